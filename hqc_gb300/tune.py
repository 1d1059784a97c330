"""Autotuner: picks the engine's launch-shape knobs by timing candidates on
this GPU at the shapes of the run at hand, and remembers the choice.

Knobs (``hqcgb_tune_set``; each changes launch shapes only, so results agree
to rounding):

* ``quad_groups``: K slices of the persistent tensor-core Fock quadrature
  (one CTA group of the destination tiles per slice; at most one CTA per
  SM).  Fewer slices leave SMs to the kernels of concurrent configurations;
  more slices use the whole GPU for one quadrature.
* ``quad_kchunk``: grid points per CTA of the tile-list form (AO counts the
  persistent form does not take).  Longer chunks mean fewer FP64 partial
  tiles to reduce but fewer CTAs and a larger working set per CTA.
  Both are timed on the PBE quadrature (``hqcgb_tc_quadrature_gga``) with
  synthetic operands of the run's shape.
* ``exx_group`` and ``exx_gram_ctas``: orbitals per exact-exchange group and
  the CTA count of its tensor-core Gram matrix.  Timed on the exchange build
  of a converged Hartree-Fock SCF (``hqcgb_exchange_rebuild``) of the run's
  shape; both are read when a plan is created.

Choices are cached per GPU name and shape in a JSON file
(``$HQCGB_TUNE_CACHE``, default ``~/.cache/hqc_gb300/tune.json``) and applied
on later runs without timing.  The reference has no counterpart: XLA picks
its own launch shapes.
"""
import ctypes
import json
import os

import numpy as np
import torch

from . import _lib

CACHE = os.environ.get("HQCGB_TUNE_CACHE",
                       os.path.join(os.path.expanduser("~"), ".cache", "hqc_gb300", "tune.json"))


def _load():
    try:
        with open(CACHE) as fh:
            return json.load(fh)
    except (OSError, ValueError):
        return {}


def _save(d):
    try:
        os.makedirs(os.path.dirname(CACHE), exist_ok=True)
        with open(CACHE, "w") as fh:
            json.dump(d, fh, indent=1, sort_keys=True)
    except OSError:
        pass  # a read-only home: the choice still applies to this process


def set_knob(name, value):
    """Set a knob (value <= 0 restores its default)."""
    _lib.check(_lib.load().hqcgb_tune_set(name.encode(), int(value)))


def get_knob(name):
    return int(_lib.load().hqcgb_tune_get(name.encode()))


def _time_ms(fn, reps):
    fn()  # warm (first launches raise shared-memory limits, build tensor maps)
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(reps):
        fn()
    b.record()
    torch.cuda.synchronize()
    return a.elapsed_time(b) / reps


def _cached(key, measure, use_cache=True):
    cache = _load() if use_cache else {}
    if key in cache:
        return cache[key], None
    best, table = measure()
    if use_cache:
        cache = _load()
        cache[key] = best
        _save(cache)
    return best, table


def tune_quadrature(nao, ng, candidates=(2048, 4096, 8192, 16384), reps=4, use_cache=True):
    """Launch shape of the PBE Fock quadrature at nao AOs on an ng^3 grid:
    the number of K slices (CTA groups) when the shape takes the persistent
    form, else the K chunk of the tile-list form.  Sets the knob and returns
    (knob, value) (with the timing table when it was measured)."""
    tiles, _ = _lib.quad_tiles(nao, False)
    ntile = int((tiles[:, 0] == 0).sum())
    if ntile:
        sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
        full = max(1, sms // ntile)
        knob, cands = "quad_groups", sorted({max(1, full // 2), max(1, (3 * full) // 4), full})
    else:
        knob, cands = "quad_kchunk", candidates
    key = f"{torch.cuda.get_device_name()}|{knob}|{nao}|{ng}"

    def measure():
        N = ng ** 3
        ld = (N + 63) // 64 * 64
        g = torch.Generator(device="cuda").manual_seed(1)
        phi = torch.zeros(nao, ld, dtype=torch.float32, device="cuda")
        phi[:, :N] = torch.randn(nao, N, generator=g, device="cuda")
        dphi = torch.zeros(3 * nao, ld, dtype=torch.float32, device="cuda")
        dphi[:, :N] = torch.randn(3 * nao, N, generator=g, device="cuda")
        w = torch.zeros(ld, dtype=torch.float32, device="cuda")
        w[:N] = torch.rand(N, generator=g, device="cuda")
        u = torch.zeros(3, ld, dtype=torch.float32, device="cuda")
        u[:, :N] = torch.randn(3, N, generator=g, device="cuda")
        table = {}
        for c in cands:
            set_knob(knob, c)
            table[c] = _time_ms(lambda: _lib.tc_quadrature_gga(phi, dphi, w, u, 1e-3, N, drain=4), reps)
        del phi, dphi
        torch.cuda.empty_cache()
        return int(min(table, key=table.get)), table

    best, table = _cached(key, measure, use_cache)
    set_knob(knob, best)
    return (knob, best), table


def tune_exchange(n, L, rs, grid, basis="gth-dzv", groups=(4, 8, 16), ctas=(152, 304, 608), reps=3,
                  use_cache=True, **scf_kw):
    """Orbital group size and Gram CTA count of the exact exchange of an
    n-atom Hartree-Fock system (box L, rs units; grid^3 points); sets and
    returns (group, ctas) (with the timing table when it was measured)."""
    from .solver import make_solver
    key = f"{torch.cuda.get_device_name()}|exx|{n}|{grid}|{basis}"
    rng = np.random.default_rng(17)
    xp = rng.uniform(0.0, L, (n, 3))

    def measure():
        lib = _lib.load()
        table = {}
        for gsz in groups:
            for c in ctas:
                set_knob("exx_group", gsz)
                set_knob("exx_gram_ctas", c)
                s = make_solver(n, L, rs, basis, precision="mixed", n_grid=grid, **scf_kw)
                s(xp)
                st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
                table[f"{gsz}x{c}"] = _time_ms(lambda: lib.hqcgb_exchange_rebuild(s.plan.handle, st), reps)
                del s
        best = min(table, key=table.get)
        return [int(v) for v in best.split("x")], table

    best, table = _cached(key, measure, use_cache)
    set_knob("exx_group", best[0])
    set_knob("exx_gram_ctas", best[1])
    return tuple(best), table
