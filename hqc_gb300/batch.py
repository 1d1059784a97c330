"""Uneven batches: energies and forces of many configurations of different
atom counts, box sizes and grids in one engine call (``hqcgb_batch_run``).

The reference batches with ``jax.vmap`` over configurations of one shape
(``test/test.py:157,179``), so a mixed set of system sizes needs one vmapped
call per shape there.  ``make_pes_batch`` takes the factory arguments of
``make_pes`` (``hqc/pbc/pes.py:10-31``) that are common to all
configurations -- basis, method, smearing, SCF controls -- and returns
``pes_batch(configs)`` for configurations that each bring their own

    (xp, L, rs, n_grid):  positions (n, 3) and box side L in rs units (as the
                          reference's xp and L), rs, grid points per axis
                          (odd for parity with the reference, solver.py:159;
                          ``grid_size(L * rs, grid_length)`` gives the
                          reference's choice).

The engine groups the configurations into size classes (n, n_grid); each of
``workers`` host threads keeps one workspace per size class and resets its
box-dependent tables per configuration, taking configurations largest first.
"""
import ctypes
import weakref

import numpy as np
import torch

from . import _lib
from .solver import RY, build_params
from .potential import potential_energy_pp_and_grad


def make_pes_batch(basis, rcut=24, tol=1e-7, max_cycle=100, diis=True, diis_space=8,
                   diis_start_cycle=1, diis_damp=0., dft=False, xc='lda,vwn', smearing=False,
                   smearing_method='fermi', smearing_sigma=0., search_method='bisect',
                   search_cycle=100, search_tol=1e-7, Gmax=15, kappa=10, precision='fp64',
                   forces=False, exx_occ_threshold=0.0, workers=1):
    """Batch PES factory.  ``pes_batch(configs)`` returns a dict:

    * ``E``: (B,) E + Vpp in Rydberg, the reference's ``pes(xp)`` per
      configuration (hqc/pbc/pes.py:78-86);
    * ``F``: (B,) free energy F + Vpp (F = E - sigma S, E without smearing),
      the value whose gradient ``grad`` is;
    * ``grad`` (forces=True): list of (n_c, 3) dF/dxp in Rydberg per rs unit;
    * ``bands`` (list of (nao_c,) Rydberg), ``Se``, ``converged``,
      ``iterations`` per configuration.
    """
    lib = _lib.load()
    if not torch.cuda.is_available():
        raise RuntimeError("hqc_gb300 needs a CUDA GPU (no CPU fallback)")
    P, keep, nao_atom = build_params(1, 1.0, 3, basis, rcut, tol, max_cycle, diis, diis_space,
                                     diis_start_cycle, diis_damp, dft, xc, smearing, smearing_method,
                                     smearing_sigma, search_method, search_cycle, search_tol,
                                     precision, forces, exx_occ_threshold)
    h = ctypes.c_void_p()
    _lib.check(lib.hqcgb_batch_create(ctypes.byref(P), float(rcut), int(workers), ctypes.byref(h)))
    device = torch.device("cuda", torch.cuda.current_device())

    def _pos(x):
        if isinstance(x, torch.Tensor):
            return x.detach().to(dtype=torch.float64)
        return torch.as_tensor(np.asarray(x, dtype=np.float64))

    def pes_batch(configs):
        B = len(configs)
        xs = [_pos(c[0]) for c in configs]
        n = np.array([x.shape[0] for x in xs], dtype=np.int32)
        grid = np.array([int(c[3]) for c in configs], dtype=np.int32)
        L_rs = np.array([float(c[1]) for c in configs])
        rs = np.array([float(c[2]) for c in configs])
        L_bohr = np.ascontiguousarray(L_rs * rs)
        xp = torch.cat([x.to(device) * r for x, r in zip(xs, rs)]).contiguous()
        nao = n.astype(np.int64) * nao_atom
        aoff = np.concatenate([[0], np.cumsum(nao)])
        xoff = np.concatenate([[0], np.cumsum(n)])
        out = dict(bands=torch.empty(int(aoff[-1]), dtype=torch.float64, device=device),
                   energies=torch.empty(B, 5, dtype=torch.float64, device=device),
                   converged=torch.zeros(B, dtype=torch.int32, device=device),
                   iterations=torch.zeros(B, dtype=torch.int32, device=device),
                   free_energy=torch.empty(B, dtype=torch.float64, device=device))
        ptr = lambda k: ctypes.c_void_p(out[k].data_ptr()) if k in out else ctypes.c_void_p(0)
        o = _lib.ScfOut(*[ptr(k) for k in ("mo_coeff", "dm", "bands", "energies", "converged",
                                            "iterations", "free_energy")])
        g = torch.empty(int(xoff[-1]), 3, dtype=torch.float64, device=device) if forces else None
        st = ctypes.c_void_p(torch.cuda.current_stream(device).cuda_stream)
        status = lib.hqcgb_batch_run(h, B, n.ctypes.data_as(_lib.c_int_p), grid.ctypes.data_as(_lib.c_int_p),
                                     L_bohr.ctypes.data_as(_lib.c_double_p), ctypes.c_void_p(xp.data_ptr()),
                                     ctypes.byref(o), ctypes.c_void_p(g.data_ptr() if g is not None else 0),
                                     st)
        _lib.check(status, allow=(0, 1))
        vpp = [potential_energy_pp_and_grad(x, Lc, r, kappa=kappa, Gmax=Gmax)
               for x, Lc, r in zip(xs, L_rs, rs)]
        Vpp = torch.stack([v[0] for v in vpp])
        e = out["energies"]
        res = dict(E=e[:, 0] * RY + Vpp, F=out["free_energy"] * RY + Vpp, Se=e[:, 4],
                   converged=out["converged"] != 0, iterations=out["iterations"].tolist(),
                   bands=[out["bands"][aoff[c]:aoff[c + 1]] * RY for c in range(B)])
        if forces:
            res["grad"] = [g[xoff[c]:xoff[c + 1]] * (RY * rs[c]) + vpp[c][1] for c in range(B)]
        return res

    pes_batch.handle = h
    pes_batch._keep = keep
    pes_batch._finalizer = weakref.finalize(pes_batch, lib.hqcgb_batch_destroy, h)
    return pes_batch
