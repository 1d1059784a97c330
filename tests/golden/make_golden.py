"""Generate golden vectors by running the reference ``hqc`` package itself.

The reference (ZihangL/hqc v0.1.12) is pure Python on top of JAX.  jaxlib is
not installable here, so this script puts ``tests/golden/_jaxshim`` (a NumPy
stand-in for the JAX API subset the reference uses, see its ``_core.py``) in
front of ``sys.path`` and imports the reference's unmodified sources from the
read-only checkout.  Every number written below is therefore produced by the
reference's own code path: ``hqc/pbc/solver.py`` (make_solver and its
hf_gamma / dft_gamma / hf_kpt / dft_kpt drivers), ``hqc/pbc/scf.py``,
``hqc/tools/smearing.py``, ``hqc/tools/excor.py``, ``hqc/pbc/gto.py``,
``hqc/pbc/potential.py``, ``hqc/pbc/overlap.py``, ``hqc/pbc/slater.py``,
``hqc/pbc/lcao.py`` and ``hqc/pbc/pes.py``.

Positions come from ``numpy.random.default_rng(seed)`` (JAX's PRNG stream is
not reproducible without jaxlib).  Output: one ``.npz`` per case in this
folder plus ``manifest.json``.  Run from the repository root:

    HQC_REFERENCE=/path/to/hqc python tests/golden/make_golden.py [case-name ...]

``HQC_REFERENCE`` names the reference checkout (default: /root/reference).
"""
import json
import os
import sys
import time
import warnings

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REFERENCE = os.environ.get("HQC_REFERENCE", "/root/reference")
sys.path.insert(0, os.path.join(HERE, "_jaxshim"))
sys.path.insert(0, REFERENCE)
warnings.filterwarnings("ignore")

import jax.numpy as jnp  # noqa: E402  (the stand-in)
from hqc.pbc.solver import make_solver  # noqa: E402
from hqc.pbc.lcao import make_lcao  # noqa: E402
from hqc.pbc.pes import make_pes  # noqa: E402
from hqc.pbc.gto import make_pbc_gto  # noqa: E402
from hqc.pbc.overlap import make_overlap  # noqa: E402
from hqc.pbc.slater import make_slater  # noqa: E402
from hqc.pbc.potential import potential_energy_pp, potential_energy, kpoints, Madelung  # noqa: E402


def box(n):
    return (4.0 / 3.0 * np.pi * n) ** (1.0 / 3.0)


def uniform_positions(n, seed):
    return np.random.default_rng(seed).uniform(0.0, box(n), (n, 3))


def bcc_positions(ncell):
    """bcc lattice, ``ncell``^3 conventional cells, in rs units."""
    n = 2 * ncell ** 3
    a = box(n) / ncell
    pts = []
    for i in range(ncell):
        for j in range(ncell):
            for k in range(ncell):
                pts.append([i, j, k])
                pts.append([i + 0.5, j + 0.5, k + 0.5])
    return np.array(pts) * a


SOLVER_KEYS = ("mo_coeff", "dm", "bands", "E", "Ki", "Vep", "Vee", "Se", "converged")

# name -> (factory, n, rs, basis, seed, kwargs)
SOLVER_CASES = {
    "hf_szv_diis": ("solver", 4, 1.5, "gth-szv", 42, dict(grid_length=0.12, tol=1e-8)),
    "hf_dzv_diis": ("solver", 4, 1.5, "gth-dzv", 42, dict(grid_length=0.12, tol=1e-8)),
    "hf_dzvp_diis": ("solver", 4, 1.5, "gth-dzvp", 42, dict(grid_length=0.12, tol=1e-8)),
    "hf_dzv_fp": ("solver", 4, 1.5, "gth-dzv", 42,
                  dict(grid_length=0.12, tol=1e-10, diis=False)),
    "hf_dzv_fermi_bisect": ("solver", 4, 1.5, "gth-dzv", 42,
                            dict(grid_length=0.12, tol=1e-8, smearing=True,
                                 smearing_method="fermi", smearing_sigma=0.1)),
    "hf_dzv_gauss_bisect": ("solver", 4, 1.5, "gth-dzv", 42,
                            dict(grid_length=0.12, tol=1e-8, smearing=True,
                                 smearing_method="gauss", smearing_sigma=0.05)),
    "hf_dzv_fermi_newton": ("lcao", 4, 1.5, "gth-dzv", 42,
                            dict(grid_length=0.12, tol=1e-8, smearing=True,
                                 smearing_method="fermi", smearing_sigma=0.1)),
    "hf_h8_szv_41": ("solver", 8, 1.25, "gth-szv", 42,
                     dict(grid_length=box(8) * 1.25 / 40.0, tol=1e-8)),
    "dft_dzv_lda": ("solver", 4, 1.5, "gth-dzv", 42,
                    dict(grid_length=0.2, tol=1e-8, dft=True, xc="lda,vwn")),
    "dft_dzv_lda_fermi": ("solver", 4, 1.5, "gth-dzv", 42,
                          dict(grid_length=0.2, tol=1e-8, dft=True, xc="lda,vwn",
                               smearing=True, smearing_method="fermi",
                               smearing_sigma=0.1)),
    "dft_szv_lda_gauss": ("solver", 4, 1.5, "gth-szv", 7,
                          dict(grid_length=0.2, tol=1e-8, dft=True, xc="lda,vwn",
                               smearing=True, smearing_method="gauss",
                               smearing_sigma=0.05)),
    "dft_szv_lda_hl": ("solver", 4, 1.5, "gth-szv", 7,
                       dict(grid_length=0.2, tol=1e-8, dft=True, xc="lda,hl")),
    "dft_szv_lda_x": ("solver", 4, 1.5, "gth-szv", 7,
                      dict(grid_length=0.2, tol=1e-8, dft=True, xc="lda,")),
    "dft_szv_lda_bh72": ("solver", 4, 1.5, "gth-szv", 7,
                         dict(grid_length=0.2, tol=1e-8, dft=True, xc="lda,bh72")),
    "dft_szv_lda_gl77": ("solver", 4, 1.5, "gth-szv", 7,
                         dict(grid_length=0.2, tol=1e-8, dft=True, xc="lda,gl77")),
    "dft_dzvp_lda": ("solver", 4, 1.5, "gth-dzvp", 42,
                     dict(grid_length=0.25, tol=1e-8, dft=True, xc="lda,vwn")),
    "hf_h8_dzv_gauss_bisect": ("solver", 8, 1.4, "gth-dzv", 1,
                               dict(grid_length=box(8) * 1.4 / 24.0, tol=1e-8,
                                    smearing=True, smearing_method="gauss",
                                    smearing_sigma=0.5 * 10000 / 157888.09)),
    "pes_dev_hf_dzv": ("pes", 4, 1.5, "gth-dzv", 42,
                       dict(grid_length=0.12, tol=1e-8, mode="dev")),
    "hf_kpt_dzv": ("solver", 4, 1.5, "gth-dzv", 42,
                   dict(grid_length=0.2, tol=1e-8, gamma=False)),
    "dft_kpt_dzv": ("solver", 4, 1.5, "gth-dzv", 42,
                    dict(grid_length=0.2, tol=1e-8, gamma=False, dft=True)),
}


def run_solver_case(name):
    factory, n, rs, basis, seed, kw = SOLVER_CASES[name]
    L = box(n)
    xp = uniform_positions(n, seed)
    kpt = None
    if not kw.get("gamma", True):
        kpt = np.random.default_rng(seed + 1).uniform(-np.pi / L / rs, np.pi / L / rs, 3)
    t0 = time.time()
    if factory == "solver":
        f = make_solver(n, L, rs, basis, **kw)
    elif factory == "lcao":
        f = make_lcao(n, L, rs, basis, **kw)
    else:
        f = make_pes(n, L, rs, basis, **kw)
    args = (jnp.array(xp.copy()),) if kpt is None else (jnp.array(xp.copy()), jnp.array(kpt))
    out = f(*args)
    rec = dict(xp=xp, n=n, rs=rs, L=L)
    if kpt is not None:
        rec["kpt"] = kpt
    if factory == "solver":
        for k, v in zip(SOLVER_KEYS, out):
            rec[k] = np.asarray(v)
    elif factory == "lcao":
        for k, v in zip(("mo_coeff", "bands", "E"), out):
            rec[k] = np.asarray(v)
    else:
        for k, v in zip(("Etot", "Ki", "Vep", "Vee", "Vpp", "Se", "converged"), out):
            rec[k] = np.asarray(v)
    meta = dict(factory=factory, n=n, rs=rs, basis=basis, seed=seed, kwargs=kw,
                seconds=round(time.time() - t0, 2))
    return rec, meta


def run_gto_case():
    """eval_pbc_ao values (``hqc/pbc/gto.py:357-369``) at random electrons."""
    n, rs = 8, 1.5
    L = box(n) * rs
    rng = np.random.default_rng(43)
    xp = rng.uniform(0.0, L, (n, 3))
    xe = rng.uniform(0.0, L, (16, 3))
    rec = dict(xp=xp, xe=xe, L=L)
    for basis in ("gth-szv", "gth-dzv", "gth-dzvp"):
        f = make_pbc_gto(basis, L)
        vals = np.stack([np.asarray(f(jnp.array(xp), jnp.array(e))) for e in xe])
        rec["ao_" + basis.replace("-", "_")] = vals
    return rec, dict(n=n, rs=rs, seeds=43)


def run_gto_kpt_case():
    """eval_pbc_ao_kpt values (``hqc/pbc/gto.py:371-427``): Bloch AOs at a
    random k-point of the first Brillouin zone, random electrons."""
    n, rs = 8, 1.5
    L = box(n) * rs
    rng = np.random.default_rng(44)
    xp = rng.uniform(0.0, L, (n, 3))
    xe = rng.uniform(0.0, L, (16, 3))
    kpt = rng.uniform(-np.pi / L, np.pi / L, 3)
    rec = dict(xp=xp, xe=xe, L=L, kpt=kpt)
    for basis in ("gth-szv", "gth-dzv", "gth-dzvp"):
        f = make_pbc_gto(basis, L, gamma=False)
        vals = np.stack([np.asarray(f(jnp.array(xp), jnp.array(e), jnp.array(kpt))) for e in xe])
        rec["ao_" + basis.replace("-", "_")] = vals
    return rec, dict(n=n, rs=rs, seeds=44)


def run_slater_case():
    """make_slater (``hqc/pbc/slater.py:7-104``): the Slater matrices of one
    electron configuration with random orthonormal orbital coefficients, for
    the ground state, an excited ``state_idx`` and a k-point (complex
    coefficients).  Positions and L in rs units, as the reference takes them."""
    n, rs, basis = 8, 1.5, "gth-dzv"
    L = box(n)
    rng = np.random.default_rng(45)
    xp = rng.uniform(0.0, L, (n, 3))
    xe = rng.uniform(0.0, L, (n, 3))
    nao = 2 * n
    mo = np.linalg.qr(rng.normal(size=(nao, nao)))[0]
    moc = mo * np.exp(1j * rng.uniform(0.0, 2 * np.pi, nao))[None, :]
    kpt = rng.uniform(-np.pi / (L * rs), np.pi / (L * rs), 3)
    idx = np.array([0, 1, 2, 5, 0, 1, 3, 4])
    rec = dict(xp=xp, xe=xe, L=L, mo=mo, moc=moc, kpt=kpt, idx=idx)
    a = (jnp.array(xp), jnp.array(xe))
    up, dn = make_slater(n, L, rs, basis)(*a, jnp.array(mo))
    rec["up"], rec["dn"] = np.asarray(up), np.asarray(dn)
    up, dn = make_slater(n, L, rs, basis, groundstate=False)(*a, jnp.array(mo), jnp.array(idx))
    rec["up_x"], rec["dn_x"] = np.asarray(up), np.asarray(dn)
    up, dn = make_slater(n, L, rs, basis, gamma=False)(*a, jnp.array(moc), jnp.array(kpt))
    rec["up_k"], rec["dn_k"] = np.asarray(up), np.asarray(dn)
    return rec, dict(n=n, rs=rs, basis=basis, seeds=45)


def run_coulomb_case():
    """potential_energy (``hqc/pbc/potential.py:69-101``) of proton + electron
    walker batches, with kpoints / Madelung (6-33), as in
    ``test/tools/observables.py:8-25``: 3D (Gmax 15, kappa 10) and a 2D case."""
    rec, meta = {}, {}
    rng = np.random.default_rng(45)
    for tag, n, rs, dim, gmax in (("h8", 8, 1.31, 3, 15), ("h16", 16, 1.5, 3, 15), ("d2", 6, 1.2, 2, 10)):
        L = box(n) if dim == 3 else np.sqrt(np.pi * n)
        x = rng.uniform(-0.5 * L, 1.5 * L, (3, 2 * n, dim))  # protons then electrons, some outside the box
        G = np.asarray(kpoints(dim, gmax))
        vpp, vep, vee = potential_energy(jnp.array(x.copy()), 10.0, G, L, rs)
        rec["x_" + tag] = x
        rec["vpp_" + tag], rec["vep_" + tag], rec["vee_" + tag] = (np.asarray(v) for v in (vpp, vep, vee))
        rec["madelung_" + tag] = np.asarray(Madelung(dim, 10.0, G))
        rec["L_" + tag] = np.asarray(L)
        meta[tag] = dict(n=n, rs=rs, dim=dim, Gmax=gmax, kappa=10.0)
    return rec, meta


def run_overlap_case():
    """make_overlap (``hqc/pbc/overlap.py:11-319``) at Gamma and at a k-point,
    rcut 18 and 24, the three bases."""
    n, rs = 4, 1.5
    L = box(n)
    rng = np.random.default_rng(46)
    xp = rng.uniform(0.0, L, (n, 3))
    kpt = rng.uniform(-np.pi / L / rs, np.pi / L / rs, 3)
    rec = dict(xp=xp, kpt=kpt, L=np.asarray(L))
    for basis in ("gth-szv", "gth-dzv", "gth-dzvp"):
        tag = basis.replace("-", "_")
        for rcut in (18, 24):
            f = make_overlap(n, L, rs, basis, rcut=rcut, gamma=True, use_jit=False)
            rec[f"S_{tag}_{rcut}"] = np.asarray(f(jnp.array(xp.copy())))
        fk = make_overlap(n, L, rs, basis, rcut=24, gamma=False, use_jit=False)
        rec[f"Sk_{tag}"] = np.asarray(fk(jnp.array(xp.copy()), jnp.array(kpt)))
    return rec, dict(n=n, rs=rs, seeds=46)


def run_vpp_case():
    """potential_energy_pp (``hqc/pbc/potential.py:103-130``)."""
    rec = {}
    meta = {}
    # (tag, positions (rs units), rs)
    cases = [("n14", uniform_positions(14, 42), 1.31),
             ("n1", np.array([[0.3, 0.2, 0.1]]), 1.0),
             ("bcc16", bcc_positions(2), 1.31),
             ("n8", uniform_positions(8, 5), 1.25)]
    for tag, xp, rs in cases:
        n = xp.shape[0]
        L = box(n)
        rec["xp_" + tag] = xp
        rec["vpp_" + tag] = np.asarray(potential_energy_pp(jnp.array(xp.copy()), L, rs))
        rec["rs_" + tag] = np.asarray(rs)
        meta[tag] = dict(n=n, rs=rs)
    return rec, meta


# Central finite differences of the reference's own make_pes energy
# (pes_gamma, hqc/pbc/pes.py:78-86: E + Vpp in Ry, xp in rs units).  The
# reference has no forces (doc/solver_algorithm.md:1210) and its SCF
# while_loop is not reverse-differentiable, so these differences of its
# energy are what pins the engine's analytic gradient to the reference.
# name -> (n, rs, basis, seed, kwargs, n_coords): n_coords coordinates drawn
# from numpy.random.default_rng(seed + 100) (None: every coordinate).  The
# SCF and the chemical-potential search run to near machine precision so the
# differences carry ~1e-8 Ry/rs of noise; smeared cases use the Newton search
# (the bisection's return rule leaves N(mu) != n, so its energy has no
# stationary free energy) and record Se so that E - sigma Se can be
# differenced as well.
FD_H = 1e-4
FD_TIGHT = dict(tol=1e-10, max_cycle=300)
FD_CASES = {
    "fd_hf_szv": (4, 1.5, "gth-szv", 42, dict(grid_length=0.12, **FD_TIGHT), None),
    "fd_hf_dzv": (4, 1.5, "gth-dzv", 42, dict(grid_length=0.12, **FD_TIGHT), None),
    "fd_hf_dzv_fermi": (4, 1.5, "gth-dzv", 42,
                        dict(grid_length=0.12, smearing=True, smearing_method="fermi",
                             smearing_sigma=0.1, search_method="newton", search_tol=1e-13,
                             search_cycle=200, **FD_TIGHT), None),
    "fd_lda_dzvp": (4, 1.5, "gth-dzvp", 42,
                    dict(grid_length=0.25, dft=True, xc="lda,vwn", **FD_TIGHT), 6),
    # single k-point (pes_kpt, hqc/pbc/pes.py:88-98): the k-point is drawn as
    # in the hf_kpt_dzv solver case and held fixed while the protons move
    "fd_hf_kpt_dzv_fermi": (4, 1.5, "gth-dzv", 42,
                            dict(grid_length=0.2, gamma=False, smearing=True,
                                 smearing_method="fermi", smearing_sigma=0.1,
                                 search_method="newton", search_tol=1e-13, search_cycle=200,
                                 **FD_TIGHT), 8),
    "fd_lda_kpt_dzv": (4, 1.5, "gth-dzv", 42,
                       dict(grid_length=0.2, gamma=False, dft=True, xc="lda,vwn", **FD_TIGHT), 6),
}


def run_fd_case(name):
    n, rs, basis, seed, kw, ncoord = FD_CASES[name]
    L = box(n)
    xp = uniform_positions(n, seed)
    t0 = time.time()
    pes = make_pes(n, L, rs, basis, mode="dev", **kw)
    sigma = kw.get("smearing_sigma", 0.0) if kw.get("smearing") else 0.0
    kpt = None
    if not kw.get("gamma", True):
        kpt = np.random.default_rng(seed + 1).uniform(-np.pi / L / rs, np.pi / L / rs, 3)

    def ev(x):
        args = (jnp.array(x.copy()),) if kpt is None else (jnp.array(x.copy()), jnp.array(kpt))
        Etot, Ki, Vep, Vee, Vpp, Se, conv = pes(*args)
        assert bool(np.asarray(conv)), "reference SCF did not converge"
        return float(np.asarray(Etot)), float(np.asarray(Se)), float(np.asarray(Vpp))

    coords = [(a, d) for a in range(n) for d in range(3)]
    if ncoord is not None:
        pick = np.random.default_rng(seed + 100).choice(len(coords), ncoord, replace=False)
        coords = [coords[i] for i in sorted(pick)]
    E0, S0, V0 = ev(xp)
    dE, dF = [], []
    for a, d in coords:
        vals = []
        for sgn in (1.0, -1.0):
            x = xp.copy()
            x[a, d] += sgn * FD_H
            vals.append(ev(x))
        (Ep, Sp, _), (Em, Sm, _) = vals
        dE.append((Ep - Em) / (2 * FD_H))
        # free energy F = E - sigma Se (sigma in Hartree, E in Ry: factor 2)
        dF.append(((Ep - 2 * sigma * Sp) - (Em - 2 * sigma * Sm)) / (2 * FD_H))
    rec = dict(xp=xp, n=n, rs=rs, L=L, h=FD_H, coords=np.array(coords), Etot=E0, Se=S0, Vpp=V0,
               dEtot=np.array(dE), dFtot=np.array(dF), sigma=sigma)
    if kpt is not None:
        rec["kpt"] = kpt
    meta = dict(factory="pes_fd", n=n, rs=rs, basis=basis, seed=seed, kwargs=kw, h=FD_H,
                coords=len(coords), seconds=round(time.time() - t0, 2))
    return rec, meta


def main(selected):
    manifest_path = os.path.join(HERE, "manifest.json")
    manifest = json.load(open(manifest_path)) if os.path.exists(manifest_path) else {}
    jobs = list(SOLVER_CASES) + ["gto_values", "gto_values_kpt", "vpp", "coulomb_pe", "overlap",
                                 "slater"] + list(FD_CASES)
    if selected:
        jobs = [j for j in jobs if j in selected]
    for name in jobs:
        t0 = time.time()
        if name == "gto_values":
            rec, meta = run_gto_case()
        elif name == "gto_values_kpt":
            rec, meta = run_gto_kpt_case()
        elif name == "coulomb_pe":
            rec, meta = run_coulomb_case()
        elif name == "overlap":
            rec, meta = run_overlap_case()
        elif name == "slater":
            rec, meta = run_slater_case()
        elif name == "vpp":
            rec, meta = run_vpp_case()
        elif name in FD_CASES:
            rec, meta = run_fd_case(name)
        else:
            rec, meta = run_solver_case(name)
        np.savez(os.path.join(HERE, name + ".npz"), **rec)
        manifest[name] = meta
        print(f"{name}: {time.time() - t0:.1f}s", {k: rec[k] for k in ("E", "converged") if k in rec},
              flush=True)
        with open(manifest_path, "w") as fh:
            json.dump(manifest, fh, indent=1, sort_keys=True)


if __name__ == "__main__":
    main(sys.argv[1:])
