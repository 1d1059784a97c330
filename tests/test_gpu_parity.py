"""GPU parity of the FP64 engine path against the reference's golden vectors
and the CPU oracle.

Tolerances (FP64 everywhere on both sides; differences come from summation
order, the Jacobi vs LAPACK eigensolver and SCF stopping noise at tol 1e-8):
energies 1e-8 Ry, bands 1e-6 Ry, density matrix 1e-6, S/T/V 1e-11, forces
1e-7 Ha/Bohr against the oracle's analytic gradient.
"""
import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu

CASES = ["hf_szv_diis", "hf_dzv_diis", "hf_dzvp_diis", "hf_dzv_fp", "hf_dzv_fermi_bisect",
         "hf_dzv_fermi_newton", "hf_h8_szv_41", "dft_dzv_lda", "dft_dzv_lda_fermi",
         "dft_szv_lda_gauss", "dft_szv_lda_hl", "dft_szv_lda_x", "dft_dzvp_lda"]


def _np(t):
    return t.detach().cpu().numpy()


def make(meta, z, **extra):
    from hqc_gb300 import make_solver, make_lcao
    kw = dict(meta["kwargs"])
    kw.pop("mode", None)
    kw.update(extra)
    if meta["factory"] == "lcao":
        return make_lcao(meta["n"], float(z["L"]), meta["rs"], meta["basis"], **kw).solver
    return make_solver(meta["n"], float(z["L"]), meta["rs"], meta["basis"], **kw)


@pytest.mark.parametrize("name", CASES)
def test_scf_matches_reference_golden(name):
    meta, z = load_golden(name)
    s = make(meta, z)
    out = s(z["xp"])
    assert abs(float(out[3]) - float(z["E"])) < 1e-8
    np.testing.assert_allclose(_np(out[2]), z["bands"], atol=1e-6)
    if "dm" in z.files:
        np.testing.assert_allclose(_np(out[1]), z["dm"], atol=1e-6)
        for k, i in (("Ki", 4), ("Vep", 5), ("Vee", 6), ("Se", 7)):
            assert abs(float(out[i]) - float(z[k])) < 1e-7, k
        assert bool(out[8]) == bool(z["converged"])


def test_pes_dev_matches_reference_golden():
    from hqc_gb300 import make_pes
    meta, z = load_golden("pes_dev_hf_dzv")
    kw = dict(meta["kwargs"])
    out = make_pes(meta["n"], float(z["L"]), meta["rs"], meta["basis"], **kw)(z["xp"])
    for k, v in zip(("Etot", "Ki", "Vep", "Vee", "Vpp", "Se"), out[:6]):
        assert abs(float(v) - float(z[k])) < 1e-8, k
    assert bool(out[6])


def test_vpp_matches_reference_golden():
    from hqc_gb300 import potential_energy_pp
    _, z = load_golden("vpp")
    for tag in ("n14", "n1", "bcc16", "n8"):
        xp = z["xp_" + tag]
        n = xp.shape[0]
        L = (4 / 3 * np.pi * n) ** (1 / 3)
        v = float(potential_energy_pp(xp, L, float(z["rs_" + tag])))
        assert abs(v - float(z["vpp_" + tag])) < 1e-10, tag


def test_components_match_oracle():
    """S, T, V, the AO grid and v_loc against the oracle at an H4 dzvp case."""
    from hqc_gb300 import make_solver
    from oracle.gpw import Solver
    n, rs = 4, 1.5
    L = (4 / 3 * np.pi * n) ** (1 / 3)
    xp = np.random.default_rng(3).uniform(0, L, (n, 3))
    s = make_solver(n, L, rs, "gth-dzvp", grid_length=0.3, dft=True, tol=1e-9)
    s(xp)
    ref = Solver(n, L, rs, "gth-dzvp", grid_length=0.3, dft=True, tol=1e-9)
    g = ref.setup_geometry(xp)
    nao = ref.st.nao
    for key, val in (("S", g["S"]), ("T", g["T"]), ("V", g["V"])):
        np.testing.assert_allclose(_np(s.plan.query(key)).reshape(nao, nao), val, atol=1e-11)
    np.testing.assert_allclose(_np(s.plan.query("vloc")), g["vloc"].ravel(), atol=1e-10)
    np.testing.assert_allclose(_np(s.plan.query("phi")), g["phi"].ravel(), atol=1e-12)


@pytest.mark.parametrize("basis,xc", [("gth-dzvp", "pbe"), ("gth-dzv", "pbe"), ("gth-szv", "lda,hl")])
def test_dft_energy_matches_oracle(basis, xc):
    """PBE has no reference implementation; the oracle is the checker."""
    from hqc_gb300 import make_solver
    from oracle.gpw import Solver
    n, rs = 4, 1.31
    L = (4 / 3 * np.pi * n) ** (1 / 3)
    xp = np.random.default_rng(7).uniform(0, L, (n, 3))
    kw = dict(grid_length=0.25, dft=True, xc=xc, tol=1e-9)
    out = make_solver(n, L, rs, basis, **kw)(xp)
    ro = Solver(n, L, rs, basis, **kw).solve(xp)
    assert abs(float(out[3]) - ro[3]) < 1e-8
    np.testing.assert_allclose(_np(out[2]), ro[2], atol=1e-6)


@pytest.mark.parametrize("basis,kw", [
    ("gth-dzvp", dict(dft=True, xc="lda,vwn")),
    ("gth-dzvp", dict(dft=True, xc="pbe")),
    ("gth-dzv", dict(dft=False)),
    ("gth-szv", dict(dft=True, xc="lda,vwn", smearing=True, smearing_sigma=0.05,
                     search_method="newton", search_tol=1e-12)),
])
def test_forces_match_oracle(basis, kw):
    from hqc_gb300 import make_solver
    from oracle.gpw import Solver
    from oracle.forces import electronic_gradient
    n, rs = 4, 1.5
    L = (4 / 3 * np.pi * n) ** (1 / 3)
    xp = np.random.default_rng(42).uniform(0, L, (n, 3))
    common = dict(grid_length=0.25, tol=1e-10, max_cycle=200)
    s = make_solver(n, L, rs, basis, forces=True, **common, **kw)
    s(xp)
    g = _np(s.plan.forces())
    ref = Solver(n, L, rs, basis, **common, **kw)
    ref.solve(xp)
    rg = electronic_gradient(ref)
    np.testing.assert_allclose(g, rg, atol=1e-7)


def test_ewald_gradient_matches_oracle():
    from hqc_gb300 import potential_energy_pp_and_grad
    from oracle.ewald import vpp
    n, rs = 16, 1.31
    L = (4 / 3 * np.pi * n) ** (1 / 3)
    xp = np.random.default_rng(5).uniform(-0.5, L + 0.5, (n, 3))
    e, g = potential_energy_pp_and_grad(xp, L, rs)
    re_, rg = vpp(xp, L, rs, grad=True)
    assert abs(float(e) - re_) < 1e-10
    np.testing.assert_allclose(_np(g), rg, atol=1e-10)


def test_failure_status_not_converged():
    """max_cycle reached is reported as converged=False, not an exception
    (scf.py:240, pes.py:111-115)."""
    from hqc_gb300 import make_solver
    meta, z = load_golden("hf_dzv_diis")
    s = make(meta, z, max_cycle=10)
    out = s(z["xp"])
    assert not bool(out[8])


def test_coincident_atoms_raise():
    """Two protons on top of each other make S singular: the engine reports
    it as an error status (raised here), not a NaN result or a device fault."""
    from hqc_gb300 import make_solver
    from hqc_gb300._lib import HqcgbError
    n, rs = 4, 1.5
    L = (4 / 3 * np.pi * n) ** (1 / 3)
    xp = np.random.default_rng(42).uniform(0, L, (n, 3))
    xp[1] = xp[0]
    s = make_solver(n, L, rs, "gth-dzv", grid_length=0.3)
    with pytest.raises(HqcgbError):
        s(xp)


@pytest.mark.parametrize("n,batch", [(1, 1), (2, 3), (33, 2), (160, 1), (270, 2)])
def test_eigensolver_matches_lapack(n, batch):
    import torch
    from hqc_gb300._lib import eigh
    rng = np.random.default_rng(n)
    M = rng.normal(size=(batch, n, n))
    M = M + np.transpose(M, (0, 2, 1))
    if n >= 160:  # a clustered spectrum like a symmetric lattice's bands
        Q = np.linalg.qr(rng.normal(size=(n, n)))[0]
        lam = np.repeat(np.linspace(-2, 3, n // 10), 10)[:n] + 1e-9 * rng.normal(size=n)
        M[0] = (Q * lam) @ Q.T
        M[0] = 0.5 * (M[0] + M[0].T)
    w, V = eigh(torch.as_tensor(M, device="cuda"))
    w, V = _np(w), _np(V)
    for b in range(batch):
        np.testing.assert_allclose(w[b], np.linalg.eigvalsh(M[b]), atol=1e-12 * max(1, np.abs(M[b]).max()))
        np.testing.assert_allclose(V[b].T @ V[b], np.eye(n), atol=1e-12)
        np.testing.assert_allclose(M[b] @ V[b], V[b] * w[b], atol=1e-11 * max(1, np.abs(M[b]).max()))


def test_h16_dzvp_pbe_forces_match_oracle():
    """A system above one warp of AOs (80) exercising every block reduction."""
    from hqc_gb300 import make_solver
    from oracle.gpw import Solver
    from oracle.forces import electronic_gradient
    n, rs = 16, 1.31
    L = (4 / 3 * np.pi * n) ** (1 / 3)
    xp = np.random.default_rng(11).uniform(0, L, (n, 3))
    kw = dict(grid_length=L * rs / 24, dft=True, xc="pbe", tol=1e-9, max_cycle=100)
    s = make_solver(n, L, rs, "gth-dzvp", forces=True, **kw)
    out = s(xp)
    g = _np(s.plan.forces())
    ref = Solver(n, L, rs, "gth-dzvp", **kw)
    ro = ref.solve(xp)
    assert abs(float(out[3]) - ro[3]) < 1e-8
    np.testing.assert_allclose(_np(out[2]), ro[2], atol=1e-6)
    np.testing.assert_allclose(g, electronic_gradient(ref), atol=1e-7)


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-7), ("mixed", 2e-6)])
def test_energy_periodic_in_lattice_translations(precision, tol):
    """Shifting protons by lattice vectors is the same crystal: energy and
    forces agree (the reference checks the periodicity of its GTO values,
    test/test_pbc_gto.py:116-127).  Not to rounding: like the reference, the
    engine does not wrap positions into the box (hqc/pbc/solver.py:722) and
    sums S and T over a fixed sphere of lattice vectors of radius 24 Bohr
    (solver.py:162-176), so a shift changes which far images of the most
    diffuse primitives are included, by about exp(-mu (24 - |R|)^2) ~ 1e-8."""
    from hqc_gb300 import make_solver
    n, rs = 8, 1.5
    L = (4 / 3 * np.pi * n) ** (1 / 3)
    xp = np.random.default_rng(21).uniform(0, L, (n, 3))
    s = make_solver(n, L, rs, "gth-dzv", grid_length=L * rs / 30, dft=True, xc="pbe", tol=1e-9,
                    precision=precision, forces=True)
    e0 = float(s(xp)[3])
    g0 = _np(s.plan.forces())
    shifted = xp + np.array([L, 0.0, -2 * L])
    shifted[3] -= np.array([0.0, L, 0.0])
    e1 = float(s(shifted)[3])
    g1 = _np(s.plan.forces())
    assert abs(e1 - e0) < tol
    np.testing.assert_allclose(g1, g0, atol=1e-6)
