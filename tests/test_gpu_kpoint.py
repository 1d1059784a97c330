"""GPU parity of the single k-point solver (make_solver(gamma=False);
hf_kpt / dft_kpt, hqc/pbc/solver.py:769-962) against the reference's
k-point goldens and the CPU oracle, and of its complex Hermitian eigensolver.

Tolerances (FP64 on both sides; differences from summation order, the
eigensolver and SCF stopping noise at tol 1e-8): energies 1e-8 Ry, bands
1e-6 Ry, density matrix 1e-6, S/T/V 1e-11, eigen-residuals 1e-12 relative.
"""
import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu


def _np(t):
    return t.detach().cpu().numpy()


def _kpt_solver(meta, z, **extra):
    from hqc_gb300 import make_solver
    kw = dict(meta["kwargs"])
    kw.update(extra)
    return make_solver(meta["n"], float(z["L"]), meta["rs"], meta["basis"], **kw)


def _hermitian(rng, n, b=1, spectrum=None):
    X = rng.normal(size=(b, n, n)) + 1j * rng.normal(size=(b, n, n))
    if spectrum is None:
        return X + np.conj(np.swapaxes(X, 1, 2))
    Q, _ = np.linalg.qr(X)
    return np.einsum("bij,j,bkj->bik", Q, spectrum, np.conj(Q))


@pytest.mark.parametrize("n,b,kind", [(1, 1, "random"), (2, 3, "random"), (37, 2, "random"),
                                      (130, 1, "random"), (64, 1, "degenerate")])
def test_eigh_herm(n, b, kind):
    import torch
    from hqc_gb300 import _lib
    rng = np.random.default_rng(n + b)
    spec = None
    if kind == "degenerate":
        spec = np.repeat(np.arange(n // 4, dtype=float), 4)  # four-fold degenerate levels
    A = _hermitian(rng, n, b, spec)
    At = torch.tensor(A, dtype=torch.complex128, device="cuda")
    w, V = _lib.eigh_herm(At)
    w, V = _np(w), _np(V)
    scale = np.abs(np.linalg.eigvalsh(A)).max()
    np.testing.assert_allclose(w, np.linalg.eigvalsh(A), atol=1e-12 * scale)
    resid = np.einsum("bij,bjk->bik", A, V) - V * w[:, None, :]
    assert np.abs(resid).max() < 1e-12 * scale
    I = np.einsum("bji,bjk->bik", np.conj(V), V)
    assert np.abs(I - np.eye(n)).max() < 1e-12
    assert np.array_equal(_np(At), A)  # input left untouched


@pytest.mark.parametrize("name", ["hf_kpt_dzv", "dft_kpt_dzv"])
def test_kpoint_scf_matches_reference_golden(name):
    meta, z = load_golden(name)
    s = _kpt_solver(meta, z)
    out = s(z["xp"], z["kpt"])
    assert abs(float(out[3]) - float(z["E"])) < 1e-8
    np.testing.assert_allclose(_np(out[2]), z["bands"], atol=1e-6)
    np.testing.assert_allclose(_np(out[1]), z["dm"], atol=1e-6)
    for k, i in (("Ki", 4), ("Vep", 5), ("Vee", 6), ("Se", 7)):
        assert abs(float(out[i]) - float(z[k])) < 1e-7, k
    assert bool(out[8]) == bool(z["converged"])
    # MO columns equal the reference's up to a phase: |c_ref^H S c| = 1
    import torch
    S = s.plan.query("S").reshape(-1, 2)
    S = _np(torch.view_as_complex(S.contiguous())).reshape(out[0].shape)
    ov = np.abs(np.sum(np.conj(z["mo_coeff"]) * (S @ _np(out[0])), axis=0))
    np.testing.assert_allclose(ov, 1.0, atol=1e-6)


def test_kpoint_integrals_match_oracle():
    """S^k, T^k (phase-weighted lattice sums) and V^k (grid quadrature)."""
    import torch
    from oracle.gpw import Solver
    meta, z = load_golden("hf_kpt_dzv")
    s = _kpt_solver(meta, z)
    s(z["xp"], z["kpt"])
    kw = dict(meta["kwargs"])
    kw.pop("gamma")
    o = Solver(meta["n"], float(z["L"]), meta["rs"], meta["basis"], **kw)
    g = o.setup_geometry(z["xp"], z["kpt"])
    nao = g["S"].shape[0]
    for key in ("S", "T", "V", "St"):
        t = s.plan.query(key).reshape(-1, 2).contiguous()
        M = _np(torch.view_as_complex(t)).reshape(nao, nao)
        ref = g["Stilde"] if key == "St" else g[key]
        np.testing.assert_allclose(M, ref, atol=1e-11, err_msg=key)


CASES = [
    # (n, basis, kwargs, seed)
    (4, "gth-dzv", dict(dft=True, xc="lda,vwn", smearing=True, smearing_sigma=0.05), 5),
    (4, "gth-szv", dict(dft=True, xc="pbe"), 6),
    (4, "gth-szv", dict(diis=False), 7),
    (4, "gth-dzvp", dict(smearing=True, smearing_method="gauss", smearing_sigma=0.02, dft=True), 8),
    (8, "gth-dzv", dict(), 9),
]


@pytest.mark.parametrize("n,basis,kw,seed", CASES)
def test_kpoint_scf_matches_oracle(n, basis, kw, seed):
    from hqc_gb300 import make_solver
    from oracle.gpw import Solver
    rng = np.random.default_rng(seed)
    rs, L = 1.5, (4 * np.pi * n / 3) ** (1 / 3)
    xp = rng.uniform(0, L, size=(n, 3))
    kpt = rng.uniform(-np.pi / L / rs, np.pi / L / rs, 3)
    common = dict(grid_length=0.2, tol=1e-8, **kw)
    out = make_solver(n, L, rs, basis, gamma=False, **common)(xp, kpt)
    ref = Solver(n, L, rs, basis, **common).solve(xp, kpt)
    assert bool(out[8]) == bool(ref[8])
    assert abs(float(out[3]) - ref[3]) < 1e-8
    np.testing.assert_allclose(_np(out[2]), ref[2], atol=1e-6)
    np.testing.assert_allclose(_np(out[1]), ref[1], atol=1e-6)
    for i in (4, 5, 6, 7):
        assert abs(float(out[i]) - ref[i]) < 1e-7, i


def test_kpoint_gamma_limit_equals_gamma_solver():
    from hqc_gb300 import make_solver
    meta, z = load_golden("hf_dzv_diis")
    kw = dict(meta["kwargs"])
    args = (meta["n"], float(z["L"]), meta["rs"], meta["basis"])
    g = make_solver(*args, **kw)(z["xp"])
    k = make_solver(*args, gamma=False, **kw)(z["xp"], np.zeros(3))
    assert abs(float(g[3]) - float(k[3])) < 1e-9
    np.testing.assert_allclose(_np(g[2]), _np(k[2]), atol=1e-8)
    np.testing.assert_allclose(_np(g[1]), _np(k[1]).real, atol=1e-8)
    assert np.abs(_np(k[1]).imag).max() < 1e-10


def test_kpoint_time_reversal_and_batch():
    """E(k) = E(-k) (H^-k = conj(H^k)); a batch over (xp, kpt) equals the
    single calls bit for bit, and pes(xp, kpt) adds the Ewald energy."""
    from hqc_gb300 import make_solver, make_pes, potential_energy_pp
    meta, z = load_golden("dft_kpt_dzv")
    kw = dict(meta["kwargs"])
    args = (meta["n"], float(z["L"]), meta["rs"], meta["basis"])
    s = make_solver(*args, **kw)
    k = np.asarray(z["kpt"])
    a = s(z["xp"], k)
    b = s(z["xp"], -k)
    assert abs(float(a[3]) - float(b[3])) < 1e-9
    np.testing.assert_allclose(_np(a[2]), _np(b[2]), atol=1e-8)
    np.testing.assert_allclose(_np(a[1]), np.conj(_np(b[1])), atol=1e-7)
    ks = np.stack([k, -k, 0.5 * k])
    batch = s(z["xp"], ks)
    for j, kk in enumerate(ks):
        one = s(z["xp"], kk)
        assert float(batch[3][j]) == float(one[3])
        assert np.array_equal(_np(batch[2][j]), _np(one[2]))
    pes = make_pes(*args, **kw)
    Vpp = float(potential_energy_pp(z["xp"], float(z["L"]), meta["rs"]))
    assert abs(float(pes(z["xp"], k)) - (float(a[3]) + Vpp)) < 1e-10


# Mixed-precision k-point solver (Hartree-Fock and LDA): grid contractions on
# the tensor cores through the real embedding of the complex AO grid, FP32
# pair transforms for the exchange, FP64 eigensolver.  Bound: the metric's
# 1e-6 Ha/atom on the energy; occupied bands within 2e-5 Ry.
MIXED_CASES = [
    ("golden", "hf_kpt_dzv", None),
    ("golden", "dft_kpt_dzv", None),
    ("random", 16, dict(smearing=True, smearing_method="fermi", smearing_sigma=0.5 * 10000 / 157888.09,
                        search_method="newton", grid_length=None)),
]


@pytest.mark.parametrize("kind,case,kw", MIXED_CASES)
def test_kpoint_mixed_matches_fp64(kind, case, kw):
    from hqc_gb300 import make_solver
    if kind == "golden":
        meta, z = load_golden(case)
        n = meta["n"]
        s64 = _kpt_solver(meta, z)
        s32 = _kpt_solver(meta, z, precision="mixed")
        xp, kpt = z["xp"], z["kpt"]
        nocc = n // 2
    else:
        n, rs = case, 1.4
        L = (4 * np.pi * n / 3) ** (1 / 3)
        rng = np.random.default_rng(11)
        xp = rng.uniform(0, L, size=(n, 3))
        kpt = rng.uniform(-np.pi / L / rs, np.pi / L / rs, 3)
        common = dict(kw, grid_length=L * rs / 48.0, tol=1e-7, max_cycle=100, gamma=False)
        s64 = make_solver(n, L, rs, "gth-dzv", **common)
        s32 = make_solver(n, L, rs, "gth-dzv", precision="mixed", **common)
        nocc = n // 2
    o64, o32 = s64(xp, kpt), s32(xp, kpt)
    dE = abs(float(o32[3]) - float(o64[3])) / 2 / n
    dB = np.abs(_np(o32[2])[:nocc] - _np(o64[2])[:nocc]).max()
    print(f"{case}: mixed vs fp64 dE = {dE:.2e} Ha/atom, occupied bands {dB:.2e} Ry, converged "
          f"{bool(o64[8])}/{bool(o32[8])} in {s64.iterations}/{s32.iterations} iterations")
    assert bool(o64[8]) and bool(o32[8])
    assert dE < 1e-6
    assert dB < 2e-5
    # the density matrix is Hermitian to rounding
    D = _np(o32[1])
    assert np.abs(D - np.conj(D.T)).max() < 1e-10
