"""make_slater (hqc/pbc/slater.py): AO values at electron positions against
the reference's golden values (generated from its eval_pbc_ao,
hqc/pbc/gto.py:357-369) and Slater matrices against the same products in
FP64 on the host, for single walkers and walker batches; the Slater matrices
also against the reference's own make_slater output."""
import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("basis", ["gth-szv", "gth-dzv", "gth-dzvp"])
def test_ao_values_match_reference_golden(basis):
    from hqc_gb300 import make_slater
    meta, z = load_golden("gto_values")
    n, rs = meta["n"], meta["rs"]
    L = float(z["L"]) / rs
    sl = make_slater(n, L, rs, basis)
    ao = sl.ao_values(z["xp"] / rs, z["xe"] / rs).cpu().numpy()
    np.testing.assert_allclose(ao, z["ao_" + basis.replace("-", "_")], atol=1e-12)


def test_slater_matrices_and_walker_batches():
    from hqc_gb300 import make_slater
    n, rs, basis = 8, 1.5, "gth-dzv"
    L = (4 / 3 * np.pi * n) ** (1 / 3)
    rng = np.random.default_rng(5)
    xp = rng.uniform(0, L, (n, 3))
    xe = rng.uniform(0, L, (4, n, 3))
    mo = np.linalg.qr(rng.normal(size=(2 * n, 2 * n)))[0]
    sl = make_slater(n, L, rs, basis)
    up, dn = sl(xp, xe, mo)
    for w in range(4):
        ao = sl.ao_values(xp, xe[w]).cpu().numpy()
        np.testing.assert_allclose(up[w].cpu().numpy(), ao[:n // 2] @ mo[:, :n // 2], atol=1e-12)
        np.testing.assert_allclose(dn[w].cpu().numpy(), ao[n // 2:] @ mo[:, :n // 2], atol=1e-12)
        u1, d1 = sl(xp, xe[w], mo)
        np.testing.assert_allclose(u1.cpu().numpy(), up[w].cpu().numpy(), atol=1e-14)
    # excited configuration and per-walker protons
    ex = make_slater(n, L, rs, basis, groundstate=False)
    idx = np.array([0, 1, 2, 5, 0, 1, 3, 4])
    xps = xp[None] + 0.01 * rng.normal(size=(4, n, 3))
    up2, dn2 = ex(xps, xe, mo, idx)
    ao = ex.ao_values(xps[2], xe[2]).cpu().numpy()
    np.testing.assert_allclose(up2[2].cpu().numpy(), ao[:4] @ mo[:, idx[:4]], atol=1e-12)
    np.testing.assert_allclose(dn2[2].cpu().numpy(), ao[4:] @ mo[:, idx[4:]], atol=1e-12)


@pytest.mark.parametrize("basis", ["gth-szv", "gth-dzv", "gth-dzvp"])
def test_ao_values_kpt_match_reference_golden(basis):
    """Bloch AOs against the reference's eval_pbc_ao_kpt (gto.py:371-427)."""
    from hqc_gb300 import make_slater
    meta, z = load_golden("gto_values_kpt")
    n, rs = meta["n"], meta["rs"]
    L = float(z["L"]) / rs
    sl = make_slater(n, L, rs, basis, gamma=False)
    ao = sl.ao_values(z["xp"] / rs, z["xe"] / rs, z["kpt"]).cpu().numpy()
    np.testing.assert_allclose(ao, z["ao_" + basis.replace("-", "_")], atol=1e-12)


def test_slater_kpt_matrices_and_walker_batches():
    """slater_kpt (hqc/pbc/slater.py:72-93): complex AO values times complex
    MOs; the k-point SCF's own mo_coeff as the orbitals."""
    from hqc_gb300 import make_slater, make_solver
    n, rs, basis = 8, 1.5, "gth-dzv"
    L = (4 / 3 * np.pi * n) ** (1 / 3)
    rng = np.random.default_rng(6)
    xp = rng.uniform(0, L, (n, 3))
    xe = rng.uniform(0, L, (3, n, 3))
    kpt = rng.uniform(-np.pi / L / rs, np.pi / L / rs, 3)
    mo = make_solver(n, L, rs, basis, grid_length=0.2, gamma=False)(xp, kpt)[0].cpu().numpy()
    sl = make_slater(n, L, rs, basis, gamma=False)
    up, dn = sl(xp, xe, mo, kpt)
    assert up.dtype.is_complex
    for w in range(3):
        ao = sl.ao_values(xp, xe[w], kpt).cpu().numpy()
        np.testing.assert_allclose(up[w].cpu().numpy(), ao[:n // 2] @ mo[:, :n // 2], atol=1e-12)
        np.testing.assert_allclose(dn[w].cpu().numpy(), ao[n // 2:] @ mo[:, :n // 2], atol=1e-12)
    ex = make_slater(n, L, rs, basis, groundstate=False, gamma=False)
    idx = np.array([0, 1, 2, 5, 0, 1, 3, 4])
    up2, dn2 = ex(xp, xe[1], mo, kpt, idx)
    ao = ex.ao_values(xp, xe[1], kpt).cpu().numpy()
    np.testing.assert_allclose(up2.cpu().numpy(), ao[:4] @ mo[:, idx[:4]], atol=1e-12)
    np.testing.assert_allclose(dn2.cpu().numpy(), ao[4:] @ mo[:, idx[4:]], atol=1e-12)
    # k = 0 reduces to the Gamma AO values
    g = make_slater(n, L, rs, basis).ao_values(xp, xe[0]).cpu().numpy()
    k0 = sl.ao_values(xp, xe[0], np.zeros(3)).cpu().numpy()
    np.testing.assert_allclose(k0.real, g, atol=1e-13)
    assert np.abs(k0.imag).max() == 0.0


def test_slater_matrices_match_reference_golden():
    """The reference's own make_slater output (ground state, an excited
    state_idx, and a k-point with complex coefficients) for one electron
    configuration."""
    from hqc_gb300 import make_slater
    meta, z = load_golden("slater")
    n, rs, basis, L = meta["n"], meta["rs"], meta["basis"], float(z["L"])
    up, dn = make_slater(n, L, rs, basis)(z["xp"], z["xe"], z["mo"])
    np.testing.assert_allclose(up.cpu().numpy(), z["up"], atol=1e-11)
    np.testing.assert_allclose(dn.cpu().numpy(), z["dn"], atol=1e-11)
    up, dn = make_slater(n, L, rs, basis, groundstate=False)(z["xp"], z["xe"], z["mo"], z["idx"])
    np.testing.assert_allclose(up.cpu().numpy(), z["up_x"], atol=1e-11)
    np.testing.assert_allclose(dn.cpu().numpy(), z["dn_x"], atol=1e-11)
    up, dn = make_slater(n, L, rs, basis, gamma=False)(z["xp"], z["xe"], z["moc"], z["kpt"])
    np.testing.assert_allclose(up.cpu().numpy(), z["up_k"], atol=1e-11)
    np.testing.assert_allclose(dn.cpu().numpy(), z["dn_k"], atol=1e-11)
