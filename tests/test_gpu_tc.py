"""The mixed path's building blocks against FP64 references of the same op:
the tcgen05 3xTF32 grid contractions (density, quadrature) against torch FP64
GEMMs on the GPU, and the mixed-precision eigensolver against LAPACK.

Tolerances: the contractions are FP32-accurate (3xTF32 products, compensated
FP32 sums), so each output element is compared against 1e-6 of the sum of
the absolute values of its terms; the eigensolver is refined to FP64, so
eigenvalues match LAPACK to 1e-12 of the matrix scale and the vectors are
orthonormal to 1e-12.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _operands(nao, N, seed):
    """GTO-like AO values (a few large, most small, all signs) and a
    density-matrix-like symmetric D."""
    import torch
    g = torch.Generator(device="cuda").manual_seed(seed)
    ld = (N + 3) // 4 * 4
    phi = torch.zeros(nao, ld, dtype=torch.float32, device="cuda")
    phi[:, :N] = (torch.randn(nao, N, generator=g, device="cuda") *
                  torch.exp(-3 * torch.rand(nao, N, generator=g, device="cuda")))
    D = torch.randn(nao, nao, generator=g, device="cuda", dtype=torch.float64)
    D = (0.5 * (D + D.T) / nao ** 0.5).float()
    return phi, D, ld


@pytest.mark.parametrize("nao,N", [(1, 1000), (20, 29791), (80, 29791), (130, 4097), (270, 531441)])
def test_tc_density_matches_fp64(nao, N):
    from hqc_gb300._lib import tc_density
    phi, D, ld = _operands(nao, N, nao)
    rho = tc_density(phi, D, N, drain=1)
    rho2 = tc_density(phi, D, N, drain=1)
    p64 = phi[:, :N].double()
    ref = ((D.double() @ p64) * p64).sum(0)
    scale = ((D.double().abs() @ p64.abs()) * p64.abs()).sum(0)
    err = ((rho - ref).abs() / scale.clamp_min(1e-30)).max().item()
    assert err < 1e-6, err
    assert bool((rho == rho2).all()), "repeated call differs"


@pytest.mark.parametrize("nao,N", [(1, 1000), (20, 29791), (80, 29791), (130, 4097), (150, 4097),
                                   (256, 4097), (270, 531441), (600, 3000), (784, 2500), (900, 2500),
                                   (1000, 2500)])
def test_tc_quadrature_matches_fp64(nao, N):
    """LDA form (symmetric tile set).  130, 256, 270 and 784 AOs take the
    persistent form (784: six full blocks and a 16-row block, the largest);
    600, 900 and 1000 AOs need 15, 36 and 36 tiles, several tile-list
    launches."""
    import torch
    from hqc_gb300._lib import tc_quadrature
    phi, _, ld = _operands(nao, N, 100 + nao)
    w = torch.zeros(ld, dtype=torch.float32, device="cuda")
    w[:N] = torch.randn(N, device="cuda", generator=torch.Generator(device="cuda").manual_seed(5))
    M = tc_quadrature(phi, w, drain=1)
    M2 = tc_quadrature(phi, w, drain=1)
    p64, w64 = phi[:, :N].double(), w[:N].double()
    ref = (p64 * w64) @ p64.T
    scale = (p64.abs() * w64.abs()) @ p64.abs().T
    err = ((M - ref).abs() / scale.clamp_min(1e-30)).max().item()
    assert err < 1e-6, err
    assert bool((M == M2).all()), "repeated call differs"


@pytest.mark.parametrize("nao,N,nuse,gga", [(1, 1000, 1, False), (20, 29791, 10, True),
                                             (80, 29791, 40, False), (130, 4097, 64, False),
                                             (130, 4097, 32, True),
                                             (270, 531441, 27, True), (270, 531441, 33, False)])
def test_tc_orbital_density_matches_fp64(nao, N, nuse, gga):
    """rho = sum_k f_k psi_k^2 against the FP64 sum_pq D_pq phi_p phi_q of
    D = C diag(f) C^T, with orthonormal-like C columns and occupations 2
    (up to 64 orbitals without the gradient, 32 with it)."""
    import torch
    from hqc_gb300._lib import tc_orbital_density
    phi, _, ld = _operands(nao, N, 200 + nao)
    dphi = None
    if gga:
        g = torch.Generator(device="cuda").manual_seed(9)
        dphi = torch.zeros(3, nao, ld, dtype=torch.float32, device="cuda")
        dphi[:, :, :N] = torch.randn(3, nao, N, generator=g, device="cuda")
    C = torch.linalg.qr(torch.randn(nao, nao, dtype=torch.float64, device="cuda",
                                    generator=torch.Generator(device="cuda").manual_seed(3)))[0]
    occ = torch.zeros(nao, dtype=torch.float64, device="cuda")
    occ[:nuse] = 2.0
    out = tc_orbital_density(phi, C, occ, N, nuse, dphi.reshape(3 * nao, ld) if gga else None)
    rho = out[0] if gga else out
    p64 = phi[:, :N].double()
    Y = C[:, :nuse] * occ[:nuse].sqrt()
    psi = Y.T @ p64
    ref = (psi ** 2).sum(0)
    scale = ((Y.abs().T @ p64.abs()) ** 2).sum(0)
    err = ((rho - ref).abs() / scale.clamp_min(1e-30)).max().item()
    assert err < 2e-6, err
    if gga:
        for c in range(3):
            dpsi = Y.T @ dphi[c, :, :N].double()
            gref = 2 * (psi * dpsi).sum(0)
            gscale = 2 * ((Y.abs().T @ p64.abs()) * (Y.abs().T @ dphi[c, :, :N].double().abs())).sum(0)
            gerr = ((out[1][c] - gref).abs() / gscale.clamp_min(1e-30)).max().item()
            assert gerr < 2e-6, (c, gerr)


@pytest.mark.parametrize("n", [1, 2, 5, 20, 32, 33, 80, 160, 270])
def test_eigh_mixed_matches_lapack(n):
    import torch
    from hqc_gb300._lib import eigh_mixed
    rng = np.random.default_rng(n)
    M = rng.normal(size=(n, n))
    M = M + M.T
    w, V = eigh_mixed(torch.as_tensor(M, device="cuda"))
    w, V = w.cpu().numpy(), V.cpu().numpy()
    s = max(1.0, np.abs(M).max())
    np.testing.assert_allclose(w, np.linalg.eigvalsh(M), atol=1e-12 * s)
    np.testing.assert_allclose(V.T @ V, np.eye(n), atol=1e-12)
    np.testing.assert_allclose(M @ V, V * w, atol=1e-11 * s)


@pytest.mark.parametrize("n", [20, 80, 270])
def test_eigh_mixed_clustered_spectrum(n):
    """Near-degenerate clusters like a symmetric lattice's bands."""
    import torch
    from hqc_gb300._lib import eigh_mixed
    rng = np.random.default_rng(7 * n)
    Q = np.linalg.qr(rng.normal(size=(n, n)))[0]
    lam = np.repeat(np.linspace(-2, 3, n // 6 + 1), 6)[:n] + 1e-7 * rng.normal(size=n)
    M = (Q * lam) @ Q.T
    M = 0.5 * (M + M.T)
    w, V = eigh_mixed(torch.as_tensor(M, device="cuda"))
    w, V = w.cpu().numpy(), V.cpu().numpy()
    np.testing.assert_allclose(w, np.linalg.eigvalsh(M), atol=1e-12 * 3)
    np.testing.assert_allclose(V.T @ V, np.eye(n), atol=1e-12)
    np.testing.assert_allclose(M @ V, V * w, atol=1e-11 * 3)


@pytest.mark.parametrize("nao,N", [(20, 4000), (129, 5000), (140, 7000), (150, 9000), (256, 6000),
                                   (270, 20000), (400, 3000), (600, 3000)])
def test_tc_quadrature_gga_matches_fp64(nao, N):
    """The PBE-form Fock quadrature (pre-split operands, non-symmetric tile
    set with the partial AO block as an N = 16 MMA, transposed on the A side)
    against FP64: M = Z phi^T + phi Z^T, Z = 0.5 w phi + dV u . grad phi."""
    import torch
    from hqc_gb300._lib import tc_quadrature_gga
    g = torch.Generator(device="cuda").manual_seed(nao)
    ld = (N + 31) // 32 * 32
    phi = torch.zeros(nao, ld, dtype=torch.float32, device="cuda")
    phi[:, :N] = torch.randn(nao, N, generator=g, device="cuda")
    dphi = torch.zeros(3, nao, ld, dtype=torch.float32, device="cuda")
    dphi[:, :, :N] = torch.randn(3, nao, N, generator=g, device="cuda")
    w = torch.zeros(ld, dtype=torch.float32, device="cuda")
    w[:N] = torch.rand(N, generator=g, device="cuda")
    u = torch.zeros(3, ld, dtype=torch.float32, device="cuda")
    u[:, :N] = torch.randn(3, N, generator=g, device="cuda")
    dV = 0.01
    M = tc_quadrature_gga(phi, dphi, w, u, dV, N, drain=1)
    P = phi[:, :N].double()
    Z = 0.5 * w[:N].double() * P + dV * torch.einsum("dg,dpg->pg", u[:, :N].double(), dphi[:, :, :N].double())
    ref = Z @ P.T + P @ Z.T
    err = (M - ref).abs().max().item() / ref.abs().max().item()
    assert err < 2e-6, err
