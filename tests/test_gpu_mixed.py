"""Mixed-precision path (tcgen05 3xTF32 grid GEMMs, FP32 FFT, FP64 small
linear algebra) against the FP64 path on the same inputs.

Tolerances are the target accuracy: total energy within 1e-6 Ha per atom
(2e-6 Ry/atom), occupied band energies within 1e-6 Ha (2e-6 Ry), the
one-off Vep matrix within 1e-6 of its largest element.  Virtual bands are
not compared: FP32-level noise in the grid quadratures is amplified by
1/s_min(S) in the near-linearly-dependent directions of the AO basis
(s_min ~ 1e-5..1e-7 for dzvp at these densities), which only the empty
high-lying states feel.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _np(t):
    return t.detach().cpu().numpy()


@pytest.mark.parametrize("n,basis,xc,seed,rs", [(4, "gth-dzvp", "lda,vwn", 3, 1.31),
                                                (16, "gth-dzvp", "pbe", 11, 1.31),
                                                (16, "gth-dzv", "lda,vwn", 5, 1.5),
                                                (8, "gth-dzvp", "pbe", 1, 1.5)])
def test_mixed_matches_fp64(n, basis, xc, seed, rs):
    from hqc_gb300 import make_solver
    L = (4 / 3 * np.pi * n) ** (1 / 3)
    xp = np.random.default_rng(seed).uniform(0, L, (n, 3))
    kw = dict(grid_length=L * rs / 30, dft=True, xc=xc, tol=1e-7, max_cycle=100)
    s64 = make_solver(n, L, rs, basis, precision="fp64", **kw)
    s32 = make_solver(n, L, rs, basis, precision="mixed", **kw)
    o64 = s64(xp)
    o32 = s32(xp)
    V64 = _np(s64.plan.query("V"))
    V32 = _np(s32.plan.query("V"))
    assert np.abs(V32 - V64).max() < 1e-6 * np.abs(V64).max()
    assert abs(float(o32[3]) - float(o64[3])) / n < 2e-6
    nocc = n // 2
    np.testing.assert_allclose(_np(o32[2])[:nocc], _np(o64[2])[:nocc], atol=2e-6)
    assert bool(o32[8])


def test_mixed_h54_bcc_pbe_energy_and_bands():
    """The benchmark workload itself: |dE| <= 1e-6 Ha/atom, bands <= 1e-6 Ha."""
    from hqc_gb300 import make_solver
    from hqc_gb300.workloads import h54_bcc_pbe
    w = h54_bcc_pbe()
    kw = dict(grid_length=w["grid_length"], dft=True, xc="pbe", tol=1e-7, max_cycle=100)
    o64 = make_solver(w["n"], w["L"], w["rs"], w["basis"], precision="fp64", **kw)(w["xp"])
    o32 = make_solver(w["n"], w["L"], w["rs"], w["basis"], precision="mixed", **kw)(w["xp"])
    dE = abs(float(o32[3]) - float(o64[3])) / 2 / w["n"]
    print(f"H54 mixed vs fp64: dE = {dE:.2e} Ha/atom")
    assert dE < 1e-6
    np.testing.assert_allclose(_np(o32[2])[:27], _np(o64[2])[:27], atol=2e-6)
    assert bool(o32[8])
