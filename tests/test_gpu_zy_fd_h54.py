"""The benchmark workload's adjoint forces against central finite
differences of the engine's own FP64 energy.

H54 bcc 3x3x3, rs 1.31, N(0, 0.1 Bohr) noise (seed 7), gth-dzvp, PBE, 81^3:
12 coordinates drawn with numpy.random.default_rng(12), central differences
with h = 1e-4 Bohr of E + Vpp from the FP64 path (SCF tol 1e-10 Ry), against
the FP64 adjoint and the mixed-precision adjoint, both within the target
force accuracy of 1e-5 Ha/Bohr (the FP64 adjoint is expected at ~1e-7).
The mixed path's own energy is not differenced: its SCF stops at its noise
floor (|dE| 2e-6 Ry), which at h = 1e-4 Bohr would dominate a difference
quotient.  Collected late (file name) because it runs 25 H54 SCFs.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_h54_adjoint_matches_fp64_finite_differences():
    from hqc_gb300 import make_pes
    from hqc_gb300.workloads import h54_bcc_pbe
    w = h54_bcc_pbe()
    n, L, rs, xp = w["n"], w["L"], w["rs"], w["xp"]
    kw = dict(dft=True, xc="pbe", grid_length=w["grid_length"], max_cycle=100, forces=True)
    # the 24 displaced energies run as one batch, 8 configurations at a time
    # (bitwise the single-call results: tests/test_gpu_batch.py)
    p64 = make_pes(n, L, rs, w["basis"], precision="fp64", tol=1e-10, concurrency=8, **kw)
    p32 = make_pes(n, L, rs, w["basis"], precision="mixed", tol=1e-7, **kw)
    _, g64 = p64.value_and_grad(xp)
    _, g32 = p32.value_and_grad(xp)
    to_ha_bohr = 1.0 / (2.0 * rs)                    # Ry per rs unit -> Ha/Bohr
    g64 = g64.cpu().numpy() * to_ha_bohr
    g32 = g32.cpu().numpy() * to_ha_bohr
    rng = np.random.default_rng(12)
    pick = rng.choice(3 * n, 12, replace=False)
    h = 1e-4 / rs                                    # 1e-4 Bohr in rs units
    xs = []
    for idx in pick:
        a, d = divmod(int(idx), 3)
        for sgn in (1.0, -1.0):
            x = xp.copy()
            x[a, d] += sgn * h
            xs.append(x)
    e = p64(np.stack(xs)).cpu().numpy()
    err64, err32 = [], []
    for i, idx in enumerate(pick):
        a, d = divmod(int(idx), 3)
        fd = (e[2 * i] - e[2 * i + 1]) / (2 * h) * to_ha_bohr
        err64.append(abs(fd - g64[a, d]))
        err32.append(abs(fd - g32[a, d]))
    print(f"H54 FD (12 coordinates, h = 1e-4 Bohr): max |FP64 adjoint - FD| = {max(err64):.2e}, "
          f"max |mixed adjoint - FD| = {max(err32):.2e} Ha/Bohr")
    assert max(err64) < 1e-6
    assert max(err32) < 1e-5
