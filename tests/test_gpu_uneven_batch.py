"""Uneven batches through one call (``make_pes_batch`` / ``hqcgb_batch_run``):
configurations of different atom counts, per-configuration rs (box sizes)
and grids -- the batched workload's H16 / H32 mix at reduced size -- must
give what one ``make_pes`` call per configuration gives (the reference's
batching is jax.vmap over one shape, test/test.py:157,179), and the FP64
energies must match the CPU oracle."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SIGMA = 0.5 * 5000 / 157888.09  # Fermi smearing at 5000 K (Hartree)


def _configs(count=6, seed=3):
    from hqc_gb300.workloads import box
    rng = np.random.default_rng(seed)
    cfgs = []
    for k in range(count):
        n, grid = (8, 25) if k % 2 == 0 else (16, 31)
        rs = rng.uniform(1.2, 1.6)
        L = box(n)
        cfgs.append((rng.uniform(0.0, L, (n, 3)), L, rs, grid))
    return cfgs


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_uneven_batch_matches_single_calls(precision):
    from hqc_gb300 import make_pes, make_pes_batch
    kw = dict(dft=False, smearing=True, smearing_method="fermi", smearing_sigma=SIGMA, tol=1e-8,
              max_cycle=100)
    cfgs = _configs()
    pb = make_pes_batch("gth-dzv", precision=precision, forces=True, workers=3, **kw)
    res = pb(cfgs)
    for c, (xp, L, rs, grid) in enumerate(cfgs):
        single = make_pes(xp.shape[0], L, rs, "gth-dzv", precision=precision, forces=True,
                          n_grid=grid, **kw)
        F, g = single.value_and_grad(xp)
        E = single(xp)
        assert single.solver.iterations == res["iterations"][c]
        assert abs(float(res["F"][c]) - float(F)) < 1e-9
        assert abs(float(res["E"][c]) - float(E)) < 1e-9
        np.testing.assert_allclose(res["grad"][c].cpu().numpy(), g.cpu().numpy(), atol=1e-9)
    # a second call, in another order, reuses the size-class workspaces
    res2 = pb(cfgs[::-1])
    np.testing.assert_allclose(res2["F"].cpu().numpy()[::-1], res["F"].cpu().numpy(), atol=1e-9)


def test_uneven_batch_fp64_matches_oracle():
    from hqc_gb300 import make_pes_batch, potential_energy_pp
    from oracle.gpw import Solver
    kw = dict(dft=False, smearing=True, smearing_method="fermi", smearing_sigma=SIGMA, tol=1e-9,
              max_cycle=100)
    cfgs = _configs(count=2, seed=5)
    res = make_pes_batch("gth-dzv", workers=2, **kw)(cfgs)
    for c, (xp, L, rs, grid) in enumerate(cfgs):
        ref = Solver(xp.shape[0], L, rs, "gth-dzv", n_grid=grid, **kw).solve(xp)
        Eel = float(res["E"][c]) - float(potential_energy_pp(xp, L, rs))
        assert abs(Eel - ref[3]) < 1e-8
        np.testing.assert_allclose(res["bands"][c].cpu().numpy(), ref[2], atol=1e-6)
