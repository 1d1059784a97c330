"""Concurrent batches (hqcgb_pes_batch with several worker plans) against
one-at-a-time calls on the same plan parameters: every configuration's
energy, bands and forces must be bit-identical, whichever worker ran it."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_batch_matches_single_calls(precision):
    import torch
    from hqc_gb300 import make_pes
    n, rs = 8, 1.5
    L = (4 / 3 * np.pi * n) ** (1 / 3)
    rng = np.random.default_rng(4)
    xps = rng.uniform(0, L, (5, n, 3))
    kw = dict(grid_length=L * rs / 30, dft=True, xc="pbe", tol=1e-8, max_cycle=100,
              precision=precision, forces=True)
    single = make_pes(n, L, rs, "gth-dzv", **kw)
    batched = make_pes(n, L, rs, "gth-dzv", concurrency=3, **kw)
    Eb, gb = batched.value_and_grad(xps)
    for b in range(xps.shape[0]):
        E, g = single.value_and_grad(xps[b])
        assert float(E) == float(Eb[b])
        assert torch.equal(g, gb[b])
    out = batched.solver(xps)
    for b in range(xps.shape[0]):
        ref = single.solver(xps[b])
        assert torch.equal(ref[2], out[2][b])
        assert float(ref[3]) == float(out[3][b])
        assert bool(ref[8]) == bool(out[8][b])


def test_batch_reports_failing_configuration():
    """Coincident atoms in one configuration: the batch raises and names it;
    the engine stays usable afterwards."""
    from hqc_gb300 import make_solver
    from hqc_gb300._lib import HqcgbError
    n, rs = 4, 1.5
    L = (4 / 3 * np.pi * n) ** (1 / 3)
    xps = np.random.default_rng(42).uniform(0, L, (3, n, 3))
    xps[1, 1] = xps[1, 0]
    s = make_solver(n, L, rs, "gth-dzv", grid_length=0.3, concurrency=2)
    with pytest.raises(HqcgbError, match="configuration 1"):
        s(xps)
    out = s(xps[[0, 2]])
    assert bool(out[8].all())
