"""The allocation-free eigensolver entry point (hqcgb_eigh_noalloc).

Some callers cannot allocate device memory (a framework that owns every
device buffer, such as an XLA custom call inside a jitted program, or a loop
that must not wait on an allocation); hqcgb_eigh_noalloc serves them with a
static device scratch array.  These tests call it through the C ABI twice in
a row and compare with the allocating entry point hqcgb_eigh, within the
eigensolver tolerances used elsewhere in the suite.  This file is collected
last so that a failure here does not hide the other tests' results.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _sym(n, seed):
    M = np.random.default_rng(seed).normal(size=(n, n))
    return M + M.T


def test_noalloc_matches_allocating_entry_point_two_calls():
    import torch
    from hqc_gb300._lib import eigh, eigh_noalloc
    for n, seed in ((270, 11), (64, 12)):  # two calls in a row, different sizes
        A = torch.as_tensor(_sym(n, seed), device="cuda")
        w_ref, V_ref = eigh(A)
        w, V = eigh_noalloc(A)
        w_ref, V_ref, w, V = (t.cpu().numpy() for t in (w_ref, V_ref, w, V))
        M = A.cpu().numpy()
        scale = max(1.0, np.abs(M).max())
        np.testing.assert_allclose(w, w_ref, atol=1e-12 * scale)
        # eigenvectors agree up to sign
        overlap = np.abs(np.sum(V * V_ref, axis=0))
        np.testing.assert_allclose(overlap, np.ones(n), atol=1e-10)
        np.testing.assert_allclose(M @ V, V * w, atol=1e-11 * scale)


def test_noalloc_rejects_sizes_beyond_its_maximum():
    import torch
    from hqc_gb300._lib import HqcgbError, eigh_noalloc, EIGH_NOALLOC_MAX_N
    A = torch.zeros(EIGH_NOALLOC_MAX_N + 1, EIGH_NOALLOC_MAX_N + 1, dtype=torch.float64,
                    device="cuda")
    with pytest.raises(HqcgbError, match="outside"):
        eigh_noalloc(A)
