"""Nuclear gradients pinned to the reference, and the free-energy pair of
``pes.value_and_grad``.

The reference has no forces (doc/solver_algorithm.md:1210) and its SCF
while_loop cannot be reverse-differentiated, so ``tests/golden/make_golden.py``
central-differences (h = 1e-4 rs units) the reference's own make_pes energy
(pes_gamma, hqc/pbc/pes.py:78-86, run unmodified over the NumPy stand-in for
JAX) on Hartree-Fock szv/dzv, a Fermi-smeared HF case (Newton mu search;
its golden also differences E - sigma Se) and an LDA dzvp case.  The
engine's analytic gradient (the adjoint plus the Ewald gradient) must match
those differences:

* FP64: within 5e-7 Ry per rs unit (1.7e-7 Ha/Bohr at rs 1.5; the finite
  differences themselves carry ~1e-7);
* mixed: within 3e-5 Ry per rs unit (1e-5 Ha/Bohr, the target accuracy).

``value_and_grad`` must return a value whose derivative is the gradient it
returns: checked by central differences of that value under Fermi and
Gaussian smearing.
"""
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = ["fd_hf_szv", "fd_hf_dzv", "fd_hf_dzv_fermi", "fd_lda_dzvp"]


def _case(name):
    g = np.load(os.path.join(HERE, name + ".npz"))
    meta = json.load(open(os.path.join(HERE, "manifest.json")))[name]
    return g, meta


@pytest.mark.parametrize("precision,tol", [("fp64", 5e-7), ("mixed", 3e-5)])
@pytest.mark.parametrize("name", CASES)
def test_gradient_matches_reference_fd(name, precision, tol):
    from hqc_gb300 import make_pes
    g, meta = _case(name)
    kw = dict(meta["kwargs"])
    n, rs, L = int(g["n"]), float(g["rs"]), float(g["L"])
    pes = make_pes(n, L, rs, meta["basis"], forces=True, precision=precision, **kw)
    F, grad = pes.value_and_grad(g["xp"])
    grad = grad.detach().cpu().numpy()
    c = g["coords"]
    an = grad[c[:, 0], c[:, 1]]
    err = np.abs(an - g["dFtot"]).max()
    # the value is the free energy E - sigma Se of the reference's own outputs
    Fref = float(g["Etot"]) - 2.0 * float(g["sigma"]) * float(g["Se"])
    print(f"{name} {precision}: max |grad - FD| = {err:.2e} Ry/rs, |F - Fref| = {abs(float(F) - Fref):.2e}")
    assert err < tol
    assert abs(float(F) - Fref) < (1e-8 if precision == "fp64" else 2e-6 * n)


@pytest.mark.parametrize("method,dft", [("fermi", False), ("gauss", False), ("fermi", True)])
def test_value_and_grad_is_a_derivative_pair(method, dft):
    """Central differences (h = 1e-4 rs) of value_and_grad's value reproduce
    its gradient on 4 coordinates, under smearing, where pes(xp) (the
    reference's internal energy E) and the gradient differ."""
    from hqc_gb300 import make_pes
    n, rs = 4, 1.5
    L = (4 / 3 * np.pi * n) ** (1 / 3)
    xp = np.random.default_rng(21).uniform(0, L, (n, 3))
    # Gaussian occupations are capped at 1 (smearing.py:52): a wider sigma
    # gives the same partial filling as Fermi's
    sigma = 0.08 if method == "fermi" else 0.25
    kw = dict(grid_length=0.2, tol=1e-11, max_cycle=300, smearing=True, smearing_method=method,
              smearing_sigma=sigma, search_method="newton", search_tol=1e-13, search_cycle=200)
    if dft:
        kw.update(dft=True, xc="lda,vwn")
    pes = make_pes(n, L, rs, "gth-dzv", forces=True, **kw)
    F0, grad = pes.value_and_grad(xp)
    grad = grad.detach().cpu().numpy()
    h = 1e-4
    for a, d in [(0, 0), (1, 2), (2, 1), (3, 0)]:
        vals = []
        for sgn in (1, -1):
            x = xp.copy()
            x[a, d] += sgn * h
            vals.append(float(pes.value_and_grad(x)[0]))
            assert pes.solver.iterations < kw["max_cycle"], "SCF did not converge"
        fd = (vals[0] - vals[1]) / (2 * h)
        print(f"{method} dft={dft} ({a},{d}): FD {fd:.9f} grad {grad[a, d]:.9f} diff {fd - grad[a, d]:.2e}")
        assert abs(fd - grad[a, d]) < 5e-7, (a, d, fd, grad[a, d])
    # E (pes) and F differ by sigma * S under smearing
    assert abs(float(pes(xp)) - float(F0)) > 1e-6
