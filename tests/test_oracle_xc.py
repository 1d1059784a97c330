"""Exact constraints of the oracle's PBE and PW92 (CPU).

The reference has no GGA, so PBE parity is unpinned; these tests pin the
oracle's functional form to properties that PBE was built to satisfy
(Perdew, Burke, Ernzerhof, PRL 77, 3865 (1996)) and PW92 to its high-density
limit, and compare PW92 with the reference's VWN (pinned by the golden
vectors), a fit to the same Ceperley-Alder data.
"""
import numpy as np

from oracle import xc

RS = np.array([0.5, 1.0, 1.31, 2.0, 3.0, 5.0, 8.0, 10.0])
RHO = 3 / (4 * np.pi * RS ** 3)


def _ex_unif(rho):
    return -3 * (3 * np.pi ** 2 * rho) ** (1 / 3) / (4 * np.pi)


def test_pbe_uniform_limit_is_lda_x_plus_pw92():
    """sigma = 0: F_x = 1 and H = 0, so PBE is Slater exchange + PW92."""
    e = xc.e_pbe(RHO, np.zeros_like(RHO))
    ref = RHO * (xc.eps_x_lda(RHO) + xc.eps_c_pw92(RS))
    np.testing.assert_allclose(e, ref, rtol=1e-14)


def test_pbe_second_order_gradient_terms_cancel():
    """PBE's mu = beta pi^2 / 3 makes the exchange and correlation
    second-order gradient terms cancel (the LDA linear response is kept):
    e(rho, sigma) - e(rho, 0) is O(sigma^2), far below the exchange term
    rho eps_x^unif mu s^2 alone."""
    assert abs(xc._MU - xc._BETA * np.pi ** 2 / 3) < 1e-15
    for rho in RHO:
        kf = (3 * np.pi ** 2 * rho) ** (1 / 3)
        for s2 in (1e-4, 1e-6):
            sigma = s2 * 4 * kf ** 2 * rho ** 2
            d = xc.e_pbe(rho, sigma) - xc.e_pbe(rho, 0.0)
            x_term = rho * _ex_unif(rho) * xc._MU * s2
            assert abs(d) < 0.05 * abs(x_term) * (s2 / 1e-4), (rho, s2, d, x_term)


def test_pbe_large_gradient_limits():
    """s -> infinity: F_x -> 1 + kappa = 1.804 (Lieb-Oxford) and the
    correlation (eps_c + H) -> 0, so e / (rho eps_x^unif) -> 1.804."""
    for rho in (1e-3, 1e-2, 0.1):
        ratio = xc.e_pbe(rho, 1e12) / (rho * _ex_unif(rho))
        assert abs(ratio - (1 + xc._KAPPA)) < 1e-6, (rho, ratio)


def test_pw92_high_density_coefficient_is_exact():
    """PW92's A is the exact high-density (RPA) coefficient (1 - ln 2)/pi^2
    of eps_c ~ A ln rs, the same constant as PBE's gamma."""
    assert abs(xc._PW["A"] - (1 - np.log(2)) / np.pi ** 2) < 1e-6
    assert abs(xc._GAMMA - (1 - np.log(2)) / np.pi ** 2) < 1e-15
    rs = np.array([1e-4, 1e-5])
    slope = (xc.eps_c_pw92(rs[0]) - xc.eps_c_pw92(rs[1])) / np.log(rs[0] / rs[1])
    assert abs(slope - xc._PW["A"]) < 2e-3 * xc._PW["A"]


def test_pw92_agrees_with_reference_vwn():
    """Both parametrise the Ceperley-Alder correlation energy; they differ by
    less than 0.5 mHa over rs 0.5-10 (about 1 % at rs 0.5)."""
    d = xc.eps_c_pw92(RS) - xc.eps_vwn(RHO)
    assert np.abs(d).max() < 5e-4, d


def test_pbe_potentials_are_the_partials():
    """v_rho = de/drho and v_sigma = de/dsigma of evaluate() against central
    finite differences of the energy, at reduced gradients s^2 in [0.1, 10]
    (for s -> 0, e - e(sigma = 0) is O(sigma^2) and a finite difference in
    sigma loses every digit to cancellation)."""
    f = xc.Functional("pbe")
    rng = np.random.default_rng(0)
    rho = 10 ** rng.uniform(-3, 0.5, 64)
    kf = (3 * np.pi ** 2 * rho) ** (1 / 3)
    sigma = 10 ** rng.uniform(-1, 1, 64) * 4 * kf ** 2 * rho ** 2
    e, vr, vs = f.evaluate(rho, sigma)
    h = 1e-6
    fr = (xc.e_pbe(rho * (1 + h), sigma) - xc.e_pbe(rho * (1 - h), sigma)) / (2 * h * rho)
    fs = (xc.e_pbe(rho, sigma * (1 + h)) - xc.e_pbe(rho, sigma * (1 - h))) / (2 * h * sigma)
    np.testing.assert_allclose(vr, fr, rtol=1e-7)
    np.testing.assert_allclose(vs, fs, rtol=1e-6)
