"""Oracle: proton-proton Ewald energy ``potential_energy_pp`` and its gradient.

Restates ``hqc/pbc/potential.py:6-67,103-130``: nearest-image real-space term
erfc(kappa d)/d, reciprocal sum over integer G with 0 < |G|^2 <= Gmax^2,
g_0 = -pi/kappa^2 and the Madelung self term, in L = 1 units; result in Ry.
The gradient (absent from the reference) differentiates the same expression.
Test infrastructure only.
"""
import numpy as np
from scipy.special import erfc


def kvectors(gmax):
    n = np.arange(-gmax, gmax + 1)
    G = np.array(np.meshgrid(n, n, n)).reshape(3, -1).T
    G2 = (G ** 2).sum(1)
    return G[(G2 <= gmax ** 2) & (G2 > 0)].astype(float)


def madelung(kappa, G):
    Gn2 = (G ** 2).sum(1)
    gk = np.exp(-np.pi ** 2 * Gn2 / kappa ** 2) / (np.pi * Gn2)
    return gk.sum() - np.pi / kappa ** 2 - 2 * kappa / np.sqrt(np.pi)


def vpp(xp, L, rs, kappa=10.0, Gmax=15, grad=False):
    """Ewald energy (Ry) of protons at ``xp`` (rs units) in a box of side L (rs units).

    With grad=True also returns dVpp/dxp in Ry per rs unit.
    """
    xp = np.asarray(xp, dtype=float)
    n = xp.shape[0]
    xw = xp - L * np.floor(xp / L)
    i, j = np.triu_indices(n, k=1)
    r = (xw[i] - xw[j]) / L
    r -= np.rint(r)
    G = kvectors(Gmax)
    Gn2 = (G ** 2).sum(1)
    gk = np.exp(-np.pi ** 2 * Gn2 / kappa ** 2) / (np.pi * Gn2)
    d = np.linalg.norm(r, axis=1)
    phase = 2 * np.pi * r @ G.T  # (pairs, nG)
    v = erfc(kappa * d) / d + np.cos(phase) @ gk - np.pi / kappa ** 2
    E = 2 * v.sum() / L / rs + n * madelung(kappa, G) / L / rs
    if not grad:
        return E
    dsr = (-2 * kappa / np.sqrt(np.pi) * np.exp(-(kappa * d) ** 2) / d - erfc(kappa * d) / d ** 2)
    dv = dsr[:, None] * r / d[:, None] - (np.sin(phase) * gk[None]) @ (2 * np.pi * G)
    # d r / d xp_i = +1/L, d r / d xp_j = -1/L
    g = np.zeros_like(xp)
    np.add.at(g, i, dv)
    np.add.at(g, j, -dv)
    return E, 2 * g / L / L / rs
