"""Oracle: proton-proton Ewald energy ``potential_energy_pp`` and its gradient,
and the proton + electron ``potential_energy`` of walker batches.

Restates ``hqc/pbc/potential.py:6-130``: nearest-image real-space term
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


def kpoints(dim, gmax):
    """Integer vectors 0 < |G|^2 <= gmax^2 (``kpoints``, potential.py:6-16)."""
    n = np.arange(-gmax, gmax + 1)
    G = np.array([g.ravel() for g in np.meshgrid(*([n] * dim))]).T
    G2 = (G ** 2).sum(1)
    return G[(G2 <= gmax ** 2) & (G2 > 0)]


def _g_terms(dim, kappa, G):
    Gn = np.linalg.norm(np.asarray(G, dtype=float), axis=1)
    if dim == 3:
        return np.exp(-np.pi ** 2 * Gn ** 2 / kappa ** 2) / (np.pi * Gn ** 2), -np.pi / kappa ** 2
    return erfc(np.pi * Gn / kappa) / Gn, -2 * np.sqrt(np.pi) / kappa


def madelung_dim(dim, kappa, G):
    """``Madelung`` (potential.py:18-33) in 2 or 3 dimensions."""
    gk, g0 = _g_terms(dim, kappa, G)
    return gk.sum() + g0 - 2 * kappa / np.sqrt(np.pi)


def potential_energy(x, kappa, G, L, rs):
    """``potential_energy`` (potential.py:69-101, with psi 35-67) of a batch of
    proton + electron configurations x (B, n, dim) in rs units, first n/2
    protons: returns (vpp, vep, vee), each (B,), pair by pair."""
    x = np.asarray(x, dtype=float)
    B, n, dim = x.shape
    G = np.asarray(G)
    gk, g0 = _g_terms(dim, kappa, G)
    i, j = np.triu_indices(n, k=1)
    Z = np.concatenate([np.ones(n // 2), -np.ones(n // 2)])
    tot = Z[i] + Z[j]
    out = np.zeros((B, 3))
    for b in range(B):
        xw = x[b] - L * np.floor(x[b] / L)
        r = (xw[i] - xw[j]) / L
        r -= np.rint(r)
        d = np.linalg.norm(r, axis=1)
        v = erfc(kappa * d) / d + np.cos(2 * np.pi * r @ G.T) @ gk + g0
        out[b] = (2 * rs / L * v[tot == 2].sum(), -2 * rs / L * v[tot == 0].sum(),
                  2 * rs / L * v[tot == -2].sum())
    return out[:, 0], out[:, 1], out[:, 2]
