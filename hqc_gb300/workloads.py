"""Synthetic proton configurations of the benchmark workloads.

Seeded with ``numpy.random.default_rng(seed)``; positions in rs units like
the reference's inputs (``hqc/pbc/solver.py:710-723``).  The reference's own
tests draw positions with jax.random (test/test_pbc_solver.py:72-80), whose
stream is not reproducible without jaxlib.
"""
import numpy as np


def box(n):
    """Box side in rs units: L = (4 pi n / 3)^(1/3)."""
    return (4.0 / 3.0 * np.pi * n) ** (1.0 / 3.0)


def uniform(n, seed):
    return np.random.default_rng(seed).uniform(0.0, box(n), (n, 3))


def bcc(ncell, rs, noise_bohr=0.0, seed=0):
    """bcc lattice of ncell^3 conventional cells (2 atoms each) with Gaussian
    displacements of standard deviation ``noise_bohr`` (Bohr)."""
    n = 2 * ncell ** 3
    a = box(n) / ncell
    pts = []
    for i in range(ncell):
        for j in range(ncell):
            for k in range(ncell):
                pts.append([i, j, k])
                pts.append([i + 0.5, j + 0.5, k + 0.5])
    xp = np.array(pts, dtype=float) * a
    if noise_bohr:
        xp = xp + np.random.default_rng(seed).normal(0.0, noise_bohr, xp.shape) / rs
    return xp


# (name) -> dict of the make_pes / make_solver arguments and positions
def h54_bcc_pbe(noise_seed=7):
    """H54 bcc 3x3x3, rs 1.31, 0.1 Bohr noise (seed 7), gth-dzvp, PBE, 81^3 grid
    (the reference's odd grid for a requested 80^3)."""
    n, rs = 54, 1.31
    L = box(n)
    return dict(n=n, L=L, rs=rs, basis="gth-dzvp", dft=True, xc="pbe",
                grid_length=L * rs / 80.0, xp=bcc(3, rs, 0.1, noise_seed))


def h8_szv_hf(seed=42):
    n, rs = 8, 1.25
    L = box(n)
    return dict(n=n, L=L, rs=rs, basis="gth-szv", dft=False, grid_length=L * rs / 40.0,
                xp=uniform(n, seed))


def h32_dzv_lda(seed=1):
    n, rs = 32, 1.4
    L = box(n)
    sigma = 0.5 * 10000 / 157888.09
    return dict(n=n, L=L, rs=rs, basis="gth-dzv", dft=True, xc="lda,vwn",
                grid_length=L * rs / 64.0, smearing=True, smearing_method="gauss",
                smearing_sigma=sigma, xp=uniform(n, seed))


def hf_fermi(n=16, rs=1.4, seed=3, count=3, grid=None):
    """Configuration family 4 at one density: H16 (or H32) dzv Hartree-Fock
    with Fermi smearing at 5000 K (sigma = 0.5 * 5000 / 157888.09 Ha), 49^3
    grid for H16 (65^3 for H32) unless `grid` points per side are given;
    `count` configurations of the family, seeded uniformly in the box."""
    L = box(n)
    sigma = 0.5 * 5000 / 157888.09
    if grid is None:
        grid = 48.0 if n == 16 else 64.0
    rng = np.random.default_rng(seed)
    return dict(n=n, L=L, rs=rs, basis="gth-dzv", dft=False, grid_length=L * rs / grid,
                smearing=True, smearing_method="fermi", smearing_sigma=sigma,
                xps=rng.uniform(0.0, L, (count, n, 3)))


def hf_uneven_batch(count=256, seed=3):
    """Configuration family 4 as one uneven batch: `count` configurations,
    the first half H16 on a 49^3 grid and the second half H32 on 65^3 (the
    reference's odd grids for the requested 48^3 / 64^3), each with its own
    rs ~ U[1.2, 1.6] and uniform positions in its box; gth-dzv Hartree-Fock
    with Fermi smearing at 5000 K (``HF_FERMI_5000K``).  Returns a list of
    (xp (n, 3) rs units, L rs units, rs, n_grid) for ``make_pes_batch``."""
    rng = np.random.default_rng(seed)
    cfgs = []
    for k in range(count):
        n, grid = (16, 49) if k < count // 2 else (32, 65)
        rs = rng.uniform(1.2, 1.6)
        L = box(n)
        cfgs.append((rng.uniform(0.0, L, (n, 3)), L, rs, grid))
    return cfgs


HF_FERMI_5000K = dict(dft=False, smearing=True, smearing_method="fermi",
                      smearing_sigma=0.5 * 5000 / 157888.09)
