"""Ewald energies of hqc/pbc/potential.py.

* ``potential_energy_pp`` (potential.py:103-130): the proton-proton energy
  (``hqcgb_ewald``): nearest-image real-space term, reciprocal sphere
  0 < |G| <= Gmax, Madelung self term, result in Rydberg.
  ``potential_energy_pp_and_grad`` also returns dVpp/dxp (Rydberg per rs
  unit), which the reference does not provide.
* ``potential_energy(x, kappa, G, L, rs)`` (potential.py:69-101): the
  (vpp, vep, vee) pair sums of proton + electron walker batches x (B, n, dim)
  (``hqcgb_coulomb_energy``), with the host helpers ``kpoints`` and
  ``Madelung`` (potential.py:6-33) that the VMC observables combine with it.
"""
import ctypes

import numpy as np
import torch

from . import _lib


def potential_energy_pp_and_grad(xp, L, rs, kappa=10, Gmax=15):
    lib = _lib.load()
    dev = torch.device("cuda", torch.cuda.current_device())
    x = xp.detach().to(device=dev, dtype=torch.float64) if isinstance(xp, torch.Tensor) else \
        torch.as_tensor(np.asarray(xp, dtype=np.float64), device=dev)
    x = x.contiguous()
    n = x.shape[0]
    e = torch.empty(1, dtype=torch.float64, device=dev)
    g = torch.empty(n, 3, dtype=torch.float64, device=dev)
    st = ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    _lib.check(lib.hqcgb_ewald(ctypes.c_void_p(x.data_ptr()), n, float(L), float(rs), float(kappa),
                               int(Gmax), ctypes.c_void_p(e.data_ptr()),
                               ctypes.c_void_p(g.data_ptr()), st))
    return e[0], g


def potential_energy_pp(xp, L, rs, kappa=10, Gmax=15):
    """Vpp in Rydberg; xp (n, 3) and L in rs units (potential.py:103-130)."""
    return potential_energy_pp_and_grad(xp, L, rs, kappa, Gmax)[0]


def kpoints(dim, Gmax):
    """Integer vectors with 0 < |G|^2 <= Gmax^2 (potential.py:6-16), (nG, dim) int."""
    m = np.arange(-Gmax, Gmax + 1)
    G = np.array([g.flatten() for g in np.meshgrid(*([m] * dim))]).T
    G2 = (G ** 2).sum(axis=-1)
    return G[(G2 <= Gmax ** 2) * (G2 > 0)]


def Madelung(dim, kappa, G):  # noqa: N802 (the reference's name)
    """Madelung constant of the unit simple-cubic (square) lattice for this
    kappa and G set (potential.py:18-33)."""
    Gn = np.linalg.norm(np.asarray(G, dtype=np.float64), axis=-1)
    if dim == 3:
        gk = np.exp(-np.pi ** 2 * Gn ** 2 / kappa ** 2) / (np.pi * Gn ** 2)
        g0 = -np.pi / kappa ** 2
    elif dim == 2:
        from scipy.special import erfc
        gk = erfc(np.pi * Gn / kappa) / Gn
        g0 = -2 * np.sqrt(np.pi) / kappa
    else:
        raise ValueError("dim must be 2 or 3")
    return gk.sum() + g0 - 2 * kappa / np.sqrt(np.pi)


def potential_energy(x, kappa, G, L, rs):
    """(vpp, vep, vee) of proton + electron configurations x (B, n, dim) in rs
    units, the first n/2 particles protons (potential.py:69-101), each (B,)."""
    lib = _lib.load()
    dev = torch.device("cuda", torch.cuda.current_device())
    xt = x.detach().to(device=dev, dtype=torch.float64) if isinstance(x, torch.Tensor) else \
        torch.as_tensor(np.asarray(x, dtype=np.float64), device=dev)
    xt = xt.contiguous()
    B, n, dim = xt.shape
    Gi = np.ascontiguousarray(np.asarray(G), dtype=np.int32).reshape(-1, dim)
    out = torch.empty(B, 3, dtype=torch.float64, device=dev)
    st = ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    _lib.check(lib.hqcgb_coulomb_energy(B, n, dim, ctypes.c_void_p(xt.data_ptr()), float(L), float(rs),
                                        float(kappa), Gi.shape[0], Gi.ctypes.data_as(_lib.c_int_p),
                                        ctypes.c_void_p(out.data_ptr()), st))
    return out[:, 0], out[:, 1], out[:, 2]
