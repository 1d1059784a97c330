"""Proton-proton Ewald energy ``potential_energy_pp`` (hqc/pbc/potential.py:103-130).

Computed by the engine (``hqcgb_ewald``): nearest-image real-space term,
reciprocal sphere 0 < |G| <= Gmax, Madelung self term, result in Rydberg.
``potential_energy_pp_and_grad`` also returns dVpp/dxp (Rydberg per rs unit),
which the reference does not provide.
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
