"""``make_slater``: Slater matrices of periodic GTO orbitals at electron
positions (hqc/pbc/slater.py:7-104), Gamma point.

``slater(xp, xe, mo_coeff)`` (groundstate=True) or
``slater(xp, xe, mo_coeff, state_idx)`` returns (slater_up, slater_dn), the
(n/2, n/2) matrices AO(xe_up) mo_coeff[:, idx_up] and the same for spin down.
xp and xe are in rs units; xe may carry a leading walker axis (W, n, 3),
with xp either shared (n, 3) or per walker (W, n, 3) -- the walker batches
the reference builds with jax.vmap.  AO values come from the engine
(hqcgb_ao_points: the reference's eval_pbc_ao, gto.py:326-369), the products
from batched DGEMMs (hqcgb_slater).
"""
import ctypes

import numpy as np
import torch

from . import _lib
from .basis import basis_tables
from .solver import lattice_1d


def make_slater(n, L, rs, basis, rcut=24, groundstate=True, gamma=True):
    assert n % 2 == 0
    if not gamma:
        raise NotImplementedError("k-point Slater matrices (gamma=False) are not implemented")
    alpha, coef, ls, carts = basis_tables(basis)
    lat = lattice_1d(L * rs, rcut)
    nb = coef.shape[0]
    keep = (alpha, coef, ls, carts, lat)

    def _dev(x):
        dev = torch.device("cuda", torch.cuda.current_device())
        if isinstance(x, torch.Tensor):
            return x.detach().to(device=dev, dtype=torch.float64).contiguous()
        return torch.as_tensor(np.asarray(x, dtype=np.float64), device=dev).contiguous()

    def ao_values(xp, xe):
        """AO values (..., n_e, n_ao) at xe for protons xp (rs units)."""
        lib = _lib.load()
        xp_t, xe_t = _dev(xp) * rs, _dev(xe) * rs
        lead = xe_t.shape[:-2]
        ne = xe_t.shape[-2]
        W = int(np.prod(lead)) if lead else 1
        groups = 1 if xp_t.dim() == 2 else W
        out = torch.empty(W * ne, n * nb, dtype=torch.float64, device=xe_t.device)
        st = ctypes.c_void_p(torch.cuda.current_stream(xe_t.device).cuda_stream)
        _lib.check(lib.hqcgb_ao_points(
            n, nb, alpha.size, keep[0].ctypes.data_as(_lib.c_double_p),
            keep[1].ctypes.data_as(_lib.c_double_p), keep[2].ctypes.data_as(_lib.c_int_p),
            keep[3].ctypes.data_as(_lib.c_int_p), lat.size, keep[4].ctypes.data_as(_lib.c_double_p),
            ctypes.c_void_p(xp_t.data_ptr()), W * ne, ne if groups > 1 else W * ne,
            ctypes.c_void_p(xe_t.data_ptr()), ctypes.c_void_p(out.data_ptr()), st))
        return out.reshape(*lead, ne, n * nb)

    def slater(xp, xe, mo_coeff, state_idx=None):
        lib = _lib.load()
        if state_idx is None:
            state_idx = np.concatenate([np.arange(n // 2), np.arange(n // 2)])
        idx = np.ascontiguousarray(np.asarray(state_idx, dtype=np.int32))
        assert idx.shape == (n,)
        xp_t, xe_t = _dev(xp) * rs, _dev(xe) * rs
        single = xe_t.dim() == 2
        xe3 = xe_t.unsqueeze(0) if single else xe_t
        W = xe3.shape[0]
        groups = 1 if xp_t.dim() == 2 else W
        mo = _dev(mo_coeff)
        up = torch.empty(W, n // 2, n // 2, dtype=torch.float64, device=xe3.device)
        dn = torch.empty_like(up)
        st = ctypes.c_void_p(torch.cuda.current_stream(xe3.device).cuda_stream)
        _lib.check(lib.hqcgb_slater(
            n, nb, alpha.size, keep[0].ctypes.data_as(_lib.c_double_p),
            keep[1].ctypes.data_as(_lib.c_double_p), keep[2].ctypes.data_as(_lib.c_int_p),
            keep[3].ctypes.data_as(_lib.c_int_p), lat.size, keep[4].ctypes.data_as(_lib.c_double_p),
            W, groups, ctypes.c_void_p(xp_t.data_ptr()), ctypes.c_void_p(xe3.contiguous().data_ptr()),
            ctypes.c_void_p(mo.data_ptr()), mo.shape[1], idx.ctypes.data_as(_lib.c_int_p),
            ctypes.c_void_p(up.data_ptr()), ctypes.c_void_p(dn.data_ptr()), st))
        return (up[0], dn[0]) if single else (up, dn)

    if groundstate:
        fn = lambda xp, xe, mo_coeff: slater(xp, xe, mo_coeff)  # noqa: E731
    else:
        fn = slater
    fn.ao_values = ao_values
    return fn
