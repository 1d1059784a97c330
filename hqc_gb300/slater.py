"""``make_slater``: Slater matrices of periodic GTO orbitals at electron
positions (hqc/pbc/slater.py:7-104), at the Gamma point or, with
``gamma=False``, at one k-point (Bloch AOs, complex; slater_kpt).

``slater(xp, xe, mo_coeff)`` (groundstate=True) or
``slater(xp, xe, mo_coeff, state_idx)`` returns (slater_up, slater_dn), the
(n/2, n/2) matrices AO(xe_up) mo_coeff[:, idx_up] and the same for spin down.
xp and xe are in rs units; xe may carry a leading walker axis (W, n, 3),
with xp either shared (n, 3) or per walker (W, n, 3) -- the walker batches
the reference builds with jax.vmap.  AO values come from the engine
(hqcgb_ao_points: the reference's eval_pbc_ao, gto.py:326-369), the products
from batched DGEMMs (hqcgb_slater).  With gamma=False the calls are
``slater(xp, xe, mo_coeff, kpt)`` / ``slater(xp, xe, mo_coeff, kpt,
state_idx)`` (kpt (3,) in 1/Bohr, mo_coeff complex) and the matrices are
complex128 (hqcgb_ao_points_kpt / hqcgb_slater_kpt, batched ZGEMMs).
"""
import ctypes

import numpy as np
import torch

from . import _lib
from .basis import basis_tables
from .solver import lattice_1d


def make_slater(n, L, rs, basis, rcut=24, groundstate=True, gamma=True):
    assert n % 2 == 0
    alpha, coef, ls, carts = basis_tables(basis)
    lat = lattice_1d(L * rs, rcut)
    nb = coef.shape[0]
    keep = (alpha, coef, ls, carts, lat)

    def _dev(x):
        dev = torch.device("cuda", torch.cuda.current_device())
        if isinstance(x, torch.Tensor):
            return x.detach().to(device=dev, dtype=torch.float64).contiguous()
        return torch.as_tensor(np.asarray(x, dtype=np.float64), device=dev).contiguous()

    def _kpt(kpt):
        k = np.ascontiguousarray(np.asarray(kpt.detach().cpu() if isinstance(kpt, torch.Tensor) else kpt,
                                            dtype=np.float64))
        assert k.shape == (3,)
        return k

    def _tables():
        return (keep[0].ctypes.data_as(_lib.c_double_p), keep[1].ctypes.data_as(_lib.c_double_p),
                keep[2].ctypes.data_as(_lib.c_int_p), keep[3].ctypes.data_as(_lib.c_int_p), lat.size,
                keep[4].ctypes.data_as(_lib.c_double_p))

    def ao_values(xp, xe, kpt=None):
        """AO values (..., n_e, n_ao) at xe for protons xp (rs units); with a
        k-point (1/Bohr) the complex Bloch AOs."""
        lib = _lib.load()
        xp_t, xe_t = _dev(xp) * rs, _dev(xe) * rs
        lead = xe_t.shape[:-2]
        ne = xe_t.shape[-2]
        W = int(np.prod(lead)) if lead else 1
        groups = 1 if xp_t.dim() == 2 else W
        dt = torch.float64 if kpt is None else torch.complex128
        out = torch.empty(W * ne, n * nb, dtype=dt, device=xe_t.device)
        st = ctypes.c_void_p(torch.cuda.current_stream(xe_t.device).cuda_stream)
        tail = (ctypes.c_void_p(xp_t.data_ptr()), W * ne, ne if groups > 1 else W * ne,
                ctypes.c_void_p(xe_t.data_ptr()), ctypes.c_void_p(out.data_ptr()), st)
        if kpt is None:
            _lib.check(lib.hqcgb_ao_points(n, nb, alpha.size, *_tables(), *tail))
        else:
            k = _kpt(kpt)
            _lib.check(lib.hqcgb_ao_points_kpt(n, nb, alpha.size, *_tables(),
                                               k.ctypes.data_as(_lib.c_double_p), *tail))
        return out.reshape(*lead, ne, n * nb)

    def slater(xp, xe, mo_coeff, state_idx=None, kpt=None):
        lib = _lib.load()
        if state_idx is None:
            state_idx = np.concatenate([np.arange(n // 2), np.arange(n // 2)])
        idx = np.ascontiguousarray(np.asarray(state_idx, dtype=np.int32))
        assert idx.shape == (n,)
        xp_t, xe_t = _dev(xp) * rs, _dev(xe) * rs
        single = xe_t.dim() == 2
        xe3 = (xe_t.unsqueeze(0) if single else xe_t).contiguous()
        W = xe3.shape[0]
        groups = 1 if xp_t.dim() == 2 else W
        if kpt is None:
            mo = _dev(mo_coeff)
            dt = torch.float64
        else:
            dev = xe3.device
            mo = (mo_coeff.detach().to(device=dev, dtype=torch.complex128) if isinstance(mo_coeff, torch.Tensor)
                  else torch.as_tensor(np.asarray(mo_coeff, dtype=np.complex128), device=dev)).contiguous()
            dt = torch.complex128
        up = torch.empty(W, n // 2, n // 2, dtype=dt, device=xe3.device)
        dn = torch.empty_like(up)
        st = ctypes.c_void_p(torch.cuda.current_stream(xe3.device).cuda_stream)
        tail = (W, groups, ctypes.c_void_p(xp_t.data_ptr()), ctypes.c_void_p(xe3.data_ptr()),
                ctypes.c_void_p(mo.data_ptr()), mo.shape[1], idx.ctypes.data_as(_lib.c_int_p),
                ctypes.c_void_p(up.data_ptr()), ctypes.c_void_p(dn.data_ptr()), st)
        if kpt is None:
            _lib.check(lib.hqcgb_slater(n, nb, alpha.size, *_tables(), *tail))
        else:
            k = _kpt(kpt)
            _lib.check(lib.hqcgb_slater_kpt(n, nb, alpha.size, *_tables(),
                                            k.ctypes.data_as(_lib.c_double_p), *tail))
        return (up[0], dn[0]) if single else (up, dn)

    if gamma:
        if groundstate:
            fn = lambda xp, xe, mo_coeff: slater(xp, xe, mo_coeff)  # noqa: E731
        else:
            fn = slater
    else:
        if groundstate:
            fn = lambda xp, xe, mo_coeff, kpt: slater(xp, xe, mo_coeff, kpt=kpt)  # noqa: E731
        else:
            fn = lambda xp, xe, mo_coeff, kpt, state_idx: slater(  # noqa: E731
                xp, xe, mo_coeff, state_idx, kpt=kpt)
    fn.ao_values = ao_values
    return fn
