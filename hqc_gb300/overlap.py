"""``make_overlap`` (hqc/pbc/overlap.py:11-319): the periodic overlap matrix
as a standalone function, ``overlap(xp)`` at the Gamma point (real) or
``overlap(xp, kpt)`` with ``gamma=False`` (complex Hermitian, kpt in 1/Bohr).

xp is in rs units; a leading batch axis (B, n, 3) -- and for k-points a kpt
batch (B, 3) -- gives (B, n_ao, n_ao), what ``jax.vmap`` returns for the
reference.  The integrals are the engine's analytic lattice sums over the
sphere |t| <= rcut (hqcgb_overlap); ``overlap.with_kinetic`` also returns the
kinetic matrix T of the same sums.  ``use_jit`` and ``remat`` are accepted for
signature compatibility.
"""
import ctypes

import numpy as np
import torch

from . import _lib
from .basis import basis_tables
from .solver import lattice_sphere


def make_overlap(n, L, rs, basis, rcut=24, gamma=True, use_jit=True, remat=False):
    alpha, coef, ls, carts = basis_tables(basis)
    L_bohr = float(L) * float(rs)
    lat = lattice_sphere(L_bohr, rcut)
    nb = coef.shape[0]
    nao = n * nb
    keep = (alpha, coef, ls, carts, lat)

    def _run(xp, kpt, kinetic):
        lib = _lib.load()
        dev = torch.device("cuda", torch.cuda.current_device())
        x = (xp.detach().to(device=dev, dtype=torch.float64) if isinstance(xp, torch.Tensor)
             else torch.as_tensor(np.asarray(xp, dtype=np.float64), device=dev))
        batched = x.dim() == 3
        k = None
        if not gamma:
            k = np.asarray(kpt.detach().cpu() if isinstance(kpt, torch.Tensor) else kpt, dtype=np.float64)
            batched = batched or k.ndim == 2
        B = x.shape[0] if x.dim() == 3 else (k.shape[0] if k is not None and k.ndim == 2 else 1)
        xs = (x.expand(B, n, 3) if x.dim() == 3 else x.reshape(1, n, 3).expand(B, n, 3)).contiguous() * rs
        dt = torch.float64 if gamma else torch.complex128
        S = torch.empty(B, nao, nao, dtype=dt, device=dev)
        T = torch.empty_like(S) if kinetic else None
        kp = None
        if k is not None:
            kk = np.ascontiguousarray(np.broadcast_to(k.reshape(-1, 3), (B, 3)))
            kp = kk.ctypes.data_as(_lib.c_double_p)
        st = ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
        _lib.check(lib.hqcgb_overlap(
            n, nb, alpha.size, keep[0].ctypes.data_as(_lib.c_double_p),
            keep[1].ctypes.data_as(_lib.c_double_p), keep[2].ctypes.data_as(_lib.c_int_p),
            keep[3].ctypes.data_as(_lib.c_int_p), lat.shape[0], keep[4].ctypes.data_as(_lib.c_double_p),
            B, ctypes.c_void_p(xs.data_ptr()), kp, ctypes.c_void_p(S.data_ptr()),
            ctypes.c_void_p(T.data_ptr() if T is not None else 0), st))
        if not batched:
            S = S[0]
            T = T[0] if T is not None else None
        return (S, T) if kinetic else S

    if gamma:
        def overlap(xp):
            return _run(xp, None, False)

        def with_kinetic(xp):
            return _run(xp, None, True)
    else:
        def overlap(xp, kpt):
            return _run(xp, kpt, False)

        def with_kinetic(xp, kpt):
            return _run(xp, kpt, True)
    overlap.with_kinetic = with_kinetic
    return overlap
