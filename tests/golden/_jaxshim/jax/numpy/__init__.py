"""``jax.numpy`` stand-in: NumPy with dual-number-aware elementary functions."""
import types as _types

import numpy as _np

from .._core import (wrap as _wrap, d_exp, d_log, d_sqrt, d_arctan, d_square,
                     d_power, d_abs, d_clip, d_sum, einsum_dual, transpose as _tr)

pi = _np.pi
e = _np.e
inf = _np.inf
nan = _np.nan
float64 = _np.float64
float32 = _np.float32
complex128 = _np.complex128
complex64 = _np.complex64
int32 = _np.int32
int64 = _np.int64
ndarray = _np.ndarray

exp = d_exp
log = d_log
sqrt = d_sqrt
arctan = d_arctan
square = d_square
power = d_power
abs = d_abs
clip = d_clip
sum = d_sum
einsum = einsum_dual


def transpose(x, axes=None):
    return _tr(x, axes)


def empty_like(x, dtype=None):
    # jax.numpy.empty_like returns zeros
    return _wrap(_np.zeros_like(_np.asarray(x), dtype=dtype))


def _wrapped(fn):
    def w(*a, **k):
        return _wrap(fn(*a, **k))
    w.__name__ = getattr(fn, "__name__", "fn")
    return w


linalg = _types.SimpleNamespace(**{k: _wrapped(getattr(_np.linalg, k)) for k in
                                   ("eigh", "solve", "norm", "det", "inv", "eigvalsh")})
fft = _types.SimpleNamespace(**{k: _wrapped(getattr(_np.fft, k)) for k in
                                ("fft", "ifft", "fftn", "ifftn", "rfft", "irfft", "fftfreq")})


def __getattr__(name):
    obj = getattr(_np, name)
    if callable(obj) and not isinstance(obj, type):
        return _wrapped(obj)
    return obj
