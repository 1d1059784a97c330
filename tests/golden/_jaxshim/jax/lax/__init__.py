"""``jax.lax`` stand-in: control flow as Python loops; erf/erf_inv from SciPy."""
import numpy as _np
import scipy.special as _sps

from .._core import d_erf as erf, wrap as _wrap


def erf_inv(x):
    return _wrap(_sps.erfinv(x))


def while_loop(cond_fun, body_fun, init_val):
    val = init_val
    while bool(cond_fun(val)):
        val = body_fun(val)
    return val


def fori_loop(lower, upper, body_fun, init_val):
    val = init_val
    for i in range(int(lower), int(upper)):
        val = body_fun(i, val)
    return val


def scan(f, init, xs, length=None):
    carry = init
    ys = []
    n = length if xs is None else _np.shape(xs)[0]
    for i in range(n):
        carry, y = f(carry, None if xs is None else xs[i])
        ys.append(y)
    if ys and isinstance(ys[0], tuple):
        return carry, tuple(_wrap(_np.stack([y[k] for y in ys])) for k in range(len(ys[0])))
    return carry, _wrap(_np.stack(ys))


def map(f, xs):  # noqa: A001  (the jax.lax name)
    return _wrap(_np.stack([f(x) for x in xs]))
