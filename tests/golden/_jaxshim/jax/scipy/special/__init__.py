"""``jax.scipy.special`` stand-in."""
import scipy.special as _sps

from ..._core import wrap as _wrap, d_erf as erf  # noqa: F401


def erfc(x):
    return _wrap(_sps.erfc(x))
