"""NumPy stand-in for the small subset of the JAX API that ``hqc.pbc`` uses.

Test infrastructure only: it lets ``tests/golden/make_golden.py`` execute the
reference's own, unmodified Python source in a container that has no jaxlib,
so that golden vectors come from the reference code path itself.

What is restated here (JAX itself, jax>=0.4, unpinned by the reference's
``setup.py:10-15``, is absent):

* ``jit`` is the identity; ``vmap`` is a Python loop over the mapped axis
  followed by a stack along ``out_axes``;
* ``lax.scan`` / ``lax.while_loop`` / ``lax.fori_loop`` are Python loops with
  JAX's documented semantics;
* ``grad`` (scalar argument) and ``jacfwd`` are forward-mode automatic
  differentiation with tagged dual numbers (Siskind & Pearlmutter's
  perturbation tags, so nested ``jacfwd(jacfwd(f), argnums=1)`` and
  ``grad(grad(f))`` are exact);
* ``jnp.fft`` / ``jnp.linalg`` map onto NumPy's pocketfft and LAPACK, which
  stand in for XLA's CPU FFT and ``eigh``.  Results therefore agree with a real
  jax_enable_x64 run to rounding, except for the eigenvector sign gauge.

Arrays returned by the ``jax.numpy`` stand-in are a NumPy subclass that adds
JAX's functional ``.at[...].set`` and turns augmented assignment into
rebinding (JAX arrays are immutable; the reference writes ``xp *= rs``).
"""
import itertools

import numpy as np
import scipy.special as _sps

_tag_counter = itertools.count(1)


def new_tag():
    return next(_tag_counter)


class JArray(np.ndarray):
    """ndarray with JAX's immutable update helpers."""

    @property
    def at(self):
        return _AtIndexer(self)

    # JAX arrays are immutable: ``x *= a`` rebinds ``x`` to a new array.
    def __iadd__(self, other):
        return np.add(self, other)

    def __isub__(self, other):
        return np.subtract(self, other)

    def __imul__(self, other):
        return np.multiply(self, other)

    def __itruediv__(self, other):
        return np.true_divide(self, other)


class _AtIndexer:
    def __init__(self, arr):
        self.arr = arr

    def __getitem__(self, idx):
        return _AtSetter(self.arr, idx)


class _AtSetter:
    def __init__(self, arr, idx):
        self.arr, self.idx = arr, idx

    def set(self, v):
        out = np.array(self.arr, copy=True).view(JArray)
        out[self.idx] = v
        return out

    def add(self, v):
        out = np.array(self.arr, copy=True).view(JArray)
        out[self.idx] += v
        return out


def wrap(x):
    if isinstance(x, np.ndarray) and not isinstance(x, JArray):
        return x.view(JArray)
    if isinstance(x, tuple) and not hasattr(x, "_fields"):
        return tuple(wrap(v) for v in x)
    return x


# ----------------------------------------------------------------------------
# Tagged dual numbers (forward-mode AD).
# ----------------------------------------------------------------------------
def tag_of(x):
    return x.tag if isinstance(x, Dual) else -1


def primal(x):
    while isinstance(x, Dual):
        x = x.val
    return x


def shape_of(x):
    return np.shape(primal(x))


class Dual:
    __array_ufunc__ = None  # make NumPy defer to our reflected operators
    __array_priority__ = 1000

    def __init__(self, val, tan, tag):
        self.val = val
        shp = shape_of(val)
        if shape_of(tan) != shp:
            tan = tan + np.zeros(shp)
        self.tan = tan
        self.tag = tag

    @property
    def shape(self):
        return shape_of(self.val)

    @property
    def ndim(self):
        return len(self.shape)

    @property
    def T(self):
        return transpose(self)

    def __getitem__(self, idx):
        return Dual(self.val[idx], self.tan[idx], self.tag)

    def reshape(self, *s):
        return Dual(self.val.reshape(*s), self.tan.reshape(*s), self.tag)

    def __len__(self):
        return self.shape[0]

    # arithmetic -------------------------------------------------------
    def __add__(self, o):
        return binop(self, o, lambda a, b: a + b, lambda a, b: 1.0, lambda a, b: 1.0)

    def __radd__(self, o):
        return binop(o, self, lambda a, b: a + b, lambda a, b: 1.0, lambda a, b: 1.0)

    def __sub__(self, o):
        return binop(self, o, lambda a, b: a - b, lambda a, b: 1.0, lambda a, b: -1.0)

    def __rsub__(self, o):
        return binop(o, self, lambda a, b: a - b, lambda a, b: 1.0, lambda a, b: -1.0)

    def __mul__(self, o):
        return binop(self, o, lambda a, b: a * b, lambda a, b: b, lambda a, b: a)

    def __rmul__(self, o):
        return binop(o, self, lambda a, b: a * b, lambda a, b: b, lambda a, b: a)

    def __truediv__(self, o):
        return binop(self, o, lambda a, b: a / b, lambda a, b: 1.0 / b,
                     lambda a, b: -a / (b * b))

    def __rtruediv__(self, o):
        return binop(o, self, lambda a, b: a / b, lambda a, b: 1.0 / b,
                     lambda a, b: -a / (b * b))

    def __neg__(self):
        return Dual(-self.val, -self.tan, self.tag)

    def __pos__(self):
        return self

    def __pow__(self, p):
        if isinstance(p, Dual):
            raise NotImplementedError("dual exponent")
        return unary(self, lambda v: v ** p, lambda v: p * v ** (p - 1))

    def __matmul__(self, o):
        return einsum_dual("...ij,...jk->...ik" if shape_of(o) and len(shape_of(o)) > 1
                           else "...ij,j->...i", self, o)

    def __rmatmul__(self, o):
        if len(shape_of(self)) == 1:
            return einsum_dual("...ij,j->...i", o, self)
        return einsum_dual("...ij,...jk->...ik", o, self)

    # comparisons act on the primal value (not differentiated)
    def __lt__(self, o):
        return primal(self) < primal(o)

    def __le__(self, o):
        return primal(self) <= primal(o)

    def __gt__(self, o):
        return primal(self) > primal(o)

    def __ge__(self, o):
        return primal(self) >= primal(o)

    def __float__(self):
        return float(primal(self))


def binop(a, b, f, da, db):
    ta, tb = tag_of(a), tag_of(b)
    t = max(ta, tb)
    if ta == t and tb == t:
        v = f(a.val, b.val)
        tan = da(a.val, b.val) * a.tan + db(a.val, b.val) * b.tan
    elif ta == t:
        v = f(a.val, b)
        tan = da(a.val, b) * a.tan
    else:
        v = f(a, b.val)
        tan = db(a, b.val) * b.tan
    return Dual(v, tan, t)


def unary(x, f, df):
    if not isinstance(x, Dual):
        return f(x)
    return Dual(f(x.val), df(x.val) * x.tan, x.tag)


def transpose(x, axes=None):
    if isinstance(x, Dual):
        return Dual(transpose(x.val, axes), transpose(x.tan, axes), x.tag)
    return np.transpose(x, axes)


def einsum_dual(subs, *ops, **kw):
    tags = [tag_of(o) for o in ops]
    t = max(tags)
    if t < 0:
        return wrap(np.einsum(subs, *ops, **kw))
    vals = [o.val if tag_of(o) == t else o for o in ops]
    v = einsum_dual(subs, *vals, **kw)
    tan = None
    for k, o in enumerate(ops):
        if tag_of(o) == t:
            args = list(vals)
            args[k] = o.tan
            term = einsum_dual(subs, *args, **kw)
            tan = term if tan is None else tan + term
    return Dual(v, tan, t)


# Dual-aware elementary functions ------------------------------------------
def d_exp(x):
    return unary(x, d_exp, d_exp) if isinstance(x, Dual) else wrap(np.exp(x))


def d_log(x):
    return unary(x, d_log, lambda v: 1.0 / v) if isinstance(x, Dual) else wrap(np.log(x))


def d_sqrt(x):
    return (unary(x, d_sqrt, lambda v: 0.5 / d_sqrt(v)) if isinstance(x, Dual)
            else wrap(np.sqrt(x)))


def d_arctan(x):
    return (unary(x, d_arctan, lambda v: 1.0 / (1.0 + v * v)) if isinstance(x, Dual)
            else wrap(np.arctan(x)))


def d_square(x):
    return unary(x, d_square, lambda v: 2.0 * v) if isinstance(x, Dual) else wrap(np.square(x))


def d_power(x, p):
    if isinstance(p, Dual):
        raise NotImplementedError("dual exponent")
    if isinstance(x, Dual):
        return unary(x, lambda v: d_power(v, p), lambda v: p * d_power(v, p - 1))
    return wrap(np.power(x, p))


def d_abs(x):
    if isinstance(x, Dual):
        return unary(x, d_abs, lambda v: np.sign(primal(v)))
    return wrap(np.abs(x))


def d_erf(x):
    if isinstance(x, Dual):
        return unary(x, d_erf, lambda v: 2.0 / np.sqrt(np.pi) * d_exp(-(v * v)))
    return wrap(_sps.erf(x))


def d_clip(x, lo, hi):
    if isinstance(x, Dual):
        p = primal(x)
        mask = ((p >= lo) & (p <= hi)).astype(float)
        return Dual(d_clip(x.val, lo, hi), mask * x.tan, x.tag)
    return wrap(np.clip(x, lo, hi))


def d_sum(x, axis=None, **kw):
    if isinstance(x, Dual):
        return Dual(d_sum(x.val, axis=axis, **kw), d_sum(x.tan, axis=axis, **kw), x.tag)
    return wrap(np.sum(x, axis=axis, **kw))


# ----------------------------------------------------------------------------
# Transformations.
# ----------------------------------------------------------------------------
def jit(f=None, *args, **kwargs):
    if f is None:
        return lambda g: g
    return f


def _take(a, i, ax):
    if isinstance(a, Dual):
        raise NotImplementedError("vmap over a dual number")
    return np.take(np.asarray(a), i, axis=ax)


def _stack(items, axis):
    if any(isinstance(v, Dual) for v in items):
        raise NotImplementedError("vmap returning a dual number")
    return wrap(np.stack([np.asarray(v) for v in items], axis=axis))


def vmap(f, in_axes=0, out_axes=0):
    def vf(*args):
        if isinstance(in_axes, (tuple, list)):
            ia = tuple(in_axes)
        else:
            ia = (in_axes,) * len(args)
        n = None
        for a, ax in zip(args, ia):
            if ax is not None:
                n = np.shape(a)[ax]
                break
        if n == 0:
            # zero-length map of a scalar-valued function (e.g. no atom pairs)
            return wrap(np.zeros((0,)))
        results = []
        for i in range(n):
            sl = [(_take(a, i, ax) if ax is not None else a) for a, ax in zip(args, ia)]
            results.append(f(*sl))
        if isinstance(results[0], tuple):
            k = len(results[0])
            oa = tuple(out_axes) if isinstance(out_axes, (tuple, list)) else (out_axes,) * k
            return tuple(_stack([r[j] for r in results], oa[j]) for j in range(k))
        return _stack(results, out_axes)

    return vf


def _extract(out, tag):
    if isinstance(out, tuple):
        return tuple(_extract(o, tag) for o in out)
    if isinstance(out, Dual) and out.tag == tag:
        return out.tan
    return wrap(np.zeros(shape_of(out)))


def grad(f, argnums=0):
    def g(*args):
        tag = new_tag()
        a = list(args)
        x = a[argnums]
        if shape_of(x):
            raise NotImplementedError("grad over an array argument")
        a[argnums] = Dual(x, 1.0, tag)
        return _extract(f(*a), tag)

    return g


def jacfwd(f, argnums=0):
    def j(*args):
        x = args[argnums]
        xs = shape_of(x)
        cols = []
        for idx in np.ndindex(*xs):
            tag = new_tag()
            e = np.zeros(xs)
            e[idx] = 1.0
            a = list(args)
            a[argnums] = Dual(x, e, tag)
            cols.append(_extract(f(*a), tag))

        def assemble(leaves):
            t = max(tag_of(v) for v in leaves)
            if t >= 0:
                # nested use: the leaves still carry an outer perturbation
                vals = [v.val if tag_of(v) == t else v for v in leaves]
                tans = [v.tan if tag_of(v) == t else np.zeros(shape_of(v)) for v in leaves]
                return Dual(assemble(vals), assemble(tans), t)
            arr = np.stack([np.asarray(v) for v in leaves], axis=-1)
            return wrap(arr.reshape(np.shape(leaves[0]) + xs))

        if isinstance(cols[0], tuple):
            return tuple(assemble([c[k] for c in cols]) for k in range(len(cols[0])))
        return assemble(cols)

    return j
