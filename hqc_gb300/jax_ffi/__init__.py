"""JAX binding of the engine: ``make_pes_jax`` returns a PES usable inside
``jax.jit`` with ``jax.grad`` / ``jax.vmap``, as the reference's ``make_pes``
(hqc/pbc/pes.py:10-153) is used.

The energy and its adjoint gradient come from one XLA FFI call
(``pes_ffi.cc``: the engine's batched SCF + forces + Ewald on XLA's stream;
the Gamma point or a single k-point)
wrapped in ``jax.custom_vjp``, so ``jax.grad(pes)`` runs the engine's
adjoint instead of differentiating through the SCF (which the reference
cannot do either: its ``lax.while_loop`` has no reverse-mode rule).  The
value is the free energy F + Vpp whose exact gradient the adjoint gives
(F = E without smearing; see ``make_pes``'s ``value_and_grad``).

Needs jaxlib with CUDA and a compiled ``pes_ffi`` library (``build.py`` in
this folder; it compiles only where jaxlib's FFI headers exist).  Importing
this module without JAX raises ImportError; nothing else in the package
depends on it.
"""
import ctypes
import os

import jax
import jax.numpy as jnp
import numpy as np

from ..pes import make_pes

HERE = os.path.dirname(os.path.abspath(__file__))
_registered = False


def register(lib_path=os.path.join(HERE, "libhqcgb_jax.so")):
    """Load the compiled handlers and register them as the CUDA targets
    "hqcgb_pes" and "hqcgb_pes_kpt" (once per process)."""
    global _registered
    if _registered:
        return
    lib = ctypes.cdll.LoadLibrary(lib_path)
    jax.ffi.register_ffi_target("hqcgb_pes", jax.ffi.pycapsule(lib.HqcgbPes), platform="CUDA")
    jax.ffi.register_ffi_target("hqcgb_pes_kpt", jax.ffi.pycapsule(lib.HqcgbPesKpt), platform="CUDA")
    _registered = True


def make_pes_jax(n, L, rs, basis, Gmax=15, kappa=10, gamma=True, **kw):
    """``pes(xp)`` -> F + Vpp (Rydberg) for xp (n, 3) or (B, n, 3) in rs
    units, differentiable with jax.grad (the engine's adjoint).  With
    ``gamma=False``, ``pes(xp, kpt)`` at a single k-point (kpt (3,) or
    (B, 3) in 1/Bohr, pes_kpt of hqc/pbc/pes.py:88-98); its gradient is
    taken with respect to xp (the k-point's cotangent is zero).  Other
    keyword arguments as ``make_pes`` (precision, dft, xc, smearing, ...)."""
    register()
    host = make_pes(n, L, rs, basis, forces=True, Gmax=Gmax, kappa=kappa, gamma=gamma, **kw)
    plan = int(host.solver.plan.handle.value)
    attrs = dict(plan=np.int64(plan), L_rs=np.float64(L), rs=np.float64(rs), kappa=np.float64(kappa),
                 gmax=np.int64(Gmax))

    def _outs(shape):
        batch = shape[:-2]
        f64 = jnp.float64
        return (jax.ShapeDtypeStruct(batch + (5,), f64), jax.ShapeDtypeStruct(batch, f64),
                jax.ShapeDtypeStruct(shape, f64), jax.ShapeDtypeStruct(batch, f64),
                jax.ShapeDtypeStruct(shape, f64), jax.ShapeDtypeStruct(batch, jnp.int32))

    def _finish(free, grad, vpp, vpp_grad):
        value = 2.0 * free + vpp                       # Hartree -> Rydberg, + Vpp
        g = 2.0 * rs * grad + vpp_grad                 # Hartree/Bohr -> Rydberg per rs unit
        return value, g

    if gamma:
        def _call(xp):
            outs = _outs(xp.shape)
            call = jax.ffi.ffi_call("hqcgb_pes", outs, vmap_method="broadcast_all")
            energies, free, grad, vpp, vpp_grad, conv = call(xp, xp * rs, **attrs)
            return _finish(free, grad, vpp, vpp_grad)

        @jax.custom_vjp
        def pes(xp):
            return _call(xp)[0]

        def fwd(xp):
            value, g = _call(xp)
            return value, g

        def bwd(g, ct):
            return (ct[..., None, None] * g,)
    else:
        def _call(xp, kpt):
            kpt = jnp.broadcast_to(kpt, xp.shape[:-2] + (3,))
            outs = _outs(xp.shape)
            call = jax.ffi.ffi_call("hqcgb_pes_kpt", outs, vmap_method="broadcast_all")
            energies, free, grad, vpp, vpp_grad, conv = call(xp, xp * rs, kpt, **attrs)
            return _finish(free, grad, vpp, vpp_grad)

        @jax.custom_vjp
        def pes(xp, kpt):
            return _call(xp, kpt)[0]

        def fwd(xp, kpt):
            value, g = _call(xp, kpt)
            return value, (g, kpt)

        def bwd(res, ct):
            g, kpt = res
            return ct[..., None, None] * g, jnp.zeros_like(kpt)

    pes.defvjp(fwd, bwd)
    pes.host = host
    return pes
