"""JAX binding of the engine: ``make_pes_jax`` returns a PES usable inside
``jax.jit`` with ``jax.grad`` / ``jax.vmap``, as the reference's ``make_pes``
(hqc/pbc/pes.py:10-153) is used.

The energy and its adjoint gradient come from one XLA FFI call
(``pes_ffi.cc``: the engine's batched SCF + forces + Ewald on XLA's stream)
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
    """Load the compiled handler and register it as the CUDA target
    "hqcgb_pes" (once per process)."""
    global _registered
    if _registered:
        return
    lib = ctypes.cdll.LoadLibrary(lib_path)
    jax.ffi.register_ffi_target("hqcgb_pes", jax.ffi.pycapsule(lib.HqcgbPes), platform="CUDA")
    _registered = True


def make_pes_jax(n, L, rs, basis, Gmax=15, kappa=10, **kw):
    """``pes(xp)`` -> F + Vpp (Rydberg) for xp (n, 3) or (B, n, 3) in rs
    units, differentiable with jax.grad (the engine's adjoint).  Other
    keyword arguments as ``make_pes`` (precision, dft, xc, smearing, ...)."""
    register()
    host = make_pes(n, L, rs, basis, forces=True, Gmax=Gmax, kappa=kappa, **kw)
    plan = int(host.solver.plan.handle.value)

    def _call(xp):
        shape = xp.shape
        batch = shape[:-2]
        f64 = jnp.float64
        outs = (jax.ShapeDtypeStruct(batch + (5,), f64), jax.ShapeDtypeStruct(batch, f64),
                jax.ShapeDtypeStruct(shape, f64), jax.ShapeDtypeStruct(batch, f64),
                jax.ShapeDtypeStruct(shape, f64), jax.ShapeDtypeStruct(batch, jnp.int32))
        call = jax.ffi.ffi_call("hqcgb_pes", outs, vmap_method="broadcast_all")
        energies, free, grad, vpp, vpp_grad, conv = call(
            xp, xp * rs, plan=np.int64(plan), L_rs=np.float64(L), rs=np.float64(rs),
            kappa=np.float64(kappa), gmax=np.int64(Gmax))
        value = 2.0 * free + vpp                       # Hartree -> Rydberg, + Vpp
        g = 2.0 * rs * grad + vpp_grad                 # Hartree/Bohr -> Rydberg per rs unit
        return value, g

    @jax.custom_vjp
    def pes(xp):
        return _call(xp)[0]

    def fwd(xp):
        value, g = _call(xp)
        return value, g

    def bwd(g, ct):
        return (ct[..., None, None] * g,)

    pes.defvjp(fwd, bwd)
    pes.host = host
    return pes
