"""Compile the XLA FFI handler ``pes_ffi.cc`` into ``libhqcgb_jax.so``.

Only where jaxlib is installed: its FFI headers come from
``jax.ffi.include_dir()``.  Links against the engine library
(``hqc_gb300/libhqcgb.so``, built first by ``hqc_gb300.build``).

    python -m hqc_gb300.jax_ffi.build
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.dirname(HERE)


def build():
    import jax  # noqa: F401  (ImportError without JAX)
    from jax import ffi
    from hqc_gb300 import build as engine
    engine.build()
    out = os.path.join(HERE, "libhqcgb_jax.so")
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-shared", os.path.join(HERE, "pes_ffi.cc"),
           "-I", ffi.include_dir(), "-I", os.path.join(PKG, "..", "include"),
           "-I", os.path.join(cuda, "include"), "-L", PKG, "-lhqcgb", "-Wl,-rpath," + PKG,
           "-o", out]
    subprocess.run(cmd, check=True)
    return out


if __name__ == "__main__":
    print(build())
    sys.exit(0)
