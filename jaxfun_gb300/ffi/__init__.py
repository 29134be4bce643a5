"""jax.ffi binding of the C ABI: the drop-in for jaxfun's jit-compiled methods.

``jfg_xla.cc`` defines one XLA FFI handler per entry point (transforms, FD
solve, variable-coefficient apply, PCG); ``jaxfun_gb300/build.py`` compiles it
into ``_lib/libjfg_xla.so`` when XLA's FFI header is available (jaxlib's
include directory or ``JFG_XLA_INCLUDE``).  ``register()`` then registers the
handlers with JAX as CUDA custom-call targets, and the functions below are
what jaxfun's ``TensorProductSpace.forward/backward/scalar_product``
(src/jaxfun/galerkin/tensorproductspace.py:330-417),
``TPMatricesLUFactors.solve`` (src/jaxfun/la/tpmatrix.py:545-587) and
``TensorMatrix.__matmul__`` (src/jaxfun/la/tensormatrix.py:54-56) would call
inside their jitted bodies.  JAX is imported lazily: this module loads
without it, and every function raises if JAX or the handler library is
missing (there is no fallback).
"""

from __future__ import annotations

import ctypes
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent.parent / "_lib" / "libjfg_xla.so"

TARGETS = {
    "jfg_tp_apply_1d": "JfgTpApply1d",
    "jfg_tp_apply_2d": "JfgTpApply2d",
    "jfg_tp_apply_3d": "JfgTpApply3d",
    "jfg_fd_solve": "JfgFdSolve",
    "jfg_varcoef_apply": "JfgVarcoefApply",
    "jfg_pcg_varcoef": "JfgPcgVarcoef",
}

_registered = False


def register() -> None:
    """Register every handler of libjfg_xla.so as a CUDA FFI target (once)."""
    global _registered
    if _registered:
        return
    import jax

    if not LIB_PATH.exists():
        raise RuntimeError(f"{LIB_PATH} is not built: XLA's FFI header was not found at build "
                           "time (set JFG_XLA_INCLUDE or install jaxlib, then rebuild)")
    lib = ctypes.cdll.LoadLibrary(str(LIB_PATH))
    for name, sym in TARGETS.items():
        jax.ffi.register_ffi_target(name, jax.ffi.pycapsule(getattr(lib, sym)),
                                    platform="CUDA")
    _registered = True


def tp_apply(mats, x):
    """y[b] = (x_ax mats[ax]) x[b] for x of shape (batch, cols...), FP64: the
    per-axis operators of a forward, backward or scalar product."""
    import jax
    import jax.numpy as jnp

    register()
    nd = len(mats)
    out = jax.ShapeDtypeStruct((x.shape[0],) + tuple(m.shape[0] for m in mats), jnp.float64)
    return jax.ffi.ffi_call(f"jfg_tp_apply_{nd}d", out)(x, *mats)


def fd_solve(E, W, lam, c0, c1, rhs):
    """U = (x W) [(x E) F / (c0[b] + c1[b] sum lam)] for rhs (batch, n, n[, n])."""
    import jax
    import jax.numpy as jnp

    register()
    out = jax.ShapeDtypeStruct(rhs.shape, jnp.float64)
    return jax.ffi.ffi_call("jfg_fd_solve", out)(E, W, lam, c0, c1, rhs)


def varcoef_apply(ops, kw, u):
    """v = A(kappa) u with the packed operators of jfg_varcoef_pack_ops_host."""
    import jax
    import jax.numpy as jnp

    register()
    out = jax.ShapeDtypeStruct(u.shape, jnp.float64)
    return jax.ffi.ffi_call("jfg_varcoef_apply", out)(ops, kw, u)


def pcg_varcoef(ops, kw, E, W, lam, fd_scale, rhs, tol=1e-10, maxiter=1000):
    """Batched FD-preconditioned FP64 PCG: returns (x, iterations per problem)."""
    import jax
    import jax.numpy as jnp
    import numpy as np

    register()
    outs = (jax.ShapeDtypeStruct(rhs.shape, jnp.float64),
            jax.ShapeDtypeStruct((rhs.shape[0],), jnp.int32))
    return jax.ffi.ffi_call("jfg_pcg_varcoef", outs)(ops, kw, E, W, lam, fd_scale, rhs,
                                                      tol=np.float64(tol),
                                                      maxiter=np.int64(maxiter))
