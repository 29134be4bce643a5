"""ctypes binding of the C ABI in ``include/jaxfun_gb300.h``.

The shared library is built in-tree (``jaxfun_gb300/_lib/libjaxfun_gb300.so``).
There is no CPU fallback: if the library cannot be loaded, every compute call
raises.  Device buffers are torch CUDA tensors; only their data pointers and
the current CUDA stream cross the boundary.
"""

from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "_lib" / "libjaxfun_gb300.so"

JFG_OK = 0
JFG_ERR_ARG = 1
JFG_ERR_CUDA = 2
JFG_ERR_NOT_CONVERGED = 3
JFG_ERR_DEVICE_TIMEOUT = 4
JFG_ERR_UNSUPPORTED = 5
JFG_ERR_WORKSPACE = 6

EPI_NONE = 0
EPI_MUL_FIELD = 1
EPI_DIV_EIG = 2


class JfgError(RuntimeError):
    """A C-ABI call returned a non-zero status."""

    def __init__(self, status: int, what: str):
        self.status = status
        msg = f"{what}: {status_string(status)} (status {status})"
        if status == JFG_ERR_CUDA and _lib is not None:
            msg += f", cuda error {_lib.jfg_last_cuda_error()}"
        super().__init__(msg)


class NotConvergedError(JfgError):
    pass


class TcConfig(C.Structure):
    _fields_ = [("operand_a_in_tmem", C.c_int), ("order", C.c_int), ("ctas", C.c_int),
                ("stages", C.c_int), ("mtile", C.c_int), ("schedule", C.c_int),
                ("store", C.c_int)]


class ContractDesc(C.Structure):
    _fields_ = [
        ("batch", C.c_int), ("nseg", C.c_int), ("M", C.c_int), ("P", C.c_int), ("K", C.c_int),
        ("op_ld", C.c_longlong), ("op_seg", C.c_longlong),
        ("in_ld", C.c_longlong), ("in_seg", C.c_longlong), ("in_batch", C.c_longlong),
        ("out_ld", C.c_longlong), ("out_seg", C.c_longlong), ("out_batch", C.c_longlong),
        ("epilogue", C.c_int),
        ("field", C.c_void_p),
        ("field_ld", C.c_longlong), ("field_seg", C.c_longlong), ("field_batch", C.c_longlong),
        ("lam_m", C.c_void_p), ("lam_p", C.c_void_p), ("c0", C.c_void_p), ("c1", C.c_void_p),
        ("alpha", C.c_double), ("beta", C.c_double),
        ("batch_list", C.c_void_p), ("batch_count", C.c_void_p),
    ]


_vp = C.c_void_p
_i = C.c_int
_sz = C.c_size_t
_d = C.c_double

# name -> (restype, argtypes)
SIGNATURES = {
    "jfg_version": (C.c_char_p, []),
    "jfg_status_string": (C.c_char_p, [_i]),
    "jfg_last_cuda_error": (_i, []),
    "jfg_device_supported": (_i, []),
    "jfg_launch_count": (C.c_longlong, []),
    "jfg_reset_launch_count": (None, []),
    "jfg_weighted_field_f64": (_i, [_i, _i, _i, _vp, _vp, _vp, _vp, _vp]),
    "jfg_exp_weighted_field_f64": (_i, [_i, _i, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "jfg_field_moments_f64": (_i, [_i, _i, _i, _vp, _vp, _vp, _vp]),
    "jfg_exp_weighted_backward_workspace_size": (_sz, [_i, _i, _i, _i]),
    "jfg_exp_weighted_backward_f64": (_i, [_i, _i, _i, _i, _vp, _vp, _i, _vp, _vp, _vp, _vp,
                                           _vp, _sz, _vp]),
    "jfg_contract_f64": (_i, [C.POINTER(ContractDesc), _vp, _vp, _vp, _vp]),
    "jfg_contract_f32": (_i, [C.POINTER(ContractDesc), _vp, _vp, _vp, _vp]),
    "jfg_contract_df64": (_i, [C.POINTER(ContractDesc), _vp, _vp, _vp, _vp]),
    "jfg_contract_tc": (_i, [C.POINTER(ContractDesc), _vp, _vp, _vp, _vp, _vp]),
    "jfg_contract_tc_bf16x3": (_i, [C.POINTER(ContractDesc), _vp, _vp, _vp, _vp, _vp]),
    "jfg_split_bf16_host": (None, [_sz, _vp, _vp, _vp]),
    "jfg_tp_apply_tc_bf16x3": (_i, [_i, _vp, _vp, _i, _vp, _vp, _vp, _vp, _vp, _sz, _vp]),
    "jfg_tc_set_store_path": (_i, [_i]),
    "jfg_tc_set_op_resident": (_i, [_i]),
    "jfg_tc_set_autotune": (_i, [_i]),
    "jfg_tc_force_config": (_i, [_vp]),
    "jfg_tc_tuned_count": (_i, []),
    "jfg_tc_tuned_entry": (_i, [_i, C.c_char_p, _sz, _vp, _vp]),
    "jfg_banded_lu_size": (_sz, [_i, _i, _i, _i]),
    "jfg_banded_lu_factor_f64": (_i, [_i, _i, _i, _vp, _vp, _vp, _vp]),
    "jfg_banded_lu_solve_f64": (_i, [_i, _i, _i, _i, _vp, _vp, _vp, C.c_longlong,
                                     C.c_longlong, _vp]),
    "jfg_contract_tc_grouped": (_i, [_i, C.POINTER(ContractDesc), _vp, _vp, _vp, _vp, _vp, _vp]),
    "jfg_tc_autotune": (_i, [_i, C.POINTER(ContractDesc), _vp, _vp, _vp, _vp, _i, _vp, _vp, _vp]),
    "jfg_split_tf32_host": (None, [_sz, _vp, _vp, _vp]),
    "jfg_tc_set_variant": (_i, [_i]),
    "jfg_device_status": (_i, []),
    "jfg_tc_set_wait_budget_ns": (_i, [C.c_ulonglong]),
    "jfg_tc_test_hold": (_i, [_i]),
    "jfg_tp_apply_workspace_size": (_sz, [_i, C.POINTER(_i), C.POINTER(_i), _i, _i]),
    "jfg_tp_apply_f64": (_i, [_i, C.POINTER(_i), C.POINTER(_i), _i, C.POINTER(_vp), _vp, _vp,
                              _vp, _sz, _vp]),
    "jfg_tp_apply_f32": (_i, [_i, C.POINTER(_i), C.POINTER(_i), _i, C.POINTER(_vp), _vp, _vp,
                              _vp, _sz, _vp]),
    "jfg_tp_apply_df64": (_i, [_i, C.POINTER(_i), C.POINTER(_i), _i, C.POINTER(_vp), _vp, _vp,
                               _vp, _sz, _vp]),
    "jfg_tp_apply_tc": (_i, [_i, C.POINTER(_i), C.POINTER(_i), _i, C.POINTER(_vp),
                             C.POINTER(_vp), _vp, _vp, _vp, _sz, _vp]),
    "jfg_tp_apply_affine_f64": (_i, [_i, C.POINTER(_i), C.POINTER(_i), _i, C.POINTER(_vp),
                                     _vp, _vp, _vp, _vp, _sz, _vp]),
    "jfg_fd_solve_workspace_size": (_sz, [_i, _i, _i, _i]),
    "jfg_fd_solve_f64": (_i, [_i, _i, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _sz, _vp]),
    "jfg_fd_solve_f32": (_i, [_i, _i, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _sz, _vp]),
    "jfg_fd_solve_tc": (_i, [_i, _i, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _sz,
                             _vp]),
    "jfg_helmholtz_workspace_size": (_sz, [_i, _i]),
    "jfg_helmholtz_apply_f64": (_i, [_i, _i, _i, _vp, _vp, _vp, _vp, _vp, _sz, _vp]),
    "jfg_helmholtz_solve_workspace_size": (_sz, [_i, _i, _i]),
    "jfg_helmholtz_grouped_workspace_size": (_sz, [_i, _vp, _vp, _vp]),
    "jfg_helmholtz_solve_grouped": (_i, [_i, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp,
                                         _vp, _vp, _vp, _d, _i, _vp, _vp, _vp, _sz, _vp]),
    "jfg_helmholtz_solve_mixed": (_i, [_i, _i, _i, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp,
                                       _vp, _d, _i, C.POINTER(_i), _vp, _sz, _vp]),
    "jfg_fd_solve_noalloc_max_bytes": (_sz, []),
    "jfg_fd_solve_f64_noalloc": (_i, [_i, _i, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "jfg_varcoef_ops_count": (_sz, [_i, _i, _i]),
    "jfg_varcoef_f16_rows": (_sz, [_i, _i]),
    "jfg_split_f16_rows_host": (None, [_i, _i, _vp, _vp, _vp, _vp]),
    "jfg_varcoef_f16_rows_nd": (_sz, [_i, _i, _i]),
    "jfg_split_f16_rows_nd_host": (None, [_i, _i, _i, _vp, _vp, _vp, _vp]),
    "jfg_split_f16_rowscaled_host": (None, [_sz, _sz, _vp, _vp, _vp, _vp]),
    "jfg_contract_tc_f16x3": (_i, [C.POINTER(ContractDesc), _vp, _vp, _vp, C.c_longlong, _vp, _vp,
                                   _vp, _vp, _vp]),
    "jfg_varcoef_pack_ops_host": (None, [_i, _i, _i, _vp, _vp, _vp]),
    "jfg_varcoef_workspace_size": (_sz, [_i, _i, _i, _i, _i]),
    "jfg_varcoef_apply_f64": (_i, [_i, _i, _i, _i, _vp, _vp, _vp, _vp, _vp, _sz, _vp]),
    "jfg_varcoef_apply_f32": (_i, [_i, _i, _i, _i, _vp, _vp, _vp, _vp, _vp, _sz, _vp]),
    "jfg_pcg_mixed_workspace_size": (_sz, [_i, _i, _i, _i]),
    "jfg_pcg_mixed_autotune": (_i, [_vp, _vp, _sz, _vp]),
    "jfg_pcg_varcoef_mixed": (_i, [_vp, _vp, _vp, _i, _d, _d, _i, _i, C.POINTER(_i),
                                   C.POINTER(_i), _vp, _sz, _vp]),
    "jfg_pcg_varcoef_mixed_guess": (_i, [_vp, _vp, _vp, _vp, _i, _d, _d, _i, _i, C.POINTER(_i),
                                         C.POINTER(_i), _vp, _sz, _vp]),
    "jfg_pcg_workspace_size": (_sz, [_i, _i, _i, _i, _i]),
    "jfg_pcg_varcoef_f64": (_i, [_i, _i, _i, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _i,
                                 _d, _i, C.POINTER(_i), _vp, _sz, _vp]),
}

_lib: C.CDLL | None = None


def load(build_if_missing: bool = True) -> C.CDLL:
    """Load the shared library (building it first if absent and nvcc exists)."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists() and build_if_missing:
        from .build import build

        build()
    if not LIB_PATH.exists():
        raise RuntimeError(
            f"jaxfun_gb300 CUDA library not found at {LIB_PATH}; run jaxfun_gb300.build.build()"
        )
    lib = C.CDLL(os.fspath(LIB_PATH))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name, None)
        if fn is None:
            continue
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def lib() -> C.CDLL:
    return load()


def status_string(s: int) -> str:
    if _lib is None:
        return str(s)
    return _lib.jfg_status_string(s).decode()


def check(status: int, what: str) -> None:
    if status == JFG_OK:
        return
    if status == JFG_ERR_NOT_CONVERGED:
        raise NotConvergedError(status, what)
    raise JfgError(status, what)


def ptr(t) -> int | None:
    """Device pointer of a torch tensor (None passes NULL)."""
    if t is None:
        return None
    return t.data_ptr()


def stream_handle(stream=None) -> int:
    import torch

    s = torch.cuda.current_stream() if stream is None else stream
    return s.cuda_stream


def int_array(vals):
    arr = (C.c_int * len(vals))(*[int(v) for v in vals])
    return arr


def ptr_array(ptrs):
    return (C.c_void_p * len(ptrs))(*ptrs)


class GemmDesc(C.Structure):
    """Mirror of jfg_gemm_desc (include/jaxfun_gb300.h)."""

    _fields_ = [
        ("batch", C.c_int), ("M", C.c_int), ("N", C.c_int), ("K", C.c_int), ("ksplit", C.c_int),
        ("lda", C.c_longlong), ("a_batch", C.c_longlong),
        ("ldb", C.c_longlong), ("b_batch", C.c_longlong),
        ("alpha", C.c_float), ("act", C.c_int),
        ("add", C.c_void_p), ("ld_add", C.c_longlong), ("add_batch", C.c_longlong),
        ("bias", C.c_void_p),
        ("gg", C.c_void_p), ("ld_gg", C.c_longlong), ("gg_batch", C.c_longlong),
        ("d32", C.c_void_p), ("ld_d32", C.c_longlong), ("d32_batch", C.c_longlong),
        ("d32_accumulate", C.c_int),
        ("pre", C.c_void_p), ("ld_pre", C.c_longlong), ("pre_batch", C.c_longlong),
        ("dbf", C.c_void_p), ("ld_dbf", C.c_longlong), ("dbf_batch", C.c_longlong),
        ("dtbf", C.c_void_p), ("ld_dtbf", C.c_longlong), ("dtbf_batch", C.c_longlong),
    ]


_ll = C.c_longlong
_f = C.c_float
SIGNATURES.update({
    "jfg_gemm_bf16": (_i, [C.POINTER(GemmDesc), _vp, _vp, _vp]),
    "jfg_sno_modemix_fwd": (_i, [_i, _i, _i, _vp, _vp, _vp, _vp]),
    "jfg_sno_modemix_bwd": (_i, [_i, _i, _i, _vp, _vp, _vp, _vp, _vp, _vp]),
    "jfg_colsum_bf16": (_i, [_ll, _i, _vp, _vp, _i, _vp]),
    "jfg_adam_step": (_i, [_ll, _vp, _vp, _vp, _vp, _f, _f, _f, _f, _i, _vp, _vp, _i, _i, _vp]),
    "jfg_sno_mse": (_i, [_ll, _vp, _ll, _vp, _vp, _vp, _vp, _vp]),
})


def tuned_configs() -> list[dict]:
    """Single-group tensor-core launch configurations chosen by the autotuner
    (jfg_tc_set_autotune / jfg_pcg_mixed_autotune), with their signatures and
    times."""
    L = lib()
    out = []
    buf = C.create_string_buffer(256)
    for i in range(L.jfg_tc_tuned_count()):
        cfg = TcConfig()
        ms = C.c_float()
        check(L.jfg_tc_tuned_entry(i, buf, 256, C.byref(cfg), C.byref(ms)), "jfg_tc_tuned_entry")
        out.append({"signature": buf.value.decode(), "ms": ms.value,
                    "operand_a_in_tmem": cfg.operand_a_in_tmem, "stages": cfg.stages,
                    "mtile": cfg.mtile or 128,
                    "schedule": {0: "default", 1: "streaming", 2: "operator-stationary"}[cfg.schedule],
                    "store": {0: "default", 1: "tma", 2: "plain"}[cfg.store]})
    return out
