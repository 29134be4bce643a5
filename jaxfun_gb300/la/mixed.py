"""Mixed-precision variable-coefficient solver: tensor-core (split-TF32) PCG
inside FP64 iterative refinement, one C-ABI call (``jfg_pcg_varcoef_mixed``).

The inner operators are the FP64 ones padded from n to nq per axis (zero rows
and columns; eigenvalues padded with ones) and split into TF32 hi/lo pairs, so
every tensor-core contraction sees 16-byte aligned rows and K a multiple of 32.
"""

from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from .. import _lib
from ..device import as_device, workspace
from .tpmatrix import TPMatricesLUFactors
from .varcoef import VarCoefMatrix, fd_preconditioner, pack_varcoef_ops


class MixedPlan(C.Structure):
    _fields_ = [
        ("ndim", C.c_int), ("n", C.c_int), ("nq", C.c_int), ("batch", C.c_int),
        ("ops64", C.c_void_p), ("kw64", C.c_void_p),
        ("ops_hi", C.c_void_p), ("ops_lo", C.c_void_p), ("kw32", C.c_void_p),
        ("E_hi", C.c_void_p), ("E_lo", C.c_void_p), ("W_hi", C.c_void_p), ("W_lo", C.c_void_p),
        ("lam", C.c_void_p), ("fd_scale", C.c_void_p), ("ops32", C.c_void_p),
        ("residual", C.c_int),
        ("precond_bf16", C.c_int),
        ("E_hi16", C.c_void_p), ("E_lo16", C.c_void_p), ("W_hi16", C.c_void_p),
        ("W_lo16", C.c_void_p),
        ("apply_f16", C.c_int),
        ("ops_hi16", C.c_void_p), ("ops_lo16", C.c_void_p), ("ops_inv16", C.c_void_p),
        ("fused_dots", C.c_int),
        ("schedule", C.c_int),
    ]


def split_bf16(a: np.ndarray) -> tuple[torch.Tensor, torch.Tensor]:
    """FP64 host array -> (hi, lo) BF16 bit patterns as int16 device tensors."""
    L = _lib.lib()
    a = np.ascontiguousarray(a, dtype=np.float64)
    hi = np.empty(a.shape, dtype=np.uint16)
    lo = np.empty(a.shape, dtype=np.uint16)
    L.jfg_split_bf16_host(a.size, a.ctypes.data, hi.ctypes.data, lo.ctypes.data)
    return (as_device(hi.view(np.int16), torch.int16), as_device(lo.view(np.int16), torch.int16))


def split_f16_rows(n: int, nq: int, ops: np.ndarray, ndim: int = 2):
    """2-D or 3-D packed operators (FP64) -> FP16 (hi, lo) bit patterns as int16
    device tensors, each operator row scaled by a power of two, and the inverse
    row scales (FP32 device tensor) for the scaled split-FP16 apply."""
    L = _lib.lib()
    a = np.ascontiguousarray(ops, dtype=np.float64)
    hi = np.empty(a.shape, dtype=np.uint16)
    lo = np.empty(a.shape, dtype=np.uint16)
    inv = np.empty(L.jfg_varcoef_f16_rows_nd(ndim, n, nq), dtype=np.float32)
    L.jfg_split_f16_rows_nd_host(ndim, n, nq, a.ctypes.data, hi.ctypes.data, lo.ctypes.data,
                                 inv.ctypes.data)
    return (as_device(hi.view(np.int16), torch.int16), as_device(lo.view(np.int16), torch.int16),
            as_device(inv, torch.float32))


def split_tf32(a: np.ndarray) -> tuple[torch.Tensor, torch.Tensor]:
    """FP64 host array -> (hi, lo) FP32 device tensors (TF32 split)."""
    L = _lib.lib()
    a = np.ascontiguousarray(a, dtype=np.float64)
    hi = np.empty(a.shape, dtype=np.float32)
    lo = np.empty(a.shape, dtype=np.float32)
    L.jfg_split_tf32_host(a.size, a.ctypes.data, hi.ctypes.data, lo.ctypes.data)
    return as_device(hi, torch.float32), as_device(lo, torch.float32)


def _pad(M: np.ndarray, rows: int, cols: int) -> np.ndarray:
    out = np.zeros((rows, cols))
    out[: M.shape[0], : M.shape[1]] = M
    return out


class MixedVarCoefSolver:
    """Solve A(kappa_b) x_b = rhs_b for a batch with the mixed-precision path."""

    def __init__(self, A: VarCoefMatrix, M: TPMatricesLUFactors | None = None,
                 residual: str = "df64", fp32_updates: bool | None = None,
                 precond: str | None = None, apply: str | None = None, fused_dots: bool = True,
                 schedule: str = "sync"):
        """``residual``: arithmetic of the refinement residual r = b - A x,
        "df64" (double-FP32 on the FP32 units) or "f64" (FP64 FMAs).
        ``fp32_updates``: once ||r|| <= 1e-4 ||b||, update r -= ||r|| A d in FP32
        instead of recomputing it (default: in 2-D only; in 3-D the operator's
        conditioning turns the FP32 update error into > 1e-10 solution error).
        ``precond``: plain "bf16" (one BF16 product per term, ~2^-8 relative),
        split-"bf16x3" (~2^-16) or split-"tf32" tensor-core passes for the
        inner fast-diagonalisation preconditioner.  Default: "bf16" in 2-D,
        "bf16x3" in 3-D.  The preconditioner tolerates the rounding: in the
        oracle's PCG at N = 128 and 256 plain BF16 left every iteration count
        unchanged, and on the benchmark's 128 problems at N = 256 it ran
        90.42 inner iterations against 90.40 with split BF16, 5.5 % faster
        (split BF16 was ~7 % faster than split TF32).  Padded sizes with
        nq % 8 != 0 use split-TF32 (the BF16 rows would not be 16-byte
        multiples).
        ``apply``: the inner operator passes as scaled split-"f16x3" (FP16
        hi/lo pairs with power-of-two scales per operator row and per problem,
        the accuracy of split TF32 at twice its MMA rate) or split-"tf32".
        Default: "f16x3" in 2-D, "tf32" in 3-D (at 32 x 128^3 the FP16 passes
        saved iterations but not time: 37.1 against 37.6 solves/s, and their
        answer error was 3.2e-11 against 2.4e-12); nq % 8 != 0 uses split-TF32.
        ``fused_dots``: take the inner PCG's p.Ap and r.M^-1 r from the
        contraction epilogues (the field pass and the divide pass) instead of
        separate dot kernels; r.M^-1 r only for a symmetric factorisation.
        ``schedule``: "sync" (default: every refinement step waits for all
        inner solves) or "flat" (each problem takes its refinement steps on its
        own, restarting its inner solve at the next 10-iteration boundary
        after it converges while the others keep iterating).  On the
        benchmark's batches the hard problems are hard in every step, so the
        flat schedule does not shorten the batch and its extra rounds cost
        more than they overlap; it pays when the slow problem changes from
        step to step."""
        if schedule not in ("flat", "sync"):
            raise ValueError(f"schedule must be 'flat' or 'sync', not {schedule!r}")
        if precond is None:
            precond = "bf16" if A.ndim == 2 else "bf16x3"
        if precond not in ("tf32", "bf16x3", "bf16"):
            raise ValueError(f"precond must be 'tf32', 'bf16x3' or 'bf16', not {precond!r}")
        if apply is None:
            apply = "f16x3" if A.ndim == 2 else "tf32"
        if apply not in ("tf32", "f16x3"):
            raise ValueError(f"apply must be 'tf32' or 'f16x3', not {apply!r}")
        if residual not in ("df64", "f64"):
            raise ValueError(f"residual must be 'df64' or 'f64', not {residual!r}")
        self.A = A
        nd, n, nq = A.ndim, A.n, A.nq
        if fp32_updates is None:
            fp32_updates = nd == 2
        s0 = A.T.basespaces[0]
        B = s0.backward_matrix(None, 0)
        D = s0.backward_matrix(None, 1)
        ops_pad = pack_varcoef_ops(nd, _pad(B, nq, nq), _pad(D, nq, nq))
        self.ops_hi, self.ops_lo = split_tf32(ops_pad)
        af = apply == "f16x3" and nq % 8 == 0
        if af:
            self.ops16 = split_f16_rows(nq, nq, ops_pad, nd)
        self.ops32 = as_device(ops_pad, torch.float32)
        self.kw32 = A.kw.to(torch.float32).contiguous()
        fac = fd_preconditioner(A.T) if M is None else M
        self.E_hi, self.E_lo = split_tf32(_pad(fac.E_host, nq, nq))
        self.W_hi, self.W_lo = split_tf32(_pad(fac.W_host, nq, nq))
        # BF16 operator rows must be 16-byte multiples (nq % 8 == 0) for TMA
        pb = precond in ("bf16x3", "bf16") and nq % 8 == 0
        p1 = pb and precond == "bf16"
        self.precond = ("bf16" if p1 else "bf16x3") if pb else "tf32"  # as run
        if pb:
            self.E16 = split_bf16(_pad(fac.E_host, nq, nq))
            self.W16 = split_bf16(_pad(fac.W_host, nq, nq))
        lam = np.ones(nq)
        lam[:n] = fac.lam_host
        # PCG scalars from the epilogues: p.Ap always (the operator is
        # symmetric by construction), r.M^-1 r when E = W^T
        fused = 1 | (2 if (fused_dots and np.array_equal(fac.E_host, fac.W_host.T)) else 0)
        if not fused_dots:
            fused = 0
        self.lam = as_device(lam, torch.float32)
        self.plan = MixedPlan(nd, n, nq, A.batch, A.ops.data_ptr(), A.kw.data_ptr(),
                              self.ops_hi.data_ptr(), self.ops_lo.data_ptr(),
                              self.kw32.data_ptr(), self.E_hi.data_ptr(), self.E_lo.data_ptr(),
                              self.W_hi.data_ptr(), self.W_lo.data_ptr(), self.lam.data_ptr(),
                              None, self.ops32.data_ptr() if fp32_updates else None,
                              1 if residual == "df64" else 0, (2 if p1 else 1) if pb else 0,
                              self.E16[0].data_ptr() if pb else None,
                              self.E16[1].data_ptr() if pb and not p1 else None,
                              self.W16[0].data_ptr() if pb else None,
                              self.W16[1].data_ptr() if pb and not p1 else None,
                              1 if af else 0,
                              self.ops16[0].data_ptr() if af else None,
                              self.ops16[1].data_ptr() if af else None,
                              self.ops16[2].data_ptr() if af else None,
                              fused, 1 if schedule == "flat" else 0)

    def autotune(self, ws=None) -> list[dict]:
        """Tune the tensor-core passes of the inner solve once (each distinct
        pass signature keeps its fastest launch configuration for the
        process); returns the tuned configurations."""
        L = _lib.lib()
        if ws is None:
            ws = workspace(self.workspace_bytes(), slot=1)
        _lib.check(L.jfg_pcg_mixed_autotune(C.byref(self.plan), ws.data_ptr(), ws.numel(),
                                            _lib.stream_handle()), "jfg_pcg_mixed_autotune")
        return _lib.tuned_configs()

    def workspace_bytes(self) -> int:
        A = self.A
        return int(_lib.lib().jfg_pcg_mixed_workspace_size(A.ndim, A.n, A.nq, A.batch))

    def solve(self, b, x0=None, tol: float = 1e-10, inner_tol: float = 5e-6,
              max_outer: int = 10, maxiter_inner: int = 1000, out=None, ws=None, guess=None):
        """Returns (x, inner_iterations, outer_iterations) per problem.

        ``x0``: an FP64 starting iterate (its residual is formed in FP64);
        ``guess``: a learned initial guess for the first inner solve (judged per
        problem against the zero start, see jfg_pcg_varcoef_mixed_guess)."""
        A = self.A
        b = as_device(b)
        if x0 is None:
            x = torch.empty_like(b) if out is None else out
        else:
            x = as_device(x0).clone() if out is None else out.copy_(as_device(x0))
        g = None if guess is None else as_device(guess)
        L = _lib.lib()
        if ws is None:
            ws = workspace(self.workspace_bytes(), slot=1)
        it_in = (C.c_int * A.batch)()
        it_out = (C.c_int * A.batch)()
        st = L.jfg_pcg_varcoef_mixed_guess(C.byref(self.plan), b.data_ptr(), x.data_ptr(),
                                           None if g is None else g.data_ptr(),
                                           0 if x0 is None else 1, float(tol), float(inner_tol),
                                           int(max_outer), int(maxiter_inner), it_in, it_out,
                                           ws.data_ptr(), ws.numel(), _lib.stream_handle())
        _lib.check(st, "jfg_pcg_varcoef_mixed")
        return x, np.array(it_in[:]), np.array(it_out[:])
