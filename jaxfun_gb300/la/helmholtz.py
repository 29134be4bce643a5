"""Batched 2-D Dirichlet Helmholtz solves with uneven N (alpha^2 u - lap u = f).

Each problem b has its own N_b and alpha_b.  Problems are grouped by size and
the whole batch is ONE C-ABI call (``jfg_helmholtz_solve_grouped``): fast-
diagonalisation corrections on the tensor cores (split-TF32, padded layout;
every pass one persistent grouped launch over all size groups, configuration
chosen by the autotuner ``jfg_tc_autotune``) inside FP64 iterative
refinement whose residual r = b - A x is applied in O(n^2) from the
closed-form mass and stiffness matrices, the refinement step captured into a
CUDA graph.  The FD factors are those of ``tpmats_lu_factor`` for
alpha^2 M (x) M + K (x) M + M (x) K (src/jaxfun/la/tpmatrix.py:1089-1233), with
the general eigendecomposition for the non-symmetric Chebyshev stiffness.
"""

from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from .. import _lib
from ..device import as_device
from ..galerkin.spaces import DIRICHLET, Chebyshev, FunctionSpace, Legendre
from .mixed import split_tf32
from .tpmatrix import fd_eig

FAMILY = {"legendre": 0, "chebyshev": 1}


class _Group:
    def __init__(self, family: str, N: int, idx: np.ndarray, alphas: np.ndarray):
        space = Legendre if family == "legendre" else Chebyshev
        V = FunctionSpace(N, space, bcs=DIRICHLET)
        self.N, self.n = N, N - 2
        self.nq = (N + 3) // 4 * 4
        self.idx = idx
        K, M = V.stiffness_matrix(), V.mass_matrix()
        lam, W, E = fd_eig(K, M)
        Ep = np.zeros((self.nq, self.nq))
        Wp = np.zeros((self.nq, self.nq))
        Ep[: self.n, : self.n] = E
        Wp[: self.n, : self.n] = W
        lp = np.ones(self.nq)
        lp[: self.n] = lam
        self.E = split_tf32(Ep)
        self.W = split_tf32(Wp)
        self.lam32 = as_device(lp, torch.float32)
        a2 = np.asarray(alphas, dtype=np.float64)[idx] ** 2
        self.alpha2 = as_device(a2)
        self.alpha2_32 = as_device(a2, torch.float32)
        self.host = (K, M, lam, W, E)


class UnevenHelmholtzSolver:
    """alpha_b^2 u - lap u = f_b on [-1,1]^2, Dirichlet, N_b per problem."""

    def __init__(self, family: str, Ns, alphas):
        if family not in FAMILY:
            raise ValueError(f"family must be one of {tuple(FAMILY)}")
        self.family = family
        self.Ns = np.asarray(Ns, dtype=int)
        self.alphas = np.asarray(alphas, dtype=np.float64)
        self.groups = [
            _Group(family, int(N), np.nonzero(self.Ns == N)[0], self.alphas)
            for N in sorted(set(self.Ns.tolist()))
        ]
        # group-major flat layout of the whole batch
        self.order = np.concatenate([g.idx for g in self.groups])
        ng = len(self.groups)
        self._n = _lib.int_array([g.n for g in self.groups])
        self._nq = _lib.int_array([g.nq for g in self.groups])
        self._batch = _lib.int_array([len(g.idx) for g in self.groups])
        self._ptrs = [_lib.ptr_array([getattr(g, a)[k].data_ptr() for g in self.groups])
                      for a, k in (("E", 0), ("E", 1), ("W", 0), ("W", 1))]
        self._lam = _lib.ptr_array([g.lam32.data_ptr() for g in self.groups])
        a2 = self.alphas[self.order] ** 2
        self.alpha2 = as_device(a2)
        self.alpha2_32 = as_device(a2, torch.float32)
        self.offsets = np.zeros(len(self.order) + 1, dtype=np.int64)
        self.offsets[1:] = np.cumsum((self.Ns[self.order] - 2) ** 2)
        L = _lib.lib()
        self._ws = torch.empty(L.jfg_helmholtz_grouped_workspace_size(ng, self._n, self._nq,
                                                                       self._batch),
                               dtype=torch.uint8, device="cuda")
        self.cfg = None  # tensor-core launch configuration (autotune())

    def autotune(self, reps: int = 3):
        """Choose the grouped tensor-core launch configuration for this batch's
        fast-diagonalisation passes (jfg_tc_autotune on scratch operands)."""
        L = _lib.lib()
        ng = len(self.groups)
        tot = sum(len(g.idx) * g.nq * g.nq for g in self.groups)
        x = torch.randn(tot, device="cuda")
        y = torch.empty_like(x)
        descs = (_lib.ContractDesc * ng)()
        ins, outs = [], []
        off = 0
        for i, g in enumerate(self.groups):
            B, q = len(g.idx), g.nq
            descs[i] = _lib.ContractDesc(batch=B, nseg=1, M=q, P=q, K=q, op_ld=q, in_ld=q,
                                         in_batch=q * q, out_ld=q, out_batch=q * q,
                                         alpha=1.0, beta=0.0)
            ins.append(x.data_ptr() + 4 * off)
            outs.append(y.data_ptr() + 4 * off)
            off += B * q * q
        best = _lib.TcConfig()
        ms = C.c_float()
        _lib.check(L.jfg_tc_autotune(ng, descs, self._ptrs[0], self._ptrs[1],
                                     _lib.ptr_array(ins), _lib.ptr_array(outs), int(reps),
                                     C.byref(best), C.byref(ms), _lib.stream_handle()),
                   "jfg_tc_autotune")
        self.cfg = best
        return {"operand_a_in_tmem": best.operand_a_in_tmem, "order": best.order,
                "ctas": best.ctas, "stages": best.stages, "mtile": best.mtile or 128,
                "pass_ms": ms.value}

    def pack(self, rhs: list) -> torch.Tensor:
        """Per-problem right-hand sides -> the flat group-major FP64 buffer."""
        return torch.cat([as_device(rhs[i]).reshape(-1) for i in self.order])

    def solve_packed(self, b: torch.Tensor, tol: float = 1e-11, max_refine: int = 8,
                     out: torch.Tensor | None = None):
        """One C-ABI call for the whole batch on packed (group-major) data.
        Returns (x packed, refinements per problem in group-major order)."""
        L = _lib.lib()
        x = torch.empty_like(b) if out is None else out
        nref = (C.c_int * len(self.order))()
        st = L.jfg_helmholtz_solve_grouped(
            FAMILY[self.family], len(self.groups), self._n, self._nq, self._batch,
            *self._ptrs, self._lam, self.alpha2.data_ptr(), self.alpha2_32.data_ptr(),
            b.data_ptr(), x.data_ptr(), float(tol), int(max_refine), nref,
            None if self.cfg is None else C.byref(self.cfg), self._ws.data_ptr(),
            self._ws.numel(), _lib.stream_handle())
        _lib.check(st, "jfg_helmholtz_solve_grouped")
        return x, np.array(nref[:])

    def unpack(self, x: torch.Tensor) -> list:
        out = [None] * len(self.Ns)
        for k, i in enumerate(self.order):
            n = int(self.Ns[i]) - 2
            out[i] = x[self.offsets[k]:self.offsets[k + 1]].view(n, n)
        return out

    def solve(self, rhs: list, tol: float = 1e-11, max_refine: int = 8):
        """rhs: list (one per problem) of (N_b-2, N_b-2) arrays/tensors.
        Returns (solutions list of FP64 device tensors, refinements per problem)."""
        x, nref = self.solve_packed(self.pack(rhs), tol, max_refine)
        refs = np.zeros(len(self.Ns), dtype=int)
        refs[self.order] = nref
        return self.unpack(x), refs

    def solve_per_group(self, rhs: list, tol: float = 1e-11, max_refine: int = 8):
        """The same solves, one C-ABI call per size group (jfg_helmholtz_solve_mixed)."""
        L = _lib.lib()
        out = [None] * len(self.Ns)
        refs = np.zeros(len(self.Ns), dtype=int)
        sh = _lib.stream_handle()
        for g in self.groups:
            Bg = len(g.idx)
            b = torch.stack([as_device(rhs[i]) for i in g.idx]).contiguous()
            x = torch.empty_like(b)
            ws = torch.empty(L.jfg_helmholtz_solve_workspace_size(g.n, g.nq, Bg),
                             dtype=torch.uint8, device=b.device)
            nref = (C.c_int * Bg)()
            st = L.jfg_helmholtz_solve_mixed(
                FAMILY[self.family], g.n, g.nq, Bg, g.E[0].data_ptr(), g.E[1].data_ptr(),
                g.W[0].data_ptr(), g.W[1].data_ptr(), g.lam32.data_ptr(), g.alpha2.data_ptr(),
                g.alpha2_32.data_ptr(), b.data_ptr(), x.data_ptr(), float(tol), int(max_refine),
                nref, ws.data_ptr(), ws.numel(), sh)
            _lib.check(st, "jfg_helmholtz_solve_mixed")
            for k, i in enumerate(g.idx):
                out[i] = x[k]
                refs[i] = nref[k]
        return out, refs


def helmholtz_apply(family: str, N: int, alpha2, u) -> torch.Tensor:
    """v = alpha2 (M (x) M) u + (K (x) M) u + (M (x) K) u (FP64, O(n^2))."""
    L = _lib.lib()
    u = as_device(u)
    batch = u.shape[0]
    n = N - 2
    a2 = as_device(np.broadcast_to(np.asarray(alpha2, dtype=np.float64), (batch,)).copy())
    v = torch.empty_like(u)
    ws = torch.empty(L.jfg_helmholtz_workspace_size(n, batch), dtype=torch.uint8,
                     device=u.device)
    st = L.jfg_helmholtz_apply_f64(FAMILY[family], n, batch, a2.data_ptr(), u.data_ptr(), None,
                                   v.data_ptr(), ws.data_ptr(), ws.numel(), _lib.stream_handle())
    _lib.check(st, "jfg_helmholtz_apply_f64")
    return v
