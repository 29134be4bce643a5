"""Batched 2-D Dirichlet Helmholtz solves with uneven N (alpha^2 u - lap u = f).

Each problem b has its own N_b and alpha_b; problems are grouped by size and
each group is one C-ABI call (``jfg_helmholtz_solve_mixed``): fast-
diagonalisation corrections on the tensor cores (split-TF32, padded layout)
inside FP64 iterative refinement whose residual r = b - A x is applied in
O(n^2) from the closed-form mass and stiffness matrices.  The FD factors are
those of ``tpmats_lu_factor`` for alpha^2 M (x) M + K (x) M + M (x) K
(src/jaxfun/la/tpmatrix.py:1089-1233), with the general eigendecomposition for
the non-symmetric Chebyshev stiffness.
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

    def solve(self, rhs: list, tol: float = 1e-11, max_refine: int = 8):
        """rhs: list (one per problem) of (N_b-2, N_b-2) arrays/tensors.
        Returns (solutions list of FP64 device tensors, refinements per problem)."""
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
