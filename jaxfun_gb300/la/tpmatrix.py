"""Kronecker-structured operators and the fast-diagonalisation solver.

Mirrors ``TPMatrix``, ``TPMatrices``, ``tpmats_lu_factor`` and
``TPMatricesLUFactors`` of src/jaxfun/la/tpmatrix.py (46-589, 1089-1233).  The
per-axis generalized eigendecomposition is one-time FP64 host setup (the
reference also calls scipy.linalg.eigh on the host); every solve runs on the
GPU as 2d per-axis contractions with the pointwise divide fused into the
epilogue of the d-th pass (``jfg_fd_solve_f64``).

Difference from the reference: for a non-symmetric stiffness (Chebyshev
Galerkin, K = -(phi_j'', phi_i)_w is upper triangular) the reference's
``eigh(A0, A1)`` reads only one triangle and returns a wrong factorisation.
Here a general eigendecomposition M^{-1} K = W Lambda W^{-1} is used and the
forward factor is E = W^{-1} M^{-1}; for symmetric pairs E = W^T exactly as in
the reference.
"""

from __future__ import annotations

import numpy as np
import scipy.linalg
import torch

from .. import _lib
from ..device import as_device, workspace
from ..galerkin.tensorproductspace import device_op, tp_apply


class SolverNotApplicable(Exception):
    """The factor structure does not admit the fast solver (src/jaxfun/la/matrixprotocol.py:30)."""


class TPMatrix:
    """coefficient * (mats[0] (x) mats[1] (x) ...), per-axis dense factors (test rows)."""

    def __init__(self, mats, coefficient: float = 1.0):
        self.mats = [np.asarray(m, dtype=np.float64) for m in mats]
        self.coefficient = float(coefficient)

    @property
    def dims(self) -> int:
        return len(self.mats)

    @property
    def shape(self):
        return tuple(m.shape[0] for m in self.mats)

    def __matmul__(self, u) -> torch.Tensor:
        out = tp_apply(self.mats, u)
        if self.coefficient != 1.0:
            out = out * self.coefficient
        return out

    def todense(self) -> np.ndarray:
        K = self.mats[0]
        for m in self.mats[1:]:
            K = np.kron(K, m)
        return self.coefficient * K


class TPMatrices:
    """Sum of TPMatrix terms (src/jaxfun/la/tpmatrix.py:296-509)."""

    def __init__(self, tpmats):
        self.tpmats = list(tpmats)
        self._lu_cache = None
        self._kron_cache = None

    def __matmul__(self, u) -> torch.Tensor:
        out = None
        for tp in self.tpmats:
            v = tp @ u
            out = v if out is None else out + v
        return out

    def todense(self) -> np.ndarray:
        return sum(tp.todense() for tp in self.tpmats)

    def lu_factor(self) -> "TPMatricesLUFactors":
        if self._lu_cache is None:
            self._lu_cache = tpmats_lu_factor(self.tpmats)
        return self._lu_cache

    def solve(self, rhs, *, method: str = "auto", kron_method: str = "auto",
              auto_threshold: int = 100) -> torch.Tensor:
        """Solve A x = rhs (leading batch axes allowed).

        method "lu": fast diagonalisation on the GPU (raises SolverNotApplicable if
        the structure does not allow it); "kron": dense Kronecker LU (small
        problems only, cuSOLVER through torch.linalg); "auto": lu, else kron —
        the dispatch of TPMatrices.solve (tpmatrix.py:429-509).  ``kron_method``
        ("auto", "banded", "rcm", "dense") and ``auto_threshold`` keep the
        reference's signature; they choose among the reference's sparse
        Kronecker solvers, whereas the Kronecker path here is always the dense
        LU, so they are validated and otherwise have no effect.
        """
        if kron_method not in ("auto", "banded", "rcm", "dense"):
            raise ValueError(f"unknown kron_method {kron_method!r}")
        if int(auto_threshold) < 0:
            raise ValueError("auto_threshold must be non-negative")
        if method in ("auto", "lu"):
            try:
                return self.lu_factor().solve(rhs)
            except SolverNotApplicable:
                if method == "lu":
                    raise
        if method not in ("auto", "kron"):
            raise ValueError(f"unknown method {method!r}")
        return self._kron_solve(rhs)

    def _kron_solve(self, rhs) -> torch.Tensor:
        if self._kron_cache is None:
            self._kron_cache = as_device(self.todense())
        A = self._kron_cache
        rhs = as_device(rhs)
        shp = self.tpmats[0].shape
        nd = len(shp)
        flat = rhs.reshape(-1, int(np.prod(shp))).T
        sol = torch.linalg.solve(A, flat)
        return sol.T.reshape(rhs.shape[: rhs.ndim - nd] + shp)


def _same(a: np.ndarray, b: np.ndarray) -> bool:
    return a.shape == b.shape and np.allclose(a, b, rtol=1e-5, atol=1e-8)


class TPMatricesLUFactors:
    """Fast-diagonalisation factors: per axis E (forward), W (backward), lam, and
    a sum-separable denominator D = c0 + c1 * sum_axes lam[i_axis]."""

    def __init__(self, E: np.ndarray, W: np.ndarray, lam: np.ndarray, c0: float, c1: float,
                 ndim: int):
        self.E_host, self.W_host, self.lam_host = E, W, lam
        self.c0, self.c1 = float(c0), float(c1)
        self.ndim = ndim
        self.n = E.shape[0]
        self._dev = {}

    def device_factors(self, dtype=torch.float64):
        t = self._dev.get(dtype)
        if t is None:
            t = (device_op(self.E_host, dtype), device_op(self.W_host, dtype),
                 as_device(self.lam_host, dtype))
            self._dev[dtype] = t
        return t

    def solve(self, rhs, c0=None, c1=None) -> torch.Tensor:
        """U = (x W) [(x E) F / (c0 + c1 * sum lam)] for every leading-batch slice.
        ``c0``/``c1`` may be per-batch arrays (default: the factored scalars)."""
        rhs = as_device(rhs)
        nd, n = self.ndim, self.n
        if tuple(rhs.shape[rhs.ndim - nd :]) != (n,) * nd:
            raise ValueError(f"rhs trailing shape {tuple(rhs.shape)} != {(n,) * nd}")
        lead = rhs.shape[: rhs.ndim - nd]
        batch = int(np.prod(lead)) if lead else 1
        out = torch.empty_like(rhs)
        if batch == 0:
            return out
        E, W, lam = self.device_factors()
        c0 = self.c0 if c0 is None else c0
        c1 = self.c1 if c1 is None else c1
        c0_t = as_device(np.broadcast_to(np.asarray(c0, dtype=np.float64), (batch,)).copy())
        c1_t = as_device(np.broadcast_to(np.asarray(c1, dtype=np.float64), (batch,)).copy())
        L = _lib.lib()
        ws = workspace(L.jfg_fd_solve_workspace_size(nd, n, batch, 8))
        st = L.jfg_fd_solve_f64(nd, n, batch, E.data_ptr(), W.data_ptr(), lam.data_ptr(),
                                c0_t.data_ptr(), c1_t.data_ptr(), rhs.data_ptr(), out.data_ptr(),
                                ws.data_ptr(), ws.numel(), _lib.stream_handle())
        _lib.check(st, "jfg_fd_solve_f64")
        return out


def fd_eig(K: np.ndarray, M: np.ndarray):
    """Return (lam, W, E) with K W = M W diag(lam) and E = W^{-1} M^{-1}.

    Symmetric K: scipy.linalg.eigh(K, M) (tpmatrix.py:1184), E = W^T.
    Non-symmetric K: general eig of M^{-1} K (real spectrum for the
    Chebyshev Dirichlet Laplacian), E = W^{-1} M^{-1}.
    """
    if np.allclose(K, K.T, rtol=1e-13, atol=1e-13 * np.abs(K).max()):
        lam, W = scipy.linalg.eigh(K, M)
        return lam, W, W.T.copy()
    lam, W = scipy.linalg.eig(np.linalg.solve(M, K))
    if np.max(np.abs(lam.imag)) > 1e-8 * np.max(np.abs(lam.real)):
        raise SolverNotApplicable("complex spectrum: not simultaneously diagonalisable in R")
    order = np.argsort(lam.real)
    lam = lam.real[order].copy()
    W = W.real[:, order].copy()
    E = np.linalg.solve(W, np.linalg.inv(M))
    return lam, W, E


def tpmats_lu_factor(A) -> TPMatricesLUFactors:
    """Diagonalisation factors for sum_k s_k (A_k0 (x) A_k1 (x) ...)
    (src/jaxfun/la/tpmatrix.py:1089-1233).

    Supported structure (the Helmholtz/Poisson family): every axis carries the
    same pair {K, M} of distinct matrices, and each term has K on at most one
    axis, with equal coefficients for the K-terms.  Raises SolverNotApplicable
    otherwise.
    """
    if isinstance(A, TPMatrix):
        A = [A]
    tpmats = list(A)
    nd = tpmats[0].dims
    distinct: list[np.ndarray] = []

    def rep(m):
        for i, r in enumerate(distinct):
            if _same(m, r):
                return i
        distinct.append(m)
        return len(distinct) - 1

    ids = [[rep(m) for m in tp.mats] for tp in tpmats]
    if len(distinct) > 2:
        raise SolverNotApplicable(f"{len(distinct)} distinct factor matrices (at most 2)")
    if len(distinct) == 1:
        raise SolverNotApplicable("single distinct factor: use a Kronecker solve")
    # identify the mass-like factor M (symmetric positive definite; the factor
    # that occurs most often, e.g. the alpha^2 M (x) M term of Helmholtz)
    counts = [sum(row.count(i) for row in ids) for i in (0, 1)]
    m_id = None
    norms = [float(np.linalg.norm(d)) for d in distinct]
    for cand in sorted((0, 1), key=lambda i: (-counts[i], norms[i])):
        X = distinct[cand]
        if np.allclose(X, X.T):
            try:
                np.linalg.cholesky(X)
                m_id = cand
                break
            except np.linalg.LinAlgError:
                continue
    if m_id is None:
        raise SolverNotApplicable("no symmetric positive definite factor")
    k_id = 1 - m_id
    c0 = 0.0
    c1 = None
    for s, row in zip([tp.coefficient for tp in tpmats], ids, strict=True):
        nk = sum(1 for i in row if i == k_id)
        if nk == 0:
            c0 += s
        elif nk == 1:
            if c1 is None:
                c1 = s
            elif not np.isclose(c1, s):
                raise SolverNotApplicable("unequal stiffness coefficients per axis")
        else:
            raise SolverNotApplicable("product of stiffness factors in one term")
    # every axis must see each K-term exactly once
    k_axes = sorted(row.index(k_id) for row in ids if k_id in row)
    if k_axes != list(range(nd)):
        raise SolverNotApplicable("stiffness factor missing on an axis")
    lam, W, E = fd_eig(distinct[k_id], distinct[m_id])
    return TPMatricesLUFactors(E, W, lam, c0, 1.0 if c1 is None else c1, nd)
