"""Variable-coefficient operator (kappa grad u, grad v) and batched PCG.

jaxfun assembles ``inner(kappa*Dot(Grad(u), Grad(v)))`` with a non-separable
kappa into a dense 4-index ``TensorMatrix`` A[i,k,j,l] (src/jaxfun/galerkin/
inner.py:445-490, 991-1024; 2-D only, O(n^4) memory) and applies it with
``einsum("ikjl,kl->ij")`` (src/jaxfun/la/tensormatrix.py:54-56).
``VarCoefMatrix`` is the same operator applied matrix-free and
sum-factorised on the GPU in 2-D and 3-D: contract the coefficients to the
gradient on the quadrature grid, multiply by kappa * w (x) w, contract back.
"""

from __future__ import annotations

import numpy as np
import torch

from .. import _lib
from ..device import as_device, workspace
from ..galerkin.tensorproductspace import TensorProductSpace
from .tpmatrix import TPMatrices, TPMatrix, tpmats_lu_factor


def pack_varcoef_ops(ndim: int, B: np.ndarray, D: np.ndarray) -> np.ndarray:
    """Packed operator set for ``jfg_varcoef_apply_*`` (host, FP64)."""
    nq, n = B.shape
    L = _lib.lib()
    out = np.empty(L.jfg_varcoef_ops_count(ndim, n, nq), dtype=np.float64)
    Bc = np.ascontiguousarray(B, dtype=np.float64)
    Dc = np.ascontiguousarray(D, dtype=np.float64)
    L.jfg_varcoef_pack_ops_host(ndim, n, nq, Bc.ctypes.data, Dc.ctypes.data, out.ctypes.data)
    return out


class VarCoefMatrix:
    """A(kappa) for (kappa grad u, grad v) on a square tensor-product space.

    ``kappa`` is the coefficient sampled on the quadrature grid, shape
    ``(*batch, nq, ..., nq)``; ``A @ u`` applies it to coefficient arrays of shape
    ``(*batch, n, ..., n)`` — the ``TensorMatrix.__matmul__`` call surface.
    """

    def __init__(self, T: TensorProductSpace, kappa):
        s0 = T.basespaces[0]
        if any(s != s0 for s in T.basespaces):
            raise ValueError("VarCoefMatrix needs the same 1-D space on every axis")
        self.T = T
        self.ndim = len(T)
        self.n = s0.dim
        self.nq = s0.num_quad_points
        kappa = as_device(kappa)
        if tuple(kappa.shape[kappa.ndim - self.ndim :]) != (self.nq,) * self.ndim:
            raise ValueError("kappa must be sampled on the quadrature grid")
        self.batch_shape = tuple(kappa.shape[: kappa.ndim - self.ndim])
        W = as_device(T.weights())
        self._finish(kappa, (kappa * W).contiguous())

    def _finish(self, kappa, kw):
        s0 = self.T.basespaces[0]
        self.kappa = kappa
        self.kw = kw
        B = s0.backward_matrix(None, 0)
        D = s0.backward_matrix(None, 1)
        self.ops_host = pack_varcoef_ops(self.ndim, B, D)
        self.ops = as_device(self.ops_host)
        self.kappa_mean = kappa.reshape(kappa.shape[: kappa.ndim - self.ndim] + (-1,)).mean(-1)

    @classmethod
    def from_log(cls, T: TensorProductSpace, g, standardize: bool = False) -> "VarCoefMatrix":
        """A(kappa) for kappa = exp(g), g sampled on the quadrature grid
        (``(*batch, nq, ..., nq)``); with ``standardize`` every problem's g is
        first shifted and scaled to mean 0 and standard deviation 1.  The
        exponential and the quadrature weighting kappa w (x) w run as one
        kernel (``jfg_exp_weighted_field_f64``), the moments as another
        (``jfg_field_moments_f64``): ``evaluate_jaxfunction_expr_quad`` for
        exp(g) (src/jaxfun/galerkin/arguments.py:928-990) without a pass over
        kappa of its own."""
        obj = cls.__new__(cls)
        s0 = T.basespaces[0]
        if any(s != s0 for s in T.basespaces):
            raise ValueError("VarCoefMatrix needs the same 1-D space on every axis")
        obj.T = T
        obj.ndim = nd = len(T)
        obj.n = s0.dim
        obj.nq = nq = s0.num_quad_points
        g = as_device(g).contiguous()
        if tuple(g.shape[g.ndim - nd :]) != (nq,) * nd:
            raise ValueError("g must be sampled on the quadrature grid")
        obj.batch_shape = tuple(g.shape[: g.ndim - nd])
        batch = obj.batch
        L = _lib.lib()
        st = _lib.stream_handle()
        w = as_device(s0.quad_points_and_weights()[1])
        kappa = torch.empty_like(g)
        kw = torch.empty_like(g)
        scale = shift = None
        if standardize:
            shift = torch.empty(batch, dtype=torch.float64, device=g.device)
            scale = torch.empty(batch, dtype=torch.float64, device=g.device)
            _lib.check(L.jfg_field_moments_f64(nd, nq, batch, g.data_ptr(), shift.data_ptr(),
                                               scale.data_ptr(), st), "field_moments")
        _lib.check(L.jfg_exp_weighted_field_f64(
            nd, nq, batch, g.data_ptr(), None if scale is None else scale.data_ptr(),
            None if shift is None else shift.data_ptr(), w.data_ptr(), kappa.data_ptr(),
            kw.data_ptr(), None, st), "exp_weighted_field")
        obj._finish(kappa, kw)
        return obj

    @classmethod
    def from_expansion(cls, T: TensorProductSpace, g_coef, standardize: bool = False
                       ) -> "VarCoefMatrix":
        """A(exp(g)) for g given by its orthogonal-basis coefficients (a
        JAXFunction's coefficients, ``(*batch, N, ..., N)``): the backward
        transform to the quadrature grid with exp and the quadrature weighting
        in the epilogue of its last pass (``jfg_exp_weighted_backward_f64``;
        with ``standardize`` that pass records per-tile moments instead and
        one more pass applies exp and the weights)."""
        obj = cls.__new__(cls)
        s0 = T.basespaces[0]
        if any(s != s0 for s in T.basespaces):
            raise ValueError("VarCoefMatrix needs the same 1-D space on every axis")
        obj.T = T
        obj.ndim = nd = len(T)
        obj.n = s0.dim
        obj.nq = nq = s0.num_quad_points
        To = T.get_orthogonal()
        o0 = To.basespaces[0]
        no = o0.dim
        g_coef = as_device(g_coef).contiguous()
        if tuple(g_coef.shape[g_coef.ndim - nd:]) != (no,) * nd:
            raise ValueError(f"g_coef must end in {(no,) * nd}")
        obj.batch_shape = tuple(g_coef.shape[: g_coef.ndim - nd])
        batch = obj.batch
        V = as_device(np.ascontiguousarray(o0.backward_matrix(nq)))
        if tuple(V.shape) != (nq, no):
            raise ValueError("the orthogonal space's backward matrix is not (nq, N)")
        w = as_device(np.array(s0.quad_points_and_weights()[1]))
        shp = obj.batch_shape + (nq,) * nd
        kappa = torch.empty(shp, dtype=torch.float64, device=g_coef.device)
        kw = torch.empty_like(kappa)
        L = _lib.lib()
        ws = workspace(L.jfg_exp_weighted_backward_workspace_size(nd, no, nq, batch))
        _lib.check(L.jfg_exp_weighted_backward_f64(
            nd, no, nq, batch, V.data_ptr(), g_coef.data_ptr(), 1 if standardize else 0,
            w.data_ptr(), kappa.data_ptr(), kw.data_ptr(), None, ws.data_ptr(), ws.numel(),
            _lib.stream_handle()), "exp_weighted_backward")
        obj._finish(kappa, kw)
        return obj

    @property
    def batch(self) -> int:
        return int(np.prod(self.batch_shape)) if self.batch_shape else 1

    def __matmul__(self, u) -> torch.Tensor:
        u = as_device(u)
        shp = self.batch_shape + (self.n,) * self.ndim
        if tuple(u.shape) != shp:
            raise ValueError(f"u shape {tuple(u.shape)} != {shp}")
        v = torch.empty_like(u)
        L = _lib.lib()
        ws = workspace(L.jfg_varcoef_workspace_size(self.ndim, self.n, self.nq, self.batch, 8))
        st = L.jfg_varcoef_apply_f64(self.ndim, self.n, self.nq, self.batch, self.ops.data_ptr(),
                                     self.kw.data_ptr(), u.data_ptr(), v.data_ptr(),
                                     ws.data_ptr(), ws.numel(), _lib.stream_handle())
        _lib.check(st, "jfg_varcoef_apply_f64")
        return v

    __call__ = __matmul__


def stiffness_mass(T: TensorProductSpace):
    """(K, M) of the first axis' space: K = (grad-like) stiffness, M = mass."""
    s = T.basespaces[0]
    return s.stiffness_matrix(), s.mass_matrix()


def poisson_tpmatrices(T: TensorProductSpace, alpha2: float = 0.0) -> TPMatrices:
    """alpha^2 M (x) M + K (x) M + M (x) K (+ 3-D analogue): the TPMatrices that
    ``inner(alpha**2*u*v - v*Div(Grad(u)))`` yields (inner.py:520-562, 749-763)."""
    K, M = stiffness_mass(T)
    nd = len(T)
    terms = []
    if alpha2 != 0.0:
        terms.append(TPMatrix([M] * nd, alpha2))
    for ax in range(nd):
        mats = [M] * nd
        mats[ax] = K
        terms.append(TPMatrix(mats, 1.0))
    return TPMatrices(terms)


def helmholtz_system(T: TensorProductSpace, f, alpha2: float = 0.0):
    """(A, b) of alpha^2 u - div grad u = f on T, Dirichlet data included:
    what ``inner(alpha**2*u*v - v*Div(Grad(u)) - v*f, kind="system")`` returns
    (inner.py:520-562, 809-984).  For a DirectSumTPS the trial function is
    u = u_h + lift; the lift's part of the bilinear form moves to the
    right-hand side, b = (f, v) - a(lift, v), so ``A.solve(b)`` gives the
    homogeneous coefficients and ``T.backward`` adds the lift back.

    A is built per axis (unequal sizes allowed; the fast solver needs equal
    axes).  ``f`` is sampled on the quadrature grid (leading batch axes
    allowed); b is one affine contraction on the GPU: the scalar product of f
    with the boundary term (a_bc is fixed, computed once in FP64) added in the
    last pass's epilogue."""
    from ..galerkin.tensorproductspace import DirectSumTPS, tp_apply_affine

    H = T.get_homogeneous().basespaces
    nd = len(H)
    K = [s.stiffness_matrix() for s in H]
    M = [s.mass_matrix() for s in H]
    terms = []
    if alpha2 != 0.0:
        terms.append(TPMatrix(M, alpha2))
    for ax in range(nd):
        mats = list(M)
        mats[ax] = K[ax]
        terms.append(TPMatrix(mats, 1.0))
    A = TPMatrices(terms)
    if not isinstance(T, DirectSumTPS):
        return A, T.scalar_product(f)
    mats, shift = helmholtz_lifting(T, alpha2)
    return A, tp_apply_affine(mats, f, shift)


def helmholtz_lifting(T, alpha2: float = 0.0):
    """(scalar-product matrices, -a(lift, v)) of a DirectSumTPS: the boundary
    lift's part of alpha^2 (u, v) + (grad u, grad v) with the homogeneous test
    functions, FP64 host setup cached on T (the lift is fixed by the data)."""
    from ..galerkin.tensorproductspace import kron_apply_host

    key = ("rhs", float(alpha2))
    cached = T._maps.get(key)
    if cached is not None:
        return cached
    H = T.get_homogeneous().basespaces
    nd = len(H)
    KM = [s.test_orthogonal_matrices() for s in H]
    Kr = [km[0] for km in KM]
    Mr = [km[1] for km in KM]
    bc = np.zeros(tuple(s.dim for s in H))
    if alpha2 != 0.0:
        bc += alpha2 * kron_apply_host(Mr, T.lift)
    for ax in range(nd):
        mats = list(Mr)
        mats[ax] = Kr[ax]
        bc += kron_apply_host(mats, T.lift)
    nf = tuple(s.num_quad_points for s in H)
    sp_mats = [np.ascontiguousarray(s.scalar_product_matrix(nf[i])) for i, s in enumerate(H)]
    shift = np.ascontiguousarray(-bc)
    shift.setflags(write=False)
    cached = (sp_mats, shift)
    T._maps[key] = cached
    return cached


def fd_preconditioner(T: TensorProductSpace):
    """Constant-coefficient (kappa = 1) fast-diagonalisation factors."""
    return tpmats_lu_factor(poisson_tpmatrices(T).tpmats)


def pcg(A: VarCoefMatrix, b, M=None, x0=None, tol: float = 1e-10, maxiter: int = 2000,
        scale=None):
    """Batched FP64 PCG on the GPU: one C-ABI call (``jfg_pcg_varcoef_f64``).

    Returns (x, iters) with per-problem iteration counts.  Each problem stops
    when sqrt(r.z / r0.z0) <= tol.  ``M`` are fast-diagonalisation factors
    (default: the constant-kappa Poisson factors); ``scale`` the per-problem
    preconditioner constant (default mean kappa; PCG is invariant to it).
    """
    if M is None:
        M = fd_preconditioner(A.T)
    b = as_device(b)
    x = torch.zeros_like(b) if x0 is None else as_device(x0).clone()
    E, W, lam = M.device_factors()
    sc = A.kappa_mean.reshape(-1) if scale is None else as_device(scale).reshape(-1)
    sc = sc.contiguous()
    L = _lib.lib()
    ws = workspace(L.jfg_pcg_workspace_size(A.ndim, A.n, A.nq, A.batch, 8))
    iters = (_lib.C.c_int * A.batch)()
    st = L.jfg_pcg_varcoef_f64(A.ndim, A.n, A.nq, A.batch, A.ops.data_ptr(), A.kw.data_ptr(),
                               E.data_ptr(), W.data_ptr(), lam.data_ptr(), sc.data_ptr(),
                               b.data_ptr(), x.data_ptr(), 0 if x0 is None else 1, float(tol),
                               int(maxiter), iters, ws.data_ptr(), ws.numel(),
                               _lib.stream_handle())
    _lib.check(st, "jfg_pcg_varcoef_f64")
    return x, np.array(iters[:], dtype=np.int64)
