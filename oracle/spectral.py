"""FP64 CPU restatement of jaxfun's spectral hot path (TEST INFRASTRUCTURE ONLY).

Every function cites the reference file:line it restates (paths relative to
the jaxfun project root).  The algorithms deliberately follow the reference,
not the GPU product: per-point recurrences for Legendre, DCTs for Chebyshev,
banded mass solves for composite forward transforms, dense ``einsum`` for the
non-separable ``TensorMatrix``.  Only tests, the smoke check and the CPU
baseline legs of ``bench.py`` use this module.
"""

from __future__ import annotations

import numpy as np
import scipy.fft
import scipy.linalg

# ---------------------------------------------------------------------------
# Quadrature
# ---------------------------------------------------------------------------


def legendre_gauss(N: int) -> tuple[np.ndarray, np.ndarray]:
    """Gauss-Legendre nodes (ascending) and weights.

    Restates ``Legendre.quad_points_and_weights`` (src/jaxfun/galerkin/
    Legendre.py:125-137) which calls ``fastgl.leggauss`` (src/jaxfun/utils/
    fastgl.py:547-567, tabulated for n<=100 and Bogaert asymptotics beyond).
    Both are the unique N-point Gauss rule; here it is obtained from
    numpy's Golub-Welsch rule polished by Newton steps on the three-term
    recurrence, which agrees with the tabulated/asymptotic values to rounding.
    """
    x, _ = np.polynomial.legendre.leggauss(N)
    for _ in range(3):
        p0 = np.ones_like(x)
        p1 = x.copy()
        for k in range(2, N + 1):
            p0, p1 = p1, ((2 * k - 1) * x * p1 - (k - 1) * p0) / k
        # p1 = P_N, p0 = P_{N-1};  P_N' = N (x P_N - P_{N-1}) / (x^2 - 1)
        dp = N * (x * p1 - p0) / (x * x - 1.0)
        x = x - p1 / dp
    p0 = np.ones_like(x)
    p1 = x.copy()
    for k in range(2, N + 1):
        p0, p1 = p1, ((2 * k - 1) * x * p1 - (k - 1) * p0) / k
    dp = N * (x * p1 - p0) / (x * x - 1.0)
    w = 2.0 / ((1.0 - x * x) * dp * dp)
    return x, w


def chebyshev_gauss(N: int) -> tuple[np.ndarray, np.ndarray]:
    """Gauss-Chebyshev nodes x_k = cos(pi + (2k+1)pi/(2N)) (ascending), w = pi/N.

    Restates src/jaxfun/galerkin/Chebyshev.py:149-170.
    """
    k = np.arange(N)
    return np.cos(np.pi + (2 * k + 1) * np.pi / (2 * N)), np.full(N, np.pi / N)


# ---------------------------------------------------------------------------
# Basis evaluation (Vandermonde and derivatives)
# ---------------------------------------------------------------------------


def legendre_vandermonde(x: np.ndarray, N: int, k: int = 0) -> np.ndarray:
    """V[q, n] = d^k/dx^k P_n(x_q), n < N.

    k=0 restates the three-term recurrence of ``Legendre.eval_basis_functions``
    (src/jaxfun/galerkin/Legendre.py:162-183).  Derivatives
    (``evaluate_basis_derivative``, src/jaxfun/galerkin/orthogonal.py:168-178,
    nested ``jacfwd``) use the exact identity
    P^{(k)}_{n+1} = P^{(k)}_{n-1} + (2n+1) P^{(k-1)}_n.
    """
    x = np.asarray(x, dtype=np.float64)
    V = np.zeros((x.size, N))
    V[:, 0] = 1.0
    if N > 1:
        V[:, 1] = x
    for n in range(1, N - 1):
        V[:, n + 1] = ((2 * n + 1) * x * V[:, n] - n * V[:, n - 1]) / (n + 1)
    for _ in range(k):
        D = np.zeros_like(V)
        if N > 1:
            D[:, 1] = V[:, 0]
        for n in range(1, N - 1):
            D[:, n + 1] = D[:, n - 1] + (2 * n + 1) * V[:, n]
        V = D
    return V


def chebyshev_vandermonde(x: np.ndarray, N: int, k: int = 0) -> np.ndarray:
    """V[q, n] = d^k/dx^k T_n(x_q).

    k=0 restates ``Chebyshev.eval_basis_functions`` (src/jaxfun/galerkin/
    Chebyshev.py:199-223, T_{n+1} = 2x T_n - T_{n-1}); derivatives use
    T^{(k)}_{n+1} = 2k T^{(k-1)}_n + 2x T^{(k)}_n - T^{(k)}_{n-1}.
    """
    x = np.asarray(x, dtype=np.float64)
    V = np.zeros((x.size, N))
    V[:, 0] = 1.0
    if N > 1:
        V[:, 1] = x
    for n in range(1, N - 1):
        V[:, n + 1] = 2 * x * V[:, n] - V[:, n - 1]
    for kk in range(1, k + 1):
        D = np.zeros_like(V)
        if N > 1:
            D[:, 1] = V[:, 0] if kk == 1 else 0.0
        for n in range(1, N - 1):
            D[:, n + 1] = 2 * kk * V[:, n] + 2 * x * D[:, n] - D[:, n - 1]
        V = D
    return V


# ---------------------------------------------------------------------------
# 1-D spaces (orthogonal and Dirichlet composite)
# ---------------------------------------------------------------------------


class Space1D:
    """A 1-D Legendre or Chebyshev space, optionally with homogeneous Dirichlet BCs.

    Dirichlet composites use the stencil phi_k = P_k - P_{k+2} (LDRD, restating
    ``get_stencil_matrix`` src/jaxfun/galerkin/composite.py:786-789), so the
    space dimension is N-2 and there are N quadrature points
    (``Composite``, src/jaxfun/galerkin/composite.py:153-187).
    """

    def __init__(self, family: str, N: int, dirichlet: bool = False):
        assert family in ("legendre", "chebyshev")
        self.family = family
        self.N = N
        self.dirichlet = dirichlet
        self.dim = N - 2 if dirichlet else N
        if family == "legendre":
            self.h = 2.0 / (2.0 * np.arange(N) + 1.0)
        else:
            self.h = np.full(N, np.pi / 2)
            self.h[0] = np.pi

    # stencil S (dim x N): S[k,k] = 1, S[k,k+2] = -1
    @property
    def S(self) -> np.ndarray:
        if not self.dirichlet:
            return np.eye(self.N)
        S = np.zeros((self.N - 2, self.N))
        k = np.arange(self.N - 2)
        S[k, k] = 1.0
        S[k, k + 2] = -1.0
        return S

    def quad(self, Nq: int | None = None):
        Nq = self.N if Nq is None else Nq
        if self.family == "legendre":
            return legendre_gauss(Nq)
        return chebyshev_gauss(Nq)

    def vandermonde_orth(self, x, k=0):
        if self.family == "legendre":
            return legendre_vandermonde(x, self.N, k)
        return chebyshev_vandermonde(x, self.N, k)

    # -- transforms along axis 0 of a (possibly batched) array ---------------

    def to_orthogonal(self, c):
        """composite.py:276-279: a = c @ S (along axis 0 here)."""
        return np.tensordot(self.S.T, c, axes=(1, 0))

    def backward(self, c, Nq=None):
        """Composite.backward (composite.py:205-208) -> orthogonal backward.

        Legendre: OrthogonalSpace.backward/evaluate (orthogonal.py:102-129,
        214-227); Chebyshev: idct (Chebyshev.py:225-241).
        """
        a = self.to_orthogonal(c)
        Nq = self.N if Nq is None else Nq
        if self.family == "legendre":
            x, _ = self.quad(Nq)
            V = legendre_vandermonde(x, self.N)
            return np.tensordot(V, a, axes=(1, 0))
        n = Nq
        if n > a.shape[0]:
            pad = [(0, n - a.shape[0])] + [(0, 0)] * (a.ndim - 1)
            a = np.pad(a, pad)
        sign = ((-1.0) ** np.arange(n)).reshape((n,) + (1,) * (a.ndim - 1))
        uh = a * sign
        return 0.5 * uh[0:1] + n * scipy.fft.idct(uh, type=2, n=n, axis=0)

    def scalar_product_orth(self, u):
        """Legendre: (u*w) @ V (orthogonal.py:264-277); Chebyshev: dct (Chebyshev.py:262-279)."""
        n = u.shape[0]
        if self.family == "legendre":
            x, w = self.quad(n)
            V = legendre_vandermonde(x, self.N)
            return np.tensordot(V.T * w[None, :], u, axes=(1, 0))
        sign = ((-1.0) ** np.arange(n)).reshape((n,) + (1,) * (u.ndim - 1))
        uh = scipy.fft.dct(u, type=2, n=n, axis=0)
        uh = uh * np.pi * sign / n / 2
        return uh[: self.N]

    def scalar_product(self, u):
        """Composite.scalar_product = S @ orthogonal scalar product (composite.py:345-349)."""
        return np.tensordot(self.S, self.scalar_product_orth(u), axes=(1, 0))

    def mass_matrix(self) -> np.ndarray:
        """S diag(h) S^T (composite.py:330-333; orthogonal mass orthogonal.py:248-254)."""
        S = self.S
        return S @ np.diag(self.h) @ S.T

    def forward(self, u):
        """Composite.forward = banded mass solve of the scalar product (composite.py:339-343,
        DiaMatrix LU diamatrix.py:1881-1925); orthogonal forward = b / h (orthogonal.py:256-262)
        or the scaled DCT (Chebyshev.py:243-260)."""
        if not self.dirichlet:
            if self.family == "chebyshev":
                n = u.shape[0]
                sign = ((-1.0) ** np.arange(n)).reshape((n,) + (1,) * (u.ndim - 1))
                uh = scipy.fft.dct(u, type=2, n=n, axis=0)
                uh[0] = uh[0] / 2
                uh = uh * sign / n
                return uh[: self.N]
            b = self.scalar_product_orth(u)
            return b / self.h.reshape((-1,) + (1,) * (u.ndim - 1))
        b = self.scalar_product(u)
        # pentadiagonal (offsets -2, 0, 2) banded solve
        M = self.mass_matrix()
        n = M.shape[0]
        ab = np.zeros((5, n))
        for off in (-2, 0, 2):
            d = np.diagonal(M, off)
            if off >= 0:
                ab[2 - off, off:] = d
            else:
                ab[2 - off, : n + off] = d
        shp = b.shape
        x = scipy.linalg.solve_banded((2, 2), ab, b.reshape(n, -1))
        return x.reshape(shp)

    # -- Galerkin matrices (test rows, trial cols) ----------------------------

    def stiffness_matrix(self) -> np.ndarray:
        """K = (phi_j', phi_i') = -(phi_j'', phi_i)_w (test i, trial j).

        Legendre Dirichlet: diag(4k+6) (``LGComposite._matrices`` (1,1)/(0,2),
        src/jaxfun/galerkin/Legendre.py:439-443, 489-493).  Chebyshev: minus
        S D2 S^T with D2 the dense (T_i, T_j'')_w of
        src/jaxfun/galerkin/Chebyshev.py:21-35 (mask cols-rows>=2, even).
        """
        assert self.dirichlet
        n = self.N - 2
        if self.family == "legendre":
            return np.diag(4.0 * np.arange(n) + 6.0)
        rows = np.arange(self.N)[:, None]
        cols = np.arange(self.N)[None, :]
        off = cols - rows
        mask = (off >= 2) & ((off - 2) % 2 == 0)
        D2 = np.where(mask, cols * (cols**2 - rows**2) * np.pi / 2, 0.0)
        S = self.S
        return -(S @ D2 @ S.T)

    def matrices_quadrature(self, i: int, j: int, Nq: int | None = None) -> np.ndarray:
        """Quadrature fallback of ``inner_bilinear`` (src/jaxfun/galerkin/inner.py:887-909):
        z = S (Pi^T diag(w) Pj) S^T, i/j the test/trial derivative orders."""
        x, w = self.quad(Nq)
        Pi = self.vandermonde_orth(x, i)
        Pj = self.vandermonde_orth(x, j)
        z = (Pi.T * w[None, :]) @ Pj
        return self.S @ z @ self.S.T


# ---------------------------------------------------------------------------
# Tensor-product transforms (tensorproductspace.py:330-417)
# ---------------------------------------------------------------------------


def _along(axis, fn, a):
    b = np.moveaxis(a, axis, 0)
    return np.moveaxis(fn(b), 0, axis)


def tp_backward(spaces, c, Nq=None):
    """TensorProductSpace.backward: 1-D backward along each axis in turn (tensorproductspace.py:330-365)."""
    for ax, V in enumerate(spaces):
        c = _along(ax, lambda b, V=V, ax=ax: V.backward(b, None if Nq is None else Nq[ax]), c)
    return c


def tp_forward(spaces, u):
    """TensorProductSpace.forward (tensorproductspace.py:395-417)."""
    for ax, V in enumerate(spaces):
        u = _along(ax, V.forward, u)
    return u


def tp_scalar_product(spaces, u):
    """TensorProductSpace.scalar_product (tensorproductspace.py:367-393)."""
    for ax, V in enumerate(spaces):
        u = _along(ax, V.scalar_product, u)
    return u


# ---------------------------------------------------------------------------
# Separable operators and solvers (src/jaxfun/la/tpmatrix.py)
# ---------------------------------------------------------------------------


def tp_apply(terms, U):
    """sum_k s_k (A_k0 (x) A_k1 (x) ...) U, per-axis matvec (tpmatrix.py:152-156, 287-289)."""
    out = np.zeros_like(U)
    for s, mats in terms:
        Z = U
        for ax, A in enumerate(mats):
            Z = np.moveaxis(np.tensordot(A, Z, axes=(1, ax)), 0, ax)
        out = out + s * Z
    return out


def kron_solve(terms, rhs):
    """Dense Kronecker assembly + LU (tpmats_to_kron / tpmats_dense_lu_factor,
    tpmatrix.py:1052-1086, 1357-1402).  Small N only."""
    A = None
    for s, mats in terms:
        K = mats[0]
        for M in mats[1:]:
            K = np.kron(K, M)
        A = s * K if A is None else A + s * K
    return np.linalg.solve(A, rhs.ravel()).reshape(rhs.shape)


def fd_factor_symmetric(K, M):
    """Per-axis generalized symmetric eigenproblem K W = M W Lambda, W^T M W = I
    (scipy.linalg.eigh(A0, A1), tpmats_lu_factor, tpmatrix.py:1171-1204)."""
    lam, W = scipy.linalg.eigh(K, M)
    return lam, W


def fd_factor_general(K, M):
    """General eigendecomposition M^{-1}K = W Lambda W^{-1} for non-symmetric K
    (Chebyshev).  The reference's eigh on a non-symmetric K is inexact; the
    correct answer is pinned against ``kron_solve``."""
    lam, W = scipy.linalg.eig(np.linalg.solve(M, K))
    order = np.argsort(lam.real)
    lam = lam.real[order]
    W = W.real[:, order]
    E = np.linalg.solve(W, np.linalg.inv(M))
    return lam, W, E


def fd_solve(F, Ws, Es, lams, c0=0.0, c1=1.0):
    """TPMatricesLUFactors.solve (tpmatrix.py:545-587) with D = c0 + c1 * sum_i lambda_i:
    Ftilde = x_i E_i F;  U = x_i W_i (Ftilde / D)."""
    d = F.ndim
    Ft = F
    for ax in range(d):
        Ft = np.moveaxis(np.tensordot(Es[ax], Ft, axes=(1, ax)), 0, ax)
    D = np.full(F.shape, c0, dtype=np.float64)
    for ax in range(d):
        shp = [1] * d
        shp[ax] = -1
        D = D + c1 * lams[ax].reshape(shp)
    U = Ft / D
    for ax in range(d):
        U = np.moveaxis(np.tensordot(Ws[ax], U, axes=(1, ax)), 0, ax)
    return U


# ---------------------------------------------------------------------------
# Variable-coefficient operator (inner.py:809-911, 991-1024; tensormatrix.py:54-56)
# ---------------------------------------------------------------------------


def multivar_factors(V: Space1D, i: int, j: int, Nq=None):
    """``inner_bilinear`` multivar branch (inner.py:887-898):
    multi = S (w * Pi^(i))^T-side factor (Nq, dim), multj = S Pj^(j)."""
    x, w = V.quad(Nq)
    Pi = V.vandermonde_orth(x, i)
    Pj = V.vandermonde_orth(x, j)
    multi = (w[:, None] * Pi) @ V.S.T
    multj = Pj @ V.S.T
    return multi, multj


def assemble_multivar(P0, P1, P2, P3, kappa):
    """A[i,k,j,l] = sum_pq P0[p,i] P1[p,k] P2[q,j] P3[q,l] kappa[p,q] (inner.py:1023)."""
    return np.einsum("pi,pk,qj,ql,pq->ikjl", P0, P1, P2, P3, kappa, optimize=True)


def tensormatrix_matvec(A, u):
    """TensorMatrix._matmul_array: v_ij = sum_kl A_ikjl u_kl (tensormatrix.py:54-56)."""
    return np.einsum("ikjl,kl->ij", A, u)


def varcoef_tensormatrix(V: Space1D, kappa):
    """Dense 4-index operator of (kappa grad u, grad v) in 2-D: the sum of the two
    multivar TensorMatrix terms jaxfun assembles for kappa*Dot(Grad(u), Grad(v))."""
    P1x, P1dx = multivar_factors(V, 1, 1)
    P0x, P0dx = multivar_factors(V, 0, 0)
    A = assemble_multivar(P1x, P1dx, P0x, P0dx, kappa)
    A += assemble_multivar(P0x, P0dx, P1x, P1dx, kappa)
    return A


def varcoef_apply(V: Space1D, kappa, U):
    """Sum-factorised (kappa grad u, grad v) in 2-D or 3-D: contract U to the
    gradient on the grid, multiply by kappa * w (x) w (x) ..., contract back.
    Equal (to rounding) to ``tensormatrix_matvec(varcoef_tensormatrix(...), U)``."""
    x, w = V.quad()
    S = V.S
    B = V.vandermonde_orth(x, 0) @ S.T  # (Nq, n)  phi_k(x_q)
    B1 = V.vandermonde_orth(x, 1) @ S.T  # (Nq, n)  phi_k'(x_q)
    d = U.ndim
    W = np.ones([w.size] * d)
    for ax in range(d):
        shp = [1] * d
        shp[ax] = -1
        W = W * w.reshape(shp)
    KW = kappa * W
    out = np.zeros(U.shape)
    for g in range(d):
        G = U
        for ax in range(d):
            M = B1 if ax == g else B
            G = np.moveaxis(np.tensordot(M, G, axes=(1, ax)), 0, ax)
        G = G * KW
        for ax in range(d):
            M = B1 if ax == g else B
            G = np.moveaxis(np.tensordot(M.T, G, axes=(1, ax)), 0, ax)
        out += G
    return out


def pcg(apply_A, b, apply_Minv, x0=None, tol=1e-12, maxiter=5000):
    """Plain FP64 preconditioned conjugate gradients (no counterpart on the
    reference's Galerkin path; it follows the textbook algorithm that
    jax.scipy.sparse.linalg.cg implements, used by src/jaxfun/pinns/
    hessoptimizer.py:97).  Stops when sqrt(r.z / r0.z0) <= tol.
    Returns (x, iterations)."""
    x = np.zeros_like(b) if x0 is None else x0.copy()
    r = b - apply_A(x) if x0 is not None else b.copy()
    z = apply_Minv(r)
    p = z.copy()
    rz = float(np.vdot(r, z))
    rz0 = float(np.vdot(b, apply_Minv(b)))
    if rz0 == 0.0:
        return x, 0
    it = 0
    while it < maxiter and np.sqrt(abs(rz) / rz0) > tol:
        q = apply_A(p)
        alpha = rz / float(np.vdot(p, q))
        x += alpha * p
        r -= alpha * q
        z = apply_Minv(r)
        rz_new = float(np.vdot(r, z))
        p = z + (rz_new / rz) * p
        rz = rz_new
        it += 1
    return x, it


# ---------------------------------------------------------------------------
# Synthetic inputs (seeded) for the benchmark configurations
# ---------------------------------------------------------------------------


def forcing_coeffs(rng, N, d):
    """f_hat ~ N(0,1) * prod_ax (1+k_ax)^-2 on N^d orthogonal coefficients."""
    z = rng.standard_normal((N,) * d)
    s = np.ones((N,) * d)
    for ax in range(d):
        shp = [1] * d
        shp[ax] = -1
        s = s * (1.0 + np.arange(N)).reshape(shp) ** -2.0
    return z * s


def random_field_coeffs(rng, N, d):
    """g_hat ~ N(0,1) * (1+|k|^2)^-1.5 on N^d orthogonal coefficients."""
    z = rng.standard_normal((N,) * d)
    k2 = np.zeros((N,) * d)
    for ax in range(d):
        shp = [1] * d
        shp[ax] = -1
        k2 = k2 + (np.arange(N, dtype=np.float64) ** 2).reshape(shp)
    return z * (1.0 + k2) ** -1.5


# ---------------------------------------------------------------------------
# Per-wavenumber banded systems (Fourier x polynomial)
# ---------------------------------------------------------------------------


def dia_to_dense(data_s, offsets, n):
    """Dense matrix of one system from column-aligned DIA data:
    A[j - off][j] = data[d][j] (``DiaMatrix`` storage, src/jaxfun/la/
    diamatrix.py:108-120, band convention of :1944)."""
    A = np.zeros((n, n))
    for d, off in enumerate(offsets):
        for j in range(n):
            i = j - off
            if 0 <= i < n:
                A[i, j] = data_s[d][j]
    return A


def wavenumber_solve(data, offsets, rhs_2d):
    """Solve B_k x_k = b_k for every wavenumber k (rows of rhs_2d, the
    polynomial axis last), as TPMatricesWavenumberSolver.solve
    (src/jaxfun/la/tpmatrix.py:590-1013) does with banded LU; here with a
    dense LAPACK solve per system (same solution to rounding)."""
    n = rhs_2d.shape[1]
    out = np.empty_like(rhs_2d)
    for k in range(rhs_2d.shape[0]):
        out[k] = np.linalg.solve(dia_to_dense(data[k], offsets, n), rhs_2d[k])
    return out


# ---------------------------------------------------------------------------
# Inhomogeneous Dirichlet data: DirectSum and DirectSumTPS
# ---------------------------------------------------------------------------


def bc_basis(family: str, N: int) -> np.ndarray:
    """Dirichlet boundary basis as orthogonal-coefficient rows (2 x N).

    Restates ``get_bc_basis`` (src/jaxfun/galerkin/composite.py:835-880) for
    {"left": D, "right": D}: A[side][j] = psi_j(x_side) for j = 0, 1 (the
    search start ``first`` = 0 gives an invertible A), S = (A^{-1})^T, so
    basis function k is 1 at boundary k and 0 at the other.
    """
    A = Space1D(family, N).vandermonde_orth(np.array([-1.0, 1.0]))[:, :2]
    S = np.zeros((2, N))
    S[:, :2] = np.linalg.solve(A, np.eye(2)).T
    return S


def _bc_eval(v, coords):
    shape = np.broadcast_shapes(*[np.shape(c) for c in coords])
    if callable(v):
        return np.broadcast_to(np.asarray(v(*coords), dtype=np.float64), shape)
    return np.full(shape, float(v))


def _solve_along0(P, b):
    """P^{-1} b along axis 0 of an array of any rank."""
    return np.linalg.solve(P, b.reshape(b.shape[0], -1)).reshape(b.shape)


class DirectSum1D:
    """Composite (+) BCGeneric with Dirichlet values (left, right), the
    reference's ``DirectSum`` (src/jaxfun/galerkin/composite.py:502-631)."""

    def __init__(self, family: str, N: int, left: float, right: float):
        self.V = Space1D(family, N, dirichlet=True)
        self.O = Space1D(family, N)
        self.B = bc_basis(family, N)
        self.vals = np.array([float(left), float(right)])

    def lift(self):
        """to_orthogonal of the boundary part: bnd_vals @ S_B (composite.py:585-591)."""
        return self.vals @ self.B

    def to_orthogonal(self, c):
        lift = self.lift().reshape((-1,) + (1,) * (np.ndim(c) - 1))
        return self.V.to_orthogonal(c) + lift

    def from_orthogonal(self, a):
        """P.solve(S (a - c_b)) with P = S S^T (composite.py:282-285, 593-600)."""
        lift = self.lift().reshape((-1,) + (1,) * (np.ndim(a) - 1))
        S = self.V.S
        return _solve_along0(S @ S.T, np.tensordot(S, a - lift, axes=(1, 0)))

    def forward(self, u):
        """orthogonal forward, then from_orthogonal (composite.py:612-616)."""
        return self.from_orthogonal(self.O.forward(u))

    def backward(self, c, Nq=None):
        return self.O.backward(self.to_orthogonal(c), Nq)

    def evaluate(self, X, c):
        return self.O.vandermonde_orth(np.asarray(X, dtype=np.float64)) @ self.to_orthogonal(c)


class LiftedTPS:
    """DirectSumTPS (src/jaxfun/galerkin/tensorproductspace.py:560-851) for
    Legendre/Chebyshev axes.  ``axes``: list of (family, N, bc) with bc
    "orth" (orthogonal space), None (homogeneous Dirichlet composite) or a
    (left, right) pair of Dirichlet values, each a number or a callable of
    all coordinates (the boundary's own coordinate fixed at the boundary).

    tpspaces are keyed by a tuple of "h" (homogeneous factor) / "b" (boundary
    factor) per axis; bndvals follow the reference's cases (:609-745).
    """

    def __init__(self, axes):
        self.axes = list(axes)
        nd = len(axes)
        self.nd = nd
        self.isbc = [isinstance(a[2], tuple) for a in axes]
        bcind = [i for i in range(nd) if self.isbc[i]]
        if nd == 3 and bcind[0] == 0:
            raise ValueError("DirectSum cannot be the first space in a 3D tensor product.")
        self.hom = [Space1D(f, N, dirichlet=(bc != "orth")) for f, N, bc in axes]
        self.orth = [Space1D(f, N) for f, N, _ in axes]
        self.Bs = [bc_basis(f, N) for f, N, _ in axes]
        self.mesh = [self.orth[i].quad()[0] for i in range(nd)]
        ends = (-1.0, 1.0)
        two = len(bcind) == 2
        # projected_bcs (:624-668): the other DirectSum's data at this one's ends
        if two:
            i0, i1 = bcind
            h0, h1 = axes[i0][2], axes[i1][2]
            proj = [[], []]
            for a in range(2):
                proj[0].append(tuple(self._fix(h0[a], {i0: ends[a], i1: ends[s]})
                                     for s in range(2)))
                proj[1].append(tuple(self._fix(h1[a], {i1: ends[a], i0: ends[s]})
                                     for s in range(2)))
        self.bndvals = {}
        keys = [("h", "b") if self.isbc[i] else ("h",) for i in range(nd)]
        import itertools

        for key in itertools.product(*keys):
            nb = [i for i in range(nd) if key[i] == "b"]
            other = [i for i in range(nd) if key[i] == "h"]
            if not nb:
                continue
            if not other:  # all boundary (2-D corners)
                self.bndvals[key] = np.array(
                    [[float(_bc_eval(v, [np.zeros(())] * nd)) for v in proj[0][a]]
                     for a in range(2)])
            elif len(other) == 1 and len(nb) == 1:  # 2-D, one boundary factor
                b, o = nb[0], other[0]
                uh = []
                for j in range(2):
                    g = _bc_eval(axes[b][2][j],
                                 [self.mesh[o] if i == o else np.array(ends[j])
                                  for i in range(nd)])
                    if two:
                        corner = proj[bcind.index(b)][j]
                        f, N, _ = axes[o]
                        cv = [float(_bc_eval(v, [np.zeros(())] * nd)) for v in corner]
                        uh.append(DirectSum1D(f, N, cv[0], cv[1]).forward(g))
                    else:
                        uh.append(self.hom[o].forward(g))
                self.bndvals[key] = np.array(uh) if b == 0 else np.array(uh).T
            elif len(other) == 2 and len(nb) == 1:  # 3-D, one boundary factor
                b = nb[0]
                o = 1 if b == 2 else 2
                uh = []
                for j in range(2):
                    G = _bc_eval(axes[b][2][j],
                                 [self.mesh[0][:, None] if i == 0 else
                                  (self.mesh[o][None, :] if i == o else np.array(ends[j]))
                                  for i in range(nd)])
                    if two:
                        # the other DirectSum's data at this boundary, as a
                        # function of (x, other coordinate)
                        vals = axes[b][2][j]
                        sub = tuple(
                            (lambda x, y, v=vals, s=s, o=o, b=b, e=ends[j]:
                             _bc_eval(v, [x, *( [ends[s], e] if o == 1 else [e, ends[s]] )]))
                            for s in range(2))
                        inner = LiftedTPS([(axes[0][0], axes[0][1], axes[0][2]),
                                           (axes[o][0], axes[o][1], sub)])
                        uh.append(inner.forward(G))
                    else:
                        uh.append(tp_forward([self.hom[0], self.hom[o]], G))
                arr = np.array(uh)
                self.bndvals[key] = arr.transpose(1, 2, 0) if b == 2 else arr.transpose(1, 0, 2)
            else:  # 3-D, two boundary factors (:739-745)
                uh = []
                for a in range(2):
                    for s in range(2):
                        g = _bc_eval(axes[1][2][a], [self.mesh[0], np.array(ends[a]),
                                                     np.array(ends[s])])
                        uh.append(self.hom[0].forward(g))
                self.bndvals[key] = np.array(uh).T.reshape((-1, 2, 2))

    @staticmethod
    def _fix(v, fixed):
        """Value of v with the coordinates in ``fixed`` substituted."""
        def f(*coords):
            c = list(coords)
            for i, e in fixed.items():
                c[i] = np.full(np.shape(c[i]), e)
            return _bc_eval(v, c)
        return f

    def _factor_to_orth(self, key, c):
        for ax in range(self.nd):
            S = self.Bs[ax] if key[ax] == "b" else self.hom[ax].S
            c = _along(ax, lambda b, S=S: np.tensordot(S.T, b, axes=(1, 0)), c)
        return c

    def lift(self):
        a = 0.0
        for key, v in self.bndvals.items():
            a = a + self._factor_to_orth(key, v)
        return a

    def to_orthogonal(self, c):
        """homogeneous to_orthogonal plus every boundary factor's (:808-823)."""
        return self._factor_to_orth(("h",) * self.nd, c) + self.lift()

    def from_orthogonal(self, a):
        """subtract the boundary factors, then the homogeneous from_orthogonal
        per axis (:825-851)."""
        d = a - self.lift()
        for ax in range(self.nd):
            if self.axes[ax][2] == "orth":
                continue
            S = self.hom[ax].S
            d = _along(ax, lambda b, S=S: _solve_along0(S @ S.T, np.tensordot(S, b, axes=(1, 0))),
                       d)
        return d

    def forward(self, u):
        return self.from_orthogonal(tp_forward(self.orth, u))

    def backward(self, c, Nq=None):
        return tp_backward(self.orth, self.to_orthogonal(c), Nq)

    def evaluate_grid(self, xs, c):
        """u on the tensor grid of points xs (one array per axis)."""
        a = self.to_orthogonal(c)
        for ax, x in enumerate(xs):
            V = self.orth[ax].vandermonde_orth(np.asarray(x, dtype=np.float64))
            a = _along(ax, lambda b, V=V: np.tensordot(V, b, axes=(1, 0)), a)
        return a

    def helmholtz_rhs(self, f, alpha2=0.0):
        """b = (f, v) - a(lift, v) for alpha^2 u - div grad u = f: the trial
        lift on the orthogonal basis with test functions of the homogeneous
        space, by quadrature (inner.py:809-911 with a DirectSum trial)."""
        b = tp_scalar_product(self.hom, f)
        lift = self.lift()
        mats_M, mats_K = [], []
        for ax in range(self.nd):
            x, w = self.orth[ax].quad()
            P0 = self.orth[ax].vandermonde_orth(x, 0)
            P2 = self.orth[ax].vandermonde_orth(x, 2)
            S = self.hom[ax].S
            mats_M.append(S @ ((P0.T * w[None, :]) @ P0))
            mats_K.append(-(S @ ((P0.T * w[None, :]) @ P2)))
        terms = []
        if alpha2 != 0.0:
            terms.append((alpha2, mats_M))
        for ax in range(self.nd):
            m = list(mats_M)
            m[ax] = mats_K[ax]
            terms.append((1.0, m))
        for s, mats in terms:
            Z = lift
            for ax, A in enumerate(mats):
                Z = np.moveaxis(np.tensordot(A, Z, axes=(1, ax)), 0, ax)
            b = b - s * Z
        return b
