"""1-D Legendre and Chebyshev spaces (orthogonal and homogeneous-Dirichlet
composite) and their dense per-axis operators.

The call surface follows jaxfun: ``Legendre(N)``, ``Chebyshev(N)``,
``FunctionSpace(N, Legendre, bcs={"left": {"D": 0}, "right": {"D": 0}})``
with ``quad_points_and_weights``, ``vandermonde``, ``evaluate_basis_derivative``,
``mass_matrix``, ``backward``, ``forward``, ``scalar_product``
(src/jaxfun/galerkin/orthogonal.py:131-277, composite.py:153-349,
functionspace.py:63-173).  Unlike the reference, every transform is a dense
contraction with a precomputed FP64 operator: the Chebyshev DCTs
(Chebyshev.py:225-279) become Vandermonde contractions and the composite mass
solve (composite.py:339-343) is folded into the forward operator.  The
operators are built once on the host in FP64 (as the reference builds its
stencils and eigendecompositions with NumPy/SciPy) and applied on the GPU.
"""

from __future__ import annotations

import functools

import numpy as np

DIRICHLET = {"left": {"D": 0}, "right": {"D": 0}}


# ---------------------------------------------------------------------------
# quadrature rules and basis recurrences (FP64 setup)
# ---------------------------------------------------------------------------


@functools.lru_cache(maxsize=64)
def legendre_gauss(N: int) -> tuple[np.ndarray, np.ndarray]:
    """Gauss-Legendre nodes (ascending) and weights by Newton iteration on P_N.

    Same rule as ``Legendre.quad_points_and_weights`` / ``fastgl.leggauss``
    (src/jaxfun/galerkin/Legendre.py:125-137, src/jaxfun/utils/fastgl.py:547-567).
    """
    k = np.arange(1, N + 1, dtype=np.float64)
    x = -np.cos(np.pi * (4.0 * k - 1.0) / (4.0 * N + 2.0))
    for _ in range(100):
        p0 = np.ones_like(x)
        p1 = x.copy()
        for m in range(2, N + 1):
            p0, p1 = p1, ((2.0 * m - 1.0) * x * p1 - (m - 1.0) * p0) / m
        dp = N * (x * p1 - p0) / (x * x - 1.0)
        dx = p1 / dp
        x = x - dx
        if np.max(np.abs(dx)) < 1e-16:
            break
    p0 = np.ones_like(x)
    p1 = x.copy()
    for m in range(2, N + 1):
        p0, p1 = p1, ((2.0 * m - 1.0) * x * p1 - (m - 1.0) * p0) / m
    dp = N * (x * p1 - p0) / (x * x - 1.0)
    w = 2.0 / ((1.0 - x * x) * dp * dp)
    x.setflags(write=False)
    w.setflags(write=False)
    return x, w


def chebyshev_gauss(N: int) -> tuple[np.ndarray, np.ndarray]:
    """x_k = cos(pi + (2k+1) pi / 2N), w_k = pi / N (src/jaxfun/galerkin/Chebyshev.py:149-170)."""
    k = np.arange(N)
    return np.cos(np.pi + (2 * k + 1) * np.pi / (2 * N)), np.full(N, np.pi / N)


def _legendre_derivs(x: np.ndarray, N: int, kmax: int) -> list[np.ndarray]:
    """[P^(0), ..., P^(kmax)] at x, each (len(x), N)."""
    out = []
    V = np.zeros((x.size, N))
    V[:, 0] = 1.0
    if N > 1:
        V[:, 1] = x
    for n in range(1, N - 1):
        V[:, n + 1] = ((2 * n + 1) * x * V[:, n] - n * V[:, n - 1]) / (n + 1)
    out.append(V)
    for _ in range(kmax):
        prev = out[-1]
        D = np.zeros_like(prev)
        if N > 1:
            D[:, 1] = prev[:, 0]
        for n in range(1, N - 1):
            D[:, n + 1] = D[:, n - 1] + (2 * n + 1) * prev[:, n]
        out.append(D)
    return out


def _chebyshev_derivs(x: np.ndarray, N: int, kmax: int) -> list[np.ndarray]:
    V = np.zeros((x.size, N))
    V[:, 0] = 1.0
    if N > 1:
        V[:, 1] = x
    for n in range(1, N - 1):
        V[:, n + 1] = 2 * x * V[:, n] - V[:, n - 1]
    out = [V]
    for kk in range(1, kmax + 1):
        prev = out[-1]
        D = np.zeros_like(prev)
        if N > 1 and kk == 1:
            D[:, 1] = 1.0
        for n in range(1, N - 1):
            D[:, n + 1] = 2 * kk * prev[:, n] + 2 * x * D[:, n] - D[:, n - 1]
        out.append(D)
    return out


# ---------------------------------------------------------------------------
# spaces
# ---------------------------------------------------------------------------


class OrthogonalSpace:
    """Orthogonal Legendre (P_k) or Chebyshev (T_k) space with N modes on [-1, 1]."""

    family = "legendre"
    is_orthogonal = True

    def __init__(self, N: int, name: str | None = None):
        if N < 2:
            raise ValueError("N must be >= 2")
        self.N = int(N)
        self.name = name or type(self).__name__
        self.bcs = None

    # -- reference-compatible properties ------------------------------------
    @property
    def dim(self) -> int:
        return self.N

    @property
    def num_quad_points(self) -> int:
        return self.N

    @property
    def orthogonal(self) -> OrthogonalSpace:
        return self

    @property
    def S(self) -> np.ndarray:
        """Stencil (identity for orthogonal spaces)."""
        return np.eye(self.N)

    def norm_squared(self) -> np.ndarray:
        if self.family == "legendre":
            return 2.0 / (2.0 * np.arange(self.N) + 1.0)
        h = np.full(self.N, np.pi / 2)
        h[0] = np.pi
        return h

    def quad_points_and_weights(self, N: int | None = None):
        N = self.N if N is None else int(N)
        if self.family == "legendre":
            return legendre_gauss(N)
        return chebyshev_gauss(N)

    def mesh(self, N: int | None = None) -> np.ndarray:
        return self.quad_points_and_weights(N)[0]

    def evaluate_basis_derivative(self, X, k: int = 0) -> np.ndarray:
        """(len(X), N) matrix of d^k/dx^k psi_j(X) (orthogonal.py:168-178)."""
        X = np.asarray(X, dtype=np.float64).ravel()
        f = _legendre_derivs if self.family == "legendre" else _chebyshev_derivs
        return f(X, self.N, k)[k] @ self.S.T

    def vandermonde(self, X) -> np.ndarray:
        return self.evaluate_basis_derivative(X, 0)

    # -- Galerkin matrices ---------------------------------------------------
    def mass_matrix(self) -> np.ndarray:
        """(psi_j, psi_i)_w: diag(h) for orthogonal, S diag(h) S^T for composites
        (orthogonal.py:248-254, composite.py:330-333)."""
        S = self.S
        return S @ np.diag(self.norm_squared()) @ S.T

    def stiffness_matrix(self) -> np.ndarray:
        """K[i, j] = -(psi_j'', psi_i)_w (test i, trial j); equals (psi_j', psi_i') for
        Legendre.  Legendre Dirichlet: diag(4k+6) (Legendre.py:439-443, 489-493);
        Chebyshev: -S D2 S^T with D2 = (T_i, T_j'')_w (Chebyshev.py:21-35)."""
        N = self.N
        rows = np.arange(N)[:, None]
        cols = np.arange(N)[None, :]
        off = cols - rows
        mask = (off >= 2) & ((off - 2) % 2 == 0)
        if self.family == "legendre":
            D2 = np.where(mask, cols * (cols + 1) - rows * (rows + 1), 0.0)
        else:
            D2 = np.where(mask, cols * (cols**2 - rows**2) * np.pi / 2, 0.0)
        S = self.S
        # "+ 0.0" turns the -0.0 entries of the negated product into +0.0, so
        # the matrix is bit-identical to the closed forms (diag(4k+6) for
        # Legendre) and LAPACK picks the same eigenvector signs for it
        return -(S @ D2 @ S.T) + 0.0

    # -- dense per-axis operators (FP64, host) -------------------------------
    @functools.lru_cache(maxsize=16)
    def backward_matrix(self, Nq: int | None = None, k: int = 0) -> np.ndarray:
        """B[q, j] = d^k psi_j(x_q) at the Nq-point rule: (Nq x dim)."""
        x, _ = self.quad_points_and_weights(Nq)
        B = self.evaluate_basis_derivative(x, k)
        B.setflags(write=False)
        return B

    @functools.lru_cache(maxsize=16)
    def scalar_product_matrix(self, Nq: int | None = None) -> np.ndarray:
        """SP[j, q] = w_q psi_j(x_q): (dim x Nq) (orthogonal.py:264-277, composite.py:345-349)."""
        x, w = self.quad_points_and_weights(Nq)
        SP = (self.evaluate_basis_derivative(x, 0) * w[:, None]).T.copy()
        SP.setflags(write=False)
        return SP

    @functools.lru_cache(maxsize=16)
    def forward_matrix(self, Nq: int | None = None) -> np.ndarray:
        """F = M^{-1} SP: (dim x Nq), mass inverse folded in
        (orthogonal.py:256-262, composite.py:339-343)."""
        F = np.linalg.solve(self.mass_matrix(), self.scalar_product_matrix(Nq))
        F.setflags(write=False)
        return F

    def __hash__(self):
        return hash((type(self), self.family, self.N, self.dirichlet))

    def __eq__(self, other):
        return (
            type(self) is type(other)
            and self.family == other.family
            and self.N == other.N
            and self.dirichlet == other.dirichlet
        )

    dirichlet = False

    # -- 1-D transforms on the GPU ------------------------------------------
    def backward(self, c, N: int | None = None):
        from .tensorproductspace import _apply_1d

        return _apply_1d(self.backward_matrix(N), c)

    def forward(self, u):
        from .tensorproductspace import _apply_1d

        return _apply_1d(self.forward_matrix(u.shape[-1]), u)

    def scalar_product(self, u):
        from .tensorproductspace import _apply_1d

        return _apply_1d(self.scalar_product_matrix(u.shape[-1]), u)


class Legendre(OrthogonalSpace):
    family = "legendre"


class Chebyshev(OrthogonalSpace):
    family = "chebyshev"


class Composite(OrthogonalSpace):
    """Homogeneous Dirichlet composite phi_k = psi_k - psi_{k+2} (LDRD stencil,
    src/jaxfun/galerkin/composite.py:786-789); dim = N - 2, N quadrature points."""

    is_orthogonal = False
    dirichlet = True

    def __init__(self, N: int, family: str, name: str | None = None):
        super().__init__(N, name)
        self.family = family
        self.bcs = DIRICHLET
        self._orth = (Legendre if family == "legendre" else Chebyshev)(N)

    @property
    def dim(self) -> int:
        return self.N - 2

    @property
    def orthogonal(self) -> OrthogonalSpace:
        return self._orth

    @property
    def S(self) -> np.ndarray:
        S = np.zeros((self.N - 2, self.N))
        k = np.arange(self.N - 2)
        S[k, k] = 1.0
        S[k, k + 2] = -1.0
        return S


def FunctionSpace(N: int, space=Legendre, bcs: dict | None = None, name: str | None = None):
    """Factory as src/jaxfun/galerkin/functionspace.py:63-173: an orthogonal space, or a
    Dirichlet composite when ``bcs`` prescribes homogeneous Dirichlet values at both ends."""
    family = space.family if isinstance(space, type) else str(space)
    if bcs is None:
        return (Legendre if family == "legendre" else Chebyshev)(N, name)
    left = bcs.get("left", {})
    right = bcs.get("right", {})
    if set(left) != {"D"} or set(right) != {"D"} or left["D"] != 0 or right["D"] != 0:
        raise NotImplementedError(
            "only homogeneous Dirichlet boundary conditions are on the GPU path"
        )
    return Composite(N, family, name)
