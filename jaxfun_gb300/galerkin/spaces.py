"""1-D Legendre and Chebyshev spaces (orthogonal, homogeneous-Dirichlet
composite, and the inhomogeneous-Dirichlet direct sum) and their dense
per-axis operators.

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


def chebyshev_gauss_vandermonde(Nq: int, N: int) -> np.ndarray:
    """T_j(x_k) at the Nq Gauss nodes, (Nq x N), from exactly reduced angles.

    x_k = cos(theta_k) with theta_k = (2 Nq - 2k - 1) pi / (2 Nq), so
    T_j(x_k) = cos(pi m / (2 Nq)) for the integer m = j (2 Nq - 2k - 1) mod 4 Nq;
    folding m into [0, Nq/2] by the symmetries of cos keeps every argument
    below pi/4, so each entry is within an ulp or two.  This is the matrix of
    the DCT that Chebyshev.backward / scalar_product apply (Chebyshev.py:225-279);
    the three-term recurrence on the rounded nodes loses ~j ulps instead.
    """
    k = np.arange(Nq, dtype=np.int64)[:, None]
    j = np.arange(N, dtype=np.int64)[None, :]
    m = (j * (2 * Nq - 2 * k - 1)) % (4 * Nq)
    m = np.where(m > 2 * Nq, 4 * Nq - m, m)
    sign = np.where(m > Nq, -1.0, 1.0)
    m = np.where(m > Nq, 2 * Nq - m, m)
    use_sin = 2 * m > Nq
    ang = np.where(use_sin, Nq - m, m) * (np.pi / (2 * Nq))
    return sign * np.where(use_sin, np.sin(ang), np.cos(ang))


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

    def mesh(self, N: int | None = None, kind: str = "quadrature") -> np.ndarray:
        """Quadrature nodes, or ``kind="uniform"``: N equispaced points on [-1, 1]
        (orthogonal.py:429-444)."""
        if kind == "uniform":
            return np.linspace(-1.0, 1.0, self.N if N is None else int(N))
        if kind != "quadrature":
            raise ValueError(f"unknown mesh kind {kind!r}")
        return self.quad_points_and_weights(N)[0]

    @functools.lru_cache(maxsize=16)
    def evaluation_matrix(self, kind: str = "quadrature", N: int | None = None) -> np.ndarray:
        """(points x dim) basis values on a quadrature or uniform mesh
        (``evaluate_mesh``, orthogonal.py:181-199)."""
        if kind == "quadrature":
            return self.backward_matrix(N)
        V = self.vandermonde(self.mesh(N, kind))
        V.setflags(write=False)
        return V

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

    def orthogonal_d2(self) -> np.ndarray:
        """D2[i, j] = (psi_i, psi_j'')_w of the orthogonal basis, closed form
        (Legendre.py:19-33, Chebyshev.py:21-35): nonzero for j - i >= 2 even."""
        N = self.N
        rows = np.arange(N)[:, None]
        cols = np.arange(N)[None, :]
        off = cols - rows
        mask = (off >= 2) & ((off - 2) % 2 == 0)
        if self.family == "legendre":
            return np.where(mask, cols * (cols + 1) - rows * (rows + 1), 0.0)
        return np.where(mask, cols * (cols**2 - rows**2) * np.pi / 2, 0.0)

    def stiffness_matrix(self) -> np.ndarray:
        """K[i, j] = -(psi_j'', psi_i)_w (test i, trial j); equals (psi_j', psi_i') for
        Legendre.  Legendre Dirichlet: diag(4k+6) (Legendre.py:439-443, 489-493);
        Chebyshev: -S D2 S^T with D2 = (T_i, T_j'')_w (Chebyshev.py:21-35)."""
        S = self.S
        # "+ 0.0" turns the -0.0 entries of the negated product into +0.0, so
        # the matrix is bit-identical to the closed forms (diag(4k+6) for
        # Legendre) and LAPACK picks the same eigenvector signs for it
        return -(S @ self.orthogonal_d2() @ S.T) + 0.0

    def test_orthogonal_matrices(self) -> tuple[np.ndarray, np.ndarray]:
        """(K_r, M_r): stiffness and mass with this space's test functions (rows)
        and the ORTHOGONAL basis as trial functions (columns), dim x N.  They
        move a boundary lift given in orthogonal coefficients to the right-hand
        side (the DirectSum trial branch of inner, inner.py:809-911)."""
        S = self.S
        return -(S @ self.orthogonal_d2()) + 0.0, S * self.norm_squared()[None, :]

    # -- dense per-axis operators (FP64, host) -------------------------------
    def _quad_basis(self, Nq: int | None, k: int) -> np.ndarray:
        """d^k psi_j at the Nq-point Gauss rule (Chebyshev values from exact angles)."""
        x, _ = self.quad_points_and_weights(Nq)
        if self.family == "chebyshev" and k == 0:
            return chebyshev_gauss_vandermonde(x.size, self.N) @ self.S.T
        return self.evaluate_basis_derivative(x, k)

    @functools.lru_cache(maxsize=16)
    def backward_matrix(self, Nq: int | None = None, k: int = 0) -> np.ndarray:
        """B[q, j] = d^k psi_j(x_q) at the Nq-point rule: (Nq x dim)."""
        B = self._quad_basis(Nq, k)
        B.setflags(write=False)
        return B

    @functools.lru_cache(maxsize=16)
    def scalar_product_matrix(self, Nq: int | None = None) -> np.ndarray:
        """SP[j, q] = w_q psi_j(x_q): (dim x Nq) (orthogonal.py:264-277, composite.py:345-349)."""
        _, w = self.quad_points_and_weights(Nq)
        SP = (self._quad_basis(Nq, 0) * w[:, None]).T.copy()
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


# ---------------------------------------------------------------------------
# inhomogeneous Dirichlet data: boundary basis and direct sum
# ---------------------------------------------------------------------------


class BCValue:
    """One Dirichlet boundary value: a number, a Python callable or a sympy
    expression.  Callables and expressions are functions of the coordinates
    of the tensor product they belong to, ``f(x)``, ``f(x, y)`` or
    ``f(x, y, z)`` (sympy symbols named x, y, z); the boundary's own
    coordinate is passed fixed at the boundary (the reference substitutes it
    away, e.g. ``ue.subs(y, 1)``, examples/helmholtz2D.py:24-26)."""

    def __init__(self, value):
        self.value = value
        self._fn = None
        if callable(value) and not _is_sympy(value):
            self._fn = value
        elif _is_sympy(value):
            import sympy as sp

            expr = sp.sympify(value)
            if not expr.free_symbols:
                self.value = float(expr)
            else:
                names = {str(t) for t in expr.free_symbols}
                if not names <= {"x", "y", "z"}:
                    raise ValueError(f"boundary value {expr} may use only x, y, z")
                syms = sp.symbols("x y z")
                # match the expression's own symbols (any assumptions) by name
                own = {str(t): t for t in expr.free_symbols}
                args = [own.get(str(t), t) for t in syms]
                self._fn = sp.lambdify(args, expr, "numpy")
                self._nargs = 3
        else:
            self.value = float(value)

    @property
    def is_constant(self) -> bool:
        return self._fn is None

    def __call__(self, *coords) -> np.ndarray:
        """Values on the broadcast of ``coords`` (one array per axis)."""
        shape = np.broadcast_shapes(*[np.shape(c) for c in coords])
        if self._fn is None:
            return np.full(shape, self.value)
        if getattr(self, "_nargs", None) == 3:
            full = list(coords) + [np.zeros(())] * (3 - len(coords))
            v = self._fn(*full)
        else:
            v = self._fn(*coords)
        return np.broadcast_to(np.asarray(v, dtype=np.float64), shape).copy()


def _is_sympy(v) -> bool:
    return type(v).__module__.startswith("sympy")


def _dirichlet_values(bcs: dict) -> tuple:
    left = bcs.get("left", {})
    right = bcs.get("right", {})
    if set(left) != {"D"} or set(right) != {"D"} or set(bcs) - {"left", "right"}:
        raise NotImplementedError(
            "only Dirichlet boundary conditions (left/right 'D') are on the GPU path"
        )
    return left["D"], right["D"]


class BCGeneric(OrthogonalSpace):
    """Boundary basis of a Dirichlet direct sum: B_0 = (psi_0 - psi_1)/2 (value 1
    at x = -1, 0 at x = 1) and B_1 = (psi_0 + psi_1)/2, the rows of S
    (BCGeneric and get_bc_basis, src/jaxfun/galerkin/composite.py:411-460,
    835-880: the inverse of the boundary-value matrix of psi_0, psi_1, the same
    for Legendre and Chebyshev since psi_0 = 1 and psi_1 = x)."""

    is_orthogonal = False
    dirichlet = "boundary"

    def __init__(self, N: int, family: str, bcs: dict, name: str | None = None):
        super().__init__(N, name)
        self.family = family
        self.bcs = bcs
        self.values = tuple(BCValue(v) for v in _dirichlet_values(bcs))
        self._orth = (Legendre if family == "legendre" else Chebyshev)(N)

    @property
    def dim(self) -> int:
        return 2

    @property
    def orthogonal(self) -> OrthogonalSpace:
        return self._orth

    @property
    def S(self) -> np.ndarray:
        S = np.zeros((2, self.N))
        S[0, :2] = (0.5, -0.5)
        S[1, :2] = (0.5, 0.5)
        return S

    def orderedvals(self) -> tuple:
        """(left, right) raw values (BoundaryConditions.orderedvals)."""
        return self.values

    def bnd_vals(self) -> np.ndarray:
        """Numeric (left, right) values (composite.py:465-472)."""
        if not all(v.is_constant for v in self.values):
            raise ValueError("boundary values are functions; evaluate them on the other axes")
        return np.array([v.value for v in self.values])


class DirectSum:
    """V = Composite (+) BCGeneric: the homogeneous Dirichlet space plus the
    boundary lift fixed by the boundary values (src/jaxfun/galerkin/
    composite.py:502-631).  Coefficients are those of the homogeneous part
    (dim = N - 2); every map to or from the orthogonal basis is affine:

      to_orthogonal(c)   = S^T c + a_bc,            a_bc = B^T (left, right)
      from_orthogonal(a) = (S S^T)^{-1} S (a - a_bc)  (composite.py:282-285)
      forward(u)         = from_orthogonal(orthogonal forward of u)
      backward(c)        = orthogonal backward of to_orthogonal(c)

    and runs on the GPU as one contraction with the constant added in the
    epilogue (``jfg_tp_apply_affine_f64``)."""

    is_orthogonal = False

    def __init__(self, a: Composite, b: BCGeneric):
        if not isinstance(b, BCGeneric):
            raise TypeError("the second summand must be a BCGeneric boundary space")
        self.basespaces = (a, b)
        self.bcs = b.bcs
        self.family = a.family
        self.N = a.N
        self.name = f"{a.name}+{b.name}"

    def __getitem__(self, i: int):
        return self.basespaces[i]

    def __len__(self) -> int:
        return 2

    def __iter__(self):
        return iter(self.basespaces)

    @property
    def dim(self) -> int:
        return self[0].dim

    @property
    def num_dofs(self) -> int:
        return self[0].dim

    @property
    def num_quad_points(self) -> int:
        return self[0].num_quad_points

    @property
    def orthogonal(self) -> OrthogonalSpace:
        return self[0].orthogonal

    def quad_points_and_weights(self, N: int | None = None):
        return self[0].quad_points_and_weights(N)

    def mesh(self, N: int | None = None, kind: str = "quadrature") -> np.ndarray:
        return self[0].mesh(N, kind)

    def get_homogeneous(self) -> Composite:
        return self[0]

    def bnd_vals(self) -> np.ndarray:
        return self[1].bnd_vals()

    # -- host FP64 setup ------------------------------------------------------
    def lift(self) -> np.ndarray:
        """a_bc: orthogonal coefficients of the boundary lift (length N)."""
        return self[1].S.T @ self.bnd_vals()

    @functools.lru_cache(maxsize=4)
    def reduce_matrix(self) -> np.ndarray:
        """R = (S S^T)^{-1} S (dim x N): Composite.from_orthogonal."""
        return reduce_matrix(self[0])

    def forward_host(self, u: np.ndarray) -> np.ndarray:
        """FP64 host projection of grid values u (setup of lifted tensor
        products: project1D onto a DirectSum, inner.py:1027-1041)."""
        a = self.orthogonal.forward_matrix(u.shape[0]) @ u
        return self.reduce_matrix() @ (a - self.lift())

    # -- GPU transforms -------------------------------------------------------
    # each map is (matrix, constant) built once per size in FP64 and applied by
    # one affine contraction; the cached arrays keep their device copies alive
    @functools.lru_cache(maxsize=32)
    def affine_map(self, kind: str, N: int | None = None) -> tuple[np.ndarray, np.ndarray]:
        """(matrix, shift) of the affine map ``kind``: "to_orthogonal",
        "from_orthogonal", "backward" (N quadrature points), "forward" (N grid
        points) or "uniform" (evaluation on N equispaced points)."""
        lift = self.lift()
        R = self.reduce_matrix()
        if kind == "to_orthogonal":
            mat, shift = self[0].S.T.copy(), lift
        elif kind == "from_orthogonal":
            mat, shift = R, -(R @ lift)
        elif kind in ("backward", "uniform"):
            k = "quadrature" if kind == "backward" else "uniform"
            mat = self[0].evaluation_matrix(k, N)
            shift = self.orthogonal.evaluation_matrix(k, N) @ lift
        elif kind == "forward":
            mat, shift = R @ self.orthogonal.forward_matrix(N), -(R @ lift)
        else:
            raise ValueError(f"unknown map {kind!r}")
        mat = np.ascontiguousarray(mat)
        shift = np.ascontiguousarray(shift)
        mat.setflags(write=False)
        shift.setflags(write=False)
        return mat, shift

    def _apply(self, kind, x, N=None):
        from .tensorproductspace import tp_apply_affine

        mat, shift = self.affine_map(kind, N)
        return tp_apply_affine([mat], x, shift)

    def to_orthogonal(self, c):
        return self._apply("to_orthogonal", c)

    def from_orthogonal(self, a):
        return self._apply("from_orthogonal", a)

    def backward(self, c, N: int | None = None):
        return self._apply("backward", c, N)

    def forward(self, u):
        return self._apply("forward", u, int(u.shape[-1]))

    def scalar_product(self, u):
        """Test functions carry no boundary part (composite.py:622-626)."""
        return self[0].scalar_product(u)

    def evaluate_mesh(self, c, kind: str = "quadrature", N: int | None = None):
        """u on the quadrature or a uniform mesh (composite.py:607-611)."""
        return self._apply("backward" if kind == "quadrature" else "uniform", c, N)

    def evaluate(self, X, c):
        """u(X) at arbitrary points (DirectSum.evaluate, composite.py:602-605)."""
        from .tensorproductspace import tp_apply_affine

        X = np.atleast_1d(np.asarray(X, dtype=np.float64))
        V = self.orthogonal.vandermonde(X)
        return tp_apply_affine([self[0].vandermonde(X)], c, V @ self.lift(), cache=False)


@functools.lru_cache(maxsize=64)
def reduce_matrix(space: OrthogonalSpace) -> np.ndarray:
    """(S S^T)^{-1} S: least-squares coefficients of a homogeneous space from
    orthogonal ones (Composite.from_orthogonal, composite.py:282-285); the
    identity for an orthogonal space."""
    S = space.S
    R = np.linalg.solve(S @ S.T, S)
    R.setflags(write=False)
    return R


def FunctionSpace(N: int, space=Legendre, bcs: dict | None = None, name: str | None = None):
    """Factory as src/jaxfun/galerkin/functionspace.py:63-173: an orthogonal
    space; a Dirichlet composite when ``bcs`` prescribes homogeneous Dirichlet
    values at both ends; a DirectSum (composite + boundary lift) for
    inhomogeneous Dirichlet values (numbers, callables or sympy expressions)."""
    family = space.family if isinstance(space, type) else str(space)
    if bcs is None:
        return (Legendre if family == "legendre" else Chebyshev)(N, name)
    left, right = _dirichlet_values(bcs)

    def _zero(v):
        if _is_sympy(v):
            import sympy as sp

            return sp.sympify(v) == 0
        return not callable(v) and float(v) == 0.0

    if _zero(left) and _zero(right):
        return Composite(N, family, name)
    return DirectSum(Composite(N, family, name), BCGeneric(N, family, bcs))
