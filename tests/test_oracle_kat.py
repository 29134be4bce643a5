"""The FP64 oracle against the reference's own known answers (CPU only)."""

import json
import os

import numpy as np
import pytest

from oracle import spectral as O

KAT = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "kat.json")))


def test_chebyshev_scalar_product_of_one():
    # src/jaxfun/galerkin/arguments.py:728-737
    V = O.Space1D("chebyshev", 4)
    b = V.scalar_product_orth(V.backward(np.ones(4)))
    assert np.allclose(b, KAT["chebyshev4_scalar_product_of_one"], rtol=0, atol=1e-15)


def test_tensormatrix_corner_x2y2():
    # tests/galerkin/test_inner.py:580-609: wrong without padding, exact with 7x7 points
    V = O.Space1D("legendre", 6)
    t = KAT["tensormatrix_x2y2_legendre6"]
    tol = KAT["atol_sqrt_ulp100"]
    for nq, ok in ((6, False), (7, True)):
        P0, P1 = O.multivar_factors(V, 0, 0, Nq=nq)
        x, _ = V.quad(nq)
        X, Y = np.meshgrid(x, x, indexing="ij")
        A = O.assemble_multivar(P0, P1, P0, P1, X**2 + Y**2)
        assert (abs(A[-1, -1, -1, -1] - t) < tol) == ok


def test_tensormatrix_corner_sqrt():
    # tests/galerkin/test_inner.py:611-650 (32x32 points)
    V = O.Space1D("legendre", 6)
    P0, P1 = O.multivar_factors(V, 0, 0, Nq=32)
    x, _ = V.quad(32)
    X, Y = np.meshgrid(x, x, indexing="ij")
    A = O.assemble_multivar(P0, P1, P0, P1, np.sqrt(X**2 + Y**2))
    assert abs(A[-1, -1, -1, -1] - KAT["tensormatrix_sqrt_legendre6"]) < KAT["atol_sqrt_ulp100"]


@pytest.mark.parametrize("family", ["legendre", "chebyshev"])
@pytest.mark.parametrize("dirichlet", [False, True])
def test_round_trip(family, dirichlet):
    # tests/galerkin/test_forward_backward.py:20-104 (ulp(100))
    V = O.Space1D(family, 8, dirichlet)
    rng = np.random.default_rng(0)
    c = rng.standard_normal((V.dim, V.dim))
    ch = O.tp_forward([V, V], O.tp_backward([V, V], c))
    assert np.linalg.norm(ch - c) < 100 * np.spacing(1.0) * 10


@pytest.mark.parametrize("family", ["legendre", "chebyshev"])
def test_poisson_manufactured(family):
    # tests/la/test_tpmatrices_solvers.py:91-104, 272-283
    V = O.Space1D(family, 16, True)
    x, _ = V.quad()
    X, Y = np.meshgrid(x, x, indexing="ij")
    f = 2 * (1 - Y**2) + 2 * (1 - X**2)
    b = O.tp_scalar_product([V, V], f)
    K, M = V.stiffness_matrix(), V.mass_matrix()
    if family == "legendre":
        lam, W = O.fd_factor_symmetric(K, M)
        E = W.T
    else:
        lam, W, E = O.fd_factor_general(K, M)
    for u in (O.kron_solve([(1.0, [K, M]), (1.0, [M, K])], b),
              O.fd_solve(b, [W, W], [E, E], [lam, lam])):
        xj = V.quad(40)[0]
        Xj, Yj = np.meshgrid(xj, xj, indexing="ij")
        uj = O.tp_backward([V, V], u, Nq=(40, 40))
        l2 = np.linalg.norm(uj - (1 - Xj**2) * (1 - Yj**2)) / 40
        assert l2 < KAT["poisson_manufactured_l2_bound"]


@pytest.mark.parametrize("family", ["legendre", "chebyshev"])
def test_closed_form_matrices_equal_quadrature(family):
    # tests/galerkin/test_precomputed_matrices.py:108-436
    V = O.Space1D(family, 12, True)
    K = V.stiffness_matrix()
    assert np.allclose(K, -V.matrices_quadrature(0, 2), rtol=1e-12, atol=1e-9)
    assert np.allclose(V.mass_matrix(), V.matrices_quadrature(0, 0), atol=1e-14)


def test_sumfactorised_equals_tensormatrix():
    V = O.Space1D("legendre", 10, True)
    rng = np.random.default_rng(2)
    kap = np.exp(0.3 * rng.standard_normal((10, 10)))
    U = rng.standard_normal((8, 8))
    A = O.varcoef_tensormatrix(V, kap)
    ref = O.tensormatrix_matvec(A, U)
    assert np.abs(O.varcoef_apply(V, kap, U) - ref).max() < 1e-12 * np.abs(ref).max()


def test_3d_varcoef_constant_kappa_is_separable():
    # constant kappa: (grad u, grad v) = K(x)M(x)M + M(x)K(x)M + M(x)M(x)K
    V = O.Space1D("legendre", 8, True)
    rng = np.random.default_rng(3)
    U = rng.standard_normal((6, 6, 6))
    K, M = V.stiffness_matrix(), V.mass_matrix()
    ref = O.tp_apply([(1.0, [K, M, M]), (1.0, [M, K, M]), (1.0, [M, M, K])], U)
    out = O.varcoef_apply(V, 2.5 * np.ones((8, 8, 8)), U)
    assert np.abs(out - 2.5 * ref).max() < 1e-12 * np.abs(ref).max()


def test_chebyshev_eigh_fd_is_wrong_general_eig_is_right():
    # the reference's eigh on the non-symmetric Chebyshev stiffness (tpmatrix.py:1184)
    V = O.Space1D("chebyshev", 24, True)
    K, M = V.stiffness_matrix(), V.mass_matrix()
    rng = np.random.default_rng(0)
    b = rng.standard_normal((22, 22))
    ref = O.kron_solve([(10.0, [M, M]), (1.0, [K, M]), (1.0, [M, K])], b)
    lam, W, E = O.fd_factor_general(K, M)
    good = O.fd_solve(b, [W, W], [E, E], [lam, lam], c0=10.0)
    assert np.abs(good - ref).max() < 1e-11 * np.abs(ref).max()
    import scipy.linalg

    lam2, W2 = scipy.linalg.eigh(K, M)  # reads one triangle only
    bad = O.fd_solve(b, [W2, W2], [W2.T, W2.T], [lam2, lam2], c0=10.0)
    assert np.abs(bad - ref).max() > 1e-3 * np.abs(ref).max()


def test_oracle_dia_convention():
    """Column-aligned DIA: data[d][j] = A[j - off_d][j] (diamatrix.py:108-120)."""
    from oracle import spectral as O

    A = np.arange(1.0, 26.0).reshape(5, 5)
    offsets = (-1, 0, 2)
    data = np.zeros((3, 5))
    for d, off in enumerate(offsets):
        for j in range(5):
            if 0 <= j - off < 5:
                data[d, j] = A[j - off, j]
    D = O.dia_to_dense(data, offsets, 5)
    mask = np.zeros((5, 5), bool)
    for off in offsets:
        mask |= np.eye(5, k=off, dtype=bool)
    assert np.array_equal(D, np.where(mask, A, 0.0))


# ---------------------------------------------------------------------------
# Docstring known answers of the Petrov-Galerkin test spaces (LegPhi_1/2,
# ChebPhi_1/2): src/jaxfun/galerkin/Legendre.py:520-546, 598-626 and
# Chebyshev.py:551-577, 629-656.  The test functions are restated from the
# reference's stencils (Legendre.py LegPhi_1 {0: 1/2, 2: -1/2}, LegPhi_2
# {0: 1/(2(2k+3)), 2: -(2k+5)/((2k+7)(2k+3)), 4: 1/(2(2k+7))}; Chebyshev.py
# ChebPhi_1 {0: 1/(pi(k+1)), 2: -1/(pi(k+1))}, ChebPhi_2 {0: 1/(2 pi (k+1)(k+2)),
# 2: -1/(pi (k^2+4k+3)), 4: 1/(2 pi (k+2)(k+3))}) on N+1 resp. N+2 orthogonal
# modes; the trial spaces are the orthogonal one, the left-Dirichlet stencil
# {0: 1, 1: 1} and the homogeneous Dirichlet composite {0: 1, 2: -1}.
# ---------------------------------------------------------------------------


def _pg_matrix(family, N, order, trial_stencil):
    M = N + order  # orthogonal modes of the test space
    Nq = N + order + 2
    big = O.Space1D(family, M)
    x, w = big.quad(Nq)
    P = big.vandermonde_orth(x, 0)  # (Nq, M)
    k = np.arange(M - 2 * order, dtype=np.float64)
    pi = np.pi
    if family == "legendre" and order == 1:
        st = {0: 0.5 + 0 * k, 2: -0.5 + 0 * k}
    elif family == "legendre":
        st = {0: 1 / (2 * (2 * k + 3)), 2: -(2 * k + 5) / (2 * k + 7) / (2 * k + 3),
              4: 1 / (2 * (2 * k + 7))}
    elif order == 1:
        st = {0: 1 / pi / (k + 1), 2: -1 / pi / (k + 1)}
    else:
        st = {0: 1 / (2 * pi * (k + 1) * (k + 2)), 2: -1 / (pi * (k**2 + 4 * k + 3)),
              4: 1 / (2 * pi * (k + 2) * (k + 3))}
    S = np.zeros((len(k), M))
    for off, c in st.items():
        S[np.arange(len(k)), np.arange(len(k)) + off] = c
    phi = P @ S.T  # test functions at the nodes
    V = O.Space1D(family, N).vandermonde_orth(x, order)  # trial derivatives
    n_trial = N - max(trial_stencil)
    T = np.zeros((n_trial, N))
    for off, c in trial_stencil.items():
        T[np.arange(n_trial), np.arange(n_trial) + off] = c
    return (phi.T * w[None, :]) @ (V @ T.T)


@pytest.mark.parametrize("family", ["legendre", "chebyshev"])
def test_petrov_galerkin_docstring_matrices(family):
    ident1 = np.eye(5, 6, k=1)
    A = _pg_matrix(family, 6, 1, {0: 1.0})
    np.testing.assert_allclose(A, ident1, atol=1e-13)
    A = _pg_matrix(family, 6, 1, {0: 1.0, 1: 1.0})  # {"left": {"D": 0}}
    np.testing.assert_allclose(A, np.eye(5) + np.eye(5, k=1), atol=1e-13)
    ident2 = np.eye(5, 7, k=2)
    A = _pg_matrix(family, 7, 2, {0: 1.0})
    np.testing.assert_allclose(A, ident2, atol=1e-12)
    # the homogeneous Dirichlet composite of the GPU path (phi_k = P_k - P_{k+2})
    A = _pg_matrix(family, 7, 2, {0: 1.0, 2: -1.0})
    np.testing.assert_allclose(A, -np.eye(5) + np.eye(5, k=2), atol=1e-12)
