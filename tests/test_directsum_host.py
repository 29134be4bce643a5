"""Inhomogeneous Dirichlet data (DirectSum / DirectSumTPS): oracle known
answers and the host-side FP64 setup of the product against the oracle.

No GPU: the lifting coefficients, the lift and every affine map's (matrices,
constant) pair are host FP64 setup; they are checked here by applying them
with NumPy.  The device path (one affine contraction per transform) is
checked in test_gpu_directsum.py.
"""

import numpy as np
import pytest

from jaxfun_gb300.galerkin import (
    BCValue,
    Chebyshev,
    Composite,
    DirectSum,
    DirectSumTPS,
    FunctionSpace,
    Legendre,
    TensorProduct,
)
from jaxfun_gb300.galerkin.tensorproductspace import kron_apply_host
from jaxfun_gb300.la.varcoef import helmholtz_lifting
from oracle import spectral as O

ULP1 = np.spacing(1.0)
ULP100 = np.spacing(100.0)
ULP1000 = np.spacing(1000.0)
CLS = {"legendre": Legendre, "chebyshev": Chebyshev}


def _mk(fam, N, bc):
    if bc == "orth":
        return CLS[fam](N)
    if bc is None:
        return FunctionSpace(N, CLS[fam], bcs={"left": {"D": 0}, "right": {"D": 0}})
    return FunctionSpace(N, CLS[fam], bcs={"left": {"D": bc[0]}, "right": {"D": bc[1]}})


def _gauss2(x, y):
    # exp(-(X^2 + Y^2)) of examples/helmholtz2D.py on (0, 1)^2, X = (x + 1)/2
    return np.exp(-(((x + 1) / 2) ** 2 + ((y + 1) / 2) ** 2))


def _f3(x, y, z):
    return np.sin(np.pi * x) * np.exp(0.5 * y + 0.3 * z)


CASES = {
    "ds_x_orth": lambda f: [(f, 8, (1.0, 2.0)), (f, 9, "orth")],
    "two_const": lambda f: [(f, 5, (1.0, 2.0)), (f, 6, (3.0, 4.0))],
    "one_func": lambda f: [(f, 10, None),
                           (f, 12, (lambda x, y: np.exp(-x**2), lambda x, y: np.cos(x)))],
    "two_func": lambda f: [(f, 16, (_gauss2, _gauss2)), (f, 14, (_gauss2, _gauss2))],
    "3d_y": lambda f: [(f, 10, None), (f, 12, (_f3, _f3)), (f, 11, None)],
    "3d_z": lambda f: [(f, 10, None), (f, 12, None), (f, 11, (_f3, _f3))],
    "3d_yz": lambda f: [(f, 10, None), (f, 12, (_f3, _f3)), (f, 11, (_f3, _f3))],
    "3d_orth_yz": lambda f: [(f, 10, "orth"), (f, 12, (_f3, _f3)), (f, 11, (_f3, _f3))],
}


def _hb(key):
    return tuple("b" if type(s).__name__ == "BCGeneric" else "h" for s in key)


def test_bc_basis_known_answers():
    """Each boundary function is 1 at its own end and 0 at the other
    (get_bc_basis, composite.py:835-880); the product's basis is the same."""
    for fam in ("legendre", "chebyshev"):
        B = O.bc_basis(fam, 7)
        V = O.Space1D(fam, 7).vandermonde_orth(np.array([-1.0, 1.0]))
        np.testing.assert_allclose(V @ B.T, np.eye(2), atol=1e-15)
        D = _mk(fam, 7, (1.0, 2.0))
        np.testing.assert_array_equal(D[1].S, B)


def test_oracle_directsum_endpoint_values():
    """FunctionSpace(6, Legendre, bcs={left: 1, right: 2}) evaluates to 1 and 2
    at the ends with zero coefficients (test_additional_coverage.py:106-117)."""
    for fam in ("legendre", "chebyshev"):
        D = O.DirectSum1D(fam, 6, 1.0, 2.0)
        np.testing.assert_allclose(D.evaluate([-1.0, 1.0], np.zeros(4)), [1.0, 2.0], atol=1e-15)


def test_oracle_directsum_roundtrip():
    """TensorProduct(DirectSum, Legendre): forward(backward(U)) == U
    (test_tensorproductspace_more.py:38-50)."""
    T = O.LiftedTPS([("legendre", 5, (1.0, 2.0)), ("legendre", 5, "orth")])
    U = np.random.default_rng(1).standard_normal((3, 5))
    np.testing.assert_allclose(T.forward(T.backward(U)), U, atol=1e-13)


@pytest.mark.parametrize("fam", ["legendre", "chebyshev"])
def test_oracle_helmholtz2d_manufactured(fam):
    """examples/helmholtz2D.py:22-51 on the reference square: Delta u + u = f
    on (0,1)^2 with u = exp(-(x^2+y^2)) on the boundary, N = 50; mapped to
    [-1,1]^2 it reads -Delta u - u/4 = -f/4.  The reference asserts
    ||u - ue|| / 100 < ulp(1000) on a 100 x 100 uniform mesh."""
    N = 50
    T = O.LiftedTPS([(fam, N, (_gauss2, _gauss2)), (fam, N, (_gauss2, _gauss2))])
    X, Y = np.meshgrid(*T.mesh, indexing="ij")
    Xp, Yp = (X + 1) / 2, (Y + 1) / 2
    f = (4 * Xp**2 + 4 * Yp**2 - 3) * np.exp(-(Xp**2 + Yp**2))
    b = T.helmholtz_rhs(-f / 4, -0.25)
    V = T.hom[0]
    K, M = V.stiffness_matrix(), V.mass_matrix()
    c = O.kron_solve([(-0.25, [M, M]), (1.0, [K, M]), (1.0, [M, K])], b)
    xu = np.linspace(-1, 1, 100)
    XU, YU = np.meshgrid(xu, xu, indexing="ij")
    err = np.linalg.norm(T.evaluate_grid([xu, xu], c) - _gauss2(XU, YU)) / 100
    assert err < ULP1000, err


def test_oracle_two_inhomogeneous_point_value():
    """Project exp(-(x^2+y^2)) onto the lifted N = 16 Legendre product and
    evaluate at the centre (test_tensorproductspace_more.py:83-98: < ulp(100))."""
    T = O.LiftedTPS([("legendre", 16, (_gauss2, _gauss2)), ("legendre", 16, (_gauss2, _gauss2))])
    X, Y = np.meshgrid(*T.mesh, indexing="ij")
    c = T.forward(_gauss2(X, Y))
    u0 = T.evaluate_grid([np.array([0.0]), np.array([0.0])], c)[0, 0]
    assert abs(u0 - _gauss2(0.0, 0.0)) < ULP100


@pytest.mark.parametrize("fam", ["legendre", "chebyshev"])
@pytest.mark.parametrize("case", list(CASES))
def test_lifting_setup_matches_oracle(fam, case):
    """bndvals (every mixed product space), the lift and the affine maps'
    FP64 host operands against the oracle's DirectSumTPS."""
    axes = CASES[case](fam)
    T = TensorProduct(*[_mk(*a) for a in axes])
    assert isinstance(T, DirectSumTPS)
    ot = O.LiftedTPS(axes)
    assert {_hb(k) for k in T.bndvals} == set(ot.bndvals)
    for key, v in T.bndvals.items():
        ov = ot.bndvals[_hb(key)]
        assert v.shape == ov.shape
        np.testing.assert_allclose(v, ov, atol=1e-13 * max(1.0, np.abs(ov).max()))
    np.testing.assert_allclose(T.lift, ot.lift(), atol=1e-13 * max(1.0, np.abs(T.lift).max()))
    rng = np.random.default_rng(7)
    c = rng.standard_normal(T.dim)
    uo = ot.backward(c)
    scale = np.abs(uo).max()
    mats, shift = T.affine_map("quadrature")
    np.testing.assert_allclose(kron_apply_host(mats, c) + shift, uo, atol=1e-12 * scale)
    mats, shift = T.affine_map("forward", T.shape)
    np.testing.assert_allclose(kron_apply_host(mats, uo) + shift, ot.forward(uo),
                               atol=1e-12 * max(1.0, np.abs(c).max()))
    mats, shift = T.affine_map("to_orthogonal")
    a = kron_apply_host(mats, c) + shift
    np.testing.assert_allclose(a, ot.to_orthogonal(c), atol=1e-13 * np.abs(a).max())
    mats, shift = T.affine_map("from_orthogonal")
    np.testing.assert_allclose(kron_apply_host(mats, a) + shift, ot.from_orthogonal(a),
                               atol=1e-12)


@pytest.mark.parametrize("fam", ["legendre", "chebyshev"])
@pytest.mark.parametrize("alpha2", [0.0, -0.25, 3.0])
def test_lifting_rhs_matches_oracle(fam, alpha2):
    """-a(lift, v): closed-form rectangular stiffness/mass (product) against
    the quadrature of inner.py:887-909 (oracle).  The oracle's quadrature of
    the Chebyshev second derivatives (entries ~N^4) is the noisier side."""
    T = TensorProduct(_mk(fam, 20, (_gauss2, _gauss2)), _mk(fam, 22, (_gauss2, _gauss2)))
    ot = O.LiftedTPS([(fam, 20, (_gauss2, _gauss2)), (fam, 22, (_gauss2, _gauss2))])
    _, shift = helmholtz_lifting(T, alpha2)
    ref = ot.helmholtz_rhs(np.zeros((20, 22)), alpha2)
    tol = 1e-12 if fam == "legendre" else 1e-10
    np.testing.assert_allclose(shift, ref, atol=tol * np.abs(ref).max())


def test_bc_value_forms_agree():
    """Numbers, callables and sympy expressions are the same boundary data."""
    sp = pytest.importorskip("sympy")
    x, y = sp.symbols("x y")
    xs = np.linspace(-1, 1, 7)
    vals = [BCValue(lambda x, y: np.exp(-x**2) * (1 + 0 * y)), BCValue(sp.exp(-x**2))]
    a, b = (v(xs, np.array(1.0)) for v in vals)
    np.testing.assert_allclose(a, b, rtol=1e-15)
    assert BCValue(sp.Integer(3)).is_constant
    np.testing.assert_array_equal(BCValue(2.5)(xs, np.array(0.0)), np.full(7, 2.5))
    T1 = TensorProduct(_mk("legendre", 8, None),
                       _mk("legendre", 9, (sp.exp(-x**2), sp.cos(x))))
    T2 = TensorProduct(_mk("legendre", 8, None),
                       _mk("legendre", 9, (lambda x, y: np.exp(-x**2),
                                           lambda x, y: np.cos(x))))
    np.testing.assert_allclose(T1.lift, T2.lift, atol=1e-15)


def test_factory_and_errors():
    """FunctionSpace returns a Composite for zero data and a DirectSum
    otherwise (functionspace.py:63-173); 3-D products cannot start with a
    DirectSum (tensorproductspace.py:617-620); the lifted product has no
    scalar product (:796-799)."""
    assert isinstance(_mk("legendre", 6, (0.0, 0.0)), Composite)
    D = _mk("legendre", 6, (1.0, 2.0))
    assert isinstance(D, DirectSum) and D.dim == 4
    np.testing.assert_array_equal(D.bnd_vals(), [1.0, 2.0])
    with pytest.raises(ValueError):
        TensorProduct(D, _mk("legendre", 6, None), _mk("legendre", 6, None))
    T = TensorProduct(_mk("legendre", 6, None), D)
    with pytest.raises(RuntimeError):
        T.scalar_product(np.zeros(T.shape))
    with pytest.raises(NotImplementedError):
        FunctionSpace(6, Legendre, bcs={"left": {"N": 1}, "right": {"D": 0}})
    assert np.all(np.isfinite(T.lift)) and T.dim == (4, 4)
    # machine-precision constants used by the device tests' bars
    assert ULP1 < ULP100 < ULP1000
