"""Inhomogeneous Dirichlet data on the GPU: DirectSum / DirectSumTPS
transforms (one affine contraction each, ``jfg_tp_apply_affine_f64``)
against the oracle, the reference's DirectSum known answers, and
manufactured solutions solved through ``helmholtz_system`` + the fast
diagonalisation solve.  FP64 throughout; tolerances are stated per test."""

import numpy as np
import pytest
import torch

from jaxfun_gb300.galerkin import (
    Chebyshev,
    DirectSumTPS,
    FunctionSpace,
    Legendre,
    TensorProduct,
    tp_apply_affine,
)
from jaxfun_gb300.galerkin.tensorproductspace import kron_apply_host
from jaxfun_gb300.la import helmholtz_system
from oracle import spectral as O
from test_directsum_host import CASES, _gauss2, _mk

pytestmark = pytest.mark.gpu

ULP100 = np.spacing(100.0)
ULP1000 = np.spacing(1000.0)
CLS = {"legendre": Legendre, "chebyshev": Chebyshev}


def _np(t):
    return t.cpu().numpy()


@pytest.mark.parametrize("fam", ["legendre", "chebyshev"])
def test_directsum_1d_vs_oracle(fam):
    """DirectSum backward / forward / to_orthogonal / from_orthogonal
    (composite.py:585-621) and the end values 1 and 2 with zero coefficients
    (test_additional_coverage.py:106-117).  Bar: 1e-13 relative."""
    D = FunctionSpace(12, CLS[fam], bcs={"left": {"D": 1.0}, "right": {"D": 2.0}})
    od = O.DirectSum1D(fam, 12, 1.0, 2.0)
    rng = np.random.default_rng(3)
    c = rng.standard_normal(10)
    u = od.backward(c)
    np.testing.assert_allclose(_np(D.backward(c)), u, atol=1e-13 * np.abs(u).max())
    np.testing.assert_allclose(_np(D.forward(u)), od.forward(u), atol=1e-13)
    a = od.to_orthogonal(c)
    np.testing.assert_allclose(_np(D.to_orthogonal(c)), a, atol=1e-14 * np.abs(a).max())
    np.testing.assert_allclose(_np(D.from_orthogonal(a)), od.from_orthogonal(a), atol=1e-13)
    ends = _np(D.evaluate([-1.0, 1.0], np.zeros(10)))
    np.testing.assert_allclose(ends, [1.0, 2.0], atol=1e-15)


@pytest.mark.parametrize("fam", ["legendre", "chebyshev"])
@pytest.mark.parametrize("case", list(CASES))
def test_directsum_tps_vs_oracle(fam, case):
    """Every lifted transform of a batch of 3 fields (one shift broadcast to
    all) against the oracle's DirectSumTPS.  Bar: 1e-12 relative."""
    axes = CASES[case](fam)
    T = TensorProduct(*[_mk(*a) for a in axes])
    ot = O.LiftedTPS(axes)
    rng = np.random.default_rng(11)
    c = rng.standard_normal((3,) + T.dim)
    u = _np(T.backward(c))
    uo = np.stack([ot.backward(ci) for ci in c])
    np.testing.assert_allclose(u, uo, atol=1e-12 * np.abs(uo).max())
    cf = _np(T.forward(uo))
    cfo = np.stack([ot.forward(ui) for ui in uo])
    np.testing.assert_allclose(cf, cfo, atol=1e-12 * max(1.0, np.abs(cfo).max()))
    np.testing.assert_allclose(cf, c, atol=1e-11 * max(1.0, np.abs(c).max()))
    a = _np(T.to_orthogonal(c))
    ao = np.stack([ot.to_orthogonal(ci) for ci in c])
    np.testing.assert_allclose(a, ao, atol=1e-13 * np.abs(ao).max())
    np.testing.assert_allclose(_np(T.from_orthogonal(ao)),
                               np.stack([ot.from_orthogonal(ai) for ai in ao]), atol=1e-12)


def test_tpspaces_sum_equals_backward():
    """Summing every product space's backward (and derivative) of its
    bndvals - or of c for the homogeneous one - gives the lifted backward
    (test_tensorproductspace_extra.py:230-262, bar sqrt(ulp(100)))."""
    T = TensorProduct(_mk("legendre", 5, (1.0, 2.0)), _mk("legendre", 6, (3.0, 4.0)))
    assert isinstance(T, DirectSumTPS)
    c = np.random.default_rng(0).standard_normal(T.dim)
    bar = np.sqrt(ULP100)
    z0 = sum(_np(v.backward(T.bndvals.get(f, c))) for f, v in T.tpspaces.items())
    assert np.linalg.norm(z0 - _np(T.backward(c))) < bar
    z0 = sum(_np(v.backward_derivative(T.bndvals.get(f, c), (1, 1)))
             for f, v in T.tpspaces.items())
    assert np.linalg.norm(z0 - _np(T.backward_derivative(c, (1, 1)))) < bar
    z0 = sum(_np(v.evaluate_mesh(T.bndvals.get(f, c), "uniform", (5, 6)))
             for f, v in T.tpspaces.items())
    assert np.linalg.norm(z0 - _np(T.evaluate_mesh(c, "uniform", (5, 6)))) < bar


def test_to_orthogonal_consistency():
    """backward(c) == orthogonal backward of to_orthogonal(c)
    (test_tensorproductspace_extra.py:194-208)."""
    T = TensorProduct(_mk("legendre", 5, (1.0, 2.0)), _mk("legendre", 6, (3.0, 4.0)))
    c = np.random.default_rng(0).standard_normal(T.dim)
    y0 = _np(T.backward(c))
    y1 = _np(T.get_orthogonal().backward(T.to_orthogonal(c)))
    assert np.linalg.norm(y0 - y1) < np.sqrt(ULP100)


def test_roundtrip_directsum_times_legendre():
    """TensorProduct(DirectSum, Legendre): forward(backward(U)) == U
    (test_tensorproductspace_more.py:38-50, jnp.allclose)."""
    T = TensorProduct(_mk("legendre", 5, (1.0, 2.0)), Legendre(5))
    U = np.random.default_rng(1).standard_normal((3, 5))
    np.testing.assert_allclose(_np(T.forward(T.backward(U))), U, rtol=1e-5, atol=1e-8)


@pytest.mark.parametrize("fam,bar", [("legendre", ULP100), ("chebyshev", 4 * ULP100)])
def test_two_inhomogeneous_point_value(fam, bar):
    """Project exp(-(x^2+y^2)) (on (0,1)^2) onto the lifted N = 16 product
    and evaluate at the centre (test_tensorproductspace_more.py:83-98: the
    reference asserts < ulp(100) for Legendre)."""
    T = TensorProduct(_mk(fam, 16, (_gauss2, _gauss2)), _mk(fam, 16, (_gauss2, _gauss2)))
    X, Y = T.mesh()
    c = T.forward(_gauss2(X, Y))
    u0 = _np(T.evaluate_mesh(c, "uniform", (3, 3)))[1, 1]
    assert abs(u0 - _gauss2(0.0, 0.0)) < bar


@pytest.mark.parametrize("fam", ["legendre", "chebyshev"])
def test_helmholtz2d_manufactured(fam):
    """examples/helmholtz2D.py:22-51: Delta u + u = f on (0,1)^2 with
    u = exp(-(x^2+y^2)) on the boundary, N = 50, mapped to [-1,1]^2
    (-Delta u - u/4 = -f/4); right-hand side with the lift moved over,
    fast-diagonalisation solve on the GPU, lifted evaluation on a 100 x 100
    uniform mesh.  The reference asserts ||u - ue|| / 100 < ulp(1000)."""
    N = 50
    T = TensorProduct(_mk(fam, N, (_gauss2, _gauss2)), _mk(fam, N, (_gauss2, _gauss2)))
    X, Y = T.mesh()
    Xp, Yp = (X + 1) / 2, (Y + 1) / 2
    f = (4 * Xp**2 + 4 * Yp**2 - 3) * np.exp(-(Xp**2 + Yp**2))
    A, b = helmholtz_system(T, -f / 4, alpha2=-0.25)
    c = A.solve(b)
    uj = _np(T.evaluate_mesh(c, "uniform", (100, 100)))
    xu = np.linspace(-1, 1, 100)
    XU, YU = np.meshgrid(xu, xu, indexing="ij")
    err = np.linalg.norm(uj - _gauss2(XU, YU)) / 100
    assert err < ULP1000, err
    # the coefficients against the oracle's dense solve of its own
    # quadrature-assembled system; the high Chebyshev modes of b carry
    # rounding amplified by the N^3 stiffness entries, which the solve damps
    ot = O.LiftedTPS([(fam, N, (_gauss2, _gauss2)), (fam, N, (_gauss2, _gauss2))])
    bo = ot.helmholtz_rhs(-f / 4, -0.25)
    V = ot.hom[0]
    K, M = V.stiffness_matrix(), V.mass_matrix()
    co = O.kron_solve([(-0.25, [M, M]), (1.0, [K, M]), (1.0, [M, K])], bo)
    np.testing.assert_allclose(_np(c), co, atol=1e-12 * np.abs(co).max())


@pytest.mark.parametrize("fam", ["legendre", "chebyshev"])
def test_poisson3d_two_inhomogeneous(fam):
    """test_tensorproductspace_extra.py:48-81 with the Fourier axis replaced
    by a homogeneous Dirichlet axis: -Delta u = f with u = (1 - x^2)
    exp(y/2 + z/3) on the y and z boundaries, N = 20.  Bars as the
    reference: ||u - ue|| < sqrt(ulp(1)) and ||forward(u) - uh|| < ulp(1000)
    (scaled by ||uh||)."""
    def ue(x, y, z):
        return (1 - x**2) * np.exp(y / 2 + z / 3)

    N = 20
    T = TensorProduct(_mk(fam, N, None), _mk(fam, N, (ue, ue)), _mk(fam, N, (ue, ue)))
    X, Y, Z = T.mesh()
    f = (2 * np.exp(Y / 2 + Z / 3) - (1 / 4 + 1 / 9) * ue(X, Y, Z))
    A, b = helmholtz_system(T, f)
    uh = A.solve(b)
    uj = _np(T.backward(uh))
    assert np.linalg.norm(uj - ue(X, Y, Z)) < np.sqrt(np.spacing(1.0))
    back = _np(T.forward(uj))
    assert np.linalg.norm(back - _np(uh)) < ULP1000 * max(1.0, np.linalg.norm(_np(uh)))


def test_affine_apply_batch_broadcast():
    """out[b] = (x_ax mats) x[b] + shift for every b (one shift, batch 4)."""
    rng = np.random.default_rng(5)
    mats = [rng.standard_normal((7, 5)), rng.standard_normal((6, 4)), rng.standard_normal((3, 9))]
    for m in mats:
        m.setflags(write=False)
    shift = rng.standard_normal((7, 6, 3))
    x = rng.standard_normal((4, 5, 4, 9))
    out = _np(tp_apply_affine(mats, torch.as_tensor(x, device="cuda"), shift, cache=False))
    ref = np.stack([kron_apply_host(mats, xi) + shift for xi in x])
    np.testing.assert_allclose(out, ref, atol=1e-13 * np.abs(ref).max())
