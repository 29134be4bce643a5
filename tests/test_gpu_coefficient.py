"""The coefficient evaluated from its logarithm (VarCoefMatrix.from_log /
from_expansion: fused exp + quadrature weighting, per-problem moments)
against kappa = exp(g) built on the host and against the oracle's backward
transform and variable-coefficient apply.  FP64; tolerances per test."""

import numpy as np
import pytest

from jaxfun_gb300.galerkin import DIRICHLET, FunctionSpace, Legendre, TensorProduct
from jaxfun_gb300.la import VarCoefMatrix
from oracle import spectral as O

pytestmark = pytest.mark.gpu


def _space(N, nd):
    D = FunctionSpace(N, Legendre, bcs=DIRICHLET)
    return TensorProduct(*([D] * nd))


@pytest.mark.parametrize("nd,N", [(2, 24), (3, 12)])
def test_from_log_matches_exp(nd, N):
    T = _space(N, nd)
    rng = np.random.default_rng(4)
    g = 0.7 * rng.standard_normal((3,) + (N,) * nd)
    A1 = VarCoefMatrix(T, np.exp(g))
    A2 = VarCoefMatrix.from_log(T, g)
    kw1, kw2 = A1.kw.cpu().numpy(), A2.kw.cpu().numpy()
    assert np.abs(kw1 - kw2).max() <= 1e-15 * np.abs(kw1).max()
    np.testing.assert_allclose(A2.kappa.cpu().numpy(), np.exp(g), rtol=1e-15)
    u = rng.standard_normal((3,) + (N - 2,) * nd)
    v1, v2 = (A1 @ u).cpu().numpy(), (A2 @ u).cpu().numpy()
    assert np.abs(v1 - v2).max() <= 1e-14 * np.abs(v1).max()


def test_from_expansion_standardized_vs_oracle():
    """g from seeded Legendre coefficients (the variable-coefficient recipe:
    backward to the grid, standardise, exponentiate), then the operator
    apply, against the oracle (1e-12 relative)."""
    N = 20
    T = _space(N, 2)
    rng = np.random.default_rng(9)
    gh = np.stack([O.random_field_coeffs(rng, N, 2) for _ in range(2)])
    A = VarCoefMatrix.from_expansion(T, gh, standardize=True)
    Vo = O.Space1D("legendre", N, True)
    Voo = O.Space1D("legendre", N, False)
    for b in range(2):
        g = O.tp_backward([Voo, Voo], gh[b])
        g = (g - g.mean()) / g.std()
        kap = np.exp(g)
        assert np.abs(A.kappa[b].cpu().numpy() - kap).max() <= 1e-12 * kap.max()
        u = rng.standard_normal((N - 2, N - 2))
        vo = O.varcoef_apply(Vo, kap, u)
        A1 = VarCoefMatrix.from_expansion(T, gh[b:b + 1], standardize=True)
        v = (A1 @ u[None]).cpu().numpy()[0]
        assert np.abs(v - vo).max() <= 1e-12 * np.abs(vo).max()


@pytest.mark.parametrize("standardize", [False, True])
@pytest.mark.parametrize("nd,N,batch", [(2, 40, 3), (2, 130, 2), (3, 14, 2)])
def test_fused_backward_matches_unfused(nd, N, batch, standardize):
    """from_expansion (backward transform with exp and the weights in its last
    pass's epilogue; standardised: per-tile moments there, combined pairwise)
    against the unfused sequence -- backward transform, two-pass moments,
    exp-weighting kernel -- on the same coefficients: kappa and kappa w to
    1e-14 relative (the standardisation's rounding differs by an ulp or so,
    and exp carries it), the operator apply to 1e-13."""
    T = _space(N, nd)
    rng = np.random.default_rng(11 + N)
    gh = np.stack([O.random_field_coeffs(rng, N, nd) for _ in range(batch)])
    A1 = VarCoefMatrix.from_expansion(T, gh, standardize=standardize)
    A2 = VarCoefMatrix.from_log(T, T.get_orthogonal().backward(gh), standardize=standardize)
    for a, b in ((A1.kappa, A2.kappa), (A1.kw, A2.kw)):
        a, b = a.cpu().numpy(), b.cpu().numpy()
        assert np.abs(a - b).max() <= 1e-14 * np.abs(b).max(), np.abs(a - b).max()
    if standardize:
        g = np.log(A1.kappa.cpu().numpy()).reshape(batch, -1)
        assert np.abs(g.mean(axis=1)).max() < 1e-13 and np.abs(g.std(axis=1) - 1).max() < 1e-13
    u = rng.standard_normal((batch,) + (N - 2,) * nd)
    v1, v2 = (A1 @ u).cpu().numpy(), (A2 @ u).cpu().numpy()
    assert np.abs(v1 - v2).max() <= 1e-13 * np.abs(v2).max()


@pytest.mark.parametrize("nd,N", [(2, 48), (3, 16)])
def test_rhs_from_expansion(nd, N):
    """scalar_product_expansion (the backward transform of f's orthogonal
    coefficients fused with the scalar product: one tensor-product apply)
    against backward then scalar_product on the GPU (1e-13) and against the
    oracle's two-step restatement (1e-12)."""
    T = _space(N, nd)
    rng = np.random.default_rng(5 + nd)
    fh = np.stack([O.forcing_coeffs(rng, N, nd) for _ in range(2)])
    b1 = T.scalar_product_expansion(fh).cpu().numpy()
    b2 = T.scalar_product(T.get_orthogonal().backward(fh)).cpu().numpy()
    assert np.abs(b1 - b2).max() <= 1e-13 * np.abs(b2).max()
    Vd = O.Space1D("legendre", N, True)
    Vo = O.Space1D("legendre", N, False)
    for i in range(2):
        ref = O.tp_scalar_product([Vd] * nd, O.tp_backward([Vo] * nd, fh[i]))
        assert np.abs(b1[i] - ref).max() <= 1e-12 * np.abs(ref).max()
