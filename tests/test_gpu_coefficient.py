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
