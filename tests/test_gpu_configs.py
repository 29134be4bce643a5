"""Parity cases shaped like the benchmark configurations (reduced sizes where
the oracle would be slow):

  config 0  2-D Poisson, Legendre Dirichlet N=64: scalar product, FD solve,
            backward, forward, each against the oracle (<= 1e-12 relative).
  config 1  batched 3-D Chebyshev transforms: FP64 path (<= 1e-12) and the
            split-TF32 tensor-core path (<= 2e-5 relative) on a round trip.
  config 2  uneven Chebyshev Helmholtz batch: FD solves at several N with
            per-problem alpha against the oracle's dense Kronecker solve.
  config 4  3-D variable-coefficient Poisson: mixed-precision solve <= 1e-10
            against a tight FP64 solve.
"""

import numpy as np
import pytest

from jaxfun_gb300.galerkin import DIRICHLET, Chebyshev, FunctionSpace, Legendre, TensorProduct
from jaxfun_gb300.la import MixedVarCoefSolver, VarCoefMatrix, pcg, poisson_tpmatrices
from oracle import spectral as O

pytestmark = pytest.mark.gpu


def rel(a, b):
    a = a.detach().cpu().numpy() if hasattr(a, "detach") else a
    return np.abs(a - b).max() / np.abs(b).max()


def test_config0_poisson_legendre_n64():
    N = 64
    D = FunctionSpace(N, Legendre, bcs=DIRICHLET)
    T = TensorProduct(D, D)
    Lo = Legendre(N)
    To = TensorProduct(Lo, Lo)
    Vo = O.Space1D("legendre", N, True)
    Voo = O.Space1D("legendre", N, False)
    fh = O.forcing_coeffs(np.random.default_rng(0), N, 2)
    f_ref = O.tp_backward([Voo, Voo], fh)
    f = To.backward(fh)
    assert rel(f, f_ref) < 1e-12
    b_ref = O.tp_scalar_product([Vo, Vo], f_ref)
    b = T.scalar_product(f_ref)
    assert rel(b, b_ref) < 1e-12
    K, M = Vo.stiffness_matrix(), Vo.mass_matrix()
    lam, W = O.fd_factor_symmetric(K, M)
    u_ref = O.fd_solve(b_ref, [W, W], [W.T, W.T], [lam, lam])
    # the two oracle solvers agree to the conditioning of the 3844^2 Kronecker system
    assert np.abs(O.kron_solve([(1.0, [K, M]), (1.0, [M, K])], b_ref) - u_ref).max() < 1e-10 * np.abs(u_ref).max()
    u = poisson_tpmatrices(T).solve(b_ref)
    assert rel(u, u_ref) < 1e-12
    uj_ref = O.tp_backward([Vo, Vo], u_ref)
    uj = T.backward(u_ref)
    assert rel(uj, uj_ref) < 1e-12
    assert rel(T.forward(uj_ref), O.tp_forward([Vo, Vo], uj_ref)) < 1e-12


@pytest.mark.parametrize("N,fields", [(32, 3), (64, 2)])
def test_config1_chebyshev_3d_roundtrip(N, fields):
    C = Chebyshev(N)
    T = TensorProduct(C, C, C)
    Vo = O.Space1D("chebyshev", N, False)
    rng = np.random.default_rng(N)
    i = np.arange(N)
    s = 1.0 / (1.0 + i[:, None, None] + i[None, :, None] + i[None, None, :]) ** 3
    c = rng.standard_normal((fields, N, N, N)) * s
    u_ref = np.stack([O.tp_backward([Vo] * 3, c[k]) for k in range(fields)])
    u64 = T.backward(c)
    assert rel(u64, u_ref) < 1e-12
    c64 = T.forward(u64)
    assert rel(c64, c) < 1e-12
    u32 = T.backward(c, precision="tc")
    assert rel(u32, u_ref) < 2e-5
    c32 = T.forward(u32, precision="tc")
    assert rel(c32, c) < 2e-5


def test_config2_uneven_helmholtz_fd_vs_kron():
    rng = np.random.default_rng(2)
    for N in (16, 32, 48):
        V = FunctionSpace(N, Chebyshev, bcs=DIRICHLET)
        T = TensorProduct(V, V)
        Vo = O.Space1D("chebyshev", N, True)
        K, M = Vo.stiffness_matrix(), Vo.mass_matrix()
        fac = poisson_tpmatrices(T, 1.0).lu_factor()
        alpha = rng.uniform(0, 50, 3)
        b = rng.standard_normal((3, N - 2, N - 2))
        x = fac.solve(b, c0=alpha**2, c1=1.0).cpu().numpy()
        for k in range(3):
            ref = O.kron_solve([(alpha[k] ** 2, [M, M]), (1.0, [K, M]), (1.0, [M, K])], b[k])
            assert rel(x[k], ref) < 1e-11, (N, k)


def test_config4_varcoef_3d_mixed():
    N, batch = 24, 2
    V = FunctionSpace(N, Legendre, bcs=DIRICHLET)
    T = TensorProduct(V, V, V)
    rng = np.random.default_rng(4)
    kap = np.exp(rng.standard_normal((batch, N, N, N)) * 0.7)
    b = rng.standard_normal((batch, N - 2, N - 2, N - 2))
    A = VarCoefMatrix(T, kap)
    xr, _ = pcg(A, b, tol=1e-14, maxiter=3000)
    x, it_in, it_out = MixedVarCoefSolver(A).solve(b, tol=3e-12)
    for k in range(batch):
        assert rel(x[k], xr[k].cpu().numpy()) < 1e-10, (it_in, it_out)
