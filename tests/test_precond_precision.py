"""CPU check of the precision argument behind the plain-BF16 preconditioner
passes: the oracle's FP64 PCG on the variable-coefficient Poisson operator,
preconditioned by the constant-coefficient fast diagonalisation computed
exactly, or with every pass's operator and input rounded to BF16 (one
product per term, FP32 accumulation), reaches the inner tolerance of the
mixed solve (5e-6) in the same number of iterations.  Problems are the
benchmark's seeded recipe (log-normal kappa, decaying forcing) at N = 64."""

import numpy as np
import pytest

from oracle import spectral as O


def bf16(a):
    """Round to BF16 (nearest even), returned as FP64."""
    u = np.ascontiguousarray(a, dtype=np.float32).view(np.uint32).astype(np.uint64)
    u = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def problem(seed, N):
    rng = np.random.default_rng(seed)
    k2 = np.add.outer(np.arange(N) ** 2.0, np.arange(N) ** 2.0)
    gh = rng.standard_normal((N, N)) * (1.0 + k2) ** -1.5
    s = np.outer((1.0 + np.arange(N)) ** -2.0, (1.0 + np.arange(N)) ** -2.0)
    fh = rng.standard_normal((N, N)) * s
    Vo = O.Space1D("legendre", N)
    g = O.tp_backward([Vo, Vo], gh)
    g = (g - g.mean()) / g.std()
    return np.exp(g), O.tp_backward([Vo, Vo], fh)


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_plain_bf16_fd_preconditioner_keeps_pcg_iterations(seed):
    N = 64
    V = O.Space1D("legendre", N, dirichlet=True)
    lam, W = O.fd_factor_symmetric(V.stiffness_matrix(), V.mass_matrix())
    E = W.T  # W^T M W = I: (K x M + M x K)^-1 = (W x W) D^-1 (W^T x W^T)
    kap, f = problem(seed, N)
    b = O.tp_scalar_product([V, V], f)
    D = kap.mean() * (lam[:, None] + lam[None, :])

    def contract(op, x, plain):
        if not plain:
            return op @ x
        return (bf16(op) @ bf16(x)).astype(np.float32).astype(np.float64)

    def fd(plain):
        def apply(R):
            F = contract(E, contract(E, R, plain).T, plain).T / D
            return contract(W, contract(W, F, plain).T, plain).T
        return apply

    A = lambda U: O.varcoef_apply(V, kap, U)  # noqa: E731
    its = {}
    for plain in (False, True):
        x, it = O.pcg(A, b, fd(plain), tol=5e-6, maxiter=500)
        r = b - A(x)
        assert np.linalg.norm(r) / np.linalg.norm(b) < 5e-5
        its[plain] = it
    assert abs(its[True] - its[False]) <= 1, its
