"""Uneven-N Dirichlet Helmholtz batches (benchmark configuration 2 shape):
structured FP64 operator apply (<= 1e-12 vs the oracle's dense matrices) and
the mixed-precision solve with FP64 refinement (<= 1e-10 vs the oracle's
dense Kronecker / general-eigenvector FD solve)."""

import numpy as np
import pytest
import torch

from jaxfun_gb300.la.helmholtz import UnevenHelmholtzSolver, helmholtz_apply
from oracle import spectral as O

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("family", ["legendre", "chebyshev"])
@pytest.mark.parametrize("N", [8, 17, 64])
def test_structured_apply_matches_dense(family, N):
    Vo = O.Space1D(family, N, True)
    K, M = Vo.stiffness_matrix(), Vo.mass_matrix()
    rng = np.random.default_rng(N)
    u = rng.standard_normal((3, N - 2, N - 2))
    a2 = np.array([0.0, 3.0, 2500.0])
    v = helmholtz_apply(family, N, a2, u).cpu().numpy()
    for b in range(3):
        ref = O.tp_apply([(a2[b], [M, M]), (1.0, [K, M]), (1.0, [M, K])], u[b])
        assert np.abs(v[b] - ref).max() < 1e-12 * np.abs(ref).max()


@pytest.mark.parametrize("mode", ["grouped", "grouped_tuned", "per_group"])
@pytest.mark.parametrize("family", ["legendre", "chebyshev"])
def test_uneven_batch_solve(family, mode):
    rng = np.random.default_rng(11)
    Ns = rng.choice([16, 32, 48, 64], size=10)
    alphas = rng.uniform(0, 50, size=10)
    rhs = []
    for N in Ns:
        fh = O.forcing_coeffs(rng, N, 2)[: N - 2, : N - 2]
        rhs.append(fh)
    S = UnevenHelmholtzSolver(family, Ns, alphas)
    # grouped on a side stream (graph-captured refinement step); tuned on the
    # default stream (steps launched directly)
    stream = torch.cuda.Stream() if mode == "grouped" else torch.cuda.current_stream()
    with torch.cuda.stream(stream):
        if mode == "grouped_tuned":
            cfg = S.autotune(reps=1)
            assert cfg["pass_ms"] > 0
        if mode == "per_group":
            xs, refs = S.solve_per_group(rhs, tol=1e-12)
        else:
            xs, refs = S.solve(rhs, tol=1e-12)
    torch.cuda.synchronize()
    for b, N in enumerate(Ns):
        Vo = O.Space1D(family, N, True)
        K, M = Vo.stiffness_matrix(), Vo.mass_matrix()
        terms = [(alphas[b] ** 2, [M, M]), (1.0, [K, M]), (1.0, [M, K])]
        if N <= 48:
            ref = O.kron_solve(terms, rhs[b])
        else:
            if family == "legendre":
                lam, W = O.fd_factor_symmetric(K, M)
                E = W.T
            else:
                lam, W, E = O.fd_factor_general(K, M)
            ref = O.fd_solve(rhs[b], [W, W], [E, E], [lam, lam], c0=alphas[b] ** 2)
        x = xs[b].cpu().numpy()
        assert np.abs(x - ref).max() < 1e-10 * np.abs(ref).max(), (N, refs[b])
    assert refs.min() >= 1
