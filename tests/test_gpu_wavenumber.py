"""Per-wavenumber banded solves (TPMatricesWavenumberSolver mirror) against
the oracle's dense per-system solve: random diagonally dominant bands, the
polynomial axis first, last or in the middle, and the Fourier x Legendre
Helmholtz systems k^2 M + K of the reference's Poisson examples.  FP64,
tolerance 1e-12 relative."""

import numpy as np
import pytest
import torch

from jaxfun_gb300.la import TPMatricesWavenumberSolver
from oracle import spectral as O

pytestmark = pytest.mark.gpu


def _random_band(rng, n_F, n_P, offsets):
    data = rng.standard_normal((n_F, len(offsets), n_P))
    d0 = list(offsets).index(0)
    data[:, d0, :] = 2.0 * len(offsets) + np.abs(data[:, d0, :])  # diagonally dominant
    return data


def _check(shape, poly_axis, offsets, seed):
    rng = np.random.default_rng(seed)
    nd = len(shape)
    fourier = [a for a in range(nd) if a != poly_axis]
    n_F = int(np.prod([shape[a] for a in fourier]))
    n_P = shape[poly_axis]
    data = _random_band(rng, n_F, n_P, offsets)
    rhs = rng.standard_normal(shape)
    S = TPMatricesWavenumberSolver(poly_axis, shape, B_data_batch=data, poly_offsets=offsets)
    x = S.solve(rhs).cpu().numpy()
    order = fourier + [poly_axis]
    rhs_2d = np.transpose(rhs, order).reshape(n_F, n_P)
    ref = O.wavenumber_solve(data, offsets, rhs_2d)
    ref = np.transpose(ref.reshape([shape[a] for a in order]), np.argsort(order))
    assert np.abs(x - ref).max() <= 1e-12 * np.abs(ref).max()


@pytest.mark.parametrize("shape,poly_axis", [((37, 40), 1), ((40, 37), 0), ((5, 24, 7), 1),
                                              ((6, 5, 30), 2)])
@pytest.mark.parametrize("offsets", [(-2, 0, 2), (-1, 0, 1, 3), (0, 1)])
def test_wavenumber_random_bands(shape, poly_axis, offsets):
    _check(shape, poly_axis, offsets, seed=len(shape) + poly_axis + len(offsets))


def test_fourier_legendre_helmholtz():
    """B_k = k^2 M + K for the Legendre Dirichlet composite (M pentadiagonal,
    K diagonal), the per-wavenumber systems of a Fourier x Legendre Poisson
    problem; compared with the dense solve of each system."""
    N, nk = 48, 33
    V = O.Space1D("legendre", N, True)
    K, M = V.stiffness_matrix(), V.mass_matrix()
    n = N - 2
    offsets = (-2, 0, 2)
    k2 = np.arange(nk, dtype=float) ** 2
    data = np.zeros((nk, 3, n))
    for kk in range(nk):
        B = k2[kk] * M + K
        for d, off in enumerate(offsets):
            for j in range(n):
                i = j - off
                if 0 <= i < n:
                    data[kk, d, j] = B[i, j]
    rhs = np.random.default_rng(3).standard_normal((nk, n))
    S = TPMatricesWavenumberSolver(1, (nk, n), B_data_batch=data, poly_offsets=offsets)
    x = S.solve(torch.as_tensor(rhs)).cpu().numpy()
    for kk in range(nk):
        ref = np.linalg.solve(k2[kk] * M + K, rhs[kk])
        assert np.abs(x[kk] - ref).max() <= 1e-12 * np.abs(ref).max()


def test_b_matrices_constructor_matches_batched_data():
    """The reference's legacy constructor (one DIA matrix per wavenumber, with
    differing offset sets) gives the same solution as the batched band data and
    as the dense solve of each system."""
    from jaxfun_gb300.la import DiaMatrix

    rng = np.random.default_rng(17)
    nk, n = 9, 31
    dense, mats = [], []
    for kk in range(nk):
        offs = (-2, 0, 2) if kk % 2 == 0 else (-1, 0, 1, 3)
        A = np.zeros((n, n))
        for o in offs:
            A += np.diag(rng.standard_normal(n - abs(o)), o)
        A += np.diag(2.0 * len(offs) + np.abs(rng.standard_normal(n)))
        dense.append(A)
        mats.append(DiaMatrix.from_dense(A, offs))
        assert np.array_equal(mats[-1].todense(), A)
    rhs = rng.standard_normal((nk, n))
    x = TPMatricesWavenumberSolver(1, (nk, n), B_matrices=mats).solve(rhs).cpu().numpy()
    union = (-2, -1, 0, 1, 2, 3)
    data = np.stack([DiaMatrix.from_dense(A, union).data for A in dense])
    xb = TPMatricesWavenumberSolver(1, (nk, n), B_data_batch=data,
                                    poly_offsets=union).solve(rhs).cpu().numpy()
    for kk in range(nk):
        ref = np.linalg.solve(dense[kk], rhs[kk])
        assert np.abs(x[kk] - ref).max() <= 1e-12 * np.abs(ref).max()
    assert np.abs(x - xb).max() <= 1e-14 * np.abs(xb).max()
