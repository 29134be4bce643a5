"""GPU parity of the FP64 path against the oracle (<= 1e-12 relative).

Every check goes through the C ABI (ctypes over libjaxfun_gb300.so)."""

import numpy as np
import pytest
import torch

from jaxfun_gb300 import _lib
from jaxfun_gb300.galerkin import DIRICHLET, Chebyshev, FunctionSpace, Legendre, TensorProduct
from jaxfun_gb300.la import VarCoefMatrix, pcg, poisson_tpmatrices, tpmats_lu_factor
from oracle import spectral as O

pytestmark = pytest.mark.gpu
TOL = 1e-12
FAM = {"legendre": Legendre, "chebyshev": Chebyshev}


def rel(a, b):
    a = a.detach().cpu().numpy() if isinstance(a, torch.Tensor) else a
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


@pytest.mark.parametrize("fam", ["legendre", "chebyshev"])
@pytest.mark.parametrize("dirichlet", [False, True])
@pytest.mark.parametrize("ndim,N", [(1, 7), (2, 17), (2, 64), (3, 12)])
def test_transforms(fam, dirichlet, ndim, N):
    V = FunctionSpace(N, FAM[fam], bcs=DIRICHLET if dirichlet else None)
    Vo = O.Space1D(fam, N, dirichlet)
    T = TensorProduct(*([V] * ndim))
    rng = np.random.default_rng(N + ndim)
    c = rng.standard_normal((V.dim,) * ndim)
    u_ref = O.tp_backward([Vo] * ndim, c)
    u = T.backward(c)
    assert rel(u, u_ref) < TOL
    assert rel(T.forward(u_ref), O.tp_forward([Vo] * ndim, u_ref)) < TOL
    assert rel(T.scalar_product(u_ref), O.tp_scalar_product([Vo] * ndim, u_ref)) < TOL


def test_transform_batched_and_padded():
    V = FunctionSpace(16, Legendre, bcs=DIRICHLET)
    Vo = O.Space1D("legendre", 16, True)
    T = TensorProduct(V, V)
    c = np.random.default_rng(1).standard_normal((3, 2, 14, 14))
    u = T.backward(c, N=(24, 20)).cpu().numpy()
    for i in range(3):
        for j in range(2):
            assert rel(u[i, j], O.tp_backward([Vo, Vo], c[i, j], Nq=(24, 20))) < TOL


@pytest.mark.parametrize("fam,alpha2", [("legendre", 0.0), ("chebyshev", 0.0), ("chebyshev", 37.0)])
@pytest.mark.parametrize("ndim", [2, 3])
def test_fd_solve_vs_kron(fam, alpha2, ndim):
    N = 12 if ndim == 2 else 8
    V = FunctionSpace(N, FAM[fam], bcs=DIRICHLET)
    Vo = O.Space1D(fam, N, True)
    T = TensorProduct(*([V] * ndim))
    A = poisson_tpmatrices(T, alpha2)
    rng = np.random.default_rng(7)
    b = rng.standard_normal((V.dim,) * ndim)
    K, M = Vo.stiffness_matrix(), Vo.mass_matrix()
    terms = [(alpha2, [M] * ndim)] if alpha2 else []
    for ax in range(ndim):
        mats = [M] * ndim
        mats[ax] = K
        terms.append((1.0, mats))
    ref = O.kron_solve(terms, b)
    x = A.solve(b, method="lu")
    assert rel(x, ref) < 1e-11


def test_fd_solve_batched_per_problem_alpha():
    N = 32
    V = FunctionSpace(N, Chebyshev, bcs=DIRICHLET)
    Vo = O.Space1D("chebyshev", N, True)
    T = TensorProduct(V, V)
    fac = tpmats_lu_factor(poisson_tpmatrices(T, 1.0).tpmats)
    rng = np.random.default_rng(3)
    b = rng.standard_normal((5, N - 2, N - 2))
    alpha2 = rng.uniform(0, 2500, 5)
    x = fac.solve(b, c0=alpha2, c1=1.0).cpu().numpy()
    K, M = Vo.stiffness_matrix(), Vo.mass_matrix()
    lam, W, E = O.fd_factor_general(K, M)
    for i in range(5):
        ref = O.fd_solve(b[i], [W, W], [E, E], [lam, lam], c0=alpha2[i])
        assert rel(x[i], ref) < 1e-11


def test_fd_legendre_n64_vs_oracle_fd():
    N = 64
    V = FunctionSpace(N, Legendre, bcs=DIRICHLET)
    Vo = O.Space1D("legendre", N, True)
    T = TensorProduct(V, V)
    b = np.random.default_rng(5).standard_normal((62, 62))
    lam, W = O.fd_factor_symmetric(Vo.stiffness_matrix(), Vo.mass_matrix())
    ref = O.fd_solve(b, [W, W], [W.T, W.T], [lam, lam])
    assert rel(poisson_tpmatrices(T).solve(b), ref) < TOL


def test_varcoef_apply_vs_tensormatrix_2d():
    N = 12
    V = FunctionSpace(N, Legendre, bcs=DIRICHLET)
    Vo = O.Space1D("legendre", N, True)
    T = TensorProduct(V, V)
    rng = np.random.default_rng(11)
    kap = np.exp(rng.standard_normal((2, N, N)))
    U = rng.standard_normal((2, N - 2, N - 2))
    v = (VarCoefMatrix(T, kap) @ U).cpu().numpy()
    for i in range(2):
        ref = O.tensormatrix_matvec(O.varcoef_tensormatrix(Vo, kap[i]), U[i])
        assert rel(v[i], ref) < TOL


@pytest.mark.parametrize("ndim,N", [(2, 64), (3, 10), (3, 17)])
def test_varcoef_apply_vs_sumfact(ndim, N):
    V = FunctionSpace(N, Legendre, bcs=DIRICHLET)
    Vo = O.Space1D("legendre", N, True)
    T = TensorProduct(*([V] * ndim))
    rng = np.random.default_rng(ndim * 100 + N)
    kap = np.exp(rng.standard_normal((N,) * ndim))
    U = rng.standard_normal((N - 2,) * ndim)
    assert rel(VarCoefMatrix(T, kap) @ U, O.varcoef_apply(Vo, kap, U)) < TOL


@pytest.mark.parametrize("ndim,N,batch", [(2, 24, 3), (3, 10, 2)])
def test_pcg_vs_direct(ndim, N, batch):
    V = FunctionSpace(N, Legendre, bcs=DIRICHLET)
    Vo = O.Space1D("legendre", N, True)
    T = TensorProduct(*([V] * ndim))
    rng = np.random.default_rng(21)
    kap = np.exp(rng.standard_normal((batch,) + (N,) * ndim))
    b = rng.standard_normal((batch,) + (N - 2,) * ndim)
    A = VarCoefMatrix(T, kap)
    x, it = pcg(A, b, tol=1e-13, maxiter=500)
    x = x.cpu().numpy()
    n = (N - 2) ** ndim
    for i in range(batch):
        # dense operator from applying the oracle to unit vectors
        cols = [O.varcoef_apply(Vo, kap[i], e.reshape((N - 2,) * ndim)).ravel() for e in np.eye(n)]
        Ad = np.array(cols).T
        ref = np.linalg.solve(Ad, b[i].ravel()).reshape(b[i].shape)
        assert rel(x[i], ref) < 1e-10, (i, it)
    assert np.all(it > 0)


def test_pcg_matches_oracle_pcg_iterations():
    N = 32
    V = FunctionSpace(N, Legendre, bcs=DIRICHLET)
    Vo = O.Space1D("legendre", N, True)
    T = TensorProduct(V, V)
    rng = np.random.default_rng(4)
    kap = np.exp(rng.standard_normal((N, N)))
    b = rng.standard_normal((N - 2, N - 2))
    x, it = pcg(VarCoefMatrix(T, kap), b[None], tol=1e-10)
    lam, W = O.fd_factor_symmetric(Vo.stiffness_matrix(), Vo.mass_matrix())
    xo, ito = O.pcg(lambda u: O.varcoef_apply(Vo, kap, u), b,
                    lambda r: O.fd_solve(r, [W, W], [W.T, W.T], [lam, lam]), tol=1e-10)
    assert abs(int(it[0]) - ito) <= 1
    assert rel(x[0], xo) < 1e-9


def test_contract_ragged_segments_epilogues():
    """Generic contraction with odd sizes, 2 segments, MUL and DIV epilogues, beta."""
    L = _lib.lib()
    rng = np.random.default_rng(0)
    B, S, M, P, K = 3, 2, 37, 53, 29
    op = rng.standard_normal((S, M, K))
    x = rng.standard_normal((B, S, P, K))
    fld = rng.standard_normal((B, S, M, P))
    out0 = rng.standard_normal((B, S, M, P))
    dev = lambda a: torch.as_tensor(a, device="cuda")  # noqa: E731
    t_op, t_x, t_f = dev(op), dev(x), dev(fld)
    ref = np.einsum("smk,bspk->bsmp", op, x)
    for epi in (0, 1, 2):
        t_out = dev(out0.copy())
        d = _lib.ContractDesc(batch=B, nseg=S, M=M, P=P, K=K, op_ld=K, op_seg=M * K,
                              in_ld=K, in_seg=P * K, in_batch=S * P * K,
                              out_ld=P, out_seg=M * P, out_batch=S * M * P,
                              epilogue=epi, alpha=0.5, beta=2.0)
        lam_m, lam_p = dev(rng.uniform(1, 2, M)), dev(rng.uniform(1, 2, P))
        c0, c1 = dev(rng.uniform(0, 1, B)), dev(rng.uniform(1, 2, B))
        if epi == 1:
            d.field, d.field_ld, d.field_seg, d.field_batch = t_f.data_ptr(), P, M * P, S * M * P
            want = ref * fld
        elif epi == 2:
            d.lam_m, d.lam_p = lam_m.data_ptr(), lam_p.data_ptr()
            d.c0, d.c1 = c0.data_ptr(), c1.data_ptr()
            den = c0.cpu().numpy()[:, None, None, None] + c1.cpu().numpy()[:, None, None, None] * (
                lam_m.cpu().numpy()[None, None, :, None] + lam_p.cpu().numpy()[None, None, None, :])
            want = ref / den
        else:
            want = ref
        want = 0.5 * want + 2.0 * out0
        st = L.jfg_contract_f64(d, t_op.data_ptr(), t_x.data_ptr(), t_out.data_ptr(),
                                _lib.stream_handle())
        assert st == 0
        assert rel(t_out, want) < TOL


def test_bad_workspace_is_reported():
    L = _lib.lib()
    rows = _lib.int_array([8, 8])
    x = torch.zeros(64, dtype=torch.float64, device="cuda")
    m = torch.zeros(64, dtype=torch.float64, device="cuda")
    st = L.jfg_tp_apply_f64(2, rows, rows, 1, _lib.ptr_array([m.data_ptr()] * 2), x.data_ptr(),
                            x.data_ptr(), None, 0, _lib.stream_handle())
    assert st == _lib.JFG_ERR_WORKSPACE


@pytest.mark.parametrize("ndim", [2, 3])
def test_tpmatrices_apply_vs_numpy_kron(ndim):
    """Separable apply (TPMatrix / TPMatrices @ u, tpmatrix.py:152-156,
    287-289) against the explicit numpy.kron product, as the reference's
    test_kron.py:206-369 checks its Kronecker assembly: random dense factors
    of unequal sizes, three terms with coefficients, a batch of 2."""
    from functools import reduce

    from jaxfun_gb300.la import TPMatrices, TPMatrix

    rng = np.random.default_rng(21)
    shape = (5, 7, 4)[:ndim]
    terms = []
    for s in (1.0, -0.5, 2.0):
        terms.append(TPMatrix([rng.standard_normal((n, n)) for n in shape], s))
    A = TPMatrices(terms)
    u = rng.standard_normal((2,) + shape)
    v = (A @ u).cpu().numpy()
    K = A.todense()
    ref = np.stack([(K @ ui.ravel()).reshape(shape) for ui in u])
    np.testing.assert_allclose(v, ref, atol=1e-13 * np.abs(ref).max())
    K2 = sum(t.coefficient * reduce(np.kron, t.mats) for t in terms)
    np.testing.assert_allclose(K, K2, atol=1e-15 * np.abs(K2).max())
