"""Double-FP32 contraction (jfg_contract_df64) against the FP64 contraction on
the same FP64 inputs, and the mixed solver with either residual arithmetic.
Tolerance 2e-13 of the output's max magnitude: K <= 512 products at ~2^-46
relative each."""

import numpy as np
import pytest
import torch

from jaxfun_gb300 import _lib

pytestmark = pytest.mark.gpu
DF_TOL = 2e-13


def _run(fn, d, op, x, out):
    st = fn(d, op.data_ptr(), x.data_ptr(), out.data_ptr(), _lib.stream_handle())
    assert st == 0, _lib.status_string(st)
    torch.cuda.synchronize()


@pytest.mark.parametrize("shape", [(512, 254, 254, 4), (254, 256, 512, 3), (37, 70, 19, 2)])
@pytest.mark.parametrize("epi", [0, 1, 2])
def test_df64_matches_f64(shape, epi):
    L = _lib.lib()
    M, P, K, B = shape
    g = torch.Generator(device="cuda").manual_seed(7)
    op = torch.randn(M, K, generator=g, dtype=torch.float64, device="cuda")
    x = torch.randn(B, P, K, generator=g, dtype=torch.float64, device="cuda")
    d = _lib.ContractDesc(batch=B, nseg=1, M=M, P=P, K=K, op_ld=K, in_ld=K, in_batch=P * K,
                          out_ld=P, out_batch=M * P, epilogue=epi, alpha=0.5, beta=0.0)
    keep = []
    if epi == 1:
        f = torch.rand(B, M, P, generator=g, dtype=torch.float64, device="cuda") + 0.5
        keep.append(f)
        d.field, d.field_ld, d.field_batch = f.data_ptr(), P, M * P
    if epi == 2:
        lm = torch.rand(M, generator=g, dtype=torch.float64, device="cuda") + 1.0
        lp = torch.rand(P, generator=g, dtype=torch.float64, device="cuda") + 1.0
        c0 = torch.rand(B, generator=g, dtype=torch.float64, device="cuda")
        keep += [lm, lp, c0]
        d.lam_m, d.lam_p, d.c0 = lm.data_ptr(), lp.data_ptr(), c0.data_ptr()
    ref = torch.empty(B, M, P, dtype=torch.float64, device="cuda")
    out = torch.empty_like(ref)
    _run(L.jfg_contract_f64, d, op, x, ref)
    _run(L.jfg_contract_df64, d, op, x, out)
    err = float((out - ref).abs().max() / ref.abs().max())
    assert err <= DF_TOL, err
    # beta accumulate
    d.beta = -1.0
    out2 = out.clone()
    _run(L.jfg_contract_df64, d, op, x, out2)
    assert float((out2 - 0.0).abs().max()) <= DF_TOL * float(ref.abs().max()) * 4


def test_mixed_residual_df64_vs_f64():
    from jaxfun_gb300.galerkin import DIRICHLET, FunctionSpace, Legendre, TensorProduct
    from jaxfun_gb300.la import MixedVarCoefSolver, VarCoefMatrix, pcg

    N = 64
    D = FunctionSpace(N, Legendre, bcs=DIRICHLET)
    T = TensorProduct(D, D)
    rng = np.random.default_rng(5)
    B = 6
    x, _ = D.quad_points_and_weights()
    X, Y = np.meshgrid(x, x, indexing="ij")
    kap = np.stack([np.exp(0.8 * np.sin((1 + s) * X + s) * np.cos((2 + s) * Y))
                    for s in range(B)])
    kap_d = torch.as_tensor(kap, device="cuda")
    b = T.scalar_product(torch.as_tensor(rng.standard_normal((B, N, N)), device="cuda"))
    A = VarCoefMatrix(T, kap_d)
    xt, _ = pcg(A, b, tol=1e-14, maxiter=3000)
    for res in ("df64", "f64"):
        xm, it_in, it_out = MixedVarCoefSolver(A, residual=res).solve(b, tol=1e-11)
        err = float(((xm - xt).abs().amax(dim=(1, 2)) / xt.abs().amax(dim=(1, 2))).max())
        assert err <= 1e-10, (res, err)


@pytest.mark.parametrize("family", ["legendre", "chebyshev"])
def test_scalar_product_df64(family):
    """TensorProductSpace.scalar_product(precision="df64") (the right-hand side
    assembly of the end-to-end solve) against the FP64 path and the oracle."""
    from jaxfun_gb300.galerkin import DIRICHLET, Chebyshev, FunctionSpace, Legendre, TensorProduct
    from oracle import spectral as O

    N = 64
    D = FunctionSpace(N, Legendre if family == "legendre" else Chebyshev, bcs=DIRICHLET)
    T = TensorProduct(D, D)
    f = np.random.default_rng(2).standard_normal((3, N, N))
    b64 = T.scalar_product(f).cpu().numpy()
    bdf = T.scalar_product(f, precision="df64").cpu().numpy()
    assert np.abs(bdf - b64).max() <= DF_TOL * np.abs(b64).max()
    V = O.Space1D(family, N, True)
    bo = np.stack([O.tp_scalar_product([V, V], fi) for fi in f])
    assert np.abs(bdf - bo).max() <= 1e-12 * np.abs(bo).max()
