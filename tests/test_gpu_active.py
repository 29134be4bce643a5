"""Active subsets of a batch (jfg_contract_desc.batch_list / batch_count): only
the listed problems are computed, each exactly as in a full launch; unlisted
problems and out-of-range entries leave the output untouched.  The PCG uses the
same lists to drop converged problems, so its per-problem results must equal
those of single-problem solves."""

import numpy as np
import pytest
import torch

from jaxfun_gb300 import _lib

pytestmark = pytest.mark.gpu


def _split(op64):
    L = _lib.lib()
    a = np.ascontiguousarray(op64, dtype=np.float64)
    hi = np.empty(a.shape, dtype=np.float32)
    lo = np.empty(a.shape, dtype=np.float32)
    L.jfg_split_tf32_host(a.size, a.ctypes.data, hi.ctypes.data, lo.ctypes.data)
    return hi, lo


def _contract(engine, op, x, out, lst=None, count=None, epi=0, field=None):
    L = _lib.lib()
    B, P, K = x.shape
    M = op.shape[0]
    d = _lib.ContractDesc(batch=B, nseg=1, M=M, P=P, K=K, op_ld=K, in_ld=K, in_batch=P * K,
                          out_ld=P, out_batch=M * P, epilogue=epi, alpha=1.0, beta=0.0)
    if epi == 1:
        d.field, d.field_ld, d.field_batch = field.data_ptr(), P, M * P
    if lst is not None:
        d.batch_list, d.batch_count = lst.data_ptr(), count.data_ptr()
    sh = _lib.stream_handle()
    if engine == "tc":
        hi, lo = (torch.as_tensor(a, device="cuda") for a in _split(op.cpu().numpy()))
        st = L.jfg_contract_tc(d, hi.data_ptr(), lo.data_ptr(), x.data_ptr(), out.data_ptr(), sh)
    elif engine == "f64":
        st = L.jfg_contract_f64(d, op.data_ptr(), x.data_ptr(), out.data_ptr(), sh)
    else:
        st = L.jfg_contract_f32(d, op.data_ptr(), x.data_ptr(), out.data_ptr(), sh)
    assert st == 0, _lib.status_string(st)
    torch.cuda.synchronize()
    assert L.jfg_device_status() == 0


@pytest.mark.parametrize("engine", ["tc", "f64", "f32"])
@pytest.mark.parametrize("epi", [0, 1])
def test_listed_problems_only(engine, epi):
    B, M, P, K = 7, 64, 128, 96
    g = torch.Generator(device="cuda").manual_seed(3)
    dt = torch.float64 if engine == "f64" else torch.float32
    op = torch.randn(M, K, generator=g, device="cuda", dtype=torch.float64)
    opd = op if engine in ("tc", "f64") else op.float()
    x = torch.randn(B, P, K, generator=g, device="cuda", dtype=torch.float64).to(dt)
    field = torch.randn(B, M, P, generator=g, device="cuda", dtype=torch.float64).to(dt)
    full = torch.zeros(B, M, P, device="cuda", dtype=dt)
    _contract(engine, opd, x, full, epi=epi, field=field)
    # list: problems 5, 0, 3, an out-of-range entry, then 6 (beyond the count)
    lst = torch.tensor([5, 0, 3, 99, 6], dtype=torch.int32, device="cuda")
    count = torch.tensor([4], dtype=torch.int32, device="cuda")
    out = torch.full((B, M, P), float("nan"), device="cuda", dtype=dt)
    _contract(engine, opd, x, out, lst, count, epi=epi, field=field)
    for b in range(B):
        if b in (5, 0, 3):
            assert torch.equal(out[b], full[b]), b
        else:
            assert torch.isnan(out[b]).all(), b
    # an empty list computes nothing
    count.zero_()
    out2 = torch.full((B, M, P), float("nan"), device="cuda", dtype=dt)
    _contract(engine, opd, x, out2, lst, count, epi=epi, field=field)
    assert torch.isnan(out2).all()


def test_pcg_batch_equals_single_solves():
    """Batched FP64 PCG with early-converging problems: each problem's result
    and iteration count equal those of the same problem solved alone."""
    from jaxfun_gb300.galerkin import DIRICHLET, FunctionSpace, Legendre, TensorProduct
    from jaxfun_gb300.la import VarCoefMatrix, pcg

    N = 32
    D = FunctionSpace(N, Legendre, bcs=DIRICHLET)
    T = TensorProduct(D, D)
    rng = np.random.default_rng(11)
    B = 5
    x, _ = D.quad_points_and_weights()
    X, Y = np.meshgrid(x, x, indexing="ij")
    # increasingly rough coefficients: iteration counts differ across the batch
    kap = np.stack([np.exp(0.3 * s * np.sin((1 + s) * X) * np.cos((2 + s) * Y))
                    for s in range(B)])
    f = rng.standard_normal((B, N, N))
    kap_d = torch.as_tensor(kap, device="cuda")
    b = T.scalar_product(torch.as_tensor(f, device="cuda"))
    A = VarCoefMatrix(T, kap_d)
    xb, itb = pcg(A, b, tol=1e-12, maxiter=500)
    itb = np.asarray(itb)
    assert len(set(itb.tolist())) > 1  # the batch really is uneven
    for i in range(B):
        Ai = VarCoefMatrix(T, kap_d[i:i + 1])
        xi, iti = pcg(Ai, b[i:i + 1], tol=1e-12, maxiter=500)
        assert int(np.asarray(iti)[0]) == int(itb[i])
        assert torch.equal(xi[0], xb[i])
