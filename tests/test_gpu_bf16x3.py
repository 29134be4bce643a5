"""Split-BF16 tensor-core contraction (jfg_contract_tc_bf16x3: hi*hi + hi*lo +
lo*hi BF16 MMAs, FP32 accumulation) against an FP64 reference of the same FP32
inputs, and the 3-D transform round trip with it.  Tolerance 6e-5 of the
output's max magnitude (BF16 pairs carry ~17 bits; one product ~2^-16).
The plain BF16 form (op_lo NULL: hi*hi only) is checked against the FP64
contraction of the BF16-rounded operands: its products are exact in FP32, so
only the FP32 accumulation differs (1e-5 of the max)."""

import numpy as np
import pytest
import torch

from jaxfun_gb300 import _lib

pytestmark = pytest.mark.gpu
B3_TOL = 6e-5


@pytest.fixture(params=[1, 2, 0], ids=["sched-auto", "op-resident", "streaming"], autouse=True)
def schedule(request):
    """Operator-stationary schedule: automatic (what large launches get),
    forced wherever the operator chunk fits, or off."""
    L = _lib.lib()
    assert L.jfg_tc_set_op_resident(request.param) == 0
    yield request.param
    L.jfg_tc_set_op_resident(0)


def split16(op64):
    L = _lib.lib()
    a = np.ascontiguousarray(op64, dtype=np.float64)
    hi = np.empty(a.shape, dtype=np.uint16)
    lo = np.empty(a.shape, dtype=np.uint16)
    L.jfg_split_bf16_host(a.size, a.ctypes.data, hi.ctypes.data, lo.ctypes.data)
    return hi, lo


def test_split_bf16_host():
    x = np.array([1.0, -3.14159265358979, 1e-3, 65504.5, 0.0])
    hi, lo = split16(x)
    f = lambda b: (b.astype(np.uint32) << 16).view(np.float32).astype(np.float64)  # noqa: E731
    approx = f(hi) + f(lo)
    assert np.all(np.abs(approx - x) <= 2.0 ** -16 * np.abs(x) + 1e-300)


def run_b3(op64, x32, epi=0, field=None, lam_m=None, lam_p=None, c0=None, single=False,
           beta=0.0):
    L = _lib.lib()
    S, M, K = op64.shape
    B, S2, P, K2 = x32.shape
    hi, lo = split16(op64)
    dev = lambda a: torch.as_tensor(np.ascontiguousarray(a), device="cuda")  # noqa: E731
    t_hi, t_lo, t_x = dev(hi.view(np.int16)), dev(lo.view(np.int16)), dev(x32)
    out = torch.zeros(B, S, M, P, dtype=torch.float32, device="cuda")
    d = _lib.ContractDesc(batch=B, nseg=S, M=M, P=P, K=K, op_ld=K, op_seg=M * K, in_ld=K,
                          in_seg=P * K, in_batch=S * P * K, out_ld=P, out_seg=M * P,
                          out_batch=S * M * P, epilogue=epi, alpha=1.0, beta=beta)
    keep = []
    if epi == 1:
        f = dev(field.astype(np.float32))
        keep.append(f)
        d.field, d.field_ld, d.field_seg, d.field_batch = f.data_ptr(), P, M * P, S * M * P
    if epi == 2:
        ts = [dev(a.astype(np.float32)) for a in (lam_m, lam_p, c0)]
        keep += ts
        d.lam_m, d.lam_p, d.c0 = (t.data_ptr() for t in ts)
    st = L.jfg_contract_tc_bf16x3(d, t_hi.data_ptr(), None if single else t_lo.data_ptr(),
                                  t_x.data_ptr(), out.data_ptr(), _lib.stream_handle())
    if single and (beta != 0.0 or epi == 1):
        return st
    assert st == 0, _lib.status_string(st)
    torch.cuda.synchronize()
    assert L.jfg_device_status() == 0
    return out.cpu().numpy().astype(np.float64)


def rel(a, b):
    return np.abs(a - b).max() / np.abs(b).max()


@pytest.mark.parametrize("B,S,M,P,K", [
    (1, 1, 256, 128, 64),
    (2, 1, 256, 256, 256),
    (1, 2, 128, 300, 96),
    (3, 1, 48, 130, 40),
    (16, 1, 128, 512, 128),
    (2, 3, 16, 128, 512),
])
def test_bf16x3_matches_fp64(B, S, M, P, K):
    rng = np.random.default_rng(M + P + K)
    op = rng.standard_normal((S, M, K))
    x = rng.standard_normal((B, S, P, K)).astype(np.float32)
    ref = np.einsum("smk,bspk->bsmp", op, x.astype(np.float64))
    assert rel(run_b3(op, x), ref) < B3_TOL


def test_bf16x3_epilogues():
    rng = np.random.default_rng(9)
    B, S, M, P, K = 2, 1, 64, 256, 128
    op = rng.standard_normal((S, M, K))
    x = rng.standard_normal((B, S, P, K)).astype(np.float32)
    ref = np.einsum("smk,bspk->bsmp", op, x.astype(np.float64))
    fld = rng.uniform(0.5, 2, (B, S, M, P)).astype(np.float32)
    assert rel(run_b3(op, x, epi=1, field=fld), ref * fld) < B3_TOL
    lam_m, lam_p, c0 = rng.uniform(1, 2, M), rng.uniform(1, 2, P), rng.uniform(0, 1, B)
    den = c0[:, None, None, None] + lam_m[None, None, :, None] + lam_p[None, None, None, :]
    assert rel(run_b3(op, x, epi=2, lam_m=lam_m, lam_p=lam_p, c0=c0), ref / den) < B3_TOL


def test_transform_roundtrip_bf16x3():
    from jaxfun_gb300.galerkin import Chebyshev, TensorProduct

    N = 64
    C = Chebyshev(N)
    T = TensorProduct(C, C, C)
    rng = np.random.default_rng(1)
    i = np.arange(N, dtype=np.float64)
    s = 1.0 / (1.0 + i[:, None, None] + i[None, :, None] + i[None, None, :]) ** 3
    c = torch.as_tensor(rng.standard_normal((2, N, N, N)) * s, device="cuda")
    u = T.backward(c)
    ref = T.forward(u)
    fwd = T.forward(u.float(), precision="bf16x3").double()
    assert float((fwd - ref).abs().max() / ref.abs().max()) < 2e-4
    back = T.backward(fwd.float(), precision="bf16x3").double()
    assert float((back - u).abs().max() / u.abs().max()) < 2e-4


def bf16_round(a):
    """Round FP32 values to BF16 (nearest even), as FP64."""
    u = np.ascontiguousarray(a, dtype=np.float32).view(np.uint32).astype(np.uint64)
    u = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


@pytest.mark.parametrize("B,S,M,P,K", [
    (2, 1, 256, 256, 256),
    (3, 1, 48, 130, 40),
    (2, 3, 16, 128, 512),
])
def test_bf16_single_matches_rounded_fp64(B, S, M, P, K):
    rng = np.random.default_rng(M + P + K + 1)
    op = rng.standard_normal((S, M, K))
    x = rng.standard_normal((B, S, P, K)).astype(np.float32)
    hi, _ = split16(op)
    oph = (hi.astype(np.uint32) << 16).view(np.float32).astype(np.float64)
    ref = np.einsum("smk,bspk->bsmp", oph, bf16_round(x))
    assert rel(run_b3(op, x, single=True), ref) < 1e-5
    # and ~2^-8 of the unrounded contraction
    ref64 = np.einsum("smk,bspk->bsmp", op, x.astype(np.float64))
    assert rel(run_b3(op, x, single=True), ref64) < 2e-2


def test_bf16_single_divide_epilogue_and_rejections():
    rng = np.random.default_rng(19)
    B, S, M, P, K = 2, 1, 64, 256, 128
    op = rng.standard_normal((S, M, K))
    x = rng.standard_normal((B, S, P, K)).astype(np.float32)
    hi, _ = split16(op)
    oph = (hi.astype(np.uint32) << 16).view(np.float32).astype(np.float64)
    ref = np.einsum("smk,bspk->bsmp", oph, bf16_round(x))
    lam_m, lam_p, c0 = rng.uniform(1, 2, M), rng.uniform(1, 2, P), rng.uniform(0, 1, B)
    den = (c0.astype(np.float32)[:, None, None, None] +
           lam_m.astype(np.float32)[None, None, :, None] +
           lam_p.astype(np.float32)[None, None, None, :])
    got = run_b3(op, x, epi=2, lam_m=lam_m, lam_p=lam_p, c0=c0, single=True)
    assert rel(got, ref / den) < 1e-5
    # the plain form has no beta and no field epilogue: refused before any launch
    fld = rng.uniform(0.5, 2, (B, S, M, P)).astype(np.float32)
    assert run_b3(op, x, epi=1, field=fld, single=True) != 0
    assert run_b3(op, x, single=True, beta=1.0) != 0
