"""Tensor-core (tcgen05, split-TF32) contraction against an FP64 reference of the
same FP32 inputs.  Tolerance: 1e-5 relative to the output's max magnitude
(three-term split TF32 with FP32 accumulation over K <= 512 terms)."""

import numpy as np
import pytest
import torch

from jaxfun_gb300 import _lib

pytestmark = pytest.mark.gpu
TC_TOL = 1e-5


@pytest.fixture(params=[1, 0], ids=["A-in-TMEM", "A-in-SMEM"], autouse=True)
def variant(request):
    L = _lib.lib()
    assert L.jfg_tc_set_variant(request.param) == 0
    yield request.param
    L.jfg_tc_set_variant(1)


def split(op64):
    L = _lib.lib()
    a = np.ascontiguousarray(op64, dtype=np.float64)
    hi = np.empty(a.shape, dtype=np.float32)
    lo = np.empty(a.shape, dtype=np.float32)
    L.jfg_split_tf32_host(a.size, a.ctypes.data, hi.ctypes.data, lo.ctypes.data)
    return hi, lo


def run_tc(op64, x32, out0=None, epi=0, field=None, lam_m=None, lam_p=None, c0=None, c1=None,
           alpha=1.0, beta=0.0):
    L = _lib.lib()
    S, M, K = op64.shape
    B, S2, P, K2 = x32.shape
    assert S2 == S and K2 == K
    hi, lo = split(op64)
    dev = lambda a: torch.as_tensor(np.ascontiguousarray(a), device="cuda")  # noqa: E731
    t_hi, t_lo, t_x = dev(hi), dev(lo), dev(x32)
    out = dev(out0.astype(np.float32)) if out0 is not None else torch.zeros(
        B, S, M, P, dtype=torch.float32, device="cuda")
    d = _lib.ContractDesc(batch=B, nseg=S, M=M, P=P, K=K, op_ld=K, op_seg=M * K, in_ld=K,
                          in_seg=P * K, in_batch=S * P * K, out_ld=P, out_seg=M * P,
                          out_batch=S * M * P, epilogue=epi, alpha=alpha, beta=beta)
    keep = []
    if epi == 1:
        f = dev(field.astype(np.float32))
        keep.append(f)
        d.field, d.field_ld, d.field_seg, d.field_batch = f.data_ptr(), P, M * P, S * M * P
    if epi == 2:
        ts = [dev(a.astype(np.float32)) for a in (lam_m, lam_p, c0, c1)]
        keep += ts
        d.lam_m, d.lam_p, d.c0, d.c1 = (t.data_ptr() for t in ts)
    st = L.jfg_contract_tc(d, t_hi.data_ptr(), t_lo.data_ptr(), t_x.data_ptr(), out.data_ptr(),
                           _lib.stream_handle())
    assert st == 0, _lib.status_string(st)
    torch.cuda.synchronize()
    assert L.jfg_device_status() == 0
    return out.cpu().numpy().astype(np.float64)


def rel(a, b):
    return np.abs(a - b).max() / np.abs(b).max()


@pytest.mark.parametrize("B,S,M,P,K", [
    (1, 1, 256, 128, 32),
    (2, 1, 256, 256, 256),
    (1, 2, 128, 300, 96),
    (3, 1, 48, 130, 64),
    (1, 1, 512, 256, 128),
    (1, 1, 254, 129, 256),
    (2, 3, 16, 128, 40),
    (300, 1, 128, 256, 64),
    (7, 2, 200, 384, 160),
])
def test_tc_matches_fp64(B, S, M, P, K):
    rng = np.random.default_rng(M + P + K)
    op = rng.standard_normal((S, M, K))
    x = rng.standard_normal((B, S, P, K)).astype(np.float32)
    ref = np.einsum("smk,bspk->bsmp", op, x.astype(np.float64))
    out = run_tc(op, x)
    assert rel(out, ref) < TC_TOL


def test_tc_epilogues():
    rng = np.random.default_rng(5)
    B, S, M, P, K = 2, 2, 64, 256, 64
    op = rng.standard_normal((S, M, K))
    x = rng.standard_normal((B, S, P, K)).astype(np.float32)
    ref = np.einsum("smk,bspk->bsmp", op, x.astype(np.float64))
    fld = rng.uniform(0.5, 2, (B, S, M, P)).astype(np.float32)
    out0 = rng.standard_normal((B, S, M, P)).astype(np.float32)
    out = run_tc(op, x, out0=out0, epi=1, field=fld, alpha=0.5, beta=2.0)
    want = 0.5 * ref * fld + 2.0 * out0
    assert rel(out, want) < TC_TOL
    lam_m, lam_p = rng.uniform(1, 2, M), rng.uniform(1, 2, P)
    c0, c1 = rng.uniform(0, 1, B), rng.uniform(1, 2, B)
    out = run_tc(op, x, epi=2, lam_m=lam_m, lam_p=lam_p, c0=c0, c1=c1)
    den = (c0[:, None, None, None].astype(np.float32).astype(np.float64)
           + c1[:, None, None, None].astype(np.float32) * (lam_m.astype(np.float32)[None, None, :, None]
                                                           + lam_p.astype(np.float32)[None, None, None, :]))
    assert rel(out, ref / den) < TC_TOL


def test_tc_rejects_misaligned_strides():
    L = _lib.lib()
    x = torch.zeros(1024, dtype=torch.float32, device="cuda")
    d = _lib.ContractDesc(batch=1, nseg=1, M=16, P=16, K=30, op_ld=30, in_ld=30, in_batch=480,
                          out_ld=16, out_batch=256, alpha=1.0)
    st = L.jfg_contract_tc(d, x.data_ptr(), x.data_ptr(), x.data_ptr(), x.data_ptr(),
                           _lib.stream_handle())
    assert st == _lib.JFG_ERR_ARG


@pytest.mark.parametrize("B,S,M,P,K,epi", [
    (2, 1, 256, 256, 256, 0),
    (3, 2, 200, 300, 96, 1),
    (2, 1, 128, 130, 64, 2),
    (1, 1, 512, 1024, 128, 0),
])
def test_tc_store_paths_agree(B, S, M, P, K, epi):
    """TMA bulk-tensor stores through shared memory and plain stores write the
    same values (out-of-range rows and columns clipped)."""
    L = _lib.lib()
    rng = np.random.default_rng(B + M + P)
    op = rng.standard_normal((S, M, K))
    x = rng.standard_normal((B, S, P, K)).astype(np.float32)
    kw = {}
    if epi == 1:
        kw["field"] = rng.uniform(0.5, 2, (B, S, M, P))
    if epi == 2:
        kw.update(lam_m=rng.uniform(1, 2, M), lam_p=rng.uniform(1, 2, P),
                  c0=rng.uniform(0, 1, B), c1=rng.uniform(1, 2, B))
    outs = []
    for path in (1, 0):
        assert L.jfg_tc_set_store_path(path) == 0
        try:
            outs.append(run_tc(op, x, out0=np.full((B, S, M, P), 7.0), epi=epi, **kw))
        finally:
            L.jfg_tc_set_store_path(1)
    assert np.array_equal(outs[0], outs[1])


def test_bounded_wait_times_out_and_context_stays_usable(variant):
    """The timeout path of the bounded mbarrier waits, in the allowed form: with
    a 200 us wait budget the epilogue waits on a barrier that nothing arrives
    on; the wait runs out, JFG_ERR_DEVICE_TIMEOUT is recorded, every other
    role's waits run out, and the kernel drains and returns.  The next launch
    with the default budget is correct against FP64 and leaves status OK."""
    L = _lib.lib()
    rng = np.random.default_rng(21)
    op = rng.standard_normal((1, 256, 256))
    x = rng.standard_normal((8, 1, 256, 256)).astype(np.float32)
    assert L.jfg_device_status() == 0
    assert L.jfg_tc_set_wait_budget_ns(200_000) == 0
    assert L.jfg_tc_test_hold(1) == 0
    try:
        hi, lo = split(op)
        dev = lambda a: torch.as_tensor(np.ascontiguousarray(a), device="cuda")  # noqa: E731
        t_hi, t_lo, t_x = dev(hi), dev(lo), dev(x)
        out = torch.zeros(8, 1, 256, 256, dtype=torch.float32, device="cuda")
        d = _lib.ContractDesc(batch=8, nseg=1, M=256, P=256, K=256, op_ld=256, op_seg=0,
                              in_ld=256, in_seg=0, in_batch=256 * 256, out_ld=256, out_seg=0,
                              out_batch=256 * 256, alpha=1.0, beta=0.0)
        st = L.jfg_contract_tc(d, t_hi.data_ptr(), t_lo.data_ptr(), t_x.data_ptr(),
                               out.data_ptr(), _lib.stream_handle())
        assert st == 0, _lib.status_string(st)
        torch.cuda.synchronize()
    finally:
        assert L.jfg_tc_test_hold(0) == 0
        assert L.jfg_tc_set_wait_budget_ns(0) == 0
    assert L.jfg_device_status() == _lib.JFG_ERR_DEVICE_TIMEOUT
    assert L.jfg_device_status() == 0  # read and cleared
    got = run_tc(op, x)
    ref = np.einsum("smk,bspk->bsmp", op, x.astype(np.float64))
    assert np.abs(got - ref).max() <= TC_TOL * np.abs(ref).max()


def run_f16(op64, x32, epi=0, field=None, in_max_scale=1.0):
    """jfg_contract_tc_f16x3: operator rows split on the host into scaled FP16
    pairs, per-problem input scale from max |x[b]| (times in_max_scale, a
    looser bound), out_max recorded.  Returns (out, out_max as floats)."""
    L = _lib.lib()
    S, M, K = op64.shape
    B, S2, P, K2 = x32.shape
    hi = np.empty((S, M, K), np.uint16)
    lo = np.empty((S, M, K), np.uint16)
    inv = np.empty(S * M, np.float32)
    a = np.ascontiguousarray(op64, dtype=np.float64)
    L.jfg_split_f16_rowscaled_host(S * M, K, a.ctypes.data, hi.ctypes.data, lo.ctypes.data,
                                   inv.ctypes.data)
    dev = lambda v: torch.as_tensor(np.ascontiguousarray(v), device="cuda")  # noqa: E731
    t_hi, t_lo, t_inv = dev(hi.view(np.int16)), dev(lo.view(np.int16)), dev(inv)
    t_x = dev(x32)
    mx = (np.abs(x32.reshape(B, -1)).max(axis=1) * in_max_scale).astype(np.float32)
    t_in = dev(mx.view(np.int32))
    t_out_max = torch.zeros(B, dtype=torch.int32, device="cuda")
    out = torch.zeros(B, S, M, P, dtype=torch.float32, device="cuda")
    d = _lib.ContractDesc(batch=B, nseg=S, M=M, P=P, K=K, op_ld=K, op_seg=M * K, in_ld=K,
                          in_seg=P * K, in_batch=S * P * K, out_ld=P, out_seg=M * P,
                          out_batch=S * M * P, epilogue=epi, alpha=1.0, beta=0.0)
    keep = []
    if epi == 1:
        f = dev(field.astype(np.float32))
        keep.append(f)
        d.field, d.field_ld, d.field_seg, d.field_batch = f.data_ptr(), P, M * P, S * M * P
    st = L.jfg_contract_tc_f16x3(d, t_hi.data_ptr(), t_lo.data_ptr(), t_inv.data_ptr(), M,
                                 t_in.data_ptr(), t_out_max.data_ptr(), t_x.data_ptr(),
                                 out.data_ptr(), _lib.stream_handle())
    assert st == 0, _lib.status_string(st)
    torch.cuda.synchronize()
    assert L.jfg_device_status() == 0
    return (out.cpu().numpy().astype(np.float64),
            t_out_max.cpu().numpy().view(np.float32).astype(np.float64))


@pytest.mark.parametrize("sched", [1, 2, 0])
@pytest.mark.parametrize("S,M,P,K,epi", [(1, 512, 256, 256, 0), (2, 256, 200, 200, 1),
                                         (1, 96, 130, 512, 0), (2, 64, 128, 512, 1)])
def test_f16x3_matches_fp64(S, M, P, K, epi, sched):
    """Scaled split-FP16 contraction against FP64 of the same FP32 inputs,
    per problem (1e-5 of each problem's output maximum), with problems of
    very different magnitudes, a zero problem, a loose input bound (2^9 too
    large) and the recorded output maxima (exact float equality)."""
    rng = np.random.default_rng(S * 1000 + M + P + K)
    B = 4
    op = rng.standard_normal((S, M, K)) * np.logspace(-3, 3, M)[None, :, None]
    x = rng.standard_normal((B, S, P, K))
    x *= np.array([1e-9, 1.0, 3e7, 0.0])[:, None, None, None]
    x = x.astype(np.float32)
    field = rng.uniform(0.1, 2.0, (B, S, M, P)) if epi == 1 else None
    ref = np.einsum("smk,bspk->bsmp", op, x.astype(np.float64))
    if epi == 1:
        ref = ref * field.astype(np.float32).astype(np.float64)
    L = _lib.lib()
    assert L.jfg_tc_set_op_resident(sched) == 0
    try:
        runs = [run_f16(op, x, epi, field, in_max_scale=bound) for bound in (1.0, 512.0)]
    finally:
        L.jfg_tc_set_op_resident(0)
    for bound, (got, omax) in zip((1.0, 512.0), runs):
        for b in range(B):
            scale = np.abs(ref[b]).max()
            if scale == 0:
                assert np.all(got[b] == 0) and omax[b] == 0
                continue
            assert np.abs(got[b] - ref[b]).max() <= TC_TOL * scale, (b, bound)
            assert omax[b] == np.abs(got[b]).max()


def test_autotuned_launch_is_correct_and_recorded():
    """With autotuning on, the first launch of a signature times its candidate
    configurations (including the operator-stationary schedule and plain
    stores) and records the winner (a signature tuned earlier in the process
    keeps its entry); the result is correct, and so is the next launch of that
    signature, which uses the recorded configuration."""
    L = _lib.lib()
    rng = np.random.default_rng(33)
    op = rng.standard_normal((1, 256, 256))
    x = rng.standard_normal((6, 1, 256, 256)).astype(np.float32)
    ref = np.einsum("smk,bspk->bsmp", op, x.astype(np.float64))
    assert L.jfg_tc_set_autotune(1) == 0
    try:
        got, _ = run_f16(op, x)
    finally:
        L.jfg_tc_set_autotune(0)
    assert L.jfg_tc_tuned_count() >= 1
    entries = _lib.tuned_configs()
    assert any("p2:b6:s1:M256:P256:K256" in e["signature"] for e in entries)
    assert np.abs(got - ref).max() <= TC_TOL * np.abs(ref).max()
    got2, _ = run_f16(op, x)
    assert np.abs(got2 - ref).max() <= TC_TOL * np.abs(ref).max()


@pytest.mark.parametrize("mtile", [0, 64])
@pytest.mark.parametrize("S,M,P,K", [(2, 256, 200, 200), (2, 256, 256, 256), (1, 130, 96, 512)])
def test_f16x3_field_forced_configs(S, M, P, K, mtile):
    """The scaled split-FP16 field-multiply pass under forced launch
    configurations (jfg_tc_force_config): TMA stores with the field fetched
    into the staging boxes, and plain stores with the field loaded per
    element, at both tile heights, against FP64 of the same FP32 inputs."""
    L = _lib.lib()
    rng = np.random.default_rng(S * 1000 + P + mtile)
    B = 9
    op = rng.standard_normal((S, M, K))
    x = rng.standard_normal((B, S, P, K)).astype(np.float32)
    field = rng.uniform(0.5, 2.0, (B, S, M, P))
    ref = np.einsum("smk,bspk->bsmp", op, x.astype(np.float64)) * field.astype(np.float32)
    scale = np.abs(ref).max()
    try:
        for store in (1, 2):
            for stages in (0, 2):
                cfg = _lib.TcConfig(operand_a_in_tmem=1, order=0, ctas=0, stages=stages,
                                    mtile=mtile, schedule=1, store=store)
                assert L.jfg_tc_force_config(_lib.C.byref(cfg)) == 0
                got, _ = run_f16(op, x, epi=1, field=field)
                assert np.abs(got - ref).max() <= TC_TOL * scale, (store, stages)
    finally:
        assert L.jfg_tc_force_config(None) == 0
