"""Grouped persistent tensor-core contraction: one launch over groups of
different shapes (the per-axis passes of uneven-N solves) gives, group by
group, exactly the result of a single-group launch, for every configuration
the autotuner can pick; the autotuner returns one of them."""

import ctypes as C

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
    return torch.as_tensor(hi, device="cuda"), torch.as_tensor(lo, device="cuda")


def _groups(epi):
    rng = np.random.default_rng(4)
    out = []
    for (nq, B) in [(32, 7), (48, 3), (128, 2), (256, 2), (160, 5)]:
        op = rng.standard_normal((nq, nq))
        hi, lo = _split(op)
        x = torch.as_tensor(rng.standard_normal((B, nq, nq)), device="cuda").float()
        d = _lib.ContractDesc(batch=B, nseg=1, M=nq, P=nq, K=nq, op_ld=nq, in_ld=nq,
                              in_batch=nq * nq, out_ld=nq, out_batch=nq * nq, epilogue=epi,
                              alpha=1.0, beta=0.0)
        keep = [hi, lo, x]
        if epi == 2:
            lam = torch.as_tensor(rng.uniform(1, 2, nq), device="cuda").float()
            c0 = torch.as_tensor(rng.uniform(0, 1, B), device="cuda").float()
            keep += [lam, c0]
            d.lam_m = d.lam_p = lam.data_ptr()
            d.c0 = c0.data_ptr()
        out.append((d, hi, lo, x, keep))
    return out


def _arrays(gs, outs):
    n = len(gs)
    descs = (_lib.ContractDesc * n)(*[g[0] for g in gs])
    ptr = lambda ts: (C.c_void_p * n)(*[t.data_ptr() for t in ts])  # noqa: E731
    return descs, ptr([g[1] for g in gs]), ptr([g[2] for g in gs]), ptr([g[3] for g in gs]), \
        ptr(outs)


@pytest.mark.parametrize("epi", [0, 2])
def test_grouped_equals_single(epi):
    L = _lib.lib()
    gs = _groups(epi)
    sh = _lib.stream_handle()
    ref = []
    for d, hi, lo, x, _ in gs:
        o = torch.empty(d.batch, d.M, d.P, device="cuda")
        assert L.jfg_contract_tc(d, hi.data_ptr(), lo.data_ptr(), x.data_ptr(), o.data_ptr(),
                                 sh) == 0
        ref.append(o)
    torch.cuda.synchronize()
    for ta in (1, 0):
        for order in (0, 1, 2):
            for stages, mt in ((0, 0), (2, 0), (0, 64)):
                outs = [torch.full_like(r, float("nan")) for r in ref]
                descs, oh, ol, ins, ops = _arrays(gs, outs)
                cfg = _lib.TcConfig(ta, order, 0, stages, mt)
                st = L.jfg_contract_tc_grouped(len(gs), descs, oh, ol, ins, ops, C.byref(cfg), sh)
                assert st == 0, _lib.status_string(st)
                torch.cuda.synchronize()
                assert L.jfg_device_status() == 0
                for o, r in zip(outs, ref):
                    if mt == 0:
                        assert torch.equal(o, r), (ta, order, stages)
                    else:  # another tile height: same products, other summation order
                        assert torch.allclose(o, r, rtol=1e-5, atol=1e-5 * float(r.abs().max()))


def test_autotune_picks_a_candidate():
    L = _lib.lib()
    gs = _groups(0)
    outs = [torch.empty(g[0].batch, g[0].M, g[0].P, device="cuda") for g in gs]
    descs, oh, ol, ins, ops = _arrays(gs, outs)
    best = _lib.TcConfig()
    ms = C.c_float()
    st = L.jfg_tc_autotune(len(gs), descs, oh, ol, ins, ops, 2, C.byref(best), C.byref(ms),
                           _lib.stream_handle())
    assert st == 0, _lib.status_string(st)
    assert best.operand_a_in_tmem in (0, 1) and best.order in (0, 1, 2)
    assert best.mtile in (0, 64)
    assert ms.value > 0
    # the cached choice is used when no configuration is passed
    outs2 = [torch.empty_like(o) for o in outs]
    descs, oh, ol, ins, ops2 = _arrays(gs, outs2)
    assert L.jfg_contract_tc_grouped(len(gs), descs, oh, ol, ins, ops2, None,
                                     _lib.stream_handle()) == 0
    torch.cuda.synchronize()
    for a, b in zip(outs, outs2):
        assert torch.equal(a, b)
