"""Benchmark: variable-coefficient 2-D Poisson solves/s at <= 1e-10 error (one GB300).

Workload (one "step"): a batch of B independent problems
  -div(kappa grad u) = f on [-1,1]^2, Legendre Dirichlet basis, N = 256 per axis
  (254^2 unknowns, 256^2 Gauss grid), kappa = exp(g) with g a Gaussian random
  field (Legendre coefficients N(0,1)(1+|k|^2)^-1.5, rescaled to std 1),
  forcing coefficients N(0,1)(1+j)^-2(1+k)^-2; seeded synthetic data.
Each problem is solved by PCG with the constant-coefficient fast-
diagonalisation preconditioner until its error against the FP64 solution is
<= 1e-10 (checked on a sample at the end).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--batch B] [--impl ours|reference]

Prints one JSON line (rank 0).  ``--impl reference`` times the CPU FP64
restatement of the reference algorithm (the oracle port) on the host cores.
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "var-coef solves/s at 1e-10 err: learned+mixed vs plain FP64 PCG, 1 GB300"
N_GRID = 256
# DRAM bytes (read + write) of one scaled split-FP16 k_contract_tc launch at
# M = 512, P = K = 256, 128 problems, from ncu (dram__bytes_read.sum +
# dram__bytes_write.sum); None until captured.
TC_TRAFFIC_PER_LAUNCH_B128 = 34.173440e6 + 8.172288e6


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            p = json.load(fh)
        return p, "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


# ---------------------------------------------------------------------------
# clocks sampler (nvidia-smi during the timed region)
# ---------------------------------------------------------------------------


class Clocks:
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "50"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if self.path is None or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------
# synthetic problems
# ---------------------------------------------------------------------------


def synth_coeffs(seed: int, N: int):
    import numpy as np

    rng = np.random.default_rng(seed)
    k2 = np.add.outer(np.arange(N) ** 2.0, np.arange(N) ** 2.0)
    gh = rng.standard_normal((N, N)) * (1.0 + k2) ** -1.5
    s = np.outer((1.0 + np.arange(N)) ** -2.0, (1.0 + np.arange(N)) ** -2.0)
    fh = rng.standard_normal((N, N)) * s
    return gh, fh


def make_problems(B: int, N: int, seed0: int = 0):
    """Return host (kappa, f) on the Gauss grid, shape (B, N, N), FP64.

    g and f are the backward transforms of the seeded Legendre coefficients,
    computed on the GPU with the library's own transform."""
    import numpy as np

    from jaxfun_gb300.galerkin import Legendre, TensorProduct

    To = TensorProduct(Legendre(N), Legendre(N))
    gh = np.empty((B, N, N))
    fh = np.empty((B, N, N))
    for b in range(B):
        gh[b], fh[b] = synth_coeffs(seed0 + b, N)
    g = To.backward(gh).cpu().numpy()
    f = To.backward(fh).cpu().numpy()
    g = (g - g.mean(axis=(1, 2), keepdims=True)) / g.std(axis=(1, 2), keepdims=True)
    return np.exp(g), f


# ---------------------------------------------------------------------------
# reference arm (CPU restatement of the reference algorithm)
# ---------------------------------------------------------------------------


def cpu_solver(N: int):
    import numpy as np

    from oracle import spectral as O

    V = O.Space1D("legendre", N, True)
    lam, W = O.fd_factor_symmetric(V.stiffness_matrix(), V.mass_matrix())

    def solve(kap, f, tol=1e-10):
        b = O.tp_scalar_product([V, V], f)
        x, it = O.pcg(lambda u: O.varcoef_apply(V, kap, u), b,
                      lambda r: O.fd_solve(r, [W, W], [W.T, W.T], [lam, lam]), tol=tol)
        return x, it

    return solve, np


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    import numpy as np  # noqa: F401

    N = N_GRID
    solve, _ = cpu_solver(N)
    # inputs: the same synthetic recipe, generated on the host by the restatement
    from oracle import spectral as O

    Vo = O.Space1D("legendre", N, False)
    probs = []
    for b in range(args.warmup + args.steps):
        gh, fh = synth_coeffs(b, N)
        g = O.tp_backward([Vo, Vo], gh)
        g = (g - g.mean()) / g.std()
        probs.append((np.exp(g), O.tp_backward([Vo, Vo], fh)))
    for b in range(args.warmup):
        solve(*probs[b])
    t0 = time.perf_counter()
    its = []
    for b in range(args.warmup, args.warmup + args.steps):
        _, it = solve(*probs[b])
        its.append(it)
    dt = time.perf_counter() - t0
    val = args.steps / dt
    cores = len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else os.cpu_count()
    line = {
        "metric": METRIC, "impl": "reference", "value": val, "unit": "solves/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * dt / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded, config recipe)",
        "config": {"workload": "varcoef-poisson-2d-legendre-N256", "N": N, "batch": 1,
                   "tol": 1e-10, "pcg_iterations_mean": float(np.mean(its))},
        "cpu_baseline": {"value": val, "unit": "solves/s", "cores": cores, "kind": "port",
                         "sample": f"{args.steps} single-problem FP64 PCG solves (N=256) with "
                                   "numpy/scipy BLAS on all host threads"},
        "e2e": {"value": val, "unit": "solves/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------
# our arm
# ---------------------------------------------------------------------------


def roofline_microbench(B: int, N: int, reps: int = 20, M: int | None = None,
                        prec: str = "f16x3", field_pass: bool = False):
    """Time the dominant kernel -- the tcgen05 contraction at the first
    variable-coefficient pass shape of the inner solve (stacked [B; D]
    operator: M = 2N quadrature rows, P = K = N padded coefficients, B problems;
    M = N gives the preconditioner pass) -- with CUDA events on its launch
    stream.  prec "f16x3": scaled split FP16 (kind::f16, the inner solve's
    operator passes); "tf32": split TF32 (kind::tf32); "bf16" / "bf16x3":
    plain / split BF16 (the preconditioner's passes, with M = N).  field_pass: the
    second operator pass instead (two segments of M = N rows, the kappa*w
    field multiplied in the epilogue).  Returns achieved numbers; FLOPs count
    each contraction once."""
    import numpy as np
    import torch

    from jaxfun_gb300 import _lib
    from jaxfun_gb300.la import split_tf32

    L = _lib.lib()
    P = K = N
    M = 2 * N if M is None else M
    S = 1
    if field_pass:
        S, M = 2, N
    rng = np.random.default_rng(0)
    op = rng.standard_normal((S * M, K))
    x = torch.randn(B, S, P, K, dtype=torch.float32, device="cuda")
    y = torch.empty(B, S, M, P, dtype=torch.float32, device="cuda")
    d = _lib.ContractDesc(batch=B, nseg=S, M=M, P=P, K=K, op_ld=K, op_seg=M * K, in_ld=K,
                          in_seg=P * K, in_batch=S * P * K, out_ld=P, out_seg=M * P,
                          out_batch=S * M * P, alpha=1.0, beta=0.0)
    if field_pass:
        fld = torch.rand(B, M, P, dtype=torch.float32, device="cuda") + 0.5
        d.epilogue = 1
        d.field, d.field_ld, d.field_seg, d.field_batch = fld.data_ptr(), P, 0, M * P
    s = torch.cuda.current_stream()
    if prec == "f16x3":
        hi = np.empty((S * M, K), np.uint16)
        lo = np.empty((S * M, K), np.uint16)
        inv = np.empty(S * M, np.float32)
        L.jfg_split_f16_rowscaled_host(S * M, K, op.ctypes.data, hi.ctypes.data, lo.ctypes.data,
                                       inv.ctypes.data)
        t_hi = torch.as_tensor(hi.view(np.int16), device="cuda")
        t_lo = torch.as_tensor(lo.view(np.int16), device="cuda")
        t_inv = torch.as_tensor(inv, device="cuda")
        in_max = x.abs().amax(dim=(1, 2, 3)).contiguous().view(torch.int32)
        out_max = torch.zeros(B, dtype=torch.int32, device="cuda")
        call = lambda: L.jfg_contract_tc_f16x3(  # noqa: E731
            d, t_hi.data_ptr(), t_lo.data_ptr(), t_inv.data_ptr(), M, in_max.data_ptr(),
            out_max.data_ptr(), x.data_ptr(), y.data_ptr(), s.cuda_stream)
    elif prec in ("bf16", "bf16x3"):
        from jaxfun_gb300.la.mixed import split_bf16

        hi, lo = split_bf16(op)
        lo_p = lo.data_ptr() if prec == "bf16x3" else None
        call = lambda: L.jfg_contract_tc_bf16x3(d, hi.data_ptr(), lo_p,  # noqa: E731
                                                x.data_ptr(), y.data_ptr(), s.cuda_stream)
    else:
        hi, lo = split_tf32(op)
        call = lambda: L.jfg_contract_tc(d, hi.data_ptr(), lo.data_ptr(),  # noqa: E731
                                         x.data_ptr(), y.data_ptr(), s.cuda_stream)
    for _ in range(3):
        _lib.check(call(), "contract_tc")
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(s)
    for _ in range(reps):
        call()
    e1.record(s)
    e1.synchronize()
    t = e0.elapsed_time(e1) / 1e3 / reps
    flops = 2.0 * M * P * K * B * S
    nbytes = 4.0 * B * S * P * (K + M) + (4.0 * B * M * P if field_pass else 0.0)
    return {"M": M, "P": P, "K": K, "S": S, "t": t, "flops": flops, "bytes": nbytes, "prec": prec,
            "tflops_alg": flops / t / 1e12,
            "tflops_issued": (1 if prec == "bf16" else 3) * flops / t / 1e12,
            "gbs": nbytes / t / 1e9}


def other_kernel_microbench(which: str, B: int, reps: int = 3):
    """CUDA-event timing of the BF16 GEMM ('gemm'), the FP64 contraction ('fp64') or
    its double-FP32 counterpart ('df64')."""
    import ctypes

    import torch

    from jaxfun_gb300 import _lib

    L = _lib.lib()
    s = torch.cuda.current_stream()
    if which == "gemm":
        M, N, K, P = 1024, 64, 4096, 4096
        A = torch.randn(M, K, device="cuda").to(torch.bfloat16)
        Bm = torch.randn(N, B * P, device="cuda").to(torch.bfloat16)
        out = torch.empty(B, M, N, device="cuda")
        d = _lib.GemmDesc(batch=B, M=M, N=N, K=K, ksplit=1, lda=K, a_batch=0, ldb=B * P,
                          b_batch=P, alpha=1.0, d32=out.data_ptr(), ld_d32=N, d32_batch=M * N)
        call = lambda: L.jfg_gemm_bf16(ctypes.byref(d), A.data_ptr(), Bm.data_ptr(),  # noqa: E731
                                       s.cuda_stream)
        flops = 2.0 * M * N * K * B
        name = "k_gemm_bf16"
    elif which in ("transform", "transform_tf32"):
        from jaxfun_gb300.galerkin import Chebyshev
        from jaxfun_gb300.galerkin.tensorproductspace import device_op_split, device_op_split_bf16

        N_ = N_GRID
        F = Chebyshev(N_).forward_matrix()
        M, P, K = N_, N_ * N_, N_
        x = torch.randn(B, P, K, device="cuda")
        y = torch.empty(B, M, P, device="cuda")
        d = _lib.ContractDesc(batch=B, nseg=1, M=M, P=P, K=K, op_ld=K, in_ld=K, in_batch=P * K,
                              out_ld=P, out_batch=M * P, alpha=1.0, beta=0.0)
        if which == "transform":
            hi, lo = device_op_split_bf16(F)
            fn = L.jfg_contract_tc_bf16x3
        else:
            hi, lo = device_op_split(F)
            fn = L.jfg_contract_tc
        call = lambda: fn(d, hi.data_ptr(), lo.data_ptr(), x.data_ptr(), y.data_ptr(),  # noqa: E731
                          s.cuda_stream)
        flops = 2.0 * M * P * K * B
        name = "k_contract_tc (" + ("split-BF16" if which == "transform" else "split-TF32") + ")"
        nbytes = 4.0 * B * P * (K + M)
    else:
        N_ = N_GRID
        n = N_ - 2
        M, P, K = 2 * N_, n, n
        op = torch.randn(M, K, dtype=torch.float64, device="cuda")
        x = torch.randn(B, P, K, dtype=torch.float64, device="cuda")
        y = torch.empty(B, M, P, dtype=torch.float64, device="cuda")
        d = _lib.ContractDesc(batch=B, nseg=1, M=M, P=P, K=K, op_ld=K, in_ld=K, in_batch=P * K,
                              out_ld=P, out_batch=M * P, alpha=1.0, beta=0.0)
        fn = L.jfg_contract_f64 if which == "fp64" else L.jfg_contract_df64
        call = lambda: fn(d, op.data_ptr(), x.data_ptr(), y.data_ptr(),  # noqa: E731
                          s.cuda_stream)
        flops = 2.0 * M * P * K * B
        name = "k_contract_simt<double>" if which == "fp64" else "k_contract_df"
    for _ in range(2):
        _lib.check(call(), name)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(s)
    for _ in range(reps):
        call()
    e1.record(s)
    e1.synchronize()
    t = e0.elapsed_time(e1) / 1e3 / reps
    out = {"kernel": name, "t": t, "tflops": flops / t / 1e12}
    if which.startswith("transform"):
        out["gbs"] = nbytes / t / 1e9
    return out


def run_transforms(args):
    """Secondary measurement (not the headline): 16 FP64 fields on the 256^3
    Chebyshev-Gauss grid, forward + backward round trip, FP64 CUDA-core path vs
    split-TF32 tensor-core path (FP32 storage); errors vs the FP64 path."""
    import numpy as np
    import torch

    from jaxfun_gb300.galerkin import Chebyshev, TensorProduct

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    N, F = args.n_transform, args.fields
    C = Chebyshev(N)
    T = TensorProduct(C, C, C)
    rng = np.random.default_rng(0)
    i = np.arange(N, dtype=np.float64)
    s = 1.0 / (1.0 + i[:, None, None] + i[None, :, None] + i[None, None, :]) ** 3
    c = torch.empty((F, N, N, N), dtype=torch.float64, device="cuda")
    for k in range(F):
        c[k] = torch.as_tensor(np.random.default_rng(k).standard_normal((N, N, N)) * s)
    u = T.backward(c)                       # FP64 grid fields (the inputs)
    u32 = u.float()
    res = {}
    for prec, x in (("f64", u), ("tc", u32), ("bf16x3", u32)):
        for _ in range(args.warmup):
            T.backward(T.forward(x, precision=prec), precision=prec)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(args.steps):
            y = T.backward(T.forward(x, precision=prec), precision=prec)
        e1.record()
        e1.synchronize()
        t = e0.elapsed_time(e1) / 1e3 / args.steps
        eb = 8 if prec == "f64" else 4
        nbytes = 6 * 2 * F * N**3 * eb          # 6 passes, each reads and writes one field set
        flops = 6 * 2.0 * N * F * N**3           # useful contraction FLOPs
        err = float((y.double() - u).abs().max() / u.abs().max())
        res[prec] = {"ms": 1e3 * t, "gbs": nbytes / t / 1e9, "tflops_alg": flops / t / 1e12,
                     "max_rel_err_vs_input": err}
    pk, kind = peaks()
    t_roof_tc = max(6 * 2.0 * N * F * N**3 / (pk["bf16_tflops"] / 2 * 1e12),
                    6 * 2 * F * N**3 * 4 / (pk["hbm_gbs"] * 1e9))
    line = {"workload": f"chebyshev-3d-N{N}-{F}fields-roundtrip", "unit": "ms per round trip",
            "f64": res["f64"], "tc": res["tc"], "bf16x3": res["bf16x3"],
            "tc_roofline_ms": 1e3 * t_roof_tc,
            "tc_roofline_frac": 1e3 * t_roof_tc / res["tc"]["ms"],
            "bf16x3_roofline_frac": 1e3 * t_roof_tc / res["bf16x3"]["ms"],
            "roofline_note": f"max(useful FLOP / (bf16 {kind} / 2), FP32 bytes / HBM {kind})"}
    print(json.dumps(line), flush=True)
    return 0


def transform_roundtrip_keys(n: int = 256, fields: int = 16, reps: int = 10):
    """Config 1 (batched 3-D Chebyshev transforms) as flat keys of the headline
    line: 16 FP64 fields on the 256^3 Chebyshev-Gauss grid, each the backward
    transform of seeded coefficients z (1+i+j+k)^-3; forward + backward round
    trip in split-BF16 on the tensor cores (FP32 storage), CUDA-event timed
    after warm-up; the roofline counts FP32 bytes read and written per pass
    (6 passes) against measured HBM bandwidth; error vs the FP64 input."""
    import numpy as np
    import torch

    from jaxfun_gb300.galerkin import Chebyshev, TensorProduct

    C = Chebyshev(n)
    T = TensorProduct(C, C, C)
    i = np.arange(n, dtype=np.float64)
    decay = 1.0 / (1.0 + i[:, None, None] + i[None, :, None] + i[None, None, :]) ** 3
    c = torch.empty((fields, n, n, n), dtype=torch.float64, device="cuda")
    for k in range(fields):
        c[k] = torch.as_tensor(np.random.default_rng(k).standard_normal((n, n, n)) * decay)
    u = T.backward(c)
    del c
    x = u.float()
    for _ in range(3):
        y = T.backward(T.forward(x, precision="bf16x3"), precision="bf16x3")
    s = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(s)
    for _ in range(reps):
        y = T.backward(T.forward(x, precision="bf16x3"), precision="bf16x3")
    e1.record(s)
    e1.synchronize()
    t = e0.elapsed_time(e1) / 1e3 / reps
    err = float((y.double() - u).abs().max() / u.abs().max())
    pk, kind = peaks()
    nbytes = 6 * 2 * fields * n**3 * 4
    flops = 6 * 2.0 * n * fields * n**3
    t_roof = max(flops / (pk["bf16_tflops"] * 1e12), nbytes / (pk["hbm_gbs"] * 1e9))
    del u, x, y
    torch.cuda.empty_cache()
    return {"transforms_workload": f"chebyshev-3d-N{n}-{fields}fields-roundtrip-bf16x3",
            "transforms_ms": 1e3 * t, "transforms_gbs": nbytes / t / 1e9,
            "transforms_roofline_ms": 1e3 * t_roof, "transforms_roofline_frac": t_roof / t,
            "transforms_max_rel_err_vs_fp64": err,
            "transforms_roofline_note": f"max(useful FLOP / bf16 {kind}, FP32 bytes / HBM {kind})"}


def run_poisson2d(args):
    """Secondary measurement (config 0): 2-D Poisson, Legendre Dirichlet, N = 64.
    One step = scalar product of f, fast-diagonalisation solve, backward to
    the grid and forward back (the reference's solve + round trip), 8 FP64
    contraction passes.  Launch/latency bound: reported as the latency of one
    problem (direct C-ABI calls, and the same step replayed as a CUDA graph)
    and as solves/s with 1024 problems per step (graph replay).  f: seeded
    coefficients z (1+j)^-2 (1+k)^-2 on 64 x 64 orthogonal Legendre modes,
    backward to the Gauss grid."""
    import numpy as np
    import torch

    from jaxfun_gb300 import _lib
    from jaxfun_gb300.galerkin import DIRICHLET, FunctionSpace, Legendre, TensorProduct
    from jaxfun_gb300.la import poisson_tpmatrices

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    L = _lib.lib()
    N = 64
    n = N - 2
    D = FunctionSpace(N, Legendre, bcs=DIRICHLET)
    T = TensorProduct(D, D)
    To = TensorProduct(Legendre(N), Legendre(N))
    E, W, lam = poisson_tpmatrices(T).lu_factor().device_factors()
    SP = torch.as_tensor(np.ascontiguousarray(D.scalar_product_matrix()), device="cuda")
    BW = torch.as_tensor(np.ascontiguousarray(D.backward_matrix()), device="cuda")
    FW = torch.as_tensor(np.ascontiguousarray(D.forward_matrix(N)), device="cuda")
    i = np.arange(N, dtype=np.float64)
    decay = 1.0 / np.outer((1.0 + i) ** 2, (1.0 + i) ** 2)
    ia = _lib.int_array

    def make(batch, stream):
        with torch.cuda.stream(stream):
            fh = np.stack([np.random.default_rng(k).standard_normal((N, N)) * decay
                           for k in range(batch)])
            f = To.backward(fh)
            buf = {"f": f, "b": torch.empty(batch, n, n, dtype=torch.float64, device="cuda"),
                   "u": torch.empty(batch, n, n, dtype=torch.float64, device="cuda"),
                   "uj": torch.empty(batch, N, N, dtype=torch.float64, device="cuda"),
                   "c": torch.empty(batch, n, n, dtype=torch.float64, device="cuda"),
                   "c0": torch.zeros(batch, dtype=torch.float64, device="cuda"),
                   "c1": torch.ones(batch, dtype=torch.float64, device="cuda")}
            wtp = L.jfg_tp_apply_workspace_size(2, ia([N, N]), ia([N, N]), batch, 8)
            buf["wtp"] = torch.empty(wtp, dtype=torch.uint8, device="cuda")
            buf["wfd"] = torch.empty(L.jfg_fd_solve_workspace_size(2, n, batch, 8),
                                     dtype=torch.uint8, device="cuda")
        sh = stream.cuda_stream
        p2 = lambda t: _lib.ptr_array([t.data_ptr()] * 2)  # noqa: E731
        args_sp = (2, ia([n, n]), ia([N, N]), batch, p2(SP))
        args_bw = (2, ia([N, N]), ia([n, n]), batch, p2(BW))
        args_fw = (2, ia([n, n]), ia([N, N]), batch, p2(FW))
        wp, wn = buf["wtp"].data_ptr(), buf["wtp"].numel()

        def step():
            _lib.check(L.jfg_tp_apply_f64(*args_sp, buf["f"].data_ptr(), buf["b"].data_ptr(),
                                          wp, wn, sh), "scalar_product")
            _lib.check(L.jfg_fd_solve_f64(2, n, batch, E.data_ptr(), W.data_ptr(),
                                          lam.data_ptr(), buf["c0"].data_ptr(),
                                          buf["c1"].data_ptr(), buf["b"].data_ptr(),
                                          buf["u"].data_ptr(), buf["wfd"].data_ptr(),
                                          buf["wfd"].numel(), sh), "fd_solve")
            _lib.check(L.jfg_tp_apply_f64(*args_bw, buf["u"].data_ptr(), buf["uj"].data_ptr(),
                                          wp, wn, sh), "backward")
            _lib.check(L.jfg_tp_apply_f64(*args_fw, buf["uj"].data_ptr(), buf["c"].data_ptr(),
                                          wp, wn, sh), "forward")
        return step, buf

    def timed(fn, stream, reps):
        for _ in range(max(3, args.warmup)):
            fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0 = time.perf_counter()
        e0.record(stream)
        for _ in range(reps):
            fn()
        e1.record(stream)
        e1.synchronize()
        return e0.elapsed_time(e1) / 1e3 / reps, (time.perf_counter() - t0) / reps

    out = {"workload": "poisson-2d-legendre-dirichlet-N64", "unit": "us / solves/s"}
    stream = torch.cuda.Stream()
    for batch, key in ((1, "single"), (args.nprob, "batched")):
        step, buf = make(batch, stream)
        with torch.cuda.stream(stream):
            dev_direct, host_direct = timed(step, stream, 200 if batch == 1 else 20)
            torch.cuda.synchronize()
            L.jfg_reset_launch_count()
            step()
            launches = int(L.jfg_launch_count())
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g, stream=stream):
                step()
            dev_graph, _ = timed(g.replay, stream, 200 if batch == 1 else 20)
        rec = {"batch": batch, "launches_per_step": launches,
               "us_per_step_direct_calls": 1e6 * host_direct,
               "us_per_step_graph": 1e6 * dev_graph,
               "solves_per_s_graph": batch / dev_graph,
               "roundtrip_max_rel": float((buf["c"] - buf["u"]).abs().max()
                                          / buf["u"].abs().max())}
        out[key] = rec
        if batch == 1:
            f1, u1 = buf["f"][0].cpu().numpy(), buf["u"][0].cpu().numpy()
    # the oracle port of the same step on the host (CPU baseline and checker)
    from oracle import spectral as O

    Vo = O.Space1D("legendre", N, True)
    K, M = Vo.stiffness_matrix(), Vo.mass_matrix()
    lamo, Wo = O.fd_factor_symmetric(K, M)
    reps = 20
    t0 = time.perf_counter()
    for _ in range(reps):
        bo = O.tp_scalar_product([Vo, Vo], f1)
        uo = O.fd_solve(bo, [Wo, Wo], [Wo.T, Wo.T], [lamo, lamo])
        ujo = O.tp_backward([Vo, Vo], uo)
        O.tp_forward([Vo, Vo], ujo)
    tcpu = (time.perf_counter() - t0) / reps
    out["max_rel_err_vs_oracle"] = float(np.abs(u1 - uo).max() / np.abs(uo).max())
    out["cpu_baseline"] = {"us_per_step": 1e6 * tcpu, "kind": "port",
                           "cores": os.cpu_count(), "sample": f"{reps} single-problem steps"}
    print(json.dumps(out), flush=True)
    return 0


def run_helmholtz(args):
    """Secondary measurement (not the headline): 1024 Chebyshev Dirichlet Helmholtz
    problems, N ~ U{32,48,...,512}, alpha ~ U[0,50], forcing coefficients
    N(0,1)(1+j)^-2(1+k)^-2; tensor-core FD corrections + FP64 refinement to
    relative residual tol; error of one problem per size vs the FP64 FD path."""
    import numpy as np
    import torch

    from jaxfun_gb300.galerkin import DIRICHLET, Chebyshev, FunctionSpace, TensorProduct
    from jaxfun_gb300.la import poisson_tpmatrices
    from jaxfun_gb300.la.helmholtz import UnevenHelmholtzSolver

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    rng = np.random.default_rng(0)
    nprob = args.nprob
    sizes = np.arange(32, 513, 16)
    Ns = rng.choice(sizes, size=nprob)
    alphas = rng.uniform(0.0, 50.0, size=nprob)
    rhs = []
    for N in Ns:
        C_ = Chebyshev(int(N))
        To = TensorProduct(C_, C_)
        D = FunctionSpace(int(N), Chebyshev, bcs=DIRICHLET)
        T = TensorProduct(D, D)
        j = np.arange(N)
        fh = rng.standard_normal((N, N)) * np.outer((1.0 + j) ** -2.0, (1.0 + j) ** -2.0)
        rhs.append(T.scalar_product(To.backward(fh)))
    S = UnevenHelmholtzSolver("chebyshev", Ns, alphas)
    stream = torch.cuda.Stream()              # a capturable stream (CUDA graph per step)
    torch.cuda.set_stream(stream)
    tuned = S.autotune()                      # untimed: picks the grouped launch config
    b = S.pack(rhs)                           # untimed: group-major flat layout
    xp = torch.empty_like(b)
    for _ in range(args.warmup):
        S.solve_packed(b, tol=args.tol, out=xp)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        _, nref = S.solve_packed(b, tol=args.tol, out=xp)
    e1.record(stream)
    e1.synchronize()
    t = e0.elapsed_time(e1) / 1e3 / args.steps
    xs = S.unpack(xp)
    refs = np.zeros(nprob, dtype=int)
    refs[S.order] = nref
    # the same batch solved one size group per call (previous structure)
    S.solve_per_group(rhs, tol=args.tol)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    S.solve_per_group(rhs, tol=args.tol)
    torch.cuda.synchronize()
    t_pg = time.perf_counter() - t0
    from jaxfun_gb300.la.helmholtz import helmholtz_apply

    errs, res_ours, res_fd = {}, {}, {}
    for g in S.groups:
        i = int(g.idx[0])
        D = FunctionSpace(g.N, Chebyshev, bcs=DIRICHLET)
        fac = poisson_tpmatrices(TensorProduct(D, D), 1.0).lu_factor()
        b = rhs[i][None]
        a2 = alphas[i] ** 2
        # reference: FP64 FD solve, refined in FP64 with the structured residual
        ref = fac.solve(b, c0=a2, c1=1.0)
        rr = lambda u: b - helmholtz_apply("chebyshev", g.N, a2, u)  # noqa: E731
        res_fd[g.N] = float(rr(ref).norm() / b.norm())
        for _ in range(3):
            ref = ref + fac.solve(rr(ref), c0=a2, c1=1.0)
        res_ours[g.N] = float(rr(xs[i][None]).norm() / b.norm())
        errs[g.N] = float((xs[i] - ref[0]).abs().max() / ref.abs().max())
    n3 = float(np.mean((Ns - 2.0) ** 3))
    fd_flops = 8.0 * n3 * nprob  # one FD pass of the batch: 4 contractions of 2 n^3
    line = {"workload": f"helmholtz-chebyshev-uneven-{nprob}x-N32..512", "unit": "solves/s",
            "solves_per_s": nprob / t, "ms_per_batch": 1e3 * t,
            "refinements_mean": float(np.mean(refs)),
            "max_rel_err_vs_fp64_refined_fd": max(errs.values()),
            "max_relres_ours": max(res_ours.values()),
            "max_relres_plain_fp64_fd": max(res_fd.values()),
            "groups": len(S.groups), "fd_pass_gflop": fd_flops / 1e9,
            "fd_tflops_algorithmic": fd_flops * float(np.mean(refs)) / t / 1e12,
            "launch_structure": "one C-ABI call: per refinement step 4 grouped persistent "
                                "tensor-core launches over all 31 size groups, CUDA graph",
            "autotuned_config": tuned,
            "per_group_calls_solves_per_s": nprob / t_pg}
    print(json.dumps(line), flush=True)
    return 0


def run_tour(args):
    """Every product kernel on moderate sizes (a few launches each), for the
    all-kernels ncu summary.  Not a measurement: prints the kernels' names."""
    import numpy as np
    import torch

    from jaxfun_gb300 import _lib
    from jaxfun_gb300.galerkin import (DIRICHLET, Chebyshev, FunctionSpace, Legendre,
                                       TensorProduct)
    from jaxfun_gb300.la import MixedVarCoefSolver, VarCoefMatrix, pcg, poisson_tpmatrices
    from jaxfun_gb300.la.helmholtz import UnevenHelmholtzSolver, helmholtz_apply
    from jaxfun_gb300.sno import train as sno_train
    from jaxfun_gb300.sno.model import SNO, SNOConfig

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    L = _lib.lib()
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    rng = np.random.default_rng(0)
    # 1. transforms: 3-D Chebyshev 128^3, 4 fields (FP64, FP32, split-TF32)
    C3 = Chebyshev(128)
    T3 = TensorProduct(C3, C3, C3)
    c = torch.as_tensor(rng.standard_normal((4, 128, 128, 128)), device="cuda")
    u = T3.backward(c)
    T3.forward(u.float(), precision="tc")
    T3.forward(u.float(), precision="bf16x3")
    T3.forward(u)
    # 2. FD solve (FP64 and the no-allocation entry point), 2-D Legendre N=256, 32 rhs
    D = FunctionSpace(256, Legendre, bcs=DIRICHLET)
    T = TensorProduct(D, D)
    fac = poisson_tpmatrices(T, 1.0).lu_factor()
    b = torch.as_tensor(rng.standard_normal((32, 254, 254)), device="cuda")
    fac.solve(b)
    # 3-D FD (eigenvalue-sum kernel), 64^3, 4 rhs
    D3 = FunctionSpace(64, Legendre, bcs=DIRICHLET)
    fac3 = poisson_tpmatrices(TensorProduct(D3, D3, D3), 1.0).lu_factor()
    fac3.solve(torch.as_tensor(rng.standard_normal((4, 62, 62, 62)), device="cuda"))
    # 3. variable-coefficient 2-D N=256, 32 problems: weighted field, FP64 apply,
    #    mixed solve (tensor-core PCG, double-FP32 and FP32 residuals), FP64 PCG
    kap_h, f_h = make_problems(32, 256)
    kap = torch.as_tensor(kap_h, device="cuda")
    A = VarCoefMatrix(T, kap)
    rhs = T.scalar_product(torch.as_tensor(f_h, device="cuda"))
    A @ rhs
    S = MixedVarCoefSolver(A)

    def bounded(fn, *a, **k):  # a few iterations of each solver are enough here
        try:
            fn(*a, **k)
        except _lib.NotConvergedError:
            pass

    w = torch.as_tensor(np.array(D.quad_points_and_weights()[1]), device="cuda")
    kw32 = torch.empty(32, 256, 256, dtype=torch.float32, device="cuda")
    _lib.check(L.jfg_weighted_field_f64(2, 256, 32, kap.data_ptr(), w.data_ptr(),
                                        A.kw.data_ptr(), kw32.data_ptr(),
                                        _lib.stream_handle()), "weighted_field")
    # two outer steps: the second updates the residual in FP32 (CUDA-core pass)
    bounded(S.solve, rhs, tol=1e-11, max_outer=2, maxiter_inner=200)
    bounded(pcg, VarCoefMatrix(T, kap[:4]), rhs[:4], tol=1e-10, maxiter=12)
    # 4. learned guess: features, inference, map back; one training step
    if os.path.exists(args.weights):
        model = sno_train.load(args.weights, batch=32)
        maps = sno_train.GridMaps()
        X, s = sno_train.features(torch.log(kap.float()), torch.as_tensor(f_h, device="cuda"),
                                  maps)
        g = sno_train.initial_guess(model, maps, X, s)
        bounded(S.solve, rhs, tol=1e-11, guess=g, max_outer=1, maxiter_inner=12)
    m = SNO(SNOConfig(batch=8), seed=0)
    Xs = torch.randn(8 * m.P, 16, device="cuda").to(torch.bfloat16)
    Bn = m.set_input(Xs)
    m.forward(Bn)
    m.backward(Bn, torch.randn(8 * m.P, device="cuda"))
    m.adam(1e-3)
    # 5. Helmholtz: structured apply, one group, and the grouped uneven batch
    Ns = rng.choice(np.arange(32, 257, 16), size=64)
    al = rng.uniform(0, 50, size=64)
    H = UnevenHelmholtzSolver("chebyshev", Ns, al)
    bounded(H.solve, [rng.standard_normal((N - 2, N - 2)) for N in Ns], tol=1e-11,
            max_refine=2)
    helmholtz_apply("chebyshev", 130, 4.0, torch.as_tensor(rng.standard_normal((8, 128, 128)),
                                                            device="cuda"))
    bounded(H.solve_per_group, [rng.standard_normal((N - 2, N - 2)) for N in Ns],
            tol=1e-11, max_refine=1)
    # 6. per-wavenumber banded solves: 4096 systems k^2 M + K (Legendre, n = 254)
    from jaxfun_gb300.la import TPMatricesWavenumberSolver

    Kd, Md = D.stiffness_matrix(), D.mass_matrix()
    n = Kd.shape[0]
    offs = (-2, 0, 2)
    k2 = np.arange(4096, dtype=float) ** 2 / 64.0
    band = np.zeros((4096, 3, n))
    for di, off in enumerate(offs):
        j = np.arange(max(off, 0), n + min(off, 0))
        band[:, di, j] = k2[:, None] * Md[j - off, j][None, :] + Kd[j - off, j][None, :]
    WS = TPMatricesWavenumberSolver(1, (4096, n), B_data_batch=band, poly_offsets=offs)
    WS.solve(torch.as_tensor(rng.standard_normal((4096, n)), device="cuda"))
    # 7. inhomogeneous Dirichlet lifting (affine transforms) and the coefficient
    #    evaluated from its logarithm (exp + weighting, moments), 32 problems
    def gb(x, y):
        return np.exp(-(x**2 + y**2))

    Dl = FunctionSpace(256, Legendre, bcs={"left": {"D": gb}, "right": {"D": gb}})
    TL = TensorProduct(Dl, Dl)
    cl = TL.backward(torch.as_tensor(rng.standard_normal((32, 254, 254)), device="cuda"))
    TL.forward(cl)
    VarCoefMatrix.from_log(T, torch.as_tensor(rng.standard_normal((32, 256, 256)),
                                              device="cuda"), standardize=True)
    torch.cuda.synchronize()
    print(json.dumps({"tour": "done", "device_status": int(L.jfg_device_status()),
                      "launches": int(L.jfg_launch_count())}), flush=True)
    return 0


def run_varcoef3d(args):
    """Secondary measurement (not the headline): 32 problems -div(kappa grad u) = f
    on 128^3 Legendre Dirichlet, kappa = exp(g) from the 3-D random-field recipe,
    mixed-precision solve vs plain FP64 PCG (on a subset), error vs a tight FP64
    solve."""
    import torch

    from jaxfun_gb300.galerkin import DIRICHLET, FunctionSpace, Legendre, TensorProduct
    from jaxfun_gb300.la import MixedVarCoefSolver, VarCoefMatrix, pcg

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    N, B = args.n3d, args.batch3d
    D = FunctionSpace(N, Legendre, bcs=DIRICHLET)
    T = TensorProduct(D, D, D)
    Lo = Legendre(N)
    To = TensorProduct(Lo, Lo, Lo)
    gen = torch.Generator(device="cuda").manual_seed(0)
    k = torch.arange(N, dtype=torch.float64, device="cuda")
    k2 = k[:, None, None] ** 2 + k[None, :, None] ** 2 + k[None, None, :] ** 2
    fs = ((1 + k[:, None, None]) * (1 + k[None, :, None]) * (1 + k[None, None, :])) ** -2.0
    gh = torch.randn((B, N, N, N), generator=gen, dtype=torch.float64, device="cuda") * (1 + k2) ** -1.5
    fh = torch.randn((B, N, N, N), generator=gen, dtype=torch.float64, device="cuda") * fs
    g = To.backward(gh)
    g = (g - g.mean(dim=(1, 2, 3), keepdim=True)) / g.std(dim=(1, 2, 3), keepdim=True)
    kap = torch.exp(g)
    b = T.scalar_product(To.backward(fh))
    A = VarCoefMatrix(T, kap)
    S = MixedVarCoefSolver(A, precond=args.precond)
    for _ in range(args.warmup):
        x, it_in, it_out = S.solve(b, tol=args.tol3d)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        x, it_in, it_out = S.solve(b, tol=args.tol3d)
    torch.cuda.synchronize()
    t = (time.perf_counter() - t0) / args.steps
    # learned initial guess (3-D spectral neural operator: 32^3 grid, 16^3 modes,
    # width 32), its inference inside the timed region
    learned = None
    w3 = os.path.join(ROOT, "jaxfun_gb300", "sno", "weights", "sno_varcoef3d_N128.npz")
    if os.path.exists(w3) and N == 128:
        from jaxfun_gb300.sno import train as sno_train

        model = sno_train.load(w3, batch=min(B, 16))
        maps = sno_train.GridMaps(N=N, n=model.cfg.n, guess_modes=args.guess_modes, ndim=3)
        f_grid = To.backward(fh)

        def solve_learned():
            X, sc = sno_train.features(torch.log(kap.float()), f_grid, maps)
            guess = sno_train.initial_guess(model, maps, X, sc)
            return S.solve(b, tol=args.tol3d, guess=guess)

        for _ in range(args.warmup):
            xl, il, ol = solve_learned()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            xl, il, ol = solve_learned()
        torch.cuda.synchronize()
        tl = (time.perf_counter() - t0) / args.steps
        learned = {"solves_per_s": B / tl, "inner_iterations_mean": float(il.mean()),
                   "outer_iterations_mean": float(ol.mean()), "x": xl}
    nf = min(B, 4)
    A4 = VarCoefMatrix(T, kap[:nf])
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    x64, it64 = pcg(A4, b[:nf], tol=args.fp64_tol3d, maxiter=3000)
    torch.cuda.synchronize()
    t64 = time.perf_counter() - t0
    xt, _ = pcg(A4, b[:nf], tol=1e-14, maxiter=4000)
    err = float(((x[:nf] - xt).abs().amax(dim=(1, 2, 3)) / xt.abs().amax(dim=(1, 2, 3))).max())
    err64 = float(((x64 - xt).abs().amax(dim=(1, 2, 3)) / xt.abs().amax(dim=(1, 2, 3))).max())
    line = {"workload": f"varcoef-poisson-3d-legendre-N{N}-batch{B}", "unit": "solves/s",
            "mixed_solves_per_s": B / t, "mixed_inner_iterations_mean": float(it_in.mean()),
            "mixed_outer_iterations_mean": float(it_out.mean()), "mixed_max_rel_err": err,
            "fp64_pcg_solves_per_s": nf / t64, "fp64_pcg_iterations_mean": float(it64.mean()),
            "fp64_pcg_max_rel_err": err64, "speedup": (B / t) / (nf / t64),
            "precond": S.precond}
    if learned is not None:
        xl = learned.pop("x")
        learned["max_rel_err"] = float(((xl[:nf] - xt).abs().amax(dim=(1, 2, 3))
                                        / xt.abs().amax(dim=(1, 2, 3))).max())
        learned["inner_iterations_saved_mean"] = (line["mixed_inner_iterations_mean"]
                                                  - learned["inner_iterations_mean"])
        learned["speedup_vs_fp64_pcg"] = learned["solves_per_s"] / (nf / t64)
        line["learned_mixed"] = learned
    print(json.dumps(line), flush=True)
    return 0


def run_ours(args):
    import numpy as np
    import torch

    from jaxfun_gb300 import _lib
    from jaxfun_gb300.galerkin import DIRICHLET, FunctionSpace, Legendre, TensorProduct
    from jaxfun_gb300.la import MixedVarCoefSolver, VarCoefMatrix

    from jaxfun_gb300 import replicas

    info = replicas.rank_info()
    world, rank, local = info.world, info.rank, info.local
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    L = _lib.lib()
    N = N_GRID
    n = N - 2
    B = args.batch
    D = FunctionSpace(N, Legendre, bcs=DIRICHLET)
    T = TensorProduct(D, D)
    kap_h, f_h = make_problems(B, N, seed0=replicas.seed_base(rank))  # own problems per rank
    # --host-loop (profiling aid): the legacy default stream, which cannot be
    # captured, so the refinement loop is host-driven and every kernel of the
    # solve is a separate launch in a profiler's list
    stream = torch.cuda.default_stream() if args.host_loop else torch.cuda.Stream()
    sh = 0 if args.host_loop else stream.cuda_stream
    with torch.cuda.stream(stream):
        # ---- resident inputs and plans (untimed setup)
        w = torch.as_tensor(np.array(D.quad_points_and_weights()[1]), device="cuda")
        kap = torch.as_tensor(kap_h, device="cuda")
        fgrid = torch.as_tensor(f_h, device="cuda")
        A = VarCoefMatrix(T, kap)                 # FP64 operator (kw = kappa w (x) w)
        solver = MixedVarCoefSolver(A, fused_dots=not args.no_fused_dots,
                                    schedule=args.schedule, precond=args.precond)
        SP = torch.as_tensor(np.array(D.scalar_product_matrix()), device="cuda")
        rhs = torch.empty(B, n, n, dtype=torch.float64, device="cuda")
        x = torch.empty(B, n, n, dtype=torch.float64, device="cuda")
        rows, cols = _lib.int_array([n, n]), _lib.int_array([N, N])
        tp_ws = torch.empty(L.jfg_tp_apply_workspace_size(2, rows, cols, B, 8),
                            dtype=torch.uint8, device="cuda")
        mws = torch.empty(solver.workspace_bytes(), dtype=torch.uint8, device="cuda")
        it_in = (_lib.C.c_int * B)()
        it_out = (_lib.C.c_int * B)()
        # learned initial guess: the trained spectral neural operator
        model = maps = None
        if not args.no_learned and os.path.exists(args.weights):
            from jaxfun_gb300.sno import train as sno_train

            model = sno_train.load(args.weights, batch=min(B, 128))
            maps = sno_train.GridMaps(guess_modes=args.guess_modes)
        guess = torch.empty(B, n, n, dtype=torch.float64, device="cuda")

    def learned_guess(kap_d=None, f_d=None):
        # network inputs (log kappa, f / rms(f), x, y) on its 64^2 grid, inference
        # on the tensor cores, and the map back to the first guess_modes^2
        # coefficients; the network reads FP32, so log kappa is taken in FP32
        # (the FP64 log alone cost ~0.5 ms per 128 problems on the FP64 units)
        kap_d = kap if kap_d is None else kap_d
        f_d = fgrid if f_d is None else f_d
        X, s = sno_train.features(torch.log(kap_d.float()), f_d, maps)
        guess.copy_(sno_train.initial_guess(model, maps, X, s))
        return guess

    def prepare(kap_d, f_d):
        # kw = kappa * w (x) w in FP64 and FP32; rhs = (f, v) scalar product in
        # double-FP32 arithmetic (FP64-class, ~3x the FP64 pipe's rate)
        _lib.check(L.jfg_weighted_field_f64(2, N, B, kap_d.data_ptr(), w.data_ptr(),
                                            A.kw.data_ptr(), solver.kw32.data_ptr(), sh),
                   "weighted_field")
        _lib.check(L.jfg_tp_apply_df64(2, rows, cols, B, _lib.ptr_array([SP.data_ptr()] * 2),
                                       f_d.data_ptr(), rhs.data_ptr(), tp_ws.data_ptr(),
                                       tp_ws.numel(), sh), "scalar_product")

    def solve(use_model=True, given=None, x_d=None, kap_d=None, f_d=None):
        g = learned_guess(kap_d, f_d) if (use_model and model is not None) else None
        if given is not None:
            g = given
        x_d = x if x_d is None else x_d
        st = L.jfg_pcg_varcoef_mixed_guess(_lib.C.byref(solver.plan), rhs.data_ptr(),
                                           x_d.data_ptr(), None if g is None else g.data_ptr(), 0,
                                           args.tol, args.inner_tol, 10, args.maxiter, it_in,
                                           it_out, mws.data_ptr(), mws.numel(), sh)
        _lib.check(st, "pcg_mixed")

    tuned_txt = None
    with torch.cuda.stream(stream):
        prepare(kap, fgrid)
        if not args.no_autotune:
            # untimed: each distinct tensor-core pass of the inner solve gets its
            # fastest launch configuration (kept for the process)
            tuned = solver.autotune(mws)
            tuned_txt = "; ".join(
                f"{t['signature'].split(':', 1)[1]} -> {t['schedule']}, {t['stages'] or 'max'} "
                f"stages, {t['store']} stores, mtile {t['mtile']} ({1e3 * t['ms']:.1f} us)"
                for t in tuned)
        for _ in range(args.warmup):
            solve()
        torch.cuda.synchronize()
        if dist is not None:
            dist.barrier()
        L.jfg_reset_launch_count()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        if args.profile:
            # a marker kernel (torch's spin kernel) before and after the timed
            # solves, so that a launch list can be cut to them
            torch.cuda._sleep(1000)
            torch.cuda.synchronize()
        with Clocks(local) as clk:
            torch.cuda.synchronize()
            e0.record(stream)
            for _ in range(args.steps):
                solve()
            e1.record(stream)
            e1.synchronize()
        if args.profile:
            torch.cuda._sleep(1000)
            torch.cuda.synchronize()
        launches = int(L.jfg_launch_count())
        t = e0.elapsed_time(e1) / 1e3
        clocks = clk.summary()
    t = replicas.max_time(t, dist, device="cuda")
    value = replicas.throughput(B * args.steps, world, t)
    its_in, its_out = np.array(it_in[:]), np.array(it_out[:])
    dev_status = int(L.jfg_device_status())
    if args.profile:
        # profiling run (launch lists): the setup, warm-up and timed solves only
        if rank == 0:
            print(json.dumps({"profile": "varcoef2d", "batch": B, "steps": args.steps,
                              "warmup": args.warmup, "ms_per_step": 1e3 * t / args.steps,
                              "launches_timed": launches, "device_status": dev_status}),
                  flush=True)
        return 0
    x_learned = x.clone()

    # ---- the same mixed solve from a zero start (what the learned guess gains)
    mixed_zero = None
    if model is not None:
        with torch.cuda.stream(stream):
            solve(use_model=False)
            torch.cuda.synchronize()
            e0.record(stream)
            for _ in range(max(1, args.steps)):
                solve(use_model=False)
            e1.record(stream)
            e1.synchronize()
            tz = e0.elapsed_time(e1) / 1e3 / max(1, args.steps)
            mixed_zero = {"solves_per_s": world * B / tz,
                          "inner_iterations_mean": float(np.mean(it_in[:])),
                          "outer_iterations_mean": float(np.mean(it_out[:])),
                          "max_rel_err": None}
            x_zero = x.clone()
        x.copy_(x_learned)

    # ---- plain FP64 PCG on the same problems (the comparison path), and the
    # accuracy check of the mixed answer against a tight FP64 solve of every
    # problem of the timed batch.  The comparator runs at the same batch, is
    # warmed up (its first call captures and instantiates its CUDA graph) and
    # stops at relative residual fp64_tol, the loosest rule that still gives
    # <= 1e-10 error on these problems (checked below).
    nf = min(B, args.fp64_batch)
    with torch.cuda.stream(stream):
        A64 = VarCoefMatrix(T, kap[:nf])
        from jaxfun_gb300.la import fd_preconditioner

        fac = fd_preconditioner(T)
        E, W, lam = fac.device_factors()
        sc = torch.ones(nf, dtype=torch.float64, device="cuda")
        ws64 = torch.empty(L.jfg_pcg_workspace_size(2, n, N, nf, 8), dtype=torch.uint8,
                           device="cuda")
        x64 = torch.empty(nf, n, n, dtype=torch.float64, device="cuda")
        it64 = (_lib.C.c_int * nf)()

        def solve64(xo, tol, its):
            st = L.jfg_pcg_varcoef_f64(2, n, N, nf, A64.ops.data_ptr(), A64.kw.data_ptr(),
                                       E.data_ptr(), W.data_ptr(), lam.data_ptr(), sc.data_ptr(),
                                       rhs[:nf].data_ptr(), xo.data_ptr(), 0, tol, args.maxiter,
                                       its, ws64.data_ptr(), ws64.numel(), sh)
            _lib.check(st, "pcg_f64")

        solve64(x64, args.fp64_tol, it64)     # warm-up (graph capture + instantiate)
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(args.fp64_steps):
            solve64(x64, args.fp64_tol, it64)
        e1.record(stream)
        e1.synchronize()
        t64 = e0.elapsed_time(e1) / 1e3 / args.fp64_steps
        xt = torch.empty_like(x64)
        solve64(xt, 1e-14, None)
        torch.cuda.synchronize()
        rel = lambda a: (a - xt).abs().amax(dim=(1, 2)) / xt.abs().amax(dim=(1, 2))  # noqa: E731
        err_mixed = float(rel(x[:nf]).max())
        err_fp64 = float(rel(x64).max())
        xt_cpu0 = xt[0].cpu().numpy()
        # What the guess can gain at this refinement schedule: the network's
        # guess error, and the same timed solve started from the tight FP64
        # solution itself (a perfect guess; the inner solve sees it rounded to
        # FP32) -- the ceiling of any learned start.
        guess_info = {}
        if model is not None and nf == B:
            gq = learned_guess()
            guess_info["learned_guess_rel_l2_mean"] = float(
                ((gq - xt).norm(dim=(1, 2)) / xt.norm(dim=(1, 2))).mean())
            guess_info["learned_guess_modes"] = int(maps.guess_modes)
            pg = xt.clone()
            solve(use_model=False, given=pg)
            torch.cuda.synchronize()
            e0.record(stream)
            for _ in range(max(1, args.steps)):
                solve(use_model=False, given=pg)
            e1.record(stream)
            e1.synchronize()
            tp = e0.elapsed_time(e1) / 1e3 / max(1, args.steps)
            guess_info["perfect_guess_solves_per_s"] = world * B / tp
            guess_info["perfect_guess_inner_iterations_mean"] = float(np.mean(it_in[:]))
            guess_info["perfect_guess_max_rel_err"] = float(rel(x).max())
            x.copy_(x_learned)
        if mixed_zero is not None:
            mixed_zero["max_rel_err"] = float(rel(x_zero[:nf]).max())
        x_cpu0 = x[0].cpu().numpy()
    fp64_value = world * nf / t64

    # ---- end to end through the C ABI with host buffers (pinned).  A serving
    # loop: the inputs of step i+1 are copied in on a copy stream while step i
    # solves, and step i's answer is read back while step i+1 solves (two
    # device sets of inputs and answers; every step's copies are inside the
    # timed region).
    kap_pin = torch.as_tensor(kap_h).pin_memory()
    f_pin = torch.as_tensor(f_h).pin_memory()
    x_pins = [torch.empty(B, n, n, dtype=torch.float64).pin_memory() for _ in range(2)]
    kap_b = [kap, torch.empty_like(kap)]
    f_b = [fgrid, torch.empty_like(fgrid)]
    x_b = [x, torch.empty_like(x)]
    cps = torch.cuda.Stream()
    ev_in = [torch.cuda.Event() for _ in range(2)]
    ev_used = [torch.cuda.Event() for _ in range(2)]
    ev_out = [torch.cuda.Event() for _ in range(2)]
    ev_read = [torch.cuda.Event() for _ in range(2)]
    e2e_steps = max(5, args.steps)

    def copy_in(j):
        with torch.cuda.stream(cps):
            cps.wait_event(ev_used[j])
            kap_b[j].copy_(kap_pin, non_blocking=True)
            f_b[j].copy_(f_pin, non_blocking=True)
            ev_in[j].record(cps)

    def serve(steps):
        for j in range(2):
            ev_used[j].record(stream)
            ev_read[j].record(stream)
        copy_in(0)
        for i in range(steps):
            j = i % 2
            if i + 1 < steps:
                copy_in(1 - j)
            with torch.cuda.stream(stream):
                stream.wait_event(ev_in[j])
                stream.wait_event(ev_read[j])
                prepare(kap_b[j], f_b[j])
                solve(x_d=x_b[j], kap_d=kap_b[j], f_d=f_b[j])
                ev_used[j].record(stream)
                ev_out[j].record(stream)
            with torch.cuda.stream(cps):
                cps.wait_event(ev_out[j])
                x_pins[j].copy_(x_b[j], non_blocking=True)
                ev_read[j].record(cps)
        torch.cuda.synchronize()

    serve(2)  # untimed: both answer buffers get their solve graph
    t0 = time.perf_counter()
    serve(e2e_steps)
    t_e2e = time.perf_counter() - t0
    for j in range(2):
        assert torch.equal(x_pins[j].to(x.device), x_b[j])
    h2d = 2 * B * N * N * 8
    d2h = B * n * n * 8

    # ---- roofline of the dominant kernel (tcgen05 contraction): roofline
    # time = max(useful FLOP / tensor peak, algorithmic bytes / HBM peak), the
    # fraction = roofline time / measured launch time, bound = the larger term
    pk, pk_kind = peaks()
    with torch.cuda.stream(stream):
        rf = roofline_microbench(B, N)
        rf32 = roofline_microbench(B, N, prec="tf32")
    f16_peak = pk["bf16_tflops"]           # dense FP16 rate = dense BF16 rate
    tf32_peak = pk["bf16_tflops"] / 2.0
    t_tensor = rf["flops"] / (f16_peak * 1e12)
    t_hbm = rf["bytes"] / (pk["hbm_gbs"] * 1e9)
    hbm_bound = t_hbm >= t_tensor
    tr = None
    if rank == 0 and not args.skip_transforms:
        with torch.cuda.stream(stream):
            tr = transform_roundtrip_keys()

    # ---- CPU baseline (bounded sample, rank 0, N=1 only); the oracle's tight
    # solve of problem 0 then checks our answer at the full size
    cpu = None
    err_oracle = err_fp64_oracle = None
    if rank == 0 and world == 1 and not args.skip_cpu:
        solve_cpu, _ = cpu_solver(N)
        t0 = time.perf_counter()
        nsamp = 0
        while nsamp < 2 or (time.perf_counter() - t0 < 10.0 and nsamp < 6):
            solve_cpu(kap_h[nsamp % B], f_h[nsamp % B])
            nsamp += 1
        dt = time.perf_counter() - t0
        cores = len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else os.cpu_count()
        cpu = {"value": nsamp / dt, "unit": "solves/s", "cores": cores, "kind": "port",
               "sample": f"{nsamp} single-problem FP64 PCG solves (N=256, tol 1e-10), "
                         "numpy/scipy on all host threads"}
        xo, _ = solve_cpu(kap_h[0], f_h[0], tol=1e-13)
        err_oracle = float(np.abs(x_cpu0 - xo).max() / np.abs(xo).max())
        err_fp64_oracle = float(np.abs(xt_cpu0 - xo).max() / np.abs(xo).max())

    if rank == 0:
        rl = {"bound": "hbm" if hbm_bound else "tensor",
              "achieved": rf["gbs"] if hbm_bound else rf["tflops_alg"],
              "peak": pk["hbm_gbs"] if hbm_bound else f16_peak,
              "unit": "GB/s" if hbm_bound else "TFLOP/s",
              "frac": max(t_tensor, t_hbm) / rf["t"],
              "traffic": (None if TC_TRAFFIC_PER_LAUNCH_B128 is None
                          else TC_TRAFFIC_PER_LAUNCH_B128 * B / 128),
              "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of one launch "
                                "at this shape with 128 problems, scaled by problems per launch",
              "kernel": "k_contract_tc<..., PREC=2> (tcgen05 kind::f16, scaled split FP16: "
                        "3 MMAs per K step)",
              "launch_M": rf["M"], "launch_P": rf["P"], "launch_K": rf["K"], "launch_batch": B,
              "launch_us": 1e6 * rf["t"], "flops_per_launch": rf["flops"],
              "bytes_per_launch": rf["bytes"],
              "roofline_us": 1e6 * max(t_tensor, t_hbm),
              "tensor_term_us": 1e6 * t_tensor, "hbm_term_us": 1e6 * t_hbm,
              "tflops_algorithmic": rf["tflops_alg"], "hbm_gbs_algorithmic": rf["gbs"],
              "tensor_frac": t_tensor / rf["t"],
              "issued_tflops": rf["tflops_issued"],
              "issued_frac": rf["tflops_issued"] / f16_peak,
              "hbm_frac": t_hbm / rf["t"],
              "tf32_variant_us": 1e6 * rf32["t"],
              "tf32_variant_frac": max(rf32["flops"] / (tf32_peak * 1e12), t_hbm) / rf32["t"],
              "peak_kind": f"{pk_kind}: HBM copy GB/s; tensor = bf16 burst (dense FP16 rate; "
                           "the split-TF32 variant against bf16 burst / 2)"}
        cfg = {"workload": "varcoef-poisson-2d-legendre-N256", "N": N, "batch": B,
               "path": ("learned guess (BF16 tcgen05 spectral neural operator) + "
                        if model is not None else "") +
                       "mixed: tcgen05 PCG (scaled split-FP16 operator, " +
                       {"bf16x3": "split-BF16", "bf16": "plain BF16",
                        "tf32": "split-TF32"}[solver.precond] +
                       " preconditioner) + FP64 refinement",
               "precond": solver.precond,
               "tol_relres": args.tol, "inner_tol": args.inner_tol,
               "inner_iterations_mean": float(its_in.mean()),
               "outer_iterations_mean": float(its_out.mean()),
               "max_rel_err_vs_fp64_tight": err_mixed,
               "err_problems_checked": nf,
               "max_rel_err_vs_oracle_problem0": err_oracle,
               "fp64_tight_vs_oracle_problem0": err_fp64_oracle,
               "fp64_pcg_solves_per_s": fp64_value,
               "fp64_pcg_batch": nf, "fp64_pcg_err": err_fp64,
               "fp64_pcg_stopping_rule": f"relres <= {args.fp64_tol:g} (loosest rule reaching "
                                         "<= 1e-10 error here; config 3 names 1e-10 relres)",
               "fp64_pcg_iterations_mean": float(np.mean(it64[:])),
               "speedup_vs_fp64_pcg": value / fp64_value,
               "device_status": dev_status,
               "autotuned_passes": tuned_txt,
               "l2": "inputs+workspace > L2 (129 MB) per step"}
        if mixed_zero is not None:
            cfg["mixed_zero_start_solves_per_s"] = mixed_zero["solves_per_s"]
            cfg["mixed_zero_start_inner_iterations_mean"] = mixed_zero["inner_iterations_mean"]
            cfg["mixed_zero_start_outer_iterations_mean"] = mixed_zero["outer_iterations_mean"]
            cfg["mixed_zero_start_max_rel_err"] = mixed_zero["max_rel_err"]
            cfg["learned_vs_zero_start_speedup"] = value / mixed_zero["solves_per_s"]
        if tr is not None:
            cfg.update(tr)
        cfg.update(guess_info)
        line = {
            "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32/f16x3+bf16x3+f64",
            "data": "synthetic (seeded; kappa=exp(GRF), config-3 recipe)",
            "config": cfg,
            "e2e": {"value": world * B * e2e_steps / t_e2e, "unit": "solves/s",
                    "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "steps": e2e_steps,
                    "copies": "pinned; step i+1's inputs copied in and step i-1's answer "
                              "read back on a copy stream while step i solves"},
            "gpu_launches": launches,
            "roofline": rl,
            "clocks": clocks,
            "cpu_baseline": cpu,
        }
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--batch", type=int, default=128)
    # stopping rules calibrated on seeded problems so that each path ends at
    # <= 1e-10 max relative error against a tight FP64 solve (checked below)
    ap.add_argument("--tol", type=float, default=1e-11, help="outer relative residual")
    # inner tolerance: the residual is updated in FP32 after the first correction,
    # and its error scales with the residual left by that correction; 5e-6 keeps
    # the answer at <= 6e-11 error with the scaled split-FP16 operator (1e-5 gave
    # 1.2e-10, and tightening the outer rule alone did not help)
    ap.add_argument("--inner-tol", type=float, default=5e-6)
    ap.add_argument("--fp64-tol", type=float, default=5e-12)
    ap.add_argument("--fp64-batch", type=int, default=128)
    ap.add_argument("--fp64-steps", type=int, default=1)
    ap.add_argument("--skip-transforms", action="store_true",
                    help="leave out the split-BF16 3-D transform round trip (config 1) keys")
    ap.add_argument("--maxiter", type=int, default=1000)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--schedule", default="sync", choices=["flat", "sync"],
                    help="refinement steps per problem (flat) or for the whole batch (sync)")
    ap.add_argument("--precond", default=None, choices=["bf16x3", "bf16", "tf32"],
                    help="arithmetic of the inner preconditioner's passes (default: the "
                         "solver's, plain BF16 in 2-D and split BF16 in 3-D)")
    ap.add_argument("--no-fused-dots", action="store_true",
                    help="inner PCG dots as separate kernels (not from the epilogues)")
    ap.add_argument("--no-autotune", action="store_true",
                    help="launch the inner solve's passes with the default configuration")
    ap.add_argument("--host-loop", action="store_true",
                    help="solve on the legacy default stream (host-driven loop, no whole-solve "
                         "graph): every kernel a separate launch for profilers")
    ap.add_argument("--profile", action="store_true",
                    help="stop after the timed solves (for ncu launch lists of the headline)")
    ap.add_argument("--no-learned", action="store_true", help="mixed solve from a zero start")
    ap.add_argument("--guess-modes", type=int, default=None,
                    help="Dirichlet modes per axis kept in the learned guess (default: 2-D 10, 3-D 16)")
    ap.add_argument("--weights", default=os.path.join(
        ROOT, "jaxfun_gb300", "sno", "weights", "sno_varcoef2d_N256.npz"))
    ap.add_argument("--kernel-only", nargs="?", const="contract", default=None,
                    choices=["contract", "contract_tf32", "contract_field",
                             "contract_field_tf32", "precond", "precond_bf16x3", "gemm",
                             "fp64", "df64", "transform", "transform_tf32"],
                    help="time one kernel and print its numbers (used for ncu captures): "
                         "contract = tcgen05 scaled split-FP16 contraction at the variable-"
                         "coefficient pass shape (M = 512, P = K = 256), B problems; "
                         "contract_tf32 = its split-TF32 variant; contract_field(_tf32) = "
                         "the second operator pass (2 segments, kappa*w field epilogue); "
                         "precond(_bf16x3) = a plain (split) BF16 preconditioner pass "
                         "(M = P = K = 256); "
                         "gemm = BF16 GEMM of the neural operator's spectral transform "
                         "(1024 x 64 x 4096 per sample, B samples); fp64 = FP64 CUDA-core "
                         "contraction at the variable-coefficient pass shape; df64 = the same "
                         "pass in double-FP32 arithmetic; transform(_tf32) = one split-BF16 "
                         "(split-TF32) pass of the 3-D 256^3 Chebyshev transform, B fields")
    ap.add_argument("--config", default="varcoef2d",
                    choices=["varcoef2d", "poisson2d", "transforms", "helmholtz", "varcoef3d",
                             "tour"],
                    help="varcoef2d: the headline; poisson2d: N = 64 Poisson solve + round "
                         "trip, latency and batched; transforms: batched 3-D Chebyshev "
                         "round trip; helmholtz: uneven Helmholtz batch; varcoef3d: 3-D "
                         "variable coefficient (secondary reports); tour: every kernel once "
                         "(for profiling)")
    ap.add_argument("--nprob", type=int, default=1024)
    ap.add_argument("--n3d", type=int, default=128)
    # 3-D stopping rules (calibrated to <= 1e-10 error on the seeded 128^3 problems)
    ap.add_argument("--tol3d", type=float, default=1e-12)
    ap.add_argument("--fp64-tol3d", type=float, default=5e-12)
    ap.add_argument("--batch3d", type=int, default=32)
    ap.add_argument("--n-transform", type=int, default=256)
    ap.add_argument("--fields", type=int, default=16)
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.config == "poisson2d":
        return run_poisson2d(args)
    if args.config == "transforms":
        return run_transforms(args)
    if args.config == "helmholtz":
        return run_helmholtz(args)
    if args.config == "varcoef3d":
        return run_varcoef3d(args)
    if args.config == "tour":
        return run_tour(args)
    if args.kernel_only:
        import torch

        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        if args.kernel_only in ("contract", "contract_tf32", "contract_field",
                                "contract_field_tf32"):
            prec = "tf32" if args.kernel_only.endswith("tf32") else "f16x3"
            out = {"kernel": "k_contract_tc",
                   **roofline_microbench(args.batch, N_GRID, reps=3, prec=prec,
                                         field_pass=args.kernel_only.startswith(
                                             "contract_field"))}
        elif args.kernel_only in ("precond", "precond_bf16x3"):
            prec = "bf16x3" if args.kernel_only.endswith("bf16x3") else "bf16"
            out = {"kernel": "k_contract_tc",
                   **roofline_microbench(args.batch, N_GRID, reps=3, M=N_GRID, prec=prec)}
        else:
            out = other_kernel_microbench(args.kernel_only, args.batch)
        print(json.dumps({"batch": args.batch, **out}), flush=True)
        return 0
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
