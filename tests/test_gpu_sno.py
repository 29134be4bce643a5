"""BF16 tcgen05 GEMM and the spectral neural operator's GPU training kernels.

The GEMM is checked against a plain PyTorch FP32 reference of the same BF16
operands (tolerance 2e-3 relative: FP32 accumulation, BF16 outputs rounded);
the network's loss and gradients against the FP64 NumPy oracle
(oracle/sno.py) fed the same BF16-rounded weights and inputs (tolerance 3e-2
relative per parameter tensor: activations are stored in BF16 on the GPU)."""

import ctypes as C

import numpy as np
import pytest
import torch

from jaxfun_gb300 import _lib
from jaxfun_gb300.sno.model import CIN, SNO, SNOConfig, transform_matrices
from oracle import sno as OS

pytestmark = pytest.mark.gpu


def gemm(A, B, M, N, K, lda, ldb, **kw):
    d = _lib.GemmDesc()
    d.batch = kw.pop("batch", 1)
    d.M, d.N, d.K, d.ksplit = M, N, K, kw.pop("ksplit", 1)
    d.lda, d.ldb = lda, ldb
    d.a_batch, d.b_batch = kw.pop("a_batch", 0), kw.pop("b_batch", 0)
    d.alpha = kw.pop("alpha", 1.0)
    d.act = kw.pop("act", 0)
    for name in ("add", "bias", "gg", "d32", "pre", "dbf", "dtbf"):
        t = kw.pop(name, None)
        setattr(d, name, None if t is None else t.data_ptr())
    for k, v in kw.items():
        setattr(d, k, v)
    st = _lib.lib().jfg_gemm_bf16(C.byref(d), A.data_ptr(), B.data_ptr(), _lib.stream_handle())
    assert st == 0, _lib.status_string(st)
    torch.cuda.synchronize()
    assert _lib.lib().jfg_device_status() == 0


def rel(a, b):
    return float((a - b).abs().max() / b.abs().max())


@pytest.mark.parametrize("M,N,K", [(128, 64, 64), (300, 16, 16), (1024, 64, 4096), (77, 200, 136)])
def test_gemm_plain(M, N, K):
    g = torch.Generator(device="cuda").manual_seed(M + N + K)
    A = torch.randn(M, K, generator=g, device="cuda").to(torch.bfloat16)
    B = torch.randn(N, K, generator=g, device="cuda").to(torch.bfloat16)
    ref = A.float() @ B.float().t()
    d32 = torch.empty(M, N, device="cuda")
    dbf = torch.empty(M, N, device="cuda", dtype=torch.bfloat16)
    dtbf = torch.empty(N, M, device="cuda", dtype=torch.bfloat16)
    gemm(A, B, M, N, K, K, K, d32=d32, ld_d32=N, dbf=dbf, ld_dbf=N, dtbf=dtbf, ld_dtbf=M)
    assert rel(d32, ref) < 1e-4
    assert rel(dbf.float(), ref) < 1e-2
    assert rel(dtbf.float().t(), ref) < 1e-2


def test_gemm_epilogues_batched_and_split():
    g = torch.Generator(device="cuda").manual_seed(7)
    Bt, P, C_, NM = 3, 256, 16, 64
    # batched with samples interleaved inside each row of B (the spectral layout)
    A = torch.randn(NM, P, generator=g, device="cuda").to(torch.bfloat16)
    Ucf = torch.randn(C_, Bt * P, generator=g, device="cuda").to(torch.bfloat16)
    out = torch.empty(Bt, NM, C_, device="cuda")
    gemm(A, Ucf, NM, C_, P, P, Bt * P, batch=Bt, b_batch=P, d32=out, ld_d32=C_,
         d32_batch=NM * C_)
    ref = torch.stack([A.float() @ Ucf[:, b * P:(b + 1) * P].float().t() for b in range(Bt)])
    assert rel(out, ref) < 1e-4
    # add + bias + GELU + pre
    R = 512
    X = torch.randn(R, C_, generator=g, device="cuda").to(torch.bfloat16)
    W = torch.randn(C_, C_, generator=g, device="cuda").to(torch.bfloat16)
    add = torch.randn(R, C_, generator=g, device="cuda")
    bias = torch.randn(C_, generator=g, device="cuda")
    pre = torch.empty(R, C_, device="cuda")
    y = torch.empty(R, C_, device="cuda")
    gemm(X, W, R, C_, C_, C_, C_, add=add, ld_add=C_, bias=bias, act=1, pre=pre, ld_pre=C_,
         d32=y, ld_d32=C_)
    z = X.float() @ W.float().t() + add + bias
    assert rel(pre, z) < 1e-4
    assert rel(y, torch.nn.functional.gelu(z)) < 1e-4
    # GELU-derivative multiply
    gg = torch.randn(R, C_, generator=g, device="cuda")
    gemm(X, W, R, C_, C_, C_, C_, gg=gg, ld_gg=C_, d32=y, ld_d32=C_)
    x = gg.clone().requires_grad_(True)
    torch.nn.functional.gelu(x).backward(torch.ones_like(x))
    assert rel(y, (X.float() @ W.float().t()) * x.grad) < 1e-4
    # split-K into an accumulator
    Kl = 8192
    A2 = torch.randn(C_, Kl, generator=g, device="cuda").to(torch.bfloat16)
    B2 = torch.randn(C_, Kl, generator=g, device="cuda").to(torch.bfloat16)
    acc = torch.zeros(C_, C_, device="cuda")
    gemm(A2, B2, C_, C_, Kl, Kl, Kl, ksplit=16, d32=acc, ld_d32=C_)
    assert rel(acc, A2.float() @ B2.float().t()) < 1e-4


def _small_model(seed=0):
    cfg = SNOConfig(n=16, width=16, modes=8, layers=2, batch=2)
    m = SNO(cfg, seed=seed)
    rng = np.random.default_rng(seed + 1)
    for k, p in m.params.items():  # non-trivial biases / projection
        if k.startswith("b") or k == "W_p2":
            p.copy_(torch.as_tensor(0.1 * rng.standard_normal(p.shape), dtype=torch.float32))
    m._sync_bf16()
    return m, cfg


def test_sno_gradients_match_oracle():
    m, cfg = _small_model()
    Bt, P = cfg.batch, cfg.n * cfg.n
    rng = np.random.default_rng(5)
    X = np.zeros((Bt * P, CIN), dtype=np.float32)
    X[:, :4] = rng.standard_normal((Bt * P, 4))
    Xb = torch.as_tensor(X, device="cuda").to(torch.bfloat16)
    tgt = torch.as_tensor(rng.standard_normal(Bt * P), dtype=torch.float32, device="cuda")
    m.set_input(Xb)
    pred = m.forward(Bt)[:, 0].clone()
    loss = m.backward(Bt, tgt)
    # oracle with the operands the GPU sees (BF16-rounded weights, transforms, inputs)
    bf = lambda t: t.to(torch.bfloat16).double().cpu().numpy()  # noqa: E731
    params = {k: (bf(v) if k in m.matrix_names() else v.double().cpu().numpy())
              for k, v in m.params.items()}
    Phi, Psi = transform_matrices(cfg.n, cfg.modes)
    Phi = bf(torch.as_tensor(Phi))
    Psi = bf(torch.as_tensor(Psi))
    loss_o, pred_o, g_o = OS.forward_backward(params, Phi, Psi, bf(Xb), tgt.double().cpu().numpy(),
                                              Bt, cfg.layers)
    assert abs(loss - loss_o) < 2e-2 * loss_o
    assert np.abs(pred.cpu().numpy() - pred_o[:, 0]).max() < 2e-2 * np.abs(pred_o[:, 0]).max()
    for k, go in g_o.items():
        gg = m.grads[k].double().cpu().numpy()
        err = np.linalg.norm(gg - go) / max(np.linalg.norm(go), 1e-30)
        assert err < 3e-2, (k, err)


def test_sno3d_gradients_match_oracle():
    """The same network on a 3-D grid (8^3 points, 4^3 modes): forward and
    backward against the oracle's explicit chain rule."""
    cfg = SNOConfig(n=8, width=16, modes=4, layers=2, batch=2, ndim=3)
    m = SNO(cfg, seed=4)
    rng = np.random.default_rng(9)
    for k, p in m.params.items():
        if k.startswith("b") or k == "W_p2":
            p.copy_(torch.as_tensor(0.1 * rng.standard_normal(p.shape), dtype=torch.float32))
    m._sync_bf16()
    Bt, P = cfg.batch, cfg.n ** 3
    X = np.zeros((Bt * P, CIN), dtype=np.float32)
    X[:, :5] = rng.standard_normal((Bt * P, 5))
    Xb = torch.as_tensor(X, device="cuda").to(torch.bfloat16)
    tgt = torch.as_tensor(rng.standard_normal(Bt * P), dtype=torch.float32, device="cuda")
    m.set_input(Xb)
    pred = m.forward(Bt)[:, 0].clone()
    loss = m.backward(Bt, tgt)
    bf = lambda t: t.to(torch.bfloat16).double().cpu().numpy()  # noqa: E731
    params = {k: (bf(v) if k in m.matrix_names() else v.double().cpu().numpy())
              for k, v in m.params.items()}
    Phi, Psi = transform_matrices(cfg.n, cfg.modes, 3)
    Phi = bf(torch.as_tensor(Phi))
    Psi = bf(torch.as_tensor(Psi))
    loss_o, pred_o, g_o = OS.forward_backward(params, Phi, Psi, bf(Xb), tgt.double().cpu().numpy(),
                                              Bt, cfg.layers)
    assert abs(loss - loss_o) < 2e-2 * loss_o
    assert np.abs(pred.cpu().numpy() - pred_o[:, 0]).max() < 2e-2 * np.abs(pred_o[:, 0]).max()
    for k, go in g_o.items():
        gg = m.grads[k].double().cpu().numpy()
        err = np.linalg.norm(gg - go) / max(np.linalg.norm(go), 1e-30)
        assert err < 3e-2, (k, err)


def test_sno_training_reduces_loss():
    m, cfg = _small_model(seed=3)
    Bt, P = cfg.batch, cfg.n * cfg.n
    rng = np.random.default_rng(9)
    X = np.zeros((Bt * P, CIN), dtype=np.float32)
    X[:, :4] = rng.standard_normal((Bt * P, 4))
    Xb = torch.as_tensor(X, device="cuda").to(torch.bfloat16)
    tgt = torch.as_tensor(np.tanh(X[:, 0] + 0.5 * X[:, 1]), device="cuda")
    losses = []
    for _ in range(60):
        m.set_input(Xb)
        m.forward(Bt)
        losses.append(m.backward(Bt, tgt))
        m.adam(3e-3)
    assert losses[-1] < 0.3 * losses[0], losses[::10]


def test_learned_guess_saves_iterations():
    """What the trained network gains: on held-out seeded problems of the
    variable-coefficient benchmark (N = 256), starting the first inner solve
    from the learned guess needs fewer inner PCG iterations than the zero
    start, and both answers are within 1e-10 of a tight FP64 solve."""
    import os

    from jaxfun_gb300.la import MixedVarCoefSolver, VarCoefMatrix, pcg
    from jaxfun_gb300.sno import train as T

    path = os.path.join(os.path.dirname(T.__file__), "weights", "sno_varcoef2d_N256.npz")
    model = T.load(path, batch=16)
    maps = T.GridMaps()
    data = T.generate(16, seed=7, maps=maps, keep_fine=True, log=lambda *_: None)
    kap, f, b, _ = data["fine"][0]
    A = VarCoefMatrix(maps.T, kap)
    S = MixedVarCoefSolver(A)
    xt, _ = pcg(A, b, tol=1e-14, maxiter=3000)
    g = T.initial_guess(model, maps, data["X"], data["s"])
    res = {}
    for name, guess in (("zero", None), ("learned", g)):
        x, it_in, _ = S.solve(b, tol=1e-11, inner_tol=1e-5, guess=guess)
        err = float(((x - xt).abs().amax(dim=(1, 2)) / xt.abs().amax(dim=(1, 2))).max())
        assert err <= 1e-10, (name, err)
        res[name] = float(np.mean(it_in))
    assert res["learned"] < 0.97 * res["zero"], res
    # the guess itself is a usable approximation (coefficient-space L2, 32 modes)
    rel = ((g - xt).norm(dim=(1, 2)) / xt.norm(dim=(1, 2))).mean()
    assert float(rel) < 0.3


def test_learned_guess_saves_iterations_3d():
    """The 3-D network (32^3 grid, 16^3 modes, width 32) on held-out 128^3
    problems: fewer inner iterations than the zero start, both answers within
    1e-10 of a tight FP64 solve (3-D stopping rule 1e-12)."""
    import os

    from jaxfun_gb300.la import MixedVarCoefSolver, VarCoefMatrix, pcg
    from jaxfun_gb300.sno import train as T

    path = os.path.join(os.path.dirname(T.__file__), "weights", "sno_varcoef3d_N128.npz")
    model = T.load(path, batch=8)
    maps = T.GridMaps(N=128, n=model.cfg.n, ndim=3)
    data = T.generate(8, seed=11, maps=maps, chunk=8, keep_fine=True, log=lambda *_: None)
    kap, f, b, _ = data["fine"][0]
    A = VarCoefMatrix(maps.T, kap)
    S = MixedVarCoefSolver(A)
    xt, _ = pcg(A, b, tol=1e-14, maxiter=4000)
    g = T.initial_guess(model, maps, data["X"], data["s"])
    res = {}
    for name, guess in (("zero", None), ("learned", g)):
        x, it_in, _ = S.solve(b, tol=1e-12, inner_tol=1e-5, guess=guess)
        err = float(((x - xt).abs().amax(dim=(1, 2, 3)) / xt.abs().amax(dim=(1, 2, 3))).max())
        assert err <= 1e-10, (name, err)
        res[name] = float(np.mean(it_in))
    assert res["learned"] < res["zero"], res
