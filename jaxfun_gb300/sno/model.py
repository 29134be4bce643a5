"""Spectral neural operator (SNO) for the variable-coefficient initial guess.

Architecture (on an n^d Legendre-Gauss grid, d = 2 or 3, channel width C, L
spectral layers, nm^d retained Legendre modes):

    lift     U0 = X W_lift^T + b_lift                       X: (logk, f/s, x, y[, z], 0...) 16 ch
    layer l  U_{l+1} = act( Psi (R_l . (Phi U_l)) + U_l W_l^T + b_l )   act = GELU except last
    project  Q = GELU(U_L W_p1^T + b_p1);  u = Q W_p2^T + b_p2   (channel 0)

Phi (nm^d x n^d) is the truncated Legendre forward transform, Psi (n^d x nm^d)
the backward transform, R_l[q] a C x C channel mixing per mode q.  Every
contraction runs on the tensor cores through ``jfg_gemm_bf16`` (BF16 operands,
FP32 accumulation, fused bias/GELU/residual/GELU-derivative epilogues that write
row-major and transposed copies); mode mixing, bias gradients, the loss and
Adam are small CUDA-core kernels.  Activations are kept in two BF16 layouts:
"cl" (rows = (sample, pixel), channels contiguous) for contractions over
channels and "cf" (channels x (sample, pixel)) for contractions over pixels.
"""

from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np
import torch

from .. import _lib
from ..galerkin.spaces import Legendre

BF = torch.bfloat16
F32 = torch.float32
CIN = 16  # input channels (padded to one BF16 MMA K step)
COUT = 16  # projection output channels (padded; channel 0 is the prediction)


@dataclass
class SNOConfig:
    n: int = 64        # grid points per axis
    width: int = 64    # channels C
    modes: int = 32    # retained modes per axis
    layers: int = 4
    batch: int = 32    # training batch
    ndim: int = 2      # 2 (n x n grid) or 3 (n x n x n grid)


def transform_matrices(n: int, modes: int, ndim: int = 2) -> tuple[np.ndarray, np.ndarray]:
    """Phi (modes^d x n^d): truncated orthogonal Legendre forward transform on
    the n-point Gauss grid in d = ndim dimensions; Psi (n^d x modes^d): the
    backward transform."""
    L = Legendre(n)
    F = L.forward_matrix()[:modes, :]      # (modes, n)
    B = L.backward_matrix()[:, :modes]     # (n, modes)
    Phi, Psi = F, B
    for _ in range(ndim - 1):
        Phi, Psi = np.kron(Phi, F), np.kron(Psi, B)
    return Phi, Psi


def _dev(a, dtype):
    return torch.as_tensor(np.ascontiguousarray(a), device="cuda").to(dtype).contiguous()


class SNO:
    """Parameters, optimizer state, activation buffers and GPU passes."""

    def __init__(self, cfg: SNOConfig, seed: int = 0):
        self.cfg = cfg
        n, C_, m, L = cfg.n, cfg.width, cfg.modes, cfg.layers
        self.P = n ** cfg.ndim
        self.NM = m ** cfg.ndim
        rng = np.random.default_rng(seed)
        Phi, Psi = transform_matrices(n, m, cfg.ndim)
        self.Phi = _dev(Phi, BF)
        self.Psi = _dev(Psi, BF)
        self.PhiT = _dev(Phi.T, BF)
        self.PsiT = _dev(Psi.T, BF)
        # ---- parameters (FP32 masters) ----
        p = {}
        p["W_lift"] = rng.standard_normal((C_, CIN)) * np.sqrt(1.0 / 4)
        p["W_lift"][:, 2 + cfg.ndim:] = 0.0  # inputs: log kappa, f, coordinates
        p["b_lift"] = np.zeros(C_)
        for l in range(L):
            p[f"W{l}"] = rng.standard_normal((C_, C_)) * np.sqrt(1.0 / C_)
            p[f"b{l}"] = np.zeros(C_)
            p[f"R{l}"] = rng.standard_normal((self.NM, C_, C_)) * (1.0 / C_)
        p["W_p1"] = rng.standard_normal((C_, C_)) * np.sqrt(2.0 / C_)
        p["b_p1"] = np.zeros(C_)
        p["W_p2"] = np.zeros((COUT, C_))
        p["W_p2"][0] = rng.standard_normal(C_) * np.sqrt(1.0 / C_)
        p["b_p2"] = np.zeros(COUT)
        self.params = {k: _dev(v, F32) for k, v in p.items()}
        self.grads = {k: torch.zeros_like(v) for k, v in self.params.items()}
        self.m = {k: torch.zeros_like(v) for k, v in self.params.items()}
        self.v = {k: torch.zeros_like(v) for k, v in self.params.items()}
        self.step_count = 0
        self._sync_bf16()
        self._bufs_batch = 0

    # ------------------------------------------------------------------ params
    def matrix_names(self):
        return ["W_lift", "W_p1", "W_p2"] + [f"W{l}" for l in range(self.cfg.layers)]

    def _sync_bf16(self):
        """BF16 copies (and transposes) of the weight matrices for the GEMMs."""
        self.wbf = {}
        self.wtbf = {}
        for k in self.matrix_names():
            self.wbf[k] = self.params[k].to(BF).contiguous()
            self.wtbf[k] = self.params[k].t().contiguous().to(BF)

    def state_dict(self) -> dict[str, np.ndarray]:
        out = {k: v.detach().cpu().numpy() for k, v in self.params.items()}
        out["_config"] = np.array([self.cfg.n, self.cfg.width, self.cfg.modes, self.cfg.layers,
                                   self.cfg.ndim])
        return out

    def load_state_dict(self, sd: dict[str, np.ndarray]):
        for k in self.params:
            self.params[k].copy_(torch.as_tensor(np.asarray(sd[k], dtype=np.float32)))
        self._sync_bf16()

    # ------------------------------------------------------------------ buffers
    def _ensure(self, Bt: int):
        if self._bufs_batch == Bt:
            return
        C_, P, NM, L = self.cfg.width, self.P, self.NM, self.cfg.layers
        R = Bt * P
        z = lambda *s, dt=BF: torch.empty(s, dtype=dt, device="cuda")  # noqa: E731
        self.X_cl, self.X_cf = z(R, CIN), z(CIN, R)
        self.U_cl = [z(R, C_) for _ in range(L + 1)]
        self.U_cf = [z(C_, R) for _ in range(L + 1)]
        self.Zpre = [z(R, C_, dt=F32) for _ in range(L)]
        self.Uhat = [z(Bt, NM, C_, dt=F32) for _ in range(L)]
        self.Wh_cf = z(Bt, C_, NM)
        self.S = z(R, C_, dt=F32)
        self.Q1pre = z(R, C_, dt=F32)
        self.Q1_cl, self.Q1_cf = z(R, C_), z(C_, R)
        self.pred = z(R, COUT, dt=F32)
        self.dq_cl, self.dq_cf = z(R, COUT), z(COUT, R)
        self.dZ_cl, self.dZ_cf = z(R, C_), z(C_, R)
        self.dZ2_cl, self.dZ2_cf = z(R, C_), z(C_, R)
        self.dWh = z(Bt, NM, C_, dt=F32)
        self.dUh_cf = z(Bt, C_, NM)
        self.T1 = z(R, C_, dt=F32)
        self.loss_acc = z(1, dt=F32)
        self._bufs_batch = Bt

    # ------------------------------------------------------------------ kernels
    def _gemm(self, A, B, M, N, K, lda, ldb, batch=1, a_batch=0, b_batch=0, ksplit=1, **kw):
        d = _lib.GemmDesc()
        d.batch, d.M, d.N, d.K, d.ksplit = batch, M, N, K, ksplit
        d.lda, d.a_batch, d.ldb, d.b_batch = lda, a_batch, ldb, b_batch
        d.alpha = kw.pop("alpha", 1.0)
        d.act = kw.pop("act", 0)
        for name in ("add", "bias", "gg", "d32", "pre", "dbf", "dtbf"):
            t = kw.pop(name, None)
            setattr(d, name, None if t is None else t.data_ptr())
        for name, val in kw.items():
            setattr(d, name, val)
        st = _lib.lib().jfg_gemm_bf16(C.byref(d), A.data_ptr(), B.data_ptr(),
                                      _lib.stream_handle())
        _lib.check(st, "jfg_gemm_bf16")

    def _colsum(self, src, rows, n, out):
        _lib.check(_lib.lib().jfg_colsum_bf16(rows, n, src.data_ptr(), out.data_ptr(), 0,
                                              _lib.stream_handle()), "colsum")

    # ------------------------------------------------------------------ passes
    def set_input(self, x_cl: torch.Tensor, train: bool = True):
        """x_cl: (Bt*P, 16) BF16 input channels (rows = (sample, pixel)).  The
        channel-first copy is kept only for training (the lift's weight
        gradient)."""
        Bt = x_cl.shape[0] // self.P
        self._ensure(Bt)
        self.X_cl.copy_(x_cl)
        if train:
            self.X_cf.copy_(x_cl.t())
        return Bt

    def forward(self, Bt: int, train: bool = True) -> torch.Tensor:
        """Forward pass on self.X_cl / X_cf; returns pred (Bt*P, 16) FP32 (col 0).
        With train=False (inference) the GEMM epilogues skip what only the
        backward pass reads: the FP32 pre-activations and the channel-first
        copies of the last spectral layer's output and of the projection's
        hidden layer."""
        C_, P, NM, L = self.cfg.width, self.P, self.NM, self.cfg.layers
        R = Bt * P
        L_ = _lib.lib()
        sh = _lib.stream_handle()
        # lift (no activation)
        self._gemm(self.X_cl, self.wbf["W_lift"], R, C_, CIN, CIN, CIN,
                   bias=self.params["b_lift"], dbf=self.U_cl[0], ld_dbf=C_,
                   dtbf=self.U_cf[0], ld_dtbf=R)
        for l in range(L):
            # Uhat[b] = Phi U_cf[:, b]^T                      (NM x C per sample)
            self._gemm(self.Phi, self.U_cf[l], NM, C_, P, P, R, batch=Bt, b_batch=P,
                       d32=self.Uhat[l], ld_d32=C_, d32_batch=NM * C_)
            _lib.check(L_.jfg_sno_modemix_fwd(Bt, NM, C_, self.params[f"R{l}"].data_ptr(),
                                              self.Uhat[l].data_ptr(), self.Wh_cf.data_ptr(), sh),
                       "modemix_fwd")
            # S[b] = Psi Wh_cf[b]^T                          (P x C per sample)
            self._gemm(self.Psi, self.Wh_cf, P, C_, NM, NM, NM, batch=Bt, b_batch=C_ * NM,
                       d32=self.S, ld_d32=C_, d32_batch=P * C_)
            last = l == L - 1
            self._gemm(self.U_cl[l], self.wbf[f"W{l}"], R, C_, C_, C_, C_,
                       add=self.S, ld_add=C_, bias=self.params[f"b{l}"],
                       act=0 if last else 1,
                       pre=None if (last or not train) else self.Zpre[l], ld_pre=C_,
                       dbf=self.U_cl[l + 1], ld_dbf=C_,
                       dtbf=self.U_cf[l + 1] if (train or not last) else None, ld_dtbf=R)
        self._gemm(self.U_cl[L], self.wbf["W_p1"], R, C_, C_, C_, C_, bias=self.params["b_p1"],
                   act=1, pre=self.Q1pre if train else None, ld_pre=C_, dbf=self.Q1_cl,
                   ld_dbf=C_, dtbf=self.Q1_cf if train else None, ld_dtbf=R)
        self._gemm(self.Q1_cl, self.wbf["W_p2"], R, COUT, C_, C_, C_, bias=self.params["b_p2"],
                   d32=self.pred, ld_d32=COUT)
        return self.pred

    def backward(self, Bt: int, target: torch.Tensor) -> float:
        """Backward pass for 0.5*mean((pred - target)^2); fills self.grads.
        Returns the loss (synchronises on its read)."""
        C_, P, NM, L = self.cfg.width, self.P, self.NM, self.cfg.layers
        R = Bt * P
        L_ = _lib.lib()
        sh = _lib.stream_handle()
        g = self.grads
        ks = max(1, min(64, R // 4096))
        self.loss_acc.zero_()
        _lib.check(L_.jfg_sno_mse(R, self.pred.data_ptr(), COUT, target.data_ptr(),
                                  self.dq_cl.data_ptr(), self.dq_cf.data_ptr(),
                                  self.loss_acc.data_ptr(), sh), "mse")
        # projection
        g["W_p2"].zero_()
        self._gemm(self.dq_cf, self.Q1_cf, COUT, C_, R, R, R, ksplit=ks, d32=g["W_p2"], ld_d32=C_)
        self._colsum(self.dq_cl, R, COUT, g["b_p2"])
        self._gemm(self.dq_cl, self.wtbf["W_p2"], R, C_, COUT, COUT, COUT, gg=self.Q1pre,
                   ld_gg=C_, dbf=self.dZ_cl, ld_dbf=C_, dtbf=self.dZ_cf, ld_dtbf=R)
        g["W_p1"].zero_()
        self._gemm(self.dZ_cf, self.U_cf[L], C_, C_, R, R, R, ksplit=ks, d32=g["W_p1"], ld_d32=C_)
        self._colsum(self.dZ_cl, R, C_, g["b_p1"])
        # dU_L (the last layer has no activation: this is its dZ)
        self._gemm(self.dZ_cl, self.wtbf["W_p1"], R, C_, C_, C_, C_, dbf=self.dZ2_cl, ld_dbf=C_,
                   dtbf=self.dZ2_cf, ld_dtbf=R)
        dz_cl, dz_cf, nz_cl, nz_cf = self.dZ2_cl, self.dZ2_cf, self.dZ_cl, self.dZ_cf
        for l in range(L - 1, -1, -1):
            g[f"W{l}"].zero_()
            self._gemm(dz_cf, self.U_cf[l], C_, C_, R, R, R, ksplit=ks, d32=g[f"W{l}"],
                       ld_d32=C_)
            self._colsum(dz_cl, R, C_, g[f"b{l}"])
            # dWh[b] = Psi^T dZ_cf[:, b]^T                   (NM x C per sample)
            self._gemm(self.PsiT, dz_cf, NM, C_, P, P, R, batch=Bt, b_batch=P, d32=self.dWh,
                       ld_d32=C_, d32_batch=NM * C_)
            _lib.check(L_.jfg_sno_modemix_bwd(Bt, NM, C_, self.params[f"R{l}"].data_ptr(),
                                              self.Uhat[l].data_ptr(), self.dWh.data_ptr(),
                                              self.dUh_cf.data_ptr(), g[f"R{l}"].data_ptr(), sh),
                       "modemix_bwd")
            # dU_l = dZ W_l + Phi^T dUh ; times GELU'(Zpre_{l-1}) for l >= 1
            self._gemm(dz_cl, self.wtbf[f"W{l}"], R, C_, C_, C_, C_, d32=self.T1, ld_d32=C_)
            gg = self.Zpre[l - 1] if l >= 1 else None
            self._gemm(self.PhiT, self.dUh_cf, P, C_, NM, NM, NM, batch=Bt, b_batch=C_ * NM,
                       add=self.T1, ld_add=C_, add_batch=P * C_, gg=gg, ld_gg=C_,
                       gg_batch=P * C_, dbf=nz_cl, ld_dbf=C_, dbf_batch=P * C_, dtbf=nz_cf,
                       ld_dtbf=R, dtbf_batch=P)
            dz_cl, dz_cf, nz_cl, nz_cf = nz_cl, nz_cf, dz_cl, dz_cf
        # lift
        g["W_lift"].zero_()
        self._gemm(dz_cf, self.X_cf, C_, CIN, R, R, R, ksplit=ks, d32=g["W_lift"], ld_d32=CIN)
        self._colsum(dz_cl, R, C_, g["b_lift"])
        return float(self.loss_acc.item()) * 0.5 / R

    def adam(self, lr: float, beta1=0.9, beta2=0.999, eps=1e-8):
        self.step_count += 1
        L_ = _lib.lib()
        sh = _lib.stream_handle()
        mats = set(self.matrix_names())
        for k, p in self.params.items():
            pb = self.wbf[k] if k in mats else None
            ptb = self.wtbf[k] if k in mats else None
            rows, cols = (p.shape[0], p.shape[1]) if k in mats else (0, 0)
            st = L_.jfg_adam_step(p.numel(), p.data_ptr(), self.grads[k].data_ptr(),
                                  self.m[k].data_ptr(), self.v[k].data_ptr(), lr, beta1, beta2,
                                  eps, self.step_count, None if pb is None else pb.data_ptr(),
                                  None if ptb is None else ptb.data_ptr(), rows, cols, sh)
            _lib.check(st, "adam")
