"""FP64 NumPy restatement of the spectral neural operator's forward pass and
its gradients (TEST INFRASTRUCTURE ONLY: the checker for the GPU training
kernels).  The network has no counterpart in the reference; this follows the
architecture documented in jaxfun_gb300/sno/model.py, with the chain rule
written out by hand (no autograd).
"""

from __future__ import annotations

import numpy as np
from scipy.special import erf


def gelu(x):
    return 0.5 * x * (1.0 + erf(x / np.sqrt(2.0)))


def gelu_grad(x):
    return 0.5 * (1.0 + erf(x / np.sqrt(2.0))) + x * np.exp(-0.5 * x * x) / np.sqrt(2.0 * np.pi)


def forward_backward(params: dict, Phi, Psi, X, target, Bt: int, layers: int):
    """X: (Bt*P, 16) inputs, target: (Bt*P,).  Returns (loss, pred, grads)."""
    P = Phi.shape[1]
    NM = Phi.shape[0]
    p = {k: np.asarray(v, dtype=np.float64) for k, v in params.items()}
    C = p["W0"].shape[0]
    R = Bt * P
    U = [X @ p["W_lift"].T + p["b_lift"]]
    Zs, Uhats = [], []
    for l in range(layers):
        Ub = U[l].reshape(Bt, P, C)
        Uhat = np.einsum("qp,bpc->bqc", Phi, Ub)
        Wh = np.einsum("qoi,bqi->bqo", p[f"R{l}"], Uhat)
        S = np.einsum("pq,bqc->bpc", Psi, Wh).reshape(R, C)
        Z = U[l] @ p[f"W{l}"].T + S + p[f"b{l}"]
        Zs.append(Z)
        Uhats.append(Uhat)
        U.append(Z if l == layers - 1 else gelu(Z))
    Q1pre = U[layers] @ p["W_p1"].T + p["b_p1"]
    Q1 = gelu(Q1pre)
    pred = Q1 @ p["W_p2"].T + p["b_p2"]
    e = pred[:, 0] - target
    loss = 0.5 * np.mean(e * e)
    g = {}
    dq = np.zeros_like(pred)
    dq[:, 0] = e / R
    g["W_p2"] = dq.T @ Q1
    g["b_p2"] = dq.sum(0)
    dZq = (dq @ p["W_p2"]) * gelu_grad(Q1pre)
    g["W_p1"] = dZq.T @ U[layers]
    g["b_p1"] = dZq.sum(0)
    dz = dZq @ p["W_p1"]
    for l in range(layers - 1, -1, -1):
        g[f"W{l}"] = dz.T @ U[l]
        g[f"b{l}"] = dz.sum(0)
        dzb = dz.reshape(Bt, P, C)
        dWh = np.einsum("pq,bpc->bqc", Psi, dzb)
        g[f"R{l}"] = np.einsum("bqo,bqi->qoi", dWh, Uhats[l])
        dUhat = np.einsum("qoi,bqo->bqi", p[f"R{l}"], dWh)
        dU = dz @ p[f"W{l}"] + np.einsum("qp,bqc->bpc", Phi, dUhat).reshape(R, C)
        dz = dU * gelu_grad(Zs[l - 1]) if l >= 1 else dU
    g["W_lift"] = dz.T @ X
    g["b_lift"] = dz.sum(0)
    return loss, pred, g
