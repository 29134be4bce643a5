"""Training data from the solver itself, training loop, and the learned
initial guess for the variable-coefficient PCG.

Data: seeded problems of the 2-D variable-coefficient Poisson benchmark
(N = 256 Legendre Dirichlet; kappa = exp(g), g a Gaussian random field with
Legendre coefficients N(0,1)(1+|k|^2)^-1.5 rescaled to std 1; forcing
coefficients N(0,1)(1+j)^-2(1+k)^-2), solved by ``MixedVarCoefSolver``.
Fields are moved to the network's 64 x 64 Legendre-Gauss grid by spectral
truncation; the forcing and the solution are scaled by the forcing's RMS
(the problem is linear in f).

    python -m jaxfun_gb300.sno.train --train 20000 --test 1000 --epochs 8 --out ckpt.npz
"""

from __future__ import annotations

import argparse
import json
import math
import time

import numpy as np
import torch

from ..galerkin import DIRICHLET, FunctionSpace, Legendre, TensorProduct, tp_apply
from ..galerkin.tensorproductspace import tp_apply_tc
from ..la import MixedVarCoefSolver, VarCoefMatrix
from .model import CIN, SNO, SNOConfig

N_FINE = 256


class GridMaps:
    """Per-axis FP64 operators between the solver's space and the network grid."""

    def __init__(self, N: int = N_FINE, n: int = 64, guess_modes: int = 32):
        self.N, self.n = N, n
        Lo, lo = Legendre(N), Legendre(n)
        # fine-grid field -> first n Legendre modes -> values on the n-point grid
        self.to_net = lo.backward_matrix() @ Lo.forward_matrix()[:n, :]
        D = FunctionSpace(N, Legendre, bcs=DIRICHLET)
        # solver coefficients (N-2) -> values on the n-point grid
        self.coef_to_net = D.backward_matrix(n)
        d = FunctionSpace(n, Legendre, bcs=DIRICHLET)
        # network-grid values -> Dirichlet coefficients (the basis functions
        # phi_k = L_k - L_{k+2} do not depend on N), padded to N-2.  Only the
        # first guess_modes are kept: the network resolves 32 Legendre modes
        # per axis and its higher-mode content is noise in the energy norm.
        G = np.zeros((N - 2, n))
        m = min(guess_modes, n - 2)
        G[:m] = d.forward_matrix()[:m]
        self.net_to_coef = G
        x = lo.mesh()
        self.X, self.Y = np.meshgrid(x, x, indexing="ij")
        self.D = D
        self.T = TensorProduct(D, D)
        self.To = TensorProduct(Lo, Lo)


def synth_batch(gen: torch.Generator, B: int, N: int, maps: GridMaps):
    """Seeded coefficients -> (kappa, f) on the fine Gauss grid (FP64, GPU)."""
    k = torch.arange(N, dtype=torch.float64, device="cuda")
    grf = (1.0 + k[:, None] ** 2 + k[None, :] ** 2) ** -1.5
    fs = ((1.0 + k[:, None]) ** -2.0) * ((1.0 + k[None, :]) ** -2.0)
    gh = torch.randn((B, N, N), generator=gen, dtype=torch.float64, device="cuda") * grf
    fh = torch.randn((B, N, N), generator=gen, dtype=torch.float64, device="cuda") * fs
    g = maps.To.backward(gh)
    g = (g - g.mean(dim=(1, 2), keepdim=True)) / g.std(dim=(1, 2), keepdim=True)
    f = maps.To.backward(fh)
    return g, f


def features(g, f, maps: GridMaps):
    """Network inputs (B*n^2, 16) FP32 and the per-sample forcing scale."""
    B = g.shape[0]
    n = maps.n
    # spectral truncation onto the network grid on the tensor cores (FP32 data)
    g64 = tp_apply_tc([maps.to_net, maps.to_net], g)
    f64 = tp_apply_tc([maps.to_net, maps.to_net], f)
    s = f64.pow(2).mean(dim=(1, 2)).sqrt().clamp_min(1e-30)
    X = torch.zeros((B, n, n, CIN), dtype=torch.float32, device="cuda")
    X[..., 0] = g64.float()
    X[..., 1] = (f64 / s[:, None, None]).float()
    X[..., 2] = torch.as_tensor(maps.X, device="cuda").float()
    X[..., 3] = torch.as_tensor(maps.Y, device="cuda").float()
    return X.reshape(B * n * n, CIN), s


def generate(nsamples: int, seed: int, maps: GridMaps, chunk: int = 128, tol: float = 1e-8,
             keep_fine: bool = False, log=print):
    """Solve nsamples seeded problems; return network inputs/targets (and the fine
    fields when keep_fine)."""
    gen = torch.Generator(device="cuda")
    gen.manual_seed(seed)
    N, n = maps.N, maps.n
    Xs, Ts, Ss, fine = [], [], [], []
    t0 = time.perf_counter()
    done = 0
    while done < nsamples:
        B = min(chunk, nsamples - done)
        g, f = synth_batch(gen, B, N, maps)
        kap = torch.exp(g)
        b = maps.T.scalar_product(f)
        A = VarCoefMatrix(maps.T, kap)
        x, _, _ = MixedVarCoefSolver(A).solve(b, tol=tol)
        X, s = features(g, f, maps)
        u64 = tp_apply([maps.coef_to_net, maps.coef_to_net], x)
        Xs.append(X.to(torch.bfloat16))
        Ts.append((u64 / s[:, None, None]).float().reshape(-1))
        Ss.append(s)
        if keep_fine:
            fine.append((kap, f, b, x))
        done += B
    torch.cuda.synchronize()
    log(f"generated {nsamples} solves in {time.perf_counter() - t0:.1f} s")
    out = {"X": torch.cat(Xs), "T": torch.cat(Ts), "s": torch.cat(Ss)}
    if keep_fine:
        out["fine"] = fine
    return out


def train(model: SNO, data: dict, epochs: int, lr: float = 1e-3, log=print, seed: int = 0):
    P = model.P
    nsamp = data["T"].numel() // P
    Bt = model.cfg.batch
    steps_per_epoch = nsamp // Bt
    total = epochs * steps_per_epoch
    rng = np.random.default_rng(seed)
    step = 0
    hist = []
    t0 = time.perf_counter()
    X = data["X"].reshape(nsamp, P, CIN)
    T = data["T"].reshape(nsamp, P)
    for ep in range(epochs):
        perm = torch.as_tensor(rng.permutation(nsamp), device="cuda")
        tot = 0.0
        for i in range(steps_per_epoch):
            idx = perm[i * Bt:(i + 1) * Bt]
            Bn = model.set_input(X[idx].reshape(Bt * P, CIN))
            model.forward(Bn)
            tgt = T[idx].reshape(-1).contiguous()
            loss = model.backward(Bn, tgt)
            cur = lr * 0.5 * (1.0 + math.cos(math.pi * step / max(1, total)))
            model.adam(cur)
            tot += loss
            step += 1
        hist.append(tot / max(1, steps_per_epoch))
        log(f"epoch {ep}: loss {hist[-1]:.4e}  ({time.perf_counter() - t0:.1f} s)")
    return hist


def predict(model: SNO, X: torch.Tensor, Bt: int | None = None) -> torch.Tensor:
    """Network prediction (nsamples, n, n) FP32 on the network grid."""
    P = model.P
    nsamp = X.shape[0] // P
    Bt = Bt or model.cfg.batch
    out = torch.empty((nsamp, P), dtype=torch.float32, device="cuda")
    for i in range(0, nsamp, Bt):
        B = min(Bt, nsamp - i)
        model.set_input(X[i * P:(i + B) * P])
        pred = model.forward(B)
        out[i:i + B] = pred[:, 0].reshape(B, P)
    n = model.cfg.n
    return out.reshape(nsamp, n, n)


def initial_guess(model: SNO, maps: GridMaps, X: torch.Tensor, s: torch.Tensor) -> torch.Tensor:
    """Learned initial guess in the solver's coefficient space (B, N-2, N-2) FP64."""
    u = predict(model, X) * s[:, None, None].float()
    return tp_apply_tc([maps.net_to_coef, maps.net_to_coef], u).double()


def relative_l2(model: SNO, data: dict) -> float:
    P = model.P
    nsamp = data["T"].numel() // P
    pred = predict(model, data["X"]).reshape(nsamp, -1)
    T = data["T"].reshape(nsamp, -1)
    return float(((pred - T).norm(dim=1) / T.norm(dim=1)).mean())


def evaluate_gain(model: SNO, maps: GridMaps, nprob: int = 128, seed: int = 3,
                  tol: float = 3e-11, inner_tol: float = 1e-5) -> dict:
    """Mixed-precision solves of held-out problems from a zero start and from the
    learned guess: iterations, time, and error against a tight FP64 solve."""
    from ..la import pcg

    data = generate(nprob, seed, maps, keep_fine=True, log=lambda *_: None)
    kap, f, b, _ = data["fine"][0] if len(data["fine"]) == 1 else [
        torch.cat([c[i] for c in data["fine"]]) for i in range(4)]
    A = VarCoefMatrix(maps.T, kap)
    S = MixedVarCoefSolver(A)
    xt, _ = pcg(A, b, tol=1e-14, maxiter=3000)
    out = {}
    for name in ("zero", "learned"):
        for rep in range(2):  # second repetition is timed
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            x0 = initial_guess(model, maps, data["X"], data["s"]) if name == "learned" else None
            x, it_in, it_out = S.solve(b, guess=x0, tol=tol, inner_tol=inner_tol)
            torch.cuda.synchronize()
            dt = time.perf_counter() - t0
        err = float(((x - xt).abs().amax(dim=(1, 2)) / xt.abs().amax(dim=(1, 2))).max())
        out[name] = {"inner_iterations_mean": float(it_in.mean()),
                     "outer_iterations_mean": float(it_out.mean()), "ms": 1e3 * dt,
                     "solves_per_s": nprob / dt, "max_rel_err": err}
    x0 = initial_guess(model, maps, data["X"], data["s"])
    out["guess_rel_err_mean"] = float(((x0 - xt).norm(dim=(1, 2)) / xt.norm(dim=(1, 2))).mean())
    return out


def save(model: SNO, path: str, meta: dict | None = None):
    sd = model.state_dict()
    arrs = {k: (v.astype(np.float16) if k.startswith("R") else v.astype(np.float32))
            for k, v in sd.items() if not k.startswith("_")}
    arrs["_config"] = sd["_config"]
    arrs["_meta"] = np.frombuffer(json.dumps(meta or {}).encode(), dtype=np.uint8)
    np.savez(path, **arrs)


def load(path: str, batch: int = 32) -> SNO:
    z = np.load(path)
    n, width, modes, layers = (int(v) for v in z["_config"])
    model = SNO(SNOConfig(n=n, width=width, modes=modes, layers=layers, batch=batch))
    model.load_state_dict({k: z[k] for k in z.files if not k.startswith("_")})
    return model


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--train", type=int, default=20000)
    ap.add_argument("--test", type=int, default=1000)
    ap.add_argument("--epochs", type=int, default=8)
    ap.add_argument("--batch", type=int, default=32)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--out", default="sno_varcoef2d_N256.npz")
    args = ap.parse_args()
    torch.cuda.set_device(0)
    maps = GridMaps()
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        tr = generate(args.train, seed=1, maps=maps)
        te = generate(args.test, seed=2, maps=maps)
        model = SNO(SNOConfig(batch=args.batch), seed=0)
        t0 = time.perf_counter()
        hist = train(model, tr, args.epochs, lr=args.lr)
        t_train = time.perf_counter() - t0
        err = relative_l2(model, te)
        gain = evaluate_gain(model, maps)
    meta = {"train": args.train, "test": args.test, "epochs": args.epochs, "lr": args.lr,
            "test_rel_l2": err, "train_loss": hist, "train_seconds": t_train, "gain": gain}
    print(json.dumps(meta))
    save(model, args.out, meta)


if __name__ == "__main__":
    main()
