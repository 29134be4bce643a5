"""Training data from the solver itself, training loop, and the learned
initial guess for the variable-coefficient PCG.

Data: seeded problems of the variable-coefficient Poisson benchmarks (2-D:
N = 256 Legendre Dirichlet, network grid 64^2, 32^2 modes; 3-D: N = 128, grid
32^3, 16^3 modes; kappa = exp(g), g a Gaussian random field with Legendre
coefficients N(0,1)(1+|k|^2)^-1.5 rescaled to std 1; forcing coefficients
N(0,1) prod_i (1+k_i)^-2), solved by ``MixedVarCoefSolver``.  Fields are moved
to the network's Legendre-Gauss grid by spectral truncation; the forcing and
the solution are scaled by the forcing's RMS (the problem is linear in f).

    python -m jaxfun_gb300.sno.train --train 20000 --test 1000 --epochs 80 --out ckpt.npz
      (the committed 2-D weights: 80 epochs, test relative L2 0.42 %)
    python -m jaxfun_gb300.sno.train --ndim 3 --N 128 --n 32 --modes 16 --width 32 ...
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

    # Dirichlet modes per axis the learned guess keeps.  Beyond them the
    # network's prediction is mostly noise relative to the solution's small
    # content there, and noise in high modes costs PCG iterations.  2-D, 128
    # problems of N = 256 solved to 1e-11: 107.9 mean inner iterations from
    # zero, 100.6 from the guess cut at 32 modes, 97.4 at 6, 95.0 at 8, 94.6
    # at 10 (smooth tapers did no better than a cut).  3-D, 32 problems of
    # N = 128: cutting below 16 modes gained nothing.
    GUESS_MODES = {2: 10, 3: 16}

    def __init__(self, N: int = N_FINE, n: int = 64, guess_modes: int | None = None,
                 ndim: int = 2):
        if guess_modes is None:
            guess_modes = self.GUESS_MODES[ndim]
        self.N, self.n, self.ndim = N, n, ndim
        self.guess_modes = guess_modes
        Lo, lo = Legendre(N), Legendre(n)
        # fine-grid field -> first n Legendre modes -> values on the n-point grid
        self.to_net = lo.backward_matrix() @ Lo.forward_matrix()[:n, :]
        D = FunctionSpace(N, Legendre, bcs=DIRICHLET)
        # solver coefficients (N-2) -> values on the n-point grid
        self.coef_to_net = D.backward_matrix(n)
        d = FunctionSpace(n, Legendre, bcs=DIRICHLET)
        # network-grid values -> Dirichlet coefficients (the basis functions
        # phi_k = L_k - L_{k+2} do not depend on N), padded to N-2; only the
        # first guess_modes are kept.
        G = np.zeros((N - 2, n))
        m = min(guess_modes, n - 2)
        G[:m] = d.forward_matrix()[:m]
        self.net_to_coef = G
        x = lo.mesh()
        self.coords = np.meshgrid(*([x] * ndim), indexing="ij")
        self.D = D
        self.T = TensorProduct(*([D] * ndim))
        self.To = TensorProduct(*([Lo] * ndim))


def _axes(maps: GridMaps) -> tuple[int, ...]:
    return tuple(range(1, 1 + maps.ndim))


def _bcast(v: torch.Tensor, ndim: int) -> torch.Tensor:
    return v.reshape((-1,) + (1,) * ndim)


def synth_batch(gen: torch.Generator, B: int, N: int, maps: GridMaps):
    """Seeded coefficients -> (kappa, f) on the fine Gauss grid (FP64, GPU)."""
    nd = maps.ndim
    k = torch.arange(N, dtype=torch.float64, device="cuda")
    ks = [k.reshape((-1,) + (1,) * (nd - 1 - i)) for i in range(nd)]
    grf = (1.0 + sum(kk ** 2 for kk in ks)) ** -1.5
    fs = 1.0
    for kk in ks:
        fs = fs * (1.0 + kk) ** -2.0
    shape = (B,) + (N,) * nd
    gh = torch.randn(shape, generator=gen, dtype=torch.float64, device="cuda") * grf
    fh = torch.randn(shape, generator=gen, dtype=torch.float64, device="cuda") * fs
    g = maps.To.backward(gh)
    ax = _axes(maps)
    g = (g - g.mean(dim=ax, keepdim=True)) / g.std(dim=ax, keepdim=True)
    f = maps.To.backward(fh)
    return g, f


def _feature_buffer(maps: GridMaps, B: int) -> torch.Tensor:
    """(B, n^d, CIN) FP32 input buffer whose coordinate channels (and zero
    padding channels) are written once and kept; only the field channels are
    rewritten per call."""
    key = (B, torch.cuda.current_device())
    cache = maps.__dict__.setdefault("_xbuf", {})
    X = cache.get(key)
    if X is None:
        n, nd = maps.n, maps.ndim
        X = torch.zeros((B,) + (n,) * nd + (CIN,), dtype=torch.float32, device="cuda")
        for i, c in enumerate(maps.coords):
            X[..., 2 + i] = torch.as_tensor(c, device="cuda").float()
        cache[key] = X
    return X


def features(g, f, maps: GridMaps):
    """Network inputs (B*n^2, 16) FP32 and the per-sample forcing scale.  The
    returned tensor is a per-(batch, device) buffer of ``maps`` that the next
    call with the same batch overwrites."""
    B = g.shape[0]
    n, nd = maps.n, maps.ndim
    # spectral truncation onto the network grid on the tensor cores (FP32 data)
    g64 = tp_apply_tc([maps.to_net] * nd, g)
    f64 = tp_apply_tc([maps.to_net] * nd, f)
    s = torch.linalg.vector_norm(f64.flatten(1), dim=1).mul_(n ** (-nd / 2)).clamp_min_(1e-30)
    X = _feature_buffer(maps, B)
    X[..., 0] = g64
    torch.div(f64, _bcast(s, nd), out=X[..., 1])
    return X.reshape(B * n ** nd, CIN), s


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
        u64 = tp_apply([maps.coef_to_net] * maps.ndim, x)
        Xs.append(X.to(torch.bfloat16))
        Ts.append((u64 / _bcast(s, maps.ndim)).float().reshape(-1))
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
        model.set_input(X[i * P:(i + B) * P], train=False)
        pred = model.forward(B, train=False)
        out[i:i + B] = pred[:, 0].reshape(B, P)
    n = model.cfg.n
    return out.reshape((nsamp,) + (n,) * model.cfg.ndim)


def initial_guess(model: SNO, maps: GridMaps, X: torch.Tensor, s: torch.Tensor) -> torch.Tensor:
    """Learned initial guess in the solver's coefficient space (B, (N-2,)*d) FP64."""
    u = predict(model, X) * _bcast(s, maps.ndim).float()
    return tp_apply_tc([maps.net_to_coef] * maps.ndim, u).double()


def relative_l2(model: SNO, data: dict) -> float:
    P = model.P
    nsamp = data["T"].numel() // P
    pred = predict(model, data["X"]).reshape(nsamp, -1)
    T = data["T"].reshape(nsamp, -1)
    return float(((pred - T).norm(dim=1) / T.norm(dim=1)).mean())


def evaluate_gain(model: SNO, maps: GridMaps, nprob: int = 128, seed: int = 3,
                  tol: float | None = None, inner_tol: float = 1e-5) -> dict:
    """Mixed-precision solves of held-out problems from a zero start and from the
    learned guess: iterations, time, and error against a tight FP64 solve.
    Default tolerance: the benchmarks' calibrated stopping rule (2-D 1e-11 on
    the relative residual, 3-D 1e-12)."""
    from ..la import pcg

    if tol is None:
        tol = 1e-11 if maps.ndim == 2 else 1e-12
    data = generate(nprob, seed, maps, keep_fine=True, log=lambda *_: None)
    kap, f, b, _ = data["fine"][0] if len(data["fine"]) == 1 else [
        torch.cat([c[i] for c in data["fine"]]) for i in range(4)]
    A = VarCoefMatrix(maps.T, kap)
    S = MixedVarCoefSolver(A)
    xt, _ = pcg(A, b, tol=1e-14, maxiter=4000)
    ax = _axes(maps)
    out = {}
    for name in ("zero", "learned"):
        for rep in range(2):  # second repetition is timed
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            x0 = initial_guess(model, maps, data["X"], data["s"]) if name == "learned" else None
            x, it_in, it_out = S.solve(b, guess=x0, tol=tol, inner_tol=inner_tol)
            torch.cuda.synchronize()
            dt = time.perf_counter() - t0
        err = float(((x - xt).abs().amax(dim=ax) / xt.abs().amax(dim=ax)).max())
        out[name] = {"inner_iterations_mean": float(it_in.mean()),
                     "outer_iterations_mean": float(it_out.mean()), "ms": 1e3 * dt,
                     "solves_per_s": nprob / dt, "max_rel_err": err}
    x0 = initial_guess(model, maps, data["X"], data["s"])
    vn = torch.linalg.vector_norm
    out["guess_rel_err_mean"] = float((vn(x0 - xt, dim=ax) / vn(xt, dim=ax)).mean())
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
    cfg = [int(v) for v in z["_config"]]
    n, width, modes, layers = cfg[:4]
    ndim = cfg[4] if len(cfg) > 4 else 2
    model = SNO(SNOConfig(n=n, width=width, modes=modes, layers=layers, batch=batch,
                          ndim=ndim))
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
    ap.add_argument("--ndim", type=int, default=2)
    ap.add_argument("--N", type=int, default=N_FINE, help="solver modes per axis")
    ap.add_argument("--n", type=int, default=64, help="network grid points per axis")
    ap.add_argument("--modes", type=int, default=32, help="network modes per axis")
    ap.add_argument("--width", type=int, default=64)
    ap.add_argument("--chunk", type=int, default=128, help="problems per generating solve")
    ap.add_argument("--gain-problems", type=int, default=128)
    ap.add_argument("--guess-modes", type=int, default=None,
                    help="Dirichlet modes per axis kept in the learned guess")
    args = ap.parse_args()
    torch.cuda.set_device(0)
    maps = GridMaps(N=args.N, n=args.n, guess_modes=args.guess_modes, ndim=args.ndim)
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        tr = generate(args.train, seed=1, maps=maps, chunk=args.chunk)
        te = generate(args.test, seed=2, maps=maps, chunk=args.chunk)
        model = SNO(SNOConfig(n=args.n, width=args.width, modes=args.modes, batch=args.batch,
                              ndim=args.ndim), seed=0)
        t0 = time.perf_counter()
        hist = train(model, tr, args.epochs, lr=args.lr)
        t_train = time.perf_counter() - t0
        err = relative_l2(model, te)
        save(model, args.out, {"train": args.train, "test": args.test, "epochs": args.epochs,
                               "test_rel_l2": err})
        gain = evaluate_gain(model, maps, nprob=args.gain_problems)
    meta = {"train": args.train, "test": args.test, "epochs": args.epochs, "lr": args.lr,
            "test_rel_l2": err, "train_loss": hist, "train_seconds": t_train, "gain": gain}
    print(json.dumps(meta))
    save(model, args.out, meta)


if __name__ == "__main__":
    main()
