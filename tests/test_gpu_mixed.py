"""Mixed-precision (tensor-core PCG + FP64 refinement) solve: <= 1e-10 relative
error against a tight FP64 solve of the same system."""

import numpy as np
import pytest

from jaxfun_gb300.galerkin import DIRICHLET, FunctionSpace, Legendre, TensorProduct
from jaxfun_gb300.la import MixedVarCoefSolver, VarCoefMatrix, pcg
from oracle import spectral as O

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.abs(a - b).max() / np.abs(b).max()


@pytest.fixture(params=[1, 2], ids=["sched-auto", "op-resident"])
def schedule(request):
    from jaxfun_gb300 import _lib

    L = _lib.lib()
    assert L.jfg_tc_set_op_resident(request.param) == 0
    yield request.param
    L.jfg_tc_set_op_resident(0)


@pytest.mark.parametrize("apply", ["f16x3", "tf32"])
@pytest.mark.parametrize("precond", ["bf16x3", "bf16", "tf32"])
@pytest.mark.parametrize("ndim,N,batch", [(2, 32, 3), (2, 64, 2), (3, 16, 2)])
def test_mixed_matches_fp64(ndim, N, batch, precond, apply, schedule):
    V = FunctionSpace(N, Legendre, bcs=DIRICHLET)
    T = TensorProduct(*([V] * ndim))
    rng = np.random.default_rng(N + ndim)
    kap = np.exp(rng.standard_normal((batch,) + (N,) * ndim))
    b = rng.standard_normal((batch,) + (N - 2,) * ndim)
    A = VarCoefMatrix(T, kap)
    xr, _ = pcg(A, b, tol=1e-14, maxiter=3000)
    x, it_in, it_out = MixedVarCoefSolver(A, precond=precond, apply=apply).solve(b, tol=1e-12)
    xr, x = xr.cpu().numpy(), x.cpu().numpy()
    for i in range(batch):
        assert rel(x[i], xr[i]) < 1e-10, (i, it_in, it_out)
    assert np.all(it_out >= 1) and np.all(it_in > 0)


def test_mixed_against_oracle_direct():
    N = 20
    V = FunctionSpace(N, Legendre, bcs=DIRICHLET)
    Vo = O.Space1D("legendre", N, True)
    T = TensorProduct(V, V)
    rng = np.random.default_rng(9)
    kap = np.exp(rng.standard_normal((N, N)))
    b = rng.standard_normal((N - 2, N - 2))
    Ad = O.varcoef_tensormatrix(Vo, kap).transpose(0, 2, 1, 3).reshape((N - 2) ** 2, -1)
    ref = np.linalg.solve(Ad, b.ravel()).reshape(b.shape)
    x, _, _ = MixedVarCoefSolver(VarCoefMatrix(T, kap[None])).solve(b[None], tol=1e-12)
    assert rel(x.cpu().numpy()[0], ref) < 1e-10


def test_mixed_with_initial_guess_and_converged_problem():
    N = 32
    V = FunctionSpace(N, Legendre, bcs=DIRICHLET)
    T = TensorProduct(V, V)
    rng = np.random.default_rng(1)
    kap = np.exp(rng.standard_normal((2, N, N)))
    b = rng.standard_normal((2, N - 2, N - 2))
    A = VarCoefMatrix(T, kap)
    xr, _ = pcg(A, b, tol=1e-14, maxiter=3000)
    x0 = xr.clone()
    x0[1] += 1e-3 * x0[1].abs().max()  # problem 0 starts converged
    x, it_in, it_out = MixedVarCoefSolver(A).solve(b, x0=x0, tol=1e-12)
    assert it_out[0] == 0 and it_out[1] >= 1
    assert rel(x.cpu().numpy()[1], xr.cpu().numpy()[1]) < 1e-10


def test_mixed_after_autotune():
    """The solver's autotune tunes every distinct tensor-core pass of its inner
    solve (2-D defaults: scaled split-FP16 operator passes, p2, and plain BF16
    preconditioner passes, p3); the solve with the tuned configurations still
    reaches 1e-10."""
    N, batch = 64, 3
    V = FunctionSpace(N, Legendre, bcs=DIRICHLET)
    T = TensorProduct(V, V)
    rng = np.random.default_rng(77)
    kap = np.exp(rng.standard_normal((batch, N, N)))
    b = rng.standard_normal((batch, N - 2, N - 2))
    A = VarCoefMatrix(T, kap)
    S = MixedVarCoefSolver(A)
    tuned = S.autotune()
    sigs = [t["signature"] for t in tuned]
    assert any(":p2:b3:" in s for s in sigs) and any(":p3:b3:" in s for s in sigs), sigs
    xr, _ = pcg(A, b, tol=1e-14, maxiter=3000)
    x, _, _ = S.solve(b, tol=1e-12)
    xr, x = xr.cpu().numpy(), x.cpu().numpy()
    for i in range(batch):
        assert rel(x[i], xr[i]) < 1e-10


def test_plain_bf16_preconditioner_keeps_iterations(schedule):
    """The preconditioner's passes in plain BF16 (one product per term,
    ~2^-8) against split BF16 (~2^-16), N = 128, 4 problems: the same answers
    (<= 1e-10 vs a tight FP64 solve) and inner iteration counts within 3 %."""
    N, batch = 128, 4
    V = FunctionSpace(N, Legendre, bcs=DIRICHLET)
    T = TensorProduct(V, V)
    rng = np.random.default_rng(128)
    kap = np.exp(0.5 * rng.standard_normal((batch, N, N)))
    b = rng.standard_normal((batch, N - 2, N - 2))
    A = VarCoefMatrix(T, kap)
    xr, _ = pcg(A, b, tol=1e-14, maxiter=4000)
    xr = xr.cpu().numpy()
    its = {}
    for precond in ("bf16x3", "bf16"):
        S = MixedVarCoefSolver(A, precond=precond)
        assert S.plan.precond_bf16 == (2 if precond == "bf16" else 1)
        x, it_in, _ = S.solve(b, tol=1e-12)
        x = x.cpu().numpy()
        for i in range(batch):
            assert rel(x[i], xr[i]) < 1e-10, (precond, i)
        its[precond] = it_in.astype(float)
    assert np.all(np.abs(its["bf16"] - its["bf16x3"]) <= 0.03 * its["bf16x3"] + 1), its


@pytest.mark.parametrize("precond", ["bf16x3", "tf32"])
def test_fused_dots_match_explicit(precond):
    """The inner PCG's p.Ap (field-pass epilogue) and r.M^-1 r (divide-pass
    epilogue) fused into the contractions give the same answers (<= 1e-10 vs
    a tight FP64 solve) and nearly the same iteration counts as the separate
    dot kernels."""
    N, batch = 64, 4
    V = FunctionSpace(N, Legendre, bcs=DIRICHLET)
    T = TensorProduct(V, V)
    rng = np.random.default_rng(91)
    kap = np.exp(rng.standard_normal((batch, N, N)))
    b = rng.standard_normal((batch, N - 2, N - 2))
    A = VarCoefMatrix(T, kap)
    xr, _ = pcg(A, b, tol=1e-14, maxiter=3000)
    xr = xr.cpu().numpy()
    its = {}
    for fused in (True, False):
        S = MixedVarCoefSolver(A, precond=precond, fused_dots=fused)
        assert S.plan.fused_dots == (3 if fused else 0)
        x, it_in, _ = S.solve(b, tol=1e-12)
        x = x.cpu().numpy()
        for i in range(batch):
            assert rel(x[i], xr[i]) < 1e-10, (fused, i)
        its[fused] = it_in.astype(float)
    assert np.all(np.abs(its[True] - its[False]) <= 0.1 * its[False] + 2), its


@pytest.mark.parametrize("ndim,N,batch", [(2, 48, 6), (3, 16, 3)])
def test_flat_schedule_matches_sync_and_fp64(ndim, N, batch):
    """Per-problem refinement steps (the flat schedule) reach the same
    <= 1e-10 answers as the synchronised schedule; a problem with a zero
    right-hand side converges at once; with a perturbed start and with a
    guess for the first inner solve as well."""
    V = FunctionSpace(N, Legendre, bcs=DIRICHLET)
    T = TensorProduct(*([V] * ndim))
    rng = np.random.default_rng(17 + ndim)
    kap = np.exp(rng.standard_normal((batch,) + (N,) * ndim) * np.linspace(0.2, 1.5, batch)
                 .reshape((batch,) + (1,) * ndim))
    b = rng.standard_normal((batch,) + (N - 2,) * ndim)
    b[1] = 0.0
    A = VarCoefMatrix(T, kap)
    xr, _ = pcg(A, b, tol=1e-14, maxiter=4000)
    xr = xr.cpu().numpy()
    res = {}
    for sched in ("flat", "sync"):
        S = MixedVarCoefSolver(A, schedule=sched)
        x, it_in, it_out = S.solve(b, tol=1e-12)
        x = x.cpu().numpy()
        assert np.all(x[1] == 0.0) and it_out[1] == 0
        for i in range(batch):
            if i != 1:
                assert rel(x[i], xr[i]) < 1e-10, (sched, i, it_in, it_out)
        res[sched] = it_in
        # from an FP64 starting iterate and from a guess
        x0 = xr + 1e-3 * rng.standard_normal(xr.shape) * np.abs(xr).max()
        x0[1] = 0.0
        x, _, _ = S.solve(b, x0=x0, tol=1e-12)
        x = x.cpu().numpy()
        g, _, _ = S.solve(b, tol=1e-12, guess=x0)
        g = g.cpu().numpy()
        for i in range(batch):
            if i != 1:
                assert rel(x[i], xr[i]) < 1e-10, (sched, "x0", i)
                assert rel(g[i], xr[i]) < 1e-10, (sched, "guess", i)
    # the same inner work per problem, within the chunk granularity
    assert np.all(np.abs(res["flat"] - res["sync"]) <= 0.25 * res["sync"] + 12), res


def test_flat_schedule_outer_budget_exhausted():
    """With one outer step allowed and a tight tolerance the flat schedule
    stops and reports non-convergence instead of looping."""
    from jaxfun_gb300 import _lib

    N = 32
    V = FunctionSpace(N, Legendre, bcs=DIRICHLET)
    T = TensorProduct(V, V)
    rng = np.random.default_rng(3)
    kap = np.exp(rng.standard_normal((2, N, N)))
    b = rng.standard_normal((2, N - 2, N - 2))
    S = MixedVarCoefSolver(VarCoefMatrix(T, kap), schedule="flat")
    with pytest.raises(_lib.JfgError) as e:
        S.solve(b, tol=1e-13, max_outer=1)
    assert e.value.status == _lib.JFG_ERR_NOT_CONVERGED


@pytest.mark.parametrize("ndim,N,batch", [(2, 48, 5), (3, 16, 3)])
@pytest.mark.parametrize("sched", ["sync", "flat"])
def test_whole_solve_graph_matches_host_loop(sched, ndim, N, batch):
    """On a stream that can be captured the whole refinement loop is one CUDA
    graph (a conditional WHILE node around an IF/ELSE choice of outer step or
    inner chunk).  It gives bit-identical answers and iteration counts to the
    host-driven loop on the legacy default stream -- from zero, from a
    starting iterate and from a guess, with a problem whose right-hand side
    is zero -- also when the cached graph is replayed on new data; an
    exhausted outer budget still reports non-convergence."""
    import torch

    from jaxfun_gb300 import _lib

    V = FunctionSpace(N, Legendre, bcs=DIRICHLET)
    T = TensorProduct(*([V] * ndim))
    rng = np.random.default_rng(29 + ndim)
    kap = np.exp(rng.standard_normal((batch,) + (N,) * ndim))
    A = VarCoefMatrix(T, kap)
    S = MixedVarCoefSolver(A, schedule=sched)
    bs = [rng.standard_normal((batch,) + (N - 2,) * ndim) for _ in range(2)]
    for b in bs:
        b[2] = 0.0
    x0 = 1e-3 * rng.standard_normal(bs[0].shape)
    x0[2] = 0.0
    side = torch.cuda.Stream()

    def run(b, stream, **kw):
        bt = torch.as_tensor(b, device="cuda")
        with torch.cuda.stream(stream):
            x, it_in, it_out = S.solve(bt, tol=1e-12, **kw)
            x = x.clone()
        torch.cuda.synchronize()
        return x.cpu().numpy(), np.array(it_in), np.array(it_out)

    legacy = torch.cuda.default_stream()
    for kw in ({}, {"x0": x0}, {"guess": x0}):
        for b in bs:  # the second right-hand side replays the cached graph
            xh, ih, oh = run(b, legacy, **kw)
            xg, ig, og = run(b, side, **kw)
            assert np.array_equal(xh, xg), (kw.keys(), np.abs(xh - xg).max())
            assert np.array_equal(ih, ig) and np.array_equal(oh, og), (ih, ig, oh, og)
            assert np.all(xg[2] == 0.0) and og[2] == 0
    with pytest.raises(_lib.JfgError) as e:
        with torch.cuda.stream(side):
            S.solve(torch.as_tensor(bs[0], device="cuda"), tol=1e-13, max_outer=1)
        torch.cuda.synchronize()
    assert e.value.status == _lib.JFG_ERR_NOT_CONVERGED
