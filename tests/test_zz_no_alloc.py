"""The allocation-free fast-diagonalisation entry point (jfg_fd_solve_f64_noalloc).

It exists for callers that cannot allocate device memory at the point where
they solve (inside a host runtime that owns all device memory and hands out no
workspace, in loops that must not block on an allocator): they pass only
inputs and outputs, and the library uses a fixed scratch array of its own.
This file is collected last so that a run stopping at the first failure has
already run every other test; it also passes alone in a fresh process.
"""

import numpy as np
import pytest
import torch

from jaxfun_gb300 import _lib
from jaxfun_gb300.galerkin import DIRICHLET, Chebyshev, FunctionSpace, Legendre, TensorProduct
from jaxfun_gb300.la import poisson_tpmatrices, tpmats_lu_factor

pytestmark = pytest.mark.gpu


def _factors(space, N, ndim, alpha2):
    V = FunctionSpace(N, space, bcs=DIRICHLET)
    T = TensorProduct(*([V] * ndim))
    return tpmats_lu_factor(poisson_tpmatrices(T, alpha2).tpmats)


def _solve_both(fac, rhs, c0, c1, check_memory=False):
    """Run the workspace entry point and the allocation-free one on the same data.

    With check_memory, also check that the allocation-free call leaves the
    device's free memory and torch's allocated bytes unchanged (only after a
    first call: with lazy module loading the first call loads the library's
    kernels and its scratch array)."""
    L = _lib.lib()
    nd, n = fac.ndim, fac.n
    batch = rhs.shape[0]
    E, W, lam = fac.device_factors()
    dev = lambda a: torch.as_tensor(np.ascontiguousarray(a), device="cuda")  # noqa: E731
    t_rhs, t_c0, t_c1 = dev(rhs), dev(c0), dev(c1)
    ref = torch.empty_like(t_rhs)
    out = torch.full_like(t_rhs, float("nan"))
    ws = torch.empty(L.jfg_fd_solve_workspace_size(nd, n, batch, 8), dtype=torch.uint8,
                     device="cuda")
    sh = _lib.stream_handle()
    st = L.jfg_fd_solve_f64(nd, n, batch, E.data_ptr(), W.data_ptr(), lam.data_ptr(),
                            t_c0.data_ptr(), t_c1.data_ptr(), t_rhs.data_ptr(), ref.data_ptr(),
                            ws.data_ptr(), ws.numel(), sh)
    assert st == 0, _lib.status_string(st)
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    used0 = torch.cuda.memory_allocated()
    st = L.jfg_fd_solve_f64_noalloc(nd, n, batch, E.data_ptr(), W.data_ptr(), lam.data_ptr(),
                                    t_c0.data_ptr(), t_c1.data_ptr(), t_rhs.data_ptr(),
                                    out.data_ptr(), sh)
    assert st == 0, _lib.status_string(st)
    torch.cuda.synchronize()
    if check_memory:
        assert torch.cuda.memory_allocated() == used0
        assert torch.cuda.mem_get_info()[0] == free0
    return ref.cpu().numpy(), out.cpu().numpy()


@pytest.mark.parametrize("space,N,ndim,alpha2", [
    (Legendre, 64, 2, 0.0),
    (Chebyshev, 48, 2, 25.0),
    (Legendre, 20, 3, 0.0),
])
def test_noalloc_matches_workspace_entry_point_twice(space, N, ndim, alpha2):
    fac = _factors(space, N, ndim, alpha2)
    rng = np.random.default_rng(N * ndim)
    for call in range(2):  # two calls in a row reuse (and must overwrite) the scratch
        batch = 3 + call
        rhs = rng.standard_normal((batch,) + (fac.n,) * ndim)
        c0 = np.full(batch, alpha2) + call
        c1 = np.ones(batch)
        ref, out = _solve_both(fac, rhs, c0, c1, check_memory=call == 1)
        assert np.all(np.isfinite(out))
        assert np.abs(out - ref).max() <= 1e-12 * np.abs(ref).max()


def test_noalloc_rejects_oversized_request():
    L = _lib.lib()
    cap = L.jfg_fd_solve_noalloc_max_bytes()
    assert cap == 32 * 1024 * 1024
    n, nd = 254, 2
    batch = cap // (n * n * 8)  # two fields of this batch exceed the array
    assert L.jfg_fd_solve_workspace_size(nd, n, batch, 8) > cap
    x = torch.zeros(8, dtype=torch.float64, device="cuda")
    p = x.data_ptr()
    st = L.jfg_fd_solve_f64_noalloc(nd, n, batch, p, p, p, None, None, p, p,
                                    _lib.stream_handle())
    assert st == _lib.JFG_ERR_WORKSPACE
    # sizes whose byte count would wrap around in size_t are rejected as well
    for n_, nd_, b_ in ((2048, 3, 2**28), (2**20, 3, 1), (65536, 2, 2**31 - 1)):
        st = L.jfg_fd_solve_f64_noalloc(nd_, n_, b_, p, p, p, None, None, p, p,
                                        _lib.stream_handle())
        assert st == _lib.JFG_ERR_WORKSPACE, (n_, nd_, b_)
    torch.cuda.synchronize()
