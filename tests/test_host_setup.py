"""Product host setup (FP64 operators) against the oracle; C-ABI library load (CPU only)."""

import re
from pathlib import Path

import numpy as np
import pytest

from jaxfun_gb300.galerkin import DIRICHLET, Chebyshev, FunctionSpace, Legendre
from jaxfun_gb300.la import fd_eig
from oracle import spectral as O

ROOT = Path(__file__).resolve().parents[1]


@pytest.mark.parametrize("N", [5, 16, 64, 257])
def test_gauss_legendre_matches_oracle(N):
    from jaxfun_gb300.galerkin import legendre_gauss

    x, w = legendre_gauss(N)
    xo, wo = O.legendre_gauss(N)
    assert np.abs(x - xo).max() < 4e-16 and np.abs(w - wo).max() < 1e-15


@pytest.mark.parametrize("space,fam", [(Legendre, "legendre"), (Chebyshev, "chebyshev")])
@pytest.mark.parametrize("bcs", [None, DIRICHLET])
def test_operators_match_oracle(space, fam, bcs):
    N = 12
    V = FunctionSpace(N, space, bcs=bcs)
    Vo = O.Space1D(fam, N, bcs is not None)
    c = np.random.default_rng(0).standard_normal(V.dim)
    assert np.abs(V.backward_matrix() @ c - Vo.backward(c)).max() < 1e-13
    u = Vo.backward(c)
    assert np.abs(V.forward_matrix() @ u - Vo.forward(u)).max() < 1e-13
    assert np.abs(V.scalar_product_matrix() @ u - Vo.scalar_product(u)).max() < 1e-13
    assert np.abs(V.mass_matrix() - Vo.mass_matrix()).max() < 1e-14
    if bcs is not None:
        assert np.abs(V.stiffness_matrix() - Vo.stiffness_matrix()).max() < 1e-9


def test_fd_eig_chebyshev_reconstructs():
    V = FunctionSpace(40, Chebyshev, bcs=DIRICHLET)
    K, M = V.stiffness_matrix(), V.mass_matrix()
    lam, W, E = fd_eig(K, M)
    assert np.all(lam > 0)
    assert np.abs(E @ M @ W - np.eye(38)).max() < 1e-9
    assert np.abs(E @ K @ W - np.diag(lam)).max() < 1e-9 * lam.max()


def _header_symbols():
    txt = (ROOT / "include" / "jaxfun_gb300.h").read_text()
    return sorted(set(re.findall(r"\b(jfg_[a-z0-9_]+)\s*\(", txt)))


def test_library_exports_every_header_symbol(lib):
    syms = _header_symbols()
    assert len(syms) > 10
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing


def test_host_side_argument_checks(lib):
    from jaxfun_gb300 import _lib

    assert lib.jfg_version().startswith(b"jaxfun_gb300")
    assert lib.jfg_status_string(_lib.JFG_ERR_ARG) == b"invalid argument"
    # NULL descriptor / bad shapes are rejected before any CUDA call
    assert lib.jfg_contract_f64(None, None, None, None, None) == _lib.JFG_ERR_ARG
    d = _lib.ContractDesc(batch=1, nseg=1, M=4, P=4, K=0)
    assert lib.jfg_contract_f64(d, None, None, None, None) == _lib.JFG_ERR_ARG
    d = _lib.ContractDesc(batch=1, nseg=1, M=4, P=4, K=4, op_ld=2, in_ld=4, out_ld=4)
    assert lib.jfg_contract_f32(d, None, None, None, None) == _lib.JFG_ERR_ARG
    rows = _lib.int_array([4, 4])
    assert lib.jfg_tp_apply_f64(4, rows, rows, 1, None, None, None, None, 0, None) == _lib.JFG_ERR_ARG
    assert lib.jfg_fd_solve_workspace_size(2, 8, 3, 8) > 0


def test_varcoef_pack_layout(lib):
    from jaxfun_gb300.la import pack_varcoef_ops

    rng = np.random.default_rng(0)
    B, D = rng.standard_normal((6, 4)), rng.standard_normal((6, 4))
    p = pack_varcoef_ops(2, B, D)
    nn = 24
    assert np.array_equal(p[:nn].reshape(6, 4), B)
    assert np.array_equal(p[nn:2 * nn].reshape(6, 4), D)
    assert np.array_equal(p[4 * nn:5 * nn].reshape(4, 6), B.T)
    assert np.array_equal(p[6 * nn:].reshape(4, 12), np.hstack([D.T, B.T]))


def test_new_entry_points_reject_bad_arguments(lib):
    """Entry points added with the lifting, the coefficient evaluation and the
    double-FP32 apply validate on the host before any CUDA call."""
    from jaxfun_gb300 import _lib

    ERR = _lib.JFG_ERR_ARG
    rows, cols = _lib.int_array([6, 6]), _lib.int_array([8, 8])
    fake = 4096  # never dereferenced: the checks fail first
    # affine apply: no shift, or output aliasing the input
    assert lib.jfg_tp_apply_affine_f64(2, rows, cols, 1, _lib.ptr_array([fake, fake]), fake,
                                       None, fake, fake, 1 << 20, None) == ERR
    assert lib.jfg_tp_apply_affine_f64(2, rows, cols, 1, _lib.ptr_array([fake, fake]), fake,
                                       fake, fake, fake, 1 << 20, None) == ERR
    assert lib.jfg_tp_apply_df64(0, rows, cols, 1, None, None, None, None, 0, None) == ERR
    # coefficient from its logarithm / moments
    assert lib.jfg_exp_weighted_field_f64(2, 8, 1, None, None, None, fake, None, fake, None,
                                          None) == ERR
    assert lib.jfg_field_moments_f64(4, 8, 1, fake, fake, fake, None) == ERR
    # mode mixing: the block owns 8 consecutive modes
    assert lib.jfg_sno_modemix_fwd(2, 10, 64, fake, fake, fake, None) == ERR
    assert lib.jfg_sno_modemix_fwd(2, 16, 65, fake, fake, fake, None) == ERR


def test_tp_apply_workspace_includes_operator_pairs(lib):
    """Two intermediate buffers (256-byte aligned) plus the operators split
    into 8-byte (hi, lo) pairs for the double-FP32 engine."""
    from jaxfun_gb300 import _lib

    def al(x):
        return (x + 255) // 256 * 256

    rows, cols = [30, 20], [32, 24]
    batch = 3
    # pass 1 contracts axis 1: (30... rotate) -> the field between passes is (20, 32)
    inter = al(batch * 20 * 32 * 8)
    ops = al((30 * 32 + 20 * 24) * 8)
    got = lib.jfg_tp_apply_workspace_size(2, _lib.int_array(rows), _lib.int_array(cols), batch, 8)
    assert got == 2 * inter + ops


def test_tpmatrices_solve_signature():
    """TPMatrices.solve keeps the reference's keywords (tpmatrix.py:429-436)
    and rejects unknown choices before any device work."""
    import inspect

    from jaxfun_gb300.la import TPMatrices

    sig = inspect.signature(TPMatrices.solve)
    for k in ("method", "kron_method", "auto_threshold"):
        assert sig.parameters[k].kind is inspect.Parameter.KEYWORD_ONLY
    A = TPMatrices([])
    with pytest.raises(ValueError):
        A.solve(np.zeros((2, 2)), kron_method="cholesky")
    with pytest.raises(ValueError):
        A.solve(np.zeros((2, 2)), method="qr")


def test_xla_ffi_handlers_declared_and_build_is_optional():
    """The jax.ffi handler source defines one handler symbol per registered
    target, the Python binding imports without JAX, and the build step skips
    the handlers cleanly when XLA's FFI header is absent."""
    import re
    from pathlib import Path

    from jaxfun_gb300 import build, ffi

    src = (Path(ffi.__file__).parent / "jfg_xla.cc").read_text()
    defined = set(re.findall(r"XLA_FFI_DEFINE_HANDLER_SYMBOL\((\w+),", src))
    assert defined == set(ffi.TARGETS.values())
    for entry in ("jfg_tp_apply_f64", "jfg_fd_solve_f64", "jfg_varcoef_apply_f64",
                  "jfg_pcg_varcoef_f64"):
        assert entry + "(" in src
    import importlib.util
    import os

    if importlib.util.find_spec("jax") is None and not os.environ.get("JFG_XLA_INCLUDE"):
        assert build.xla_include_dir() is None
        assert build.build_xla_ffi("nvcc", build.OUTDIR / build.LIBNAME) is None


def test_f16_row_split_rounding_and_reconstruction():
    """Host split of operator rows into scaled FP16 (hi, lo): hi is the
    round-to-nearest-even FP16 of the scaled FP32 value (numpy's float16
    conversion of the same FP32 value, subnormals and ties included), the
    scaled row max lies in [2^14, 2^15), and hi + lo reproduces each row to
    2^-22 of its maximum."""
    import ctypes as C

    import numpy as np

    from jaxfun_gb300 import _lib

    L = _lib.lib()
    rng = np.random.default_rng(3)
    rows, cols = 6, 300
    a = rng.standard_normal((rows, cols)) * np.logspace(-12, 12, rows)[:, None]
    a[1, :] *= np.exp(rng.uniform(-30, 0, cols))  # wide range inside a row
    a[2] = 0.0
    # row 3: no scaling (max in [2^14, 2^15)), FP16 edge values
    edge = np.array([20000.0, 2.0 ** -25, 2.0 ** -25 * 1.0001, 2.0 ** -24, 3 * 2.0 ** -25,
                     2.0 ** -14, 2.0 ** -14 * (1 - 2.0 ** -11), 1 + 2.0 ** -11, 1 + 3 * 2.0 ** -11,
                     -1 - 2.0 ** -11, 5.96e-8, 6.1e-5, 1e-3, -1e-7])
    a[3] = 0.0
    a[3, : edge.size] = edge
    hi = np.empty((rows, cols), np.uint16)
    lo = np.empty((rows, cols), np.uint16)
    inv = np.empty(rows, np.float32)
    L.jfg_split_f16_rowscaled_host(rows, cols, a.ctypes.data, hi.ctypes.data, lo.ctypes.data,
                                   inv.ctypes.data)
    for r in range(rows):
        s = 1.0 / float(inv[r])
        v = a[r] * s
        if np.abs(a[r]).max() > 0:
            assert 2.0 ** 14 <= np.abs(v).max() < 2.0 ** 15
        ref_hi = v.astype(np.float32).astype(np.float16).view(np.uint16)
        assert np.array_equal(hi[r], ref_hi), r
        rem = (v - hi[r].view(np.float16).astype(np.float64)).astype(np.float32)
        assert np.array_equal(lo[r], rem.astype(np.float16).view(np.uint16)), r
        back = (hi[r].view(np.float16).astype(np.float64)
                + lo[r].view(np.float16).astype(np.float64)) * float(inv[r])
        assert np.abs(back - a[r]).max() <= 2.0 ** -22 * max(np.abs(a[r]).max(), 1e-300)
    assert inv[3] == 1.0


def test_f16_packed_operator_split_2d_and_3d():
    """The packed variable-coefficient operators split block by block into
    row-scaled FP16 pairs: the row count (2-D 4 nq + 3 n, 3-D 5 nq + 3 n) and,
    row by row in the blocks' order, the same scales and bits as the plain
    row split of that block."""
    import numpy as np

    from jaxfun_gb300 import _lib

    L = _lib.lib()
    n = nq = 24
    nn = n * nq
    rng = np.random.default_rng(8)
    for ndim, blocks in ((2, [(0, 2 * nq, n), (2 * nn, 2 * nq, n), (4 * nn, 2 * n, nq),
                              (6 * nn, n, 2 * nq)]),
                         (3, [(0, 2 * nq, n), (2 * nn, 3 * nq, n), (5 * nn, 3 * n, nq)])):
        rows = L.jfg_varcoef_f16_rows_nd(ndim, n, nq)
        assert rows == (4 * nq + 3 * n if ndim == 2 else 5 * nq + 3 * n)
        ops = rng.standard_normal(8 * nn) * 10.0 ** rng.uniform(-3, 3, 8 * nn)
        hi = np.zeros(8 * nn, np.uint16)
        lo = np.zeros(8 * nn, np.uint16)
        inv = np.zeros(rows, np.float32)
        L.jfg_split_f16_rows_nd_host(ndim, n, nq, ops.ctypes.data, hi.ctypes.data,
                                     lo.ctypes.data, inv.ctypes.data)
        r0 = 0
        for off, nr, ln in blocks:
            blk = np.ascontiguousarray(ops[off: off + nr * ln])
            h2 = np.zeros(nr * ln, np.uint16)
            l2 = np.zeros(nr * ln, np.uint16)
            i2 = np.zeros(nr, np.float32)
            L.jfg_split_f16_rowscaled_host(nr, ln, blk.ctypes.data, h2.ctypes.data,
                                           l2.ctypes.data, i2.ctypes.data)
            assert np.array_equal(hi[off: off + nr * ln], h2)
            assert np.array_equal(lo[off: off + nr * ln], l2)
            assert np.array_equal(inv[r0: r0 + nr], i2)
            r0 += nr
        assert r0 == rows
