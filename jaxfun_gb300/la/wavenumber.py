"""Per-wavenumber solver for Fourier x polynomial tensor-product systems.

Mirrors ``TPMatricesWavenumberSolver`` (src/jaxfun/la/tpmatrix.py:590-1013):
every axis but one is Fourier (diagonal per-axis matrices), so the system
splits into one 1-D banded polynomial system B_k per combination of Fourier
wavenumbers.  The GB300 path factors all B_k at once without pivoting
(``jfg_banded_lu_factor_f64``, one thread per system, factors interleaved
across systems for coalesced access) and solves every right-hand side with one
launch (``jfg_banded_lu_solve_f64``) directly in the caller's layout, without
the reference's transposes.
"""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np
import torch

from .. import _lib
from ..device import as_device


@dataclass(frozen=True)
class DiaMatrix:
    """Square banded matrix in jaxfun's column-aligned DIA storage
    (src/jaxfun/la/diamatrix.py:100-160): ``data[d][j] = A[j - offsets[d]][j]``
    (upper diagonals start at column ``off``, lower ones at column 0), shape
    ``(n_diags, n)``.  A host-side container for the per-wavenumber systems."""

    data: np.ndarray
    offsets: tuple[int, ...]

    @staticmethod
    def from_dense(a, offsets: tuple[int, ...]) -> "DiaMatrix":
        a = np.asarray(a, dtype=np.float64)
        n = a.shape[0]
        if a.shape != (n, n):
            raise ValueError("DiaMatrix.from_dense needs a square matrix")
        data = np.zeros((len(offsets), n))
        for d, off in enumerate(offsets):
            j = np.arange(max(0, off), min(n, n + off))
            data[d, j] = a[j - off, j]
        return DiaMatrix(data, tuple(int(o) for o in offsets))

    @property
    def shape(self) -> tuple[int, int]:
        n = self.data.shape[1]
        return (n, n)

    def todense(self) -> np.ndarray:
        n = self.data.shape[1]
        a = np.zeros((n, n))
        for d, off in enumerate(self.offsets):
            j = np.arange(max(0, off), min(n, n + off))
            a[j - off, j] = self.data[d, j]
        return a


def _stack_dia(B_matrices) -> tuple[np.ndarray, tuple[int, ...]]:
    """Per-wavenumber DIA matrices (objects with ``data`` and ``offsets``, or
    ``(data, offsets)`` pairs) aligned on the union of their offsets:
    (n_F, n_diags, n_P) band data, the legacy ``B_matrices`` input of the
    reference (src/jaxfun/la/tpmatrix.py:823-845)."""
    mats = []
    for B in B_matrices:
        data, offs = (B.data, B.offsets) if hasattr(B, "offsets") else B
        data = np.asarray(data.cpu() if torch.is_tensor(data) else data, dtype=np.float64)
        offs = tuple(int(o) for o in offs)
        if data.ndim != 2 or data.shape[0] != len(offs):
            raise ValueError("each B matrix needs data of shape (len(offsets), n)")
        mats.append((data, offs))
    if not mats:
        raise ValueError("B_matrices is empty")
    n_P = mats[0][0].shape[1]
    if any(d.shape[1] != n_P for d, _ in mats):
        raise ValueError("all B matrices must have the same size")
    union = tuple(sorted({o for _, offs in mats for o in offs}))
    out = np.zeros((len(mats), len(union), n_P))
    for k, (data, offs) in enumerate(mats):
        for d, o in enumerate(offs):
            out[k, union.index(o)] += data[d]
    return out, union


class TPMatricesWavenumberSolver:
    """``B_data_batch`` (n_F, n_diags, n_P): the per-wavenumber band data in
    jaxfun's column-aligned DIA convention (data[k][d][j] = B_k[j - off_d][j]),
    wavenumbers in C order over the Fourier axes of ``shape``; ``poly_offsets``
    the diagonal offsets; ``poly_axis`` the polynomial axis of ``shape``.
    Alternatively ``B_matrices``: one DIA matrix per wavenumber (``DiaMatrix``
    or any object with ``data`` and ``offsets``), stacked on the union of
    their offsets and factored by the same batched kernel.  The argument
    order is the reference's (src/jaxfun/la/tpmatrix.py:718-725)."""

    def __init__(self, poly_axis: int, shape: tuple[int, ...], B_matrices=None,
                 B_data_batch=None, poly_offsets: tuple[int, ...] | None = None):
        if B_data_batch is None or poly_offsets is None:
            if B_matrices is None:
                raise ValueError("either B_data_batch + poly_offsets or B_matrices is required")
            B_data_batch, poly_offsets = _stack_dia(B_matrices)
        self.poly_axis = int(poly_axis)
        self.shape = tuple(int(s) for s in shape)
        nd = len(self.shape)
        if not 0 <= self.poly_axis < nd:
            raise ValueError(f"poly_axis {poly_axis} out of range for shape {shape}")
        data = as_device(B_data_batch)
        n_F, n_diag, n_P = data.shape
        fourier = [a for a in range(nd) if a != self.poly_axis]
        if n_P != self.shape[self.poly_axis] or n_F != int(np.prod([self.shape[a] for a in fourier])):
            raise ValueError("B_data_batch does not match shape / poly_axis")
        if len(poly_offsets) != n_diag:
            raise ValueError("one offset per diagonal is required")
        self.offsets = tuple(int(o) for o in poly_offsets)
        self.p = max(0, -min(self.offsets))
        self.q = max(0, max(self.offsets))
        self.n_F, self.n_P = n_F, n_P
        L = _lib.lib()
        self.lu = torch.empty(L.jfg_banded_lu_size(n_F, n_P, self.p, self.q) // 8,
                              dtype=torch.float64, device=data.device)
        _lib.check(L.jfg_banded_lu_factor_f64(n_F, n_P, n_diag, _lib.int_array(self.offsets),
                                              data.contiguous().data_ptr(), self.lu.data_ptr(),
                                              _lib.stream_handle()), "jfg_banded_lu_factor_f64")
        # strides of (wavenumber, polynomial index) in a C-order array of `shape`
        st = [int(np.prod(self.shape[a + 1:])) for a in range(nd)]
        self.elem_stride = st[self.poly_axis]
        fshape = [self.shape[a] for a in fourier]
        fstr = [st[a] for a in fourier]
        # wavenumber k (C order over the Fourier axes) -> offset; regular only if
        # the Fourier axes are contiguous in the strides, else one call per slab
        self._fourier_shape, self._fourier_strides = fshape, fstr

    def solve(self, rhs) -> torch.Tensor:
        """Solution with the shape of ``rhs`` (= ``shape``)."""
        rhs = as_device(rhs).contiguous()
        if tuple(rhs.shape) != self.shape:
            raise ValueError(f"rhs shape {tuple(rhs.shape)} != {self.shape}")
        x = torch.empty_like(rhs)
        L = _lib.lib()
        sh = _lib.stream_handle()
        fshape, fstr = self._fourier_shape, self._fourier_strides
        if not fshape:
            fshape, fstr = [1], [0]
        # the innermost Fourier axis is one strided batch; outer Fourier axes loop
        inner_n, inner_s = fshape[-1], fstr[-1]
        outer = [range(s) for s in fshape[:-1]]
        for idx in np.ndindex(*[len(r) for r in outer]) if outer else [()]:
            base = sum(i * s for i, s in zip(idx, fstr[:-1]))
            k0 = int(np.ravel_multi_index(idx + (0,), fshape)) if outer else 0
            # a contiguous run of inner_n systems starting at wavenumber k0
            lu_view = self._lu_slice(k0, inner_n)
            _lib.check(L.jfg_banded_lu_solve_f64(inner_n, self.n_P, self.p, self.q,
                                                 lu_view.data_ptr(),
                                                 rhs.data_ptr() + 8 * base,
                                                 x.data_ptr() + 8 * base, inner_s,
                                                 self.elem_stride, sh),
                       "jfg_banded_lu_solve_f64")
        return x

    def _lu_slice(self, k0: int, cnt: int) -> torch.Tensor:
        """Factors of systems k0 .. k0+cnt-1 re-packed contiguously (interleaved)."""
        if k0 == 0 and cnt == self.n_F:
            return self.lu
        key = (k0, cnt)
        cache = self.__dict__.setdefault("_slices", {})
        t = cache.get(key)
        if t is None:
            bw = self.p + self.q + 1
            t = self.lu.view(bw * self.n_P, self.n_F)[:, k0:k0 + cnt].contiguous()
            cache[key] = t
        return t
