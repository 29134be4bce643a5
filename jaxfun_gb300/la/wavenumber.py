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

import numpy as np
import torch

from .. import _lib
from ..device import as_device


class TPMatricesWavenumberSolver:
    """``B_data_batch`` (n_F, n_diags, n_P): the per-wavenumber band data in
    jaxfun's column-aligned DIA convention (data[k][d][j] = B_k[j - off_d][j]),
    wavenumbers in C order over the Fourier axes of ``shape``; ``poly_offsets``
    the diagonal offsets; ``poly_axis`` the polynomial axis of ``shape``."""

    def __init__(self, poly_axis: int, shape: tuple[int, ...], B_data_batch,
                 poly_offsets: tuple[int, ...]):
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
