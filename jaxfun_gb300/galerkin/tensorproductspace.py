"""Tensor-product spaces with GPU transforms.

``TensorProductSpace.backward / forward / scalar_product`` keep the signatures of
src/jaxfun/galerkin/tensorproductspace.py:330-417.  Each transform is one C-ABI
call (``jfg_tp_apply_f64``): d per-axis contraction passes on the GPU, each
contracting the last axis and writing it first, so the field crosses HBM once
per axis.  Leading batch dimensions are allowed (independent fields).
"""

from __future__ import annotations

import numpy as np
import torch

from .. import _lib
from ..device import as_device, workspace
from .spaces import OrthogonalSpace

_OP_CACHE: dict[tuple, torch.Tensor] = {}


def device_op(mat: np.ndarray, dtype=torch.float64) -> torch.Tensor:
    """Upload (once) a host FP64 operator matrix."""
    key = (id(mat), mat.shape, dtype, torch.cuda.current_device())
    t = _OP_CACHE.get(key)
    if t is None:
        t = as_device(mat, dtype)
        _OP_CACHE[key] = t
        # keep the host array alive as long as its device copy is cached
        _OP_CACHE[("host",) + key] = mat  # type: ignore[assignment]
    return t


def tp_apply(mats: list[np.ndarray], x, dtype=torch.float64) -> torch.Tensor:
    """out = (x_ax mats[ax]) x over the trailing len(mats) axes of ``x``."""
    nd = len(mats)
    x = as_device(x, dtype)
    if x.ndim < nd:
        raise ValueError(f"array of rank {x.ndim} for a {nd}-axis transform")
    cols = [m.shape[1] for m in mats]
    rows = [m.shape[0] for m in mats]
    if list(x.shape[x.ndim - nd :]) != cols:
        raise ValueError(f"trailing shape {tuple(x.shape[x.ndim - nd:])} != {tuple(cols)}")
    lead = x.shape[: x.ndim - nd]
    batch = int(np.prod(lead)) if lead else 1
    out = torch.empty(lead + tuple(rows), dtype=dtype, device=x.device)
    if batch == 0:
        return out
    L = _lib.lib()
    r_a, c_a = _lib.int_array(rows), _lib.int_array(cols)
    eb = 8 if dtype == torch.float64 else 4
    ws_bytes = L.jfg_tp_apply_workspace_size(nd, r_a, c_a, batch, eb)
    ws = workspace(ws_bytes)
    ops = [device_op(m, dtype) for m in mats]
    fn = L.jfg_tp_apply_f64 if dtype == torch.float64 else L.jfg_tp_apply_f32
    st = fn(nd, r_a, c_a, batch, _lib.ptr_array([o.data_ptr() for o in ops]), x.data_ptr(),
            out.data_ptr(), ws.data_ptr(), ws.numel(), _lib.stream_handle())
    _lib.check(st, "jfg_tp_apply")
    return out


_SPLIT_CACHE: dict[tuple, tuple] = {}


def device_op_split(mat: np.ndarray):
    """Upload (once) the TF32 (hi, lo) split of a host FP64 operator."""
    key = (id(mat), mat.shape, torch.cuda.current_device())
    t = _SPLIT_CACHE.get(key)
    if t is None:
        from ..la.mixed import split_tf32

        t = split_tf32(mat) + (mat,)
        _SPLIT_CACHE[key] = t
    return t[0], t[1]


def tp_apply_tc(mats: list[np.ndarray], x) -> torch.Tensor:
    """Tensor-core (split-TF32, tcgen05) version of ``tp_apply``: FP32 data."""
    nd = len(mats)
    x = as_device(x, torch.float32)
    cols = [m.shape[1] for m in mats]
    rows = [m.shape[0] for m in mats]
    if list(x.shape[x.ndim - nd :]) != cols:
        raise ValueError(f"trailing shape {tuple(x.shape[x.ndim - nd:])} != {tuple(cols)}")
    lead = x.shape[: x.ndim - nd]
    batch = int(np.prod(lead)) if lead else 1
    out = torch.empty(lead + tuple(rows), dtype=torch.float32, device=x.device)
    if batch == 0:
        return out
    L = _lib.lib()
    r_a, c_a = _lib.int_array(rows), _lib.int_array(cols)
    ws = workspace(L.jfg_tp_apply_workspace_size(nd, r_a, c_a, batch, 4))
    ops = [device_op_split(m) for m in mats]
    st = L.jfg_tp_apply_tc(nd, r_a, c_a, batch, _lib.ptr_array([o[0].data_ptr() for o in ops]),
                           _lib.ptr_array([o[1].data_ptr() for o in ops]), x.data_ptr(),
                           out.data_ptr(), ws.data_ptr(), ws.numel(), _lib.stream_handle())
    _lib.check(st, "jfg_tp_apply_tc")
    return out


_SPLIT16_CACHE: dict[tuple, tuple] = {}


def device_op_split_bf16(mat: np.ndarray):
    """Upload (once) the BF16 (hi, lo) split of a host FP64 operator."""
    key = (id(mat), mat.shape, torch.cuda.current_device())
    t = _SPLIT16_CACHE.get(key)
    if t is None:
        a = np.ascontiguousarray(mat, dtype=np.float64)
        hi = np.empty(a.shape, dtype=np.uint16)
        lo = np.empty(a.shape, dtype=np.uint16)
        _lib.lib().jfg_split_bf16_host(a.size, a.ctypes.data, hi.ctypes.data, lo.ctypes.data)
        t = (torch.as_tensor(hi.view(np.int16), device="cuda"),
             torch.as_tensor(lo.view(np.int16), device="cuda"), mat)
        _SPLIT16_CACHE[key] = t
    return t[0], t[1]


def tp_apply_bf16x3(mats: list[np.ndarray], x) -> torch.Tensor:
    """Tensor-core version of ``tp_apply`` with split-BF16 operators (three BF16
    MMAs per product, FP32 accumulation): FP32 data, for HBM-bound transforms."""
    nd = len(mats)
    x = as_device(x, torch.float32)
    cols = [m.shape[1] for m in mats]
    rows = [m.shape[0] for m in mats]
    if list(x.shape[x.ndim - nd :]) != cols:
        raise ValueError(f"trailing shape {tuple(x.shape[x.ndim - nd:])} != {tuple(cols)}")
    lead = x.shape[: x.ndim - nd]
    batch = int(np.prod(lead)) if lead else 1
    out = torch.empty(lead + tuple(rows), dtype=torch.float32, device=x.device)
    if batch == 0:
        return out
    L = _lib.lib()
    r_a, c_a = _lib.int_array(rows), _lib.int_array(cols)
    ws = workspace(L.jfg_tp_apply_workspace_size(nd, r_a, c_a, batch, 4))
    ops = [device_op_split_bf16(m) for m in mats]
    st = L.jfg_tp_apply_tc_bf16x3(nd, r_a, c_a, batch,
                                  _lib.ptr_array([o[0].data_ptr() for o in ops]),
                                  _lib.ptr_array([o[1].data_ptr() for o in ops]), x.data_ptr(),
                                  out.data_ptr(), ws.data_ptr(), ws.numel(),
                                  _lib.stream_handle())
    _lib.check(st, "jfg_tp_apply_tc_bf16x3")
    return out


def _apply_1d(mat: np.ndarray, x) -> torch.Tensor:
    return tp_apply([mat], x)


class TensorProductSpace:
    """d-dimensional tensor product of 1-D spaces (d in {1, 2, 3})."""

    def __init__(self, basespaces, name: str = "T"):
        self.basespaces: list[OrthogonalSpace] = list(basespaces)
        if not 1 <= len(self.basespaces) <= 3:
            raise ValueError("1, 2 or 3 axes are supported")
        self.name = name

    def __len__(self) -> int:
        return len(self.basespaces)

    def __getitem__(self, i: int) -> OrthogonalSpace:
        return self.basespaces[i]

    def __iter__(self):
        return iter(self.basespaces)

    @property
    def dims(self) -> int:
        return len(self)

    @property
    def shape(self) -> tuple[int, ...]:
        """Physical (quadrature) shape."""
        return tuple(s.num_quad_points for s in self.basespaces)

    @property
    def dim(self) -> tuple[int, ...]:
        """Spectral shape."""
        return tuple(s.dim for s in self.basespaces)

    @property
    def is_orthogonal(self) -> bool:
        return all(s.is_orthogonal for s in self.basespaces)

    def mesh(self, N=None, broadcast: bool = True):
        xs = [s.mesh(None if N is None else N[i]) for i, s in enumerate(self.basespaces)]
        if not broadcast:
            return xs
        return np.meshgrid(*xs, indexing="ij")

    def weights(self) -> np.ndarray:
        ws = [s.quad_points_and_weights()[1] for s in self.basespaces]
        W = ws[0]
        for w in ws[1:]:
            W = np.multiply.outer(W, w)
        return W

    # ---- transforms (tensorproductspace.py:330-417) -------------------------
    # precision: "f64" (FP64 CUDA cores, parity path), "bf16x3" (FP32 data,
    # split-BF16 operators, three BF16 MMAs per product) or "tc" (FP32 data,
    # split-TF32 tcgen05 contractions)
    def _apply(self, mats, x, precision):
        if precision == "f64":
            return tp_apply(mats, x)
        if precision == "bf16x3":
            return tp_apply_bf16x3(mats, x)
        if precision == "tc":
            return tp_apply_tc(mats, x)
        raise ValueError(f"unknown precision {precision!r}")

    def backward(self, c, N: tuple[int | None, ...] | None = None,
                 precision: str = "f64") -> torch.Tensor:
        mats = [
            s.backward_matrix(None if N is None else N[i]) for i, s in enumerate(self.basespaces)
        ]
        return self._apply(mats, c, precision)

    def forward(self, u, precision: str = "f64") -> torch.Tensor:
        nd = len(self)
        shp = tuple(u.shape[-nd:])
        mats = [s.forward_matrix(shp[i]) for i, s in enumerate(self.basespaces)]
        return self._apply(mats, u, precision)

    def scalar_product(self, u, precision: str = "f64") -> torch.Tensor:
        nd = len(self)
        shp = tuple(u.shape[-nd:])
        mats = [s.scalar_product_matrix(shp[i]) for i, s in enumerate(self.basespaces)]
        return self._apply(mats, u, precision)

    def backward_derivative(self, c, k: tuple[int, ...]) -> torch.Tensor:
        """d^k u / dx^k on the quadrature grid (per-axis derivative orders)."""
        mats = [s.backward_matrix(None, k[i]) for i, s in enumerate(self.basespaces)]
        return tp_apply(mats, c)


def TensorProduct(*basespaces, name: str = "T") -> TensorProductSpace:
    """Factory (src/jaxfun/galerkin/tensorproductspace.py:507-557)."""
    return TensorProductSpace(basespaces, name=name)
