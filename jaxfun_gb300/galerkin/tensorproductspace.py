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


def tp_apply(mats: list[np.ndarray], x, dtype=torch.float64, df: bool = False) -> torch.Tensor:
    """out = (x_ax mats[ax]) x over the trailing len(mats) axes of ``x``.
    ``df``: FP64 data with double-FP32 arithmetic (``jfg_tp_apply_df64``)."""
    nd = len(mats)
    if df and dtype != torch.float64:
        raise ValueError("the double-FP32 engine takes FP64 data")
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
    fn = (L.jfg_tp_apply_df64 if df else L.jfg_tp_apply_f64) if dtype == torch.float64 \
        else L.jfg_tp_apply_f32
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


def tp_apply_affine(mats: list[np.ndarray], x, shift: np.ndarray, cache: bool = True
                    ) -> torch.Tensor:
    """out = (x_ax mats[ax]) x + shift over the trailing len(mats) axes of ``x``,
    the same ``shift`` (host FP64, shape = the output's trailing shape) for
    every leading index: one ``jfg_tp_apply_affine_f64`` call, the constant
    added in the last pass's epilogue.  ``cache=False`` uploads the operands
    without keeping device copies (one-off evaluation points)."""
    nd = len(mats)
    x = as_device(x, torch.float64)
    if x.ndim < nd:
        raise ValueError(f"array of rank {x.ndim} for a {nd}-axis transform")
    cols = [m.shape[1] for m in mats]
    rows = [m.shape[0] for m in mats]
    if list(x.shape[x.ndim - nd :]) != cols:
        raise ValueError(f"trailing shape {tuple(x.shape[x.ndim - nd:])} != {tuple(cols)}")
    if tuple(np.shape(shift)) != tuple(rows):
        raise ValueError(f"shift shape {np.shape(shift)} != {tuple(rows)}")
    lead = x.shape[: x.ndim - nd]
    batch = int(np.prod(lead)) if lead else 1
    out = torch.empty(lead + tuple(rows), dtype=torch.float64, device=x.device)
    if batch == 0:
        return out
    up = device_op if cache else (lambda m: as_device(np.ascontiguousarray(m), torch.float64))
    ops = [up(m) for m in mats]
    sh = up(shift)
    x = x.contiguous()
    L = _lib.lib()
    r_a, c_a = _lib.int_array(rows), _lib.int_array(cols)
    ws = workspace(L.jfg_tp_apply_workspace_size(nd, r_a, c_a, batch, 8))
    st = L.jfg_tp_apply_affine_f64(nd, r_a, c_a, batch,
                                   _lib.ptr_array([o.data_ptr() for o in ops]), x.data_ptr(),
                                   sh.data_ptr(), out.data_ptr(), ws.data_ptr(), ws.numel(),
                                   _lib.stream_handle())
    _lib.check(st, "jfg_tp_apply_affine_f64")
    return out


_SPB_CACHE: dict = {}


def _sp_backward_matrix(test, source) -> np.ndarray:
    """SP_test B_source at the test space's quadrature rule: (dim_test x
    dim_source), the scalar product of a source-space expansion."""
    key = (id(test), id(source))
    hit = _SPB_CACHE.get(key)
    if hit is not None and hit[0] is test and hit[1] is source:
        return hit[2]
    nq = test.num_quad_points
    M = test.scalar_product_matrix(nq) @ source.backward_matrix(nq)
    M.setflags(write=False)
    _SPB_CACHE[key] = (test, source, M)
    return M


def _apply_1d(mat: np.ndarray, x) -> torch.Tensor:
    return tp_apply([mat], x)


def kron_apply_host(mats: list[np.ndarray], a: np.ndarray) -> np.ndarray:
    """FP64 host (x_ax mats[ax]) a for the small one-time lifting setup."""
    for ax, m in enumerate(mats):
        a = np.moveaxis(np.tensordot(m, a, axes=(1, ax)), 0, ax)
    return a


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
    # precision: "f64" (FP64 CUDA cores, parity path), "df64" (FP64 data,
    # double-FP32 arithmetic on the FP32 pipe, ~1e-14), "bf16x3" (FP32 data,
    # split-BF16 operators, three BF16 MMAs per product) or "tc" (FP32 data,
    # split-TF32 tcgen05 contractions)
    def _apply(self, mats, x, precision):
        if precision == "f64":
            return tp_apply(mats, x)
        if precision == "df64":
            return tp_apply(mats, x, df=True)
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

    def scalar_product_expansion(self, coef, source: "TensorProductSpace | None" = None,
                                 precision: str = "f64") -> torch.Tensor:
        """(f, v) for every test function v of this space, with f given by its
        coefficients in ``source`` (default: this space's orthogonal space) --
        inner(f*v) of a JAXFunction f (inner.py:914-984 on the values that
        evaluate_jaxfunction_expr_quad, arguments.py:928-990, produces).  The
        backward transform of f and the scalar product are fused per axis into
        one operator, SP_ax B_ax (FP64 host product, cached), so the whole
        right-hand side is ONE tensor-product apply: half the passes of
        backward then scalar_product, and f's grid values never exist."""
        src = self.get_orthogonal() if source is None else source
        if len(src) != len(self):
            raise ValueError("source space has a different dimension")
        mats = [_sp_backward_matrix(s, t) for s, t in zip(self.basespaces, src.basespaces)]
        return self._apply(mats, coef, precision)

    def backward_derivative(self, c, k: tuple[int, ...]) -> torch.Tensor:
        """d^k u / dx^k on the quadrature grid (per-axis derivative orders)."""
        mats = [s.backward_matrix(None, k[i]) for i, s in enumerate(self.basespaces)]
        return tp_apply(mats, c)

    def evaluate_mesh(self, c, kind: str = "quadrature", N=None) -> torch.Tensor:
        """u on the tensor mesh of quadrature or equispaced ("uniform") points
        (tensorproductspace.py evaluate_mesh, orthogonal.py:181-199)."""
        mats = [s.evaluation_matrix(kind, None if N is None else N[i])
                for i, s in enumerate(self.basespaces)]
        return tp_apply(mats, c)

    def get_homogeneous(self) -> "TensorProductSpace":
        return self

    def get_orthogonal(self) -> "TensorProductSpace":
        return TensorProductSpace([s.orthogonal for s in self.basespaces], name=self.name)


# ---------------------------------------------------------------------------
# inhomogeneous Dirichlet data: DirectSumTPS (tensorproductspace.py:560-851)
# ---------------------------------------------------------------------------

_ENDS = (-1.0, 1.0)


def _project(space, g: np.ndarray) -> np.ndarray:
    """project1D of grid values onto a homogeneous or orthogonal 1-D space:
    its forward transform (inner.py:1027-1041, Composite.forward)."""
    return space.forward_matrix(g.shape[0]) @ g


def _project_lifted(space, corner: np.ndarray, g: np.ndarray) -> np.ndarray:
    """project1D onto space (+) boundary basis with Dirichlet values ``corner``:
    DirectSum.forward = R (F_orth g - B^T corner) (composite.py:612-621)."""
    from .spaces import BCGeneric, reduce_matrix

    B = BCGeneric(space.N, space.family, {"left": {"D": 0.0}, "right": {"D": 0.0}}).S
    F = space.orthogonal.forward_matrix(g.shape[0])
    return reduce_matrix(space) @ (F @ g - B.T @ corner)


def _nested_forward(X, D, bnd: np.ndarray, G: np.ndarray) -> np.ndarray:
    """Forward of the 2-D lifted product X (x) (D (+) B') with the boundary
    coefficients ``bnd`` (nx, 2) of (X, B'): DirectSumTPS.forward =
    (R_X (x) R_D)(orthogonal forward of G - lift) (tensorproductspace.py:786-790,
    825-851)."""
    from .spaces import BCGeneric, reduce_matrix

    B = BCGeneric(D.N, D.family, {"left": {"D": 0.0}, "right": {"D": 0.0}}).S
    lift = X.S.T @ bnd @ B
    Fx = X.orthogonal.forward_matrix(G.shape[0])
    Fd = D.orthogonal.forward_matrix(G.shape[1])
    return reduce_matrix(X) @ (Fx @ G @ Fd.T - lift) @ reduce_matrix(D).T


def lifting_coefficients(spaces) -> dict:
    """Boundary coefficients of every mixed (homogeneous x boundary) product
    space, keyed by the tuple of 1-D spaces, restating the cases of
    DirectSumTPS.__init__ (tensorproductspace.py:609-745): one or two
    inhomogeneous axes in 2-D, and in 3-D behind a homogeneous first axis.
    Host FP64 setup, done once per space."""
    from .spaces import DirectSum

    nd = len(spaces)
    ds = [isinstance(s, DirectSum) for s in spaces]
    hom = [s[0] if d else s for s, d in zip(spaces, ds, strict=True)]
    bnd = [s[1] if d else None for s, d in zip(spaces, ds, strict=True)]
    x = [h.mesh() for h in hom]
    e = [np.array(v) for v in _ENDS]
    out: dict = {}
    if nd == 2:
        if ds[0] and ds[1]:
            h, g = bnd[0].values, bnd[1].values
            # corners: axis-0 data h_a at y = end_b (projected_bcs[0])
            out[(bnd[0], bnd[1])] = np.array(
                [[float(h[a](e[a], e[b])) for b in range(2)] for a in range(2)])
            uh = []
            for j in range(2):
                corner = np.array([float(g[j](e[s], e[j])) for s in range(2)])
                uh.append(_project_lifted(hom[0], corner, g[j](x[0], e[j])))
            out[(hom[0], bnd[1])] = np.array(uh).T
            uh = []
            for j in range(2):
                corner = np.array([float(h[j](e[j], e[s])) for s in range(2)])
                uh.append(_project_lifted(hom[1], corner, h[j](e[j], x[1])))
            out[(bnd[0], hom[1])] = np.array(uh)
        else:
            a = 0 if ds[0] else 1
            o = 1 - a
            vals = bnd[a].values
            uh = []
            for j in range(2):
                coords = [None, None]
                coords[a] = e[j]
                coords[o] = x[o]
                uh.append(_project(hom[o], vals[j](*coords)))
            key = [hom[0], hom[1]]
            key[a] = bnd[a]
            out[tuple(key)] = np.array(uh) if a == 0 else np.array(uh).T
        return out
    # 3-D: axis 0 is homogeneous (or orthogonal)
    X = hom[0]
    xg = x[0][:, None]
    if ds[1] and ds[2]:
        h, g = bnd[1].values, bnd[2].values  # h_a(x, z) at y = end_a; g_b(x, y) at z = end_b
        uh = []
        for j in range(2):
            G = g[j](xg, x[1][None, :], e[j])
            nb = np.stack([_project(X, g[j](x[0], e[s], e[j])) for s in range(2)], axis=1)
            uh.append(_nested_forward(X, hom[1], nb, G))
        out[(X, hom[1], bnd[2])] = np.array(uh).transpose(1, 2, 0)
        uh = []
        for j in range(2):
            G = h[j](xg, e[j], x[2][None, :])
            nb = np.stack([_project(X, h[j](x[0], e[j], e[s])) for s in range(2)], axis=1)
            uh.append(_nested_forward(X, hom[2], nb, G))
        out[(X, bnd[1], hom[2])] = np.array(uh).transpose(1, 0, 2)
        uh = [_project(X, h[a](x[0], e[a], e[b])) for a in range(2) for b in range(2)]
        out[(X, bnd[1], bnd[2])] = np.array(uh).T.reshape(-1, 2, 2)
        return out
    a = 1 if ds[1] else 2
    o = 3 - a
    vals = bnd[a].values
    Fx = X.forward_matrix(x[0].shape[0])
    Fo = hom[o].forward_matrix(x[o].shape[0])
    uh = []
    for j in range(2):
        coords = [xg, None, None]
        coords[a] = e[j]
        coords[o] = x[o][None, :]
        G = np.broadcast_to(vals[j](*coords), (x[0].shape[0], x[o].shape[0]))
        uh.append(Fx @ G @ Fo.T)
    key = [X, hom[1], hom[2]]
    key[a] = bnd[a]
    out[tuple(key)] = (np.array(uh).transpose(1, 2, 0) if a == 2
                       else np.array(uh).transpose(1, 0, 2))
    return out


class DirectSumTPS(TensorProductSpace):
    """Tensor product in which one or two axes are DirectSums (inhomogeneous
    Dirichlet data), src/jaxfun/galerkin/tensorproductspace.py:560-851.

    ``tpspaces`` holds every product of homogeneous and boundary factors and
    ``bndvals`` the fixed boundary coefficients of the mixed ones (computed
    once on the host in FP64).  Their sum in orthogonal coefficients is the
    lift a_bc, so every transform is affine in the homogeneous coefficients c
    and runs as ONE GPU call (``jfg_tp_apply_affine_f64``: d per-axis passes,
    the constant added in the last pass's epilogue):

      backward(c)        = (x V_i) c + (x V_orth,i) a_bc
      to_orthogonal(c)   = (x S_i^T) c + a_bc
      from_orthogonal(a) = (x R_i) a - (x R_i) a_bc,   R = (S S^T)^{-1} S
      forward(u)         = (x R_i F_orth,i) u - (x R_i) a_bc
    """

    def __init__(self, basespaces, name: str = "DSTPS"):
        import itertools

        from .spaces import DirectSum

        super().__init__(basespaces, name=name)
        nd = len(self.basespaces)
        bcidx = [i for i, s in enumerate(self.basespaces) if isinstance(s, DirectSum)]
        if nd < 2 or not bcidx:
            raise ValueError("DirectSumTPS needs 2 or 3 axes, at least one a DirectSum")
        if nd == 3 and bcidx[0] == 0:
            raise ValueError("DirectSum cannot be the first space in a 3D tensor product.")
        self.homogeneous_spaces = [s[0] if isinstance(s, DirectSum) else s
                                   for s in self.basespaces]
        choices = [tuple(s) if isinstance(s, DirectSum) else (s,) for s in self.basespaces]
        self.tpspaces = {
            combo: TensorProductSpace(combo, name=f"{name}{i}")
            for i, combo in enumerate(itertools.product(*choices))
        }
        self.bndvals = lifting_coefficients(self.basespaces)
        lift = np.zeros(tuple(s.N for s in self.homogeneous_spaces))
        for combo, vals in self.bndvals.items():
            lift += kron_apply_host([s.S.T for s in combo], vals)
        lift.setflags(write=False)
        self.lift = lift
        self._maps: dict = {}

    @property
    def dim(self) -> tuple[int, ...]:
        return tuple(s.dim for s in self.homogeneous_spaces)

    @property
    def num_dofs(self) -> tuple[int, ...]:
        return self.dim

    @property
    def is_orthogonal(self) -> bool:
        return False

    def get_homogeneous(self) -> TensorProductSpace:
        return TensorProductSpace(self.homogeneous_spaces, name=self.name)

    def get_orthogonal(self) -> TensorProductSpace:
        return TensorProductSpace([s.orthogonal for s in self.homogeneous_spaces],
                                  name=self.name)

    def affine_map(self, kind: str, N=None):
        """(per-axis matrices, shift) of one affine map, cached per size."""
        from .spaces import reduce_matrix

        key = (kind, None if N is None else tuple(N))
        m = self._maps.get(key)
        if m is not None:
            return m
        H = self.homogeneous_spaces
        R = [reduce_matrix(s) for s in H]
        if kind == "to_orthogonal":
            mats, shift = [s.S.T.copy() for s in H], self.lift
        elif kind == "from_orthogonal":
            mats, shift = R, -kron_apply_host(R, self.lift)
        elif kind in ("quadrature", "uniform"):
            Ns = [None] * len(H) if N is None else list(N)
            mats = [s.evaluation_matrix(kind, Ns[i]) for i, s in enumerate(H)]
            shift = kron_apply_host(
                [s.orthogonal.evaluation_matrix(kind, Ns[i]) for i, s in enumerate(H)],
                self.lift)
        elif kind == "forward":
            mats = [R[i] @ s.orthogonal.forward_matrix(N[i]) for i, s in enumerate(H)]
            shift = -kron_apply_host(R, self.lift)
        else:
            raise ValueError(f"unknown map {kind!r}")
        mats = [np.ascontiguousarray(a) for a in mats]
        shift = np.ascontiguousarray(shift)
        for a in mats + [shift]:
            a.setflags(write=False)
        self._maps[key] = (mats, shift)
        return mats, shift

    def _affine(self, kind, x, N=None, precision="f64"):
        if precision != "f64":
            raise ValueError("lifted (DirectSum) transforms run in FP64")
        mats, shift = self.affine_map(kind, N)
        return tp_apply_affine(mats, x, shift)

    def backward(self, c, N=None, precision: str = "f64") -> torch.Tensor:
        return self._affine("quadrature", c, N, precision)

    def evaluate_mesh(self, c, kind: str = "quadrature", N=None) -> torch.Tensor:
        return self._affine(kind, c, N)

    def forward(self, u, precision: str = "f64") -> torch.Tensor:
        nd = len(self)
        return self._affine("forward", u, tuple(int(n) for n in u.shape[-nd:]), precision)

    def to_orthogonal(self, c) -> torch.Tensor:
        return self._affine("to_orthogonal", c)

    def from_orthogonal(self, a) -> torch.Tensor:
        return self._affine("from_orthogonal", a)

    def scalar_product(self, u, precision: str = "f64"):
        raise RuntimeError(
            "Scalar product requires homogeneous test space (call on get_homogeneous())")

    def backward_derivative(self, c, k: tuple[int, ...]) -> torch.Tensor:
        """d^k u / dx^k including the lift's derivatives."""
        key = ("derivative", tuple(k))
        if key not in self._maps:
            H = self.homogeneous_spaces
            mats = [s.backward_matrix(None, k[i]) for i, s in enumerate(H)]
            shift = kron_apply_host([s.orthogonal.backward_matrix(None, k[i])
                                     for i, s in enumerate(H)], self.lift)
            shift.setflags(write=False)
            self._maps[key] = (mats, shift)
        mats, shift = self._maps[key]
        return tp_apply_affine(mats, c, shift)


def TensorProduct(*basespaces, name: str = "T") -> TensorProductSpace:
    """Factory (src/jaxfun/galerkin/tensorproductspace.py:507-557): a
    DirectSumTPS when any axis carries inhomogeneous Dirichlet data."""
    from .spaces import DirectSum

    if any(isinstance(s, DirectSum) for s in basespaces):
        return DirectSumTPS(basespaces, name=name)
    return TensorProductSpace(basespaces, name=name)
