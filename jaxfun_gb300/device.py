"""Device plumbing: CUDA tensors, streams and reusable workspaces (torch is used
for device memory and streams only; all arithmetic runs in the library)."""

from __future__ import annotations

import numpy as np
import torch

_WORKSPACES: dict[tuple[int, int], torch.Tensor] = {}


def device() -> torch.device:
    if not torch.cuda.is_available():
        raise RuntimeError("jaxfun_gb300 requires a CUDA device (GB300, sm_103a); none is visible")
    return torch.device("cuda", torch.cuda.current_device())


def as_device(a, dtype=torch.float64) -> torch.Tensor:
    """Return ``a`` as a contiguous CUDA tensor of ``dtype`` (copying host arrays)."""
    if isinstance(a, torch.Tensor):
        t = a
        if t.device.type != "cuda":
            t = t.to(device())
        if t.dtype != dtype:
            t = t.to(dtype)
        return t.contiguous()
    a = np.ascontiguousarray(a)
    if not a.flags.writeable:  # cached read-only operators: torch wants a writable view
        a = a.copy()
    return torch.as_tensor(a, dtype=dtype, device=device())


def workspace(nbytes: int, slot: int = 0) -> torch.Tensor:
    """A cached uint8 device buffer of at least ``nbytes`` for the current stream
    (calls on one stream are ordered, so reuse between calls is safe)."""
    key = (torch.cuda.current_stream().cuda_stream, slot)
    buf = _WORKSPACES.get(key)
    if buf is None or buf.numel() < nbytes:
        buf = torch.empty(max(int(nbytes), 256), dtype=torch.uint8, device=device())
        _WORKSPACES[key] = buf
    return buf


def free_workspaces() -> None:
    _WORKSPACES.clear()
