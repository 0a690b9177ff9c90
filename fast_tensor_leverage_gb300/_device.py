"""Device plumbing shared by the host classes: CUDA device/stream lookup,
argument validation for the reference-shaped numpy entry points, and pinned
staging buffers for device<->host copies."""
from __future__ import annotations

import numpy as np
import torch

from . import _lib


def cuda_device(device=None) -> torch.device:
    if not torch.cuda.is_available():
        raise RuntimeError("fast_tensor_leverage_gb300 needs a CUDA device (there is no CPU fallback)")
    _lib.lib()  # fail loudly if the extension is missing
    if device is None:
        return torch.device("cuda", torch.cuda.current_device())
    d = torch.device(device)
    if d.type != "cuda":
        raise ValueError(f"device must be a CUDA device, got {d}")
    return d if d.index is not None else torch.device("cuda", torch.cuda.current_device())


def stream_ptr(device: torch.device, stream=None) -> int:
    s = stream if stream is not None else torch.cuda.current_stream(device)
    return int(s.cuda_stream)


def ptr(t: torch.Tensor | None):
    return None if t is None else int(t.data_ptr())


def require_numpy_out(a, dtype, name: str, min_size: int | None = None, shape=None) -> np.ndarray:
    """Outputs are written in place, so a wrong dtype or a non-contiguous
    array (which the reference's bindings silently copy, losing the result)
    is rejected."""
    if not isinstance(a, np.ndarray):
        raise TypeError(f"{name} must be a numpy.ndarray, got {type(a).__name__}")
    if a.dtype != dtype:
        raise TypeError(f"{name} must have dtype {np.dtype(dtype).name}, got {a.dtype}")
    if not a.flags["C_CONTIGUOUS"] or not a.flags["WRITEABLE"]:
        raise ValueError(f"{name} must be a writeable C-contiguous array")
    if shape is not None and tuple(a.shape) != tuple(shape):
        raise ValueError(f"{name} must have shape {tuple(shape)}, got {a.shape}")
    if min_size is not None and a.size < min_size:
        raise ValueError(f"{name} holds {a.size} elements, needs at least {min_size}")
    return a


def as_factor(u, R: int, name: str) -> np.ndarray:
    if isinstance(u, torch.Tensor):
        u = u.detach().cpu().numpy()
    a = np.asarray(u)
    if a.ndim != 2:
        raise ValueError(f"{name} must be 2-D, got shape {a.shape}")
    if a.shape[1] != R:
        raise ValueError(f"{name} has {a.shape[1]} columns, expected R={R}")
    if a.shape[0] < 1:
        raise ValueError(f"{name} has no rows")
    return np.ascontiguousarray(a, dtype=np.float64)


class PinnedStage:
    """Reusable pinned host buffers keyed by (shape, dtype)."""

    def __init__(self):
        self._bufs = {}

    def get(self, shape, dtype) -> torch.Tensor:
        key = (tuple(shape), dtype)
        buf = self._bufs.get(key)
        if buf is None:
            buf = torch.empty(shape, dtype=dtype, pin_memory=True)
            self._bufs[key] = buf
        return buf
