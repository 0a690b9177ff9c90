"""Device plumbing shared by the host classes: CUDA device/stream lookup,
argument validation for the reference-shaped numpy entry points, and pinned
staging buffers for device<->host copies."""
from __future__ import annotations

import ctypes
import threading
import weakref

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


class HostRegistry:
    """Page-locks caller-owned numpy output arrays (ftl_host_register) the
    first time results are copied into them, so the copies are DMA transfers
    instead of staged pageable ones; the registration is dropped
    (ftl_host_unregister) when the array that owns the memory is garbage
    collected, before numpy frees it.  Arrays below `min_bytes`, views of
    memory numpy does not own, and buffers whose pages the runtime refuses
    to register stay pageable (the copies are then synchronous, as before)."""

    def __init__(self, min_bytes: int = 1 << 16, register=None, unregister=None):
        self.min_bytes = int(min_bytes)
        self._reg = register or self._c_register
        self._unreg = unregister or self._c_unregister
        self._live = {}          # id(owner) -> (data pointer, nbytes)
        self._lock = threading.Lock()

    @staticmethod
    def _c_register(ptr: int, nbytes: int) -> bool:
        ok = ctypes.c_int(0)
        _lib.call("ftl_host_register", ptr, nbytes, ctypes.byref(ok))
        return bool(ok.value)

    @staticmethod
    def _c_unregister(ptr: int) -> None:
        _lib.call("ftl_host_unregister", ptr)

    @staticmethod
    def _owner(a: np.ndarray):
        o = a
        while isinstance(o.base, np.ndarray):
            o = o.base
        return o if (o.base is None and o.flags["OWNDATA"]) else None

    def pinned(self, a: np.ndarray) -> bool:
        """True when `a`'s memory is page-locked (registering it now if it
        qualifies)."""
        o = self._owner(a)
        if o is None or o.nbytes < self.min_bytes:
            return False
        key, ptr, nb = id(o), int(o.ctypes.data), int(o.nbytes)
        with self._lock:
            if self._live.get(key) == (ptr, nb):
                return True
            if key in self._live:
                return False
            if not self._reg(ptr, nb):
                return False
            self._live[key] = (ptr, nb)
        weakref.finalize(o, self._drop, key, ptr)
        return True

    def _drop(self, key: int, ptr: int) -> None:
        with self._lock:
            self._live.pop(key, None)
        self._unreg(ptr)

    def __len__(self) -> int:
        return len(self._live)


HOST_REGISTRY = HostRegistry()


def copy_to_numpy(dst: np.ndarray, src: torch.Tensor, stream=None) -> bool:
    """dst (numpy, same number of elements and item size as src) <- src
    (CUDA tensor).  Page-locked destinations get an asynchronous DMA copy on
    `stream` (the caller synchronises); returns whether the copy is still in
    flight."""
    t = torch.from_numpy(dst)
    if HOST_REGISTRY.pinned(dst):
        with torch.cuda.stream(stream) if stream is not None else _nullctx():
            t.copy_(src.view(t.shape), non_blocking=True)
        return True
    t.copy_(src.view(t.shape))
    return False


class _nullctx:
    def __enter__(self):
        return self

    def __exit__(self, *a):
        return False
