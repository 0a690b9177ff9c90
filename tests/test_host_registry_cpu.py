"""CPU: the page-lock registry of caller-owned output arrays (which arrays
qualify, one registration per owning array, release when the owner is
garbage collected), with the CUDA registration calls faked."""
import gc

import numpy as np

from fast_tensor_leverage_gb300._device import HostRegistry


def make():
    calls = {"reg": [], "unreg": []}
    r = HostRegistry(min_bytes=1024, register=lambda p, n: calls["reg"].append((p, n)) or True,
                     unregister=lambda p: calls["unreg"].append(p))
    return r, calls


def test_owner_registered_once_and_released():
    r, calls = make()
    a = np.zeros((64, 64))
    assert r.pinned(a) and r.pinned(a.reshape(-1)[:100]) and r.pinned(a[3])   # views share the owner
    assert calls["reg"] == [(a.ctypes.data, a.nbytes)] and len(r) == 1
    ptr = a.ctypes.data
    del a
    gc.collect()
    assert calls["unreg"] == [ptr] and len(r) == 0


def test_small_foreign_and_refused_buffers_stay_pageable():
    r, calls = make()
    assert not r.pinned(np.zeros(10))                        # below min_bytes
    buf = bytearray(1 << 16)
    assert not r.pinned(np.frombuffer(buf, dtype=np.float64))   # memory owned by another object
    refused = HostRegistry(min_bytes=1, register=lambda p, n: False, unregister=lambda p: None)
    assert not refused.pinned(np.zeros(1000)) and len(refused) == 0
    assert calls["reg"] == []
