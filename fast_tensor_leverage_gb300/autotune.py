"""Autotuner of the kernel variants (no counterpart in the reference, whose
tuning knobs are compile flags).

Some kernels are compiled in several variants that give identical results
with different launch shapes (see ftl_tune_variants in include/ftl.h): the
FP32 draw on wrapped-diagonal trees (16 < R <= 32) descends 1, 2 or 3
samples per warp in lockstep.  Which is fastest depends on the GPU and the
workload, so the tuner times every variant on a live sampler (CUDA events
around the descent launches), selects the fastest for the current device
(ftl_tune_set) and records it in a JSON cache keyed by GPU name, kernel
family, rank and precision.  Later processes apply the cached choice without
timing (Sampler(..., autotune="cached"), the default).

Cache file: $FTL_TUNE_CACHE, else ~/.cache/fast_tensor_leverage_gb300/tune.json.
"""
from __future__ import annotations

import ctypes
import json
import os
import statistics
import tempfile
from pathlib import Path

from . import _lib

FAMILY_DRAW = 0
FAMILY_NAMES = {FAMILY_DRAW: "draw"}


def cache_path() -> Path:
    env = os.environ.get("FTL_TUNE_CACHE")
    if env:
        return Path(env)
    return Path.home() / ".cache" / "fast_tensor_leverage_gb300" / "tune.json"


def cache_key(gpu: str, family: int, R: int, prec: int) -> str:
    return f"{gpu}|{FAMILY_NAMES.get(family, family)}|R={R}|prec={prec}"


def load_cache(path: Path | None = None) -> dict:
    path = cache_path() if path is None else Path(path)
    try:
        d = json.loads(path.read_text())
        return d if isinstance(d, dict) else {}
    except (OSError, ValueError):
        return {}


def save_cache(entries: dict, path: Path | None = None) -> None:
    """Merge `entries` into the cache file (written atomically)."""
    path = cache_path() if path is None else Path(path)
    d = load_cache(path)
    d.update(entries)
    path.parent.mkdir(parents=True, exist_ok=True)
    fd, tmp = tempfile.mkstemp(dir=str(path.parent), prefix=".tune", suffix=".json")
    with os.fdopen(fd, "w") as f:
        json.dump(d, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def variants(family: int, R: int, prec: int) -> tuple[int, int]:
    """(number of variants, default variant) of a kernel family for R, prec."""
    n, dflt = ctypes.c_int(), ctypes.c_int()
    _lib.call("ftl_tune_variants", family, R, prec, ctypes.byref(n), ctypes.byref(dflt))
    return n.value, dflt.value


def set_variant(family: int, R: int, prec: int, variant: int) -> None:
    _lib.call("ftl_tune_set", family, R, prec, int(variant))


def get_variant(family: int, R: int, prec: int) -> int:
    v = ctypes.c_int()
    _lib.call("ftl_tune_get", family, R, prec, ctypes.byref(v))
    return v.value


def choose(timings: dict[int, float], default: int) -> int:
    """Fastest variant; within 1% of the default's time the default wins
    (timing noise should not flip the choice)."""
    best = min(timings, key=timings.get)
    if default in timings and timings[default] <= 1.01 * timings[best]:
        return default
    return best


def gpu_name(device=None) -> str:
    import torch
    return torch.cuda.get_device_name(device)


def apply_cached(R: int, prec: int, family: int = FAMILY_DRAW, device=None, path=None):
    """Select the cached variant for (this GPU, family, R, prec), if any;
    returns it, or None when the cache has no entry."""
    entry = load_cache(path).get(cache_key(gpu_name(device), family, R, prec))
    if not entry:
        return None
    n, _ = variants(family, R, prec)
    v = int(entry.get("variant", -1))
    if not 0 <= v < n:
        return None
    set_variant(family, R, prec, v)
    return v


def tune_draw(sampler, j=None, reps: int = 10, warmup: int = 3, store: bool = True, path=None) -> dict:
    """Time every FP32 draw variant on `sampler` (draws excluding mode j,
    default none), select the fastest on the sampler's device and, with
    `store`, record it in the cache.  Returns {"variant": v, "ms": {v: ms}}."""
    import torch
    prec = sampler._prec
    R = sampler.R
    n, dflt = variants(FAMILY_DRAW, R, prec)
    jj = sampler.N + 1 if j is None else int(j)
    if n <= 1:
        return {"variant": dflt, "ms": {}}
    timings = {}
    saved_ctr = sampler.counter
    for v in range(n):
        set_variant(FAMILY_DRAW, R, prec, v)
        for _ in range(warmup):
            sampler.draw(jj)
        torch.cuda.synchronize(sampler.device)
        sampler.descent_events = []
        for _ in range(reps):
            sampler.draw(jj)
        torch.cuda.synchronize(sampler.device)
        timings[v] = statistics.median(a.elapsed_time(b) for a, b in sampler.descent_events)
        sampler.descent_events = None
    sampler.counter = saved_ctr  # tuning draws do not consume the caller's stream
    best = choose(timings, dflt)
    set_variant(FAMILY_DRAW, R, prec, best)
    if store:
        save_cache({cache_key(gpu_name(sampler.device), FAMILY_DRAW, R, prec):
                    {"variant": best, "ms": {str(k): t for k, t in timings.items()},
                     "workload": {"N": sampler.N, "dims": sampler.dims, "J": sampler.J}}}, path)
    return {"variant": best, "ms": timings}
