"""Serving loop with continuous batching for exact KRP sampling and CP-ALS
requests on one GPU.

Requests of uneven N, I, R and J arrive over time.  The engine:
  * admits them in arrival order as HBM budget and request slots free up
    (first fit: a request that does not fit yet does not block smaller ones
    behind it for more than `max_bypass` admissions);
  * keeps each admitted request's factors, partition trees and workspaces
    resident on the device until it completes, and gives it its own CUDA
    stream, so admitted requests overlap on the device;
  * packs the descents of concurrent sampling requests that share rank and
    precision into ONE launch (ftl_krp_sample_packed, up to FTL_MAX_PACK
    requests), after each request's computeM on its own stream;
  * runs CP-ALS requests sweep by sweep, each sweep replaying a captured CUDA
    graph after the first (eager) sweep;
  * records arrival, admission and completion times; latency = completion -
    arrival.

Sampling results are identical to a standalone Sampler.draw with the same
seed (the packed launch runs the same per-sample code); CP-ALS results equal
a standalone run up to the order of floating-point atomic additions in the
MTTKRP.
"""
from __future__ import annotations

import ctypes
import time
from collections import deque
from dataclasses import dataclass, field

import numpy as np
import torch

from . import _device as D
from . import _lib
from .als import ALS
from .sampler import Sampler
from .tensors import LowRankTensor, SparseTensor


@dataclass
class SampleRequest:
    """Draw J samples from the KRP of `factors` (list of float64 (I_k, R)
    arrays or CUDA tensors), excluding mode j (j >= N: none)."""
    factors: list
    J: int
    j: int = 1 << 30
    precision: str = "fp32"
    seed: int = 0


@dataclass
class ALSRequest:
    """`sweeps` sweeps of randomized CP-ALS on a sparse tensor (idx (nnz, N)
    uint32 or int32 CUDA tensor, vals, dims), rank R, J samples per update,
    factors from PyLowRank-style Gaussian init with `seed`."""
    idx: object
    vals: object
    dims: list
    R: int
    J: int
    sweeps: int = 5
    precision: str = "fp32"
    seed: int = 0
    sampler_seed: int = 1


@dataclass
class Handle:
    rid: int
    request: object
    arrival: float
    admitted: float = None
    done: float = None
    result: dict = None
    bytes: int = 0
    # runtime state
    _stream: object = None
    _obj: object = None
    _event: object = None
    _sweeps_done: int = 0
    _stage: str = "pending"
    _bypassed: int = 0

    @property
    def latency(self) -> float | None:
        return None if self.done is None else self.done - self.arrival


def estimate_bytes(req) -> int:
    """Device bytes a request holds while admitted (factors, trees,
    workspaces, outputs; ALS also the sorted nonzeros)."""
    if isinstance(req, SampleRequest):
        R, N, J = int(req.factors[0].shape[1]), len(req.factors), int(req.J)
        prec = _lib.PREC[req.precision]
        total = 0
        for f in req.factors:
            I = int(f.shape[0])
            total += I * R * 8 + _lib.tree_bytes(I, min(R, I), R, prec)
        e, m, l, p = _lib.plan_sizes(N, R, prec)
        return total + e + m + l + p + N * J * 8 + J * R * 8 + J * 8 + (1 << 20)
    if isinstance(req, ALSRequest):
        N, R, J = len(req.dims), int(req.R), int(req.J)
        nnz = int(req.idx.shape[0])
        prec = _lib.PREC[req.precision]
        total = nnz * (4 * N + 8) + N * nnz * (8 + 4 + 8) * 2
        for I in req.dims:
            total += 2 * I * R * 8 + _lib.tree_bytes(I, min(R, I), R, prec)
        e, m, l, p = _lib.plan_sizes(N, R, prec)
        return total + e + m + l + p + max(req.dims) * R * 8 + J * (N * 8 + R * 8 + 64) + (4 << 20)
    raise TypeError(f"unknown request type {type(req).__name__}")


class ServingEngine:
    def __init__(self, hbm_budget_bytes: int, max_active: int = 32, device=None, pack: bool = True,
                 max_bypass: int = 8, graph_als: bool = True):
        self.device = D.cuda_device(device)
        self.budget = int(hbm_budget_bytes)
        self.max_active = int(max_active)
        self.pack = pack
        self.max_bypass = max_bypass
        self.graph_als = graph_als
        self.pending: deque[Handle] = deque()
        self.active: list[Handle] = []
        self.finished: list[Handle] = []
        self.in_use = 0
        self._next = 0
        self._pack_stream = torch.cuda.Stream(self.device)
        self._streams = [torch.cuda.Stream(self.device) for _ in range(self.max_active)]
        self.t0 = time.perf_counter()
        self.packed_launches = 0
        self.max_in_use = 0

    def now(self) -> float:
        return time.perf_counter() - self.t0

    # ---------------------------------------------------------------- API
    def submit(self, request, arrival: float | None = None) -> Handle:
        h = Handle(self._next, request, self.now() if arrival is None else arrival)
        h.bytes = estimate_bytes(request)
        if h.bytes > self.budget:
            raise ValueError(f"request {h.rid} needs {h.bytes} bytes, more than the whole budget {self.budget}")
        self._next += 1
        self.pending.append(h)
        return h

    def idle(self) -> bool:
        return not self.pending and not self.active

    def tick(self) -> None:
        self._retire()
        self._admit()
        self._issue()

    def run(self, arrivals=None, poll_sleep: float = 0.0) -> list[Handle]:
        """Drive the loop.  `arrivals`: iterable of (time_s, request) sorted by
        time; each is submitted when the engine clock reaches its time."""
        todo = deque(arrivals or [])
        while todo or not self.idle():
            t = self.now()
            while todo and todo[0][0] <= t:
                at, req = todo.popleft()
                self.submit(req, arrival=at)
            self.tick()
            if poll_sleep:
                time.sleep(poll_sleep)
        return self.finished

    # ----------------------------------------------------------- internals
    def _admit(self) -> None:
        sizes = [h.bytes for h in self.pending]
        bypassed = [h._bypassed for h in self.pending]
        take = admission_order(sizes, bypassed, self.in_use, self.budget,
                               self.max_active - len(self.active), self.max_bypass)
        if not take:
            return
        chosen = set(take)
        pend = list(self.pending)
        for k, h in enumerate(pend):
            if k not in chosen:
                h._bypassed += sum(1 for i in take if i > k)
        for i in take:
            self._start(pend[i])
        self.pending = deque(h for k, h in enumerate(pend) if k not in chosen)
        self.max_in_use = max(self.max_in_use, self.in_use)

    def _start(self, h: Handle) -> None:
        h.admitted = self.now()
        self.in_use += h.bytes
        # streams come from a fixed pool, so the caching allocator can reuse
        # the blocks of finished requests
        if not self._streams:
            self._streams.append(torch.cuda.Stream(self.device))
        h._stream = self._streams.pop()
        req = h.request
        with torch.cuda.stream(h._stream):
            if isinstance(req, SampleRequest):
                h._obj = Sampler(req.factors, req.J, int(req.factors[0].shape[1]), "efficient",
                                 precision=req.precision, seed=req.seed, device=self.device)
                h._stage = "ready"
            else:
                sp = SparseTensor(req.idx, req.vals, "sort", dims=req.dims, device=self.device)
                rng = np.random.default_rng(req.seed)
                U = [rng.normal(size=(i, req.R)) for i in req.dims]
                lr = LowRankTensor(req.R, U, device=self.device, sync_host=False)
                lr.renormalize_columns(-1)
                als = ALS(lr, sp)
                als.initialize_ds_als(req.J, "efficient", precision=req.precision, seed=req.sampler_seed)
                h._obj = (sp, lr, als)
                h._stage = "als"
        self.active.append(h)

    def _issue(self) -> None:
        ready = [h for h in self.active if h._stage == "ready"]
        if ready:
            self._issue_sampling(ready)
        for h in self.active:
            if h._stage == "als":
                self._issue_als_sweep(h)

    def _issue_sampling(self, ready: list[Handle]) -> None:
        groups: dict[tuple, list[Handle]] = {}
        for h in ready:
            s: Sampler = h._obj
            groups.setdefault((s.R, s.precision), []).append(h)
        for (R, prec), hs in groups.items():
            for i in range(0, len(hs), 16 if self.pack else 1):
                chunk = hs[i:i + (16 if self.pack else 1)]
                ev = []
                for h in chunk:
                    s: Sampler = h._obj
                    j = h.request.j
                    _lib.call("ftl_krp_compute_m", ctypes.byref(s._plan), j, int(h._stream.cuda_stream))
                    e = torch.cuda.Event()
                    e.record(h._stream)
                    ev.append(e)
                ps = self._pack_stream
                for e in ev:
                    ps.wait_event(e)
                n = len(chunk)
                plans = (ctypes.POINTER(_lib.KRPPlan) * n)(*[ctypes.pointer(h._obj._plan) for h in chunk])
                js = (ctypes.c_uint32 * n)(*[min(h.request.j, 1 << 31) for h in chunk])
                smp = (ctypes.c_void_p * n)(*[h._obj.samples_dev.data_ptr() for h in chunk])
                hh = (ctypes.c_void_p * n)(*[h._obj.h_dev.data_ptr() for h in chunk])
                ww = (ctypes.c_void_p * n)(*[h._obj.weights_dev.data_ptr() for h in chunk])
                seeds = (ctypes.c_uint64 * n)(*[h._obj.seed for h in chunk])
                ctrs = (ctypes.c_uint64 * n)(*[h._obj.counter for h in chunk])
                _lib.call("ftl_krp_sample_packed", plans, n, js, smp, hh, ww, None, seeds, ctrs,
                          int(ps.cuda_stream))
                self.packed_launches += 1
                done = torch.cuda.Event()
                done.record(ps)
                for h in chunk:
                    h._obj.counter += 2 * h._obj.N * h._obj.J
                    h._event = done
                    h._stage = "running"

    def _issue_als_sweep(self, h: Handle) -> None:
        sp, lr, als = h._obj
        req: ALSRequest = h.request
        if h._event is not None and not h._event.query():
            return  # previous sweep still on the device
        with torch.cuda.stream(h._stream):
            if h._sweeps_done == 0 or not self.graph_als:
                for j in range(lr.N):
                    als.execute_ds_als_update(j, True, True)
                if self.graph_als and req.sweeps > 1:
                    als.capture_sweep()
            else:
                als.replay_sweep()
            h._sweeps_done += 1
            e = torch.cuda.Event()
            e.record(h._stream)
            h._event = e
        if h._sweeps_done >= req.sweeps:
            h._stage = "running"

    def _retire(self) -> None:
        keep = []
        for h in self.active:
            if h._stage == "running" and h._event is not None and h._event.query():
                self._finish(h)
            else:
                keep.append(h)
        self.active = keep

    def _finish(self, h: Handle) -> None:
        if isinstance(h.request, SampleRequest):
            s: Sampler = h._obj
            h.result = {"samples": s.samples_dev.cpu().numpy().view(np.uint64),
                        "h": s.h_dev.cpu().numpy(), "weights": s.weights_dev.cpu().numpy()}
        else:
            sp, lr, als = h._obj
            resid = sp.compute_residual_normsq(lr.sigma_dev, lr.U_dev)
            h.result = {"U": [u.cpu().numpy() for u in lr.U_dev], "sigma": lr.sigma,
                        "fit": 1.0 - np.sqrt(max(resid, 0.0) / sp.get_normsq())}
        h.done = self.now()
        h._obj = None
        self._streams.append(h._stream)
        h._stream = None
        h._event = None
        self.in_use -= h.bytes
        self.finished.append(h)


def admission_order(sizes, bypassed, in_use: int, budget: int, free_slots: int, max_bypass: int) -> list[int]:
    """Indices (into the pending queue, oldest first) to admit now: walk the
    queue, take every request that fits in the remaining budget while slots
    remain; a request that does not fit is skipped unless it has already
    been bypassed max_bypass times, in which case nothing behind it is
    admitted (so large requests cannot starve)."""
    take, used = [], in_use
    for i, (b, nb) in enumerate(zip(sizes, bypassed)):
        if len(take) >= free_slots:
            break
        if used + b <= budget:
            take.append(i)
            used += b
        elif nb >= max_bypass:
            break
    return take


def latency_stats(handles) -> dict:
    lat = np.array([h.latency for h in handles if h.latency is not None])
    if lat.size == 0:
        return {}
    return {"p50_ms": float(np.percentile(lat, 50) * 1e3), "p99_ms": float(np.percentile(lat, 99) * 1e3),
            "mean_ms": float(lat.mean() * 1e3), "count": int(lat.size)}
