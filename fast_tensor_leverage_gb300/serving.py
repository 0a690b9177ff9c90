"""Serving loop with continuous batching for exact KRP sampling and CP-ALS
requests on one GPU.

Requests of uneven N, I, R and J arrive over time.  The engine:
  * admits them in arrival order as HBM budget and request slots free up
    (first fit: a request that does not fit yet does not block smaller ones
    behind it for more than `max_bypass` admissions);
  * keeps each admitted request's factors, partition trees and workspaces
    resident on the device until it completes; admission work (factor and
    tree construction, computeM, sparse sorting) runs on one set-up stream,
    so freed memory is reused by later requests;
  * packs the descents of concurrent sampling requests that share rank and
    precision into ONE launch (ftl_krp_sample_packed, up to FTL_MAX_PACK
    requests) on a draw stream, after their set-up;
  * gives each CP-ALS request its own stream for its sweeps, so requests
    overlap on the device;
  * copies results to pinned host memory on the stream that made them, so
    completion needs no host synchronisation;
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
class GaussianFactors:
    """Factor matrices made on the device when the request is admitted:
    float64 tensors of N(0, 1) entries (drawn in FP32), dims[k] x R, from
    torch's CUDA generator seeded with `seed` (so a request gives the same
    factors alone or in a mix)."""
    dims: list
    R: int
    seed: int = 0

    def materialize(self, device) -> list:
        # normals drawn in FP32 and widened: float64 tensors of N(0, 1) values
        # at a fraction of the cost of FP64 transcendentals on this GPU
        g = torch.Generator(device=device)
        g.manual_seed(int(self.seed))
        return [torch.randn((int(I), int(self.R)), dtype=torch.float32, device=device, generator=g).double()
                for I in self.dims]


@dataclass
class SyntheticSparse:
    """A sparse tensor made on the device when the request is admitted:
    synthetic.sparse_powerlaw_tensor(dims, nnz, s, seed)."""
    dims: list
    nnz: int
    s: float = 1.1
    seed: int = 0

    def materialize(self, device):
        from .synthetic import sparse_powerlaw_tensor
        return sparse_powerlaw_tensor(self.dims, int(self.nnz), self.s, seed=int(self.seed), device=device)


@dataclass
class SampleRequest:
    """Draw J samples from the KRP of `factors` (list of float64 (I_k, R)
    arrays or CUDA tensors, or a GaussianFactors spec), excluding mode j
    (j >= N: none)."""
    factors: object
    J: int
    j: int = 1 << 30
    precision: str = "fp32"
    seed: int = 0
    budget_s: float = 0.0   # > 0: device-time budget of its draw (FTL_E_TIMEOUT past it)


@dataclass
class ALSRequest:
    """`sweeps` sweeps of randomized CP-ALS on a sparse tensor (idx (nnz, N)
    uint32 or int32 CUDA tensor, vals, dims; or idx a SyntheticSparse spec
    and vals None), rank R, J samples per update; the initial factors are
    GaussianFactors(dims, R, seed), made on the device, with unit columns."""
    idx: object
    vals: object
    dims: list
    R: int
    J: int
    sweeps: int = 5
    precision: str = "fp32"
    seed: int = 0
    sampler_seed: int = 1
    return_factors: bool = True   # False: the result holds sigma and the fit only


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
    _host: list = None
    status: str = "ok"            # "ok", "cancelled" or "timeout" once done
    _cancel: object = None        # pinned host flag the packed draw reads while it runs
    _slot: int = 0                # index of the request in its packed launch

    def cancel(self) -> None:
        """Cancel the request: a pending one is dropped at the next tick, a
        running draw stops at its next check of the flag (its status becomes
        "cancelled"), a CP-ALS request issues no further sweep."""
        if self._cancel is not None:
            self._cancel[0] = 1
        self.status = "cancelled" if self.done is None else self.status

    @property
    def latency(self) -> float | None:
        return None if self.done is None else self.done - self.arrival


def estimate_bytes(req) -> int:
    """Device bytes a request holds while admitted (factors, trees,
    workspaces, outputs; ALS also the sorted nonzeros)."""
    if isinstance(req, SampleRequest):
        dims, R = _factor_shapes(req.factors)
        N, J = len(dims), int(req.J)
        prec = _lib.PREC[req.precision]
        total = 0
        for I in dims:   # FP64 factor (+ FP32 copy in FP32 mode) and tree
            total += I * R * (8 if prec == 0 else 12) + _lib.tree_bytes(I, min(R, I), R, prec)
        e, m, l, p = _lib.plan_sizes(N, R, prec)
        return total + e + m + l + p + N * J * 8 + J * R * 8 + J * 8 + (1 << 20)
    if isinstance(req, ALSRequest):
        N, R, J = len(req.dims), int(req.R), int(req.J)
        prec = _lib.PREC[req.precision]
        if isinstance(req.idx, SyntheticSparse):
            nnz = int(req.idx.nnz)
            # generation transients: oversampled int64 columns, sort permutations
            gen = int(nnz * 1.35) * (8 * N + 8 * 3 + 1)
        else:
            nnz, gen = int(req.idx.shape[0]), 0
        total = max(gen, nnz * (4 * N + 8)) + N * nnz * (8 + 4 + 8) * 2
        for I in req.dims:
            total += 2 * I * R * 8 + _lib.tree_bytes(I, min(R, I), R, prec)
        e, m, l, p = _lib.plan_sizes(N, R, prec)
        return total + e + m + l + p + max(req.dims) * R * 8 + J * (N * 8 + R * 8 + 64) + (4 << 20)
    raise TypeError(f"unknown request type {type(req).__name__}")


def _factor_shapes(factors) -> tuple[list, int]:
    if isinstance(factors, GaussianFactors):
        return [int(I) for I in factors.dims], int(factors.R)
    return [int(f.shape[0]) for f in factors], int(factors[0].shape[1])


# bytes of ftl_pack_status: the start time (8) and FTL_MAX_PACK statuses (4 each)
_PACK_STATUS_BYTES = 8 + 4 * 16


class ServingEngine:
    def __init__(self, hbm_budget_bytes: int, max_active: int = 32, device=None, pack: bool = True,
                 max_bypass: int = 8, graph_als: bool = True, reserve: bool = False):
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
        # Admission work (factors, trees, computeM, sparse sorting, ALS
        # buffers) runs on one stream: torch's caching allocator keys free
        # blocks by the allocating stream, so memory freed by finished
        # requests is reused by the next ones instead of stranding in
        # per-stream caches.
        self._setup_stream = torch.cuda.Stream(self.device)
        self._streams = [torch.cuda.Stream(self.device) for _ in range(self.max_active)]
        if reserve:
            # Map the whole budget once: later requests split cached blocks
            # instead of asking the CUDA driver (cudaMalloc) for memory while other requests
            # run (large device allocations can synchronise the device).
            with torch.cuda.stream(self._setup_stream):
                block = torch.empty(self.budget, dtype=torch.uint8, device=self.device)
                del block
        self.t0 = time.perf_counter()
        self.packed_launches = 0
        self.max_in_use = 0
        self.host_s = {"admit": 0.0, "issue": 0.0, "retire": 0.0}
        self.start_s: list[float] = []   # host seconds spent admitting each request
        self.start_log: list[tuple] = []  # (seconds, kind, N, R, max I, bytes) per admission

    def now(self) -> float:
        return time.perf_counter() - self.t0

    # ---------------------------------------------------------------- API
    def submit(self, request, arrival: float | None = None) -> Handle:
        h = Handle(self._next, request, self.now() if arrival is None else arrival)
        h.bytes = estimate_bytes(request)
        if h.bytes > self.budget:
            raise ValueError(f"request {h.rid} needs {h.bytes} bytes, more than the whole budget {self.budget}")
        self._next += 1
        h._cancel = torch.zeros(1, dtype=torch.int32, pin_memory=True)
        self.pending.append(h)
        return h

    def idle(self) -> bool:
        return not self.pending and not self.active

    def tick(self) -> None:
        t0 = time.perf_counter()
        self._retire()
        t1 = time.perf_counter()
        self._admit()
        t2 = time.perf_counter()
        self._issue()
        t3 = time.perf_counter()
        hs = self.host_s
        hs["retire"] += t1 - t0
        hs["admit"] += t2 - t1
        hs["issue"] += t3 - t2

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
        # cancelled before admission: done without device work
        for h in [h for h in self.pending if h.status == "cancelled"]:
            self.pending.remove(h)
            h.done = self.now()
            h.result = {"status": "cancelled"}
            self.finished.append(h)
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
        t_start = time.perf_counter()
        h.admitted = self.now()
        self.in_use += h.bytes
        req = h.request
        st = self._setup_stream
        with torch.cuda.stream(st):
            if isinstance(req, SampleRequest):
                factors = req.factors
                if isinstance(factors, GaussianFactors):
                    factors = factors.materialize(self.device)
                s = Sampler(factors, req.J, _factor_shapes(factors)[1], "efficient",
                            precision=req.precision, seed=req.seed, device=self.device, overlap_computem=False)
                _lib.call("ftl_krp_compute_m", ctypes.byref(s._plan), min(req.j, 1 << 31), int(st.cuda_stream))
                h._obj = s
                h._event = torch.cuda.Event()
                h._event.record(st)
                h._stage = "ready"
            else:
                idx, vals = req.idx, req.vals
                if isinstance(idx, SyntheticSparse):
                    idx, vals = idx.materialize(self.device)
                sp = SparseTensor(idx, vals, "sort", dims=req.dims, device=self.device)
                U = GaussianFactors(req.dims, req.R, seed=req.seed).materialize(self.device)
                lr = LowRankTensor(req.R, U, device=self.device, sync_host=False)
                lr.renormalize_columns(-1)
                als = ALS(lr, sp)
                als.initialize_ds_als(req.J, "efficient", precision=req.precision, seed=req.sampler_seed)
                h._obj = (sp, lr, als)
                h._stage = "als"
        if h._stage == "als":
            # sweeps run on the request's own stream, after its set-up
            if not self._streams:
                self._streams.append(torch.cuda.Stream(self.device))
            h._stream = self._streams.pop()
            h._stream.wait_stream(st)
        self.active.append(h)
        dt = time.perf_counter() - t_start
        self.start_s.append(dt)
        if isinstance(req, SampleRequest):
            dims, R = _factor_shapes(req.factors)
        else:
            dims, R = req.dims, req.R
        self.start_log.append((dt, "sample" if isinstance(req, SampleRequest) else "als", len(dims), R,
                               max(dims), h.bytes))

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
                ps = self._pack_stream
                for h in chunk:
                    ps.wait_event(h._event)   # set-up and computeM done
                n = len(chunk)
                plans = (ctypes.POINTER(_lib.KRPPlan) * n)(*[ctypes.pointer(h._obj._plan) for h in chunk])
                js = (ctypes.c_uint32 * n)(*[min(h.request.j, 1 << 31) for h in chunk])
                smp = (ctypes.c_void_p * n)(*[h._obj.samples_dev.data_ptr() for h in chunk])
                hh = (ctypes.c_void_p * n)(*[h._obj.h_dev.data_ptr() for h in chunk])
                ww = (ctypes.c_void_p * n)(*[h._obj.weights_dev.data_ptr() for h in chunk])
                seeds = (ctypes.c_uint64 * n)(*[h._obj.seed for h in chunk])
                ctrs = (ctypes.c_uint64 * n)(*[h._obj.counter for h in chunk])
                # serving controls: every request's cancel flag, and the
                # launch's time budget = the tightest request budget
                cancel = (ctypes.c_void_p * n)(*[h._cancel.data_ptr() for h in chunk])
                budgets = [h.request.budget_s for h in chunk if h.request.budget_s > 0]
                budget_ns = int(min(budgets) * 1e9) if budgets else 0
                with torch.cuda.stream(ps):
                    status = torch.empty(_PACK_STATUS_BYTES, dtype=torch.uint8, device=self.device)
                _lib.call("ftl_krp_sample_packed_ctl", plans, n, js, smp, hh, ww, None, seeds, ctrs,
                          cancel, budget_ns, status.data_ptr(), int(ps.cuda_stream))
                self.packed_launches += 1
                # results to pinned host buffers on the same stream: completion
                # needs no host synchronisation
                with torch.cuda.stream(ps):
                    st_host = torch.empty(_PACK_STATUS_BYTES, dtype=torch.uint8, pin_memory=True)
                    st_host.copy_(status, non_blocking=True)
                    for k, h in enumerate(chunk):
                        s: Sampler = h._obj
                        srcs = (s.samples_dev, s.h_dev, s.weights_dev)
                        h._host = [torch.empty(t.shape, dtype=t.dtype, pin_memory=True) for t in srcs]
                        for dst, src in zip(h._host, srcs):
                            dst.copy_(src, non_blocking=True)
                        h._host.append(st_host)
                        h._slot = k
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
        if h._cancel is not None and int(h._cancel[0]) != 0:
            # cancelled: no further sweep; retire once the last one is done
            h.status = "cancelled"
            h._host = None
            h._stage = "running"
            if h._event is None:
                h._event = torch.cuda.Event()
                h._event.record(h._stream)
            return
        with torch.cuda.stream(h._stream):
            if h._sweeps_done == 0 or not self.graph_als:
                for j in range(lr.N):
                    als.execute_ds_als_update(j, True, True)
                if self.graph_als and req.sweeps > 1:
                    als.capture_sweep()
            else:
                als.replay_sweep()
            h._sweeps_done += 1
            if h._sweeps_done >= req.sweeps:
                # the fit terms and the result copies follow the last sweep on
                # this stream
                terms = sp.residual_terms_async(lr.sigma_dev, lr.U_dev)
                srcs = [terms, lr.sigma_dev, sp._normsq_dev]
                if req.return_factors:
                    srcs += list(lr.U_dev)
                h._host = [torch.empty(t.shape, dtype=t.dtype, pin_memory=True) for t in srcs]
                for dst, src in zip(h._host, srcs):
                    dst.copy_(src, non_blocking=True)
                h._stage = "running"
            e = torch.cuda.Event()
            e.record(h._stream)
            h._event = e

    def _retire(self) -> None:
        keep = []
        for h in self.active:
            if h._stage == "running" and h._event is not None and h._event.query():
                self._finish(h)
            else:
                keep.append(h)
        self.active = keep

    def _finish(self, h: Handle) -> None:
        # h._event covers the result copies: the pinned buffers are complete
        if h._host is None:
            h.result = {"status": h.status}
        elif isinstance(h.request, SampleRequest):
            samples, hh, w, st = h._host
            code = int(st.numpy()[8:].view(np.uint32)[h._slot])
            h.status = {0: "ok", _lib.FTL_E_CANCELLED: "cancelled", _lib.FTL_E_TIMEOUT: "timeout"}.get(code, "error")
            if h.status == "ok":
                h.result = {"samples": samples.numpy().view(np.uint64), "h": hh.numpy(), "weights": w.numpy(),
                            "status": "ok"}
            else:
                h.result = {"status": h.status}  # the draw stopped early: no results
        else:
            terms, sigma, normsq = (t.numpy() for t in h._host[:3])
            resid = float(terms[0] + terms[1])
            h.status = "ok"  # every sweep ran (a cancel after the last one came too late)
            h.result = {"sigma": sigma, "fit": 1.0 - np.sqrt(max(resid, 0.0) / float(normsq[0])), "status": "ok"}
            if h.request.return_factors:
                h.result["U"] = [t.numpy() for t in h._host[3:]]
        h._host = None
        h.done = self.now()
        h._obj = None
        if h._stream is not None:
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
    """Latency percentiles (completion - arrival), split into the wait for
    admission (admitted - arrival) and the service time (completion -
    admitted)."""
    hs = [h for h in handles if h.latency is not None]
    if not hs:
        return {}
    lat = np.array([h.latency for h in hs])
    wait = np.array([h.admitted - h.arrival for h in hs])
    serv = np.array([h.done - h.admitted for h in hs])
    pc = lambda a, q: float(np.percentile(a, q) * 1e3)
    return {"p50_ms": pc(lat, 50), "p99_ms": pc(lat, 99), "mean_ms": float(lat.mean() * 1e3), "count": len(hs),
            "wait_p50_ms": pc(wait, 50), "wait_p99_ms": pc(wait, 99),
            "service_p50_ms": pc(serv, 50), "service_p99_ms": pc(serv, 99)}


def als_dims_cap(N: int, key_bits: int = 62) -> int:
    """Largest mode size for which every mode's fiber keys (mixed-radix over
    the other N - 1 modes) stay below 2^key_bits when all modes share it."""
    return int(2 ** (key_bits / (N - 1)))


def poisson_request_stream(seed: int, rate: float, duration: float, als_fraction: float = 0.2,
                           precision: str = "fp32", ranks=(8, 16, 32, 64, 128),
                           I_range=(1e4, 1e7), J_log2_range=(10, 17), nnz_range=(1e5, 3e6),
                           als_sweeps: int = 5) -> list:
    """A seeded mixed request stream: arrivals of a Poisson process with mean
    `rate` per second over `duration` seconds; each request is CP-ALS with
    probability `als_fraction`, else sampling.  N uniform in {3..6}, every
    mode size log-uniform in I_range, R uniform over `ranks`, J log-uniform
    in 2^J_log2_range, float64 N(0, 1) factors made on the device.  Sampling
    requests exclude a mode j uniform in {0..N} (N: none excluded).  CP-ALS
    requests run `als_sweeps` sweeps on a Zipf(1.1) sparse tensor with nnz
    log-uniform in nnz_range; their mode sizes are capped at als_dims_cap(N)
    (lower bound min(I_range[0], cap / 4)) so fiber keys fit 62 bits, and
    they return sigma and the fit (not the factors).
    Returns [(arrival_s, request), ...] sorted by arrival."""
    rng = np.random.default_rng(seed)
    out, t = [], 0.0
    lo, hi = np.log10(I_range[0]), np.log10(I_range[1])
    while True:
        t += float(rng.exponential(1.0 / rate))
        if t >= duration:
            break
        N = int(rng.integers(3, 7))
        R = int(ranks[int(rng.integers(0, len(ranks)))])
        J = int(round(2.0 ** rng.uniform(*J_log2_range)))
        s = int(rng.integers(0, 1 << 62))
        if rng.random() < als_fraction:
            cap = als_dims_cap(N)
            a_hi = min(hi, np.log10(cap))
            a_lo = min(lo, a_hi - np.log10(4.0))
            dims = [int(round(10 ** rng.uniform(a_lo, a_hi))) for _ in range(N)]
            nnz = int(round(10 ** rng.uniform(np.log10(nnz_range[0]), np.log10(nnz_range[1]))))
            req = ALSRequest(SyntheticSparse(dims, nnz, 1.1, seed=s), None, dims, R, J, sweeps=als_sweeps,
                             precision=precision, seed=s + 1, sampler_seed=s + 2, return_factors=False)
        else:
            dims = [int(round(10 ** rng.uniform(lo, hi))) for _ in range(N)]
            req = SampleRequest(GaussianFactors(dims, R, seed=s), J, j=int(rng.integers(0, N + 1)),
                                precision=precision, seed=s + 1)
        out.append((t, req))
    return out
