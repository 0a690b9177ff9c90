"""Sampler: drop-in for the reference's exact KRP leverage sampler,
`Sampler(matrices, J, R, "efficient")` with KRPDrawSamples and
KRPDrawSamples_materialize (cpp_ext/als_module.cpp:30-82 over
cpp_ext/efficient_krp_sampler.hpp).

Factors and partition trees live on the GPU for the sampler's lifetime; a
draw is one computeM launch pair plus one fused descent launch
(ftl_krp_draw).  The numpy entry points copy the results back into the
caller's arrays; `draw()` returns device tensors without a host round trip.
"""
from __future__ import annotations

import ctypes
import secrets

import numpy as np
import torch

from . import _device as D
from . import _lib


class Sampler:
    def __init__(self, U, J: int, R: int, type: str = "efficient", *, precision: str = "fp64",
                 seed: int | None = None, device=None, factor_shadows: bool = True,
                 overlap_computem: bool = True, autotune="cached"):
        if type != "efficient":
            raise ValueError(
                f"Unsupported argument {type!r} passed for sampler construction "
                "(only the exact 'efficient' sampler is implemented)")
        if precision not in _lib.PREC:
            raise ValueError(f"precision must be one of {sorted(_lib.PREC)}, got {precision!r}")
        U = list(U)
        N, J, R = len(U), int(J), int(R)
        if not (1 <= N <= _lib.MAX_MODES):
            raise ValueError(f"need 1..{_lib.MAX_MODES} factor matrices, got {N}")
        if not (1 <= R <= _lib.MAX_RANK):
            raise ValueError(f"R={R} outside [1, {_lib.MAX_RANK}]")
        if J < 1:
            raise ValueError(f"J={J} must be positive")
        factors = [self._factor_input(u, R, f"matrices[{k}]") for k, u in enumerate(U)]
        self.N, self.J, self.R = N, J, R
        self.precision = precision
        self._prec = _lib.PREC[precision]
        self.device = D.cuda_device(device)
        self.dims = [int(f.shape[0]) for f in factors]
        self.F = [min(R, n) for n in self.dims]
        self.P = R * (R + 1) // 2
        self._plan_prec = _lib.storage_prec(self._prec)   # what the draws see
        tdt = torch.float64 if precision == "fp64" else torch.float32
        dev = self.device
        self.U = [f.to(dev, torch.float64).contiguous() if isinstance(f, torch.Tensor)
                  else torch.from_numpy(f).to(dev) for f in factors]
        # FP32 mode: FP32 copies of the factors for the leaf scans (half the
        # leaf-block bytes, same results); refreshed with each tree
        self.U32 = ([torch.empty((n, R), dtype=torch.float32, device=dev) for n in self.dims]
                    if precision != "fp64" and factor_shadows else None)
        self.trees = []
        for k in range(N):
            nb = _lib.tree_bytes(self.dims[k], self.F[k], R, self._prec)
            self.trees.append(torch.empty(nb // tdt.itemsize, dtype=tdt, device=dev))
        eig_b, M_b, lam_b, p32_b = _lib.plan_sizes(N, R, self._prec)
        # Per-draw workspaces (eigen trees, computeM matrices).  With
        # overlap_computem there are two sets: computeM of the next draw runs
        # on a side stream into the other set while the current descent runs
        # (computeM is a few single-CTA kernels that would otherwise leave the
        # GPU idle between descents).  Every draw still does all its work.
        self._ws_sets = []
        for _ in range(2 if overlap_computem else 1):
            self._ws_sets.append((torch.empty(eig_b // tdt.itemsize, dtype=tdt, device=dev),
                                  torch.zeros(M_b // 8, dtype=torch.float64, device=dev),
                                  torch.zeros(lam_b // 8, dtype=torch.float64, device=dev),
                                  torch.zeros(p32_b // 4, dtype=torch.float32, device=dev)))
        self.eig_G, self.M, self.lam, self.pinv32 = self._ws_sets[0]
        self.samples_dev = torch.zeros((N, J), dtype=torch.int64, device=dev)
        self.h_dev = torch.empty((J, R), dtype=torch.float64, device=dev)
        self.weights_dev = torch.empty(J, dtype=torch.float64, device=dev)
        self.seed = int(seed) if seed is not None else secrets.randbits(63)
        self.counter = 0
        self._overlap = overlap_computem
        self._plans = [_lib.KRPPlan() for _ in self._ws_sets]
        self._plan = self._plans[0]        # the plan of the last draw
        self._next_set = 0
        if overlap_computem:
            # high priority: the computeM CTAs are dispatched ahead of the
            # queued blocks of the running descent as soon as an SM frees up
            self._cm_stream = torch.cuda.Stream(dev, priority=-1)
            self._cm_done = [torch.cuda.Event() for _ in self._ws_sets]
            self._set_free = [None] * len(self._ws_sets)
        # (set, j) of a computeM launched ahead for the next draw: after two
        # draws with the same j, the next draw's computeM (same trees, same
        # j: the same result) is launched right behind the current descent,
        # so callers that wait for every draw (copies to the host) still get
        # it overlapped.  Each draw still runs exactly one computeM.
        self._spec = None
        self._last_j = None
        self._tree_ev = torch.cuda.Event()
        # optional list: each draw appends a (start, end) pair of timing
        # events recorded on the launching stream around its descent launch
        self.descent_events = None
        self._refresh_plan()
        for k in range(N):
            self.update_sampler(k)
        # kernel variants: "cached" applies the autotuner's recorded choice
        # for this GPU (if any); True also times the variants when there is
        # none; False leaves the current selection
        self.tuning = None
        if autotune:
            from . import autotune as AT
            v = AT.apply_cached(R, self._prec, device=self.device)
            if v is None and autotune is True:
                self.tuning = AT.tune_draw(self)
            else:
                self.tuning = {"variant": v, "cached": v is not None}

    @staticmethod
    def _factor_input(u, R: int, name: str):
        # CUDA tensors stay on the device; everything else becomes float64 numpy
        if isinstance(u, torch.Tensor) and u.is_cuda:
            if u.dim() != 2 or u.shape[1] != R or u.shape[0] < 1:
                raise ValueError(f"{name} must be (I, {R}), got {tuple(u.shape)}")
            return u
        return D.as_factor(u, R, name)

    # ----------------------------------------------------------- plumbing
    def _refresh_plan(self) -> None:
        for p, (eig, M, lam, p32) in zip(self._plans, self._ws_sets):
            p.N, p.R, p.J, p.prec = self.N, self.R, self.J, self._plan_prec
            for k in range(self.N):
                p.dims[k] = self.dims[k]
                p.U[k] = self.U[k].data_ptr()
                p.U32[k] = self.U32[k].data_ptr() if self.U32 is not None else None
                p.gram_G[k] = self.trees[k].data_ptr()
            p.eig_G = eig.data_ptr()
            p.M = M.data_ptr()
            p.lambda_ = lam.data_ptr()
            p.pinv32 = p32.data_ptr()

    def _stream(self, stream=None) -> int:
        return D.stream_ptr(self.device, stream)

    # ------------------------------------------------------------ updates
    def update_sampler(self, j: int, stream=None) -> None:
        """Rebuild the Gram tree of factor j from its device copy
        (EfficientKRPSampler::update_sampler, efficient_krp_sampler.hpp:73-75)."""
        if getattr(self, "_spec", None) is not None:
            # a computeM launched ahead reads the trees: let it finish, then
            # drop it (its result belongs to the old trees)
            main = stream if stream is not None else torch.cuda.current_stream(self.device)
            main.wait_event(self._cm_done[self._spec[0]])
            self._spec = None
        # the tree and (FP32 trees with copies) the FP32 copy of the factor
        # for the leaf scans, in one pass over the factor
        _lib.call("ftl_tree_build_ex", self.U[j].data_ptr(), self.dims[j], self.R, self.F[j],
                  self._prec, self.trees[j].data_ptr(),
                  self.U32[j].data_ptr() if self.U32 is not None else None, self._stream(stream))
        # computeM on the side stream must see this tree
        self._tree_ev.record(stream if stream is not None else torch.cuda.current_stream(self.device))

    def set_factor(self, j: int, U, stream=None) -> None:
        """Replace factor j (same shape) and rebuild its tree."""
        if isinstance(U, torch.Tensor) and U.is_cuda:
            self.U[j].copy_(U.reshape(self.dims[j], self.R))
        else:
            f = D.as_factor(U, self.R, "U")
            if f.shape[0] != self.dims[j]:
                raise ValueError(f"factor {j} has {self.dims[j]} rows, got {f.shape[0]}")
            self.U[j].copy_(torch.from_numpy(f))
        self.update_sampler(j, stream)

    # -------------------------------------------------------------- draws
    def draw(self, j: int, draws=None, *, stream=None):
        """Draw J samples excluding mode j (j >= N: none excluded).  Returns
        device tensors (samples N x J int64 holding the uint64 row indices,
        h J x R, weights J); they are overwritten by the next draw.
        `draws` (2N x J uniforms, the reference's layout; numpy or CUDA
        tensor, or a pinned CPU tensor, copied without blocking) replaces the
        in-kernel Philox stream."""
        j = int(j)
        if j < 0:
            raise ValueError(f"j={j} must be non-negative")
        main = stream if stream is not None else torch.cuda.current_stream(self.device)
        plan = self._plan
        if self._overlap:
            b = self._next_set
            self._next_set = (b + 1) % len(self._plans)
            plan, cm = self._plans[b], self._cm_stream
            if self._spec != (b, j):
                self._launch_computem(b, j)
            self._spec = None
        d_ptr = None
        if draws is not None:
            n = 2 * self.N * self.J
            with torch.cuda.stream(main):
                if isinstance(draws, torch.Tensor):
                    dt = draws.to(self.device, torch.float64, non_blocking=draws.is_pinned()).reshape(-1)
                    dt = dt.contiguous()
                else:
                    dt = torch.from_numpy(np.ascontiguousarray(np.asarray(draws, dtype=np.float64)).reshape(-1))
                    dt = dt.to(self.device, non_blocking=False)
            if dt.numel() != n:
                raise ValueError(f"draws must hold 2*N*J = {n} uniforms, got {dt.numel()}")
            self._draws_keep = dt
            d_ptr = dt.data_ptr()
        if self._overlap:
            main.wait_event(self._cm_done[b])
            ev0 = self._timing_event(main)
            _lib.call("ftl_krp_sample", ctypes.byref(plan), j, self.samples_dev.data_ptr(),
                      self.h_dev.data_ptr(), self.weights_dev.data_ptr(), d_ptr, self.seed,
                      self.counter, int(main.cuda_stream))
            self._timing_event(main, ev0)
            ev = torch.cuda.Event()
            ev.record(main)
            self._set_free[b] = ev
            self._plan = plan
            self.eig_G, self.M, self.lam, self.pinv32 = self._ws_sets[b]
            if self._last_j == j:
                nb = self._next_set
                self._launch_computem(nb, j)
                self._spec = (nb, j)
            self._last_j = j
        else:
            _lib.call("ftl_krp_draw", ctypes.byref(plan), j, self.samples_dev.data_ptr(),
                      self.h_dev.data_ptr(), self.weights_dev.data_ptr(), d_ptr, self.seed,
                      self.counter, int(main.cuda_stream))
        if d_ptr is None:
            self.counter += 2 * self.N * self.J
        return self.samples_dev, self.h_dev, self.weights_dev

    def _timing_event(self, stream, start=None):
        # records a timing event on `stream` when descent_events is a list;
        # with `start`, appends the (start, end) pair
        if self.descent_events is None:
            return None
        ev = torch.cuda.Event(enable_timing=True)
        ev.record(stream)
        if start is not None:
            self.descent_events.append((start, ev))
        return ev

    def _launch_computem(self, b: int, j: int) -> None:
        # computeM into workspace set b after the trees it reads and after the
        # descent that last read set b (it does not need the uniforms, so it
        # is launched before they are copied); the descent waits for _cm_done[b]
        cm = self._cm_stream
        cm.wait_event(self._tree_ev)
        if self._set_free[b] is not None:
            cm.wait_event(self._set_free[b])
        _lib.call("ftl_krp_compute_m", ctypes.byref(self._plans[b]), j, int(cm.cuda_stream))
        self._cm_done[b].record(cm)

    def _rows(self, j: int):
        return [k for k in range(self.N) if k != j]

    def _copy_rows_out(self, j: int, s_out) -> bool:
        # straight from the device into the caller's array (one copy; rows of
        # excluded modes are left as they are, as in the reference); returns
        # whether a copy is still in flight (page-locked destination)
        N, J = self.N, self.J
        flat = s_out.reshape(-1)[: N * J].reshape(N, J).view(np.int64)
        if j >= N:
            return D.copy_to_numpy(flat, self.samples_dev)
        pending = False
        for k in self._rows(j):
            pending |= D.copy_to_numpy(flat[k], self.samples_dev[k])
        return pending

    def KRPDrawSamples(self, j: int, samples, draws=None) -> None:
        """Draw J samples from the KRP of all factors except j into
        samples (N x J uint64, row j untouched when j < N), in place."""
        s_out = D.require_numpy_out(samples, np.uint64, "samples", min_size=self.N * self.J)
        self.draw(j, draws)
        if self._copy_rows_out(int(j), s_out):
            torch.cuda.current_stream(self.device).synchronize()

    def KRPDrawSamples_materialize(self, j: int, samples, h_out, weights_out, draws=None) -> None:
        """KRPDrawSamples plus copies of the sampled KRP rows h (J x R) and the
        importance weights (J) (als_module.cpp:70-81)."""
        N, J, R = self.N, self.J, self.R
        s_out = D.require_numpy_out(samples, np.uint64, "samples", min_size=N * J)
        h_np = D.require_numpy_out(h_out, np.float64, "h_out", min_size=J * R)
        w_np = D.require_numpy_out(weights_out, np.float64, "weights_out", min_size=J)
        self.draw(j, draws)
        # results straight into the caller's arrays: DMA copies once the
        # arrays are page-locked (registered on first use, released when they
        # are garbage collected), then one wait for all of them
        pending = self._copy_rows_out(int(j), s_out)
        pending |= D.copy_to_numpy(h_np.reshape(-1)[: J * R], self.h_dev.reshape(-1))
        pending |= D.copy_to_numpy(w_np.reshape(-1)[:J], self.weights_dev)
        if pending:
            torch.cuda.current_stream(self.device).synchronize()

    # ------------------------------------------------------- inspection
    @property
    def h(self) -> np.ndarray:
        return self.h_dev.cpu().numpy()

    @property
    def weights(self) -> np.ndarray:
        return self.weights_dev.cpu().numpy()

    def gram_tree(self, k: int) -> np.ndarray:
        """Node Grams of factor k's tree, (node_count, P) packed upper
        triangles (whatever the device layout), as FP64."""
        _, S, pos = _lib.node_layout(self.R, self._plan_prec)
        return self.trees[k].double().cpu().numpy().reshape(-1, S)[:, pos].copy()

    def eigen_tree(self, k: int) -> np.ndarray:
        _, S, pos = _lib.node_layout(self.R, self._plan_prec)
        e = self.eig_G.double().cpu().numpy().reshape(self.N, 2 * self.R - 1, S)
        return e[k][:, pos].copy()

    def workspace_M(self) -> np.ndarray:
        # the (2N+3) R x R slots; the status word and packed pseudo-inverse follow
        RR = self.R * self.R
        return self.M.cpu().numpy()[: (2 * self.N + 3) * RR].reshape(-1, self.R, self.R)
