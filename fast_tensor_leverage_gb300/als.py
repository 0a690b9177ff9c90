"""Randomized CP-ALS (STS-CP): drop-in for the reference's ALS class
(cpp_ext/als.hpp:18-271, bound in cpp_ext/als_module.cpp:111-115) and its
Python driver (als.py:59-107, tensors.py:16-53), on the GPU.

One sampled update of mode j (execute_ds_als_update, als.hpp:57-220):
  draw J samples excluding j -> fiber keys of the samples (modes != j,
  uint32-cast) -> dedup with multiplicities -> FP64 Gram of the
  sqrt(w * count)-scaled sampled KRP rows -> FP64 pseudo-inverse (rank cap
  min(unique, R), eigenvalue cut 1e-11) -> sparse MTTKRP of the
  (w * count)-scaled rows (one balanced pass over the nonzeros sorted by
  output row, probing the dedup hash table for each nonzero's fiber) ->
  U_j = MTTKRP
  pinv -> column renormalisation -> rebuild of mode j's partition tree.
Every step is a kernel of libftl_gb300; the only host synchronisation is the
optional mirror of the updated factor into the caller's numpy array.
"""
from __future__ import annotations

import ctypes
import time

import numpy as np
import torch

from . import _device as D
from . import _lib
from .sampler import Sampler
from .tensors import DenseTensor, LowRankTensor, SparseTensor, _ptrs, _Workspace, factor_gram


class ALS:
    def __init__(self, cp_decomp: LowRankTensor, ground_truth: SparseTensor):
        if not isinstance(cp_decomp, LowRankTensor):
            raise TypeError("cp_decomp must be a fast_tensor_leverage_gb300.LowRankTensor")
        if not isinstance(ground_truth, (SparseTensor, LowRankTensor, DenseTensor)):
            raise TypeError("ground_truth must be a SparseTensor, LowRankTensor or DenseTensor "
                            "of fast_tensor_leverage_gb300")
        if ground_truth is cp_decomp:
            raise ValueError("the decomposition cannot be its own ground truth")
        if ground_truth.N != cp_decomp.N:
            raise ValueError("tensor and decomposition disagree on the number of modes")
        for k in range(cp_decomp.N):
            if ground_truth.dims[k] > cp_decomp.dims[k]:
                raise ValueError(f"mode {k}: tensor index range {ground_truth.dims[k]} exceeds factor rows "
                                 f"{cp_decomp.dims[k]}")
        self.cp_decomp = cp_decomp
        self.ground_truth = ground_truth
        self.device = cp_decomp.device
        self.sampler: Sampler | None = None
        self.J = None
        self._eager_done = False
        self._ws = _Workspace(self.device)
        self.last_update = {}

    def initialize_ds_als(self, J: int, sampler_type: str = "efficient", *, precision: str = "fp64",
                          seed: int | None = None) -> None:
        """Create the sampler over the decomposition's factors
        (als.hpp:39-55).  Only the exact 'efficient' sampler exists here."""
        if sampler_type != "efficient":
            raise ValueError(f"sampler type {sampler_type!r} is not implemented (only 'efficient')")
        lr = self.cp_decomp
        self.J = int(J)
        # the sampler shares the factors' device storage, so solves written
        # into lr.U_dev[j] are what update_sampler(j) rebuilds from
        # no FP32 factor copies: every update rebuilds one tree, and a copy pass
        # over a (mostly zero) factor would cost more than the leaf scans save
        self.sampler = Sampler(lr.U_dev, self.J, lr.R, "efficient", precision=precision, seed=seed,
                               device=self.device, factor_shadows=False, overlap_computem=False)
        assert all(a.data_ptr() == b.data_ptr() for a, b in zip(self.sampler.U, lr.U_dev))
        dev, R, J = self.device, lr.R, self.J
        self._keys = torch.empty(J, dtype=torch.int64, device=dev)
        self._ukeys = torch.empty(J, dtype=torch.int64, device=dev)
        self._urep = torch.empty(J, dtype=torch.int32, device=dev)
        self._ucnt = torch.empty(J, dtype=torch.int32, device=dev)
        self._nuniq = torch.zeros(1, dtype=torch.int64, device=dev)
        self._gram = torch.empty((R, R), dtype=torch.float64, device=dev)
        self._pinv = torch.empty((R, R), dtype=torch.float64, device=dev)
        self._vscr = torch.empty((R, R), dtype=torch.float64, device=dev)
        self._hp = torch.empty((J, R), dtype=torch.float64, device=dev)   # sampled rows times pinv
        self._dims_c = (ctypes.c_int64 * lr.N)(*lr.dims)
        # every buffer an update uses is sized here, so updates (and captured
        # sweeps) allocate nothing
        self._ws.get("dedup", _lib.ws_bytes("dedup", J))
        if isinstance(self.ground_truth, SparseTensor):
            self._ws.get("mttkrp_rows", _lib.ws_bytes("mttkrp_rows", J, R))
        if isinstance(self.ground_truth, LowRankTensor):
            self.ground_truth._ws.get("lowrank_mttkrp", _lib.ws_bytes("lowrank_mttkrp", self.ground_truth.R, R))
        self._ws.get("gram", _lib.ws_bytes("gram", R))
        lr._ws.get("colnorm", _lib.ws_bytes("colnorm", R))
        if getattr(lr, "_norms", None) is None:
            lr._norms = torch.empty((lr.N, R), dtype=torch.float64, device=dev)
        self._ctr_dev = torch.zeros(1, dtype=torch.int64, device=dev)
        self._gdraws = torch.empty(2 * lr.N * J, dtype=torch.float64, device=dev)

    # ------------------------------------------------------------------ updates
    def execute_ds_als_update(self, j: int, renormalize: bool = True, update_sampler: bool = True,
                              draws=None) -> None:
        if self.sampler is None:
            raise RuntimeError("initialize_ds_als must be called first")
        lr, gt = self.cp_decomp, self.ground_truth
        N, R, J = lr.N, lr.R, self.J
        j = int(j)
        st = D.stream_ptr(self.device)
        self._eager_done = True
        samples, h, w = self.sampler.draw(j, draws)
        # fiber keys of the samples on modes != j (samples are N x J)
        _lib.call("ftl_fiber_keys", samples.data_ptr(), 1, J, 1, J, N, self._dims_c, j, self._keys.data_ptr(), st)
        nb = _lib.ws_bytes("dedup", J)
        _lib.call("ftl_dedup", self._keys.data_ptr(), J, self._ws.get("dedup", nb).data_ptr(), nb,
                  self._ukeys.data_ptr(), self._urep.data_ptr(), self._ucnt.data_ptr(), self._nuniq.data_ptr(), st)
        gb = _lib.ws_bytes("gram", R)
        _lib.call("ftl_weighted_gram", h.data_ptr(), self._urep.data_ptr(), w.data_ptr(), self._ucnt.data_ptr(),
                  self._nuniq.data_ptr(), J, R, self._ws.get("gram", gb).data_ptr(), gb, self._gram.data_ptr(), st)
        _lib.call("ftl_pinv_square", self._gram.data_ptr(), R, R, self._nuniq.data_ptr(), 1e-11,
                  self._pinv.data_ptr(), self._vscr.data_ptr(), st)
        I_j = lr.dims[j]
        # U_j = MTTKRP pinv (als.hpp:189-203) with MTTKRP = sum_z coef_z e_row(z)
        # h_rep(z)^T, i.e. U_j = sum_z coef_z e_row(z) (h_rep(z)^T pinv): the J
        # sampled rows are multiplied by pinv first (J x R^2 FP64 instead of
        # I_j x R^2) and the MTTKRP accumulates straight into U_j.
        hp = self._hp
        _lib.call("ftl_solve_rows", h.data_ptr(), self._pinv.data_ptr(), J, R, hp.data_ptr(), st)
        out = lr.U_dev[j]
        if not isinstance(gt, SparseTensor):
            # black-box right-hand side (black_box_tensor.hpp:21-67): low-rank
            # shortcut or dense fiber gather, rows past gt.dims[j] zeroed
            gt._sampled_mttkrp_dev(samples.data_ptr(), J, self._urep.data_ptr(), self._ucnt.data_ptr(),
                                   self._nuniq.data_ptr(), w.data_ptr(), hp.data_ptr(), R, j, out.data_ptr(), I_j, st)
        elif I_j == gt.dims[j]:
            # one balanced pass over the nonzeros sorted by output row
            rrows, rkeys, rvals = gt.rows[j]
            mb = _lib.ws_bytes("mttkrp_rows", J, R)
            _lib.call("ftl_sparse_mttkrp_rows", rrows.data_ptr(), rkeys.data_ptr(), rvals.data_ptr(), gt.nnz,
                      self._ukeys.data_ptr(), self._urep.data_ptr(), self._ucnt.data_ptr(), self._nuniq.data_ptr(),
                      J, J, w.data_ptr(), hp.data_ptr(), R, self._ws.get("mttkrp_rows", mb).data_ptr(), mb,
                      out.data_ptr(), I_j, st)
        else:
            skeys, idxj, vj = gt.lookups[j]
            _lib.call("ftl_sparse_mttkrp", skeys.data_ptr(), idxj.data_ptr(), vj.data_ptr(), gt.nnz,
                      self._ukeys.data_ptr(), self._urep.data_ptr(), w.data_ptr(), self._ucnt.data_ptr(),
                      self._nuniq.data_ptr(), J, hp.data_ptr(), R, out.data_ptr(), I_j, st)
        if renormalize:
            lr.renormalize_columns(j)          # mirrors to the host array when lr.sync_host
        elif lr.sync_host:
            lr.sync_host_copies(j)
        if update_sampler:
            self.sampler.update_sampler(j)

    def execute_exact_als_update(self, j: int, renormalize: bool = True, update_sampler: bool = True) -> None:
        """Exact least-squares update of mode j (als.hpp:222-270): Gram
        Hadamard chain of the other factors, its pseudo-inverse, the exact
        MTTKRP over all nonzeros, the solve and renormalisation.  Like the
        reference, the sampler's tree of mode j is not rebuilt here."""
        lr, gt = self.cp_decomp, self.ground_truth
        N, R = lr.N, lr.R
        j = int(j)
        st = D.stream_ptr(self.device)
        G = [factor_gram(u, self._ws, st) for u in lr.U_dev]
        gram = torch.empty((R, R), dtype=torch.float64, device=self.device)
        _lib.call("ftl_gram_hadamard", _ptrs(G), N, R, j, None, None, gram.data_ptr(), None, st)
        pinv = torch.empty((R, R), dtype=torch.float64, device=self.device)
        vscr = torch.empty((R, R), dtype=torch.float64, device=self.device)
        _lib.call("ftl_pinv_square", gram.data_ptr(), R, R, None, 1e-11, pinv.data_ptr(), vscr.data_ptr(), st)
        I_j = lr.dims[j]
        mt = torch.empty((I_j, R), dtype=torch.float64, device=self.device)
        if isinstance(gt, DenseTensor):
            # the reference's DenseTensor has no exact MTTKRP (tensor.hpp:21-23 leaves it empty)
            raise NotImplementedError("exact ALS updates against a DenseTensor are not supported")
        gt._exact_mttkrp_dev(lr.U_dev, j, mt.data_ptr(), I_j, st)
        _lib.call("ftl_solve_rows", mt.data_ptr(), pinv.data_ptr(), I_j, R, lr.U_dev[j].data_ptr(), st)
        if renormalize:
            lr.renormalize_columns(j)
        elif lr.sync_host:
            lr.sync_host_copies(j)

    def num_unique_samples(self) -> int:
        return int(self._nuniq.item())

    # ------------------------------------------------------- captured sweeps
    def capture_sweep(self, renormalize: bool = True, update_sampler: bool = True) -> None:
        """Capture one sweep (a sampled update of every mode) as a CUDA
        graph.  Its uniforms come from the Philox stream of the sampler's seed
        at a device-resident counter that the graph advances, so every replay
        draws fresh samples -- the same uniforms the eager updates would use
        from the current counter on.  The decomposition must keep its factors
        on the device (sync_host=False)."""
        if self.sampler is None:
            raise RuntimeError("initialize_ds_als must be called first")
        lr = self.cp_decomp
        if lr.sync_host:
            raise RuntimeError("graph capture needs LowRankTensor(..., sync_host=False)")
        N, J = lr.N, self.J
        dev = self.device
        cur = torch.cuda.current_stream(dev)
        # no host round trip: the counter is filled on the device
        self._ctr_dev.fill_(self.sampler.counter)

        def sweep():
            st = D.stream_ptr(dev)
            for j in range(N):
                _lib.call("ftl_philox_uniforms_dev", self._gdraws.data_ptr(), 2 * N * J, self.sampler.seed,
                          self._ctr_dev.data_ptr(), st)
                self.execute_ds_als_update(j, renormalize, update_sampler, draws=self._gdraws)

        # Capture on a side stream with the graph API directly: nothing runs
        # while capturing, so no warm-up or device-wide synchronisation is
        # needed (torch.cuda.graph's context manager would synchronise the
        # whole device and empty the allocator cache, stalling every other
        # stream).  Workspaces and kernel attributes were settled by eager
        # updates, which must precede the capture.
        if not self._eager_done:
            raise RuntimeError("run one eager sampled update before capture_sweep")
        self._graph = torch.cuda.CUDAGraph()
        cap = torch.cuda.Stream(dev)
        cap.wait_stream(cur)
        with torch.cuda.stream(cap):
            self._graph.capture_begin()
            try:
                sweep()
            finally:
                self._graph.capture_end()
        cur.wait_stream(cap)

    def replay_sweep(self) -> None:
        """Run one captured sweep on the current stream.  The device counter
        is first refilled from the host one (a stream-ordered fill), so eager
        updates made between replays advance the stream the replay draws from
        and no uniforms are reused."""
        self._ctr_dev.fill_(self.sampler.counter)
        self._graph.replay()
        # keep the host copy of the Philox counter in step with the device one
        N, J = self.cp_decomp.N, self.J
        self.sampler.counter += N * 2 * N * J


# ------------------------------------------------------------ Python driver

class PyDenseTensor:
    """The reference's PyDenseTensor (tensors.py:122-130): a dense array as
    an ALS right-hand side (FP32 or FP64, kept in its precision)."""

    def __init__(self, data):
        self.ten = DenseTensor(data, 10000)
        self.N = self.ten.N
        self.dims = list(self.ten.dims)


class PyLowRank:
    """The reference's PyLowRank (tensors.py:16-53): Gaussian factors from
    numpy.random.default_rng(seed), wrapped in a LowRankTensor."""

    def __init__(self, dims, R, allow_rhs_mttkrp=False, init_method="gaussian", seed=None, **kw):
        if init_method != "gaussian":
            raise ValueError("only init_method='gaussian' exists")
        rng = np.random.default_rng(seed)
        self.dims = list(dims)
        self.N = len(self.dims)
        self.R = int(R)
        self.U = [rng.normal(size=(i, R)) for i in self.dims]
        self.ten = LowRankTensor(R, 10000, self.U, **kw) if allow_rhs_mttkrp else LowRankTensor(R, self.U, **kw)

    def set_sigma(self, new_sigma):
        self.ten.set_sigma(new_sigma)

    def compute_diff_resid(self, rhs) -> float:
        normsq = rhs.ten.compute_residual_normsq(self.ten.sigma_dev, self.ten.U_dev)
        return float(np.sqrt(max(normsq, 0.0)))

    def compute_exact_fit(self, rhs) -> float:
        return 1.0 - self.compute_diff_resid(rhs) / np.sqrt(rhs.ten.get_normsq())


class PySparseTensor:
    """In-memory stand-in for the reference's HDF5-backed PySparseTensor
    (tensors.py:85-113): indices (nnz, N) uint32 already shifted to zero,
    values, optional log(1 + x) preprocessing."""

    def __init__(self, idx, vals, lookup="sort", preprocessing=None, dims=None):
        vals = np.asarray(vals, dtype=np.float64)
        if preprocessing == "log_count":
            vals = np.log(vals + 1.0)
        elif preprocessing is not None:
            raise ValueError(f"Unknown preprocessing option {preprocessing!r}")
        self.tensor_idxs = np.ascontiguousarray(idx, dtype=np.uint32)
        self.values = vals
        self.N = self.tensor_idxs.shape[1]
        self.nnz = self.tensor_idxs.shape[0]
        self.dims = list(dims) if dims is not None else [int(v) + 1 for v in self.tensor_idxs.max(axis=0)]
        self.ten = SparseTensor(self.tensor_idxs, self.values, lookup, dims=self.dims)


def als_prod(lhs: PyLowRank, rhs, J: int, method: str, max_iter: int, stop_tolerance: float,
             epoch_length: int = 5, verbose: bool = False, precision: str = "fp64", seed=None) -> dict:
    """The reference's sweep loop (als.py:59-107): per sweep one update per
    mode, the exact fit every `epoch_length` sweeps, and its stopping rule
    (stop once the best of the last three fits is not above the best before
    them by stop_tolerance)."""
    als = ALS(lhs.ten, rhs.ten)
    if method != "exact":
        als.initialize_ds_als(J, method, precision=precision, seed=seed)
    iterations, fits, update_times, fit_times = [0], [lhs.compute_exact_fit(rhs)], [], []
    if verbose:
        print(f"Before ALS:\tFit: {fits[-1]}")
    for i in range(max_iter):
        for j in range(lhs.N):
            torch.cuda.synchronize(lhs.ten.device)
            t0 = time.time()
            if method == "exact":
                als.execute_exact_als_update(j, True, True)
            else:
                als.execute_ds_als_update(j, True, True)
            torch.cuda.synchronize(lhs.ten.device)
            update_times.append(time.time() - t0)
        if (i + 1) % epoch_length == 0:
            t0 = time.time()
            iterations.append(i + 1)
            fits.append(lhs.compute_exact_fit(rhs))
            fit_times.append(time.time() - t0)
            if verbose:
                print(f"Iteration: {i + 1}\tFit: {fits[-1]}")
            if len(fits) > 4 and np.max(fits[-3:]) < np.max(fits[:-3]) + stop_tolerance:
                break
    return {"iterations": iterations, "fits": fits, "update_times": update_times,
            "fit_computation_times": fit_times}
