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
                 seed: int | None = None, device=None, factor_shadows: bool = True):
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
        tdt = torch.float64 if precision == "fp64" else torch.float32
        dev = self.device
        self.U = [f.to(dev, torch.float64).contiguous() if isinstance(f, torch.Tensor)
                  else torch.from_numpy(f).to(dev) for f in factors]
        # FP32 mode: FP32 copies of the factors for the leaf scans (half the
        # leaf-block bytes, same results); refreshed with each tree
        self.U32 = ([torch.empty((n, R), dtype=torch.float32, device=dev) for n in self.dims]
                    if precision == "fp32" and factor_shadows else None)
        self.trees = []
        for k in range(N):
            nb = _lib.tree_bytes(self.dims[k], self.F[k], R, self._prec)
            self.trees.append(torch.empty(nb // tdt.itemsize, dtype=tdt, device=dev))
        eig_b, M_b, lam_b, p32_b = _lib.plan_sizes(N, R, self._prec)
        self.eig_G = torch.empty(eig_b // tdt.itemsize, dtype=tdt, device=dev)
        self.M = torch.zeros(M_b // 8, dtype=torch.float64, device=dev)
        self.lam = torch.zeros(lam_b // 8, dtype=torch.float64, device=dev)
        self.pinv32 = torch.zeros(p32_b // 4, dtype=torch.float32, device=dev)
        self.samples_dev = torch.zeros((N, J), dtype=torch.int64, device=dev)
        self.h_dev = torch.empty((J, R), dtype=torch.float64, device=dev)
        self.weights_dev = torch.empty(J, dtype=torch.float64, device=dev)
        self.seed = int(seed) if seed is not None else secrets.randbits(63)
        self.counter = 0
        self._stage = D.PinnedStage()
        self._plan = _lib.KRPPlan()
        self._refresh_plan()
        for k in range(N):
            self.update_sampler(k)

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
        p = self._plan
        p.N, p.R, p.J, p.prec = self.N, self.R, self.J, self._prec
        for k in range(self.N):
            p.dims[k] = self.dims[k]
            p.U[k] = self.U[k].data_ptr()
            p.U32[k] = self.U32[k].data_ptr() if self.U32 is not None else None
            p.gram_G[k] = self.trees[k].data_ptr()
        p.eig_G = self.eig_G.data_ptr()
        p.M = self.M.data_ptr()
        p.lambda_ = self.lam.data_ptr()
        p.pinv32 = self.pinv32.data_ptr()

    def _stream(self, stream=None) -> int:
        return D.stream_ptr(self.device, stream)

    # ------------------------------------------------------------ updates
    def update_sampler(self, j: int, stream=None) -> None:
        """Rebuild the Gram tree of factor j from its device copy
        (EfficientKRPSampler::update_sampler, efficient_krp_sampler.hpp:73-75)."""
        _lib.call("ftl_tree_build", self.U[j].data_ptr(), self.dims[j], self.R, self.F[j],
                  self._prec, self.trees[j].data_ptr(), self._stream(stream))
        if self.U32 is not None:
            _lib.call("ftl_factor_shadow", self.U[j].data_ptr(), self.dims[j] * self.R, self.U32[j].data_ptr(),
                      self._stream(stream))

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
        tensor) replaces the in-kernel Philox stream."""
        j = int(j)
        if j < 0:
            raise ValueError(f"j={j} must be non-negative")
        d_ptr = None
        if draws is not None:
            n = 2 * self.N * self.J
            if isinstance(draws, torch.Tensor):
                dt = draws.to(self.device, torch.float64).reshape(-1).contiguous()
            else:
                dt = torch.from_numpy(np.ascontiguousarray(np.asarray(draws, dtype=np.float64)).reshape(-1))
                dt = dt.to(self.device, non_blocking=False)
            if dt.numel() != n:
                raise ValueError(f"draws must hold 2*N*J = {n} uniforms, got {dt.numel()}")
            self._draws_keep = dt
            d_ptr = dt.data_ptr()
        _lib.call("ftl_krp_draw", ctypes.byref(self._plan), j, self.samples_dev.data_ptr(),
                  self.h_dev.data_ptr(), self.weights_dev.data_ptr(), d_ptr, self.seed,
                  self.counter, self._stream(stream))
        if d_ptr is None:
            self.counter += 2 * self.N * self.J
        return self.samples_dev, self.h_dev, self.weights_dev

    def _rows(self, j: int):
        return [k for k in range(self.N) if k != j]

    def KRPDrawSamples(self, j: int, samples, draws=None) -> None:
        """Draw J samples from the KRP of all factors except j into
        samples (N x J uint64, row j untouched when j < N), in place."""
        N, J = self.N, self.J
        s_out = D.require_numpy_out(samples, np.uint64, "samples", min_size=N * J)
        self.draw(j, draws)
        stage = self._stage.get((N, J), torch.int64)
        stage.copy_(self.samples_dev, non_blocking=True)
        torch.cuda.current_stream(self.device).synchronize()
        flat = s_out.reshape(-1)[: N * J].reshape(N, J)
        host = stage.numpy().view(np.uint64)
        for k in self._rows(j):
            flat[k] = host[k]

    def KRPDrawSamples_materialize(self, j: int, samples, h_out, weights_out, draws=None) -> None:
        """KRPDrawSamples plus copies of the sampled KRP rows h (J x R) and the
        importance weights (J) (als_module.cpp:70-81)."""
        N, J, R = self.N, self.J, self.R
        s_out = D.require_numpy_out(samples, np.uint64, "samples", min_size=N * J)
        h_np = D.require_numpy_out(h_out, np.float64, "h_out", min_size=J * R)
        w_np = D.require_numpy_out(weights_out, np.float64, "weights_out", min_size=J)
        self.draw(j, draws)
        s_st = self._stage.get((N, J), torch.int64)
        h_st = self._stage.get((J, R), torch.float64)
        w_st = self._stage.get((J,), torch.float64)
        s_st.copy_(self.samples_dev, non_blocking=True)
        h_st.copy_(self.h_dev, non_blocking=True)
        w_st.copy_(self.weights_dev, non_blocking=True)
        torch.cuda.current_stream(self.device).synchronize()
        flat = s_out.reshape(-1)[: N * J].reshape(N, J)
        host = s_st.numpy().view(np.uint64)
        for k in self._rows(j):
            flat[k] = host[k]
        h_np.reshape(-1)[: J * R] = h_st.numpy().reshape(-1)
        w_np.reshape(-1)[:J] = w_st.numpy()

    # ------------------------------------------------------- inspection
    @property
    def h(self) -> np.ndarray:
        return self.h_dev.cpu().numpy()

    @property
    def weights(self) -> np.ndarray:
        return self.weights_dev.cpu().numpy()

    def _stride(self) -> int:
        w = 16 // (8 if self.precision == "fp64" else 4)
        return (self.P + w - 1) // w * w

    def gram_tree(self, k: int) -> np.ndarray:
        """Node Grams of factor k's tree, (node_count, P) packed, as FP64."""
        S = self._stride()
        return self.trees[k].double().cpu().numpy().reshape(-1, S)[:, : self.P].copy()

    def eigen_tree(self, k: int) -> np.ndarray:
        S = self._stride()
        e = self.eig_G.double().cpu().numpy().reshape(self.N, 2 * self.R - 1, S)
        return e[k, :, : self.P].copy()

    def workspace_M(self) -> np.ndarray:
        return self.M.cpu().numpy().reshape(-1, self.R, self.R)
