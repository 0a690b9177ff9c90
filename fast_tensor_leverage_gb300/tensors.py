"""LowRankTensor and SparseTensor: drop-ins for the reference's tensor
classes on the CP-ALS path (cpp_ext/low_rank_tensor.hpp:13-303,
cpp_ext/sparse_tensor.hpp:25-213, bound in cpp_ext/als_module.cpp:85-107),
with factors and nonzeros resident on the GPU."""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _device as D
from . import _lib


def _ptrs(tensors) -> ctypes.Array:
    arr = (ctypes.c_void_p * len(tensors))()
    for k, t in enumerate(tensors):
        arr[k] = t.data_ptr()
    return arr


class _Workspace:
    """Device scratch buffers reused across calls, keyed by name."""

    def __init__(self, device):
        self.device = device
        self._bufs = {}

    def get(self, name: str, nbytes: int) -> torch.Tensor:
        b = self._bufs.get(name)
        if b is None or b.numel() < nbytes:
            b = torch.empty(max(nbytes, 16), dtype=torch.uint8, device=self.device)
            self._bufs[name] = b
        return b


def factor_gram(U_dev: torch.Tensor, ws: _Workspace, stream: int, out: torch.Tensor | None = None) -> torch.Tensor:
    """FP64 U^T U (R x R) on the device."""
    I, R = U_dev.shape
    if out is None:
        out = torch.empty((R, R), dtype=torch.float64, device=U_dev.device)
    gb = _lib.ws_bytes("gram", R)
    w = ws.get("gram", gb)
    _lib.call("ftl_weighted_gram", U_dev.data_ptr(), None, None, None, None, I, R, w.data_ptr(), gb,
              out.data_ptr(), stream)
    return out


class LowRankTensor:
    """CP model sum_r sigma_r u_r^(1) o ... o u_r^(N).

    LowRankTensor(R, U_list) or LowRankTensor(R, max_rhs_rows, U_list), as in
    the reference.  U_list holds float64 (I_k, R) C-contiguous numpy arrays,
    kept by reference; ALS updates are mirrored back into them (set
    `sync_host=False` to keep the factors on the device only and call
    `sync_host_copies()` when the host arrays are needed).  U_list may
    instead hold float64 CUDA tensors (with sync_host=False): the factors
    then live on the device only."""

    def __init__(self, R, *args, device=None, sync_host: bool = True):
        if len(args) == 1:
            U_list, self.max_rhs_rows, self.is_static = args[0], None, False
        elif len(args) == 2:
            self.max_rhs_rows, U_list = int(args[0]), args[1]
            self.is_static = True
        else:
            raise TypeError("LowRankTensor(R, U_list) or LowRankTensor(R, max_rhs_rows, U_list)")
        self.R = int(R)
        U_list = list(U_list)
        self.N = len(U_list)
        if not (1 <= self.N <= _lib.MAX_MODES) or not (1 <= self.R <= _lib.MAX_RANK):
            raise ValueError(f"bad N={self.N} or R={self.R}")
        on_device = all(isinstance(u, torch.Tensor) and u.is_cuda for u in U_list)
        for k, u in enumerate(U_list):
            if not on_device:
                D.require_numpy_out(u, np.float64, f"U[{k}]")
            if u.ndim != 2 or u.shape[1] != self.R:
                raise ValueError(f"U[{k}] must be (I_k, {self.R}), got {tuple(u.shape)}")
        self.dims = [int(u.shape[0]) for u in U_list]
        self.device = D.cuda_device(device)
        if on_device:
            # device-only factors (no host arrays to mirror into)
            if sync_host:
                raise ValueError("CUDA factor tensors need sync_host=False")
            self.U = None
            self.U_dev = [u.to(self.device, torch.float64).contiguous() for u in U_list]
        else:
            self.U = U_list
            self.U_dev = [torch.from_numpy(u).to(self.device) for u in self.U]
        self.sigma_dev = torch.ones(self.R, dtype=torch.float64, device=self.device)
        self.sync_host = sync_host
        self._ws = _Workspace(self.device)
        self._normsq = None
        if self.is_static:
            self._normsq = self._chain_sum_self()
        # additive counter-hash Gaussian noise of the tensor as a right-hand
        # side (set_noise); 0: none
        self.noise_sigma = 0.0
        self.noise_seed = 0
        self._dims_c = (ctypes.c_int64 * self.N)(*self.dims)

    def set_noise(self, sigma: float, seed: int = 0) -> None:
        """Make this tensor, as a right-hand side, X + sigma Z with Z one
        standard normal per entry, a function of the entry's index and
        `seed` (ftl_noise_*: never stored).  Sampled MTTKRPs, evaluated
        entries and materialised fibers include the noise; the norms and
        residuals are their expectations over Z (the cross term with Z has
        mean zero, the noise energy sigma^2 prod(dims) is added)."""
        if sigma < 0:
            raise ValueError("sigma must be >= 0")
        self.noise_sigma = float(sigma)
        self.noise_seed = int(seed)

    def set_noise_snr(self, snr_db: float, seed: int = 0) -> float:
        """set_noise with sigma for a signal-to-noise ratio of `snr_db`:
        sigma^2 prod(dims) = ||[[sigma; U]]||^2 10^(-snr_db / 10).  Returns sigma."""
        sig = float(np.sqrt(self._chain_sum_self() * 10.0 ** (-snr_db / 10.0) / float(np.prod(self.dims, dtype=np.float64))))
        self.set_noise(sig, seed)
        return sig

    def noise_energy(self) -> float:
        """sigma^2 prod(dims): the expected squared norm of the noise."""
        return self.noise_sigma ** 2 * float(np.prod(self.dims, dtype=np.float64))

    # ---------------------------------------------------------- plumbing
    def _stream(self) -> int:
        return D.stream_ptr(self.device)

    def upload(self, k: int | None = None) -> None:
        """Copy host factor(s) to the device (after editing the numpy arrays)."""
        if self.U is None:
            raise RuntimeError("this LowRankTensor has device factors only")
        for i in range(self.N) if k is None else [k]:
            self.U_dev[i].copy_(torch.from_numpy(self.U[i]))

    def sync_host_copies(self, k: int | None = None) -> None:
        if self.U is None:
            raise RuntimeError("this LowRankTensor has device factors only")
        for i in range(self.N) if k is None else [k]:
            self.U[i][...] = self.U_dev[i].cpu().numpy()

    @property
    def sigma(self) -> np.ndarray:
        return self.sigma_dev.cpu().numpy()

    # ------------------------------------------------------------ sigma
    def get_sigma(self, out, j: int = -1) -> None:
        o = D.require_numpy_out(out, np.float64, "sigma_out", min_size=self.R)
        o.reshape(-1)[: self.R] = self.sigma

    def set_sigma(self, sigma_in) -> None:
        s = np.ascontiguousarray(np.asarray(sigma_in, dtype=np.float64).reshape(-1)[: self.R])
        self.sigma_dev.copy_(torch.from_numpy(s))

    # ---------------------------------------------------- perturbation
    def multiply_random_factor_entries(self, rho: float, A: float, seed: int | None = None) -> None:
        """Multiply each factor entry by A with probability rho, independently
        (LowRankTensor::multiply_random_factor_entries,
        low_rank_tensor.hpp:289-303, which draws from an unseeded generator;
        here `seed` makes it reproducible, None draws a fresh one).  Like the
        reference it does not touch a sampler built on these factors: call
        its update_sampler afterwards."""
        import secrets
        if not 0.0 <= float(rho) <= 1.0:
            raise ValueError(f"rho={rho} outside [0, 1]")
        g = torch.Generator(device=self.device)
        g.manual_seed(secrets.randbits(63) if seed is None else int(seed))
        for k in range(self.N):
            hit = torch.rand(self.U_dev[k].shape, generator=g, device=self.device, dtype=torch.float64) < float(rho)
            self.U_dev[k][hit] *= float(A)
        self._normsq = None if not self.is_static else self._chain_sum_self()
        if self.sync_host:
            self.sync_host_copies()

    # ------------------------------------------------------ renormalise
    def renormalize_columns(self, j: int) -> None:
        """Divide the columns of factor j (j = -1: every factor) by their
        norms (norms <= 1e-7 count as 1); sigma <- the norms of factor j, or
        the product over all factors for j = -1
        (low_rank_tensor.hpp:203-260)."""
        st = self._stream()
        nb = _lib.ws_bytes("colnorm", self.R)
        w = self._ws.get("colnorm", nb)
        modes = range(self.N) if j == -1 else [j]
        if getattr(self, "_norms", None) is None:
            self._norms = torch.empty((self.N, self.R), dtype=torch.float64, device=self.device)
        norms = self._norms
        for i in modes:
            _lib.call("ftl_renormalize_columns", self.U_dev[i].data_ptr(), self.dims[i], self.R,
                      norms[i].data_ptr(), w.data_ptr(), nb, 1, st)
        if j == -1:
            self.sigma_dev.copy_(torch.prod(norms, dim=0))
        else:
            self.sigma_dev.copy_(norms[j])
        self._normsq = None if not self.is_static else self._normsq
        if self.sync_host:
            for i in modes:
                self.sync_host_copies(i)

    # ------------------------------------------------------------ norms
    def grams(self) -> list[torch.Tensor]:
        st = self._stream()
        return [factor_gram(u, self._ws, st) for u in self.U_dev]

    def _chain_sum_self(self) -> float:
        G = self.grams()
        out = torch.empty(1, dtype=torch.float64, device=self.device)
        _lib.call("ftl_gram_hadamard", _ptrs(G), self.N, self.R, -1, self.sigma_dev.data_ptr(),
                  self.sigma_dev.data_ptr(), None, out.data_ptr(), self._stream())
        return float(out.item())

    def get_normsq(self) -> float:
        """||model||^2 = sum_rs sigma_r sigma_s prod_k (U_k^T U_k)_rs
        (low_rank_tensor.hpp:70-76), plus the expected noise energy when
        set_noise is in effect."""
        if not self.is_static or self._normsq is None:
            return self._chain_sum_self() + self.noise_energy()
        return self._normsq + self.noise_energy()


# --------------------------------------------------- low-rank as a tensor
# (LowRankTensor as the right-hand side of ALS or a fit; the reference's
# BlackBoxTensor / Tensor interface, cpp_ext/low_rank_tensor.hpp:70-280)

def _lr_other(lr, sigma, U_list, R):
    st = D.stream_ptr(lr.device)
    if isinstance(sigma, torch.Tensor):
        sig = sigma.to(lr.device, torch.float64).contiguous()
    else:
        sig = torch.from_numpy(np.ascontiguousarray(np.asarray(sigma, dtype=np.float64).reshape(-1)[:R])).to(lr.device)
    Ud = []
    for k, u in enumerate(U_list):
        if isinstance(u, torch.Tensor) and u.is_cuda:
            Ud.append(u.to(lr.device, torch.float64).contiguous())
        else:
            Ud.append(torch.from_numpy(D.as_factor(u, R, f"U[{k}]")).to(lr.device))
    return st, sig, Ud


def _chain_sum(ws, st, A, Ra, sa, B, Rb, sb) -> torch.Tensor:
    """sum_rs sa_r sb_s prod_k (A_k^T B_k)_rs on the device (ATB_chain_prod_sum)."""
    dev = A[0].device
    nb = _lib.ws_bytes("cross_gram", Ra, Rb)
    w = ws.get("cross", nb)
    G = []
    for a, b in zip(A, B):
        g = torch.empty((Ra, Rb), dtype=torch.float64, device=dev)
        _lib.call("ftl_cross_gram", a.data_ptr(), Ra, b.data_ptr(), Rb, a.shape[0], w.data_ptr(), nb, g.data_ptr(), st)
        G.append(g)
    out = torch.empty(1, dtype=torch.float64, device=dev)
    _lib.call("ftl_chain_prod", _ptrs(G), len(G), Ra, Rb, -1, sa.data_ptr(), sb.data_ptr(), None, out.data_ptr(), st)
    return out


def _lr_compute_residual_normsq(self, sigma, U_list) -> float:
    """||self - [[sigma; U]]||^2 = ||self||^2 + ||other||^2 - 2 <other, self>
    by Gram chains (LowRankTensor::compute_residual_normsq,
    low_rank_tensor.hpp:78-89), clamped at 0 like the reference."""
    Ro = len(np.asarray(sigma).reshape(-1)) if not isinstance(sigma, torch.Tensor) else int(sigma.numel())
    st, sig, Ud = _lr_other(self, sigma, U_list, Ro)
    t_self = _chain_sum(self._ws, st, self.U_dev, self.R, self.sigma_dev, self.U_dev, self.R, self.sigma_dev)
    t_other = _chain_sum(self._ws, st, Ud, Ro, sig, Ud, Ro, sig)
    t_cross = _chain_sum(self._ws, st, Ud, Ro, sig, self.U_dev, self.R, self.sigma_dev)
    v = torch.cat([t_self, t_other, t_cross]).cpu().numpy()
    # with noise: plus its expected energy (the cross term with Z has mean 0)
    return max(float(v[0] + v[1] - 2.0 * v[2]), 0.0) + self.noise_energy()


def _lr_evaluate_indices(self, indices, result) -> None:
    """result[z] = sum_r sigma_r prod_k U_k[indices[z, k], r]
    (LowRankTensor::evaluate_indices, low_rank_tensor.hpp:262-280)."""
    idx = np.ascontiguousarray(np.asarray(indices, dtype=np.uint32))
    n = idx.shape[0]
    out = D.require_numpy_out(result, np.float64, "result", min_size=n)
    if idx.ndim != 2 or idx.shape[1] != self.N:
        raise ValueError(f"indices must be (n, {self.N})")
    idx_d = torch.from_numpy(idx.view(np.int32)).to(self.device)
    o = torch.empty(n, dtype=torch.float64, device=self.device)
    _lib.call("ftl_lowrank_evaluate", _ptrs(self.U_dev), self.N, self.R, self.sigma_dev.data_ptr(), idx_d.data_ptr(),
              0, n, o.data_ptr(), D.stream_ptr(self.device))
    if self.noise_sigma:
        _lib.call("ftl_noise_add_at", self._dims_c, self.N, self.noise_seed, self.noise_sigma, idx_d.data_ptr(), 0, n,
                  o.data_ptr(), D.stream_ptr(self.device))
    out.reshape(-1)[:n] = o.cpu().numpy()


def _lr_materialize_rhs(self, samples, j: int, rhs_buf) -> None:
    """Fibers at the samples (n x N uint64): j >= N: rhs_buf (n x R) = sigma o
    prod_k U_k[s_k]; else rhs_buf (n x I_j) = that row times U_j^T
    (LowRankTensor::materialize_rhs, low_rank_tensor.hpp:91-135)."""
    S = np.ascontiguousarray(np.asarray(samples, dtype=np.uint64))
    n, j = S.shape[0], int(j)
    cols = self.R if j >= self.N else self.dims[j]
    out = D.require_numpy_out(rhs_buf, np.float64, "rhs_buf", min_size=n * cols)
    S_d = torch.from_numpy(S.view(np.int64)).to(self.device)
    o = torch.empty((n, cols), dtype=torch.float64, device=self.device)
    _lib.call("ftl_lowrank_materialize", _ptrs(self.U_dev), self.N, self.R, self.sigma_dev.data_ptr(), S_d.data_ptr(),
              n, j, self.dims[j] if j < self.N else 0, o.data_ptr(), D.stream_ptr(self.device))
    if self.noise_sigma and j < self.N:
        _lib.call("ftl_noise_add_fibers", self._dims_c, self.N, self.noise_seed, self.noise_sigma, S_d.data_ptr(), n,
                  j, o.data_ptr(), D.stream_ptr(self.device))
    out.reshape(-1)[: n * cols] = o.cpu().numpy().reshape(-1)


def _lr_sampled_mttkrp_dev(self, samples, J, urep, ucnt, nuniq, w, h, R, j, out, out_rows, stream) -> None:
    nb = _lib.ws_bytes("lowrank_mttkrp", self.R, R)
    ws = self._ws.get("lowrank_mttkrp", nb)
    _lib.call("ftl_lowrank_sampled_mttkrp", _ptrs(self.U_dev), self.sigma_dev.data_ptr(), self.N, self.R, j,
              samples, J, urep, ucnt, nuniq, J, w, h, R, ws.data_ptr(), nb, out, self.dims[j], out_rows, stream)
    if self.noise_sigma:
        _lib.call("ftl_noise_sampled_mttkrp", self._dims_c, self.N, j, self.noise_seed, self.noise_sigma, samples, J,
                  urep, ucnt, nuniq, J, w, h, R, out, out_rows, stream)


def _lr_execute_downsampled_mttkrp_py(self, samples, lhs, j: int, result) -> None:
    """result (I_j x R) = sum over the rows s of samples (J x N uint64) of
    fiber_s (x) lhs[s] (BlackBoxTensor::execute_downsampled_mttkrp,
    black_box_tensor.hpp:21-67), through the low-rank shortcut."""
    S = np.ascontiguousarray(np.asarray(samples, dtype=np.uint64))
    L = np.ascontiguousarray(np.asarray(lhs, dtype=np.float64))
    J, R = L.shape
    out = D.require_numpy_out(result, np.float64, "result", min_size=self.dims[j] * R)
    S_d = torch.from_numpy(np.ascontiguousarray(S.T).view(np.int64)).to(self.device)   # N x J
    L_d = torch.from_numpy(L).to(self.device)
    o = torch.empty((self.dims[j], R), dtype=torch.float64, device=self.device)
    _lr_sampled_mttkrp_dev(self, S_d.data_ptr(), J, None, None, None, None, L_d.data_ptr(), R, int(j), o.data_ptr(),
                           self.dims[j], D.stream_ptr(self.device))
    out.reshape(-1)[: self.dims[j] * R] = o.cpu().numpy().reshape(-1)


def _lr_exact_mttkrp_dev(self, U_L, j: int, out, out_rows, stream) -> None:
    """out = U_j (sigma 1^T o prod_{k != j} U_k^T U_L,k)
    (LowRankTensor::execute_exact_mttkrp, low_rank_tensor.hpp:147-180)."""
    R_L = int(U_L[0].shape[1])
    nb = _lib.ws_bytes("cross_gram", self.R, R_L)
    w = self._ws.get("cross", nb)
    G = []
    for k in range(self.N):
        g = torch.empty((self.R, R_L), dtype=torch.float64, device=self.device)
        if k != j:
            _lib.call("ftl_cross_gram", self.U_dev[k].data_ptr(), self.R, U_L[k].data_ptr(), R_L, self.dims[k],
                      w.data_ptr(), nb, g.data_ptr(), stream)
        G.append(g)
    M = torch.empty((self.R, R_L), dtype=torch.float64, device=self.device)
    _lib.call("ftl_chain_prod", _ptrs(G), self.N, self.R, R_L, j, self.sigma_dev.data_ptr(), None, M.data_ptr(),
              None, stream)
    _lib.call("ftl_rows_times", self.U_dev[j].data_ptr(), self.dims[j], self.R, M.data_ptr(), R_L, out, out_rows,
              stream)


LowRankTensor.compute_residual_normsq = _lr_compute_residual_normsq
LowRankTensor.evaluate_indices = _lr_evaluate_indices
LowRankTensor.materialize_rhs = _lr_materialize_rhs
LowRankTensor.execute_downsampled_mttkrp_py = _lr_execute_downsampled_mttkrp_py
LowRankTensor._sampled_mttkrp_dev = _lr_sampled_mttkrp_dev
LowRankTensor._exact_mttkrp_dev = _lr_exact_mttkrp_dev


class DenseTensor:
    """Dense row-major tensor (FP64 or FP32) resident on the device, usable
    as the right-hand side of ALS (DenseTensor<VAL_T>,
    cpp_ext/dense_tensor.hpp:13-59).  `data`: numpy array or CUDA tensor.
    Unlike the reference (whose DenseTensor has no residual), get_normsq and
    compute_residual_normsq are implemented."""

    def __init__(self, data, max_rhs_rows: int = 10000, *, device=None):
        self.device = D.cuda_device(device)
        if isinstance(data, torch.Tensor):
            t = data.to(self.device).contiguous()
        else:
            a = np.asarray(data)
            if a.dtype not in (np.float32, np.float64):
                a = a.astype(np.float64)
            t = torch.from_numpy(np.ascontiguousarray(a)).to(self.device)
        if t.dtype not in (torch.float32, torch.float64):
            t = t.to(torch.float64)
        self.T_dev = t
        self.is_f32 = t.dtype == torch.float32
        self.dims = [int(d) for d in t.shape]
        self.N = len(self.dims)
        self.max_rhs_rows = int(max_rhs_rows)
        self._dims_c = (ctypes.c_int64 * self.N)(*self.dims)
        self._ws = _Workspace(self.device)
        self._normsq = None

    def _terms(self, sigma, U_list, R):
        st = D.stream_ptr(self.device)
        nb = _lib.ws_bytes("dense_residual")
        out = torch.empty(2, dtype=torch.float64, device=self.device)
        if U_list is None:
            _lib.call("ftl_dense_residual_terms", self.T_dev.data_ptr(), int(self.is_f32), self._dims_c, self.N, None,
                      None, 1, self._ws.get("dense", nb).data_ptr(), nb, out.data_ptr(), st)
        else:
            _, sig, Ud = _lr_other(self, sigma, U_list, R)
            _lib.call("ftl_dense_residual_terms", self.T_dev.data_ptr(), int(self.is_f32), self._dims_c, self.N,
                      _ptrs(Ud), sig.data_ptr(), R, self._ws.get("dense", nb).data_ptr(), nb, out.data_ptr(), st)
        return out.cpu().numpy()

    def get_normsq(self) -> float:
        if self._normsq is None:
            self._normsq = float(self._terms(None, None, 1)[1])
        return self._normsq

    def compute_residual_normsq(self, sigma, U_list) -> float:
        R = int(sigma.numel()) if isinstance(sigma, torch.Tensor) else len(np.asarray(sigma).reshape(-1))
        return float(self._terms(sigma, U_list, R)[0])

    def materialize_rhs(self, samples, j: int, rhs_buf) -> None:
        """rhs_buf (n x I_j) = the fibers at the samples (n x N uint64)
        (DenseTensor::materialize_rhs, dense_tensor.hpp:38-59)."""
        S = np.ascontiguousarray(np.asarray(samples, dtype=np.uint64))
        n, j = S.shape[0], int(j)
        out = D.require_numpy_out(rhs_buf, np.float64, "rhs_buf", min_size=n * self.dims[j])
        S_d = torch.from_numpy(S.view(np.int64)).to(self.device)
        o = torch.empty((n, self.dims[j]), dtype=torch.float64, device=self.device)
        _lib.call("ftl_dense_materialize", self.T_dev.data_ptr(), int(self.is_f32), self._dims_c, self.N, j,
                  S_d.data_ptr(), n, o.data_ptr(), D.stream_ptr(self.device))
        out.reshape(-1)[: n * self.dims[j]] = o.cpu().numpy().reshape(-1)

    def _sampled_mttkrp_dev(self, samples, J, urep, ucnt, nuniq, w, h, R, j, out, out_rows, stream) -> None:
        _lib.call("ftl_dense_sampled_mttkrp", self.T_dev.data_ptr(), int(self.is_f32), self._dims_c, self.N, j,
                  samples, J, urep, ucnt, nuniq, J, w, h, R, out, out_rows, stream)

    def execute_downsampled_mttkrp_py(self, samples, lhs, j: int, result) -> None:
        """result (I_j x R) = sum over the rows s of samples (J x N uint64) of
        fiber_s (x) lhs[s] (BlackBoxTensor::execute_downsampled_mttkrp)."""
        S = np.ascontiguousarray(np.asarray(samples, dtype=np.uint64))
        L = np.ascontiguousarray(np.asarray(lhs, dtype=np.float64))
        J, R = L.shape
        out = D.require_numpy_out(result, np.float64, "result", min_size=self.dims[j] * R)
        S_d = torch.from_numpy(np.ascontiguousarray(S.T).view(np.int64)).to(self.device)
        L_d = torch.from_numpy(L).to(self.device)
        o = torch.empty((self.dims[j], R), dtype=torch.float64, device=self.device)
        self._sampled_mttkrp_dev(S_d.data_ptr(), J, None, None, None, None, L_d.data_ptr(), R, int(j), o.data_ptr(),
                                 self.dims[j], D.stream_ptr(self.device))
        out.reshape(-1)[: self.dims[j] * R] = o.cpu().numpy().reshape(-1)


def DenseTensor_double(data, max_rhs_rows: int = 10000):
    """The reference's DenseTensor_double binding (als_module.cpp:99-100)."""
    return DenseTensor(np.asarray(data, dtype=np.float64), max_rhs_rows)


def DenseTensor_float(data, max_rhs_rows: int = 10000):
    """The reference's DenseTensor_float binding (als_module.cpp:101-102)."""
    return DenseTensor(np.asarray(data, dtype=np.float32), max_rhs_rows)



class SparseTensor:
    """COO tensor with one sorted fiber lookup per mode
    (SparseTensor, sparse_tensor.hpp:46-77; SortIdxLookup ctor,
    sort_lookup.hpp:33-60).  idx: (nnz, N) uint32, vals: (nnz,) float64."""

    def __init__(self, idx, vals, method: str = "sort", *, dims=None, device=None):
        if method != "sort":
            raise ValueError(f"Unknown lookup method {method!r} (only 'sort' is implemented)")
        self.device = D.cuda_device(device)
        dev = self.device
        st = D.stream_ptr(dev)
        if isinstance(idx, torch.Tensor) and idx.is_cuda:
            # device-resident input: (nnz, N) int32 holding the uint32 indices
            if idx.dim() != 2 or idx.dtype != torch.int32:
                raise TypeError("a CUDA idx must be a (nnz, N) int32 tensor")
            self.idx_dev = idx.contiguous()
            self.vals_dev = vals.to(dev, torch.float64).contiguous().reshape(-1)
            if dims is None:
                dims = (self.idx_dev.to(torch.int64).amax(dim=0) + 1).tolist()
        else:
            idx = np.asarray(idx)
            if idx.ndim != 2 or idx.dtype != np.uint32:
                raise TypeError("idx must be a (nnz, N) uint32 array")
            v = np.ascontiguousarray(np.asarray(vals, dtype=np.float64).reshape(-1))
            self.idx_dev = torch.from_numpy(np.ascontiguousarray(idx).view(np.int32)).to(dev)
            self.vals_dev = torch.from_numpy(v).to(dev)
            if dims is None:
                dims = (idx.max(axis=0).astype(np.int64) + 1) if idx.shape[0] else np.ones(idx.shape[1], np.int64)
        if self.vals_dev.shape[0] != self.idx_dev.shape[0]:
            raise ValueError("idx and vals disagree on nnz")
        self.nnz, self.N = int(self.idx_dev.shape[0]), int(self.idx_dev.shape[1])
        self.dims = [int(d) for d in dims]
        dims_c = (ctypes.c_int64 * self.N)(*self.dims)
        self._ws = _Workspace(dev)
        self.lookups = []   # per mode: fiber keys sorted, their mode-j index and value
        self.rows = []      # per mode: nonzeros sorted by mode-j index (index, fiber key, value)
        for j in range(self.N):
            keys = torch.empty(self.nnz, dtype=torch.int64, device=dev)
            _lib.call("ftl_fiber_keys", self.idx_dev.data_ptr(), 0, self.nnz, self.N, 1, self.N, dims_c, j,
                      keys.data_ptr(), st)
            # one-off construction sorts (keys < 2^63, so the signed order is
            # the unsigned order)
            skeys, perm = torch.sort(keys)
            idxj = torch.empty(self.nnz, dtype=torch.int32, device=dev)
            vj = torch.empty(self.nnz, dtype=torch.float64, device=dev)
            _lib.call("ftl_sparse_gather", perm.data_ptr(), self.idx_dev.data_ptr(), self.vals_dev.data_ptr(),
                      self.nnz, self.N, j, idxj.data_ptr(), vj.data_ptr(), st)
            del perm
            self.lookups.append((skeys, idxj, vj))
            col = self.idx_dev[:, j]
            rperm = torch.argsort(col, stable=True)
            self.rows.append((col[rperm].contiguous(), keys[rperm].contiguous(), self.vals_dev[rperm].contiguous()))
            del keys, rperm, col
        nb = _lib.ws_bytes("fit")
        out = torch.empty(1, dtype=torch.float64, device=dev)
        _lib.call("ftl_sum_squares", self.vals_dev.data_ptr(), self.nnz, self._ws.get("fit", nb).data_ptr(), nb,
                  out.data_ptr(), st)
        # read on first use: construction does not wait for the device
        self._normsq_dev = out
        self._normsq_ev = torch.cuda.Event()
        self._normsq_ev.record(torch.cuda.current_stream(dev))
        self._normsq = None
        self._dims_c = dims_c

    @property
    def normsq(self) -> float:
        if self._normsq is None:
            self._normsq_ev.synchronize()   # the sum ran on the construction stream
            self._normsq = float(self._normsq_dev.item())
        return self._normsq

    def get_normsq(self) -> float:
        return self.normsq

    def _factor_dev(self, U_list, R):
        out = []
        for k, u in enumerate(U_list):
            if isinstance(u, torch.Tensor) and u.is_cuda:
                out.append(u.to(torch.float64).contiguous())
            else:
                out.append(torch.from_numpy(D.as_factor(u, R, f"U[{k}]")).to(self.device))
        return out

    def compute_residual_normsq(self, sigma, U_list) -> float:
        """||X - [[sigma; U]]||^2 = sum_nnz (v^2 - 2 v model) + ||model||^2
        (sparse_tensor.hpp:117-119, sort_lookup.hpp:134-197).  U_list items
        may be numpy arrays or CUDA tensors (a LowRankTensor's U_dev)."""
        t = self.residual_terms_async(sigma, U_list).cpu().numpy()
        return float(t[0] + t[1])

    def residual_terms_async(self, sigma, U_list) -> torch.Tensor:
        """The two terms of compute_residual_normsq as a (2,) CUDA tensor,
        enqueued on the current stream without waiting for them."""
        st = D.stream_ptr(self.device)
        if isinstance(sigma, torch.Tensor):
            sig = sigma.to(self.device, torch.float64).contiguous()
        else:
            sig = torch.from_numpy(np.ascontiguousarray(np.asarray(sigma, dtype=np.float64))).to(self.device)
        R = int(sig.numel())
        Ud = self._factor_dev(U_list, R)
        nb = _lib.ws_bytes("fit")
        terms = torch.empty(2, dtype=torch.float64, device=self.device)
        _lib.call("ftl_sparse_residual_terms", self.idx_dev.data_ptr(), self.vals_dev.data_ptr(), self.nnz, self.N,
                  _ptrs(Ud), sig.data_ptr(), R, self._ws.get("fit", nb).data_ptr(), nb, terms[0:1].data_ptr(), st)
        G = [factor_gram(u, self._ws, st) for u in Ud]
        _lib.call("ftl_gram_hadamard", _ptrs(G), self.N, R, -1, sig.data_ptr(), sig.data_ptr(), None,
                  terms[1:2].data_ptr(), st)
        return terms

    def _exact_mttkrp_dev(self, U_L, j: int, out, out_rows, stream) -> None:
        R = int(U_L[0].shape[1])
        _lib.call("ftl_sparse_exact_mttkrp", self.idx_dev.data_ptr(), self.vals_dev.data_ptr(), self.nnz, self.N, j,
                  _ptrs(U_L), R, out, out_rows, stream)

    def execute_rrf(self, lr: "LowRankTensor", seed: int | None = None) -> None:
        """Randomized range-finder initialisation of `lr` (SparseTensor::
        execute_rrf, sparse_tensor.hpp:84-92): for every mode j, U_j = X_(j)
        Omega_j with one N(0,1) R-vector per fiber of mode j, then
        lr.renormalize_columns(-1).  The vectors come from a counter-based
        generator keyed by `seed` (random when None, as in the reference)."""
        import secrets
        if lr.N != self.N or lr.device != self.device:
            raise ValueError("tensor and decomposition disagree on modes or device")
        for k in range(self.N):
            if self.dims[k] > lr.dims[k]:
                raise ValueError(f"mode {k}: tensor index range {self.dims[k]} exceeds factor rows {lr.dims[k]}")
        seed = secrets.randbits(63) if seed is None else int(seed)
        st = D.stream_ptr(self.device)
        for j in range(self.N):
            rrows, rkeys, rvals = self.rows[j]
            _lib.call("ftl_sparse_rrf", rrows.data_ptr(), rkeys.data_ptr(), rvals.data_ptr(), self.nnz, lr.R,
                      seed, j, lr.U_dev[j].data_ptr(), lr.dims[j], st)
        lr.renormalize_columns(-1)

    def execute_downsampled_mttkrp_py(self, samples, lhs, j: int, result) -> None:
        """result (I_j x R) = sum over the rows i of samples (J x N uint64) of
        the fiber of samples[i] (modes != j) times lhs[i]
        (sparse_tensor.hpp:95-115)."""
        s = np.ascontiguousarray(np.asarray(samples, dtype=np.uint64))
        J, N = s.shape
        if N != self.N:
            raise ValueError(f"samples has {N} modes, tensor {self.N}")
        lhs_np = np.ascontiguousarray(np.asarray(lhs, dtype=np.float64))
        R = lhs_np.shape[1]
        out = D.require_numpy_out(result, np.float64, "result")
        if out.shape != (self.dims[j], R) and out.shape[0] < self.dims[j]:
            raise ValueError(f"result must be ({self.dims[j]}, {R})")
        dev = self.device
        st = D.stream_ptr(dev)
        s_d = torch.from_numpy(s.view(np.int64)).to(dev)
        keys = torch.empty(J, dtype=torch.int64, device=dev)
        _lib.call("ftl_fiber_keys", s_d.data_ptr(), 1, J, N, 1, N, self._dims_c, j, keys.data_ptr(), st)
        lhs_d = torch.from_numpy(lhs_np).to(dev)
        I_j = out.shape[0]
        o = torch.empty((I_j, R), dtype=torch.float64, device=dev)
        skeys, idxj, vj = self.lookups[j]
        _lib.call("ftl_sparse_mttkrp", skeys.data_ptr(), idxj.data_ptr(), vj.data_ptr(), self.nnz, keys.data_ptr(),
                  None, None, None, None, J, lhs_d.data_ptr(), R, o.data_ptr(), I_j, st)
        out[...] = o.cpu().numpy()
