"""CPU oracle of the exact KRP leverage sampler -- TEST INFRASTRUCTURE ONLY.

Imported only by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
leg, always as the checker and never as the measured or shipped path.

The heavy loops (tree build, descents, Philox) are the C restatement in
ftl_oracle.c; this module restates the orchestration of
EfficientKRPSampler (vbharadwaj-bk/fast_tensor_leverage,
cpp_ext/efficient_krp_sampler.hpp) in numpy, with numpy.linalg.eigh on the
upper triangle standing in for LAPACKE_dsyev(..., 'V', 'U', ...).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
LIB = BUILD / "libftl_oracle.so"

_lib = None


def build(force: bool = False) -> Path:
    src = HERE / "ftl_oracle.c"
    if not force and LIB.exists() and LIB.stat().st_mtime >= src.stat().st_mtime:
        return LIB
    BUILD.mkdir(exist_ok=True)
    tmp = BUILD / "libftl_oracle.so.tmp"
    cmd = ["gcc", "-O3", "-fopenmp", "-shared", "-fPIC", "-std=c11", str(src), "-o", str(tmp), "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(str(LIB))
        P = ctypes.c_void_p
        i64 = ctypes.c_int64
        L.orc_geometry.argtypes = [i64, i64, P]
        L.orc_tree_build.argtypes = [P, i64, ctypes.c_int, i64, P]
        L.orc_tree_scale.argtypes = [P, P, i64, ctypes.c_int, P]
        L.orc_pt_sample.argtypes = [P, P, i64, ctypes.c_int, i64, P, P, P, P, i64, P]
        L.orc_philox_uniforms.argtypes = [ctypes.c_uint64, ctypes.c_uint64, i64, P]
        L.orc_philox4x32_10.argtypes = [P, P, P]
        L.orc_num_threads.restype = ctypes.c_int
        L.orc_set_num_threads.argtypes = [ctypes.c_int]
        _lib = L
    return _lib


def _p(a: np.ndarray):
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(ctypes.c_void_p)


GEOM_KEYS = (
    "n", "F", "leaf_count", "node_count", "lfill_level", "lfill_count", "total_levels",
    "nodes_upto_lfill", "nodes_before_lfill", "complete_level_offset",
)


def geometry(n: int, F: int) -> dict:
    out = np.zeros(10, dtype=np.int64)
    lib().orc_geometry(n, F, _p(out))
    return dict(zip(GEOM_KEYS, (int(v) for v in out)))


def packed_size(R: int) -> int:
    return R * (R + 1) // 2


def packed_to_upper(Gp: np.ndarray, R: int) -> np.ndarray:
    """Packed upper triangles (..., P) -> full (..., R, R) with a zero lower
    triangle, the reference's node layout."""
    iu = np.triu_indices(R)
    out = np.zeros(Gp.shape[:-1] + (R, R))
    out[..., iu[0], iu[1]] = Gp
    return out


def upper_to_packed(G: np.ndarray, R: int) -> np.ndarray:
    iu = np.triu_indices(R)
    return np.ascontiguousarray(G[..., iu[0], iu[1]])


def tree_build(U: np.ndarray, F: int) -> np.ndarray:
    U = np.ascontiguousarray(U, dtype=np.float64)
    n, R = U.shape
    g = geometry(n, F)
    G = np.empty((g["node_count"], packed_size(R)))
    lib().orc_tree_build(_p(U), n, R, F, _p(G))
    return G


def tree_scale(G: np.ndarray, R: int, mat_packed: np.ndarray) -> np.ndarray:
    out = np.empty_like(G)
    m = np.ascontiguousarray(mat_packed, dtype=np.float64)
    lib().orc_tree_scale(_p(G), _p(out), G.shape[0], R, _p(m))
    return out


def pt_sample(G, U, F, h, scaled_h, samples, draws, margin=None):
    """PartitionTree::PTSample_internal: in place on h and samples."""
    n, R = U.shape
    J = scaled_h.shape[0]
    lib().orc_pt_sample(
        _p(G), _p(U), n, R, F, _p(h), _p(scaled_h), _p(samples), _p(draws), J,
        _p(margin) if margin is not None else None,
    )


def philox_uniforms(seed: int, ctr: int, n: int) -> np.ndarray:
    out = np.empty(n)
    lib().orc_philox_uniforms(seed, ctr, n, _p(out))
    return out


def philox4x32_10(ctr, key) -> list:
    c = np.asarray(ctr, dtype=np.uint32)
    k = np.asarray(key, dtype=np.uint32)
    out = np.zeros(4, dtype=np.uint32)
    lib().orc_philox4x32_10(_p(c), _p(k), _p(out))
    return [int(v) for v in out]


def set_threads(n: int) -> None:
    lib().orc_set_num_threads(int(n))


def num_threads() -> int:
    return int(lib().orc_num_threads())


class OracleKRPSampler:
    """EfficientKRPSampler (cpp_ext/efficient_krp_sampler.hpp:16-275) with
    injected uniforms, on the CPU."""

    def __init__(self, U_list, J: int, R: int):
        self.U = [np.ascontiguousarray(u, dtype=np.float64) for u in U_list]
        self.N = len(self.U)
        self.J = int(J)
        self.R = int(R)
        self.F = [min(R, u.shape[0]) for u in self.U]  # ctor :52
        self.gram = [tree_build(u, f) for u, f in zip(self.U, self.F)]
        self.eig = [None] * self.N
        self.h = None
        self.weights = None
        self.pinv = None

    def update_sampler(self, j: int) -> None:  # :73-75
        self.gram[j] = tree_build(self.U[j], self.F[j])

    def _norm_j(self, j: int) -> int:
        # j == N indexes past the reference's eigenvector list (undefined
        # there); every j >= N is taken as "no mode excluded".
        return j if j < self.N else self.N + 1

    def compute_m(self, j: int) -> None:
        """computeM, :90-194."""
        N, R = self.N, self.R
        j = self._norm_j(j)
        M = np.zeros((N + 2, R, R))
        M[N] = 1.0
        roots = [packed_to_upper(self.gram[k][0], R) for k in range(N)]
        last = N
        for k in range(N - 1, -1, -1):  # :95-105
            if k != j:
                M[k] = roots[k] * M[last]
                last = k
        if j == 0:  # :108-110
            M[0] = M[1].copy()
        M[N + 1] = M[0]
        lam, V = np.linalg.eigh(M[0], UPLO="U")  # :118-124
        keep = lam > 1e-8
        WN = np.zeros((R, R))
        for v in range(R):  # :126-138
            if keep[v]:
                WN[:, R - 1 - v] = V[:, v] / np.sqrt(lam[v])
        pinv = WN @ WN.T  # :140-150 (dsyrk, upper)
        M[N] = WN
        self.lam0 = lam
        for k in range(N - 1, 0, -1):  # :154-161
            if k != j:
                M[k] = M[k] * pinv
        self.lam = {}
        for k in range(N, 0, -1):  # :164-184
            if k != j:
                if k < N:
                    lk, Vk = np.linalg.eigh(M[k], UPLO="U")
                    self.lam[k] = lk
                    # negative rounding noise is clamped (the reference takes
                    # sqrt of it and gets NaN)
                    M[k] = Vk * np.sqrt(np.maximum(lk, 0.0))[None, :]
                M[k] = M[k].T.copy()
        for k in range(N - 1, -1, -1):  # :187-193
            if k != j:
                offset = k + 2 if k + 1 == j else k + 1
                Gk = tree_build(np.ascontiguousarray(M[offset]), 1)
                self.eig[k] = tree_scale(Gk, R, self.gram[k][0])
        self.M = M
        self.pinv = pinv

    def draw(self, j: int, draws: np.ndarray, samples: np.ndarray | None = None,
             want_margin: bool = False):
        """KRPDrawSamples with injected uniforms (2N x J layout), :209-268.
        Returns samples (N x J uint64); sets self.h, self.weights and, if
        asked, self.margin (per-sample smallest decision margin)."""
        N, J, R = self.N, self.J, self.R
        draws = np.ascontiguousarray(draws, dtype=np.float64).reshape(-1)
        assert draws.size == 2 * N * J
        self.compute_m(j)
        jn = self._norm_j(j)
        if samples is None:
            samples = np.zeros((N, J), dtype=np.uint64)
        h = np.ones((J, R))
        margin = np.full(J, np.inf) if want_margin else None
        mtmp = np.empty(J) if want_margin else None
        for k in range(N):
            if k == jn:
                continue
            scaled_h = h.copy()
            offset = k + 2 if k + 1 == jn else k + 1
            row = np.zeros(J, dtype=np.uint64)
            W = np.ascontiguousarray(self.M[offset])
            pt_sample(self.eig[k], W, 1, scaled_h, h, row,
                      np.ascontiguousarray(draws[k * J:(k + 1) * J]), mtmp)
            if want_margin:
                np.minimum(margin, mtmp, out=margin)
            pt_sample(self.gram[k], self.U[k], self.F[k], h, scaled_h, row,
                      np.ascontiguousarray(draws[N * J + k * J:N * J + (k + 1) * J]), mtmp)
            if want_margin:
                np.minimum(margin, mtmp, out=margin)
            samples[k] = row
        # compute_DAGAT (sampler.hpp:94-123): dsymm with the upper triangle,
        # then per-row dot products; w = R / (lev * J) (:264-267)
        temp = h @ np.triu(self.pinv) + h @ np.triu(self.pinv, 1).T
        lev = np.einsum("ij,ij->i", h, temp)
        self.h = h
        self.weights = R / (lev * J)
        self.margin = margin
        return samples


def krp_leverage(U_list, pinv_of=None):
    """Exact leverage scores of every row of the (small) KRP of U_list, rows
    in the reference's flattening (first factor slowest): lev = k^T pinv(G) k
    with G = Hadamard product of the factor Grams."""
    R = U_list[0].shape[1]
    G = np.ones((R, R))
    for u in U_list:
        G = G * (u.T @ u)
    pinv = np.linalg.pinv(G) if pinv_of is None else pinv_of
    rows = U_list[0]
    for u in U_list[1:]:
        rows = np.einsum("ir,jr->ijr", rows, u).reshape(-1, R)
    return np.einsum("ir,rs,is->i", rows, pinv, rows)


# ------------------------------------------------------------------ CP-ALS

def pinv_square(M: np.ndarray, target_rank: int, tol: float) -> np.ndarray:
    """compute_pinv_square (cpp_ext/common.h:228-269): eigendecomposition of
    the upper triangle, keep eigenpair v (ascending) when v >= R - target and
    lambda_v > tol, return W W^T with W's kept columns v / sqrt(lambda_v)."""
    R = M.shape[0]
    lam, V = np.linalg.eigh(M, UPLO="U")
    W = np.zeros((R, R))
    for v in range(R):
        if v >= R - target_rank and lam[v] > tol:
            W[:, v] = V[:, v] / np.sqrt(lam[v])
    return W @ W.T


def fiber_keys(idx: np.ndarray, dims, j: int) -> np.ndarray:
    """Mixed-radix key of the indices of the modes != j (first mode most
    significant): the order of the reference's comparators on modes != j."""
    N = idx.shape[1]
    key = np.zeros(idx.shape[0], dtype=np.uint64)
    for k in range(N):
        if k == j:
            continue
        key = key * np.uint64(dims[k]) + idx[:, k].astype(np.uint64)
    return key


class OracleALS:
    """ALS::execute_ds_als_update (cpp_ext/als.hpp:57-220) restated in numpy
    over OracleKRPSampler, for a COO sparse tensor (SortIdxLookup semantics,
    cpp_ext/sort_lookup.hpp:69-132)."""

    def __init__(self, U_list, sigma, idx, vals, J: int, dims=None, rhs=None, lookups=None):
        self.U = [np.array(u, dtype=np.float64, copy=True) for u in U_list]
        self.N = len(self.U)
        self.R = self.U[0].shape[1]
        self.sigma = np.array(sigma, dtype=np.float64, copy=True)
        self.rhs = rhs          # a black-box right-hand side (OracleLowRankRHS / OracleDenseRHS)
        self.dims = list(dims) if dims is not None else [u.shape[0] for u in self.U]
        self.J = J
        self.sampler = OracleKRPSampler(self.U, J, self.R)
        self.lookups = []
        if rhs is not None:
            return
        self.idx = np.ascontiguousarray(idx, dtype=np.uint32)
        self.vals = np.asarray(vals, dtype=np.float64)
        if lookups is not None:
            # per mode (sorted fiber keys, their mode-j indices, their values),
            # the stable sort below made elsewhere
            self.lookups = [(np.asarray(k, dtype=np.uint64), np.asarray(i, dtype=np.int64),
                             np.asarray(v, dtype=np.float64)) for k, i, v in lookups]
            return
        for j in range(self.N):
            k = fiber_keys(self.idx, self.dims, j)
            perm = np.argsort(k, kind="stable")
            self.lookups.append((k[perm], self.idx[perm, j].astype(np.int64), self.vals[perm]))

    def update(self, j: int, draws, renormalize: bool = True, update_sampler: bool = True):
        N, R, J = self.N, self.R, self.J
        self.sampler.U = self.U
        samples = self.sampler.draw(j, draws)
        h, w = self.sampler.h, self.sampler.weights
        T = samples.T.astype(np.uint32).astype(np.int64)          # als.hpp:76-81
        keys = fiber_keys(T, self.dims, j)
        uk, first, counts = np.unique(keys, return_index=True, return_counts=True)
        wd = w[first] * counts                                      # :125-153
        hd = h[first] * np.sqrt(wd)[:, None]                        # :155-160
        pinv = pinv_square(hd.T @ hd, min(len(uk), R), 1e-11)       # :164-165
        hd = hd * np.sqrt(wd)[:, None]                              # :169-174
        if self.rhs is not None:                                    # black_box_tensor.hpp:21-67
            out = np.zeros((self.U[j].shape[0], R))
            fib = self.rhs.fibers(T[first], j)                      # unique samples x I_j
            out[: fib.shape[1]] = fib.T @ hd
            self.U[j] = out @ pinv
            return self._finish_update(j, renormalize, update_sampler, samples)
        skeys, sidx, svals = self.lookups[j]
        lo = np.searchsorted(skeys, uk, side="left")
        hi = np.searchsorted(skeys, uk, side="right")
        out = np.zeros((self.U[j].shape[0], R))
        for u in range(len(uk)):
            for z in range(lo[u], hi[u]):
                out[sidx[z]] += svals[z] * hd[u]
        self.U[j] = out @ pinv                                      # :189-203
        return self._finish_update(j, renormalize, update_sampler, samples)

    def _finish_update(self, j, renormalize, update_sampler, samples):
        if renormalize:                                             # low_rank_tensor.hpp:203-260
            norms = np.sqrt((self.U[j] ** 2).sum(axis=0))
            norms[norms <= 1e-7] = 1.0
            self.U[j] = self.U[j] / norms
            self.sigma = norms
        if update_sampler:
            self.sampler.U[j] = self.U[j]
            self.sampler.update_sampler(j)
        self.last_samples = samples
        return self.U[j]

    def residual_normsq(self) -> float:
        model = np.ones((self.idx.shape[0], self.R)) * self.sigma[None, :]
        for k in range(self.N):
            model = model * self.U[k][self.idx[:, k]]
        m = model.sum(axis=1)
        G = np.outer(self.sigma, self.sigma)
        for k in range(self.N):
            G = G * (self.U[k].T @ self.U[k])
        return float(np.sum(self.vals ** 2 - 2 * self.vals * m) + G.sum())


def fiber_normals(seed: int, mode: int, key: int, R: int) -> np.ndarray:
    """The R standard normals of one fiber in the GPU range finder
    (ftl_sparse_rrf): Philox4x32-10 block p = (counter (key lo, key hi, p,
    mode), key seed), u1 = ((x0 >> 8) + 1) 2^-24, u2 = (x1 >> 8) 2^-24,
    columns 2p, 2p+1 = sqrt(-2 ln u1) (cos, sin)(2 pi u2), here in FP64."""
    out = np.empty(2 * ((R + 1) // 2))
    kk = [seed & 0xFFFFFFFF, seed >> 32]
    for p in range((R + 1) // 2):
        x = philox4x32_10([key & 0xFFFFFFFF, key >> 32, p, mode], kk)
        u1 = ((x[0] >> 8) + 1) / 16777216.0
        u2 = (x[1] >> 8) / 16777216.0
        r = np.sqrt(-2.0 * np.log(u1))
        out[2 * p], out[2 * p + 1] = r * np.cos(2 * np.pi * u2), r * np.sin(2 * np.pi * u2)
    return out[:R]


def rrf(idx: np.ndarray, vals: np.ndarray, dims, rows, R: int, seed: int) -> list:
    """Restatement of SparseTensor::execute_rrf (sparse_tensor.hpp:84-92,
    sort_lookup.hpp:262-353) before the final renormalisation: for every mode
    j, U_j[idx_j] += v * g(fiber), one Gaussian vector per fiber (the modes
    != j), with the GPU's counter-based vectors; `rows` = factor row counts."""
    idx = np.asarray(idx, dtype=np.int64)
    out = []
    for j in range(len(dims)):
        keys = fiber_keys(idx, dims, j)
        U = np.zeros((rows[j], R))
        cache = {}
        for z in range(idx.shape[0]):
            k = int(keys[z])
            if k not in cache:
                cache[k] = fiber_normals(seed, j, k, R)
            U[idx[z, j]] += vals[z] * cache[k]
        out.append(U)
    return out


class OracleLowRankRHS:
    """A low-rank right-hand side [[sigma; V]] (LowRankTensor as a
    BlackBoxTensor, low_rank_tensor.hpp:91-135): the fiber of sample s along
    mode j is V_j (sigma o prod_{k != j} V_k[s_k])."""

    def __init__(self, V, sigma):
        self.V = [np.asarray(v, dtype=np.float64) for v in V]
        self.sigma = np.asarray(sigma, dtype=np.float64)

    def partial(self, S, j):
        P = np.ones((S.shape[0], self.sigma.size)) * self.sigma[None, :]
        for k, v in enumerate(self.V):
            if k != j:
                P = P * v[S[:, k]]
        return P

    def fibers(self, S, j):
        return self.partial(S, j) @ self.V[j].T

    def evaluate(self, idx):
        return self.partial(np.asarray(idx, dtype=np.int64), -1).sum(axis=1)

    def residual_normsq(self, sigma, U):
        """||[[sigma; U]] - [[s; V]]||^2 by Gram chains (low_rank_tensor.hpp:78-89)."""
        def chain(A, sa, B, sb):
            G = np.outer(sa, sb)
            for a, b in zip(A, B):
                G = G * (a.T @ b)
            return G.sum()
        return max(chain(self.V, self.sigma, self.V, self.sigma) + chain(U, sigma, U, sigma)
                   - 2 * chain(U, sigma, self.V, self.sigma), 0.0)


class OracleDenseRHS:
    """A dense right-hand side (DenseTensor, dense_tensor.hpp:38-59): the
    fiber of sample s along mode j is T[s_0, .., :, .., s_{N-1}]."""

    def __init__(self, T):
        self.T = np.asarray(T, dtype=np.float64)

    def fibers(self, S, j):
        N = self.T.ndim
        out = np.empty((S.shape[0], self.T.shape[j]))
        for i in range(S.shape[0]):
            out[i] = self.T[tuple(S[i, k] if k != j else slice(None) for k in range(N))]
        return out
