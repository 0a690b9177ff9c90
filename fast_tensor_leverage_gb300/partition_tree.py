"""PartitionTree: drop-in for the reference's standalone tree module
(cpp_ext/partition_tree.cpp:4-59, PartitionTree(n, F, J, R) with build_tree,
PTSample, get_G0 and multiply_against_numpy_buffer), backed by the CUDA tree
build (ftl_tree_build) and warp-per-sample descent (ftl_tree_sample)."""
from __future__ import annotations

import numpy as np
import torch

from . import _device as D
from . import _lib


class PartitionTree:
    def __init__(self, n: int, F: int, J: int, R: int, *, precision: str = "fp64", device=None):
        if precision not in _lib.PREC:
            raise ValueError(f"precision must be one of {sorted(_lib.PREC)}, got {precision!r}")
        n, F, J, R = int(n), int(F), int(J), int(R)
        if not (1 <= R <= _lib.MAX_RANK):
            raise ValueError(f"R={R} outside [1, {_lib.MAX_RANK}]")
        if not (1 <= F <= _lib.MAX_RANK):
            raise ValueError(f"F={F} outside [1, {_lib.MAX_RANK}]")
        if n < 1 or J < 0:
            raise ValueError(f"bad n={n} or J={J}")
        self.n, self.F, self.J, self.R = n, F, J, R
        self.precision = precision
        self._prec = _lib.PREC[precision]
        self.device = D.cuda_device(device)
        g = _lib.tree_geometry(n, F)
        self.leaf_count, self.node_count = g.leaf_count, g.node_count
        self.lfill_level = g.lfill_level
        self.P = R * (R + 1) // 2
        dt = torch.float64 if precision == "fp64" else torch.float32
        nbytes = _lib.tree_bytes(n, F, R, self._prec)
        self.S = nbytes // (self.node_count * dt.itemsize)  # values per node (ftl_node_layout)
        self.G = torch.zeros(nbytes // dt.itemsize, dtype=dt, device=self.device)
        self._G_unmultiplied = None
        self._U = None

    def build_tree(self, U) -> None:
        """PartitionTree::build_tree (partition_tree.hpp:120-170)."""
        u = D.as_factor(U, self.R, "U")
        if u.shape[0] != self.n:
            raise ValueError(f"U has {u.shape[0]} rows, tree covers n={self.n}")
        self._U = torch.from_numpy(u).to(self.device)
        self._G_unmultiplied = None
        _lib.call("ftl_tree_build", D.ptr(self._U), self.n, self.R, self.F, self._prec,
                  D.ptr(self.G), D.stream_ptr(self.device))

    def multiply_against_numpy_buffer(self, mat) -> None:
        """Multiply every node Gram elementwise by mat (R x R, upper triangle
        used), keeping the unmultiplied Grams for later calls
        (partition_tree.hpp:183-199)."""
        m = np.asarray(mat, dtype=np.float64).reshape(self.R, self.R)
        iu = np.triu_indices(self.R)
        packed = torch.from_numpy(np.ascontiguousarray(m[iu])).to(self.device)
        if self._G_unmultiplied is None:
            self._G_unmultiplied = self.G.clone()
        _lib.call("ftl_tree_scale", D.ptr(self._G_unmultiplied), D.ptr(self.G), self.node_count,
                  self.R, self._prec, D.ptr(packed), D.stream_ptr(self.device))

    def get_G0(self, out) -> None:
        """Root Gram into out (R x R): upper triangle, zero lower triangle, as
        the reference stores it (partition_tree.hpp:172-177)."""
        o = D.require_numpy_out(out, np.float64, "out", min_size=self.R * self.R)
        _, _, pos = _lib.node_layout(self.R, self._prec)
        root = self.G[: self.S].double().cpu().numpy()[pos]
        full = np.zeros((self.R, self.R))
        full[np.triu_indices(self.R)] = root
        o.reshape(-1)[: self.R * self.R] = full.reshape(-1)

    def get_G(self) -> np.ndarray:
        """All node Grams as packed upper triangles, (node_count, P), whatever
        the device layout."""
        _, _, pos = _lib.node_layout(self.R, self._prec)
        return self.G.double().cpu().numpy().reshape(self.node_count, self.S)[:, pos].copy()

    def PTSample(self, U, h, scaled_h, samples, random_draws) -> None:
        """PartitionTree::PTSample (partition_tree.hpp:216-405): for every row
        i of scaled_h draw a row of U with probability proportional to
        (U[row] . scaled_h[i])^2 using random_draws[i]; samples[i] <- row,
        h[i] *= U[row].  h and samples are updated in place."""
        J = self.J
        h_np = D.require_numpy_out(h, np.float64, "h", shape=(J, self.R))
        s_np = D.require_numpy_out(samples, np.uint64, "samples", min_size=J)
        sh = np.ascontiguousarray(np.asarray(scaled_h, dtype=np.float64).reshape(J, self.R))
        dr = np.ascontiguousarray(np.asarray(random_draws, dtype=np.float64).reshape(-1)[:J])
        u = D.as_factor(U, self.R, "U")
        if u.shape[0] != self.n:
            raise ValueError(f"U has {u.shape[0]} rows, tree covers n={self.n}")
        dev = self.device
        U_d = torch.from_numpy(u).to(dev)
        h_d = torch.from_numpy(h_np).to(dev)
        sh_d = torch.from_numpy(sh).to(dev)
        dr_d = torch.from_numpy(dr).to(dev)
        s_d = torch.empty(J, dtype=torch.int64, device=dev)
        _lib.call("ftl_tree_sample", D.ptr(self.G), self._prec, D.ptr(U_d), self.n, self.R, self.F,
                  D.ptr(h_d), D.ptr(sh_d), D.ptr(s_d), D.ptr(dr_d), J, D.stream_ptr(dev))
        h_np[...] = h_d.cpu().numpy()
        s_np.reshape(-1)[:J] = s_d.cpu().numpy().view(np.uint64)
