"""Seeded synthetic workloads standing in for datasets that are not available
here (the FROSTT tensors the reference benchmarks on).

sparse_powerlaw_tensor: a 3-mode sparse tensor with per-mode bounded
Zipf(s) indices (inverse-CDF of the continuous power law on [1, dim + 1)),
duplicate index tuples removed, values log(1 + x) of lognormal(0, 1) draws --
the shape, index skew and value distribution of the amazon-reviews stand-in.
Generated on the GPU with torch's seeded generator.
"""
from __future__ import annotations

import torch


def _zipf_indices(n: int, dim: int, s: float, gen: torch.Generator, device) -> torch.Tensor:
    u = torch.rand(n, generator=gen, device=device, dtype=torch.float64)
    a = 1.0 - s
    hi = float(dim + 1) ** a
    x = (1.0 + u * (hi - 1.0)) ** (1.0 / a)      # continuous power law on [1, dim + 1)
    return (x.floor().to(torch.int64) - 1).clamp_(0, dim - 1)


def sparse_powerlaw_tensor(dims, nnz: int, s: float = 1.1, seed: int = 0, device="cuda",
                           oversample: float = 1.35):
    """Returns (idx int32 (nnz', 3) CUDA tensor holding uint32 indices, values
    float64 (nnz',)), nnz' <= nnz unique tuples sorted lexicographically."""
    assert len(dims) == 3
    gen = torch.Generator(device=device)
    gen.manual_seed(seed)
    m = int(nnz * oversample)
    i0 = _zipf_indices(m, dims[0], s, gen, device)
    i1 = _zipf_indices(m, dims[1], s, gen, device)
    i2 = _zipf_indices(m, dims[2], s, gen, device)
    # unique tuples: lexicographic sort by (i0, i1 * d2 + i2) (two stable sorts)
    lo = i1 * dims[2] + i2
    o = torch.argsort(lo, stable=True)
    o = o[torch.argsort(i0[o], stable=True)]
    i0, lo = i0[o], lo[o]
    keep = torch.ones(m, dtype=torch.bool, device=device)
    keep[1:] = (i0[1:] != i0[:-1]) | (lo[1:] != lo[:-1])
    i0, lo = i0[keep][:nnz], lo[keep][:nnz]
    idx = torch.stack([i0, lo // dims[2], lo % dims[2]], dim=1).to(torch.int32)
    vals = torch.log1p(torch.exp(torch.randn(idx.shape[0], generator=gen, device=device, dtype=torch.float64)))
    return idx.contiguous(), vals
