"""Seeded synthetic workloads standing in for datasets that are not available
here (the FROSTT tensors the reference benchmarks on).

sparse_powerlaw_tensor: an N-mode sparse tensor with per-mode bounded
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
    """Returns (idx int32 (nnz', N) CUDA tensor holding uint32 indices, values
    float64 (nnz',)), nnz' <= nnz unique tuples sorted lexicographically."""
    N = len(dims)
    assert N >= 2 and all(0 < d <= 1 << 32 for d in dims)
    gen = torch.Generator(device=device)
    gen.manual_seed(seed)
    m = int(nnz * oversample)
    cols = [_zipf_indices(m, int(d), s, gen, device) for d in dims]
    # lexicographic order: stable sorts from the last mode to the first
    o = torch.argsort(cols[N - 1], stable=True)
    for k in range(N - 2, -1, -1):
        o = o[torch.argsort(cols[k][o], stable=True)]
    cols = [c[o] for c in cols]
    keep = torch.zeros(m, dtype=torch.bool, device=device)
    keep[0] = True
    for c in cols:
        keep[1:] |= c[1:] != c[:-1]
    idx = torch.stack([c[keep][:nnz] for c in cols], dim=1).to(torch.int32)
    del cols, keep, o
    vals = torch.log1p(torch.exp(torch.randn(idx.shape[0], generator=gen, device=device, dtype=torch.float64)))
    return idx.contiguous(), vals
