"""GPU parity of the exact KRP sampler and the partition tree against the
reference's golden outputs and the CPU oracle.

Tolerances:
  * FP64 mode: sample indices bit-exact.  A sample may differ only if the
    oracle's smallest decision margin for it (distance between a uniform and
    a cutoff it was compared with) is below NEAR_TIE -- the quadratic forms
    are summed in a different order than the reference's BLAS, so decisions
    that close are rounding-dependent.  h of a matching sample is bit-exact
    (the same rows multiplied in the same order); weights within 1e-9
    relative (FP64 pseudo-inverse from a Jacobi eigensolver vs LAPACK).
  * FP32 mode: index agreement with the FP64 oracle >= 99% (>= 97% for
    R > 32: the per-mode eigendecompositions run in FP32 and, where the
    eigenvalues of a per-mode matrix cluster, FP32 eigenvectors mix within
    the cluster, which moves the uniform -> component map but not the
    distribution), weights within 1e-3 relative, and the empirical
    distribution within sampling noise of the exact leverage distribution
    (total variation).
"""
import numpy as np
import pytest
import torch

from oracle import oracle as O
from tests._golden import included_rows, krp_cases, load_krp, load_tree, tree_cases

pytestmark = pytest.mark.gpu

NEAR_TIE = 1e-10


@pytest.fixture(scope="module")
def ftl():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import fast_tensor_leverage_gb300 as m
    return m


def check_indices(got, want, margin, rows, max_ties_frac=1e-3):
    mism = (got[rows] != want[rows]).any(axis=0)
    n = int(mism.sum())
    if n:
        assert margin is not None, f"{n} mismatching samples"
        assert np.all(margin[mism] < NEAR_TIE), (
            f"{n} mismatches, margins {np.sort(margin[mism])[-5:]}")
        assert n <= max(1, max_ties_frac * got.shape[1])
    return mism


@pytest.mark.parametrize("name", krp_cases())
def test_fp64_draw_matches_reference_golden(ftl, name):
    c = load_krp(name)
    N, J, R, j = c["N"], c["J"], c["R"], c["j"]
    s = ftl.Sampler(c["U"], J, R, "efficient", precision="fp64")
    samples = np.zeros((N, J), dtype=np.uint64)
    h = np.zeros((J, R))
    w = np.zeros(J)
    s.KRPDrawSamples_materialize(j, samples, h, w, draws=c["draws"])
    o = O.OracleKRPSampler(c["U"], J, R)
    o.draw(j, c["draws"], want_margin=True)
    rows = included_rows(N, j)
    mism = check_indices(samples, c["samples"], o.margin, rows)
    ok = ~mism
    assert np.array_equal(h[ok], c["h"][ok])
    np.testing.assert_allclose(w[ok], c["weights"][ok], rtol=1e-9)
    # row j is left untouched when a mode is excluded
    if j < N:
        assert not samples[j].any()


@pytest.mark.parametrize("N,dims,R,J,j,seed", [
    (4, [1000] * 4, 8, 10000, 5, 101),       # README shape, none excluded
    (3, [1001] * 3, 8, 5000, 1, 102),        # partial leaf, mode excluded
    (3, [2048, 777, 4096], 32, 4000, 0, 103),
    (3, [300, 1500, 64], 25, 3000, 2, 104),  # R not a power of two, F = R
    (2, [5000, 3000], 64, 2000, 3, 105),     # R > 32: shared-memory forms
    (2, [600, 700], 128, 600, 3, 106),       # R = 128: eigenvectors in scratch
    (4, [300, 400, 350, 500], 128, 400, 1, 111),  # R = 128, four modes, one excluded
    (3, [20, 30, 40], 32, 1500, 4, 107),     # I < R: F = I, single-leaf trees
    (6, [50, 60, 70, 80, 90, 100], 16, 2000, 3, 108),
    (4, [17, 50, 9, 23], 5, 1500, 2, 109),   # odd R with N + 1 odd: unaligned dense slots
    (5, [33, 44, 55, 66, 77], 7, 1500, 6, 110),
])
def test_fp64_draw_matches_oracle(ftl, N, dims, R, J, j, seed):
    rng = np.random.default_rng(seed)
    U = [rng.normal(size=(n, R)) for n in dims]
    rows_heavy = rng.choice(dims[0], size=max(1, dims[0] // 100), replace=False)
    U[0][rows_heavy] *= 100.0
    draws = rng.random(2 * N * J)
    s = ftl.Sampler(U, J, R, "efficient", precision="fp64")
    samples = np.zeros((N, J), dtype=np.uint64)
    h = np.zeros((J, R))
    w = np.zeros(J)
    s.KRPDrawSamples_materialize(j, samples, h, w, draws=draws)
    o = O.OracleKRPSampler(U, J, R)
    ref = o.draw(j, draws, want_margin=True)
    rows = included_rows(N, j if j < N else N + 1)
    mism = check_indices(samples, ref, o.margin, rows)
    ok = ~mism
    assert np.array_equal(h[ok], o.h[ok])
    np.testing.assert_allclose(w[ok], o.weights[ok], rtol=1e-9)


@pytest.fixture(scope="module")
def c2_case(ftl):
    """The benchmarked sampling shape: N = 3 factors of I = 2^23 rows x
    R = 32, N(0,1) entries with 1% of each factor's rows x100 (made on the
    device, seeded), with the CPU oracle's FP64 trees over the same values."""
    N, I, R = 3, 1 << 23, 32
    g = torch.Generator(device="cuda")
    g.manual_seed(2323)
    U = []
    for _ in range(N):
        u = torch.randn(I, R, device="cuda", dtype=torch.float64, generator=g)
        u[torch.randperm(I, device="cuda", generator=g)[: I // 100]] *= 100.0
        U.append(u)
    U_host = [u.cpu().numpy() for u in U]
    import os
    O.set_threads(os.cpu_count() or 1)
    return {"N": N, "I": I, "R": R, "U": U, "U_host": U_host, "oracle": O.OracleKRPSampler(U_host, 4096, R)}


@pytest.mark.parametrize("j,min_agree", [(4, 0.90), (0, 0.80)])
def test_c2_scale_draw_matches_oracle(ftl, c2_case, j, min_agree):
    """At the benchmarked size (18-level Gram trees, I = 2^23): FP64 draws
    match the oracle index for index (except near-ties, oracle margin below
    NEAR_TIE), h bit-exact, weights within 1e-9.  Mixed-precision draws given
    the same uniforms agree with the oracle's samples on >= 90% (j = N+1) /
    80% (j = 0) of samples, with h bit-exact and weights within 1e-3 where
    they agree: FP32 forms place the 2^23 row boundaries of each mode's CDF
    about 1e-7 from their FP64 positions, and where per-mode eigenvalues
    cluster the FP32 eigenbasis differs inside the cluster, so the same
    uniform can land on a neighbouring row although the sampled law is the
    same (test_c2_like_law_matches_exact_marginals checks the law)."""
    N, R, J = c2_case["N"], c2_case["R"], 4096
    o = c2_case["oracle"]
    rng = np.random.default_rng(77 + j)
    draws = rng.random(2 * N * J)
    ref = o.draw(j, draws, want_margin=True).copy()
    margin, h_ref, w_ref = o.margin.copy(), o.h.copy(), o.weights.copy()
    rows = included_rows(N, j if j < N else N + 1)
    for precision in ("fp64", "fp32"):
        s = ftl.Sampler(c2_case["U"], J, R, "efficient", precision=precision, seed=1)
        samples = np.zeros((N, J), dtype=np.uint64)
        h = np.zeros((J, R))
        w = np.zeros(J)
        s.KRPDrawSamples_materialize(j, samples, h, w, draws=draws)
        if precision == "fp64":
            mism = check_indices(samples, ref, margin, rows)
            ok = ~mism
            assert np.array_equal(h[ok], h_ref[ok])
            np.testing.assert_allclose(w[ok], w_ref[ok], rtol=1e-9)
        else:
            agree = (samples[rows] == ref[rows]).all(axis=0)
            assert agree.mean() >= min_agree, agree.mean()
            assert np.array_equal(h[agree], h_ref[agree])
            np.testing.assert_allclose(w[agree], w_ref[agree], rtol=1e-3)
        del s
        torch.cuda.empty_cache()


def _exact_subtree_marginals(trees64, R, j, k, level):
    """P(mode-k sample row lies under node c) for the nodes c of `level` of
    mode k's tree: sum_ab G_c[a,b] M_k[a,b] / rank with M_k = pinv(prod over
    the sampled modes of the root Grams) o prod over the sampled modes other
    than k of the root Grams (the leverage law of the KRP, summed over the
    other modes' rows), from the FP64 node Grams (packed, stride 528)."""
    P = R * (R + 1) // 2
    iu = torch.triu_indices(R, R, device="cuda")

    def full(packed):
        M = torch.zeros((packed.shape[0], R, R), dtype=torch.float64, device="cuda")
        M[:, iu[0], iu[1]] = packed
        M[:, iu[1], iu[0]] = packed
        return M

    S = 528  # FP64 node stride at R = 32
    roots = {m: full(t.view(-1, S)[:1, :P])[0] for m, t in enumerate(trees64)}
    modes = [m for m in roots if m != j]
    prod = torch.ones((R, R), dtype=torch.float64, device="cuda")
    for m in modes:
        prod = prod * roots[m]
    Mk = torch.linalg.pinv(prod, hermitian=True)
    for m in modes:
        if m != k:
            Mk = Mk * roots[m]
    nodes = trees64[k].view(-1, S)[(1 << level) - 1:(1 << (level + 1)) - 1, :P]
    p = (full(nodes) * Mk).sum((1, 2))
    return (p / p.sum()).cpu().numpy()


@pytest.mark.parametrize("j", [4, 0])
def test_c2_like_law_matches_exact_marginals(ftl, j):
    """The sampled law itself at the C2 shape but 2^20 rows (15-level trees,
    1% of rows x100): for every sampled mode, the frequencies of 2^23 draws'
    rows per subtree at tree levels 4 and 8 against the exact subtree
    probabilities, in FP64 and in mixed precision.  Total variation within
    1.5x the sampling noise of that many draws (+1e-4)."""
    N, I, R, Jd, reps = 3, 1 << 20, 32, 1 << 20, 8
    g = torch.Generator(device="cuda")
    g.manual_seed(77)
    U = []
    for _ in range(N):
        u = torch.randn(I, R, device="cuda", dtype=torch.float64, generator=g)
        u[torch.randperm(I, device="cuda", generator=g)[: I // 100]] *= 100.0
        U.append(u)
    s64 = ftl.Sampler(U, Jd, R, "efficient", precision="fp64", seed=5)
    depth = 15  # 2^20 rows / 32 per leaf = 2^15 leaves, complete tree
    for precision in ("fp64", "fp32"):
        s = s64 if precision == "fp64" else ftl.Sampler(U, Jd, R, "efficient", precision=precision, seed=5)
        counts = {(k, L): torch.zeros(1 << L, dtype=torch.int64, device="cuda")
                  for k in range(N) if k != j for L in (4, 8)}
        for _ in range(reps):
            smp = s.draw(j)[0]
            for (k, L), c in counts.items():
                c += torch.bincount((smp[k] // 32) >> (depth - L), minlength=1 << L)
        for (k, L), c in counts.items():
            p = _exact_subtree_marginals(s64.trees, R, j, k, L)
            emp = c.cpu().numpy() / (reps * Jd)
            tv = 0.5 * np.abs(emp - p).sum()
            noise = 0.5 * np.sum(np.sqrt(2 * p / (np.pi * reps * Jd)))
            assert tv <= 1.5 * noise + 1e-4, (precision, k, L, tv, noise)


def test_readme_shape_marginals_match_exact(ftl):
    """The README configuration (N = 4 factors of 1000 x 8, a KRP of 10^12
    rows): the per-mode marginal of 2^24 draws over each mode's 1000 rows
    against the exact marginal p_k(i) = u_i^T [pinv(prod_m G_m) o prod_{m != k}
    G_m] u_i / rank (computed in FP64 from the factors), FP64 and mixed."""
    rng = np.random.default_rng(2024)
    N, I, R, Jd, reps = 4, 1000, 8, 1 << 21, 8
    U = [rng.normal(size=(I, R)) for _ in range(N)]
    G = [u.T @ u for u in U]
    prod = np.ones((R, R))
    for m in range(N):
        prod = prod * G[m]
    pinv = np.linalg.pinv(prod, hermitian=True)
    for precision in ("fp64", "fp32"):
        s = ftl.Sampler(U, Jd, R, "efficient", precision=precision, seed=9)
        counts = torch.zeros((N, I), dtype=torch.int64, device="cuda")
        for _ in range(reps):
            smp = s.draw(N + 1)[0]
            for k in range(N):
                counts[k] += torch.bincount(smp[k], minlength=I)
        emp = counts.cpu().numpy() / (reps * Jd)
        for k in range(N):
            Mk = pinv.copy()
            for m in range(N):
                if m != k:
                    Mk = Mk * G[m]
            p = np.einsum("ia,ab,ib->i", U[k], Mk, U[k])
            p = p / p.sum()
            tv = 0.5 * np.abs(emp[k] - p).sum()
            noise = 0.5 * np.sum(np.sqrt(2 * p / (np.pi * reps * Jd)))
            assert tv <= 1.5 * noise + 1e-4, (precision, k, tv, noise)


def test_philox_stream_equals_injected_oracle_uniforms(ftl):
    rng = np.random.default_rng(7)
    N, I, R, J = 4, 1000, 8, 10000
    U = [rng.normal(size=(I, R)) for _ in range(N)]
    seed = 0x1234_5678_9ABC
    s = ftl.Sampler(U, J, R, "efficient", precision="fp64", seed=seed)
    dev = torch.empty(2 * N * J, dtype=torch.float64, device="cuda")
    from fast_tensor_leverage_gb300 import _lib
    _lib.call("ftl_philox_uniforms", dev.data_ptr(), dev.numel(), seed, 0,
              torch.cuda.current_stream().cuda_stream)
    uni = O.philox_uniforms(seed, 0, 2 * N * J)
    assert np.array_equal(dev.cpu().numpy(), uni)
    samples = np.zeros((N, J), dtype=np.uint64)
    s.KRPDrawSamples(N + 1, samples)  # in-kernel Philox, counter 0
    o = O.OracleKRPSampler(U, J, R)
    ref = o.draw(N + 1, uni, want_margin=True)
    check_indices(samples, ref, o.margin, list(range(N)))
    # the next call continues the stream
    samples2 = np.zeros((N, J), dtype=np.uint64)
    s.KRPDrawSamples(N + 1, samples2)
    ref2 = o.draw(N + 1, O.philox_uniforms(seed, 2 * N * J, 2 * N * J), want_margin=True)
    check_indices(samples2, ref2, o.margin, list(range(N)))


@pytest.mark.parametrize("N,dims,R,J,j", [
    (4, [1000] * 4, 8, 10000, 5),
    (3, [4096, 2048, 3000], 32, 4000, 1),
    (2, [5000, 3000], 64, 2000, 3),
    (3, [20, 30, 40], 32, 3000, 4),   # rank-deficient Grams: Jacobi pseudo-inverse path
    (4, [170, 500, 90, 230], 5, 3000, 1),
    (3, [500, 600, 700], 128, 1500, 1),
])
def test_fp32_draw_agrees_with_fp64_oracle(ftl, N, dims, R, J, j):
    rng = np.random.default_rng(31 + R)
    U = [rng.normal(size=(n, R)) for n in dims]
    draws = rng.random(2 * N * J)
    s = ftl.Sampler(U, J, R, "efficient", precision="fp32")
    samples = np.zeros((N, J), dtype=np.uint64)
    h = np.zeros((J, R))
    w = np.zeros(J)
    s.KRPDrawSamples_materialize(j, samples, h, w, draws=draws)
    o = O.OracleKRPSampler(U, J, R)
    ref = o.draw(j, draws)
    rows = included_rows(N, j if j < N else N + 1)
    agree = (samples[rows] == ref[rows]).all(axis=0)
    assert agree.mean() >= (0.99 if R <= 32 else 0.97), agree.mean()
    np.testing.assert_allclose(w[agree], o.weights[agree], rtol=1e-3)
    assert np.array_equal(h[agree], o.h[agree])


@pytest.mark.parametrize("precision,N,I,R", [
    ("fp64", 3, 8, 8), ("fp32", 3, 8, 8),     # the reference's distribution check shape
    ("fp32", 2, 16, 16),                      # wider rank, mixed precision
])
def test_distribution_matches_exact_leverage(ftl, precision, N, I, R):
    """Empirical distribution of 2^26 draws from the KRP of small factors
    (I^N rows, 1% of entries x10 as in the reference's distribution check)
    against the brute-force FP64 leverage scores."""
    rng = np.random.default_rng(2023)
    U = [rng.normal(size=(I, R)) for _ in range(N)]
    for u in U:
        u[rng.random(u.shape) < 0.01] *= 10.0
    lev = O.krp_leverage(U)
    p = lev / lev.sum()
    J = 1 << 23
    s = ftl.Sampler(U, J, R, "efficient", precision=precision, seed=99)
    counts = torch.zeros(I ** N, dtype=torch.int64, device="cuda")
    offs = torch.tensor([I ** (N - 1 - k) for k in range(N)], device="cuda", dtype=torch.int64)
    reps = 8
    w_err = 0.0
    for _ in range(reps):
        samples, h, w = s.draw(N + 1)
        flat = (samples * offs[:, None]).sum(0)
        counts += torch.bincount(flat, minlength=I ** N)
        lev_s = torch.from_numpy(lev).cuda()[flat]
        w_err = max(w_err, float(((w * J * lev_s / R) - 1).abs().max()))
    emp = counts.cpu().numpy() / (reps * J)
    tv = 0.5 * np.abs(emp - p).sum()
    noise = 0.5 * np.sum(np.sqrt(2 * p / (np.pi * reps * J)))
    assert tv <= 1.3 * noise + 1e-4, (tv, noise)
    assert tv < 1e-3
    assert w_err < (1e-9 if precision == "fp64" else 1e-3), w_err


# ---------------------------------------------------------------- tree level

@pytest.mark.parametrize("name", tree_cases())
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_tree_build_and_sample_match_reference_golden(ftl, name, precision):
    c = load_tree(name)
    n, F, R, J = (int(c[k]) for k in ("n", "F", "R", "J"))
    t = ftl.PartitionTree(n, F, J, R, precision=precision)
    t.build_tree(c["U"])
    G = t.get_G()
    scale = np.abs(c["G_packed"]).max()
    tol = 1e-12 if precision == "fp64" else 2e-6
    np.testing.assert_allclose(G, c["G_packed"], rtol=0, atol=tol * scale * max(1, np.log2(n)))
    G0 = np.zeros((R, R))
    t.get_G0(G0)
    assert np.array_equal(np.tril(G0, -1), np.zeros((R, R)))
    h = c["h"].copy()
    samples = np.zeros(J, dtype=np.uint64)
    t.PTSample(c["U"], h, c["scaled_h"], samples, c["draws"])
    if precision == "fp64":
        Go = O.tree_build(c["U"], F)
        margin = np.zeros(J)
        s_o = np.zeros(J, dtype=np.uint64)
        O.pt_sample(Go, c["U"], F, c["h"].copy(), np.ascontiguousarray(c["scaled_h"]), s_o,
                    c["draws"], margin)
        mism = samples != c["samples"]
        assert np.all(margin[mism] < NEAR_TIE)
        assert np.array_equal(h[~mism], c["h_out"][~mism])
    else:
        assert (samples == c["samples"]).mean() >= 0.99


def test_tree_scale_matches_oracle(ftl):
    rng = np.random.default_rng(5)
    n, F, R = 500, 8, 8
    U = rng.normal(size=(n, R))
    mat = rng.normal(size=(R, R))
    t = ftl.PartitionTree(n, F, 10, R, precision="fp64")
    t.build_tree(U)
    t.multiply_against_numpy_buffer(mat)
    t.multiply_against_numpy_buffer(mat)  # applied to the unmultiplied Grams again
    Go = O.tree_scale(O.tree_build(U, F), R, O.upper_to_packed(mat, R))
    np.testing.assert_allclose(t.get_G(), Go, rtol=1e-13, atol=1e-13)


def test_large_tree_build_fp32_vs_fp64(ftl):
    """Complete tree of 2^20 rows, R = 32: FP32 build within FP32 rounding of
    the FP64 build at every node."""
    rng = np.random.default_rng(9)
    n, R = 1 << 20, 32
    U = rng.normal(size=(n, R))
    t64 = ftl.PartitionTree(n, R, 1, R, precision="fp64")
    t32 = ftl.PartitionTree(n, R, 1, R, precision="fp32")
    t64.build_tree(U)
    t32.build_tree(U)
    a, b = t64.get_G(), t32.get_G()
    diag = np.array([k * R - k * (k - 1) // 2 for k in range(R)])
    node_scale = a[:, diag].max(axis=1, keepdims=True)
    assert np.max(np.abs(a - b) / node_scale) < 1e-5
    # root against numpy
    Gr = U.T @ U
    np.testing.assert_allclose(a[0], Gr[np.triu_indices(R)], rtol=1e-10, atol=1e-8)


@pytest.mark.parametrize("R,rows_per_block", [(32, 32), (64, 64), (16, 5)])
def test_fp32_draw_never_selects_zero_rows(ftl, R, rows_per_block):
    """Factors whose rows are mostly exact zeros in long runs (the rows of an
    ALS factor that no sampled fiber touched): every sampled row must have a
    positive leverage, so every weight is finite and positive.  The FP32
    descent carries right-child masses as parent - left, so without the
    careful re-descent rounding can walk into an all-zero subtree."""
    rng = np.random.default_rng(77 + R)
    N, I, J = 3, 20000, 1 << 17
    U = []
    for k in range(N):
        u = np.zeros((I, R))
        live = rng.choice(I // rows_per_block, size=I // rows_per_block // 9, replace=False)
        for b in live:
            r = b * rows_per_block + rng.integers(0, rows_per_block)
            u[r] = rng.normal(size=R) * 10.0 ** rng.uniform(-3, 3)
        U.append(u)
    s = ftl.Sampler(U, J, R, "efficient", precision="fp32", seed=5)
    zero = [torch.from_numpy(~u.any(axis=1)).cuda() for u in U]
    for j in (N + 1, 0, 2):
        for _ in range(4):
            samples, h, w = s.draw(j)
            for k in range(N):
                if k == j:
                    continue
                assert not bool(zero[k][samples[k]].any()), f"mode {k}: a zero row was sampled"
            assert bool(torch.isfinite(w).all()) and bool((w > 0).all())
            assert bool((h.abs().sum(dim=1) > 0).all())


def test_pinv_square_with_nan_input_completes(ftl):
    """A NaN Gram (from a non-finite weight) must give a NaN result, not
    out-of-range eigenvector indexes: the eigenvalue sort ranks NaN last."""
    from fast_tensor_leverage_gb300 import _lib
    for R in (8, 64):
        M = torch.eye(R, dtype=torch.float64, device="cuda")
        M[1, 2] = M[2, 1] = float("nan")
        M[3, 3] = float("nan")
        out = torch.empty_like(M)
        vs = torch.empty_like(M)
        _lib.call("ftl_pinv_square", M.data_ptr(), R, R, None, 1e-11, out.data_ptr(), vs.data_ptr(),
                  torch.cuda.current_stream().cuda_stream)
        torch.cuda.synchronize()
        # the context is healthy and a finite input still inverts exactly
        G = torch.eye(R, dtype=torch.float64, device="cuda") * 4.0
        _lib.call("ftl_pinv_square", G.data_ptr(), R, R, None, 1e-11, out.data_ptr(), vs.data_ptr(),
                  torch.cuda.current_stream().cuda_stream)
        torch.cuda.synchronize()
        torch.testing.assert_close(out, torch.eye(R, dtype=torch.float64, device="cuda") / 4.0)


@pytest.mark.parametrize("R,j", [(32, 4), (64, 1), (128, 0), (25, 2)])
def test_fp32_factor_shadows_give_identical_draws(ftl, R, j):
    """FP32 draws whose leaf scans read the FP32 factor copies equal those
    reading the FP64 rows, bit for bit (the scan rounds the rows to FP32
    either way), alone and in a packed launch."""
    rng = np.random.default_rng(50 + R)
    dims = [3000, 2217, 4100]
    U = [rng.normal(size=(n, R)) for n in dims]
    U[1][rng.choice(dims[1], 40, replace=False)] *= 50.0
    J = 6000
    a = ftl.Sampler(U, J, R, "efficient", precision="fp32", seed=11)
    b = ftl.Sampler(U, J, R, "efficient", precision="fp32", seed=11, factor_shadows=False)
    assert a.U32 is not None and b.U32 is None
    for _ in range(2):
        sa, ha, wa = (t.clone() for t in a.draw(j))
        sb, hb, wb = (t.clone() for t in b.draw(j))
        assert torch.equal(sa, sb) and torch.equal(ha, hb) and torch.equal(wa, wb)
    # packed: shadowed plans together, then a mix (falls back to FP64 rows)
    from fast_tensor_leverage_gb300 import _lib
    import ctypes
    st = torch.cuda.current_stream().cuda_stream
    for plans_of in ((a, a), (a, b)):
        for s in plans_of:
            _lib.call("ftl_krp_compute_m", ctypes.byref(s._plan), j, st)
        # zeros: the excluded mode's row is left as it is, like the sampler's own buffer
        outs = [(torch.zeros_like(s.samples_dev), torch.empty_like(s.h_dev), torch.empty_like(s.weights_dev))
                for s in plans_of]
        b.samples_dev.zero_()
        n = len(plans_of)
        _lib.call("ftl_krp_sample_packed", (ctypes.POINTER(_lib.KRPPlan) * n)(*[ctypes.pointer(s._plan) for s in plans_of]),
                  n, (ctypes.c_uint32 * n)(*[j] * n), (ctypes.c_void_p * n)(*[o[0].data_ptr() for o in outs]),
                  (ctypes.c_void_p * n)(*[o[1].data_ptr() for o in outs]),
                  (ctypes.c_void_p * n)(*[o[2].data_ptr() for o in outs]), None,
                  (ctypes.c_uint64 * n)(*[11] * n), (ctypes.c_uint64 * n)(*[0] * n), st)
        _lib.call("ftl_krp_compute_m", ctypes.byref(b._plan), j, st)
        _lib.call("ftl_krp_sample", ctypes.byref(b._plan), j, b.samples_dev.data_ptr(), b.h_dev.data_ptr(),
                  b.weights_dev.data_ptr(), None, 11, 0, st)
        for o in outs:
            assert torch.equal(o[0], b.samples_dev) and torch.equal(o[1], b.h_dev) and torch.equal(o[2], b.weights_dev)


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_computem_launched_ahead_matches_fresh_draws(ftl, precision):
    """After two draws with the same j the sampler launches the next draw's
    computeM behind the current descent.  Every draw must equal a fresh
    sampler's draw on the same factors and uniforms: repeated j, a changed j
    (the launched-ahead result is discarded), and a factor replaced through
    set_factor between draws (its tree rebuild invalidates it)."""
    rng = np.random.default_rng(77)
    N, R, J = 3, 16, 4000
    dims = [900, 1300, 700]
    U = [rng.normal(size=(d, R)) for d in dims]
    s = ftl.Sampler([u.copy() for u in U], J, R, "efficient", precision=precision)

    def fresh(Uc, j, dr):
        f = ftl.Sampler([u.copy() for u in Uc], J, R, "efficient", precision=precision, overlap_computem=False)
        out = np.zeros((N, J), dtype=np.uint64)
        h = np.zeros((J, R))
        w = np.zeros(J)
        f.KRPDrawSamples_materialize(j, out, h, w, draws=dr)
        return out, h, w

    for step, j in enumerate([1, 1, 1, 1, 2, 1, 1, "swap", 1, 1, 0]):
        if j == "swap":
            U[0] = rng.normal(size=(dims[0], R))
            s.set_factor(0, U[0])
            continue
        dr = rng.random(2 * N * J)
        out = np.zeros((N, J), dtype=np.uint64)
        h = np.zeros((J, R))
        w = np.zeros(J)
        s.KRPDrawSamples_materialize(j, out, h, w, draws=dr)
        ro, rh, rw = fresh(U, j, dr)
        rows = [k for k in range(N) if k != j]
        assert (out[rows] == ro[rows]).all(), f"step {step} (j={j}): samples differ"
        np.testing.assert_array_equal(h, rh)
        np.testing.assert_array_equal(w, rw)


@pytest.mark.parametrize("precision,shadows", [("fp64", 0), ("fp32", 0), ("fp32", 1)])
def test_sampler_handle_matches_python_sampler(ftl, precision, shadows):
    """The handle API (ftl_sampler_create / set_factor / draw / destroy, for
    hosts that are not Python) gives the Python Sampler's draws bit for bit:
    factors copied from host arrays, injected uniforms, j excluded and none
    excluded; then factor 1 replaced through the device pointer and
    ftl_sampler_update."""
    import ctypes
    from fast_tensor_leverage_gb300 import _lib
    rng = np.random.default_rng(404)
    N, R, J = 3, 24, 3000
    dims = [700, 1100, 90]
    U = [np.ascontiguousarray(rng.normal(size=(d, R))) for d in dims]
    prec = _lib.PREC[precision]
    st = torch.cuda.current_stream().cuda_stream
    h = ctypes.c_void_p()
    dims_c = (ctypes.c_int64 * N)(*dims)
    _lib.call("ftl_sampler_create", N, dims_c, R, J, prec, shadows, ctypes.byref(h))
    try:
        for k in range(N):
            _lib.call("ftl_sampler_set_factor", h, k, U[k].ctypes.data, 1, st)
        for step, j in enumerate([1, 3, 1]):
            if step == 2:
                U[1] = np.ascontiguousarray(rng.normal(size=(dims[1], R)))
                # write the handle's device factor directly, then rebuild its tree
                dptr = ctypes.c_void_p()
                _lib.call("ftl_sampler_factor", h, 1, ctypes.byref(dptr))
                dev = torch.from_numpy(U[1]).cuda()
                torch.cuda.synchronize()
                view = type("DevView", (), {"__cuda_array_interface__": {
                    "shape": (dims[1], R), "typestr": "<f8", "data": (dptr.value, False), "version": 3}})()
                torch.as_tensor(view, device="cuda").copy_(dev)
                _lib.call("ftl_sampler_update", h, 1, st)
            dr = rng.random(2 * N * J)
            drd = torch.from_numpy(dr).cuda()
            smp = torch.zeros((N, J), dtype=torch.int64, device="cuda")
            hh = torch.empty((J, R), dtype=torch.float64, device="cuda")
            ww = torch.empty(J, dtype=torch.float64, device="cuda")
            _lib.call("ftl_sampler_draw", h, j, smp.data_ptr(), hh.data_ptr(), ww.data_ptr(), drd.data_ptr(),
                      0, 0, st)
            ref = ftl.Sampler([u.copy() for u in U], J, R, "efficient", precision=precision, overlap_computem=False)
            rs, rh, rw = ref.draw(j, dr)
            rows = [k for k in range(N) if k != j]
            assert torch.equal(smp[rows], rs[rows]), f"step {step}: samples differ"
            assert torch.equal(hh, rh) and torch.equal(ww, rw)
    finally:
        _lib.call("ftl_sampler_destroy", h)


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_sketched_least_squares_residual_ratio(ftl, precision):
    """The reference's accuracy benchmark (benchmarks/accuracy_tests_residual.py:
    21-79) restated as an assertion: solve min ||A x - b|| over the KRP A of
    three 40 x 8 factors (64,000 rows) from J = 4,000 leverage samples with
    their importance weights, and compare the full residual with the exact
    least-squares residual: the ratio is 1 + O(R / J); the oracle's samples
    give 1.0001 here, uniform sampling of the same size 1.007."""
    rng = np.random.default_rng(2024)
    N, I, R, J = 3, 40, 8, 4000
    U = [rng.normal(size=(I, R)) for _ in range(N)]
    for u in U:
        heavy = rng.choice(I, size=2, replace=False)
        u[heavy] *= 30.0
    A = np.einsum("ir,jr,kr->ijkr", *U).reshape(-1, R)
    b = A @ rng.normal(size=R) + 0.5 * rng.normal(size=A.shape[0]) * np.abs(A).mean()
    x_exact = np.linalg.lstsq(A, b, rcond=None)[0]
    r_exact = np.linalg.norm(A @ x_exact - b)
    s = ftl.Sampler([u.copy() for u in U], J, R, "efficient", precision=precision, seed=5)
    samples = np.zeros((N, J), dtype=np.uint64)
    h = np.zeros((J, R))
    w = np.zeros(J)
    s.KRPDrawSamples_materialize(N + 1, samples, h, w)
    rows = (samples[0].astype(np.int64) * I + samples[1].astype(np.int64)) * I + samples[2].astype(np.int64)
    np.testing.assert_allclose(h, A[rows], rtol=1e-12, atol=1e-12 * np.abs(A).max())
    sw = np.sqrt(w)
    x_s = np.linalg.lstsq(sw[:, None] * h, sw * b[rows], rcond=None)[0]
    ratio = np.linalg.norm(A @ x_s - b) / r_exact
    assert ratio < 1.01, ratio


@pytest.mark.parametrize("R,dims", [(32, [70_000, 33_000, 50_021]), (25, [40_000, 9_999, 30_000])])
def test_draw_variants_are_bit_identical(ftl, R, dims, tmp_path, monkeypatch):
    """Every compiled variant of the FP32 draw on wrapped-diagonal trees (1,
    2 or 3 samples descended per warp with the query weights in registers,
    3, 4 or 6 with them in shared memory) gives the same samples, h and
    weights bit for bit -- the autotuner only chooses the speed -- and the
    tuner times them, selects one and records it in its cache."""
    from fast_tensor_leverage_gb300 import _lib
    from fast_tensor_leverage_gb300 import autotune as AT
    monkeypatch.setenv("FTL_TUNE_CACHE", str(tmp_path / "tune.json"))
    rng = np.random.default_rng(R)
    U = [rng.normal(size=(n, R)) for n in dims]
    N, J = len(dims), 3001
    s = ftl.Sampler(U, J, R, "efficient", precision="fp32", seed=4, autotune=False)
    n, dflt = AT.variants(AT.FAMILY_DRAW, R, _lib.PREC["fp32"])
    assert n == 6
    outs = []
    for v in range(n):
        AT.set_variant(AT.FAMILY_DRAW, R, _lib.PREC["fp32"], v)
        for j in (N + 1, 1):
            s.counter = 0
            smp, h, w = s.draw(j)
            outs.append((v, j, smp.clone(), h.clone(), w.clone()))
    for v, j, smp, h, w in outs:
        ref = next(o for o in outs if o[0] == 0 and o[1] == j)
        assert torch.equal(smp, ref[2]) and torch.equal(h, ref[3]) and torch.equal(w, ref[4]), (v, j)
    res = AT.tune_draw(s, reps=3, warmup=1)
    assert set(res["ms"]) == set(range(6)) and AT.get_variant(AT.FAMILY_DRAW, R, 1) == res["variant"]
    assert AT.load_cache()[AT.cache_key(AT.gpu_name(), AT.FAMILY_DRAW, R, 1)]["variant"] == res["variant"]
    AT.set_variant(AT.FAMILY_DRAW, R, _lib.PREC["fp32"], -1)
