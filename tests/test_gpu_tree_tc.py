"""GPU: partition trees whose leaf Grams run on the tensor cores (tcgen05,
TMA-fed) -- tree precisions tf32x3 (hi/lo split of the FP32-rounded factor,
three products, FP32 accumulation) and bf16 (BF16-rounded factor, FP32
accumulation) -- against the FP64 Grams of the same factor.

Tolerances (entrywise, relative to sqrt(G_aa G_bb) of the FP64 node):
  * tf32x3 (and the FP32 CUDA-core build): 6e-6 -- each product carries
    about 2^-21 relative error, and the FP32 sums over a leaf's 32 rows and
    up to 20 levels above it add about 50 roundings of 2^-24 on a root path;
  * bf16: 1.6e-2 -- each factor entry is rounded to 8 significant bits.
The FP32 copy of the factor written by the same pass equals the factor
rounded to nearest FP32 exactly, and no bounded device wait ran out."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

TOL = {"tf32x3": 6e-6, "bf16": 1.6e-2, "fp32": 6e-6}


@pytest.fixture(scope="module")
def ftl():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import fast_tensor_leverage_gb300 as m
    return m


def build(ftl, U, R, F, precision, with_copy=True):
    from fast_tensor_leverage_gb300 import _lib
    n = U.shape[0]
    t = ftl.PartitionTree(n, F, 1, R, precision=precision)
    Ud = torch.from_numpy(U).cuda()
    U32 = torch.empty((n, R), dtype=torch.float32, device="cuda") if with_copy else None
    _lib.call("ftl_tree_build_ex", Ud.data_ptr(), n, R, F, _lib.PREC[precision], t.G.data_ptr(),
              U32.data_ptr() if with_copy else None, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    return t.get_G(), (U32.cpu().numpy() if with_copy else None)


def check_close(G, G64, R, tol):
    iu = np.triu_indices(R)
    d = np.zeros((G64.shape[0], R))
    for k, (a, b) in enumerate(zip(*iu)):
        if a == b:
            d[:, a] = G64[:, k]
    scale = np.sqrt(np.maximum(d[:, iu[0]] * d[:, iu[1]], 1e-300))
    err = np.abs(G - G64) / scale
    assert np.nanmax(err) <= tol, (np.nanmax(err), np.unravel_index(np.nanargmax(err), err.shape))


@pytest.mark.parametrize("n,R,F", [
    (1 << 16, 32, 32),        # tensor-map copies, wrapped-diagonal nodes, complete tree
    (100_003, 32, 32),        # partial last leaf and tile
    (50_000, 25, 25),         # odd R: untiled bulk copies with a ragged tail, R < 32
    (40_000, 16, 16),         # packed nodes (R <= 16)
    (7_777, 8, 8),
    (20, 32, 20),             # F = n < R: one leaf
    (1000, 24, 12),           # F < R
    (8, 4, 4),                # R = 4: 32-byte rows, box taller than the factor
    (1000, 4, 4),
])
@pytest.mark.parametrize("precision", ["tf32x3", "bf16"])
def test_tensor_core_tree_matches_fp64(ftl, n, R, F, precision):
    from fast_tensor_leverage_gb300 import _lib
    rng = np.random.default_rng(n + R)
    U = rng.normal(size=(n, R))
    U[rng.random(n) < 0.01] *= 100.0
    G64, _ = build(ftl, U, R, F, "fp64", with_copy=False)
    G, U32 = build(ftl, U, R, F, precision)
    check_close(G, G64, R, TOL[precision])
    assert np.array_equal(U32, U.astype(np.float32))
    assert _lib.device_status() == 0


def test_cuda_core_fp32_tree_writes_the_fp32_copy(ftl):
    """The FP32 CUDA-core build (integer FP64 -> FP32 rounding) writes the
    same FP32 copy and agrees with the FP64 tree."""
    rng = np.random.default_rng(5)
    n, R = 30_000, 32
    U = rng.normal(size=(n, R))
    G64, _ = build(ftl, U, R, R, "fp64", with_copy=False)
    G, U32 = build(ftl, U, R, R, "fp32")
    check_close(G, G64, R, TOL["fp32"])
    assert np.array_equal(U32, U.astype(np.float32))


def test_fp64_to_fp32_rounding_edge_values(ftl):
    """Integer rounding of the leaf builds at the edges: halfway cases (ties
    to even), values next to the FP32 range limits, zeros of both signs and
    FP64 subnormals, against numpy's round-to-nearest conversion."""
    R = 8
    vals = [0.0, -0.0, 1.0, -1.0, 1.0 + 2.0 ** -24, 1.0 + 3 * 2.0 ** -24, 1.0 + 2.0 ** -24 + 2.0 ** -40,
            np.nextafter(1.0, 2.0), 3.4028234663852886e38, 1.1754943508222875e-38, 1.0e-39, 5e-324,
            -2.5e-310, 1.0e30, -7.123456789e-20, 0.1, 1.0 / 3.0]
    U = np.zeros((64, R))
    U.flat[: len(vals)] = vals
    for precision in ("fp32", "tf32x3"):
        _, U32 = build(ftl, U, R, R, precision)
        assert np.array_equal(U32.view(np.uint32), U.astype(np.float32).view(np.uint32)), precision


def test_sampler_tensor_core_trees_draw_like_fp64(ftl):
    """A sampler on tf32x3 trees agrees with the FP64 sampler's indices on
    nearly every sample and its weights to 1e-3, on a well-conditioned KRP."""
    rng = np.random.default_rng(3)
    N, I, R, J = 3, 5000, 32, 4000
    U = [rng.normal(size=(I, R)) for _ in range(N)]
    draws = rng.random(2 * N * J)
    out = {}
    for precision in ("fp64", "tf32x3", "bf16"):
        s = ftl.Sampler(U, J, R, "efficient", precision=precision)
        samples = np.zeros((N, J), dtype=np.uint64)
        h = np.zeros((J, R))
        w = np.zeros(J)
        s.KRPDrawSamples_materialize(N + 1, samples, h, w, draws=draws)
        out[precision] = (samples, w)
    agree = (out["tf32x3"][0] == out["fp64"][0]).all(axis=0)
    assert agree.mean() >= 0.99, agree.mean()
    np.testing.assert_allclose(out["tf32x3"][1][agree], out["fp64"][1][agree], rtol=1e-3)
    agree_bf = (out["bf16"][0] == out["fp64"][0]).all(axis=0)
    assert agree_bf.mean() >= 0.5, agree_bf.mean()
