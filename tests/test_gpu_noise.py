"""GPU: counter-hash Gaussian noise on black-box tensors (ftl_noise_*):
entries, fibers and the sampled MTTKRP term against a numpy restatement of
the noise function (FP64 Box-Muller from the same 24-bit uniforms; the
device evaluates it in FP32, so values agree to about 1e-6 relative), the
noise's first two moments, and CP-ALS on a noisy low-rank tensor."""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

M64 = (1 << 64) - 1


@pytest.fixture(scope="module")
def ftl():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import fast_tensor_leverage_gb300 as m
    return m


def noise_np(L, seed):
    """Z at linear indices L (uint64 array): SplitMix64 finaliser of
    L * 0x9E3779B97F4A7C15 + seed, u1 = ((z >> 40) + 1) 2^-24, u2 = ((z >> 16)
    mod 2^24) 2^-24, Z = sqrt(-2 ln u1) cos(2 pi u2)."""
    z = [((int(l) * 0x9E3779B97F4A7C15) + seed) & M64 for l in np.asarray(L).reshape(-1)]
    out = np.empty(len(z))
    for n, x in enumerate(z):
        x = ((x ^ (x >> 30)) * 0xBF58476D1CE4E5B9) & M64
        x = ((x ^ (x >> 27)) * 0x94D049BB133111EB) & M64
        x ^= x >> 31
        u1 = ((x >> 40) + 1) / 16777216.0
        u2 = ((x >> 16) & 0xFFFFFF) / 16777216.0
        out[n] = np.sqrt(-2.0 * np.log(u1)) * np.cos(2.0 * np.pi * u2)
    return out.reshape(np.shape(L))


def linear(idx, dims):
    L = np.zeros(idx.shape[0], dtype=object)
    for k, d in enumerate(dims):
        L = L * d + idx[:, k].astype(object)
    return L


def test_noise_entries_and_fibers(ftl):
    from fast_tensor_leverage_gb300 import _lib
    rng = np.random.default_rng(1)
    dims = [65536, 65536, 65536, 65536]   # prod = 2^64: linear indices use every bit
    dims_c = (ctypes.c_int64 * 4)(*dims)
    idx = rng.integers(0, 65536, size=(3000, 4)).astype(np.uint64)
    idx[0] = [65535, 65535, 65535, 65535]
    idx[1] = 0
    out = torch.zeros(3000, dtype=torch.float64, device="cuda")
    idx_d = torch.from_numpy(idx.view(np.int64)).cuda()
    _lib.call("ftl_noise_add_at", dims_c, 4, 12345, 2.0, idx_d.data_ptr(), 1, 3000, out.data_ptr(),
              torch.cuda.current_stream().cuda_stream)
    ref = 2.0 * noise_np(linear(idx, dims), 12345)
    np.testing.assert_allclose(out.cpu().numpy(), ref, rtol=2e-6, atol=2e-6)
    # fibers along mode 2 at 5 samples
    fib = torch.zeros((5, 65536), dtype=torch.float64, device="cuda")
    _lib.call("ftl_noise_add_fibers", dims_c, 4, 12345, 1.0, idx_d.data_ptr(), 5, 2, fib.data_ptr(),
              torch.cuda.current_stream().cuda_stream)
    for z in range(5):
        cols = rng.integers(0, 65536, size=40)
        t = np.repeat(idx[z:z + 1], 40, axis=0)
        t[:, 2] = cols
        np.testing.assert_allclose(fib[z].cpu().numpy()[cols], noise_np(linear(t, dims), 12345), rtol=2e-6,
                                   atol=2e-6)


def test_noise_moments(ftl):
    from fast_tensor_leverage_gb300 import _lib
    n = 1 << 22
    dims = [1 << 11, 1 << 11]
    idx = torch.stack(torch.meshgrid(torch.arange(1 << 11), torch.arange(1 << 11), indexing="ij"), -1).reshape(-1, 2)
    idx = idx.to(torch.int64).cuda()
    out = torch.zeros(n, dtype=torch.float64, device="cuda")
    _lib.call("ftl_noise_add_at", (ctypes.c_int64 * 2)(*dims), 2, 7, 1.0, idx.data_ptr(), 1, n, out.data_ptr(),
              torch.cuda.current_stream().cuda_stream)
    assert abs(float(out.mean())) < 5.0 / np.sqrt(n)
    assert abs(float(out.var()) - 1.0) < 5.0 * np.sqrt(2.0 / n)
    assert abs(float((out ** 3).mean())) < 0.01 and abs(float((out ** 4).mean()) - 3.0) < 0.03


def test_noise_sampled_mttkrp_matches_numpy(ftl):
    """out[i, c] += sigma sum_u w[rep_u] cnt_u Z(i, s_u) h[rep_u, c] with
    repeated samples collapsed by urep/ucnt, on top of existing values."""
    from fast_tensor_leverage_gb300 import _lib
    rng = np.random.default_rng(5)
    dims = [37, 200, 29, 13]
    N, j, R, J = 4, 1, 7, 500
    S = np.stack([rng.integers(0, d, size=J) for d in dims]).astype(np.uint64)  # N x J
    nu = 300
    urep = np.sort(rng.choice(J, size=nu, replace=False)).astype(np.int32)
    ucnt = rng.integers(1, 4, size=nu).astype(np.int32)
    w = rng.random(J) + 0.5
    h = rng.normal(size=(J, R))
    sigma = 0.3
    out0 = rng.normal(size=(dims[j] + 3, R))
    out = torch.from_numpy(out0.copy()).cuda()
    st = torch.cuda.current_stream().cuda_stream
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    S_d, urep_d, ucnt_d, w_d, h_d = dev(S.view(np.int64)), dev(urep), dev(ucnt), dev(w), dev(h)
    nuniq = torch.tensor([nu], dtype=torch.int64, device="cuda")
    _lib.call("ftl_noise_sampled_mttkrp", (ctypes.c_int64 * N)(*dims), N, j, 99, sigma, S_d.data_ptr(), J,
              urep_d.data_ptr(), ucnt_d.data_ptr(), nuniq.data_ptr(), J, w_d.data_ptr(), h_d.data_ptr(), R,
              out.data_ptr(), dims[j] + 3, st)
    ref = out0.copy()
    for u in range(nu):
        rep = urep[u]
        t = np.repeat(S[:, rep][None, :], dims[j], axis=0)
        t[:, j] = np.arange(dims[j])
        Z = noise_np(linear(t.astype(np.uint64), dims), 99)
        ref[:dims[j]] += sigma * w[rep] * ucnt[u] * np.outer(Z, h[rep])
    np.testing.assert_allclose(out.cpu().numpy(), ref, rtol=1e-5, atol=1e-5 * np.abs(ref).max())


def test_als_on_noisy_low_rank_tensor(ftl):
    """CP-ALS against a rank-4 tensor with noise at SNR 20 dB, started from
    the true factors: the expected fit of the true factors is 1 - sqrt(1 /
    101), and two sampled sweeps (FP64 and mixed sampling) stay within 1e-3
    of it -- the noise enters the sampled MTTKRP at its true scale (a wrong
    scale would pull the factors off by far more).  Without noise the same
    sweeps keep the fit above 0.999."""
    from fast_tensor_leverage_gb300.serving import GaussianFactors
    dims, Rt, J = [300, 250, 280], 4, 8000
    U_true = GaussianFactors(dims, Rt, seed=3).materialize(torch.device("cuda", 0))
    target = 1.0 - np.sqrt(1.0 / 101.0)
    for snr in (None, 20.0):
        rhs_ten = ftl.LowRankTensor(Rt, 10000, [u.clone() for u in U_true], sync_host=False)
        if snr is not None:
            rhs_ten.set_noise_snr(snr, seed=8)
        rhs = type("Rhs", (), {})()
        rhs.ten = rhs_ten
        for prec in ("fp64", "fp32"):
            lhs = ftl.PyLowRank(dims, Rt, seed=7, sync_host=False)
            for k in range(3):
                lhs.ten.U_dev[k].copy_(U_true[k])
            lhs.ten.renormalize_columns(-1)
            als = ftl.ALS(lhs.ten, rhs_ten)
            als.initialize_ds_als(J, "efficient", precision=prec, seed=11)
            for _ in range(2):
                for jj in range(3):
                    als.execute_ds_als_update(jj, True, True)
            fit = lhs.compute_exact_fit(rhs)
            if snr is None:
                assert fit > 0.999, (prec, fit)
            else:
                assert abs(fit - target) < 1e-3, (prec, fit, target)
