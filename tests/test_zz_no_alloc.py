"""GPU: ftl_krp_draw_static, the draw entry point that allocates nothing, for
callers that cannot call cudaMalloc (hosts whose device memory is reserved up
front by another runtime, or request paths that must not allocate because
cudaMalloc can synchronise the device or fail under memory pressure).  Its
scratch lives in a fixed static device array.

Called through the C ABI and compared with ftl_krp_draw on the same inputs,
twice in a row (the array keeps the previous call's contents), plus the size
limit.  Tolerance as in the other FP64 parity tests: identical sample indices
and h, weights within 1e-9 relative (the two entry points run the same
kernels, so they agree exactly in practice).

This file is named so pytest collects it last.
"""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ftl():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import fast_tensor_leverage_gb300 as m
    return m


def _static_draw(s, j, draws_dev, samples, h, w):
    from fast_tensor_leverage_gb300 import _lib
    N = s.N
    dims = (ctypes.c_int64 * N)(*s.dims)
    U = (ctypes.c_void_p * N)(*[u.data_ptr() for u in s.U])
    G = (ctypes.c_void_p * N)(*[t.data_ptr() for t in s.trees])
    _lib.call("ftl_krp_draw_static", N, s.R, s.J, s._prec, dims, U, G, j,
              samples.data_ptr(), h.data_ptr(), w.data_ptr(), draws_dev.data_ptr(), 0, 0,
              torch.cuda.current_stream().cuda_stream)


def _regular_draw(s, j, draws_dev, samples, h, w):
    from fast_tensor_leverage_gb300 import _lib
    _lib.call("ftl_krp_draw", ctypes.byref(s._plan), j, samples.data_ptr(), h.data_ptr(),
              w.data_ptr(), draws_dev.data_ptr(), 0, 0, torch.cuda.current_stream().cuda_stream)


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_static_draw_matches_regular_draw_twice(ftl, precision):
    rng = np.random.default_rng(77)
    N, R, J = 3, 32, 4000
    dims = [3000, 1001, 2048]
    U = [rng.normal(size=(n, R)) for n in dims]
    s = ftl.Sampler(U, J, R, "efficient", precision=precision)
    dev = s.device
    for call, j in enumerate([N + 1, 1]):  # two calls in a row, different set-ups
        draws = torch.from_numpy(rng.random(2 * N * J)).to(dev)
        outs = []
        for fn in (_regular_draw, _static_draw):
            samples = torch.zeros((N, J), dtype=torch.int64, device=dev)
            h = torch.zeros((J, R), dtype=torch.float64, device=dev)
            w = torch.zeros(J, dtype=torch.float64, device=dev)
            fn(s, j, draws, samples, h, w)
            torch.cuda.synchronize()
            outs.append((samples.cpu().numpy(), h.cpu().numpy(), w.cpu().numpy()))
        (s0, h0, w0), (s1, h1, w1) = outs
        assert np.array_equal(s0, s1), f"call {call}: sample indices differ"
        assert np.array_equal(h0, h1), f"call {call}: h differs"
        np.testing.assert_allclose(w1, w0, rtol=1e-9, atol=0)


def test_static_draw_rejects_oversized_configuration(ftl):
    from fast_tensor_leverage_gb300 import _lib
    N, R = 16, 128  # 16 eigen trees of 255 x 8256 FP64 values: far beyond the array
    dims = (ctypes.c_int64 * N)(*([1000] * N))
    ptrs = (ctypes.c_void_p * N)(*([1] * N))
    with pytest.raises(_lib.FTLError) as ei:
        _lib.call("ftl_krp_draw_static", N, R, 100, 0, dims, ptrs, ptrs, N + 1,
                  1, None, None, None, 0, 0, None)
    assert ei.value.status == 1
    assert "static array" in str(ei.value)
