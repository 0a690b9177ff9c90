"""GPU: results of the reference-shaped draw calls are copied by DMA into
page-locked caller arrays (registered on first use, released when the
array is garbage collected) with the same values as the device results."""
import gc

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


def test_materialize_into_page_locked_arrays(ftl):
    from fast_tensor_leverage_gb300 import _device as D
    rng = np.random.default_rng(3)
    N, I, R, J = 3, 20000, 32, 40000
    U = [rng.normal(size=(I, R)) for _ in range(N)]
    s = ftl.Sampler(U, J, R, "efficient", precision="fp32", seed=3)
    draws = rng.random(2 * N * J)
    n0 = len(D.HOST_REGISTRY)
    samples = np.zeros((N, J), dtype=np.uint64)     # 0.96 MB: page-locked on first use
    h = np.zeros((J, R))                             # 10 MB
    w = np.zeros(J)                                  # 320 KB
    tiny = np.zeros(100)                             # below the registry's threshold: stays pageable
    for rep in range(2):
        samples[:] = 0
        h[:] = 0
        w[:] = 0
        s.KRPDrawSamples_materialize(N + 1, samples, h, w, draws=draws)
        assert len(D.HOST_REGISTRY) == n0 + 3 and not D.HOST_REGISTRY.pinned(tiny)
        assert np.array_equal(samples.view(np.int64), s.samples_dev.cpu().numpy())
        assert np.array_equal(h, s.h_dev.cpu().numpy()) and np.array_equal(w, s.weights_dev.cpu().numpy())
    # a view into the registered array is copied into the same pages
    h2 = h[: J // 2]
    s.KRPDrawSamples(1, samples, draws=draws)
    assert len(D.HOST_REGISTRY) == n0 + 3 and h2.base is h
    del h, h2
    gc.collect()
    assert len(D.HOST_REGISTRY) == n0 + 2
    del samples, w
    gc.collect()
    assert len(D.HOST_REGISTRY) == n0
