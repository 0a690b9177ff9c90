"""CPU: argument validation of the reference-shaped Python API happens before
any device work, so it is testable without a GPU."""
import numpy as np
import pytest

import fast_tensor_leverage_gb300 as ftl
from fast_tensor_leverage_gb300 import _device as D


def test_unsupported_sampler_type_raises():
    U = [np.zeros((10, 4)) for _ in range(3)]
    with pytest.raises(ValueError, match="Unsupported"):
        ftl.Sampler(U, 100, 4, "larsen_kolda")


def test_bad_shapes_raise():
    with pytest.raises(ValueError):
        ftl.Sampler([np.zeros((10, 5))], 100, 4, "efficient")
    with pytest.raises(ValueError):
        ftl.Sampler([np.zeros((10, 4))] * 17, 100, 4, "efficient")
    with pytest.raises(ValueError):
        ftl.Sampler([np.zeros((10, 4))], 0, 4, "efficient")
    with pytest.raises(ValueError):
        ftl.Sampler([np.zeros((10, 200))], 10, 200, "efficient")
    with pytest.raises(ValueError):
        ftl.Sampler([np.zeros((10, 4))], 10, 4, "efficient", precision="fp16")


def test_output_arrays_are_checked_not_copied():
    a = np.zeros((3, 10), dtype=np.int64)
    with pytest.raises(TypeError):
        D.require_numpy_out(a, np.uint64, "samples")
    b = np.zeros((10, 3), dtype=np.uint64).T
    with pytest.raises(ValueError):
        D.require_numpy_out(b, np.uint64, "samples")
    c = np.zeros(5, dtype=np.uint64)
    with pytest.raises(ValueError):
        D.require_numpy_out(c, np.uint64, "samples", min_size=30)
    ok = np.zeros((3, 10), dtype=np.uint64)
    assert D.require_numpy_out(ok, np.uint64, "samples", min_size=30) is ok


def test_no_cpu_fallback_without_cuda():
    import torch
    if torch.cuda.is_available():
        pytest.skip("CUDA present")
    with pytest.raises(RuntimeError, match="CUDA"):
        ftl.Sampler([np.ones((10, 4))] * 2, 10, 4, "efficient")
