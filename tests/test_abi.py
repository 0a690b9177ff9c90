"""CPU: the C-ABI library loads and exports every entry point include/ftl.h
declares; host-only entry points (geometry, sizes, argument validation) work
without a GPU and agree with the oracle."""
import ctypes
import re

import numpy as np
import pytest

from fast_tensor_leverage_gb300 import _lib
from oracle import oracle as O
from tests.conftest import REPO


def declared_functions():
    text = (REPO / "include" / "ftl.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(ftl_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_entry_points():
    names = declared_functions()
    assert "ftl_krp_draw" in names and "ftl_tree_build" in names and len(names) >= 10


def test_library_exports_every_declared_symbol():
    L = ctypes.CDLL(str(_lib.LIB_PATH))
    missing = [n for n in declared_functions() if not hasattr(L, n)]
    assert not missing, f"missing exports: {missing}"
    # and the Python binding covers all of them
    assert set(declared_functions()) <= set(_lib.SIGNATURES), \
        set(declared_functions()) - set(_lib.SIGNATURES)


@pytest.mark.parametrize("n,F", [(1, 1), (5, 8), (8, 8), (1000, 8), (1001, 8), (520, 8),
                                 (13, 1), (8388608, 32), (4800000, 25), (65536, 64), (777, 16)])
def test_geometry_matches_oracle(n, F):
    g = _lib.tree_geometry(n, F)
    o = O.geometry(n, F)
    for k in O.GEOM_KEYS:
        assert getattr(g, k) == o[k], k


def test_sizes():
    R = 32
    P = R * (R + 1) // 2
    # FP32 nodes at 16 < R <= 32 use the wrapped-diagonal layout (544 values)
    assert _lib.tree_bytes(2**23, 32, R, _lib.PREC["fp32"]) == (2 * 2**18 - 1) * 544 * 4
    assert _lib.tree_bytes(2**10, 16, 16, _lib.PREC["fp32"]) == (2 * 2**6 - 1) * 136 * 4
    assert _lib.tree_bytes(1001, 8, 8, _lib.PREC["fp64"]) == (2 * 126 - 1) * 36 * 8
    e, m, l, p = _lib.plan_sizes(3, R, _lib.PREC["fp64"])
    assert e == 3 * (2 * R - 1) * P * 8 and l == 4 * R * 8 and p == 544 * 4  # pinv32: one FP32 node
    assert m >= 5 * R * R * 8


@pytest.mark.parametrize("call", [
    lambda: _lib.call("ftl_tree_build", None, 10, 8, 8, 0, None, None),
    lambda: _lib.call("ftl_tree_build", 1, 10, 0, 8, 0, 1, None),
    lambda: _lib.call("ftl_tree_build", 1, 10, 129, 8, 0, 1, None),
    lambda: _lib.call("ftl_tree_build", 1, 10, 8, 8, 7, 1, None),
    lambda: _lib.call("ftl_tree_build", 16, 10, 8, 8, 0, 24, None),   # unaligned tree
    lambda: _lib.call("ftl_tree_sample", 24, 0, 16, 10, 8, 8, 16, 16, 16, 16, 5, None),
    lambda: _lib.call("ftl_tree_sample", 1, 0, 1, 10, 8, 0, 1, 1, 1, 1, 5, None),
    lambda: _lib.tree_geometry(0, 8),
    lambda: _lib.plan_sizes(0, 8, 0),
    lambda: _lib.plan_sizes(17, 8, 0),
    lambda: _lib.call("ftl_krp_draw", None, 0, 1, None, None, None, 0, 0, None),
])
def test_invalid_arguments_return_ftl_e_arg(call):
    with pytest.raises(_lib.FTLError) as ei:
        call()
    assert ei.value.status == 1  # FTL_E_ARG, raised before any CUDA call


def test_plan_validation_rejects_bad_plans():
    plan = _lib.KRPPlan()
    plan.N, plan.R, plan.J, plan.prec = 3, 8, 100, 0
    with pytest.raises(_lib.FTLError) as ei:  # null workspaces
        _lib.call("ftl_krp_compute_m", ctypes.byref(plan), 0, None)
    assert ei.value.status == 1
    plan.N = 0
    with pytest.raises(_lib.FTLError):
        _lib.call("ftl_krp_compute_m", ctypes.byref(plan), 0, None)


def test_sampler_handle_rejects_bad_shapes_without_touching_the_device():
    """ftl_sampler_create validates its arguments before any allocation."""
    h = ctypes.c_void_p(12345)
    dims = (ctypes.c_int64 * 3)(10, 20, 30)
    L = _lib.lib()
    for N, R, J, prec in [(0, 8, 10, 0), (3, 0, 10, 0), (3, 8, 0, 0), (3, 8, 10, 7), (3, 200, 10, 0)]:
        assert L.ftl_sampler_create(N, dims, R, J, prec, 0, ctypes.byref(h)) == 1
        assert h.value is None
    assert L.ftl_sampler_destroy(None) == 0


def test_sparse_and_als_handles_reject_bad_arguments_without_touching_the_device():
    """ftl_sparse_create / ftl_als_create validate before any allocation or copy."""
    L = _lib.lib()
    X = ctypes.c_void_p(7)
    idx = (ctypes.c_uint32 * 6)(0, 0, 1, 1, 2, 2)
    vals = (ctypes.c_double * 3)(1.0, 2.0, 3.0)
    dims = (ctypes.c_int64 * 2)(3, 3)
    for nnz, N in [(0, 2), (3, 1), (3, 17)]:
        assert L.ftl_sparse_create(idx, vals, nnz, N, dims, 1, None, ctypes.byref(X)) == 1
        assert X.value is None
    bad_dims = (ctypes.c_int64 * 2)(3, 0)
    assert L.ftl_sparse_create(idx, vals, 3, 2, bad_dims, 1, None, ctypes.byref(X)) == 1
    A = ctypes.c_void_p(9)
    assert L.ftl_als_create(None, 8, 100, 0, 1, ctypes.byref(A)) == 1
    assert L.ftl_sparse_destroy(None) == 0 and L.ftl_als_destroy(None) == 0


@pytest.mark.parametrize("R,prec", [(8, "fp32"), (16, "fp32"), (17, "fp32"), (25, "fp32"), (32, "fp32"),
                                    (33, "fp32"), (32, "fp64"), (5, "fp64"), (128, "fp32")])
def test_node_layout_positions(R, prec):
    """Every upper-triangle element has its own position inside the node
    stride; the wrapped-diagonal layout (FP32, 16 < R <= 32) puts (a, b) at
    diagonal (b - a) mod 32 of row a (or of row b past distance 16)."""
    import numpy as np
    lay, S, pos = _lib.node_layout(R, _lib.PREC[prec])
    P = R * (R + 1) // 2
    assert pos.shape == (P,) and len(set(pos.tolist())) == P and pos.min() >= 0 and pos.max() < S
    assert S * (4 if prec == "fp32" else 8) % 16 == 0
    if prec == "fp32" and 16 < R <= 32:
        assert lay == 1 and S == 544
        e = 0
        for a in range(R):
            for b in range(a, R):
                d = (b - a) % 32
                r, dd = (a, d) if d <= 16 else (b, 32 - d)
                want = ((dd // 4) * 32 + r) * 4 + dd % 4 if dd < 16 else 512 + r
                assert pos[e] == want
                e += 1
    else:
        assert lay == 0 and np.array_equal(pos, np.arange(P))
