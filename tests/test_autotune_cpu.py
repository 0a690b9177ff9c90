"""CPU: the autotuner's cache and selection logic, and the per-device
variant table of the C ABI (ftl_tune_*), without a GPU."""
import json

import pytest

from fast_tensor_leverage_gb300 import _lib
from fast_tensor_leverage_gb300 import autotune as AT


def test_cache_round_trip_and_merge(tmp_path):
    path = tmp_path / "t.json"
    assert AT.load_cache(path) == {}
    k1 = AT.cache_key("NVIDIA GB300", AT.FAMILY_DRAW, 32, 1)
    k2 = AT.cache_key("NVIDIA GB300", AT.FAMILY_DRAW, 25, 1)
    assert k1 != k2 and "R=32" in k1 and "draw" in k1
    AT.save_cache({k1: {"variant": 2, "ms": {"0": 1.0}}}, path)
    AT.save_cache({k2: {"variant": 0}}, path)
    d = AT.load_cache(path)
    assert d[k1]["variant"] == 2 and d[k2]["variant"] == 0
    path.write_text("not json")
    assert AT.load_cache(path) == {}


def test_choose_prefers_default_within_noise():
    assert AT.choose({0: 1.00, 1: 0.90, 2: 0.95}, default=2) == 1
    assert AT.choose({0: 1.00, 1: 0.995, 2: 1.0}, default=2) == 2   # within 1%: keep the default
    assert AT.choose({0: 0.5}, default=0) == 0


def test_variant_table_through_the_c_abi():
    # FP32 trees at 16 < R <= 32 have six draw variants, default 2
    n, d = AT.variants(AT.FAMILY_DRAW, 32, _lib.PREC["fp32"])
    assert (n, d) == (6, 2)
    assert AT.variants(AT.FAMILY_DRAW, 25, _lib.PREC["tf32x3"]) == (6, 2)
    assert AT.variants(AT.FAMILY_DRAW, 64, _lib.PREC["fp32"]) == (1, 0)
    assert AT.variants(AT.FAMILY_DRAW, 32, _lib.PREC["fp64"]) == (1, 0)
    assert AT.get_variant(AT.FAMILY_DRAW, 32, 1) == 2
    AT.set_variant(AT.FAMILY_DRAW, 32, 1, 0)
    assert AT.get_variant(AT.FAMILY_DRAW, 32, 1) == 0
    assert AT.get_variant(AT.FAMILY_DRAW, 20, 2) == 0      # same class: FP32 nodes, DIAG32 layout
    AT.set_variant(AT.FAMILY_DRAW, 32, 1, -1)               # back to the default
    assert AT.get_variant(AT.FAMILY_DRAW, 32, 1) == 2
    with pytest.raises(_lib.FTLError):
        AT.set_variant(AT.FAMILY_DRAW, 32, 1, 6)
    with pytest.raises(_lib.FTLError):
        AT.set_variant(7, 32, 1, 0)
