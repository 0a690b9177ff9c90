"""ctypes binding of libftl_gb300.so (C ABI declared in include/ftl.h).

The library is loaded from the package's in-tree _build/ folder.  There is no
CPU fallback: if the library is missing or CUDA is unavailable, using the
package raises.
"""
from __future__ import annotations

import ctypes
import os
from pathlib import Path

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "_build" / "libftl_gb300.so"

FTL_OK = 0
FTL_E_TIMEOUT = 4
FTL_E_CANCELLED = 5
STATUS_NAMES = {
    1: "FTL_E_ARG",
    2: "FTL_E_OOM",
    3: "FTL_E_CUDA",
    4: "FTL_E_TIMEOUT",
    5: "FTL_E_CANCELLED",
    6: "FTL_E_UNSUPPORTED",
}
# tree precisions: fp64 and fp32 trees computed in their precision; tf32x3
# and bf16 trees store FP32 nodes whose leaf Grams come from the tensor cores
PREC = {"fp64": 0, "fp32": 1, "tf32x3": 2, "bf16": 3}


def storage_prec(prec: int) -> int:
    """The node precision plans and draws see (FP64 or FP32)."""
    return 0 if prec == 0 else 1
MAX_MODES = 16
MAX_RANK = 128


class FTLError(RuntimeError):
    """A libftl_gb300 call returned a non-zero status."""

    def __init__(self, status: int, message: str):
        self.status = status
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")


class TreeGeom(ctypes.Structure):
    _fields_ = [(k, ctypes.c_int64) for k in (
        "n", "F", "leaf_count", "node_count", "lfill_level", "lfill_count", "total_levels",
        "nodes_upto_lfill", "nodes_before_lfill", "complete_level_offset")]


class KRPPlan(ctypes.Structure):
    _fields_ = [
        ("N", ctypes.c_int),
        ("R", ctypes.c_int),
        ("J", ctypes.c_int64),
        ("prec", ctypes.c_int),
        ("dims", ctypes.c_int64 * MAX_MODES),
        ("U", ctypes.c_void_p * MAX_MODES),
        ("gram_G", ctypes.c_void_p * MAX_MODES),
        ("eig_G", ctypes.c_void_p),
        ("M", ctypes.c_void_p),
        ("lambda_", ctypes.c_void_p),
        ("pinv32", ctypes.c_void_p),
        ("U32", ctypes.c_void_p * MAX_MODES),
    ]


_lib = None

_P = ctypes.c_void_p
_I64 = ctypes.c_int64
_INT = ctypes.c_int
_U32 = ctypes.c_uint32
_U64 = ctypes.c_uint64
_SZP = ctypes.POINTER(ctypes.c_size_t)

SIGNATURES = {
    "ftl_last_error": ([], ctypes.c_char_p),
    "ftl_abi_version": ([], _INT),
    "ftl_sampler_create": ([_INT, _P, _INT, _I64, _INT, _INT, ctypes.POINTER(_P)], _INT),
    "ftl_sampler_set_factor": ([_P, _INT, _P, _INT, _P], _INT),
    "ftl_sampler_update": ([_P, _INT, _P], _INT),
    "ftl_sampler_factor": ([_P, _INT, ctypes.POINTER(_P)], _INT),
    "ftl_sampler_draw": ([_P, ctypes.c_uint32, _P, _P, _P, _P, ctypes.c_uint64, ctypes.c_uint64, _P], _INT),
    "ftl_sampler_destroy": ([_P], _INT),
    "ftl_sparse_create": ([_P, _P, _I64, _INT, _P, _INT, _P, ctypes.POINTER(_P)], _INT),
    "ftl_sparse_normsq": ([_P, ctypes.POINTER(ctypes.c_double)], _INT),
    "ftl_sparse_destroy": ([_P], _INT),
    "ftl_als_create": ([_P, _INT, _I64, _INT, ctypes.c_uint64, ctypes.POINTER(_P)], _INT),
    "ftl_als_set_factor": ([_P, _INT, _P, _INT, _P], _INT),
    "ftl_als_set_sigma": ([_P, _P, _INT, _P], _INT),
    "ftl_als_factor": ([_P, _INT, ctypes.POINTER(_P)], _INT),
    "ftl_als_sigma": ([_P, ctypes.POINTER(_P)], _INT),
    "ftl_als_samples": ([_P, ctypes.POINTER(_P)], _INT),
    "ftl_als_renormalize": ([_P, _INT, _P], _INT),
    "ftl_als_init_rrf": ([_P, ctypes.c_uint64, _P], _INT),
    "ftl_als_update": ([_P, _INT, _INT, _INT, _P, _P], _INT),
    "ftl_als_fit": ([_P, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double), _P], _INT),
    "ftl_als_destroy": ([_P], _INT),
    "ftl_lowrank_mttkrp_workspace_bytes": ([_INT, _INT, _P], _INT),
    "ftl_lowrank_sampled_mttkrp": ([_P, _P, _INT, _INT, _INT, _P, _I64, _P, _P, _P, _I64, _P, _P, _INT, _P,
                                    ctypes.c_size_t, _P, _I64, _I64, _P], _INT),
    "ftl_dense_sampled_mttkrp": ([_P, _INT, _P, _INT, _INT, _P, _I64, _P, _P, _P, _I64, _P, _P, _INT, _P, _I64,
                                  _P], _INT),
    "ftl_dense_materialize": ([_P, _INT, _P, _INT, _INT, _P, _I64, _P, _P], _INT),
    "ftl_dense_residual_workspace_bytes": ([_P], _INT),
    "ftl_dense_residual_terms": ([_P, _INT, _P, _INT, _P, _P, _INT, _P, ctypes.c_size_t, _P, _P], _INT),
    "ftl_lowrank_evaluate": ([_P, _INT, _INT, _P, _P, _INT, _I64, _P, _P], _INT),
    "ftl_noise_sampled_mttkrp": ([_P, _INT, _INT, _U64, ctypes.c_double, _P, _I64, _P, _P, _P, _I64, _P, _P, _INT,
                                  _P, _I64, _P], _INT),
    "ftl_noise_add_at": ([_P, _INT, _U64, ctypes.c_double, _P, _INT, _I64, _P, _P], _INT),
    "ftl_host_register": ([_P, ctypes.c_size_t, ctypes.POINTER(_INT)], _INT),
    "ftl_host_unregister": ([_P], _INT),
    "ftl_noise_add_fibers": ([_P, _INT, _U64, ctypes.c_double, _P, _I64, _INT, _P, _P], _INT),
    "ftl_lowrank_materialize": ([_P, _INT, _INT, _P, _P, _I64, _INT, _I64, _P, _P], _INT),
    "ftl_cross_gram_workspace_bytes": ([_INT, _INT, _P], _INT),
    "ftl_cross_gram": ([_P, _INT, _P, _INT, _I64, _P, ctypes.c_size_t, _P, _P], _INT),
    "ftl_chain_prod": ([_P, _INT, _INT, _INT, _INT, _P, _P, _P, _P, _P], _INT),
    "ftl_rows_times": ([_P, _I64, _INT, _P, _INT, _P, _I64, _P], _INT),
    "ftl_sparse_rrf": ([_P, _P, _P, _I64, _INT, _U64, ctypes.c_uint32, _P, _I64, _P], _INT),
    "ftl_factor_shadow": ([_P, _I64, _P, _P], _INT),
    "ftl_tree_geometry": ([_I64, _I64, ctypes.POINTER(TreeGeom)], _INT),
    "ftl_tree_bytes": ([_I64, _I64, _INT, _INT, _SZP], _INT),
    "ftl_krp_sample_packed_ctl": ([_P, _INT, _P, _P, _P, _P, _P, _P, _P, _P, _U64, _P, _P], _INT),
    "ftl_tune_variants": ([_INT, _INT, _INT, ctypes.POINTER(_INT), ctypes.POINTER(_INT)], _INT),
    "ftl_tune_set": ([_INT, _INT, _INT, _INT], _INT),
    "ftl_tune_get": ([_INT, _INT, _INT, ctypes.POINTER(_INT)], _INT),
    "ftl_node_layout": ([_INT, _INT, ctypes.POINTER(_INT), ctypes.POINTER(_INT), _P], _INT),
    "ftl_tree_build": ([_P, _I64, _INT, _I64, _INT, _P, _P], _INT),
    "ftl_tree_build_ex": ([_P, _I64, _INT, _I64, _INT, _P, _P, _P], _INT),
    "ftl_device_status": ([ctypes.POINTER(ctypes.c_uint32)], _INT),
    "ftl_tree_scale": ([_P, _P, _I64, _INT, _INT, _P, _P], _INT),
    "ftl_tree_sample": ([_P, _INT, _P, _I64, _INT, _I64, _P, _P, _P, _P, _I64, _P], _INT),
    "ftl_krp_plan_sizes": ([_INT, _INT, _INT, _SZP, _SZP, _SZP, _SZP], _INT),
    "ftl_krp_compute_m": ([ctypes.POINTER(KRPPlan), _U32, _P], _INT),
    "ftl_krp_draw": ([ctypes.POINTER(KRPPlan), _U32, _P, _P, _P, _P, _U64, _U64, _P], _INT),
    "ftl_krp_sample": ([ctypes.POINTER(KRPPlan), _U32, _P, _P, _P, _P, _U64, _U64, _P], _INT),
    "ftl_krp_draw_static": ([_INT, _INT, _I64, _INT, _P, _P, _P, _U32, _P, _P, _P, _P, _U64, _U64, _P], _INT),
    "ftl_fiber_keys": ([_P, _INT, _I64, _I64, _I64, _INT, _P, _INT, _P, _P], _INT),
    "ftl_sparse_gather": ([_P, _P, _P, _I64, _INT, _INT, _P, _P, _P], _INT),
    "ftl_dedup_workspace_bytes": ([_I64, _SZP], _INT),
    "ftl_dedup": ([_P, _I64, _P, ctypes.c_size_t, _P, _P, _P, _P, _P], _INT),
    "ftl_gram_workspace_bytes": ([_INT, _SZP], _INT),
    "ftl_weighted_gram": ([_P, _P, _P, _P, _P, _I64, _INT, _P, ctypes.c_size_t, _P, _P], _INT),
    "ftl_pinv_square": ([_P, _INT, _INT, _P, ctypes.c_double, _P, _P, _P], _INT),
    "ftl_sparse_mttkrp": ([_P, _P, _P, _I64, _P, _P, _P, _P, _P, _I64, _P, _INT, _P, _I64, _P], _INT),
    "ftl_mttkrp_rows_workspace_bytes": ([_I64, _INT, _SZP], _INT),
    "ftl_sparse_mttkrp_rows": ([_P, _P, _P, _I64, _P, _P, _P, _P, _I64, _I64, _P, _P, _INT, _P, ctypes.c_size_t, _P, _I64, _P],
                               _INT),
    "ftl_solve_rows": ([_P, _P, _I64, _INT, _P, _P], _INT),
    "ftl_colnorm_workspace_bytes": ([_INT, _SZP], _INT),
    "ftl_renormalize_columns": ([_P, _I64, _INT, _P, _P, ctypes.c_size_t, _INT, _P], _INT),
    "ftl_fit_workspace_bytes": ([_SZP], _INT),
    "ftl_sparse_residual_terms": ([_P, _P, _I64, _INT, _P, _P, _INT, _P, ctypes.c_size_t, _P, _P], _INT),
    "ftl_sum_squares": ([_P, _I64, _P, ctypes.c_size_t, _P, _P], _INT),
    "ftl_sparse_exact_mttkrp": ([_P, _P, _I64, _INT, _INT, _P, _INT, _P, _I64, _P], _INT),
    "ftl_gram_hadamard": ([_P, _INT, _INT, _INT, _P, _P, _P, _P, _P], _INT),
    "ftl_krp_sample_packed": ([_P, _INT, _P, _P, _P, _P, _P, _P, _P, _P], _INT),
    "ftl_philox_uniforms_dev": ([_P, _I64, _U64, _P, _P], _INT),
    "ftl_philox_uniforms": ([_P, _I64, _U64, _U64, _P], _INT),
}


def lib():
    """Load libftl_gb300.so (built by fast_tensor_leverage_gb300.build)."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise ImportError(
                f"{LIB_PATH} is missing: build it with `python -m fast_tensor_leverage_gb300.build` "
                "(there is no CPU fallback)")
        L = ctypes.CDLL(str(LIB_PATH), mode=os.RTLD_NOW | getattr(os, "RTLD_LOCAL", 0))
        for name, (args, res) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = res
        _lib = L
    return _lib


def check(status: int, what: str = "") -> None:
    if status != FTL_OK:
        msg = lib().ftl_last_error().decode(errors="replace")
        raise FTLError(status, f"{what}: {msg}" if what else msg)


def call(name: str, *args) -> None:
    check(getattr(lib(), name)(*args))


def tree_geometry(n: int, F: int) -> TreeGeom:
    g = TreeGeom()
    call("ftl_tree_geometry", n, F, ctypes.byref(g))
    return g


def tree_bytes(n: int, F: int, R: int, prec: int) -> int:
    out = ctypes.c_size_t()
    call("ftl_tree_bytes", n, F, R, prec, ctypes.byref(out))
    return out.value


def node_layout(R: int, prec: int):
    """(layout, stride, pos): the node layout id (0 packed, 1 wrapped
    diagonals), values per node, and the position inside a node of every
    upper-triangle element in row-major order (a numpy int32 array of
    R(R+1)/2 entries)."""
    import numpy as np
    lay, stride = _INT(), _INT()
    pos = np.zeros(R * (R + 1) // 2, dtype=np.int32)
    call("ftl_node_layout", R, prec, ctypes.byref(lay), ctypes.byref(stride), pos.ctypes.data)
    return lay.value, stride.value, pos


def device_status() -> int:
    """Status bits of device-side bounded waits that ran out since the last
    call (waits for the device; cleared on read)."""
    v = ctypes.c_uint32()
    call("ftl_device_status", ctypes.byref(v))
    return v.value


def ws_bytes(name: str, *args) -> int:
    """Workspace size query: name is one of dedup / mttkrp_rows / gram / colnorm / fit / ..."""
    out = ctypes.c_size_t()
    call(f"ftl_{name}_workspace_bytes", *args, ctypes.byref(out))
    return out.value


def plan_sizes(N: int, R: int, prec: int):
    e, m, l, p = (ctypes.c_size_t() for _ in range(4))
    call("ftl_krp_plan_sizes", N, R, prec, ctypes.byref(e), ctypes.byref(m), ctypes.byref(l), ctypes.byref(p))
    return e.value, m.value, l.value, p.value
