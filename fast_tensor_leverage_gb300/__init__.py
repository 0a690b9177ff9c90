"""GB300-native exact leverage-score sampling from Khatri-Rao products.

Drop-in replacements for the reference's Python API on this path
(vbharadwaj-bk/fast_tensor_leverage, cpp_ext/als_module.cpp and
cpp_ext/partition_tree.cpp), backed by sm_103a CUDA kernels behind the C ABI
of include/ftl.h.
"""
from ._lib import FTLError, PREC
from .als import ALS, PyDenseTensor, PyLowRank, PySparseTensor, als_prod
from .partition_tree import PartitionTree
from .sampler import Sampler
from .tensors import DenseTensor, DenseTensor_double, DenseTensor_float, LowRankTensor, SparseTensor

__all__ = ["FTLError", "PREC", "PartitionTree", "Sampler", "LowRankTensor", "SparseTensor", "DenseTensor",
           "DenseTensor_double", "DenseTensor_float", "PyDenseTensor", "ALS",
           "PyLowRank", "PySparseTensor", "als_prod"]
