"""axia_gpu -- host side of the GB300 linear-static backend for Axia.

The compute runs in libaxia_gpu.so (C ABI, include/axia_gpu.h); this package
binds it with ctypes and mirrors the reference's solver-selection and *STATIC
interfaces so callers and tests read like the reference's own.
"""
from . import _lib, meshgen  # noqa: F401
from ._lib import AxiaError, load  # noqa: F401
from .backend import SparseBackend, parse_sparse_backend, set_sparse_backend, sparse_backend, with_sparse_backend  # noqa: F401
from .context import GpuContext  # noqa: F401
from .static import StaticResult, solve_linear  # noqa: F401
