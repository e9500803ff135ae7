"""ctypes binding of libaxia_gpu.so (declarations in include/axia_gpu.h).

This is the binding a host of the C ABI writes (a Rust host declares the same
functions in an extern "C" block).  Loading fails loudly when the library is
missing: there is no CPU fallback behind this module.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

PKG_DIR = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(PKG_DIR, "libaxia_gpu.so")

OK = 0
ERR_INVALID_ARG = 1
ERR_SINGULAR_JACOBIAN = 2
ERR_NEG_JACOBIAN = 3
ERR_MATERIAL = 4
ERR_NOT_CONVERGED = 5
ERR_ZERO_PIVOT = 6
ERR_NO_FREE_DOF = 9
ERR_NONFINITE = 10
ERR_CUDA = 11
ERR_OOM = 12
ERR_TIMEOUT = 13
ERR_STATE = 14
ERR_TOO_LARGE = 15

STATUS_NAMES = {v: k for k, v in dict(
    OK=OK, INVALID_ARG=ERR_INVALID_ARG, SINGULAR_JACOBIAN=ERR_SINGULAR_JACOBIAN, NEG_JACOBIAN=ERR_NEG_JACOBIAN,
    MATERIAL=ERR_MATERIAL, NOT_CONVERGED=ERR_NOT_CONVERGED, ZERO_PIVOT=ERR_ZERO_PIVOT, NO_FREE_DOF=ERR_NO_FREE_DOF,
    NONFINITE=ERR_NONFINITE, CUDA=ERR_CUDA, OOM=ERR_OOM, TIMEOUT=ERR_TIMEOUT, STATE=ERR_STATE,
    TOO_LARGE=ERR_TOO_LARGE).items()}

PREC_FP64 = 0
PREC_MIXED = 1
REFINE_RESTART = 0
REFINE_RELIABLE = 1
ASM_CSR64 = 1
ASM_CSR32 = 2
ASM_BSR64 = 4
ASM_BSR32 = 8
ASM_SYM32 = 16
ASM_BSR32LO = 32
FORMAT_CSR = 0
FORMAT_BSR3 = 1
FORMAT_BSR3_SYM = 2
KRYLOV_PER_CASE = 0
KRYLOV_BLOCK = 1
ELEMENT_DWORD = 0
ELEMENT_FP64 = 1
PRECOND_JACOBI = 0
PRECOND_COARSE = 1


class Mesh(C.Structure):
    _fields_ = [("n_nodes", C.c_int64), ("coords", C.c_void_p), ("n_elem", C.c_int64), ("nn", C.c_int32),
                ("reduced", C.c_int32), ("conn", C.c_void_p), ("e_elem", C.c_void_p), ("e", C.c_double),
                ("nu", C.c_double)]


class SolveOpts(C.Structure):
    _fields_ = [("rtol", C.c_double), ("max_iter", C.c_int64), ("precision", C.c_int32),
                ("refine_mode", C.c_int32), ("inner_rtol", C.c_double), ("max_outer", C.c_int32),
                ("spmv_lanes", C.c_int32), ("matrix_format", C.c_int32), ("spmv_vec", C.c_int32),
                ("preconditioner", C.c_int32), ("coarse_nodes", C.c_int32), ("krylov", C.c_int32),
                ("reserved", C.c_int32)]


class SolveInfo(C.Structure):
    _fields_ = [("n_free", C.c_int64), ("nnz", C.c_int64), ("iters", C.c_int64), ("outer_iters", C.c_int64),
                ("residual", C.c_double), ("bnorm", C.c_double), ("true_residual", C.c_double),
                ("ms_setup", C.c_double), ("ms_assemble", C.c_double), ("ms_solve", C.c_double),
                ("ms_pcg_kernel", C.c_double), ("pcg_launches", C.c_int64), ("bad_index", C.c_int64), ("status", C.c_int32), ("reserved", C.c_int32)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_ if k != "reserved"}


# (name, restype, argtypes) of every exported symbol -- the same list as include/axia_gpu.h
_P = C.c_void_p
SIGNATURES = [
    ("axia_gpu_abi_version", C.c_int32, []),
    ("axia_gpu_create", _P, [C.c_int32, C.POINTER(C.c_int32)]),
    ("axia_gpu_destroy", None, [_P]),
    ("axia_gpu_last_error", C.c_char_p, [_P]),
    ("axia_gpu_element_ke", C.c_int32, [_P, C.c_int32, C.c_int32, C.c_int64, _P, _P, C.c_double, _P, _P,
                                        C.POINTER(C.c_int64)]),
    ("axia_gpu_element_ke_noalloc", C.c_int32, [C.c_int32, C.c_int32, C.c_int64, _P, _P, C.c_double, _P, _P,
                                                C.POINTER(C.c_int64)]),
    ("axia_face_loads", C.c_int32, [C.c_int32, C.c_int64, _P, _P, C.c_int64, _P, _P, _P, _P, C.POINTER(C.c_int64)]),
    ("axia_gpu_setup", C.c_int32, [_P, C.POINTER(Mesh), C.c_int64, _P, _P]),
    ("axia_gpu_assemble", C.c_int32, [_P, C.c_int32]),
    ("axia_gpu_assemble_ex", C.c_int32, [_P, C.c_int32]),
    ("axia_gpu_solve", C.c_int32, [_P, _P, _P, C.POINTER(SolveOpts), C.POINTER(SolveInfo)]),
    ("axia_gpu_solve_device", C.c_int32, [_P, _P, _P, C.POINTER(SolveOpts), C.POINTER(SolveInfo)]),
    ("axia_gpu_set_stream", C.c_int32, [_P, _P]),
    ("axia_gpu_kernel_launches", C.c_int64, [_P]),
    ("axia_gpu_check_wait_limit", C.c_int32, [_P, C.c_int64, C.POINTER(C.c_int32), C.POINTER(C.c_double)]),
    ("axia_gpu_fma_rate", C.c_int32, [_P, C.c_int32, C.POINTER(C.c_double)]),
    ("axia_gpu_spmv_device", C.c_int32, [_P, C.c_int32, _P, _P, C.c_int32]),
    ("axia_gpu_bsr_spmv_device", C.c_int32, [_P, C.c_int32, _P, _P, C.c_int32, C.c_int32]),
    ("axia_gpu_sym_spmv_device", C.c_int32, [_P, _P, _P, C.c_int32]),
    ("axia_gpu_sym_blocks", C.c_int64, [_P, C.POINTER(C.c_int64)]),
    ("axia_gpu_node_blocks", C.c_int64, [_P]),
    ("axia_gpu_assemble_times", C.c_int32, [_P, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    ("axia_gpu_set_element_arith", C.c_int32, [_P, C.c_int32]),
    ("axia_gpu_coarse_size", C.c_int32, [_P, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
    ("axia_gpu_setup_multi", C.c_int32, [_P, C.c_int32, C.POINTER(Mesh), _P, _P, _P]),
    ("axia_gpu_solve_multi", C.c_int32, [_P, _P, _P, C.POINTER(SolveOpts), C.POINTER(SolveInfo), _P, _P]),
    ("axia_gpu_solve_multi_device", C.c_int32, [_P, _P, _P, C.POINTER(SolveOpts), C.POINTER(SolveInfo), _P, _P]),
    ("axia_gpu_solve_batched", C.c_int32, [_P, C.c_int32, _P, _P, C.POINTER(SolveOpts), C.POINTER(SolveInfo), _P]),
    ("axia_gpu_solve_batched_device", C.c_int32, [_P, C.c_int32, _P, _P, C.POINTER(SolveOpts), C.POINTER(SolveInfo),
                                                  _P]),
    ("axia_gpu_element_energy", C.c_int32, [_P, _P, _P, _P]),
    ("axia_gpu_recover", C.c_int32, [_P, _P, _P, C.c_double, _P, _P, _P, _P, _P]),
    ("axia_gpu_solve_triplets", C.c_int32, [_P, C.c_int64, C.c_int64, _P, _P, _P, _P, _P, C.POINTER(SolveOpts),
                                            C.POINTER(SolveInfo)]),
    ("axia_gpu_autotune", C.c_int32, [_P, C.c_char_p, C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                                      C.POINTER(C.c_double)]),
    ("axia_gpu_autotune_batched", C.c_int32, [_P, C.c_char_p, C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                                              C.POINTER(C.c_double)]),
    ("axia_dofmap_build", C.c_int32, [C.c_int64, C.c_int64, _P, _P, C.c_int64, _P, _P, _P, _P, _P,
                                      C.POINTER(C.c_void_p)]),
    ("axia_dofmap_n_ind", C.c_int64, [_P]),
    ("axia_dofmap_export", C.c_int64, [_P, _P, _P, _P, _P, _P]),
    ("axia_dofmap_free", None, [_P]),
    ("axia_gpu_solve_reduced", C.c_int32, [_P, _P, C.c_int64, _P, _P, _P, _P, _P, C.POINTER(SolveOpts),
                                           C.POINTER(SolveInfo)]),
    ("axia_gpu_solve_csr", C.c_int32, [_P, C.c_int64, _P, _P, _P, _P, _P, C.POINTER(SolveOpts),
                                       C.POINTER(SolveInfo)]),
    ("axia_gpu_recover_device", C.c_int32, [_P, _P, _P, C.c_double, _P, _P, _P, _P, _P]),
    ("axia_gpu_compliance_forward", C.c_int32, [_P, _P, C.c_double, C.c_double, _P, _P, C.POINTER(C.c_double),
                                                C.POINTER(SolveOpts), C.POINTER(SolveInfo)]),
    ("axia_gpu_compliance_backward", C.c_int32, [_P, _P]),
    ("axia_gpu_system_size", C.c_int32, [_P, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
    ("axia_gpu_export_system", C.c_int32, [_P, _P, _P, _P, _P, _P]),
    ("axia_gpu_export_dofmap", C.c_int32, [_P, _P]),
]

_lib = None


class AxiaError(RuntimeError):
    """A non-OK status of the C ABI, with the library's message."""

    def __init__(self, code, msg=""):
        super().__init__(f"{STATUS_NAMES.get(code, code)}: {msg}")
        self.code = code


def load(path: str | None = None):
    """Loads libaxia_gpu.so (building it first if it is absent and nvcc exists)."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        import importlib.util
        spec = importlib.util.spec_from_file_location("_axia_build", os.path.join(PKG_DIR, "build.py"))
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        mod.build()
    lib = C.CDLL(path)
    for name, res, args in SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def ptr(a: np.ndarray | None):
    return None if a is None else a.ctypes.data
