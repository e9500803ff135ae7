"""Solver selection with the GPU backends added to the reference's enum.

Mirrors solver/src/backend.rs: the SparseBackend enum (backend.rs:9-27) with
two new variants, Gpu = 8 (FP64 Jacobi-PCG on the GPU) and GpuMixed = 9 (FP32
inner PCG with FP64 refinement), the process-wide default plus thread-local
override (backend.rs:49-89), AXIA_SOLVER (backend.rs:69-80) and the alias
parser (backend.rs:91-110) with "gpu" / "cuda" / "gpu-mixed" added.
"""
from __future__ import annotations

import contextlib
import enum
import os
import threading


class SparseBackend(enum.IntEnum):
    Auto = 0
    Mkl = 1
    Panua = 2
    Pardiso = 3
    Faer = 4
    Rivrs = 5
    Cholesky = 6
    Pcg = 7
    Gpu = 8
    GpuMixed = 9

    def as_str(self) -> str:
        return {SparseBackend.Gpu: "gpu", SparseBackend.GpuMixed: "gpu-mixed"}.get(self, self.name.lower())

    def is_gpu(self) -> bool:
        return self in (SparseBackend.Gpu, SparseBackend.GpuMixed)


_ALIASES = {
    "auto": SparseBackend.Auto, "default": SparseBackend.Auto,
    "mkl": SparseBackend.Mkl, "intel": SparseBackend.Mkl, "pardiso-mkl": SparseBackend.Mkl,
    "intel-mkl": SparseBackend.Mkl,
    "panua": SparseBackend.Panua, "pardiso-panua": SparseBackend.Panua,
    "pardiso": SparseBackend.Pardiso,
    "faer": SparseBackend.Faer, "supernodal": SparseBackend.Faer, "llt": SparseBackend.Faer,
    "rivrs": SparseBackend.Rivrs, "rivrs-sparse": SparseBackend.Rivrs, "ldlt": SparseBackend.Rivrs,
    "cholesky": SparseBackend.Cholesky, "dense": SparseBackend.Cholesky, "chol": SparseBackend.Cholesky,
    "pcg": SparseBackend.Pcg, "cg": SparseBackend.Pcg,
    "gpu": SparseBackend.Gpu, "cuda": SparseBackend.Gpu, "gpu-fp64": SparseBackend.Gpu,
    "gpu-mixed": SparseBackend.GpuMixed, "cuda-mixed": SparseBackend.GpuMixed, "mixed": SparseBackend.GpuMixed,
}


class BackendError(ValueError):
    pass


def parse_sparse_backend(s: str) -> SparseBackend:
    t = s.strip().lower()
    if t.startswith("--solver="):
        t = t[len("--solver="):]
    try:
        return _ALIASES[t]
    except KeyError:
        raise BackendError(f"unbekannter Sparse-Solver '{s}'. Erlaubt: auto, mkl, panua, pardiso, faer, rivrs, "
                           f"cholesky, pcg, gpu, gpu-mixed") from None


_process = SparseBackend.Auto
_tls = threading.local()


def set_sparse_backend(b: SparseBackend) -> None:
    global _process
    _process = SparseBackend(b)


def sparse_backend() -> SparseBackend:
    b = getattr(_tls, "b", None)
    return b if b is not None else _process


def apply_env_solver() -> None:
    global _process
    if _process != SparseBackend.Auto:
        return
    raw = os.environ.get("AXIA_SOLVER")
    if raw is None:
        return
    try:
        _process = parse_sparse_backend(raw)
    except BackendError:
        pass


@contextlib.contextmanager
def with_sparse_backend(b: SparseBackend):
    prev = getattr(_tls, "b", None)
    _tls.b = SparseBackend(b)
    try:
        yield
    finally:
        _tls.b = prev
