"""The DOF map with multi-point constraints (axia_dofmap_* of the C ABI).

Mirrors the reference's DofMap (solver/src/constraint.rs:16-136): u = u0 + T x
with MPCs u_slave = sum alpha u_master + u0 given as (slave, [(master, alpha),
...], u0) tuples, like the reference's Mpc struct.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L


def mpc_arrays(mpcs):
    """(slave, [(master, alpha), ...], u0) tuples -> (slave, ptr, master, alpha, u0) arrays."""
    slave = np.array([m[0] for m in mpcs], np.int64)
    ptr = np.zeros(len(mpcs) + 1, np.int64)
    for k, m in enumerate(mpcs):
        ptr[k + 1] = ptr[k] + len(m[1])
    master = np.array([t[0] for m in mpcs for t in m[1]], np.int64)
    alpha = np.array([t[1] for m in mpcs for t in m[1]], np.float64)
    u0 = np.array([m[2] for m in mpcs], np.float64)
    return slave, ptr, master, alpha, u0


class DofMap:
    """DofMap::build on the host side of the library."""

    def __init__(self, ndof, presc_dof, presc_val, mpcs=()):
        lib = L.load()
        self._lib = lib
        self.h = C.c_void_p()
        pd = np.ascontiguousarray(presc_dof, np.int64)
        pv = np.ascontiguousarray(presc_val, np.float64)
        sl, ptr, ma, al, u0 = mpc_arrays(list(mpcs))
        st = lib.axia_dofmap_build(int(ndof), pd.shape[0], L.ptr(pd), L.ptr(pv), sl.shape[0], L.ptr(sl), L.ptr(ptr),
                                   L.ptr(ma), L.ptr(al), L.ptr(u0), C.byref(self.h))
        if st:
            raise L.AxiaError(st, "dofmap_build")
        self.ndof = int(ndof)
        self.n_ind = int(lib.axia_dofmap_n_ind(self.h))

    def export(self):
        """(t_ptr, t_col, t_val, u0, ind_of)."""
        nnz = int(self._lib.axia_dofmap_export(self.h, None, None, None, None, None))
        t_ptr = np.zeros(self.ndof + 1, np.int64)
        t_col = np.zeros(max(nnz, 1), np.int64)
        t_val = np.zeros(max(nnz, 1))
        u0 = np.zeros(self.ndof)
        ind_of = np.zeros(self.ndof, np.int64)
        self._lib.axia_dofmap_export(self.h, L.ptr(t_ptr), L.ptr(t_col), L.ptr(t_val), L.ptr(u0), L.ptr(ind_of))
        return t_ptr, t_col[:nnz], t_val[:nnz], u0, ind_of

    def __del__(self):
        try:
            if self.h:
                self._lib.axia_dofmap_free(self.h)
        except Exception:
            pass
