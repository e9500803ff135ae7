"""ctypes wrapper of the CPU oracle (oracle/axia_oracle.cpp).

TEST INFRASTRUCTURE ONLY: the checker used by tests/, __graft_entry__.smoke()
and bench.py's CPU-baseline leg.  The product library never imports this.
Every function restates a reference function; the C++ file cites them.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = os.path.join(_HERE, "liboracle.so")
_lib = None

STATUS = {0: "OK", 1: "INVALID_ARG", 2: "SINGULAR_JACOBIAN", 3: "NEG_JACOBIAN", 4: "MATERIAL",
          5: "NOT_CONVERGED", 6: "ZERO_PIVOT", 7: "INDEFINITE", 8: "SINGULAR", 9: "NO_FREE_DOF"}

SOLVER_CHOLESKY = 1
SOLVER_PCG = 2

_d = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_i32 = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_i64 = np.ctypeslib.ndpointer(dtype=np.int64, flags="C_CONTIGUOUS")


class OracleError(RuntimeError):
    def __init__(self, code, where=""):
        super().__init__(f"oracle {where}: {STATUS.get(code, code)}")
        self.code = code


def build(force=False):
    if force or not os.path.exists(_LIB) or os.path.getmtime(_LIB) < os.path.getmtime(
            os.path.join(_HERE, "axia_oracle.cpp")):
        subprocess.run(["bash", os.path.join(_HERE, "build_oracle.sh")], check=True)


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(_LIB)
        L.or_hex8_shape.argtypes = [C.c_double] * 3 + [_d, _d]
        L.or_hex20_shape.argtypes = [C.c_double] * 3 + [_d, _d]
        L.or_quad8_shape.argtypes = [C.c_double] * 2 + [_d, _d]
        L.or_invert3.argtypes = [_d, _d, _d]
        L.or_d_iso_3d.argtypes = [C.c_double, C.c_double, _d]
        L.or_element_ke.argtypes = [C.c_int, _d, C.c_double, C.c_double, C.c_int, _d, _d]
        L.or_face_pressure.argtypes = [C.c_int, _d, C.c_int, C.c_double, _d]
        L.or_face_loads.argtypes = [C.c_int64, _d, C.c_int, _i32, C.c_int64, _i64, _i32, _d, _d,
                                    C.POINTER(C.c_int64)]
        L.or_solve_static.argtypes = [C.c_int64, _d, C.c_int, C.c_int, C.c_int64, _i32, _d, C.c_double,
                                      C.c_int64, _i64, _d, _d, C.c_int, C.c_double, C.c_int64, C.c_int,
                                      C.c_int, _d, C.c_void_p, _d, C.POINTER(C.c_void_p), C.c_void_p]
        L.or_csr_n.argtypes = [C.c_void_p]
        L.or_csr_n.restype = C.c_int64
        L.or_csr_nnz.argtypes = [C.c_void_p]
        L.or_csr_nnz.restype = C.c_int64
        L.or_csr_export.argtypes = [C.c_void_p, _i64, _i64, _d]
        L.or_csr_free.argtypes = [C.c_void_p]
        L.or_solve_kff.argtypes = [C.c_int64, C.c_int64, _i64, _i64, _d, _d, C.c_int, C.c_double,
                                   C.c_int64, C.c_int, _d, _d]
        L.or_residual_ok.argtypes = [C.c_double, C.c_double]
        L.or_residual_multi.argtypes = [C.c_int64, _d, C.c_int, C.c_int, C.c_int64, _i32, _d, C.c_double,
                                        C.c_int64, _d, _d, _d, C.c_int, C.POINTER(C.c_int64)]
        L.or_nodal_stress.argtypes = [C.c_int64, _d, C.c_int, C.c_int, C.c_int64, _i32, _d, C.c_double, _d, _d,
                                      C.c_void_p, C.c_void_p, C.POINTER(C.c_int64)]
        L.or_reactions.argtypes = [C.c_int64, _d, C.c_int, C.c_int, C.c_int64, _i32, _d, C.c_double, _d, _d, _d,
                                   C.POINTER(C.c_int64)]
        L.or_dofmap_build.argtypes = [C.c_int64, C.c_int64, _i64, _d, C.c_int64, _i64, _i64, _i64, _d, _d,
                                      C.POINTER(C.c_void_p)]
        L.or_dofmap_n_ind.argtypes = [C.c_void_p]
        L.or_dofmap_n_ind.restype = C.c_int64
        L.or_dofmap_export.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        L.or_dofmap_export.restype = C.c_int64
        L.or_dofmap_free.argtypes = [C.c_void_p]
        L.or_solve_reduced.argtypes = [C.c_void_p, C.c_int64, _i64, _i64, _d, _d, C.c_int, C.c_double, C.c_int64,
                                       _d, _d, C.POINTER(C.c_void_p), C.c_void_p]
        L.or_compliance_grad.argtypes = [C.c_int64, _d, C.c_int, C.c_int, C.c_int64, _i32, _d, C.c_double,
                                         C.c_double, C.c_double, _d, _d, C.POINTER(C.c_int64)]
        _lib = L
    return _lib


def hex8_shape(xi, eta, zeta):
    n, dn = np.zeros(8), np.zeros(24)
    lib().or_hex8_shape(xi, eta, zeta, n, dn)
    return n, dn.reshape(8, 3)


def hex20_shape(xi, eta, zeta):
    n, dn = np.zeros(20), np.zeros(60)
    lib().or_hex20_shape(xi, eta, zeta, n, dn)
    return n, dn.reshape(20, 3)


def quad8_shape(xi, eta):
    n, dn = np.zeros(8), np.zeros(16)
    lib().or_quad8_shape(xi, eta, n, dn)
    return n, dn.reshape(8, 2)


def invert3(a):
    inv, det = np.zeros(9), np.zeros(1)
    st = lib().or_invert3(np.ascontiguousarray(a, dtype=np.float64).ravel(), inv, det)
    if st:
        raise OracleError(st, "invert3")
    return inv.reshape(3, 3), float(det[0])


def d_iso_3d(e, nu):
    d = np.zeros(36)
    st = lib().or_d_iso_3d(e, nu, d)
    if st:
        raise OracleError(st, "d_iso_3d")
    return d.reshape(6, 6)


def element_ke(xyz, e, nu, reduced=False):
    xyz = np.ascontiguousarray(xyz, dtype=np.float64)
    nn = xyz.shape[0]
    ke, vol = np.zeros((3 * nn) ** 2), np.zeros(1)
    st = lib().or_element_ke(nn, xyz.ravel(), e, nu, int(reduced), ke, vol)
    if st:
        raise OracleError(st, "element_ke")
    return ke.reshape(3 * nn, 3 * nn), float(vol[0])


def face_pressure(xyz, face, p):
    xyz = np.ascontiguousarray(xyz, dtype=np.float64)
    nn = xyz.shape[0]
    fe = np.zeros(3 * nn)
    st = lib().or_face_pressure(nn, xyz.ravel(), int(face), float(p), fe)
    if st:
        raise OracleError(st, "face_pressure")
    return fe


def load_vector(model):
    """CLOAD vector plus the DLOAD face pressures in list order (the full f)."""
    f = np.array(model.cload, dtype=np.float64, copy=True)
    if model.dload_elem.shape[0]:
        bad = C.c_int64(-1)
        st = lib().or_face_loads(model.n_nodes, np.ascontiguousarray(model.coords).ravel(), model.nn,
                                 np.ascontiguousarray(model.conn, dtype=np.int32).ravel(),
                                 model.dload_elem.shape[0], np.ascontiguousarray(model.dload_elem, np.int64),
                                 np.ascontiguousarray(model.dload_face, np.int32),
                                 np.ascontiguousarray(model.dload_p, np.float64), f, C.byref(bad))
        if st:
            raise OracleError(st, f"face load {bad.value}")
    return f


class StaticResult:
    pass


def solve_static(model, solver=SOLVER_PCG, tol=1e-8, max_iter=0, nthreads=1, f=None, autospc=True,
                 keep_csr=False, reactions=False):
    """The restated *STATIC path; returns u_full, info and optionally the K_ff CSR (int64 arrays)."""
    L = lib()
    if f is None:
        f = load_vector(model)
    u = np.zeros(model.ndof)
    rf = np.zeros(model.ndof) if reactions else None
    info = np.zeros(12)
    h = C.c_void_p()
    n_free_guess = model.ndof
    rhs = np.zeros(n_free_guess) if keep_csr else None
    st = L.or_solve_static(model.n_nodes, np.ascontiguousarray(model.coords).ravel(), model.nn,
                           int(model.reduced), model.n_elem,
                           np.ascontiguousarray(model.conn, dtype=np.int32).ravel(),
                           np.ascontiguousarray(model.e_elem, np.float64), float(model.nu),
                           model.bc_dof.shape[0], np.ascontiguousarray(model.bc_dof, np.int64),
                           np.ascontiguousarray(model.bc_val, np.float64), np.ascontiguousarray(f, np.float64),
                           int(solver), float(tol), int(max_iter), int(nthreads), int(autospc), u,
                           rf.ctypes.data if rf is not None else None, info,
                           C.byref(h) if keep_csr else None, rhs.ctypes.data if keep_csr else None)
    if st:
        raise OracleError(st, f"solve_static (element {int(info[11])})")
    r = StaticResult()
    r.u = u
    r.rf = rf
    r.n_free = int(info[0])
    r.nnz = int(info[1])
    r.iters = int(info[2])
    r.residual = float(info[3])
    r.t_assembly, r.t_reduce, r.t_csr, r.t_solve, r.t_total = (float(v) for v in info[4:9])
    r.n_triplets = int(info[9])
    r.bnorm = float(info[10])
    r.f = f
    if keep_csr:
        n, nnz = L.or_csr_n(h), L.or_csr_nnz(h)
        indptr, indices, data = np.zeros(n + 1, np.int64), np.zeros(nnz, np.int64), np.zeros(nnz)
        L.or_csr_export(h, indptr, indices, data)
        L.or_csr_free(h)
        r.indptr, r.indices, r.data = indptr, indices, data
        r.rhs = rhs[:n].copy()
    return r


def solve_kff(n, ti, tj, tv, rhs, solver=SOLVER_PCG, tol=1e-8, max_iter=0, nthreads=1):
    """csr_from_triplets + dense Cholesky or PCG on caller triplets; returns (x, iters, residual)."""
    x, info = np.zeros(n), np.zeros(2)
    st = lib().or_solve_kff(int(n), len(tv), np.ascontiguousarray(ti, np.int64),
                            np.ascontiguousarray(tj, np.int64), np.ascontiguousarray(tv, np.float64),
                            np.ascontiguousarray(rhs, np.float64), int(solver), float(tol), int(max_iter),
                            int(nthreads), x, info)
    if st:
        raise OracleError(st, "solve_kff")
    return x, int(info[0]), float(info[1])


def nodal_stress(model, u_full, elem_mean=False):
    """Nodal averaged Voigt stresses [n_nodes][6] and von Mises [n_nodes]
    (and, with elem_mean, the element means [n_elem][6])."""
    st_ = np.zeros((model.n_nodes, 6))
    vm = np.zeros(model.n_nodes)
    em = np.zeros((model.n_elem, 6))
    bad = C.c_int64(-1)
    st = lib().or_nodal_stress(model.n_nodes, np.ascontiguousarray(model.coords).ravel(), model.nn,
                               int(model.reduced), model.n_elem,
                               np.ascontiguousarray(model.conn, dtype=np.int32).ravel(),
                               np.ascontiguousarray(model.e_elem, np.float64), float(model.nu),
                               np.ascontiguousarray(u_full, np.float64), st_.ravel(), vm.ctypes.data,
                               em.ctypes.data, C.byref(bad))
    if st:
        raise OracleError(st, f"nodal_stress element {bad.value}")
    return (st_, vm, em) if elem_mean else (st_, vm)


def nodal_strain(stress, e, nu):
    """Strain from the averaged stress (analysis.rs:1160-1172)."""
    s = np.asarray(stress, dtype=np.float64)
    tr = s[:, 0] + s[:, 1] + s[:, 2]
    out = np.zeros_like(s)
    for c in range(3):
        out[:, c] = ((1.0 + nu) * s[:, c] - nu * tr) / e
    g2 = e / (1.0 + nu)
    out[:, 3:] = s[:, 3:] / g2
    return out


def reactions(model, u_full, f_full):
    """K u - f over all DOFs (reactions at prescribed DOFs)."""
    rf = np.zeros(model.ndof)
    bad = C.c_int64(-1)
    st = lib().or_reactions(model.n_nodes, np.ascontiguousarray(model.coords).ravel(), model.nn, int(model.reduced),
                            model.n_elem, np.ascontiguousarray(model.conn, dtype=np.int32).ravel(),
                            np.ascontiguousarray(model.e_elem, np.float64), float(model.nu),
                            np.ascontiguousarray(u_full, np.float64), np.ascontiguousarray(f_full, np.float64), rf,
                            C.byref(bad))
    if st:
        raise OracleError(st, f"reactions element {bad.value}")
    return rf


def residual_multi(model, u, f, nthreads=None):
    """K u - f for one vector (u[ndof]) or several (u[k][ndof], f the same shape or
    one f for all) with the oracle's own element stiffness, element by element
    (no K stored), the element loop split over nthreads (default: all cores)."""
    u = np.ascontiguousarray(u, np.float64)
    one = u.ndim == 1
    U = u.reshape(1, -1) if one else u
    F = np.ascontiguousarray(np.broadcast_to(f, U.shape), np.float64)
    out = np.zeros_like(U)
    nt = int(nthreads or os.cpu_count() or 1)
    bad = C.c_int64(-1)
    st = lib().or_residual_multi(model.n_nodes, np.ascontiguousarray(model.coords).ravel(), model.nn,
                                 int(model.reduced), model.n_elem,
                                 np.ascontiguousarray(model.conn, dtype=np.int32).ravel(),
                                 np.ascontiguousarray(model.e_elem, np.float64), float(model.nu), U.shape[0],
                                 U.ravel(), F.ravel(), out.ravel(), nt, C.byref(bad))
    if st:
        raise OracleError(st, f"residual element {bad.value}")
    return out[0] if one else out


def free_mask(model):
    """True on the DOFs no boundary condition prescribes (the model's SPCs only)."""
    m = np.ones(model.ndof, bool)
    m[np.asarray(model.bc_dof, np.int64)] = False
    return m


def relative_residual(model, u, f, nthreads=None):
    """||(K u - f)_free|| / ||f_free|| per vector with the oracle's K: the residual of a
    solution computed elsewhere under the oracle's own assembly (prescribed values zero)."""
    r = residual_multi(model, u, f, nthreads)
    m = free_mask(model)
    F = np.broadcast_to(f, np.shape(u))
    if r.ndim == 1:
        return float(np.linalg.norm(r[m]) / np.linalg.norm(F[m]))
    return np.linalg.norm(r[:, m], axis=1) / np.linalg.norm(F[:, m], axis=1)


def residual_ok(residual, bnorm):
    return bool(lib().or_residual_ok(float(residual), float(bnorm)))


def compliance_grad(model, rho, pexp, e0, u_full):
    g = np.zeros(model.n_elem)
    bad = C.c_int64(-1)
    st = lib().or_compliance_grad(model.n_nodes, np.ascontiguousarray(model.coords).ravel(), model.nn,
                                  int(model.reduced), model.n_elem,
                                  np.ascontiguousarray(model.conn, dtype=np.int32).ravel(),
                                  np.ascontiguousarray(rho, np.float64), float(pexp), float(e0),
                                  float(model.nu), np.ascontiguousarray(u_full, np.float64), g, C.byref(bad))
    if st:
        raise OracleError(st, f"compliance_grad element {bad.value}")
    return g


def direct_solve(indptr, indices, data, rhs):
    """Sparse direct solve of K_ff x = rhs with SciPy's SuperLU: the stand-in for the
    reference's faer LL^T (faer 0.24.4 is a Rust crate with no build here)."""
    import scipy.sparse as sp
    import scipy.sparse.linalg as spla
    n = indptr.shape[0] - 1
    K = sp.csr_matrix((data, indices, indptr), shape=(n, n)).tocsc()
    return spla.splu(K, permc_spec="COLAMD").solve(rhs)


def mpc_arrays(mpcs):
    """(slave, [(master, alpha), ...], u0) tuples -> flat arrays (slave, ptr, master, alpha, u0)."""
    slave = np.array([m[0] for m in mpcs], np.int64)
    ptr = np.zeros(len(mpcs) + 1, np.int64)
    for k, m in enumerate(mpcs):
        ptr[k + 1] = ptr[k] + len(m[1])
    master = np.array([t[0] for m in mpcs for t in m[1]], np.int64)
    alpha = np.array([t[1] for m in mpcs for t in m[1]], np.float64)
    u0 = np.array([m[2] for m in mpcs], np.float64)
    return slave, ptr, master, alpha, u0


class DofMap:
    """DofMap::build with MPCs (constraint.rs:26-136): T as CSR over full DOFs and u0."""

    def __init__(self, ndof, presc_dof, presc_val, mpcs):
        L = lib()
        self.h = C.c_void_p()
        sl, ptr, ma, al, u0 = mpc_arrays(mpcs)
        st = L.or_dofmap_build(int(ndof), len(presc_dof), np.ascontiguousarray(presc_dof, np.int64),
                               np.ascontiguousarray(presc_val, np.float64), len(mpcs), sl, ptr,
                               ma if ma.size else np.zeros(1, np.int64), al if al.size else np.zeros(1),
                               u0 if u0.size else np.zeros(1), C.byref(self.h))
        if st:
            raise OracleError(st, "dofmap_build")
        self.ndof = int(ndof)
        self.n_ind = int(L.or_dofmap_n_ind(self.h))
        nnz = int(L.or_dofmap_export(self.h, None, None, None, None))
        self.t_ptr = np.zeros(ndof + 1, np.int64)
        self.t_col = np.zeros(max(nnz, 1), np.int64)
        self.t_val = np.zeros(max(nnz, 1))
        self.u0 = np.zeros(ndof)
        L.or_dofmap_export(self.h, self.t_ptr.ctypes.data, self.t_col.ctypes.data, self.t_val.ctypes.data,
                           self.u0.ctypes.data)
        self.t_col, self.t_val = self.t_col[:nnz], self.t_val[:nnz]

    def solve(self, ti, tj, tv, f_full, solver=SOLVER_CHOLESKY, tol=1e-8, max_iter=0):
        """reduce -> csr_from_triplets -> solve -> reconstruct; returns u_full, info, (indptr, indices, data), rhs."""
        L = lib()
        u = np.zeros(self.ndof)
        info = np.zeros(2)
        h = C.c_void_p()
        rhs = np.zeros(max(self.n_ind, 1))
        st = L.or_solve_reduced(self.h, len(tv), np.ascontiguousarray(ti, np.int64), np.ascontiguousarray(tj, np.int64),
                                np.ascontiguousarray(tv, np.float64), np.ascontiguousarray(f_full, np.float64),
                                int(solver), float(tol), int(max_iter), u, info, C.byref(h), rhs.ctypes.data)
        csr = None
        if h.value:
            n, nnz = L.or_csr_n(h), L.or_csr_nnz(h)
            indptr, indices, data = np.zeros(n + 1, np.int64), np.zeros(nnz, np.int64), np.zeros(nnz)
            L.or_csr_export(h, indptr, indices, data)
            L.or_csr_free(h)
            csr = (indptr, indices, data)
        if st:
            raise OracleError(st, "solve_reduced")
        return u, info, csr, rhs[:self.n_ind]

    def __del__(self):
        try:
            if self.h:
                lib().or_dofmap_free(self.h)
        except Exception:
            pass


def element_triplets(model):
    """Full-DOF element triplets in the reference's push order (analysis.rs:651-668):
    elements ascending, Ke row-major, zero entries skipped."""
    ti, tj, tv = [], [], []
    for e in range(model.n_elem):
        ke, _ = element_ke(model.coords[model.conn[e]], float(model.e_elem[e]), model.nu, reduced=model.reduced)
        g = (3 * model.conn[e][:, None].astype(np.int64) + np.arange(3)).ravel()
        I, J = np.meshgrid(g, g, indexing="ij")
        keep = ke != 0.0
        ti.append(I[keep])
        tj.append(J[keep])
        tv.append(ke[keep])
    return np.concatenate(ti), np.concatenate(tj), np.concatenate(tv)
