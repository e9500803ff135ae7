"""Host-side wrapper of one GPU context of the C ABI."""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import _lib as L


def _c(a, dtype):
    return np.ascontiguousarray(a, dtype=dtype)


class GpuContext:
    """One libaxia_gpu context: setup (symbolic) -> assemble (numeric) -> solve."""

    def __init__(self, device: int = 0):
        self.lib = L.load()
        st = C.c_int32(0)
        self.h = self.lib.axia_gpu_create(device, C.byref(st))
        if not self.h:
            raise L.AxiaError(st.value, f"cannot create a context on CUDA device {device}")
        self._keep = []

    def close(self):
        if getattr(self, "h", None):
            self.lib.axia_gpu_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, code, what=""):
        if code != L.OK:
            msg = self.lib.axia_gpu_last_error(self.h)
            raise L.AxiaError(code, f"{what}: {msg.decode() if msg else ''}")

    # -- element_ke ---------------------------------------------------------
    def element_ke(self, xyz, e, nu, reduced=False):
        """Batched element stiffness: xyz (n_elem, nn, 3), e (n_elem,) -> ke (n_elem, 3nn, 3nn), vol."""
        xyz = _c(xyz, np.float64)
        if xyz.ndim == 2:
            xyz = xyz[None]
        n_elem, nn = xyz.shape[0], xyz.shape[1]
        e = _c(np.broadcast_to(np.asarray(e, np.float64), (n_elem,)), np.float64)
        ke = np.zeros((n_elem, 3 * nn, 3 * nn))
        vol = np.zeros(n_elem)
        bad = C.c_int64(-1)
        code = self.lib.axia_gpu_element_ke(self.h, nn, int(reduced), n_elem, L.ptr(xyz), L.ptr(e), float(nu),
                                            L.ptr(ke), L.ptr(vol), C.byref(bad))
        if code != L.OK:
            err = L.AxiaError(code, self.lib.axia_gpu_last_error(self.h).decode())
            err.bad_index = bad.value
            raise err
        return ke, vol

    # -- model --------------------------------------------------------------
    def setup(self, model):
        self.model = model
        self._coords = _c(model.coords, np.float64)
        self._conn = _c(model.conn, np.int32)
        self._e = _c(model.e_elem, np.float64)
        self._bc_dof = _c(model.bc_dof, np.int64)
        self._bc_val = _c(model.bc_val, np.float64)
        m = L.Mesh(model.n_nodes, L.ptr(self._coords), model.n_elem, model.nn, int(model.reduced),
                   L.ptr(self._conn), L.ptr(self._e), 0.0, float(model.nu))
        self._check(self.lib.axia_gpu_setup(self.h, C.byref(m), self._bc_dof.shape[0], L.ptr(self._bc_dof),
                                            L.ptr(self._bc_val)), "setup")
        self._refresh_sizes()
        return self

    def _refresh_sizes(self):
        n, nnz = C.c_int64(), C.c_int64()
        self.lib.axia_gpu_system_size(self.h, C.byref(n), C.byref(nnz))
        self.n_free, self.nnz = n.value, nnz.value

    def setup_multi(self, models):
        """Several independent meshes as one context (concatenated node and element lists)."""
        self.models = list(models)
        n = len(self.models)
        keep = []
        meshes = (L.Mesh * n)()
        nbc = np.zeros(n, np.int64)
        dof_ptrs = (C.c_void_p * n)()
        val_ptrs = (C.c_void_p * n)()
        for k, m in enumerate(self.models):
            co, cn, e = _c(m.coords, np.float64), _c(m.conn, np.int32), _c(m.e_elem, np.float64)
            bd, bv = _c(m.bc_dof, np.int64), _c(m.bc_val, np.float64)
            keep += [co, cn, e, bd, bv]
            meshes[k] = L.Mesh(m.n_nodes, L.ptr(co), m.n_elem, m.nn, int(m.reduced), L.ptr(cn), L.ptr(e), 0.0,
                               float(m.nu))
            nbc[k] = bd.shape[0]
            dof_ptrs[k] = L.ptr(bd)
            val_ptrs[k] = L.ptr(bv)
        self._check(self.lib.axia_gpu_setup_multi(self.h, n, meshes, L.ptr(nbc), C.cast(dof_ptrs, C.c_void_p),
                                                  C.cast(val_ptrs, C.c_void_p)), "setup_multi")
        self._multi_keep = keep
        self.node0 = np.concatenate([[0], np.cumsum([m.n_nodes for m in self.models])]).astype(np.int64)
        nf, nnz = C.c_int64(), C.c_int64()
        self.lib.axia_gpu_system_size(self.h, C.byref(nf), C.byref(nnz))
        self.n_free, self.nnz = nf.value, nnz.value
        self.model = None
        return self

    def solve_multi(self, f_full, **kw):
        """Solve all meshes of setup_multi: concatenated f -> (u, info, rel_res, iters)."""
        f = _c(f_full, np.float64)
        u = np.zeros_like(f)
        n = len(self.models)
        rel, its = np.zeros(n), np.zeros(n, np.int64)
        kw.setdefault("inner_rtol", 0.01)
        o = self.opts(**kw)
        info = L.SolveInfo()
        self._check(self.lib.axia_gpu_solve_multi(self.h, L.ptr(f), L.ptr(u), C.byref(o), C.byref(info), L.ptr(rel),
                                                  L.ptr(its)), "solve_multi")
        return u, info, rel, its

    def solve_multi_device(self, f_dev_ptr, u_dev_ptr, **kw):
        n = len(self.models)
        rel, its = np.zeros(n), np.zeros(n, np.int64)
        kw.setdefault("inner_rtol", 0.01)
        o = self.opts(**kw)
        info = L.SolveInfo()
        self._check(self.lib.axia_gpu_solve_multi_device(self.h, C.c_void_p(f_dev_ptr), C.c_void_p(u_dev_ptr),
                                                         C.byref(o), C.byref(info), L.ptr(rel), L.ptr(its)),
                    "solve_multi")
        return info, rel, its

    def assemble(self, precision=L.PREC_FP64):
        self._check(self.lib.axia_gpu_assemble(self.h, int(precision)), "assemble")
        return self

    def assemble_ex(self, flags):
        """Build the matrix forms named by ASM_* flags (CSR / node-block, FP64 / FP32)."""
        self._check(self.lib.axia_gpu_assemble_ex(self.h, int(flags)), "assemble_ex")
        return self

    def load_vector(self, model=None):
        """CLOAD vector plus the DLOAD face pressures (host, library routine)."""
        model = model or self.model
        f = np.array(model.cload, dtype=np.float64, copy=True)
        if model.dload_elem.shape[0]:
            bad = C.c_int64(-1)
            el, fc, pp = _c(model.dload_elem, np.int64), _c(model.dload_face, np.int32), _c(model.dload_p, np.float64)
            code = self.lib.axia_face_loads(model.nn, model.n_nodes, L.ptr(_c(model.coords, np.float64)),
                                            L.ptr(_c(model.conn, np.int32)), el.shape[0], L.ptr(el), L.ptr(fc),
                                            L.ptr(pp), L.ptr(f), C.byref(bad))
            if code != L.OK:
                raise L.AxiaError(code, f"face load {bad.value}")
        return f

    @staticmethod
    def opts(rtol=1e-8, max_iter=0, precision=L.PREC_FP64, refine_mode=L.REFINE_RESTART, inner_rtol=1e-3,
             max_outer=50, spmv_lanes=0, matrix_format=L.FORMAT_CSR, spmv_vec=0, preconditioner=0,
             coarse_nodes=0, krylov=L.KRYLOV_PER_CASE):
        return L.SolveOpts(rtol, max_iter, precision, refine_mode, inner_rtol, max_outer, spmv_lanes,
                           matrix_format, spmv_vec, preconditioner, coarse_nodes, krylov, 0)

    def set_stream(self, stream_handle: int | None):
        """Issue the context's work on a caller's cudaStream_t (None: own stream)."""
        self._check(self.lib.axia_gpu_set_stream(self.h, C.c_void_p(stream_handle or 0)), "set_stream")

    def assemble_times(self):
        """(element kernel ms, gather ms) of the last numeric assembly (CUDA events)."""
        a, b = C.c_double(0.0), C.c_double(0.0)
        self._check(self.lib.axia_gpu_assemble_times(self.h, C.byref(a), C.byref(b)), "assemble_times")
        return a.value, b.value

    def set_element_arith(self, arith):
        """C3D8 / C3D20(R) element stiffness arithmetic: _lib.ELEMENT_DWORD (FP32-pair
        double words, default) or _lib.ELEMENT_FP64."""
        self._check(self.lib.axia_gpu_set_element_arith(self.h, int(arith)), "set_element_arith")
        return self

    def n_blocks(self) -> int:
        """3x3 node blocks of the node-block form."""
        return int(self.lib.axia_gpu_node_blocks(self.h))

    def coarse_size(self):
        """(subdomains, coarse unknowns) of the last two-level solve."""
        ns, nc = C.c_int64(0), C.c_int64(0)
        self._check(self.lib.axia_gpu_coarse_size(self.h, C.byref(ns), C.byref(nc)), "coarse_size")
        return int(ns.value), int(nc.value)

    def kernel_launches(self) -> int:
        return int(self.lib.axia_gpu_kernel_launches(self.h))

    def check_wait_limit(self, limit_us: int):
        """Run one device wait that cannot complete with the given limit;
        returns (status the host saw, probe kernel ms)."""
        st = C.c_int32(0)
        ms = C.c_double(0.0)
        self._check(self.lib.axia_gpu_check_wait_limit(self.h, int(limit_us), C.byref(st), C.byref(ms)),
                    "check_wait_limit")
        return int(st.value), float(ms.value)

    def fma_rate(self, precision=L.PREC_FP64) -> float:
        """Measured FMA throughput of the device in TFLOP/s (FP64 or FP32)."""
        t = C.c_double(0.0)
        self._check(self.lib.axia_gpu_fma_rate(self.h, int(precision), C.byref(t)), "fma_rate")
        return float(t.value)

    def spmv_device(self, precision, x_dev_ptr, y_dev_ptr, lanes=0):
        self._check(self.lib.axia_gpu_spmv_device(self.h, int(precision), C.c_void_p(x_dev_ptr),
                                                  C.c_void_p(y_dev_ptr), int(lanes)), "spmv")

    def bsr_spmv_device(self, precision, x_dev_ptr, y_dev_ptr, lanes=0, vec=0):
        self._check(self.lib.axia_gpu_bsr_spmv_device(self.h, int(precision), C.c_void_p(x_dev_ptr),
                                                      C.c_void_p(y_dev_ptr), int(lanes), int(vec)), "bsr_spmv")

    def sym_spmv_device(self, x_dev_ptr, y_dev_ptr, lanes=0):
        """y = K x (FP32) with the matrix in symmetric storage (AXIA_ASM_SYM32)."""
        self._check(self.lib.axia_gpu_sym_spmv_device(self.h, C.c_void_p(x_dev_ptr), C.c_void_p(y_dev_ptr),
                                                      int(lanes)), "sym_spmv")

    def sym_blocks(self):
        """(stored upper blocks incl. padding, lower-list entries) of the symmetric form."""
        nl = C.c_int64(0)
        nu = int(self.lib.axia_gpu_sym_blocks(self.h, C.byref(nl)))
        return nu, int(nl.value)

    def solve(self, f_full, out=None, **kw):
        """u for the load vector f_full (host arrays; out: a float64 array of the same
        size to write u into, e.g. in pinned memory)."""
        f = _c(f_full, np.float64)
        u = np.zeros_like(f) if out is None else out
        o = self.opts(**kw)
        info = L.SolveInfo()
        self._check(self.lib.axia_gpu_solve(self.h, L.ptr(f), L.ptr(u), C.byref(o), C.byref(info)), "solve")
        return u, info

    def solve_device(self, f_dev_ptr, u_dev_ptr, **kw):
        o = self.opts(**kw)
        info = L.SolveInfo()
        self._check(self.lib.axia_gpu_solve_device(self.h, C.c_void_p(f_dev_ptr), C.c_void_p(u_dev_ptr), C.byref(o),
                                                   C.byref(info)), "solve_device")
        return info

    def element_energy(self, u_full, v_full=None):
        """s_e = u_e^T K_e(E=1) v_e for every element (v defaults to u)."""
        u = _c(u_full, np.float64)
        v = u if v_full is None else _c(v_full, np.float64)
        s = np.zeros(self.model.n_elem)
        self._check(self.lib.axia_gpu_element_energy(self.h, L.ptr(u), L.ptr(v), L.ptr(s)), "element_energy")
        return s

    def recover(self, u_full, f_full=None, e_strain=None):
        """Nodal stresses [n][6], strains [n][6], von Mises [n], reactions K u - f [ndof]
        and element mean stresses [n_elem][6] for the displacement u_full."""
        m = self.model
        u = _c(u_full, np.float64)
        f = None if f_full is None else _c(f_full, np.float64)
        if e_strain is None:
            e_strain = float(np.asarray(m.e_elem, dtype=np.float64).ravel()[0]) if m.n_elem else 1.0
        stress = np.zeros((m.n_nodes, 6))
        strain = np.zeros((m.n_nodes, 6))
        vm = np.zeros(m.n_nodes)
        rf = np.zeros(m.ndof)
        emean = np.zeros((m.n_elem, 6))
        self._check(self.lib.axia_gpu_recover(self.h, L.ptr(u), None if f is None else L.ptr(f), float(e_strain),
                                              L.ptr(stress), L.ptr(strain), L.ptr(vm), L.ptr(rf), L.ptr(emean)),
                    "recover")
        return stress, strain, vm, rf, emean

    def recover_device(self, u_ptr, f_ptr, e_strain, stress_ptr=None, strain_ptr=None, vm_ptr=None, rf_ptr=None,
                       elem_ptr=None):
        """Device-pointer form of recover (ordered on the context's stream)."""
        self._check(self.lib.axia_gpu_recover_device(self.h, u_ptr, f_ptr, float(e_strain), stress_ptr, strain_ptr,
                                                     vm_ptr, rf_ptr, elem_ptr), "recover_device")

    def compliance_forward(self, rho, penal, e0, f_full, **kw):
        """SIMP forward: E = e0 rho^penal, solve, return (u, C, info)."""
        r = _c(rho, np.float64)
        f = _c(f_full, np.float64)
        u = np.zeros_like(f)
        c = C.c_double(0.0)
        o = self.opts(**kw)
        info = L.SolveInfo()
        self._check(self.lib.axia_gpu_compliance_forward(self.h, L.ptr(r), float(penal), float(e0), L.ptr(f), L.ptr(u),
                                                         C.byref(c), C.byref(o), C.byref(info)), "compliance_forward")
        return u, c.value, info

    def compliance_backward(self):
        """dC/drho_e for every element from the last forward call."""
        g = np.zeros(self.model.n_elem)
        self._check(self.lib.axia_gpu_compliance_backward(self.h, L.ptr(g)), "compliance_backward")
        return g

    def solve_batched(self, F, **kw):
        """Solve many load cases (F: (nrhs, ndof)) -> U (nrhs, ndof), info, per-case relative residuals."""
        Fm = _c(np.atleast_2d(F), np.float64)
        nrhs = Fm.shape[0]
        U = np.zeros_like(Fm)
        rel = np.zeros(nrhs)
        kw.setdefault("inner_rtol", 0.01)
        o = self.opts(**kw)
        info = L.SolveInfo()
        self._check(self.lib.axia_gpu_solve_batched(self.h, nrhs, L.ptr(Fm), L.ptr(U), C.byref(o), C.byref(info),
                                                    L.ptr(rel)), "solve_batched")
        return U, info, rel

    def solve_batched_device(self, nrhs, F_dev_ptr, U_dev_ptr, rel=None, **kw):
        kw.setdefault("inner_rtol", 0.01)
        o = self.opts(**kw)
        info = L.SolveInfo()
        rel = np.zeros(nrhs) if rel is None else rel
        self._check(self.lib.axia_gpu_solve_batched_device(self.h, nrhs, C.c_void_p(F_dev_ptr), C.c_void_p(U_dev_ptr),
                                                           C.byref(o), C.byref(info), L.ptr(rel)), "solve_batched")
        return info, rel

    def autotune(self, cache_path=None):
        """Time the node-block layouts of the mixed solver on the assembled mesh and keep
        the fastest for later solves; returns (lanes, vec, us_per_iter)."""
        lanes, vec, us = C.c_int32(), C.c_int32(), C.c_double()
        path = None if cache_path is None else os.fsencode(cache_path)
        self._check(self.lib.axia_gpu_autotune(self.h, path, C.byref(lanes), C.byref(vec), C.byref(us)), "autotune")
        return lanes.value, vec.value, us.value

    def autotune_batched(self, cache_path=None):
        """Time the tiles of the batched load-case kernel on the assembled mesh and keep the
        fastest for later batched solves; returns (cases_per_lane, blocks_per_step, us_per_iter)."""
        tc, tu, us = C.c_int32(), C.c_int32(), C.c_double()
        path = None if cache_path is None else os.fsencode(cache_path)
        self._check(self.lib.axia_gpu_autotune_batched(self.h, path, C.byref(tc), C.byref(tu), C.byref(us)),
                    "autotune_batched")
        return tc.value, tu.value, us.value

    def solve_kff(self, n, trips, rhs, **kw):
        """solve_kff on the GPU (linalg.rs:311 with PCG): trips = (i, j, v) arrays in the
        caller's order; returns (x, info).  Replaces any mesh set up on the context."""
        ti = _c(trips[0], np.int64)
        tj = _c(trips[1], np.int64)
        tv = _c(trips[2], np.float64)
        b = _c(rhs, np.float64)
        x = np.zeros(int(n))
        kw.setdefault("rtol", 1e-8)
        o = self.opts(**kw)
        info = L.SolveInfo()
        self.model = None
        try:
            self._check(self.lib.axia_gpu_solve_triplets(self.h, int(n), int(ti.shape[0]), L.ptr(ti), L.ptr(tj),
                                                         L.ptr(tv), L.ptr(b), L.ptr(x), C.byref(o), C.byref(info)),
                        "solve_kff")
        finally:
            self._refresh_sizes()
        return x, info

    def solve_reduced(self, dofmap, trips, f_full, **kw):
        """The MPC path of solve_linear: DofMap::reduce of full-DOF triplets and the load,
        csr_from_triplets, PCG, reconstruct; returns (u_full, info)."""
        ti = _c(trips[0], np.int64)
        tj = _c(trips[1], np.int64)
        tv = _c(trips[2], np.float64)
        f = _c(f_full, np.float64)
        u = np.zeros(dofmap.ndof)
        kw.setdefault("rtol", 1e-8)
        o = self.opts(**kw)
        info = L.SolveInfo()
        self.model = None
        try:
            self._check(self.lib.axia_gpu_solve_reduced(self.h, dofmap.h, int(ti.shape[0]), L.ptr(ti), L.ptr(tj),
                                                        L.ptr(tv), L.ptr(f), L.ptr(u), C.byref(o), C.byref(info)),
                        "solve_reduced")
        finally:
            self._refresh_sizes()
        return u, info

    def solve_csr(self, n, indptr, indices, data, rhs, **kw):
        """The same for a caller's CSR (int64 indptr / indices, full symmetric storage)."""
        p = _c(indptr, np.int64)
        c = _c(indices, np.int64)
        v = _c(data, np.float64)
        b = _c(rhs, np.float64)
        x = np.zeros(int(n))
        kw.setdefault("rtol", 1e-8)
        o = self.opts(**kw)
        info = L.SolveInfo()
        self.model = None
        try:
            self._check(self.lib.axia_gpu_solve_csr(self.h, int(n), L.ptr(p), L.ptr(c), L.ptr(v), L.ptr(b), L.ptr(x),
                                                    C.byref(o), C.byref(info)), "solve_csr")
        finally:
            self._refresh_sizes()
        return x, info

    def export_system(self):
        """K_ff as (rowptr, col, val), the Jacobi diagonal and K_fp u0."""
        rp = np.zeros(self.n_free + 1, np.int32)
        col = np.zeros(self.nnz, np.int32)
        val = np.zeros(self.nnz)
        dg = np.zeros(self.n_free)
        kf = np.zeros(self.n_free)
        self._check(self.lib.axia_gpu_export_system(self.h, L.ptr(rp), L.ptr(col), L.ptr(val), L.ptr(dg), L.ptr(kf)),
                    "export_system")
        return rp, col, val, dg, kf

    def export_dofmap(self):
        out = np.zeros(3 * self.model.n_nodes, np.int32)
        self._check(self.lib.axia_gpu_export_dofmap(self.h, L.ptr(out)), "export_dofmap")
        return out
