#!/usr/bin/env python
"""Static-solve throughput of the GB300 backend (one JSON line on rank 0).

Workload (default): C3D8 block of 100^3 unit elements (1,030,301 nodes), x=0
clamped, uniform 1 MPa pressure on x=L, interior nodes perturbed by up to
+-0.15 h (seeded), E=210000, nu=0.3 -> 3,060,300 free DOFs, 242,991,882
entries of K_ff.  The matrix (2.9 GB FP64) is far larger than the 129 MB L2,
so no flush is needed between steps.

A step = numeric assembly (element stiffness + gather into K_ff + Dirichlet
elimination) + PCG solve to ||r|| <= 1e-10 ||b|| + reconstruct, on inputs
already resident in HBM (the symbolic setup is done once, before timing).
  value : MDOF/s of the mixed-precision path (FP32 inner CG with FP64
          reliable updates on the node-block form, preconditioned by the
          diagonal plus a coarse space of subdomain rigid-body modes),
          n_free / step time; the coarse operator is rebuilt in every step
  mixed : the same with the diagonal preconditioner only (the reference's)
  fp64  : the plain FP64 Jacobi-PCG path timed the same way
  e2e   : the same metric through the C ABI with host buffers (pinned): setup
          (mesh upload + symbolic) + assemble + solve(host f -> host u) per step
--impl reference times the CPU restatement of the reference's path on the
host cores instead (see cpu_baseline).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "axia-fem_gb300"))

METRIC = "MDOF/s static solve, mixed vs FP64 PCG at rel err ≤1e-8; SpMV HBM GB/s"
PEAKS_FALLBACK = {"hbm_gbs": 6800.0}
CPU_SAMPLE_N = 50          # edge count of the CPU-baseline sample block (also timed on the GPU)
RTOL = 1e-10


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return d, "measured"
    return PEAKS_FALLBACK, "fallback"


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.p = None

    def __enter__(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                      stderr=subprocess.DEVNULL)
        except FileNotFoundError:
            self.p = None
        return self

    def __exit__(self, *a):
        if self.p:
            self.p.terminate()
            try:
                self.p.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.p.kill()

    def summary(self):
        self.f.flush()
        rows = [r.split(",") for r in open(self.f.name).read().strip().splitlines() if r.strip()]
        os.unlink(self.f.name)
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            r = [x.strip() for x in r]
            if len(r) < 9:
                continue
            try:
                sm.append(float(r[1]))
                mx = float(r[2])
            except ValueError:
                continue
            for k, name in enumerate(names):
                if r[5 + k].lower() == "active":
                    reasons.add(name)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


# DRAM bytes per algorithmic byte of pcg_bsr_reliable_kernel<8, 4>, from the ncu
# capture of the same kernel on the 60^3 block (75.49 GB over 300 iterations
# against 273.5 MB of algorithmic bytes per iteration; the matrix, padding
# included, is streamed once per iteration and the CG vectors stay in L2);
# scaled to a launch here by its algorithmic bytes (traffic grows with the
# iteration count and the matrix size).
MIXED_TRAFFIC_PER_ALG_BYTE = 0.920
# the same for pcg_bsr_reliable_kernel<8, 4, true> (two-level), from its ncu
# capture on the 60^3 block (52.73 GB over 198 iterations and 5 FP64 updates
# against 57.48 GB of algorithmic bytes, 64 subdomains)
COARSE_TRAFFIC_PER_ALG_BYTE = 0.919


def spmv_bytes(nnz, n, vbytes):
    """Algorithmic bytes of y = K x in CSR with int32 indices: values, columns,
    row pointers, x once, y once."""
    return vbytes * nnz + 4 * nnz + 4 * (n + 1) + 2 * vbytes * n


def pcg_iter_bytes(nnz, n, vbytes):
    """Algorithmic bytes of one PCG iteration of the persistent kernel:
    SpMV (values, columns, row pointers, p once, q written) + x/r update
    (x r+w, p r, r r+w, q r, dinv r) + p update (r r, dinv r, p r+w)."""
    return (vbytes + 4) * nnz + 4 * (n + 1) + 2 * vbytes * n + 7 * vbytes * n + 4 * vbytes * n


def bsr_spmv_bytes(nblocks, n_nodes, vbytes):
    """Algorithmic bytes of y = K x in the node-block form: 9 values and one
    int32 block column per block, int32 block-row pointers, x and y once."""
    return (9 * vbytes + 4) * nblocks + 4 * (n_nodes + 1) + 2 * vbytes * 3 * n_nodes


def bsr_pcg_iter_bytes(nblocks, n_nodes, vbytes):
    """One CG iteration on the node-block form (full-DOF vectors)."""
    nd = 3 * n_nodes
    return (9 * vbytes + 4) * nblocks + 4 * (n_nodes + 1) + 2 * vbytes * nd + 11 * vbytes * nd


def sym_spmv_bytes(nbu, nbl, n_nodes):
    """Algorithmic bytes of y = K x in the symmetric node-block form: each stored
    block (9 FP32 values + int32 column, pad blocks included) once, one
    (row, position) pair per lower entry, both row-pointer arrays, x and y once
    (the transposed re-reads of stored blocks are not counted: they are the
    same bytes)."""
    return 40 * nbu + 8 * nbl + 8 * (n_nodes + 1) + 2 * 4 * 3 * n_nodes


def sym_pcg_iter_bytes(nbu, nbl, n_nodes):
    """One CG iteration with the symmetric FP32 matrix (full-DOF vectors)."""
    nd = 3 * n_nodes
    return 40 * nbu + 8 * nbl + 8 * (n_nodes + 1) + 2 * 4 * nd + 11 * 4 * nd


def coarse_iter_bytes(n_nodes, n_coarse):
    """Extra algorithmic bytes of one two-level CG iteration: the per-node
    subdomain geometry (16 B) and node order (4 B) once, the dense coarse
    inverse (n_coarse rows of n_coarse rounded up to 64 floats) once."""
    ncp = (n_coarse + 63) // 64 * 64
    return 20 * n_nodes + 4 * n_coarse * ncp


def batch_iter_bytes(nblocks, n_nodes, n_coarse, nrhs=32):
    """One iteration of the 32-case kernel: the FP32 node-block matrix once
    (values + block columns, unpadded), the block-row pointers, 13 passes over
    [3 n_nodes][32] FP32 vectors (SpMV: P gathered once, Q written, P read for
    p.q; update: X, R read+written, P, Q read; search direction: R read, P
    read+written) and, with a coarse space, its per-iteration bytes."""
    b = (9 * 4 + 4) * nblocks + 4 * (n_nodes + 1) + 13 * 4 * nrhs * 3 * n_nodes
    if n_coarse:
        b += coarse_iter_bytes(n_nodes, n_coarse)
    return b


def batch_update_bytes(nblocks, n_nodes, nrhs=32):
    """One FP64 reliable update of the 32-case kernel: X += X32 (X read+written,
    X32 read+written), the FP64 matrix once, X gathered once, B read, R32 written."""
    nd = 3 * n_nodes
    return (9 * 8 + 4) * nblocks + 4 * (n_nodes + 1) + nrhs * nd * (8 + 8 + 4 + 4 + 8 + 8 + 4)


def element_fp64_flops(nn, ng):
    """FP64 operations of element_ke_kernel per element (FMA = 2 flops): per Gauss
    point 15 nn + 19 FMA (J, cofactors, det J, c_a) and 6 nn + 19 MUL (cofactors,
    c_a, h_a = (w / det J) c_a, w / det J); NE FMA per Gauss point for A_ab over
    the NE upper-triangle entries; NE MUL + NE FMA for K_ab from A and 3 FMA per
    node pair for the trace term; 2 ADD per node pair for the traces.  For C3D8
    that is 3920 FMA + 836 MUL + 72 ADD, the DFMA / DMUL / DADD counts ncu reads
    for the kernel (8,748 flop)."""
    ne = 9 * nn * (nn - 1) // 2 + 6 * nn
    nb = nn * (nn + 1) // 2
    fma = ng * (15 * nn + 19) + ne * ng + ne + 3 * nb
    other = ng * (6 * nn + 19) + ne + 2 * nb
    return 2 * fma + other


def gather_bytes(n_elem, nn, nblocks, n_nodes):
    """Algorithmic bytes of the gather into the node-block forms (FP64 + FP32):
    each (element, node) reads its 3 rows of Ke (9 nn doubles) and its element
    code, the node's adjacency and incidence; the 9 value planes are written in
    FP64 and FP32 and the inverse diagonals (FP64, FP32) once."""
    return n_elem * nn * (9 * nn * 8 + 4 + 4 * nn) + nblocks * (4 + 9 * 12) + 3 * n_nodes * 12 + 16 * n_nodes


def recover_bytes(n_elem, nn, n_nodes):
    """Algorithmic bytes of stress recovery + reactions: per element the
    connectivity twice, E once, 9 doubles per (element, node) written and read
    back; per node coordinates, u, f and the incidence pointer read, stress,
    strain, von Mises and reactions written."""
    per_elem = 2 * 4 * nn + 8 + 2 * 72 * nn + 48
    per_node = 24 + 24 + 24 + 8 + 48 + 48 + 8 + 24
    return per_elem * n_elem + per_node * n_nodes


def cpu_baseline(n=CPU_SAMPLE_N, threads=1):
    """The CPU restatement of the reference's *STATIC path (oracle/) on a
    bounded sample: the same block, loads and BCs at n^3, full path
    (element loop -> triplets -> reduce -> CSR -> Jacobi PCG to rtol 1e-10;
    the PCG's vector work over `threads` OpenMP threads)."""
    from axia_gpu import meshgen
    from oracle import oracle as O
    m = meshgen.block_c3d8_pressure(n=n)
    f = O.load_vector(m)
    t0 = time.perf_counter()
    r = O.solve_static(m, solver=O.SOLVER_PCG, tol=RTOL, nthreads=threads, f=f)
    dt = time.perf_counter() - t0
    return {"value": r.n_free / dt / 1e6, "unit": "MDOF/s", "cores": threads, "kind": "port",
            "sample": f"C3D8 {n}^3 block, same loads/BCs, full path to rtol {RTOL:g} "
                      f"({r.n_free} free DOFs, {r.iters} PCG iterations, {dt:.2f} s)",
            "seconds": dt, "iters": r.iters, "n_free": r.n_free,
            "phases_s": {"element_loop": r.t_assembly, "reduce": r.t_reduce, "csr_from_triplets": r.t_csr,
                         "pcg": r.t_solve}}


def oracle_residuals(model, sols, f, group=4):
    """||(K_oracle u - f)_free|| / ||f_free|| of each solution, with the oracle's own
    element stiffness applied element by element over all host threads (no K
    stored, no code shared with the library): the full-size accuracy check.
    sols: {name: u[ndof]} (one load f) or {name: U[k][ndof]} (f is [k][ndof]);
    vectors go through the element loop `group` at a time."""
    import numpy as np
    from oracle import oracle as O
    t0 = time.perf_counter()
    names, vecs, loads = [], [], []
    for name, u in sols.items():
        u = np.asarray(u)
        if u.ndim == 1:
            names.append(name)
            vecs.append(u)
            loads.append(f)
        else:
            for k in range(u.shape[0]):
                names.append(name)
                vecs.append(u[k])
                loads.append(f[k])
    res = []
    for k in range(0, len(vecs), group):
        res.extend(O.relative_residual(model, np.stack(vecs[k:k + group]), np.stack(loads[k:k + group])))
    out = {}
    for name, r in zip(names, res):
        out[name] = max(out.get(name, 0.0), float(r))
    return {"rel_residual_free": out, "seconds": time.perf_counter() - t0, "threads": os.cpu_count() or 1,
            "what": "||(K u - f)_free|| / ||f_free|| with K the oracle's element stiffness (restated "
                    "hex8/hex20_stiffness), applied element by element on the host; max over load cases"}


class Timer:
    """CUDA events on the stream the library launches on (torch's current stream)."""

    def __init__(self, torch, stream):
        self.torch, self.stream = torch, stream

    def __call__(self, fn, warmup, steps):
        torch = self.torch
        out, ms = None, []
        for k in range(warmup + steps):
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            with torch.cuda.stream(self.stream):
                a.record(self.stream)
                out = fn()
                b.record(self.stream)
            b.synchronize()
            if k >= warmup:
                ms.append(a.elapsed_time(b))
        return sum(ms) / len(ms), out


def _gpu_env(args):
    import torch
    from axia_gpu import GpuContext
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    ctx = GpuContext(local)
    stream = torch.cuda.Stream()
    ctx.set_stream(stream.cuda_stream)
    return torch, ctx, stream, Timer(torch, stream), local


def _line(args, workload, value, ms, extra):
    out = {"metric": METRIC, "value": value, "unit": "MDOF/s", "n_gpus": 1, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "data": "synthetic (seeded structured hexahedral meshes)",
           "config": {"workload": workload}}
    out.update(extra)
    print(json.dumps(out))


def same_sample_leg(args, local, n=CPU_SAMPLE_N):
    """The GPU on the CPU baseline's own sample (the n^3 block): the reference's
    algorithm (FP64 CSR Jacobi-PCG) and the headline path (mixed, two-level),
    each as assemble + solve on resident inputs, and the headline path through
    the C ABI with pinned host buffers (setup + assemble + solve + copy back)."""
    import numpy as np
    import torch
    from axia_gpu import GpuContext, _lib as L, meshgen
    model = meshgen.block_c3d8_pressure(n=n)
    ctx = GpuContext(local)
    stream = torch.cuda.Stream()
    ctx.set_stream(stream.cuda_stream)
    timer = Timer(torch, stream)
    ctx.setup(model)
    f_host = ctx.load_vector(model)
    f_dev = torch.from_numpy(f_host).to(f"cuda:{local}")
    u64, uco = torch.empty_like(f_dev), torch.empty_like(f_dev)
    coarse_kw = dict(precision=L.PREC_MIXED, refine_mode=L.REFINE_RELIABLE, inner_rtol=args.delta,
                     matrix_format=L.FORMAT_BSR3, preconditioner=L.PRECOND_COARSE, coarse_nodes=args.coarse_nodes)

    def step64():  # the reference's algorithm throughout (FP64 element stiffness too)
        ctx.set_element_arith(L.ELEMENT_FP64)
        ctx.assemble_ex(L.ASM_CSR64)
        info = ctx.solve_device(f_dev.data_ptr(), u64.data_ptr(), rtol=RTOL, precision=L.PREC_FP64)
        ctx.set_element_arith(L.ELEMENT_DWORD)
        return info

    def stepco():
        ctx.assemble_ex(L.ASM_BSR64 | L.ASM_BSR32)
        return ctx.solve_device(f_dev.data_ptr(), uco.data_ptr(), rtol=RTOL, **coarse_kw)
    ms64, i64 = timer(step64, args.warmup, args.steps)
    msco, ico = timer(stepco, args.warmup, args.steps)
    f_pin = torch.empty(f_host.shape, dtype=torch.float64, pin_memory=True).numpy()
    f_pin[...] = f_host
    u_pin = torch.empty(f_host.shape, dtype=torch.float64, pin_memory=True).numpy()
    ctx.set_stream(None)
    ts = []
    for k in range(args.warmup + args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ctx.setup(model)
        ctx.assemble_ex(L.ASM_BSR64 | L.ASM_BSR32)
        ctx.solve(f_pin, out=u_pin, rtol=RTOL, **coarse_kw)
        if k >= args.warmup:
            ts.append(time.perf_counter() - t0)
    e2e_ms = 1e3 * sum(ts) / len(ts)
    nf = ctx.n_free
    u64h = u64.cpu().numpy()
    out = {"workload": f"C3D8 block {n}^3 (the CPU baseline's sample), same loads/BCs", "n_free": nf,
           "fp64_jacobi": {"value": nf / (ms64 * 1e-3) / 1e6, "ms_per_step": ms64, "iters": i64.iters,
                           "algorithm": "FP64 CSR Jacobi-PCG (the reference's)"},
           "mixed_coarse": {"value": nf / (msco * 1e-3) / 1e6, "ms_per_step": msco, "iters": ico.iters,
                            "rel_err_vs_fp64": float(np.linalg.norm(uco.cpu().numpy() - u64h) / np.linalg.norm(u64h))},
           "mixed_coarse_e2e": {"value": nf / (e2e_ms * 1e-3) / 1e6, "ms_per_step": e2e_ms}}
    ctx.close()
    return out


def run_c3(args):
    """C3D20 50^3 block, base clamped, random top traction: mixed (FP32 node-block
    inner CG, FP64 reliable updates) vs FP64 CSR PCG, both to rtol 1e-10."""
    import numpy as np
    from axia_gpu import _lib as L, meshgen
    torch, ctx, stream, timer, local = _gpu_env(args)
    n = args.n if args.n != 100 else 50
    m = meshgen.block_c3d20_traction(n=n)
    ctx.setup(m)
    f = torch.from_numpy(ctx.load_vector(m)).to(f"cuda:{local}")
    u64, umx = torch.empty_like(f), torch.empty_like(f)

    def step64():  # the reference's algorithm throughout (FP64 element stiffness too)
        ctx.set_element_arith(L.ELEMENT_FP64)
        ctx.assemble_ex(L.ASM_CSR64)
        info = ctx.solve_device(f.data_ptr(), u64.data_ptr(), rtol=RTOL, spmv_lanes=args.lanes64)
        ctx.set_element_arith(L.ELEMENT_DWORD)
        return info

    def stepmx():
        ctx.assemble_ex(L.ASM_BSR64 | L.ASM_BSR32)
        return ctx.solve_device(f.data_ptr(), umx.data_ptr(), rtol=RTOL, precision=L.PREC_MIXED,
                                refine_mode=L.REFINE_RELIABLE, inner_rtol=args.delta, matrix_format=L.FORMAT_BSR3,
                                spmv_lanes=args.lanes32)
    uco = torch.empty_like(f)

    def stepco():
        ctx.assemble_ex(L.ASM_BSR64 | L.ASM_BSR32)
        return ctx.solve_device(f.data_ptr(), uco.data_ptr(), rtol=RTOL, precision=L.PREC_MIXED,
                                refine_mode=L.REFINE_RELIABLE, inner_rtol=args.delta, matrix_format=L.FORMAT_BSR3,
                                spmv_lanes=args.lanes32, preconditioner=L.PRECOND_COARSE,
                                coarse_nodes=args.coarse_nodes)
    ms64, i64 = timer(step64, args.warmup, args.steps)
    msmx, imx = timer(stepmx, args.warmup, args.steps)
    msco, ico = timer(stepco, args.warmup, args.steps)
    rel = float(torch.linalg.norm(umx - u64) / torch.linalg.norm(u64))
    relco = float(torch.linalg.norm(uco - u64) / torch.linalg.norm(u64))
    oracle_check = oracle_residuals(m, {"fp64": u64.cpu().numpy(), "mixed": umx.cpu().numpy(),
                                        "mixed_coarse": uco.cpu().numpy()}, f.cpu().numpy())
    nf = ctx.n_free
    n_sub, n_coarse = ctx.coarse_size()
    _line(args, f"C3D20 block {n}^3, 27-point Gauss, E=70000 nu=0.33, base clamped, top traction N(0,1)",
          nf / (msco * 1e-3) / 1e6, msco,
          {"dtype": "f32+f64", "config": {"workload": f"C3D20 {n}^3", "n_free": nf, "nnz_kff": ctx.nnz,
                                          "node_blocks": ctx.n_blocks(), "rtol": RTOL,
                                          "preconditioner": f"diagonal + coarse space ({n_sub} subdomains)"},
           "mixed_coarse": {"ms_per_step": msco, "inner_iters": ico.iters, "reliable_updates": ico.outer_iters,
                            "ms_assemble": ico.ms_assemble, "ms_pcg_kernel": ico.ms_pcg_kernel,
                            "true_rel_residual": ico.true_residual / ico.bnorm, "rel_err_vs_fp64": relco,
                            "subdomains": n_sub, "coarse_unknowns": n_coarse},
           "fp64": {"value": nf / (ms64 * 1e-3) / 1e6, "ms_per_step": ms64, "iters": i64.iters,
                    "ms_assemble": i64.ms_assemble, "true_rel_residual": i64.true_residual / i64.bnorm},
           "mixed": {"ms_per_step": msmx, "inner_iters": imx.iters, "reliable_updates": imx.outer_iters,
                     "ms_assemble": imx.ms_assemble, "true_rel_residual": imx.true_residual / imx.bnorm,
                     "rel_err_vs_fp64": rel},
           "speedup_mixed_vs_fp64": ms64 / msco, "speedup_mixed_jacobi_vs_fp64": ms64 / msmx,
           "oracle_check": oracle_check})


def run_c4a(args):
    """C3D8 80^3 block with 32 random surface load cases in one batched launch."""
    from axia_gpu import _lib as L, meshgen
    torch, ctx, stream, timer, local = _gpu_env(args)
    n = args.n if args.n != 100 else 80
    m = meshgen.block_c3d8_multiload(n=n, nrhs=32)
    ctx.setup(m)
    F = torch.from_numpy(m.cload_batch).to(f"cuda:{local}")
    U = torch.empty_like(F)
    # tile of the batched kernel, picked by the library's autotuner (untimed)
    ctx.assemble_ex(L.ASM_BSR64 | L.ASM_BSR32)
    btc, btu, bus = ctx.autotune_batched()

    # the FP32 low parts: reliable updates in double words between kernel segments
    LO = L.ASM_BSR64 | L.ASM_BSR32 | L.ASM_BSR32LO

    def step_jacobi():
        ctx.assemble_ex(LO)
        return ctx.solve_batched_device(32, F.data_ptr(), Uj.data_ptr(), rtol=RTOL, inner_rtol=args.delta)

    def step():
        ctx.assemble_ex(LO)
        return ctx.solve_batched_device(32, F.data_ptr(), U.data_ptr(), rtol=RTOL, inner_rtol=args.delta,
                                        preconditioner=L.PRECOND_COARSE, coarse_nodes=args.coarse_nodes)
    Uj = torch.empty_like(F)
    Ub = torch.empty_like(F)

    def step_block():
        ctx.assemble_ex(L.ASM_BSR64 | L.ASM_BSR32)
        return ctx.solve_batched_device(32, F.data_ptr(), Ub.data_ptr(), rtol=RTOL, inner_rtol=args.delta,
                                        preconditioner=L.PRECOND_COARSE, coarse_nodes=args.coarse_nodes,
                                        krylov=L.KRYLOV_BLOCK)
    msj, (infoj, relj) = timer(step_jacobi, args.warmup, args.steps)
    ms, (info, rel) = timer(step, args.warmup, args.steps)
    msb, (infob, relb) = timer(step_block, args.warmup, args.steps)
    n_sub, n_coarse = ctx.coarse_size()
    err_j = float(torch.linalg.norm(U - Uj) / torch.linalg.norm(Uj))
    # one case through the single-RHS mixed path for comparison
    u1 = torch.empty(m.ndof, dtype=torch.float64, device=f"cuda:{local}")

    def single():
        return ctx.solve_device(F[0].data_ptr(), u1.data_ptr(), rtol=RTOL, precision=L.PREC_MIXED,
                                refine_mode=L.REFINE_RELIABLE, inner_rtol=args.delta, matrix_format=L.FORMAT_BSR3,
                                preconditioner=L.PRECOND_COARSE, coarse_nodes=args.coarse_nodes)
    ms1, i1 = timer(single, 1, 2)
    err = float(torch.linalg.norm(U[0] - u1) / torch.linalg.norm(u1))
    pk, pk_kind = peaks()
    nblocks = ctx.n_blocks()
    bbytes = batch_iter_bytes(nblocks, m.n_nodes, n_coarse) * info.iters + \
        batch_update_bytes(nblocks, m.n_nodes) * info.outer_iters
    bach = bbytes / (info.ms_pcg_kernel * 1e-3) / 1e9
    broof = {"bound": "hbm", "achieved": bach, "peak": pk["hbm_gbs"], "unit": "GB/s", "frac": bach / pk["hbm_gbs"],
             "bytes_per_launch": bbytes, "ms_per_launch": info.ms_pcg_kernel,
             "us_per_iteration": 1e3 * info.ms_pcg_kernel / max(info.iters, 1),
             "kernel": "pcg_bsr_multi_kernel (32 load cases, two-level)", "peak_source": f"{pk_kind} hbm_gbs"}
    oracle_check = oracle_residuals(m, {"batched_coarse": U.cpu().numpy(), "batched_jacobi": Uj.cpu().numpy(),
                                        "block_coarse": Ub.cpu().numpy()}, m.cload_batch)
    err_b = float(torch.linalg.norm(Ub - U) / torch.linalg.norm(U))
    nf = ctx.n_free
    _line(args, f"C3D8 block {n}^3, x=0 clamped, 32 load cases (5% of surface nodes, N(0,1))",
          32 * nf / (ms * 1e-3) / 1e6, ms,
          {"dtype": "f32+f64", "config": {"workload": f"C3D8 {n}^3 x 32 load cases", "n_free": nf, "rhs": 32,
                                          "preconditioner": f"diagonal + coarse space ({n_sub} subdomains)"},
           "tile": {"cases_per_lane": btc, "blocks_per_step": btu, "us_per_iter_tuning": bus},
           "roofline": broof,
           "batched": {"iters": info.iters, "reliable_updates": info.outer_iters, "max_rel_residual": float(rel.max()),
                       "ms_kernel": info.ms_pcg_kernel, "coarse_unknowns": n_coarse,
                       "rel_err_vs_jacobi_batched": err_j},
           "batched_jacobi": {"ms_per_step": msj, "iters": infoj.iters, "reliable_updates": infoj.outer_iters,
                              "max_rel_residual": float(relj.max()), "ms_kernel": infoj.ms_pcg_kernel},
           "block": {"ms_per_step": msb, "value": 32 * nf / (msb * 1e-3) / 1e6, "iters": infob.iters,
                     "reliable_updates": infob.outer_iters, "max_rel_residual": float(relb.max()),
                     "ms_solve_launches": infob.ms_pcg_kernel, "rel_err_vs_per_case": err_b,
                     "method": "block PCG, one Krylov block for the 32 cases (breakdown-free, orthonormalized "
                               "directions), two-level preconditioner, FP64 reliable updates"},
           "speedup_block_vs_per_case": ms / msb,
           "single_case": {"ms": ms1, "iters": i1.iters, "rel_err_batched_vs_single": err},
           "speedup_vs_32_single_solves": 32 * ms1 / ms, "oracle_check": oracle_check})


def run_c4b(args):
    """64 independent C3D8 cubes (edges 10..40) in one cooperative launch from a CUDA graph.
    With N ranks (torchrun), every rank takes a disjoint subset of the meshes balanced by
    the work estimate (no collective on the data path); the job time is the slowest
    rank's and the value all 64 meshes' DOFs over it (total work fixed: strong scaling)."""
    import numpy as np
    from axia_gpu import _lib as L, meshgen, replicas
    torch, ctx, stream, timer, local = _gpu_env(args)
    rank, _, world = replicas.world()
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    cubes_all = meshgen.cube_family(count=64, lo=10, hi=40)
    work = [replicas.mesh_work(c.n_nodes, (3 * (c.shape[0] + 1) - 2) ** 3) for c in cubes_all]
    mine = replicas.partition_meshes(work, world)[rank]
    cubes = [cubes_all[k] for k in mine]
    ctx.setup_multi(cubes)
    f = torch.from_numpy(np.concatenate([c.cload for c in cubes])).to(f"cuda:{local}")
    u = torch.empty_like(f)

    def step_jacobi():
        ctx.assemble_ex(L.ASM_BSR64 | L.ASM_BSR32)
        return ctx.solve_multi_device(f.data_ptr(), u.data_ptr(), rtol=RTOL, inner_rtol=args.delta)

    def step():
        ctx.assemble_ex(L.ASM_BSR64 | L.ASM_BSR32)
        return ctx.solve_multi_device(f.data_ptr(), u.data_ptr(), rtol=RTOL, inner_rtol=args.delta,
                                      preconditioner=L.PRECOND_COARSE, coarse_nodes=(args.coarse_nodes or 2000) // 2)
    msj, (infoj, relj, itsj) = timer(step_jacobi, args.warmup, args.steps)
    uj = u.clone()
    if dist is not None:
        torch.cuda.synchronize()
        dist.barrier()
    ms, (info, rel, its) = timer(step, args.warmup, args.steps)
    ms_job = replicas.max_over_ranks(ms, dist, f"cuda:{local}")
    msj_job = replicas.max_over_ranks(msj, dist, f"cuda:{local}")
    err_j = float(torch.linalg.norm(u - uj) / torch.linalg.norm(uj))
    n_sub, n_coarse = ctx.coarse_size()
    uh = u.cpu().numpy()
    t0 = time.perf_counter()
    worst = 0.0
    for k, c in enumerate(cubes):
        chk = oracle_residuals(c, {"u": uh[3 * ctx.node0[k]:3 * ctx.node0[k + 1]]}, c.cload)
        worst = max(worst, chk["rel_residual_free"]["u"])
    worst = replicas.max_over_ranks(worst, dist, f"cuda:{local}")
    oracle_check = {"rel_residual_free": {"multi_coarse_worst_mesh": worst}, "seconds": time.perf_counter() - t0,
                    "what": "per mesh ||(K u - f)_free|| / ||f_free|| with the oracle's element stiffness; "
                            "the worst of the 64 meshes"}
    nf_all = sum(int(c.n_free) for c in cubes_all)
    if dist is not None:
        dist.destroy_process_group()
    if rank != 0:
        return
    _line(args, "64 C3D8 cubes, edge counts U{10..40} (seeded), x=0 clamped, random surface loads",
          nf_all / (ms_job * 1e-3) / 1e6, ms_job,
          {"dtype": "f32+f64", "n_gpus": world, "scaling": "strong",
           "config": {"workload": "64 cubes", "n_free": nf_all, "meshes": 64,
                      "sizes": [int(c.shape[0]) for c in cubes_all],
                      "preconditioner": f"diagonal + per-mesh coarse spaces ({n_sub} subdomains on rank 0)",
                      "parallelism": f"meshes split over {world} rank(s) by work estimate, no collective"},
           "multi": {"max_iters": int(its.max()), "min_iters": int(its.min()), "max_rel_residual": float(rel.max()),
                     "ms_kernel": info.ms_pcg_kernel, "ms_assemble": info.ms_assemble,
                     "rel_err_vs_diagonal": err_j, "coarse_unknowns": n_coarse, "rank0_meshes": len(mine)},
           "multi_diagonal": {"ms_per_step": msj_job, "max_iters": int(itsj.max()), "ms_kernel": infoj.ms_pcg_kernel},
           "oracle_check": oracle_check})


def run_c5(args):
    """SIMP beam 100x50x50: FP64 forward solve, adjoint gradient of all elements,
    checked against central differences (h = 1e-6) on 20 seeded elements."""
    import numpy as np
    from axia_gpu import _lib as L, meshgen
    from oracle import oracle as O
    torch, ctx, stream, timer, local = _gpu_env(args)
    m = meshgen.simp_beam(nx=100, ny=50, nz=50)
    ctx.setup(m)
    f = ctx.load_vector(m)
    # forward solves: FP64 CSR Jacobi-PCG (the reference's algorithm) and the mixed
    # node-block solve with the two-level preconditioner, both to rtol 1e-12
    fwd = dict(rtol=1e-12, precision=L.PREC_MIXED, refine_mode=L.REFINE_RELIABLE, inner_rtol=args.delta,
               matrix_format=L.FORMAT_BSR3, preconditioner=L.PRECOND_COARSE, coarse_nodes=args.coarse_nodes)
    ctx.set_element_arith(L.ELEMENT_FP64)  # the reference's algorithm throughout
    ctx.compliance_forward(m.rho, m.pexp, m.e0, f, rtol=1e-12)  # warm-up
    t0 = time.perf_counter()
    u64, c64, info64 = ctx.compliance_forward(m.rho, m.pexp, m.e0, f, rtol=1e-12)
    t_fwd64 = time.perf_counter() - t0
    ctx.set_element_arith(L.ELEMENT_DWORD)
    ctx.compliance_forward(m.rho, m.pexp, m.e0, f, **fwd)  # warm-up
    t0 = time.perf_counter()
    u, c, info = ctx.compliance_forward(m.rho, m.pexp, m.e0, f, **fwd)
    t_fwd = time.perf_counter() - t0
    rel_u = float(np.linalg.norm(u - u64) / np.linalg.norm(u64))
    t0 = time.perf_counter()
    g = ctx.compliance_backward()
    t_bwd = time.perf_counter() - t0
    rng = np.random.default_rng(20261203)
    pick = rng.choice(m.n_elem, 20, replace=False)
    h = 1e-6
    worst_exact, worst_direct = 0.0, 0.0
    for k in pick:
        rp, rm = m.rho.copy(), m.rho.copy()
        rp[k] += h
        rm[k] -= h
        up, cp, _ = ctx.compliance_forward(rp, m.pexp, m.e0, f, **fwd)
        um, cm, _ = ctx.compliance_forward(rm, m.pexp, m.e0, f, **fwd)
        d = (3 * m.conn[k][:, None] + np.arange(3)).ravel()
        ke, _ = O.element_ke(m.coords[m.conn[k]], 1.0, m.nu)
        dc = -(m.e0 * rp[k] ** m.pexp - m.e0 * rm[k] ** m.pexp) * (up[d] @ ke @ um[d])
        worst_exact = max(worst_exact, abs(dc / (2 * h) - g[k]) / abs(g[k]))
        worst_direct = max(worst_direct, abs((cp - cm) / (2 * h) - g[k]) / abs(g[k]))
    m.e_elem = m.e0 * m.rho ** m.pexp
    g_cpu = O.compliance_grad(m, m.rho, m.pexp, m.e0, u)
    oracle_check = oracle_residuals(m, {"forward_fp64": u64, "forward_mixed_coarse": u}, f)
    nf = ctx.n_free
    _line(args, "SIMP beam 100x50x50 C3D8, E=rho^3, rho~U[0.3,1], tip load", nf / t_fwd / 1e6, t_fwd * 1e3,
          {"dtype": "f32+f64", "config": {"workload": "C3D8 100x50x50 SIMP", "n_free": nf, "elements": m.n_elem,
                                          "forward": "mixed node-block, two-level preconditioner, rtol 1e-12"},
           "forward": {"iters": info.iters, "reliable_updates": info.outer_iters, "ms_solve": info.ms_solve,
                       "ms_total": t_fwd * 1e3, "compliance": c, "rel_err_vs_fp64": rel_u},
           "forward_fp64": {"iters": info64.iters, "ms_solve": info64.ms_solve, "ms_total": t_fwd64 * 1e3,
                            "compliance": c64},
           "backward_ms": t_bwd * 1e3,
           "gradient_vs_cpu_analytic_max_rel": float(np.abs(g - g_cpu).max() / np.abs(g_cpu).max()),
           "fd_20_elements": {"h": h, "max_rel_err_exact_difference": worst_exact,
                              "max_rel_err_direct_difference": worst_direct},
           "oracle_check": oracle_check})


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    vals = []
    info = None
    for k in range(args.warmup + args.steps):
        b = cpu_baseline(CPU_SAMPLE_N, threads)
        if k >= args.warmup:
            vals.append(b["value"])
            info = b
    v = statistics.median(vals)
    out = {"metric": METRIC, "value": v, "unit": "MDOF/s", "impl": "reference", "n_gpus": args.gpus,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": info["seconds"] * 1e3,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
           "data": "synthetic (seeded structured C3D8 block)",
           "config": {"workload": f"C3D8 block {CPU_SAMPLE_N}^3 sample of the 100^3 pressure block",
                      "rtol": RTOL, "threads": threads},
           "cpu_baseline": {"value": v, "unit": "MDOF/s", "cores": threads, "kind": "port",
                            "sample": info["sample"]},
           "e2e": {"value": v, "unit": "MDOF/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=100, help="edge count of the C3D8 block")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--lanes64", type=int, default=0)
    ap.add_argument("--lanes32", type=int, default=0)
    ap.add_argument("--lanes32csr", type=int, default=0)
    ap.add_argument("--delta", type=float, default=0.01, help="reliable-update residual reduction")
    ap.add_argument("--coarse-nodes", type=int, default=0,
                    help="nodes per subdomain of the coarse space (0: the library default, about 512 "
                         "subdomains of at least ~13,500 matrix node blocks)")
    ap.add_argument("--fp64-updates", action="store_true",
                    help="--only batch: FP64 reliable updates inside the kernel (no FP32 low parts)")
    ap.add_argument("--only", choices=["mixed", "coarse", "fp64", "spmv", "batch", "assemble"], default=None,
                    help="run one solve (or SpMV sweep) once and exit: the profiling entry")
    ap.add_argument("--max-iter", type=int, default=0, help="with --only: cap the CG iterations")
    ap.add_argument("--krylov", choices=["per-case", "block"], default="per-case",
                    help="with --only batch: one recurrence per load case, or the block PCG")
    ap.add_argument("--precond", choices=["jacobi", "coarse"], default="jacobi",
                    help="with --only batch: the diagonal or the two-level preconditioner")
    ap.add_argument("--workload", choices=["c2", "c3", "c4a", "c4b", "c5"], default="c2",
                    help="c2 (default): the 100^3 C3D8 block; others: the remaining configurations")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
        return
    if args.workload != "c2" and not (args.only == "assemble" and args.workload == "c3"):
        {"c3": run_c3, "c4a": run_c4a, "c4b": run_c4b, "c5": run_c5}[args.workload](args)
        return

    import numpy as np
    import torch

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    from axia_gpu import GpuContext, _lib as L, meshgen, replicas

    if args.only == "batch":
        # one batched solve of 32 load cases on an n^3 block: the profiling entry of the batched kernel
        m = meshgen.block_c3d8_multiload(n=args.n, nrhs=32)
        ctx = GpuContext(local)
        ctx.setup(m)
        ctx.assemble_ex(L.ASM_BSR64 | L.ASM_BSR32 | (0 if args.fp64_updates else L.ASM_BSR32LO))
        F = torch.from_numpy(m.cload_batch).to(f"cuda:{local}")
        U = torch.empty_like(F)
        try:
            kry = L.KRYLOV_BLOCK if args.krylov == "block" else L.KRYLOV_PER_CASE
            pre = L.PRECOND_COARSE if args.precond == "coarse" else L.PRECOND_JACOBI
            info, rel = ctx.solve_batched_device(32, F.data_ptr(), U.data_ptr(), rtol=RTOL, inner_rtol=args.delta,
                                                 max_iter=args.max_iter, krylov=kry, preconditioner=pre,
                                                 coarse_nodes=args.coarse_nodes)
            print(json.dumps({"only": "batch", "iters": info.iters, "updates": info.outer_iters, "ms_kernel": info.ms_pcg_kernel, "max_rel": float(max(rel))}))
        except Exception as e:  # a capped iteration count ends as NOT_CONVERGED
            print(json.dumps({"only": "batch", "status": str(e)[:120]}))
        torch.cuda.synchronize()
        return

    if args.only == "assemble" and args.workload == "c3":
        model = meshgen.block_c3d20_traction(n=args.n)  # the profiling entry of the C3D20 assembly
    else:
        model = meshgen.block_c3d8_pressure(n=args.n)
    ctx = GpuContext(local)
    stream = torch.cuda.Stream()
    ctx.set_stream(stream.cuda_stream)
    f_host = ctx.load_vector(model)
    t0 = time.perf_counter()
    ctx.setup(model)
    setup_s = time.perf_counter() - t0
    n, nnz = ctx.n_free, ctx.nnz
    f_dev = torch.from_numpy(f_host).to(f"cuda:{local}")
    u64 = torch.empty_like(f_dev)
    umx = torch.empty_like(f_dev)

    if args.only:
        if args.only == "assemble":
            # numeric assembly only (element kernel + gather into both node-block forms), three times
            for _ in range(3):
                ctx.assemble_ex(L.ASM_BSR64 | L.ASM_BSR32)
            el, ga = ctx.assemble_times()
            print(json.dumps({"only": "assemble", "ms_element": el, "ms_gather": ga, "n_elem": model.n_elem}))
            torch.cuda.synchronize()
            return
        if args.only == "spmv":
            ctx.assemble_ex(L.ASM_CSR64 | L.ASM_CSR32 | L.ASM_BSR64 | L.ASM_BSR32 | L.ASM_SYM32)
            nd = 3 * model.n_nodes
            xf32 = torch.rand(nd, device=f"cuda:{local}")
            yf32 = torch.empty_like(xf32)
            with torch.cuda.stream(stream):
                for _ in range(5):
                    ctx.bsr_spmv_device(L.PREC_MIXED, xf32.data_ptr(), yf32.data_ptr(), args.lanes32)
                for _ in range(5):
                    ctx.sym_spmv_device(xf32.data_ptr(), yf32.data_ptr(), 0)
        else:
            mixed = args.only in ("mixed", "coarse")
            ctx.assemble_ex((L.ASM_BSR64 | L.ASM_BSR32) if mixed else L.ASM_CSR64)
            kw = dict(precision=L.PREC_MIXED, refine_mode=L.REFINE_RELIABLE, inner_rtol=args.delta,
                      matrix_format=L.FORMAT_BSR3) if mixed else dict(precision=L.PREC_FP64)
            if args.only == "coarse":
                kw.update(preconditioner=L.PRECOND_COARSE, coarse_nodes=args.coarse_nodes)
            try:
                with torch.cuda.stream(stream):
                    info = ctx.solve_device(f_dev.data_ptr(), u64.data_ptr(), rtol=RTOL, max_iter=args.max_iter, **kw)
                print(json.dumps({"only": args.only, "iters": info.iters, "updates": info.outer_iters,
                                  "ms_kernel": info.ms_pcg_kernel, "n_nodes": model.n_nodes,
                                  "node_blocks": ctx.n_blocks(), "coarse": ctx.coarse_size()}))
            except Exception as e:  # a capped iteration count ends as NOT_CONVERGED
                print(json.dumps({"only": args.only, "status": str(e)[:120]}))
        torch.cuda.synchronize()
        return

    def barrier():
        torch.cuda.synchronize()
        if dist is not None:
            dist.barrier()

    def timed(asm_flags, solve_kw, u_dev, arith=L.ELEMENT_DWORD):
        ctx.set_element_arith(arith)
        infos = []
        times = []
        for k in range(args.warmup + args.steps):
            if k == args.warmup:
                barrier()
                l0 = ctx.kernel_launches()
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            with torch.cuda.stream(stream):
                a.record(stream)
                ctx.assemble_ex(asm_flags)
                info = ctx.solve_device(f_dev.data_ptr(), u_dev.data_ptr(), rtol=RTOL, **solve_kw)
                b.record(stream)
            b.synchronize()
            if k >= args.warmup:
                times.append(a.elapsed_time(b))
                infos.append(info.as_dict())
        barrier()
        launches = ctx.kernel_launches() - l0
        ctx.set_element_arith(L.ELEMENT_DWORD)
        ms = sum(times) / len(times)
        ms = replicas.max_over_ranks(ms, dist, f"cuda:{local}")
        return ms, infos, launches

    fp64_kw = dict(precision=L.PREC_FP64, spmv_lanes=args.lanes64, matrix_format=L.FORMAT_CSR)
    mixed_kw = dict(precision=L.PREC_MIXED, refine_mode=L.REFINE_RELIABLE, inner_rtol=args.delta,
                    spmv_lanes=args.lanes32, matrix_format=L.FORMAT_BSR3)
    mixed_csr_kw = dict(precision=L.PREC_MIXED, refine_mode=L.REFINE_RELIABLE, inner_rtol=args.delta,
                        spmv_lanes=args.lanes32csr, matrix_format=L.FORMAT_CSR)
    coarse_kw = dict(mixed_kw, preconditioner=L.PRECOND_COARSE, coarse_nodes=args.coarse_nodes)
    sym_kw = dict(coarse_kw, matrix_format=L.FORMAT_BSR3_SYM, spmv_lanes=0)
    umc = torch.empty_like(f_dev)
    uco = torch.empty_like(f_dev)
    ucs = torch.empty_like(f_dev)
    # layout of the FP32 inner loop, picked by the library's autotuner (untimed)
    ctx.assemble_ex(L.ASM_BSR64 | L.ASM_BSR32)
    tuned = {"lanes": None, "vec": None}
    if not args.lanes32:
        lanes_t, vec_t, us_t = ctx.autotune()
        tuned = {"lanes": lanes_t, "vec": vec_t, "us_per_iter": us_t}
    with ClockSampler(local) as clk:
        # the reference's algorithm throughout: FP64 element stiffness and assembly sums
        ms64, inf64, la64 = timed(L.ASM_CSR64, fp64_kw, u64, L.ELEMENT_FP64)
        msmx, infmx, lamx = timed(L.ASM_BSR64 | L.ASM_BSR32, mixed_kw, umx)
        msmc, infmc, lamc = timed(L.ASM_CSR64 | L.ASM_CSR32, mixed_csr_kw, umc)
        msco, infco, laco = timed(L.ASM_BSR64 | L.ASM_BSR32, coarse_kw, uco)
        mscs, infcs, lacs = timed(L.ASM_BSR64 | L.ASM_SYM32, sym_kw, ucs)
    clocks = clk.summary()
    n_sub, n_coarse = ctx.coarse_size()

    # standalone SpMV bandwidth: CSR FP64 / FP32 (K_ff, n_free vectors) and the
    # node-block form FP64 / FP32 (full-DOF vectors)
    nd = 3 * model.n_nodes
    spmv = {}
    x64 = torch.rand(n, dtype=torch.float64, device=f"cuda:{local}")
    y64 = torch.empty_like(x64)
    x32 = x64.float()
    y32 = torch.empty_like(x32)
    xf64 = torch.rand(nd, dtype=torch.float64, device=f"cuda:{local}")
    yf64 = torch.empty_like(xf64)
    xf32 = xf64.float()
    yf32 = torch.empty_like(xf32)
    nblocks = ctx.n_blocks()
    nbu, nbl = ctx.sym_blocks()
    cases = (("csr_fp64", ctx.spmv_device, L.PREC_FP64, x64, y64, spmv_bytes(nnz, n, 8), args.lanes64),
             ("csr_fp32", ctx.spmv_device, L.PREC_MIXED, x32, y32, spmv_bytes(nnz, n, 4), args.lanes32csr),
             ("bsr_fp64", ctx.bsr_spmv_device, L.PREC_FP64, xf64, yf64, bsr_spmv_bytes(nblocks, model.n_nodes, 8), 0),
             ("bsr_fp32", ctx.bsr_spmv_device, L.PREC_MIXED, xf32, yf32, bsr_spmv_bytes(nblocks, model.n_nodes, 4),
              args.lanes32),
             ("sym_fp32", lambda prec, x, y, lanes: ctx.sym_spmv_device(x, y, lanes), L.PREC_MIXED, xf32, yf32,
              sym_spmv_bytes(nbu, nbl, model.n_nodes), 0))
    for name, fn, prec, x, y, nbytes, lanes in cases:
        if name.startswith("csr"):
            ctx.assemble_ex(L.ASM_CSR64 | L.ASM_CSR32)
        elif name.startswith("sym"):
            ctx.assemble_ex(L.ASM_BSR64 | L.ASM_SYM32)
        else:
            ctx.assemble_ex(L.ASM_BSR64 | L.ASM_BSR32)
        with torch.cuda.stream(stream):
            for _ in range(3):
                fn(prec, x.data_ptr(), y.data_ptr(), lanes)
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            reps = 20
            a.record(stream)
            for _ in range(reps):
                fn(prec, x.data_ptr(), y.data_ptr(), lanes)
            b.record(stream)
        b.synchronize()
        ms = a.elapsed_time(b) / reps
        spmv[name] = {"ms": ms, "gbs": nbytes / (ms * 1e-3) / 1e9, "bytes": nbytes}

    pk, pk_kind = peaks()
    hbm = pk["hbm_gbs"]
    for v in spmv.values():
        v["frac_of_hbm"] = v["gbs"] / hbm

    # assembly phases (CUDA events inside the library), in both element
    # arithmetics: double words on the FP32 pipe (the default; issue bound) and
    # FP64 (the reference's; FP64-pipe bound), each against the measured FP64 FMA
    # rate in FP64-equivalent flops, the gathers against HBM
    def asm_times(arith):
        ctx.set_element_arith(arith)
        t = []
        for _ in range(4):
            ctx.assemble_ex(L.ASM_BSR64 | L.ASM_BSR32)
            t.append(ctx.assemble_times())
        ctx.set_element_arith(L.ELEMENT_DWORD)
        return statistics.median(a[0] for a in t[1:]), statistics.median(a[1] for a in t[1:])
    ms_el64, ms_ga64 = asm_times(L.ELEMENT_FP64)
    ms_el, ms_ga = asm_times(L.ELEMENT_DWORD)
    ctx.assemble_ex(L.ASM_BSR64 | L.ASM_BSR32)
    fp64_peak = ctx.fma_rate(L.PREC_FP64)
    fp32_peak = ctx.fma_rate(L.PREC_MIXED)
    el_flops = element_fp64_flops(model.nn, 8) * model.n_elem
    ga_bytes = gather_bytes(model.n_elem, model.nn, nblocks, model.n_nodes)
    assembly = {"ms_element": ms_el, "ms_gather": ms_ga,
                "element": {"kernel": "element_ke_dw_kernel<8,8,8>",
                            "arith": "double words (FP32 pairs, 48 significant bits) on the FP32 pipe",
                            "bound": "instruction issue (about 3,700 warp instructions per element)",
                            "fp64_equivalent_flops": el_flops,
                            "fp64_equivalent_tflops": el_flops / (ms_el * 1e-3) / 1e12,
                            "x_fp64_fma_peak": el_flops / (ms_el * 1e-3) / 1e12 / fp64_peak,
                            "canonical_flops_per_element": 32872},
                "element_fp64": {"kernel": "element_ke_kernel<8,8,8>", "bound": "fp64 pipe", "ms": ms_el64,
                                 "achieved_tflops": el_flops / (ms_el64 * 1e-3) / 1e12, "peak_tflops": fp64_peak,
                                 "frac": el_flops / (ms_el64 * 1e-3) / 1e12 / fp64_peak,
                                 "peak_source": "axia_gpu_fma_rate (FP64 FMA chains on every SM, CUDA events)"},
                "gather": {"kernel": "k_gather<true,8> (double-word sums)", "bound": "hbm", "bytes": ga_bytes,
                           "achieved_gbs": ga_bytes / (ms_ga * 1e-3) / 1e9,
                           "frac": ga_bytes / (ms_ga * 1e-3) / 1e9 / hbm},
                "gather_fp64": {"kernel": "k_gather<false,8> (FP64 sums)", "ms": ms_ga64,
                                "frac": ga_bytes / (ms_ga64 * 1e-3) / 1e9 / hbm},
                "fp32_fma_tflops_measured": fp32_peak}

    # post-solve recovery of the mixed solution: nodal stress, strain, von Mises,
    # element means and reactions K u - f (two kernels)
    nn_ = model.n_nodes
    rec_out = {k: torch.empty(sz, dtype=torch.float64, device=f"cuda:{local}")
               for k, sz in (("stress", 6 * nn_), ("strain", 6 * nn_), ("vm", nn_), ("rf", nd),
                             ("elem", 6 * model.n_elem))}
    e_ref = float(model.e_elem[0])

    def recover():
        ctx.recover_device(umx.data_ptr(), f_dev.data_ptr(), e_ref, rec_out["stress"].data_ptr(),
                           rec_out["strain"].data_ptr(), rec_out["vm"].data_ptr(), rec_out["rf"].data_ptr(),
                           rec_out["elem"].data_ptr())
    ms_rec, _ = Timer(torch, stream)(recover, 3, 10)
    rec_bytes = recover_bytes(model.n_elem, model.nn, nn_)
    recovery = {"ms": ms_rec, "bytes": rec_bytes, "gbs": rec_bytes / (ms_rec * 1e-3) / 1e9,
                "kernels": "element_recover_kernel<8,8> + k_recover_nodes",
                "bound": "fp64 pipe (about 7 kFLOP per C3D8 element)"}

    # accuracy: mixed vs FP64 solution, both with true FP64 residual <= 1e-10 ||b||, and both
    # against an FP64 solve to rtol 1e-12 (untimed; the direct oracle does not reach 3M DOF)
    u64h = u64.cpu().numpy()
    rel_mx = float(np.linalg.norm(umx.cpu().numpy() - u64h) / np.linalg.norm(u64h))
    rel_mc = float(np.linalg.norm(umc.cpu().numpy() - u64h) / np.linalg.norm(u64h))
    rel_co = float(np.linalg.norm(uco.cpu().numpy() - u64h) / np.linalg.norm(u64h))
    rel_cs = float(np.linalg.norm(ucs.cpu().numpy() - u64h) / np.linalg.norm(u64h))
    ctx.set_element_arith(L.ELEMENT_FP64)
    ctx.assemble_ex(L.ASM_CSR64)
    utight = torch.empty_like(f_dev)
    with torch.cuda.stream(stream):
        itight = ctx.solve_device(f_dev.data_ptr(), utight.data_ptr(), rtol=1e-12, precision=L.PREC_FP64)
    torch.cuda.synchronize()
    ctx.set_element_arith(L.ELEMENT_DWORD)
    uth = utight.cpu().numpy()
    tight = {"rtol": 1e-12, "iters": itight.iters, "true_rel_residual": itight.true_residual / itight.bnorm,
             "rel_err_fp64": float(np.linalg.norm(u64h - uth) / np.linalg.norm(uth)),
             "rel_err_mixed": float(np.linalg.norm(umx.cpu().numpy() - uth) / np.linalg.norm(uth)),
             "rel_err_mixed_csr": float(np.linalg.norm(umc.cpu().numpy() - uth) / np.linalg.norm(uth)),
             "rel_err_mixed_coarse": float(np.linalg.norm(uco.cpu().numpy() - uth) / np.linalg.norm(uth)),
             "rel_err_mixed_coarse_sym": float(np.linalg.norm(ucs.cpu().numpy() - uth) / np.linalg.norm(uth))}

    # full-size residual of every solution under the oracle's own stiffness (host, untimed)
    oracle_check = oracle_residuals(model, {"fp64": u64h, "mixed": umx.cpu().numpy(), "mixed_csr": umc.cpu().numpy(),
                                            "mixed_coarse": uco.cpu().numpy(), "mixed_coarse_sym": ucs.cpu().numpy(),
                                            "fp64_rtol_1e-12": uth}, f_host)

    last64, lastmx, lastmc, lastco, lastcs = inf64[-1], infmx[-1], infmc[-1], infco[-1], infcs[-1]
    itcs = statistics.mean(i["iters"] for i in infcs)
    kcs_ms = statistics.mean(i["ms_pcg_kernel"] for i in infcs)
    updcs = statistics.mean(i["outer_iters"] for i in infcs)
    bytescs = ((sym_pcg_iter_bytes(nbu, nbl, model.n_nodes) + coarse_iter_bytes(model.n_nodes, n_coarse)) * itcs +
               bsr_spmv_bytes(nblocks, model.n_nodes, 8) * updcs)
    achcs = bytescs / (kcs_ms * 1e-3) / 1e9
    mdofs_co = n / (msco * 1e-3) / 1e6 * world
    mdofs = n / (msmx * 1e-3) / 1e6 * world
    mdofs64 = n / (ms64 * 1e-3) / 1e6 * world
    mdofsmc = n / (msmc * 1e-3) / 1e6 * world

    # roofline of the dominant kernel: the persistent FP32 node-block PCG of the mixed step
    it32 = statistics.mean(i["iters"] for i in infmx)
    k32_ms = statistics.mean(i["ms_pcg_kernel"] for i in infmx)
    upd = statistics.mean(i["outer_iters"] for i in infmx)
    bytes32 = bsr_pcg_iter_bytes(nblocks, model.n_nodes, 4) * it32 + bsr_spmv_bytes(nblocks, model.n_nodes, 8) * upd
    ach32 = bytes32 / (k32_ms * 1e-3) / 1e9
    it64 = statistics.mean(i["iters"] for i in inf64)
    k64_ms = statistics.mean(i["ms_pcg_kernel"] for i in inf64)
    bytes64 = pcg_iter_bytes(nnz, n, 8) * it64
    ach64 = bytes64 / (k64_ms * 1e-3) / 1e9
    itco = statistics.mean(i["iters"] for i in infco)
    kco_ms = statistics.mean(i["ms_pcg_kernel"] for i in infco)
    updco = statistics.mean(i["outer_iters"] for i in infco)
    bytesco = ((bsr_pcg_iter_bytes(nblocks, model.n_nodes, 4) + coarse_iter_bytes(model.n_nodes, n_coarse)) * itco +
               bsr_spmv_bytes(nblocks, model.n_nodes, 8) * updco)
    achco = bytesco / (kco_ms * 1e-3) / 1e9
    itmc = statistics.mean(i["iters"] for i in infmc)
    kmc_ms = statistics.mean(i["ms_pcg_kernel"] for i in infmc)
    bytesmc = pcg_iter_bytes(nnz, n, 4) * itmc
    achmc = bytesmc / (kmc_ms * 1e-3) / 1e9

    e2e = None
    if not args.no_e2e:
        # through the C ABI with host buffers: setup (mesh upload) + assemble + solve (host f -> host u)
        # the inputs live in pinned host memory (as a caller's buffers would); u goes to pinned memory
        import copy

        def pinned(a):
            t = torch.empty(a.shape, dtype=getattr(torch, str(a.dtype)), pin_memory=True)
            arr = t.numpy()
            arr[...] = a
            return arr
        pm = copy.copy(model)
        pm.coords, pm.conn = pinned(np.ascontiguousarray(model.coords)), pinned(model.conn.astype(np.int32))
        pm.e_elem, pm.bc_dof, pm.bc_val = pinned(model.e_elem), pinned(model.bc_dof), pinned(model.bc_val)
        f_pin, u_pin = pinned(f_host), pinned(np.zeros_like(f_host))
        h2d = (pm.coords.nbytes + pm.conn.nbytes + pm.e_elem.nbytes + pm.bc_dof.nbytes + pm.bc_val.nbytes +
               f_pin.nbytes)
        d2h = u_pin.nbytes
        ctx.set_stream(None)
        mixed_kw["spmv_lanes"] = args.lanes32
        ts, phases = [], []
        for k in range(args.warmup + args.steps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            ctx.setup(pm)  # every call of the C ABI returns after its device work
            t1 = time.perf_counter()
            ctx.assemble_ex(L.ASM_BSR64 | L.ASM_BSR32)
            t2 = time.perf_counter()
            u, info = ctx.solve(f_pin, out=u_pin, rtol=RTOL, **coarse_kw)
            t3 = time.perf_counter()
            if k >= args.warmup:
                ts.append(t3 - t0)
                phases.append((t1 - t0, t2 - t1, t3 - t2))
        e2e_s = sum(ts) / len(ts)
        e2e_s = replicas.max_over_ranks(e2e_s, dist, f"cuda:{local}")
        e2e = {"value": n / e2e_s / 1e6 * world, "unit": "MDOF/s", "h2d_bytes_per_step": int(h2d),
               "d2h_bytes_per_step": int(d2h), "ms_per_step": e2e_s * 1e3,
               "phases_ms": {"setup (mesh upload + symbolic)": 1e3 * statistics.median(p[0] for p in phases),
                             "assemble": 1e3 * statistics.median(p[1] for p in phases),
                             "solve (f upload, coarse operator, CG, u copy back)":
                                 1e3 * statistics.median(p[2] for p in phases)}}

    same = None
    if rank == 0 and not args.no_cpu:
        same = same_sample_leg(args, local)
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        cpu = cpu_baseline(CPU_SAMPLE_N, os.cpu_count() or 1)
        cpu_iters, cpu_s = cpu.pop("iters"), cpu.pop("seconds")
        cpu.pop("n_free")
        if same is not None:
            same["cpu"] = {"value": cpu["value"], "iters": cpu_iters, "seconds": cpu_s, "threads": cpu["cores"],
                           "phases_s": cpu.pop("phases_s")}
            same["gpu_over_cpu_same_algorithm"] = same["fp64_jacobi"]["value"] / cpu["value"]
            same["gpu_over_cpu_headline"] = same["mixed_coarse"]["value"] / cpu["value"]
            same["gpu_over_cpu_headline_e2e"] = same["mixed_coarse_e2e"]["value"] / cpu["value"]
            same["jacobi_iterations"] = {f"{CPU_SAMPLE_N}^3 (CPU)": cpu_iters,
                                         f"{CPU_SAMPLE_N}^3 (GPU FP64)": same["fp64_jacobi"]["iters"],
                                         f"{args.n}^3 (GPU FP64)": inf64[-1]["iters"]}
        else:
            cpu.pop("phases_s", None)

    if rank != 0:
        if dist is not None:
            dist.destroy_process_group()
        return
    out = {
        "metric": METRIC, "value": mdofs_co, "unit": "MDOF/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": msco, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic (seeded perturbed structured C3D8 block)",
        "config": {"workload": f"C3D8 block {args.n}^3 unit elements, x=0 clamped, p=1 MPa on x=L, "
                               f"interior nodes perturbed +-0.15h", "n_free": n, "nnz_kff": nnz,
                   "rtol": RTOL, "step": "assemble + solve (symbolic setup once; the coarse operator is "
                                         "rebuilt from K in every step)",
                   "preconditioner": f"diagonal + coarse space ({n_sub} subdomains, {n_coarse} rigid-body modes)",
                   "l2": "inputs (2.9 GB matrix) larger than L2, no flush", "parallelism": f"replicas x{world}"},
        "fp64": {"value": mdofs64, "ms_per_step": ms64, "iters": last64["iters"], "format": "CSR int32",
                 "ms_assemble": last64["ms_assemble"], "ms_solve": last64["ms_solve"],
                 "true_rel_residual": last64["true_residual"] / last64["bnorm"]},
        "mixed_coarse": {"value": mdofs_co, "ms_per_step": msco, "inner_iters": lastco["iters"],
                         "reliable_updates": lastco["outer_iters"], "subdomains": n_sub, "coarse_unknowns": n_coarse,
                         "format": "3x3 node blocks, int32 block columns",
                         "ms_assemble": lastco["ms_assemble"], "ms_solve": lastco["ms_solve"],
                         "ms_pcg_kernel": lastco["ms_pcg_kernel"],
                         "ms_coarse_setup": lastco["ms_solve"] - lastco["ms_pcg_kernel"],
                         "true_rel_residual": lastco["true_residual"] / lastco["bnorm"], "rel_err_vs_fp64": rel_co},
        "mixed_coarse_sym": {"value": n / (mscs * 1e-3) / 1e6 * world, "ms_per_step": mscs,
                             "inner_iters": lastcs["iters"], "reliable_updates": lastcs["outer_iters"],
                             "format": "FP32 symmetric node blocks (upper blocks stored once) + FP64 node blocks",
                             "ms_assemble": lastcs["ms_assemble"], "ms_solve": lastcs["ms_solve"],
                             "ms_pcg_kernel": lastcs["ms_pcg_kernel"],
                             "true_rel_residual": lastcs["true_residual"] / lastcs["bnorm"], "rel_err_vs_fp64": rel_cs,
                             "roofline": {"achieved": achcs, "frac": achcs / hbm, "bytes_per_launch": bytescs,
                                          "ms_per_launch": kcs_ms}},
        "mixed": {"value": mdofs, "ms_per_step": msmx, "inner_iters": lastmx["iters"],
                  "reliable_updates": lastmx["outer_iters"], "format": "3x3 node blocks, int32 block columns",
                  "ms_assemble": lastmx["ms_assemble"], "ms_solve": lastmx["ms_solve"],
                  "true_rel_residual": lastmx["true_residual"] / lastmx["bnorm"], "rel_err_vs_fp64": rel_mx},
        "mixed_csr": {"value": mdofsmc, "ms_per_step": msmc, "inner_iters": lastmc["iters"],
                      "reliable_updates": lastmc["outer_iters"], "format": "CSR int32",
                      "ms_assemble": lastmc["ms_assemble"], "ms_solve": lastmc["ms_solve"],
                      "true_rel_residual": lastmc["true_residual"] / lastmc["bnorm"], "rel_err_vs_fp64": rel_mc},
        "vs_fp64_rtol_1e-12": tight,
        "layout_fp32": tuned,
        "speedup_mixed_vs_fp64": ms64 / msco,
        "speedup_mixed_jacobi_vs_fp64": ms64 / msmx,
        "speedup_coarse_vs_jacobi": msmx / msco,
        "speedup_mixed_vs_fp64_solve": last64["ms_solve"] / lastmx["ms_solve"],
        "speedup_mixed_csr_vs_fp64": ms64 / msmc,
        "setup_ms": setup_s * 1e3,
        "spmv": spmv,
        "recovery": recovery,
        "roofline": {"bound": "hbm", "achieved": achco, "peak": hbm, "unit": "GB/s", "frac": achco / hbm,
                     "traffic": None if COARSE_TRAFFIC_PER_ALG_BYTE is None else bytesco * COARSE_TRAFFIC_PER_ALG_BYTE,
                     "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of the same kernel at 60^3, "
                                       "per algorithmic byte, scaled to this launch",
                     "kernel": "pcg_bsr_reliable_kernel<8,4,true> (FP32 node-block CG, two-level preconditioner, "
                               "FP64 updates)",
                     "peak_source": f"{pk_kind} hbm_gbs", "bytes_per_launch": bytesco, "ms_per_launch": kco_ms},
        "roofline_mixed_jacobi": {"bound": "hbm", "achieved": ach32, "peak": hbm, "unit": "GB/s", "frac": ach32 / hbm,
                     "traffic": bytes32 * MIXED_TRAFFIC_PER_ALG_BYTE,
                     "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of the same kernel at 60^3, "
                                       "per algorithmic byte, scaled to this launch",
                     "kernel": "pcg_bsr_reliable_kernel (FP32 node-block CG + FP64 updates)",
                     "peak_source": f"{pk_kind} hbm_gbs", "bytes_per_launch": bytes32, "ms_per_launch": k32_ms},
        "roofline_fp64_pcg": {"bound": "hbm", "achieved": ach64, "peak": hbm, "unit": "GB/s", "frac": ach64 / hbm,
                              "kernel": "pcg_kernel<double> (CSR)", "ms_per_launch": k64_ms,
                              "bytes_per_launch": bytes64},
        "roofline_mixed_csr_pcg": {"bound": "hbm", "achieved": achmc, "peak": hbm, "unit": "GB/s",
                                   "frac": achmc / hbm, "kernel": "pcg_reliable_kernel (CSR FP32 + FP64 updates)",
                                   "ms_per_launch": kmc_ms, "bytes_per_launch": bytesmc},
        "assembly": assembly,
        "oracle_check": oracle_check,
        "same_sample": same,
        "gpu_launches": int(la64 + lamx + lamc + laco + lacs),
        "clocks": clocks,
        "e2e": e2e,
        "cpu_baseline": cpu,
    }
    print(json.dumps(out))
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
