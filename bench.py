"""Benchmark: miniFE CG solve to a 1e-8 relative residual on one GB300.

Workload (the FP64 GPU configuration): nx = ny = nz = 256 Hex8 box, 16,974,593
unknowns, 454,756,609 CSR nonzeros (FP64 values, int32 columns), reference
boundary conditions, unpreconditioned CG from x0 = 0 to ||r|| <= 1e-8 ||r0||.
A "step" is one full CG solve on the assembled system (assembly is timed
separately and reported beside it).  The matrix (5.5 GB) is far larger than
the 129 MB L2, so no L2 flush is needed between steps.

Keys beyond the base contract:
  e2e          the same solve through the host drop-in call
               (mfe_cg_solve_host: host CSR and b in pinned memory copied to the
               device inside the timed region, x copied back)
  roofline     the dominant kernel (the verified FP64 stencil SpMV) timed with
               CUDA events on its stream against the measured FP64 pipe rate,
               its HBM fraction beside it; traffic from the committed ncu
               summary.  fp64_csr_values carries the same solve with the CSR
               values and the box CSR SpMV's roofline against HBM.
  cpu_baseline the OpenMP CG port (oracle/cpu_baseline.c) on the host cores:
               one whole solve of the same system to the same tolerance
  --impl reference  times that CPU baseline as the reference arm, one whole
               solve per timed step.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

DIMS = (256, 256, 256)
TOL = 1e-8
METRIC = "CG time to 1e-8 rel. residual, mixed vs FP64 on GB300; SpMV GB/s vs HBM roof"
# FP64 FMA throughput of this machine's GB300 (597 G FMA/s = 1.19 TFLOP/s, 1.90
# FMA/clk/SM), measured with an FMA-only kernel; see profiles/.
FP64_PEAK_TFLOPS = 1.194


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def traffic_from_profile(key="bytes_per_launch_256"):
    """Per-launch DRAM bytes of an SpMV kernel at 256^3 from the committed
    ncu summary (captured on a smaller box, scaled by the units processed)."""
    path = os.path.join(ROOT, "profiles", "spmv_traffic.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d[key])
    except Exception:
        return None


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        sm.sort()
        med = sm[len(sm) // 2] if sm else None
        return {"sm_mhz": med, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_setup(ngpus):
    import torch
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if torch.cuda.is_available():
            torch.cuda.set_device(local)
        dist.init_process_group(backend=backend)
    elif torch.cuda.is_available():
        torch.cuda.set_device(0)
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(world, v):
    if world == 1:
        return v
    import torch
    import torch.distributed as dist
    dev = "cuda" if torch.cuda.is_available() else "cpu"
    t = torch.tensor([v], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# --------------------------------------------------------------------------
# CPU baseline (oracle/cpu_baseline.c, OpenMP port of the openmp/ variant)
# --------------------------------------------------------------------------
def workload_config(world, n, nnz, dims=DIMS):
    """The `config` both arms print: the 256^3 FP64 CG to 1e-8 relative."""
    return {"workload": "cg_f64_%d^3_to_1e-8_rel" % dims[0], "nx": dims[0], "ny": dims[1],
            "nz": dims[2], "rows": n, "nnz": nnz, "tol_rel": TOL,
            "l2": "inputs larger than L2", "parallelism": "replicas" if world > 1 else "single"}


def cpu_cg_solve(ro, cols, vals, b, max_iter=5000, tol=TOL, tol_mode=1):
    """One OpenMP CG solve from x0 = 0 (relative tolerance by default);
    returns (seconds, iterations, threads, x)."""
    import ctypes
    import numpy as np
    from oracle import oracle as O
    L = O.cpubase()
    x = np.zeros(b.size)
    nr = ctypes.c_double()
    t0 = time.perf_counter()
    it = L.cpub_cg_solve(b.size, ro, cols, vals, b, x, int(max_iter), float(tol), int(tol_mode),
                         ctypes.byref(nr))
    t1 = time.perf_counter()
    return t1 - t0, int(it), int(L.cpub_num_threads()), x


def host_system(A, b):
    """Copy the device system to host numpy arrays (bit-identical to the
    oracle's assembly, which the parity tests establish)."""
    import numpy as np
    ro = A.row_offsets.cpu().numpy()
    cols = A.packed_cols.cpu().numpy()
    vals = A.packed_coefs.cpu().numpy()
    bh = b.cpu().numpy()
    return (np.ascontiguousarray(ro), np.ascontiguousarray(cols), np.ascontiguousarray(vals),
            np.ascontiguousarray(bh))


def run_reference(args):
    """Reference arm: the OpenMP CG port on all host cores.  Every timed step
    is one whole solve of the 256^3 system from x0 = 0 to the 1e-8 relative
    residual (its own iteration count, measured, not scaled).  Warm-up steps
    are bounded: a short solve (--ref-warmup-iters iterations) each, which
    pages the arrays in and starts the thread pool."""
    world, rank, local = dist_setup(args.gpus)
    if rank != 0:
        return 0
    from oracle import oracle as O
    O.build()
    # the system is built on the host by the oracle (the reference's element
    # loop restated), so no GPU code runs in this arm
    dims = (args.ref_dims,) * 3
    t0 = time.perf_counter()
    ro, cols, vals, bh = O.build_system(*dims)
    log("reference arm: host assembly of %dx%dx%d took %.1f s" % (*dims, time.perf_counter() - t0))
    for _ in range(args.warmup):
        cpu_cg_solve(ro, cols, vals, bh, max_iter=args.ref_warmup_iters)
    ts, its = [], []
    threads = 1
    for _ in range(args.steps):
        dt, it, threads, _ = cpu_cg_solve(ro, cols, vals, bh)
        ts.append(dt)
        its.append(it)
        log("reference arm: solve %.2f s, %d iterations" % (dt, it))
    value = sum(ts) / len(ts)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": value * 1e3, "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (miniFE %d^3 box generated on the host by the oracle)" % dims[0],
        "config": workload_config(1, ro.size - 1, cols.size, dims),
        "iterations": {"min": min(its), "max": max(its)},
        "cpu_baseline": {"value": value, "unit": "s", "cores": threads, "kind": "port",
                         "sample": "whole OpenMP CG solves of the %d^3 system to 1e-8 relative "
                                   "(%d-%d iterations), one per step, averaged over %d steps"
                                   % (dims[0], min(its), max(its), args.steps)},
        "e2e": {"value": value, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# --------------------------------------------------------------------------
# GPU arm
# --------------------------------------------------------------------------
def run_gpu(args):
    import numpy as np
    import torch
    world, rank, local = dist_setup(args.gpus)
    import minife_gb300 as M
    dev = torch.cuda.current_device()
    n, nnz = M.box_dims(*DIMS)
    stream = torch.cuda.current_stream()

    # assembly (timed separately, like the reference's "FE assembly Time")
    A = M.CSRMatrix.empty_box(*DIMS)
    b = torch.empty(n, dtype=torch.float64, device="cuda")
    M.assemble_FE_data(*DIMS, A, b, impose_bc=True)
    torch.cuda.synchronize()
    ta = []
    for _ in range(2):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        M.assemble_FE_data(*DIMS, A, b, impose_bc=True)
        e1.record(stream)
        torch.cuda.synchronize()
        ta.append(e0.elapsed_time(e1) * 1e-3)
    t_assembly = min(ta)

    def time_solves(op):
        """CUDA-event time per whole FP64 solve with the given operator."""
        xx = torch.zeros_like(b)
        for _ in range(args.warmup):
            xx.zero_()
            M.cg_solve(A, b, xx, max_iter=5000, tol=TOL, tol_mode="relative", f64_operator=op)
        torch.cuda.synchronize()
        barrier(world)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        its = []
        for _ in range(args.steps):
            xx.zero_()
            r = M.cg_solve(A, b, xx, max_iter=5000, tol=TOL, tol_mode="relative", f64_operator=op)
            its.append(r.num_iters)
        e1.record(stream)
        torch.cuda.synchronize()
        barrier(world)
        return max_over_ranks(world, e0.elapsed_time(e1) * 1e-3 / args.steps), r, xx

    sampler = ClockSampler(dev) if rank == 0 else None
    if sampler:
        sampler.start()
    # headline: the FP64 solve as mfe_cg_solve runs it by default (the
    # verified FP64 stencil operator; its per-call check of every entry of A
    # and the final residual with the CSR values are inside the timed region)
    t_step, res, x = time_solves("auto")
    rel = res.normr / res.normr0
    final_rel = res.final_resid / res.normr0
    rc, err = M.verify_solution(*DIMS, x)
    # the same solve with the CSR values (matvec_std) for every product
    t_csr, res_csr, x_csr = time_solves("csr")
    d_ops = float((x - x_csr).norm() / x_csr.norm())
    del x_csr

    # dominant kernels timed alone on the same stream with CUDA events: the
    # FP64 stencil SpMV of the headline solve and the CSR SpMV (with its
    # fused p.Ap in the CSR solve)
    p = torch.randn(n, dtype=torch.float64, device="cuda")
    Ap = torch.empty_like(p)
    S = M.Stencil64(A)

    def time_kernel(fn, R=20):
        for _ in range(3):
            fn()
        torch.cuda.synchronize()
        k0 = torch.cuda.Event(enable_timing=True)
        k1 = torch.cuda.Event(enable_timing=True)
        k0.record(stream)
        for _ in range(R):
            fn()
        k1.record(stream)
        torch.cuda.synchronize()
        return k0.elapsed_time(k1) * 1e-3 / R

    t_st = time_kernel(lambda: M.matvec_stencil64(S, p, Ap))
    t_spmv = time_kernel(lambda: M.matvec(A, p, Ap))
    clocks = sampler.stop() if sampler else None
    # stencil SpMV: x read once and y written once (16 B/row); 13.5 FP64
    # operations per row (class sums 3.5, two plane partials 8, final add 1,
    # p.Ap 1; the timed standalone launch has no dot: 12.5)
    st_bytes = 16 * n
    st_ops = 12.5 * n
    # the box-structured CSR kernel reads the values only (columns and row
    # offsets follow from the box): 8 bytes per nonzero + x and y once
    spmv_bytes = nnz * 8 + 2 * n * 8
    csr_equiv_bytes = nnz * (8 + 4) + (n + 1) * 4 + 2 * n * 8
    # CG iteration bytes: stencil SpMV 16 B/row, update 48, p update 24
    iter_bytes_st = 88 * n
    iter_bytes_csr = nnz * 8 + 11 * n * 8
    peak, peak_kind = peaks()
    achieved = spmv_bytes / t_spmv / 1e9
    traffic = traffic_from_profile()

    # e2e through the host drop-in call (pinned host CSR, copies inside).
    # Each call is timed on its own; the host x is zeroed between calls,
    # outside the timed region, as the reference arm allocates its x outside.
    # The call copies the values, b and x in and x out.  With x0 = 0 it
    # starts the stencil solve at once, while the values are copied and
    # checked on a second stream and the host threads check the layout; the
    # result counts once all have passed (a verified box layout is not
    # copied).
    e2e = None
    if not args.no_e2e:
        ro_h = A.row_offsets.cpu().pin_memory()
        cols_h = A.packed_cols.cpu().pin_memory()
        vals_h = A.packed_coefs.cpu().pin_memory()
        b_h = b.cpu().pin_memory()
        x_h = torch.zeros(n, dtype=torch.float64).pin_memory()
        M.cg_solve_host(ro_h, cols_h, vals_h, b_h, x_h, max_iter=5000, tol=TOL,
                        tol_mode="relative")
        barrier(world)
        t_calls = 0.0
        for _ in range(args.steps):
            x_h.zero_()
            t0 = time.perf_counter()
            r2 = M.cg_solve_host(ro_h, cols_h, vals_h, b_h, x_h, max_iter=5000, tol=TOL,
                                 tol_mode="relative")
            t_calls += time.perf_counter() - t0
        barrier(world)
        t_e2e = max_over_ranks(world, t_calls / args.steps)
        h2d = 8 * nnz + 8 * n + 8 * n
        e2e = {"value": t_e2e, "unit": "s", "h2d_bytes_per_step": h2d,
               "d2h_bytes_per_step": 8 * n, "iterations": r2.num_iters,
               "ratio_to_device_solve": t_e2e / t_step,
               "structure": "row offsets and columns checked on the host against the box "
                            "layout, not copied",
               "start": ("speculative: the solve ran beside the values copy and checks"
                         if r2.inner_operator == "stencil64" and r2.fp64_spmvs == 1
                         else "after the values copy"),
               "csr_products": r2.fp64_spmvs}
        del ro_h, cols_h, vals_h

    # mixed precision (FP32 inner operator and vectors, FP64 dots and reliable
    # updates) to the same FP64-verified tolerance, same system, same timing
    # rules.  The default inner operator is the verified FP32 stencil (its
    # per-call verification of every row is inside the timed region); the
    # FP32 copy of the values (prepared once, outside) is timed beside it.
    mixed = None
    if not args.no_mixed:
        x64 = x.clone()
        xm = torch.zeros_like(b)
        from minife_gb300 import autotune
        if args.refine_k > 0:
            mcfg = {"refine_k": args.refine_k, "inner_tol": 0.01, "cached": None}
        else:
            mcfg = autotune.tune_mixed(A, b, tol=TOL, reps=1)

        def time_mixed(A32):
            kw = dict(max_iter=5000, tol=TOL, tol_mode="relative", precision="mixed",
                      refine_k=mcfg["refine_k"], inner_tol=mcfg["inner_tol"], A32=A32)
            for _ in range(args.warmup):
                xm.zero_()
                M.cg_solve(A, b, xm, **kw)
            torch.cuda.synchronize()
            barrier(world)
            m0 = torch.cuda.Event(enable_timing=True)
            m1 = torch.cuda.Event(enable_timing=True)
            m0.record(stream)
            for _ in range(args.steps):
                xm.zero_()
                rm = M.cg_solve(A, b, xm, **kw)
            m1.record(stream)
            torch.cuda.synchronize()
            barrier(world)
            return max_over_ranks(world, m0.elapsed_time(m1) * 1e-3 / args.steps), rm

        A32 = M.to_f32(A)
        t_values, rv = time_mixed(A32)
        del A32
        t_mixed, rm = time_mixed(None)
        rcm, errm = M.verify_solution(*DIMS, xm)
        diff = xm - x64
        mixed = {"value": t_mixed, "unit": "s", "speedup_vs_fp64": t_step / t_mixed,
                 "speedup_vs_fp64_csr_values": t_csr / t_mixed,
                 "inner_operator": rm.inner_operator,
                 "inner_iterations": rm.num_iters, "reliable_updates": rm.refinements,
                 "tuning": {"refine_k": mcfg["refine_k"], "inner_tol": mcfg["inner_tol"]},
                 "tuned_from_cache": mcfg.get("cached"), "status": rm.status,
                 "final_rel_resid_fp64": rm.final_resid / rm.normr0,
                 "err_vs_fp64_solution": {"rel_l2": float(diff.norm() / x64.norm()),
                                          "max_abs": float(diff.abs().max())},
                 "analytic_check": {"max_err": errm, "passed": rcm == 0},
                 "values_copy": {"value": t_values, "unit": "s",
                                 "speedup_vs_fp64": t_step / t_values,
                                 "inner_iterations": rv.num_iters, "status": rv.status},
                 "dtype": "f32 inner operator/vectors, f64 dots/scalars/solution"}
        del xm, x64

    # launches of the timed headline region: per CG iteration the SpMV, the
    # update and the p update; per solve the stencil check (table, its reset
    # and the row-by-row check), the initial residual, the graph's begin
    # node and the final residual with the CSR values
    gpu_launches = args.steps * (3 * res.num_iters + 6)

    # the rows after the hot path on the same system: ELL storage and the
    # Jacobi-preconditioned CG
    next_rows = None if args.no_next else bench_next_rows(args, world, stream, A, b)

    # batched uneven boxes and multi-RHS: measured after the headline system
    # is released, so their stores have the memory
    batch = multi = adjoint = small = None
    if rank == 0 and not args.no_cpu:
        ro, cols, vals, bh = host_system(A, b)
    else:
        ro = cols = vals = bh = None
    if not args.no_batch or not args.no_multi or not args.no_adjoint:
        del A, b, x, p, Ap
        torch.cuda.empty_cache()
        if not args.no_batch:
            batch = bench_batch(args, world, stream)
        if not args.no_multi:
            multi = bench_multi(args, world, stream)
        if not args.no_adjoint:
            adjoint = bench_adjoint(args, world, stream)
    if not args.no_small:
        small = bench_small(args, world, stream)

    cpu = None
    if rank == 0 and not args.no_cpu:
        dt, it_cpu, threads, _ = cpu_cg_solve(ro, cols, vals, bh)
        cpu = {"value": dt, "unit": "s", "cores": threads, "kind": "port",
               "sample": "one whole OpenMP CG solve of the 256^3 system to 1e-8 relative "
                         "(%d iterations)" % it_cpu}

    if rank == 0:
        line = {
            "metric": METRIC, "value": t_step, "unit": "s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_step * 1e3,
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (miniFE 256^3 box generated on the device; matrix 5.5 GB > L2, "
                    "no flush needed)",
            "config": workload_config(world, n, nnz),
            "iterations": res.num_iters,
            "operator": res.inner_operator,
            "final_rel_resid": final_rel, "reported_rel_normr": rel,
            "analytic_check": {"max_err": err, "passed": rc == 0},
            "ms_per_iter": t_step / res.num_iters * 1e3,
            "cg_hbm_gbs": iter_bytes_st * res.num_iters / t_step / 1e9,
            "assembly_s": t_assembly,
            "fp64_csr_values": {
                "value": t_csr, "unit": "s", "iterations": res_csr.num_iters,
                "speedup_of_headline": t_csr / t_step,
                "final_rel_resid": res_csr.final_resid / res_csr.normr0,
                "rel_l2_diff_vs_headline_x": d_ops,
                "ms_per_iter": t_csr / res_csr.num_iters * 1e3,
                "cg_hbm_gbs": iter_bytes_csr * res_csr.num_iters / t_csr / 1e9,
                "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                             "frac": achieved / peak, "traffic": traffic,
                             "kernel": "k_spmv_box<double> (FP64 box-structured CSR SpMV)",
                             "algorithmic_bytes": spmv_bytes,
                             "peak_kind": peak_kind + " (HBM copy)",
                             "csr_equivalent_gbs": csr_equiv_bytes / t_spmv / 1e9,
                             "fp64_pipe": {"achieved_gops": nnz / t_spmv / 1e9,
                                           "peak_gops": FP64_PEAK_TFLOPS / 2 * 1e3,
                                           "frac": nnz / t_spmv / 1e9 / (FP64_PEAK_TFLOPS / 2 * 1e3)}},
            },
            "mixed": mixed,
            "next_rows": next_rows,
            "batch": batch,
            "multi_rhs": multi,
            "adjoint": adjoint,
            "small_30cubed": small,
            "roofline": {"bound": "fp64", "achieved": st_ops / t_st / 1e9,
                         "peak": FP64_PEAK_TFLOPS / 2 * 1e3, "unit": "G FP64 op/s",
                         "frac": st_ops / t_st / 1e9 / (FP64_PEAK_TFLOPS / 2 * 1e3),
                         "traffic": traffic_from_profile("st64_bytes_per_launch_256"),
                         "kernel": "k_spmv_st64 (verified FP64 stencil SpMV, 12.5 FP64 operations "
                                   "per row without the fused dot)",
                         "kernel_ms": t_st * 1e3, "algorithmic_ops": st_ops,
                         "peak_kind": "measured (FP64 FMA-only kernel, one operation per FMA)",
                         "hbm": {"achieved_gbs": st_bytes / t_st / 1e9, "peak_gbs": peak,
                                 "frac": st_bytes / t_st / 1e9 / peak,
                                 "algorithmic_bytes": st_bytes}},
            "e2e": e2e,
            "cpu_baseline": cpu,
            "gpu_launches": gpu_launches,
            "clocks": clocks,
        }
        print(json.dumps(line), flush=True)
    return 0


SEED = 20261201  # S: adjoint conductivity S, target S + 1, FD elements S + 2, batch S + 3


def bench_next_rows(args, world, stream, A, b):
    """The rows after the hot path, measured on the 256^3 system: ELL storage
    (ELLMatrix: 27 entries per row, the reference's padded layout) -- its
    conversion from the CSR, its matvec against the bytes it moves (every
    padded entry's value and column, x and y once) and the FP64 CG with it to
    1e-8 relative -- the Jacobi-preconditioned CG to 1e-8 relative on the
    CSR, and a CSR that is not a box matrix: its FP64 CG to 1e-8 and its
    matvec against the bytes it moves.  CUDA events, warm-up first."""
    import torch
    import minife_gb300 as M
    n = A.nrows
    peak, _ = peaks()

    def ev_time(fn, reps):
        fn()
        torch.cuda.synchronize()
        barrier(world)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        out = None
        for _ in range(reps):
            out = fn()
        e1.record(stream)
        torch.cuda.synchronize()
        barrier(world)
        return max_over_ranks(world, e0.elapsed_time(e1) * 1e-3 / reps), out

    t_conv, E = ev_time(lambda: M.ELLMatrix.from_csr(A), 1)
    K = E.num_cols_per_row
    x = torch.randn(n, dtype=torch.float64, device="cuda")
    y = torch.empty_like(x)
    t_mv, _ = ev_time(lambda: M.matvec_ell(E, x, y), 10)
    ell_bytes = n * K * (8 + 4) + 2 * n * 8
    # the sliced copy the ELL CG iterates on (the same entries, 32-row
    # slices column-major)
    t_sconv, S = ev_time(lambda: M.SELLMatrix.from_ell(E), 1)
    t_smv, _ = ev_time(lambda: M.matvec_sell(S, x, y), 10)
    sell_bytes = M.SELLMatrix.entries(n, K) * (8 + 4) + 2 * n * 8
    del S
    torch.cuda.empty_cache()
    xs = torch.zeros_like(b)

    def ell_solve():
        xs.zero_()
        return M.cg_solve_ell(E, b, xs, max_iter=5000, tol=TOL, tol_mode="relative")

    t_ell, r_ell = ev_time(ell_solve, 1)
    ell_rel = r_ell.final_resid / r_ell.normr0
    del E, x, y
    torch.cuda.empty_cache()

    def pcg_solve():
        xs.zero_()
        return M.cg_solve(A, b, xs, max_iter=5000, tol=TOL, tol_mode="relative", precond="jacobi")

    t_pcg, r_pcg = ev_time(pcg_solve, 1)

    # any CSR that is not a box matrix: the same operator with one interior
    # row's columns (and values) rotated, so the box layout check fails and
    # the FP64 CG iterates on a sliced copy of the CSR
    Nx = DIMS[0] + 1
    row = (Nx * Nx) * (DIMS[2] // 2) + Nx * (DIMS[1] // 2) + DIMS[0] // 2
    a, e = int(A.row_offsets[row]), int(A.row_offsets[row + 1])
    gcols = A.packed_cols.clone()
    gvals = A.packed_coefs.clone()
    gcols[a:e] = torch.roll(gcols[a:e], 1)
    gvals[a:e] = torch.roll(gvals[a:e], 1)
    G = M.CSRMatrix(A.row_offsets, gcols, gvals)

    def gen_solve():
        xs.zero_()
        return M.cg_solve(G, b, xs, max_iter=5000, tol=TOL, tol_mode="relative")

    t_gen, r_gen = ev_time(gen_solve, 1)
    # the same CSR's matvec: the warp-staged kernel (rows of <= 32 entries)
    xg = torch.randn(n, dtype=torch.float64, device="cuda")
    yg = torch.empty_like(xg)
    t_gmv, _ = ev_time(lambda: M.matvec(G, xg, yg), 10)
    gen_bytes = A.nnz * (8 + 4) + n * 20
    del xs, G, gcols, gvals, xg, yg
    torch.cuda.empty_cache()
    return {
        "ell": {"conversion_s": t_conv, "cg_s": t_ell, "iterations": r_ell.num_iters,
                "final_rel_resid": ell_rel, "ncols_per_row": K,
                "cg_operator": "sliced ELL copy (32-row slices), made inside the call",
                "spmv": {"ms": t_mv * 1e3, "bytes": ell_bytes,
                         "achieved_gbs": ell_bytes / t_mv / 1e9, "peak_gbs": peak,
                         "frac": ell_bytes / t_mv / 1e9 / peak},
                "sell_conversion_s": t_sconv,
                "sell_spmv": {"ms": t_smv * 1e3, "bytes": sell_bytes,
                              "achieved_gbs": sell_bytes / t_smv / 1e9, "peak_gbs": peak,
                              "frac": sell_bytes / t_smv / 1e9 / peak,
                              "fp64_fma_frac": n * K / t_smv / (FP64_PEAK_TFLOPS * 0.5e12)}},
        "pcg_jacobi": {"value": t_pcg, "unit": "s", "iterations": r_pcg.num_iters,
                       "final_rel_resid": r_pcg.final_resid / r_pcg.normr0,
                       "operator": r_pcg.inner_operator},
        "generic_csr_cg": {"value": t_gen, "unit": "s", "iterations": r_gen.num_iters,
                           "final_rel_resid": r_gen.final_resid / r_gen.normr0,
                           "what": "FP64 CG on a CSR that is not a box matrix (one row's "
                                   "columns rotated): the iterations on its sliced copy",
                           "spmv": {"ms": t_gmv * 1e3, "bytes": gen_bytes,
                                    "achieved_gbs": gen_bytes / t_gmv / 1e9, "peak_gbs": peak,
                                    "frac": gen_bytes / t_gmv / 1e9 / peak,
                                    "kernel": "k_spmv_staged (a warp per 32-row group)"}},
    }


def bench_small(args, world, stream):
    """The reference's CPU-sized case, 30^3 (29,791 rows): FP64 CG to 1e-8
    relative (max 200 iterations) and to the reference's own stop (absolute
    DBL_EPSILON, max 200), GPU time per solve by CUDA events, beside the
    OpenMP CPU baseline on the same host arrays (rank 0)."""
    import torch
    import minife_gb300 as M
    A, b = M.build_system(30, 30, 30)
    out = {"system": "30^3", "rows": A.nrows, "nnz": A.nnz}
    for name, tol, mode in (("rel_1e-8", TOL, "relative"), ("abs_eps", 2.220446049250313e-16, "absolute")):
        x = torch.zeros_like(b)
        for _ in range(args.warmup):
            x.zero_()
            r = M.cg_solve(A, b, x, max_iter=200, tol=tol, tol_mode=mode)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            x.zero_()
            r = M.cg_solve(A, b, x, max_iter=200, tol=tol, tol_mode=mode)
        e1.record(stream)
        torch.cuda.synchronize()
        out[name] = {"gpu_s": max_over_ranks(world, e0.elapsed_time(e1) * 1e-3 / args.steps),
                     "iterations": r.num_iters, "normr": r.normr}
    if not args.no_cpu and (world == 1 or int(os.environ.get("RANK", "0")) == 0):
        import ctypes
        import numpy as np
        from oracle import oracle as O
        ro, cols, vals, bh = host_system(A, b)
        L = O.cpubase()
        nr = ctypes.c_double()
        best = None
        for _ in range(3):
            xh = np.zeros(bh.size)
            t0 = time.perf_counter()
            L.cpub_cg_solve(bh.size, ro, cols, vals, bh, xh, 200, TOL, 1, ctypes.byref(nr))
            dt = time.perf_counter() - t0
            best = dt if best is None else min(best, dt)
        out["cpu_port_rel_1e-8_s"] = best
        out["cpu_cores"] = int(L.cpub_num_threads())
    return out


def bench_adjoint(args, world, stream):
    """Gradient of L = 1/2 ||u - u_target||^2 with respect to per-element
    conductivity on 128^3 (2,097,152 elements): kappa = exp(g), g ~ N(0, 0.5^2)
    (seed S), u_target = the solution at kappa * exp(N(0, 0.05^2)) (seed S + 1),
    FP64 forward and adjoint CG to 1e-10 relative.  Timed: the native
    mfe_adjoint_grad call (assembly with kappa, forward solve, adjoint solve,
    element contraction), CUDA events.  Checked: central differences h = 1e-6
    on 64 elements drawn with seed S + 2 (error relative to the gradient's
    largest magnitude, as the tests; the per-element relative error of
    near-zero components is reported beside it)."""
    import torch
    from minife_gb300 import adjoint as ad
    d = args.adjoint_dims
    E = d ** 3
    g0 = torch.Generator().manual_seed(SEED)
    kappa = torch.exp(0.5 * torch.randn(E, generator=g0, dtype=torch.float64)).cuda()
    g1 = torch.Generator().manual_seed(SEED + 1)
    kt = kappa * torch.exp(0.05 * torch.randn(E, generator=g1, dtype=torch.float64)).cuda()
    u_target = ad.solve(kt, (d, d, d), tol=1e-12).detach()
    for _ in range(max(1, args.warmup)):
        ad.grad_l2(kappa, (d, d, d), u_target, tol=1e-10)
    torch.cuda.synchronize()
    barrier(world)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    steps = max(1, min(args.steps, 3))
    e0.record(stream)
    for _ in range(steps):
        loss, grad, u = ad.grad_l2(kappa, (d, d, d), u_target, tol=1e-10)
    e1.record(stream)
    torch.cuda.synchronize()
    barrier(world)
    t = max_over_ranks(world, e0.elapsed_time(e1) * 1e-3 / steps)
    g2 = torch.Generator().manual_seed(SEED + 2)
    elems = torch.randperm(E, generator=g2)[:args.adjoint_fd]
    fd = ad.finite_difference(kappa, (d, d, d), u_target, elems.tolist(), h=1e-6)
    ga = grad[elems.cuda()].cpu()
    err_scaled = float((ga - fd).abs().max() / grad.abs().max().cpu())
    rel = float(((ga - fd).abs() / fd.abs().clamp_min(1e-300)).max())
    return {"value": t, "unit": "s", "system": "%d^3" % d, "elements": E,
            "what": "one gradient: assembly with kappa, FP64 forward + adjoint CG to 1e-10, "
                    "element contraction (mfe_adjoint_grad)",
            "loss": loss, "fd_elements": int(elems.numel()), "fd_h": 1e-6,
            "fd_max_err_over_max_grad": err_scaled, "fd_max_rel_err_per_element": rel}


def batch_dims(nbox=96, lo=32, hi=160, seed=20261204):
    """Seeded uneven boxes: nx, ny, nz uniform in {lo..hi} (the first nbox
    of the 96-box sequence)."""
    import numpy as np
    rng = np.random.default_rng(seed)
    dims = [tuple(int(v) for v in rng.integers(lo, hi + 1, size=3)) for _ in range(96)]
    return dims[:nbox]


def bench_batch(args, world, stream):
    """96 uneven boxes (seeded, each dimension uniform in 32..160), each with
    the miniFE right-hand side, assembled once and solved together in mixed
    precision to 1e-8 relative (every box stopping on its true FP64
    residual), launch shape and refine_k from the autotuner.  Timed: the
    batched solve (one graph launch) per step; the sequential baseline is
    the same boxes solved one after another with the single-box mixed
    solver at the same refine_k."""
    import torch
    import minife_gb300 as M
    from minife_gb300 import autotune
    dims = batch_dims()
    bt = M.Batch(dims)
    rows, nnz, t_asm, _ = bt.info()
    cfg = autotune.tune_batch(bt, precision="mixed", tol=TOL, probe_iters=30, reps=1)
    x = torch.empty(bt.offsets[-1], dtype=torch.float64, device="cuda")
    for _ in range(max(1, args.warmup - 1)):
        bt.solve(max_iter=5000, tol=TOL, tol_mode="relative", precision="mixed",
                 refine_k=cfg["refine_k"], x=x)
    torch.cuda.synchronize()
    barrier(world)
    ts = []
    for _ in range(args.steps):
        _, res = bt.solve(max_iter=5000, tol=TOL, tol_mode="relative", precision="mixed",
                          refine_k=cfg["refine_k"], x=x)
        ts.append(res[0].times[4])
    barrier(world)
    t = max_over_ranks(world, sum(ts) / len(ts))
    its = [r.num_iters for r in res]
    work = sum(r.num_iters * M.box_dims(*d)[1] for r, d in zip(res, dims))
    _, res64 = bt.solve(max_iter=5000, tol=TOL, tol_mode="relative", precision="f64", x=x)
    out = {"boxes": len(dims), "dims": "seeded U{32..160}^3 (numpy default_rng(20261204))",
           "rows": rows, "nnz": nnz, "assembly_s": t_asm, "value": t, "unit": "s",
           "tuning": {k: cfg[k] for k in ("spmv_rows", "spmv_stages", "chunk_rows", "refine_k")},
           "tuned_from_cache": cfg.get("cached", False),
           "iterations": {"min": min(its), "max": max(its)},
           "all_converged": all(r.status == 0 for r in res),
           "max_rel_resid": max(r.final_resid / r.normr0 for r in res),
           "nnz_iterations_per_s": work / t,
           "fp64_batched_s": res64[0].times[4]}
    bt.close()
    del x
    if not args.no_seq:
        t_seq = 0.0
        for d in dims:
            A, b = M.build_system(*d)
            xx = torch.zeros_like(b)
            r = M.cg_solve(A, b, xx, max_iter=5000, tol=TOL, tol_mode="relative",
                           precision="mixed", refine_k=cfg["refine_k"])
            t_seq += r.total_time
            del A, b, xx
        out["sequential_mixed_s"] = t_seq
        out["sequential_refine_k"] = cfg["refine_k"]
        out["speedup_vs_sequential"] = t_seq / t
    return out


def bench_multi(args, world, stream):
    """32 seeded random-normal right-hand sides on the 128^3 system, solved
    together (one SpMM per iteration) in mixed precision to 1e-8 relative,
    launch shape and reliable-update policy from the autotuner; beside it the
    same 32 solves one after another with the single-box mixed solver
    (its own tuned policy for this box)."""
    import torch
    import minife_gb300 as M
    from minife_gb300 import autotune
    A, b = M.build_system(128, 128, 128)
    g = torch.Generator(device="cpu").manual_seed(0)
    B = torch.randn(A.nrows, 32, generator=g, dtype=torch.float64).cuda().contiguous()
    X = torch.zeros_like(B)
    cfg = autotune.tune_multi(A, B, X, tol=TOL, reps=1)
    kw = dict(max_iter=5000, tol=TOL, tol_mode="relative", precision="mixed",
              refine_k=cfg["refine_k"], inner_tol=cfg["inner_tol"])
    for _ in range(max(1, args.warmup - 1)):
        X.zero_()
        M.cg_solve_multi(A, B, X, **kw)
    torch.cuda.synchronize()
    barrier(world)
    ts = []
    for _ in range(args.steps):
        X.zero_()
        res = M.cg_solve_multi(A, B, X, **kw)
        ts.append(res[0].times[4])
    t = max_over_ranks(world, sum(ts) / len(ts))
    out = {"rhs": 32, "system": "128^3", "value": t, "unit": "s",
           "inner_operator": res[0].inner_operator,
           "tuning": {k: cfg[k] for k in ("z_chunk", "refine_k", "inner_tol")},
           "tuned_from_cache": cfg.get("cached", False),
           "iterations_max": max(r.num_iters for r in res),
           "reliable_updates": res[0].refinements,
           "all_converged": all(r.status == 0 for r in res),
           "max_rel_resid": max(r.final_resid / r.normr0 for r in res)}
    if not args.no_seq:
        scfg = autotune.tune_mixed(A, b, tol=TOL, reps=1)
        t_seq = 0.0
        for j in range(32):
            bj = B[:, j].contiguous()
            xj = torch.zeros_like(bj)
            r = M.cg_solve(A, bj, xj, max_iter=5000, tol=TOL, tol_mode="relative",
                           precision="mixed", refine_k=scfg["refine_k"],
                           inner_tol=scfg["inner_tol"])
            t_seq += r.total_time
        out["sequential_mixed_s"] = t_seq
        out["sequential_tuning"] = {"refine_k": scfg["refine_k"], "inner_tol": scfg["inner_tol"]}
        out["speedup_vs_sequential"] = t_seq / t
    return out


def run_probe(args):
    """Small fixed workloads for profiler captures (ncu): 'spmv' = the box
    system at --dims^3, three FP64 and three FP32 matvecs; 'st64' = the
    system and three products with its verified FP64 stencil; 'sell' = the
    system's ELL layout, its sliced copy and the CSR without box dimensions,
    three products with each; 'cgfull' = the
    system, one whole FP64 solve to 1e-8 (--op) and the analytic check; 'cg' = the system
    and a 4-iteration CG solve; 'multi' = the system and a 6-iteration
    mixed-precision solve of 32 right-hand sides (reliable update every 3);
    'batch' = the first --nbox of the seeded uneven boxes solved together in
    mixed precision to 1e-8 (default shape, refine_k 50); 'mixed' = the
    system solved in mixed precision to 1e-8 (--refine-k)."""
    import torch
    import minife_gb300 as M
    torch.cuda.set_device(0)
    if args.probe == "batch":
        dims = batch_dims(args.nbox)
        x, off, res = M.batch_solve_boxes(dims, max_iter=5000, tol=TOL, tol_mode="relative",
                                          precision="mixed", refine_k=50)
        torch.cuda.synchronize()
        print("probe batch %d boxes done: %d iterations, solve %.3f s"
              % (len(dims), max(r.num_iters for r in res), res[0].times[4]))
        return 0
    d = args.dims
    A, b = M.build_system(d, d, d)
    if args.probe == "cgfull":
        # one whole FP64 solve to 1e-8 (--op: the operator) and the analytic
        # check, each timed with CUDA events
        x = torch.zeros_like(b)
        st = torch.cuda.current_stream()
        e = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
        e[0].record(st)
        r = M.cg_solve(A, b, x, max_iter=5000, tol=TOL, tol_mode="relative", f64_operator=args.op)
        e[1].record(st)
        rc, err = M.verify_solution(d, d, d, x)
        e[2].record(st)
        torch.cuda.synchronize()
        print("cgfull %s: %d iterations, operator %s, solve %.4f s, verify_solution %.3f ms "
              "(max err %.4f)" % (args.op, r.num_iters, r.inner_operator,
                                  e[0].elapsed_time(e[1]) * 1e-3, e[1].elapsed_time(e[2]), err))
    elif args.probe == "st64":
        x = torch.randn(A.nrows, dtype=torch.float64, device="cuda")
        y = torch.empty_like(x)
        S = M.Stencil64(A)
        for _ in range(3):
            M.matvec_stencil64(S, x, y)
    elif args.probe == "sell":
        # the reference's ELL layout, its sliced copy and the CSR without its
        # box dimensions (the generic kernel), three products with each
        x = torch.randn(A.nrows, dtype=torch.float64, device="cuda")
        y = torch.empty_like(x)
        E = M.ELLMatrix.from_csr(A)
        S = M.SELLMatrix.from_ell(E)
        G = M.CSRMatrix(A.row_offsets, A.packed_cols, A.packed_coefs)
        for _ in range(3):
            M.matvec_ell(E, x, y)
        for _ in range(3):
            M.matvec_sell(S, x, y)
        for _ in range(3):
            M.matvec(G, x, y)
    elif args.probe == "spmv":
        x = torch.randn(A.nrows, dtype=torch.float64, device="cuda")
        y = torch.empty_like(x)
        for _ in range(3):
            M.matvec(A, x, y)
        A32 = M.to_f32(A)
        x32 = x.float()
        y32 = torch.empty_like(x32)
        for _ in range(3):
            M.matvec(A32, x32, y32)
    elif args.probe == "batch":
        pass
    elif args.probe == "mixed":
        x = torch.zeros_like(b)
        r = M.cg_solve(A, b, x, max_iter=5000, tol=TOL, tol_mode="relative", precision="mixed",
                       refine_k=args.refine_k)
        print("mixed: %d inner iterations, %d reliable updates" % (r.num_iters, r.refinements))
    elif args.probe == "multi":
        g = torch.Generator(device="cpu").manual_seed(0)
        B = torch.randn(A.nrows, 32, generator=g, dtype=torch.float64).cuda().contiguous()
        X = torch.zeros_like(B)
        M.cg_solve_multi(A, B, X, max_iter=6, tol=TOL, tol_mode="relative", precision="mixed",
                         refine_k=3)
    else:
        x = torch.zeros_like(b)
        M.cg_solve(A, b, x, max_iter=4, tol=TOL, tol_mode="relative")
    torch.cuda.synchronize()
    print("probe %s %d^3 done" % (args.probe, d))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--probe", choices=["spmv", "st64", "sell", "cg", "cgfull", "mixed", "multi",
                                        "batch"],
                    default=None,
                    help="run a small fixed workload for a profiler capture and exit")
    ap.add_argument("--dims", type=int, default=128)
    ap.add_argument("--op", choices=["auto", "csr"], default="auto",
                    help="probe cgfull: the FP64 operator")
    ap.add_argument("--nbox", type=int, default=96, help="boxes of the batch probe")
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-mixed", action="store_true")
    ap.add_argument("--no-batch", action="store_true",
                    help="skip the 96-box batched solve")
    ap.add_argument("--no-small", action="store_true", help="skip the 30^3 case")
    ap.add_argument("--no-next", action="store_true",
                    help="skip the ELL and Jacobi-PCG legs (the rows after the hot path)")
    ap.add_argument("--no-adjoint", action="store_true",
                    help="skip the adjoint-gradient leg (128^3 gradient + FD spot check)")
    ap.add_argument("--adjoint-dims", type=int, default=128)
    ap.add_argument("--adjoint-fd", type=int, default=64, help="elements of the FD spot check")
    ap.add_argument("--no-multi", action="store_true",
                    help="skip the 32-right-hand-side solve")
    ap.add_argument("--no-seq", action="store_true",
                    help="skip the sequential baselines of the batched and multi-RHS solves")
    ap.add_argument("--refine-k", type=int, default=0,
                    help="mixed solver: reliable update at least every k inner iterations "
                         "(0: the autotuner's choice)")
    ap.add_argument("--ref-dims", type=int, default=DIMS[0],
                    help="reference arm: box edge of the system (the metric's is 256)")
    ap.add_argument("--ref-warmup-iters", type=int, default=20,
                    help="reference arm: CG iterations of each (untimed) warm-up solve")
    args = ap.parse_args()
    if args.probe:
        return run_probe(args)
    if args.impl == "reference":
        return run_reference(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
