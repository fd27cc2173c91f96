"""Benchmark: Bloch-Torrey signals/s on one GB300 (contract: one JSON line).

Workload (default): the two-compartment permeable box -- [-10,10]^3 um, 40^3
Kuhn-split cubes (384,000 tets), inner compartment = cells with centroid
x^2 + y^2 < 36 (interface nodes duplicated), D = 3e-3 um^2/us in both,
kappa = 1e-5 um/us, PGSE delta = 10600 us, Delta = 43100 us, dt = 200 us
(270 Crank-Nicolson steps), b in {1000, 3000} s/mm^2, gdir (0,1,0), u0 = 1.
All inputs are synthetic and deterministic (seed 0).

A "step" is one pass of the hot path over the whole batch: every signal of the
workload integrated over all 270 time steps by libbtgpu.  ``value`` is the
batched mixed-precision path (FP32 inner Jacobi-COCG, double-float residuals,
outer rtol 1e-9; its signals agree with the FP64 path to <= 1e-6, checked in
the line as ``plain_fp64.max_rel_err_mixed_vs_fp64``), measured with the mesh
already resident and assembled; ``plain_fp64`` times the FP64 path (rtol 1e-12,
the reference-parity path) on the same workload.  ``e2e`` repeats the
measurement through the public C-ABI calls from host buffers (mesh upload and
device graph build, coefficient upload, assembly, schedule, solve, signals back
to the host).

``batched`` is the batched form on the eight-cylinder 64^3 workload: 64 of its
512 signals (Fibonacci directions x b-values, PGSE and cos-OGSE) in one
mixed-precision launch against the FP64 path on two of the same signals.

``uneven`` runs 16 small meshes of uneven size in one persistent launch
(bt_solve_multi) against one launch per mesh.

``--impl reference`` times the CPU restatement of the reference's solve path
(two-field real system, Jacobi-BiCGSTAB rtol 1e-9 as GCloudDmriSolver.py
ships it) with one process per host core, on a bounded sample of time steps.
"""

import argparse
import importlib
import json
import math
import multiprocessing as mp
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
PKG = "dmri-fem-cloud_gb300"

WORKLOADS = {
    "cfg1": "one compartment, [-10,10]^3 um box, 20^3 Kuhn cubes (48,000 tets), D=3e-3, PGSE 10600/43100 us, "
            "b=1000, gdir (1,0,0), dt=200 us",
    "cfg2": "two compartments, [-10,10]^3 um box, 40^3 Kuhn cubes (384,000 tets), cylinder x^2+y^2<36, "
            "D=3e-3, kappa=1e-5, PGSE 10600/43100 us, b in {1000,3000}, gdir (0,1,0), dt=200 us",
    "cfg3": "eight seeded non-overlapping z-cylinders (radii U[2,5]) in a [-15,15]^3 um box, 64^3 Kuhn cubes "
            "(1.57M tets), kappa=5e-5, D=3e-3, 64 Fibonacci directions x 8 b in [500,4000] = 512 signals, "
            "directions 0-31 PGSE 10600/43100 us, 32-63 cos-OGSE (one period over delta), dt=200 us",
}


def alg_bytes_fp64(n, nnz, steps, iters):
    """Minimum unique bytes of the FP64 single-RHS solve of one signal (one
    k_step64 launch).

    per COCG iteration: nnz*(4 + 8 + 8) (column, A_re, J_g) + 4n (row offsets)
      + n*16*(2 + 7 + 1) (SpMV p in / q out, update x,r,p,q in + x,r,p out, diagonal)
    per time step (right-hand side): nnz*(4 + 3*8) + 4n + 2n*16
    """
    per_iter = nnz * 20 + 4 * n + 160 * n
    per_step = nnz * 28 + 4 * n + 32 * n
    return steps * per_step + iters * per_iter


def alg_bytes_mixed(n, nnz, nsig, steps, iters, sweeps):
    """Minimum unique bytes of one k_batched launch of `nsig` signals.

    Each signal is two FP32 complex slots (Re / Im right-hand sides, 8 bytes a
    value).  per inner iteration and signal-dof: 2 slots x (gather z 8 + p,q in
    16 + p,q out 16 + p,q,d,r in 32 + d,r,z out 24) = 192 B, plus the matrix
    nnz*(4 + 16) once per iteration for the whole batch.  Per time step and
    signal-dof: residual at u_n (gather u 16, r out 16) + extrapolated-guess
    correction (gather two history vectors 16, r in/out 32, u in 8, history out
    8, restart of the five slot vectors 80) = 176 B, matrix nnz*(4 + 8 + 32) +
    nnz*(4 + 32).  Per refinement sweep and signal-dof: gather d 16, u and r
    in/out as double-float 64, history in/out 16, restart 80 = 176 B, matrix
    nnz*(4 + 32).
    """
    return (iters * (192 * n * nsig + 20 * nnz) + sweeps * (176 * n * nsig + 36 * nnz)
            + steps * (176 * n * nsig + 80 * nnz))


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[3:7]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------- CPU legs ---
def _cpu_sample_worker(args):
    """One bounded sample: `steps` time steps of one signal of the workload on
    the CPU restatement (literal two-field system, Jacobi-BiCGSTAB rtol 1e-9)."""
    name, steps, sig_index = args
    sys.path.insert(0, ROOT)
    import oracle
    pkg = importlib.import_module(PKG)
    w = pkg.meshgen.workload(name)
    s2 = oracle.two_field_system(w["xyz"], w["tets"], w["region"], np.asarray(w["D"]), 0.0, w["kappa"] or 0.0,
                                 multiple=w["multiple"])
    b, g, _ = w["signals"][sig_index % len(w["signals"])]
    prof = oracle.PGSE(10600, 43100)
    q = oracle.bvalue_to_q(b, prof.int4gb())
    r = oracle.solve_two_field(s2, prof, q, g, w["dt"], solver="bicgstab", rtol=1e-9, atol=1e-10,
                               max_steps=steps)
    return r.elapsed, r.steps


def cpu_baseline(name, steps, workers):
    """signals/s of the CPU restatement: `workers` processes (spawned) each
    integrate `steps` of the 270 steps of one signal; throughput is scaled to
    whole signals."""
    total_steps = 270
    # one thread per worker process: BLAS / OpenMP pools would oversubscribe the
    # cores (the variables are read when a spawned worker loads numpy)
    for var in ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS", "BLIS_NUM_THREADS"):
        os.environ[var] = "1"
    t0 = time.perf_counter()
    ctx = mp.get_context("spawn")
    with ctx.Pool(workers) as pool:
        res = pool.map(_cpu_sample_worker, [(name, steps, i) for i in range(workers)])
    wall = time.perf_counter() - t0
    per_step = max(e / s for e, s in res)      # slowest worker's solve time per step
    sig_per_s = workers / (per_step * total_steps)
    return {"value": sig_per_s, "unit": "signals/s", "cores": workers, "kind": "port",
            "sample": "%d of %d Crank-Nicolson steps of one %s signal per process (time of the solve loop, "
                      "assembly excluded), %d process(es); wall %.1f s" % (steps, total_steps, name, workers, wall)}


# ---------------------------------------------------------------- GPU leg ----
def gpu_run(args):
    import torch
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    pkg = importlib.import_module(PKG)
    replicas = importlib.import_module(PKG + ".replicas")
    pkg._native.load(pkg.build())
    w = pkg.meshgen.workload(args.workload)
    prof = w["profiles"]
    fns, fos = zip(*[pkg.sequences.profile_samples(p, w["dt"]) for p in prof])
    fn, fo = np.array(fns), np.array(fos)
    int4 = [p.int4gb() for p in prof]
    sig = w["signals"]
    q = np.array([pkg.sequences.b_to_q(b, int4[pi]) for b, _, pi in sig])
    g = np.array([gd for _, gd, _ in sig], np.float64)
    g /= np.linalg.norm(g, axis=1, keepdims=True)
    pidx = np.array([pi for _, _, pi in sig], np.int32)
    nr = w["n_regions"]
    rc = None if w["multiple"] else np.zeros(nr, np.int32)
    prec = pkg.PRECISION_MIXED if args.precision == "mixed" else pkg.PRECISION_FP64
    rtol = args.rtol if args.rtol else (1e-12 if prec == pkg.PRECISION_FP64 else 1e-9)

    stream = torch.cuda.current_stream()
    ctx = pkg.Context(local)
    ctx.set_stream(stream.cuda_stream)
    ctx.mesh_upload(w["xyz"], w["tets"], w["region"], nr, rc)
    ctx.set_coefficients(w["D"], w["invT2"], w["kappa"])
    ctx.assemble()
    ctx.set_schedule(fn, fo, w["dt"])
    info = ctx.info()
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")   # 512 MB > L2
    n_sig = len(sig)

    def timed(precision, tol, steps, warmup):
        """W untimed + K timed solves of the whole batch; CUDA events on the
        library's stream (torch's current stream), L2 flushed between steps."""
        for _ in range(warmup):
            ctx.solve(q, g, pidx, None, precision, tol, args.maxit)
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        evs, outs = [], []
        with ClockSampler(local) as clk:
            torch.cuda.synchronize()
            for _ in range(steps):
                flush.zero_()
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                outs.append(ctx.solve(q, g, pidx, None, precision, tol, args.maxit))
                e1.record(stream)
                evs.append((e0, e1))
            torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        tot = replicas.max_over_ranks(sum(a.elapsed_time(b) for a, b in evs), device="cuda")
        return tot, outs, clk.summary()

    peaks_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(peaks_path):
        peak, peak_src = json.load(open(peaks_path))["hbm_gbs"], "measured"
    else:
        peak, peak_src = 6800.0, "fallback"
    l2_note = ("L2-resident: the working set fits the 129 MB L2 within a step, so achieved/HBM-peak counts "
               "L2-served bytes" if info["nnz"] * 44 + info["n_dofs"] * n_sig * 400 < 100e6 else
               "working set larger than L2")

    def roofline(kind, st):
        if kind == "fp64":
            iters = st["total_iterations"] / n_sig
            byts = alg_bytes_fp64(info["n_dofs"], info["nnz"], st["steps"], iters)
            launch_ms = st["stepper_ms"] / n_sig
            kern = "k_step64 (persistent FP64 CN/COCG stepper, one launch per signal)"
        else:
            launches = max(1, -(-n_sig // 256))
            per = n_sig / launches
            iters = st["total_iterations"] / n_sig                 # inner iterations per launch
            sweeps = st["refinements"] / launches
            byts = alg_bytes_mixed(info["n_dofs"], info["nnz"], per, st["steps"], iters, sweeps)
            launch_ms = st["stepper_ms"] / launches
            kern = "k_batched (persistent mixed-precision batched stepper, %d signal(s) per launch)" % per
        ach = byts / (launch_ms / 1e3) / 1e9
        tr = None
        tpath = os.path.join(ROOT, "profiles", "traffic.json")
        if os.path.exists(tpath):
            t = json.load(open(tpath)).get("%s:%s" % (args.workload, kind))
            tr = t["bytes_per_launch"] if t else None
        return {"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak,
                "traffic": tr, "kernel": kern, "bytes_per_launch": byts, "launch_ms": launch_ms,
                "peak_source": peak_src + " hbm_gbs (copy)", "note": l2_note}

    prec_main = pkg.PRECISION_MIXED if args.precision == "mixed" else pkg.PRECISION_FP64
    tol_main = args.rtol if args.rtol else (1e-9 if prec_main == pkg.PRECISION_MIXED else 1e-12)
    total_ms, outs, clocks = timed(prec_main, tol_main, args.steps, args.warmup)
    value = world * n_sig * args.steps / (total_ms / 1e3)
    st = outs[-1]["stats"]
    norm = outs[-1]["signal"] / outs[-1]["S0"]
    kind = "mixed" if prec_main == pkg.PRECISION_MIXED else "fp64"
    roof = roofline(kind, st)
    launches = st["kernel_launches"]

    plain = None
    if prec_main == pkg.PRECISION_MIXED and args.fp64_steps > 0:
        t64, o64, c64 = timed(pkg.PRECISION_FP64, 1e-12, args.fp64_steps, max(1, min(args.warmup, 2)))
        s64 = o64[-1]["stats"]
        n64 = o64[-1]["signal"] / o64[-1]["S0"]
        plain = {"value": world * n_sig * args.fp64_steps / (t64 / 1e3), "unit": "signals/s",
                 "ms_per_step": t64 / args.fp64_steps, "steps": args.fp64_steps, "rtol": 1e-12,
                 "normalized_signals": [float(v) for v in n64],
                 "iterations_per_signal": s64["total_iterations"] / n_sig,
                 "roofline": roofline("fp64", s64), "clocks": c64}
        plain["mixed_over_plain"] = value / plain["value"]
        plain["max_rel_err_mixed_vs_fp64"] = float(np.max(np.abs(norm - n64) / np.abs(n64)))

    batched = batched_leg(args, pkg, stream, flush, peak, peak_src) if args.batched_signals > 0 else None
    uneven = uneven_leg(args, pkg, stream, flush) if args.uneven_meshes > 0 else None
    adjoint = adjoint_leg(args, pkg, stream, flush) if args.adjoint_signals > 0 else None

    # end to end through the public C-ABI from host buffers
    e2e_ms = []
    h2d = (w["xyz"].nbytes + w["tets"].astype(np.int32).nbytes + w["region"].astype(np.int32).nbytes
           + 8 * nr * (2 + nr) + fn.nbytes + fo.nbytes + q.nbytes + g.nbytes + pidx.nbytes)
    d2h = 8 * (n_sig + 1)
    for _ in range(args.e2e_steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        c2 = pkg.Context(local)
        c2.set_stream(stream.cuda_stream)
        c2.mesh_upload(w["xyz"], w["tets"], w["region"], nr, rc)
        c2.set_coefficients(w["D"], w["invT2"], w["kappa"])
        c2.assemble()
        c2.set_schedule(fn, fo, w["dt"])
        o2 = c2.solve(q, g, pidx, None, prec_main, tol_main, args.maxit)
        _ = float(o2["signal"][0])                          # result on the host
        e2e_ms.append((time.perf_counter() - t0) * 1e3)
        c2.close()
    e2e_value = n_sig / (statistics.median(e2e_ms) / 1e3) * world if e2e_ms else None

    res = None
    if rank == 0:
        cpu = cpu_baseline(args.workload, args.cpu_sample_steps, 1) if args.cpu_sample_steps > 0 else None
        res = {
            "metric": "Bloch-Torrey signals/s on 1 GB300 at <=1e-6 rel err (%s)" % args.workload,
            "value": value, "unit": "signals/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": total_ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None,
            "dtype": "f64" if kind == "fp64" else "f32 (inner COCG) + double-float residuals",
            "data": "synthetic (seeded Kuhn box mesh and centroid markers; no dataset)",
            "config": {"workload": args.workload + ": " + WORKLOADS.get(args.workload, ""),
                       "signals_per_step": n_sig, "precision": kind, "rtol": tol_main,
                       "n_dofs": info["n_dofs"], "nnz": info["nnz"], "time_steps": st["steps"],
                       "l2": "flushed between timed steps (512 MB write)",
                       "parallelism": "replicas" if world > 1 else "single GPU"},
            "normalized_signals": [float(v) for v in norm],
            "iterations_per_signal": st["total_iterations"] / n_sig,
            "roofline": roof,
            "plain_fp64": plain,
            "batched": batched,
            "uneven": uneven,
            "adjoint": adjoint,
            "cpu_baseline": cpu,
            "e2e": {"value": e2e_value, "unit": "signals/s", "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h),
                    "what": "bt_create+bt_mesh_upload (device graph build)+bt_set_coefficients+bt_assemble+"
                            "bt_set_schedule+bt_solve, host arrays in, signals out; median of %d" % len(e2e_ms)},
            "gpu_launches": int(launches) * args.steps,
            "clocks": clocks,
        }
        print(json.dumps(res))
    ctx.close()
    if world > 1:
        torch.distributed.destroy_process_group()
    return res


def batched_leg(args, pkg, stream, flush, peak, peak_src):
    """The batched form on the eight-cylinder 64^3 workload: the first
    `batched_signals` of its 512 signals (directions x b-values, PGSE and
    cos-OGSE) in one mixed-precision launch, against the FP64 path on two of the
    same signals (one FP64 launch per signal).  L2 flushed before each timed
    launch."""
    import torch
    w = pkg.meshgen.workload("cfg3")
    prof = w["profiles"]
    fns, fos = zip(*[pkg.sequences.profile_samples(p, w["dt"]) for p in prof])
    int4 = [p.int4gb() for p in prof]
    sig = w["signals"]
    idx = np.linspace(0, len(sig) - 1, args.batched_signals).astype(int)
    sel = [sig[i] for i in idx]
    q = np.array([pkg.sequences.b_to_q(b, int4[pi]) for b, _, pi in sel])
    g = np.array([gd for _, gd, _ in sel], np.float64)
    g /= np.linalg.norm(g, axis=1, keepdims=True)
    pidx = np.array([pi for _, _, pi in sel], np.int32)
    ctx = pkg.Context(int(os.environ.get("LOCAL_RANK", "0")))
    ctx.set_stream(stream.cuda_stream)
    ctx.mesh_upload(w["xyz"], w["tets"], w["region"], w["n_regions"], None)
    ctx.set_coefficients(w["D"], w["invT2"], w["kappa"])
    ctx.assemble()
    ctx.set_schedule(np.array(fns), np.array(fos), w["dt"])
    info = ctx.info()

    def timed(fn):
        flush.zero_()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        out = fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1), out

    ctx.solve(q, g, pidx, None, pkg.PRECISION_MIXED, 1e-9, args.maxit)          # warm-up (autotuner)
    ms_mix, out = timed(lambda: ctx.solve(q, g, pidx, None, pkg.PRECISION_MIXED, 1e-9, args.maxit))
    two = [0, len(q) - 1]
    ms_64, o64 = timed(lambda: ctx.solve(q[two], g[two], pidx[two], None, pkg.PRECISION_FP64, 1e-12, args.maxit))
    st = out["stats"]
    n_sig = len(q)
    iters = st["total_iterations"] / n_sig
    byts = alg_bytes_mixed(info["n_dofs"], info["nnz"], n_sig, st["steps"], iters, st["refinements"])
    ach = byts / (st["stepper_ms"] / 1e3) / 1e9
    err = float(np.max(np.abs(out["signal"][two] - o64["signal"]) / np.abs(o64["signal"])))
    v_mix = n_sig / (ms_mix / 1e3)
    v_64 = len(two) / (ms_64 / 1e3)
    ctx.close()
    return {"workload": "cfg3: " + WORKLOADS["cfg3"], "signals": n_sig, "n_dofs": info["n_dofs"], "nnz": info["nnz"],
            "value": v_mix, "unit": "signals/s", "ms": ms_mix,
            "plain_fp64_value": v_64, "plain_fp64_signals_timed": len(two),
            "mixed_over_plain": v_mix / v_64, "max_rel_err_mixed_vs_fp64": err,
            "iterations_per_signal": iters, "refinements": st["refinements"],
            "roofline": {"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak,
                         "bytes_per_launch": byts, "launch_ms": st["stepper_ms"],
                         "peak_source": peak_src + " hbm_gbs (copy)",
                         "note": "algorithmic bytes (bench.alg_bytes_mixed); working set larger than L2"}}


def adjoint_leg(args, pkg, stream, flush):
    """Gradients: the layered-sphere 48^3 workload (4 layers, per-layer D and T2,
    per-interface kappa), the first `adjoint_signals` of its 120 signals spread
    evenly; the batched mixed-precision adjoint (bt_adjoint_batch, one set of
    launches) against the FP64 adjoint of one signal (bt_adjoint), and the
    gradient error of that signal."""
    import torch
    w = pkg.meshgen.workload("cfg4")
    prof = w["profiles"]
    fns, fos = zip(*[pkg.sequences.profile_samples(p, w["dt"]) for p in prof])
    sig = w["signals"]
    idx = np.linspace(0, len(sig) - 1, args.adjoint_signals).astype(int)
    sel = [sig[i] for i in idx]
    q = np.array([pkg.sequences.b_to_q(b, prof[pi].int4gb()) for b, _, pi in sel])
    g = np.array([gd for _, gd, _ in sel], np.float64)
    g /= np.linalg.norm(g, axis=1, keepdims=True)
    ctx = pkg.Context(int(os.environ.get("LOCAL_RANK", "0")))
    ctx.set_stream(stream.cuda_stream)
    ctx.mesh_upload(w["xyz"], w["tets"], w["region"], w["n_regions"], None)
    ctx.set_coefficients(w["D"], w["invT2"], w["kappa"])
    ctx.assemble()
    ctx.set_schedule(np.array(fns), np.array(fos), w["dt"])

    def timed(fn_):
        flush.zero_()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        out = fn_()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1), out

    ctx.solve(q, g, None, None, pkg.PRECISION_MIXED, 1e-9, args.maxit)          # warm-up (autotuner)
    ms_b, out = timed(lambda: ctx.adjoint_batch(q, g, rtol=1e-9, max_iterations=args.maxit))
    ms_64, ref = timed(lambda: ctx.adjoint(q[0], g[0], rtol=1e-12, max_iterations=args.maxit))
    err = {k: float(np.max(np.abs(out[k][0] - ref[k])) / np.max(np.abs(ref[k])))
           for k in ("dD", "dinvT2", "dkappa")}
    info = ctx.info()
    ctx.close()
    n = len(q)
    return {"workload": "layered sphere 48^3 (4 regions, D/T2 per layer, kappa per interface), PGSE, "
                        "%d signals in one batched adjoint" % n,
            "n_dofs": info["n_dofs"], "signals": n,
            "batched_mixed": {"gradients_per_s": n / (ms_b / 1e3), "ms": ms_b,
                              "parameters_per_signal": "D x4, 1/T2 x4, kappa x3"},
            "fp64_one_signal": {"gradients_per_s": 1.0 / (ms_64 / 1e3), "ms": ms_64},
            "ratio": (n / ms_b) / (1.0 / ms_64),
            "max_rel_err_vs_fp64_adjoint": err,
            "signal_rel_err": float(abs(out["signal"][0] - ref["signal"]) / abs(ref["signal"]))}


def uneven_leg(args, pkg, stream, flush):
    """Several meshes of uneven size in one persistent launch (bt_solve_multi):
    `uneven_meshes` seeded boxes of 8^3 ... 24^3 Kuhn cubes of 1.5 um with
    random z-cylinders (D 3e-3 / 2e-3, kappa U[1e-5,1e-4]), 4 b-values along one
    direction each, PGSE; against one launch per mesh, and the largest mesh
    against the FP64 path."""
    import torch
    meshes = pkg.meshgen.uneven_meshes(count=args.uneven_meshes, seed=0, nmin=8, nmax=24, cube=1.5)
    p = pkg.sequences.pgse(10600, 43100)
    fn, fo = pkg.sequences.profile_samples(p, 200.0)
    qs = [pkg.sequences.b_to_q(b, p.int4gb()) for b in (1000.0, 2000.0, 3000.0, 4000.0)]
    gs = [[0.36, 0.48, 0.8]] * 4
    ctxs = []
    for m in meshes:
        c = pkg.Context(int(os.environ.get("LOCAL_RANK", "0")))
        c.set_stream(stream.cuda_stream)
        c.mesh_upload(m["xyz"], m["tets"], m["region"], 2)
        c.set_coefficients(m["D"], None, m["kappa"])
        c.assemble()
        c.set_schedule(fn, fo, 200.0)
        ctxs.append(c)
    n = len(ctxs)

    def timed(fn_):
        flush.zero_()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        out = fn_()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1), out

    pkg.solve_multi(ctxs, [qs] * n, [gs] * n, rtol=1e-9)                          # warm-up (tuning)
    ms_one, out = timed(lambda: pkg.solve_multi(ctxs, [qs] * n, [gs] * n, rtol=1e-9))
    for c in ctxs:
        c.solve(qs, gs, precision=pkg.PRECISION_MIXED, rtol=1e-9)                # warm-up (tuning)
    ms_sep, _ = timed(lambda: [c.solve(qs, gs, precision=pkg.PRECISION_MIXED, rtol=1e-9) for c in ctxs])
    r64 = ctxs[-1].solve(qs, gs, precision=pkg.PRECISION_FP64, rtol=1e-12, max_iterations=20000)["signal"]
    err = float(np.max(np.abs(out["signal"][-1] - r64) / np.abs(r64)))
    dofs = [c.info()["n_dofs"] for c in ctxs]
    for c in ctxs:
        c.close()
    nsig = 4 * n
    return {"workload": "%d seeded cylinder boxes, 8^3..24^3 Kuhn cubes of 1.5 um (%d..%d dofs), 4 b-values each, "
                        "PGSE 10600/43100 us" % (n, min(dofs), max(dofs)),
            "signals": nsig, "value": nsig / (ms_one / 1e3), "unit": "signals/s", "ms": ms_one,
            "separate_launches_value": nsig / (ms_sep / 1e3), "one_launch_over_separate": ms_sep / ms_one,
            "max_rel_err_vs_fp64_largest_mesh": err}


def batched_profile(args):
    """One short launch for a profiler: the batched leg's 64 signals on the
    eight-cylinder 64^3 workload, schedule cut to `batched_profile` steps inside
    the first gradient pulse, geometry fixed (lanes-per-row 32, two blocks per
    SM, interleaved rows) so that no autotuner trial runs first."""
    pkg = importlib.import_module(PKG)
    pkg._native.load(pkg.build())
    w = pkg.meshgen.workload("cfg3")
    n = args.batched_profile
    fns, fos = zip(*[pkg.sequences.profile_samples(p, w["dt"]) for p in w["profiles"]])
    fn, fo = np.array(fns)[:, 20:20 + n], np.array(fos)[:, 20:20 + n]
    int4 = [p.int4gb() for p in w["profiles"]]
    sig = w["signals"]
    sel = [sig[i] for i in np.linspace(0, len(sig) - 1, args.batched_signals).astype(int)]
    q = np.array([pkg.sequences.b_to_q(b, int4[pi]) for b, _, pi in sel])
    g = np.array([gd for _, gd, _ in sel], np.float64)
    g /= np.linalg.norm(g, axis=1, keepdims=True)
    pidx = np.array([pi for _, _, pi in sel], np.int32)
    ctx = pkg.Context(0)
    ctx.mesh_upload(w["xyz"], w["tets"], w["region"], w["n_regions"], None)
    ctx.set_coefficients(w["D"], w["invT2"], w["kappa"])
    ctx.assemble()
    ctx.set_schedule(fn, fo, w["dt"])
    for key, val in (("mixed.lanes_per_row", 32), ("mixed.blocks_per_sm", 2), ("mixed.blocked_rows", 0)):
        ctx.set_option(key, val)
    st = ctx.solve(q, g, pidx, None, pkg.PRECISION_MIXED, 1e-9, args.maxit)["stats"]
    print(json.dumps({"batched_profile_steps": st["steps"], "stepper_ms": st["stepper_ms"],
                      "inner_iterations": st["total_iterations"] / len(q), "refinements": st["refinements"]}))
    ctx.close()


def reference_run(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    workers = os.cpu_count() or 1
    vals = []
    for _ in range(args.warmup_ref):
        pass
    for _ in range(args.ref_steps):
        vals.append(cpu_baseline(args.workload, args.cpu_sample_steps_ref, workers))
    v = statistics.median(x["value"] for x in vals)
    out = {"metric": "Bloch-Torrey signals/s on 1 GB300 at <=1e-6 rel err (%s)" % args.workload,
           "value": v, "unit": "signals/s", "n_gpus": int(os.environ.get("WORLD_SIZE", "1")),
           "steps": args.ref_steps, "warmup": 0, "higher_is_better": True, "scaling": "weak",
           "impl": "reference", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "config": {"workload": args.workload + ": " + WORKLOADS.get(args.workload, "")},
           "cpu_baseline": {"value": v, "unit": "signals/s", "cores": workers, "kind": "port",
                            "sample": vals[-1]["sample"]},
           "e2e": {"value": v, "unit": "signals/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="cfg2", choices=sorted(WORKLOADS))
    ap.add_argument("--precision", default="mixed", choices=["fp64", "mixed"])
    ap.add_argument("--fp64-steps", type=int, default=3, help="timed steps of the plain FP64 path (0: skip)")
    ap.add_argument("--rtol", type=float, default=None)
    ap.add_argument("--maxit", type=int, default=5000)
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--cpu-sample-steps", type=int, default=8)
    ap.add_argument("--cpu-sample-steps-ref", type=int, default=6)
    ap.add_argument("--batched-profile", type=int, default=0,
                    help="only one short batched launch of this many steps, for a profiler")
    ap.add_argument("--adjoint-signals", type=int, default=16,
                    help="signals of the batched-adjoint leg on the 48^3 layered sphere (0: skip)")
    ap.add_argument("--uneven-meshes", type=int, default=16,
                    help="meshes of the uneven multi-mesh leg (0: skip)")
    ap.add_argument("--batched-signals", type=int, default=64,
                    help="signals of the eight-cylinder 64^3 batched leg (0: skip)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 0)
    args.warmup_e2e = 0
    args.warmup_ref = 0
    args.ref_steps = max(1, min(args.steps, 3))
    if args.batched_profile > 0:
        batched_profile(args)
    elif args.impl == "reference":
        reference_run(args)
    else:
        gpu_run(args)


if __name__ == "__main__":
    main()
