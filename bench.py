"""Benchmark: Bloch-Torrey signals/s on one GB300 (contract: one JSON line).

Headline (``value``): the plain FP64 path on the two-compartment permeable box,
the configuration stated as plain FP64 -- [-10,10]^3 um, 40^3 Kuhn-split cubes
(384,000 tets), inner compartment = cells with centroid x^2 + y^2 < 36
(interface nodes duplicated), D = 3e-3 um^2/us in both, kappa = 1e-5 um/us,
PGSE delta = 10600 us, Delta = 43100 us, dt = 200 us (270 Crank-Nicolson
steps), b in {1000, 3000} s/mm^2, gdir (0,1,0), u0 = 1.  A "step" is one pass
of the hot path over the batch: both signals integrated over all 270 time
steps by libbtgpu's FP64 stepper (COCG to ||r|| <= 1e-12 ||b|| per step), mesh
resident and assembled.  Each signal's error against the oracle's committed
SuperLU solution of the same workload (tests/golden/oracle_signals.json) is
printed in the line.  ``e2e`` repeats the measurement through the public C-ABI
calls from host buffers (mesh upload and device graph build, coefficient
upload, assembly, schedule, solve, signals back to the host).

Legs (each its own timed region, named workload, precision and error):

* ``mixed_cfg2``: the batched mixed-precision path (FP32 inner Jacobi-COCG on
  Re/Im right-hand sides, double-float residuals and refinement, FP64 signal)
  on the same 40^3 workload, its error per signal against the oracle and its
  ratio to the FP64 path;
* ``batched``: the eight-cylinder 64^3 workload with all 512 signals (64
  Fibonacci directions x 8 b-values, PGSE and cos-OGSE) in two 256-signal
  launches, against the FP64 path timed on signals spread over the 512; the
  mixed-vs-FP64 error of every signal (the FP64 values of all 512 are the
  committed fixture tests/golden/gpu_fp64_cfg3_signals.json, written by the FP64
  path on a GB300, which is pinned to the oracle at 1e-9; the spread sample is
  re-checked live);
* ``uneven``: 16 small meshes of uneven size in one persistent launch
  (bt_solve_multi) against one launch per mesh;
* ``adjoint``: batched mixed-precision gradients on the 48^3 layered sphere
  against the FP64 adjoint;
* ``cfg5`` (``--cfg5 128``, off by default: several minutes): the uneven batch
  of 16 meshes of 24^3 ... 96^3 cubes, 2,048 signals, forward (bt_solve_multi)
  and gradients (bt_adjoint_multi).

``--impl reference`` times the CPU restatement of the reference's solve path
(two-field real system, Jacobi-BiCGSTAB rtol 1e-9 as GCloudDmriSolver.py ships
it): one whole 270-step signal per process, set-up included, one process per
host core.
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
METRIC = "Bloch-Torrey signals/s on 1 GB300 at ≤1e-6 rel err, batched vs plain FP64; HBM %"
L2_BYTES = 129e6          # GB300 L2

WORKLOADS = {
    "cfg1": "plain FP64, one compartment, [-10,10]^3 um box, 20^3 Kuhn cubes (48,000 tets), D=3e-3, "
            "PGSE 10600/43100 us, b=1000, gdir (1,0,0), dt=200 us",
    "cfg2": "plain FP64 two-compartment permeable: [-10,10]^3 um box, 40^3 Kuhn cubes (384,000 tets), "
            "cylinder x^2+y^2<36 (staircase, interface nodes duplicated), D=3e-3 both, kappa=1e-5, Neumann, "
            "PGSE 10600/43100 us, b in {1000,3000}, gdir (0,1,0), dt=200 us, u0=1",
    "cfg3": "batched + mixed precision: eight seeded non-overlapping z-cylinders (radii U[2,5]) in a "
            "[-15,15]^3 um box, 64^3 Kuhn cubes (1.57M tets), kappa=5e-5, D=3e-3, 64 Fibonacci directions x 8 b "
            "in [500,4000] = 512 signals, directions 0-31 PGSE 10600/43100 us, 32-63 cos-OGSE (one period over "
            "delta), dt=200 us",
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


def alg_bytes_fp64_pair(n, nnz, its):
    """Minimum unique bytes of one k_step64_pair launch (two signals of one
    direction; its[j][k] = COCG iterations of signal j at step k).

    The matrix (column, A_re, J_g: nnz*20 + 4n) is read once per pair iteration,
    max(its[0][k], its[1][k]) of them at step k; the vector traffic (160n) is per
    signal and iteration.  Per step: the right-hand-side matrix once
    (nnz*28 + 4n) and 32n of vectors per signal.
    """
    its = np.asarray(its, np.int64)
    per_step = (nnz * 28 + 4 * n) * its.shape[1] + 2 * 32 * n * its.shape[1]
    return per_step + (nnz * 20 + 4 * n) * int(its.max(axis=0).sum()) + 160 * n * int(its.sum())


def alg_bytes_mixed(n, nnz, nsig, steps, iters, sweeps):
    """Minimum unique bytes of one k_batched launch of `nsig` signals.

    Each signal is two FP32 complex slots (Re / Im right-hand sides, 8 bytes a
    value).  per inner iteration and signal-dof: 2 slots x (gather z 8 + p,q in
    16 + p,q out 16 + p,q,d,r in 32 + d,r,z out 24) = 192 B, plus the matrix
    nnz*(4 + 16) once per iteration for the whole batch.  Per time step and
    signal-dof: residual at u_n (gather u 16, r out 16) + extrapolated-guess
    correction (gather the offset 8, r in/out 32, u in 8, correction out 8,
    backward-difference table in 24 / out 24, restart of the five slot vectors
    80) = 216 B, matrix nnz*(4 + 8 + 32) + nnz*(4 + 32).  Per refinement sweep
    and signal-dof: gather d 16, u and r in/out as double-float 64, correction
    in/out 16, table in 24, next offset out 8, restart 80 = 208 B, matrix
    nnz*(4 + 32).
    """
    return (iters * (192 * n * nsig + 20 * nnz) + sweeps * (208 * n * nsig + 36 * nnz)
            + steps * (216 * n * nsig + 80 * nnz))


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


def load_json(*parts):
    path = os.path.join(ROOT, *parts)
    if not os.path.exists(path):
        return None
    with open(path) as fh:
        return json.load(fh)


def peak_hbm():
    pk = load_json("MEASURED_PEAKS.json")
    if pk and "hbm_gbs" in pk:
        return float(pk["hbm_gbs"]), "measured hbm_gbs (copy), MEASURED_PEAKS.json"
    return 6800.0, "fallback 6.8 TB/s"


def golden_cfg2():
    """Oracle normalised signals of the full 40^3 workload, keyed by b."""
    g = load_json("tests", "golden", "oracle_signals.json")
    for case in (g or {}).get("cases", []):
        if case["workload"] == "cfg2" and case["n"] is None:
            return {float(s["b"]): s["normalized"] for s in case["signals"]}
    return {}


# ---------------------------------------------------------------- CPU legs ---
def _cpu_signal_worker(args):
    """One whole signal on the CPU restatement of the reference's solve path:
    the literal two-field system (set-up: mesh + assembly of the forms, as one
    GCloudDmriSolver.py job does) and all 270 Crank-Nicolson steps with
    Jacobi-BiCGSTAB rtol 1e-9 / atol 1e-10 (GCloudDmriSolver.py:219-222)."""
    name, sig_index = args
    sys.path.insert(0, ROOT)
    import oracle
    pkg = importlib.import_module(PKG)
    t0 = time.perf_counter()
    w = pkg.meshgen.workload(name)
    s2 = oracle.two_field_system(w["xyz"], w["tets"], w["region"], np.asarray(w["D"]), 0.0, w["kappa"] or 0.0,
                                 multiple=w["multiple"])
    b, g, _ = w["signals"][sig_index % len(w["signals"])]
    prof = oracle.PGSE(10600, 43100)
    q = oracle.bvalue_to_q(b, prof.int4gb())
    t1 = time.perf_counter()
    r = oracle.solve_two_field(s2, prof, q, g, w["dt"], solver="bicgstab", rtol=1e-9, atol=1e-10)
    t2 = time.perf_counter()
    it = np.asarray(r.iterations)
    return {"setup_s": t1 - t0, "solve_s": t2 - t1, "steps": r.steps, "normalized": r.normalized, "b": b,
            "iterations": [float(it[:53].mean()), float(it[53:216].mean()), float(it[216:].mean())]}


def cpu_baseline(name, workers):
    """signals/s of the CPU restatement: `workers` spawned processes, each
    integrating one whole signal (set-up included); throughput = workers /
    the slowest worker's time."""
    for var in ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS", "BLIS_NUM_THREADS"):
        os.environ[var] = "1"    # one BLAS thread per process: a pool of them would oversubscribe the cores
    t0 = time.perf_counter()
    with mp.get_context("spawn").Pool(workers) as pool:
        res = pool.map(_cpu_signal_worker, [(name, i) for i in range(workers)])
    wall = time.perf_counter() - t0
    per = max(r["setup_s"] + r["solve_s"] for r in res)
    solve = max(r["solve_s"] for r in res)
    it = np.mean([r["iterations"] for r in res], axis=0)
    return {"value": workers / per, "unit": "signals/s", "cores": workers, "kind": "port",
            "solve_only_value": workers / solve,
            "sample": "%d whole signal(s) of the %s workload (all %d Crank-Nicolson steps, set-up included: mesh + "
                      "assembly of the two-field forms), one per process, %d process(es) on %d core(s); slowest "
                      "process %.1f s (solve %.1f s); BiCGSTAB iterations per step in the f=1 / f=0 / f=-1 regimes "
                      "%.1f / %.1f / %.1f; wall %.1f s"
                      % (workers, name, res[0]["steps"], workers, workers, per, solve, it[0], it[1], it[2], wall),
            "normalized_signals": [r["normalized"] for r in res[:2]]}


# ---------------------------------------------------------------- GPU legs ---
def _event_timer(stream, flush):
    import torch

    def timed(fn):
        flush.zero_()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        out = fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1), out
    return timed


def _signal_arrays(pkg, w, sel):
    prof = w["profiles"]
    int4 = [p.int4gb() for p in prof]
    q = np.array([pkg.sequences.b_to_q(b, int4[pi]) for b, _, pi in sel])
    g = np.array([gd for _, gd, _ in sel], np.float64)
    g /= np.linalg.norm(g, axis=1, keepdims=True)
    pidx = np.array([pi for _, _, pi in sel], np.int32)
    return q, g, pidx


def _context(pkg, w, local, stream):
    ctx = pkg.Context(local)
    ctx.set_stream(stream.cuda_stream)
    rc = None if w["multiple"] else np.zeros(w["n_regions"], np.int32)
    ctx.mesh_upload(w["xyz"], w["tets"], w["region"], w["n_regions"], rc)
    ctx.set_coefficients(w["D"], w["invT2"], w["kappa"])
    ctx.assemble()
    fns, fos = zip(*[pkg.sequences.profile_samples(p, w["dt"]) for p in w["profiles"]])
    ctx.set_schedule(np.array(fns), np.array(fos), w["dt"])
    return ctx, np.array(fns), np.array(fos)


NOMINAL_HBM_GBS = 7900.0   # GB300 HBM3e nominal, for reference beside the measured copy bandwidth


def roofline_fp64(info, st, its, peak, peak_src, traffic):
    """Roofline of the headline's stepper launches.  its[j][k]: iterations of
    signal j at step k.  Two signals of one direction share a k_step64_pair
    launch (5 kernel launches per pair, 3 per single signal)."""
    n_sig = len(its)
    paired = n_sig == 2 and st["kernel_launches"] == 5
    if paired:
        byts = alg_bytes_fp64_pair(info["n_dofs"], info["nnz"], its)
        launch_ms = st["stepper_ms"]
        kernel = "k_step64_pair (persistent FP64 CN/COCG stepper, the two signals of one direction in one launch)"
    else:
        byts = alg_bytes_fp64(info["n_dofs"], info["nnz"], st["steps"], st["total_iterations"] / n_sig)
        launch_ms = st["stepper_ms"] / n_sig
        kernel = "k_step64 (persistent FP64 CN/COCG stepper, one launch per signal)"
    ach = byts / (launch_ms / 1e3) / 1e9
    out = {"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak,
           "traffic": traffic.get("bytes_per_launch") if traffic else None,
           "kernel": kernel, "bytes_per_launch": byts, "launch_ms": launch_ms, "peak_source": peak_src,
           "frac_of_nominal_7900": ach / NOMINAL_HBM_GBS}
    if traffic:
        out["note"] = ("L2-resident: ncu counts %.0f MB of DRAM traffic per launch of %s, %.3f%% of the %.0f GB "
                       "of algorithmic bytes, so `achieved` counts L2-served bytes and `frac` is not an HBM "
                       "fraction; the stepper is bound by the FP64 pipe (GB300 runs FP64 at a small fraction of "
                       "FP32; %s)"
                       % (traffic["bytes_per_launch"] / 1e6, traffic.get("kernel", "the stepper"),
                          100.0 * traffic["bytes_per_launch"] / byts, byts / 1e9,
                          "profiles/k_step64_pair_cfg2.md: FP64 pipe active 61.6% of peak" if paired
                          else "profiles/k_step64_cfg2.md: FP64 pipe active 59% of peak"))
    else:
        out["note"] = "no DRAM capture for this workload"
    return out


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
    w = pkg.meshgen.workload("cfg2")
    # the whole job's signal list: b in {1000, 3000} x one direction per rank
    # ((0,1,0) on one GPU, as the configuration states); each rank integrates
    # its contiguous shard (replicas only: no data-path collective)
    dirs = [(0.0, 1.0, 0.0)] if world == 1 else [tuple(d) for d in pkg.meshgen.fibonacci_directions(world)]
    job = [(b, d, 0) for d in dirs for b in (1000.0, 3000.0)]
    mine = replicas.shard(len(job), rank, world)
    sel = [job[i] for i in mine]
    q, g, pidx = _signal_arrays(pkg, w, sel)
    n_sig = len(sel)
    stream = torch.cuda.current_stream()
    ctx, fn, fo = _context(pkg, w, local, stream)
    info = ctx.info()
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")   # 512 MB > L2
    peak, peak_src = peak_hbm()
    traffic = load_json("profiles", "traffic.json") or {}

    def timed_steps(precision, tol, steps, warmup):
        """W untimed + K timed solves of the shard; CUDA events on the
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

    # ---- headline: plain FP64 path
    total_ms, outs, clocks = timed_steps(pkg.PRECISION_FP64, 1e-12, args.steps, args.warmup)
    value = len(job) * args.steps / (total_ms / 1e3)
    st = outs[-1]["stats"]
    norm = outs[-1]["signal"] / outs[-1]["S0"]
    its = ctx.iterations(n_sig, st["steps"])
    gathered = replicas.gather_signals(mine, norm, len(job), device="cuda")
    roof = roofline_fp64(info, st, its, peak, peak_src, traffic.get("cfg2:fp64"))
    gold = golden_cfg2()
    err_oracle = [abs(float(v) - gold[b]) / abs(gold[b]) for (b, _, _), v in zip(sel, norm)
                  if tuple(dirs[0]) == (0.0, 1.0, 0.0) and b in gold] if rank == 0 else []

    legs = {}
    if world == 1 and args.mixed_steps > 0:
        legs["mixed_cfg2"] = mixed_cfg2_leg(args, pkg, ctx, q, g, pidx, norm, total_ms / args.steps, gold, sel,
                                            traffic.get("cfg2:mixed"), info, peak, peak_src, timed_steps)
    # end to end through the public C-ABI from host buffers
    e2e_ms = []
    rc = None if w["multiple"] else np.zeros(w["n_regions"], np.int32)
    nr = w["n_regions"]
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
        o2 = c2.solve(q, g, pidx, None, pkg.PRECISION_FP64, 1e-12, args.maxit)
        _ = float(o2["signal"][0])                          # result on the host
        e2e_ms.append((time.perf_counter() - t0) * 1e3)
        c2.close()
    e2e_ms_max = replicas.max_over_ranks(statistics.median(e2e_ms), device="cuda") if e2e_ms else None
    e2e_value = len(job) / (e2e_ms_max / 1e3) if e2e_ms else None
    ctx.close()

    if world == 1:
        stream_legs = (("batched", batched_leg, args.batched_signals), ("uneven", uneven_leg, args.uneven_meshes),
                       ("adjoint", adjoint_leg, args.adjoint_signals), ("strong", strong_leg, args.strong_signals),
                       ("cfg5", cfg5_leg, args.cfg5))
        for key, fnc, n in stream_legs:
            if n > 0:
                legs[key] = fnc(args, pkg, stream, flush, peak, peak_src, traffic)

    res = None
    if rank == 0:
        cpu = cpu_baseline("cfg2", 1) if args.cpu_signals > 0 else None
        res = {
            "metric": METRIC,
            "value": value, "unit": "signals/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": total_ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None,
            "dtype": "f64",
            "data": "synthetic (seeded Kuhn box mesh and centroid markers; no dataset)",
            "config": {"workload": "cfg2: " + WORKLOADS["cfg2"],
                       "signals_per_step": len(job), "signals_per_gpu": n_sig, "precision": "fp64", "rtol": 1e-12,
                       "n_dofs": info["n_dofs"], "nnz": info["nnz"], "time_steps": st["steps"],
                       "l2": "flushed between timed steps (512 MB write); the workload itself is L2-resident",
                       "parallelism": "replicas, signal list sharded over ranks" if world > 1 else "single GPU"},
            "normalized_signals": [float(v) for v in gathered[:, 0]] if gathered is not None else None,
            "rel_err_vs_oracle": err_oracle,
            "max_rel_err_vs_oracle": max(err_oracle) if err_oracle else None,
            "iterations_per_signal": st["total_iterations"] / n_sig,
            "roofline": roof,
            "cpu_baseline": cpu,
            "e2e": {"value": e2e_value, "unit": "signals/s", "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h),
                    "what": "bt_create+bt_mesh_upload (device graph build)+bt_set_coefficients+bt_assemble+"
                            "bt_set_schedule+bt_solve (FP64), host arrays in, signals out; median of %d"
                            % len(e2e_ms)},
            "gpu_launches": int(st["kernel_launches"]) * args.steps,
            "clocks": clocks,
        }
        res.update(legs)
        print(json.dumps(res))
    if world > 1:
        torch.distributed.destroy_process_group()
    return res


def mixed_cfg2_leg(args, pkg, ctx, q, g, pidx, n64, ms64, gold, sel, traffic, info, peak, peak_src, timed_steps):
    """The batched mixed-precision path on the same 40^3 workload (2 signals in
    one launch), its per-signal error against the oracle and the FP64 path."""
    tot, outs, clk = timed_steps(pkg.PRECISION_MIXED, 1e-9, args.mixed_steps, 2)
    st = outs[-1]["stats"]
    nm = outs[-1]["signal"] / outs[-1]["S0"]
    n_sig = len(q)
    iters = st["total_iterations"] / n_sig
    byts = alg_bytes_mixed(info["n_dofs"], info["nnz"], n_sig, st["steps"], iters, st["refinements"])
    launch_ms = st["stepper_ms"]
    ach = byts / (launch_ms / 1e3) / 1e9
    roof = {"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak,
            "traffic": traffic.get("bytes_per_launch") if traffic else None,
            "kernel": "k_batched (persistent mixed-precision stepper, %d signals per launch)" % n_sig,
            "bytes_per_launch": byts, "launch_ms": launch_ms, "peak_source": peak_src,
           "frac_of_nominal_7900": ach / NOMINAL_HBM_GBS}
    if traffic:
        roof["note"] = ("L2-resident: ncu counts %.0f MB of DRAM traffic per launch, %.2f%% of the algorithmic "
                        "bytes; `frac` counts L2-served bytes" % (traffic["bytes_per_launch"] / 1e6,
                                                                  100.0 * traffic["bytes_per_launch"] / byts))
    err_or = [abs(float(v) - gold[b]) / abs(gold[b]) for (b, _, _), v in zip(sel, nm) if b in gold]
    value = n_sig * args.mixed_steps / (tot / 1e3)
    return {"workload": "cfg2 (the headline's workload) on the mixed-precision path", "precision": "mixed",
            "dtype": "f32 inner COCG + double-float (FP32 pair, ~44 bit) residual, refinement and state; FP64 signal "
                     "sum (a deviation from FP64 residuals, chosen because GB300's FP64 issue rate is low)",
            "rtol": 1e-9, "signals": n_sig, "value": value, "unit": "signals/s", "ms_per_step": tot / args.mixed_steps,
            "steps": args.mixed_steps, "mixed_over_plain_fp64": value / (n_sig / (ms64 / 1e3)),
            "rel_err_vs_oracle": err_or, "rel_err_vs_fp64": [float(abs(a - b) / abs(b)) for a, b in zip(nm, n64)],
            "iterations_per_signal": iters, "refinements": st["refinements"], "roofline": roof, "clocks": clk}


def batched_leg(args, pkg, stream, flush, peak, peak_src, traffic):
    """All 512 signals of the eight-cylinder 64^3 workload on the mixed path
    (two launches of 256), against the FP64 path on `fp64_sample` signals
    spread over the 512, and the error of every signal against the FP64 values
    of the committed fixture."""
    w = pkg.meshgen.workload("cfg3")
    sig = w["signals"][:args.batched_signals]
    q, g, pidx = _signal_arrays(pkg, w, sig)
    local = int(os.environ.get("LOCAL_RANK", "0"))
    ctx, fn, fo = _context(pkg, w, local, stream)
    info = ctx.info()
    timed = _event_timer(stream, flush)
    # warm-up: the autotuner's 3-step trials for this batch size, on a short schedule
    ctx.set_schedule(fn[:, :4], fo[:, :4], w["dt"])
    ctx.solve(q[:256], g[:256], pidx[:256], None, pkg.PRECISION_MIXED, 1e-9, args.maxit)
    ctx.set_schedule(fn, fo, w["dt"])
    ms_mix, out = timed(lambda: ctx.solve(q, g, pidx, None, pkg.PRECISION_MIXED, 1e-9, args.maxit))
    n_sig = len(q)
    nm = out["signal"] / out["S0"]
    samp = np.unique(np.linspace(0, n_sig - 1, max(1, args.fp64_sample)).astype(int))
    ms_64, o64 = timed(lambda: ctx.solve(q[samp], g[samp], pidx[samp], None, pkg.PRECISION_FP64, 1e-12, args.maxit))
    n64 = o64["signal"] / o64["S0"]
    err_live = np.abs(nm[samp] - n64) / np.abs(n64)
    fx = load_json("tests", "golden", "gpu_fp64_cfg3_signals.json")
    per_signal = None
    if fx and len(fx.get("normalized", [])) >= n_sig:
        ref = np.asarray(fx["normalized"][:n_sig])
        per_signal = (np.abs(nm - ref) / np.abs(ref)).tolist()
    st = out["stats"]
    launches = -(-n_sig // 256)
    per = n_sig / launches
    iters = st["total_iterations"] / n_sig
    byts = alg_bytes_mixed(info["n_dofs"], info["nnz"], per, st["steps"], iters, st["refinements"] / launches)
    launch_ms = st["stepper_ms"] / launches
    ach = byts / (launch_ms / 1e3) / 1e9
    Rp = 2 * int(per)
    wset = info["n_dofs"] * (Rp * 8 * 6 + (Rp // 2) * 8 * 7) + info["nnz"] * 44
    tr = (traffic or {}).get("cfg3:mixed")
    v_mix = n_sig / (ms_mix / 1e3)
    v_64 = len(samp) / (ms_64 / 1e3)
    ctx.close()
    return {"workload": "cfg3: " + WORKLOADS["cfg3"], "precision": "mixed", "signals": n_sig,
            "launches": launches, "n_dofs": info["n_dofs"], "nnz": info["nnz"],
            "value": v_mix, "unit": "signals/s", "ms": ms_mix,
            "plain_fp64_value": v_64, "plain_fp64_signals_timed": len(samp),
            "mixed_over_plain": v_mix / v_64,
            "max_rel_err_vs_fp64_live": float(err_live.max()),
            "rel_err_vs_fp64_all_signals": per_signal,
            "max_rel_err_vs_fp64_all_signals": max(per_signal) if per_signal else None,
            "fp64_reference": ("tests/golden/gpu_fp64_cfg3_signals.json (FP64 path, rtol 1e-12, every signal) and "
                               "%d signals re-run live" % len(samp)),
            "iterations_per_signal": iters, "refinements": st["refinements"],
            "roofline": {"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak,
                         "traffic": tr.get("bytes_per_launch") if tr else None,
                         "bytes_per_launch": byts, "launch_ms": launch_ms, "peak_source": peak_src,
                         "frac_of_nominal_7900": ach / NOMINAL_HBM_GBS,
                         "note": "algorithmic bytes (bench.alg_bytes_mixed); working set %.1f GB, %.0fx the L2"
                                 % (wset / 1e9, wset / L2_BYTES)}}


def adjoint_leg(args, pkg, stream, flush, peak, peak_src, traffic):
    """Gradients: the layered-sphere 48^3 workload (4 layers, per-layer D and T2,
    per-interface kappa), `adjoint_signals` of its 120 signals spread evenly
    (default: all 120); the batched mixed-precision adjoint (bt_adjoint_batch)
    against the FP64 adjoint (bt_adjoint) of five spread signals."""
    w = pkg.meshgen.workload("cfg4")
    sig = w["signals"]
    idx = np.linspace(0, len(sig) - 1, args.adjoint_signals).astype(int)
    q, g, _ = _signal_arrays(pkg, w, [sig[i] for i in idx])
    local = int(os.environ.get("LOCAL_RANK", "0"))
    ctx, _, _ = _context(pkg, w, local, stream)
    timed = _event_timer(stream, flush)
    ctx.solve(q, g, None, None, pkg.PRECISION_MIXED, 1e-9, args.maxit)          # warm-up (autotuner)
    ms_b, out = timed(lambda: ctx.adjoint_batch(q, g, rtol=1e-9, max_iterations=args.maxit))
    chk = sorted(set(np.linspace(0, len(q) - 1, min(5, len(q))).astype(int).tolist()))
    ms_64 = []
    err = {"dD": 0.0, "dinvT2": 0.0, "dkappa": 0.0}
    sig_err = 0.0
    for k in chk:
        m, ref = timed(lambda: ctx.adjoint(q[k], g[k], rtol=1e-12, max_iterations=args.maxit))
        ms_64.append(m)
        for key in err:
            err[key] = max(err[key], float(np.max(np.abs(out[key][k] - ref[key])) / np.max(np.abs(ref[key]))))
        sig_err = max(sig_err, float(abs(out["signal"][k] - ref["signal"]) / abs(ref["signal"])))
    info = ctx.info()
    ctx.close()
    n = len(q)
    v64 = 1.0 / (statistics.mean(ms_64) / 1e3)
    return {"workload": "layered sphere 48^3 (4 regions, D/T2 per layer, kappa per interface), PGSE, "
                        "%d signals in one batched adjoint" % n,
            "n_dofs": info["n_dofs"], "signals": n,
            "batched_mixed": {"gradients_per_s": n / (ms_b / 1e3), "ms": ms_b,
                              "parameters_per_signal": "D x4, 1/T2 x4, kappa x3"},
            "fp64_adjoint": {"gradients_per_s": v64, "ms_per_signal": statistics.mean(ms_64),
                             "signals_checked": chk},
            "ratio": (n / (ms_b / 1e3)) / v64,
            "max_rel_err_vs_fp64_adjoint": err, "signal_rel_err": sig_err}


def uneven_leg(args, pkg, stream, flush, peak, peak_src, traffic):
    """Several meshes of uneven size in one persistent launch (bt_solve_multi):
    `uneven_meshes` seeded boxes of 8^3 ... 24^3 Kuhn cubes of 1.5 um with
    random z-cylinders (D 3e-3 / 2e-3, kappa U[1e-5,1e-4]), 4 b-values along one
    direction each, PGSE; against one launch per mesh, and the largest mesh
    against the FP64 path."""
    meshes = pkg.meshgen.uneven_meshes(count=args.uneven_meshes, seed=0, nmin=8, nmax=24, cube=1.5)
    p = pkg.sequences.pgse(10600, 43100)
    fn, fo = pkg.sequences.profile_samples(p, 200.0)
    qs = [pkg.sequences.b_to_q(b, p.int4gb()) for b in (1000.0, 2000.0, 3000.0, 4000.0)]
    gs = [[0.36, 0.48, 0.8]] * 4
    ctxs = []
    local = int(os.environ.get("LOCAL_RANK", "0"))
    for m in meshes:
        c = pkg.Context(local)
        c.set_stream(stream.cuda_stream)
        c.mesh_upload(m["xyz"], m["tets"], m["region"], 2)
        c.set_coefficients(m["D"], None, m["kappa"])
        c.assemble()
        c.set_schedule(fn, fo, 200.0)
        ctxs.append(c)
    n = len(ctxs)
    timed = _event_timer(stream, flush)
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
            "precision": "mixed", "signals": nsig, "value": nsig / (ms_one / 1e3), "unit": "signals/s", "ms": ms_one,
            "separate_launches_value": nsig / (ms_sep / 1e3), "one_launch_over_separate": ms_sep / ms_one,
            "max_rel_err_vs_fp64_largest_mesh": err}


def strong_leg(args, pkg, stream, flush, peak, peak_src, traffic):
    """Strong pseudo-periodic form (IsDomainPeriodic = True): the workload of
    tests/golden/oracle_strong_signals.json (12^3 Kuhn box of 4/3 um cubes, a
    z-cylinder on whole cubes, periodic in x, y, z, PGSE 10600/43100 us, 270
    steps, 4 signals), FP64 Jacobi-BiCGSTAB: the 4 signals in one batched launch
    and one launch each, and 32 signals (the 4 among them) in one batched launch,
    every fixture signal against the oracle's value."""
    gold = load_json("tests", "golden", "oracle_strong_signals.json")
    if gold is None:
        return {"unavailable": "tests/golden/oracle_strong_signals.json missing"}
    s = gold["setup"]
    lo, hi = s["box"]
    xyz, tets = pkg.meshgen.kuhn_box(lo, hi, s["cubes_per_axis"])
    X = xyz[tets]
    c = 0.5 * (X.min(axis=1) + X.max(axis=1))
    reg = (c[:, 0] ** 2 + c[:, 1] ** 2 < s["radius"] ** 2).astype(np.int32)
    p = pkg.sequences.pgse(s["delta"], s["Delta"])
    fn, fo = pkg.sequences.profile_samples(p, s["dt"])
    ctx = pkg.Context(int(os.environ.get("LOCAL_RANK", "0")))
    ctx.set_stream(stream.cuda_stream)
    ctx.mesh_upload(xyz, tets, reg, 2)
    ctx.set_coefficients(s["D"], None, np.array([[0.0, s["kappa"]], [s["kappa"], 0.0]]))
    ctx.assemble()
    ctx.set_periodic_mode("strong")
    ctx.set_periodic(s["periodic_dir"])
    ctx.set_schedule(fn, fo, s["dt"])
    ctx.set_schedule_integral(*pkg.sequences.integral_samples(p, s["dt"]))
    sig = gold["signals"][:max(1, args.strong_signals)]
    q = np.array([g["q"] for g in sig])
    gd = np.array([np.asarray(g["g"]) / np.linalg.norm(g["g"]) for g in sig])
    ctx.solve(q, gd, rtol=1e-12, max_iterations=20000)                     # warm-up (folded system set-up)
    timed = _event_timer(stream, flush)
    ms, out = timed(lambda: ctx.solve(q, gd, rtol=1e-12, max_iterations=20000))   # one batched launch
    err = [abs(float(out["signal"][i]) - g["signal"]) / abs(g["signal"]) for i, g in enumerate(sig)]
    info = ctx.strong_periodic_info()
    st = out["stats"]
    ctx.set_option("strong.batch", 0)                                        # one launch per signal
    ms1, out1 = timed(lambda: ctx.solve(q, gd, rtol=1e-12, max_iterations=20000))
    err1 = [abs(float(out1["signal"][i]) - g["signal"]) / abs(g["signal"]) for i, g in enumerate(sig)]
    ctx.set_option("strong.batch", 1)
    # 32 signals (8 Fibonacci directions x b 1000..4000 with the fixture's four among
    # them): one batched launch, a lane per signal and direction
    dirs = pkg.meshgen.fibonacci_directions(8)
    qb = list(q) + [pkg.sequences.b_to_q(b, p.int4gb()) for d in dirs for b in (1000.0, 2000.0, 3000.0, 4000.0)][:28]
    gb = list(gd) + [d / np.linalg.norm(d) for d in dirs for b in (1000.0, 2000.0, 3000.0, 4000.0)][:28]
    qb, gb = np.array(qb), np.array(gb)
    msb, outb = timed(lambda: ctx.solve(qb, gb, rtol=1e-12, max_iterations=20000))
    errb = [abs(float(outb["signal"][i]) - g["signal"]) / abs(g["signal"]) for i, g in enumerate(sig)]
    ctx.close()
    return {"workload": "strong pseudo-periodic box: 12^3 Kuhn cubes of 4/3 um, z-cylinder r 5 um, periodic x/y/z, "
                        "D 3e-3/2e-3, kappa 1e-5, PGSE 10600/43100 us, 270 steps",
            "precision": "fp64", "solver": "Jacobi-BiCGSTAB, rtol 1e-12", "signals": len(sig),
            "value": len(sig) / (ms / 1e3), "unit": "signals/s", "ms": ms,
            "folded_dofs": info["n_dofs"], "vertex_classes": info["n_classes"],
            "iterations_per_launch": st["total_iterations"] / len(sig),
            "rel_err_vs_oracle": err, "max_rel_err_vs_oracle": max(err),
            "single_launches": {"value": len(sig) / (ms1 / 1e3), "ms": ms1, "max_rel_err_vs_oracle": max(err1)},
            "batch_32": {"what": "32 signals: the fixture's 4 and 7 more Fibonacci directions x b 1000..4000, one "
                                 "batched launch (a lane per signal)",
                         "value": 32 / (msb / 1e3), "unit": "signals/s", "ms": msb,
                         "over_single_launches": (32 / (msb / 1e3)) / (len(sig) / (ms1 / 1e3)),
                         "rel_err_vs_oracle_fixture_signals": errb}}


def cfg5_leg(args, pkg, stream, flush, peak, peak_src, traffic):
    """The uneven batch: 16 seeded boxes of 24^3 ... 96^3 Kuhn cubes of 0.5 um
    (edge counts stepped evenly) with random non-overlapping z-cylinders (radii
    U[1.5,5] um up to an area fraction U[0.1,0.4]), kappa U[1e-5,1e-4], D_in 2e-3,
    D_out 3e-3; `cfg5` signals per mesh from 32 Fibonacci directions x b in
    {1000, 2000, 3000, 4000} (128: the whole 2,048-signal workload), PGSE.  Times
    the forward solve of every mesh (bt_solve_multi) and the gradients dS/dD,
    dS/d(1/T2), dS/dkappa of every signal (bt_adjoint_multi), and checks one
    signal of every mesh against the FP64 path and the gradients of four meshes
    against the FP64 adjoint."""
    meshes = pkg.meshgen.uneven_meshes(count=16, seed=0, nmin=24, nmax=96, cube=0.5)
    p = pkg.sequences.pgse(10600, 43100)
    fn, fo = pkg.sequences.profile_samples(p, 200.0)
    dirs = pkg.meshgen.fibonacci_directions(32)
    allsig = [(b, d) for d in dirs for b in (1000.0, 2000.0, 3000.0, 4000.0)]
    pick = np.linspace(0, len(allsig) - 1, min(args.cfg5, len(allsig))).astype(int)
    qs = [pkg.sequences.b_to_q(allsig[i][0], p.int4gb()) for i in pick]
    gs = [allsig[i][1] for i in pick]
    local = int(os.environ.get("LOCAL_RANK", "0"))
    ctxs = []
    for m in meshes:
        c = pkg.Context(local)
        c.set_stream(stream.cuda_stream)
        c.mesh_upload(m["xyz"], m["tets"], m["region"], 2)
        c.set_coefficients(m["D"], None, m["kappa"])
        c.assemble()
        c.set_schedule(fn[:4], fo[:4], 200.0)
        ctxs.append(c)
    n = len(ctxs)
    pkg.solve_multi(ctxs, [qs] * n, [gs] * n, rtol=1e-9)            # warm-up: the autotuner's trials
    for c in ctxs:
        c.set_schedule(fn, fo, 200.0)
    timed = _event_timer(stream, flush)
    ms_f, fw = timed(lambda: pkg.solve_multi(ctxs, [qs] * n, [gs] * n, rtol=1e-9))
    ms_a, ad = timed(lambda: pkg.adjoint_multi(ctxs, [qs] * n, [gs] * n, rtol=1e-9))
    nsig = n * len(qs)
    err_f, err_a = [], []
    for k, c in enumerate(ctxs):
        i = (5 * k) % len(qs)
        r64 = c.solve([qs[i]], [gs[i]], precision=pkg.PRECISION_FP64, rtol=1e-12, max_iterations=20000)["signal"][0]
        err_f.append(float(abs(fw["signal"][k][i] - r64) / abs(r64)))
        err_a.append(float(abs(ad["signal"][k][i] - r64) / abs(r64)))
    gerr = {}
    for k in (0, 5, 10, 15):
        c = ctxs[k]
        i = (5 * k) % len(qs)
        ref = c.adjoint(qs[i], gs[i], rtol=1e-12, max_iterations=20000)
        for key in ("dD", "dinvT2", "dkappa"):
            e = float(np.max(np.abs(ad[key][k][i] - ref[key])) / np.max(np.abs(ref[key])))
            gerr[key] = max(gerr.get(key, 0.0), e)
    dofs = [c.info()["n_dofs"] for c in ctxs]
    cells = [c.info()["n_cells"] for c in ctxs]
    for c in ctxs:
        c.close()
    return {"workload": "cfg5: 16 seeded cylinder boxes, %d^3..%d^3 Kuhn cubes of 0.5 um (%d..%d dofs, up to %d "
                        "tets), kappa U[1e-5,1e-4], D_in 2e-3 / D_out 3e-3, %d signals per mesh (32 Fibonacci "
                        "directions x b 1000..4000), PGSE 10600/43100 us, dt 200 us"
                        % (meshes[0]["n"], meshes[-1]["n"], min(dofs), max(dofs), max(cells), len(qs)),
            "precision": "mixed", "signals": nsig, "dofs_per_mesh": dofs,
            "forward": {"value": nsig / (ms_f / 1e3), "unit": "signals/s", "ms": ms_f,
                        "max_rel_err_vs_fp64_one_signal_per_mesh": max(err_f)},
            "gradients": {"value": nsig / (ms_a / 1e3), "unit": "gradients/s", "ms": ms_a,
                          "parameters_per_signal": "D x2, 1/T2 x2, kappa x1",
                          "signal_rel_err_vs_fp64": max(err_a),
                          "max_rel_err_vs_fp64_adjoint_meshes_0_5_10_15": gerr}}


def batched_profile(args):
    """One short launch for a profiler: `profile_signals` signals of the
    eight-cylinder 64^3 workload, schedule cut to `batched_profile` steps inside
    the first gradient pulse, geometry fixed (lanes-per-row 32, two blocks per
    SM, interleaved rows) so that no autotuner trial runs first."""
    pkg = importlib.import_module(PKG)
    pkg._native.load(pkg.build())
    w = pkg.meshgen.workload("cfg3")
    n = args.batched_profile
    fns, fos = zip(*[pkg.sequences.profile_samples(p, w["dt"]) for p in w["profiles"]])
    fn, fo = np.array(fns)[:, 20:20 + n], np.array(fos)[:, 20:20 + n]
    sig = w["signals"]
    sel = [sig[i] for i in np.linspace(0, len(sig) - 1, args.profile_signals).astype(int)]
    q, g, pidx = _signal_arrays(pkg, w, sel)
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
    vals = [cpu_baseline("cfg2", workers) for _ in range(args.ref_steps)]
    v = statistics.median(x["value"] for x in vals)
    out = {"metric": METRIC,
           "value": v, "unit": "signals/s", "n_gpus": int(os.environ.get("WORLD_SIZE", "1")),
           "steps": args.ref_steps, "warmup": 0, "higher_is_better": True, "scaling": "weak",
           "impl": "reference", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "config": {"workload": "cfg2: " + WORKLOADS["cfg2"]},
           "cpu_baseline": {"value": v, "unit": "signals/s", "cores": workers, "kind": "port",
                            "solve_only_value": statistics.median(x["solve_only_value"] for x in vals),
                            "sample": vals[-1]["sample"]},
           "e2e": {"value": v, "unit": "signals/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--maxit", type=int, default=20000)
    ap.add_argument("--mixed-steps", type=int, default=5, help="timed steps of the mixed leg on 40^3 (0: skip)")
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--cpu-signals", type=int, default=1, help="whole-signal CPU baseline on one core (0: skip)")
    ap.add_argument("--batched-profile", type=int, default=0,
                    help="only one short batched launch of this many steps, for a profiler")
    ap.add_argument("--profile-signals", type=int, default=64, help="signals of the --batched-profile launch")
    ap.add_argument("--batched-signals", type=int, default=512,
                    help="signals of the eight-cylinder 64^3 batched leg (0: skip)")
    ap.add_argument("--fp64-sample", type=int, default=8, help="FP64 signals timed against the batched leg")
    ap.add_argument("--adjoint-signals", type=int, default=120,
                    help="signals of the batched-adjoint leg on the 48^3 layered sphere (0: skip)")
    ap.add_argument("--uneven-meshes", type=int, default=16,
                    help="meshes of the uneven multi-mesh leg (0: skip)")
    ap.add_argument("--strong-signals", type=int, default=4,
                    help="signals of the strong pseudo-periodic leg (0: skip)")
    ap.add_argument("--cfg5", type=int, default=0,
                    help="signals per mesh of the 16-mesh 24^3..96^3 forward + adjoint leg (128: the whole "
                         "workload, several minutes; 0: skip)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 0)
    args.ref_steps = max(1, min(args.steps, 2))
    if args.batched_profile > 0:
        batched_profile(args)
    elif args.impl == "reference":
        reference_run(args)
    else:
        gpu_run(args)


if __name__ == "__main__":
    main()
