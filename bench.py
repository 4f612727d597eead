#!/usr/bin/env python
"""Benchmark: Projected-Newton iterations/s of the sparse per-element
derivative path on one GB300 (TinyAD's eval_with_hessian_proj +
newton_direction + line_search loop, tests/NewtonTest.cc:69-75).

Default workload: the large mixed-precision parametrisation -- symmetric
Dirichlet on a jittered, lifted disk from a 1024 x 1024 grid (1.64M faces,
1.64M variables), Tutte initial UVs -- in mixed precision (FP32 element
Hessians, projection and PCG; FP64 values, gradient, line-search energy and
refinement).  One step = one Newton iteration (element eval + projection +
assembly + PCG solve + line search) on the device-resident state.

Also reported: the same loop in FP64 (the plain drop-in), element-Hessians/s,
kernel roofline figures, an end-to-end figure through the C ABI with host
buffers, and the CPU restatement of the reference path timed on this host.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--workload disk1024|disk64|tet48] [--precision mixed|fp64]
"""
from __future__ import annotations

import argparse
import json
import os
import platform
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "Newton iters/s & element-Hessians/s, mixed vs FP64 GPU at 1e-8 energy err"
# Algorithmic flops per element of the element kernels: the library's
# symmetric Dirichlet evaluation (packed forward-mode scalar over the d(N-1)
# non-constant vertices, plus the lift of the first vertex's derivatives) and
# its translation-deflated PSD projection (averaged over seeded elements),
# counted by oracle/flop_count.sh with op-counting scalar types.
ELEM_FLOPS = {6: 3283, 12: 49256}
UNIT = "Newton iters/s"
# DRAM bytes per launch (dram__bytes_read.sum + dram__bytes_write.sum) of the
# element kernels (K1 + K2) and of the PCG SpMV, each read from one ncu
# capture of that kernel on the named workload -- figures of that capture, not
# measured by this run (reported with "traffic_source"); workloads without a
# capture report null
TRAFFIC_FROM_CAPTURE = {("disk1024", "mixed"): {"elem": (131.3e6 + 195.9e6) + (157.5e6 + 100.1e6), "spmv": 138.0e6 + 5.1e6}}
TRAFFIC_SOURCE = "one ncu capture of the kernel on this workload and precision (not measured in this run)"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="disk1024")
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--no-fp64", action="store_true", help="skip the FP64 comparison leg")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-extra", action="store_true",
                    help="skip the summaries of the other configurations (tet48, adjoint254, batch256)")
    ap.add_argument("--kernels-only", action="store_true",
                    help="profile the main kernels once at the initial state (for ncu captures) and exit")
    return ap.parse_args()


def reduce_max(v: float, dist, device) -> float:
    """Max over ranks (timings: the slowest rank defines the step time)."""
    if dist is None:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def aggregate_rate(world: int, steps: int, seconds: float) -> float:
    """Whole-job rate for weak scaling: every rank runs its own mesh replica."""
    return world * steps / seconds


def make_workload(name: str, rank: int = 0):
    from tinyad_gb300 import meshes
    if name.startswith("disk"):
        grid = int(name[4:])
        return meshes.disk_param(grid, seed=2 + 1000 * rank, name=name)
    if name.startswith("tet"):
        return meshes.tet_twist(int(name[3:]), seed=1 + 1000 * rank, name=name)
    raise SystemExit(f"unknown workload {name}")


def workload_desc(w) -> str:
    if w.name.startswith("disk"):
        return (f"{w.name}: symmetric Dirichlet planar parametrisation of a jittered, lifted disk from a "
                f"{w.info['grid']}x{w.info['grid']} grid ({w.info['n_faces']} faces, {w.info['n_verts']} vertices), "
                f"Tutte initial UVs, k=6")
    return (f"{w.name}: {w.info['cells']}^3 cube, 6 tets/cube ({w.info['n_tets']} tets, {w.info['n_verts']} vertices), "
            f"symmetric Dirichlet k=12 + z=0 pin / z=1 45-degree twist penalties")


# ---------------------------------------------------------------------------
# clocks sampled during the timed region
# NVML clock-event reason bits (nvml.h, nvmlClocksEventReason*)
_NVML_REASONS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown", 0x40: "hw_thermal_slowdown",
                 0x80: "hw_power_brake_slowdown"}


class ClockSampler:
    """Samples the SM clock and the clock-event reasons of this process's GPU
    every ~2 ms through NVML (read-only queries), so that even a timed region
    of a few tens of milliseconds gets samples; mark() / unmark() bracket the
    timed region.  Falls back to `nvidia-smi -lms 100` when NVML cannot be
    loaded."""

    def __init__(self, cuda_index: int = 0, period_s: float = 0.002):
        self.cuda_index = cuda_index
        self.period = period_s
        self.samples = []          # (t, sm_mhz, reasons_mask, in_region)
        self.max_mhz = None
        self.in_region = False
        self.stop = threading.Event()
        self.proc = None
        self.source = None

    def _nvml_handle(self):
        import ctypes
        lib = ctypes.CDLL("libnvidia-ml.so.1")
        if lib.nvmlInit_v2() != 0:
            raise OSError("nvmlInit failed")
        h = ctypes.c_void_p()
        ok = False
        try:
            import torch
            uuid = str(torch.cuda.get_device_properties(self.cuda_index).uuid)
            ok = lib.nvmlDeviceGetHandleByUUID(("GPU-" + uuid).encode(), ctypes.byref(h)) == 0
        except Exception:
            ok = False
        if not ok:
            vis = os.environ.get("CUDA_VISIBLE_DEVICES", "")
            ids = [v for v in vis.split(",") if v.strip()]
            idx = int(ids[self.cuda_index]) if ids and ids[self.cuda_index].strip().isdigit() else self.cuda_index
            if lib.nvmlDeviceGetHandleByIndex_v2(idx, ctypes.byref(h)) != 0:
                raise OSError("no NVML handle")
        return lib, h

    def _run_nvml(self, lib, h):
        import ctypes
        clk = ctypes.c_uint()
        mask = ctypes.c_ulonglong()
        get_reasons = getattr(lib, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
            lib.nvmlDeviceGetCurrentClocksThrottleReasons
        while not self.stop.is_set():
            if lib.nvmlDeviceGetClockInfo(h, 1, ctypes.byref(clk)) == 0:   # NVML_CLOCK_SM
                r = get_reasons(h, ctypes.byref(mask))
                self.samples.append((time.perf_counter(), float(clk.value), int(mask.value) if r == 0 else 0,
                                     self.in_region))
            time.sleep(self.period)

    def __enter__(self):
        try:
            import ctypes
            lib, h = self._nvml_handle()
            mx = ctypes.c_uint()
            if lib.nvmlDeviceGetMaxClockInfo(h, 1, ctypes.byref(mx)) == 0:
                self.max_mhz = float(mx.value)
            self.source = "nvml (2 ms polling)"
            self.t = threading.Thread(target=self._run_nvml, args=(lib, h), daemon=True)
            self.t.start()
        except Exception:
            self._start_smi()
        return self

    def _start_smi(self):
        q = ("clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        bits = [0x8, 0x40, 0x20, 0x4]
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                          "-i", str(self.cuda_index), "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.source = "nvidia-smi -lms 100"

            def read():
                for line in self.proc.stdout:
                    parts = [x.strip() for x in line.split(",")]
                    try:
                        sm, mx = float(parts[0]), float(parts[1])
                    except (ValueError, IndexError):
                        continue
                    self.max_mhz = mx
                    m = sum(b for b, v in zip(bits, parts[2:6]) if v.lower() in ("active", "1", "yes"))
                    self.samples.append((time.perf_counter(), sm, m, self.in_region))
            self.t = threading.Thread(target=read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def mark(self):
        self.in_region = True

    def unmark(self):
        self.in_region = False

    def __exit__(self, *a):
        self.stop.set()
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        elif getattr(self, "t", None) is not None:
            self.t.join(timeout=1)

    def summary(self) -> dict:
        region = [s for s in self.samples if s[3]]
        use = region if region else self.samples
        sm = sorted(s[1] for s in use)
        mask = 0
        for s in use:
            mask |= s[2]
        reasons = sorted(nm for bit, nm in _NVML_REASONS.items() if mask & bit)
        return {"sm_mhz": sm[len(sm) // 2] if sm else None, "sm_max_mhz": self.max_mhz, "reasons": reasons,
                "samples": len(sm), "window": "timed region" if region else "whole run (no sample inside the region)",
                "source": self.source}


# ---------------------------------------------------------------------------
# CPU baseline: the oracle (restatement of the reference's OpenMP path)
# ---------------------------------------------------------------------------
CPU_SAMPLE = "disk512"
CPU_SAMPLE_MAX_ELEMENTS = 500_000   # a workload up to this size is timed whole


def cpu_sample(full_w):
    """The mesh the CPU legs time: the workload itself up to
    CPU_SAMPLE_MAX_ELEMENTS elements, else a smaller mesh of the same family
    (512-grid disk / 24^3 tet cube), scaled to the workload by element count."""
    if full_w.n_elements <= CPU_SAMPLE_MAX_ELEMENTS:
        return full_w
    return make_workload("tet24" if full_w.name.startswith("tet") else CPU_SAMPLE)


def host_cpu() -> dict:
    """The host the CPU legs ran on: hardware threads and the CPU model (lscpu's
    "Model name", else /proc/cpuinfo's "model name", else the machine type)."""
    model = None
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        model = next((l.split(":", 1)[1].strip() for l in out.splitlines() if l.startswith("Model name")), None)
    except (OSError, subprocess.SubprocessError):
        pass
    if not model:
        try:
            with open("/proc/cpuinfo") as f:
                model = next((l.split(":", 1)[1].strip() for l in f if l.lower().startswith("model name")), None)
        except OSError:
            pass
    return {"nproc": os.cpu_count(), "model": model or platform.machine()}


def cpu_baseline(full_w, threads: int | None = None) -> dict:
    """One oracle Projected-Newton iteration (OpenMP element eval, serial
    scatter + triplet sort, sparse LDL^T, Armijo) on cpu_sample(full_w),
    scaled to the benchmark mesh by element count."""
    from oracle import pyoracle
    w = cpu_sample(full_w)
    CPU = w.name
    nthreads = threads if threads else -1
    p = pyoracle.Problem.from_workload(w, n_threads=nthreads)
    t0 = time.perf_counter()
    x, fh, times = p.newton(w.x0, 1)
    dt = time.perf_counter() - t0
    scale = w.n_elements / full_w.n_elements
    return {"value": (1.0 / dt) * scale, "unit": UNIT, "cores": p.n_threads, "kind": "port",
            "sample": (f"1 Projected-Newton iteration of the oracle (CPU restatement of the reference path: OpenMP "
                       f"element eval + projection, serial triplet assembly, sparse LDL^T, Armijo) on {CPU} "
                       f"({w.n_elements} elements) = {dt:.2f} s, scaled by elements to {full_w.n_elements} "
                       f"(linear scaling; the LDL^T grows faster, so this favours the CPU)"),
            "stage_s": {"eval_assemble": times[0], "ldlt": times[1], "line_search": times[2]}, "host": host_cpu()}


REF_TIME_LIMIT_S = 150.0   # timed Newton iterations of the reference arm stop once the next would pass this


def run_reference(args):
    """--impl reference: the reference's CPU path (its restatement in oracle/;
    the reference itself needs Eigen 3, absent here) on the benchmark's own
    workload, with the reference's default thread count (all hardware threads
    but one, Parallel.hh:20-31).  The linear solver's pattern analysis (the
    Hessian's sparsity, the fill-reducing ordering and the symbolic LDL^T) runs
    untimed first, as the reference caches it across iterations
    (LinearSolver.hh:12-19).  Full Newton iterations are then timed one at a
    time, as many as fit REF_TIME_LIMIT_S (at least one, at most --steps), after
    the requested warm-up iterations when they are cheap: on the 1.64M-face
    disk one iteration takes about a minute, so only one warm-up iteration
    runs there, and "steps" / "warmup" give the counts actually run."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from oracle import pyoracle
    w = make_workload(args.workload)
    threads = max(1, (os.cpu_count() or 2) - 1)
    p = pyoracle.Problem.from_workload(w, n_threads=threads)
    t0 = time.perf_counter()
    p.prepare_solver(w.x0)
    t_prep = time.perf_counter() - t0
    x = w.x0.copy()
    # warm-up iterations while they are cheap: all W when W times the first
    # one's cost fits half the time limit, else only that first one
    warm = 0
    if args.warmup > 0:
        t0 = time.perf_counter()
        x, _, _ = p.newton(x, 1)
        t_first = time.perf_counter() - t0
        warm = 1
        if args.warmup * t_first <= 0.5 * REF_TIME_LIMIT_S:
            for _ in range(args.warmup - 1):
                x, _, _ = p.newton(x, 1)
            warm = args.warmup
    per_iter, stages = [], np.zeros(3)
    total = 0.0
    while len(per_iter) < max(1, args.steps):
        t0 = time.perf_counter()
        x, _, times = p.newton(x, 1)
        dt = time.perf_counter() - t0
        per_iter.append(dt)
        stages += times[:3]
        total += dt
        if total + dt > REF_TIME_LIMIT_S:
            break
    n = len(per_iter)
    v = n / total
    sample = (f"{n} Projected-Newton iteration(s) (iterations {warm + 1}..{warm + n} from the Tutte initial state, "
              f"after {warm} untimed warm-up iteration(s)) of the oracle, the CPU restatement of the reference path "
              f"(OpenMP element evaluation + projection, serial triplet assembly, sparse LDL^T with a "
              f"nested-dissection ordering, Armijo), on the benchmark workload itself ({w.name}, {w.n_elements} "
              f"elements); pattern analysis {t_prep:.1f} s untimed; iterations stop at a {REF_TIME_LIMIT_S:.0f} s limit")
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": n, "steps_requested": args.steps, "warmup": warm, "warmup_requested": args.warmup,
            "ms_per_step": total / n * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic (seeded generator)",
            "config": {"workload": workload_desc(w)},
            "seconds_per_iteration": per_iter,
            "stage_s": {"eval_assemble": stages[0], "factor_solve": stages[1], "line_search": stages[2]},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": p.n_threads, "kind": "port", "sample": sample,
                             "host": host_cpu()},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# batched solves (config 4): 256 disks, face counts log-uniform in [1k, 50k]
# ---------------------------------------------------------------------------
def measure_batch(args, rank: int, n_meshes: int, sequential: bool = True) -> dict:
    """The batched-solve workload: n_meshes disk parametrisations with face
    counts log-uniform in [1k, 50k], one CUDA graph per batched Newton
    iteration; mixed and FP64, and (sequential) the same meshes solved one
    problem at a time with the same algorithm."""
    import torch
    import tinyad_gb300 as tad
    from tinyad_gb300 import meshes

    t0 = time.perf_counter()
    ws = meshes.disk_batch(n_meshes, 1000, 50000, seed=4 + rank)
    t_gen = time.perf_counter() - t0
    n_faces = sum(w.n_elements for w in ws)
    res = {}
    clk = ClockSampler(torch.cuda.current_device()).__enter__()
    for name, prec in (("mixed", tad.PREC_MIXED), ("fp64", tad.PREC_FP64)):
        b = tad.Batch(ws, precision=prec, pcg_rel_tol=1e-2, pcg_max_iters=64)
        x = torch.from_numpy(b.x0()).cuda()
        # warm-up iterations, then the launch shape is tuned on the state the timed iterations start from
        b.newton_solve_device(x.data_ptr(), args.warmup)
        tune = b.autotune(x.data_ptr())
        stream = torch.cuda.ExternalStream(b.stream_ptr)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        if name == "mixed":
            clk.mark()
            torch.cuda.profiler.start()   # an ncu launch list with --profile-from-start off covers these iterations
        e0.record(stream)
        b.newton_solve_device(x.data_ptr(), args.steps)
        e1.record(stream)
        torch.cuda.synchronize()
        if name == "mixed":
            torch.cuda.profiler.stop()
        clk.unmark()
        ms = e0.elapsed_time(e1)
        fh = b.newton_solve_device(x.data_ptr(), 1, history=True)
        res[name] = {"batch_iters_per_s": args.steps / (ms / 1e3), "mesh_iters_per_s": n_meshes * args.steps / (ms / 1e3),
                     "ms_per_iteration": ms / args.steps, "autotune": tune,
                     "element_hessians_per_s": n_faces * args.steps / (ms / 1e3),
                     "mean_final_energy": float(np.mean(fh[-1]))}
        del b
    # sequential baseline: the same meshes one problem at a time, one iteration each, with the batch's
    # algorithm (block-Jacobi PCG without the AMG restart, at most 16 Armijo trials)
    seq = []
    t_seq = None
    if sequential:
        fns = [tad.ScalarFunction.from_workload(w, precision=tad.PREC_MIXED, pcg_rel_tol=1e-2, pcg_max_iters=64,
                                                preconditioner=0, ls_max_iters=16) for w in ws]
        xs = [torch.from_numpy(w.x0.copy()).cuda() for w in ws]
        for fn, xx in zip(fns, xs):
            fn.newton_solve_device(xx.data_ptr(), args.warmup)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(max(1, args.steps // 2)):
            for fn, xx in zip(fns, xs):
                fn.newton_solve_device(xx.data_ptr(), 1)
        torch.cuda.synchronize()
        t_seq = (time.perf_counter() - t0) / max(1, args.steps // 2)
        del fns, xs
    line = {"metric": METRIC, "value": res["mixed"]["batch_iters_per_s"], "unit": "batched Newton iters/s",
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": res["mixed"]["ms_per_iteration"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 Hessian/PCG + f64 value/gradient", "data": "synthetic (seeded generator)",
            "config": {"workload": f"batch{n_meshes}: {n_meshes} disk parametrisations, faces log-uniform in [1k, 50k] "
                                   f"({n_faces} faces total), one CUDA graph per batched Newton iteration",
                       "newton": "per mesh: PCG tol 1e-2, <= 64 iterations, 16 Armijo trials",
                       "mesh_generation_s": round(t_gen, 1)},
            "mixed": res["mixed"], "fp64": res["fp64"],
            "mixed_vs_fp64": res["mixed"]["batch_iters_per_s"] / res["fp64"]["batch_iters_per_s"],
            "sequential_single_problem_ms_per_iteration": t_seq * 1e3 if t_seq else None,
            "batched_vs_sequential": t_seq * 1e3 / res["mixed"]["ms_per_iteration"] if t_seq else None}
    clk.__exit__(None, None, None)
    line["clocks"] = clk.summary()
    return line


def run_batch(args, rank: int):
    n_meshes = int(args.workload[5:]) if len(args.workload) > 5 else 256
    print(json.dumps(measure_batch(args, rank, n_meshes)), flush=True)


def measure_adjoint(args, grid: int = 254) -> dict:
    """The adjoint workload: a ~100k-triangle pinned disk parametrisation
    (254^2 grid) solved to |g| < 1e-9 in FP64; loss L = 1/2 |x* - target|^2
    with target = x* + N(0, 0.01^2) noise; dL/d(rest positions) by the device
    adjoint (solve H lambda = dL/dx on the exact Hessian, contract lambda with
    the per-element mixed derivatives).  Checked against central differences
    of re-solved minimisers (h = 1e-6, 64 seeded unit directions) and against
    the oracle's CPU adjoint; the GPU adjoint and the CPU adjoint are timed."""
    import torch
    import tinyad_gb300 as tad
    from tinyad_gb300 import meshes

    n_dirs = 64
    t0 = time.perf_counter()
    w = meshes.disk_param_pinned(grid, seed=11)
    t_gen = time.perf_counter() - t0
    x, fn = tad.solve_minimiser(w, w.x0, newton_iters=60, full_steps=3)
    _, g = fn.eval_with_gradient(x)
    gnorm = float(np.linalg.norm(g))
    rng = np.random.default_rng(12)
    target = x + rng.normal(scale=0.01, size=x.size)
    dLdx = x - target
    # GPU adjoint: warm-up, then timed (host in / host out, the C ABI call)
    fn.adjoint_rest_gradient(x, dLdx, w.rest, projected=False)
    torch.cuda.synchronize()
    reps = max(1, args.steps)
    t0 = time.perf_counter()
    for _ in range(reps):
        grad, lam, iters = fn.adjoint_rest_gradient(x, dLdx, w.rest, projected=False)
    t_gpu = (time.perf_counter() - t0) / reps
    # central differences of re-solved minimisers
    h = 1e-6
    fd_err = []
    t0 = time.perf_counter()
    for _ in range(n_dirs):
        dP = rng.normal(size=w.rest.shape)
        dP /= np.linalg.norm(dP)
        Ls = []
        for sgn in (1.0, -1.0):
            xs, _ = tad.solve_minimiser(meshes.with_rest(w, w.rest + sgn * h * dP), x, newton_iters=3, full_steps=2)
            Ls.append(0.5 * float(np.sum((xs - target) ** 2)))
        fd = (Ls[0] - Ls[1]) / (2 * h)
        an = float(np.sum(grad * dP))
        fd_err.append(abs(fd - an) / max(abs(fd), 1e-12))
    t_fd = time.perf_counter() - t0
    cpu = None
    if not args.no_cpu:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import pyoracle
        p = pyoracle.Problem.from_workload(w, n_threads=max(1, (os.cpu_count() or 2) - 1))
        t0 = time.perf_counter()
        g_cpu, lam_cpu = p.adjoint_rest_gradient(x, dLdx, w.rest, projected=False)
        t_cpu = time.perf_counter() - t0
        cpu = {"value": 1.0 / t_cpu, "unit": "adjoint gradients/s", "cores": max(1, (os.cpu_count() or 2) - 1),
               "kind": "port", "seconds": t_cpu,
               "sample": f"the oracle's adjoint (LDL^T solve + AD<15> mixed blocks) on the same {w.n_elements}-face problem",
               "rel_err_gpu_vs_cpu_gradient": float(np.linalg.norm(grad.reshape(-1) - np.reshape(g_cpu, -1)) /
                                                    np.linalg.norm(np.reshape(g_cpu, -1))),
               "rel_err_gpu_vs_cpu_lambda": float(np.linalg.norm(lam - lam_cpu) / np.linalg.norm(lam_cpu))}
    line = {"metric": "adjoint dL/d(rest positions) at a converged parametrisation", "value": 1.0 / t_gpu,
            "unit": "adjoint gradients/s", "n_gpus": 1, "steps": reps, "warmup": 1, "ms_per_step": t_gpu * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded generator)",
            "config": {"workload": f"adjoint{grid}: pinned disk parametrisation from a {grid}x{grid} grid "
                                   f"({w.n_elements} faces, {w.n_handles} vertices), loss 1/2|x*-target|^2, "
                                   f"target = x* + N(0, 0.01^2)", "mesh_generation_s": round(t_gen, 1)},
            "converged_grad_norm": gnorm, "adjoint_pcg_iters": int(iters),
            "fd_check": {"directions": n_dirs, "h": h, "max_rel_err": max(fd_err), "median_rel_err": float(np.median(fd_err)),
                         "seconds": t_fd},
            "cpu_baseline": cpu}
    return line


def run_adjoint(args, rank: int):
    grid = int(args.workload[7:]) if len(args.workload) > 7 else 254
    print(json.dumps(measure_adjoint(args, grid)), flush=True)


def measure_newton(args, name: str) -> dict:
    """Newton iterations/s of workload `name` in mixed precision and FP64 over
    its solve: an untimed solve from the initial state (up to 30 iterations)
    gives the converged energy and the number of iterations n that reach
    1e-8 of it; then n iterations from the initial state are timed as one
    solver call (CUDA events on the library's stream).  A tetrahedral cube
    converges in a few iterations, after which the steps only move the
    energy at rounding level (and the line search may stop the solve), so a
    fixed window after W warm-up iterations would time no real work."""
    import torch
    import tinyad_gb300 as tad
    w = make_workload(name)
    settings = dict(pcg_rel_tol=1e-2, pcg_max_iters=2000, forcing=0, refine_max_iters=3, refine_rel_tol=1e-8)
    out = {"workload": workload_desc(w),
           "protocol": "iterations from the initial state until the energy is within 1e-8 of the converged energy, "
                       "timed as one solver call after an untimed solve"}
    for pname, prec in (("mixed", tad.PREC_MIXED), ("fp64", tad.PREC_FP64)):
        fn = tad.ScalarFunction.from_workload(w, precision=prec, **settings)
        fn.finalize()
        x = torch.from_numpy(w.x0.copy()).cuda()
        fh_all = fn.newton_solve_device(x.data_ptr(), 30)
        torch.cuda.synchronize()
        f_conv = float(np.min(fh_all))
        n = next(i for i, f in enumerate(fh_all) if f - f_conv <= 1e-8 * abs(f_conv))
        n = max(n, 1)
        x.copy_(torch.from_numpy(w.x0))
        s = torch.cuda.ExternalStream(fn.stream_ptr)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(s)
        fh = fn.newton_solve_device(x.data_ptr(), n)
        e1.record(s)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        st = fn.last_solve_stats()
        done = len(fh) - 1
        out[pname] = {"iters": done, "iters_per_s": done / (ms / 1e3), "ms_per_step": ms / max(done, 1),
                      "seconds": ms / 1e3, "pcg_iters_per_step": st["pcg_iters"] / max(done, 1),
                      "f_final": float(fh[-1]), "f_converged": f_conv}
        del fn, x
        torch.cuda.empty_cache()
    out["mixed_vs_fp64"] = out["mixed"]["iters_per_s"] / out["fp64"]["iters_per_s"]
    out["mixed_vs_fp64_time_to_1e-8"] = out["fp64"]["seconds"] / out["mixed"]["seconds"]
    out["final_energy_rel_diff"] = abs(out["mixed"]["f_converged"] - out["fp64"]["f_converged"]) / abs(out["fp64"]["f_converged"])
    return out


def summary_adjoint(line: dict) -> dict:
    keys = ("value", "unit", "ms_per_step", "converged_grad_norm", "adjoint_pcg_iters", "fd_check")
    out = {k: line[k] for k in keys}
    out["workload"] = line["config"]["workload"]
    cpu = line.get("cpu_baseline") or {}
    out["cpu_oracle_seconds"] = cpu.get("seconds")
    out["rel_err_gpu_vs_cpu_gradient"] = cpu.get("rel_err_gpu_vs_cpu_gradient")
    return out


def summary_batch(line: dict) -> dict:
    return {"workload": line["config"]["workload"], "mixed_batched_iters_per_s": line["mixed"]["batch_iters_per_s"],
            "fp64_batched_iters_per_s": line["fp64"]["batch_iters_per_s"], "mixed_vs_fp64": line["mixed_vs_fp64"],
            "mixed_ms_per_iteration": line["mixed"]["ms_per_iteration"]}





# ---------------------------------------------------------------------------
# our arm
# ---------------------------------------------------------------------------
def main():
    args = parse()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        return run_reference(args)

    import torch
    import tinyad_gb300 as tad

    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    def barrier():
        if dist is not None:
            dist.barrier()

    if args.workload.startswith("batch"):
        return run_batch(args, rank)
    if args.workload.startswith("adjoint"):
        return run_adjoint(args, rank)

    prec = tad.PREC_MIXED if args.precision == "mixed" else tad.PREC_FP64
    t_gen = time.perf_counter()
    w = make_workload(args.workload, rank)
    t_gen = time.perf_counter() - t_gen
    # the same inexact-Newton policy for both precisions: PCG to 1e-2 relative
    # residual (<= 2000 iterations), the fastest-converging mixed policy measured
    settings = dict(pcg_rel_tol=1e-2, pcg_max_iters=2000, forcing=0, refine_max_iters=3, refine_rel_tol=1e-8)

    def make_fn(p):
        fn = tad.ScalarFunction.from_workload(w, precision=p, **settings)
        fn.finalize()
        return fn

    fn = make_fn(prec)
    stream = torch.cuda.ExternalStream(fn.stream_ptr)
    x = torch.from_numpy(w.x0.copy()).cuda()
    if args.kernels_only:
        prof = fn.profile_kernels(x.data_ptr(), reps=3)
        if rank == 0:
            print(json.dumps({"kernels_ms_per_launch": prof, "workload": workload_desc(w), "precision": args.precision}))
        return

    stage = {"ms_eval": 0.0, "ms_assemble": 0.0, "ms_pcg": 0.0, "ms_linesearch": 0.0, "pcg_iters": 0, "ls_trials": 0}
    fh = None
    with ClockSampler(local) as clk:
        # warm-up
        fn.newton_solve_device(x.data_ptr(), args.warmup)
        torch.cuda.synchronize()
        x_warm = x.clone()
        barrier()
        # timed region: K Newton iterations on the device-resident state
        launches0 = fn.launch_count
        torch.cuda.synchronize()
        barrier()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        clk.mark()
        # the timed region is also the profiler range (a no-op unless a
        # profiler started with --profile-from-start off is attached)
        torch.cuda.profiler.start()
        e0.record(stream)
        # the K iterations as one solver call, as a Newton solve runs them
        fh = fn.newton_solve_device(x.data_ptr(), args.steps)
        e1.record(stream)
        st = fn.last_solve_stats()
        for k in stage:
            stage[k] += st[k]
        torch.cuda.synchronize()
        torch.cuda.profiler.stop()
        clk.unmark()
        ms = e0.elapsed_time(e1)
        launches = fn.launch_count - launches0
        if len(fh) - 1 != args.steps:
            raise RuntimeError(f"the solve stopped after {len(fh) - 1} of {args.steps} iterations")
    ms = reduce_max(ms, dist, "cuda")
    value = aggregate_rate(world, args.steps, ms / 1e3)

    # end to end through the C ABI with host buffers (pinned), one call per
    # step, the same protocol as the timed region: W untimed warm-up calls
    # from the initial state, then the K timed calls (Newton iterations
    # W+1..W+K, as above); every call copies x in and out
    n = w.n_vars
    xh = torch.empty(n, dtype=torch.float64, pin_memory=True)
    xh.copy_(torch.from_numpy(w.x0))
    xh_np = xh.numpy()
    for _ in range(args.warmup):
        fn.newton_solve_inplace(xh_np, 1)
    torch.cuda.synchronize()
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        fn.newton_solve_inplace(xh_np, 1)
    t_e2e = time.perf_counter() - t0
    t_e2e = reduce_max(t_e2e, dist, "cuda")
    e2e = {"value": aggregate_rate(world, args.steps, t_e2e), "unit": UNIT, "h2d_bytes_per_step": 8 * n, "d2h_bytes_per_step": 8 * n + 8,
           "path": "tad_newton_solve (C ABI), one call per Newton iteration with pinned host x copied in and out every "
                   "call; W untimed warm-up calls from the initial state, then the K timed calls (iterations W+1..W+K, "
                   "as the timed region)"}

    # kernel figures at the final state (CUDA events on the library stream)
    prof = fn.profile_kernels(x.data_ptr(), reps=5)
    nb = fn.hessian_pattern()[1].size // (w.var_dim ** 2)
    vb = 4 if prec == tad.PREC_MIXED else 8
    # fused SpMV: H blocks + column ids + row pointers + z gathered once + Ap, p read and written
    spmv_bytes = nb * (w.var_dim ** 2 * vb + 4) + (w.n_handles + 1) * 4 + 5 * n * vb
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    hbm = float(peaks.get("hbm_gbs", 6800.0))
    hbm_src = "measured" if "hbm_gbs" in peaks else "fallback"
    spmv_gbs = spmv_bytes / (prof["spmv"] * 1e-3) / 1e9
    # element Hessians (K1 + K2, all terms) per second of their own kernel time
    elem_hess_per_s = world * w.n_elements / (prof["elem_hessian"] / 1e3)
    # K6 runs only for trials the speculative first trial did not cover: its
    # launches are in the launch list, not estimated here
    share = {"spmv": stage["pcg_iters"] * prof["spmv"] / ms, "pcg_update": stage["pcg_iters"] * prof["pcg_update"] / ms,
             "elem_hessian": args.steps * prof["elem_hessian"] / ms, "assemble": args.steps * prof["assemble"] / ms}
    traffic = TRAFFIC_FROM_CAPTURE.get((args.workload, args.precision), {})
    timing_note = "CUDA events around a captured CUDA graph of the kernel's launches, as the solver runs them"
    spmv_name = ("k_pcg_spmv_sell (sliced-ELL SpMV + p update + p.Ap)" if w.var_dim == 3
                 else "k_pcg_spmv_fused (BSR SpMV + p update + p.Ap)")
    roof_spmv = {"bound": "hbm", "kernel": spmv_name, "achieved": spmv_gbs, "timing": timing_note,
                 "peak": hbm, "unit": "GB/s", "frac": spmv_gbs / hbm, "traffic": traffic.get("spmv"),
                 "traffic_source": TRAFFIC_SOURCE if traffic.get("spmv") else None,
                 "peak_source": f"{hbm_src} copy bandwidth (MEASURED_PEAKS.json hbm_gbs)",
                 "algorithmic_bytes_per_launch": spmv_bytes, "ms_per_launch": prof["spmv"]}
    fp_peak = tad.measure_fma_peak(prec)
    k_elem = w.var_dim * w.terms[0].valence
    elem_flops = ELEM_FLOPS.get(k_elem, 0) * w.terms[0].handles.shape[0]
    elem_tf = elem_flops / (prof["elem_hessian"] * 1e-3) / 1e12
    elem_name = ("k_elem_grad_lanes + k_elem_hess_lanes + k_project_blocks (lane-split Double<k> evaluation + "
                 "PSD projection)" if (k_elem == 12 and prec == tad.PREC_MIXED)
                 else "k_elem_hessian + k_project_blocks (Double<k> evaluation + PSD projection)")
    roof_elem = {"bound": "fp32 CUDA-core pipe" if prec == tad.PREC_MIXED else "fp64 CUDA-core pipe",
                 "kernel": elem_name, "achieved": elem_tf, "timing": timing_note,
                 "peak": fp_peak, "unit": "TFLOP/s", "frac": elem_tf / fp_peak, "traffic": traffic.get("elem"),
                 "traffic_unit": "bytes per launch", "traffic_source": TRAFFIC_SOURCE if traffic.get("elem") else None,
                 "flops_source": "op counting of the library's arithmetic (oracle/flop_count.sh), not a counter",
                 "peak_source": "measured FMA throughput (tad_measure_fma_peak, this GPU)",
                 "algorithmic_flops_per_launch": elem_flops,
                 "flops_per_element": ELEM_FLOPS.get(k_elem, 0), "ms_per_launch": prof["elem_hessian"]}
    roofline = dict(roof_elem if share["elem_hessian"] >= share["spmv"] else roof_spmv)
    roofline["share_of_timed_region_est"] = share
    kernels = {k: round(v, 5) for k, v in prof.items()}

    # FP64 plain path on the same workload (the drop-in), same protocol
    fp64 = None
    if not args.no_fp64 and prec == tad.PREC_MIXED:
        fd = make_fn(tad.PREC_FP64)
        xd = torch.from_numpy(w.x0.copy()).cuda()
        fd.newton_solve_device(xd.data_ptr(), args.warmup)
        torch.cuda.synchronize()
        sd = torch.cuda.ExternalStream(fd.stream_ptr)
        a0, a1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        st64 = {"ms_eval": 0.0, "ms_assemble": 0.0, "pcg_iters": 0}
        a0.record(sd)
        fd.newton_solve_device(xd.data_ptr(), args.steps)
        a1.record(sd)
        torch.cuda.synchronize()
        s2 = fd.last_solve_stats()
        for k in st64:
            st64[k] += s2[k]
        t64 = a0.elapsed_time(a1) / 1e3
        prof64 = fd.profile_kernels(xd.data_ptr(), reps=2)
        fp64 = {"value": args.steps / t64, "unit": UNIT, "steps": args.steps,
                "element_hessians_per_s": w.n_elements / (prof64["elem_hessian"] / 1e3),
                "pcg_iters_per_step": st64["pcg_iters"] / args.steps,
                "kernels_ms": {k: round(v, 5) for k, v in prof64.items()},
                "fp64_fma_peak_tflops": tad.measure_fma_peak(tad.PREC_FP64)}
        del fd

    # solve to 1e-8 energy error: mixed and FP64 from the initial state until the
    # energy is within 1e-8 of the converged FP64 energy
    solve = None
    if not args.no_fp64 and prec == tad.PREC_MIXED and rank == 0:
        def run_to_convergence(p, max_iter=200, max_s=40.0):
            f_ = make_fn(p)
            xx = torch.from_numpy(w.x0.copy()).cuda()
            hist = []
            t_start = time.perf_counter()
            while len(hist) < max_iter and time.perf_counter() - t_start < max_s:
                fh_ = f_.newton_solve_device(xx.data_ptr(), 1)
                torch.cuda.synchronize()
                hist.append((time.perf_counter() - t_start, float(fh_[-1])))
                if len(hist) > 3 and abs(hist[-1][1] - hist[-3][1]) <= 1e-12 * abs(hist[-1][1]):
                    break
            return hist
        h64 = run_to_convergence(tad.PREC_FP64)
        hmx = run_to_convergence(tad.PREC_MIXED)
        fstar = min(h64[-1][1], hmx[-1][1])

        def reach(hist):
            for i, (t_, f_) in enumerate(hist):
                if f_ <= fstar * (1 + 1e-8):
                    return {"iters": i + 1, "seconds": t_}
            return None
        solve = {"f_converged_fp64": h64[-1][1], "f_converged_mixed": hmx[-1][1],
                 "final_energy_rel_err_mixed_vs_fp64": abs(hmx[-1][1] - h64[-1][1]) / abs(h64[-1][1]),
                 "to_1e-8_fp64": reach(h64), "to_1e-8_mixed": reach(hmx)}
        # error of the mixed path against FP64 at the post-warm-up state: f, g
        # and H of the evaluation, and the Newton step of the timed
        # configuration (PCG to 1e-2) in both precisions
        xw = x_warm.cpu().numpy()
        e64 = tad.ScalarFunction.from_workload(w, precision=tad.PREC_FP64, **settings)
        emx = tad.ScalarFunction.from_workload(w, precision=tad.PREC_MIXED, **settings)
        f64, g64, H64 = e64.eval_with_hessian_proj(xw)
        fmx, gmx, Hmx = emx.eval_with_hessian_proj(xw)
        d64, _, _ = e64.newton_direction(xw)
        dmx, _, _ = emx.newton_direction(xw)
        solve["errors_mixed_vs_fp64_at_step_W"] = {
            "f": abs(fmx - f64) / abs(f64),
            "g": float(np.linalg.norm(gmx - g64) / np.linalg.norm(g64)),
            "H_frobenius": float(np.linalg.norm((Hmx - H64).data) / np.linalg.norm(H64.data)),
            "newton_step_pcg_1e-2": float(np.linalg.norm(dmx - d64) / np.linalg.norm(d64)),
            "predicted_decrease_g_dot_d": float(abs(g64 @ dmx - g64 @ d64) / abs(g64 @ d64))}
        del e64, emx
        if w.name.startswith("disk"):
            # a tight (1e-10) Newton step on a well-posed problem: the same family
            # with two pinned boundary vertices (no rigid null space), near its
            # minimiser; on the unconstrained mesh a tight step is dominated by the
            # eps-regularised rigid motions and is arbitrary in any precision
            from tinyad_gb300 import meshes
            wp = meshes.disk_param_pinned(128, seed=6)
            xs, _ = tad.solve_minimiser(wp, wp.x0)
            xp = xs + np.random.default_rng(8).normal(scale=1e-4, size=xs.size)
            tight = dict(pcg_rel_tol=1e-10, pcg_max_iters=20000, refine_max_iters=8, refine_rel_tol=1e-10)
            p64 = tad.ScalarFunction.from_workload(wp, precision=tad.PREC_FP64, **tight)
            pmx = tad.ScalarFunction.from_workload(wp, precision=tad.PREC_MIXED, **tight)
            d64, _, _ = p64.newton_direction(xp)
            dmx, _, _ = pmx.newton_direction(xp)
            solve["errors_mixed_vs_fp64_tight_step"] = {
                "workload": f"disk128_pinned ({wp.n_elements} faces), minimiser + 1e-4 noise, PCG to 1e-10",
                "newton_step": float(np.linalg.norm(dmx - d64) / np.linalg.norm(d64))}
            del p64, pmx

    cpu = None
    if not args.no_cpu and rank == 0 and world == 1:
        cpu = cpu_baseline(w)

    # the other configurations of the benchmark, summarised (single GPU only)
    configs = None
    if not args.no_extra and world == 1 and rank == 0 and args.workload == "disk1024":
        del fn
        torch.cuda.empty_cache()
        configs = {}
        for key, job in (("tet48", lambda: measure_newton(args, "tet48")),
                         ("adjoint254", lambda: summary_adjoint(measure_adjoint(args))),
                         ("batch256", lambda: summary_batch(measure_batch(args, rank, 256, sequential=False)))):
            t0 = time.perf_counter()
            try:
                configs[key] = job()
            except Exception as e:   # a failed summary must not lose the headline line
                configs[key] = {"error": f"{type(e).__name__}: {e}"}
            configs[key]["wall_s"] = round(time.perf_counter() - t0, 1)
            torch.cuda.empty_cache()

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 Hessian/PCG + f64 value/gradient" if prec == tad.PREC_MIXED else "f64",
        "data": "synthetic (seeded generator)",
        "config": {"workload": workload_desc(w), "precision": args.precision,
                   "n_vars": n, "n_elements": w.n_elements, "hessian_nnz": int(nb * w.var_dim ** 2),
                   "newton": "projected Newton, eps=1e-9, block-Jacobi PCG to 1e-2 relative residual (<= 2000 "
                             "iterations), Armijo line search (0.8, 1e-4, 64); steps W+1..W+K from the initial state",
                   "parallelism": f"replicas x{world}" if world > 1 else "single GPU",
                   "l2": "inputs larger than L2: per-step working set (element blocks 157 MB, BSR Hessian, vectors) > 126 MB",
                   "mesh_generation_s": round(t_gen, 2)},
        "element_hessians_per_s": elem_hess_per_s,
        "stages_ms_per_step": {k: v / args.steps for k, v in stage.items()},
        "stages_note": "an accepted speculative first trial evaluates and assembles the next iteration's derivatives "
                       "inside the line-search stage (ms_linesearch); ms_eval / ms_assemble then count only iterations "
                       "that evaluate at their start",
        "kernels_ms_per_launch": kernels,
        "fp_pipe_peak_tflops": fp_peak,
        "f_history": [float(v) for v in fh],
        "roofline": roofline,
        "roofline_spmv": roof_spmv,
        "roofline_elem": roof_elem,
        "e2e": e2e,
        "fp64_path": fp64,
        "mixed_vs_fp64_iters_per_s": (value / fp64["value"]) if fp64 else None,
        "time_to_1e-8_energy": ({"mixed": solve["to_1e-8_mixed"], "fp64": solve["to_1e-8_fp64"],
                                 "note": "Newton iterations and seconds from the initial state until the energy is "
                                         "within 1e-8 of the converged energy, one solver call per iteration"}
                                if solve else None),
        "solve": solve,
        "configs": configs,
        "cpu_baseline": cpu,
        "clocks": clk.summary(),
        "gpu_launches": int(launches),
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
