#!/usr/bin/env python3
"""Benchmark of the 7-point fp32 diffusion sweep at 512^3 on one GB300.

Workload (the reference's diffusion benchmark, examples/diffusion-benchmark,
at 512^3): f_new = cc*c + cw*w + ce*e + cs*s + cn*n + cb*b + ct*t with
cc=0.4 and the six neighbour weights 0.1, neighbours clamped at the faces,
double-buffered (two PSStencilMaps, g1->g2 and g2->g1).  One bench step is one
time step: one sweep over all 512^3 cells.  Inputs: uniform[0,1) from the
SplitMix64 stream, seed 1.

Printed JSON line (one, rank 0):
  value      GLUPS (giga lattice-site updates per second) with the grids
             resident in HBM, timed with CUDA events on the runtime's stream;
  e2e        the same metric for one whole job through the public C API with
             host buffers: PSGridCopyin (pinned host -> device), PSStencilRun of
             K steps, PSGridCopyout (device -> pinned host);
  roofline   achieved HBM GB/s of the sweep kernel (8 algorithmic bytes per
             cell update: one fp32 read, one fp32 write) against the measured
             copy bandwidth in MEASURED_PEAKS.json;
  cpu_baseline  the CPU restatement of the REF target (oracle/) on the host
             cores, OpenMP over z, on a bounded sample of the same workload.

Further keys of the same line (leave them out with --no-extras), each with
its own CUDA-event timing, roofline and CPU baseline:
  himeno     19-point Himeno Jacobi at 257x257x513 with the fused
             residual, max(K, 50) sweeps, 56 algorithmic bytes per interior
             cell update;
  batch      48 uneven grids (half diffusion, half Himeno), 200
             steps each, batched against 48 separate runs;
  diffusion64  64^3 x 100 steps + PSReduce sum (the REF program's
             configuration), device and end to end;
  reduce     PSReduce over a 512^3 float grid, GB/s.

--impl reference times only the CPU implementation (the reference's REF
target restated in C, all host threads) on the same metric: each step one
sweep of the whole 512^3 field.
Multi-GPU (torchrun): independent replicas, one per GPU (the path has no
data exchange); value is the sum over ranks.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N = 512
COEF = (0.1, 0.1, 0.1, 0.1, 0.1, 0.1, 0.4)  # ce cw cn cs ct cb cc
BYTES_PER_LUP = 8
METRIC = "GLUPS, 7-point fp32 diffusion 512^3 (clamped, double-buffered)"
WORKLOAD = "7-point fp32 diffusion 512x512x512, clamped, cc=0.4 others 0.1"


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Dist:
    """Barrier and max/sum over ranks (gloo on CPU tensors) for replicas."""

    def __init__(self):
        self.ws, self.rank, self.local = dist_env()
        self.pg = None
        if self.ws > 1:
            import torch.distributed as td
            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            td.init_process_group("gloo")
            self.td = td

    def barrier(self):
        if self.ws > 1:
            self.td.barrier()

    def reduce(self, v, op):
        if self.ws == 1:
            return v
        import torch
        t = torch.tensor([float(v)], dtype=torch.float64)
        self.td.all_reduce(t, op=getattr(self.td.ReduceOp, op))
        return float(t.item())

    def close(self):
        if self.ws > 1:
            self.td.destroy_process_group()


class ClockSampler:
    """nvidia-smi clock / throttle sampling around the timed region.

    start() returns once the first sample has arrived, and stop() waits for
    one sample taken after it was called, so even a timed region shorter
    than the 100 ms sampling period is bracketed by samples under load."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self, wait=3.0):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
            return
        t0 = time.perf_counter()
        while not self.lines and time.perf_counter() - t0 < wait:
            time.sleep(0.005)

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append((time.perf_counter(), line.strip()))

    def stop(self, wait=1.0):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no nvidia-smi"]}
        t_stop = time.perf_counter()
        while (not self.lines or self.lines[-1][0] < t_stop) and \
                time.perf_counter() - t_stop < wait:
            time.sleep(0.005)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.t.join(timeout=2)
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown",
                 "sw_power_cap"]
        for _, line in self.lines:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm),
                "window": "from before the warm-up to the first sample after the timed region"}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profiled_traffic(name="diffusion7_512.md"):
    """dram bytes (read + write) of one launch of a kernel at the bench's
    full size, from the committed ncu summary of that capture
    (profiles/<name>, line `traffic_bytes_per_launch:`)."""
    p = os.path.join(ROOT, "profiles", name)
    if not os.path.exists(p):
        return None
    for line in open(p):
        if line.startswith("traffic_bytes_per_launch:"):
            try:
                return float(line.split(":", 1)[1].split()[0])
            except ValueError:
                return None
    return None


# ---------------------------------------------------------------------------
# CPU legs (the oracle is the checker and the CPU baseline only)
# ---------------------------------------------------------------------------

def host_threads():
    """Host cores this process may use.  torchrun sets OMP_NUM_THREADS=1 for
    its ranks; the CPU legs (rank 0 alone) take every core regardless."""
    try:
        return len(os.sched_getaffinity(0))
    except (AttributeError, OSError):
        return os.cpu_count() or 1


def cpu_sweeps(seconds, nthreads=0, zslab=None):
    """Times oracle sweeps of the 512^3 workload on host cores until about
    `seconds` have elapsed.  With zslab, each sweep covers z in [0, zslab)
    of the full grid (a bounded sample).  Returns (glups, sweeps, threads)."""
    from oracle import pyoracle
    from physis_gb300 import synth
    nt = nthreads if nthreads > 0 else host_threads()
    f1 = synth.uniform((N, N, N), 1)
    f2 = np.zeros_like(f1)
    zs = zslab or N
    dom = (0, N, 0, N, 0, zs)
    pyoracle.sweep7(pyoracle.V_DIFFUSION7, f1, f2, dom, COEF, nthreads=nt)
    t0 = time.perf_counter()
    sweeps = 0
    while True:
        pyoracle.sweep7(pyoracle.V_DIFFUSION7, f1, f2, dom, COEF, nthreads=nt)
        f1, f2 = f2, f1
        sweeps += 1
        el = time.perf_counter() - t0
        if el >= seconds:
            break
    return N * N * zs * sweeps / el / 1e9, sweeps, nt


def run_reference(args, dist):
    if dist.rank != 0:
        return
    from oracle import pyoracle
    from physis_gb300 import synth
    nt = host_threads()
    f1 = synth.uniform((N, N, N), 1)
    f2 = np.zeros_like(f1)
    dom = (0, N, 0, N, 0, N)
    for _ in range(args.warmup):
        pyoracle.sweep7(pyoracle.V_DIFFUSION7, f1, f2, dom, COEF, nthreads=nt)
        f1, f2 = f2, f1
    t0 = time.perf_counter()
    for _ in range(args.steps):
        pyoracle.sweep7(pyoracle.V_DIFFUSION7, f1, f2, dom, COEF, nthreads=nt)
        f1, f2 = f2, f1
    el = time.perf_counter() - t0
    value = float(N) ** 3 * args.steps / el / 1e9
    sample = (f"one step = one REF-order sweep of the whole {N}^3 field "
              f"({N ** 3} cells), OpenMP over z")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "GLUPS",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": el / args.steps * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic uniform[0,1) seed 1 (SplitMix64)",
        "config": {"workload": WORKLOAD, "grid": [N, N, N],
                   "implementation": "oracle/ps_oracle.c: C restatement of the "
                   "Physis REF target (the reference's REF runtime needs Boost and "
                   "its translator; neither builds here)"},
        "cpu_baseline": {"value": value, "unit": "GLUPS", "cores": nt,
                         "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": "GLUPS", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# The reference's own hand-written CUDA diffusion kernels, on the same GPU
# ---------------------------------------------------------------------------

# (label, cubin, mangled name, block, grid(n), dynamic smem, steps per launch):
# launch geometry of examples/diffusion-benchmark/diffusion3d_cuda.cu:322-333,
# diffusion3d_cuda_shared.cu:110-121 and diffusion3d_cuda_temporal_blocking.cu:
# 289-309 (block sizes diffusion3d_cuda.h:15, 50-51 and
# diffusion3d_cuda_temporal_blocking.h:16-17).
REF_CUDA = [
    ("diffusion_kernel (thread per x,y column, block 64x4; the translator's "
     "CUDA target has this shape)", "diffusion3d_cuda.cubin",
     "_ZN11diffusion3d16diffusion_kernelEPfS0_iiifffffff", (64, 4, 1),
     lambda n: (n // 64, n // 4, 1), 0, 1),
    ("diffusion_kernel_shared (2.5D shared memory, block 128x2)",
     "diffusion3d_cuda_shared.cubin",
     "_ZN11diffusion3d23diffusion_kernel_sharedEPfS0_iiifffffff", (128, 2, 1),
     lambda n: (n // 128, n // 2, 1), 0, 1),
    ("diffusion_kernel_temporal_blocking2 (2 steps per launch, block 32x16)",
     "diffusion3d_cuda_temporal_blocking.cubin",
     "_ZN11diffusion3d35diffusion_kernel_temporal_blocking2EPfS0_iiifffffff",
     (32, 16, 1), lambda n: ((n + 29) // 30, (n + 13) // 14, 1), 3 * 32 * 16 * 4, 2),
]


def reference_cuda_kernels(ps, g1, g2, steps):
    """Times the reference's hand-written CUDA diffusion kernels, compiled
    from its sources for sm_103a (oracle/Makefile, cubins in oracle/_ref/),
    on the same 512^3 grids and stream.  GLUPS per kernel, or why not."""
    import ctypes
    L = ps.lib()
    n = N
    if ps.lib().PSGridPitch(g1.handle) != n * 4:
        return {"unavailable": "needs dense rows (pitch == nx*4)"}
    try:
        cu = ctypes.CDLL("libcuda.so.1")
    except OSError as e:
        return {"unavailable": f"libcuda.so.1: {e}"}
    cu.cuInit(0)
    out = {}
    ptrs = [ctypes.c_void_p(L.PSGridDevicePtr(g1.handle)),
            ctypes.c_void_p(L.PSGridDevicePtr(g2.handle))]
    stream = ctypes.c_void_p(L.PSGetStream())
    for label, cubin, sym, block, gridf, smem, per in REF_CUDA:
        path = os.path.join(ROOT, "oracle", "_ref", cubin)
        if not os.path.exists(path):
            out[label] = "unavailable: cubin not built (needs the reference tree)"
            continue
        mod, fn = ctypes.c_void_p(), ctypes.c_void_p()
        if cu.cuModuleLoad(ctypes.byref(mod), path.encode()) != 0 or \
                cu.cuModuleGetFunction(ctypes.byref(fn), mod, sym.encode()) != 0:
            out[label] = "unavailable: cuModuleLoad/GetFunction failed"
            continue
        grid = gridf(n)
        coefs = [ctypes.c_float(c) for c in COEF]  # ce cw cn cs ct cb cc

        def launch(i):
            a = [ptrs[i % 2], ptrs[(i + 1) % 2], ctypes.c_int(n), ctypes.c_int(n),
                 ctypes.c_int(n)] + coefs
            params = (ctypes.c_void_p * len(a))(
                *[ctypes.cast(ctypes.pointer(x), ctypes.c_void_p) for x in a])
            return cu.cuLaunchKernel(fn, grid[0], grid[1], grid[2], block[0], block[1],
                                     block[2], smem, stream, params, None)

        count = max(1, steps // per)
        rc = 0
        for i in range(3):
            rc |= launch(i)
        L.PSEventRecord(4)
        for i in range(count):
            rc |= launch(i)
        L.PSEventRecord(5)
        ms = L.PSEventElapsedMs(4, 5)
        cu.cuModuleUnload(mod)
        if rc != 0:
            out[label] = f"unavailable: cuLaunchKernel returned {rc}"
            continue
        out[label] = {"glups": float(n) ** 3 * count * per / (ms / 1e3) / 1e9,
                      "ms_per_step": ms / (count * per)}
    return out


# ---------------------------------------------------------------------------
# GPU leg
# ---------------------------------------------------------------------------

def run_gpu(args, dist):
    os.environ.setdefault("PS_DEVICE", str(dist.local))
    import physis_gb300 as ps
    from physis_gb300 import synth
    ps.init()
    L = ps.lib()
    shape = (N, N, N)
    init = synth.uniform(shape, 1)
    g1, g2 = ps.Grid(shape), ps.Grid(shape)
    g1.copyin(init)
    g2.copyin(init)
    dom = ps.full_domain(shape)
    if args.warps or args.rows or args.ns or args.ctas:
        ps.set_launch_shape(ps.PS_KERNEL_DIFFUSION7, warps=args.warps,
                            rows=args.rows, ns=args.ns, ctas_per_sm=args.ctas)
    if args.temporal > 1:
        tw, tr, tn = (int(v) for v in args.tshape.split(","))
        ps.set_temporal(ps.PS_KERNEL_DIFFUSION7, args.temporal, warps=tw, rows=tr, ns=tn)
    if args.fma:
        ps.set_fma(True)
    m1 = ps.stencil_map(ps.PS_KERNEL_DIFFUSION7, dom, [g1, g2], COEF)
    m2 = ps.stencil_map(ps.PS_KERNEL_DIFFUSION7, dom, [g2, g1], COEF)
    K, W = args.steps, args.warmup

    def steps(k):
        # k single-map steps, alternating direction (PSStencilRun per map)
        pairs, rem = divmod(k, 2)
        if pairs:
            ps.stencil_run([m1, m2], pairs)
        if rem:
            ps.stencil_run([m1], 1)

    clocks = ClockSampler(dist.local)
    clocks.start()
    attempt = 0
    while True:
        steps(W)
        ps.synchronize()
        dist.barrier()
        n0 = ps.launch_count()
        L.PSEventRecord(0)
        steps(K)
        L.PSEventRecord(1)
        ps.synchronize()
        ms = L.PSEventElapsedMs(0, 1)
        launches = ps.launch_count() - n0
        dist.barrier()
        clk = clocks.stop()
        bad = {"hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown"}
        if attempt == 0 and bad & set(clk.get("reasons", [])):
            attempt += 1
            clocks = ClockSampler(dist.local)
            clocks.start()
            continue
        break
    ps.check()
    ms_max = dist.reduce(ms, "MAX")
    cells = float(N) ** 3
    value = dist.ws * cells * K / (ms_max / 1e3) / 1e9

    # end to end through the public API with pinned host buffers
    import ctypes
    nbytes = N * N * N * 4
    hin = L.PSHostAlloc(nbytes)
    hout = L.PSHostAlloc(nbytes)
    ctypes.memmove(hin, init.ctypes.data, nbytes)
    dist.barrier()
    t0 = time.perf_counter()
    L.PSGridCopyin(g1.handle, hin)
    steps(K)
    L.PSGridCopyout(g1.handle if K % 2 == 0 else g2.handle, hout)
    e2e_s = time.perf_counter() - t0
    ps.check()
    e2e_max = dist.reduce(e2e_s, "MAX")
    e2e = dist.ws * cells * K / e2e_max / 1e9
    L.PSHostFree(hin)
    L.PSHostFree(hout)

    # the same run with temporal blocking: k = 2 steps per pass on a fixed
    # shape, then the autotuner's choice among plain shapes and temporal
    # depths (its trials run inside the warm-up, then K timed steps).  Both
    # bit-exact (no contraction: contracted passes drift past 1e-5 of REF
    # before the 1000 steps of this workload, so they are not reported).
    temporal = None
    if args.temporal == 1 and not args.no_extras:
        temporal = {"k": 2, "tshape": "8,4,3", "steps": K, "bit_exact": True}
        ps.set_temporal(ps.PS_KERNEL_DIFFUSION7, 2, warps=8, rows=4, ns=3)
        steps(W)
        ps.synchronize()
        dist.barrier()
        L.PSEventRecord(0)
        steps(K)
        L.PSEventRecord(1)
        ps.synchronize()
        tms = dist.reduce(L.PSEventElapsedMs(0, 1), "MAX")
        temporal["glups"] = dist.ws * cells * K / (tms / 1e3) / 1e9
        ps.set_temporal(ps.PS_KERNEL_DIFFUSION7, 1)
        ps.set_autotune(True)
        steps(max(W, 400))
        ps.synchronize()
        tuned, shape_t, k_t, tshape_t = ps.stencil_plan(m1)
        dist.barrier()
        L.PSEventRecord(0)
        steps(K)
        L.PSEventRecord(1)
        ps.synchronize()
        tms = dist.reduce(L.PSEventElapsedMs(0, 1), "MAX")
        temporal["autotuned"] = {"glups": dist.ws * cells * K / (tms / 1e3) / 1e9,
                                 "tuned": tuned, "k": k_t, "launch_shape": list(shape_t),
                                 "temporal_shape": list(tshape_t)}
        ps.set_autotune(False)
        ps.check()

    peak, peak_kind = measured_peaks()
    achieved = cells * BYTES_PER_LUP / (ms / K / 1e3) / 1e9
    traffic = profiled_traffic()
    ref_cuda = None
    if dist.rank == 0 and not args.no_cpu_baseline:
        ref_cuda = reference_cuda_kernels(ps, g1, g2, min(K, 200))
    shape_used = ps.get_launch_shape(ps.PS_KERNEL_DIFFUSION7)

    # the other headline configurations, each with its own CUDA-event timing,
    # roofline and CPU baseline (Himeno 257x257x513, 48 uneven grids, 64^3 x 100
    # steps, PSReduce over 512^3)
    extras = {}
    if not args.no_extras:
        with_cpu = dist.rank == 0 and not args.no_cpu_baseline
        hk = max(K, 50) + (max(K, 50) % 2)
        extras["himeno"] = himeno_measure(ps, dist, hk, W, args.cpu_seconds / 2, with_cpu)
        extras["batch"] = batch_measure(ps, dist, 200, False, args.cpu_seconds / 2, with_cpu)
        if dist.rank == 0:
            extras["diffusion64"] = diffusion64_measure(ps)
            extras["reduce"] = reduce_measure(ps, cpu=with_cpu)

    cpu = None
    if dist.rank == 0 and not args.no_cpu_baseline:
        glups, sweeps, nt = cpu_sweeps(args.cpu_seconds)
        cpu = {"value": glups, "unit": "GLUPS", "cores": nt, "kind": "port",
               "sample": f"{sweeps} REF-order sweeps of the full 512^3 field "
                         f"(oracle/ps_oracle.c, OpenMP over z, "
                         f"{args.cpu_seconds:.0f} s budget)"}
    if dist.rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "GLUPS",
            "n_gpus": dist.ws, "steps": K, "warmup": W,
            "ms_per_step": ms_max / K, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic uniform[0,1) seed 1 (SplitMix64)",
            "config": {
                "workload": WORKLOAD, "grid": [N, N, N],
                "parallelism": f"replicas{dist.ws}" if dist.ws > 1 else "single-gpu",
                "l2": "inputs larger than L2 (two 512 MiB grids vs 129 MB L2)",
                "launch_shape": {"warps": shape_used[0], "rows": shape_used[1],
                                 "ns": shape_used[2],
                                 "ctas_per_sm": shape_used[4] or "auto"},
                "e2e_job": "PSGridCopyin(pinned) + K steps + PSGridCopyout(pinned)",
                "temporal_k": args.temporal,
                "temporal_tshape": args.tshape if args.temporal > 1 else None,
                "fma": bool(args.fma),
            },
            "e2e": {"value": e2e, "unit": "GLUPS",
                    "h2d_bytes_per_step": nbytes / K,
                    "d2h_bytes_per_step": nbytes / K,
                    "job_seconds": e2e_max},
            "gpu_launches": int(launches),
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak,
                         "unit": "GB/s", "frac": achieved / peak,
                         "traffic": traffic, "peak_source": peak_kind,
                         "bytes_per_lup": BYTES_PER_LUP},
            "hbm_gbs_achieved": achieved,
            "clocks": clk,
            "cpu_baseline": cpu,
            "reference_cuda_kernels": ref_cuda,
            "temporal_blocking": temporal,
        }
        line.update(extras)
        print(json.dumps(line), flush=True)
    g1.free()
    g2.free()


# ---------------------------------------------------------------------------
# 64^3 x 100 steps + PSReduce, and the grid form of PSReduce
# ---------------------------------------------------------------------------

def diffusion64_measure(ps, reps=20):
    """64^3 clamped diffusion, seed 0, 100 steps (50 iterations of the two
    maps) and a PSReduce sum of the final grid, as the reference's REF
    program runs it.  Device: CUDA events around the 100 steps.  e2e: the
    whole job through the public API with pinned host buffers
    (PSGridCopyin + PSStencilRun + PSReduce + PSGridCopyout), wall clock,
    best of `reps`.  CPU: the REF port, sequential like the REF target."""
    import ctypes
    from oracle import pyoracle
    from physis_gb300 import synth
    L = ps.lib()
    n, steps = 64, 100
    shape = (n, n, n)
    init = synth.uniform(shape, 0)
    g1, g2 = ps.Grid(shape), ps.Grid(shape)
    dom = ps.full_domain(shape)
    m1 = ps.stencil_map(ps.PS_KERNEL_DIFFUSION7, dom, [g1, g2], COEF)
    m2 = ps.stencil_map(ps.PS_KERNEL_DIFFUSION7, dom, [g2, g1], COEF)
    nbytes = init.nbytes
    hin, hout = L.PSHostAlloc(nbytes), L.PSHostAlloc(nbytes)
    ctypes.memmove(hin, init.ctypes.data, nbytes)
    total = np.zeros(1, np.float32)

    def timed_jobs():
        dev_ms, job_s = [], []
        for r in range(reps + 3):
            L.PSGridCopyin(g1.handle, hin)
            ps.synchronize()
            L.PSEventRecord(0)
            ps.stencil_run([m1, m2], steps // 2)
            L.PSEventRecord(1)
            ps.synchronize()
            t0 = time.perf_counter()
            L.PSGridCopyin(g1.handle, hin)
            ps.stencil_run([m1, m2], steps // 2)
            L.PSReduceGridV(total.ctypes.data_as(ctypes.c_void_p), ps.PS_SUM, g1.handle)
            L.PSGridCopyout(g1.handle, hout)
            el = time.perf_counter() - t0
            if r >= 3:
                dev_ms.append(L.PSEventElapsedMs(0, 1))
                job_s.append(el)
        ps.check()
        out = np.empty_like(init)
        ctypes.memmove(out.ctypes.data, hout, nbytes)
        return float(np.median(dev_ms)), float(min(job_s)), out, float(total[0])

    dms, js, got, tsum = timed_jobs()
    # The same jobs with the library's autotuner on (PSSetAutotune): its trials
    # (launch shapes and bit-identical temporal depths) run in untimed jobs,
    # then the tuned plan is timed the same way.
    ps.set_autotune(True)
    for _ in range(3):
        L.PSGridCopyin(g1.handle, hin)
        ps.stencil_run([m1, m2], steps // 2)
    ps.synchronize()
    tuned, shape_t, k_t, tshape_t = ps.stencil_plan(m1)
    dms_t, js_t, got_t, tsum_t = timed_jobs()
    ps.set_autotune(False)
    total[0] = tsum
    L.PSHostFree(hin)
    L.PSHostFree(hout)
    g1.free()
    g2.free()
    # the oracle: bit-exact grid, FP64 sum; then its time, sequential
    r1, r2 = init.copy(), np.zeros_like(init)
    t0 = time.perf_counter()
    pyoracle.run7(pyoracle.V_DIFFUSION7, r1, r2, (0, n, 0, n, 0, n), COEF, iter=steps // 2)
    ref_sum = pyoracle.reduce_ref(r1, pyoracle.PS_SUM)
    cpu_s = time.perf_counter() - t0
    exact = pyoracle.reduce_fp64(r1, pyoracle.PS_SUM)
    cells = float(n) ** 3
    return {
        "workload": "7-point fp32 diffusion 64^3, seed 0, 100 steps + PSReduce sum "
                    "(the reference REF program's configuration)",
        "value": cells * steps / (dms / 1e3) / 1e9, "unit": "GLUPS",
        "us_per_step": dms / steps * 1e3,
        "steps": steps, "reps": reps,
        "e2e": {"value": cells * steps / js / 1e9, "unit": "GLUPS", "job_us": js * 1e6,
                "h2d_bytes_per_step": nbytes / steps, "d2h_bytes_per_step": (nbytes + 4) / steps,
                "what": "PSGridCopyin(pinned) + PSStencilRun(50 x 2 maps) + PSReduce + "
                        "PSGridCopyout(pinned), wall clock, best of reps"},
        "bit_exact_vs_oracle": bool(np.array_equal(got.view(np.uint32), r1.view(np.uint32))),
        "autotuned": {
            "value": cells * steps / (dms_t / 1e3) / 1e9, "unit": "GLUPS",
            "us_per_step": dms_t / steps * 1e3,
            "e2e": {"value": cells * steps / js_t / 1e9, "unit": "GLUPS", "job_us": js_t * 1e6},
            "plan": {"tuned": tuned, "temporal_k": k_t, "launch_shape": list(shape_t),
                     "temporal_shape": list(tshape_t)},
            "bit_exact_vs_oracle": bool(np.array_equal(got_t.view(np.uint32),
                                                       r1.view(np.uint32))),
            "sum_rel_err": abs(tsum_t - exact) / abs(exact),
            "what": "the same jobs after PSSetAutotune(1) tuned the run in untimed jobs"},
        "reduce": {"value": float(total[0]), "fp64_oracle": exact,
                   "rel_err": abs(float(total[0]) - exact) / abs(exact),
                   "ref_fold": float(ref_sum)},
        "roofline": {"bound": "launch/latency",
                     "what": "1 MiB grids stay in L2; 100 dependent sweeps of 262,144 cells"},
        "cpu_baseline": {"value": cells * steps / cpu_s / 1e9, "unit": "GLUPS", "cores": 1,
                         "kind": "port",
                         "sample": "the whole job (100 REF-order sweeps + REF PSReduce fold), "
                                   "sequential as the REF target runs it"},
    }


def reduce_measure(ps, reps=20, cpu=True):
    """PSReduce (grid form, PS_SUM) over a 512^3 float grid.  Device: the
    reduction kernel launched `reps` times back to back on the runtime
    stream (through PSReduceNoAlloc, which launches the same kernel with the
    same CTA count) between CUDA events: 4 algorithmic bytes per element.
    Call: wall clock of PSReduce itself (launch, 8-byte readback,
    synchronisation).  CPU: the REF fold (sequential, as the REF target)."""
    import ctypes
    from physis_gb300 import synth
    L = ps.lib()
    n = 512
    shape = (n, n, n)
    init = synth.uniform(shape, 3)
    g = ps.Grid(shape)
    g.copyin(init)
    slot = ps.Grid((1,), np.float64)
    stream = L.PSGetStream()
    for _ in range(3):
        L.PSReduceNoAlloc(g.dev_ptr, g.pitch, n, n, n, ps.PS_FLOAT, ps.PS_SUM, slot.dev_ptr,
                          stream)
    ps.synchronize()
    n0 = ps.launch_count()
    L.PSEventRecord(0)
    for _ in range(reps):
        L.PSReduceNoAlloc(g.dev_ptr, g.pitch, n, n, n, ps.PS_FLOAT, ps.PS_SUM, slot.dev_ptr,
                          stream)
    L.PSEventRecord(1)
    ps.synchronize()
    ms = L.PSEventElapsedMs(0, 1) / reps
    out = np.zeros(1, np.float32)
    calls = []
    for _ in range(reps):
        t0 = time.perf_counter()
        L.PSReduceGridV(out.ctypes.data_as(ctypes.c_void_p), ps.PS_SUM, g.handle)
        calls.append(time.perf_counter() - t0)
    ps.check()
    v64 = ps.reduce_f64(g, ps.PS_SUM)
    exact = float(init.astype(np.float64).sum())
    g.free()
    slot.free()
    peak, peak_kind = measured_peaks()
    nbytes = float(n) ** 3 * 4
    res = {
        "workload": "PSReduce PS_SUM over a 512^3 float grid (uniform[0,1), seed 3)",
        "value": nbytes / (ms / 1e3) / 1e9, "unit": "GB/s", "us_per_reduction": ms * 1e3,
        "call_us_median": float(np.median(calls)) * 1e6,
        "rel_err_vs_fp64": abs(v64 - exact) / exact,
        "roofline": {"bound": "hbm", "achieved": nbytes / (ms / 1e3) / 1e9, "peak": peak,
                     "unit": "GB/s", "frac": nbytes / (ms / 1e3) / 1e9 / peak,
                     "traffic": profiled_traffic("reduce_512.md"), "peak_source": peak_kind,
                     "bytes_per_element": 4},
        "l2": "512 MiB grid > L2",
        "cpu_baseline": None,
    }
    if cpu:
        from oracle import pyoracle
        t0 = time.perf_counter()
        pyoracle.reduce_ref(init, pyoracle.PS_SUM)
        el = time.perf_counter() - t0
        res["cpu_baseline"] = {"value": nbytes / el / 1e9, "unit": "GB/s", "cores": 1,
                               "kind": "port",
                               "sample": "one REF PSReduce fold of the whole grid "
                                         "(sequential, as the REF target)"}
    return res


# ---------------------------------------------------------------------------
# Himeno 19-point Jacobi with the fused residual, 257x257x513
# ---------------------------------------------------------------------------

HIM = (257, 257, 513)  # nx, ny, nz
HIM_BYTES_PER_LUP = 56
HIM_METRIC = ("GLUPS, Himeno 19-point Jacobi fp32 257x257x513 with the fused "
              "sum-of-squares residual per sweep")


def himeno_arrays(nx, ny, nz):
    """Set-up of himenobmtxpa_physis.c:126-141: p = k^2/(K-1)^2 (k = z),
    a0=a1=a2=1, a3=1/6, b*=0, c*=1, bnd 1 inside / 0 on the faces, wrk1=0,
    in the map's grid order p0 p1 a0 a1 a2 a3 b0 b1 b2 c0 c1 c2 bnd wrk1."""
    shape = (nz, ny, nx)
    z = np.arange(nz, dtype=np.int64)
    pz = (z * z).astype(np.float32) / np.float32((nz - 1) * (nz - 1))
    p0 = np.ascontiguousarray(np.broadcast_to(pz[:, None, None], shape))
    one = np.ones(shape, np.float32)
    zero = np.zeros(shape, np.float32)
    bnd = np.zeros(shape, np.float32)
    bnd[1:-1, 1:-1, 1:-1] = 1.0
    return [p0, p0.copy(), one, one, one, np.full(shape, np.float32(1.0 / 6.0)),
            zero, zero, zero, one, one, one, bnd, zero]


def himeno_measure(ps, dist, K, W, cpu_seconds, with_cpu):
    """Config 3: K fused-residual sweeps of the 257x257x513 Himeno set-up
    with resident grids (CUDA events on the runtime stream), one e2e job,
    and the REF port on host cores.  Returns the JSON object."""
    L = ps.lib()
    nx, ny, nz = HIM
    shape = (nz, ny, nx)
    arrays = himeno_arrays(nx, ny, nz)
    gs = [ps.Grid(shape) for _ in range(14)]
    for g, a in zip(gs, arrays):
        g.copyin(a)
    dom = ps.domain(1, nx - 1, 1, ny - 1, 1, nz - 1)
    omega = np.float32(0.8)
    k = ps.PS_KERNEL_HIMENO19_GOSA
    m1 = ps.stencil_map(k, dom, gs, [omega])
    m2 = ps.stencil_map(k, dom, [gs[1], gs[0]] + gs[2:], [omega])

    def sweeps(n):
        pairs, rem = divmod(n, 2)
        if pairs:
            ps.stencil_run([m1, m2], pairs)
        if rem:
            ps.stencil_run([m1], 1)

    clocks = ClockSampler(dist.local)
    clocks.start()
    sweeps(W)
    ps.synchronize()
    dist.barrier()
    n0 = ps.launch_count()
    L.PSEventRecord(0)
    sweeps(K)
    L.PSEventRecord(1)
    ps.synchronize()
    ms = L.PSEventElapsedMs(0, 1)
    launches = ps.launch_count() - n0
    dist.barrier()
    clk = clocks.stop()
    lups = float(nx - 2) * (ny - 2) * (nz - 2)
    ms_max = dist.reduce(ms, "MAX")
    value = dist.ws * lups * K / (ms_max / 1e3) / 1e9

    # end to end: copy p in (pinned), K sweeps each returning its residual to
    # the host through PSReduce's kernel form, copy p out (pinned)
    import ctypes
    nbytes = nx * ny * nz * 4
    hin = L.PSHostAlloc(nbytes)
    hout = L.PSHostAlloc(nbytes)
    ctypes.memmove(hin, arrays[0].ctypes.data, nbytes)
    dist.barrier()
    t0 = time.perf_counter()
    L.PSGridCopyin(gs[0].handle, hin)
    gosa = None
    for s_ in range(K):
        a, b = (gs[0], gs[1]) if s_ % 2 == 0 else (gs[1], gs[0])
        gosa = ps.reduce_kernel(ps.PS_SUM, k, dom, [a, b] + gs[2:], [omega])
    L.PSGridCopyout((gs[0] if K % 2 == 0 else gs[1]).handle, hout)
    e2e_s = time.perf_counter() - t0
    ps.check()
    e2e_max = dist.reduce(e2e_s, "MAX")
    L.PSHostFree(hin)
    L.PSHostFree(hout)

    peak, peak_kind = measured_peaks()
    achieved = lups * HIM_BYTES_PER_LUP / (ms / K / 1e3) / 1e9
    cpu = None
    if dist.rank == 0 and with_cpu:
        from oracle import pyoracle
        nt = host_threads()
        g = [a.copy() for a in arrays]
        zs = 64
        d = (1, nx - 1, 1, ny - 1, 1, zs + 1)
        pyoracle.himeno19(g, d, omega, nthreads=nt)
        t0 = time.perf_counter()
        n = 0
        while time.perf_counter() - t0 < cpu_seconds:
            pyoracle.himeno19(g, d, omega, nthreads=nt)
            g[0], g[1] = g[1], g[0]
            n += 1
        el = time.perf_counter() - t0
        cpu = {"value": (nx - 2) * (ny - 2) * zs * n / el / 1e9, "unit": "GLUPS",
               "cores": nt, "kind": "port",
               "sample": f"{n} REF-order sweeps (with the residual) of z in [1,{zs + 1}) "
                         f"(oracle/ps_oracle.c, OpenMP over z)"}
    shape_used = ps.get_launch_shape(k)
    out = {
        "metric": HIM_METRIC, "value": value, "unit": "GLUPS",
        "n_gpus": dist.ws, "steps": K, "warmup": W,
        "ms_per_step": ms_max / K, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "Himeno benchmark set-up (deterministic), omega 0.8",
        "config": {"workload": "Himeno 19-point Jacobi 257x257x513, interior "
                               "255x255x511, residual fused per sweep",
                   "grid": [nx, ny, nz], "l2": "14 grids of 139 MB, > L2",
                   "launch_shape": {"warps": shape_used[0], "ns": shape_used[2],
                                    "ns2": shape_used[3]},
                   "e2e_job": "PSGridCopyin(p) + K PSReduce kernel-form sweeps "
                              "(residual to host each) + PSGridCopyout(p)"},
        "e2e": {"value": dist.ws * lups * K / e2e_max / 1e9, "unit": "GLUPS",
                "h2d_bytes_per_step": nbytes / K,
                "d2h_bytes_per_step": nbytes / K + 4,
                "job_seconds": e2e_max, "last_gosa": float(gosa)},
        "gpu_launches": int(launches),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak,
                     "unit": "GB/s", "frac": achieved / peak,
                     "traffic": profiled_traffic("himeno19_traffic_257x257x513.md"),
                     "peak_source": peak_kind,
                     "bytes_per_lup": HIM_BYTES_PER_LUP},
        "clocks": clk,
        "cpu_baseline": cpu,
    }
    for g in gs:
        g.free()
    return out


def run_gpu_himeno(args, dist):
    os.environ.setdefault("PS_DEVICE", str(dist.local))
    import physis_gb300 as ps
    ps.init()
    out = himeno_measure(ps, dist, args.steps, args.warmup, args.cpu_seconds,
                         not args.no_cpu_baseline)
    if dist.rank == 0:
        print(json.dumps(out), flush=True)


# ---------------------------------------------------------------------------
# Batched uneven grids (48 problems)
# ---------------------------------------------------------------------------

def batch_dims(seed=2, n=48, xy=(32, 320), z=(32, 512)):
    """(nx, ny, nz) per problem: X, Y in xy, Z in z, rounded to multiples of
    8, from the SplitMix64 stream with the given seed."""
    from physis_gb300 import synth
    u = synth.uniform((n, 3), seed).astype(np.float64)
    dims = []
    for a, b, c in u:
        nx = int(round((xy[0] + a * (xy[1] - xy[0])) / 8)) * 8
        ny = int(round((xy[0] + b * (xy[1] - xy[0])) / 8)) * 8
        nz = int(round((z[0] + c * (z[1] - z[0])) / 8)) * 8
        dims.append((nx, ny, nz))
    return dims


def batch_measure(ps, dist, steps_per_problem, small, cpu_seconds, with_cpu):
    """Config 4: 48 uneven grids (24 diffusion, 24 Himeno) batched against
    the same work as 48 separate runs, both with resident grids, one e2e
    job, and the REF port on host cores over a bounded sample.  Returns the
    JSON object."""
    from physis_gb300 import synth
    L = ps.lib()
    if small:
        dims = batch_dims(xy=(16, 64), z=(16, 64))
        label = "48 small grids, X,Y,Z in [16,64] (multiples of 8)"
    else:
        dims = batch_dims()
        label = "48 grids, X,Y in [32,320], Z in [32,512] (multiples of 8)"
    runs, grids, inputs, host = [], [], [], []
    lups = 0.0
    algo_bytes = 0.0
    for i, (nx, ny, nz) in enumerate(dims):
        shape = (nz, ny, nx)
        init = synth.uniform(shape, 100 + i)
        if i % 2 == 0:  # 7-point diffusion
            g1, g2 = ps.Grid(shape), ps.Grid(shape)
            g1.copyin(init)
            dom = ps.full_domain(shape)
            runs.append([ps.stencil_map(ps.PS_KERNEL_DIFFUSION7, dom, [g1, g2], COEF),
                         ps.stencil_map(ps.PS_KERNEL_DIFFUSION7, dom, [g2, g1], COEF)])
            grids.append([g1, g2])
            inputs.append([(g1, init)])
            host.append(("diffusion", init))
            lups += float(nx) * ny * nz
            algo_bytes += 8.0 * nx * ny * nz
        else:  # Himeno 19-point, config-3 coefficients, p uniform
            arrays = himeno_arrays(nx, ny, nz)
            arrays[0] = init
            arrays[1] = init.copy()
            gs = [ps.Grid(shape) for _ in range(14)]
            for g, a in zip(gs, arrays):
                g.copyin(a)
            dom = ps.domain(1, nx - 1, 1, ny - 1, 1, nz - 1)
            runs.append([ps.stencil_map(ps.PS_KERNEL_HIMENO19, dom, gs, [0.8]),
                         ps.stencil_map(ps.PS_KERNEL_HIMENO19, dom,
                                        [gs[1], gs[0]] + gs[2:], [0.8])])
            grids.append(gs)
            inputs.append([(gs[0], init), (gs[1], init)])
            host.append(("himeno", arrays))
            n_in = float(nx - 2) * (ny - 2) * (nz - 2)
            lups += n_in
            algo_bytes += 56.0 * n_in
    it = max(1, steps_per_problem // 2)
    b = ps.batch_create(runs)
    ps.batch_run(b, 2)  # warm-up (also builds the graph cache on longer runs)
    ps.synchronize()
    clocks = ClockSampler(dist.local)
    clocks.start()
    n0 = ps.launch_count()
    L.PSEventRecord(0)
    ps.batch_run(b, it)
    L.PSEventRecord(1)
    ps.synchronize()
    ms_batch = L.PSEventElapsedMs(0, 1)
    launches = ps.launch_count() - n0
    clk = clocks.stop()
    # the same work as 48 separate runs, one after another on the same stream
    for r in runs:
        ps.stencil_run(r, 2)
    ps.synchronize()
    L.PSEventRecord(2)
    for r in runs:
        ps.stencil_run(r, it)
    L.PSEventRecord(3)
    ps.synchronize()
    ms_sep = L.PSEventElapsedMs(2, 3)
    steps = 2 * it
    value = lups * steps / (ms_batch / 1e3) / 1e9
    # end to end: copy every problem's input in (pinned), run, copy all out
    import ctypes
    pinned = []
    for lst in inputs:
        for g, a in lst:
            h = L.PSHostAlloc(a.nbytes)
            ctypes.memmove(h, a.ctypes.data, a.nbytes)
            pinned.append((g, h, a.nbytes))
    t0 = time.perf_counter()
    for g, h, _ in pinned:
        L.PSGridCopyinAsync(g.handle, h)
    ps.batch_run(b, it)
    for g, h, _ in pinned:
        L.PSGridCopyoutAsync(g.handle, h)
    ps.synchronize()
    e2e_s = time.perf_counter() - t0
    ps.check()
    nbytes = sum(n for _, _, n in pinned)
    for _, h, _ in pinned:
        L.PSHostFree(h)
    cpu = None
    if with_cpu and dist.rank == 0:
        # REF-order sweeps of the problems in batch order, one sweep each,
        # until the time budget is used (a bounded sample of the workload)
        from oracle import pyoracle
        nt = host_threads()
        done_lups, t0 = 0.0, time.perf_counter()
        n_sw = 0
        while time.perf_counter() - t0 < cpu_seconds:
            kind, a = host[n_sw % len(host)]
            if kind == "diffusion":
                nz, ny, nx = a.shape
                pyoracle.sweep7(pyoracle.V_DIFFUSION7, a, np.empty_like(a),
                                (0, nx, 0, ny, 0, nz), COEF, nthreads=nt)
                done_lups += float(a.size)
            else:
                nz, ny, nx = a[0].shape
                g = [x.copy() if j < 2 else x for j, x in enumerate(a)]
                pyoracle.himeno19(g, (1, nx - 1, 1, ny - 1, 1, nz - 1), np.float32(0.8),
                                  nthreads=nt)
                done_lups += float(nx - 2) * (ny - 2) * (nz - 2)
            n_sw += 1
        el = time.perf_counter() - t0
        cpu = {"value": done_lups / el / 1e9, "unit": "GLUPS", "cores": nt, "kind": "port",
               "sample": f"{n_sw} REF-order sweeps, one per problem in batch order "
                         f"(oracle/ps_oracle.c, OpenMP over z)"}
    peak, peak_kind = measured_peaks()
    achieved = algo_bytes * steps / (ms_batch / 1e3) / 1e9
    out = {
        "metric": "GLUPS, 48 uneven fp32 grids (24 x 7-point diffusion, 24 x Himeno "
                  "19-point) batched",
        "value": value, "unit": "GLUPS", "n_gpus": 1, "steps": steps, "warmup": 4,
        "ms_per_step": ms_batch / steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32",
        "data": "synthetic uniform[0,1) fields, dims from SplitMix64 seed 2",
        "config": {"workload": label,
                   "cells": lups, "separate_runs_glups": lups * steps / (ms_sep / 1e3) / 1e9,
                   "batch_over_separate": ms_sep / ms_batch,
                   "l2": "inputs larger than L2 (about 13 GB of grids)" if not small
                         else "fits L2"},
        "e2e": {"value": lups * steps / e2e_s / 1e9, "unit": "GLUPS",
                "h2d_bytes_per_step": nbytes / steps, "d2h_bytes_per_step": nbytes / steps},
        "gpu_launches": int(launches),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": None, "peak_source": peak_kind},
        "clocks": clk,
        "cpu_baseline": cpu,
    }
    ps.batch_free(b)
    for gs in grids:
        for g in gs:
            g.free()
    return out


def run_gpu_batch(args, dist):
    os.environ.setdefault("PS_DEVICE", str(dist.local))
    import physis_gb300 as ps
    ps.init()
    out = batch_measure(ps, dist, args.steps, args.batch_small, args.cpu_seconds,
                        not args.no_cpu_baseline)
    if dist.rank == 0:
        print(json.dumps(out), flush=True)


# ---------------------------------------------------------------------------
# Point-list stencils (27-point periodic sum; 7-point diffusion as points)
# ---------------------------------------------------------------------------

P27 = [(x, y, z) for z in (-1, 0, 1) for (x, y) in
       [(0, 0), (1, 0), (-1, 0), (0, 1), (1, 1), (-1, 1), (0, -1), (1, -1), (-1, -1)]]
P7 = [(0, 0, 0), (-1, 0, 0), (1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, -1), (0, 0, 1)]


# The clamped diffusion stencil in the reference's stencil language, the way
# examples/diffusion-benchmark/diffusion3d_physis.c:29-58 writes it
# (neighbours replaced by the centre at the faces; scalars in map order
# ce cw cn cs ct cb cc).
FN_DIFFUSION = r"""
void diffusion(const int x, const int y, const int z, PSGrid3DFloat g1, PSGrid3DFloat g2,
               float ce, float cw, float cn, float cs, float ct, float cb, float cc) {
  int nx = PSGridDim(g1, 0), ny = PSGridDim(g1, 1), nz = PSGridDim(g1, 2);
  float c = PSGridGet(g1, x, y, z);
  float w = (x == 0) ? c : PSGridGet(g1, x - 1, y, z);
  float e = (x == nx - 1) ? c : PSGridGet(g1, x + 1, y, z);
  float n = (y == 0) ? c : PSGridGet(g1, x, y - 1, z);
  float s = (y == ny - 1) ? c : PSGridGet(g1, x, y + 1, z);
  float b = (z == 0) ? c : PSGridGet(g1, x, y, z - 1);
  float t = (z == nz - 1) ? c : PSGridGet(g1, x, y, z + 1);
  PSGridEmit(g2, cc * c + cw * w + ce * e + cs * s + cn * n + cb * b + ct * t);
}
"""

# The 27-point sum of tests/system_tests/test_cases/test_27-pt.c: the 27
# terms added left to right in the test's order.
FN27 = r"""
void sum27(const int x, const int y, const int z, PSGrid3DFloat g1, PSGrid3DFloat g2) {
  const int dx[9] = {0, 1, -1, 0, 1, -1, 0, 1, -1};
  const int dy[9] = {0, 0, 0, 1, 1, 1, -1, -1, -1};
  float v = PSGridGet(g1, x, y, z - 1);
  for (int dz = -1; dz <= 1; ++dz)
    for (int i = (dz == -1) ? 1 : 0; i < 9; ++i)
      v = v + PSGridGet(g1, x + dx[i], y + dy[i], z + dz);
  PSGridEmit(g2, v);
}
"""


def run_gpu_points(args, dist):
    """K sweeps of a point stencil over an N^3 float grid, ping-pong.

    points27: the 27-point unit-weight periodic sum of
    tests/system_tests/test_cases/test_27-pt-periodic.c at N^3.
    points7: the clamped 7-point diffusion (cc=0.4, others 0.1) as a point
    stencil, to compare the generic kernel with the dedicated one.
    """
    os.environ.setdefault("PS_DEVICE", str(dist.local))
    import physis_gb300 as ps
    from physis_gb300 import synth
    ps.init()
    L = ps.lib()
    shape = (N, N, N)
    init = synth.uniform(shape, 1)
    g1, g2 = ps.Grid(shape), ps.Grid(shape)
    g1.copyin(init)
    g2.copyin(init)
    dom = ps.full_domain(shape)
    if args.workload == "points27":
        k = ps.point_stencil(P27, boundary=ps.BOUNDARY_NONE)
        dom = ps.domain(1, N - 1, 1, N - 1, 1, N - 1)
        label = f"27-point sum fp32 {N}^3 interior (point stencil)"
    elif args.workload == "points7":
        k = ps.point_stencil(P7, weights=[0.4] + [0.1] * 6, boundary=ps.BOUNDARY_CLAMP)
        label = f"7-point clamped diffusion fp32 {N}^3 as a point stencil"
    elif args.workload == "function27":
        k = ps.stencil_function(FN27, "sum27")
        dom = ps.domain(1, N - 1, 1, N - 1, 1, N - 1)
        label = f"27-point sum fp32 {N}^3 interior (compiled stencil function)"
    else:
        k = ps.stencil_function(FN_DIFFUSION, "diffusion")
        label = f"7-point clamped diffusion fp32 {N}^3 (compiled stencil function)"
    if (args.warps or args.rows) and args.workload.startswith("points"):
        ps.set_launch_shape(k, warps=args.warps, rows=args.rows)
    sc = list(COEF) if args.workload == "function7" else []
    m1 = ps.stencil_map(k, dom, [g1, g2], sc)
    m2 = ps.stencil_map(k, dom, [g2, g1], sc)
    K, W = args.steps, args.warmup

    def steps(n):
        pairs, rem = divmod(n, 2)
        if pairs:
            ps.stencil_run([m1, m2], pairs)
        if rem:
            ps.stencil_run([m1], 1)

    clocks = ClockSampler(dist.local)
    clocks.start()
    steps(W)
    ps.synchronize()
    dist.barrier()
    n0 = ps.launch_count()
    L.PSEventRecord(0)
    steps(K)
    L.PSEventRecord(1)
    ps.synchronize()
    ms = L.PSEventElapsedMs(0, 1)
    launches = ps.launch_count() - n0
    dist.barrier()
    clk = clocks.stop()
    ps.check()
    ms_max = dist.reduce(ms, "MAX")
    cells = float(N) ** 3 if not args.workload.endswith("27") else float(N - 2) ** 3
    value = dist.ws * cells * K / (ms_max / 1e3) / 1e9
    peak, peak_kind = measured_peaks()
    achieved = cells * BYTES_PER_LUP / (ms / K / 1e3) / 1e9
    if dist.rank == 0:
        line = {
            "metric": f"GLUPS, {label}", "value": value, "unit": "GLUPS",
            "n_gpus": dist.ws, "steps": K, "warmup": W, "ms_per_step": ms_max / K,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic uniform[0,1) seed 1 (SplitMix64)",
            "config": {"workload": label, "grid": [N, N, N],
                       "launch_shape": (list(ps.get_launch_shape(k)[:2])
                                        if args.workload.startswith("points")
                                        else ("64x4 threads, one per (x, y), z-chunked"
                                              if os.environ.get("PS_FUNCTION_TILED") == "0"
                                              else "64x16 tiles of 256 threads, z-chunked, "
                                                   "staged grids in shared memory")),
                       "l2": "inputs larger than L2" if N >= 256 else "fits L2"},
            "gpu_launches": int(launches),
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak,
                         "unit": "GB/s", "frac": achieved / peak, "traffic": None,
                         "peak_source": peak_kind, "bytes_per_lup": BYTES_PER_LUP},
            "clocks": clk,
        }
        print(json.dumps(line), flush=True)
    g1.free()
    g2.free()


# ---------------------------------------------------------------------------
# Learned warm start for the 19-point Jacobi solve
# ---------------------------------------------------------------------------

def measured_bf16_tflops():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        for k in ("bf16_tflops", "bf16_tflops_burst"):
            if k in d:
                return float(d[k]), "measured"
    return 1900.0, "fallback"


def run_gpu_warmstart(args, dist):
    """Train the warm-start network on solved instances, then time the
    held-out Jacobi solves to relative residual 1e-6 from zero, from the
    network's prediction, and from the prediction followed by learned
    restarts (prediction and restart time included)."""
    import torch
    import physis_gb300 as ps
    from physis_gb300 import warmstart as ws
    ps.init()
    if args.ws_full:
        # the specified 129 x 129 x 257 (x, y, z); 16^3 blocks give the network
        # the same 17 x 9 x 9 coarse grid as the reduced instances; 16
        # instances side by side in x keep the sweep's 128-wide tiles full
        shape, factor, nsx, per_stack, chunk = (257, 129, 129), 16, 16, 64, 2000
    else:
        shape, factor, nsx, per_stack, chunk = (args.ws_nz, args.ws_ny, args.ws_nx), 4, 15, 300, 256
    nu = args.ws_nu or 2 * factor * factor
    snapshots = ([int(v) for v in args.ws_snapshots.split(",") if v.strip()] or
                 [nu, 4 * nu, 16 * nu, 64 * nu])
    rng = np.random.default_rng(args.ws_seed)
    workers = min(16, os.cpu_count() or 1)
    t0 = time.perf_counter()
    data = ws.Dataset(rng, args.ws_train, shape, factor, nsx=nsx, per_stack=per_stack, tol=1e-7,
                      chunk=chunk, max_sweeps=args.ws_max_sweeps, workers=workers,
                      mirrors=args.ws_mirrors, snapshots=snapshots)
    data_s = time.perf_counter() - t0
    net = ws.Net(seed=1)
    per_epoch = max(1, data.x.shape[0] // 32)
    epochs = max(1, round(args.ws_steps / per_epoch))
    hist, train_s = ws.train(net, data, epochs=epochs, batch=32, lr=2e-3)

    held = ws.make_instances(rng, args.ws_held, shape, workers)
    st = ws.Stack(held, shape, nsx=min(nsx, args.ws_held))
    echunk = 500 if args.ws_full else 32
    stack_gb = 14 * 4 * float(np.prod(st.gshape)) / 1e9
    zeros = np.zeros(st.gshape, np.float32)

    def reset():
        st.grids[0].copyin(zeros)
        st.grids[1].copyin(zeros)

    scales = (data.wscale, data.pscale)
    pm = args.ws_predict_mirrors
    K = args.ws_restarts
    # Sweep counts, checked every `echunk` sweeps.  Float32 Jacobi has a
    # residual floor near 1e-7 * ||p|| / ||ss(0)||; instances whose floor lies
    # above 1e-6 never get there from any start and are left out of the
    # comparison (counted in the output).
    reset()
    zero = st.solve(1e-6, echunk, args.ws_max_sweeps)
    modes = {"single": 0}
    if K > 0:
        modes["restarts"] = K
    counts, r_start = {}, {}
    for name, k in modes.items():
        reset()
        used = ws.predict_into(net, st, scales, factor, pm, restarts=k, nu=nu,
                               restart_mirrors=args.ws_restart_mirrors,
                               pullback=args.ws_pullback)
        r_start[name] = st.residuals()
        c = st.solve(1e-6, echunk, args.ws_max_sweeps)
        counts[name] = np.where(c > 0, c + used, c)
    both = zero > 0
    for c in counts.values():
        both &= c > 0
    nz_sw = int(zero[both].max())
    final_sw = {name: int((counts[name][both] - modes[name] * nu).max()) for name in modes}

    def timed(k, n):
        reset()
        ps.synchronize()
        torch.cuda.synchronize()
        t = time.perf_counter()
        if k is not None:
            ws.predict_into(net, st, scales, factor, pm, restarts=k, nu=nu,
                            restart_mirrors=args.ws_restart_mirrors, pullback=args.ws_pullback)
        st.sweeps(n)
        ps.synchronize()
        return time.perf_counter() - t

    for _ in range(max(args.warmup, 3) // 3):  # warm-up of every path
        timed(None, 32)
        for k in modes.values():
            timed(k, 32)
    reps = 1 if args.ws_full else 2
    tz = min(timed(None, nz_sw) for _ in range(reps))
    ok_zero = int((st.residuals()[both] <= 1e-6).sum())
    secs, oks = {}, {}
    for name, k in modes.items():
        secs[name] = min(timed(k, final_sw[name]) for _ in range(reps))
        # instances at or below 1e-6 after the timed run (a few whose float32
        # floor lies just under 1e-6 can drift back above it between checks)
        oks[name] = int((st.residuals()[both] <= 1e-6).sum())

    # Ceiling of the coarse representation (--ws-ceiling): the held-out
    # instances solved on to 1e-7, their exact block-centre samples upsampled
    # as a perfect network output would be, and the sweeps to 1e-6 from there.
    ceiling = None
    if args.ws_ceiling:
        import ctypes
        reset()
        st.solve(1e-7, echunk * 8, args.ws_max_sweeps * 2)
        zc, yc, xc = ws.coarse_shape(shape, factor)
        exact = torch.empty(st.count * zc * yc * xc, dtype=torch.float32, device="cuda")
        fe = st.fields(factor, 1.0, 1.0, True)
        ws._ok(ps.lib().PSWarmStartPoolTarget(ctypes.byref(fe), ws._p(exact), None))
        for g in (st.grids[0], st.grids[1]):
            ws._ok(ps.lib().PSWarmStartUpsample(ctypes.byref(fe), ws._p(exact),
                                                ctypes.c_void_p(g.dev_ptr), None))
        ps.synchronize()
        best = st.solve(1e-6, echunk, args.ws_max_sweeps)
        ok = both & (best > 0)
        ceiling = {"sweeps_mean": float(best[ok].mean()),
                   "sweeps_ratio_mean": float(zero[ok].mean() / best[ok].mean()),
                   "what": "single-shot warm start from the exact solution's block-centre "
                           "samples"}

    # tensor roofline of the network's forward pass over the training set
    zc, yc, xc = data.dims1
    nvox = data.x.shape[0] * zc * yc * xc
    x = data.x.reshape(-1)
    net.forward(x, (data.x.shape[0], zc, yc, xc))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(5):
        net.forward(x, (data.x.shape[0], zc, yc, xc))
    torch.cuda.synchronize()
    fwd_ms = (time.perf_counter() - t0) / 5 * 1e3
    flops = 2.0 * 27 * 16 * 16 * nvox * ws.LAYERS
    peak, peak_kind = measured_bf16_tflops()
    tflops = flops / (fwd_ms / 1e3) / 1e12
    st.free()
    head = "restarts" if "restarts" in modes else "single"

    def mode_out(name):
        return {"sweeps_mean": float(counts[name][both].mean()),
                "sweeps_max": int(counts[name][both].max()),
                "seconds": secs[name], "speedup_wall": tz / secs[name],
                "sweeps_ratio_mean": float(zero[both].mean() / counts[name][both].mean()),
                "at_1e-6_after_timed_run": oks[name],
                "initial_residual_median": float(np.median(r_start[name])),
                "restarts": modes[name], "sweeps_per_restart": nu if modes[name] else 0,
                "pullback": args.ws_pullback if modes[name] else 0.0}

    line = {
        "metric": "Poisson time-to-1e-6 resid, learned vs plain (speed-up of the warm start)",
        "value": tz / secs[head], "unit": "x", "n_gpus": 1, "steps": args.ws_held,
        "warmup": max(args.warmup, 3), "ms_per_step": secs[head] / args.ws_held * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+bf16",
        "data": f"synthetic seeded instances (seed {args.ws_seed}), {args.ws_train} solved for training "
                f"(x {len(data.flips)} mirror images, + {len(snapshots)} solve iterates each "
                f"for the restarts), {args.ws_held} held out",
        "config": {"workload": f"learned warm start, 19-point Jacobi {shape[2]}x{shape[1]}x"
                               f"{shape[0]} (x,y,z" +
                               ("; the specified size)" if args.ws_full
                                else "; reduced from 129x129x257)"),
                   "pool_factor": factor, "sweep_count_resolution": echunk,
                   "network": f"pool {factor}^3 (9 channels) -> 6 conv 3x3x3 x16 (BF16, FP32 acc.) "
                              "-> Catmull-Rom",
                   "headline": head,
                   "epochs": epochs, "adam_steps": epochs * per_epoch, "batch": 32,
                   "mirror_images": len(data.flips), "training_snapshots": snapshots,
                   "prediction_mirror_images": len(ws.mirror_images(shape, pm)),
                   "l2": f"held-out stack: 14 arrays, {stack_gb:.1f} GB in all, > L2"},
        "compared_instances": int(both.sum()),
        "below_1e-6_unreachable": {"zero_start": int((zero <= 0).sum()),
                                   **{name: int((counts[name] <= 0).sum()) for name in modes}},
        "zero_start": {"sweeps_mean": float(zero[both].mean()), "sweeps_max": nz_sw,
                       "seconds": tz, "at_1e-6_after_timed_run": ok_zero},
        "warm_start": mode_out("single"),
        "warm_start_restarts": mode_out("restarts") if "restarts" in modes else None,
        "training": {"seconds": train_s, "loss_first_epoch": hist[0],
                     "loss_last_epoch": hist[-1]},
        "network_forward_ms": fwd_ms,
        "representation_ceiling": ceiling,
        "dataset": {"seconds": data_s, "solve_seconds": data.solve_seconds,
                    "target_sweeps_mean": float(data.sweeps.mean())},
        "roofline": {"bound": "tensor", "achieved": tflops, "peak": peak, "unit": "TFLOP/s",
                     "frac": tflops / peak, "traffic": None, "peak_source": peak_kind,
                     "what": "network forward over the training set (tcgen05 BF16 implicit GEMM)"},
        "gpu_launches": None,
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extras", action="store_true",
                    help="diffusion: leave out the temporal/himeno/batch/diffusion64/reduce "
                         "keys (the plain sweep alone, e.g. for a profiler)")
    ap.add_argument("--warps", type=int, default=0)
    ap.add_argument("--rows", type=int, default=0)
    ap.add_argument("--ns", type=int, default=0)
    ap.add_argument("--ctas", type=int, default=0)
    ap.add_argument("--n", type=int, default=512,
                    help="grid edge (default 512; smaller only for profiling)")
    ap.add_argument("--batch-small", action="store_true",
                    help="batch workload with 48 small grids (launch-bound regime)")
    ap.add_argument("--workload", default="diffusion",
                    choices=["diffusion", "himeno", "batch", "points27", "points7",
                             "function7", "function27", "warmstart", "reduce"],
                    help="diffusion: 7-point 512^3 (the headline); himeno: "
                         "19-point Jacobi 257x257x513 with fused residual")
    ap.add_argument("--temporal", type=int, default=1,
                    help="diffusion: temporal blocking depth k (1 = plain sweeps)")
    ap.add_argument("--tshape", default="8,4,3",
                    help="warps,rows,ring stages of the temporal passes")
    ap.add_argument("--fma", action="store_true",
                    help="diffusion: temporal passes contract multiply-adds "
                         "(PSSetFusedMultiplyAdd; results within 1e-5 of REF)")
    ap.add_argument("--ws-train", type=int, default=4096)
    ap.add_argument("--ws-held", type=int, default=256)
    ap.add_argument("--ws-steps", type=int, default=25600,
                    help="warm start: Adam steps (minibatches of 32) of training")
    ap.add_argument("--ws-mirrors", type=int, default=16,
                    help="warm start: training pairs per solved instance (its mirror images)")
    ap.add_argument("--ws-predict-mirrors", type=int, default=16,
                    help="warm start: mirror images whose predictions are averaged")
    ap.add_argument("--ws-ceiling", action="store_true",
                    help="warm start: also time the solve from the exact solution's "
                         "block-centre samples (the coarse representation's ceiling)")
    ap.add_argument("--ws-nx", type=int, default=33)
    ap.add_argument("--ws-ny", type=int, default=33)
    ap.add_argument("--ws-nz", type=int, default=65)
    ap.add_argument("--ws-max-sweeps", type=int, default=12000)
    ap.add_argument("--ws-restarts", type=int, default=4,
                    help="warm start: learned restarts after the prediction (0: single shot)")
    ap.add_argument("--ws-seed", type=int, default=5,
                    help="warm start: seed of the training and held-out instances")
    ap.add_argument("--ws-pullback", type=float, default=1e-4,
                    help="warm start: relative pull of the restarted iterate toward zero "
                         "(keeps float32 Jacobi out of 2-cycles near the tolerance)")
    ap.add_argument("--ws-restart-mirrors", type=int, default=16,
                    help="warm start: mirror images averaged in each restart's prediction")
    ap.add_argument("--ws-nu", type=int, default=0,
                    help="warm start: Jacobi sweeps before each learned restart (even; "
                         "0: 2 x pooling factor^2, i.e. 32 reduced, 512 at --ws-full)")
    ap.add_argument("--ws-snapshots", default="",
                    help="warm start: sweep counts of the target solves whose iterates "
                         "train the restarts (comma-separated, even; default: nu x 1, 4, "
                         "16, 64)")
    ap.add_argument("--ws-full", action="store_true",
                    help="warm start at 129x129x257 (use --ws-train/--ws-held "
                         "to size it, e.g. 128/32, and --ws-max-sweeps 100000)")
    args = ap.parse_args()
    global N
    N = args.n
    if args.warmup < 3:
        args.warmup = 3
    dist = Dist()
    try:
        if args.impl == "reference":
            run_reference(args, dist)
        elif args.workload == "himeno":
            run_gpu_himeno(args, dist)
        elif args.workload == "batch":
            run_gpu_batch(args, dist)
        elif args.workload == "warmstart":
            run_gpu_warmstart(args, dist)
        elif args.workload == "reduce":
            os.environ.setdefault("PS_DEVICE", str(dist.local))
            import physis_gb300 as ps
            ps.init()
            out = reduce_measure(ps, reps=max(args.steps, 3), cpu=not args.no_cpu_baseline)
            if dist.rank == 0:
                print(json.dumps(out), flush=True)
        elif args.workload in ("points27", "points7", "function7", "function27"):
            run_gpu_points(args, dist)
        else:
            run_gpu(args, dist)
    finally:
        dist.close()


if __name__ == "__main__":
    main()
