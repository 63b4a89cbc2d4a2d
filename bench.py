"""Benchmark of the QMCkl basis-evaluation path on GB300: MO vgl points/s.

A step is one evaluation of the hot path for one batch of points: touch the context (new
point set) and provide mo_vgl = AO vgl (fused kernel) + MO contraction, for the medium
workload (40 nuclei, 600 s/p/d/f shells -> 1188 AOs, 300 MOs, 256 walkers x 160 electrons
= 40960 points; seeded synthetic data). `value` is measured with the inputs resident in
HBM and timed with CUDA events on the library's stream; `e2e` is the same metric through
the C ABI with host buffers (points copied in, mo_vgl copied out every step). The working
set (ao_vgl 1.95 GB + mo_vgl 0.49 GB per step) is far larger than the 129 MB L2, so no L2
flush is inserted between steps.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--form fp64|mixed]

Under torchrun (N > 1) each rank runs an independent replica on its own GPU ("replicas
only": the path has no exchange step); value = all points / max-over-ranks time.
`--impl reference` times the reference algorithm on the host cores (the oracle port in
oracle/, all threads) on the same workload and prints the same JSON line.
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "MO vgl points/sec on 1 GB300: mixed vs FP64 form at <=1e-6 rel err; % roofline"
FALLBACK_HBM_GBS = 6800.0


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=100)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--form", choices=["fp64", "mixed"], default=None)
    p.add_argument("--walkers", type=int, default=256)
    p.add_argument("--electrons", type=int, default=160)
    p.add_argument("--cpu-seconds", type=float, default=8.0, help="wall budget of the CPU baseline sample")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-batched", action="store_true", help="skip the batched-form measurement")
    p.add_argument("--long-steps", type=int, default=200,
                   help="steps of the headline form's second, longer timed region (0: skip it)")
    p.add_argument("--batch-molecules", type=int, default=64, help="molecules of the batched workload")
    p.add_argument("--batch-walkers", type=int, default=32, help="walkers per molecule of the batched workload")
    return p.parse_args()


class Dist:
    """Rank bookkeeping; torch.distributed (gloo, CPU) only for the N > 1 barrier/max."""

    def __init__(self):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local_rank = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch.distributed as dist

            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            dist.init_process_group("gloo", rank=self.rank, world_size=self.world)
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, x):
        if not self.pg:
            return x
        import torch

        t = torch.tensor([float(x)], dtype=torch.float64)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def sum(self, x):
        if not self.pg:
            return x
        import torch

        t = torch.tensor([float(x)], dtype=torch.float64)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.SUM)
        return float(t.item())


class NvmlSampler:
    """SM clock and clock-event reasons read through NVML (libnvidia-ml, read-only queries) every
    2 ms on a host thread during a timed region: the timed regions here last tens of
    milliseconds, shorter than nvidia-smi's sampling period."""

    REASONS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown", 0x40: "hw_thermal_slowdown"}

    def __init__(self, gpu, period=0.002):
        self.gpu, self.period = gpu, period
        self.samples, self.reasons, self.max_mhz = [], set(), None
        self.ok = False
        try:
            self.nv = ctypes.CDLL("libnvidia-ml.so.1")
            if self.nv.nvmlInit_v2() != 0:
                return
            self.h = ctypes.c_void_p()
            if self.nv.nvmlDeviceGetHandleByIndex_v2(ctypes.c_uint(gpu), ctypes.byref(self.h)) != 0:
                self.nv.nvmlShutdown()
                return
            m = ctypes.c_uint()
            if self.nv.nvmlDeviceGetMaxClockInfo(self.h, 1, ctypes.byref(m)) == 0:
                self.max_mhz = float(m.value)
            self.reason_fn = getattr(self.nv, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
                getattr(self.nv, "nvmlDeviceGetCurrentClocksThrottleReasons")
            self.ok = True
        except (OSError, AttributeError):
            self.ok = False

    def _run(self):
        mhz, r = ctypes.c_uint(), ctypes.c_ulonglong()
        while not self.stop:
            if self.nv.nvmlDeviceGetClockInfo(self.h, 1, ctypes.byref(mhz)) == 0:
                self.samples.append(float(mhz.value))
            if self.reason_fn(self.h, ctypes.byref(r)) == 0:
                for bit, name in self.REASONS.items():
                    if r.value & bit:
                        self.reasons.add(name)
            time.sleep(self.period)

    def __enter__(self):
        if self.ok:
            self.stop = False
            self.t = threading.Thread(target=self._run, daemon=True)
            self.t.start()
        return self

    def __exit__(self, *exc):
        if self.ok:
            self.stop = True
            self.t.join()
            self.nv.nvmlShutdown()  # balances the nvmlInit of this sampler
            self.ok = False

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": self.max_mhz, "reasons": ["unsampled"], "samples": 0,
                    "source": "nvml"}
        return {"sm_mhz": statistics.median(self.samples), "sm_max_mhz": self.max_mhz,
                "reasons": sorted(self.reasons), "samples": len(self.samples), "source": "nvml, every 2 ms"}


def clock_sampler(gpu):
    """NVML sampling where the driver's library loads, else nvidia-smi."""
    s = NvmlSampler(gpu)
    return s if s.ok else ClockSampler(gpu)


def cpu_model():
    """The host CPU's model name (lscpu, which also names Arm cores; else /proc/cpuinfo)."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.strip().lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        for line in open("/proc/cpuinfo"):
            if line.lower().startswith(("model name", "cpu model")):
                return line.split(":", 1)[1].strip()
    except OSError:
        pass
    import platform

    return platform.processor() or platform.machine()


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled every 50 ms during a timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            # the timed region starts once nvidia-smi is sampling
            t0 = time.time()
            while not self.lines and time.time() - t0 < 3.0 and self.proc.poll() is None:
                time.sleep(0.01)
            self.skip = len(self.lines)
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
        sm, smax, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines[getattr(self, "skip", 0):]:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = max(smax, float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax, "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return d, "measured"
    return {"hbm_gbs": FALLBACK_HBM_GBS}, "fallback"


def ncu_traffic():
    """Per-point DRAM bytes (and FP64-pipe activity and FP64 thread instructions per point, where
    measured) of the dominant kernels from the committed ncu summary (profiles/ncu_traffic.txt,
    lines `kernel=<name> dram_bytes_per_point=<x> [fp64_pipe_active=<f>] [fp64_inst_per_point=<n>]`)."""
    out, pipe = {}, {}
    path = os.path.join(ROOT, "profiles", "ncu_traffic.txt")
    if os.path.exists(path):
        for line in open(path):
            if line.startswith("kernel="):
                kv = dict(t.split("=", 1) for t in line.split())
                out[kv["kernel"]] = float(kv["dram_bytes_per_point"])
                for key in ("fp64_pipe_active", "tensor_pipe_active", "fp64_inst_per_point"):
                    if key in kv:
                        pipe.setdefault(kv["kernel"], {})[key + "_ncu"] = float(kv[key])
    return out, pipe


def cpu_baseline(s, seconds, threads=None):
    """The reference algorithm (oracle port, all host threads) on the whole workload, repeated
    until `seconds` of wall time (at least once): returns points/s, threads and the sample, and
    the last result (the oracle's mo_vgl of the workload)."""
    from oracle import oracle

    L = oracle.lib()
    if threads:
        L.oracle_set_num_threads(threads)
    nthreads = L.oracle_num_threads()
    t_total, reps, out = 0.0, 0, None
    while reps == 0 or (t_total < seconds and reps < 20):
        t0 = time.perf_counter()
        out = oracle.forward(s, want=("mo_vgl",))["mo_vgl"]
        t_total += time.perf_counter() - t0
        reps += 1
    return (s.point_num * reps / t_total, nthreads,
            "the whole workload (%d points) x %d, %.1f s wall" % (s.point_num, reps, t_total), out)


def run_reference(args, dist):
    from qmckl_sycl_gb300.systems import config_medium

    if dist.rank != 0:
        return
    s = config_medium(0, args.walkers, args.electrons)
    from oracle import oracle

    nthreads = oracle.lib().oracle_num_threads()
    times = []
    # one step = the whole workload (every point), as the GPU arm's step
    for i in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        oracle.forward(s, want=("mo_vgl",))
        dt = time.perf_counter() - t0
        if i >= args.warmup:
            times.append(dt)
    v = s.point_num * len(times) / sum(times)
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "points/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sum(times) / len(times),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": config_dict(s), "form": REF_FORM,
        "cpu_baseline": {"value": v, "unit": "points/s", "cores": nthreads, "cpu": cpu_model(), "kind": "port",
                         "sample": "the whole workload (%d points) per step" % s.point_num},
        "e2e": {"value": v, "unit": "points/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# what the reference arm runs (the same workload and config as this arm's)
REF_FORM = "reference CPU path: the oracle port of src/qmckl_ao_sycl.cpp + src/qmckl_mo_sycl.cpp, FP64, all host threads"


def config_dict(s):
    return {"workload": "medium: %d nuclei, %d shells, %d primitives, %d AOs, %d MOs, %d points" % (
        s.nucl_num, s.shell_num, s.prim_num, s.ao_num, s.mo_num, s.point_num),
            "nucl_num": s.nucl_num, "shell_num": s.shell_num, "prim_num": s.prim_num, "ao_num": s.ao_num,
            "mo_num": s.mo_num, "point_num": s.point_num, "seed": 0,
            "l2": "no flush: per-step working set %.2f GB (ao_vgl + mo_vgl) > 129 MB L2" % (
                8.0 * 5 * s.point_num * (s.ao_num + s.mo_num) / 1e9)}


def time_form(ctx, s, form, steps, warmup, dist, clocks=None):
    from qmckl_sycl_gb300 import PRECISION_FP64, PRECISION_SPLIT_BF16

    ctx.set_precision(PRECISION_FP64 if form == "fp64" else PRECISION_SPLIT_BF16)
    ctx.set_async(True)
    for _ in range(warmup):
        ctx.touch()
        ctx.call("provide_mo_basis_mo_vgl")
    ctx.synchronize()
    ctx.reset_kernel_stats()
    dist.barrier()
    ctx.synchronize()
    sampler = clocks or _NullCtx()
    with sampler:
        ctx.call("timer_start")
        for _ in range(steps):
            ctx.touch()
            ctx.call("provide_mo_basis_mo_vgl")
        ms = ctypes.c_double(0)
        ctx.call("timer_stop", ctypes.byref(ms))
    ctx.synchronize()
    stats = ctx.kernel_stats()
    launches = ctx.launch_count()
    ctx.set_async(False)
    return ms.value, stats, launches


class _NullCtx:
    def __enter__(self):
        return self

    def __exit__(self, *a):
        return False


def time_e2e(ctx, s, steps, warmup):
    """Through the C ABI with host buffers: page-locked coordinates in, mo_vgl out."""
    L = ctx.L
    P, M = s.point_num, s.mo_num
    coord = np.ascontiguousarray(s.coord)
    out = np.empty((P, 5, M))
    ctx.call("host_register", coord.ctypes.data_as(ctypes.c_void_p), coord.nbytes)
    ctx.call("host_register", out.ctypes.data_as(ctypes.c_void_p), out.nbytes)
    cptr = coord.ctypes.data_as(ctypes.c_void_p)
    optr = out.ctypes.data_as(ctypes.c_void_p)
    try:
        for i in range(warmup + steps):
            if i == warmup:
                t0 = time.perf_counter()
            ctx.call("set_point", b"N", P, cptr, 3 * P)
            ctx.call("get_mo_basis_mo_vgl", optr, out.size)
        dt = time.perf_counter() - t0
    finally:
        ctx.call("host_unregister", coord.ctypes.data_as(ctypes.c_void_p))
        ctx.call("host_unregister", out.ctypes.data_as(ctypes.c_void_p))
    return dt, coord.nbytes, out.nbytes, out


def time_batched(dist, steps, warmup, peaks, fp64_peak, molecules=64, walkers=32, with_oracle=False):
    """The batched form on the 64-molecule workload: every member's MO vgl per step through
    qmckl_batch_provide_mo_vgl_device (graph replay, autotuned), both precision forms, plus
    one profiled pass with ordinary launches for the per-stage times."""
    from qmckl_sycl_gb300 import Batch, Context, config_batched

    systems = config_batched(0, molecules=molecules, walkers=walkers)
    ctxs = []
    for sy in systems:
        c = Context(dist.local_rank)
        c.load_system(sy)
        ctxs.append(c)
    lead = ctxs[0]
    b = Batch(ctxs)
    P = sum(sy.point_num for sy in systems)
    ao_bytes = {"fp64": sum((8.0 * 5 * sy.ao_num + 24.0) * sy.point_num for sy in systems),
                "mixed": sum((6.0 * 5 * sy.ao_num + 24.0) * sy.point_num for sy in systems)}
    flops = sum(10.0 * sy.ao_num * sy.mo_num * sy.point_num for sy in systems)
    out = {"workload": "batched: %d molecules (%d-%d nuclei, %d-%d AOs, %d-%d MOs), %d walkers x 2N electrons "
                       "each, %d points in total" % (
                           len(systems), min(x.nucl_num for x in systems), max(x.nucl_num for x in systems),
                           min(x.ao_num for x in systems), max(x.ao_num for x in systems),
                           min(x.mo_num for x in systems), max(x.mo_num for x in systems), walkers, P),
           "point_num": P, "forms": {}}
    ref = None
    for form, mode in (("fp64", 0), ("mixed", 1)):
        b.set_precision(mode)
        b.set_async(False)
        b.touch()
        b.provide_mo_vgl()  # autotunes this shape, captures the graph
        b.set_async(True)
        for _ in range(warmup):
            b.touch()
            b.provide_mo_vgl()
        b.synchronize()
        dist.barrier()
        lead.call("timer_start")
        for _ in range(steps):
            b.touch()
            b.provide_mo_vgl()
        ms = ctypes.c_double(0)
        lead.call("timer_stop", ctypes.byref(ms))
        b.synchronize()
        b.set_async(False)
        t = dist.max(ms.value)
        lead.set_profiling(True)
        lead.reset_kernel_stats()
        for _ in range(2):
            b.touch()
            b.provide_mo_vgl()
        stats = lead.kernel_stats()
        lead.set_profiling(False)
        kern = {}
        for k, st in stats.items():
            n, tot = st
            if n <= 0:
                continue
            kms = tot / n
            if k.startswith("batch_ao_vgl"):
                a = ao_bytes[form] / (kms * 1e-3) / 1e9
                kern[k] = {"bound": "hbm", "achieved": a, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                           "ms_per_launch": kms, "frac": a / peaks["hbm_gbs"]}
            elif k.startswith("batch_mo_vgl"):
                pk = fp64_peak if form == "fp64" else peaks.get("bf16_tflops", 1909.5)
                a = flops / (kms * 1e-3) / 1e12
                kern[k] = {"bound": "tensor", "achieved": a, "peak": pk, "unit": "TFLOP/s", "ms_per_launch": kms,
                           "frac": a / pk}
            else:
                kern[k] = {"ms_per_launch": kms}
        out["forms"][form] = {"value": dist.sum(P * steps) / (t * 1e-3), "ms_per_step": t / steps,
                              "tuning": list(b.tuning()), "launches_per_step": b.launch_count(),
                              "graph": True, "kernels": kern}
        if form == "fp64":
            ref = [c.get_mo_vgl(sy.point_num) for c, sy in zip(ctxs, systems)]
        else:
            worst = np.zeros(5)
            worst_o = {"fp64": np.zeros(5), "mixed": np.zeros(5)}
            for c, sy, r in zip(ctxs, systems, ref):
                g = c.get_mo_vgl(sy.point_num)
                worst = np.maximum(worst, np.abs(g - r).max(axis=(0, 2)) / np.abs(r).max(axis=(0, 2)))
                if with_oracle:
                    from oracle import oracle

                    o = oracle.forward(sy, want=("mo_vgl",))["mo_vgl"]
                    sc = np.abs(o).max(axis=(0, 2))
                    worst_o["fp64"] = np.maximum(worst_o["fp64"], np.abs(r - o).max(axis=(0, 2)) / sc)
                    worst_o["mixed"] = np.maximum(worst_o["mixed"], np.abs(g - o).max(axis=(0, 2)) / sc)
            out["mixed_vs_fp64_error"] = {"max_rel_normwise_over_molecules": [float(x) for x in worst]}
            if with_oracle:
                out["error_vs_oracle"] = {f: {"max_rel_normwise_over_molecules": [float(x) for x in w]}
                                          for f, w in worst_o.items()}
    out["mixed_over_fp64"] = out["forms"]["mixed"]["value"] / out["forms"]["fp64"]["value"]
    b.close()
    for c in ctxs:
        c.close()
    return out


def time_shared_exponentials(dist, steps, warmup, points=40960):
    """Shared exponentials (the per-nucleus distinct exponents of finalize_hpc) on two
    contracted bases with `points` points around their nuclei: the CHBrClF molecule of the
    reference's tests (5 nuclei, 297 primitives, 133 distinct exponents per nucleus, 263 AOs,
    224 MOs) and the generally contracted synthetic basis (20 nuclei, 2060 primitives, 26
    distinct exponents per nucleus, 1100 AOs, 300 MOs). Per form: the fused AO kernel's time
    with sharing off, on, and as chosen automatically, and the automatic choice's points/s."""
    from qmckl_sycl_gb300 import (PRECISION_FP64, PRECISION_SPLIT_BF16, SHARED_EXP_AUTO, SHARED_EXP_OFF,
                                  SHARED_EXP_ON, Context)
    from qmckl_sycl_gb300.systems import System, config_contracted

    base = System.from_npz(os.path.join(ROOT, "tests", "golden", "chbrclf.npz"))
    rng = np.random.default_rng(3)
    nuc = base.nucl_coord.T[rng.integers(0, base.nucl_num, points)]
    systems = [("chbrclf", base.with_points(nuc + rng.normal(scale=1.5, size=(points, 3)))),
               ("contracted", config_contracted(0, points))]
    out = {}
    k = max(5, min(steps, 20))
    for label, sy in systems:
        ctx = Context(dist.local_rank)
        ctx.load_system(sy)
        entry = {"workload": "%s: %d nuclei, %d shells, %d primitives, %d AOs, %d MOs, %d points" % (
            label, sy.nucl_num, sy.shell_num, sy.prim_num, sy.ao_num, sy.mo_num, points)}
        for form, prec, kname, call in (
                ("fp64", PRECISION_FP64, "ao_vgl_fused", "provide_ao_basis_ao_vgl"),
                ("mixed", PRECISION_SPLIT_BF16, "ao_vgl_fused_bf16_planes", "provide_mo_basis_mo_vgl")):
            ctx.set_precision(prec)
            res = {}
            for mlabel, mode in (("off", SHARED_EXP_OFF), ("on", SHARED_EXP_ON), ("auto", SHARED_EXP_AUTO)):
                ctx.set_shared_exponentials(mode)
                for _ in range(warmup):
                    ctx.touch()
                    ctx.call(call)
                ctx.synchronize()
                ctx.set_profiling(True)
                ctx.reset_kernel_stats()
                ctx.call("timer_start")
                for _ in range(k):
                    ctx.touch()
                    ctx.call(call)
                ms = ctypes.c_double(0)
                ctx.call("timer_stop", ctypes.byref(ms))
                st = ctx.kernel_stats()
                ctx.set_profiling(False)
                n, tot = st.get(kname, (0, 0.0))
                res[mlabel] = (tot / n if n else None, ms.value / k)
                if mlabel == "auto":
                    res["auto_active"] = ctx.shared_exponentials()
            entry[form] = {"ao_kernel": kname, "ao_ms_off": res["off"][0], "ao_ms_on": res["on"][0],
                           "ao_ms_auto": res["auto"][0], "auto_shares": res["auto_active"],
                           "ao_speedup_on": res["off"][0] / res["on"][0] if res["off"][0] and res["on"][0] else None,
                           "step_ms_auto": res["auto"][1], "points_per_s_auto": points / (res["auto"][1] * 1e-3)}
        ctx.close()
        out[label] = entry
    return out


def time_adjoint(dist, steps, warmup, fp64_peak):
    """The adjoint form on its workload (8 nuclei, ~200 AOs, 64 MOs, 2048 points): one step =
    new points + qmckl_vjp_mo_vgl_device for all three gradients (coefficients, exponents,
    coordinates), W ~ N(0, 1) resident on the device."""
    from qmckl_sycl_gb300 import Context, config_adjoint

    sy = config_adjoint(0)
    P, A, M, K = sy.point_num, sy.ao_num, sy.mo_num, sy.prim_num
    ctx = Context(dist.local_rank)
    ctx.load_system(sy)
    w = np.random.default_rng(5).normal(size=(P, 5, M))
    wd = ctx.upload(w)
    dc = ctx.buffer("dc", 8 * M * A)
    de = ctx.buffer("de", 8 * K)
    dx = ctx.buffer("dx", 8 * 3 * P)

    def step():
        ctx.touch()
        ctx.call("vjp_mo_vgl", wd.ptr, w.size, dc.ptr, M * A, de.ptr, K, dx.ptr, 3 * P)

    ctx.set_async(True)
    for _ in range(warmup):
        step()
    ctx.synchronize()
    dist.barrier()
    reps = max(steps, 20)
    ctx.call("timer_start")
    for _ in range(reps):
        step()
    ms = ctypes.c_double(0)
    ctx.call("timer_stop", ctypes.byref(ms))
    ctx.synchronize()
    ctx.set_async(False)
    t = dist.max(ms.value) / reps
    ctx.set_profiling(True)
    ctx.reset_kernel_stats()
    for _ in range(3):
        step()
    stats = ctx.kernel_stats()
    ctx.close()
    kern = {}
    gemm_flops = 2.0 * 5 * P * M * A
    for k, (n, tot) in stats.items():
        if n <= 0:
            continue
        kms = tot / n
        kern[k] = {"ms_per_launch": kms, "launches_per_step": n / 3.0}
        if k in ("vjp_ao_adjoint_dgemm", "vjp_coefficient_dgemm"):
            kern[k].update({"bound": "tensor", "achieved": gemm_flops / (kms * 1e-3) / 1e12, "peak": fp64_peak,
                            "unit": "TFLOP/s"})
            kern[k]["frac"] = kern[k]["achieved"] / fp64_peak
    return {"workload": "adjoint: %d nuclei, %d shells, %d primitives, %d AOs, %d MOs, %d points; L = sum(W * mo_vgl), "
                        "W ~ N(0,1); gradients w.r.t. C, exponents, coordinates (FP64)" % (
                            sy.nucl_num, sy.shell_num, K, A, M, P),
            "value": dist.sum(P) / (t * 1e-3), "unit": "points/s", "ms_per_step": t, "kernels": kern}


def main():
    args = parse()
    dist = Dist()
    if args.impl == "reference":
        run_reference(args, dist)
        return
    from qmckl_sycl_gb300 import Context, config_medium

    s = config_medium(0, args.walkers, args.electrons)
    P, A, M = s.point_num, s.ao_num, s.mo_num
    ctx = Context(dist.local_rank)
    ctx.set_profiling(True)
    ctx.load_system(s)
    fp64_peak = ctypes.c_double(0)
    ctx.call("measure_fp64_peak", ctypes.byref(fp64_peak))
    peaks, peak_src = measured_peaks()
    traffic, fp64_pipe = ncu_traffic()

    forms = ["fp64"]
    try:
        ctx.set_precision(1)
        ctx.touch()
        ctx.call("provide_mo_basis_mo_vgl")
        forms.append("mixed")
    except Exception:
        pass
    ctx.set_precision(0)
    headline = args.form or ("mixed" if "mixed" in forms else "fp64")

    results = {}
    samplers = {f: clock_sampler(dist.local_rank) for f in forms}
    clocks = samplers[headline]
    for form in forms:
        # the FP64 form (150 ms a step) is timed on at most 10 steps when it is not the headline
        k = args.steps if form == headline else min(args.steps, 10)
        ms, stats, launches = time_form(ctx, s, form, k, args.warmup, dist, samplers[form])
        t = dist.max(ms)
        total_points = dist.sum(P * k)
        results[form] = dict(ms=t, value=total_points / (t * 1e-3), stats=stats, launches=launches, steps=k)

    # the headline form once more over a longer timed region (at least 200 steps), with its own
    # clock record: the timed region of K steps lasts only tens of milliseconds
    long_run = None
    if args.long_steps > 0:
        long_k = max(args.long_steps, args.steps)
        long_clocks = clock_sampler(dist.local_rank)
        ms_long, _, _ = time_form(ctx, s, headline, long_k, args.warmup, dist, long_clocks)
        t_long = dist.max(ms_long)
        long_run = {"steps": long_k, "value": dist.sum(P * long_k) / (t_long * 1e-3),
                    "ms_per_step": t_long / long_k, "clocks": long_clocks.summary()}

    # CPU baseline: the oracle port on the whole workload (rank 0, one GPU), whose result is also
    # the reference for the error of both forms below
    cpu, oracle_mo = None, None
    if dist.rank == 0 and dist.world == 1 and not args.no_cpu_baseline:
        v, cores, sample, oracle_mo = cpu_baseline(s, args.cpu_seconds)
        cpu = {"value": v, "unit": "points/s", "cores": cores, "cpu": cpu_model(), "kind": "port", "sample": sample}

    def errors(got, ref):
        scale = np.abs(ref).max(axis=(0, 2))
        diff = np.abs(got - ref)
        big = np.abs(ref) >= 1e-3 * scale[None, :, None]  # elementwise relative error where |ref| is not tiny
        rel = np.where(big, diff / np.where(big, np.abs(ref), 1.0), 0.0)
        return {"max_abs": [float(x) for x in diff.max(axis=(0, 2))],
                "max_rel_normwise": [float(x) for x in diff.max(axis=(0, 2)) / scale],
                "max_rel_elementwise_where_ref_ge_1e-3_max": [float(x) for x in rel.max(axis=(0, 2))]}

    # accuracy of the mixed form against the FP64 form and against the oracle, on the same inputs
    acc = acc_oracle = None
    if "mixed" in forms:
        ctx.set_precision(0)
        ctx.touch()
        ref = ctx.get_mo_vgl(P)
        ctx.set_precision(1)
        ctx.touch()
        got = ctx.get_mo_vgl(P)
        acc = errors(got, ref)
        if oracle_mo is not None:
            acc_oracle = {"mixed": errors(got, oracle_mo), "fp64": errors(ref, oracle_mo),
                          "points": P, "components": ["value", "d/dx", "d/dy", "d/dz", "laplacian"]}
        del ref, got

    # end to end through the C ABI with host buffers (headline form), as a caller runs it: without
    # the per-launch timing events (the host-buffer path launches ~30 kernels and copies a step)
    ctx.set_precision(0 if headline == "fp64" else 1)
    ctx.set_profiling(False)
    e2e_dt, h2d, d2h, _ = time_e2e(ctx, s, args.steps, min(args.warmup, 2))
    ctx.set_profiling(True)
    e2e_dt = dist.max(e2e_dt)
    e2e_value = dist.sum(P * args.steps) / e2e_dt

    def roof(form):
        st = results[form]["stats"]
        out = {}
        # AO kernel: algorithmic bytes 8 (5A + 3) per point (the FP64 ao_vgl written, coordinates
        # read) for both forms; the split-BF16 form's kernel writes three BF16 planes instead (6
        # bytes per element), reported beside it
        for k in ("ao_vgl_fused", "ao_vgl_fused_bf16_planes"):
            if st.get(k, (0, 0))[0] > 0:
                n, tot = st[k]
                ms = tot / max(n, 1)
                alg = (8.0 * 5 * A + 24.0) * P
                out[k] = {"bound": "hbm", "achieved": alg / (ms * 1e-3) / 1e9, "peak": peaks["hbm_gbs"],
                          "unit": "GB/s", "ms_per_launch": ms, "traffic": traffic.get(k, 0) * P or None,
                          "algorithmic_bytes": alg}
                out[k]["frac"] = out[k]["achieved"] / peaks["hbm_gbs"]
                if k == "ao_vgl_fused_bf16_planes":
                    written = (6.0 * 5 * A + 24.0) * P
                    out[k]["planes_bytes"] = written
                    out[k]["planes_frac"] = written / (ms * 1e-3) / 1e9 / peaks["hbm_gbs"]
                # what bounds it on GB300 is the latency of its FP64 chains, not HBM: the FP64-pipe
                # activity ncu measured on the same kernel
                out[k].update({kk: v for kk, v in fp64_pipe.get(k, {}).items() if kk != "fp64_inst_per_point_ncu"})
        for k in ("mo_vgl_dgemm", "mo_vgl_split_bf16"):
            if st.get(k, (0, 0))[0] > 0:
                n, tot = st[k]
                ms = tot / max(n, 1)
                flops = 10.0 * A * M * P
                pk = fp64_peak.value if k == "mo_vgl_dgemm" else peaks.get("bf16_tflops", 1909.5)
                out[k] = {"bound": "tensor", "achieved": flops / (ms * 1e-3) / 1e12, "peak": pk, "unit": "TFLOP/s",
                          "ms_per_launch": ms, "traffic": traffic.get(k, 0) * P or None}
                out[k]["frac"] = out[k]["achieved"] / pk
                out[k].update(fp64_pipe.get(k, {}))
                if k == "mo_vgl_split_bf16":
                    # the split executes six BF16 products per algorithmic one (on 64-padded K and
                    # 16-padded column tiles); the algorithmic figure above counts 10 A M per point
                    out[k]["bf16_products"] = 6
                    out[k]["bf16_work_frac"] = 6.0 * out[k]["frac"]
                    out[k]["note"] = ("frac counts the algorithmic 10 A M FLOPs per point; the kernel executes "
                                      "six BF16 products per algorithmic one: bf16_work_frac")
        return out

    rf = {f: roof(f) for f in forms}
    head = rf[headline]
    dom = max(head, key=lambda k: head[k]["ms_per_launch"])
    roofline = dict(head[dom])
    roofline["kernel"] = dom
    roofline["peak_source"] = ("live DMMA m16n8k4 f64 probe (MEASURED_PEAKS.json has no FP64 figure)"
                               if dom == "mo_vgl_dgemm" else "%s MEASURED_PEAKS.json" % peak_src)

    adj = time_adjoint(dist, args.steps, args.warmup, fp64_peak.value)
    shared = time_shared_exponentials(dist, args.steps, args.warmup)
    bt = None
    if not args.no_batched:
        bt = time_batched(dist, args.steps, args.warmup, peaks, fp64_peak.value, args.batch_molecules,
                          args.batch_walkers, with_oracle=dist.rank == 0 and not args.no_cpu_baseline)
        bt["mixed_over_plain_fp64_medium"] = bt["forms"]["mixed"]["value"] / results["fp64"]["value"]
    if dist.rank != 0:
        return
    hr = results[headline]
    line = {
        "metric": METRIC, "value": hr["value"], "unit": "points/s", "n_gpus": dist.world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": hr["ms"] / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64" if headline == "fp64" else "f64+bf16x3",
        "data": "synthetic (seeded generator with the medium configuration's shapes and distributions)",
        "config": config_dict(s), "form": "split-BF16 (mixed)" if headline == "mixed" else "FP64 (plain)",
        "roofline": roofline, "cpu_baseline": cpu,
        "e2e": {"value": e2e_value, "unit": "points/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "gpu_launches": hr["launches"], "clocks": clocks.summary(),
        "clocks_by_form": {f: samplers[f].summary() for f in forms},
        "forms": {f: {"value": results[f]["value"], "ms_per_step": results[f]["ms"] / results[f]["steps"],
                      "steps": results[f]["steps"], "kernels": rf[f]} for f in forms},
        "fp64_peak_tflops": fp64_peak.value, "long_run": long_run,
    }
    if acc:
        line["mixed_vs_fp64_error"] = acc
    if acc_oracle:
        line["error_vs_oracle"] = acc_oracle
        line["mixed_over_fp64"] = results["mixed"]["value"] / results["fp64"]["value"]
    line["adjoint"] = adj
    line["shared_exponentials"] = shared
    if bt:
        line["batched"] = bt
    print(json.dumps(line), flush=True)
    ctx.close()


if __name__ == "__main__":
    main()
