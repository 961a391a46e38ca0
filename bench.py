#!/usr/bin/env python
"""Benchmark of the Lennard-Jones neighbour-list force path on GB300.

Workload (the reference's rho = 0.5 comparison case at 108,000 particles):
FCC 30^3 cells x 4 = 108,000 particles, rho = 0.5, periodic cubic box
L = (N / rho)^(1/3) = 60, jitter U[-0.05, 0.05) per coordinate from
mt19937_64(20240601), cutoff 3.0 (CL2 = 9), search radius 3.3, i-sorted int32
CSR half list (~37.6 partners per particle) built on the device, AoS double4
and SoA positions, dt = 0.005.

A step is one force call (p += F dt over the whole system).  L2 is flushed
(512 MiB write) before every timed step; each step is timed with CUDA events
on the engine's stream.  `value` is the best mixed-precision variant in
G pair-interactions/s = P_half / t_call / 1e9 (P_half = i<j list pairs, the
same count for gather and scatter); the FP64 path is reported beside it.

e2e runs the reference's measure() through the C ABI (lj_measure_aos): host
q, p and the CSR list uploaded from pinned memory, 100 force calls, p
downloaded, every step.

--impl reference times the reference's CPU force routine restated in C (the
oracle; gather over the full list on every host core, project-written
OpenMP -- the reference itself is single-threaded) on the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

NCELL, DENSITY, JITTER, SEED = 30, 0.5, 0.05, 20240601
RC, RS, DT = 3.0, 3.3, 0.005
METRIC = "G pair-interactions/s, mixed vs plain FP64, same GB300, force rel err <=1e-5"
UNIT = "G pair-interactions/s"
WORKLOAD = ("LJ force call, FCC 108,000 particles, rho=0.5, periodic L=60, rc=3.0, "
            "search 3.3, i-sorted int32 CSR, dt=0.005")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--e2e-steps", type=int, default=5)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-autotune", action="store_true",
                    help="time the 'auto' variants with the engine's default launch shapes "
                         "(what the tuner picks on this workload) instead of tuning first; "
                         "for runs under a profiler, whose per-launch overhead swamps the "
                         "tuner's timings")
    ap.add_argument("--shape", action="append", default=[],
                    help="extra mixed AoS gather variant KERNEL,LANES,UNROLL (e.g. 3,4,2 for "
                         "the cell-tiled kernel), timed beside the default variants")
    ap.add_argument("--workload", default="rho0.5_108k",
                    choices=["rho0.5_108k", "rho1_108k", "precision_1m", "large_8m",
                             "batch_512"],
                    help="rho0.5_108k: the headline force benchmark; rho1_108k: the same at "
                         "rho = 1; precision_1m: 1,000,188-particle mixed MD with force "
                         "errors against FP64 every 100 steps; large_8m: 8,001,504-particle "
                         "MD, mixed and FP64 back to back; batch_512: 512 replicas of "
                         "uneven N in one mixed MD loop")
    return ap.parse_args()


# ---------------------------------------------------------------------------
# distributed plumbing (replicas only: every rank runs its own system)
# ---------------------------------------------------------------------------
class Dist:
    def __init__(self, backend):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch.distributed as dist
            dist.init_process_group(backend=backend)
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, v, device=None):
        if not self.pg:
            return v
        import torch
        t = torch.tensor([v], dtype=torch.float64, device=device)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def sum(self, v, device=None):
        if not self.pg:
            return v
        import torch
        t = torch.tensor([v], dtype=torch.float64, device=device)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.SUM)
        return float(t.item())

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()


# ---------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------
class _Nvml:
    """Read-only NVML queries through ctypes (the library ships with the
    driver): SM clock, its maximum, power and the active clock-event reasons
    of one device.  Nothing here sets anything."""
    SM = 1  # NVML_CLOCK_SM
    REASONS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown",
               0x40: "hw_thermal_slowdown", 0x80: "hw_power_brake_slowdown"}

    def __init__(self, cuda_index):
        import ctypes
        self.c = ctypes
        self.lib = ctypes.CDLL("libnvidia-ml.so.1")
        if self.lib.nvmlInit_v2() != 0:
            raise OSError("nvmlInit failed")
        self.h = ctypes.c_void_p()
        bus = self._bus_id(cuda_index)
        rc = (self.lib.nvmlDeviceGetHandleByPciBusId_v2(bus.encode(), ctypes.byref(self.h))
              if bus else self.lib.nvmlDeviceGetHandleByIndex_v2(cuda_index,
                                                                 ctypes.byref(self.h)))
        if rc != 0:
            self.lib.nvmlShutdown()
            raise OSError("no NVML handle for CUDA device %d" % cuda_index)
        self.reasons_fn = getattr(self.lib, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
            self.lib.nvmlDeviceGetCurrentClocksThrottleReasons
        self.max_mhz = self._uint(self.lib.nvmlDeviceGetMaxClockInfo, self.SM)

    @staticmethod
    def _bus_id(cuda_index):
        # NVML numbers devices in PCI order, CUDA by CUDA_VISIBLE_DEVICES:
        # match them by bus id where torch reports it
        try:
            import torch
            pr = torch.cuda.get_device_properties(cuda_index)
            return "%08X:%02X:%02X.0" % (pr.pci_domain_id, pr.pci_bus_id, pr.pci_device_id)
        except (AttributeError, RuntimeError, AssertionError):
            return None

    def _uint(self, fn, *args):
        v = self.c.c_uint()
        return v.value if fn(self.h, *args, self.c.byref(v)) == 0 else None

    def sample(self):
        r = self.c.c_ulonglong()
        ok = self.reasons_fn(self.h, self.c.byref(r)) == 0
        return (self._uint(self.lib.nvmlDeviceGetClockInfo, self.SM),
                self._uint(self.lib.nvmlDeviceGetPowerUsage),
                [nm for bit, nm in self.REASONS.items() if ok and r.value & bit])

    def close(self):
        self.lib.nvmlShutdown()


class ClockSampler:
    """SM clock and clock-event reasons sampled during a timed region: NVML
    every 2 ms where the library loads, else `nvidia-smi -lms 100`."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
    PERIOD_S = 0.002

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.nvml = None
        self.lines = []
        self.samples = []  # (sm MHz, power mW, reasons) from NVML
        self.stop = threading.Event()

    def __enter__(self):
        try:
            self.nvml = _Nvml(self.gpu)
            self.samples.append(self.nvml.sample())
            self.t = threading.Thread(target=self._poll, daemon=True)
            self.t.start()
            return self
        except (OSError, AttributeError):
            self.nvml = None
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (FileNotFoundError, OSError):
            self.proc = None
        return self

    def _poll(self):
        while not self.stop.wait(self.PERIOD_S):
            self.samples.append(self.nvml.sample())

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.nvml:
            self.stop.set()
            self.t.join(timeout=5)
            self.samples.append(self.nvml.sample())
            self.nvml.close()
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if self.nvml:
            sm = [s[0] for s in self.samples if s[0] is not None]
            pw = [s[1] / 1e3 for s in self.samples if s[1] is not None]
            reasons = sorted({nm for s in self.samples for nm in s[2]})
            if sm:
                return {"sm_mhz": statistics.median(sm), "sm_min_mhz": min(sm),
                        "sm_max_mhz": self.nvml.max_mhz, "reasons": reasons,
                        "power_w_median": statistics.median(pw) if pw else None,
                        "samples": len(sm), "source": "nvml, every 2 ms"}
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm), "source": "nvidia-smi -lms 100"}


def merge_clocks(parts):
    """One clock record from several sampled segments: the median of the
    segments' medians, the lowest clock seen and every reason seen."""
    got = [c for c in parts if c.get("samples")]
    if not got:
        return parts[0] if parts else None
    out = dict(got[0])
    out["sm_mhz"] = statistics.median(c["sm_mhz"] for c in got)
    if all("sm_min_mhz" in c for c in got):
        out["sm_min_mhz"] = min(c["sm_min_mhz"] for c in got)
    pw = [c["power_w_median"] for c in got if c.get("power_w_median") is not None]
    if pw:
        out["power_w_median"] = statistics.median(pw)
    out["reasons"] = sorted({r for c in got for r in c["reasons"]})
    out["samples"] = sum(c["samples"] for c in got)
    return out


# ---------------------------------------------------------------------------
# roofline constants
# ---------------------------------------------------------------------------
def peaks():
    f = ROOT / "MEASURED_PEAKS.json"
    if f.exists():
        d = json.loads(f.read_text())
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


def profiled_traffic(name):
    """dram bytes per launch recorded from an ncu capture under profiles/."""
    f = ROOT / "profiles" / name
    if not f.exists():
        return None
    for line in f.read_text().splitlines():
        if line.startswith("traffic_bytes_per_launch:"):
            return float(line.split(":")[1].split()[0])
    return None


def profiled_metric(name, metric):
    """One metric value (a number) from the `- `metric`: value unit` lines of an
    ncu summary under profiles/."""
    f = ROOT / "profiles" / name
    if not f.exists():
        return None
    key = f"- `{metric}`:"
    for line in f.read_text().splitlines():
        if line.startswith(key):
            try:
                return float(line[len(key):].split()[0])
            except (IndexError, ValueError):
                return None
    return None


# FP64 add / FMA issue rate measured on this machine's GB300 (one op per lane):
# 503 G/s, i.e. ~1.0 TFLOP/s counting an FMA as two
FP64_PEAK_OPS = 503e9


def pair_kernel_bytes(method, layout, P, N):
    """Compulsory bytes of the pair kernel alone: list indices, the 16-byte
    fixed-point image read once, number_of_partners + pointer, p read +
    written (AoS: a 32-byte record)."""
    per_n = (16 + 8 + 64) if layout == "aos" else (16 + 8 + 48)
    return (8 if method == "gather" else 4) * P + per_n * N


def algorithmic_bytes(method, layout, P, N):
    # compulsory traffic per force call (each datum once): list indices, q, p
    # read + write, number_of_partners + pointer
    per_n = 104 if layout == "aos" else 80
    return (8 if method == "gather" else 4) * P + per_n * N


# ---------------------------------------------------------------------------
# our arm
# ---------------------------------------------------------------------------
def run_ours(args, dist, density=DENSITY):
    import torch
    import lj_gpu_gb300 as lj
    from lj_gpu_gb300 import _build

    _build.build()
    dev = torch.device("cuda", dist.local)
    torch.cuda.set_device(dev)
    stream = torch.cuda.current_stream()
    q, L = lj.init_fcc(NCELL, density, JITTER, SEED)
    N = q.shape[0]
    qd = torch.from_numpy(q).to(dev)
    qs = [torch.from_numpy(np.ascontiguousarray(q[:, d])).to(dev) for d in range(3)]
    ctx = lj.Context(dist.local, stream=stream)
    t0 = time.perf_counter()
    ctx.build_list(qd, RS, box=L)
    torch.cuda.synchronize()
    t_build = time.perf_counter() - t0
    _, P, max_half = ctx.list_info("half")
    _, P_full, max_full = ctx.list_info("full")
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    def time_variant(prec, method, layout, shape, steps, warmup):
        k, g, u = shape if shape else (0, 0, 0)
        opts = lj.make_opts(dt=DT, cl2=RC * RC, box=L, precision=prec, method=method,
                            kernel=k, lanes=g, unroll=u)
        pd = torch.zeros_like(qd)
        ps = [torch.zeros(N, dtype=torch.float64, device=dev) for _ in range(3)]

        def call():
            if layout == "aos":
                ctx.force_aos(qd, pd, opts)
            else:
                ctx.force_soa(*qs, *ps, opts)

        for _ in range(warmup):
            flush.add_(1.0)
            call()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
              for _ in range(steps)]
        torch.cuda.synchronize()
        dist.barrier()
        for a, b in ev:
            flush.add_(1.0)  # > L2: every timed call starts cold
            a.record(stream)
            call()
            b.record(stream)
        torch.cuda.synchronize()
        dist.barrier()
        ms = [a.elapsed_time(b) for a, b in ev]
        return sum(ms)

    # the engine's autotuner picks the launch shape of the AoS calls that
    # leave the launch fields at their defaults ("auto" below)
    tuned = {}
    for prec in ("mixed", "fp64"):
        if args.no_autotune:
            tuned[prec] = {"method": "gather" if prec == "mixed" else "scatter",
                           "kernel": "default", "note": "autotuner skipped (--no-autotune)"}
            continue
        best, ms_t = ctx.autotune(qd, lj.make_opts(dt=DT, cl2=RC * RC, box=L, precision=prec),
                                  reps=5)
        tuned[prec] = {"method": {1: "gather", 2: "scatter"}[best.method], "kernel": best.kernel,
                       "lanes": best.lanes, "unroll": best.unroll, "block": best.block,
                       "ms_warm": ms_t}
    variants = [("mixed", "auto", "aos", None), ("mixed", "gather", "soa", None),
                ("mixed", "scatter", "aos", None), ("fp64", "auto", "aos", None),
                ("fp64", "scatter", "soa", None), ("fp64", "gather", "aos", None)]
    for s in args.shape:
        variants.append(("mixed", "gather", "aos", tuple(int(x) for x in s.split(","))))
    key = lambda v: "/".join(v[:3]) + ("/k%dg%du%d" % v[3] if v[3] else "")
    by_key = {key(v): v for v in variants}
    results = {}
    clocks = None
    for v in variants:
        steps = args.steps if v[0] == "mixed" else max(3, min(args.steps, 20))
        if v == ("mixed", "auto", "aos", None):
            with ClockSampler(dist.local) as cs:
                ms = time_variant(*v, steps, args.warmup)
            clocks = cs.summary()
        else:
            ms = time_variant(*v, steps, max(3, min(args.warmup, 5)))
        t_max = dist.max(ms / steps / 1e3, dev)  # seconds per call, slowest rank
        results[key(v)] = {"s_per_call": t_max, "steps": steps,
                                "gpairs": dist.world * P / t_max / 1e9}

    # explicit --shape variants are reported, not taken as the headline
    best_mixed = max((k for k in results if k.startswith("mixed") and by_key[k][3] is None),
                     key=lambda k: results[k]["gpairs"])
    best_fp64 = max((k for k in results if k.startswith("fp64")),
                    key=lambda k: results[k]["gpairs"])
    head = results[best_mixed]
    prec, method, layout, _ = by_key[best_mixed]
    if method == "auto":
        method = tuned[prec]["method"]

    # pair-kernel time of the headline variant (engine-side CUDA events
    # between the position-image pass and the pair kernel)
    def stage_times(variant, steps):
        ctx.set_timing(True)
        time_variant(*by_key[variant], steps, 0)
        t = ctx.get_timing()
        ctx.set_timing(False)
        return t[0] / t[3], t[1] / t[3]
    t_image_ms, t_pair_ms = stage_times(best_mixed, args.steps)

    # reported, never the headline: the mixed gather over the full list with
    # every row shuffled (the reference's random_shfl lists), same engine
    # defaults, in a context of its own
    fnp, fptr, flst = ctx.get_list_csr("full")
    lj.shuffle_rows(fnp, fptr, flst, seed=10)
    ctx2 = lj.Context(dist.local, stream=stream)
    ctx2.set_list_csr(torch.from_numpy(fnp).to(dev), torch.from_numpy(fptr).to(dev),
                      torch.from_numpy(flst).to(dev), kind="full")
    opts2 = lj.make_opts(dt=DT, cl2=RC * RC, box=L, precision="mixed", method="gather")
    pd2 = torch.zeros_like(qd)
    for _ in range(3):
        flush.add_(1.0)
        ctx2.force_aos(qd, pd2, opts2)
    ev2 = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
           for _ in range(20)]
    for a, b in ev2:
        flush.add_(1.0)
        a.record(stream)
        ctx2.force_aos(qd, pd2, opts2)
        b.record(stream)
    torch.cuda.synchronize()
    ms2 = sum(a.elapsed_time(b) for a, b in ev2) / len(ev2)
    shuffled = dist.world * P / dist.max(ms2 / 1e3, dev) / 1e9
    ctx2.close()
    t_image64_ms, t_pair64_ms = stage_times(best_fp64, max(3, min(args.steps, 20)))

    # e2e: the reference's measure() through the C ABI with pinned host buffers
    e2e = None
    if args.e2e_steps > 0:
        kind = "full" if method == "gather" else "half"
        np_, ptr_, lst_ = ctx.get_list_csr(kind)
        pin = lambda a: torch.from_numpy(a).pin_memory()
        h_np, h_ptr, h_lst = pin(np_), pin(ptr_), pin(lst_)
        ctx.set_list_csr(h_np, h_ptr, h_lst, kind=kind)
        hq = pin(q)
        hp = torch.zeros_like(hq).pin_memory()
        opts = lj.make_opts(dt=DT, cl2=RC * RC, box=L, precision=prec, method=method)
        ctx.measure_aos(hq, hp, opts, calls=100)  # warm-up
        dist.barrier()
        tot = 0.0
        for _ in range(args.e2e_steps):
            ms_total, _ = ctx.measure_aos(hq, hp, opts, calls=100)
            tot += ms_total
        dist.barrier()
        t_step = dist.max(tot / args.e2e_steps / 1e3, dev)
        h2d = hq.numel() * 8 * 2 + (h_np.numel() + h_ptr.numel() + h_lst.numel()) * 4
        e2e = {"value": dist.world * P * 100 / t_step / 1e9, "unit": UNIT,
               "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(hp.numel() * 8),
               "step": "lj_measure_aos: H2D q,p,CSR + 100 force calls + D2H p",
               "ms_per_step": t_step * 1e3}

    hbm, peak_kind = peaks()
    alg = pair_kernel_bytes(method, layout, P, N)
    achieved = alg / (t_pair_ms * 1e-3) / 1e9
    # DRAM traffic per launch from the committed ncu capture of this kernel on
    # this workload (the AoS and SoA gathers at rho 0.5); other workloads and
    # kernels have none
    prof = f"force_mixed_gather_{layout}_108k_rho0.5.txt"
    matches = density == DENSITY and method == "gather"
    traffic = profiled_traffic(prof) if matches else None
    roofline = {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                "frac": achieved / hbm, "traffic": traffic,
                "traffic_source": f"profiles/{prof}" if traffic else None,
                "peak_kind": peak_kind,
                "kernel": f"pair kernel of {best_mixed}, shape {tuned['mixed']}",
                "algorithmic_bytes_per_launch": alg,
                "kernel_ms": t_pair_ms, "position_image_ms": t_image_ms,
                "force_call_bytes": algorithmic_bytes(method, layout, P, N),
                "force_call_frac": algorithmic_bytes(method, layout, P, N)
                / head["s_per_call"] / 1e9 / hbm}
    if traffic:
        # the pipe that bounds this kernel (random 16-B gathers through L1),
        # from the same capture: wavefronts as a fraction of the pipe's peak
        l1 = profiled_metric(prof, "l1tex__data_pipe_lsu_wavefronts.avg.pct_of_peak_sustained_elapsed")
        dram = profiled_metric(prof, "gpu__dram_throughput.avg.pct_of_peak_sustained_elapsed")
        roofline["l1_data_pipe_frac"] = l1 / 100 if l1 is not None else None
        roofline["dram_throughput_frac"] = dram / 100 if dram is not None else None
    fp = results[best_fp64]
    fp_m, fp_l = best_fp64.split("/")[1], best_fp64.split("/")[2]
    if fp_m == "auto":
        fp_m = tuned["fp64"]["method"]
    # FP64 arithmetic per pair inside the cutoff (scatter): 20 FP64 ops; the
    # inside fraction of a search-radius list is (rc / rs)^3 for a uniform
    # density
    inside = (RC / RS) ** 3
    dp_ops = P * inside * (20 if fp_m == "scatter" else 34)
    fp64 = {"value": fp["gpairs"], "variant": best_fp64, "ms_per_call": fp["s_per_call"] * 1e3,
            "pair_kernel_ms": t_pair64_ms,
            "hbm_frac": algorithmic_bytes(fp_m, fp_l, P, N) / fp["s_per_call"] / 1e9 / hbm,
            "fp64_ops_per_call": dp_ops,
            "fp64_pipe_frac": dp_ops / (t_pair64_ms * 1e-3) / FP64_PEAK_OPS,
            "fp64_peak_ops_per_s": FP64_PEAK_OPS,
            "mixed_over_fp64": head["gpairs"] / fp["gpairs"]}

    cpu = None
    if dist.rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_baseline(q, L, P, sample_calls=5 if density <= 0.5 else 2)

    line = {
        "metric": METRIC, "value": dist.world * P / head["s_per_call"] / 1e9, "unit": UNIT,
        "n_gpus": dist.world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": head["s_per_call"] * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 pair math, f64 q/p",
        "data": "synthetic",
        "config": {"workload": WORKLOAD.replace("rho=0.5", f"rho={density}").replace(
                       "L=60", f"L={L:.4g}"), "N": N, "pairs_half": P, "pairs_full": P_full,
                   "max_row_half": max_half, "max_row_full": max_full, "box": L,
                   "variant": best_mixed, "step": "one force call",
                   "l2": "flushed before every timed call (512 MiB write)",
                   "list_build_s": t_build, "parallelism": f"replicas x{dist.world}"},
        "e2e": e2e, "roofline": roofline, "cpu_baseline": cpu, "fp64": fp64,
        "variants": dict({k: round(v["gpairs"], 3) for k, v in results.items()},
                         **{"mixed/gather/aos/shuffled_rows": round(shuffled, 3)}),
        "autotuned": tuned,
        "clocks": clocks, "gpu_launches": 2 * args.steps,
        "gpu_launches_note": "headline timed region: position-image pass + pair kernel per step",
    }
    ctx.close()
    return line


# ---------------------------------------------------------------------------
# MD workloads
# ---------------------------------------------------------------------------
def force_errors(torch, lj, L, qd, rs=RS):
    """Mixed vs FP64 forces of the engine on the same positions (the FP64 path
    is held to 1e-12 of the oracle by the parity tests)."""
    ctx = lj.Context(qd.device.index or 0, stream=torch.cuda.current_stream())
    ctx.build_list(qd, rs, box=L)
    out = {}
    for prec in ("mixed", "fp64"):
        p = torch.zeros_like(qd)
        ctx.force_aos(qd, p, lj.make_opts(dt=1.0, cl2=RC * RC, box=L, precision=prec))
        out[prec] = p[:, :3]
    torch.cuda.synchronize()
    d = torch.linalg.norm(out["mixed"] - out["fp64"], dim=1)
    r = torch.linalg.norm(out["fp64"], dim=1)
    rms = torch.sqrt(torch.mean(r * r))
    per = d / r
    ctx.close()
    return {"max_rel": float(per.max()), "rms_rel": float(torch.sqrt(torch.mean(per * per))),
            "max_rel_rms": float(d.max() / rms), "global_rel": float(torch.linalg.norm(d) /
                                                                     torch.linalg.norm(r))}


def md_step_bytes(P, N, rebuilds_per_step, mixed=True):
    """Algorithmic HBM bytes of one MD step: the force call (gather over the
    full list 8 P + 104 N, or scatter over the half list 4 P + 104 N), the
    drift (q read + write, p read, image write, reference image read: 112 N)
    and the list rows written by rebuilds, amortised (4 B per entry)."""
    entries = 2 * P if mixed else P
    return 4 * entries + 104 * N + 112 * N + 4 * entries * rebuilds_per_step


def run_precision(args, dist):
    """1,000,188 particles (FCC 63^3 x 4), rho = 1, rc 3.0, skin 0.3, MB momenta
    at T* = 1, 1,000 mixed velocity-Verlet steps at dt = 0.005."""
    import torch
    import lj_gpu_gb300 as lj
    from lj_gpu_gb300 import _build
    _build.build()
    dev = torch.device("cuda", dist.local)
    torch.cuda.set_device(dev)
    q, L = lj.init_fcc(63, 1.0, JITTER, SEED)
    N = q.shape[0]
    p = lj.init_momenta(N, 1.0, SEED + 1)
    qd, pd = torch.from_numpy(q).to(dev), torch.from_numpy(p).to(dev)
    errors = [dict(step=0, **force_errors(torch, lj, L, qd))]
    ctx = lj.Context(dist.local, stream=torch.cuda.current_stream())
    prm = lj.make_md_params(DT, RC, RS - RC, L, precision="mixed", record_every=100)
    records, ms, rebuilds, clock_samples = [], 0.0, 0, []
    for seg in range(10):
        with ClockSampler(dist.local) as cs:
            recs, st = ctx.md_run(qd, pd, prm, 100)
        clock_samples.append(cs.summary())
        ms += st["ms_total"]
        rebuilds += st["rebuilds"]
        records += [(r[0] + 100 * seg, r[1], r[2]) for r in recs if seg == 0 or r[0] > 0]
        errors.append(dict(step=100 * (seg + 1), **force_errors(torch, lj, L, qd)))
    e0 = records[0][1] + records[0][2]
    drift = max(abs(r[1] + r[2] - e0) for r in records) / abs(e0)
    ctx.build_list(qd, RS, box=L, kinds=("half",))
    P = ctx.list_info("half")[1]
    ctx.close()
    hbm, _ = peaks()
    sb = md_step_bytes(P, N, rebuilds / 1000)
    return {"metric": "mixed-precision MD force error vs FP64 and energy drift",
            "workload": "precision_1m", "N": N, "box": L, "steps": 1000, "dt": DT,
            "ms_per_step": ms / 1000, "rebuilds": rebuilds, "pairs_half": P,
            "gpairs": P / (ms / 1000 * 1e-3) / 1e9,
            "hbm_gbs": sb / (ms / 1000 * 1e-3) / 1e9,
            "hbm_frac": sb / (ms / 1000 * 1e-3) / 1e9 / hbm,
            "max_rel_rms_force_error": max(e["max_rel_rms"] for e in errors),
            "global_rel_force_error": max(e["global_rel"] for e in errors),
            "force_errors": errors, "energy_drift_rel": drift,
            "energies": [{"step": r[0], "kinetic": r[1], "potential": r[2]} for r in records],
            "clocks": merge_clocks(clock_samples),
            "note": "the cut, unshifted potential (the reference's) jumps when pairs cross "
                    "rc, so total energy drifts in FP64 too; force errors are against the "
                    "engine's FP64 path on the same positions"}


def run_large(args, dist):
    """8,001,504 particles (FCC 126^3 x 4), rho = 1, rc 3.0, skin 0.3, MB
    momenta at T* = 1, 500 steps at dt = 0.005 with a rebuild every 20 steps,
    mixed then FP64 from the same initial state."""
    import torch
    import lj_gpu_gb300 as lj
    from lj_gpu_gb300 import _build
    _build.build()
    dev = torch.device("cuda", dist.local)
    torch.cuda.set_device(dev)
    steps = 500 if args.steps >= 100 else args.steps
    q, L = lj.init_fcc(126, 1.0, JITTER, SEED)
    N = q.shape[0]
    p = lj.init_momenta(N, 1.0, SEED + 1)
    hbm, _ = peaks()
    out = {"metric": "MD ns/step and HBM GB/s, mixed vs FP64", "workload": "large_8m", "N": N,
           "box": L, "steps": steps, "dt": DT, "rebuild_every": 20}
    for prec in ("mixed", "fp64"):
        qd, pd = torch.from_numpy(q).to(dev), torch.from_numpy(p).to(dev)
        ctx = lj.Context(dist.local, stream=torch.cuda.current_stream())
        prm = lj.make_md_params(DT, RC, RS - RC, L, precision=prec, record_every=steps,
                                rebuild_every=20)
        with ClockSampler(dist.local) as cs:
            recs, st = ctx.md_run(qd, pd, prm, steps)
        ctx.build_list(qd, RS, box=L, kinds=("half",))
        _, P, _ = ctx.list_info("half")
        ctx.close()
        ms = st["ms_total"] / steps
        step_bytes = md_step_bytes(P, N, 1 / 20, mixed=prec == "mixed")
        out[prec] = {"ms_per_step": ms, "ns_per_step_per_particle": ms * 1e6 / N,
                     "gpairs": P / (ms * 1e-3) / 1e9, "hbm_gbs": step_bytes / (ms * 1e-3) / 1e9,
                     "hbm_frac": step_bytes / (ms * 1e-3) / 1e9 / hbm,
                     "rebuilds": st["rebuilds"], "pairs_half": P,
                     "energy_first_last": [recs[0][1] + recs[0][2], recs[-1][1] + recs[-1][2]],
                     "clocks": cs.summary()}
        del qd, pd
        torch.cuda.empty_cache()
    out["mixed_over_fp64"] = out["fp64"]["ms_per_step"] / out["mixed"]["ms_per_step"]
    return out


def run_batch(args, dist):
    """512 replicas, N log-uniform in [256, 16384] (seeded) -> n = round((N/4)^(1/3))
    FCC cells, rho from {0.5, 0.8, 1.0}, rc 2.5, skin 0.3, MB momenta at T* = 1,
    1,000 mixed velocity-Verlet steps at dt = 0.005 in one batched loop."""
    import torch
    import lj_gpu_gb300 as lj
    from lj_gpu_gb300 import _build
    _build.build()
    dev = torch.device("cuda", dist.local)
    torch.cuda.set_device(dev)
    rng = np.random.default_rng(SEED)
    steps = 1000 if args.steps >= 100 else args.steps
    qs, ps, boxes, offs, specs = [], [], [], [0], []
    for r in range(512):
        ndraw = float(np.exp(rng.uniform(np.log(256), np.log(16384))))
        nc = int(round((ndraw / 4) ** (1 / 3)))
        rho = float(rng.choice([0.5, 0.8, 1.0]))
        q, L = lj.init_fcc(nc, rho, JITTER, SEED + 1000 + r)
        p = lj.init_momenta(q.shape[0], 1.0, SEED + 5000 + r)
        qs.append(q)
        ps.append(p)
        boxes.append([L, L, L])
        offs.append(offs[-1] + q.shape[0])
        specs.append((nc, rho))
    q, p = np.concatenate(qs), np.concatenate(ps)
    qd, pd = torch.from_numpy(q).to(dev), torch.from_numpy(p).to(dev)
    prm = lj.make_md_params(DT, 2.5, 0.3, 1.0, precision="mixed", record_every=steps)
    ctx = lj.Context(dist.local, stream=torch.cuda.current_stream())
    with ClockSampler(dist.local) as cs:
        en, st, shapes = ctx.batch_run(qd, pd, np.array(offs, np.int32), np.array(boxes), prm,
                                       steps)
    ctx.close()
    # half-list pairs within rc + skin per replica, counted once on the device
    pairs = 0
    ctx = lj.Context(dist.local, stream=torch.cuda.current_stream())
    for r in range(512):
        a, b = offs[r], offs[r + 1]
        ctx.build_list(qd[a:b].contiguous(), 2.8, box=boxes[r], kinds=("half",))
        pairs += ctx.list_info("half")[1]
    ctx.close()
    e0 = en[0, :, 0] + en[0, :, 1]
    e1 = en[-1, :, 0] + en[-1, :, 1]
    ms = st["ms_total"] / steps
    hbm, _ = peaks()
    sb = md_step_bytes(pairs, q.shape[0], st["rebuilds"] / max(steps, 1))
    return {"metric": "batched MD G pair-interactions/s (mixed)", "workload": "batch_512",
            "replicas": 512, "N_total": int(q.shape[0]), "N_min": int(min(np.diff(offs))),
            "N_max": int(max(np.diff(offs))), "steps": steps, "ms_per_step": ms,
            "gpairs": pairs / (ms * 1e-3) / 1e9, "pairs_half_within_list_radius": int(pairs),
            "hbm_gbs": sb / (ms * 1e-3) / 1e9, "hbm_frac": sb / (ms * 1e-3) / 1e9 / hbm,
            "rebuilds": st["rebuilds"],
            "size_classes": [{"rows": int(s[0]), "lanes": int(s[1]), "entries_in_flight": int(s[2])}
                             for s in shapes if s[0] > 0],
            "energy_change_rel_max": float(np.max(np.abs(e1 - e0) / np.abs(e0))),
            "clocks": cs.summary(),
            "note": "graph-captured step chunks with flag-guarded on-device rebuilds; per-class "
                    "gather shapes timed at start-up"}


# ---------------------------------------------------------------------------
# CPU legs (oracle: the reference's algorithm restated in C)
# ---------------------------------------------------------------------------
def cpu_baseline(q, L, P, sample_calls=5):
    sys.path.insert(0, str(ROOT / "tests"))
    import oracle_lib as ol
    full = ol.build_list(q, RS, box=L, full=True)
    threads = ol.oracle().lj_or_max_threads()
    p = np.zeros_like(q)
    ol.force_gather_aos(q, p, *full, cl2=RC * RC, dt=DT, box=L, threads=threads)  # warm
    t0 = time.perf_counter()
    ol.force_gather_aos(q, p, *full, cl2=RC * RC, dt=DT, box=L, calls=sample_calls,
                        threads=threads)
    t = time.perf_counter() - t0
    half = ol.build_list(q, RS, box=L)
    t1 = time.perf_counter()
    ol.force_sorted_aos(q, p, *half, cl2=RC * RC, dt=DT, box=L, calls=1)
    t_single = time.perf_counter() - t1
    t2 = time.perf_counter()
    ol.force_sorted_soa(q, p, *half, cl2=RC * RC, dt=DT, box=L, calls=1)
    t_single_soa = time.perf_counter() - t2
    return {"value": P * sample_calls / t / 1e9, "unit": UNIT, "cores": threads,
            "kind": "port", "cpu": cpu_model(), "nproc": os.cpu_count(),
            "sample": f"{sample_calls} full force calls of the 108,000-particle system, "
                      "OpenMP gather over the full list (project-written parallelisation)",
            "single_thread_force_sorted": P / t_single / 1e9,
            "single_thread_force_sorted_soa": P / t_single_soa / 1e9}


def cpu_model():
    """The host CPU as lscpu names it (architecture and model)."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
    except (OSError, subprocess.SubprocessError):
        out = ""
    info = {}
    for line in out.splitlines():
        k, _, v = line.partition(":")
        info[k.strip()] = v.strip()
    parts = [info.get("Architecture"), info.get("Vendor ID"), info.get("Model name")]
    return ", ".join(x for x in parts if x) or None


def run_reference(args, dist):
    if dist.rank != 0:
        return None
    sys.path.insert(0, str(ROOT / "tests"))
    import oracle_lib as ol
    q, L = ol.init_fcc_periodic(NCELL, DENSITY, JITTER, SEED)
    full = ol.build_list(q, RS, box=L, full=True)
    half = ol.build_list(q, RS, box=L)
    P = len(half[2])
    threads = ol.oracle().lj_or_max_threads()
    p = np.zeros_like(q)
    for _ in range(args.warmup):
        ol.force_gather_aos(q, p, *full, cl2=RC * RC, dt=DT, box=L, threads=threads)
    t0 = time.perf_counter()
    ol.force_gather_aos(q, p, *full, cl2=RC * RC, dt=DT, box=L, calls=args.steps,
                        threads=threads)
    t = time.perf_counter() - t0
    v = P * args.steps / t / 1e9
    return {
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": dist.world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": t / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic",
        "config": {"workload": WORKLOAD, "N": q.shape[0], "pairs_half": P,
                   "step": "one force call", "parallelism": "host cores"},
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                         "cpu": cpu_model(), "nproc": os.cpu_count(),
                         "sample": "every step is one full force call of the workload "
                                   "(C restatement of the reference routine, OpenMP gather)"},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def main():
    args = parse()
    if args.impl == "reference":
        dist = Dist("gloo")
        line = run_reference(args, dist)
    else:
        dist = Dist("nccl")
        if args.workload == "precision_1m":
            line = run_precision(args, dist)
        elif args.workload == "large_8m":
            line = run_large(args, dist)
        elif args.workload == "batch_512":
            line = run_batch(args, dist)
        else:
            line = run_ours(args, dist, 1.0 if args.workload == "rho1_108k" else DENSITY)
    if dist.rank == 0 and line is not None:
        print(json.dumps(line))
    dist.close()


if __name__ == "__main__":
    main()
