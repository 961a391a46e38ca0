#!/usr/bin/env python
"""Benchmark of the Lennard-Jones neighbour-list force path on GB300.

Default workload (md_8m): the large single system -- FCC 126^3 cells x 4 =
8,001,504 particles, rho = 1, periodic cubic box L = (N / rho)^(1/3) =
200.0, jitter U[-0.05, 0.05) per coordinate from mt19937_64(20240601),
Maxwell-Boltzmann momenta at T* = 1, cutoff 3.0, skin 0.3 (list radius 3.3),
velocity Verlet at dt = 0.005 with the neighbour list rebuilt on the device
every 20 steps.  Mixed precision and plain FP64 run back to back from the
same initial state, each in its own context.

A step is one MD step (drift, guarded rebuild, force kick).  W warm-up
steps, then K steps timed with CUDA events on the engine's stream, bracketed
by a barrier and a device synchronize.  `value` = P_half / t_step / 1e9 in
G pair-interactions/s, P_half = i<j pairs within the list radius at the last
build (the reference's count).  The working set (list rows 9.2 GB, positions
and images 0.5 GB) is far larger than L2, so no flush is needed.  The force
errors (per-particle max and RMS relative |dF| / |F|, and max |dF| / rms |F|)
compare the mixed force of the final MD positions with the oracle's FP64
force over the same list.

e2e: per step, the pinned host q and p copied to the device, lj_md_run over
20 steps (one rebuild period, including its list build), q and p copied back.

--impl reference times the reference's CPU force routine restated in C (the
oracle; gather over the full list on every host core, project-written
OpenMP -- the reference itself is single-threaded) on the same 8M system, one
sixteenth of the rows per step.

Other workloads (--workload): rho0.5_108k / rho1_108k (one force call of the
108,000-particle comparison cases, every variant), precision_1m (1,000 MD
steps at 1,000,188 particles with force errors every 100 steps) and
batch_512 (512 replicas in one batched MD loop).
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


def force_workload(n, density, box):
    return (f"LJ force call, FCC {n:,} particles, rho={density:g}, periodic L={box:.4g}, "
            "rc=3.0, search 3.3, i-sorted int32 CSR, dt=0.005")


WORKLOAD = force_workload(4 * NCELL ** 3, DENSITY, 60.0)
NCELL_8M, REBUILD_8M, E2E_CHUNK = 126, 20, 20
NCELL_MD = {"md_8m": 126, "md_1m": 63}
PAIRS_HALF_1M = 73_261_786  # half-list pairs of the md_1m capture under profiles/


def md_workload(ncell):
    n = 4 * ncell ** 3
    return (f"LJ MD step, FCC {n:,} particles, rho=1, periodic L={n ** (1 / 3):.0f}, MB "
            "momenta T*=1, rc=3.0, skin 0.3, device list rebuild every 20 steps, velocity "
            "Verlet dt=0.005; mixed and FP64 back to back")


WORKLOAD_8M = md_workload(NCELL_8M)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=500)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--kick-lanes", type=int, default=0,
                    help="MD workloads: lanes per row of the mixed gather kick (0: default)")
    ap.add_argument("--l2-window", type=float, default=0.0,
                    help="force-call workloads: run on a side stream with an L2 persistence "
                         "window of this hit ratio over the position image "
                         "(lj_ctx_set_l2_window)")
    ap.add_argument("--chunk-graphs", action="store_true",
                    help="MD workloads: launch the captured step chunks from the host "
                         "instead of the persistent WHILE-node graph, so that a profiler "
                         "can capture the step's kernels one by one")
    ap.add_argument("--no-autotune", action="store_true",
                    help="time the 'auto' variants with the engine's default launch shapes "
                         "(what the tuner picks on this workload) instead of tuning first; "
                         "for runs under a profiler, whose per-launch overhead swamps the "
                         "tuner's timings")
    ap.add_argument("--shape", action="append", default=[],
                    help="extra mixed AoS gather variant KERNEL,LANES,UNROLL (e.g. 3,4,2 for "
                         "the cell-tiled kernel), timed beside the default variants")
    ap.add_argument("--workload", default="md_8m",
                    choices=["md_8m", "md_1m", "rho1_1m", "rho0.5_108k", "rho1_108k", "precision_1m", "batch_512"],
                    help="md_8m: 8,001,504-particle MD, mixed and FP64 back to back (the "
                         "headline); rho0.5_108k / rho1_108k: one force call of the 108,000-"
                         "particle cases, every variant; md_1m: md_8m's step at 1,000,188 "
                         "particles (the size the kernel profiles are captured on); rho1_1m: "
                         "every force variant at 1,000,188 particles, rho = 1; precision_1m: 1,000,188-particle "
                         "mixed MD with force errors every 100 steps; batch_512: 512 "
                         "replicas of uneven N in one mixed MD loop")
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
def run_ours(args, dist, density=DENSITY, ncell=NCELL):
    import torch
    import lj_gpu_gb300 as lj
    from lj_gpu_gb300 import _build

    _build.build()
    dev = torch.device("cuda", dist.local)
    torch.cuda.set_device(dev)
    stream = torch.cuda.current_stream()
    q, L = lj.init_fcc(ncell, density, JITTER, SEED)
    N = q.shape[0]
    qd = torch.from_numpy(q).to(dev)
    qs = [torch.from_numpy(np.ascontiguousarray(q[:, d])).to(dev) for d in range(3)]
    ctx = lj.Context(dist.local, stream=stream)
    if args.l2_window:
        ctx.set_l2_window(args.l2_window)
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

    # force error of the mixed default (and the FP64 scatter) against the
    # oracle's FP64 force_sorted over the device-built half list
    ferr = None
    if dist.rank == 0 and not args.no_cpu_baseline:
        sys.path.insert(0, str(ROOT / "tests"))
        import oracle_lib as ol
        half = ctx.get_list_csr("half")
        po = ol.force_sorted_aos(q, np.zeros_like(q), *half, cl2=RC * RC, dt=1.0, box=L)
        ferr = {}
        for fprec in ("mixed", "fp64"):
            pm = torch.zeros_like(qd)
            ctx.force_aos(qd, pm, lj.make_opts(dt=1.0, cl2=RC * RC, box=L, precision=fprec))
            ferr[fprec] = per_particle_errors(pm[:, :3].cpu().numpy(), po[:, :3])
        ferr["reference"] = "oracle FP64 force_sorted, default launch shapes"
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
        tot = calc = 0.0
        for _ in range(args.e2e_steps):
            ms_total, ms_calc = ctx.measure_aos(hq, hp, opts, calls=100)
            tot += ms_total
            calc += ms_calc
        dist.barrier()
        t_step = dist.max(tot / args.e2e_steps / 1e3, dev)
        h2d = hq.numel() * 8 * 2 + (h_np.numel() + h_ptr.numel() + h_lst.numel()) * 4
        e2e = {"value": dist.world * P * 100 / t_step / 1e9, "unit": UNIT,
               "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(hp.numel() * 8),
               "step": "lj_measure_aos: H2D q,p,CSR + 100 force calls + D2H p",
               "ms_per_step": t_step * 1e3, "force_calls_ms": calc / args.e2e_steps}

    hbm, peak_kind = peaks()
    alg = pair_kernel_bytes(method, layout, P, N)
    achieved = alg / (t_pair_ms * 1e-3) / 1e9
    # DRAM traffic per launch from a committed ncu capture of this kernel on
    # this workload: the 108,000-particle captures under profiles/ are of the
    # FP32-term gather (LJ_PREC_MIXED_FP32), not of the two-float default
    # timed here, so this line carries none
    prof = f"force_mixed_gather_{layout}_108k_rho0.5.txt"
    traffic = None
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
    # the FP64 pipe's busy fraction comes from the committed ncu capture of
    # the FP64 scatter on this workload (a counter, not a model)
    fp_prof = "force_fp64_scatter_108k_rho0.5.txt"
    fp_pipe = (profiled_metric(fp_prof, "sm__pipe_fp64_cycles_active.avg.pct_of_peak_sustained_active")
               if density == DENSITY and fp_m == "scatter" else None)
    fp64 = {"value": fp["gpairs"], "variant": best_fp64, "ms_per_call": fp["s_per_call"] * 1e3,
            "pair_kernel_ms": t_pair64_ms,
            "hbm_frac": algorithmic_bytes(fp_m, fp_l, P, N) / fp["s_per_call"] / 1e9 / hbm,
            "fp64_pipe_frac": fp_pipe / 100 if fp_pipe is not None else None,
            "fp64_pipe_frac_source": f"profiles/{fp_prof}" if fp_pipe is not None else None,
            "mixed_over_fp64": head["gpairs"] / fp["gpairs"]}

    cpu = None
    if dist.rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_baseline(q, L, P, sample_calls=5 if density <= 0.5 else 2)

    line = {
        "metric": METRIC, "value": dist.world * P / head["s_per_call"] / 1e9, "unit": UNIT,
        "n_gpus": dist.world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": head["s_per_call"] * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 two-float pair math, f64 q/p",
        "data": "synthetic",
        "config": {"workload": force_workload(N, density, L), "N": N, "pairs_half": P, "pairs_full": P_full,
                   "max_row_half": max_half, "max_row_full": max_full, "box": L,
                   "variant": best_mixed, "step": "one force call",
                   "l2": "flushed before every timed call (512 MiB write)",
                   "list_build_s": t_build, "parallelism": f"replicas x{dist.world}"},
        "e2e": e2e, "roofline": roofline, "cpu_baseline": cpu, "fp64": fp64,
        "force_error": ferr,
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
def force_errors(torch, lj, L, qd, rs=RS, oracle=False):
    """Mixed against FP64 forces on the same positions and device-built list:
    the engine's FP64 path (held to 1e-12 of the oracle by the parity tests),
    and with `oracle` also the oracle's FP64 gather on the host cores
    (`vs_oracle`)."""
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
    res = {"max_rel": float(per.max()), "rms_rel": float(torch.sqrt(torch.mean(per * per))),
           "max_rel_rms": float(d.max() / rms), "global_rel": float(torch.linalg.norm(d) /
                                                                    torch.linalg.norm(r))}
    if oracle:
        sys.path.insert(0, str(ROOT / "tests"))
        import oracle_lib as ol
        npp, ptr_, lst = ctx.get_list_csr("full")
        qh = qd.cpu().numpy()
        po = np.zeros_like(qh)
        ol.force_gather_aos(qh, po, npp, ptr_, lst, cl2=RC * RC, dt=1.0, box=L,
                            threads=ol.oracle().lj_or_max_threads())
        res["vs_oracle"] = per_particle_errors(out["mixed"].cpu().numpy(), po[:, :3])
    ctx.close()
    return res


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
    errors = [dict(step=0, **force_errors(torch, lj, L, qd, oracle=not args.no_cpu_baseline))]
    ctx = lj.Context(dist.local, stream=torch.cuda.current_stream())
    prm = lj.make_md_params(DT, RC, RS - RC, L, precision="mixed", record_every=100,
                            chunk_graphs=args.chunk_graphs)
    records, ms, rebuilds, clock_samples = [], 0.0, 0, []
    for seg in range(10):
        with ClockSampler(dist.local) as cs:
            recs, st = ctx.md_run(qd, pd, prm, 100)
        clock_samples.append(cs.summary())
        ms += st["ms_total"]
        rebuilds += st["rebuilds"]
        records += [(r[0] + 100 * seg, r[1], r[2]) for r in recs if seg == 0 or r[0] > 0]
        errors.append(dict(step=100 * (seg + 1),
                           **force_errors(torch, lj, L, qd, oracle=not args.no_cpu_baseline)))
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
            "max_rel_force_error": max(e["max_rel"] for e in errors),
            "max_rel_force_error_vs_oracle": max((e["vs_oracle"]["max_rel"] for e in errors
                                                  if "vs_oracle" in e), default=None),
            "max_rel_rms_force_error": max(e["max_rel_rms"] for e in errors),
            "global_rel_force_error": max(e["global_rel"] for e in errors),
            "force_errors": errors, "energy_drift_rel": drift,
            "energies": [{"step": r[0], "kinetic": r[1], "potential": r[2]} for r in records],
            "clocks": merge_clocks(clock_samples),
            "note": "the cut, unshifted potential (the reference's) jumps when pairs cross "
                    "rc, so total energy drifts in FP64 too; force errors are against the "
                    "engine's FP64 path and (vs_oracle) the oracle's FP64 gather on the same "
                    "positions and list"}


def per_particle_errors(test, ref):
    """Relative force errors of `test` against `ref` (N x 3 arrays): the
    per-particle max and RMS of |dF_i| / |F_i|, and max |dF_i| / rms |F|."""
    d = np.linalg.norm(test - ref, axis=1)
    r = np.linalg.norm(ref, axis=1)
    per = d / np.where(r > 0, r, np.inf)
    return {"max_rel": float(per.max()), "rms_rel": float(np.sqrt(np.mean(per * per))),
            "max_rel_rms": float(d.max() / np.sqrt(np.mean(r * r)))}


def run_md8m(args, dist):
    """The large single system, mixed then FP64 from the same initial state
    (see the module docstring)."""
    import torch
    import lj_gpu_gb300 as lj
    from lj_gpu_gb300 import _build
    _build.build()
    dev = torch.device("cuda", dist.local)
    torch.cuda.set_device(dev)
    stream = torch.cuda.current_stream()
    ncell = NCELL_MD[args.workload]
    q, L = lj.init_fcc(ncell, 1.0, JITTER, SEED)
    N = q.shape[0]
    p0 = lj.init_momenta(N, 1.0, SEED + 1)
    K, W = args.steps, args.warmup
    hbm, peak_kind = peaks()
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    runs, final_q = {}, {}
    for prec in ("mixed", "fp64"):
        qd, pd = torch.from_numpy(q).to(dev), torch.from_numpy(p0).to(dev)
        ctx = lj.Context(dist.local, stream=stream)
        prm = lj.make_md_params(DT, RC, RS - RC, L, precision=prec, rebuild_every=REBUILD_8M,
                                chunk_graphs=args.chunk_graphs, kick_lanes=args.kick_lanes)
        ctx.md_run(qd, pd, prm, W, max_records=0)  # warm-up: its own build + W steps
        ev = (torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
        torch.cuda.synchronize()
        dist.barrier()
        with ClockSampler(dist.local) as cs:
            ev[0].record(stream)
            _, st = ctx.md_run(qd, pd, prm, K, max_records=0)
            ev[1].record(stream)
            torch.cuda.synchronize()
        dist.barrier()
        t_step = dist.max(ev[0].elapsed_time(ev[1]) / K / 1e3, dev)
        # the list at the final positions: its pair count, and the pair
        # kernel of a force call over it timed on the engine's stream (the MD
        # step runs the same kernel over padded rows inside a graph)
        ctx.build_list(qd, RS, box=L)
        _, P, _ = ctx.list_info("half")
        opts = lj.make_opts(dt=DT, cl2=RC * RC, box=L, precision=prec,
                            method="gather" if prec == "mixed" else "scatter")
        pk = torch.zeros_like(qd)
        for _ in range(3):
            flush.add_(1.0)
            ctx.force_aos(qd, pk, opts)
        torch.cuda.synchronize()
        ctx.set_timing(True)
        for _ in range(10):
            flush.add_(1.0)
            ctx.force_aos(qd, pk, opts)
        torch.cuda.synchronize()
        tm = ctx.get_timing()
        ctx.set_timing(False)
        runs[prec] = {"t_step": t_step, "P": P, "stats": st, "clocks": cs.summary(),
                      "pair_ms": tm[1] / tm[3], "image_ms": tm[0] / tm[3]}
        if prec == "mixed":
            final_q["mixed"] = qd
            keep_ctx = ctx
        else:
            ctx.close()
        del pd, pk
    ctx = keep_ctx
    qd = final_q["mixed"]
    P = runs["mixed"]["P"]

    # forces of the final mixed positions: mixed and FP64 engine paths, and
    # the oracle's FP64 gather over the same (device-built) full list
    def force_of(prec):
        pz = torch.zeros_like(qd)
        ctx.force_aos(qd, pz, lj.make_opts(dt=1.0, cl2=RC * RC, box=L, precision=prec,
                                            method="gather" if prec == "mixed" else "scatter"))
        torch.cuda.synchronize()
        return pz[:, :3].cpu().numpy()
    f_mixed, f_fp64 = force_of("mixed"), force_of("fp64")
    errors = {"vs_engine_fp64": per_particle_errors(f_mixed, f_fp64)}
    cpu = None
    if dist.rank == 0 and not args.no_cpu_baseline:
        sys.path.insert(0, str(ROOT / "tests"))
        import oracle_lib as ol
        npp, ptr_, lst = ctx.get_list_csr("full")
        qh = qd.cpu().numpy()
        threads = ol.oracle().lj_or_max_threads()
        po = np.zeros_like(qh)
        t0 = time.perf_counter()
        ol.force_gather_aos(qh, po, npp, ptr_, lst, cl2=RC * RC, dt=1.0, box=L, threads=threads)
        t_cpu = time.perf_counter() - t0
        errors["vs_oracle"] = per_particle_errors(f_mixed, po[:, :3])
        errors["fp64_vs_oracle"] = per_particle_errors(f_fp64, po[:, :3])
        cpu = {"value": P / t_cpu / 1e9, "unit": UNIT, "cores": threads, "kind": "port",
               "cpu": cpu_model(), "nproc": os.cpu_count(), "seconds": t_cpu,
               "sample": f"one full-list force call of the {N:,}-particle system at the "
                         "final mixed MD positions (OpenMP gather over every host core, "
                         "project-written parallelisation); value counts its P_half pairs"}
        del npp, ptr_, lst
    err = errors.get("vs_oracle", errors["vs_engine_fp64"])

    # e2e: pinned host state in, the MD loop over one rebuild period, state out
    # (lj_md_run_host: the copy of p in runs beside the initial list build,
    # the copy of q out beside the final half kick)
    e2e = None
    if args.e2e_steps > 0:
        hq = torch.from_numpy(q).pin_memory()
        hp = torch.from_numpy(p0).pin_memory()
        prm = lj.make_md_params(DT, RC, RS - RC, L, precision="mixed", rebuild_every=REBUILD_8M)

        def e2e_step():
            # host q, p in and out through the host entry (page-locked, updated
            # in place: each step continues the trajectory)
            ctx.md_run_host(hq, hp, prm, E2E_CHUNK, max_records=0)
        e2e_step()  # warm-up
        dist.barrier()
        t0 = time.perf_counter()
        for _ in range(args.e2e_steps):
            e2e_step()
        t_e = dist.max((time.perf_counter() - t0) / args.e2e_steps, dev)
        nbytes = hq.numel() * 8 + hp.numel() * 8
        e2e = {"value": dist.world * P * E2E_CHUNK / t_e / 1e9, "unit": UNIT,
               "h2d_bytes_per_step": int(nbytes), "d2h_bytes_per_step": int(nbytes),
               "ms_per_step": t_e * 1e3,
               "step": f"lj_md_run_host: pinned host q, p -> device, {E2E_CHUNK} MD steps (the "
                       "initial list build included), q, p -> host; host wall clock",
               "md_steps_per_step": E2E_CHUNK}
    ctx.close()

    mx, fp = runs["mixed"], runs["fp64"]
    alg = pair_kernel_bytes("gather", "aos", P, N)
    prof = "force_mixed_seg_gather_md_1m.txt"
    tr1m = profiled_traffic(prof)
    # the 1M capture's DRAM bytes scaled to this launch by the list entries
    # (traffic grows with the entries; the image and p terms scale with N alike)
    traffic = tr1m * (P / PAIRS_HALF_1M) if tr1m else None
    roofline = {"bound": "hbm", "achieved": alg / (mx["pair_ms"] * 1e-3) / 1e9, "peak": hbm,
                "unit": "GB/s", "frac": alg / (mx["pair_ms"] * 1e-3) / 1e9 / hbm,
                "traffic": traffic,
                "traffic_source": (f"profiles/{prof}, scaled by list entries from the 1,000,188-"
                                   "particle capture") if traffic else None,
                "peak_kind": peak_kind,
                "kernel": "k_gather_mixed_seg (FP32 far part, two-float near part; one lane "
                          "per row, 4 entries in flight), timed in force calls at the final MD "
                          "positions",
                "algorithmic_bytes_per_launch": alg, "kernel_ms": mx["pair_ms"],
                "position_image_ms": mx["image_ms"],
                "md_step_bytes": md_step_bytes(P, N, 1 / REBUILD_8M),
                "md_step_gbs": md_step_bytes(P, N, 1 / REBUILD_8M) / mx["t_step"] / 1e9,
                "md_step_frac": md_step_bytes(P, N, 1 / REBUILD_8M) / mx["t_step"] / 1e9 / hbm}
    # what bounds the kernel instead of HBM, from the same capture: issue, the
    # ALU pipe and the L1 data pipe
    for key, metric in (("issue_active_frac", "smsp__issue_active.avg.pct_of_peak_sustained_active"),
                        ("alu_pipe_frac", "sm__pipe_alu_cycles_active.avg.pct_of_peak_sustained_active"),
                        ("fma_pipe_frac", "sm__pipe_fma_cycles_active.avg.pct_of_peak_sustained_active"),
                        ("l1_data_pipe_frac",
                         "l1tex__data_pipe_lsu_wavefronts.avg.pct_of_peak_sustained_elapsed")):
        v = profiled_metric(prof, metric)
        if v is not None:
            roofline[key] = v / 100
    roofline["limiter"] = ("instruction issue and the ALU and L1 data pipes (two-float pair "
                           "terms); HBM is not the bound")
    fp_prof = "force_fp64_scatter_md_1m.txt"
    fp_pipe = profiled_metric(fp_prof, "sm__pipe_fp64_cycles_active.avg.pct_of_peak_sustained_active")
    fp64 = {"value": dist.world * fp["P"] / fp["t_step"] / 1e9, "ms_per_step": fp["t_step"] * 1e3,
            "ns_per_particle_step": fp["t_step"] * 1e9 / N,
            "md_step_hbm_gbs": md_step_bytes(fp["P"], N, 1 / REBUILD_8M, mixed=False)
            / fp["t_step"] / 1e9,
            "pairs_half": fp["P"], "pair_kernel_ms": fp["pair_ms"],
            "kernel": "k_scatter_fp64_c (compacted half-list scatter)",
            "md_step_hbm_frac": md_step_bytes(fp["P"], N, 1 / REBUILD_8M, mixed=False)
            / fp["t_step"] / 1e9 / hbm,
            "fp64_pipe_frac": fp_pipe / 100 if fp_pipe is not None else None,
            "fp64_pipe_frac_source": f"profiles/{fp_prof}" if fp_pipe is not None else None,
            "rebuilds": fp["stats"]["rebuilds"], "gpu_launches": fp["stats"]["launches"],
            "clocks": fp["clocks"]}
    line = {
        "metric": METRIC, "value": dist.world * P / mx["t_step"] / 1e9, "unit": UNIT,
        "n_gpus": dist.world, "steps": K, "warmup": W, "ms_per_step": mx["t_step"] * 1e3,
        "ns_per_step": mx["t_step"] * 1e9, "ns_per_particle_step": mx["t_step"] * 1e9 / N,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 two-float pair math, f64 q/p", "data": "synthetic",
        "config": {"workload": md_workload(ncell), "N": N, "box": L, "pairs_half": P,
                   "step": "one MD step (drift, guarded rebuild, force kick)",
                   "rebuild_every": REBUILD_8M, "rebuilds": mx["stats"]["rebuilds"],
                   "l2": "working set (list rows ~9 GB) far larger than L2; no flush",
                   "parallelism": f"replicas x{dist.world}"},
        "force_error": dict(err, reference="oracle FP64 gather" if "vs_oracle" in errors
                            else "engine FP64 path", positions="final mixed MD state"),
        "force_errors": errors,
        "fp64": fp64,
        "mixed_over_fp64": {"md_step": fp["t_step"] / mx["t_step"],
                            "pair_kernel": fp["pair_ms"] / mx["pair_ms"]},
        "e2e": e2e, "roofline": roofline, "cpu_baseline": cpu,
        "clocks": mx["clocks"], "gpu_launches": mx["stats"]["launches"],
        "gpu_launches_note": "kernels of the timed mixed lj_md_run (graph nodes counted by "
                             "the engine)",
    }
    return line


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
    prm = lj.make_md_params(DT, 2.5, 0.3, 1.0, precision="mixed", record_every=steps,
                            chunk_graphs=args.chunk_graphs)
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
    # force errors at the final positions of a sample of replicas (smallest,
    # largest, the first of each density): the engine's mixed force against
    # the oracle's FP64 force_sorted over the same list
    sizes = np.diff(offs)
    sample = sorted({int(np.argmin(sizes)), int(np.argmax(sizes))} |
                    {next(r for r in range(512) if specs[r][1] == rho) for rho in (0.5, 0.8, 1.0)})
    errors = None
    if not args.no_cpu_baseline:
        sys.path.insert(0, str(ROOT / "tests"))
        import oracle_lib as ol
        worst = {"max_rel": 0.0, "rms_rel": 0.0, "max_rel_rms": 0.0}
        for r in sample:
            a, b = offs[r], offs[r + 1]
            qr = qd[a:b].contiguous()
            ctx.build_list(qr, 2.8, box=boxes[r], kinds=("half", "full"))
            half = ctx.get_list_csr("half")
            pm = torch.zeros_like(qr)
            ctx.force_aos(qr, pm, lj.make_opts(dt=1.0, cl2=2.5 * 2.5, box=boxes[r],
                                                precision="mixed", method="gather"))
            qh = qr.cpu().numpy()
            po = ol.force_sorted_aos(qh, np.zeros_like(qh), *half, cl2=2.5 * 2.5, dt=1.0,
                                     box=boxes[r][0])
            e = per_particle_errors(pm[:, :3].cpu().numpy(), po[:, :3])
            worst = {k: max(worst[k], e[k]) for k in worst}
        errors = dict(worst, replicas=sample, reference="oracle FP64 force_sorted",
                      positions="final batched MD state",
                      test="lj_force_aos mixed gather of each sampled replica (the batch "
                           "kernel itself is checked against the oracle's integrator by "
                           "tests/test_batch_gpu.py)")
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
            "force_error": errors,
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
    threads = ol.oracle().lj_or_max_threads()
    if args.workload == "md_8m":
        # the 8,001,504-particle system; a step is the force call over one
        # sixteenth of its rows (a fixed slice, its list built once)
        q, L = ol.init_fcc_periodic(NCELL_8M, 1.0, JITTER, SEED)
        n = q.shape[0]
        row1 = n // 16
        npp, ptr_, lst = ol.build_rows(q, RS, 0, row1, box=L, full=True)
        P = int(npp.sum()) // 2  # the slice's share of the half-list pairs
        p = np.zeros_like(q)
        for _ in range(args.warmup):
            ol.force_gather_rows_aos(q, p, 0, npp, ptr_, lst, cl2=RC * RC, dt=DT, box=L,
                                     threads=threads)
        t0 = time.perf_counter()
        ol.force_gather_rows_aos(q, p, 0, npp, ptr_, lst, cl2=RC * RC, dt=DT, box=L,
                                 calls=args.steps, threads=threads)
        t = time.perf_counter() - t0
        workload, sample = WORKLOAD_8M, (
            f"every step is the force call over rows 0..{row1 - 1} (1/16) of the "
            "8,001,504-particle system, full-list gather (C restatement of the reference "
            "routine, project-written OpenMP); value counts that slice's P_half share")
        config = {"workload": workload, "N": n, "rows_per_step": row1, "pairs_half": P,
                  "step": "force call over 1/16 of the rows", "parallelism": "host cores"}
    else:
        # the system of the chosen workload: 1,000,188 particles at rho 1 for
        # the 1M workloads, 108,000 at rho 1 or 0.5 otherwise (the replica
        # batch has no counterpart in the reference: the 108k force call)
        big = args.workload in ("md_1m", "precision_1m", "rho1_1m")
        ncell = 63 if big else NCELL
        rho = 1.0 if big or args.workload == "rho1_108k" else DENSITY
        q, L = ol.init_fcc_periodic(ncell, rho, JITTER, SEED)
        full = ol.build_list(q, RS, box=L, full=True)
        P = len(full[2]) // 2
        p = np.zeros_like(q)
        for _ in range(args.warmup):
            ol.force_gather_aos(q, p, *full, cl2=RC * RC, dt=DT, box=L, threads=threads)
        t0 = time.perf_counter()
        ol.force_gather_aos(q, p, *full, cl2=RC * RC, dt=DT, box=L, calls=args.steps,
                            threads=threads)
        t = time.perf_counter() - t0
        workload = (md_workload(ncell) if args.workload in NCELL_MD
                    else force_workload(q.shape[0], rho, L))
        sample = ("every step is one full force call of the workload's system (C "
                  "restatement of the reference routine, OpenMP gather)")
        config = {"workload": workload, "N": q.shape[0], "pairs_half": P,
                  "step": "one force call", "parallelism": "host cores"}
    v = P * args.steps / t / 1e9
    return {
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": dist.world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": t / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": config,
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                         "cpu": cpu_model(), "nproc": os.cpu_count(), "sample": sample},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def main():
    args = parse()
    if args.impl == "reference":
        dist = Dist("gloo")
        line = run_reference(args, dist)
    else:
        dist = Dist("nccl")
        if args.workload in NCELL_MD:
            line = run_md8m(args, dist)
        elif args.workload == "precision_1m":
            line = run_precision(args, dist)
        elif args.workload == "batch_512":
            line = run_batch(args, dist)
        else:
            import contextlib
            import torch
            # the L2 window is a stream attribute: a side stream for that run
            side = (torch.cuda.stream(torch.cuda.Stream(device=dist.local)) if args.l2_window
                    else contextlib.nullcontext())
            with side:
                if args.workload == "rho1_1m":
                    line = run_ours(args, dist, 1.0, ncell=63)
                else:
                    line = run_ours(args, dist,
                                    1.0 if args.workload == "rho1_108k" else DENSITY)
            if line is not None and args.l2_window:
                line["config"]["l2_window_hit_ratio"] = args.l2_window
    if dist.rank == 0 and line is not None:
        print(json.dumps(line))
    dist.close()


if __name__ == "__main__":
    main()
