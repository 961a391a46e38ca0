"""Summaries of ncu captures in the text form kept beside the kernels' numbers.

Two inputs, both ncu CSV written on the GPU machine and read anywhere:

* a report's raw page (``ncu -i <report>.ncu-rep --page raw --csv``, or a
  ``--metrics ... --csv`` capture): one summary block per captured launch
  with the metrics named in METRICS, and a ``traffic_bytes_per_launch`` line
  (DRAM read + write) that bench.py reads back;
* a launch list (``ncu --metrics gpu__time_duration.sum --csv``): per kernel
  its launches, total time, average time and share of the listed time.

Usage::

    python -m lj_gpu_gb300.ncu_summary raw REPORT.csv [--kernel REGEX] [--title T]
    python -m lj_gpu_gb300.ncu_summary launches LAUNCHES.csv [--skip N]
"""
from __future__ import annotations

import argparse
import csv
import io
import re
import sys
from collections import OrderedDict

# the metrics a kernel summary reports, in this order (absent ones are skipped)
METRICS = [
    "Kernel Name",
    "launch__grid_size",
    "launch__block_size",
    "launch__registers_per_thread",
    "gpu__time_duration.sum",
    "dram__bytes_read.sum",
    "dram__bytes_write.sum",
    "gpu__dram_throughput.avg.pct_of_peak_sustained_elapsed",
    "lts__t_sector_hit_rate.pct",
    "l1tex__t_sector_hit_rate.pct",
    "l1tex__data_pipe_lsu_wavefronts.avg.pct_of_peak_sustained_elapsed",
    "l1tex__t_sectors_pipe_lsu_mem_global_op_ld.sum",
    "l1tex__t_requests_pipe_lsu_mem_global_op_ld.sum",
    "sm__throughput.avg.pct_of_peak_sustained_elapsed",
    "smsp__issue_active.avg.pct_of_peak_sustained_active",
    "sm__warps_active.avg.pct_of_peak_sustained_active",
    "launch__occupancy_limit_registers",
    "sm__pipe_fma_cycles_active.avg.pct_of_peak_sustained_active",
    "sm__pipe_alu_cycles_active.avg.pct_of_peak_sustained_active",
    "sm__pipe_fp64_cycles_active.avg.pct_of_peak_sustained_active",
    "sm__pipe_tensor_cycles_active.avg.pct_of_peak_sustained_active",
    "smsp__inst_executed.sum",
    "smsp__thread_inst_executed.sum",
    "smsp__average_warps_issue_stalled_long_scoreboard_per_issue_active.ratio",
    "smsp__average_warps_issue_stalled_short_scoreboard_per_issue_active.ratio",
    "smsp__average_warps_issue_stalled_wait_per_issue_active.ratio",
    "smsp__average_warps_issue_stalled_math_pipe_throttle_per_issue_active.ratio",
    "smsp__average_warps_issue_stalled_not_selected_per_issue_active.ratio",
    "smsp__average_warps_issue_stalled_tex_throttle_per_issue_active.ratio",
    "smsp__average_warps_issue_stalled_barrier_per_issue_active.ratio",
]

_SCALE = {"byte": 1.0, "Kbyte": 1e3, "Mbyte": 1e6, "Gbyte": 1e9, "Tbyte": 1e12,
          "KB": 1e3, "MB": 1e6, "GB": 1e9}
_TIME = {"ns": 1e-3, "nsecond": 1e-3, "us": 1.0, "usecond": 1.0, "ms": 1e3, "msecond": 1e3,
         "s": 1e6, "second": 1e6}


def _rows(text):
    """CSV rows of an ncu log, skipping the lines ncu prints before the table."""
    lines = [l for l in text.splitlines() if l.startswith('"')]
    return list(csv.reader(io.StringIO("\n".join(lines))))


def _number(v):
    return float(v.replace(",", ""))


def launches_raw(text):
    """Launches of a report's raw page or of a long-form metrics capture, as
    a list of OrderedDict metric -> (value, unit)."""
    rows = _rows(text)
    if not rows:
        return []
    head = rows[0]
    if "Metric Name" in head:  # long form: one row per (launch, metric)
        ki, mi, vi, ui = (head.index(k) for k in ("ID", "Metric Name", "Metric Value",
                                                  "Metric Unit"))
        kn = head.index("Kernel Name")
        out = OrderedDict()
        for r in rows[1:]:
            d = out.setdefault(r[ki], OrderedDict([("Kernel Name", (r[kn], ""))]))
            d[r[mi]] = (r[vi], r[ui])
        return list(out.values())
    # raw page: a header row, a units row, then one row per launch
    units = rows[1] if len(rows) > 1 else [""] * len(head)
    out = []
    for r in rows[2:]:
        out.append(OrderedDict((h, (v, u)) for h, v, u in zip(head, r, units)))
    return out


def summarise_launch(d):
    """The summary lines of one launch, and its DRAM bytes (or None)."""
    lines = []
    for m in METRICS:
        if m in d:
            v, u = d[m]
            lines.append(f"- `{m}`: {v}{(' ' + u) if u else ''}")
    traffic = None
    try:
        rd, ru = d["dram__bytes_read.sum"]
        wr, wu = d["dram__bytes_write.sum"]
        traffic = _number(rd) * _SCALE.get(ru, 1.0) + _number(wr) * _SCALE.get(wu, 1.0)
    except (KeyError, ValueError):
        pass
    return lines, traffic


def summarise_raw(text, kernel=None, title=None):
    out = []
    if title:
        out.append(f"# {title}\n")
    for d in launches_raw(text):
        name = d.get("Kernel Name", ("", ""))[0]
        if kernel and not re.search(kernel, name):
            continue
        lines, traffic = summarise_launch(d)
        out.extend(lines)
        if traffic is not None:
            out.append("")
            out.append(f"traffic_bytes_per_launch: {traffic:.0f}")
        out.append("")
    return "\n".join(out)


def summarise_launches(text, skip=0):
    """Per kernel: launches, total and average device time, share."""
    rows = _rows(text)
    if not rows:
        return ""
    head = rows[0]
    kn, mi, vi, ui = (head.index(k) for k in ("Kernel Name", "Metric Name", "Metric Value",
                                              "Metric Unit"))
    agg = OrderedDict()
    seen = 0
    for r in rows[1:]:
        if r[mi] != "gpu__time_duration.sum":
            continue
        seen += 1
        if seen <= skip:
            continue
        us = _number(r[vi]) * _TIME.get(r[ui], 1.0)
        name = r[kn].split("(")[0]
        a = agg.setdefault(name, [0, 0.0])
        a[0] += 1
        a[1] += us
    total = sum(v[1] for v in agg.values()) or 1.0
    out = ["| kernel | launches | total ms | avg us | share |", "|---|---|---|---|---|"]
    for name, (n, us) in sorted(agg.items(), key=lambda x: -x[1][1]):
        out.append(f"| `{name}` | {n} | {us / 1e3:.3f} | {us / n:.1f} | {100 * us / total:.1f} % |")
    out.append(f"| total | {sum(v[0] for v in agg.values())} | {total / 1e3:.3f} | | 100 % |")
    return "\n".join(out)


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    sub = ap.add_subparsers(dest="cmd", required=True)
    a = sub.add_parser("raw")
    a.add_argument("csv")
    a.add_argument("--kernel")
    a.add_argument("--title")
    b = sub.add_parser("launches")
    b.add_argument("csv")
    b.add_argument("--skip", type=int, default=0)
    args = ap.parse_args(argv)
    text = open(args.csv).read()
    if args.cmd == "raw":
        sys.stdout.write(summarise_raw(text, args.kernel, args.title) + "\n")
    else:
        sys.stdout.write(summarise_launches(text, args.skip) + "\n")


if __name__ == "__main__":
    main()
