"""Regenerates the golden fixtures in this directory from the reference itself.

    python tests/golden/make_golden.py --ref <reference checkout>

Needs the reference sources (read-only) and an x86-64 host: it builds the
reference's own cpu_ref routines with oracle/Makefile (`make ref`, outputs in
oracle/_ref/, never committed) and runs them on small inputs.  Each reference
run happens in a fresh process, because cpu_ref keeps its state (and its jitter
generator, a function-local static) in globals.

Outputs (all committed):
  ref_density0.5.dat, ref_density1.dat   copies of the reference's ref_data/
                                          golden prints (10 rows of p, %.10f)
  cpuref_rho0.5_L10.npz   the reference's own init() with L = 10 (N = 500,
                          rho = 0.5, open box), its makepair()/sortpair() list
                          and p after 100 calls of every AoS and SoA routine
  cpuref_rho1_L8.npz      rho = 1.0 FCC (N = 500) from the oracle's restatement
                          of init() (pinned bitwise to the reference at rho = 0.5),
                          the reference's makepair()/sortpair() list and p after
                          100 calls of the reference routines
"""
from __future__ import annotations

import argparse
import multiprocessing as mp
import shutil
import subprocess
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT / "tests"))

AOS_ROUTINES = ["pair", "sorted", "next", "intrin", "intrin_mat_transpose", "sorted_z",
                "sorted_z_intrin"]
SOA_ROUTINES = ["pair", "sorted", "next", "intrin"]
CALLS = 100


def _run_reference(layout: str, q: np.ndarray | None, box_len: float, out):
    import oracle_lib as ol
    R = ol.load_ref(layout)
    if q is None:
        n = R.ref_init(box_len)
        q = np.zeros((n, 4))
        R.ref_get_positions(q)
    else:
        n = q.shape[0]
        R.ref_set_positions(n, np.ascontiguousarray(q))
    npairs = R.ref_makepair()
    R.ref_sortpair()
    npp = np.zeros(n, np.int32)
    ptr = np.zeros(n, np.int32)
    lst = np.zeros(npairs, np.int32)
    R.ref_get_csr(npp, ptr, lst)
    ii = np.zeros(npairs, np.int32)
    jj = np.zeros(npairs, np.int32)
    R.ref_get_pairs(ii, jj)
    res = {"q": q, "np": npp, "ptr": ptr, "list": lst, "i": ii, "j": jj}
    for name in (AOS_ROUTINES if layout == "aos" else SOA_ROUTINES):
        R.ref_set_momenta(np.zeros((n, 4)))
        assert R.ref_run(name.encode(), CALLS) == 0, name
        p = np.zeros((n, 4))
        R.ref_get_momenta(p)
        res[f"p_{layout}_{name}"] = p
    out.put(res)


def run_reference(layout, q, box_len):
    ctx = mp.get_context("spawn")
    qu = ctx.Queue()
    pr = ctx.Process(target=_run_reference, args=(layout, q, box_len, qu))
    pr.start()
    res = qu.get()
    pr.join()
    assert pr.exitcode == 0
    return res


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", required=True, help="the reference checkout")
    a = ap.parse_args()
    ref = Path(a.ref)
    subprocess.run(["make", "-s", "-C", str(ROOT / "oracle"), "ref", f"REF={ref}"], check=True)
    for src, dst in (("density0.5.dat", "ref_density0.5.dat"), ("density1.dat",
                                                               "ref_density1.dat")):
        shutil.copyfile(ref / "ref_data" / src, HERE / dst)

    # reference init(), rho = 0.5 compiled in, L = 10 -> 5^3 cells, N = 500
    aos = run_reference("aos", None, 10.0)
    soa = run_reference("soa", aos["q"], 10.0)
    for k in ("np", "ptr", "list"):
        assert np.array_equal(aos[k], soa[k])
    fx = dict(aos)
    fx.update({k: v for k, v in soa.items() if k.startswith("p_")})
    fx["meta"] = np.array([0.5, 10.0, 9.0, 0.001, 3.3, CALLS])
    np.savez_compressed(HERE / "cpuref_rho0.5_L10.npz", **fx)

    # rho = 1: positions from the oracle restatement of init()
    import oracle_lib as ol
    q1 = ol.init_reference(1.0, 8.0)
    aos1 = run_reference("aos", q1, 8.0)
    soa1 = run_reference("soa", q1, 8.0)
    fx1 = dict(aos1)
    fx1.update({k: v for k, v in soa1.items() if k.startswith("p_")})
    fx1["meta"] = np.array([1.0, 8.0, 9.0, 0.001, 3.3, CALLS])
    np.savez_compressed(HERE / "cpuref_rho1_L8.npz", **fx1)
    for f in sorted(HERE.iterdir()):
        print(f.name, f.stat().st_size)


if __name__ == "__main__":
    main()
