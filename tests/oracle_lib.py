"""ctypes binding of the CPU oracle (oracle/lj_oracle.c) and, where it was
built, of the reference's own cpu_ref routines (oracle/_ref).

Test infrastructure only: the engine never imports this module.
"""
from __future__ import annotations

import ctypes as C
import platform
import re
import subprocess
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent.parent
ORACLE_DIR = ROOT / "oracle"
ORACLE_LIB = ORACLE_DIR / "_build" / "liblj_oracle.so"
REF_AOS = ORACLE_DIR / "_ref" / "libljref_aos.so"
REF_SOA = ORACLE_DIR / "_ref" / "libljref_soa.so"

_dp = np.ctypeslib.ndpointer(np.float64, flags="C")
_ip = np.ctypeslib.ndpointer(np.int32, flags="C")
_V = C.c_void_p

_oracle = None


def build_oracle() -> Path:
    subprocess.run(["make", "-s", "-C", str(ORACLE_DIR)], check=True)
    return ORACLE_LIB


def oracle() -> C.CDLL:
    global _oracle
    if _oracle is None:
        if not ORACLE_LIB.exists() or ORACLE_LIB.stat().st_mtime < (
                ORACLE_DIR / "lj_oracle.c").stat().st_mtime:
            build_oracle()
        L = C.CDLL(str(ORACLE_LIB))
        sig = {
            "lj_or_init_reference": (C.c_int, [C.c_double, C.c_double, _dp, C.c_int]),
            "lj_or_init_fcc_periodic": (C.c_int, [C.c_int, C.c_double, C.c_double, C.c_uint64,
                                                  _dp, C.c_int, C.POINTER(C.c_double)]),
            "lj_or_build_half_brute": (C.c_int64, [_dp, C.c_int, C.c_double, _V, _ip, _ip, _ip,
                                                   C.c_int64]),
            "lj_or_build_list_cells": (C.c_int64, [_dp, C.c_int, C.c_double, _V, C.c_int, _ip,
                                                   _ip, _ip, C.c_int64]),
            "lj_or_csr_to_pairs": (None, [C.c_int, _ip, _ip, _ip, _ip, _ip]),
            "lj_or_force_pair_aos": (None, [_dp, _dp, C.c_int64, _ip, _ip, C.c_double,
                                            C.c_double, _V]),
            "lj_or_force_sorted_aos": (None, [_dp, _dp, C.c_int, _ip, _ip, _ip, C.c_double,
                                              C.c_double, _V]),
            "lj_or_force_sorted_soa": (None, [_dp, _dp, _dp, _dp, _dp, _dp, C.c_int, _ip, _ip,
                                              _ip, C.c_double, C.c_double, _V]),
            "lj_or_build_rows_cells": (C.c_int64, [_dp, C.c_int, C.c_double, _V, C.c_int,
                                                   C.c_int, C.c_int, _ip, _ip, _ip, C.c_int64]),
            "lj_or_force_gather_rows_aos": (None, [_dp, _dp, C.c_int, C.c_int, _ip, _ip, _ip,
                                                   C.c_double, C.c_double, _V, C.c_int]),
            "lj_or_force_gather_aos": (None, [_dp, _dp, C.c_int, _ip, _ip, _ip, C.c_double,
                                              C.c_double, _V, C.c_int]),
            "lj_or_max_threads": (C.c_int, []),
            "lj_or_potential_half": (C.c_double, [_dp, C.c_int, _ip, _ip, _ip, C.c_double, _V]),
            "lj_or_kinetic": (C.c_double, [_dp, C.c_int]),
            "lj_or_drift": (None, [_dp, _dp, C.c_int, C.c_double, _V]),
            "lj_or_mt32_seed": (None, [_V, C.c_uint32]),
            "lj_or_mt32_next": (C.c_uint32, [_V]),
            "lj_or_mt64_seed": (None, [_V, C.c_uint64]),
            "lj_or_mt64_next": (C.c_uint64, [_V]),
        }
        for k, (r, a) in sig.items():
            f = getattr(L, k)
            f.restype, f.argtypes = r, a
        _oracle = L
    return _oracle


def _box(box):
    if box is None:
        return None, None
    b = np.ascontiguousarray(np.broadcast_to(np.asarray(box, np.float64), (3,)))
    return b, b.ctypes.data


# ---------------------------------------------------------------------------
# convenience wrappers
# ---------------------------------------------------------------------------
def init_reference(density=0.5, L=50.0):
    cap = 4 * (int(L / (4.0 / density) ** (1 / 3)) + 1) ** 3
    q = np.zeros((cap, 4))
    n = oracle().lj_or_init_reference(density, L, q, cap)
    return q[:n].copy()


def init_fcc_periodic(ncell, density, jitter=0.05, seed=20240601):
    n = 4 * ncell ** 3
    q = np.zeros((n, 4))
    L = C.c_double()
    got = oracle().lj_or_init_fcc_periodic(ncell, density, jitter, seed, q, n, C.byref(L))
    assert got == n
    return q, L.value


def build_list(q, search, box=None, full=False, cap=None):
    n = q.shape[0]
    cap = cap or max(16, int(n * 200))
    npp = np.zeros(n, np.int32)
    ptr = np.zeros(n, np.int32)
    lst = np.zeros(cap, np.int32)
    b, bp = _box(box)
    e = oracle().lj_or_build_list_cells(np.ascontiguousarray(q), n, search * search, bp,
                                        1 if full else 0, npp, ptr, lst, cap)
    if e < 0:
        raise RuntimeError("oracle list overflow")
    return npp, ptr, lst[:e].copy()


def build_rows(q, search, row0, row1, box=None, full=False, cap=None):
    """Rows [row0, row1) of build_list's list (npp, ptr indexed by i - row0)."""
    n = q.shape[0]
    m = row1 - row0
    cap = cap or max(16, int(m * 200))
    npp = np.zeros(m, np.int32)
    ptr = np.zeros(m, np.int32)
    lst = np.zeros(cap, np.int32)
    b, bp = _box(box)
    e = oracle().lj_or_build_rows_cells(np.ascontiguousarray(q), n, search * search, bp,
                                        1 if full else 0, row0, row1, npp, ptr, lst, cap)
    if e < 0:
        raise RuntimeError("oracle list overflow")
    return npp, ptr, lst[:e].copy()


def force_gather_rows_aos(q, p, row0, npp, ptr, lst, cl2=9.0, dt=0.001, box=None, calls=1,
                          threads=1):
    """The gather over rows [row0, row0 + len(npp)) of a build_rows list."""
    b, bp = _box(box)
    for _ in range(calls):
        oracle().lj_or_force_gather_rows_aos(q, p, row0, row0 + len(npp), npp, ptr, lst, cl2,
                                             dt, bp, threads)
    return p


def build_half_brute(q, search, box=None):
    n = q.shape[0]
    cap = max(16, n * 200)
    npp = np.zeros(n, np.int32)
    ptr = np.zeros(n, np.int32)
    lst = np.zeros(cap, np.int32)
    b, bp = _box(box)
    e = oracle().lj_or_build_half_brute(np.ascontiguousarray(q), n, search * search, bp, npp,
                                        ptr, lst, cap)
    return npp, ptr, lst[:e].copy()


def csr_to_pairs(npp, ptr, lst):
    ii = np.zeros(len(lst), np.int32)
    jj = np.zeros(len(lst), np.int32)
    oracle().lj_or_csr_to_pairs(len(npp), npp, ptr, np.ascontiguousarray(lst, np.int32), ii, jj)
    return ii, jj


def force_sorted_aos(q, p, npp, ptr, lst, cl2=9.0, dt=0.001, box=None, calls=1):
    b, bp = _box(box)
    for _ in range(calls):
        oracle().lj_or_force_sorted_aos(q, p, q.shape[0], npp, ptr, lst, cl2, dt, bp)
    return p


def velocity_verlet(q, p, L, rc, dt, steps):
    """FP64 velocity Verlet (m = 1) in the periodic cubic box L: kick dt/2,
    drift, kick dt/2 per step, each kick the restated force_sorted
    (cpu_ref/force_aos.cpp:192-224) over a half list rebuilt from the current
    positions (radius rc + 0.2), so only the cutoff decides membership.
    Returns new (q, p); the inputs are not modified."""
    q, p = q.copy(), p.copy()
    box = np.array([L, L, L], np.float64)
    for _ in range(steps):
        half = build_list(q, rc + 0.2, box=L)
        force_sorted_aos(q, p, *half, cl2=rc * rc, dt=0.5 * dt, box=L)
        oracle().lj_or_drift(q, p, q.shape[0], dt, box.ctypes.data)
        half = build_list(q, rc + 0.2, box=L)
        force_sorted_aos(q, p, *half, cl2=rc * rc, dt=0.5 * dt, box=L)
    return q, p


def periodic_diff(a, b, L):
    """Minimum-image difference of the positions of two AoS arrays."""
    d = a[:, :3] - b[:, :3]
    return d - L * np.round(d / L)


def force_sorted_soa(q, p, npp, ptr, lst, cl2=9.0, dt=0.001, box=None, calls=1):
    """q, p given as (n, 4) arrays; converted to the SoA rows the reference uses."""
    b, bp = _box(box)
    qx, qy, qz = (np.ascontiguousarray(q[:, d]) for d in range(3))
    px, py, pz = (np.ascontiguousarray(p[:, d]) for d in range(3))
    for _ in range(calls):
        oracle().lj_or_force_sorted_soa(qx, qy, qz, px, py, pz, q.shape[0], npp, ptr, lst, cl2,
                                        dt, bp)
    p[:, 0], p[:, 1], p[:, 2] = px, py, pz
    return p


def force_pair_aos(q, p, ii, jj, cl2=9.0, dt=0.001, box=None, calls=1):
    b, bp = _box(box)
    for _ in range(calls):
        oracle().lj_or_force_pair_aos(q, p, len(ii), ii, jj, cl2, dt, bp)
    return p


def force_gather_aos(q, p, npp, ptr, lst, cl2=9.0, dt=0.001, box=None, calls=1, threads=1):
    b, bp = _box(box)
    for _ in range(calls):
        oracle().lj_or_force_gather_aos(q, p, q.shape[0], npp, ptr, lst, cl2, dt, bp, threads)
    return p


def potential_half(q, npp, ptr, lst, cl2=9.0, box=None):
    b, bp = _box(box)
    return oracle().lj_or_potential_half(q, q.shape[0], npp, ptr, lst, cl2, bp)


def golden_rows(p):
    """The reference's print_results (cpu_ref/force_aos.cpp:622-630)."""
    n = p.shape[0]
    idx = list(range(5)) + list(range(n - 5, n))
    return ["%.10f %.10f %.10f" % (p[i, 0], p[i, 1], p[i, 2]) for i in idx]


# ---------------------------------------------------------------------------
# per-particle error metrics (relative errors on the 3-vector, never per
# component)
# ---------------------------------------------------------------------------
def rel_errors(test, ref):
    d = np.linalg.norm(np.asarray(test)[:, :3] - np.asarray(ref)[:, :3], axis=1)
    r = np.linalg.norm(np.asarray(ref)[:, :3], axis=1)
    rms = float(np.sqrt(np.mean(r * r))) if len(r) else 0.0
    with np.errstate(divide="ignore", invalid="ignore"):
        per = np.where(r > 0, d / r, np.where(d > 0, np.inf, 0.0))
    return {
        "max_rel": float(per.max()) if len(per) else 0.0,
        "max_rel_rms": float(d.max() / rms) if rms > 0 else 0.0,
        "global_rel": float(np.sqrt(np.sum(d * d)) / np.sqrt(np.sum(r * r))) if rms > 0 else 0.0,
        "rms_rel": float(np.sqrt(np.mean(per[np.isfinite(per)] ** 2))) if len(per) else 0.0,
    }


# ---------------------------------------------------------------------------
# reference cpu_ref libraries (built here from the read-only sources; x86-64)
# ---------------------------------------------------------------------------
def ref_available() -> bool:
    return REF_AOS.exists() and REF_SOA.exists() and platform.machine() in ("x86_64", "AMD64")


def load_ref(layout="aos") -> C.CDLL:
    L = C.CDLL(str(REF_AOS if layout == "aos" else REF_SOA))
    L.ref_init.argtypes = [C.c_double]
    L.ref_set_positions.argtypes = [C.c_int, _dp]
    L.ref_get_positions.argtypes = [_dp]
    L.ref_set_momenta.argtypes = [_dp]
    L.ref_get_momenta.argtypes = [_dp]
    L.ref_set_pairs.argtypes = [C.c_long, _ip, _ip]
    L.ref_get_pairs.argtypes = [_ip, _ip]
    L.ref_get_csr.argtypes = [_ip, _ip, _ip]
    L.ref_run.argtypes = [C.c_char_p, C.c_int]
    return L


# ---------------------------------------------------------------------------
# the reference's CUDA kernels (oracle/_ref/refcuda.cubin, built from the
# reference checkout by `make -C oracle refcuda`) and their loader
# ---------------------------------------------------------------------------
REFCUDA_CUBIN = ORACLE_DIR / "_ref" / "refcuda.cubin"
REFCUDA_LOADER = ORACLE_DIR / "_build" / "librefcuda.so"
_refcuda = None


def refcuda_available() -> bool:
    return REFCUDA_CUBIN.exists()


def load_refcuda():
    """Loads the cubin into the current CUDA context (call after the CUDA
    runtime is initialised).  Returns (lib, {(kernel_name, vec): index})."""
    global _refcuda
    if _refcuda is not None:
        return _refcuda
    build_oracle()
    L = C.CDLL(str(REFCUDA_LOADER))
    L.rc_load.argtypes = [C.c_char_p]
    L.rc_name.restype = C.c_char_p
    L.rc_name.argtypes = [C.c_int]
    L.rc_launch.argtypes = [C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_int32,
                            C.c_double, C.c_double, C.c_void_p, C.c_void_p, C.c_void_p,
                            C.c_void_p]
    count = L.rc_load(str(REFCUDA_CUBIN).encode())
    if count <= 0:
        raise RuntimeError(f"loading {REFCUDA_CUBIN} failed ({count})")
    table = {}
    for k in range(count):
        name = L.rc_name(k).decode()
        m = re.match(r"_Z(\d+)", name)  # Itanium mangling: length-prefixed name
        if not m:
            continue
        base = name[m.end():m.end() + int(m.group(1))]
        rest = name[m.end() + int(m.group(1)):]
        vec = "double4" if rest.startswith("I7double4") else "double3"
        table[(base, vec)] = k
    _refcuda = (L, table)
    return _refcuda
