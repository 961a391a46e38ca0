"""lj_gpu_gb300 -- Python binding of the GB300 Lennard-Jones force engine.

The engine is the shared library built from ``csrc/`` (C++ host code and
sm_103a CUDA kernels) behind the C ABI declared in ``include/lj_gb300.h``.
This module is a thin ctypes layer over that ABI, used by the tests and the
benchmark; it accepts torch tensors (device or host) or numpy arrays and
passes their raw pointers through.  There is no Python or CPU implementation
of the force path: if the library is missing, every call raises.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path
from typing import Optional

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "_build" / "liblj_gb300.so"

# status codes (lj_gb300.h)
LJ_OK = 0
LJ_ERR_INVALID_ARGUMENT = 1
LJ_ERR_BAD_LIST = 2
LJ_ERR_CUDA = 3
LJ_ERR_OUT_OF_MEMORY = 4
LJ_ERR_LIST_OVERFLOW = 5
LJ_ERR_TIMEOUT = 6
LJ_ERR_NO_LIST = 7
LJ_ERR_UNSUPPORTED = 8

PREC_FP64, PREC_MIXED, PREC_MIXED_FP32 = 0, 1, 2
LIST_HALF, LIST_FULL = 0, 1
WHERE_HOST, WHERE_DEVICE = 0, 1
METHOD_AUTO, METHOD_GATHER_FULL, METHOD_SCATTER_HALF = 0, 1, 2

# "mixed": two-float pair terms (per-particle error ~1e-9 of FP64);
# "mixed_fp32": single FP32 pair terms (faster, ~1e-6 of the RMS force)
_PRECISION = {"fp64": PREC_FP64, "mixed": PREC_MIXED, "mixed_fp32": PREC_MIXED_FP32}
_METHOD = {"auto": METHOD_AUTO, "gather": METHOD_GATHER_FULL, "scatter": METHOD_SCATTER_HALF}
_KIND = {"half": LIST_HALF, "full": LIST_FULL}


class LJError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"[{status}] {message}")
        self.status = status


class ForceOpts(C.Structure):
    _fields_ = [
        ("dt", C.c_double),
        ("cl2", C.c_double),
        ("box", C.c_double * 3),
        ("periodic", C.c_int32),
        ("precision", C.c_int32),
        ("method", C.c_int32),
        ("lanes", C.c_int32),
        ("block", C.c_int32),
        ("kernel", C.c_int32),
        ("unroll", C.c_int32),
        ("ff_all", C.c_int32),
    ]


def make_opts(dt=0.001, cl2=9.0, box=None, precision="fp64", method="auto", lanes=0,
              block=0, kernel=0, unroll=0, ff_all=False) -> ForceOpts:
    o = ForceOpts()
    o.dt, o.cl2 = float(dt), float(cl2)
    if box is not None:
        b = [float(box)] * 3 if isinstance(box, (int, float)) else [float(v) for v in box]
        o.box[0], o.box[1], o.box[2] = b
        o.periodic = 1
    o.precision = _PRECISION[precision] if isinstance(precision, str) else int(precision)
    o.method = _METHOD[method] if isinstance(method, str) else int(method)
    o.lanes, o.block = int(lanes), int(block)
    o.kernel, o.unroll = int(kernel), int(unroll)
    o.ff_all = 1 if ff_all else 0
    return o


LJ_LAYOUT_AOS, LJ_LAYOUT_SOA, LJ_LAYOUT_Z = 0, 1, 2
LAYOUTS = {"aos": LJ_LAYOUT_AOS, "soa": LJ_LAYOUT_SOA, "z": LJ_LAYOUT_Z}


class TuneResult(C.Structure):
    _fields_ = [("best", ForceOpts), ("layout", C.c_int32), ("from_cache", C.c_int32),
                ("timed", C.c_int32), ("reserved", C.c_int32), ("ms", C.c_double),
                ("key", C.c_char * 160)]


class MdParams(C.Structure):
    _fields_ = [
        ("dt", C.c_double), ("rc", C.c_double), ("skin", C.c_double), ("box", C.c_double * 3),
        ("precision", C.c_int32), ("record_every", C.c_int32), ("graph_steps", C.c_int32),
        ("rebuild_every", C.c_int32), ("ff_all", C.c_int32), ("chunk_graphs", C.c_int32),
        ("kick_lanes", C.c_int32), ("reserved", C.c_int32),
    ]


class MdRecord(C.Structure):
    _fields_ = [("step", C.c_int64), ("kinetic", C.c_double), ("potential", C.c_double)]


class MdStats(C.Structure):
    _fields_ = [("steps", C.c_int64), ("rebuilds", C.c_int64), ("ms_total", C.c_double),
                ("list_capacity", C.c_int64), ("launches", C.c_int64),
                ("loop_graph", C.c_int32), ("initial_build", C.c_int32)]


def make_md_params(dt, rc, skin, box, precision="mixed", record_every=0, graph_steps=0,
                   rebuild_every=0, ff_all=False, chunk_graphs=False, kick_lanes=0):
    m = MdParams()
    m.dt, m.rc, m.skin = float(dt), float(rc), float(skin)
    b = [float(box)] * 3 if isinstance(box, (int, float)) else [float(v) for v in box]
    m.box[0], m.box[1], m.box[2] = b
    m.precision = _PRECISION[precision] if isinstance(precision, str) else int(precision)
    m.record_every, m.graph_steps = int(record_every), int(graph_steps)
    m.rebuild_every = int(rebuild_every)
    m.ff_all = 1 if ff_all else 0
    m.chunk_graphs = 1 if chunk_graphs else 0
    m.kick_lanes = int(kick_lanes)
    return m


_lib: Optional[C.CDLL] = None

_P = C.c_void_p
_SIGNATURES = {
    "lj_force_opts_default": (None, [_P]),
    "lj_abi_version": (C.c_int, []),
    "lj_status_string": (C.c_char_p, [C.c_int]),
    "lj_ctx_create": (C.c_int, [C.POINTER(C.c_void_p), C.c_int]),
    "lj_ctx_destroy": (None, [_P]),
    "lj_ctx_last_error": (C.c_char_p, [_P]),
    "lj_ctx_set_stream": (C.c_int, [_P, _P]),
    "lj_ctx_set_timing": (C.c_int, [_P, C.c_int32]),
    "lj_ctx_set_l2_window": (C.c_int, [_P, C.c_double]),
    "lj_ctx_get_timing": (C.c_int, [_P, C.POINTER(C.c_double), C.POINTER(C.c_int64)]),
    "lj_list_set_csr": (C.c_int, [_P, C.c_int32, _P, _P, _P, C.c_int64, C.c_int32, C.c_int32]),
    "lj_list_set_pairs": (C.c_int, [_P, C.c_int32, _P, _P, C.c_int64, C.c_int32]),
    "lj_list_get_csr": (C.c_int, [_P, C.c_int32, _P, _P, _P, C.c_int64,
                                  C.POINTER(C.c_int64), C.c_int32]),
    "lj_list_info": (C.c_int, [_P, C.c_int32, C.POINTER(C.c_int32), C.POINTER(C.c_int64),
                               C.POINTER(C.c_int32)]),
    "lj_force_aos": (C.c_int, [_P, _P, _P, C.c_int32, C.POINTER(ForceOpts)]),
    "lj_force_soa": (C.c_int, [_P, _P, _P, _P, _P, _P, _P, C.c_int32, C.POINTER(ForceOpts)]),
    "lj_force_csr_fp64_aos": (C.c_int, [_P, _P, C.c_int32, C.c_double, C.c_double, _P, _P, _P,
                                        C.c_int32, _P, _P]),
    "lj_force_pairs_fp64_aos": (C.c_int, [_P, _P, C.c_int32, C.c_double, C.c_double, _P, _P,
                                          C.c_int64, _P, _P]),
    "lj_measure_aos": (C.c_int, [_P, _P, _P, C.c_int32, C.POINTER(ForceOpts), C.c_int32,
                                 C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    "lj_init_reference": (C.c_int, [C.c_double, C.c_double, _P, C.c_int32,
                                    C.POINTER(C.c_int32)]),
    "lj_init_fcc": (C.c_int, [C.c_int32, C.c_double, C.c_double, C.c_uint64, _P, C.c_int32,
                              C.POINTER(C.c_double)]),
    "lj_init_momenta": (C.c_int, [_P, C.c_int32, C.c_double, C.c_uint64]),
    "lj_list_build": (C.c_int, [_P, _P, C.c_int32, C.c_double, _P, C.c_int32]),
    "lj_batch_run": (C.c_int, [_P, _P, _P, C.c_int32, C.c_int32, _P, _P, C.POINTER(MdParams),
                               C.c_int32, _P, C.c_int32, C.POINTER(C.c_int32),
                               C.POINTER(MdStats), _P]),
    "lj_force_z": (C.c_int, [_P, _P, C.c_int32, C.POINTER(ForceOpts)]),
    "lj_list_set_ell": (C.c_int, [_P, C.c_int32, _P, _P, C.c_int64, C.c_int64, C.c_int32,
                                  C.c_int32]),
    "lj_list_get_ell": (C.c_int, [_P, C.c_int32, _P, _P, C.c_int64, C.c_int64, C.c_int32]),
    "lj_list_shuffle_rows": (C.c_int, [C.c_int32, _P, _P, _P, C.c_uint32]),
    "lj_cache_write_text": (C.c_int, [C.c_char_p, C.c_int32, _P, _P, _P, C.c_int64]),
    "lj_cache_read_text": (C.c_int, [C.c_char_p, C.c_int32, _P, _P, _P, C.c_int64,
                                     C.POINTER(C.c_int64)]),
    "lj_pairdat_write": (C.c_int, [C.c_char_p, C.c_int32, _P, _P, C.c_int64]),
    "lj_pairdat_read": (C.c_int, [C.c_char_p, C.c_int32, _P, _P, _P, C.c_int64,
                                  C.POINTER(C.c_int64)]),
    "lj_autotune_aos": (C.c_int, [_P, _P, C.c_int32, C.POINTER(ForceOpts), C.c_int32,
                                  C.POINTER(ForceOpts), C.POINTER(C.c_double)]),
    "lj_autotune": (C.c_int, [_P, _P, C.c_int32, C.POINTER(ForceOpts), C.c_int32, C.c_int32,
                              C.c_char_p, C.POINTER(TuneResult)]),
    "lj_md_run": (C.c_int, [_P, _P, _P, C.c_int32, C.POINTER(MdParams), C.c_int32,
                            C.POINTER(MdRecord), C.c_int32, C.POINTER(C.c_int32),
                            C.POINTER(MdStats)]),
    "lj_md_run_host": (C.c_int, [_P, _P, _P, C.c_int32, C.POINTER(MdParams), C.c_int32,
                                 C.POINTER(MdRecord), C.c_int32, C.POINTER(C.c_int32),
                                 C.POINTER(MdStats)]),
    "lj_force_mixed_noalloc_aos": (C.c_int, [_P, _P, C.c_int32, C.c_double, C.c_double, _P,
                                             _P, _P, _P, _P]),
}

NOALLOC_MAX_PARTICLES = 1 << 20

EXPORTED = tuple(_SIGNATURES)


def lib() -> C.CDLL:
    """Loads the engine library; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise ImportError(
                f"lj_gpu_gb300 native library missing at {LIB_PATH}; build it with "
                "`python -m lj_gpu_gb300._build` (needs nvcc)")
        L = C.CDLL(str(LIB_PATH))
        for name, (res, args) in _SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def ptr(x) -> int:
    """Raw address of a torch tensor / numpy array (None -> 0)."""
    if x is None:
        return 0
    if hasattr(x, "data_ptr"):
        return x.data_ptr()
    if hasattr(x, "ctypes"):
        return x.ctypes.data
    return int(x)


def _where(x) -> int:
    if hasattr(x, "is_cuda"):
        return WHERE_DEVICE if x.is_cuda else WHERE_HOST
    return WHERE_HOST


def _check_contig(*xs):
    for x in xs:
        if x is None:
            continue
        ok = x.is_contiguous() if hasattr(x, "is_contiguous") else x.flags["C_CONTIGUOUS"]
        if not ok:
            raise ValueError("arrays passed to the engine must be contiguous")


class Context:
    """Owns an lj_ctx: the installed neighbour list and the engine's scratch."""

    def __init__(self, device: int = 0, stream=None):
        L = lib()
        h = C.c_void_p()
        st = L.lj_ctx_create(C.byref(h), int(device))
        if st != LJ_OK:
            raise LJError(st, f"lj_ctx_create: {L.lj_status_string(st).decode()}")
        self._h = h
        self.device = device
        if stream is not None:
            self.set_stream(stream)

    def close(self):
        if getattr(self, "_h", None):
            lib().lj_ctx_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def handle(self):
        return self._h

    def _check(self, st: int, what: str):
        if st != LJ_OK:
            msg = lib().lj_ctx_last_error(self._h).decode()
            raise LJError(st, f"{what}: {msg or lib().lj_status_string(st).decode()}")

    def set_stream(self, stream):
        s = stream.cuda_stream if hasattr(stream, "cuda_stream") else int(stream or 0)
        self._check(lib().lj_ctx_set_stream(self._h, s), "set_stream")

    def set_l2_window(self, hit_ratio):
        """L2 persistence window over the position image for mixed force calls
        (lj_ctx_set_l2_window); 0 turns it off."""
        self._check(lib().lj_ctx_set_l2_window(self._h, float(hit_ratio)), "set_l2_window")

    def set_timing(self, on=True):
        self._check(lib().lj_ctx_set_timing(self._h, 1 if on else 0), "set_timing")

    def get_timing(self):
        """(ms position-image passes, ms pair kernels, ms both, calls) since reset."""
        ms = (C.c_double * 3)()
        calls = C.c_int64()
        self._check(lib().lj_ctx_get_timing(self._h, ms, C.byref(calls)), "get_timing")
        return ms[0], ms[1], ms[2], calls.value

    def set_list_csr(self, number_of_partners, pointer, sorted_list, kind="half", n=None):
        _check_contig(number_of_partners, pointer, sorted_list)
        n = len(number_of_partners) if n is None else n
        st = lib().lj_list_set_csr(self._h, n, ptr(number_of_partners), ptr(pointer),
                                   ptr(sorted_list), len(sorted_list), _KIND[kind],
                                   _where(sorted_list))
        self._check(st, "set_list_csr")

    def set_list_pairs(self, n, i_particles, j_particles):
        _check_contig(i_particles, j_particles)
        st = lib().lj_list_set_pairs(self._h, n, ptr(i_particles), ptr(j_particles),
                                     len(i_particles), _where(i_particles))
        self._check(st, "set_list_pairs")

    def build_list(self, q, search_radius, box=None, kinds=("half", "full")):
        """On-device cell-list build of the neighbour list of AoS device q."""
        _check_contig(q)
        bits = (1 if "half" in kinds else 0) | (2 if "full" in kinds else 0)
        bx = _box3(box)
        st = lib().lj_list_build(self._h, ptr(q), q.shape[0], float(search_radius),
                                 C.cast(bx, C.c_void_p) if bx else None, bits)
        self._check(st, "build_list")

    def list_info(self, kind="half"):
        n, e, m = C.c_int32(), C.c_int64(), C.c_int32()
        self._check(lib().lj_list_info(self._h, _KIND[kind], C.byref(n), C.byref(e),
                                       C.byref(m)), "list_info")
        return n.value, e.value, m.value

    def get_list_csr(self, kind="half"):
        """Returns (number_of_partners, pointer, sorted_list) as numpy arrays."""
        import numpy as np
        n, e, _ = self.list_info(kind)
        a = np.zeros(n, np.int32)
        b = np.zeros(n, np.int32)
        c = np.zeros(max(e, 1), np.int32)
        got = C.c_int64()
        self._check(lib().lj_list_get_csr(self._h, _KIND[kind], ptr(a), ptr(b), ptr(c), e,
                                          C.byref(got), WHERE_HOST), "get_list_csr")
        return a, b, c[:got.value]

    def force_aos(self, q, p, opts: ForceOpts, n=None):
        _check_contig(q, p)
        n = q.shape[0] if n is None else n
        self._check(lib().lj_force_aos(self._h, ptr(q), ptr(p), n, C.byref(opts)), "force_aos")

    def force_z(self, z, opts: ForceOpts, n=None):
        """Interleaved z[n][8] = {q.xyzw, p.xyzw} layout."""
        _check_contig(z)
        n = z.shape[0] if n is None else n
        self._check(lib().lj_force_z(self._h, ptr(z), n, C.byref(opts)), "force_z")

    def set_list_ell(self, number_of_partners, transposed_list, width, kind="full"):
        _check_contig(number_of_partners, transposed_list)
        st = lib().lj_list_set_ell(self._h, len(number_of_partners), ptr(number_of_partners),
                                   ptr(transposed_list), int(width), len(transposed_list),
                                   _KIND[kind], _where(transposed_list))
        self._check(st, "set_list_ell")

    def get_list_ell(self, width, kind="full"):
        import numpy as np
        n, _, mr = self.list_info(kind)
        npp = np.zeros(n, np.int32)
        ell = np.zeros(max(1, mr * int(width)), np.int32)
        self._check(lib().lj_list_get_ell(self._h, _KIND[kind], ptr(npp), ptr(ell), int(width),
                                          len(ell), WHERE_HOST), "get_list_ell")
        return npp, ell

    def force_soa(self, qx, qy, qz, px, py, pz, opts: ForceOpts, n=None):
        _check_contig(qx, qy, qz, px, py, pz)
        n = qx.shape[0] if n is None else n
        st = lib().lj_force_soa(self._h, ptr(qx), ptr(qy), ptr(qz), ptr(px), ptr(py), ptr(pz),
                                n, C.byref(opts))
        self._check(st, "force_soa")

    def autotune(self, q, opts: ForceOpts, reps=5):
        """Fastest launch shape for the installed list; returns (opts, ms per call)."""
        _check_contig(q)
        best = ForceOpts()
        ms = C.c_double()
        self._check(lib().lj_autotune_aos(self._h, ptr(q), q.shape[0], C.byref(opts), reps,
                                          C.byref(best), C.byref(ms)), "autotune")
        return best, ms.value

    def autotune_layouts(self, q, opts: ForceOpts, reps=5, layouts=("aos",), cache=None):
        """lj_autotune: launch shapes, the transposed list (kernel 5) and the
        particle layouts named in `layouts`, with an optional cache file.
        Returns a dict: opts, layout (name), ms, from_cache, timed, key."""
        _check_contig(q)
        mask = 0
        for name in layouts:
            mask |= 1 << LAYOUTS[name]
        r = TuneResult()
        path = None if cache is None else str(cache).encode()
        self._check(lib().lj_autotune(self._h, ptr(q), q.shape[0], C.byref(opts), reps, mask,
                                      path, C.byref(r)), "autotune")
        names = {v: k for k, v in LAYOUTS.items()}
        return {"opts": r.best, "layout": names[r.layout], "ms": r.ms,
                "from_cache": bool(r.from_cache), "timed": r.timed, "key": r.key.decode()}

    def md_run(self, q, p, params: MdParams, nsteps, max_records=64):
        """Velocity Verlet on device AoS q, p (in place); returns (records, stats)
        with records a list of (step, kinetic, potential)."""
        _check_contig(q, p)
        recs = (MdRecord * max(1, max_records))()
        nrec = C.c_int32()
        st = MdStats()
        s = lib().lj_md_run(self._h, ptr(q), ptr(p), q.shape[0], C.byref(params), int(nsteps),
                            recs, max_records, C.byref(nrec), C.byref(st))
        self._check(s, "md_run")
        return ([(recs[k].step, recs[k].kinetic, recs[k].potential) for k in range(nrec.value)],
                {"steps": st.steps, "rebuilds": st.rebuilds, "ms_total": st.ms_total,
                 "list_capacity": st.list_capacity, "launches": st.launches,
                 "loop_graph": st.loop_graph, "initial_build": st.initial_build})

    def md_run_host(self, q, p, params: MdParams, nsteps, max_records=64):
        """lj_md_run_host: velocity Verlet over host AoS (n, 4) float64 arrays
        (numpy arrays or CPU tensors, page-locked for overlapped copies),
        updated in place; returns (records, stats) as md_run."""
        import numpy as np
        for a in (q, p):
            arr = a.numpy() if hasattr(a, "numpy") else a
            if not (isinstance(arr, np.ndarray) and arr.dtype == np.float64 and arr.ndim == 2
                    and arr.shape[1] == 4 and arr.flags.c_contiguous):
                raise ValueError("q and p must be C-contiguous float64 arrays of shape (n, 4)")
        hq = q.numpy() if hasattr(q, "numpy") else q
        hp = p.numpy() if hasattr(p, "numpy") else p
        if hq.shape != hp.shape:
            raise ValueError("q and p must have the same shape")
        recs = (MdRecord * max(1, max_records))()
        nrec = C.c_int32()
        st = MdStats()
        s = lib().lj_md_run_host(self._h, hq.ctypes.data, hp.ctypes.data, hq.shape[0],
                                 C.byref(params), int(nsteps), recs, max_records,
                                 C.byref(nrec), C.byref(st))
        self._check(s, "md_run_host")
        return ([(recs[k].step, recs[k].kinetic, recs[k].potential) for k in range(nrec.value)],
                {"steps": st.steps, "rebuilds": st.rebuilds, "ms_total": st.ms_total,
                 "list_capacity": st.list_capacity, "launches": st.launches,
                 "loop_graph": st.loop_graph, "initial_build": st.initial_build})

    def batch_run(self, q, p, offsets, boxes, params: MdParams, nsteps, max_records=16):
        """Replica batch (see lj_batch_run).  offsets: n_replicas + 1 ints, boxes:
        (n_replicas, 3).  Returns (energies[rec, replica, (K, U)], stats, shapes)."""
        import numpy as np
        _check_contig(q, p)
        offs = np.ascontiguousarray(offsets, np.int32)
        bx = np.ascontiguousarray(boxes, np.float64)
        R = len(offs) - 1
        en = np.zeros((max(1, max_records), R, 2))
        nrec = C.c_int32()
        st = MdStats()
        shapes = np.zeros(9, np.int32)
        s = lib().lj_batch_run(self._h, ptr(q), ptr(p), q.shape[0], R, ptr(offs), ptr(bx),
                               C.byref(params), int(nsteps), ptr(en), max_records,
                               C.byref(nrec), C.byref(st), ptr(shapes))
        self._check(s, "batch_run")
        return (en[:nrec.value], {"steps": st.steps, "rebuilds": st.rebuilds,
                                  "ms_total": st.ms_total}, shapes.reshape(3, 3))

    def measure_aos(self, q_host, p_host, opts: ForceOpts, calls=100):
        """The reference's measure(): H2D, `calls` force calls, D2H; returns
        (ms_total, ms_calc)."""
        _check_contig(q_host, p_host)
        a, b = C.c_double(), C.c_double()
        st = lib().lj_measure_aos(self._h, ptr(q_host), ptr(p_host), q_host.shape[0],
                                  C.byref(opts), calls, C.byref(a), C.byref(b))
        self._check(st, "measure_aos")
        return a.value, b.value


def _box3(box):
    if box is None:
        return None
    b = [float(box)] * 3 if isinstance(box, (int, float)) else [float(v) for v in box]
    return (C.c_double * 3)(*b)


def init_reference(density=0.5, box_len=50.0):
    """The reference's init(): FCC + U[0, 0.1) jitter from mt19937(2); (n, 4) array."""
    import numpy as np
    n = C.c_int32()
    lib().lj_init_reference(density, box_len, None, 0, C.byref(n))
    q = np.zeros((n.value, 4))
    st = lib().lj_init_reference(density, box_len, ptr(q), n.value, C.byref(n))
    if st != LJ_OK:
        raise LJError(st, "lj_init_reference")
    return q


def init_fcc(ncell, density, jitter=0.05, seed=20240601):
    """Periodic jittered FCC; returns ((n, 4) array, box length)."""
    import numpy as np
    n = 4 * ncell ** 3
    q = np.zeros((n, 4))
    L = C.c_double()
    st = lib().lj_init_fcc(ncell, density, jitter, seed, ptr(q), n, C.byref(L))
    if st != LJ_OK:
        raise LJError(st, "lj_init_fcc")
    return q, L.value


def init_momenta(n, temperature=1.0, seed=1):
    import numpy as np
    p = np.zeros((n, 4))
    st = lib().lj_init_momenta(ptr(p), n, temperature, seed)
    if st != LJ_OK:
        raise LJError(st, "lj_init_momenta")
    return p


def _status(st, what):
    if st != LJ_OK:
        raise LJError(st, f"{what}: {lib().lj_status_string(st).decode()}")


def shuffle_rows(npp, ptr_, lst, seed=10):
    """random_shfl: shuffles the rows of host CSR arrays in place."""
    _status(lib().lj_list_shuffle_rows(len(npp), ptr(npp), ptr(ptr_), ptr(lst), seed),
            "shuffle_rows")


def cache_write_text(path, npp, ptr_, lst):
    _status(lib().lj_cache_write_text(str(path).encode(), len(npp), ptr(npp), ptr(ptr_),
                                      ptr(lst), len(lst)), "cache_write_text")


def cache_read_text(path, n, capacity):
    import numpy as np
    npp, ptr_ = np.zeros(n, np.int32), np.zeros(n, np.int32)
    lst = np.zeros(max(1, capacity), np.int32)
    ne = C.c_int64()
    _status(lib().lj_cache_read_text(str(path).encode(), n, ptr(npp), ptr(ptr_), ptr(lst),
                                     capacity, C.byref(ne)), "cache_read_text")
    return npp, ptr_, lst[:ne.value]


def pairdat_write(path, n, ii, jj):
    _status(lib().lj_pairdat_write(str(path).encode(), n, ptr(ii), ptr(jj), len(ii)),
            "pairdat_write")


def pairdat_read(path, n, capacity):
    import numpy as np
    npp = np.zeros(n, np.int32)
    ii, jj = np.zeros(max(1, capacity), np.int32), np.zeros(max(1, capacity), np.int32)
    k = C.c_int64()
    _status(lib().lj_pairdat_read(str(path).encode(), n, ptr(npp), ptr(ii), ptr(jj), capacity,
                                  C.byref(k)), "pairdat_read")
    return npp, ii[:k.value], jj[:k.value]


def force_csr_fp64_aos(q, p, dt, cl2, sorted_list, number_of_partners, pointer, kind="full",
                       box=None, stream=0):
    """Stateless FP64 drop-in for one reference kernel launch."""
    import ctypes
    bx = None
    if box is not None:
        b = [float(box)] * 3 if isinstance(box, (int, float)) else [float(v) for v in box]
        bx = (ctypes.c_double * 3)(*b)
    st = lib().lj_force_csr_fp64_aos(ptr(q), ptr(p), q.shape[0], float(dt), float(cl2),
                                     ptr(sorted_list), ptr(number_of_partners), ptr(pointer),
                                     _KIND[kind], C.cast(bx, C.c_void_p) if bx else None,
                                     stream)
    if st != LJ_OK:
        raise LJError(st, "lj_force_csr_fp64_aos")


def force_mixed_noalloc_aos(q, p, dt, cl2, sorted_list, number_of_partners, pointer, box=None,
                            stream=0):
    """Mixed-precision gather over a full list with no allocation by the
    engine: for callers that cannot allocate device memory.  Its scratch is a
    static device array for at most NOALLOC_MAX_PARTICLES particles, shared by
    every call (calls that overlap on the GPU race)."""
    bx = _box3(box)
    st = lib().lj_force_mixed_noalloc_aos(ptr(q), ptr(p), q.shape[0], float(dt), float(cl2),
                                          ptr(sorted_list), ptr(number_of_partners),
                                          ptr(pointer), C.cast(bx, C.c_void_p) if bx else None,
                                          stream)
    if st != LJ_OK:
        raise LJError(st, "lj_force_mixed_noalloc_aos")


def force_pairs_fp64_aos(q, p, dt, cl2, i_particles, j_particles, box=None, stream=0):
    """force_pair on the device (FP64, atomics on both ends)."""
    bx = None
    if box is not None:
        b = [float(box)] * 3 if isinstance(box, (int, float)) else [float(v) for v in box]
        bx = (C.c_double * 3)(*b)
    st = lib().lj_force_pairs_fp64_aos(ptr(q), ptr(p), q.shape[0], float(dt), float(cl2),
                                       ptr(i_particles), ptr(j_particles), len(i_particles),
                                       C.cast(bx, C.c_void_p) if bx else None, stream)
    if st != LJ_OK:
        raise LJError(st, "lj_force_pairs_fp64_aos")
