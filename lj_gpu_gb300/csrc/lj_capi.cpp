// lj_capi.cpp -- implementation of the C ABI in include/lj_gb300.h.
//
// Host-side C++: argument checking, list installation (validation, half->full
// expansion), buffer management and kernel dispatch.  No arithmetic of the
// force path runs here; every force call is a CUDA launch on the context's
// stream.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "lj_gb300.h"
#include "lj_internal.h"
#include "lj_nlist.h"

using namespace ljg;

#include "lj_ctx.h"

namespace {

int fail(lj_ctx* ctx, int code, const char* fmt, ...) {
  if (ctx) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    ctx->err = buf;
  }
  return code;
}

}  // namespace

int lj_fail(lj_ctx* ctx, int code, const char* fmt, ...) {
  if (ctx) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    ctx->err = buf;
  }
  return code;
}

namespace {

int cuda_fail(lj_ctx* ctx, cudaError_t e, const char* what) {
  return fail(ctx, e == cudaErrorMemoryAllocation ? LJ_ERR_OUT_OF_MEMORY : LJ_ERR_CUDA,
              "%s: %s", what, cudaGetErrorString(e));
}

#define LJ_CUDA(ctx, call, what)                 \
  do {                                           \
    cudaError_t e_ = (call);                     \
    if (e_ != cudaSuccess) return cuda_fail(ctx, e_, what); \
  } while (0)

bool pow2_lanes(int v) { return v == 1 || v == 2 || v == 4 || v == 8 || v == 16 || v == 32; }

int check_opts(lj_ctx* ctx, const lj_force_opts* o) {
  if (!o) return fail(ctx, LJ_ERR_INVALID_ARGUMENT, "opts is NULL");
  if (!(o->precision == LJ_PREC_FP64 || o->precision == LJ_PREC_MIXED ||
        o->precision == LJ_PREC_MIXED_FP32))
    return fail(ctx, LJ_ERR_INVALID_ARGUMENT, "unknown precision %d", o->precision);
  if (o->method < LJ_METHOD_AUTO || o->method > LJ_METHOD_SCATTER_HALF)
    return fail(ctx, LJ_ERR_INVALID_ARGUMENT, "unknown method %d", o->method);
  if (o->lanes != 0 && !pow2_lanes(o->lanes))
    return fail(ctx, LJ_ERR_INVALID_ARGUMENT, "lanes must be 0 or a power of two <= 32");
  if (o->block != 0 && (o->block < 64 || o->block > 256 || (o->block % 32) != 0))
    return fail(ctx, LJ_ERR_INVALID_ARGUMENT, "block must be 0 or a multiple of 32 in [64, 256]");
  if (o->kernel < 0 || o->kernel > 5)
    return fail(ctx, LJ_ERR_INVALID_ARGUMENT, "kernel must be 0 (default) or 1..5");
  if (o->unroll < 0) return fail(ctx, LJ_ERR_INVALID_ARGUMENT, "unroll must be >= 0");
  if (o->ff_all != 0 && o->ff_all != 1)
    return fail(ctx, LJ_ERR_INVALID_ARGUMENT, "ff_all must be 0 or 1");
  if (!(o->cl2 >= 0.0) || !std::isfinite(o->dt))
    return fail(ctx, LJ_ERR_INVALID_ARGUMENT, "cl2 must be >= 0 and dt finite");
  if (o->periodic) {
    for (int d = 0; d < 3; d++)
      if (!(o->box[d] > 0.0) || !std::isfinite(o->box[d]))
        return fail(ctx, LJ_ERR_INVALID_ARGUMENT, "periodic box lengths must be > 0");
    const double mn = std::min(o->box[0], std::min(o->box[1], o->box[2]));
    if (o->cl2 > 0.25 * mn * mn)
      return fail(ctx, LJ_ERR_INVALID_ARGUMENT,
                  "cutoff exceeds half the box: the minimum image is ambiguous");
  }
  return LJ_OK;
}

Periodic make_periodic(const lj_force_opts* o) {
  Periodic b{};
  b.on = o->periodic ? 1 : 0;
  for (int d = 0; d < 3; d++) {
    b.len[d] = b.on ? o->box[d] : 0.0;
    b.half[d] = 0.5 * b.len[d];
  }
  return b;
}

// Defaults measured on GB300 (108,000 particles, rho = 0.5 and 1.0, cold L2):
//   mixed gather  : kernel 2, 4 lanes per row, 4 entries per lane in flight
//   FP64 scatter  : kernel 2 (compacted, RED on both ends)
//   FP64 gather   : kernel 2 (compacted, one warp per row)
int default_lanes(int precision, int method, int kernel, int64_t entries, int n) {
  const double avg = n > 0 ? (double)entries / n : 0.0;
  // two-float gathers are issue-bound: one lane per row wastes the fewest
  // slots on row ends and group sums (1M rho = 1: 139 G pair/s against 115
  // with 4 lanes); FP32 pair terms are bound by the L1 gathers and keep 4
  if (kernel >= 2 && precision == LJ_PREC_MIXED && method == LJ_METHOD_GATHER_FULL)
    return avg <= 24 ? 2 : 1;
  if (kernel >= 2 && precision != LJ_PREC_FP64) return avg <= 24 ? 2 : 4;
  if (precision == LJ_PREC_FP64 && method == LJ_METHOD_SCATTER_HALF) return avg <= 12 ? 2 : 4;
  if (avg <= 12) return 2;
  if (avg <= 24) return 4;
  if (avg <= 96) return 8;
  return 16;
}


int copy_in(lj_ctx* ctx, int32_t* dst, const int32_t* src, size_t count, int where) {
  if (count == 0) return LJ_OK;
  LJ_CUDA(ctx,
          cudaMemcpyAsync(dst, src, count * sizeof(int32_t),
                          where == LJ_WHERE_HOST ? cudaMemcpyHostToDevice
                                                 : cudaMemcpyDeviceToDevice,
                          ctx->stream),
          "list copy");
  return LJ_OK;
}

// Builds ctx->full from ctx->half on the device.
int expand_full(lj_ctx* ctx) {
  const Csr h = ctx->half.csr();
  const int n = h.n;
  if ((int64_t)2 * h.entries > 0x7fffffffll)
    return fail(ctx, LJ_ERR_UNSUPPORTED, "full list would exceed 2^31-1 entries");
  LJ_CUDA(ctx, ctx->tmp_i32a.ensure((size_t)n), "alloc");
  LJ_CUDA(ctx, ctx->tmp_off.ensure((size_t)n + 1), "alloc");
  LJ_CUDA(ctx, ctx->tmp_scan.ensure(scan_tmp_bytes(n)), "alloc");
  LJ_CUDA(ctx, launch_full_from_half_count(h, ctx->tmp_i32a.ptr, ctx->stream), "count");
  LJ_CUDA(ctx, launch_scan_counts(ctx->tmp_i32a.ptr, n, ctx->tmp_off.ptr, ctx->tmp_scan.ptr,
                                  ctx->tmp_scan.cap, ctx->stream), "scan");
  int64_t total = 0;
  LJ_CUDA(ctx, cudaMemcpyAsync(&total, ctx->tmp_off.ptr + n, sizeof total,
                               cudaMemcpyDeviceToHost, ctx->stream), "total");
  LJ_CUDA(ctx, cudaStreamSynchronize(ctx->stream), "sync");
  DevList& f = ctx->full;
  f.valid = false;
  LJ_CUDA(ctx, f.np.ensure((size_t)n), "alloc");
  LJ_CUDA(ctx, f.ptr.ensure((size_t)n), "alloc");
  LJ_CUDA(ctx, f.list.ensure((size_t)total), "alloc");
  LJ_CUDA(ctx, ctx->tmp_i32b.ensure((size_t)total), "alloc");
  LJ_CUDA(ctx, launch_full_from_half_fill(h, ctx->tmp_off.ptr, ctx->tmp_i32a.ptr,
                                          ctx->tmp_i32b.ptr, ctx->stream), "fill");
  LJ_CUDA(ctx, launch_sort_rows_into(ctx->tmp_off.ptr, n, ctx->tmp_i32b.ptr, f.list.ptr,
                                     ctx->stream), "sort");
  LJ_CUDA(ctx, ctx->err2.ensure(2), "alloc");
  LJ_CUDA(ctx, launch_offsets_to_ptr(ctx->tmp_off.ptr, n, f.ptr.ptr, f.np.ptr, ctx->err2.ptr,
                                     ctx->stream), "ptr");
  int32_t mr = 0;
  LJ_CUDA(ctx, cudaMemcpyAsync(&mr, ctx->err2.ptr, sizeof mr, cudaMemcpyDeviceToHost,
                               ctx->stream), "max row");
  LJ_CUDA(ctx, cudaStreamSynchronize(ctx->stream), "sync");
  f.n = n;
  f.entries = total;
  f.max_row = mr;
  f.valid = true;
  return LJ_OK;
}

// Keeps beside ctx->full a copy whose rows start on 16-byte boundaries (each
// row zero-padded to a multiple of 4 entries), read by the mixed gather's
// vector index loads.  Lists beyond 2^31 padded entries keep the scalar path.
int build_aligned(lj_ctx* ctx) {
  DevList& f = ctx->full;
  f.avalid = false;
  f.svalid = f.savalid = false;
  f.evalid = false;
  const int n = f.n;
  if (!f.valid || n == 0) return LJ_OK;
  cudaStream_t s = ctx->stream;
  LJ_CUDA(ctx, ctx->tmp_i32a.ensure((size_t)n), "alloc");
  LJ_CUDA(ctx, f.aoff.ensure((size_t)n + 1), "alloc");
  LJ_CUDA(ctx, ctx->tmp_scan.ensure(scan_tmp_bytes(n)), "alloc");
  LJ_CUDA(ctx, launch_round4(f.np.ptr, n, ctx->tmp_i32a.ptr, s), "round");
  LJ_CUDA(ctx, launch_scan_counts(ctx->tmp_i32a.ptr, n, f.aoff.ptr, ctx->tmp_scan.ptr,
                                  ctx->tmp_scan.cap, s), "scan");
  int64_t total = 0;
  LJ_CUDA(ctx, cudaMemcpyAsync(&total, f.aoff.ptr + n, sizeof total, cudaMemcpyDeviceToHost, s),
          "total");
  LJ_CUDA(ctx, cudaStreamSynchronize(s), "sync");
  if (total > 0x7fffffffll) return LJ_OK;
  LJ_CUDA(ctx, f.aptr.ensure((size_t)n), "alloc");
  LJ_CUDA(ctx, f.alist.ensure((size_t)std::max<int64_t>(total, 4)), "alloc");
  LJ_CUDA(ctx, launch_copy_rows4(f.np.ptr, f.ptr.ptr, f.list.ptr, f.aoff.ptr, n, f.alist.ptr,
                                 f.aptr.ptr, s), "aligned copy");
  f.aentries = total;
  f.avalid = true;
  return LJ_OK;
}

// Copies a caller CSR into the context, validates it, and stores it compact:
// rows in i order, contiguous, pointer[i] = sum of the earlier row lengths
// (what sortpair produces).  Kernels that sweep several rows as one flat range
// rely on that.
int install_csr(lj_ctx* ctx, int32_t n, const int32_t* np, const int32_t* ptr,
                const int32_t* list, int64_t entries, int32_t kind, int32_t where) {
  DevList& l = kind == LJ_LIST_HALF ? ctx->half : ctx->full;
  ctx->half.valid = false;
  ctx->full.valid = false;
  ctx->full.avalid = false;
  ctx->full.svalid = ctx->full.savalid = false;
  ctx->full.evalid = false;
  ctx->tiled.valid = false;
  LJ_CUDA(ctx, l.np.ensure((size_t)n), "alloc");
  LJ_CUDA(ctx, l.ptr.ensure((size_t)n), "alloc");
  LJ_CUDA(ctx, ctx->tmp_i32a.ensure((size_t)n), "alloc");
  LJ_CUDA(ctx, ctx->tmp_i32b.ensure((size_t)entries), "alloc");
  int rc;
  if ((rc = copy_in(ctx, l.np.ptr, np, (size_t)n, where))) return rc;
  if ((rc = copy_in(ctx, ctx->tmp_i32a.ptr, ptr, (size_t)n, where))) return rc;
  if ((rc = copy_in(ctx, ctx->tmp_i32b.ptr, list, (size_t)entries, where))) return rc;
  // validation runs on the caller's layout, as check_loadedpair does
  const Csr raw{n, entries, l.np.ptr, ctx->tmp_i32a.ptr, ctx->tmp_i32b.ptr, 0, 0};
  {
    LJ_CUDA(ctx, ctx->err2.ensure(2), "alloc");
    const int32_t init[2] = {0, 0x7fffffff};
    LJ_CUDA(ctx, cudaMemcpyAsync(ctx->err2.ptr, init, sizeof init, cudaMemcpyHostToDevice,
                                 ctx->stream), "err init");
    LJ_CUDA(ctx, launch_validate_csr(raw, ctx->err2.ptr, ctx->stream), "validate");
    int32_t out[2];
    LJ_CUDA(ctx, cudaMemcpyAsync(out, ctx->err2.ptr, sizeof out, cudaMemcpyDeviceToHost,
                                 ctx->stream), "err read");
    LJ_CUDA(ctx, cudaStreamSynchronize(ctx->stream), "validate sync");
    switch (out[0]) {
      case 0: break;
      case 1: return fail(ctx, LJ_ERR_BAD_LIST, "number_of_partners[%d] out of range", out[1]);
      case 2: return fail(ctx, LJ_ERR_BAD_LIST, "pointer[%d] out of range", out[1]);
      case 3: return fail(ctx, LJ_ERR_BAD_LIST, "row %d runs past the end of the list", out[1]);
      default: return fail(ctx, LJ_ERR_BAD_LIST, "sorted_list[%d] out of range", out[1]);
    }
  }
  LJ_CUDA(ctx, ctx->tmp_off.ensure((size_t)n + 1), "alloc");
  LJ_CUDA(ctx, ctx->tmp_scan.ensure(scan_tmp_bytes(n)), "alloc");
  LJ_CUDA(ctx, launch_scan_counts(l.np.ptr, n, ctx->tmp_off.ptr, ctx->tmp_scan.ptr,
                                  ctx->tmp_scan.cap, ctx->stream), "scan");
  int64_t total = 0;
  LJ_CUDA(ctx, cudaMemcpyAsync(&total, ctx->tmp_off.ptr + n, sizeof total,
                               cudaMemcpyDeviceToHost, ctx->stream), "total");
  LJ_CUDA(ctx, cudaStreamSynchronize(ctx->stream), "sync");
  LJ_CUDA(ctx, l.list.ensure((size_t)std::max<int64_t>(total, 1)), "alloc");
  LJ_CUDA(ctx, launch_compact_rows(l.np.ptr, ctx->tmp_i32a.ptr, ctx->tmp_i32b.ptr,
                                   ctx->tmp_off.ptr, n, l.list.ptr, ctx->stream), "compact");
  LJ_CUDA(ctx, launch_offsets_to_ptr(ctx->tmp_off.ptr, n, l.ptr.ptr, l.np.ptr, ctx->err2.ptr,
                                     ctx->stream), "ptr");
  int32_t mr = 0;
  LJ_CUDA(ctx, cudaMemcpyAsync(&mr, ctx->err2.ptr, sizeof mr, cudaMemcpyDeviceToHost,
                               ctx->stream), "max row");
  LJ_CUDA(ctx, cudaStreamSynchronize(ctx->stream), "sync");
  l.n = n;
  l.entries = total;
  l.max_row = mr;
  l.valid = true;
  if (kind == LJ_LIST_HALF) {
    if ((rc = expand_full(ctx))) {
      ctx->half.valid = false;
      return rc;
    }
  }
  return build_aligned(ctx);
}

int resolve_method(lj_ctx* ctx, const lj_force_opts* o, int* method) {
  int m = o->method;
  if (m == LJ_METHOD_AUTO) {
    if (o->precision == LJ_PREC_FP64 && o->kernel != 5)
      m = ctx->half.valid ? LJ_METHOD_SCATTER_HALF : LJ_METHOD_GATHER_FULL;
    else
      m = LJ_METHOD_GATHER_FULL;
  }
  if (m == LJ_METHOD_SCATTER_HALF && !ctx->half.valid)
    return fail(ctx, ctx->full.valid ? LJ_ERR_UNSUPPORTED : LJ_ERR_NO_LIST,
                "scatter over a half list needs a half list installed");
  if (m == LJ_METHOD_GATHER_FULL && !ctx->full.valid)
    return fail(ctx, LJ_ERR_NO_LIST, "no neighbour list installed");
  *method = m;
  return LJ_OK;
}

// The transposed copy of the full list for the ELL gather (kernel 5), built
// from the installed CSR when missing (or when `refresh`, after the CSR was
// uploaded again).
int ensure_ell(lj_ctx* ctx, bool refresh = false) {
  DevList& f = ctx->full;
  if (f.evalid && !refresh) return LJ_OK;
  f.evalid = false;
  const size_t words = std::max<size_t>((size_t)f.n * (size_t)std::max(f.max_row, 0), 1);
  LJ_CUDA(ctx, f.ell.ensure(words), "alloc");
  LJ_CUDA(ctx, launch_csr_to_ell(f.np.ptr, f.ptr.ptr, f.list.ptr, f.n, f.n, f.ell.ptr,
                                 ctx->stream), "transposed list");
  f.evalid = true;
  return LJ_OK;
}

// Three events per timed force call: before the position-image pass, before
// the pair kernel, after it.
cudaEvent_t* timing_slot(lj_ctx* ctx) {
  if (!ctx->timing) return nullptr;
  while (ctx->tev.size() < ctx->tev_used + 3) {
    cudaEvent_t e;
    if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
    ctx->tev.push_back(e);
  }
  cudaEvent_t* s = ctx->tev.data() + ctx->tev_used;
  ctx->tev_used += 3;
  return s;
}

// A configuration chosen by lj_autotune_aos replaces the engine defaults when
// the caller leaves method (AUTO) and every launch field at zero, for the
// same precision, layout, boundary kind and list.
int layout_of(const Particles& part) {
  return part.soa ? LJ_LAYOUT_SOA : (part.stride == 8 ? LJ_LAYOUT_Z : LJ_LAYOUT_AOS);
}

const lj_force_opts* apply_tuned(lj_ctx* ctx, const lj_force_opts* o, int layout,
                                 lj_force_opts* scratch) {
  if (o->method != LJ_METHOD_AUTO || o->kernel || o->lanes || o->unroll || o->block) return o;
  for (const auto& t : ctx->tuned) {
    if (t.precision == o->precision && t.layout == layout && t.periodic == (o->periodic != 0) &&
        t.entries_half == ctx->half.entries && t.entries_full == ctx->full.entries &&
        t.n == (ctx->full.valid ? ctx->full.n : ctx->half.n)) {
      *scratch = *o;
      scratch->method = t.method;
      scratch->kernel = t.kernel;
      scratch->lanes = t.lanes;
      scratch->unroll = t.unroll;
      scratch->block = t.block;
      return scratch;
    }
  }
  return o;
}

// Access-policy window over the n-entry position image on the context's
// stream (lj_ctx_set_l2_window): persisting hits for l2_hit_ratio of it,
// within the device's largest window and the persisting L2 this context
// reserves on first use.
int set_l2_window(lj_ctx* ctx, const int4* image, int32_t n) {
  if (!ctx->stream)
    return fail(ctx, LJ_ERR_UNSUPPORTED,
                "the L2 window is a stream attribute: set a stream (lj_ctx_set_stream) first");
  int dev = ctx->device, max_window = 0, max_persist = 0;
  LJ_CUDA(ctx, cudaDeviceGetAttribute(&max_window, cudaDevAttrMaxAccessPolicyWindowSize, dev),
          "attribute");
  LJ_CUDA(ctx, cudaDeviceGetAttribute(&max_persist, cudaDevAttrMaxPersistingL2CacheSize, dev),
          "attribute");
  const size_t bytes = std::min<size_t>((size_t)n * sizeof(int4), (size_t)max_window);
  if (bytes == 0 || max_persist <= 0) return LJ_OK;  // no persisting L2 on this part
  if (!ctx->l2_limit_set) {
    LJ_CUDA(ctx, cudaDeviceGetLimit(&ctx->l2_limit_prev, cudaLimitPersistingL2CacheSize),
            "limit");
    LJ_CUDA(ctx, cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize,
                                    std::min<size_t>(bytes, (size_t)max_persist)),
            "limit");
    ctx->l2_limit_set = true;
  }
  cudaStreamAttrValue v{};
  v.accessPolicyWindow.base_ptr = const_cast<int4*>(image);
  v.accessPolicyWindow.num_bytes = bytes;
  v.accessPolicyWindow.hitRatio = (float)ctx->l2_hit_ratio;
  v.accessPolicyWindow.hitProp = cudaAccessPropertyPersisting;
  v.accessPolicyWindow.missProp = cudaAccessPropertyStreaming;
  LJ_CUDA(ctx, cudaStreamSetAttribute(ctx->stream, cudaStreamAttributeAccessPolicyWindow, &v),
          "window");
  return LJ_OK;
}

int run_force(lj_ctx* ctx, const Particles& part, int32_t n, const lj_force_opts* o_in) {
  int rc = check_opts(ctx, o_in);
  if (rc) return rc;
  lj_force_opts tuned_opts;
  const lj_force_opts* o = apply_tuned(ctx, o_in, layout_of(part), &tuned_opts);
  int method = LJ_METHOD_GATHER_FULL;
  if ((rc = resolve_method(ctx, o, &method))) return rc;
  const DevList& l = method == LJ_METHOD_SCATTER_HALF ? ctx->half : ctx->full;
  if (n != l.n)
    return fail(ctx, LJ_ERR_INVALID_ARGUMENT, "n = %d but the installed list has %d rows", n,
                l.n);
  ForceLaunch L{};
  L.part = part;
  L.csr = l.csr();
  L.box = make_periodic(o);
  L.dt = o->dt;
  L.cl2 = o->cl2;
  L.precision = o->precision;
  L.method = method;
  const bool mixed = o->precision != LJ_PREC_FP64;
  // The cell-tiled gather (kernel 3, FP32 pair terms only) runs only when
  // asked for or chosen by lj_autotune_aos; it needs the tiled rows
  // lj_list_build leaves behind.
  const bool tiled_ok = ctx->tiled.valid && o->precision == LJ_PREC_MIXED_FP32 &&
                        method == LJ_METHOD_GATHER_FULL && ctx->full.n == n;
  L.kernel = o->kernel ? o->kernel : 2;  // unrolled gather / scatter (mixed), compacted (FP64)
  if (L.kernel == 3 && !tiled_ok) L.kernel = 2;  // no tiled list: unrolled gather
  if (L.kernel == 4 && !(mixed && method == LJ_METHOD_GATHER_FULL && ctx->full.avalid &&
                         ctx->full.n == n))
    L.kernel = 2;  // no aligned copy: scalar index loads
  // the mixed scatter has kernels 1 (simple) and 2 (unrolled, vector atomics)
  if (L.kernel > 2 && method == LJ_METHOD_SCATTER_HALF) L.kernel = 2;
  // kernel 5: gather over the transposed copy of the full list, one lane per row
  if (L.kernel == 5) {
    if (o->lanes > 1)
      return fail(ctx, LJ_ERR_INVALID_ARGUMENT, "kernel 5 takes one lane per row (lanes 0 or 1)");
    if (mixed && o->unroll && o->unroll != 2 && o->unroll != 4)
      return fail(ctx, LJ_ERR_INVALID_ARGUMENT, "kernel 5 takes unroll 0, 2 or 4");
    if ((rc = ensure_ell(ctx))) return rc;
  }
  L.unroll = o->unroll ? o->unroll : 4;
  if (L.kernel == 4 && L.unroll != 4)
    return fail(ctx, LJ_ERR_INVALID_ARGUMENT, "kernel 4 takes 4 entries per lane (unroll 0 or 4)");
  if (L.kernel == 2 && !(L.unroll == 1 || L.unroll == 2 || L.unroll == 4 || L.unroll == 8))
    return fail(ctx, LJ_ERR_INVALID_ARGUMENT, "unroll must be 1, 2, 4 or 8");
  if (o->precision == LJ_PREC_MIXED && (L.kernel == 2 || method == LJ_METHOD_SCATTER_HALF) &&
      !(L.unroll == 2 || L.unroll == 4))
    return fail(ctx, LJ_ERR_UNSUPPORTED, "two-float pair terms take unroll 2 or 4");
  if (L.kernel == 3 && !(L.unroll == 2 || L.unroll == 4))
    return fail(ctx, LJ_ERR_INVALID_ARGUMENT, "unroll must be 2 or 4 for kernel 3");
  L.lanes = o->lanes ? o->lanes : default_lanes(o->precision, method, L.kernel, l.entries, l.n);
  if (L.kernel == 5) {
    L.lanes = 1;
    L.csr = ctx->full.ecsr();
  }
  if (L.kernel == 4) {  // kernel 2 over the 16-byte-aligned copy, vector index loads
    L.csr = ctx->full.acsr();
    L.kernel = 2;
  }
  L.block = o->block ? o->block : 128;
  if (n == 0) return LJ_OK;
  const bool fixed = mixed || L.kernel == 2;
  cudaEvent_t* tv = timing_slot(ctx);
  if (tv) LJ_CUDA(ctx, cudaEventRecord(tv[0], ctx->stream), "event");
  if (fixed) {
    LJ_CUDA(ctx, ctx->qfix.ensure((size_t)n), "alloc");
    L.qfix = ctx->qfix.ptr;
    if (!L.box.on) {
      // the fixed-point frame of an open box follows the per-axis bounds of
      // the coordinates; the kernels read it on the device (no host round
      // trip per call)
      LJ_CUDA(ctx, ctx->oframe.ensure(kOpenFrameWords), "alloc");
      if (!ctx->oframe_armed) {
        LJ_CUDA(ctx, launch_open_frame_init(ctx->oframe.ptr, ctx->stream), "frame init");
        ctx->oframe_armed = true;
      }
      LJ_CUDA(ctx, launch_open_bounds(part, n, ctx->oframe.ptr, ctx->stream), "bounds");
      make_device_frame(L, ctx->oframe.ptr);
    } else {
      make_fixed_frame(L);
    }
    if (mixed && method == LJ_METHOD_SCATTER_HALF) {
      // one float4 per particle (FP32 terms) or two (two-float terms)
      const size_t per = o->precision == LJ_PREC_MIXED ? 8 : 4;
      LJ_CUDA(ctx, ctx->fscratch.ensure(per * (size_t)n), "alloc");
      L.fscratch = ctx->fscratch.ptr;
      L.scratch_zeroed = 1;  // the image pass below clears it
    }
    if (L.kernel == 3 && L.aniso) L.kernel = 2;
    if (L.kernel == 3) {
      auto& T = ctx->tiled;
      TiledList tl{};
      tl.n = n;
      tl.ncells = T.grid.ncells;
      for (int d = 0; d < 3; d++) tl.gnc[d] = T.grid.nc[d];
      tl.periodic = T.grid.periodic;
      tl.order = T.order.ptr;
      tl.start = T.start.ptr;
      tl.rows = T.rows.ptr;
      tl.cnt = T.cnt.ptr;
      tl.maxrow = T.maxrow;
      tl.maxc_shift = T.maxc_shift;
      LJ_CUDA(ctx, launch_fixed_image_sorted(L, T.order.ptr, T.cq.ptr, ctx->stream), "image");
      if (tv) LJ_CUDA(ctx, cudaEventRecord(tv[1], ctx->stream), "event");
      LJ_CUDA(ctx, launch_force_tiled(L, tl, T.cq.ptr, ctx->stream), "tiled force");
      if (tv) LJ_CUDA(ctx, cudaEventRecord(tv[2], ctx->stream), "event");
      return LJ_OK;
    }
    LJ_CUDA(ctx, launch_fixed_image(L, ctx->stream), "fixed image");
    // two-float gathers (kernels 2 and 4) run the segment gather over a
    // near-first copy of the full list, ordered from these positions the
    // first time; later positions change its speed, not its precision
    if (o->precision == LJ_PREC_MIXED && method == LJ_METHOD_GATHER_FULL && L.kernel == 2 &&
        !o->ff_all) {
      DevList& f = ctx->full;
      const bool al = L.csr.aligned4 != 0;
      bool& ok = al ? f.savalid : f.svalid;
      DevBuf<int32_t>& buf = al ? f.salist : f.slist;
      DevBuf<int32_t>& nn = al ? f.sann : f.snn;
      if (!ok) {
        LJ_CUDA(ctx, buf.ensure((size_t)std::max<int64_t>(al ? f.aentries : f.entries, 4)),
                "alloc");
        LJ_CUDA(ctx, nn.ensure((size_t)n), "alloc");
        LJ_CUDA(ctx, launch_partition_near(L, L.csr, buf.ptr, nn.ptr, nullptr, ctx->stream),
                "near-first rows");
        ok = true;
      }
      if (!ctx->closef_zeroed) {
        LJ_CUDA(ctx, ctx->closef.ensure(3), "alloc");
        LJ_CUDA(ctx, cudaMemsetAsync(ctx->closef.ptr, 0, 3 * sizeof(int32_t), ctx->stream),
                "memset");
        ctx->closef_zeroed = true;
      }
      LJ_CUDA(ctx, ctx->closeq.ensure((size_t)n), "alloc");
      L.close_flag = ctx->closef.ptr;
      L.close_rows = ctx->closeq.ptr;
      // near part [0, nn), far part [nn, np) of every row
      L.csr.list = buf.ptr;
      L.far = L.csr;
      L.far.first = nn.ptr;
      L.csr.np = nn.ptr;
      L.split = 1;
    }
  }
  const bool window = ctx->l2_hit_ratio > 0.0 && L.qfix && n > 0;
  if (window && (rc = set_l2_window(ctx, L.qfix, n))) return rc;
  if (tv) LJ_CUDA(ctx, cudaEventRecord(tv[1], ctx->stream), "event");
  if (L.kernel == 5) LJ_CUDA(ctx, launch_force_ell(L, ctx->stream), "force launch");
  else LJ_CUDA(ctx, launch_force(L, ctx->stream), "force launch");
  if (tv) LJ_CUDA(ctx, cudaEventRecord(tv[2], ctx->stream), "event");
  if (window) {  // later launches on the stream run without the window
    cudaStreamAttrValue off{};
    off.accessPolicyWindow.num_bytes = 0;
    LJ_CUDA(ctx, cudaStreamSetAttribute(ctx->stream, cudaStreamAttributeAccessPolicyWindow, &off),
            "window off");
  }
  return LJ_OK;
}

bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

// ---- autotuner ---------------------------------------------------------------
struct TuneCand {
  int method, kernel, lanes, unroll, block;
};

// Launch shapes worth timing for this precision, method and installed lists.
std::vector<TuneCand> tune_candidates(lj_ctx* ctx, const lj_force_opts* opts) {
  std::vector<TuneCand> cands;
  const bool mixed = opts->precision != LJ_PREC_FP64;
  const bool ff = opts->precision == LJ_PREC_MIXED;  // two-float pair terms
  const bool try_gather = ctx->full.valid && opts->method != LJ_METHOD_SCATTER_HALF;
  const bool try_scatter = ctx->half.valid && opts->method != LJ_METHOD_GATHER_FULL;
  for (int block : {128, 256}) {
    if (try_gather) {
      if (mixed) {
        if (!ff && ctx->tiled.valid && block == 128)
          for (int g : {2, 4, 8})
            for (int u : {2, 4}) cands.push_back({LJ_METHOD_GATHER_FULL, 3, g, u, 128});
        for (int g : {1, 2, 4, 8})
          for (int u : {2, 4, 8})
            if (!(ff && u == 8)) cands.push_back({LJ_METHOD_GATHER_FULL, 2, g, u, block});
        if (ctx->full.avalid)
          for (int g : {1, 2, 4, 8}) cands.push_back({LJ_METHOD_GATHER_FULL, 4, g, 4, block});
        for (int g : {4, 8, 16}) cands.push_back({LJ_METHOD_GATHER_FULL, 1, g, 0, block});
        for (int u : {2, 4}) cands.push_back({LJ_METHOD_GATHER_FULL, 5, 1, u, block});
      } else {
        if (block == 128) cands.push_back({LJ_METHOD_GATHER_FULL, 2, 0, 0, 128});
        for (int g : {4, 8}) cands.push_back({LJ_METHOD_GATHER_FULL, 1, g, 0, block});
        cands.push_back({LJ_METHOD_GATHER_FULL, 5, 1, 0, block});
      }
    }
    if (try_scatter) {
      if (!mixed && block == 128)
        for (int g : {1, 2, 4, 8}) cands.push_back({LJ_METHOD_SCATTER_HALF, 2, g, 0, 128});
      if (mixed)
        for (int g : {1, 2, 4, 8})
          for (int u : {2, 4}) cands.push_back({LJ_METHOD_SCATTER_HALF, 2, g, u, block});
      if (!ff)  // two-float scatters always run kernel 2
        for (int g : {2, 4, 8}) cands.push_back({LJ_METHOD_SCATTER_HALF, 1, g, 0, block});
    }
  }
  return cands;
}

lj_force_opts with_shape(const lj_force_opts* opts, const TuneCand& c) {
  lj_force_opts o = *opts;
  o.method = c.method;
  o.kernel = c.kernel;
  o.lanes = c.lanes;
  o.unroll = c.unroll;
  o.block = c.block;
  return o;
}

// Mean time of `reps` calls of shape c on `part`, each call after a write
// larger than L2 (a force call on a list that does not fit in L2 -- or a
// benchmark that flushes -- starts cold; warm-cache timings favour other
// shapes).  One untimed call first (warm-up and validity).
int time_shape(lj_ctx* ctx, const Particles& part, int32_t n, const lj_force_opts* opts,
               const TuneCand& c, int reps, double* ms_out) {
  const lj_force_opts o = with_shape(opts, c);
  int rc = run_force(ctx, part, n, &o);
  if (rc) return rc;
  float ms = 0.f;
  for (int r = 0; r < reps; r++) {
    LJ_CUDA(ctx, cudaMemsetAsync(ctx->tune_flush.ptr, r & 0xff, ctx->tune_flush.cap, ctx->stream),
            "flush");
    LJ_CUDA(ctx, cudaEventRecord(ctx->ev[0], ctx->stream), "event");
    if ((rc = run_force(ctx, part, n, &o))) return rc;
    LJ_CUDA(ctx, cudaEventRecord(ctx->ev[1], ctx->stream), "event");
    LJ_CUDA(ctx, cudaEventSynchronize(ctx->ev[1]), "sync");
    float t = 0.f;
    cudaEventElapsedTime(&t, ctx->ev[0], ctx->ev[1]);
    ms += t;
  }
  *ms_out = ms / reps;
  return LJ_OK;
}

// The particles of one layout for timing: AoS is the caller's q (momenta in
// tune_p); SoA and z are copies of q the tuner makes (momenta zeroed).
int tune_particles(lj_ctx* ctx, const double* q, int32_t n, int layout, Particles* part) {
  *part = Particles{};
  cudaStream_t s = ctx->stream;
  if (layout == LJ_LAYOUT_AOS) {
    part->q = q;
    part->p = ctx->tune_p.ptr;
    return LJ_OK;
  }
  if (layout == LJ_LAYOUT_SOA) {
    LJ_CUDA(ctx, ctx->tune_soa.ensure(6 * (size_t)n), "alloc");
    double* b = ctx->tune_soa.ptr;
    for (int d = 0; d < 3; d++)
      LJ_CUDA(ctx, cudaMemcpy2DAsync(b + (size_t)d * n, sizeof(double), q + d, 4 * sizeof(double),
                                     sizeof(double), (size_t)n, cudaMemcpyDeviceToDevice, s),
              "SoA copy");
    LJ_CUDA(ctx, cudaMemsetAsync(b + 3 * (size_t)n, 0, 3 * sizeof(double) * (size_t)n, s),
            "memset");
    part->soa = 1;
    part->qx = b;
    part->qy = b + n;
    part->qz = b + 2 * (size_t)n;
    part->px = b + 3 * (size_t)n;
    part->py = b + 4 * (size_t)n;
    part->pz = b + 5 * (size_t)n;
    return LJ_OK;
  }
  LJ_CUDA(ctx, ctx->tune_z.ensure(8 * (size_t)n), "alloc");
  double* z = ctx->tune_z.ptr;
  LJ_CUDA(ctx, cudaMemsetAsync(z, 0, 8 * sizeof(double) * (size_t)n, s), "memset");
  LJ_CUDA(ctx, cudaMemcpy2DAsync(z, 8 * sizeof(double), q, 4 * sizeof(double), 4 * sizeof(double),
                                 (size_t)n, cudaMemcpyDeviceToDevice, s),
          "z copy");
  part->stride = 8;
  part->q = z;
  part->p = z + 4;
  return LJ_OK;
}

// The cache key of a tuning problem (see lj_tune_result::key).
std::string tune_key(lj_ctx* ctx, int32_t n, const lj_force_opts* opts, int layouts) {
  cudaDeviceProp prop{};
  cudaGetDeviceProperties(&prop, ctx->device);
  std::string gpu = prop.name;
  for (char& ch : gpu)
    if (ch == ' ' || ch == '\t' || ch == '|') ch = '_';
  double mean = 0.0;
  if (ctx->full.valid && ctx->full.n > 0) mean = (double)ctx->full.entries / ctx->full.n;
  else if (ctx->half.valid && ctx->half.n > 0) mean = 2.0 * (double)ctx->half.entries / ctx->half.n;
  const int nclass = n > 0 ? (int)std::floor(std::log2((double)n)) : 0;
  const int rclass = mean > 0.0 ? (int)std::lround(2.0 * std::log2(mean)) : -1;
  char buf[160];
  std::snprintf(buf, sizeof buf, "%s|sm%d|n2^%d|row2^%d/2|prec%d|pbc%d|m%d|lay%d",
                gpu.c_str(), prop.multiProcessorCount, nclass, rclass, opts->precision,
                opts->periodic ? 1 : 0, opts->method, layouts);
  return buf;
}

// Cache file: one line per entry, "key method kernel lanes unroll block
// layout ms"; the last line of a key wins.
bool cache_lookup(const char* path, const std::string& key, TuneCand* c, int* layout, double* ms) {
  FILE* f = std::fopen(path, "r");
  if (!f) return false;
  char line[512];
  bool found = false;
  while (std::fgets(line, sizeof line, f)) {
    char k[256];
    TuneCand t{};
    int lay = 0;
    double m = 0.0;
    if (std::sscanf(line, "%255s %d %d %d %d %d %d %lf", k, &t.method, &t.kernel, &t.lanes,
                    &t.unroll, &t.block, &lay, &m) == 8 &&
        key == k) {
      *c = t;
      *layout = lay;
      *ms = m;
      found = true;
    }
  }
  std::fclose(f);
  return found;
}

void remember_tuned(lj_ctx* ctx, const lj_force_opts* opts, int32_t n, int layout,
                    const TuneCand& c) {
  lj_ctx::Tuned t{};
  t.precision = opts->precision;
  t.layout = layout;
  t.periodic = opts->periodic != 0;
  t.n = n;
  t.entries_half = ctx->half.entries;
  t.entries_full = ctx->full.entries;
  t.method = c.method;
  t.kernel = c.kernel;
  t.lanes = c.lanes;
  t.unroll = c.unroll;
  t.block = c.block;
  auto& v = ctx->tuned;
  v.erase(std::remove_if(v.begin(), v.end(), [&](const lj_ctx::Tuned& x) {
            return x.precision == t.precision && x.layout == t.layout && x.periodic == t.periodic;
          }),
          v.end());
  v.push_back(t);
}

int autotune(lj_ctx* ctx, const double* q, int32_t n, const lj_force_opts* opts, int reps,
             int layouts, const char* cache_path, lj_tune_result* out) {
  int rc = check_opts(ctx, opts);
  if (rc) return rc;
  if (n < 1 || !q || !aligned16(q)) return fail(ctx, LJ_ERR_INVALID_ARGUMENT, "bad q or n");
  if (!ctx->half.valid && !ctx->full.valid) return fail(ctx, LJ_ERR_NO_LIST, "no list installed");
  if (cudaSetDevice(ctx->device) != cudaSuccess) return fail(ctx, LJ_ERR_CUDA, "set device");
  *out = lj_tune_result{};
  const std::string key = tune_key(ctx, n, opts, layouts);
  std::snprintf(out->key, sizeof out->key, "%s", key.c_str());
  TuneCand win{};
  int win_layout = LJ_LAYOUT_AOS;
  double best_ms = 1e300;
  if (cache_path && cache_lookup(cache_path, key, &win, &win_layout, &best_ms)) {
    out->from_cache = 1;
  } else {
    std::vector<TuneCand> cands = tune_candidates(ctx, opts);
    if (cands.empty()) return fail(ctx, LJ_ERR_NO_LIST, "no list for the requested method");
    LJ_CUDA(ctx, ctx->tune_p.ensure(4 * (size_t)n), "alloc");
    LJ_CUDA(ctx, ctx->tune_flush.ensure((size_t)256 << 20), "alloc");  // > L2 (126 MB)
    const bool was_timing = ctx->timing;
    ctx->timing = false;
    struct Timed {
      TuneCand c;
      double ms;
    };
    std::vector<Timed> aos;
    Particles part{};
    for (const TuneCand& c : cands) {
      double ms = 0.0;
      if ((rc = tune_particles(ctx, q, n, LJ_LAYOUT_AOS, &part)) ||
          (rc = time_shape(ctx, part, n, opts, c, reps, &ms))) {
        ctx->timing = was_timing;
        return rc;
      }
      out->timed++;
      aos.push_back({c, ms});
    }
    std::stable_sort(aos.begin(), aos.end(),
                     [](const Timed& a, const Timed& b) { return a.ms < b.ms; });
    if (layouts & (1 << LJ_LAYOUT_AOS)) {
      win = aos[0].c;
      best_ms = aos[0].ms;
    }
    // the other layouts: the three fastest AoS shapes again
    for (int lay : {LJ_LAYOUT_SOA, LJ_LAYOUT_Z}) {
      if (!(layouts & (1 << lay))) continue;
      if ((rc = tune_particles(ctx, q, n, lay, &part))) {
        ctx->timing = was_timing;
        return rc;
      }
      for (size_t k = 0; k < aos.size() && k < 3; k++) {
        double ms = 0.0;
        if ((rc = time_shape(ctx, part, n, opts, aos[k].c, reps, &ms))) {
          ctx->timing = was_timing;
          return rc;
        }
        out->timed++;
        if (ms < best_ms) {
          best_ms = ms;
          win = aos[k].c;
          win_layout = lay;
        }
      }
    }
    ctx->timing = was_timing;
    if (cache_path) {
      if (FILE* f = std::fopen(cache_path, "a")) {
        std::fprintf(f, "%s %d %d %d %d %d %d %.6g\n", key.c_str(), win.method, win.kernel,
                     win.lanes, win.unroll, win.block, win_layout, best_ms);
        std::fclose(f);
      }
    }
  }
  out->best = with_shape(opts, win);
  out->layout = win_layout;
  out->ms = best_ms;
  remember_tuned(ctx, opts, n, win_layout, win);
  return LJ_OK;
}

}  // namespace

extern "C" {

void lj_force_opts_default(lj_force_opts* o) {
  if (!o) return;
  std::memset(o, 0, sizeof *o);
  o->dt = 0.001;
  o->cl2 = 9.0;
  o->precision = LJ_PREC_FP64;
  o->method = LJ_METHOD_AUTO;
}

int lj_abi_version(void) { return LJ_GB300_ABI_VERSION; }

const char* lj_status_string(int s) {
  switch (s) {
    case LJ_OK: return "ok";
    case LJ_ERR_INVALID_ARGUMENT: return "invalid argument";
    case LJ_ERR_BAD_LIST: return "neighbour list failed validation";
    case LJ_ERR_CUDA: return "CUDA error";
    case LJ_ERR_OUT_OF_MEMORY: return "out of memory";
    case LJ_ERR_LIST_OVERFLOW: return "list capacity exceeded";
    case LJ_ERR_TIMEOUT: return "device wait timed out";
    case LJ_ERR_NO_LIST: return "no neighbour list installed";
    case LJ_ERR_UNSUPPORTED: return "unsupported combination";
    default: return "unknown status";
  }
}

int lj_ctx_create(lj_ctx** out, int device) {
  if (!out) return LJ_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) return LJ_ERR_CUDA;
  if (device < 0 || device >= count) return LJ_ERR_INVALID_ARGUMENT;
  if (cudaSetDevice(device) != cudaSuccess) return LJ_ERR_CUDA;
  lj_ctx* c = new (std::nothrow) lj_ctx();
  if (!c) return LJ_ERR_OUT_OF_MEMORY;
  c->device = device;
  for (auto& e : c->ev)
    if (cudaEventCreate(&e) != cudaSuccess) {
      lj_ctx_destroy(c);
      return LJ_ERR_CUDA;
    }
  *out = c;
  return LJ_OK;
}

void lj_ctx_destroy(lj_ctx* ctx) {
  if (!ctx) return;
  cudaSetDevice(ctx->device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  else cudaDeviceSynchronize();
  if (ctx->l2_limit_set) {  // the persisting-L2 reservation this context made
    cudaCtxResetPersistingL2Cache();
    cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, ctx->l2_limit_prev);
  }
  for (auto& e : ctx->ev)
    if (e) cudaEventDestroy(e);
  for (auto& e : ctx->tev) cudaEventDestroy(e);
  delete ctx;
}

const char* lj_ctx_last_error(const lj_ctx* ctx) { return ctx ? ctx->err.c_str() : ""; }

int lj_ctx_set_l2_window(lj_ctx* ctx, double hit_ratio) {
  if (!ctx) return LJ_ERR_INVALID_ARGUMENT;
  ctx->err.clear();
  if (!(hit_ratio >= 0.0 && hit_ratio <= 1.0))
    return fail(ctx, LJ_ERR_INVALID_ARGUMENT, "hit_ratio must be in [0, 1]");
  ctx->l2_hit_ratio = hit_ratio;
  return LJ_OK;
}

int lj_ctx_set_timing(lj_ctx* ctx, int32_t on) {
  if (!ctx) return LJ_ERR_INVALID_ARGUMENT;
  if (cudaSetDevice(ctx->device) != cudaSuccess) return fail(ctx, LJ_ERR_CUDA, "set device");
  if (ctx->tev_used) cudaStreamSynchronize(ctx->stream);
  ctx->timing = on != 0;
  ctx->tev_used = 0;
  ctx->t_ms[0] = ctx->t_ms[1] = ctx->t_ms[2] = 0.0;
  ctx->t_calls = 0;
  return LJ_OK;
}

int lj_ctx_get_timing(lj_ctx* ctx, double* ms, int64_t* calls) {
  if (!ctx) return LJ_ERR_INVALID_ARGUMENT;
  if (cudaSetDevice(ctx->device) != cudaSuccess) return fail(ctx, LJ_ERR_CUDA, "set device");
  for (size_t k = 0; k + 2 < ctx->tev_used; k += 3) {
    LJ_CUDA(ctx, cudaEventSynchronize(ctx->tev[k + 2]), "event sync");
    float a = 0.f, b = 0.f;
    LJ_CUDA(ctx, cudaEventElapsedTime(&a, ctx->tev[k], ctx->tev[k + 1]), "elapsed");
    LJ_CUDA(ctx, cudaEventElapsedTime(&b, ctx->tev[k + 1], ctx->tev[k + 2]), "elapsed");
    ctx->t_ms[0] += a;
    ctx->t_ms[1] += b;
    ctx->t_ms[2] += a + b;
    ctx->t_calls++;
  }
  ctx->tev_used = 0;
  if (ms) {
    ms[0] = ctx->t_ms[0];
    ms[1] = ctx->t_ms[1];
    ms[2] = ctx->t_ms[2];
  }
  if (calls) *calls = ctx->t_calls;
  return LJ_OK;
}

int lj_ctx_set_stream(lj_ctx* ctx, void* stream) {
  if (!ctx) return LJ_ERR_INVALID_ARGUMENT;
  ctx->stream = static_cast<cudaStream_t>(stream);
  return LJ_OK;
}

int lj_list_set_csr(lj_ctx* ctx, int32_t n, const int32_t* np, const int32_t* ptr,
                    const int32_t* list, int64_t entries, int32_t kind, int32_t where) {
  if (!ctx) return LJ_ERR_INVALID_ARGUMENT;
  ctx->err.clear();
  if (n < 0 || entries < 0 || entries > 0x7fffffffll)
    return fail(ctx, LJ_ERR_INVALID_ARGUMENT, "n and n_entries must be in [0, 2^31)");
  if (kind != LJ_LIST_HALF && kind != LJ_LIST_FULL)
    return fail(ctx, LJ_ERR_INVALID_ARGUMENT, "unknown list kind %d", kind);
  if (where != LJ_WHERE_HOST && where != LJ_WHERE_DEVICE)
    return fail(ctx, LJ_ERR_INVALID_ARGUMENT, "unknown location %d", where);
  if ((n > 0 && (!np || !ptr)) || (entries > 0 && !list))
    return fail(ctx, LJ_ERR_INVALID_ARGUMENT, "null list array");
  if (cudaSetDevice(ctx->device) != cudaSuccess) return fail(ctx, LJ_ERR_CUDA, "set device");
  int rc = install_csr(ctx, n, np, ptr, list, entries, kind, where);
  if (rc) return rc;
  ctx->list_from_host = where == LJ_WHERE_HOST;
  ctx->host_kind = kind;
  if (ctx->list_from_host) {
    // the compact form actually installed, re-uploaded by lj_measure_aos
    const DevList& l = kind == LJ_LIST_HALF ? ctx->half : ctx->full;
    ctx->h_np.resize((size_t)n);
    ctx->h_ptr.resize((size_t)n);
    ctx->h_list.resize((size_t)l.entries);
    if (n > 0) {
      LJ_CUDA(ctx, cudaMemcpy(ctx->h_np.data(), l.np.ptr, sizeof(int32_t) * (size_t)n,
                              cudaMemcpyDeviceToHost), "copy");
      LJ_CUDA(ctx, cudaMemcpy(ctx->h_ptr.data(), l.ptr.ptr, sizeof(int32_t) * (size_t)n,
                              cudaMemcpyDeviceToHost), "copy");
    }
    if (l.entries > 0)
      LJ_CUDA(ctx, cudaMemcpy(ctx->h_list.data(), l.list.ptr,
                              sizeof(int32_t) * (size_t)l.entries, cudaMemcpyDeviceToHost),
              "copy");
  } else {
    ctx->h_np.clear();
    ctx->h_ptr.clear();
    ctx->h_list.clear();
  }
  return LJ_OK;
}

int lj_list_set_pairs(lj_ctx* ctx, int32_t n, const int32_t* ip, const int32_t* jp,
                      int64_t npairs, int32_t where) {
  if (!ctx) return LJ_ERR_INVALID_ARGUMENT;
  ctx->err.clear();
  if (n < 0 || npairs < 0 || npairs > 0x7fffffffll)
    return fail(ctx, LJ_ERR_INVALID_ARGUMENT, "n and n_pairs must be in [0, 2^31)");
  if (where != LJ_WHERE_HOST && where != LJ_WHERE_DEVICE)
    return fail(ctx, LJ_ERR_INVALID_ARGUMENT, "unknown location %d", where);
  if (npairs > 0 && (!ip || !jp)) return fail(ctx, LJ_ERR_INVALID_ARGUMENT, "null pair array");
  if (cudaSetDevice(ctx->device) != cudaSuccess) return fail(ctx, LJ_ERR_CUDA, "set device");
  // Pair arrays in makepair order (non-decreasing i) are sorted on the device:
  // the CSR list is then j_particles itself.  Any other order is sorted with a
  // stable counting sort on the host, as the reference's sortpair does.
  std::vector<int32_t> hi, hj;
  const int32_t* dj = jp;
  bool sorted_input = true;
  if (where == LJ_WHERE_HOST) {
    for (int64_t k = 1; k < npairs && sorted_input; k++) sorted_input = ip[k - 1] <= ip[k];
  }
  if (where == LJ_WHERE_DEVICE) {
    LJ_CUDA(ctx, ctx->tmp_i32a.ensure((size_t)n), "alloc");
    LJ_CUDA(ctx, ctx->err2.ensure(2), "alloc");
    const int32_t init[2] = {0, 0x7fffffff};
    LJ_CUDA(ctx, cudaMemcpyAsync(ctx->err2.ptr, init, sizeof init, cudaMemcpyHostToDevice,
                                 ctx->stream), "err init");
    LJ_CUDA(ctx, launch_pairs_count(ip, npairs, n, ctx->tmp_i32a.ptr, ctx->err2.ptr,
                                    ctx->stream), "pairs count");
    int32_t out[2];
    LJ_CUDA(ctx, cudaMemcpyAsync(out, ctx->err2.ptr, sizeof out, cudaMemcpyDeviceToHost,
                                 ctx->stream), "err read");
    LJ_CUDA(ctx, cudaStreamSynchronize(ctx->stream), "sync");
    if (out[0] == 4) return fail(ctx, LJ_ERR_BAD_LIST, "i_particles[%d] out of range", out[1]);
    sorted_input = out[0] == 0;
    if (!sorted_input) {
      hi.resize((size_t)npairs);
      hj.resize((size_t)npairs);
      LJ_CUDA(ctx, cudaMemcpy(hi.data(), ip, sizeof(int32_t) * (size_t)npairs,
                              cudaMemcpyDeviceToHost), "pairs read");
      LJ_CUDA(ctx, cudaMemcpy(hj.data(), jp, sizeof(int32_t) * (size_t)npairs,
                              cudaMemcpyDeviceToHost), "pairs read");
      ip = hi.data();
      jp = hj.data();
      where = LJ_WHERE_HOST;
    }
  }
  if (where == LJ_WHERE_HOST) {
    std::vector<int32_t> np((size_t)n, 0), ptr((size_t)n, 0), list((size_t)npairs);
    for (int64_t k = 0; k < npairs; k++) {
      if (ip[k] < 0 || ip[k] >= n)
        return fail(ctx, LJ_ERR_BAD_LIST, "i_particles[%lld] out of range", (long long)k);
      np[(size_t)ip[k]]++;
    }
    int64_t pos = 0;
    for (int i = 0; i < n; i++) {
      ptr[(size_t)i] = (int32_t)pos;
      pos += np[(size_t)i];
    }
    std::vector<int32_t> cur(ptr);
    for (int64_t k = 0; k < npairs; k++) list[(size_t)cur[(size_t)ip[k]]++] = jp[k];
    return lj_list_set_csr(ctx, n, np.data(), ptr.data(), list.data(), npairs, LJ_LIST_HALF,
                           LJ_WHERE_HOST);
  }
  // device, non-decreasing i: counts are in tmp_i32a; offsets by scan
  LJ_CUDA(ctx, ctx->tmp_off.ensure((size_t)n + 1), "alloc");
  LJ_CUDA(ctx, ctx->tmp_scan.ensure(scan_tmp_bytes(n)), "alloc");
  LJ_CUDA(ctx, launch_scan_counts(ctx->tmp_i32a.ptr, n, ctx->tmp_off.ptr, ctx->tmp_scan.ptr,
                                  ctx->tmp_scan.cap, ctx->stream), "scan");
  DevBuf<int32_t> np_d, ptr_d;
  LJ_CUDA(ctx, np_d.ensure((size_t)n), "alloc");
  LJ_CUDA(ctx, ptr_d.ensure((size_t)n), "alloc");
  LJ_CUDA(ctx, ctx->err2.ensure(2), "alloc");
  LJ_CUDA(ctx, launch_offsets_to_ptr(ctx->tmp_off.ptr, n, ptr_d.ptr, np_d.ptr, ctx->err2.ptr,
                                     ctx->stream), "ptr");
  LJ_CUDA(ctx, cudaStreamSynchronize(ctx->stream), "sync");
  return lj_list_set_csr(ctx, n, np_d.ptr, ptr_d.ptr, dj, npairs, LJ_LIST_HALF,
                         LJ_WHERE_DEVICE);
}

int lj_list_get_csr(lj_ctx* ctx, int32_t kind, int32_t* np, int32_t* ptr, int32_t* list,
                    int64_t capacity, int64_t* n_entries, int32_t where) {
  if (!ctx) return LJ_ERR_INVALID_ARGUMENT;
  if (kind != LJ_LIST_HALF && kind != LJ_LIST_FULL)
    return fail(ctx, LJ_ERR_INVALID_ARGUMENT, "unknown list kind %d", kind);
  if (where != LJ_WHERE_HOST && where != LJ_WHERE_DEVICE)
    return fail(ctx, LJ_ERR_INVALID_ARGUMENT, "unknown location %d", where);
  const DevList& l = kind == LJ_LIST_HALF ? ctx->half : ctx->full;
  if (!l.valid) return fail(ctx, LJ_ERR_NO_LIST, "no list of that kind installed");
  if (n_entries) *n_entries = l.entries;
  if (capacity < l.entries) return fail(ctx, LJ_ERR_LIST_OVERFLOW, "capacity too small");
  if ((l.n > 0 && (!np || !ptr)) || (l.entries > 0 && !list))
    return fail(ctx, LJ_ERR_INVALID_ARGUMENT, "null output array");
  if (cudaSetDevice(ctx->device) != cudaSuccess) return fail(ctx, LJ_ERR_CUDA, "set device");
  const cudaMemcpyKind k =
      where == LJ_WHERE_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
  if (l.n > 0) {
    LJ_CUDA(ctx, cudaMemcpyAsync(np, l.np.ptr, sizeof(int32_t) * (size_t)l.n, k, ctx->stream),
            "copy");
    LJ_CUDA(ctx, cudaMemcpyAsync(ptr, l.ptr.ptr, sizeof(int32_t) * (size_t)l.n, k, ctx->stream),
            "copy");
  }
  if (l.entries > 0)
    LJ_CUDA(ctx, cudaMemcpyAsync(list, l.list.ptr, sizeof(int32_t) * (size_t)l.entries, k,
                                 ctx->stream), "copy");
  LJ_CUDA(ctx, cudaStreamSynchronize(ctx->stream), "sync");
  return LJ_OK;
}

int lj_list_info(const lj_ctx* ctx, int32_t kind, int32_t* n, int64_t* n_entries,
                 int32_t* max_row) {
  if (!ctx || (kind != LJ_LIST_HALF && kind != LJ_LIST_FULL)) return LJ_ERR_INVALID_ARGUMENT;
  const DevList& l = kind == LJ_LIST_HALF ? ctx->half : ctx->full;
  if (n) *n = l.valid ? l.n : 0;
  if (n_entries) *n_entries = l.valid ? l.entries : 0;
  if (max_row) *max_row = l.valid ? l.max_row : 0;
  return LJ_OK;
}

int lj_force_aos(lj_ctx* ctx, const double* q, double* p, int32_t n, const lj_force_opts* o) {
  if (!ctx) return LJ_ERR_INVALID_ARGUMENT;
  ctx->err.clear();
  if (n < 0) return fail(ctx, LJ_ERR_INVALID_ARGUMENT, "n < 0");
  if (n > 0 && (!q || !p)) return fail(ctx, LJ_ERR_INVALID_ARGUMENT, "null q or p");
  if (!aligned16(q) || !aligned16(p))
    return fail(ctx, LJ_ERR_INVALID_ARGUMENT, "AoS q and p must be 16-byte aligned");
  if (cudaSetDevice(ctx->device) != cudaSuccess) return fail(ctx, LJ_ERR_CUDA, "set device");
  Particles part{};
  part.soa = 0;
  part.q = q;
  part.p = p;
  return run_force(ctx, part, n, o);
}

int lj_force_soa(lj_ctx* ctx, const double* qx, const double* qy, const double* qz, double* px,
                 double* py, double* pz, int32_t n, const lj_force_opts* o) {
  if (!ctx) return LJ_ERR_INVALID_ARGUMENT;
  ctx->err.clear();
  if (n < 0) return fail(ctx, LJ_ERR_INVALID_ARGUMENT, "n < 0");
  if (n > 0 && (!qx || !qy || !qz || !px || !py || !pz))
    return fail(ctx, LJ_ERR_INVALID_ARGUMENT, "null SoA array");
  if (cudaSetDevice(ctx->device) != cudaSuccess) return fail(ctx, LJ_ERR_CUDA, "set device");
  Particles part{};
  part.soa = 1;
  part.qx = qx;
  part.qy = qy;
  part.qz = qz;
  part.px = px;
  part.py = py;
  part.pz = pz;
  return run_force(ctx, part, n, o);
}

int lj_force_z(lj_ctx* ctx, double* z, int32_t n, const lj_force_opts* o) {
  if (!ctx) return LJ_ERR_INVALID_ARGUMENT;
  ctx->err.clear();
  if (n < 0) return fail(ctx, LJ_ERR_INVALID_ARGUMENT, "n < 0");
  if (n > 0 && !z) return fail(ctx, LJ_ERR_INVALID_ARGUMENT, "null z");
  if (!aligned16(z)) return fail(ctx, LJ_ERR_INVALID_ARGUMENT, "z must be 16-byte aligned");
  if (cudaSetDevice(ctx->device) != cudaSuccess) return fail(ctx, LJ_ERR_CUDA, "set device");
  Particles part{};
  part.soa = 0;
  part.stride = 8;
  part.q = z;
  part.p = z + 4;
  return run_force(ctx, part, n, o);
}

int lj_list_set_ell(lj_ctx* ctx, int32_t n, const int32_t* np, const int32_t* ell,
                    int64_t width, int64_t ell_len, int32_t kind, int32_t where) {
  if (!ctx) return LJ_ERR_INVALID_ARGUMENT;
  ctx->err.clear();
  if (n < 0 || width < n || ell_len < 0 || (n > 0 && (!np || (!ell && ell_len > 0))))
    return fail(ctx, LJ_ERR_INVALID_ARGUMENT, "bad ELL arguments (width must be >= n)");
  if (kind != LJ_LIST_HALF && kind != LJ_LIST_FULL)
    return fail(ctx, LJ_ERR_INVALID_ARGUMENT, "unknown list kind %d", kind);
  if (where != LJ_WHERE_HOST && where != LJ_WHERE_DEVICE)
    return fail(ctx, LJ_ERR_INVALID_ARGUMENT, "unknown location %d", where);
  if (cudaSetDevice(ctx->device) != cudaSuccess) return fail(ctx, LJ_ERR_CUDA, "set device");
  cudaStream_t s = ctx->stream;
  DevBuf<int32_t> d_np, d_ell, d_ptr, d_list;
  DevBuf<int64_t> d_off;
  LJ_CUDA(ctx, d_np.ensure((size_t)n), "alloc");
  LJ_CUDA(ctx, d_ell.ensure((size_t)ell_len), "alloc");
  int rc;
  if ((rc = copy_in(ctx, d_np.ptr, np, (size_t)n, where))) return rc;
  if ((rc = copy_in(ctx, d_ell.ptr, ell, (size_t)ell_len, where))) return rc;
  LJ_CUDA(ctx, ctx->err2.ensure(2), "alloc");
  const int32_t init[2] = {0, 0x7fffffff};
  LJ_CUDA(ctx, cudaMemcpyAsync(ctx->err2.ptr, init, sizeof init, cudaMemcpyHostToDevice, s),
          "err init");
  LJ_CUDA(ctx, launch_ell_check(d_np.ptr, n, width, ell_len, ctx->err2.ptr, s), "check");
  int32_t out[2];
  LJ_CUDA(ctx, cudaMemcpyAsync(out, ctx->err2.ptr, sizeof out, cudaMemcpyDeviceToHost, s),
          "read");
  LJ_CUDA(ctx, cudaStreamSynchronize(s), "sync");
  if (out[0] == 1)
    return fail(ctx, LJ_ERR_BAD_LIST, "number_of_partners[%d] out of range", out[1]);
  if (out[0] == 3)
    return fail(ctx, LJ_ERR_BAD_LIST, "row %d runs past the end of the transposed list", out[1]);
  LJ_CUDA(ctx, d_off.ensure((size_t)n + 1), "alloc");
  LJ_CUDA(ctx, ctx->tmp_scan.ensure(scan_tmp_bytes(n)), "alloc");
  LJ_CUDA(ctx, launch_scan_counts(d_np.ptr, n, d_off.ptr, ctx->tmp_scan.ptr, ctx->tmp_scan.cap,
                                  s), "scan");
  int64_t total = 0;
  LJ_CUDA(ctx, cudaMemcpyAsync(&total, d_off.ptr + n, sizeof total, cudaMemcpyDeviceToHost, s),
          "total");
  LJ_CUDA(ctx, cudaStreamSynchronize(s), "sync");
  if (total > 0x7fffffffll) return fail(ctx, LJ_ERR_UNSUPPORTED, "list exceeds 2^31 entries");
  LJ_CUDA(ctx, d_list.ensure((size_t)std::max<int64_t>(total, 1)), "alloc");
  LJ_CUDA(ctx, d_ptr.ensure((size_t)n), "alloc");
  LJ_CUDA(ctx, launch_ell_to_csr(d_np.ptr, d_ell.ptr, n, width, d_off.ptr, d_list.ptr, s),
          "transpose");
  LJ_CUDA(ctx, launch_offsets_to_ptr(d_off.ptr, n, d_ptr.ptr, d_np.ptr, ctx->err2.ptr, s), "ptr");
  LJ_CUDA(ctx, cudaStreamSynchronize(s), "sync");
  return lj_list_set_csr(ctx, n, d_np.ptr, d_ptr.ptr, d_list.ptr, total, kind, LJ_WHERE_DEVICE);
}

int lj_list_get_ell(lj_ctx* ctx, int32_t kind, int32_t* np, int32_t* ell, int64_t width,
                    int64_t ell_len, int32_t where) {
  if (!ctx) return LJ_ERR_INVALID_ARGUMENT;
  ctx->err.clear();
  if (kind != LJ_LIST_HALF && kind != LJ_LIST_FULL)
    return fail(ctx, LJ_ERR_INVALID_ARGUMENT, "unknown list kind %d", kind);
  if (where != LJ_WHERE_HOST && where != LJ_WHERE_DEVICE)
    return fail(ctx, LJ_ERR_INVALID_ARGUMENT, "unknown location %d", where);
  const DevList& l = kind == LJ_LIST_HALF ? ctx->half : ctx->full;
  if (!l.valid) return fail(ctx, LJ_ERR_NO_LIST, "no list of that kind installed");
  if (width < l.n) return fail(ctx, LJ_ERR_INVALID_ARGUMENT, "width must be >= n");
  if ((int64_t)l.max_row * width > ell_len)
    return fail(ctx, LJ_ERR_LIST_OVERFLOW, "transposed list needs %lld entries",
                (long long)((int64_t)l.max_row * width));
  if (l.n > 0 && (!np || !ell)) return fail(ctx, LJ_ERR_INVALID_ARGUMENT, "null output");
  if (cudaSetDevice(ctx->device) != cudaSuccess) return fail(ctx, LJ_ERR_CUDA, "set device");
  cudaStream_t s = ctx->stream;
  DevBuf<int32_t> d_ell;
  int32_t* dst = ell;
  if (where == LJ_WHERE_HOST) {
    LJ_CUDA(ctx, d_ell.ensure((size_t)std::max<int64_t>(ell_len, 1)), "alloc");
    dst = d_ell.ptr;
  }
  // zero-filled first, as make_transposed_pairlist does (set_val(0))
  LJ_CUDA(ctx, cudaMemsetAsync(dst, 0, sizeof(int32_t) * (size_t)ell_len, s), "memset");
  LJ_CUDA(ctx, launch_csr_to_ell(l.np.ptr, l.ptr.ptr, l.list.ptr, l.n, width, dst, s),
          "transpose");
  const cudaMemcpyKind k = where == LJ_WHERE_HOST ? cudaMemcpyDeviceToHost
                                                  : cudaMemcpyDeviceToDevice;
  if (where == LJ_WHERE_HOST)
    LJ_CUDA(ctx, cudaMemcpyAsync(ell, dst, sizeof(int32_t) * (size_t)ell_len, k, s), "copy");
  if (l.n > 0)
    LJ_CUDA(ctx, cudaMemcpyAsync(np, l.np.ptr, sizeof(int32_t) * (size_t)l.n, k, s), "copy");
  LJ_CUDA(ctx, cudaStreamSynchronize(s), "sync");
  return LJ_OK;
}

int lj_force_csr_fp64_aos(const double* q, double* p, int32_t n, double dt, double cl2,
                          const int32_t* list, const int32_t* np, const int32_t* ptr,
                          int32_t kind, const double* box, void* stream) {
  if (n < 0 || (n > 0 && (!q || !p || !np || !ptr))) return LJ_ERR_INVALID_ARGUMENT;
  if (kind != LJ_LIST_HALF && kind != LJ_LIST_FULL) return LJ_ERR_INVALID_ARGUMENT;
  if (!aligned16(q) || !aligned16(p)) return LJ_ERR_INVALID_ARGUMENT;
  if (!(cl2 >= 0.0) || !std::isfinite(dt)) return LJ_ERR_INVALID_ARGUMENT;
  if (n == 0) return LJ_OK;
  ForceLaunch L{};
  L.part.soa = 0;
  L.part.q = q;
  L.part.p = p;
  L.csr = Csr{n, 0, np, ptr, list, 0, 0};
  if (box) {
    L.box.on = 1;
    for (int d = 0; d < 3; d++) {
      if (!(box[d] > 0.0)) return LJ_ERR_INVALID_ARGUMENT;
      L.box.len[d] = box[d];
      L.box.half[d] = 0.5 * box[d];
    }
  }
  L.dt = dt;
  L.cl2 = cl2;
  L.precision = LJ_PREC_FP64;
  L.method = kind == LJ_LIST_FULL ? LJ_METHOD_GATHER_FULL : LJ_METHOD_SCATTER_HALF;
  L.lanes = 8;
  L.block = 128;
  L.kernel = 1;
  return launch_force(L, static_cast<cudaStream_t>(stream)) == cudaSuccess ? LJ_OK
                                                                          : LJ_ERR_CUDA;
}

int lj_force_pairs_fp64_aos(const double* q, double* p, int32_t n, double dt, double cl2,
                            const int32_t* ip, const int32_t* jp, int64_t npairs,
                            const double* box, void* stream) {
  if (n < 0 || npairs < 0 || (npairs > 0 && (!q || !p || !ip || !jp)))
    return LJ_ERR_INVALID_ARGUMENT;
  if (!aligned16(q) || !aligned16(p)) return LJ_ERR_INVALID_ARGUMENT;
  if (!(cl2 >= 0.0) || !std::isfinite(dt)) return LJ_ERR_INVALID_ARGUMENT;
  Particles part{};
  part.q = q;
  part.p = p;
  Periodic b{};
  if (box) {
    b.on = 1;
    for (int d = 0; d < 3; d++) {
      if (!(box[d] > 0.0)) return LJ_ERR_INVALID_ARGUMENT;
      b.len[d] = box[d];
      b.half[d] = 0.5 * box[d];
    }
  }
  return launch_force_pairs(part, n, ip, jp, npairs, b, dt, cl2,
                            static_cast<cudaStream_t>(stream)) == cudaSuccess
             ? LJ_OK
             : LJ_ERR_CUDA;
}

int lj_list_build(lj_ctx* ctx, const double* q, int32_t n, double rs, const double* box,
                  int32_t kinds) {
  if (!ctx) return LJ_ERR_INVALID_ARGUMENT;
  ctx->err.clear();
  if (n < 0 || (n > 0 && !q)) return fail(ctx, LJ_ERR_INVALID_ARGUMENT, "bad n or q");
  if (!aligned16(q)) return fail(ctx, LJ_ERR_INVALID_ARGUMENT, "q must be 16-byte aligned");
  if (!(rs > 0.0) || !std::isfinite(rs))
    return fail(ctx, LJ_ERR_INVALID_ARGUMENT, "search radius must be > 0");
  if (kinds < 1 || kinds > 3) return fail(ctx, LJ_ERR_INVALID_ARGUMENT, "kinds must be 1..3");
  if (cudaSetDevice(ctx->device) != cudaSuccess) return fail(ctx, LJ_ERR_CUDA, "set device");
  const bool want_half = kinds & LJ_BUILD_HALF, want_full = kinds & LJ_BUILD_FULL;
  cudaStream_t s = ctx->stream;
  CellGrid g{};
  ForceLaunch F{};
  F.part.soa = 0;
  F.part.q = q;
  F.csr.n = n;
  double open_lo[3] = {0, 0, 0}, open_hi[3] = {0, 0, 0};
  if (box) {
    g.periodic = 1;
    for (int d = 0; d < 3; d++) {
      if (!(box[d] > 0.0) || !std::isfinite(box[d]))
        return fail(ctx, LJ_ERR_INVALID_ARGUMENT, "box lengths must be > 0");
      if (rs > 0.5 * box[d])
        return fail(ctx, LJ_ERR_INVALID_ARGUMENT,
                    "search radius exceeds half the box: the minimum image is ambiguous");
      F.box.on = 1;
      F.box.len[d] = box[d];
      F.box.half[d] = 0.5 * box[d];
      g.nc[d] = std::max(1, (int)std::floor(box[d] / rs));
      g.nc[d] = std::min(g.nc[d], 1024);
      g.lo[d] = 0.0;
      g.inv_w[d] = g.nc[d] / box[d];
    }
  } else {
    double lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
    if (n > 0) {
      LJ_CUDA(ctx, ctx->b_minmax.ensure(6), "alloc");
      LJ_CUDA(ctx, launch_minmax(q, n, ctx->b_minmax.ptr, s), "minmax");
      unsigned long long k6[6];
      LJ_CUDA(ctx, cudaMemcpyAsync(k6, ctx->b_minmax.ptr, sizeof k6, cudaMemcpyDeviceToHost, s),
              "minmax read");
      LJ_CUDA(ctx, cudaStreamSynchronize(s), "sync");
      for (int d = 0; d < 3; d++) {
        hi[d] = key_to_double(k6[d]);
        lo[d] = key_to_double(~k6[3 + d]);
        if (!std::isfinite(lo[d]) || !std::isfinite(hi[d]))
          return fail(ctx, LJ_ERR_INVALID_ARGUMENT, "non-finite position");
        open_lo[d] = lo[d];
        open_hi[d] = hi[d];
      }
    }
    // at most ~2 n cells overall, every side >= rs
    const double cap = std::cbrt(2.0 * std::max(n, 1)) + 1.0;
    for (int d = 0; d < 3; d++) {
      const double ext = (hi[d] - lo[d]) * (1.0 + 1e-12) + 1e-300;
      g.nc[d] = std::max(1, std::min((int)std::floor(ext / rs), (int)cap));
      g.lo[d] = lo[d];
      g.inv_w[d] = g.nc[d] / ext;
    }
  }
  g.ncells = g.nc[0] * g.nc[1] * g.nc[2];
  make_fixed_frame(F);
  if (!box && n > 0) {
    // the open frame the force calls choose on the device, for these bounds
    int kf;
    long long org[3];
    host_open_frame(open_lo, open_hi, &kf, org);
    make_open_frame(F, kf, org);
  }
  LJ_CUDA(ctx, ctx->qfix.ensure((size_t)std::max(n, 1)), "alloc");
  F.qfix = ctx->qfix.ptr;
  LJ_CUDA(ctx, ctx->b_cell.ensure((size_t)n), "alloc");
  LJ_CUDA(ctx, ctx->b_order.ensure((size_t)n), "alloc");
  LJ_CUDA(ctx, ctx->b_cq.ensure((size_t)n), "alloc");
  LJ_CUDA(ctx, ctx->b_count.ensure((size_t)g.ncells), "alloc");
  LJ_CUDA(ctx, ctx->b_cursor.ensure((size_t)g.ncells), "alloc");
  LJ_CUDA(ctx, ctx->b_start.ensure((size_t)g.ncells + 1), "alloc");
  LJ_CUDA(ctx, ctx->tmp_scan.ensure(scan_tmp_bytes(std::max(g.ncells, n))), "alloc");
  if (n > 0) LJ_CUDA(ctx, launch_fixed_image(F, s), "fixed image");
  LJ_CUDA(ctx, launch_bin(q, n, g, ctx->b_cell.ptr, ctx->b_count.ptr, s), "bin");
  LJ_CUDA(ctx, launch_scan_counts(ctx->b_count.ptr, g.ncells, ctx->b_start.ptr, ctx->tmp_scan.ptr,
                                  ctx->tmp_scan.cap, s), "cell scan");
  LJ_CUDA(ctx, launch_place(ctx->b_cell.ptr, n, ctx->b_start.ptr, ctx->b_cursor.ptr, g.ncells,
                            ctx->qfix.ptr, ctx->b_order.ptr, ctx->b_cq.ptr, s), "place");
  // per-cell ordering (deterministic walks)
  LJ_CUDA(ctx, ctx->b_order2.ensure((size_t)n), "alloc");
  LJ_CUDA(ctx, ctx->b_cq2.ensure((size_t)n), "alloc");
  LJ_CUDA(ctx, launch_sort_cells(ctx->b_start.ptr, g.ncells, ctx->b_order.ptr, ctx->b_cq.ptr,
                                 ctx->b_order2.ptr, ctx->b_cq2.ptr, s), "cell sort");
  BuildArgs a{};
  a.q = q;
  a.n = n;
  a.grid = g;
  a.search = rs;
  for (int d = 0; d < 3; d++) {
    a.box[d] = box ? box[d] : 0.0;
    a.unit[d] = F.unit[d];
  }
  a.aniso = F.aniso;
  a.start = ctx->b_start.ptr;
  a.order = ctx->b_order2.ptr;
  a.cq = ctx->b_cq2.ptr;
  a.cell = ctx->b_cell.ptr;
  // padded row length from the mean density of the occupied volume, doubled
  // and rebuilt if any row does not fit
  double vol = 1.0;
  for (int d = 0; d < 3; d++) vol *= g.nc[d] / g.inv_w[d];
  const double per = 4.18879 * rs * rs * rs * (std::max(n, 1) / std::max(vol, 1e-300));
  int maxrow = std::max(32, ((int)std::ceil(per * 1.5) + 32 + 31) / 32 * 32);
  ctx->half.valid = false;
  ctx->full.valid = false;
  ctx->full.avalid = false;
  ctx->full.svalid = ctx->full.savalid = false;
  ctx->full.evalid = false;
  ctx->tiled.valid = false;
  int full_maxrow = 0;
  LJ_CUDA(ctx, ctx->err2.ensure(2), "alloc");
  LJ_CUDA(ctx, ctx->b_cnt_half.ensure((size_t)n), "alloc");
  LJ_CUDA(ctx, ctx->b_off_half.ensure((size_t)n + 1), "alloc");
  for (int kind = 0; kind < 2; kind++) {
    if (!(kind == 0 ? want_half : want_full)) continue;
    for (;;) {
      if (maxrow > 1 << 20)
        return fail(ctx, LJ_ERR_LIST_OVERFLOW, "a neighbour row exceeds 2^20 entries");
      LJ_CUDA(ctx, ctx->tmp_i32a.ensure((size_t)n * maxrow), "alloc");
      LJ_CUDA(ctx, cudaMemsetAsync(ctx->err2.ptr, 0, sizeof(int32_t), s), "memset");
      LJ_CUDA(ctx, launch_build_rows(a, kind == 0, maxrow, ctx->tmp_i32a.ptr,
                                     ctx->b_cnt_half.ptr, ctx->err2.ptr, s), "row build");
      int32_t ovf = 0;
      LJ_CUDA(ctx, cudaMemcpyAsync(&ovf, ctx->err2.ptr, sizeof ovf, cudaMemcpyDeviceToHost, s),
              "read");
      LJ_CUDA(ctx, cudaStreamSynchronize(s), "sync");
      if (!ovf) break;
      maxrow *= 2;
    }
    if (kind == 1) full_maxrow = maxrow;
    int64_t total = 0;
    LJ_CUDA(ctx, launch_scan_counts(ctx->b_cnt_half.ptr, n, ctx->b_off_half.ptr, ctx->tmp_scan.ptr,
                                    ctx->tmp_scan.cap, s), "row scan");
    LJ_CUDA(ctx, cudaMemcpyAsync(&total, ctx->b_off_half.ptr + n, sizeof total,
                                 cudaMemcpyDeviceToHost, s), "total");
    LJ_CUDA(ctx, cudaStreamSynchronize(s), "sync");
    if (total > 0x7fffffffll)
      return fail(ctx, LJ_ERR_LIST_OVERFLOW, "list would exceed 2^31-1 entries");
    DevList& l = kind == 0 ? ctx->half : ctx->full;
    LJ_CUDA(ctx, ctx->tmp_i32b.ensure((size_t)std::max<int64_t>(total, 1)), "alloc");
    LJ_CUDA(ctx, launch_compact_padded(ctx->b_cnt_half.ptr, ctx->tmp_i32a.ptr, maxrow,
                                       ctx->b_off_half.ptr, n, ctx->tmp_i32b.ptr, s), "compact");
    LJ_CUDA(ctx, l.np.ensure((size_t)n), "alloc");
    LJ_CUDA(ctx, l.ptr.ensure((size_t)n), "alloc");
    LJ_CUDA(ctx, l.list.ensure((size_t)std::max<int64_t>(total, 1)), "alloc");
    // rows ascending in j, as makepair + sortpair produce them
    LJ_CUDA(ctx, launch_sort_rows_into(ctx->b_off_half.ptr, n, ctx->tmp_i32b.ptr, l.list.ptr, s),
            "row sort");
    LJ_CUDA(ctx, launch_offsets_to_ptr(ctx->b_off_half.ptr, n, l.ptr.ptr, l.np.ptr,
                                       ctx->err2.ptr + 1, s), "ptr");
    int32_t mr = 0;
    LJ_CUDA(ctx, cudaMemcpyAsync(&mr, ctx->err2.ptr + 1, sizeof mr, cudaMemcpyDeviceToHost, s),
            "read");
    LJ_CUDA(ctx, cudaStreamSynchronize(s), "sync");
    l.n = n;
    l.entries = total;
    l.max_row = mr;
    l.valid = true;
  }
  if (want_full && !F.aniso && n > 0) {
    // cell-tiled form of the full list: 16-bit indices into the 27-cell tile
    std::vector<int32_t> counts((size_t)g.ncells);
    LJ_CUDA(ctx, cudaMemcpyAsync(counts.data(), ctx->b_count.ptr, sizeof(int32_t) * g.ncells,
                                 cudaMemcpyDeviceToHost, s), "counts");
    LJ_CUDA(ctx, cudaStreamSynchronize(s), "sync");
    int maxocc = 1;
    for (int v : counts) maxocc = std::max(maxocc, v);
    int shift = 5;
    while ((1 << shift) < maxocc) shift++;
    if (27 * (1 << shift) <= 65536 && 27 * (16 << shift) <= 200 * 1024) {
      {
        auto& T = ctx->tiled;
        T.grid = g;
        T.maxrow = full_maxrow;
        T.maxc_shift = shift;
        LJ_CUDA(ctx, T.rows.ensure((size_t)n * full_maxrow), "alloc");
        LJ_CUDA(ctx, T.cnt.ensure((size_t)n), "alloc");
        LJ_CUDA(ctx, T.order.ensure((size_t)n), "alloc");
        LJ_CUDA(ctx, T.start.ensure((size_t)g.ncells + 1), "alloc");
        LJ_CUDA(ctx, T.cq.ensure((size_t)n), "alloc");
        LJ_CUDA(ctx, cudaMemcpyAsync(T.order.ptr, ctx->b_order2.ptr, sizeof(int32_t) * n,
                                     cudaMemcpyDeviceToDevice, s), "copy");
        LJ_CUDA(ctx, cudaMemcpyAsync(T.start.ptr, ctx->b_start.ptr,
                                     sizeof(int64_t) * ((size_t)g.ncells + 1),
                                     cudaMemcpyDeviceToDevice, s), "copy");
        LJ_CUDA(ctx, cudaMemsetAsync(ctx->err2.ptr, 0, sizeof(int32_t), s), "memset");
        LJ_CUDA(ctx, launch_build_rows_local(a, full_maxrow, shift, T.rows.ptr, T.cnt.ptr,
                                             ctx->err2.ptr, s), "tiled rows");
        int32_t ovf = 0;
        LJ_CUDA(ctx, cudaMemcpyAsync(&ovf, ctx->err2.ptr, sizeof ovf, cudaMemcpyDeviceToHost, s),
                "read");
        LJ_CUDA(ctx, cudaStreamSynchronize(s), "sync");
        T.valid = ovf == 0;
      }
    }
  }
  ctx->list_from_host = false;
  ctx->h_np.clear();
  ctx->h_ptr.clear();
  ctx->h_list.clear();
  return want_full ? build_aligned(ctx) : LJ_OK;
}

int lj_autotune_aos(lj_ctx* ctx, const double* q, int32_t n, const lj_force_opts* opts,
                    int32_t reps, lj_force_opts* best, double* ms_best) {
  if (!ctx) return LJ_ERR_INVALID_ARGUMENT;
  ctx->err.clear();
  if (!best || reps < 1) return fail(ctx, LJ_ERR_INVALID_ARGUMENT, "best is NULL or reps < 1");
  lj_tune_result r{};
  const int rc = autotune(ctx, q, n, opts, reps, 1 << LJ_LAYOUT_AOS, nullptr, &r);
  if (rc) return rc;
  *best = r.best;
  if (ms_best) *ms_best = r.ms;
  return LJ_OK;
}

int lj_autotune(lj_ctx* ctx, const double* q, int32_t n, const lj_force_opts* opts,
                int32_t reps, int32_t layouts, const char* cache_path, lj_tune_result* out) {
  if (!ctx) return LJ_ERR_INVALID_ARGUMENT;
  ctx->err.clear();
  if (!out || reps < 1) return fail(ctx, LJ_ERR_INVALID_ARGUMENT, "out is NULL or reps < 1");
  if (layouts < 0 || layouts > 7)
    return fail(ctx, LJ_ERR_INVALID_ARGUMENT, "layouts must be a mask of 1 << LJ_LAYOUT_*");
  return autotune(ctx, q, n, opts, reps, layouts ? layouts : 1 << LJ_LAYOUT_AOS, cache_path, out);
}

int lj_measure_aos(lj_ctx* ctx, const double* q_host, double* p_host, int32_t n,
                   const lj_force_opts* o, int32_t calls, double* ms_total, double* ms_calc) {
  if (!ctx) return LJ_ERR_INVALID_ARGUMENT;
  ctx->err.clear();
  if (n < 0 || calls < 0) return fail(ctx, LJ_ERR_INVALID_ARGUMENT, "n and calls must be >= 0");
  if (n > 0 && (!q_host || !p_host)) return fail(ctx, LJ_ERR_INVALID_ARGUMENT, "null q or p");
  int rc = check_opts(ctx, o);
  if (rc) return rc;
  if (!ctx->half.valid && !ctx->full.valid) return fail(ctx, LJ_ERR_NO_LIST, "no list installed");
  const int32_t rows = ctx->full.valid ? ctx->full.n : ctx->half.n;
  if (n != rows)
    return fail(ctx, LJ_ERR_INVALID_ARGUMENT, "n = %d but the installed list has %d rows", n,
                rows);
  if (cudaSetDevice(ctx->device) != cudaSuccess) return fail(ctx, LJ_ERR_CUDA, "set device");
  const size_t bytes = sizeof(double) * 4 * (size_t)n;
  LJ_CUDA(ctx, ctx->mq.ensure(4 * (size_t)n), "alloc");
  LJ_CUDA(ctx, ctx->mp.ensure(4 * (size_t)n), "alloc");
  cudaStream_t s = ctx->stream;
  LJ_CUDA(ctx, cudaEventRecord(ctx->ev[0], s), "event");
  // copy_to_gpu (cuda/force_cuda.cu:302-312): q, p and the list arrays
  LJ_CUDA(ctx, cudaMemcpyAsync(ctx->mq.ptr, q_host, bytes, cudaMemcpyHostToDevice, s), "H2D q");
  LJ_CUDA(ctx, cudaMemcpyAsync(ctx->mp.ptr, p_host, bytes, cudaMemcpyHostToDevice, s), "H2D p");
  if (ctx->list_from_host) {
    DevList& l = ctx->host_kind == LJ_LIST_HALF ? ctx->half : ctx->full;
    if ((rc = copy_in(ctx, l.np.ptr, ctx->h_np.data(), ctx->h_np.size(), LJ_WHERE_HOST)))
      return rc;
    if ((rc = copy_in(ctx, l.ptr.ptr, ctx->h_ptr.data(), ctx->h_ptr.size(), LJ_WHERE_HOST)))
      return rc;
    if ((rc = copy_in(ctx, l.list.ptr, ctx->h_list.data(), ctx->h_list.size(), LJ_WHERE_HOST)))
      return rc;
    if (ctx->host_kind == LJ_LIST_FULL && l.avalid)  // the gather reads the aligned copy
      LJ_CUDA(ctx, launch_copy_rows4(l.np.ptr, l.ptr.ptr, l.list.ptr, l.aoff.ptr, l.n,
                                     l.alist.ptr, l.aptr.ptr, s), "aligned copy");
    if (ctx->host_kind == LJ_LIST_FULL && l.evalid && (rc = ensure_ell(ctx, true)))
      return rc;  // and kernel 5 its transposed copy
  }
  LJ_CUDA(ctx, cudaEventRecord(ctx->ev[1], s), "event");
  Particles part{};
  part.q = ctx->mq.ptr;
  part.p = ctx->mp.ptr;
  for (int c = 0; c < calls; c++)
    if ((rc = run_force(ctx, part, n, o))) return rc;
  LJ_CUDA(ctx, cudaEventRecord(ctx->ev[2], s), "event");
  LJ_CUDA(ctx, cudaMemcpyAsync(p_host, ctx->mp.ptr, bytes, cudaMemcpyDeviceToHost, s), "D2H p");
  LJ_CUDA(ctx, cudaStreamSynchronize(s), "sync");
  float t_all = 0.f, t_calc = 0.f;
  cudaEvent_t end;
  LJ_CUDA(ctx, cudaEventCreate(&end), "event");
  cudaEventRecord(end, s);
  cudaEventSynchronize(end);
  cudaEventElapsedTime(&t_all, ctx->ev[0], end);
  cudaEventElapsedTime(&t_calc, ctx->ev[1], ctx->ev[2]);
  cudaEventDestroy(end);
  if (ms_total) *ms_total = t_all;
  if (ms_calc) *ms_calc = t_calc;
  return LJ_OK;
}

}  // extern "C"
