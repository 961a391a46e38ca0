// lj_md.cu -- velocity-Verlet molecular dynamics around the force path.
//
// The reference never integrates (its 100 "steps" re-kick p from a fixed q,
// cpu_ref/force_aos.cpp:592-601); this loop extends the path with the
// integrator and on-device list rebuilds an MD code needs around it.
//
// One step (m = 1, force routine = kick p += F dt):
//   drift   q += p dt, wrap into [0, L), fixed-point image of q, and the
//           displacement against the image at the last list build; any
//           particle beyond skin/2 raises the rebuild flag        (k_md_drift)
//   rebuild fixed-shape, flag-guarded kernels: cell binning, counting sort,
//           per-cell ordering, warp-cooperative row build into padded rows
//           (+ compaction for the FP64 scatter); they do nothing on steps
//           that need no rebuild
//   kick    the mixed gather (or FP64 compacted scatter) with dt
// Half kicks of consecutive steps are merged into one full kick; they are
// split only where synchronous momenta are needed (energy records and the
// end), so a run of S steps costs S + 1 + records force calls.  The steps
// between two records run as one launch of a persistent graph (LoopGraph: a
// WHILE node over `graph_steps` captured steps, counted down on the device),
// or, where a conditional node cannot be built, as back-to-back launches of
// a graph of `graph_steps` steps.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "lj_ctx.h"
#include "lj_nlist.h"

namespace ljg {
namespace {

enum {
  F_REBUILD = 0,  // a rebuild is due this step
  F_FILL = 1,     // the rebuild fits the capacity (fill, sort, offsets run)
  F_OVERFLOW = 2, // a rebuild did not fit
  F_COUNT = 3,    // rebuilds done
  F_MAXROW = 4,   // longest row of the last build
  F_STEP = 5,     // steps taken (drives rebuild_every)
  F_CLOSE = 6,    // three words for k_seg_close_terms (6..8)
  F_LOOP = 9,     // chunks left in the persistent loop
  F_WORDS = 10
};

__global__ void __launch_bounds__(256) k_md_drift(double* __restrict__ q,
                                                  const double* __restrict__ p, int n, double dt,
                                                  double lx, double ly, double lz, FixedAxis ax,
                                                  FixedAxis ay, FixedAxis az,
                                                  int4* __restrict__ qfix,
                                                  const int4* __restrict__ qref, float ux,
                                                  float uy, float uz, float half_skin2,
                                                  int rebuild_every,
                                                  int32_t* __restrict__ flags) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i == 0) {
    // step counter; flags[F_STEP] is read by no other thread of this kernel
    const int stepno = flags[F_STEP] + 1;
    flags[F_STEP] = stepno;
    if (rebuild_every > 0 && stepno % rebuild_every == 0) flags[F_REBUILD] = 1;
  }
  if (i >= n) return;
  double* qi = q + 4 * (size_t)i;
  const double* pi = p + 4 * (size_t)i;
  const double2 pxy = *reinterpret_cast<const double2*>(pi);
  const double pz = pi[2];
  double2 xy = *reinterpret_cast<double2*>(qi);
  double z = qi[2];
  xy.x = wrap_into_box(fma(pxy.x, dt, xy.x), lx);
  xy.y = wrap_into_box(fma(pxy.y, dt, xy.y), ly);
  z = wrap_into_box(fma(pz, dt, z), lz);
  *reinterpret_cast<double2*>(qi) = xy;
  qi[2] = z;
  const int4 x = pack_image(to_fixed_fine(xy.x, ax), to_fixed_fine(xy.y, ay),
                            to_fixed_fine(z, az));
  qfix[i] = x;
  const int4 r = qref[i];
  const float dx = (float)wrap_sub(x.x, r.x) * ux, dy = (float)wrap_sub(x.y, r.y) * uy,
              dz = (float)wrap_sub(x.z, r.z) * uz;
  if (fmaf(dz, dz, fmaf(dy, dy, dx * dx)) > half_skin2) flags[F_REBUILD] = 1;
}

// Raises the rebuild flag when a particle of the image qfix lies more than
// skin/2 from its position at the last build (the drift's check, for the
// positions a run starts from).
__global__ void k_md_moved(const int4* __restrict__ qfix, const int4* __restrict__ qref, int n,
                           float ux, float uy, float uz, float half_skin2,
                           int32_t* __restrict__ flags) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int4 x = qfix[i], r = qref[i];
    const float dx = (float)wrap_sub(x.x, r.x) * ux, dy = (float)wrap_sub(x.y, r.y) * uy,
                dz = (float)wrap_sub(x.z, r.z) * uz;
    if (fmaf(dz, dz, fmaf(dy, dy, dx * dx)) > half_skin2) flags[F_REBUILD] = 1;
  }
}

__global__ void k_md_copy_ref(const int4* __restrict__ qfix, int4* __restrict__ qref, int n,
                              const int32_t* __restrict__ flags) {
  if (!flags[F_REBUILD]) return;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    qref[i] = qfix[i];
}

__global__ void k_md_finish(int32_t* flags) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  if (flags[F_REBUILD]) flags[F_COUNT] += 1;
  flags[F_REBUILD] = 0;
}

__global__ void k_md_set(int32_t* flags, int word, int value) {
  if (threadIdx.x == 0 && blockIdx.x == 0) flags[word] = value;
}

// Potential energy sum over pairs j > i of 4 (r^-12 - r^-6) for r2 <= cl2.
// Mixed: FP32 pair math from the fixed-point image, Kahan per thread, FP64
// across threads.  FP64: the FP64 kernels' arithmetic.
template <bool FP64>
__global__ void __launch_bounds__(256) k_md_potential(const double* __restrict__ q,
                                                      const int4* __restrict__ qfix, Csr c,
                                                      double lx, double ly, double lz,
                                                      float k_hi, float k_lo, float cl2u_lo,
                                                      float cl2u_hi, double cl2,
                                                      double* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double u = 0.0;
  if (i < c.n) {
    const int cnt = c.np[i];
    const int64_t k0 = row_start(c, i);
    const double* qi = q + 4 * (size_t)i;
    const double len[3] = {lx, ly, lz};
    long long hb[3];
    for (int d = 0; d < 3; d++) hb[d] = __double_as_longlong(0.5 * len[d]);
    float s = 0.f, comp = 0.f;
    const int4 xi = qfix[i];
    for (int m = 0; m < cnt; m++) {
      const int j = c.list[k0 + m];
      if (j <= i) continue;
      const double* qj = q + 4 * (size_t)j;
      if (FP64) {
        double d[3];
        for (int x = 0; x < 3; x++) d[x] = min_image_fp64(qj[x] - qi[x], len[x], hb[x]);
        const double r2 = fma(d[2], d[2], fma(d[0], d[0], d[1] * d[1]));
        if (r2 > cl2) continue;
        const double ir6 = 1.0 / (r2 * r2 * r2);
        u += 4.0 * ir6 * (ir6 - 1.0);
      } else {
        const int4 xj = qfix[j];
        const float dx = (float)wrap_sub(xj.x, xi.x), dy = (float)wrap_sub(xj.y, xi.y),
                    dz = (float)wrap_sub(xj.z, xi.z);
        const float r2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
        bool in = r2 <= cl2u_lo;
        if (!in && r2 <= cl2u_hi) {
          double d[3];
          for (int x = 0; x < 3; x++) d[x] = min_image_fp64(qj[x] - qi[x], len[x], hb[x]);
          in = !(fma(d[2], d[2], fma(d[0], d[0], d[1] * d[1])) > cl2);
        }
        if (!in) continue;
        float inv = 1.0f / r2;
        inv = fmaf(inv, k_hi, inv * k_lo);
        const float ir6 = inv * inv * inv;
        const float e = 4.0f * ir6 * (ir6 - 1.0f);
        const float y = e - comp;
        const float t = s + y;
        comp = (t - s) - y;
        s = t;
      }
    }
    if (!FP64) u = (double)s - (double)comp;
  }
  for (int o = 16; o > 0; o >>= 1) u += __shfl_xor_sync(0xffffffffu, u, o);
  if ((threadIdx.x & 31) == 0 && u != 0.0) atomicAdd(out, u);
}

__global__ void __launch_bounds__(256) k_md_kinetic(const double* __restrict__ p, int n,
                                                    double* __restrict__ out) {
  double k = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double* b = p + 4 * (size_t)i;
    k += 0.5 * (b[0] * b[0] + b[1] * b[1] + b[2] * b[2]);
  }
  for (int o = 16; o > 0; o >>= 1) k += __shfl_xor_sync(0xffffffffu, k, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(out, k);
}

int grid1(int64_t n, int b) { return (int)std::max<int64_t>(1, (n + b - 1) / b); }

}  // namespace

struct MdState {
  int n = 0;
  int64_t cap = 0;
  CellGrid grid{};
  ForceLaunch kick_full{}, kick_half{};
  BuildArgs build{};
  int maxrow = 0;          // capacity of the rows in use (full, half or near part)
  int maxrow_full = 0, maxrow_near = 0, maxrow_far = 0;
  DevBuf<int4> qfix, qref, cq, cq2;
  DevBuf<int32_t> flags, cell, count, cursor, order, order2, cnt, ptr, rows, list;
  // split two-float kicks: rows / cnt hold every row's near part, rows2 /
  // cnt2 the far part (launch_build_rows_split)
  DevBuf<int32_t> rows2, cnt2;
  DevBuf<int32_t> closeq;  // rows with far entries inside 2.0 sigma (k_gather_mixed_seg)
  // The list of the last completed run, kept for the next: it holds while
  // every particle stays within skin/2 of its position at that build (qref,
  // checked when the next run starts) and the particle count, box, cutoff,
  // skin and list kind (list_key) and the list's buffers are unchanged.
  bool list_kept = false;
  double list_key[7] = {};
  const void* list_bufs[6] = {};
  // the bytes of every argument the step graph was captured with (launch
  // structs, buffer pointers, sizes): equal bytes relaunch it as it is
  std::vector<unsigned char> graph_sig;
  int64_t graph_step_kernels = -1;
  int64_t cap2 = 0;
  bool split = false;
  DevBuf<int64_t> start, off;
  DevBuf<unsigned char> scan_tmp;
  DevBuf<double> energy;
  cudaStream_t own_stream = nullptr;
  cudaGraphExec_t graph = nullptr;
  int graph_steps = 0;
  LoopGraph loop;
  ~MdState() {
    if (graph) cudaGraphExecDestroy(graph);
    if (own_stream) cudaStreamDestroy(own_stream);
  }
};

void md_state_delete(MdState* m) { delete m; }

}  // namespace ljg

using namespace ljg;

namespace {

#define MD_CUDA(ctx, call, what)                                                        \
  do {                                                                                  \
    cudaError_t e_ = (call);                                                            \
    if (e_ != cudaSuccess)                                                              \
      return lj_fail(ctx, e_ == cudaErrorMemoryAllocation ? LJ_ERR_OUT_OF_MEMORY : LJ_ERR_CUDA, \
                     "%s: %s", what, cudaGetErrorString(e_));                           \
  } while (0)

// The fixed-shape rebuild sequence (guarded by flags[F_REBUILD]): bin, cell
// offsets, placement, per-cell ordering, warp-cooperative row build into the
// padded rows.  The mixed gather reads the padded rows directly; the FP64
// scatter sweeps rows flat, so its rows are compacted (scan + copy).
cudaError_t md_rebuild(MdState& m, bool compact, const ForceLaunch& kick, cudaStream_t s) {
  const int32_t* g = m.flags.ptr + F_REBUILD;
  cudaError_t e;
  if ((e = launch_bin(m.build.q, m.n, m.grid, m.cell.ptr, m.count.ptr, s, g))) return e;
  if ((e = launch_scan_counts(m.count.ptr, m.grid.ncells, m.start.ptr, m.scan_tmp.ptr,
                              m.scan_tmp.cap, s, g)))
    return e;
  if ((e = launch_place(m.cell.ptr, m.n, m.start.ptr, m.cursor.ptr, m.grid.ncells, m.qfix.ptr,
                        m.order.ptr, m.cq.ptr, s, g)))
    return e;
  if ((e = launch_sort_cells(m.start.ptr, m.grid.ncells, m.order.ptr, m.cq.ptr, m.order2.ptr,
                             m.cq2.ptr, s, g)))
    return e;
  if (m.split)
    e = launch_build_rows_split(m.build, m.maxrow, m.rows.ptr, m.cnt.ptr, m.maxrow_far,
                                m.rows2.ptr, m.cnt2.ptr, m.flags.ptr + F_OVERFLOW, s, g);
  else
    e = launch_build_rows(m.build, m.build.want_half != 0, m.maxrow, m.rows.ptr, m.cnt.ptr,
                          m.flags.ptr + F_OVERFLOW, s, g);
  if (e) return e;
  if (compact) {
    if ((e = launch_scan_counts(m.cnt.ptr, m.n, m.off.ptr, m.scan_tmp.ptr, m.scan_tmp.cap, s, g)))
      return e;
    if ((e = launch_compact_padded(m.cnt.ptr, m.rows.ptr, m.maxrow, m.off.ptr, m.n, m.list.ptr,
                                   s, g)))
      return e;
    if ((e = launch_offsets_to_ptr(m.off.ptr, m.n, m.ptr.ptr, m.cnt.ptr, m.flags.ptr + F_MAXROW,
                                   s, g)))
      return e;
  }
  k_md_copy_ref<<<std::min(grid1(m.n, 256), 152 * 8), 256, 0, s>>>(m.qfix.ptr, m.qref.ptr, m.n, m.flags.ptr);
  k_md_finish<<<1, 32, 0, s>>>(m.flags.ptr);
  return cudaGetLastError();
}

struct DriftArgs {
  double* q;
  const double* p;
  double dt;
  double len[3];
  float unit[3];
  float half_skin2;
  int rebuild_every;
};

// Host buffers of lj_md_run_host.  q goes to the device on the run's stream
// before the initial build; p on a side stream, waited for before its first
// use, so that its copy runs beside the build.  At the end q, final once the
// last drift has run, goes back on the side stream beside the final half
// kick, and p on the run's stream.
struct HostIo {
  double* q;
  double* p;
  size_t bytes;
  cudaStream_t side;
  cudaEvent_t ev_in, ev_p, ev_q, ev_side_done;
  bool q_queued = false;  // the copy of q back to the host is queued
};

cudaError_t md_step(MdState& m, const DriftArgs& d, const ForceLaunch& kick, cudaStream_t s,
                    HostIo* io = nullptr) {
  k_md_drift<<<grid1(m.n, 256), 256, 0, s>>>(
      d.q, d.p, m.n, d.dt, d.len[0], d.len[1], d.len[2], kick.axis[0], kick.axis[1],
      kick.axis[2], m.qfix.ptr, m.qref.ptr, d.unit[0], d.unit[1], d.unit[2], d.half_skin2,
      d.rebuild_every, m.flags.ptr);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  if ((e = md_rebuild(m, kick.method == LJ_METHOD_SCATTER_HALF, kick, s))) return e;
  if (io) {  // the last step: q is final, its copy back runs beside the kick
    if ((e = cudaEventRecord(io->ev_q, s)) || (e = cudaStreamWaitEvent(io->side, io->ev_q, 0)) ||
        (e = cudaMemcpyAsync(io->q, d.q, io->bytes, cudaMemcpyDeviceToHost, io->side)))
      return e;
    io->q_queued = true;
  }
  return launch_force(kick, s);
}

// Kernel nodes of a captured graph: the kernels one replay launches.
int64_t graph_kernels(cudaGraph_t g) {
  size_t n = 0;
  if (cudaGraphGetNodes(g, nullptr, &n) != cudaSuccess || n == 0) return 0;
  std::vector<cudaGraphNode_t> nodes(n);
  if (cudaGraphGetNodes(g, nodes.data(), &n) != cudaSuccess) return 0;
  int64_t k = 0;
  for (size_t a = 0; a < n; a++) {
    cudaGraphNodeType t;
    if (cudaGraphNodeGetType(nodes[a], &t) == cudaSuccess && t == cudaGraphNodeTypeKernel) k++;
  }
  return k;
}

}  // namespace

// lj_md_run over device q, p; with io, over the host buffers it names (the
// device q, p are then the context's staging arrays).
static int md_run(lj_ctx* ctx, double* q, double* p, int32_t n, const lj_md_params* prm,
                  int32_t nsteps, lj_md_record* records, int32_t max_records,
                  int32_t* n_records, lj_md_stats* stats, HostIo* io) {
  if (!ctx) return LJ_ERR_INVALID_ARGUMENT;
  ctx->err.clear();
  if (n_records) *n_records = 0;
  if (!prm || n < 1 || nsteps < 0 || !q || !p)
    return lj_fail(ctx, LJ_ERR_INVALID_ARGUMENT, "bad MD arguments");
  if ((reinterpret_cast<uintptr_t>(q) | reinterpret_cast<uintptr_t>(p)) & 15u)
    return lj_fail(ctx, LJ_ERR_INVALID_ARGUMENT, "q and p must be 16-byte aligned");
  if (!(prm->dt > 0.0) || !(prm->rc > 0.0) || !(prm->skin >= 0.0))
    return lj_fail(ctx, LJ_ERR_INVALID_ARGUMENT, "dt, rc must be > 0 and skin >= 0");
  if (prm->precision != LJ_PREC_MIXED && prm->precision != LJ_PREC_MIXED_FP32 &&
      prm->precision != LJ_PREC_FP64)
    return lj_fail(ctx, LJ_ERR_INVALID_ARGUMENT, "unknown precision");
  if (!(prm->kick_lanes == 0 || prm->kick_lanes == 1 || prm->kick_lanes == 2 ||
        prm->kick_lanes == 4 || prm->kick_lanes == 8))
    return lj_fail(ctx, LJ_ERR_INVALID_ARGUMENT, "kick_lanes must be 0, 1, 2, 4 or 8");
  const double rs = prm->rc + prm->skin;
  for (int d = 0; d < 3; d++)
    if (!(prm->box[d] > 2.0 * rs))
      return lj_fail(ctx, LJ_ERR_INVALID_ARGUMENT,
                     "box must exceed twice the list radius (minimum image)");
  if (cudaSetDevice(ctx->device) != cudaSuccess)
    return lj_fail(ctx, LJ_ERR_CUDA, "set device");
  if (!ctx->md) ctx->md.reset(new MdState());
  MdState& m = *ctx->md;
  // the previous run's list, if this run has its particle count, box,
  // cutoff, skin and list kind (its buffers are compared after sizing)
  const double key[7] = {(double)n, prm->box[0], prm->box[1], prm->box[2], prm->rc,
                         prm->skin, (double)(prm->precision * 2 + (prm->ff_all ? 1 : 0))};
  bool reuse = m.list_kept && std::memcmp(key, m.list_key, sizeof key) == 0;
  m.list_kept = false;  // until this run completes
  cudaStream_t s = ctx->stream;
  if (!s) {
    // graphs cannot be captured on the legacy stream: run on our own stream,
    // ordered after everything the caller queued on the legacy stream
    if (!m.own_stream) MD_CUDA(ctx, cudaStreamCreateWithFlags(&m.own_stream, cudaStreamNonBlocking),
                               "stream");
    MD_CUDA(ctx, cudaStreamSynchronize(nullptr), "sync");
    s = m.own_stream;
  }
  const bool mixed = prm->precision != LJ_PREC_FP64;

  // ---- buffers and constants -------------------------------------------
  m.n = n;
  const double vol = prm->box[0] * prm->box[1] * prm->box[2];
  const double per = 4.18879 * rs * rs * rs * (n / vol);  // full-list partners / particle
  // two-float kicks split every row into a near and a far part at the build
  m.split = prm->precision == LJ_PREC_MIXED && !prm->ff_all;
  // padded row lengths: the mean row plus room for density fluctuations
  auto padded = [](double mean) { return ((int)std::ceil(mean * 1.5) + 32 + 31) / 32 * 32; };
  if (m.split) {
    const double rn = std::min(kFarSplit, rs);
    const double per_near = 4.18879 * rn * rn * rn * (n / vol);
    m.maxrow_near = std::max(m.maxrow_near, padded(per_near));
    m.maxrow_far = std::max(m.maxrow_far, padded(per - per_near));
    m.maxrow = m.maxrow_near;
    m.cap2 = (int64_t)n * m.maxrow_far;
  } else {
    m.maxrow_full = std::max(m.maxrow_full, padded(per));
    m.maxrow = m.maxrow_full;
  }
  m.cap = (int64_t)n * m.maxrow;
  if (!mixed && per * 0.5 * n * 1.3 > 0x7fffffff)
    return lj_fail(ctx, LJ_ERR_UNSUPPORTED, "compacted half list would exceed 2^31 entries");
  for (int d = 0; d < 3; d++) {
    m.grid.nc[d] = std::max(1, std::min(1024, (int)std::floor(prm->box[d] / rs)));
    m.grid.lo[d] = 0.0;
    m.grid.inv_w[d] = m.grid.nc[d] / prm->box[d];
  }
  m.grid.ncells = m.grid.nc[0] * m.grid.nc[1] * m.grid.nc[2];
  m.grid.periodic = 1;
  MD_CUDA(ctx, m.qfix.ensure(n), "alloc");
  MD_CUDA(ctx, m.qref.ensure(n), "alloc");
  MD_CUDA(ctx, m.cq.ensure(n), "alloc");
  MD_CUDA(ctx, m.cq2.ensure(n), "alloc");
  MD_CUDA(ctx, m.flags.ensure(F_WORDS), "alloc");
  MD_CUDA(ctx, m.cell.ensure(n), "alloc");
  MD_CUDA(ctx, m.order.ensure(n), "alloc");
  MD_CUDA(ctx, m.order2.ensure(n), "alloc");
  MD_CUDA(ctx, m.cnt.ensure(n), "alloc");
  MD_CUDA(ctx, m.ptr.ensure(n), "alloc");
  MD_CUDA(ctx, m.count.ensure(m.grid.ncells), "alloc");
  MD_CUDA(ctx, m.cursor.ensure(m.grid.ncells), "alloc");
  MD_CUDA(ctx, m.start.ensure((size_t)m.grid.ncells + 1), "alloc");
  MD_CUDA(ctx, m.off.ensure((size_t)n + 1), "alloc");
  MD_CUDA(ctx, m.scan_tmp.ensure(scan_tmp_bytes(std::max(n, m.grid.ncells))), "alloc");
  MD_CUDA(ctx, m.rows.ensure((size_t)m.cap), "alloc");
  if (m.split) {
    MD_CUDA(ctx, m.rows2.ensure((size_t)m.cap2), "alloc");
    MD_CUDA(ctx, m.cnt2.ensure(n), "alloc");
    MD_CUDA(ctx, m.closeq.ensure(n), "alloc");
  }
  // the compacted half list holds about half of the padded capacity
  const int64_t half_cap = std::min<int64_t>(m.cap, 0x7fffffffll);
  if (!mixed) MD_CUDA(ctx, m.list.ensure((size_t)half_cap), "alloc");
  MD_CUDA(ctx, m.energy.ensure(2), "alloc");
  // a kept list needs the buffers it was built into
  const void* bufs[6] = {m.rows.ptr, m.cnt.ptr, m.rows2.ptr, m.cnt2.ptr, m.order2.ptr,
                         m.list.ptr};
  reuse = reuse && std::memcmp(bufs, m.list_bufs, sizeof bufs) == 0;
  MD_CUDA(ctx, cudaMemsetAsync(m.flags.ptr, 0, sizeof(int32_t) * F_WORDS, s), "memset");

  ForceLaunch K{};
  K.part.soa = 0;
  K.part.q = q;
  K.part.p = p;
  // mixed: padded rows read in place (64-bit row starts i * maxrow); FP64:
  // compacted rows with int32 offsets
  K.csr = mixed ? Csr{n, m.cap, m.cnt.ptr, nullptr, m.rows.ptr, (int64_t)m.maxrow, 1}
                : Csr{n, m.cap, m.cnt.ptr, m.ptr.ptr, m.list.ptr, 0, 0};
  K.split = m.split ? 1 : 0;
  if (m.split) {
    K.far = Csr{n, m.cap2, m.cnt2.ptr, nullptr, m.rows2.ptr, (int64_t)m.maxrow_far, 1};
    // rows visited in the cell order of the last build (k_sort_cells' slot
    // order): a warp's rows stay neighbours in space however far the
    // particles have moved from their initial order
    K.rowperm = m.order2.ptr;
  }
  K.close_flag = m.flags.ptr + F_CLOSE;
  K.close_rows = m.split ? m.closeq.ptr : nullptr;
  K.box.on = 1;
  for (int d = 0; d < 3; d++) {
    K.box.len[d] = prm->box[d];
    K.box.half[d] = 0.5 * prm->box[d];
  }
  K.cl2 = prm->rc * prm->rc;
  K.precision = prm->precision;
  K.method = mixed ? LJ_METHOD_GATHER_FULL : LJ_METHOD_SCATTER_HALF;
  K.kernel = 2;
  K.unroll = 4;
  // two-float kicks take one lane per row by default (issue-bound: fewest
  // slots lost at row ends), FP32 kicks four (bound by the L1 gathers)
  K.lanes = prm->kick_lanes && mixed ? prm->kick_lanes
                                     : (prm->precision == LJ_PREC_MIXED ? 1 : 4);
  K.block = 128;
  K.qfix = m.qfix.ptr;
  make_fixed_frame(K);
  ForceLaunch Kfull = K, Khalf = K;
  Kfull.dt = prm->dt;
  Khalf.dt = 0.5 * prm->dt;

  BuildArgs& b = m.build;
  b = BuildArgs{};
  b.q = q;
  b.n = n;
  b.grid = m.grid;
  b.search = rs;
  for (int d = 0; d < 3; d++) {
    b.box[d] = prm->box[d];
    b.unit[d] = K.unit[d];
  }
  b.aniso = K.aniso;
  b.start = m.start.ptr;
  b.order = m.order2.ptr;  // per-cell sorted order (k_sort_cells output)
  b.cq = m.cq2.ptr;
  b.cell = m.cell.ptr;
  b.superset = 1;  // the force kernels and energies apply the cutoff
  b.near = kFarSplit;
  b.want_half = mixed ? 0 : 1;
  b.want_full = mixed ? 1 : 0;

  DriftArgs D{};
  D.q = q;
  D.p = p;
  D.dt = prm->dt;
  for (int d = 0; d < 3; d++) {
    D.len[d] = prm->box[d];
    D.unit[d] = (float)K.unit[d];
  }
  D.half_skin2 = (float)(0.25 * prm->skin * prm->skin);
  D.rebuild_every = prm->rebuild_every > 0 ? prm->rebuild_every : 0;

  cudaEvent_t t0, t1;
  MD_CUDA(ctx, cudaEventCreate(&t0), "event");
  MD_CUDA(ctx, cudaEventCreate(&t1), "event");
  struct EvGuard {
    cudaEvent_t a, b;
    ~EvGuard() {
      cudaEventDestroy(a);
      cudaEventDestroy(b);
    }
  } evg{t0, t1};
  MD_CUDA(ctx, cudaEventRecord(t0, s), "event");
  if (io) {
    MD_CUDA(ctx, cudaEventRecord(io->ev_in, s), "event");  // after the caller's earlier work
    MD_CUDA(ctx, cudaMemcpyAsync(q, io->q, io->bytes, cudaMemcpyHostToDevice, s), "H2D q");
    MD_CUDA(ctx, cudaStreamWaitEvent(io->side, io->ev_in, 0), "wait");
    MD_CUDA(ctx, cudaMemcpyAsync(p, io->p, io->bytes, cudaMemcpyHostToDevice, io->side),
            "H2D p");
    MD_CUDA(ctx, cudaEventRecord(io->ev_p, io->side), "event");
  }

  // ---- initial image and list (one captured graph, so that its kernels are
  // counted) -------------------------------------------------------------------
  int64_t launches = 0;
  {
    cudaGraph_t g = nullptr;
    cudaGraphExec_t ge = nullptr;
    MD_CUDA(ctx, cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal), "capture");
    cudaError_t ce = launch_fixed_image(K, s);
    if (ce == cudaSuccess) {
      if (reuse)  // rebuild only if a particle moved beyond skin/2 since that build
        k_md_moved<<<std::min(grid1(n, 256), 152 * 8), 256, 0, s>>>(
            m.qfix.ptr, m.qref.ptr, n, D.unit[0], D.unit[1], D.unit[2], D.half_skin2,
            m.flags.ptr);
      else
        k_md_set<<<1, 32, 0, s>>>(m.flags.ptr, F_REBUILD, 1);
      ce = md_rebuild(m, !mixed, K, s);
    }
    cudaError_t ee = cudaStreamEndCapture(s, &g);
    if (ce == cudaSuccess && ee == cudaSuccess) {
      launches += graph_kernels(g);
      ce = cudaGraphInstantiate(&ge, g, 0);
      if (ce == cudaSuccess) ce = cudaGraphLaunch(ge, s);
      if (ge) cudaGraphExecDestroy(ge);
    }
    if (g) cudaGraphDestroy(g);
    if (ce != cudaSuccess || ee != cudaSuccess)
      return lj_fail(ctx, LJ_ERR_CUDA, "initial build: %s",
                     cudaGetErrorString(ce != cudaSuccess ? ce : ee));
  }

  int32_t nrec = 0;
  auto read_flags = [&](int32_t* f) -> int {
    MD_CUDA(ctx, cudaMemcpyAsync(f, m.flags.ptr, sizeof(int32_t) * F_WORDS,
                                 cudaMemcpyDeviceToHost, s), "flags");
    MD_CUDA(ctx, cudaStreamSynchronize(s), "sync");
    return LJ_OK;
  };
  auto record = [&](int64_t step) -> int {
    if (!records || nrec >= max_records) return LJ_OK;
    MD_CUDA(ctx, cudaMemsetAsync(m.energy.ptr, 0, 2 * sizeof(double), s), "memset");
    const double u2 = K.unit[0] * K.unit[0];
    const double cl2u = K.cl2 / u2;
    const float khi = (float)(1.0 / u2), klo = (float)(1.0 / u2 - (double)khi);
    const double band = cutoff_band(std::sqrt(cl2u), kCoarseQuantumErr, kBandFp32);
    // split rows: the near and the far part of every row in turn
    for (int part = 0; part < (K.split ? 2 : 1); part++) {
      const Csr c = part ? K.far : K.csr;
      if (mixed && !K.aniso)
        k_md_potential<false><<<grid1(n, 256), 256, 0, s>>>(
            q, m.qfix.ptr, c, K.box.len[0], K.box.len[1], K.box.len[2], khi, klo,
            (float)(cl2u * (1 - band)), (float)(cl2u * (1 + band)), K.cl2, m.energy.ptr + 1);
      else
        k_md_potential<true><<<grid1(n, 256), 256, 0, s>>>(
            q, m.qfix.ptr, c, K.box.len[0], K.box.len[1], K.box.len[2], 0.f, 0.f, 0.f, 0.f,
            K.cl2, m.energy.ptr + 1);
      launches++;
    }
    k_md_kinetic<<<std::min(grid1(n, 256), 1024), 256, 0, s>>>(p, n, m.energy.ptr);
    launches++;
    double e[2];
    MD_CUDA(ctx, cudaGetLastError(), "energy");
    MD_CUDA(ctx, cudaMemcpyAsync(e, m.energy.ptr, sizeof e, cudaMemcpyDeviceToHost, s), "energy");
    MD_CUDA(ctx, cudaStreamSynchronize(s), "sync");
    records[nrec].step = step;
    records[nrec].kinetic = e[0];
    records[nrec].potential = e[1];
    nrec++;
    return LJ_OK;
  };

  int32_t f[F_WORDS];
  int rc;
  if (io) MD_CUDA(ctx, cudaStreamWaitEvent(s, io->ev_p, 0), "wait");  // p's first use follows
  if ((rc = read_flags(f))) return rc;
  const int32_t initial_build = f[F_COUNT];  // 0: the previous run's list holds
  if (f[F_OVERFLOW])
    return lj_fail(ctx, LJ_ERR_LIST_OVERFLOW, "a neighbour row exceeds %d entries", m.maxrow);
  if ((rc = record(0))) return rc;

  // ---- the persistent loop over chunks of `graph_steps` plain steps --------
  const int gsteps = prm->graph_steps > 0 ? prm->graph_steps : 20;
  int64_t step_kernels = -1;  // kernels of one step (from the captured graph)
  std::vector<unsigned char> sig;
  auto put = [&](const void* v, size_t bytes) {
    const auto* c = static_cast<const unsigned char*>(v);
    sig.insert(sig.end(), c, c + bytes);
  };
  put(&Kfull, sizeof Kfull);
  put(&D, sizeof D);
  put(&m.build, sizeof m.build);
  put(&m.grid, sizeof m.grid);
  const void* used[] = {m.qfix.ptr,  m.qref.ptr,  m.cq.ptr,    m.cq2.ptr,   m.flags.ptr,
                        m.cell.ptr,  m.count.ptr, m.cursor.ptr, m.order.ptr, m.order2.ptr,
                        m.cnt.ptr,   m.ptr.ptr,   m.rows.ptr,  m.list.ptr,  m.rows2.ptr,
                        m.cnt2.ptr,  m.closeq.ptr, m.start.ptr, m.off.ptr,  m.scan_tmp.ptr};
  put(used, sizeof used);
  const int64_t sizes[] = {(int64_t)m.scan_tmp.cap, m.maxrow, m.maxrow_far, m.cap, m.cap2,
                           m.n, gsteps, prm->chunk_graphs};
  put(sizes, sizeof sizes);
  const bool cached = gsteps > 1 && (m.loop.exec || m.graph) && sig == m.graph_sig;
  if (cached) {
    step_kernels = m.graph_step_kernels;
  } else {
    m.graph_sig.clear();
    if (m.graph) {
      cudaGraphExecDestroy(m.graph);
      m.graph = nullptr;
    }
    m.loop.reset();
    if (gsteps > 1 && !prm->chunk_graphs &&
        m.loop.build(s, m.flags.ptr + F_LOOP, m.flags.ptr + F_OVERFLOW,
                     [&](cudaStream_t cs) {
                       cudaError_t ce = cudaSuccess;
                       for (int k = 0; k < gsteps && ce == cudaSuccess; k++)
                         ce = md_step(m, D, Kfull, cs);
                       return ce;
                     }) == cudaSuccess) {
      step_kernels = m.loop.kernels_per_chunk / gsteps;
      m.graph_steps = gsteps;
    } else if (gsteps > 1) {  // no conditional node: chunk graphs launched back to back
      cudaGraph_t g = nullptr;
      MD_CUDA(ctx, cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal), "capture");
      cudaError_t ce = cudaSuccess;
      for (int k = 0; k < gsteps && ce == cudaSuccess; k++) ce = md_step(m, D, Kfull, s);
      cudaError_t ee = cudaStreamEndCapture(s, &g);
      if (ce != cudaSuccess || ee != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        return lj_fail(ctx, LJ_ERR_CUDA, "graph capture: %s",
                       cudaGetErrorString(ce != cudaSuccess ? ce : ee));
      }
      step_kernels = graph_kernels(g) / gsteps;
      ce = cudaGraphInstantiate(&m.graph, g, 0);
      cudaGraphDestroy(g);
      if (ce != cudaSuccess) return lj_fail(ctx, LJ_ERR_CUDA, "graph instantiate");
      m.graph_steps = gsteps;
    }
    if (m.loop.exec || m.graph) {
      m.graph_sig = sig;
      m.graph_step_kernels = step_kernels;
    }
  }

  // ---- integrate -------------------------------------------------------------
  const int every = prm->record_every > 0 ? prm->record_every : nsteps;
  if (nsteps > 0) MD_CUDA(ctx, launch_force(Khalf, s), "kick");  // p(1/2)
  int64_t kicks = nsteps > 0 ? 1 : 0;  // each launch_force of the MD path is one kernel
  int64_t step = 0;
  while (step < nsteps) {
    int64_t stop = std::min<int64_t>(nsteps, (step / every + 1) * every);
    int64_t plain = stop - step - 1;
    const int64_t chunks = m.graph_steps > 0 ? plain / m.graph_steps : 0;
    if (chunks > 0 && m.loop.exec) {
      MD_CUDA(ctx, m.loop.launch((int32_t)chunks, s), "loop launch");
      plain -= chunks * m.graph_steps;
      launches += 1 + chunks;  // the count write and each pass's loop kernel
    }
    while (m.graph && plain >= m.graph_steps) {
      MD_CUDA(ctx, cudaGraphLaunch(m.graph, s), "graph launch");
      plain -= m.graph_steps;
    }
    for (; plain > 0; plain--) MD_CUDA(ctx, md_step(m, D, Kfull, s), "step");
    MD_CUDA(ctx, md_step(m, D, Khalf, s, stop == nsteps ? io : nullptr),
            "step");  // p(stop), synchronous
    if ((rc = read_flags(f))) return rc;
    if (f[F_OVERFLOW])
      return lj_fail(ctx, LJ_ERR_LIST_OVERFLOW,
                     "a neighbour row exceeded its capacity of %d entries", m.maxrow);
    if (stop % every == 0 || stop == nsteps)
      if ((rc = record(stop))) return rc;
    if (stop < nsteps) {
      MD_CUDA(ctx, launch_force(Khalf, s), "kick");
      kicks++;
    }
    step = stop;
  }
  if (io) {
    if (!io->q_queued)
      MD_CUDA(ctx, cudaMemcpyAsync(io->q, q, io->bytes, cudaMemcpyDeviceToHost, s), "D2H q");
    MD_CUDA(ctx, cudaMemcpyAsync(io->p, p, io->bytes, cudaMemcpyDeviceToHost, s), "D2H p");
    MD_CUDA(ctx, cudaEventRecord(io->ev_side_done, io->side), "event");
    MD_CUDA(ctx, cudaStreamWaitEvent(s, io->ev_side_done, 0), "wait");
  }
  MD_CUDA(ctx, cudaEventRecord(t1, s), "event");
  if ((rc = read_flags(f))) return rc;
  float ms = 0.f;
  cudaEventElapsedTime(&ms, t0, t1);
  if (stats) {
    stats->steps = nsteps;
    stats->rebuilds = f[F_COUNT] - initial_build;  // the initial build counts there too
    stats->ms_total = ms;
    stats->list_capacity = m.cap;
    stats->launches = step_kernels < 0 ? -1 : launches + kicks + nsteps * step_kernels;
    stats->loop_graph = m.loop.exec ? 1 : 0;
    stats->initial_build = initial_build;
  }
  if (n_records) *n_records = nrec;
  if (!ctx->stream) MD_CUDA(ctx, cudaStreamSynchronize(s), "sync");
  std::memcpy(m.list_key, key, sizeof key);
  std::memcpy(m.list_bufs, bufs, sizeof bufs);
  m.list_kept = true;
  return LJ_OK;
}

extern "C" int lj_md_run(lj_ctx* ctx, double* q, double* p, int32_t n, const lj_md_params* prm,
                         int32_t nsteps, lj_md_record* records, int32_t max_records,
                         int32_t* n_records, lj_md_stats* stats) {
  return md_run(ctx, q, p, n, prm, nsteps, records, max_records, n_records, stats, nullptr);
}

extern "C" int lj_md_run_host(lj_ctx* ctx, double* q, double* p, int32_t n,
                              const lj_md_params* prm, int32_t nsteps, lj_md_record* records,
                              int32_t max_records, int32_t* n_records, lj_md_stats* stats) {
  if (!ctx) return LJ_ERR_INVALID_ARGUMENT;
  ctx->err.clear();
  if (n_records) *n_records = 0;
  if (!q || !p || n < 1) return lj_fail(ctx, LJ_ERR_INVALID_ARGUMENT, "bad MD arguments");
  if (cudaSetDevice(ctx->device) != cudaSuccess) return lj_fail(ctx, LJ_ERR_CUDA, "set device");
  const size_t bytes = sizeof(double) * 4 * (size_t)n;
  MD_CUDA(ctx, ctx->mq.ensure(4 * (size_t)n), "alloc");
  MD_CUDA(ctx, ctx->mp.ensure(4 * (size_t)n), "alloc");
  HostIo io{q, p, bytes, nullptr, {}, {}, {}, {}};
  // the side stream and events live for this call; the guard waits for every
  // copy on the side stream before the host buffers are handed back
  struct Guard {
    HostIo& io;
    ~Guard() {
      if (io.side) {
        cudaStreamSynchronize(io.side);
        cudaStreamDestroy(io.side);
      }
      for (cudaEvent_t e : {io.ev_in, io.ev_p, io.ev_q, io.ev_side_done})
        if (e) cudaEventDestroy(e);
    }
  } guard{io};
  MD_CUDA(ctx, cudaStreamCreateWithFlags(&io.side, cudaStreamNonBlocking), "stream");
  for (cudaEvent_t* e : {&io.ev_in, &io.ev_p, &io.ev_q, &io.ev_side_done})
    MD_CUDA(ctx, cudaEventCreateWithFlags(e, cudaEventDisableTiming), "event");
  const int rc = md_run(ctx, ctx->mq.ptr, ctx->mp.ptr, n, prm, nsteps, records, max_records,
                        n_records, stats, &io);
  // the run's stream may still hold copies of the host buffers (on errors too)
  cudaStream_t s = ctx->stream ? ctx->stream : (ctx->md ? ctx->md->own_stream : nullptr);
  const cudaError_t se = s ? cudaStreamSynchronize(s) : cudaSuccess;
  if (rc) return rc;
  MD_CUDA(ctx, se, "sync");
  return LJ_OK;
}
