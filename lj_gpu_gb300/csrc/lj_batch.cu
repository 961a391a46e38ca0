// lj_batch.cu -- many independent replicas in one velocity-Verlet loop.
//
// The replicas (uneven N, own cubic box and density) are concatenated into one
// particle array; a replica table gives each its box, fixed-point frame and
// the range of its cells in one global cell numbering.  Every stage of the MD
// step (lj_md.cu) runs once over the whole batch: drift, flag-guarded rebuild
// (binning, cell offsets, placement, per-cell ordering, row build), and the
// mixed gather, which is launched once per size class of rows with the launch
// shape the class's own timing picked.  Two-float kicks split every row into
// a near part (two-float terms) and a far part (FP32 terms) when the skin
// allows it (BatchState::split).  Steps between energy records are
// replayed from a captured CUDA graph.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "lj_ctx.h"
#include "lj_nlist.h"

namespace ljg {
namespace {

enum { B_REBUILD = 0, B_OVERFLOW = 2, B_COUNT = 3, B_STEP = 5, B_LOOP = 6, B_WORDS = 8 };

__global__ void __launch_bounds__(256) k_batch_drift(double* __restrict__ q,
                                                     const double* __restrict__ p, int n,
                                                     double dt, const int32_t* __restrict__ rid,
                                                     const ReplicaInfo* __restrict__ reps,
                                                     int4* __restrict__ qfix,
                                                     const int4* __restrict__ qref,
                                                     float half_skin2, int rebuild_every,
                                                     int32_t* __restrict__ flags) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i == 0) {
    const int stepno = flags[B_STEP] + 1;
    flags[B_STEP] = stepno;
    if (rebuild_every > 0 && stepno % rebuild_every == 0) flags[B_REBUILD] = 1;
  }
  if (i >= n) return;
  const ReplicaInfo& R = reps[rid[i]];
  double* qi = q + 4 * (size_t)i;
  const double* pi = p + 4 * (size_t)i;
  const double x = wrap_into_box(fma(pi[0], dt, qi[0]), R.len[0]);
  const double y = wrap_into_box(fma(pi[1], dt, qi[1]), R.len[1]);
  const double z = wrap_into_box(fma(pi[2], dt, qi[2]), R.len[2]);
  qi[0] = x;
  qi[1] = y;
  qi[2] = z;
  const int4 X = pack_image(to_fixed_fine(x, R.ax[0]), to_fixed_fine(y, R.ax[1]),
                            to_fixed_fine(z, R.ax[2]));
  qfix[i] = X;
  const int4 r = qref[i];
  const float dx = (float)wrap_sub(X.x, r.x) * R.unit_f[0];
  const float dy = (float)wrap_sub(X.y, r.y) * R.unit_f[1];
  const float dz = (float)wrap_sub(X.z, r.z) * R.unit_f[2];
  if (fmaf(dz, dz, fmaf(dy, dy, dx * dx)) > half_skin2) flags[B_REBUILD] = 1;
}

__global__ void k_batch_image(const double* __restrict__ q, int n,
                              const int32_t* __restrict__ rid,
                              const ReplicaInfo* __restrict__ reps, int4* __restrict__ qfix) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const ReplicaInfo& R = reps[rid[i]];
  const double* b = q + 4 * (size_t)i;
  qfix[i] = pack_image(to_fixed_fine(b[0], R.ax[0]), to_fixed_fine(b[1], R.ax[1]),
                       to_fixed_fine(b[2], R.ax[2]));
}

__global__ void k_batch_copy_ref(const int4* __restrict__ qfix, int4* __restrict__ qref, int n,
                                 const int32_t* __restrict__ flags) {
  if (!flags[B_REBUILD]) return;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    qref[i] = qfix[i];
}

__global__ void k_batch_finish(int32_t* flags) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  if (flags[B_REBUILD]) flags[B_COUNT] += 1;
  flags[B_REBUILD] = 0;
}

__global__ void k_batch_set(int32_t* flags, int word, int value) {
  if (threadIdx.x == 0 && blockIdx.x == 0) flags[word] = value;
}

// Per-replica energies: kinetic (FP64, when `kinetic`) and potential over
// the pairs j > i of the rows of c with r2 <= rc^2 (FP32 from the image with
// Kahan sums; FP64 re-decision of the cutoff band), each replica into its
// own pair of accumulators.  Split rows take one launch per part.
__global__ void __launch_bounds__(256) k_batch_energy(
    const double* __restrict__ q, const double* __restrict__ p, const int4* __restrict__ qfix,
    Csr c, const int32_t* __restrict__ rid, const ReplicaInfo* __restrict__ reps, double cl2,
    double* __restrict__ out, bool kinetic) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= c.n) return;
  const int r = rid[i];
  const ReplicaInfo& R = reps[r];
  const double* pi = p + 4 * (size_t)i;
  const double kin = 0.5 * (pi[0] * pi[0] + pi[1] * pi[1] + pi[2] * pi[2]);
  const int cnt = c.np[i];
  const int64_t k0 = row_start(c, i);
  const int4 xi = qfix[i];
  const double* qi = q + 4 * (size_t)i;
  float s = 0.f, comp = 0.f;
  for (int m = 0; m < cnt; m++) {
    const int j = c.list[k0 + m];
    if (j <= i) continue;
    const int4 xj = qfix[j];
    const float dx = (float)wrap_sub(xj.x, xi.x), dy = (float)wrap_sub(xj.y, xi.y),
                dz = (float)wrap_sub(xj.z, xi.z);
    const float r2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
    bool in = r2 <= R.cl2u_lo;
    if (!in && r2 <= R.cl2u_hi) {
      const double* qj = q + 4 * (size_t)j;
      double d[3];
      for (int x = 0; x < 3; x++) d[x] = min_image_fp64(qj[x] - qi[x], R.len[x], R.half_bits[x]);
      in = !(fma(d[2], d[2], fma(d[0], d[0], d[1] * d[1])) > cl2);
    }
    if (!in) continue;
    float inv = 1.0f / r2;
    inv = fmaf(inv, R.k_hi, inv * R.k_lo);
    const float ir6 = inv * inv * inv;
    const float e = 4.0f * ir6 * (ir6 - 1.0f);
    const float y = e - comp;
    const float t = s + y;
    comp = (t - s) - y;
    s = t;
  }
  if (kinetic) atomicAdd(out + 2 * r, kin);
  const double u = (double)s - (double)comp;
  if (u != 0.0) atomicAdd(out + 2 * r + 1, u);
}

int gridn(int64_t n, int b) { return (int)std::max<int64_t>(1, (n + b - 1) / b); }

void split(double v, float& hi, float& lo) {
  hi = (float)v;
  lo = (float)(v - (double)hi);
}

}  // namespace

struct BatchState {
  int n = 0, R = 0, ncells = 0, maxrow = 0;
  // split rows (two-float kicks): rows / cnt hold every row's near part,
  // rows2 / cnt2 its far part (maxrow each); closef (three words) and closeq
  // (a slot per particle) the close queue of far entries inside kFarCheck
  bool split = false;
  DevBuf<ReplicaInfo> reps;
  DevBuf<int32_t> rid, cell_rid, flags, cell, count, cursor, order, order2, cnt, rows, classrows;
  DevBuf<int32_t> rows2, cnt2, closef, closeq;
  DevBuf<int4> qfix, qref, cq, cq2;
  DevBuf<int64_t> start;
  DevBuf<unsigned char> scan_tmp;
  DevBuf<double> energy, ptmp;
  cudaStream_t own_stream = nullptr;
  ~BatchState() {
    if (own_stream) cudaStreamDestroy(own_stream);
  }
};

}  // namespace ljg

using namespace ljg;

namespace {

struct SizeClass {
  int first, count;  // range in the class-ordered row list
  int lanes, unroll;
  bool vec;          // 16-byte index loads (unroll 4; rows are 16-byte aligned)
  double ms;
};

#define B_CUDA(ctx, call, what)                                                        \
  do {                                                                                 \
    cudaError_t e_ = (call);                                                           \
    if (e_ != cudaSuccess)                                                             \
      return lj_fail(ctx, e_ == cudaErrorMemoryAllocation ? LJ_ERR_OUT_OF_MEMORY : LJ_ERR_CUDA, \
                     "%s: %s", what, cudaGetErrorString(e_));                          \
  } while (0)

cudaError_t batch_rebuild(BatchState& b, const double* q, double sl2, cudaStream_t s) {
  const int32_t* g = b.flags.ptr + B_REBUILD;
  cudaError_t e;
  if ((e = launch_bin_batch(q, b.n, b.rid.ptr, b.reps.ptr, b.ncells, b.cell.ptr, b.count.ptr, s,
                            g)))
    return e;
  if ((e = launch_scan_counts(b.count.ptr, b.ncells, b.start.ptr, b.scan_tmp.ptr, b.scan_tmp.cap,
                              s, g)))
    return e;
  if ((e = launch_place(b.cell.ptr, b.n, b.start.ptr, b.cursor.ptr, b.ncells, b.qfix.ptr,
                        b.order.ptr, b.cq.ptr, s, g)))
    return e;
  if ((e = launch_sort_cells(b.start.ptr, b.ncells, b.order.ptr, b.cq.ptr, b.order2.ptr,
                             b.cq2.ptr, s, g)))
    return e;
  if ((e = launch_build_rows_batch(q, b.reps.ptr, b.cell_rid.ptr, b.ncells, sl2, b.start.ptr,
                                   b.order2.ptr, b.cq2.ptr, b.maxrow, b.rows.ptr, b.cnt.ptr,
                                   b.split ? b.rows2.ptr : nullptr,
                                   b.split ? b.cnt2.ptr : nullptr, b.flags.ptr + B_OVERFLOW, s,
                                   g)))
    return e;
  k_batch_copy_ref<<<std::min(gridn(b.n, 256), 152 * 8), 256, 0, s>>>(b.qfix.ptr, b.qref.ptr, b.n, b.flags.ptr);
  k_batch_finish<<<1, 32, 0, s>>>(b.flags.ptr);
  return cudaGetLastError();
}

cudaError_t batch_kick(BatchState& b, const Particles& part, const std::vector<SizeClass>& cls,
                       double dt, double cl2, bool ff, cudaStream_t s) {
  const Csr c{b.n, 0, b.cnt.ptr, nullptr, b.rows.ptr, (int64_t)b.maxrow, 1};
  const Csr far{b.n, 0, b.cnt2.ptr, nullptr, b.rows2.ptr, (int64_t)b.maxrow, 1};
  for (const SizeClass& k : cls) {
    cudaError_t e = launch_force_batch(part, c, b.qfix.ptr, b.rid.ptr, b.reps.ptr,
                                       b.classrows.ptr + k.first, k.count, dt, cl2, k.lanes,
                                       k.unroll, k.vec, ff, s, b.split ? &far : nullptr,
                                       b.closef.ptr, b.closeq.ptr);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

}  // namespace

extern "C" int lj_batch_run(lj_ctx* ctx, double* q, double* p, int32_t n_total,
                            int32_t n_replicas, const int32_t* offsets, const double* boxes,
                            const lj_md_params* prm, int32_t nsteps, double* energies,
                            int32_t max_records, int32_t* n_records, lj_md_stats* stats,
                            int32_t* class_shapes) {
  if (!ctx) return LJ_ERR_INVALID_ARGUMENT;
  ctx->err.clear();
  if (n_records) *n_records = 0;
  if (!prm || !offsets || !boxes || !q || !p || n_total < 1 || n_replicas < 1 || nsteps < 0)
    return lj_fail(ctx, LJ_ERR_INVALID_ARGUMENT, "bad batch arguments");
  if ((reinterpret_cast<uintptr_t>(q) | reinterpret_cast<uintptr_t>(p)) & 15u)
    return lj_fail(ctx, LJ_ERR_INVALID_ARGUMENT, "q and p must be 16-byte aligned");
  if (prm->precision != LJ_PREC_MIXED && prm->precision != LJ_PREC_MIXED_FP32)
    return lj_fail(ctx, LJ_ERR_UNSUPPORTED, "the batch runs the mixed path");
  const bool ff = prm->precision == LJ_PREC_MIXED;  // two-float pair terms
  if (!(prm->dt > 0.0) || !(prm->rc > 0.0) || !(prm->skin >= 0.0))
    return lj_fail(ctx, LJ_ERR_INVALID_ARGUMENT, "dt, rc must be > 0 and skin >= 0");
  if (offsets[0] != 0 || offsets[n_replicas] != n_total)
    return lj_fail(ctx, LJ_ERR_INVALID_ARGUMENT, "offsets must run from 0 to n_total");
  const double rs = prm->rc + prm->skin;
  if (cudaSetDevice(ctx->device) != cudaSuccess) return lj_fail(ctx, LJ_ERR_CUDA, "set device");
  if (!ctx->batch) ctx->batch.reset(new BatchState());
  BatchState& b = *ctx->batch;
  cudaStream_t s = ctx->stream;
  if (!s) {
    if (!b.own_stream)
      B_CUDA(ctx, cudaStreamCreateWithFlags(&b.own_stream, cudaStreamNonBlocking), "stream");
    B_CUDA(ctx, cudaStreamSynchronize(nullptr), "sync");
    s = b.own_stream;
  }

  // ---- replica table, cell numbering, size classes (host) -----------------
  const int R = n_replicas;
  std::vector<ReplicaInfo> reps((size_t)R);
  std::vector<int32_t> rid((size_t)n_total), cell_rid;
  std::vector<std::vector<int32_t>> class_rows(3);
  int ncells = 0;
  double max_per = 0.0;
  std::vector<int> rep_class((size_t)R);
  for (int r = 0; r < R; r++) {
    const int off = offsets[r], cnt = offsets[r + 1] - offsets[r];
    if (cnt < 1) return lj_fail(ctx, LJ_ERR_INVALID_ARGUMENT, "replica %d is empty", r);
    const double* bx = boxes + 3 * r;
    if (!(bx[0] > 2.0 * rs) || bx[0] != bx[1] || bx[1] != bx[2])
      return lj_fail(ctx, LJ_ERR_INVALID_ARGUMENT,
                     "replica %d: boxes must be cubic and exceed twice the list radius", r);
    ReplicaInfo& I = reps[(size_t)r];
    std::memset(&I, 0, sizeof I);
    ForceLaunch F{};
    F.box.on = 1;
    for (int d = 0; d < 3; d++) {
      F.box.len[d] = bx[d];
      F.box.half[d] = 0.5 * bx[d];
    }
    make_fixed_frame(F);
    const double u = F.unit[0], u2 = u * u;
    for (int d = 0; d < 3; d++) {
      I.ax[d] = F.axis[d];
      I.len[d] = bx[d];
      const double h = 0.5 * bx[d];
      std::memcpy(&I.half_bits[d], &h, sizeof h);
      I.unit_f[d] = (float)u;
      I.nc[d] = std::max(1, (int)std::floor(bx[d] / rs));
      I.inv_w[d] = I.nc[d] / bx[d];
    }
    split(1.0 / u2, I.k_hi, I.k_lo);
    const double cl2u = prm->rc * prm->rc / u2, sl2u = rs * rs / u2;
    // cutoff and list bands: FP32 arithmetic plus the coarse quantum, and for
    // two-float terms the float comparison plus the fine quantum
    const double bc = cutoff_band(std::sqrt(cl2u), kCoarseQuantumErr, kBandFp32);
    const double bf = cutoff_band(std::sqrt(cl2u), kCoarseQuantumErr / 1024.0, kBandFF);
    // the list build's separations also carry the rounding of positions
    // relative to the cell origin (two cell widths, 8 W 2^-24)
    const double wmax = 4294967296.0 / std::min(I.nc[0], std::min(I.nc[1], I.nc[2]));
    const double bs = cutoff_band(std::sqrt(sl2u), kCoarseQuantumErr + 8.0 * wmax * 0x1p-24,
                                  kBandFp32);
    I.cl2u_lo = (float)(cl2u * (1 - bc));
    I.cl2u_hi = (float)(cl2u * (1 + bc));
    I.cl2f_lo = (float)(cl2u * (1 - bf));
    I.cl2f_hi = (float)(cl2u * (1 + bf));
    I.sl2u_lo = (float)(sl2u * (1 - bs));
    I.sl2u_hi = (float)(sl2u * (1 + bs));
    I.near2u = (float)(kFarSplit * kFarSplit / u2);
    I.nearc2u = (float)(kFarCheck * kFarCheck / u2);
    I.unit = u;
    I.cell_base = ncells;
    I.offset = off;
    I.count = cnt;
    const int rc_cells = I.nc[0] * I.nc[1] * I.nc[2];
    ncells += rc_cells;
    for (int c = 0; c < rc_cells; c++) cell_rid.push_back(r);
    for (int i = off; i < off + cnt; i++) rid[(size_t)i] = r;
    // size class from the expected full row length
    const double per = 4.18879 * rs * rs * rs * cnt / (bx[0] * bx[1] * bx[2]);
    max_per = std::max(max_per, per);
    const int cls = per <= 48 ? 0 : (per <= 96 ? 1 : 2);
    rep_class[(size_t)r] = cls;
    for (int i = off; i < off + cnt; i++) class_rows[(size_t)cls].push_back(i);
  }
  std::vector<int32_t> rows_flat;
  std::vector<SizeClass> cls;
  for (int k = 0; k < 3; k++) {
    if (class_rows[(size_t)k].empty()) continue;
    cls.push_back({(int)rows_flat.size(), (int)class_rows[(size_t)k].size(), 4, 4, false, 0.0});
    rows_flat.insert(rows_flat.end(), class_rows[(size_t)k].begin(), class_rows[(size_t)k].end());
  }
  b.n = n_total;
  b.R = R;
  b.ncells = ncells;
  b.maxrow = ((int)std::ceil(max_per * 1.6) + 32 + 31) / 32 * 32;
  B_CUDA(ctx, b.reps.ensure((size_t)R), "alloc");
  B_CUDA(ctx, b.rid.ensure((size_t)n_total), "alloc");
  B_CUDA(ctx, b.cell_rid.ensure((size_t)ncells), "alloc");
  B_CUDA(ctx, b.classrows.ensure(rows_flat.size()), "alloc");
  B_CUDA(ctx, b.flags.ensure(B_WORDS), "alloc");
  B_CUDA(ctx, b.cell.ensure((size_t)n_total), "alloc");
  B_CUDA(ctx, b.count.ensure((size_t)ncells), "alloc");
  B_CUDA(ctx, b.cursor.ensure((size_t)ncells), "alloc");
  B_CUDA(ctx, b.start.ensure((size_t)ncells + 1), "alloc");
  B_CUDA(ctx, b.order.ensure((size_t)n_total), "alloc");
  B_CUDA(ctx, b.order2.ensure((size_t)n_total), "alloc");
  B_CUDA(ctx, b.cnt.ensure((size_t)n_total), "alloc");
  B_CUDA(ctx, b.rows.ensure((size_t)n_total * b.maxrow), "alloc");
  // two-float kicks split the rows; far pairs that come inside kFarCheck
  // before the next rebuild go through the close queue
  b.split = ff && !prm->ff_all;
  if (b.split) {
    B_CUDA(ctx, b.rows2.ensure((size_t)n_total * b.maxrow), "alloc");
    B_CUDA(ctx, b.cnt2.ensure((size_t)n_total), "alloc");
    B_CUDA(ctx, b.closef.ensure(3), "alloc");
    B_CUDA(ctx, b.closeq.ensure((size_t)n_total), "alloc");
    B_CUDA(ctx, cudaMemsetAsync(b.closef.ptr, 0, 3 * sizeof(int32_t), s), "memset");
  }
  B_CUDA(ctx, b.qfix.ensure((size_t)n_total), "alloc");
  B_CUDA(ctx, b.qref.ensure((size_t)n_total), "alloc");
  B_CUDA(ctx, b.cq.ensure((size_t)n_total), "alloc");
  B_CUDA(ctx, b.cq2.ensure((size_t)n_total), "alloc");
  B_CUDA(ctx, b.scan_tmp.ensure(scan_tmp_bytes(std::max(ncells, n_total))), "alloc");
  B_CUDA(ctx, b.energy.ensure(2 * (size_t)R), "alloc");
  B_CUDA(ctx, b.ptmp.ensure(4 * (size_t)n_total), "alloc");
  B_CUDA(ctx, cudaMemcpyAsync(b.reps.ptr, reps.data(), sizeof(ReplicaInfo) * R,
                              cudaMemcpyHostToDevice, s), "upload");
  B_CUDA(ctx, cudaMemcpyAsync(b.rid.ptr, rid.data(), sizeof(int32_t) * n_total,
                              cudaMemcpyHostToDevice, s), "upload");
  B_CUDA(ctx, cudaMemcpyAsync(b.cell_rid.ptr, cell_rid.data(), sizeof(int32_t) * ncells,
                              cudaMemcpyHostToDevice, s), "upload");
  B_CUDA(ctx, cudaMemcpyAsync(b.classrows.ptr, rows_flat.data(),
                              sizeof(int32_t) * rows_flat.size(), cudaMemcpyHostToDevice, s),
         "upload");
  B_CUDA(ctx, cudaMemsetAsync(b.flags.ptr, 0, sizeof(int32_t) * B_WORDS, s), "memset");

  const double sl2 = rs * rs, cl2 = prm->rc * prm->rc;
  Particles part{};
  part.q = q;
  part.p = p;

  // ---- initial image and list ----------------------------------------------
  k_batch_image<<<gridn(n_total, 256), 256, 0, s>>>(q, n_total, b.rid.ptr, b.reps.ptr, b.qfix.ptr);
  k_batch_set<<<1, 32, 0, s>>>(b.flags.ptr, B_REBUILD, 1);
  B_CUDA(ctx, batch_rebuild(b, q, sl2, s), "initial build");
  int32_t f[B_WORDS];
  auto read_flags = [&]() -> int {
    B_CUDA(ctx, cudaMemcpyAsync(f, b.flags.ptr, sizeof f, cudaMemcpyDeviceToHost, s), "flags");
    B_CUDA(ctx, cudaStreamSynchronize(s), "sync");
    return LJ_OK;
  };
  int rc;
  if ((rc = read_flags())) return rc;
  if (f[B_OVERFLOW])
    return lj_fail(ctx, LJ_ERR_LIST_OVERFLOW, "a neighbour row exceeds %d entries", b.maxrow);

  // ---- per-class launch shapes: time candidates on the class's rows -------
  {
    Particles tp = part;
    tp.p = b.ptmp.ptr;
    const Csr c{b.n, 0, b.cnt.ptr, nullptr, b.rows.ptr, (int64_t)b.maxrow, 1};
    const Csr far{b.n, 0, b.cnt2.ptr, nullptr, b.rows2.ptr, (int64_t)b.maxrow, 1};
    const Csr* fp = b.split ? &far : nullptr;
    cudaEvent_t e0, e1;
    B_CUDA(ctx, cudaEventCreate(&e0), "event");
    B_CUDA(ctx, cudaEventCreate(&e1), "event");
    // lanes, entries in flight, 16-byte index loads
    const int shapes[][3] = {{1, 2, 0}, {1, 4, 0}, {2, 4, 0}, {4, 2, 0}, {4, 4, 0},
                             {8, 2, 0}, {8, 4, 0}, {1, 4, 1}, {2, 4, 1}, {4, 4, 1},
                             {8, 4, 1}};
    for (SizeClass& k : cls) {
      k.ms = 1e300;
      for (const auto& sh : shapes) {
        cudaError_t e = launch_force_batch(tp, c, b.qfix.ptr, b.rid.ptr, b.reps.ptr,
                                           b.classrows.ptr + k.first, k.count, prm->dt, cl2,
                                           sh[0], sh[1], sh[2] != 0, ff, s, fp, b.closef.ptr,
                                           b.closeq.ptr);
        cudaEventRecord(e0, s);
        for (int rep = 0; rep < 3 && e == cudaSuccess; rep++)
          e = launch_force_batch(tp, c, b.qfix.ptr, b.rid.ptr, b.reps.ptr,
                                 b.classrows.ptr + k.first, k.count, prm->dt, cl2, sh[0], sh[1],
                                 sh[2] != 0, ff, s, fp, b.closef.ptr, b.closeq.ptr);
        cudaEventRecord(e1, s);
        if (e != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess) {
          cudaEventDestroy(e0);
          cudaEventDestroy(e1);
          return lj_fail(ctx, LJ_ERR_CUDA, "class tuning launch failed");
        }
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms / 3 < k.ms) {
          k.ms = ms / 3;
          k.lanes = sh[0];
          k.unroll = sh[1];
          k.vec = sh[2] != 0;
        }
      }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
  }
  if (class_shapes)
    for (size_t k = 0; k < 3; k++) {
      class_shapes[3 * k + 0] = k < cls.size() ? cls[k].count : 0;
      class_shapes[3 * k + 1] = k < cls.size() ? cls[k].lanes : 0;
      class_shapes[3 * k + 2] = k < cls.size() ? cls[k].unroll : 0;
    }

  // ---- step machinery ---------------------------------------------------------
  const float half_skin2 = (float)(0.25 * prm->skin * prm->skin);
  const int rebuild_every = prm->rebuild_every > 0 ? prm->rebuild_every : 0;
  auto step = [&](double kick_dt) -> cudaError_t {
    k_batch_drift<<<gridn(n_total, 256), 256, 0, s>>>(q, p, n_total, prm->dt, b.rid.ptr,
                                                      b.reps.ptr, b.qfix.ptr, b.qref.ptr,
                                                      half_skin2, rebuild_every, b.flags.ptr);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    if ((e = batch_rebuild(b, q, sl2, s))) return e;
    return batch_kick(b, part, cls, kick_dt, cl2, ff, s);
  };
  int32_t nrec = 0;
  auto record = [&](int64_t stepno) -> int {
    if (!energies || nrec >= max_records) return LJ_OK;
    B_CUDA(ctx, cudaMemsetAsync(b.energy.ptr, 0, 2 * sizeof(double) * R, s), "memset");
    const Csr c{b.n, 0, b.cnt.ptr, nullptr, b.rows.ptr, (int64_t)b.maxrow, 1};
    k_batch_energy<<<gridn(n_total, 256), 256, 0, s>>>(q, p, b.qfix.ptr, c, b.rid.ptr, b.reps.ptr,
                                                      cl2, b.energy.ptr, true);
    if (b.split) {
      const Csr far{b.n, 0, b.cnt2.ptr, nullptr, b.rows2.ptr, (int64_t)b.maxrow, 1};
      k_batch_energy<<<gridn(n_total, 256), 256, 0, s>>>(q, p, b.qfix.ptr, far, b.rid.ptr,
                                                        b.reps.ptr, cl2, b.energy.ptr, false);
    }
    B_CUDA(ctx, cudaGetLastError(), "energy");
    B_CUDA(ctx, cudaMemcpyAsync(energies + (size_t)nrec * 2 * R, b.energy.ptr,
                                2 * sizeof(double) * R, cudaMemcpyDeviceToHost, s), "energy");
    B_CUDA(ctx, cudaStreamSynchronize(s), "sync");
    (void)stepno;
    nrec++;
    return LJ_OK;
  };

  cudaEvent_t t0, t1;
  B_CUDA(ctx, cudaEventCreate(&t0), "event");
  B_CUDA(ctx, cudaEventCreate(&t1), "event");
  struct EvGuard {
    cudaEvent_t a, c;
    ~EvGuard() {
      cudaEventDestroy(a);
      cudaEventDestroy(c);
    }
  } evg{t0, t1};
  if ((rc = record(0))) return rc;
  B_CUDA(ctx, cudaEventRecord(t0, s), "event");

  // the steps between records: one launch of the persistent loop graph, or
  // (no conditional node) chunk graphs launched back to back
  const int gsteps = prm->graph_steps > 0 ? prm->graph_steps : 20;
  cudaGraphExec_t graph = nullptr;
  struct GraphGuard {
    cudaGraphExec_t* g;
    ~GraphGuard() {
      if (*g) cudaGraphExecDestroy(*g);
    }
  } gg{&graph};
  LoopGraph loop;
  if (gsteps > 1 && !prm->chunk_graphs && loop.build(s, b.flags.ptr + B_LOOP, b.flags.ptr + B_OVERFLOW,
                               [&](cudaStream_t) {
                                 cudaError_t ce = cudaSuccess;
                                 for (int k = 0; k < gsteps && ce == cudaSuccess; k++)
                                   ce = step(prm->dt);
                                 return ce;
                               }) == cudaSuccess) {
    // the loop runs the chunks
  } else if (gsteps > 1) {
    cudaGraph_t g = nullptr;
    B_CUDA(ctx, cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal), "capture");
    cudaError_t ce = cudaSuccess;
    for (int k = 0; k < gsteps && ce == cudaSuccess; k++) ce = step(prm->dt);
    cudaError_t ee = cudaStreamEndCapture(s, &g);
    if (ce != cudaSuccess || ee != cudaSuccess) {
      if (g) cudaGraphDestroy(g);
      return lj_fail(ctx, LJ_ERR_CUDA, "graph capture: %s",
                     cudaGetErrorString(ce != cudaSuccess ? ce : ee));
    }
    ce = cudaGraphInstantiate(&graph, g, 0);
    cudaGraphDestroy(g);
    if (ce != cudaSuccess) return lj_fail(ctx, LJ_ERR_CUDA, "graph instantiate");
  }
  const int every = prm->record_every > 0 ? prm->record_every : nsteps;
  if (nsteps > 0) B_CUDA(ctx, batch_kick(b, part, cls, 0.5 * prm->dt, cl2, ff, s), "kick");
  int64_t done = 0;
  while (done < nsteps) {
    const int64_t stop = std::min<int64_t>(nsteps, (done / every + 1) * every);
    int64_t plain = stop - done - 1;
    if (loop.exec && plain >= gsteps) {
      B_CUDA(ctx, loop.launch((int32_t)(plain / gsteps), s), "loop launch");
      plain %= gsteps;
    }
    while (graph && plain >= gsteps) {
      B_CUDA(ctx, cudaGraphLaunch(graph, s), "graph launch");
      plain -= gsteps;
    }
    for (; plain > 0; plain--) B_CUDA(ctx, step(prm->dt), "step");
    B_CUDA(ctx, step(0.5 * prm->dt), "step");
    if ((rc = read_flags())) return rc;
    if (f[B_OVERFLOW])
      return lj_fail(ctx, LJ_ERR_LIST_OVERFLOW, "a neighbour row exceeded %d entries", b.maxrow);
    if (stop % every == 0 || stop == nsteps)
      if ((rc = record(stop))) return rc;
    if (stop < nsteps) B_CUDA(ctx, batch_kick(b, part, cls, 0.5 * prm->dt, cl2, ff, s), "kick");
    done = stop;
  }
  B_CUDA(ctx, cudaEventRecord(t1, s), "event");
  if ((rc = read_flags())) return rc;
  float ms = 0.f;
  cudaEventElapsedTime(&ms, t0, t1);
  if (stats) {
    stats->steps = nsteps;
    stats->rebuilds = f[B_COUNT] - 1;  // the initial build is counted by the finish kernel
    stats->ms_total = ms;
    stats->list_capacity = (int64_t)n_total * b.maxrow;
    stats->launches = -1;
    stats->loop_graph = loop.exec ? 1 : 0;
  }
  if (n_records) *n_records = nrec;
  return LJ_OK;
}

namespace ljg {
void batch_state_delete(BatchState* b) { delete b; }
}  // namespace ljg
