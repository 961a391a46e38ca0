// lj_nlist.cu -- on-device cell-list binning and neighbour-list build.
//
// Replaces the reference's host O(N^2) makepair + sortpair
// (cpu_ref/force_aos.cpp:100-140, cuda/force_cuda.cu:122-163):
//
//   1. bin:   cell of every particle (cell side >= search radius), counts
//   2. sort:  counting sort of particle indices by cell; the fixed-point
//             positions are gathered into cell order for coalesced reads
//   3. count: per particle, candidates in the 27 surrounding cells that pass
//             r2 < rs^2 (half: j > i, full: j != i)
//   4. scan:  row offsets
//   5. fill:  same walk, writing j
//   6. sort rows ascending (rank sort), so the CSR equals the reference's
//
// Membership is decided in FP32 from the exact int32 fixed-point separation;
// candidates within a relative 4e-6 of the search sphere are re-decided in
// FP64 with the reference's expression (dx = q_i - q_j), so the list is the
// reference's list without spending FP64 on every candidate.
#include "lj_internal.h"
#include "lj_nlist.h"

namespace ljg {
namespace {

__device__ __forceinline__ int wrap_cell(int c, int nc) {
  c %= nc;
  return c < 0 ? c + nc : c;
}

__device__ __forceinline__ bool off_guard(const int32_t* guard) {
  return guard && *(volatile const int32_t*)guard == 0;
}

__global__ void k_bin(const double* __restrict__ q, int n, CellGrid g, int32_t* __restrict__ cell,
                      int32_t* __restrict__ count, const int32_t* guard) {
  if (off_guard(guard)) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double* b = q + 4 * (size_t)i;
  int c[3];
  for (int d = 0; d < 3; d++) {
    const double t = (b[d] - g.lo[d]) * g.inv_w[d];
    int ci = (int)floor(t);
    if (g.periodic) ci = wrap_cell(ci, g.nc[d]);
    else ci = min(max(ci, 0), g.nc[d] - 1);
    c[d] = ci;
  }
  const int id = (c[2] * g.nc[1] + c[1]) * g.nc[0] + c[0];
  cell[i] = id;
  atomicAdd(count + id, 1);
}

__global__ void k_place(const int32_t* __restrict__ cell, int n, const int64_t* __restrict__ start,
                        int32_t* __restrict__ cursor, const int4* __restrict__ qfix,
                        int32_t* __restrict__ order, int4* __restrict__ cq,
                        const int32_t* guard) {
  if (off_guard(guard)) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int c = cell[i];
  const int slot = (int)start[c] + atomicAdd(cursor + c, 1);
  order[slot] = i;
  cq[slot] = qfix[i];
}

struct BuildConsts {
  float sl2_lo, sl2_hi;  // certainly inside / possibly inside, fixed units^2
  float u_hi[3], u_lo[3];
  int aniso;
  int periodic;
  double len[3];
  long long half_bits[3];
  double sl2;
};

// The reference's membership test (makepair: dx = q_i - q_j, r2 < SL2), FP64.
__device__ __forceinline__ bool within_fp64(const double* q, int i, int j, const BuildConsts& k) {
  const double* a = q + 4 * (size_t)i;
  const double* b = q + 4 * (size_t)j;
  double d[3];
  for (int x = 0; x < 3; x++) {
    d[x] = a[x] - b[x];
    if (k.periodic) d[x] = min_image_fp64(d[x], k.len[x], k.half_bits[x]);
  }
  const double r2 = fma(d[2], d[2], fma(d[1], d[1], d[0] * d[0]));
  return r2 < k.sl2;
}

__device__ __forceinline__ bool within(const int4& a, const int4& b, const double* q, int i,
                                       int j, const BuildConsts& k) {
  float dx = (float)wrap_sub(a.x, b.x), dy = (float)wrap_sub(a.y, b.y),
        dz = (float)wrap_sub(a.z, b.z);
  if (k.aniso) {
    dx = fmaf(dx, k.u_hi[0], dx * k.u_lo[0]);
    dy = fmaf(dy, k.u_hi[1], dy * k.u_lo[1]);
    dz = fmaf(dz, k.u_hi[2], dz * k.u_lo[2]);
  }
  const float r2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
  if (r2 < k.sl2_lo) return true;
  if (!(r2 < k.sl2_hi)) return false;
  return within_fp64(q, i, j, k);
}

// Visits the candidate cells of particle i's cell.  Along an axis with fewer
// than 3 cells every cell is visited once; otherwise c-1, c, c+1 (wrapped when
// periodic, clipped when open).
template <typename F>
__device__ __forceinline__ void for_neighbour_cells(int cid, const CellGrid& g, F&& f) {
  const int cx = cid % g.nc[0], cy = (cid / g.nc[0]) % g.nc[1], cz = cid / (g.nc[0] * g.nc[1]);
  int lo[3], hi[3];
  const int c[3] = {cx, cy, cz};
  for (int d = 0; d < 3; d++) {
    if (g.nc[d] < 3) {
      lo[d] = 0;
      hi[d] = g.nc[d] - 1;
    } else if (g.periodic) {
      lo[d] = c[d] - 1;
      hi[d] = c[d] + 1;
    } else {
      lo[d] = max(c[d] - 1, 0);
      hi[d] = min(c[d] + 1, g.nc[d] - 1);
    }
  }
  for (int z = lo[2]; z <= hi[2]; z++)
    for (int y = lo[1]; y <= hi[1]; y++)
      for (int x = lo[0]; x <= hi[0]; x++) {
        const int wx = g.nc[0] < 3 ? x : wrap_cell(x, g.nc[0]);
        const int wy = g.nc[1] < 3 ? y : wrap_cell(y, g.nc[1]);
        const int wz = g.nc[2] < 3 ? z : wrap_cell(z, g.nc[2]);
        f((wz * g.nc[1] + wy) * g.nc[0] + wx);
      }
}

// One thread per particle, in cell order (slot s), so neighbouring threads
// read the same cells.  pass 0 counts, pass 1 writes.
template <bool FILL>
__global__ void __launch_bounds__(128) k_walk(const double* __restrict__ q, int n, CellGrid g,
                                              const int64_t* __restrict__ start,
                                              const int32_t* __restrict__ order,
                                              const int4* __restrict__ cq,
                                              const int32_t* __restrict__ cell, BuildConsts k,
                                              int want_half, int want_full,
                                              int32_t* __restrict__ cnt_half,
                                              int32_t* __restrict__ cnt_full,
                                              const int64_t* __restrict__ off_half,
                                              const int64_t* __restrict__ off_full,
                                              int32_t* __restrict__ out_half,
                                              int32_t* __restrict__ out_full,
                                              const int32_t* guard) {
  if (off_guard(guard)) return;
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  const int i = order[s];
  const int4 xi = cq[s];
  int nh = 0, nf = 0;
  int64_t wh = 0, wf = 0;
  if (FILL) {
    if (want_half) wh = off_half[i];
    if (want_full) wf = off_full[i];
  }
  for_neighbour_cells(cell[i], g, [&](int c) {
    const int b = (int)start[c], e = (int)start[c + 1];
    for (int t = b; t < e; t++) {
      const int j = order[t];
      if (j == i) continue;
      if (!want_full && j < i) continue;
      if (!within(xi, cq[t], q, i, j, k)) continue;
      if (want_full) {
        if (FILL) out_full[wf + nf] = j;
        nf++;
      }
      if (want_half && j > i) {
        if (FILL) out_half[wh + nh] = j;
        nh++;
      }
    }
  });
  if (!FILL) {
    if (want_half) cnt_half[i] = nh;
    if (want_full) cnt_full[i] = nf;
  }
}

__global__ void k_minmax(const double* __restrict__ q, int n, unsigned long long* out) {
  // out[0..2]: max over +x (as ordered keys), out[3..5]: max over -x
  unsigned long long mx[3] = {0, 0, 0}, mn[3] = {0, 0, 0};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    for (int d = 0; d < 3; d++) {
      const double v = q[4 * (size_t)i + d];
      // order-preserving key of a double
      unsigned long long b = (unsigned long long)__double_as_longlong(v);
      b = (b >> 63) ? ~b : (b | 0x8000000000000000ull);
      unsigned long long nb = ~b;
      mx[d] = max(mx[d], b);
      mn[d] = max(mn[d], nb);
    }
  for (int d = 0; d < 3; d++) {
    for (int o = 16; o > 0; o >>= 1) {
      mx[d] = max(mx[d], __shfl_xor_sync(kFullMask, mx[d], o));
      mn[d] = max(mn[d], __shfl_xor_sync(kFullMask, mn[d], o));
    }
    if ((threadIdx.x & 31) == 0) {
      atomicMax(out + d, mx[d]);
      atomicMax(out + 3 + d, mn[d]);
    }
  }
}

int grid_of(int64_t work, int block, int cap) {
  int64_t g = (work + block - 1) / block;
  if (g < 1) g = 1;
  if (cap > 0 && g > cap) g = cap;
  return (int)g;
}

}  // namespace

double key_to_double(unsigned long long k) {
  const unsigned long long b = (k >> 63) ? (k & 0x7fffffffffffffffull) : ~k;
  double v;
  std::memcpy(&v, &b, sizeof v);
  return v;
}

cudaError_t launch_minmax(const double* q, int n, unsigned long long* out6, cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(out6, 0, 6 * sizeof(unsigned long long), s);
  if (e != cudaSuccess || n == 0) return e;
  k_minmax<<<grid_of(n, 256, 1024), 256, 0, s>>>(q, n, out6);
  return cudaGetLastError();
}

cudaError_t launch_bin(const double* q, int n, const CellGrid& g, int32_t* cell, int32_t* count,
                       cudaStream_t s, const int32_t* guard) {
  cudaError_t e = guard ? launch_zero_i32(count, g.ncells, guard, s)
                        : cudaMemsetAsync(count, 0, sizeof(int32_t) * (size_t)g.ncells, s);
  if (e != cudaSuccess || n == 0) return e;
  k_bin<<<grid_of(n, 256, 0), 256, 0, s>>>(q, n, g, cell, count, guard);
  return cudaGetLastError();
}

cudaError_t launch_place(const int32_t* cell, int n, const int64_t* start, int32_t* cursor,
                         int ncells, const int4* qfix, int32_t* order, int4* cq, cudaStream_t s,
                         const int32_t* guard) {
  cudaError_t e = guard ? launch_zero_i32(cursor, ncells, guard, s)
                        : cudaMemsetAsync(cursor, 0, sizeof(int32_t) * (size_t)ncells, s);
  if (e != cudaSuccess || n == 0) return e;
  k_place<<<grid_of(n, 256, 0), 256, 0, s>>>(cell, n, start, cursor, qfix, order, cq, guard);
  return cudaGetLastError();
}

cudaError_t launch_walk(const BuildArgs& a, bool fill, cudaStream_t s, const int32_t* guard) {
  if (a.n == 0) return cudaSuccess;
  BuildConsts k{};
  const double u2 = a.aniso ? 1.0 : a.unit[0] * a.unit[0];
  const double sl2u = a.search * a.search / u2;
  k.sl2_lo = (float)(sl2u * (1.0 - 4e-6));
  k.sl2_hi = (float)(sl2u * (1.0 + 4e-6));
  for (int d = 0; d < 3; d++) {
    k.u_hi[d] = (float)a.unit[d];
    k.u_lo[d] = (float)(a.unit[d] - (double)k.u_hi[d]);
    k.len[d] = a.grid.periodic ? a.box[d] : 0.0;
    const double h = 0.5 * k.len[d];
    long long hb;
    std::memcpy(&hb, &h, sizeof hb);
    k.half_bits[d] = hb;
  }
  k.aniso = a.aniso;
  k.periodic = a.grid.periodic;
  k.sl2 = a.search * a.search;
  const int blocks = grid_of(a.n, 128, 0);
  if (fill)
    k_walk<true><<<blocks, 128, 0, s>>>(a.q, a.n, a.grid, a.start, a.order, a.cq, a.cell, k,
                                        a.want_half, a.want_full, nullptr, nullptr, a.off_half,
                                        a.off_full, a.out_half, a.out_full, guard);
  else
    k_walk<false><<<blocks, 128, 0, s>>>(a.q, a.n, a.grid, a.start, a.order, a.cq, a.cell, k,
                                         a.want_half, a.want_full, a.cnt_half, a.cnt_full,
                                         nullptr, nullptr, nullptr, nullptr, guard);
  return cudaGetLastError();
}

}  // namespace ljg
