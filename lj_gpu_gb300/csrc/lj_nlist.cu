// lj_nlist.cu -- on-device cell-list binning and neighbour-list build.
//
// Replaces the reference's host O(N^2) makepair + sortpair
// (cpu_ref/force_aos.cpp:100-140, cuda/force_cuda.cu:122-163):
//
//   1. bin:   cell of every particle (cell side >= search radius), counts
//   2. sort:  counting sort of particle indices by cell; the fixed-point
//             positions are gathered into cell order for coalesced reads
//   3. order: the slots of every cell sorted by particle index (deterministic)
//   4. rows:  one warp per cell walks the 27 surrounding cells and writes the
//             j with r2 < rs^2 (half: j > i, full: j != i) into padded rows
//   5. scan + compact into a CSR; rows sorted ascending (rank sort), so the
//             CSR equals the reference's
//
// Membership is decided in FP32 from the exact int32 fixed-point separation;
// candidates within a relative 4e-6 of the search sphere are re-decided in
// FP64 with the reference's expression (dx = q_i - q_j), so the list is the
// reference's list without spending FP64 on every candidate.
#include "lj_cells.cuh"
#include "lj_internal.h"
#include "lj_nlist.h"

namespace ljg {
namespace {


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

// Deterministic order inside every cell: the slots of cell c sorted by
// particle index (one warp per cell, stable rank sort, out of place).  The
// counting-sort placement before it uses atomics, so its order varies run to
// run; this makes every later walk -- and every floating-point sum over a
// row -- reproducible.
__global__ void k_sort_cells(const int64_t* __restrict__ start, int ncells,
                             const int32_t* __restrict__ order, const int4* __restrict__ cq,
                             int32_t* __restrict__ order2, int4* __restrict__ cq2,
                             const int32_t* guard) {
  if (off_guard(guard)) return;
  const int lane = threadIdx.x & 31;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  for (int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; c < ncells; c += nwarps) {
    const int s0 = (int)start[c], s1 = (int)start[c + 1];
    for (int a = s0 + lane; a < s1; a += 32) {
      const int v = order[a];
      int rank = 0;
      for (int b = s0; b < s1; b++) rank += order[b] < v;  // indices are distinct
      order2[s0 + rank] = v;
      cq2[s0 + rank] = cq[a];
    }
  }
}

// Warp-cooperative neighbour build into a padded row layout (row i at
// i * maxrow, length cnt[i]).  One warp per cell: the lanes hold up to 32 of
// the cell's particles; every neighbour cell is read 32 particles at a time
// with coalesced loads and broadcast to all lanes by shuffles, so a candidate
// costs shuffles and FP32/integer arithmetic instead of a scattered load.
// Rows come out in cell-walk order (deterministic after k_sort_cells).  A row
// longer than maxrow is truncated and raises *overflow.
template <bool HALF>
__global__ void __launch_bounds__(128) k_build_rows(const double* __restrict__ q, CellGrid g,
                                                    const int64_t* __restrict__ start,
                                                    const int32_t* __restrict__ order,
                                                    const int4* __restrict__ cq, BuildConsts k,
                                                    int maxrow, int32_t* __restrict__ rows,
                                                    int32_t* __restrict__ cnt,
                                                    int32_t* __restrict__ overflow,
                                                    const int32_t* guard) {
  if (off_guard(guard)) return;
  const int lane = threadIdx.x & 31;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  for (int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; c < g.ncells; c += nwarps) {
    const int s0 = (int)start[c], s1 = (int)start[c + 1];
    for (int a = s0; a < s1; a += 32) {
      const bool act = a + lane < s1;
      const int i = act ? order[a + lane] : -1;
      const int4 xi = act ? cq[a + lane] : make_int4(0, 0, 0, 0);
      const size_t base = act ? (size_t)i * (size_t)maxrow : 0;
      int count = 0;
      for_neighbour_cells(c, g, [&](int c2) {
        const int t0 = (int)start[c2], t1 = (int)start[c2 + 1];
        for (int b = t0; b < t1; b += 32) {
          int jl = -1;
          int4 xl = make_int4(0, 0, 0, 0);
          if (b + lane < t1) {
            jl = order[b + lane];
            xl = cq[b + lane];
          }
          const int m = min(32, t1 - b);
          for (int kk = 0; kk < m; kk++) {
            const int j = __shfl_sync(kFullMask, jl, kk);
            int4 xj;
            xj.x = __shfl_sync(kFullMask, xl.x, kk);
            xj.y = __shfl_sync(kFullMask, xl.y, kk);
            xj.z = __shfl_sync(kFullMask, xl.z, kk);
            xj.w = 0;
            if (act && j != i && (!HALF || j > i) && within(xi, xj, q, i, j, k)) {
              if (count < maxrow) rows[base + count] = j;
              count++;
            }
          }
        }
      });
      if (act) {
        cnt[i] = min(count, maxrow);
        if (count > maxrow) atomicMax(overflow, 1);
      }
    }
  }
}

// Batched binning: every replica has its own grid starting at cell_base.
__global__ void k_bin_batch(const double* __restrict__ q, int n, const int32_t* __restrict__ rid,
                            const ReplicaInfo* __restrict__ reps, int32_t* __restrict__ cell,
                            int32_t* __restrict__ count, const int32_t* guard) {
  if (off_guard(guard)) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const ReplicaInfo& R = reps[rid[i]];
  const double* b = q + 4 * (size_t)i;
  int c[3];
  for (int d = 0; d < 3; d++) c[d] = wrap_cell((int)floor(b[d] * R.inv_w[d]), R.nc[d]);
  const int id = R.cell_base + (c[2] * R.nc[1] + c[1]) * R.nc[0] + c[0];
  cell[i] = id;
  atomicAdd(count + id, 1);
}

// Batched warp-cooperative row build (full rows): as k_build_rows, with the
// cell's replica supplying the local grid and the membership constants.
__global__ void __launch_bounds__(128) k_build_rows_batch(
    const double* __restrict__ q, const ReplicaInfo* __restrict__ reps,
    const int32_t* __restrict__ cell_rid, int ncells, double sl2,
    const int64_t* __restrict__ start, const int32_t* __restrict__ order,
    const int4* __restrict__ cq, int maxrow, int32_t* __restrict__ rows,
    int32_t* __restrict__ cnt, int32_t* __restrict__ overflow, const int32_t* guard) {
  if (off_guard(guard)) return;
  const int lane = threadIdx.x & 31;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  for (int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; c < ncells; c += nwarps) {
    const ReplicaInfo& R = reps[cell_rid[c]];
    CellGrid g{};
    for (int d = 0; d < 3; d++) g.nc[d] = R.nc[d];
    g.ncells = R.nc[0] * R.nc[1] * R.nc[2];
    g.periodic = 1;
    BuildConsts k{};
    k.sl2_lo = R.sl2u_lo;
    k.sl2_hi = R.sl2u_hi;
    k.aniso = 0;
    k.periodic = 1;
    for (int d = 0; d < 3; d++) {
      k.len[d] = R.len[d];
      k.half_bits[d] = R.half_bits[d];
    }
    k.sl2 = sl2;
    const int s0 = (int)start[c], s1 = (int)start[c + 1];
    for (int a = s0; a < s1; a += 32) {
      const bool act = a + lane < s1;
      const int i = act ? order[a + lane] : -1;
      const int4 xi = act ? cq[a + lane] : make_int4(0, 0, 0, 0);
      const size_t base = act ? (size_t)i * (size_t)maxrow : 0;
      int count = 0;
      for_neighbour_cells(c - R.cell_base, g, [&](int c2l) {
        const int c2 = R.cell_base + c2l;
        const int t0 = (int)start[c2], t1 = (int)start[c2 + 1];
        for (int b = t0; b < t1; b += 32) {
          int jl = -1;
          int4 xl = make_int4(0, 0, 0, 0);
          if (b + lane < t1) {
            jl = order[b + lane];
            xl = cq[b + lane];
          }
          const int m = min(32, t1 - b);
          for (int kk = 0; kk < m; kk++) {
            const int j = __shfl_sync(kFullMask, jl, kk);
            int4 xj;
            xj.x = __shfl_sync(kFullMask, xl.x, kk);
            xj.y = __shfl_sync(kFullMask, xl.y, kk);
            xj.z = __shfl_sync(kFullMask, xl.z, kk);
            xj.w = 0;
            if (act && j != i && within(xi, xj, q, i, j, k)) {
              if (count < maxrow) rows[base + count] = j;
              count++;
            }
          }
        }
      });
      if (act) {
        cnt[i] = min(count, maxrow);
        if (count > maxrow) atomicMax(overflow, 1);
      }
    }
  }
}

// The same walk as k_build_rows (full rows), writing for every slot s a
// padded row of 16-bit local indices: nb * maxc + (slot in that cell), nb the
// walk position of the neighbour cell.  The cell-tiled gather stages the
// neighbour cells in that order and reads positions from shared memory.
__global__ void __launch_bounds__(128) k_build_rows_local(
    const double* __restrict__ q, CellGrid g, const int64_t* __restrict__ start,
    const int32_t* __restrict__ order, const int4* __restrict__ cq, BuildConsts k, int maxrow,
    int maxc_shift, uint16_t* __restrict__ rows, int32_t* __restrict__ cnt,
    int32_t* __restrict__ overflow) {
  const int lane = threadIdx.x & 31;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  for (int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; c < g.ncells; c += nwarps) {
    const int s0 = (int)start[c], s1 = (int)start[c + 1];
    for (int a = s0; a < s1; a += 32) {
      const bool act = a + lane < s1;
      const int i = act ? order[a + lane] : -1;
      const int4 xi = act ? cq[a + lane] : make_int4(0, 0, 0, 0);
      const size_t base = act ? (size_t)(a + lane) * (size_t)maxrow : 0;
      int count = 0, nb = 0;
      for_neighbour_cells(c, g, [&](int c2) {
        const int t0 = (int)start[c2], t1 = (int)start[c2 + 1];
        for (int b = t0; b < t1; b += 32) {
          int jl = -1;
          int4 xl = make_int4(0, 0, 0, 0);
          if (b + lane < t1) {
            jl = order[b + lane];
            xl = cq[b + lane];
          }
          const int m = min(32, t1 - b);
          for (int kk = 0; kk < m; kk++) {
            const int j = __shfl_sync(kFullMask, jl, kk);
            int4 xj;
            xj.x = __shfl_sync(kFullMask, xl.x, kk);
            xj.y = __shfl_sync(kFullMask, xl.y, kk);
            xj.z = __shfl_sync(kFullMask, xl.z, kk);
            xj.w = 0;
            if (act && j != i && within(xi, xj, q, i, j, k)) {
              if (count < maxrow) rows[base + count] = (uint16_t)((nb << maxc_shift) + (b + kk - t0));
              count++;
            }
          }
        }
        nb++;
      });
      if (act) {
        cnt[a + lane] = min(count, maxrow);
        if (count > maxrow) atomicMax(overflow, 1);
      }
    }
  }
}

// Compact copy of padded rows: out[off[i] + m] = rows[i * maxrow + m].
__global__ void k_compact_padded(const int32_t* __restrict__ cnt, const int32_t* __restrict__ rows,
                                 int maxrow, const int64_t* __restrict__ off, int n,
                                 int32_t* __restrict__ out, const int32_t* guard) {
  if (off_guard(guard)) return;
  const int lane = threadIdx.x & 31;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  for (int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < n; i += nwarps) {
    const int c = cnt[i];
    const size_t a = (size_t)i * (size_t)maxrow;
    const int64_t b = off[i];
    for (int m = lane; m < c; m += 32) out[b + m] = rows[a + m];
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

BuildConsts make_build_consts(const BuildArgs& a) {
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
  return k;
}


cudaError_t launch_sort_cells(const int64_t* start, int ncells, const int32_t* order,
                              const int4* cq, int32_t* order2, int4* cq2, cudaStream_t s,
                              const int32_t* guard) {
  k_sort_cells<<<grid_of((int64_t)ncells * 32, 256, 152 * 64), 256, 0, s>>>(
      start, ncells, order, cq, order2, cq2, guard);
  return cudaGetLastError();
}

cudaError_t launch_build_rows(const BuildArgs& a, bool half, int maxrow, int32_t* rows,
                              int32_t* cnt, int32_t* overflow, cudaStream_t s,
                              const int32_t* guard) {
  if (a.n == 0) return cudaSuccess;
  const BuildConsts k = make_build_consts(a);
  const int blocks = grid_of((int64_t)a.grid.ncells * 32, 128, 152 * 64);
  if (half)
    k_build_rows<true><<<blocks, 128, 0, s>>>(a.q, a.grid, a.start, a.order, a.cq, k, maxrow,
                                              rows, cnt, overflow, guard);
  else
    k_build_rows<false><<<blocks, 128, 0, s>>>(a.q, a.grid, a.start, a.order, a.cq, k, maxrow,
                                               rows, cnt, overflow, guard);
  return cudaGetLastError();
}

cudaError_t launch_build_rows_local(const BuildArgs& a, int maxrow, int maxc_shift,
                                    uint16_t* rows, int32_t* cnt, int32_t* overflow,
                                    cudaStream_t s) {
  if (a.n == 0) return cudaSuccess;
  const BuildConsts k = make_build_consts(a);
  const int blocks = grid_of((int64_t)a.grid.ncells * 32, 128, 152 * 64);
  k_build_rows_local<<<blocks, 128, 0, s>>>(a.q, a.grid, a.start, a.order, a.cq, k, maxrow,
                                            maxc_shift, rows, cnt, overflow);
  return cudaGetLastError();
}

cudaError_t launch_compact_padded(const int32_t* cnt, const int32_t* rows, int maxrow,
                                  const int64_t* off, int n, int32_t* out, cudaStream_t s,
                                  const int32_t* guard) {
  if (n > 0)
    k_compact_padded<<<grid_of((int64_t)n * 32, 256, 152 * 64), 256, 0, s>>>(
        cnt, rows, maxrow, off, n, out, guard);
  return cudaGetLastError();
}


cudaError_t launch_bin_batch(const double* q, int n, const int32_t* rid, const ReplicaInfo* reps,
                             int ncells, int32_t* cell, int32_t* count, cudaStream_t s,
                             const int32_t* guard) {
  cudaError_t e = launch_zero_i32(count, ncells, guard, s);
  if (e != cudaSuccess || n == 0) return e;
  k_bin_batch<<<grid_of(n, 256, 0), 256, 0, s>>>(q, n, rid, reps, cell, count, guard);
  return cudaGetLastError();
}

cudaError_t launch_build_rows_batch(const double* q, const ReplicaInfo* reps,
                                    const int32_t* cell_rid, int ncells, double sl2,
                                    const int64_t* start, const int32_t* order, const int4* cq,
                                    int maxrow, int32_t* rows, int32_t* cnt, int32_t* overflow,
                                    cudaStream_t s, const int32_t* guard) {
  const int blocks = grid_of((int64_t)ncells * 32, 128, 152 * 64);
  k_build_rows_batch<<<blocks, 128, 0, s>>>(q, reps, cell_rid, ncells, sl2, start, order, cq,
                                            maxrow, rows, cnt, overflow, guard);
  return cudaGetLastError();
}

}  // namespace ljg
