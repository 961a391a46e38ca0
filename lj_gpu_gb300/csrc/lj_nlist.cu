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
// candidates within a band of the search sphere (FP32 rounding plus the
// position quantum, cutoff_band) are re-decided in FP64 with the reference's
// expression (dx = q_i - q_j), so the list is the reference's list without
// spending FP64 on every candidate.  Verlet lists of the MD and batch loops
// (whose users apply the cutoff) skip that re-decision and keep every
// candidate below the upper edge of the band.
#include <algorithm>
#include <cmath>
#include <type_traits>

#include "lj_cells.cuh"
#include "lj_internal.h"
#include "lj_nlist.h"

namespace ljg {
namespace {


__device__ __forceinline__ bool off_guard(const int32_t* guard) {
  return guard && *(volatile const int32_t*)guard == 0;
}

// Grids are capped near one resident wave (152 SMs) and the kernels stride
// over their work: a guarded launch whose flag is off then costs one short
// wave of exiting blocks instead of one block per 256 particles.  The row
// builds take their cap from their own occupancy (one_wave).
constexpr int kResidentBlocks256 = 152 * 8;   // 256-thread blocks

__global__ void k_bin(const double* __restrict__ q, int n, CellGrid g, int32_t* __restrict__ cell,
                      int32_t* __restrict__ count, const int32_t* guard) {
  if (off_guard(guard)) return;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
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
}

__global__ void k_place(const int32_t* __restrict__ cell, int n, const int64_t* __restrict__ start,
                        int32_t* __restrict__ cursor, const int4* __restrict__ qfix,
                        int32_t* __restrict__ order, int4* __restrict__ cq,
                        const int32_t* guard) {
  if (off_guard(guard)) return;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int c = cell[i];
    const int slot = (int)start[c] + atomicAdd(cursor + c, 1);
    order[slot] = i;
    cq[slot] = qfix[i];
  }
}

struct BuildConsts {
  float sl2_lo, sl2_hi;  // certainly inside / possibly inside, fixed units^2
  float near2;           // ROWS_SPLIT: near part below this FP32 r2
  float u_hi[3], u_lo[3];
  int aniso;
  int periodic;
  double len[3];
  long long half_bits[3];
  double sl2;
};

// The reference's membership test (makepair: dx = q_i - q_j, r2 < SL2), FP64,
// with r2 contracted into fused multiply-adds as the reference's build does.
__device__ __forceinline__ bool within_fp64(const double* q, int i, int j, const BuildConsts& k) {
  const double* a = q + 4 * (size_t)i;
  const double* b = q + 4 * (size_t)j;
  double d[3];
  for (int x = 0; x < 3; x++) {
    d[x] = a[x] - b[x];
    if (k.periodic) d[x] = min_image_fp64(d[x], k.len[x], k.half_bits[x]);
  }
  const double r2 = fma(d[2], d[2], fma(d[0], d[0], d[1] * d[1]));
  return r2 < k.sl2;
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

// Warp-cooperative neighbour build into padded rows.  One warp per cell:
// the candidates of the 27-cell walk are flattened into one sequence (walk
// order, then slot order inside each cell) and the lanes hold 32 consecutive
// candidates, loaded with coalesced reads.  Up to 64 of the cell's own
// particles are staged in shared memory; the warp tests all 32 candidates
// against one of them per step and keeps the step's ballot for that
// particle.  After a chunk of candidates every lane appends its particles'
// hits, in candidate order, to their rows, so rows come out in walk order
// (deterministic after k_sort_cells).
//
// Membership is decided in FP32 on positions relative to the cell's first
// particle: every staged particle and candidate is converted once per chunk
// from the exact int32 fixed-point image, so a test costs three subtractions
// and three multiply-adds.  The conversion error is part of the band of the
// search sphere (make_build_consts); a candidate inside the band is
// re-decided in FP64 with the reference's expression (EXACT), or kept (the
// superset lists of the MD and batch loops, whose users apply the cutoff).
// Rows longer than their capacity are truncated and raise *overflow.
constexpr int kBuildBlock = 128;
constexpr int kBuildWarps = kBuildBlock / 32;
constexpr int kStage = 64;  // cell particles staged per candidate walk

// ROWS_SPLIT: full rows in two parts, the candidates with FP32 r2 below
// BuildConsts::near2 into rows / cnt and the others into rows2 / cnt2.
enum RowMode { ROWS_FULL = 0, ROWS_HALF = 1, ROWS_LOCAL = 2, ROWS_SPLIT = 3 };

struct BuildStage {
  float4 xr[kStage];      // position relative to the cell origin, particle index bits in w
  int4 xi[kStage];        // fixed-point image, particle index in w
  // staged particle t: x = its hits among the chunk's candidates, y (ROWS_SPLIT)
  // the near ones among them; one 8-byte store per test
  uint2 bal[kStage];
  int js[32];             // the chunk's candidates (particle index)
  int loc[32];            // and their 16-bit local indices (ROWS_LOCAL)
  int nb_start[32];       // first slot of each walk cell
  int nb_pref[32];        // candidates before it in the flattened walk
};

struct RowOut {
  int32_t* rows;     // particle-indexed rows (i * maxrow), or
  uint16_t* lrows;   // slot-indexed 16-bit local rows (ROWS_LOCAL)
  int32_t* cnt;
  int maxrow;
  int maxc_shift;    // ROWS_LOCAL: walk position << maxc_shift | slot
  int32_t* rows2;    // ROWS_SPLIT: far part (i * maxrow2), cnt2 entries
  int32_t* cnt2;
  int maxrow2;
  int32_t* overflow;
};

// Rows of the particles in cell c (see above).  EXACT: the reference's
// membership (FP64 re-decision in the band); otherwise every candidate with
// FP32 r2 < sl2_hi, a superset by at most the band.
template <int MODE, bool ANISO, bool EXACT>
__device__ __forceinline__ void build_cell_rows(int c, int cell_base, const CellGrid& g,
                                                const int64_t* __restrict__ start,
                                                const int32_t* __restrict__ order,
                                                const int4* __restrict__ cq, const double* q,
                                                const BuildConsts& k, const RowOut& out,
                                                BuildStage& ws, int lane) {
  int nnb;
  const int c2 = neighbour_cell_at(c, g, lane, &nnb);
  int st = 0, n2 = 0;
  if (c2 >= 0) {
    const int64_t a = start[cell_base + c2];
    st = (int)a;
    n2 = (int)(start[cell_base + c2 + 1] - a);
  }
  int incl = n2;
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    const int v = __shfl_up_sync(kFullMask, incl, off);
    if (lane >= off) incl += v;
  }
  const int total = __shfl_sync(kFullMask, incl, 31);
  // flattened index of the centre cell's first slot
  const int self_pref =
      __shfl_sync(kFullMask, incl - n2, __ffs(__ballot_sync(kFullMask, c2 == c)) - 1);
  if (lane < nnb) {
    ws.nb_start[lane] = st;
    ws.nb_pref[lane] = incl - n2;
  }
  const int s0 = (int)start[cell_base + c], s1 = (int)start[cell_base + c + 1];
  if (s1 <= s0) {
    __syncwarp();
    return;
  }
  // Separations: on periodic grids of fewer than five cells along an axis a
  // candidate may lie more than half a box from the cell origin, so those
  // take the minimum image of every pair from the int32 image (DIRECT);
  // elsewhere positions relative to the cell's first particle are exact
  // differences and are converted to FP32 once.
  const bool direct = g.periodic && min(g.nc[0], min(g.nc[1], g.nc[2])) <= 4;
  const int4 o = cq[s0];
  auto rel = [&](const int4& x) {
    float dx = (float)wrap_sub(x.x, o.x), dy = (float)wrap_sub(x.y, o.y),
          dz = (float)wrap_sub(x.z, o.z);
    if (ANISO) {
      dx = fmaf(dx, k.u_hi[0], dx * k.u_lo[0]);
      dy = fmaf(dy, k.u_hi[1], dy * k.u_lo[1]);
      dz = fmaf(dz, k.u_hi[2], dz * k.u_lo[2]);
    }
    return make_float3(dx, dy, dz);
  };
  // FP32 r2 of staged particle t and this lane's candidate (image xj or
  // relative position cr)
  auto pair_r2 = [&](auto direct_tag, int t, const int4& xj, const float3& cr) {
    float dx, dy, dz;
    if (decltype(direct_tag)::value) {
      const int4 x = ws.xi[t];
      dx = (float)wrap_sub(x.x, xj.x);
      dy = (float)wrap_sub(x.y, xj.y);
      dz = (float)wrap_sub(x.z, xj.z);
      if (ANISO) {
        dx = fmaf(dx, k.u_hi[0], dx * k.u_lo[0]);
        dy = fmaf(dy, k.u_hi[1], dy * k.u_lo[1]);
        dz = fmaf(dz, k.u_hi[2], dz * k.u_lo[2]);
      }
    } else {
      const float4 x = ws.xr[t];
      dx = x.x - cr.x;
      dy = x.y - cr.y;
      dz = x.z - cr.z;
    }
    return fmaf(dz, dz, fmaf(dy, dy, dx * dx));
  };
  const float inf = __int_as_float(0x7f800000);
  for (int a = s0; a < s1; a += kStage) {
    const int ni = min(kStage, s1 - a);
    // staged particles t = lane and lane + 32 belong to this lane
    auto stage = [&](int t) {
      if (t >= ni) return -1;
      const int i = order[a + t];
      const int4 x = cq[a + t];
      const float3 r = rel(x);
      ws.xr[t] = make_float4(r.x, r.y, r.z, __int_as_float(i));
      ws.xi[t] = make_int4(x.x, x.y, x.z, i);
      return i;
    };
    const int i0 = stage(lane), i1 = stage(lane + 32);
    __syncwarp();
    int len0 = 0, len1 = 0, far0 = 0, far1 = 0;
    for (int base = 0; base < total; base += 32) {
      const int gi = base + lane;
      const bool act = gi < total;
      int nb = 0;  // walk cell holding candidate gi: last nb with nb_pref[nb] <= gi
#pragma unroll
      for (int step = 16; step > 0; step >>= 1)
        if (nb + step < nnb && ws.nb_pref[nb + step] <= gi) nb += step;
      const int r = gi - ws.nb_pref[nb];
      int j = -1;
      int4 xj = make_int4(0, 0, 0, 0);
      float3 cr = make_float3(inf, inf, inf);  // an absent candidate is never a hit
      if (act) {
        j = order[ws.nb_start[nb] + r];
        xj = cq[ws.nb_start[nb] + r];
        cr = rel(xj);
      }
      ws.js[lane] = j;
      if (MODE == ROWS_LOCAL) ws.loc[lane] = (nb << out.maxc_shift) + r;
      // every staged particle against this chunk's candidates
      auto tests = [&](auto direct_tag) {
        bool band = false;  // a hit of this candidate lies in the band (EXACT)
#pragma unroll 4
        for (int t = 0; t < ni; t++) {
          float r2 = pair_r2(direct_tag, t, xj, cr);
          if (decltype(direct_tag)::value && !act) r2 = inf;
          const bool hit = (MODE != ROWS_HALF || j > ws.xi[t].w) && r2 < k.sl2_hi;
          const unsigned bal = __ballot_sync(kFullMask, hit);
          if (EXACT) band |= hit && !(r2 < k.sl2_lo);
          const unsigned nbal =
              MODE == ROWS_SPLIT ? __ballot_sync(kFullMask, r2 < k.near2) : 0u;
          if (lane == 0) ws.bal[t] = make_uint2(bal, nbal);
        }
        __syncwarp();
        if (EXACT && __any_sync(kFullMask, band)) {
          // rare: this lane's hits in the band, re-decided in FP64
          if (band) {
            for (int t = 0; t < ni; t++) {
              const float r2 = pair_r2(direct_tag, t, xj, cr);
              const int i = ws.xi[t].w;
              const bool hit = (MODE != ROWS_HALF || j > i) && r2 < k.sl2_hi;
              if (hit && !(r2 < k.sl2_lo) && !within_fp64(q, i, j, k))
                atomicAnd(&ws.bal[t].x, ~(1u << lane));
            }
          }
          __syncwarp();
        }
      };
      if (direct) tests(std::true_type{});
      else tests(std::false_type{});
      // this chunk's hits of staged particle t (particle i) onto its rows
      auto append = [&](int t, int i, int& len, int& len2) {
        const uint2 bn = ws.bal[t];
        unsigned mine = bn.x;
        if (MODE != ROWS_HALF) {  // a particle is its own candidate once
          const int d = self_pref + (a - s0) + t - base;
          if (d >= 0 && d < 32) mine &= ~(1u << d);
        }
        const unsigned nearm = bn.y;
        const size_t rb = (size_t)(MODE == ROWS_LOCAL ? a + t : i) * (size_t)out.maxrow;
        const size_t rb2 = MODE == ROWS_SPLIT ? (size_t)i * (size_t)out.maxrow2 : 0;
        // near hits, then far hits (ROWS_SPLIT), each in candidate order: two
        // branch-free loops, so lanes whose hits differ in kind do not run
        // both paths every iteration
        unsigned mn = MODE == ROWS_SPLIT ? (mine & nearm) : mine;
        while (mn) {
          const int b = __ffs(mn) - 1;
          mn &= mn - 1u;
          if (len < out.maxrow) {
            if (MODE == ROWS_LOCAL) out.lrows[rb + len] = (uint16_t)ws.loc[b];
            else out.rows[rb + len] = ws.js[b];
          }
          len++;
        }
        if (MODE == ROWS_SPLIT) {
          unsigned mf = mine & ~nearm;
          while (mf) {
            const int b = __ffs(mf) - 1;
            mf &= mf - 1u;
            if (len2 < out.maxrow2) out.rows2[rb2 + len2] = ws.js[b];
            len2++;
          }
        }
      };
      if (lane < ni) append(lane, i0, len0, far0);
      if (lane + 32 < ni) append(lane + 32, i1, len1, far1);
      __syncwarp();
    }
    auto finish = [&](int t, int i, int len, int len2) {
      out.cnt[MODE == ROWS_LOCAL ? a + t : i] = min(len, out.maxrow);
      if (MODE == ROWS_SPLIT) out.cnt2[i] = min(len2, out.maxrow2);
      if (len > out.maxrow || (MODE == ROWS_SPLIT && len2 > out.maxrow2))
        atomicMax(out.overflow, 1);
    };
    if (lane < ni) finish(lane, i0, len0, far0);
    if (lane + 32 < ni) finish(lane + 32, i1, len1, far1);
    __syncwarp();
  }
  __syncwarp();
}

template <int MODE, bool ANISO, bool EXACT>
__global__ void __launch_bounds__(kBuildBlock) k_build_rows(
    const double* __restrict__ q, CellGrid g, const int64_t* __restrict__ start,
    const int32_t* __restrict__ order, const int4* __restrict__ cq, BuildConsts k, RowOut out,
    const int32_t* guard) {
  if (off_guard(guard)) return;
  __shared__ BuildStage stage[kBuildWarps];
  const int lane = threadIdx.x & 31;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  for (int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; c < g.ncells; c += nwarps)
    build_cell_rows<MODE, ANISO, EXACT>(c, 0, g, start, order, cq, q, k, out,
                                        stage[threadIdx.x >> 5], lane);
}

// Batched binning: every replica has its own grid starting at cell_base.
__global__ void k_bin_batch(const double* __restrict__ q, int n, const int32_t* __restrict__ rid,
                            const ReplicaInfo* __restrict__ reps, int32_t* __restrict__ cell,
                            int32_t* __restrict__ count, const int32_t* guard) {
  if (off_guard(guard)) return;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const ReplicaInfo& R = reps[rid[i]];
    const double* b = q + 4 * (size_t)i;
    int c[3];
    for (int d = 0; d < 3; d++) c[d] = wrap_cell((int)floor(b[d] * R.inv_w[d]), R.nc[d]);
    const int id = R.cell_base + (c[2] * R.nc[1] + c[1]) * R.nc[0] + c[0];
    cell[i] = id;
    atomicAdd(count + id, 1);
  }
}

// Batched row build (full rows): as k_build_rows, with the cell's replica
// supplying the local grid and the membership constants.
// SPLIT: rows in a near and a far part (ROWS_SPLIT) at the replica's near2u.
template <bool SPLIT>
__global__ void __launch_bounds__(kBuildBlock) k_build_rows_batch(
    const double* __restrict__ q, const ReplicaInfo* __restrict__ reps,
    const int32_t* __restrict__ cell_rid, int ncells, double sl2,
    const int64_t* __restrict__ start, const int32_t* __restrict__ order,
    const int4* __restrict__ cq, int maxrow, int32_t* __restrict__ rows,
    int32_t* __restrict__ cnt, int32_t* __restrict__ rows2, int32_t* __restrict__ cnt2,
    int32_t* __restrict__ overflow, const int32_t* guard) {
  if (off_guard(guard)) return;
  __shared__ BuildStage stage[kBuildWarps];
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
    k.near2 = R.near2u;
    RowOut out{};
    out.rows = rows;
    out.cnt = cnt;
    out.maxrow = maxrow;
    out.rows2 = rows2;
    out.cnt2 = cnt2;
    out.maxrow2 = maxrow;
    out.overflow = overflow;
    build_cell_rows<SPLIT ? ROWS_SPLIT : ROWS_FULL, false, false>(
        c - R.cell_base, R.cell_base, g, start, order, cq, q, k, out, stage[threadIdx.x >> 5],
        lane);
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

// Blocks of `kernel` that the whole GPU holds at once with `block` threads:
// the grid of a grid-stride kernel that should run as exactly one wave (a
// partial second wave would run its blocks at low occupancy after the
// first).  Computed once per kernel instantiation (occupancy queries do not
// touch a stream, so this is safe during stream capture).
template <typename Kernel>
int one_wave(Kernel kernel, int block) {
  static const int blocks = [&] {
    int dev = 0, sms = 0, per = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
      sms = 152;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, block, 0) != cudaSuccess ||
        per < 1)
      per = 1;
    return sms * per;
  }();
  return blocks;
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
  k_bin<<<grid_of(n, 256, kResidentBlocks256), 256, 0, s>>>(q, n, g, cell, count, guard);
  return cudaGetLastError();
}

cudaError_t launch_place(const int32_t* cell, int n, const int64_t* start, int32_t* cursor,
                         int ncells, const int4* qfix, int32_t* order, int4* cq, cudaStream_t s,
                         const int32_t* guard) {
  cudaError_t e = guard ? launch_zero_i32(cursor, ncells, guard, s)
                        : cudaMemsetAsync(cursor, 0, sizeof(int32_t) * (size_t)ncells, s);
  if (e != cudaSuccess || n == 0) return e;
  k_place<<<grid_of(n, 256, kResidentBlocks256), 256, 0, s>>>(cell, n, start, cursor, qfix, order, cq, guard);
  return cudaGetLastError();
}

BuildConsts make_build_consts(const BuildArgs& a) {
  BuildConsts k{};
  const double u2 = a.aniso ? 1.0 : a.unit[0] * a.unit[0];
  const double sl2u = a.search * a.search / u2;
  // FP32 r2 from the coarse image: arithmetic band plus the separation
  // error, which is the coarse quantum plus the rounding of the positions
  // relative to the cell origin (each within two cell widths W of it: at
  // most 6 W 2^-24 on a separation, 8 W with the anisotropic scaling)
  const double umax = std::max(a.unit[0], std::max(a.unit[1], a.unit[2]));
  double wmax = 0.0;  // widest cell, in the units of sl2u
  for (int d = 0; d < 3; d++)
    wmax = std::max(wmax, (1.0 / a.grid.inv_w[d]) / (a.aniso ? 1.0 : a.unit[d]));
  const double qerr = kCoarseQuantumErr * (a.aniso ? umax : 1.0) + 8.0 * wmax * 0x1p-24;
  const double band = cutoff_band(std::sqrt(sl2u), qerr, kBandFp32);
  k.sl2_lo = (float)(sl2u * (1.0 - band));
  k.sl2_hi = (float)(sl2u * (1.0 + band));
  k.near2 = (float)(a.near * a.near / u2);
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
  k_sort_cells<<<grid_of((int64_t)ncells * 32, 256, kResidentBlocks256), 256, 0, s>>>(
      start, ncells, order, cq, order2, cq2, guard);
  return cudaGetLastError();
}

cudaError_t launch_build_rows(const BuildArgs& a, bool half, int maxrow, int32_t* rows,
                              int32_t* cnt, int32_t* overflow, cudaStream_t s,
                              const int32_t* guard) {
  if (a.n == 0) return cudaSuccess;
  const BuildConsts k = make_build_consts(a);
  RowOut out{};
  out.rows = rows;
  out.cnt = cnt;
  out.maxrow = maxrow;
  out.overflow = overflow;
  auto go = [&](auto mode, auto aniso, auto exact) {
    const auto kfn =
        k_build_rows<decltype(mode)::value, decltype(aniso)::value, decltype(exact)::value>;
    const int blocks =
        grid_of((int64_t)a.grid.ncells * 32, kBuildBlock, one_wave(kfn, kBuildBlock));
    kfn<<<blocks, kBuildBlock, 0, s>>>(a.q, a.grid, a.start, a.order, a.cq, k, out, guard);
    return cudaGetLastError();
  };
  using H = std::integral_constant<int, ROWS_HALF>;
  using F = std::integral_constant<int, ROWS_FULL>;
  using T = std::true_type;
  using N = std::false_type;
  if (a.superset) {
    if (a.aniso) return half ? go(H{}, T{}, N{}) : go(F{}, T{}, N{});
    return half ? go(H{}, N{}, N{}) : go(F{}, N{}, N{});
  }
  if (a.aniso) return half ? go(H{}, T{}, T{}) : go(F{}, T{}, T{});
  return half ? go(H{}, N{}, T{}) : go(F{}, N{}, T{});
}

cudaError_t launch_build_rows_local(const BuildArgs& a, int maxrow, int maxc_shift,
                                    uint16_t* rows, int32_t* cnt, int32_t* overflow,
                                    cudaStream_t s) {
  if (a.n == 0) return cudaSuccess;
  const BuildConsts k = make_build_consts(a);
  const int blocks = grid_of((int64_t)a.grid.ncells * 32, kBuildBlock,
                             one_wave(k_build_rows<ROWS_LOCAL, false, false>, kBuildBlock));
  RowOut out{};
  out.lrows = rows;
  out.cnt = cnt;
  out.maxrow = maxrow;
  out.maxc_shift = maxc_shift;
  out.overflow = overflow;
  // the cell-tiled kernel applies the cutoff itself; isotropic frames only
  k_build_rows<ROWS_LOCAL, false, false><<<blocks, kBuildBlock, 0, s>>>(
      a.q, a.grid, a.start, a.order, a.cq, k, out, nullptr);
  return cudaGetLastError();
}

cudaError_t launch_build_rows_split(const BuildArgs& a, int maxrow, int32_t* rows, int32_t* cnt,
                                    int maxrow2, int32_t* rows2, int32_t* cnt2,
                                    int32_t* overflow, cudaStream_t s, const int32_t* guard) {
  if (a.n == 0) return cudaSuccess;
  const BuildConsts k = make_build_consts(a);
  RowOut out{};
  out.rows = rows;
  out.cnt = cnt;
  out.maxrow = maxrow;
  out.rows2 = rows2;
  out.cnt2 = cnt2;
  out.maxrow2 = maxrow2;
  out.overflow = overflow;
  auto go = [&](auto kfn) {
    const int blocks =
        grid_of((int64_t)a.grid.ncells * 32, kBuildBlock, one_wave(kfn, kBuildBlock));
    kfn<<<blocks, kBuildBlock, 0, s>>>(a.q, a.grid, a.start, a.order, a.cq, k, out, guard);
    return cudaGetLastError();
  };
  if (a.aniso) return go(k_build_rows<ROWS_SPLIT, true, false>);
  return go(k_build_rows<ROWS_SPLIT, false, false>);
}

cudaError_t launch_compact_padded(const int32_t* cnt, const int32_t* rows, int maxrow,
                                  const int64_t* off, int n, int32_t* out, cudaStream_t s,
                                  const int32_t* guard) {
  if (n > 0)
    k_compact_padded<<<grid_of((int64_t)n * 32, 256, kResidentBlocks256), 256, 0, s>>>(
        cnt, rows, maxrow, off, n, out, guard);
  return cudaGetLastError();
}


cudaError_t launch_bin_batch(const double* q, int n, const int32_t* rid, const ReplicaInfo* reps,
                             int ncells, int32_t* cell, int32_t* count, cudaStream_t s,
                             const int32_t* guard) {
  cudaError_t e = launch_zero_i32(count, ncells, guard, s);
  if (e != cudaSuccess || n == 0) return e;
  k_bin_batch<<<grid_of(n, 256, kResidentBlocks256), 256, 0, s>>>(q, n, rid, reps, cell, count, guard);
  return cudaGetLastError();
}

cudaError_t launch_build_rows_batch(const double* q, const ReplicaInfo* reps,
                                    const int32_t* cell_rid, int ncells, double sl2,
                                    const int64_t* start, const int32_t* order, const int4* cq,
                                    int maxrow, int32_t* rows, int32_t* cnt, int32_t* rows2,
                                    int32_t* cnt2, int32_t* overflow, cudaStream_t s,
                                    const int32_t* guard) {
  auto go = [&](auto kfn) {
    const int blocks = grid_of((int64_t)ncells * 32, kBuildBlock, one_wave(kfn, kBuildBlock));
    kfn<<<blocks, kBuildBlock, 0, s>>>(q, reps, cell_rid, ncells, sl2, start, order, cq, maxrow,
                                       rows, cnt, rows2, cnt2, overflow, guard);
    return cudaGetLastError();
  };
  return rows2 ? go(k_build_rows_batch<true>) : go(k_build_rows_batch<false>);
}

}  // namespace ljg
