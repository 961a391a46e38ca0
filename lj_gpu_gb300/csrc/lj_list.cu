// lj_list.cu -- device kernels that install and reshape neighbour lists.
//
//   validate   : check_loadedpair (cuda/force_cuda.cu:183-201) plus row bounds
//   scan       : exclusive prefix sum of per-row counts into int64 offsets
//   half->full : every half-list pair (i, j) lands in row i and row j; rows are
//                then rank-sorted so the full list is canonical (ascending j),
//                the order the reference's full makepair produces
//                (cuda/force_cuda.cu:133-162)
//   pairs      : (i, j) pair arrays with non-decreasing i -> CSR counts, as
//                sortpair does for makepair output (cpu_ref/force_aos.cpp:100-120)
#include "lj_internal.h"

namespace ljg {
namespace {

constexpr int kScanThreads = 512;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;

// Kernels that may sit in a captured graph take an optional guard: when it
// is non-null and *guard == 0 the kernel does nothing (fixed-shape rebuilds
// of the MD loop run only on the steps that need them).
__device__ __forceinline__ bool guarded_off(const int32_t* guard) {
  return guard && *(volatile const int32_t*)guard == 0;
}

__global__ void k_zero_i32(int32_t* p, int64_t count, const int32_t* guard) {
  if (guarded_off(guard)) return;
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < count;
       k += (int64_t)gridDim.x * blockDim.x)
    p[k] = 0;
}

__device__ __forceinline__ void report(int32_t* err, int code, int32_t index) {
  atomicMax(err + 0, code);
  atomicMin(err + 1, index);
}

__global__ void k_validate_rows(Csr c, int32_t* err) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < c.n; i += gridDim.x * blockDim.x) {
    const int32_t np = c.np[i], p = c.ptr[i];
    if (np < 0 || np >= c.n) report(err, 1, i);
    else if (p < 0 || (int64_t)p > c.entries) report(err, 2, i);
    else if ((int64_t)p + np > c.entries) report(err, 3, i);
  }
}

__global__ void k_validate_entries(Csr c, int32_t* err) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < c.entries;
       k += (int64_t)gridDim.x * blockDim.x) {
    const int32_t j = c.list[k];
    if (j < 0 || j >= c.n) report(err, 4, (int32_t)(k < 0x7fffffff ? k : 0x7fffffff));
  }
}

// block-wide inclusive scan of one int64 per thread
__device__ int64_t block_scan_incl(int64_t v, int64_t* warp_tot) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int off = 1; off < 32; off <<= 1) {
    const int64_t o = __shfl_up_sync(kFullMask, v, off);
    if (lane >= off) v += o;
  }
  if (lane == 31) warp_tot[w] = v;
  __syncthreads();
  if (w == 0) {
    const int nw = blockDim.x >> 5;
    int64_t t = lane < nw ? warp_tot[lane] : 0;
    for (int off = 1; off < 32; off <<= 1) {
      const int64_t o = __shfl_up_sync(kFullMask, t, off);
      if (lane >= off) t += o;
    }
    if (lane < nw) warp_tot[lane] = t;
  }
  __syncthreads();
  if (w > 0) v += warp_tot[w - 1];
  return v;
}

__global__ void __launch_bounds__(kScanThreads) k_scan_tiles(const int32_t* in, int n,
                                                            int64_t* tile_sum,
                                                            const int32_t* guard) {
  if (guarded_off(guard)) return;
  __shared__ int64_t wt[32];
  const int64_t base = (int64_t)blockIdx.x * kScanTile + threadIdx.x * kScanItems;
  int64_t s = 0;
  for (int k = 0; k < kScanItems; k++)
    if (base + k < n) s += in[base + k];
  s = block_scan_incl(s, wt);
  if (threadIdx.x == blockDim.x - 1) tile_sum[blockIdx.x] = s;
}

// exclusive scan of the tile sums in place (one block, serial over chunks)
__global__ void __launch_bounds__(kScanThreads) k_scan_tile_sums(int64_t* tile_sum, int nt,
                                                                const int32_t* guard) {
  if (guarded_off(guard)) return;
  __shared__ int64_t wt[32];
  __shared__ int64_t carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int base = 0; base < nt; base += kScanThreads) {
    const int idx = base + threadIdx.x;
    const int64_t v = idx < nt ? tile_sum[idx] : 0;
    const int64_t incl = block_scan_incl(v, wt);
    const int64_t c = carry;
    if (idx < nt) tile_sum[idx] = c + incl - v;
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) carry = c + incl;
    __syncthreads();
  }
}

__global__ void __launch_bounds__(kScanThreads) k_scan_apply(const int32_t* in, int n,
                                                            const int64_t* tile_off,
                                                            int64_t* out, const int32_t* guard) {
  if (guarded_off(guard)) return;
  __shared__ int64_t wt[32];
  const int64_t base = (int64_t)blockIdx.x * kScanTile + threadIdx.x * kScanItems;
  int32_t v[kScanItems];
  int64_t s = 0;
  for (int k = 0; k < kScanItems; k++) {
    v[k] = base + k < n ? in[base + k] : 0;
    s += v[k];
  }
  int64_t run = block_scan_incl(s, wt) - s + tile_off[blockIdx.x];
  for (int k = 0; k < kScanItems; k++) {
    if (base + k < n) out[base + k] = run;
    run += v[k];
  }
  if (base + kScanItems >= n && base < n) out[n] = run;  // thread holding the last item
}

__global__ void k_count_as_j(Csr half, int32_t* deg) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < half.entries;
       k += (int64_t)gridDim.x * blockDim.x)
    atomicAdd(deg + half.list[k], 1);
}

__global__ void k_fill_full(Csr half, const int64_t* off, int32_t* cursor, int32_t* out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < half.n; i += gridDim.x * blockDim.x) {
    const int32_t cnt = half.np[i], k0 = half.ptr[i];
    for (int m = 0; m < cnt; m++) {
      const int32_t j = half.list[k0 + m];
      out[off[i] + atomicAdd(cursor + i, 1)] = j;
      out[off[j] + atomicAdd(cursor + j, 1)] = i;
    }
  }
}

// one warp per row: stable rank sort, O(len^2 / 32) compares per lane
__global__ void k_sort_rows(const int64_t* off, int n, const int32_t* in, int32_t* out,
                            const int32_t* guard) {
  if (guarded_off(guard)) return;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  for (int i = warp; i < n; i += nwarps) {
    const int64_t b = off[i];
    const int len = (int)(off[i + 1] - b);
    for (int a = lane; a < len; a += 32) {
      const int32_t v = in[b + a];
      int rank = 0;
      for (int c = 0; c < len; c++) {
        const int32_t w = in[b + c];
        rank += (w < v) || (w == v && c < a);
      }
      out[b + rank] = v;
    }
  }
}

__global__ void k_offsets_to_ptr(const int64_t* off, int n, int32_t* ptr, int32_t* np,
                                 int32_t* max_row, const int32_t* guard) {
  if (guarded_off(guard)) return;
  int m = 0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    ptr[i] = (int32_t)off[i];
    const int c = (int)(off[i + 1] - off[i]);
    np[i] = c;
    m = max(m, c);
  }
  for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(kFullMask, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(max_row, m);
}

// Row lengths rounded up to a multiple of 4 (16-byte row starts).
__global__ void k_round4(const int32_t* __restrict__ np, int n, int32_t* __restrict__ out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    out[i] = (np[i] + 3) & ~3;
}

// Copies row i of (np, ptr, list) to out[off[i] ...], zero-filling up to the
// next multiple of 4; aptr[i] = off[i].
__global__ void k_copy_rows4(const int32_t* __restrict__ np, const int32_t* __restrict__ ptr,
                             const int32_t* __restrict__ list, const int64_t* __restrict__ off,
                             int n, int32_t* __restrict__ out, int32_t* __restrict__ aptr) {
  const int lane = threadIdx.x & 31;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  for (int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < n; i += nwarps) {
    const int c = np[i], cp = (c + 3) & ~3;
    const int64_t a = ptr[i], b = off[i];
    for (int m = lane; m < cp; m += 32) out[b + m] = m < c ? list[a + m] : 0;
    if (lane == 0) aptr[i] = (int32_t)b;
  }
}

__global__ void k_pairs_count(const int32_t* ip, int64_t npairs, int n, int32_t* cnt,
                              int32_t* err) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < npairs;
       k += (int64_t)gridDim.x * blockDim.x) {
    const int32_t i = ip[k];
    if (i < 0 || i >= n) {
      report(err, 4, (int32_t)(k < 0x7fffffff ? k : 0x7fffffff));
      continue;
    }
    if (k > 0 && ip[k - 1] > i) report(err, 5, (int32_t)(k < 0x7fffffff ? k : 0x7fffffff));
    atomicAdd(cnt + i, 1);
  }
}

// out[off[i] + m] = in[ptr[i] + m] for m < np[i]: a compact, contiguous CSR
__global__ void k_compact_rows(const int32_t* __restrict__ np, const int32_t* __restrict__ ptr,
                               const int32_t* __restrict__ in, const int64_t* __restrict__ off,
                               int n, int32_t* __restrict__ out) {
  const int lane = threadIdx.x & 31;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  for (int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < n; i += nwarps) {
    const int c = np[i], a = ptr[i];
    const int64_t b = off[i];
    for (int m = lane; m < c; m += 32) out[b + m] = in[a + m];
  }
}

// The reference's transposed ("ELL") list: entry k of row i at
// list[i + k * width] (cuda/force_cuda.cu:229-240).  Bounds of every row are
// checked against the array length first.
__global__ void k_ell_check(const int32_t* np, int n, int64_t width, int64_t len, int32_t* err) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int c = np[i];
    if (c < 0 || c >= n) report(err, 1, i);
    else if (c > 0 && (int64_t)i + (int64_t)(c - 1) * width >= len) report(err, 3, i);
  }
}

__global__ void k_ell_to_csr(const int32_t* np, const int32_t* ell, int n, int64_t width,
                             const int64_t* off, int32_t* out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int c = np[i];
    for (int k = 0; k < c; k++) out[off[i] + k] = ell[(int64_t)i + (int64_t)k * width];
  }
}

__global__ void k_csr_to_ell(const int32_t* np, const int32_t* ptr, const int32_t* list, int n,
                             int64_t width, int32_t* ell) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int c = np[i], a = ptr[i];
    for (int k = 0; k < c; k++) ell[(int64_t)i + (int64_t)k * width] = list[a + k];
  }
}

int grid_for(int64_t work, int block) {
  int64_t g = (work + block - 1) / block;
  if (g < 1) g = 1;
  if (g > 152 * 16) g = 152 * 16;
  return (int)g;
}

}  // namespace

cudaError_t launch_validate_csr(const Csr& c, int32_t* err, cudaStream_t s) {
  if (c.n > 0) k_validate_rows<<<grid_for(c.n, 256), 256, 0, s>>>(c, err);
  if (c.entries > 0) k_validate_entries<<<grid_for(c.entries, 256), 256, 0, s>>>(c, err);
  return cudaGetLastError();
}

size_t scan_tmp_bytes(int n) {
  const int tiles = (n + kScanTile - 1) / kScanTile;
  return sizeof(int64_t) * (size_t)(tiles > 0 ? tiles : 1);
}

cudaError_t launch_ell_check(const int32_t* np, int n, int64_t width, int64_t len, int32_t* err,
                             cudaStream_t s) {
  if (n > 0) k_ell_check<<<grid_for(n, 256), 256, 0, s>>>(np, n, width, len, err);
  return cudaGetLastError();
}

cudaError_t launch_ell_to_csr(const int32_t* np, const int32_t* ell, int n, int64_t width,
                              const int64_t* off, int32_t* out, cudaStream_t s) {
  if (n > 0) k_ell_to_csr<<<grid_for(n, 128), 128, 0, s>>>(np, ell, n, width, off, out);
  return cudaGetLastError();
}

cudaError_t launch_csr_to_ell(const int32_t* np, const int32_t* ptr, const int32_t* list, int n,
                              int64_t width, int32_t* ell, cudaStream_t s) {
  if (n > 0) k_csr_to_ell<<<grid_for(n, 128), 128, 0, s>>>(np, ptr, list, n, width, ell);
  return cudaGetLastError();
}

cudaError_t launch_zero_i32(int32_t* p, int64_t count, const int32_t* guard, cudaStream_t s) {
  if (count > 0) k_zero_i32<<<grid_for(count, 256), 256, 0, s>>>(p, count, guard);
  return cudaGetLastError();
}

cudaError_t launch_scan_counts(const int32_t* counts, int n, int64_t* out, void* tmp,
                               size_t tmp_bytes, cudaStream_t s, const int32_t* guard) {
  if (n == 0) {
    if (guard) return cudaErrorInvalidValue;  // guarded scans need n > 0
    return cudaMemsetAsync(out, 0, sizeof(int64_t), s);
  }
  const int tiles = (n + kScanTile - 1) / kScanTile;
  if (tmp_bytes < sizeof(int64_t) * (size_t)tiles) return cudaErrorInvalidValue;
  auto* ts = static_cast<int64_t*>(tmp);
  k_scan_tiles<<<tiles, kScanThreads, 0, s>>>(counts, n, ts, guard);
  k_scan_tile_sums<<<1, kScanThreads, 0, s>>>(ts, tiles, guard);
  k_scan_apply<<<tiles, kScanThreads, 0, s>>>(counts, n, ts, out, guard);
  return cudaGetLastError();
}

cudaError_t launch_full_from_half_count(const Csr& half, int32_t* deg, cudaStream_t s) {
  cudaError_t e = cudaMemcpyAsync(deg, half.np, sizeof(int32_t) * (size_t)half.n,
                                  cudaMemcpyDeviceToDevice, s);
  if (e != cudaSuccess) return e;
  if (half.entries > 0) k_count_as_j<<<grid_for(half.entries, 256), 256, 0, s>>>(half, deg);
  return cudaGetLastError();
}

cudaError_t launch_full_from_half_fill(const Csr& half, const int64_t* off, int32_t* cursor,
                                       int32_t* full_list, cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(cursor, 0, sizeof(int32_t) * (size_t)half.n, s);
  if (e != cudaSuccess) return e;
  if (half.n > 0)
    k_fill_full<<<grid_for(half.n, 128), 128, 0, s>>>(half, off, cursor, full_list);
  return cudaGetLastError();
}

cudaError_t launch_sort_rows_into(const int64_t* off, int n, const int32_t* in, int32_t* out,
                                  cudaStream_t s, const int32_t* guard) {
  if (n > 0)
    k_sort_rows<<<grid_for((int64_t)n * 32, 256), 256, 0, s>>>(off, n, in, out, guard);
  return cudaGetLastError();
}

cudaError_t launch_compact_rows(const int32_t* np, const int32_t* ptr, const int32_t* in,
                                const int64_t* off, int n, int32_t* out, cudaStream_t s) {
  if (n > 0) k_compact_rows<<<grid_for((int64_t)n * 32, 256), 256, 0, s>>>(np, ptr, in, off, n, out);
  return cudaGetLastError();
}

cudaError_t launch_round4(const int32_t* np, int n, int32_t* out, cudaStream_t s) {
  if (n > 0) k_round4<<<grid_for(n, 256), 256, 0, s>>>(np, n, out);
  return cudaGetLastError();
}

cudaError_t launch_copy_rows4(const int32_t* np, const int32_t* ptr, const int32_t* list,
                              const int64_t* off, int n, int32_t* out, int32_t* aptr,
                              cudaStream_t s) {
  if (n > 0)
    k_copy_rows4<<<grid_for((int64_t)n * 32, 256), 256, 0, s>>>(np, ptr, list, off, n, out, aptr);
  return cudaGetLastError();
}

cudaError_t launch_offsets_to_ptr(const int64_t* off, int n, int32_t* ptr, int32_t* np,
                                  int32_t* max_row, cudaStream_t s, const int32_t* guard) {
  cudaError_t e = guard ? launch_zero_i32(max_row, 1, guard, s)
                        : cudaMemsetAsync(max_row, 0, sizeof(int32_t), s);
  if (e != cudaSuccess) return e;
  if (n > 0)
    k_offsets_to_ptr<<<grid_for(n, 256), 256, 0, s>>>(off, n, ptr, np, max_row, guard);
  return cudaGetLastError();
}

cudaError_t launch_pairs_count(const int32_t* ip, int64_t npairs, int n, int32_t* cnt,
                               int32_t* err, cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(cnt, 0, sizeof(int32_t) * (size_t)n, s);
  if (e != cudaSuccess) return e;
  if (npairs > 0) k_pairs_count<<<grid_for(npairs, 256), 256, 0, s>>>(ip, npairs, n, cnt, err);
  return cudaGetLastError();
}

}  // namespace ljg
