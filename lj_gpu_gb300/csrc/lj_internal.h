// lj_internal.h -- declarations shared between the C-ABI layer and the CUDA
// translation units.  Not part of the public interface.
#pragma once

#include <cstdint>
#include <functional>
#include <cuda_runtime.h>

#include "lj_common.cuh"

namespace ljg {

// The persistent step loop of the MD and batch runs (lj_graph.cu): a graph
// whose one node is a WHILE node over `chunk` (captured once), run `chunks`
// times per launch from a device counter, or fewer if *stop_word turns
// nonzero.
struct LoopGraph {
  cudaGraphExec_t exec = nullptr;
  int32_t* counter = nullptr;
  int64_t kernels_per_chunk = 0;  // kernels one pass of the body launches
  LoopGraph() = default;
  LoopGraph(const LoopGraph&) = delete;
  LoopGraph& operator=(const LoopGraph&) = delete;
  ~LoopGraph() { reset(); }
  void reset();
  cudaError_t build(cudaStream_t s, int32_t* counter_word, const int32_t* stop_word,
                    const std::function<cudaError_t(cudaStream_t)>& chunk);
  cudaError_t launch(int32_t chunks, cudaStream_t s);
};

// Where q / p live and how they are laid out.
struct Particles {
  int soa;              // 0: AoS, 1: three arrays
  int stride;           // AoS record length in doubles (0 means 4; 8 for the
                        // interleaved z[N][8] = {q.xyzw, p.xyzw} layout)
  const double* q;      // AoS
  double* p;            // AoS
  const double* qx;     // SoA
  const double* qy;
  const double* qz;
  double* px;
  double* py;
  double* pz;
};

// A device CSR list.  Rows start at ptr[i], or, when ptr is null, at
// i * stride (padded rows with a 64-bit start; kernels that accept this say
// so).
struct Csr {
  int n;
  int64_t entries;
  const int32_t* np;
  const int32_t* ptr;
  const int32_t* list;
  int64_t stride;
  int aligned4;  // every row starts on a 16-byte boundary and is readable to a multiple of 4
  // optional: row i's entries start at first[i] (the far part of a
  // near-first row); its entries are then [first[i], np[i])
  const int32_t* first;
};

__device__ __forceinline__ int64_t row_start(const Csr& c, int i) {
  return c.ptr ? (int64_t)__ldg(c.ptr + i) : (int64_t)i * c.stride;
}

struct Periodic {
  int on;
  double len[3];
  double half[3];
};

// One replica of a batch (cubic periodic box).  Positions of every replica are
// normalised to the 2^32 fixed-point period of its own box, so pair kernels
// need only the per-row unit constants below.
struct ReplicaInfo {
  FixedAxis ax[3];
  double len[3];
  long long half_bits[3];
  float unit_f[3];          // length per fixed unit
  float k_hi, k_lo;         // 1 / unit^2, split in two floats
  float cl2u_lo, cl2u_hi;   // cutoff^2 in fixed units^2, -/+ the FP32 band
  float cl2f_lo, cl2f_hi;   // the same, -/+ the band of two-float pair terms
  float sl2u_lo, sl2u_hi;   // list radius^2 in fixed units^2, -/+ the FP32 band
  float near2u;             // split rows: near part below this r2 at the build (fixed units^2)
  float nearc2u;            // far entries closer than this (kFarCheck) take two-float terms
  double unit;              // length per fixed unit (FP64)
  double inv_w[3];          // cells per unit length
  int nc[3];
  int cell_base;            // first global cell of this replica
  int offset, count;        // particle range
};

// Everything one force launch needs.
struct ForceLaunch {
  Particles part;
  Csr csr;
  Periodic box;
  double dt;
  double cl2;
  int precision;   // LJ_PREC_* (LJ_PREC_MIXED: two-float pair terms)
  int method;      // LJ_METHOD_GATHER_FULL / LJ_METHOD_SCATTER_HALF (resolved)
  int lanes;       // 1..32
  int block;       // threads per block
  int kernel;      // 1: simple strided, 2: unrolled (mixed) / compacted (FP64)
  int unroll;      // entries in flight per lane (kernel 2, mixed)
  // two-float gathers over rows in two parts: csr holds the near part of
  // every row (two-float terms), far the rest (FP32 terms); see
  // k_gather_mixed_seg
  int split;
  Csr far;
  // three device words, zero between calls (k_seg_close_terms clears them),
  // and the close queue: n row slots
  int32_t* close_flag;
  int32_t* close_rows;
  // split rows: the order in which the segment gather visits them (nullptr:
  // row order); the MD loop passes the cell order of its last build
  const int32_t* rowperm;
  // mixed precision only
  int4* qfix;      // n entries, written by the fixed-image pass
  float* fscratch; // 4 n floats, one float4 per particle (scatter-half mixed only)
  // launch_fixed_image zeroes fscratch (when set) with the image, and
  // launch_force then skips its own clear; callers that write the image some
  // other way leave this 0
  int scratch_zeroed;
  FixedAxis axis[3];
  long long origin[3];  // fine-unit origin subtracted from every coordinate
  double unit[3];  // length per coarse fixed unit on each axis
  int aniso;       // axes with different units
  // Open boxes: the device frame words (kOpenFrameWords long longs written
  // by launch_open_bounds on the same stream).  When set, the kernels take
  // the fixed-point frame from them and the host frame above is the coarse
  // exponent 0 frame they rescale; no host round trip.
  const long long* open_frame;
};

// Fills axis[] / unit[] / aniso for a periodic box, or the coarse exponent 0
// frame of an open box.
void make_fixed_frame(ForceLaunch& L);
// Open box with the frame chosen on the device (launch_open_bounds into
// words): sets L.open_frame and the exponent 0 host frame the kernels rescale.
void make_device_frame(ForceLaunch& L, const long long* words);
// The open frame the device would choose for these per-axis bounds: fine
// exponent kf (coarse unit 2^(10 - kf)) and fine origins.
void host_open_frame(const double* mn, const double* mx, int* kf, long long* origin);
// An open frame chosen on the host (host_open_frame) into L.
void make_open_frame(ForceLaunch& L, int kf, const long long* origin);

// Cell-tiled full list (built with the list, see lj_nlist.cu): particles in
// cell order (order[s], cells [start[c], start[c+1])), and for every slot s a
// padded row of 16-bit local indices nb * maxc + t -- the t-th particle of
// the nb-th neighbour cell in the walk order of for_neighbour_cells.
struct TiledList {
  int n;
  int ncells;
  int gnc[3];
  int periodic;
  const int32_t* order;
  const int64_t* start;
  const uint16_t* rows;
  const int32_t* cnt;
  int maxrow;
  int maxc_shift;  // maxc = 1 << maxc_shift (>= largest cell)
};

// Position image in cell order: cq[s] = fixed(q[order[s]]).
cudaError_t launch_fixed_image_sorted(const ForceLaunch& L, const int32_t* order, int4* cq,
                                      cudaStream_t s);
// Mixed gather, one CTA per cell staging its neighbour cells in shared memory.
cudaError_t launch_force_tiled(const ForceLaunch& L, const TiledList& T, const int4* cq,
                               cudaStream_t s);

// Batched mixed gather over the rows `rows[0..nrows)` (one size class) of a
// replica batch; padded rows (C.ptr == nullptr).  `far` (two-float terms
// only): rows split into the near part c and the far part *far, with the
// close queue (close_flag: three device words, zero between launches;
// close_rows: a slot per particle) for far entries that came inside
// kFarCheck, whose terms a second pass adds before the call returns.
cudaError_t launch_force_batch(const Particles& part, const Csr& c, const int4* qfix,
                               const int32_t* rid, const ReplicaInfo* reps,
                               const int32_t* rows, int nrows, double dt, double cl2, int lanes,
                               int unroll, bool vec, bool ff, cudaStream_t s,
                               const Csr* far = nullptr, int32_t* close_flag = nullptr,
                               int32_t* close_rows = nullptr);

// Launchers (return cudaError_t of the launch)
cudaError_t launch_fixed_image(const ForceLaunch& L, cudaStream_t s);
// Near-first copy of the rows of `in` (same row starts) into `out` for the
// segment gather (L's frame), near counts into nn; L's position image must
// be current.  `guard` (optional): nothing happens while *guard == 0.
cudaError_t launch_partition_near(const ForceLaunch& L, const Csr& in, int32_t* out, int32_t* nn,
                                  const int32_t* guard, cudaStream_t s);
cudaError_t launch_force(const ForceLaunch& L, cudaStream_t s);
// Gather over the transposed full list (kernel 5): L.csr = {n, entries, np,
// nullptr, ell, stride = n}; FP64, FP32 or two-float terms by L.precision,
// unroll 2 or 4 for the mixed precisions.
cudaError_t launch_force_ell(const ForceLaunch& L, cudaStream_t s);
cudaError_t launch_force_pairs(const Particles& part, int n, const int32_t* ip,
                               const int32_t* jp, int64_t npairs, const Periodic& box,
                               double dt, double cl2, cudaStream_t s);
// Open-box frame words (kOpenFrameWords long longs): launch_open_frame_init
// once after allocating them, then launch_open_bounds before every image
// pass (it leaves the frame in the words and re-arms them).
cudaError_t launch_open_frame_init(long long* words, cudaStream_t s);
cudaError_t launch_open_bounds(const Particles& part, int n, long long* words, cudaStream_t s);

// ---- list kernels (lj_list.cu) ----
// Validation; writes into err[0] a nonzero code and err[1] the first bad
// index (the smallest is kept).
cudaError_t launch_validate_csr(const Csr& c, int32_t* err, cudaStream_t s);
// Exclusive scan of n int32 counts into out[0..n] (out[n] = total, int64).
// Transposed ("ELL") lists: entry k of row i at ell[i + k * width].
cudaError_t launch_ell_check(const int32_t* np, int n, int64_t width, int64_t len, int32_t* err,
                             cudaStream_t s);
cudaError_t launch_ell_to_csr(const int32_t* np, const int32_t* ell, int n, int64_t width,
                              const int64_t* off, int32_t* out, cudaStream_t s);
cudaError_t launch_csr_to_ell(const int32_t* np, const int32_t* ptr, const int32_t* list, int n,
                              int64_t width, int32_t* ell, cudaStream_t s);
// Kernels that take `guard` do nothing while *guard == 0 (nullptr: always run).
cudaError_t launch_zero_i32(int32_t* p, int64_t count, const int32_t* guard, cudaStream_t s);
cudaError_t launch_scan_counts(const int32_t* counts, int n, int64_t* out, void* tmp,
                               size_t tmp_bytes, cudaStream_t s,
                               const int32_t* guard = nullptr);
size_t scan_tmp_bytes(int n);
// Full list from a half list: counts, offsets, fill, per-row sort.
cudaError_t launch_full_from_half_count(const Csr& half, int32_t* deg, cudaStream_t s);
cudaError_t launch_full_from_half_fill(const Csr& half, const int64_t* off, int32_t* cursor,
                                       int32_t* full_list, cudaStream_t s);
// Rows [off[i], off[i+1]) of `in` sorted ascending (stable) into `out`.
cudaError_t launch_sort_rows_into(const int64_t* off, int n, const int32_t* in, int32_t* out,
                                  cudaStream_t s, const int32_t* guard = nullptr);
// Compact copy of CSR rows: out[off[i] + m] = in[ptr[i] + m], m < np[i].
cudaError_t launch_compact_rows(const int32_t* np, const int32_t* ptr, const int32_t* in,
                                const int64_t* off, int n, int32_t* out, cudaStream_t s);
// 16-byte-aligned copy of a CSR: rows padded with zeros to multiples of 4.
cudaError_t launch_round4(const int32_t* np, int n, int32_t* out, cudaStream_t s);
cudaError_t launch_copy_rows4(const int32_t* np, const int32_t* ptr, const int32_t* list,
                              const int64_t* off, int n, int32_t* out, int32_t* aptr,
                              cudaStream_t s);
cudaError_t launch_offsets_to_ptr(const int64_t* off, int n, int32_t* ptr, int32_t* np,
                                  int32_t* max_row, cudaStream_t s,
                                  const int32_t* guard = nullptr);
// (i, j) pairs with non-decreasing i into CSR rows: counts per i.
cudaError_t launch_pairs_count(const int32_t* ip, int64_t npairs, int n, int32_t* cnt,
                               int32_t* err, cudaStream_t s);

}  // namespace ljg
