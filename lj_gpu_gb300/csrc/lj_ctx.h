// lj_ctx.h -- definition of the opaque lj_ctx and its device buffers
// (shared by the C-ABI translation units).  Not part of the public interface.
#pragma once

#include <cuda_runtime.h>

#include <memory>
#include <string>
#include <vector>

#include "lj_gb300.h"
#include "lj_internal.h"
#include "lj_nlist.h"

namespace ljg {

// Grow-only device buffer.
template <typename T>
struct DevBuf {
  T* ptr = nullptr;
  size_t cap = 0;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  ~DevBuf() { release(); }
  void release() {
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    cap = 0;
  }
  cudaError_t ensure(size_t count) {
    if (count <= cap && ptr) return cudaSuccess;
    release();
    const size_t c = count > 0 ? count : 1;
    cudaError_t e = cudaMalloc(reinterpret_cast<void**>(&ptr), c * sizeof(T));
    if (e != cudaSuccess) {
      ptr = nullptr;
      return e;
    }
    cap = c;
    return cudaSuccess;
  }
};

struct DevList {
  DevBuf<int32_t> np, ptr, list;
  int n = 0;
  int64_t entries = 0;
  int max_row = 0;
  bool valid = false;
  Csr csr() const { return Csr{n, entries, np.ptr, ptr.ptr, list.ptr, 0, 0}; }
  // copy with 16-byte row starts (rows zero-padded to multiples of 4) for the
  // vector index loads of the mixed gather; full lists only
  DevBuf<int32_t> aptr, alist;
  DevBuf<int64_t> aoff;  // n + 1 row offsets of the copy
  int64_t aentries = 0;
  bool avalid = false;
  Csr acsr() const { return Csr{n, entries, np.ptr, aptr.ptr, alist.ptr, 0, 1}; }
  // near-first copies of list and alist (k_partition_near, from the
  // positions of the first two-float gather after the list changed) with
  // their near counts; reset whenever the list changes
  DevBuf<int32_t> slist, snn, salist, sann;
  bool svalid = false, savalid = false;
  // transposed copy for the ELL gather (kernel 5): entry k of row i at
  // ell[i + k n], n x max_row words; built on first use, reset with the list
  DevBuf<int32_t> ell;
  bool evalid = false;
  Csr ecsr() const { return Csr{n, entries, np.ptr, nullptr, ell.ptr, n, 0}; }
};

struct MdState;  // lj_md.cu
void md_state_delete(MdState* m);
struct MdStateDeleter {
  void operator()(MdState* m) const { md_state_delete(m); }
};
struct BatchState;  // lj_batch.cu
void batch_state_delete(BatchState* b);
struct BatchStateDeleter {
  void operator()(BatchState* b) const { batch_state_delete(b); }
};

}  // namespace ljg

struct lj_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::string err;
  ljg::DevList half, full;
  // host copies when the list came from host memory (re-uploaded by measure)
  bool list_from_host = false;
  int32_t host_kind = LJ_LIST_HALF;
  std::vector<int32_t> h_np, h_ptr, h_list;
  // scratch
  ljg::DevBuf<int4> qfix;
  ljg::DevBuf<float> fscratch;
  // open-box frame words (kOpenFrameWords), armed once by k_open_frame_init
  ljg::DevBuf<long long> oframe;
  bool oframe_armed = false;
  // the segment gather's close-entry flag (two words, zeroed once)
  ljg::DevBuf<int32_t> closef, closeq;
  bool closef_zeroed = false;
  ljg::DevBuf<int32_t> err2;
  ljg::DevBuf<int32_t> tmp_i32a, tmp_i32b;
  ljg::DevBuf<int64_t> tmp_off;
  ljg::DevBuf<unsigned char> tmp_scan;
  ljg::DevBuf<double> mq, mp;  // device q / p for lj_measure_aos
  // neighbour build
  ljg::DevBuf<int32_t> b_cell, b_count, b_cursor, b_order, b_cnt_half;
  ljg::DevBuf<int64_t> b_start, b_off_half;
  ljg::DevBuf<int4> b_cq, b_cq2;
  ljg::DevBuf<int32_t> b_order2;
  ljg::DevBuf<unsigned long long> b_minmax;
  cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};
  // per-stage timing (lj_ctx_set_timing): event triples around force calls
  bool timing = false;
  // L2 access-policy window over the position image for mixed force calls
  // (lj_ctx_set_l2_window); the persisting-L2 limit found before the first
  // use is restored at destroy
  double l2_hit_ratio = 0.0;
  bool l2_limit_set = false;
  size_t l2_limit_prev = 0;
  std::vector<cudaEvent_t> tev;  // pool, 3 per recorded call
  size_t tev_used = 0;
  double t_ms[3] = {0, 0, 0};
  int64_t t_calls = 0;
  // cell-tiled form of the full list built by lj_list_build (kernel 3)
  struct Tiled {
    bool valid = false;
    ljg::CellGrid grid{};
    int maxrow = 0, maxc_shift = 0;
    ljg::DevBuf<uint16_t> rows;
    ljg::DevBuf<int32_t> cnt, order;
    ljg::DevBuf<int64_t> start;
    ljg::DevBuf<int4> cq;  // per-call cell-ordered position image
  } tiled;
  // autotuner (lj_autotune_aos): scratch p and the chosen shapes
  ljg::DevBuf<double> tune_p;
  ljg::DevBuf<double> tune_soa;  // q and p as six arrays (SoA candidates)
  ljg::DevBuf<double> tune_z;    // interleaved z[n][8] (z-layout candidates)
  ljg::DevBuf<unsigned char> tune_flush;  // written between timed tuner calls (> L2)
  struct Tuned {
    int precision, layout, periodic, n;  // layout: LJ_LAYOUT_*
    int64_t entries_half, entries_full;
    int method, kernel, lanes, unroll, block;
  };
  std::vector<Tuned> tuned;
  // molecular dynamics state (lj_md_run)
  std::unique_ptr<ljg::MdState, ljg::MdStateDeleter> md;
  // replica batch state (lj_batch_run)
  std::unique_ptr<ljg::BatchState, ljg::BatchStateDeleter> batch;
};

// Error reporting shared by the C-ABI translation units.
int lj_fail(lj_ctx* ctx, int code, const char* fmt, ...);
