// lj_force_batch.cu -- launches of the replica-batch gather (FP32 or
// two-float pair terms, per-row replica constants) and of the cell-tiled
// gather (kernel 3, FP32 pair terms).
#include "lj_force_kernels.cuh"

namespace ljg {

cudaError_t launch_force_tiled(const ForceLaunch& L, const TiledList& T, const int4* cq,
                               cudaStream_t s) {
  if (T.ncells == 0 || T.n == 0) return cudaSuccess;
  const MixedConsts K = make_mixed_consts(L);
  // FP32 pair terms only (run_force sends two-float calls to kernel 2)
  if (L.aniso || L.precision != LJ_PREC_MIXED_FP32) return cudaErrorNotSupported;
  const size_t smem = sizeof(int4) * 27 * ((size_t)1 << T.maxc_shift);
  const bool pbc = L.box.on != 0, soa = L.part.soa != 0;
  auto go = [&](auto u) -> cudaError_t {
    constexpr int U = decltype(u)::value;
    return dispatch_lanes(L.lanes, [&](auto g) {
      return dispatch_bools(pbc, soa, [&](auto P, auto S) {
        constexpr int G = decltype(g)::value;
        auto kfn = k_gather_mixed_tiled<G, U, P.value, S.value>;
        if (smem > 48 * 1024) {
          cudaError_t e = cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                               (int)smem);
          if (e != cudaSuccess) return e;
        }
        kfn<<<T.ncells, kTiledThreads, smem, s>>>(L.part, T, cq, K);
        return cudaGetLastError();
      });
    });
  };
  switch (L.unroll) {
    case 2: return go(std::integral_constant<int, 2>{});
    case 4: return go(std::integral_constant<int, 4>{});
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_force_batch(const Particles& part, const Csr& c, const int4* qfix,
                               const int32_t* rid, const ReplicaInfo* reps,
                               const int32_t* rows, int nrows, double dt, double cl2, int lanes,
                               int unroll, bool vec, bool ff, cudaStream_t s, const Csr* far,
                               int32_t* close_flag, int32_t* close_rows) {
  if (far && (!ff || !close_flag || !close_rows ||
              (vec && (far->ptr || far->stride % 4 != 0))))
    return cudaErrorInvalidValue;
  if (vec && (unroll != 4 || c.ptr || c.stride % 4 != 0)) return cudaErrorInvalidValue;
  if (nrows <= 0) return cudaSuccess;
  long long cl2_bits;
  std::memcpy(&cl2_bits, &cl2, sizeof cl2_bits);
  const int block = 128;
  const int blocks = (int)(((long long)nrows * lanes + block - 1) / block);
  auto go = [&](auto u) -> cudaError_t {
    constexpr int U = decltype(u)::value;
    return dispatch_lanes(lanes, [&](auto g) {
      constexpr int G = decltype(g)::value;
      auto run = [&](auto F) {
        constexpr bool FF = decltype(F)::value;
        if (far) {  // split rows: far part in FP32 terms, near part in two-float terms
          if (U == 4 && vec)
            k_gather_mixed_batch_seg<G, 4, true><<<blocks, block, 0, s>>>(
                part, c, *far, qfix, rid, reps, rows, nrows, dt, cl2_bits, close_flag,
                close_rows);
          else
            k_gather_mixed_batch_seg<G, U, false><<<blocks, block, 0, s>>>(
                part, c, *far, qfix, rid, reps, rows, nrows, dt, cl2_bits, close_flag,
                close_rows);
          // queued rows with far entries inside kFarCheck, a warp per row (a
          // no-op unless the flag is up)
          const int cb = (int)std::min<long long>(((long long)nrows * 32 + 255) / 256, 152 * 4);
          k_batch_close_terms<32><<<cb, 256, 0, s>>>(part, *far, qfix, rid, reps, dt, cl2_bits,
                                                     close_flag, close_rows);
          return;
        }
        if (U == 4 && vec)
          k_gather_mixed_batch<G, 4, true, FF>
              <<<blocks, block, 0, s>>>(part, c, qfix, rid, reps, rows, nrows, dt, cl2_bits);
        else
          k_gather_mixed_batch<G, U, false, FF>
              <<<blocks, block, 0, s>>>(part, c, qfix, rid, reps, rows, nrows, dt, cl2_bits);
      };
      if (ff) run(std::true_type{});
      else run(std::false_type{});
      return cudaGetLastError();
    });
  };
  switch (unroll) {
    case 2: return go(std::integral_constant<int, 2>{});
    case 4: return go(std::integral_constant<int, 4>{});
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace ljg
