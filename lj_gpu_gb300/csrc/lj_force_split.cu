// lj_force_split.cu -- launch of the segment gather (LJ_PREC_MIXED, kernels
// 2 and 4 over rows in a near and a far part): two-float terms for the near
// part, FP32 terms for the far part (k_gather_mixed_seg).
#include "lj_force_kernels.cuh"

namespace ljg {

cudaError_t launch_mixed_ff_split(const ForceLaunch& L, const MixedConsts& K, cudaStream_t s) {
  const int n = L.csr.n;
  const int block = L.block;
  const int blocks = (int)(((long long)n * L.lanes + block - 1) / block);
  const bool pbc = L.box.on != 0, soa = L.part.soa != 0;
  const bool vec = L.unroll == 4 && L.csr.aligned4 && L.far.aligned4;
  auto go = [&](auto u, auto v) -> cudaError_t {
    constexpr int U = decltype(u)::value;
    constexpr bool V = decltype(v)::value;
    return dispatch_lanes(L.lanes, [&](auto g) {
      return dispatch_bools(pbc, soa, [&](auto P, auto S) {
        constexpr int G = decltype(g)::value;
        cudaError_t e;
        if (L.aniso)
          e = launch_dependent(k_gather_mixed_seg<G, U, P.value, S.value, true, V>, blocks,
                               block, s, L.part, L.csr, L.far, L.qfix, K, L.close_flag,
                               L.close_rows, L.rowperm);
        else
          e = launch_dependent(k_gather_mixed_seg<G, U, P.value, S.value, false, V>, blocks,
                               block, s, L.part, L.csr, L.far, L.qfix, K, L.close_flag,
                               L.close_rows, L.rowperm);
        if (e != cudaSuccess) return e;
        // queued rows with far entries that came inside 2.0 sigma, a warp per
        // row (a no-op unless the flag is up)
        const int cb = (int)std::min<long long>(((long long)n * 32 + 255) / 256, 152 * 4);
        if (L.aniso)
          k_seg_close_terms<32, P.value, S.value, true>
              <<<cb, 256, 0, s>>>(L.part, L.far, L.qfix, K, L.close_flag, L.close_rows);
        else
          k_seg_close_terms<32, P.value, S.value, false>
              <<<cb, 256, 0, s>>>(L.part, L.far, L.qfix, K, L.close_flag, L.close_rows);
        return cudaGetLastError();
      });
    });
  };
  using T = std::true_type;
  using N = std::false_type;
  if (vec) return go(std::integral_constant<int, 4>{}, T{});
  if (L.unroll == 4) return go(std::integral_constant<int, 4>{}, N{});
  return go(std::integral_constant<int, 2>{}, N{});
}

}  // namespace ljg
