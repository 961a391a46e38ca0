// lj_force_ff_scatter.cu -- launch of the mixed scatter with two-float pair
// terms (LJ_PREC_MIXED, half list): the scatter into the two-float4
// per-particle scratch (snapped leading parts and remainders) and the kick
// from it.  2 or 4 entries in flight per lane.
#include "lj_force_kernels.cuh"

namespace ljg {

cudaError_t launch_mixed_ff_scatter(const ForceLaunch& L, const MixedConsts& K, cudaStream_t s) {
  const int n = L.csr.n;
  const int block = L.block;
  const int blocks = (int)(((long long)n * L.lanes + block - 1) / block);
  const bool pbc = L.box.on != 0, soa = L.part.soa != 0;
  if (!L.scratch_zeroed) {
    cudaError_t e = cudaMemsetAsync(L.fscratch, 0, sizeof(float) * 8 * (size_t)n, s);
    if (e != cudaSuccess) return e;
  }
  auto go = [&](auto u) -> cudaError_t {
    constexpr int U = decltype(u)::value;
    return dispatch_lanes(L.lanes, [&](auto g) {
      return dispatch_bools(pbc, soa, [&](auto P, auto S) {
        constexpr int G = decltype(g)::value;
        float4* fa = reinterpret_cast<float4*>(L.fscratch);
        if (L.aniso)
          return launch_dependent(k_scatter_mixed_ff<G, U, P.value, S.value, true>, blocks,
                                  block, s, L.part, L.csr, L.qfix, fa, K);
        return launch_dependent(k_scatter_mixed_ff<G, U, P.value, S.value, false>, blocks, block,
                                s, L.part, L.csr, L.qfix, fa, K);
      });
    });
  };
  cudaError_t e;
  switch (L.unroll) {
    case 2: e = go(std::integral_constant<int, 2>{}); break;
    case 4: e = go(std::integral_constant<int, 4>{}); break;
    default: return cudaErrorInvalidValue;
  }
  if (e != cudaSuccess) return e;
  const int kb = (n + 255) / 256;
  const float* fs = static_cast<const float*>(L.fscratch);
  return soa ? launch_dependent(k_kick_from_scratch<true, true>, kb, 256, s, L.part, n, fs, K)
             : launch_dependent(k_kick_from_scratch<false, true>, kb, 256, s, L.part, n, fs, K);
}

}  // namespace ljg
