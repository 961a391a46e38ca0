// lj_force_split.cu -- launch of the split two-float gather (LJ_PREC_MIXED,
// kernels 2 and 4 over rows ordered near | in range | beyond): each warp step
// takes two-float, FP32 or no pair terms by its own r2.
#include "lj_force_kernels.cuh"

namespace ljg {

cudaError_t launch_mixed_ff_split(const ForceLaunch& L, const MixedConsts& K, cudaStream_t s) {
  const int n = L.csr.n;
  const int block = L.block;
  const int blocks = (int)(((long long)n * L.lanes + block - 1) / block);
  const bool pbc = L.box.on != 0, soa = L.part.soa != 0;
  auto go = [&](auto u) -> cudaError_t {
    constexpr int U = decltype(u)::value;
    return dispatch_lanes(L.lanes, [&](auto g) {
      return dispatch_bools(pbc, soa, [&](auto P, auto S) {
        constexpr int G = decltype(g)::value;
        const int4* qf = L.qfix;
        if (U == 4 && L.csr.aligned4) {
          if (L.aniso)
            return launch_dependent(
                k_gather_mixed_u<G, 4, P.value, S.value, true, true, true, true>, blocks, block,
                s, L.part, L.csr, qf, K);
          return launch_dependent(
              k_gather_mixed_u<G, 4, P.value, S.value, false, true, true, true>, blocks, block, s,
              L.part, L.csr, qf, K);
        }
        if (L.aniso)
          return launch_dependent(
              k_gather_mixed_u<G, U, P.value, S.value, true, false, true, true>, blocks, block, s,
              L.part, L.csr, qf, K);
        return launch_dependent(
            k_gather_mixed_u<G, U, P.value, S.value, false, false, true, true>, blocks, block, s,
            L.part, L.csr, qf, K);
      });
    });
  };
  switch (L.unroll) {
    case 2: return go(std::integral_constant<int, 2>{});
    case 4: return go(std::integral_constant<int, 4>{});
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace ljg
