// lj_force_ff.cu -- launches of the mixed gathers with two-float pair terms
// (LJ_PREC_MIXED): the unrolled gather (kernel 2, and kernel 4's 16-byte
// index loads) and the simple gather (kernel 1); near-first rows go to the
// near/far split (lj_force_split.cu).  Two-float terms take 2 or 4 entries
// in flight per lane.
#include "lj_force_kernels.cuh"

namespace ljg {

cudaError_t launch_mixed_ff_gather(const ForceLaunch& L, const MixedConsts& K, cudaStream_t s) {
  const int n = L.csr.n;
  const int block = L.block;
  const int blocks = (int)(((long long)n * L.lanes + block - 1) / block);
  const bool pbc = L.box.on != 0, soa = L.part.soa != 0;
  if (L.kernel == 1) {
    return dispatch_lanes(L.lanes, [&](auto g) {
      return dispatch_bools(pbc, soa, [&](auto P, auto S) {
        constexpr int G = decltype(g)::value;
        if (L.aniso)
          k_gather_mixed<G, P.value, S.value, true, true>
              <<<blocks, block, 0, s>>>(L.part, L.csr, L.qfix, K);
        else
          k_gather_mixed<G, P.value, S.value, false, true>
              <<<blocks, block, 0, s>>>(L.part, L.csr, L.qfix, K);
        return cudaGetLastError();
      });
    });
  }
  if (L.split) return launch_mixed_ff_split(L, K, s);  // ordered rows
  auto go = [&](auto u) -> cudaError_t {
    constexpr int U = decltype(u)::value;
    return dispatch_lanes(L.lanes, [&](auto g) {
      return dispatch_bools(pbc, soa, [&](auto P, auto S) {
        constexpr int G = decltype(g)::value;
        const int4* qf = L.qfix;
        if (U == 4 && L.csr.aligned4) {
          if (L.aniso)
            return launch_dependent(k_gather_mixed_u<G, 4, P.value, S.value, true, true, true>,
                                    blocks, block, s, L.part, L.csr, qf, K);
          return launch_dependent(k_gather_mixed_u<G, 4, P.value, S.value, false, true, true>,
                                  blocks, block, s, L.part, L.csr, qf, K);
        }
        if (L.aniso)
          return launch_dependent(k_gather_mixed_u<G, U, P.value, S.value, true, false, true>,
                                  blocks, block, s, L.part, L.csr, qf, K);
        return launch_dependent(k_gather_mixed_u<G, U, P.value, S.value, false, false, true>,
                                blocks, block, s, L.part, L.csr, qf, K);
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
