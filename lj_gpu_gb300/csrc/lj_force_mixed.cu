// lj_force_mixed.cu -- launches of the mixed kernels with FP32 pair terms
// (LJ_PREC_MIXED_FP32): the unrolled and simple gathers over the full list,
// the unrolled and simple scatters over the half list with the kick from
// their per-particle scratch.
#include "lj_force_kernels.cuh"

namespace ljg {

cudaError_t launch_mixed_fp32(const ForceLaunch& L, const MixedConsts& K, cudaStream_t s) {
  const int n = L.csr.n;
  const int block = L.block;
  const int blocks = (int)(((long long)n * L.lanes + block - 1) / block);
  const bool pbc = L.box.on != 0, soa = L.part.soa != 0;
  const bool gather = L.method == LJ_METHOD_GATHER_FULL;
  auto with_unroll = [&](auto&& f) -> cudaError_t {
    switch (L.unroll) {
      case 1: return f(std::integral_constant<int, 1>{});
      case 2: return f(std::integral_constant<int, 2>{});
      case 4: return f(std::integral_constant<int, 4>{});
      case 8: return f(std::integral_constant<int, 8>{});
      default: return cudaErrorInvalidValue;
    }
  };
  if (gather && L.kernel == 2) {
    return with_unroll([&](auto u) -> cudaError_t {
      constexpr int U = decltype(u)::value;
      return dispatch_lanes(L.lanes, [&](auto g) {
        return dispatch_bools(pbc, soa, [&](auto P, auto S) {
          constexpr int G = decltype(g)::value;
          const int4* qf = L.qfix;
          if (U == 4 && L.csr.aligned4) {
            if (L.aniso)
              return launch_dependent(k_gather_mixed_u<G, 4, P.value, S.value, true, true>,
                                      blocks, block, s, L.part, L.csr, qf, K);
            return launch_dependent(k_gather_mixed_u<G, 4, P.value, S.value, false, true>,
                                    blocks, block, s, L.part, L.csr, qf, K);
          }
          if (L.aniso)
            return launch_dependent(k_gather_mixed_u<G, U, P.value, S.value, true>, blocks,
                                    block, s, L.part, L.csr, qf, K);
          return launch_dependent(k_gather_mixed_u<G, U, P.value, S.value, false>, blocks,
                                  block, s, L.part, L.csr, qf, K);
        });
      });
    });
  }
  if (!gather && !L.scratch_zeroed) {
    cudaError_t e = cudaMemsetAsync(L.fscratch, 0, sizeof(float) * 4 * (size_t)n, s);
    if (e != cudaSuccess) return e;
  }
  if (!gather && L.kernel == 2) {
    cudaError_t e = with_unroll([&](auto u) -> cudaError_t {
      constexpr int U = decltype(u)::value;
      return dispatch_lanes(L.lanes, [&](auto g) {
        return dispatch_bools(pbc, soa, [&](auto P, auto S) {
          constexpr int G = decltype(g)::value;
          float4* fa = reinterpret_cast<float4*>(L.fscratch);
          if (L.aniso)
            return launch_dependent(k_scatter_mixed_u<G, U, P.value, S.value, true>, blocks,
                                    block, s, L.part, L.csr, L.qfix, fa, K);
          return launch_dependent(k_scatter_mixed_u<G, U, P.value, S.value, false>, blocks,
                                  block, s, L.part, L.csr, L.qfix, fa, K);
        });
      });
    });
    if (e != cudaSuccess) return e;
    const int kb = (n + 255) / 256;
    const float* fs = static_cast<const float*>(L.fscratch);
    return soa ? launch_dependent(k_kick_from_scratch<true>, kb, 256, s, L.part, n, fs, K)
               : launch_dependent(k_kick_from_scratch<false>, kb, 256, s, L.part, n, fs, K);
  }
  cudaError_t e = dispatch_lanes(L.lanes, [&](auto g) {
    return dispatch_bools(pbc, soa, [&](auto P, auto S) {
      constexpr int G = decltype(g)::value;
      if (gather) {
        if (L.aniso)
          k_gather_mixed<G, P.value, S.value, true>
              <<<blocks, block, 0, s>>>(L.part, L.csr, L.qfix, K);
        else
          k_gather_mixed<G, P.value, S.value, false>
              <<<blocks, block, 0, s>>>(L.part, L.csr, L.qfix, K);
      } else {
        if (L.aniso)
          k_scatter_mixed<G, P.value, S.value, true>
              <<<blocks, block, 0, s>>>(L.part, L.csr, L.qfix, L.fscratch, K);
        else
          k_scatter_mixed<G, P.value, S.value, false>
              <<<blocks, block, 0, s>>>(L.part, L.csr, L.qfix, L.fscratch, K);
      }
      return cudaGetLastError();
    });
  });
  if (e != cudaSuccess || gather) return e;
  const int kb = (n + 255) / 256;
  if (soa) k_kick_from_scratch<true><<<kb, 256, 0, s>>>(L.part, n, L.fscratch, K);
  else k_kick_from_scratch<false><<<kb, 256, 0, s>>>(L.part, n, L.fscratch, K);
  return cudaGetLastError();
}

}  // namespace ljg
