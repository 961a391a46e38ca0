// lj_force_ell.cu -- gather over the transposed ("ELL") full list (kernel 5).
//
// Entry k of row i sits at ell[i + k n]: the layout of the reference's
// transposed list (cuda/force_cuda.cu:229-240), which its fastest K40 kernels
// read directly (force_kernel_memopt2, cuda/kernel.cuh:102-134, and
// force_kernel_unrolling2, :547-620).  One lane per row, so the index loads
// of a warp step are 32 consecutive words; the pair arithmetic is that of
// the row-major kernels with one lane per row (FP64: kernel 1; mixed: kernel
// 2 with every pair in the precision's own terms), so results are bitwise
// those of the row-major list with that shape.
#include "lj_force_kernels.cuh"

namespace ljg {

cudaError_t launch_force_ell(const ForceLaunch& L, cudaStream_t s) {
  const int n = L.csr.n;
  if (n == 0) return cudaSuccess;
  const int block = L.block;
  const int blocks = (n + block - 1) / block;
  const bool pbc = L.box.on != 0, soa = L.part.soa != 0;
  if (L.precision == LJ_PREC_FP64) {
    const Fp64Consts K = make_fp64_consts(L.box, L.dt, L.cl2);
    return dispatch_bools(pbc, soa, [&](auto P, auto S) {
      k_gather_fp64<1, P.value, S.value, true><<<blocks, block, 0, s>>>(L.part, L.csr, K);
      return cudaGetLastError();
    });
  }
  const MixedConsts K = make_mixed_consts(L);
  const bool ff = L.precision == LJ_PREC_MIXED;
  auto go = [&](auto u) -> cudaError_t {
    constexpr int U = decltype(u)::value;
    return dispatch_bools(pbc, soa, [&](auto P, auto S) {
      constexpr bool PB = P.value, SO = S.value;
      if (ff) {
        if (L.aniso)
          return launch_dependent(k_gather_mixed_u<1, U, PB, SO, true, false, true, true>, blocks,
                                  block, s, L.part, L.csr, L.qfix, K);
        return launch_dependent(k_gather_mixed_u<1, U, PB, SO, false, false, true, true>, blocks,
                                block, s, L.part, L.csr, L.qfix, K);
      }
      if (L.aniso)
        return launch_dependent(k_gather_mixed_u<1, U, PB, SO, true, false, false, true>, blocks,
                                block, s, L.part, L.csr, L.qfix, K);
      return launch_dependent(k_gather_mixed_u<1, U, PB, SO, false, false, false, true>, blocks,
                              block, s, L.part, L.csr, L.qfix, K);
    });
  };
  switch (L.unroll) {
    case 2: return go(std::integral_constant<int, 2>{});
    case 4: return go(std::integral_constant<int, 4>{});
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace ljg
