// refcuda.cu -- TEST INFRASTRUCTURE ONLY.
//
// Device code of the reference's own CUDA force kernels, compiled unmodified
// from the reference checkout (cuda/kernel.cuh, cuda/device_util.cuh; the
// include path points there) into oracle/_ref/refcuda.cubin, so the tests can
// run and time them on the same GPU beside the engine (the "reference CUDA
// comparator").  This file only instantiates the templates the reference's
// driver measures (cuda/force_cuda.cu:398-443, MEASURE_FOR_ALLTYPES with
// double3 and double4); the loader (refcuda_loader.cpp) launches them by name
// with the reference's argument list (cuda/kernel.cuh:5-13).
#include <cstdint>

#include "kernel.cuh"

#define LJ_REF_INST(K, V)                                                                   \
  template __global__ void K<V, double>(const V*, V*, const int32_t, const double,         \
                                        const double, const int32_t*, const int32_t*,      \
                                        const int32_t*);
#define LJ_REF_INST2(K) LJ_REF_INST(K, double3) LJ_REF_INST(K, double4)

// gather over the full list (cuda/force_cuda.cu:427-441)
LJ_REF_INST2(force_kernel_plain)
LJ_REF_INST2(force_kernel_memopt)
LJ_REF_INST2(force_kernel_memopt3)
LJ_REF_INST2(force_kernel_unrolling2)
LJ_REF_INST2(force_kernel_warp_unroll)
LJ_REF_INST2(force_kernel_warp_unroll2)
// scatter over the half list with FP64 atomics (cuda/force_cuda.cu:418-424)
LJ_REF_INST2(force_kernel_plain_with_aar)
LJ_REF_INST2(force_kernel_memopt3_with_aar)
LJ_REF_INST2(force_kernel_warp_unroll_with_aar)
