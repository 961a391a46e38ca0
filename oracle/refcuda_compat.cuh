// refcuda_compat.cuh -- TEST INFRASTRUCTURE ONLY.
//
// Forced include (nvcc -include) when the reference's cuda/kernel.cuh is
// compiled for sm_103a.  The reference was written for pre-Volta GPUs and
// calls the implicit-mask shuffle __shfl_down (cuda/device_util.cuh:12-19),
// which CUDA no longer declares for sm_70 and later.  Its callers are
// warp-uniform reductions after the lane loops, so the full-warp
// __shfl_down_sync is the same operation.  Nothing of the reference is changed.
#pragma once

#if defined(__CUDA_ARCH__) && __CUDA_ARCH__ >= 700
template <typename T>
__device__ __forceinline__ T __shfl_down(T var, unsigned int delta) {
  return __shfl_down_sync(0xffffffffu, var, delta);
}
#endif
