// lj_force_kernels.cuh -- the force kernels and their launch helpers, shared
// by the translation units that instantiate them (lj_force.cu: FP64 paths,
// images and frames; lj_force_mixed.cu: FP32 pair terms; lj_force_ff.cu,
// lj_force_split.cu and lj_force_ff_scatter.cu: two-float pair terms;
// lj_force_batch.cu: replica batches and the cell-tiled gather).  Spreading the instantiations over
// several files lets them compile in parallel.
//
// One force call is the kick p_i += sum_j df(r_ij) (q_j - q_i) with
// df = (24 r^-8 - 48 r^-14) dt for r2 <= cl2, the arithmetic of
// cpu_ref/force_aos.cpp:206-218 and cuda/kernel.cuh:22-31.
//
// Work mapping: a group of G lanes (G = 1..32, a power of two) owns one
// i-particle and strides through its CSR row; the group's partial sums are
// combined with xor shuffles (the role of warp_segment_reduce,
// cuda/device_util.cuh:12-19, generalised to sub-warp groups).
//
//   FP64 gather (full list):   row sums only, one plain RMW of p_i.
//   FP64 scatter (half list):  p_j -= f with RED.F64, p_i += row sum with one
//                              atomic per row (the _with_aar kernels).
//   mixed gather / scatter:    positions from the 42-bit fixed image, pair
//                              terms in FP32 or two-float arithmetic with
//                              compensated sums, FP64 only in the final
//                              p += F dt.
#pragma once

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <type_traits>

#include "lj_cells.cuh"
#include "lj_ff.cuh"
#include "lj_gb300.h"
#include "lj_internal.h"

namespace ljg {

// Constants of one launch, kept in registers / constant bank.
struct Fp64Consts {
  double c24, c48;  // 24 dt, 48 dt
  long long cl2_bits;
  double len[3];
  long long half_bits[3];
};

struct MixedConsts {
  float cl2_lo, cl2_hi;  // r2 (pair units) certainly inside / possibly inside
  float k_hi, k_lo;      // 1/unit^2 split in two floats (isotropic frames)
  float u_hi[3], u_lo[3];  // per-axis unit split in two floats (anisotropic)
  double fscale[3];      // kick scale per axis: unit dt (FP32 terms) or 24 unit dt
                         // (two-float terms); dt or 24 dt with anisotropic units
  int fexp;              // the kick scales by fscale * 2^fexp (device-chosen open frames)
  // open frames chosen on the device: cutoff band rebuilt per launch from
  // the frame's quantum (see cutoff_band)
  float cl2_0;           // cl2 in coarse units^2 of the kf = 10 frame
  float band_base;       // arithmetic part of the relative band
  float qerr;            // quantisation error of a separation, coarse units
  // two-float terms: the scatter's j-side sums snap the leading part of each
  // term to multiples of 2^qexp pair units, so float atomics add them exactly
  float snap;            // 1.5 * 2^(23 + qexp): (x + snap) - snap rounds x to that grid
  // near/far split of two-float gathers (k_gather_mixed_split): FP32 terms
  // beyond the split radius, with the FP32 cutoff band for those terms
  float cl2s_lo, cl2s_hi;  // r2 band of FP32 terms (pair units)
  float near2;           // r2 (pair units) below which a term is always two-float
  float near_build2;     // r2 (pair units) of the near-first ordering (k_partition_near)
  Fp64Consts f64;        // for the rare FP64 cutoff decision
  const long long* open_frame;  // device-chosen open-box frame, see frame_consts
};
namespace {

// ---------------------------------------------------------------------------
// particle access
// ---------------------------------------------------------------------------
__device__ __forceinline__ size_t rec(const Particles& P, int i) {
  return (size_t)i * (size_t)(P.stride ? P.stride : 4);
}

template <bool SOA>
__device__ __forceinline__ double3 load_q(const Particles& P, int i) {
  if (SOA) return make_double3(__ldg(P.qx + i), __ldg(P.qy + i), __ldg(P.qz + i));
  const double* b = P.q + rec(P, i);
  const double2 xy = __ldg(reinterpret_cast<const double2*>(b));
  return make_double3(xy.x, xy.y, __ldg(b + 2));
}

template <bool SOA>
__device__ __forceinline__ void add_p(const Particles& P, int i, double fx, double fy,
                                      double fz) {
  if (SOA) {
    P.px[i] += fx;
    P.py[i] += fy;
    P.pz[i] += fz;
  } else {
    double* b = P.p + rec(P, i);
    double2 xy = *reinterpret_cast<double2*>(b);
    xy.x += fx;
    xy.y += fy;
    *reinterpret_cast<double2*>(b) = xy;
    b[2] += fz;
  }
}

// p_i[axis] += v (one component; several lanes may each apply one).
template <bool SOA>
__device__ __forceinline__ void add_p_axis(const Particles& P, int i, int axis, double v) {
  double* a;
  if (SOA) a = (axis == 0 ? P.px : (axis == 1 ? P.py : P.pz)) + i;
  else a = P.p + rec(P, i) + axis;
  *a += v;
}

// Sums x, y and z over the 32 lanes of a warp with 6 FP64 adds instead of
// 15 (the FP64 pipe charges every warp instruction in full).  The halves of
// the warp split the components as the sums narrow: after the offset-16 step
// the lower half carries x and y and the upper half z, after the offset-8
// step lanes with bit 3 clear carry x and the others y.  Returns this lane's
// total: x in lanes 0-7, y in lanes 8-15, z in lanes 16-31.
__device__ __forceinline__ double warp_reduce3_fp64(double x, double y, double z, int lane) {
  const bool up = (lane & 16) != 0, b3 = (lane & 8) != 0;
  double s1 = up ? z : x, s2 = up ? 0.0 : y;
  const double o1 = up ? x : z, o2 = up ? y : 0.0;
  s1 += __shfl_xor_sync(kFullMask, o1, 16);
  s2 += __shfl_xor_sync(kFullMask, o2, 16);
  double keep = (up || !b3) ? s1 : s2;
  const double send = (up || b3) ? s1 : s2;
  keep += __shfl_xor_sync(kFullMask, send, 8);
#pragma unroll
  for (int off = 4; off > 0; off >>= 1) keep += __shfl_xor_sync(kFullMask, keep, off);
  return keep;
}

// v * 2^k exactly, by adding k to the exponent field: integer instructions
// only (FP64 issue is scarce on this part).  Zero, subnormal, inf/NaN and
// results that would leave the normal range take ldexp.
__device__ __forceinline__ double scale_pow2(double v, int k) {
  const long long b = __double_as_longlong(v);
  const int e = (int)((b >> 52) & 0x7ff);
  if (e == 0 || e == 0x7ff || e + k <= 0 || e + k >= 0x7ff) return ldexp(v, k);
  return __longlong_as_double(b + (long long)k * (1ll << 52));
}

// p_i = fma(f, s, p_i) per component: the single FP64 operation the mixed
// path spends per particle and axis (s scaled by 2^fexp when fexp != 0).
template <bool SOA>
__device__ __forceinline__ void kick_p(const Particles& P, int i, double fx, double fy,
                                       double fz, const double* s, int fexp = 0) {
  double s0 = s[0], s1 = s[1], s2 = s[2];
  if (fexp) {
    s0 = scale_pow2(s0, fexp);
    s1 = scale_pow2(s1, fexp);
    s2 = scale_pow2(s2, fexp);
  }
  if (SOA) {
    P.px[i] = fma(fx, s0, P.px[i]);
    P.py[i] = fma(fy, s1, P.py[i]);
    P.pz[i] = fma(fz, s2, P.pz[i]);
  } else {
    double* b = P.p + rec(P, i);
    double2 xy = *reinterpret_cast<double2*>(b);
    xy.x = fma(fx, s0, xy.x);
    xy.y = fma(fy, s1, xy.y);
    *reinterpret_cast<double2*>(b) = xy;
    b[2] = fma(fz, s2, b[2]);
  }
}

// A compensated FP32 sum hi + lo widened to FP64: FF keeps both parts (one
// FP64 add), otherwise hi + lo is rounded to float first.
template <bool FF>
__device__ __forceinline__ double widen_sum(float hi, float lo) {
  if (FF) return widen_f32(hi) + widen_f32(lo);
  return widen_f32(__fadd_rn(hi, lo));
}

// The kick of a gather row whose G lanes all hold the compensated sums
// (hi, lo) per axis.  With G >= 4 lanes 0, 1, 2 each apply one axis: one
// FP64 FMA instruction per warp instead of three (FP64 issue is charged per
// warp instruction, whatever the active lanes), with the same per-axis
// arithmetic as kick_p.
template <bool SOA, int G, bool FF = false>
__device__ __forceinline__ void kick_group(const Particles& P, int i, int lane, bool valid,
                                           float hx, float lx, float hy, float ly, float hz,
                                           float lz, const double* s, int fexp) {
  if (G < 4) {
    if (valid && lane == 0) kick_p<SOA>(P, i, widen_sum<FF>(hx, lx), widen_sum<FF>(hy, ly),
                                        widen_sum<FF>(hz, lz), s, fexp);
    return;
  }
  if (!valid || lane > 2) return;
  const float h = lane == 0 ? hx : (lane == 1 ? hy : hz);
  const float l = lane == 0 ? lx : (lane == 1 ? ly : lz);
  double sc = lane == 0 ? s[0] : (lane == 1 ? s[1] : s[2]);
  if (fexp) sc = scale_pow2(sc, fexp);
  double* a;
  if (SOA) a = (lane == 0 ? P.px : (lane == 1 ? P.py : P.pz)) + i;
  else a = P.p + rec(P, i) + lane;
  *a = fma(widen_sum<FF>(h, l), sc, *a);
}

template <bool SOA>
__device__ __forceinline__ void red_p(const Particles& P, int i, double fx, double fy,
                                      double fz) {
  if (SOA) {
    atomicAdd(P.px + i, fx);
    atomicAdd(P.py + i, fy);
    atomicAdd(P.pz + i, fz);
  } else {
    double* b = P.p + rec(P, i);
    atomicAdd(b + 0, fx);
    atomicAdd(b + 1, fy);
    atomicAdd(b + 2, fz);
  }
}

__device__ __forceinline__ double flip_sign(double x) {
  return __hiloint2double(__double2hiint(x) ^ (int)0x80000000, __double2loint(x));
}


// Separation q_j - q_i with the minimum image, FP64 (same expression on every
// path so FP64 and mixed kernels agree on the cutoff mask).
template <bool PBC>
__device__ __forceinline__ double3 sep_fp64(const double3& qi, const double3& qj,
                                            const Fp64Consts& k) {
  double dx = qj.x - qi.x, dy = qj.y - qi.y, dz = qj.z - qi.z;
  if (PBC) {
    dx = min_image_fp64(dx, k.len[0], k.half_bits[0]);
    dy = min_image_fp64(dy, k.len[1], k.half_bits[1]);
    dz = min_image_fp64(dz, k.len[2], k.half_bits[2]);
  }
  return make_double3(dx, dy, dz);
}

// dx^2 + dy^2 + dz^2 contracted as the reference's build contracts it
// (GCC with fused multiply-add: fma(dz, dz, fma(dx, dx, dy dy))), so the FP64
// r2 -- and with it the cutoff mask -- is bitwise the reference's, even for
// pairs within an ulp of CL2.
__device__ __forceinline__ double r2_fp64(const double3& d) {
  return fma(d.z, d.z, fma(d.x, d.x, d.y * d.y));
}

// true when the reference would skip the pair (r2 > CL2); NaN is not skipped,
// exactly as `if (r2 > CL2) continue;` behaves.
__device__ __forceinline__ bool beyond_cutoff(double r2, long long cl2_bits) {
  const long long b = dbits(r2);
  return b > cl2_bits && b <= 0x7ff0000000000000ll;
}

// df of the reference formula, with dt folded into the constants.
__device__ __forceinline__ double df_fp64(double r2, const Fp64Consts& k) {
  const double inv = rcp_fp64_in_range(r2) ? rcp_fp64(r2) : 1.0 / r2;
  const double r6 = inv * inv * inv;
  return (r6 * inv) * fma(-k.c48, r6, k.c24);
}

// Address of entry k of row i: row-major rows (CSR, or padded rows when
// C.ptr is null) at k0 + k, or with ELL the transposed ("ELL") list of the
// reference, entry k of row i at i + k C.stride (C.stride = the column
// length, cuda/force_cuda.cu:229-240).  ELL kernels run one lane per row, so
// a warp's index loads of one step are consecutive words.
template <bool ELL>
__device__ __forceinline__ int64_t entry_addr(const Csr& C, int i, int64_t k0, int k) {
  return ELL ? (int64_t)i + (int64_t)k * C.stride : k0 + k;
}

// ---------------------------------------------------------------------------
// FP64 gather over the full list
// ---------------------------------------------------------------------------
template <int G, bool PBC, bool SOA, bool ELL = false>
__global__ void __launch_bounds__(256) k_gather_fp64(const Particles P, const Csr C,
                                                     const Fp64Consts K) {
  static_assert(!ELL || G == 1, "the transposed list takes one lane per row");
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = t / G;
  const int lane = t & (G - 1);
  const bool valid = i < C.n;
  int cnt = 0;
  int64_t k0 = 0;
  double3 qi = make_double3(0, 0, 0);
  if (valid) {
    cnt = __ldg(C.np + i);
    if (!ELL) k0 = __ldg(C.ptr + i);
    qi = load_q<SOA>(P, i);
  }
  double fx = 0.0, fy = 0.0, fz = 0.0;
  for (int k = lane; k < cnt; k += G) {
    const int j = __ldg(C.list + entry_addr<ELL>(C, i, k0, k));
    const double3 d = sep_fp64<PBC>(qi, load_q<SOA>(P, j), K);
    const double r2 = r2_fp64(d);
    if (beyond_cutoff(r2, K.cl2_bits)) continue;
    const double df = df_fp64(r2, K);
    fx = fma(df, d.x, fx);
    fy = fma(df, d.y, fy);
    fz = fma(df, d.z, fz);
  }
  if (G > 1) {
    fx = group_reduce_fp64<G>(fx);
    fy = group_reduce_fp64<G>(fy);
    fz = group_reduce_fp64<G>(fz);
  }
  if (valid && lane == 0) add_p<SOA>(P, i, fx, fy, fz);
}

// ---------------------------------------------------------------------------
// FP64 scatter over the half list
// ---------------------------------------------------------------------------
template <int G, bool PBC, bool SOA>
__global__ void __launch_bounds__(256) k_scatter_fp64(const Particles P, const Csr C,
                                                      const Fp64Consts K) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = t / G;
  const int lane = t & (G - 1);
  const bool valid = i < C.n;
  int cnt = 0, k0 = 0;
  double3 qi = make_double3(0, 0, 0);
  if (valid) {
    cnt = __ldg(C.np + i);
    k0 = __ldg(C.ptr + i);
    qi = load_q<SOA>(P, i);
  }
  double fx = 0.0, fy = 0.0, fz = 0.0;
  for (int k = lane; k < cnt; k += G) {
    const int j = __ldg(C.list + k0 + k);
    const double3 d = sep_fp64<PBC>(qi, load_q<SOA>(P, j), K);
    const double r2 = r2_fp64(d);
    if (beyond_cutoff(r2, K.cl2_bits)) continue;
    const double ndf = flip_sign(df_fp64(r2, K));
    const double jx = ndf * d.x, jy = ndf * d.y, jz = ndf * d.z;
    fx -= jx;
    fy -= jy;
    fz -= jz;
    red_p<SOA>(P, j, jx, jy, jz);
  }
  if (G > 1) {
    fx = group_reduce_fp64<G>(fx);
    fy = group_reduce_fp64<G>(fy);
    fz = group_reduce_fp64<G>(fz);
  }
  if (valid && lane == 0) red_p<SOA>(P, i, fx, fy, fz);
}

// ---------------------------------------------------------------------------
// force_pair on the device: unsorted pair array, both ends by atomics
// ---------------------------------------------------------------------------
template <bool PBC>
__global__ void __launch_bounds__(256) k_pairs_fp64(const Particles P, const int32_t* ip,
                                                    const int32_t* jp, int64_t npairs,
                                                    const Fp64Consts K) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < npairs;
       k += (int64_t)gridDim.x * blockDim.x) {
    const int i = __ldg(ip + k), j = __ldg(jp + k);
    const double3 d = sep_fp64<PBC>(load_q<false>(P, i), load_q<false>(P, j), K);
    const double r2 = r2_fp64(d);
    if (beyond_cutoff(r2, K.cl2_bits)) continue;
    const double df = df_fp64(r2, K);
    const double fx = df * d.x, fy = df * d.y, fz = df * d.z;
    red_p<false>(P, i, fx, fy, fz);
    red_p<false>(P, j, flip_sign(fx), flip_sign(fy), flip_sign(fz));
  }
}

// ---------------------------------------------------------------------------
// Mixed precision
// ---------------------------------------------------------------------------

// Constants of the frame in use.  With an open box whose frame is chosen on
// the device (coarse scale 2^k, k = kf - 10), the host built them for k = 0;
// every frame-dependent one scales exactly by a power of two, and the band
// follows the quantum.
// The relative cutoff band in float (per thread: no FP64 issue).
__device__ __forceinline__ float cutoff_band_f(float rc, float q, float base) {
  return base + (3.4641016f * rc * q + 3.0f * q * q) / (rc * rc);
}

__device__ __forceinline__ MixedConsts frame_consts(const MixedConsts& K0) {
  MixedConsts K = K0;
  if (K0.open_frame) {
    const int k = (int)K0.open_frame[kOfExp] - kFineBits;
    const float cl2u = ldexpf(K0.cl2_0, 2 * k);
    const float rc = sqrtf(cl2u);
    const float band = cutoff_band_f(rc, K0.qerr, K0.band_base);
    K.cl2_lo = cl2u * (1.0f - band);
    K.cl2_hi = cl2u * (1.0f + band);
    const float band32 = cutoff_band_f(rc, (float)kCoarseQuantumErr, (float)kBandFp32);
    K.cl2s_lo = cl2u * (1.0f - band32);
    K.cl2s_hi = cl2u * (1.0f + band32);
    K.near2 = ldexpf(K0.near2, 2 * k);
    K.near_build2 = ldexpf(K0.near_build2, 2 * k);
    K.k_hi = ldexpf(K0.k_hi, 2 * k);
    K.k_lo = ldexpf(K0.k_lo, 2 * k);
    K.snap = ldexpf(K0.snap, k);
    K.fexp = -k;  // fscale is scaled where the kick reads it
  }
  return K;
}

// Coarse axes and fine origins of the frame in use (open frames from the
// device words, else the host's axes and origins).
struct ImageFrame {
  FixedAxis ax[3];
  long long org[3];
};

__device__ __forceinline__ ImageFrame image_frame(const ImageFrame& f0,
                                                  const long long* open_frame) {
  if (!open_frame) return f0;
  ImageFrame f;
  const FixedAxis a = pow2_axis((int)open_frame[kOfExp] - kFineBits);
  for (int d = 0; d < 3; d++) {
    f.ax[d] = a;
    f.org[d] = open_frame[kOfOrigin + d];
  }
  return f;
}

ImageFrame host_image_frame(const ForceLaunch& L) {
  ImageFrame f;
  for (int d = 0; d < 3; d++) {
    f.ax[d] = L.axis[d];
    f.org[d] = L.origin[d];
  }
  return f;
}

__device__ __forceinline__ int4 image_of(const double3& q, const ImageFrame& f) {
  return pack_image(to_fixed_fine(q.x, f.ax[0]) - f.org[0], to_fixed_fine(q.y, f.ax[1]) - f.org[1],
                    to_fixed_fine(q.z, f.ax[2]) - f.org[2]);
}

template <bool SOA>
__global__ void __launch_bounds__(256) k_fixed_image(const Particles P, int n,
                                                     const ImageFrame f0,
                                                     const long long* open_frame,
                                                     int4* __restrict__ out,
                                                     float4* __restrict__ zero_acc, int acc_len) {
  // the pair kernel that follows may launch now (it waits for this grid)
  asm volatile("griddepcontrol.launch_dependents;");
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const ImageFrame f = image_frame(f0, open_frame);
  out[i] = image_of(load_q<SOA>(P, i), f);
  // the mixed scatter's force accumulators (acc_len float4 per particle),
  // cleared here instead of by a separate memset launch
  for (int k = 0; k < acc_len; k++)
    zero_acc[(size_t)acc_len * i + k] = make_float4(0.f, 0.f, 0.f, 0.f);
}

// Open-box frame on the device: per-axis min / max of the coordinates into
// the frame words, and in the last block to finish, the frame itself (fine
// exponent from the largest extent and |coordinate|, origin = trunc(min 2^kf)).
// The last block re-arms the keys and the block counter for the next call,
// so the words need initialising once (k_open_frame_init).
__host__ __device__ __forceinline__ void open_frame_from_bounds(const double* mn, const double* mx,
                                                                long long* kf_out,
                                                                long long* origin) {
  double amax = 0.0, ext = 0.0;
  for (int d = 0; d < 3; d++) {
    const double a = fabs(mn[d]) > fabs(mx[d]) ? fabs(mn[d]) : fabs(mx[d]);
    if (!(a <= amax)) amax = a;
    const double e = mx[d] - mn[d];
    if (!(e <= ext)) ext = e;
  }
  unsigned long long ab, eb;
  memcpy(&ab, &amax, sizeof ab);
  memcpy(&eb, &ext, sizeof eb);
  const int kf = open_frame_kf(ab, eb);
  *kf_out = kf;
  for (int d = 0; d < 3; d++) {
    const double o = trunc(ldexp(mn[d], kf));
    origin[d] = (o == o && fabs(o) < 9.0e18) ? (long long)o : 0;
  }
}

__global__ void k_open_frame_init(unsigned long long* w) {
  const int t = threadIdx.x;
  if (t < 3) {
    w[kOfMin + t] = ~0ull;
    w[kOfMax + t] = 0ull;
  }
  if (t == 0) w[kOfDone] = 0ull;
}

template <bool SOA>
__global__ void __launch_bounds__(256) k_open_bounds(const Particles P, int n,
                                                     unsigned long long* w) {
  unsigned long long mn[3] = {~0ull, ~0ull, ~0ull}, mx[3] = {0ull, 0ull, 0ull};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double3 q = load_q<SOA>(P, i);
    const unsigned long long k[3] = {order_key((unsigned long long)dbits(q.x)),
                                     order_key((unsigned long long)dbits(q.y)),
                                     order_key((unsigned long long)dbits(q.z))};
    for (int d = 0; d < 3; d++) {
      mn[d] = min(mn[d], k[d]);
      mx[d] = max(mx[d], k[d]);
    }
  }
  for (int d = 0; d < 3; d++)
    for (int off = 16; off > 0; off >>= 1) {
      mn[d] = min(mn[d], __shfl_xor_sync(kFullMask, mn[d], off));
      mx[d] = max(mx[d], __shfl_xor_sync(kFullMask, mx[d], off));
    }
  if ((threadIdx.x & 31) == 0)
    for (int d = 0; d < 3; d++) {
      atomicMin(w + kOfMin + d, mn[d]);
      atomicMax(w + kOfMax + d, mx[d]);
    }
  __threadfence();
  __syncthreads();
  __shared__ bool last;
  if (threadIdx.x == 0) last = atomicAdd(w + kOfDone, 1ull) == gridDim.x - 1;
  __syncthreads();
  if (!last || threadIdx.x != 0) return;
  __threadfence();
  volatile unsigned long long* vw = w;
  double lo[3], hi[3];
  for (int d = 0; d < 3; d++) {
    lo[d] = __longlong_as_double((long long)order_unkey(vw[kOfMin + d]));
    hi[d] = __longlong_as_double((long long)order_unkey(vw[kOfMax + d]));
  }
  long long kf, org[3];
  open_frame_from_bounds(lo, hi, &kf, org);
  long long* f = reinterpret_cast<long long*>(w);
  f[kOfExp] = kf;
  for (int d = 0; d < 3; d++) f[kOfOrigin + d] = org[d];
  for (int d = 0; d < 3; d++) {
    vw[kOfMin + d] = ~0ull;
    vw[kOfMax + d] = 0ull;
  }
  vw[kOfDone] = 0ull;
}

// Separation in pair units: fixed units (isotropic frame) or length
// (anisotropic frame, unit applied per axis as a two-float product).
template <bool ANISO>
__device__ __forceinline__ float3 sep_mixed(const int4& a, const int4& b,
                                            const MixedConsts& k) {
  float dx = (float)wrap_sub(b.x, a.x);
  float dy = (float)wrap_sub(b.y, a.y);
  float dz = (float)wrap_sub(b.z, a.z);
  if (ANISO) {
    dx = fmaf(dx, k.u_hi[0], dx * k.u_lo[0]);
    dy = fmaf(dy, k.u_hi[1], dy * k.u_lo[1]);
    dz = fmaf(dz, k.u_hi[2], dz * k.u_lo[2]);
  }
  return make_float3(dx, dy, dz);
}

// Pair inside the cutoff?  Decided in FP32 away from the cutoff surface; for
// the few pairs within a relative 4e-6 of it, recomputed in FP64 from the
// FP64 positions with the FP64 kernels' expression, so the mixed mask is the
// FP64 mask.
template <bool PBC, bool SOA>
__device__ __forceinline__ bool inside_mixed(float r2, const Particles& P, int i, int j,
                                             const MixedConsts& k) {
  if (r2 <= k.cl2_lo) return true;
  if (!(r2 <= k.cl2_hi)) return false;
  const double3 d = sep_fp64<PBC>(load_q<SOA>(P, i), load_q<SOA>(P, j), k.f64);
  return !beyond_cutoff(r2_fp64(d), k.f64.cl2_bits);
}

// df / dt in pair units (24 r^-8 - 48 r^-14, r^-2 rescaled by 1/unit^2)
template <bool ANISO>
__device__ __forceinline__ float df_mixed(float r2, const MixedConsts& k) {
  float inv;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(inv) : "f"(r2));
  inv = fmaf(inv, fmaf(-r2, inv, 1.0f), inv);
  if (!ANISO) inv = fmaf(inv, k.k_hi, inv * k.k_lo);
  const float r6 = inv * inv * inv;
  return (r6 * inv) * fmaf(-48.0f, r6, 24.0f);
}

// Row sums of a mixed kernel: Kahan-compensated FP32 sums of FP32 pair terms,
// or (FF) two-float pair terms through AccFF.
template <bool FF>
struct RowSums;

template <>
struct RowSums<false> {
  KahanF x, y, z;
  __device__ __forceinline__ void init() {
    x.init();
    y.init();
    z.init();
  }
  __device__ __forceinline__ void get(float& hx, float& lx, float& hy, float& ly, float& hz,
                                      float& lz) const {
    hx = x.s, lx = -x.c, hy = y.s, ly = -y.c, hz = z.s, lz = -z.c;
  }
};

template <>
struct RowSums<true> {
  AccFF x, y, z;
  __device__ __forceinline__ void init() {
    x.init();
    y.init();
    z.init();
  }
  __device__ __forceinline__ void get(float& hx, float& lx, float& hy, float& ly, float& hz,
                                      float& lz) const {
    x.get(hx, lx);
    y.get(hy, ly);
    z.get(hz, lz);
  }
};

// The two-float pair term of i (image xi, low fields li) and j (image xj)
// added to the row sums when the pair is inside the cutoff.  in_mode 0
// decides from r2 (setting bit u of border inside the band), 1 and 2 force
// the pair in or out (the FP64 re-decision).  Returns r2 in pair units.
template <bool ANISO>
__device__ __forceinline__ float pair_term_ff(const int4& xi, const int (&li)[3], const int4& xj,
                                              const MixedConsts& K, RowSums<true>& acc,
                                              int in_mode, bool ok, unsigned& border, int u) {
  float a[3], b[3], S, s;
  pair_sep_ff<ANISO>(xi, li[0], li[1], li[2], xj, K.u_hi, K.u_lo, a, b, S, s);
  bool in;
  if (in_mode == 0) {
    in = ok && S <= K.cl2_lo;
    if (ok && S > K.cl2_lo && S <= K.cl2_hi) border |= 1u << u;
  } else {
    in = in_mode == 1;
  }
  ff g = pair_g_ff<ANISO>(S, s, K.k_hi, K.k_lo);
  if (!in) g = ff{0.f, 0.f};
  acc.x.add(g, a[0], b[0]);
  acc.y.add(g, a[1], b[1]);
  acc.z.add(g, a[2], b[2]);
  return S;
}

// pair_term_ff (in_mode 0) of two pairs, (i, j0) at slot u and (i, j1) at
// slot u + 1, with packed instructions (lj_ff.cuh): each row sum receives the
// term of u and then that of u + 1, bit for bit as two pair_term_ff calls.
template <bool ANISO>
__device__ __forceinline__ void pair_term_ff2(const int4& xi, const int (&li)[3], const int4& xj0,
                                              const int4& xj1, const MixedConsts& K,
                                              RowSums<true>& acc, bool ok0, bool ok1,
                                              unsigned& border, int u) {
  f2 a[3], b[3], S, s;
  pair_sep_ff2<ANISO>(xi, li[0], li[1], li[2], xj0, xj1, K.u_hi, K.u_lo, a, b, S, s);
  float S0, S1;
  f2_unpack(S, S0, S1);
  const bool in0 = ok0 && S0 <= K.cl2_lo, in1 = ok1 && S1 <= K.cl2_lo;
  if (ok0 && S0 > K.cl2_lo && S0 <= K.cl2_hi) border |= 1u << u;
  if (ok1 && S1 > K.cl2_lo && S1 <= K.cl2_hi) border |= 2u << u;
  ff2 g = pair_g_ff2<ANISO>(S, s, K.k_hi, K.k_lo);
  float gh0, gh1, gl0, gl1;
  f2_unpack(g.h, gh0, gh1);
  f2_unpack(g.l, gl0, gl1);
  if (!in0) gh0 = gl0 = 0.f;
  if (!in1) gh1 = gl1 = 0.f;
  g = ff2{f2_pack(gh0, gh1), f2_pack(gl0, gl1)};
  AccFF* axes[3] = {&acc.x, &acc.y, &acc.z};
#pragma unroll
  for (int d = 0; d < 3; d++) {
    f2 p, e;
    term_parts2(g, a[d], b[d], p, e);
    float p0, p1, e0, e1;
    f2_unpack(p, p0, p1);
    f2_unpack(e, e0, e1);
    axes[d]->add_parts(p0, e0);
    axes[d]->add_parts(p1, e1);
  }
}

// The two-float terms (in_mode 0) of the U slots of one step, two at a time
// with packed instructions (PK, U even) or one at a time.
template <bool ANISO, bool PK, int U>
__device__ __forceinline__ void step_terms_ff(const int4& xi, const int (&li)[3],
                                              const int4 (&xj)[U], const bool (&ok)[U],
                                              const MixedConsts& K, RowSums<true>& acc,
                                              unsigned& border) {
  static_assert(!PK || U % 2 == 0, "packed terms go in pairs");
  if constexpr (PK) {
#pragma unroll
    for (int u = 0; u < U; u += 2)
      pair_term_ff2<ANISO>(xi, li, xj[u], xj[u + 1], K, acc, ok[u], ok[u + 1], border, u);
  } else {
#pragma unroll
    for (int u = 0; u < U; u++) pair_term_ff<ANISO>(xi, li, xj[u], K, acc, 0, ok[u], border, u);
  }
}

template <int G, bool PBC, bool SOA, bool ANISO, bool FF = false>
__global__ void __launch_bounds__(256) k_gather_mixed(const Particles P, const Csr C,
                                                      const int4* __restrict__ qfix,
                                                      const MixedConsts K0) {
  // a periodic frame is fixed on the host; an open one may come from the device
  const MixedConsts K = PBC ? K0 : frame_consts(K0);
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = t / G;
  const int lane = t & (G - 1);
  const bool valid = i < C.n;
  int cnt = 0, k0 = 0;
  int4 xi = make_int4(0, 0, 0, 0);
  if (valid) {
    cnt = __ldg(C.np + i);
    k0 = __ldg(C.ptr + i);
    xi = __ldg(qfix + i);
  }
  int li[3];
  image_lo(xi.w, li[0], li[1], li[2]);
  RowSums<FF> acc;
  acc.init();
  for (int k = lane; k < cnt; k += G) {
    const int j = __ldg(C.list + k0 + k);
    const int4 xj = __ldg(qfix + j);
    if constexpr (FF) {
      unsigned border = 0u;
      const float r2 = pair_term_ff<ANISO>(xi, li, xj, K, acc, 0, true, border, 0);
      if (border && inside_mixed<PBC, SOA>(r2, P, i, j, K))
        pair_term_ff<ANISO>(xi, li, xj, K, acc, 1, true, border, 0);
    } else {
      const float3 d = sep_mixed<ANISO>(xi, xj, K);
      const float r2 = fmaf(d.z, d.z, fmaf(d.y, d.y, d.x * d.x));
      if (!inside_mixed<PBC, SOA>(r2, P, i, j, K)) continue;
      const float df = df_mixed<ANISO>(r2, K);
      acc.x.add(df * d.x);
      acc.y.add(df * d.y);
      acc.z.add(df * d.z);
    }
  }
  float hx, lx, hy, ly, hz, lz;
  acc.get(hx, lx, hy, ly, hz, lz);
  if (G > 1) {
    group_reduce_comp<G>(hx, lx);
    group_reduce_comp<G>(hy, ly);
    group_reduce_comp<G>(hz, lz);
  }
  kick_group<SOA, G, FF>(P, i, lane, valid, hx, lx, hy, ly, hz, lz, K.fscale, K.fexp);
}

// Unrolled mixed gather (kernel 2).  The row loop runs to the longest row of
// the warp, so every lane takes part in every iteration (no divergence, warp
// votes are safe); each lane issues U independent index loads and U position
// gathers before any arithmetic, which keeps U x 32 gathers in flight per
// warp; the next step's indices load while this step's positions are in
// flight, so the index -> position chain is exposed once per row, not once
// per step.  Pairs outside the cutoff are masked with a select, not a branch.  The
// U terms of one step are summed in FP32 and the step sum enters the Kahan
// accumulator, so compensation costs 12/U operations per pair.  FF: every
// term is a two-float pair term (lj_ff.cuh) entering the compensated sums on
// its own.
// Accepts padded rows (C.ptr == nullptr, row i at i * C.stride).  VEC
// (U == 4, rows on 16-byte boundaries and readable to a multiple of 4): lane
// l of a row takes the 4 consecutive entries base + 4 l .. + 3 with one
// 16-byte load, which quarters the index-load instructions and the L1
// wavefronts they cost (a 32-lane scalar index load touches one line per row).
// ELL (G = 1): the transposed list (entry_addr).
template <int G, int U, bool PBC, bool SOA, bool ANISO, bool VEC = false, bool FF = false,
          bool ELL = false, bool PK = (FF && !ELL && U % 2 == 0)>
__global__ void __launch_bounds__(256) k_gather_mixed_u(const Particles P, const Csr C,
                                                        const int4* __restrict__ qfix,
                                                        const MixedConsts K0) {
  static_assert(!VEC || U == 4, "vector index loads take 4 entries per lane");
  static_assert(!ELL || (G == 1 && !VEC), "the transposed list takes one lane per row");
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = t / G;
  const int lane = t & (G - 1);
  // Launched as a programmatic dependent of the image pass: nothing the
  // stream wrote before may be read until the preceding grid has finished.
  asm volatile("griddepcontrol.wait;" ::: "memory");
  // a periodic frame is fixed on the host; an open one may come from the device
  const MixedConsts K = PBC ? K0 : frame_consts(K0);
  const bool valid = i < C.n;
  int cnt = 0;
  int64_t k0 = 0;
  int4 xi = make_int4(0, 0, 0, 0);
  if (valid) {
    cnt = __ldg(C.np + i);
    if (!ELL) k0 = row_start(C, i);
    xi = __ldg(qfix + i);
  }
  int cmax = cnt;
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) cmax = max(cmax, __shfl_xor_sync(kFullMask, cmax, off));
  int li[3];
  image_lo(xi.w, li[0], li[1], li[2]);
  RowSums<FF> acc;
  acc.init();
  // entry of step `base` taken by (lane, u)
  auto entry = [&](int base, int u) { return VEC ? base + 4 * lane + u : base + lane + u * G; };
  auto load_idx = [&](int base, int* jn) {
    if (VEC) {
      int4 v = make_int4(0, 0, 0, 0);
      if (entry(base, 0) < cnt)
        v = __ldg(reinterpret_cast<const int4*>(C.list + k0 + entry(base, 0)));
      jn[0] = v.x;
      jn[1] = v.y;
      jn[2] = v.z;
      jn[3] = v.w;
    } else {
#pragma unroll
      for (int u = 0; u < U; u++)
        jn[u] = entry(base, u) < cnt
                    ? __ldg(C.list + entry_addr<ELL>(C, i, k0, entry(base, u)))
                    : 0;
    }
  };
  int jn[U];
  load_idx(0, jn);
  for (int base = 0; base < cmax; base += G * U) {
    int jj[U];
    bool ok[U];
#pragma unroll
    for (int u = 0; u < U; u++) {
      ok[u] = entry(base, u) < cnt;
      jj[u] = ok[u] ? jn[u] : 0;
    }
    int4 xj[U];
#pragma unroll
    for (int u = 0; u < U; u++) xj[u] = __ldg(qfix + jj[u]);
    load_idx(base + G * U, jn);
    unsigned border = 0u;
    if constexpr (FF) {
#pragma unroll
      step_terms_ff<ANISO, PK, U>(xi, li, xj, ok, K, acc, border);
      if (__any_sync(kFullMask, border != 0u)) {
#pragma unroll
        for (int u = 0; u < U; u++) {
          if (!(border & (1u << u))) continue;
          const double3 d64 = sep_fp64<PBC>(load_q<SOA>(P, i), load_q<SOA>(P, jj[u]), K.f64);
          if (beyond_cutoff(r2_fp64(d64), K.f64.cl2_bits)) continue;
          pair_term_ff<ANISO>(xi, li, xj[u], K, acc, 1, true, border, u);
        }
      }
    } else {
      float sx = 0.f, sy = 0.f, sz = 0.f;
#pragma unroll
      for (int u = 0; u < U; u++) {
        const float3 d = sep_mixed<ANISO>(xi, xj[u], K);
        const float r2 = fmaf(d.z, d.z, fmaf(d.y, d.y, d.x * d.x));
        const bool in = ok[u] && r2 <= K.cl2_lo;
        if (ok[u] && r2 > K.cl2_lo && r2 <= K.cl2_hi) border |= 1u << u;
        float df = df_mixed<ANISO>(r2, K);
        df = in ? df : 0.0f;
        sx = fmaf(df, d.x, sx);
        sy = fmaf(df, d.y, sy);
        sz = fmaf(df, d.z, sz);
      }
      if (__any_sync(kFullMask, border != 0u)) {
#pragma unroll
        for (int u = 0; u < U; u++) {
          if (!(border & (1u << u))) continue;
          const double3 d64 = sep_fp64<PBC>(load_q<SOA>(P, i), load_q<SOA>(P, jj[u]), K.f64);
          if (beyond_cutoff(r2_fp64(d64), K.f64.cl2_bits)) continue;
          const float3 d = sep_mixed<ANISO>(xi, xj[u], K);
          const float r2 = fmaf(d.z, d.z, fmaf(d.y, d.y, d.x * d.x));
          const float df = df_mixed<ANISO>(r2, K);
          sx = fmaf(df, d.x, sx);
          sy = fmaf(df, d.y, sy);
          sz = fmaf(df, d.z, sz);
        }
      }
      acc.x.add(sx);
      acc.y.add(sy);
      acc.z.add(sz);
    }
  }
  float hx, lx, hy, ly, hz, lz;
  acc.get(hx, lx, hy, ly, hz, lz);
  if (G > 1) {
    group_reduce_comp<G>(hx, lx);
    group_reduce_comp<G>(hy, ly);
    group_reduce_comp<G>(hz, lz);
  }
  kick_group<SOA, G, FF>(P, i, lane, valid, hx, lx, hy, ly, hz, lz, K.fscale, K.fexp);
}

// Orders every row near-first for the segment gather: the entries with FP32
// r2 (coarse image) below K.near_build2 first, in list order, the others
// after them in reverse list order; nn[i] receives the near count.  Rows
// keep their starts (out has the layout of C).  One warp per row, rows in a
// grid-stride loop.
template <bool PBC, bool ANISO>
__global__ void __launch_bounds__(128) k_partition_near(const Csr C, const int4* __restrict__ qfix,
                                                        const MixedConsts K0,
                                                        int32_t* __restrict__ out,
                                                        int32_t* __restrict__ nn,
                                                        const int32_t* guard) {
  if (guard && *(volatile const int32_t*)guard == 0) return;
  const MixedConsts K = PBC ? K0 : frame_consts(K0);
  const int lane = threadIdx.x & 31;
  const unsigned lt = (1u << lane) - 1u;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  for (int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < C.n; i += nwarps) {
    const int cnt = __ldg(C.np + i);
    const int64_t k0 = row_start(C, i);
    const int4 xi = __ldg(qfix + i);
    int nacc = 0, facc = 0;
    for (int base = 0; base < cnt; base += 32) {
      const int k = base + lane;
      const bool ok = k < cnt;
      int j = 0;
      bool near = false;
      if (ok) {
        j = __ldg(C.list + k0 + k);
        const float3 d = sep_mixed<ANISO>(xi, __ldg(qfix + j), K);
        near = fmaf(d.z, d.z, fmaf(d.y, d.y, d.x * d.x)) < K.near_build2;
      }
      const unsigned bn = __ballot_sync(kFullMask, near);
      const unsigned bf = __ballot_sync(kFullMask, ok && !near);
      if (near) out[k0 + nacc + __popc(bn & lt)] = j;
      else if (ok) out[k0 + cnt - 1 - (facc + __popc(bf & lt))] = j;
      nacc += __popc(bn);
      facc += __popc(bf);
    }
    if (lane == 0) nn[i] = nacc;
  }
}

// Walks entries [first, np) of row i of C (first = C.first[i], or 0) in
// steps of G * U entries per row group, U per lane, the indices loaded one
// step ahead, calling body(xj, jj, ok) per step.  VEC: 16-byte index loads
// of 4 consecutive entries per lane (rows start on 16-byte boundaries and
// are readable to a multiple of 4); the walk starts at `first` rounded down
// to a multiple of 4 with the entries before it masked.
template <int G, int U, bool VEC, class Body>
__device__ __forceinline__ void walk_row(const Csr& C, int i, bool valid, int lane,
                                         const int4* __restrict__ qfix, Body&& body) {
  static_assert(!VEC || U == 4, "vector index loads take 4 entries per lane");
  int end = 0, first = 0, from = 0;
  int64_t k0 = 0;
  if (valid) {
    end = __ldg(C.np + i);
    first = C.first ? __ldg(C.first + i) : 0;
    from = VEC ? (first & ~3) : first;
    k0 = row_start(C, i) + from;
  }
  int cmax = end - from;
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) cmax = max(cmax, __shfl_xor_sync(kFullMask, cmax, off));
  const int lim = end - from, skip = first - from;
  auto entry = [&](int base, int u) { return VEC ? base + 4 * lane + u : base + lane + u * G; };
  auto load_idx = [&](int base, int* jn) {
    if (VEC) {
      int4 v = make_int4(0, 0, 0, 0);
      if (entry(base, 0) < lim) v = __ldg(reinterpret_cast<const int4*>(C.list + k0 + entry(base, 0)));
      jn[0] = v.x;
      jn[1] = v.y;
      jn[2] = v.z;
      jn[3] = v.w;
    } else {
#pragma unroll
      for (int u = 0; u < U; u++)
        jn[u] = entry(base, u) < lim ? __ldg(C.list + k0 + entry(base, u)) : 0;
    }
  };
  int jn[U];
  load_idx(0, jn);
  for (int base = 0; base < cmax; base += G * U) {
    int jj[U];
    bool ok[U];
#pragma unroll
    for (int u = 0; u < U; u++) {
      const int e = entry(base, u);
      ok[u] = e < lim && (!VEC || e >= skip);
      jj[u] = ok[u] ? jn[u] : 0;
    }
    int4 xj[U];
#pragma unroll
    for (int u = 0; u < U; u++) xj[u] = __ldg(qfix + jj[u]);
    load_idx(base + G * U, jn);
    body(xj, jj, ok);
  }
}

// Close queue of the segment gathers: the first lane of each row group with
// a far entry inside kFarCheck (`missed` on any lane of the group) puts row
// i onto close_rows, one slot per row (warp-aggregated on the length
// close_flag[2]), and raises close_flag[0].  Called by whole warps.
template <int G>
__device__ __forceinline__ void queue_close_row(bool missed, int i, int32_t* close_flag,
                                                int32_t* close_rows) {
  const unsigned mb = __ballot_sync(kFullMask, missed);
  if (!mb) return;
  const int wl = threadIdx.x & 31;
  const unsigned gmask = G == 32 ? kFullMask : ((1u << G) - 1u);
  const bool lead = (wl & (G - 1)) == 0 && ((mb >> wl) & gmask) != 0u;
  const unsigned lm = __ballot_sync(kFullMask, lead);
  int slot = 0;
  if (wl == 0) {
    slot = atomicAdd(close_flag + 2, __popc(lm));
    atomicExch(close_flag, 1);
  }
  slot = __shfl_sync(kFullMask, slot, 0) + __popc(lm & ((1u << wl) - 1u));
  if (lead) close_rows[slot] = i;
}

// Segment gather (LJ_PREC_MIXED over rows in two parts): C holds every row's
// near part, F its far part (k_partition_near's order, or the split rows of
// the MD build).  The far part runs first in FP32 terms from the coarse image
// (the FP32 kernels' arithmetic and cutoff band) into compensated FP32 sums,
// which then seed the two-float sums of the near part's two-float terms.  A
// far entry closer than K.near2 (2.0 sigma) -- a pair that moved in since
// the rows were split -- is skipped there: its row goes once onto the close
// queue (close_rows, count in close_flag[2]) and raises close_flag[0], and
// k_seg_close_terms then adds the two-float terms of the queued rows' close
// entries, so the split decides the speed, never the precision.
template <int G, int U, bool PBC, bool SOA, bool ANISO, bool VEC>
__global__ void __launch_bounds__(256, 3) k_gather_mixed_seg(const Particles P, const Csr C,
                                                          const Csr F,
                                                          const int4* __restrict__ qfix,
                                                          const MixedConsts K0,
                                                          int32_t* close_flag,
                                                          int32_t* __restrict__ close_rows,
                                                          const int32_t* __restrict__ rowperm) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int row = t / G;
  const int lane = t & (G - 1);
  // launched as a programmatic dependent of the image pass
  asm volatile("griddepcontrol.wait;" ::: "memory");
  const MixedConsts K = PBC ? K0 : frame_consts(K0);
  const bool valid = row < C.n;
  // rows visited in `rowperm` order when given (the MD loop passes the cell
  // order of its last build, so a warp's rows stay neighbours in space)
  const int i = valid && rowperm ? __ldg(rowperm + row) : row;
  const int4 xi = valid ? __ldg(qfix + i) : make_int4(0, 0, 0, 0);
  int li[3];
  image_lo(xi.w, li[0], li[1], li[2]);
  // FP64 cutoff decision of a pair in the band
  auto inside64 = [&](int j) {
    const double3 d64 = sep_fp64<PBC>(load_q<SOA>(P, i), load_q<SOA>(P, j), K.f64);
    return !beyond_cutoff(r2_fp64(d64), K.f64.cl2_bits);
  };
  // ---- far part: FP32 terms
  bool missed = false;
  RowSums<true> acc;
  {
    RowSums<false> acc32;
    acc32.init();
    walk_row<G, U, VEC>(F, i, valid, lane, qfix, [&](const int4* xj, const int* jj, const bool* ok) {
      float3 d[U];
      float r2[U];
      bool any = false;
#pragma unroll
      for (int u = 0; u < U; u++) {
        d[u] = sep_mixed<ANISO>(xi, xj[u], K);
        r2[u] = fmaf(d[u].z, d[u].z, fmaf(d[u].y, d[u].y, d[u].x * d[u].x));
        if (ok[u] && r2[u] < K.near2) missed = true;
        any |= ok[u] && r2[u] <= K.cl2s_hi;
      }
      if (!__any_sync(kFullMask, any)) return;  // the whole step beyond the cutoff
      float sx = 0.f, sy = 0.f, sz = 0.f;
      unsigned border = 0u;
#pragma unroll
      for (int u = 0; u < U; u++) {
        const bool use = ok[u] && !(r2[u] < K.near2);
        const bool in = use && r2[u] <= K.cl2s_lo;
        if (use && r2[u] > K.cl2s_lo && r2[u] <= K.cl2s_hi) border |= 1u << u;
        float df = df_mixed<ANISO>(r2[u], K);
        df = in ? df : 0.0f;
        sx = fmaf(df, d[u].x, sx);
        sy = fmaf(df, d[u].y, sy);
        sz = fmaf(df, d[u].z, sz);
      }
      if (__any_sync(kFullMask, border != 0u)) {
#pragma unroll
        for (int u = 0; u < U; u++) {
          if (!(border & (1u << u)) || !inside64(jj[u])) continue;
          const float df = df_mixed<ANISO>(r2[u], K);
          sx = fmaf(df, d[u].x, sx);
          sy = fmaf(df, d[u].y, sy);
          sz = fmaf(df, d[u].z, sz);
        }
      }
      acc32.x.add(sx);
      acc32.y.add(sy);
      acc32.z.add(sz);
    });
    // FP32 terms carry the 24 of df; the two-float sums and kick do not
    float h[6];
    acc32.get(h[0], h[1], h[2], h[3], h[4], h[5]);
    const float r24 = 0.041666668f;
    acc.x.hi = __fmul_rn(h[0], r24);
    acc.x.lo = __fmul_rn(h[1], r24);
    acc.y.hi = __fmul_rn(h[2], r24);
    acc.y.lo = __fmul_rn(h[3], r24);
    acc.z.hi = __fmul_rn(h[4], r24);
    acc.z.lo = __fmul_rn(h[5], r24);
  }
  // rare: far entries that moved inside K.near2 since the split are left to
  // k_seg_close_terms (its own kernel, so that its registers do not add to
  // this one's); the first lane of each row group with such an entry queues
  // the row, one slot per row (the queue holds n rows)
  queue_close_row<G>(missed, i, close_flag, close_rows);
  // ---- near part: two-float terms
  walk_row<G, U, VEC>(C, i, valid, lane, qfix, [&](const int4 (&xj)[U], const int* jj,
                                                    const bool (&ok)[U]) {
    unsigned border = 0u;
    step_terms_ff<ANISO, U % 2 == 0, U>(xi, li, xj, ok, K, acc, border);
    if (__any_sync(kFullMask, border != 0u)) {
#pragma unroll
      for (int u = 0; u < U; u++)
        if ((border & (1u << u)) && inside64(jj[u]))
          pair_term_ff<ANISO>(xi, li, xj[u], K, acc, 1, true, border, u);
    }
  });
  float hx, lx, hy, ly, hz, lz;
  acc.get(hx, lx, hy, ly, hz, lz);
  if (G > 1) {
    group_reduce_comp<G>(hx, lx);
    group_reduce_comp<G>(hy, ly);
    group_reduce_comp<G>(hz, lz);
  }
  kick_group<SOA, G, true>(P, i, lane, valid, hx, lx, hy, ly, hz, lz, K.fscale, K.fexp);
}

// The two-float terms of the far-part entries closer than K.near2 (FP32 r2,
// the far walk's own test) of the rows k_gather_mixed_seg queued (rows[0,
// flag[2]), each row once), kicked into p, when it raised flag[0]; otherwise
// every block returns at once.  A warp per queued row (G = 32, one entry per
// lane and step), so that a few queued rows do not wait on one lane walking
// a whole row.  The last block to finish clears flag[0], its counter flag[1]
// and the queue length flag[2].
template <int G, bool PBC, bool SOA, bool ANISO>
__global__ void __launch_bounds__(256) k_seg_close_terms(const Particles P, const Csr F,
                                                         const int4* __restrict__ qfix,
                                                         const MixedConsts K0, int32_t* flag,
                                                         const int32_t* __restrict__ queue) {
  if (*(volatile int32_t*)flag == 0) return;
  const MixedConsts K = PBC ? K0 : frame_consts(K0);
  const int lane = threadIdx.x & (G - 1);
  const int groups = (gridDim.x * blockDim.x) / G;
  const int queued = min(*(volatile int32_t*)(flag + 2), F.n);
  const int rows = (queued + groups - 1) / groups * groups;  // whole warps take every pass
  for (int r = (blockIdx.x * blockDim.x + threadIdx.x) / G; r < rows; r += groups) {
    const bool valid = r < queued;
    const int i = valid ? __ldg(queue + r) : 0;
    const int4 xi = valid ? __ldg(qfix + i) : make_int4(0, 0, 0, 0);
    int li[3];
    image_lo(xi.w, li[0], li[1], li[2]);
    RowSums<true> acc;
    acc.init();
    walk_row<G, 1, false>(F, i, valid, lane, qfix, [&](const int4* xj, const int* jj,
                                                       const bool* ok) {
      const float3 d = sep_mixed<ANISO>(xi, xj[0], K);
      const bool close = ok[0] && fmaf(d.z, d.z, fmaf(d.y, d.y, d.x * d.x)) < K.near2;
      unsigned border = 0u;
      pair_term_ff<ANISO>(xi, li, xj[0], K, acc, 0, close, border, 0);
      if (border) {
        const double3 d64 = sep_fp64<PBC>(load_q<SOA>(P, i), load_q<SOA>(P, jj[0]), K.f64);
        if (!beyond_cutoff(r2_fp64(d64), K.f64.cl2_bits))
          pair_term_ff<ANISO>(xi, li, xj[0], K, acc, 1, true, border, 0);
      }
    });
    float hx, lx, hy, ly, hz, lz;
    acc.get(hx, lx, hy, ly, hz, lz);
    if (G > 1) {
      group_reduce_comp<G>(hx, lx);
      group_reduce_comp<G>(hy, ly);
      group_reduce_comp<G>(hz, lz);
    }
    kick_group<SOA, G, true>(P, i, lane, valid, hx, lx, hy, ly, hz, lz, K.fscale, K.fexp);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    if (atomicAdd(flag + 1, 1) == (int)gridDim.x - 1) {
      flag[0] = 0;
      flag[1] = 0;
      flag[2] = 0;
    }
  }
}

// Batched mixed gather: as k_gather_mixed_u, with every constant that depends
// on the box (unit, cutoff in fixed units, FP64 image shift) read per row
// from the row's replica.  Groups walk the row list of one size class.  FF:
// two-float pair terms as in k_gather_mixed_u.
template <int G, int U, bool VEC, bool FF = false>
__global__ void __launch_bounds__(256) k_gather_mixed_batch(
    const Particles P, const Csr C, const int4* __restrict__ qfix, const int32_t* __restrict__ rid,
    const ReplicaInfo* __restrict__ reps, const int32_t* __restrict__ rows, int nrows, double dt,
    long long cl2_bits) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int g = t / G;
  const int lane = t & (G - 1);
  const bool valid = g < nrows;
  int cnt = 0, i = 0, r = 0;
  int64_t k0 = 0;
  int4 xi = make_int4(0, 0, 0, 0);
  // only the constants of the pair loop are held in registers; the rare FP64
  // cutoff decision and the kick read the replica table where they need it
  MixedConsts K{};
  if (valid) {
    i = __ldg(rows + g);
    cnt = __ldg(C.np + i);
    k0 = row_start(C, i);
    xi = __ldg(qfix + i);
    r = __ldg(rid + i);
    const ReplicaInfo& R = reps[r];
    K.k_hi = R.k_hi;
    K.k_lo = R.k_lo;
    K.cl2_lo = FF ? R.cl2f_lo : R.cl2u_lo;
    K.cl2_hi = FF ? R.cl2f_hi : R.cl2u_hi;
  }
  int cmax = cnt;
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) cmax = max(cmax, __shfl_xor_sync(kFullMask, cmax, off));
  int li[3];
  image_lo(xi.w, li[0], li[1], li[2]);
  RowSums<FF> acc;
  acc.init();
  static_assert(!VEC || U == 4, "vector index loads take 4 entries per lane");
  // entry of step `base` taken by (lane, u); VEC as in k_gather_mixed_u
  auto entry = [&](int base, int u) { return VEC ? base + 4 * lane + u : base + lane + u * G; };
  auto load_idx = [&](int base, int* jn) {
    if (VEC) {
      int4 v = make_int4(0, 0, 0, 0);
      if (entry(base, 0) < cnt)
        v = __ldg(reinterpret_cast<const int4*>(C.list + k0 + entry(base, 0)));
      jn[0] = v.x;
      jn[1] = v.y;
      jn[2] = v.z;
      jn[3] = v.w;
    } else {
#pragma unroll
      for (int u = 0; u < U; u++)
        jn[u] = entry(base, u) < cnt ? __ldg(C.list + k0 + entry(base, u)) : 0;
    }
  };
  int jn[U];
  load_idx(0, jn);
  for (int base = 0; base < cmax; base += G * U) {
    int jj[U];
    bool ok[U];
#pragma unroll
    for (int u = 0; u < U; u++) {
      ok[u] = entry(base, u) < cnt;
      jj[u] = ok[u] ? jn[u] : 0;
    }
    int4 xj[U];
#pragma unroll
    for (int u = 0; u < U; u++) xj[u] = __ldg(qfix + jj[u]);
    load_idx(base + G * U, jn);
    unsigned border = 0u;
    // the rare FP64 cutoff decision of entry u (replica constants read here)
    auto inside_fp64 = [&](int u) {
      const ReplicaInfo& R = reps[r];
      Fp64Consts f64{};
      f64.cl2_bits = cl2_bits;
      for (int d = 0; d < 3; d++) {
        f64.len[d] = R.len[d];
        f64.half_bits[d] = R.half_bits[d];
      }
      const double3 d64 = sep_fp64<true>(load_q<false>(P, i), load_q<false>(P, jj[u]), f64);
      return !beyond_cutoff(r2_fp64(d64), cl2_bits);
    };
    if constexpr (FF) {
      step_terms_ff<false, U % 2 == 0, U>(xi, li, xj, ok, K, acc, border);
      if (__any_sync(kFullMask, border != 0u)) {
#pragma unroll
        for (int u = 0; u < U; u++) {
          if (!(border & (1u << u)) || !inside_fp64(u)) continue;
          pair_term_ff<false>(xi, li, xj[u], K, acc, 1, true, border, u);
        }
      }
    } else {
      float sx = 0.f, sy = 0.f, sz = 0.f;
#pragma unroll
      for (int u = 0; u < U; u++) {
        const float3 d = sep_mixed<false>(xi, xj[u], K);
        const float r2 = fmaf(d.z, d.z, fmaf(d.y, d.y, d.x * d.x));
        const bool in = ok[u] && r2 <= K.cl2_lo;
        if (ok[u] && r2 > K.cl2_lo && r2 <= K.cl2_hi) border |= 1u << u;
        float df = df_mixed<false>(r2, K);
        df = in ? df : 0.0f;
        sx = fmaf(df, d.x, sx);
        sy = fmaf(df, d.y, sy);
        sz = fmaf(df, d.z, sz);
      }
      if (__any_sync(kFullMask, border != 0u)) {
#pragma unroll
        for (int u = 0; u < U; u++) {
          if (!(border & (1u << u)) || !inside_fp64(u)) continue;
          const float3 d = sep_mixed<false>(xi, xj[u], K);
          const float r2 = fmaf(d.z, d.z, fmaf(d.y, d.y, d.x * d.x));
          const float df = df_mixed<false>(r2, K);
          sx = fmaf(df, d.x, sx);
          sy = fmaf(df, d.y, sy);
          sz = fmaf(df, d.z, sz);
        }
      }
      acc.x.add(sx);
      acc.y.add(sy);
      acc.z.add(sz);
    }
  }
  float hx, lx, hy, ly, hz, lz;
  acc.get(hx, lx, hy, ly, hz, lz);
  if (G > 1) {
    group_reduce_comp<G>(hx, lx);
    group_reduce_comp<G>(hy, ly);
    group_reduce_comp<G>(hz, lz);
  }
  // kick scale: unit dt for FP32 terms, 24 unit dt for two-float terms
  const double kf = valid ? reps[r].unit * dt * (FF ? 24.0 : 1.0) : 0.0;
  const double fs[3] = {kf, kf, kf};
  kick_group<false, G, FF>(P, i, lane, valid, hx, lx, hy, ly, hz, lz, fs, 0);
}

// Batched segment gather over the split rows of the replica batch: as
// k_gather_mixed_seg, with the row's replica constants, over the rows of one
// size class.  The far part (F) runs first in FP32 terms, whose compensated
// sums seed the two-float sums of the near part (C).  A far entry closer
// than the replica's kFarCheck is skipped there and its row queued (once)
// for k_batch_close_terms, as in the single-system segment gather.
template <int G, int U, bool VEC>
__global__ void __launch_bounds__(256, 3) k_gather_mixed_batch_seg(
    const Particles P, const Csr C, const Csr F, const int4* __restrict__ qfix,
    const int32_t* __restrict__ rid, const ReplicaInfo* __restrict__ reps,
    const int32_t* __restrict__ rows, int nrows, double dt, long long cl2_bits,
    int32_t* close_flag, int32_t* __restrict__ close_rows) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int g = t / G;
  const int lane = t & (G - 1);
  const bool valid = g < nrows;
  int i = 0, r = 0;
  int4 xi = make_int4(0, 0, 0, 0);
  MixedConsts K{};
  if (valid) {
    i = __ldg(rows + g);
    xi = __ldg(qfix + i);
    r = __ldg(rid + i);
    const ReplicaInfo& R = reps[r];
    K.k_hi = R.k_hi;
    K.k_lo = R.k_lo;
    K.cl2_lo = R.cl2f_lo;  // two-float terms
    K.cl2_hi = R.cl2f_hi;
    K.cl2s_lo = R.cl2u_lo;  // FP32 terms
    K.cl2s_hi = R.cl2u_hi;
    K.near2 = R.nearc2u;
  }
  int li[3];
  image_lo(xi.w, li[0], li[1], li[2]);
  // the rare FP64 cutoff decision (replica constants read here)
  auto inside_fp64 = [&](int j) {
    const ReplicaInfo& R = reps[r];
    Fp64Consts f64{};
    f64.cl2_bits = cl2_bits;
    for (int d = 0; d < 3; d++) {
      f64.len[d] = R.len[d];
      f64.half_bits[d] = R.half_bits[d];
    }
    const double3 d64 = sep_fp64<true>(load_q<false>(P, i), load_q<false>(P, j), f64);
    return !beyond_cutoff(r2_fp64(d64), cl2_bits);
  };
  // ---- far part: FP32 terms
  bool missed = false;
  RowSums<true> acc;
  {
    RowSums<false> acc32;
    acc32.init();
    walk_row<G, U, VEC>(F, i, valid, lane, qfix, [&](const int4* xj, const int* jj,
                                                     const bool* ok) {
      float sx = 0.f, sy = 0.f, sz = 0.f;
      unsigned border = 0u;
      float3 d[U];
      float r2[U];
#pragma unroll
      for (int u = 0; u < U; u++) {
        d[u] = sep_mixed<false>(xi, xj[u], K);
        r2[u] = fmaf(d[u].z, d[u].z, fmaf(d[u].y, d[u].y, d[u].x * d[u].x));
        const bool use = ok[u] && !(r2[u] < K.near2);  // closer ones: the close pass
        if (ok[u] && r2[u] < K.near2) missed = true;
        const bool in = use && r2[u] <= K.cl2s_lo;
        if (use && r2[u] > K.cl2s_lo && r2[u] <= K.cl2s_hi) border |= 1u << u;
        float df = df_mixed<false>(r2[u], K);
        df = in ? df : 0.0f;
        sx = fmaf(df, d[u].x, sx);
        sy = fmaf(df, d[u].y, sy);
        sz = fmaf(df, d[u].z, sz);
      }
      if (__any_sync(kFullMask, border != 0u)) {
#pragma unroll
        for (int u = 0; u < U; u++) {
          if (!(border & (1u << u)) || !inside_fp64(jj[u])) continue;
          const float df = df_mixed<false>(r2[u], K);
          sx = fmaf(df, d[u].x, sx);
          sy = fmaf(df, d[u].y, sy);
          sz = fmaf(df, d[u].z, sz);
        }
      }
      acc32.x.add(sx);
      acc32.y.add(sy);
      acc32.z.add(sz);
    });
    // FP32 terms carry the 24 of df; the two-float sums and kick do not
    float h[6];
    acc32.get(h[0], h[1], h[2], h[3], h[4], h[5]);
    const float r24 = 0.041666668f;
    acc.x.hi = __fmul_rn(h[0], r24);
    acc.x.lo = __fmul_rn(h[1], r24);
    acc.y.hi = __fmul_rn(h[2], r24);
    acc.y.lo = __fmul_rn(h[3], r24);
    acc.z.hi = __fmul_rn(h[4], r24);
    acc.z.lo = __fmul_rn(h[5], r24);
  }
  queue_close_row<G>(missed, i, close_flag, close_rows);
  // ---- near part: two-float terms
  walk_row<G, U, VEC>(C, i, valid, lane, qfix, [&](const int4 (&xj)[U], const int* jj,
                                                   const bool (&ok)[U]) {
    unsigned border = 0u;
    step_terms_ff<false, U % 2 == 0, U>(xi, li, xj, ok, K, acc, border);
    if (__any_sync(kFullMask, border != 0u)) {
#pragma unroll
      for (int u = 0; u < U; u++)
        if ((border & (1u << u)) && inside_fp64(jj[u]))
          pair_term_ff<false>(xi, li, xj[u], K, acc, 1, true, border, u);
    }
  });
  float hx, lx, hy, ly, hz, lz;
  acc.get(hx, lx, hy, ly, hz, lz);
  if (G > 1) {
    group_reduce_comp<G>(hx, lx);
    group_reduce_comp<G>(hy, ly);
    group_reduce_comp<G>(hz, lz);
  }
  const double kf = valid ? reps[r].unit * dt * 24.0 : 0.0;
  const double fs[3] = {kf, kf, kf};
  kick_group<false, G, true>(P, i, lane, valid, hx, lx, hy, ly, hz, lz, fs, 0);
}

// The close pass of the replica batch: as k_seg_close_terms over the rows
// k_gather_mixed_batch_seg queued, a warp per row, with the row's replica
// constants (two-float cutoff band, pair-unit scale, FP64 box, kick scale).
template <int G>
__global__ void __launch_bounds__(256) k_batch_close_terms(
    const Particles P, const Csr F, const int4* __restrict__ qfix,
    const int32_t* __restrict__ rid, const ReplicaInfo* __restrict__ reps, double dt,
    long long cl2_bits, int32_t* flag, const int32_t* __restrict__ queue) {
  if (*(volatile int32_t*)flag == 0) return;
  const int lane = threadIdx.x & (G - 1);
  const int groups = (gridDim.x * blockDim.x) / G;
  const int queued = min(*(volatile int32_t*)(flag + 2), F.n);
  const int nr = (queued + groups - 1) / groups * groups;  // whole warps take every pass
  for (int t = (blockIdx.x * blockDim.x + threadIdx.x) / G; t < nr; t += groups) {
    const bool valid = t < queued;
    const int i = valid ? __ldg(queue + t) : 0;
    const int r = valid ? __ldg(rid + i) : 0;
    const ReplicaInfo& R = reps[r];
    MixedConsts K{};
    K.k_hi = R.k_hi;
    K.k_lo = R.k_lo;
    K.cl2_lo = R.cl2f_lo;
    K.cl2_hi = R.cl2f_hi;
    const float near2 = R.nearc2u;
    const int4 xi = valid ? __ldg(qfix + i) : make_int4(0, 0, 0, 0);
    int li[3];
    image_lo(xi.w, li[0], li[1], li[2]);
    RowSums<true> acc;
    acc.init();
    walk_row<G, 1, false>(F, i, valid, lane, qfix, [&](const int4* xj, const int* jj,
                                                       const bool* ok) {
      const float3 d = sep_mixed<false>(xi, xj[0], K);
      const bool close = ok[0] && fmaf(d.z, d.z, fmaf(d.y, d.y, d.x * d.x)) < near2;
      unsigned border = 0u;
      pair_term_ff<false>(xi, li, xj[0], K, acc, 0, close, border, 0);
      if (border) {
        Fp64Consts f64{};
        f64.cl2_bits = cl2_bits;
        for (int a = 0; a < 3; a++) {
          f64.len[a] = R.len[a];
          f64.half_bits[a] = R.half_bits[a];
        }
        const double3 d64 = sep_fp64<true>(load_q<false>(P, i), load_q<false>(P, jj[0]), f64);
        if (!beyond_cutoff(r2_fp64(d64), cl2_bits))
          pair_term_ff<false>(xi, li, xj[0], K, acc, 1, true, border, 0);
      }
    });
    float hx, lx, hy, ly, hz, lz;
    acc.get(hx, lx, hy, ly, hz, lz);
    if (G > 1) {
      group_reduce_comp<G>(hx, lx);
      group_reduce_comp<G>(hy, ly);
      group_reduce_comp<G>(hz, lz);
    }
    const double kf = valid ? R.unit * dt * 24.0 : 0.0;
    const double fs[3] = {kf, kf, kf};
    kick_group<false, G, true>(P, i, lane, valid, hx, lx, hy, ly, hz, lz, fs, 0);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    if (atomicAdd(flag + 1, 1) == (int)gridDim.x - 1) {
      flag[0] = 0;
      flag[1] = 0;
      flag[2] = 0;
    }
  }
}

// Cell-tiled mixed gather (kernel 3).  One CTA per cell: it copies the
// fixed-point positions of its (up to 27) neighbour cells -- contiguous runs of
// the cell-ordered image -- into shared memory, then walks the rows of its
// own particles, whose entries are 16-bit indices into that tile.  Every
// position a pair needs is read from shared memory; the list bytes halve.
// Arithmetic, masking, compensation and the FP64 kick are those of
// k_gather_mixed_u.
constexpr int kTiledThreads = 128;

template <int G, int U, bool PBC, bool SOA>
__global__ void __launch_bounds__(kTiledThreads) k_gather_mixed_tiled(
    const Particles P, const TiledList T, const int4* __restrict__ cq, const MixedConsts K0) {
  // a periodic frame is fixed on the host; an open one may come from the device
  const MixedConsts K = PBC ? K0 : frame_consts(K0);
  extern __shared__ int4 tile[];
  __shared__ int nstart[27], ncount[27];
  __shared__ int nnb, centre;
  const int c = blockIdx.x;
  if (threadIdx.x < 27) {
    CellGrid g{};
    g.nc[0] = T.gnc[0];
    g.nc[1] = T.gnc[1];
    g.nc[2] = T.gnc[2];
    g.ncells = T.ncells;
    g.periodic = T.periodic;
    int count;
    const int c2 = neighbour_cell_at(c, g, threadIdx.x, &count);
    if (c2 >= 0) {
      const int64_t a = __ldg(T.start + c2), b = __ldg(T.start + c2 + 1);
      nstart[threadIdx.x] = (int)a;
      ncount[threadIdx.x] = (int)(b - a);
      if (c2 == c) centre = threadIdx.x;
    }
    if (threadIdx.x == 0) nnb = count;
  }
  __syncthreads();
  const int warp = threadIdx.x >> 5, wl = threadIdx.x & 31;
  for (int nb = warp; nb < nnb; nb += kTiledThreads / 32)
    for (int t = wl; t < ncount[nb]; t += 32) tile[(nb << T.maxc_shift) + t] = __ldg(cq + nstart[nb] + t);
  __syncthreads();
  const int s0 = nstart[centre], s1 = s0 + ncount[centre];
  const int lane = threadIdx.x & (G - 1);
  const unsigned mask = (1u << T.maxc_shift) - 1u;
  for (int base = s0; base < s1; base += kTiledThreads / G) {
    const int s = base + threadIdx.x / G;
    const bool valid = s < s1;
    int cnt = 0, i = 0;
    int4 xi = make_int4(0, 0, 0, 0);
    const uint16_t* row = T.rows;
    if (valid) {
      cnt = __ldg(T.cnt + s);
      i = __ldg(T.order + s);
      xi = tile[(centre << T.maxc_shift) + (s - s0)];
      row = T.rows + (size_t)s * (size_t)T.maxrow;
    }
    int cmax = cnt;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1)
      cmax = max(cmax, __shfl_xor_sync(kFullMask, cmax, off));
    KahanF ax, ay, az;
    ax.init();
    ay.init();
    az.init();
    for (int kb = 0; kb < cmax; kb += G * U) {
      unsigned loc[U];
      bool ok[U];
#pragma unroll
      for (int u = 0; u < U; u++) {
        const int k = kb + lane + u * G;
        ok[u] = k < cnt;
        loc[u] = ok[u] ? (unsigned)__ldg(row + k) : 0u;
      }
      float sx = 0.f, sy = 0.f, sz = 0.f;
      unsigned border = 0u;
#pragma unroll
      for (int u = 0; u < U; u++) {
        const float3 d = sep_mixed<false>(xi, tile[loc[u]], K);
        const float r2 = fmaf(d.z, d.z, fmaf(d.y, d.y, d.x * d.x));
        const bool in = ok[u] && r2 <= K.cl2_lo;
        if (ok[u] && r2 > K.cl2_lo && r2 <= K.cl2_hi) border |= 1u << u;
        float df = df_mixed<false>(r2, K);
        df = in ? df : 0.0f;
        sx = fmaf(df, d.x, sx);
        sy = fmaf(df, d.y, sy);
        sz = fmaf(df, d.z, sz);
      }
      if (__any_sync(kFullMask, border != 0u)) {
#pragma unroll
        for (int u = 0; u < U; u++) {
          if (!(border & (1u << u))) continue;
          const int j = __ldg(T.order + nstart[loc[u] >> T.maxc_shift] + (int)(loc[u] & mask));
          const double3 d64 = sep_fp64<PBC>(load_q<SOA>(P, i), load_q<SOA>(P, j), K.f64);
          if (beyond_cutoff(r2_fp64(d64), K.f64.cl2_bits)) continue;
          const float3 d = sep_mixed<false>(xi, tile[loc[u]], K);
          const float r2 = fmaf(d.z, d.z, fmaf(d.y, d.y, d.x * d.x));
          const float df = df_mixed<false>(r2, K);
          sx = fmaf(df, d.x, sx);
          sy = fmaf(df, d.y, sy);
          sz = fmaf(df, d.z, sz);
        }
      }
      ax.add(sx);
      ay.add(sy);
      az.add(sz);
    }
    float hx = ax.s, lx = -ax.c, hy = ay.s, ly = -ay.c, hz = az.s, lz = -az.c;
    if (G > 1) {
      group_reduce_comp<G>(hx, lx);
      group_reduce_comp<G>(hy, ly);
      group_reduce_comp<G>(hz, lz);
    }
    kick_group<SOA, G>(P, i, lane, valid, hx, lx, hy, ly, hz, lz, K.fscale, K.fexp);
  }
}

template <bool SOA>
__global__ void __launch_bounds__(256) k_fixed_image_sorted(const Particles P, int n,
                                                            const int32_t* __restrict__ order,
                                                            const ImageFrame f0,
                                                            const long long* open_frame,
                                                            int4* __restrict__ cq) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  const ImageFrame f = image_frame(f0, open_frame);
  cq[s] = image_of(load_q<SOA>(P, __ldg(order + s)), f);
}

// Compacted FP64 gather (kernel 2).  One warp per row.  Candidates are
// screened in FP32 from the fixed-point image (cheap), the survivors (inside
// the cutoff or within 4e-6 of it) are queued in shared memory, and the FP64
// arithmetic runs on full batches of 32 queued pairs, so the FP64 pipe --
// the bottleneck of this path on GB300 -- does not idle on pairs beyond the
// cutoff or on the ragged end of a strided row.  The exact FP64 mask is
// applied to every queued pair.
constexpr int kCompactWarps = 4;

template <bool PBC, bool SOA>
__device__ __forceinline__ void fp64_pair_acc(const Particles& P, const double3& qi, int j,
                                              const Fp64Consts& k, double& fx, double& fy,
                                              double& fz) {
  const double3 d = sep_fp64<PBC>(qi, load_q<SOA>(P, j), k);
  const double r2 = r2_fp64(d);
  if (beyond_cutoff(r2, k.cl2_bits)) return;
  const double df = df_fp64(r2, k);
  fx = fma(df, d.x, fx);
  fy = fma(df, d.y, fy);
  fz = fma(df, d.z, fz);
}

template <bool PBC, bool SOA, bool ANISO>
__global__ void __launch_bounds__(32 * kCompactWarps) k_gather_fp64_c(
    const Particles P, const Csr C, const int4* __restrict__ qfix, const MixedConsts K0) {
  // a periodic frame is fixed on the host; an open one may come from the device
  const MixedConsts K = PBC ? K0 : frame_consts(K0);
  __shared__ int queue[kCompactWarps][64];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int i = blockIdx.x * kCompactWarps + w;
  if (i >= C.n) return;  // warp-uniform
  int* q = queue[w];
  const int cnt = __ldg(C.np + i), k0 = __ldg(C.ptr + i);
  const int4 xi = __ldg(qfix + i);
  const double3 qi = load_q<SOA>(P, i);
  const unsigned lt = (1u << lane) - 1u;
  double fx = 0.0, fy = 0.0, fz = 0.0;
  int qn = 0;
  for (int base = 0; base < cnt; base += 32) {
    const int k = base + lane;
    bool cand = false;
    int j = 0;
    if (k < cnt) {
      j = __ldg(C.list + k0 + k);
      const float3 d = sep_mixed<ANISO>(xi, __ldg(qfix + j), K);
      cand = fmaf(d.z, d.z, fmaf(d.y, d.y, d.x * d.x)) <= K.cl2_hi;
    }
    const unsigned b = __ballot_sync(kFullMask, cand);
    if (cand) q[qn + __popc(b & lt)] = j;
    qn += __popc(b);
    __syncwarp();
    if (qn >= 32) {
      fp64_pair_acc<PBC, SOA>(P, qi, q[lane], K.f64, fx, fy, fz);
      __syncwarp();
      if (lane < qn - 32) q[lane] = q[lane + 32];
      qn -= 32;
      __syncwarp();
    }
  }
  if (lane < qn) fp64_pair_acc<PBC, SOA>(P, qi, q[lane], K.f64, fx, fy, fz);
  const double total = warp_reduce3_fp64(fx, fy, fz, lane);
  if ((lane & 7) == 0 && lane < 24) add_p_axis<SOA>(P, i, lane >> 3, total);
}

// Compacted FP64 scatter over the half list (kernel 2).  A warp owns 32
// consecutive rows; their entries are contiguous (the context keeps a compact
// CSR), so the warp sweeps them flat, 32 entries per step, each lane finding
// its entry's row by a shuffle binary search over the rows' start offsets.
// Candidates are screened in FP32 from the fixed-point image; survivors are
// queued as (i, j) in shared memory and the FP64 arithmetic runs on full
// batches of 32.  Both ends are updated with RED.F64 (p_i += f, p_j -= f), so
// a batch may span rows and no lane waits for a row to end.
constexpr int kScatterWarps = 4;

template <bool PBC, bool SOA>
__device__ __forceinline__ void fp64_pair_red(const Particles& P, int i, int j,
                                              const Fp64Consts& k) {
  const double3 d = sep_fp64<PBC>(load_q<SOA>(P, i), load_q<SOA>(P, j), k);
  const double r2 = r2_fp64(d);
  if (beyond_cutoff(r2, k.cl2_bits)) return;
  const double df = df_fp64(r2, k);
  const double fx = df * d.x, fy = df * d.y, fz = df * d.z;
  red_p<SOA>(P, i, fx, fy, fz);
  red_p<SOA>(P, j, flip_sign(fx), flip_sign(fy), flip_sign(fz));
}

// R rows per warp (32, 16, 8 or 4): fewer rows per warp give more warps,
// which the FP64 pipe needs for latency hiding on lists of ~1e5 rows, but a
// larger share of partly filled last batches.
template <bool PBC, bool SOA, bool ANISO, int R = 32>
__global__ void __launch_bounds__(32 * kScatterWarps) k_scatter_fp64_c(
    const Particles P, const Csr C, const int4* __restrict__ qfix, const MixedConsts K0) {
  static_assert(R == 4 || R == 8 || R == 16 || R == 32, "rows per warp");
  // a periodic frame is fixed on the host; an open one may come from the device
  const MixedConsts K = PBC ? K0 : frame_consts(K0);
  __shared__ int2 queue[kScatterWarps][64];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int r0 = (blockIdx.x * kScatterWarps + w) * R;
  if (r0 >= C.n) return;  // warp-uniform
  const int nrows = min(R, C.n - r0);
  int2* q = queue[w];
  // start offset of row r0 + lane (rows past the end start at e1)
  const int my_start = lane < nrows ? __ldg(C.ptr + r0 + lane) : 0x7fffffff;
  const int e0 = __shfl_sync(kFullMask, my_start, 0);
  const int last = nrows - 1;
  const int e1 = __shfl_sync(kFullMask, my_start, last) + __ldg(C.np + r0 + last);
  const unsigned lt = (1u << lane) - 1u;
  int qn = 0;
  for (int base = e0; base < e1; base += 32) {
    const int k = base + lane;
    // row of entry k: the largest r with start(r) <= k (all lanes search, so
    // every shuffle is executed by the full warp; r + step stays below 32)
    int r = 0;
#pragma unroll
    for (int step = R / 2; step > 0; step >>= 1) {
      const int s = __shfl_sync(kFullMask, my_start, r + step);
      if (s <= k) r += step;
    }
    bool cand = false;
    const int i = r0 + r;
    int j = 0;
    if (k < e1) {
      j = __ldg(C.list + k);
      const float3 d = sep_mixed<ANISO>(__ldg(qfix + i), __ldg(qfix + j), K);
      cand = fmaf(d.z, d.z, fmaf(d.y, d.y, d.x * d.x)) <= K.cl2_hi;
    }
    const unsigned b = __ballot_sync(kFullMask, cand);
    if (cand) q[qn + __popc(b & lt)] = make_int2(i, j);
    qn += __popc(b);
    __syncwarp();
    if (qn >= 32) {
      const int2 e = q[lane];
      fp64_pair_red<PBC, SOA>(P, e.x, e.y, K.f64);
      __syncwarp();
      if (lane < qn - 32) q[lane] = q[lane + 32];
      qn -= 32;
      __syncwarp();
    }
  }
  if (lane < qn) {
    const int2 e = q[lane];
    fp64_pair_red<PBC, SOA>(P, e.x, e.y, K.f64);
  }
}

// Mixed scatter: FP32 partial forces per particle in a scratch array
// (compensation lost on the j side), then one FP64 kick per particle.
template <int G, bool PBC, bool SOA, bool ANISO>
__global__ void __launch_bounds__(256) k_scatter_mixed(const Particles P, const Csr C,
                                                       const int4* __restrict__ qfix,
                                                       float* __restrict__ facc,
                                                       const MixedConsts K0) {
  // a periodic frame is fixed on the host; an open one may come from the device
  const MixedConsts K = PBC ? K0 : frame_consts(K0);
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = t / G;
  const int lane = t & (G - 1);
  const bool valid = i < C.n;
  int cnt = 0, k0 = 0;
  int4 xi = make_int4(0, 0, 0, 0);
  if (valid) {
    cnt = __ldg(C.np + i);
    k0 = __ldg(C.ptr + i);
    xi = __ldg(qfix + i);
  }
  KahanF ax, ay, az;
  ax.init();
  ay.init();
  az.init();
  for (int k = lane; k < cnt; k += G) {
    const int j = __ldg(C.list + k0 + k);
    const float3 d = sep_mixed<ANISO>(xi, __ldg(qfix + j), K);
    const float r2 = fmaf(d.z, d.z, fmaf(d.y, d.y, d.x * d.x));
    if (!inside_mixed<PBC, SOA>(r2, P, i, j, K)) continue;
    const float df = df_mixed<ANISO>(r2, K);
    const float fx = df * d.x, fy = df * d.y, fz = df * d.z;
    ax.add(fx);
    ay.add(fy);
    az.add(fz);
    atomicAdd(facc + 4 * (size_t)j + 0, -fx);
    atomicAdd(facc + 4 * (size_t)j + 1, -fy);
    atomicAdd(facc + 4 * (size_t)j + 2, -fz);
  }
  float hx = ax.s, lx = -ax.c, hy = ay.s, ly = -ay.c, hz = az.s, lz = -az.c;
  if (G > 1) {
    group_reduce_comp<G>(hx, lx);
    group_reduce_comp<G>(hy, ly);
    group_reduce_comp<G>(hz, lz);
  }
  if (valid && lane == 0) {
    atomicAdd(facc + 4 * (size_t)i + 0, hx + lx);
    atomicAdd(facc + 4 * (size_t)i + 1, hy + ly);
    atomicAdd(facc + 4 * (size_t)i + 2, hz + lz);
  }
}

// Unrolled mixed scatter over the half list (mixed kernel 2): the traversal
// of k_gather_mixed_u (G lanes per row, U entries in flight, next indices
// prefetched, FP32 step sums into a Kahan accumulator for i), each pair's
// reaction on j added with one 16-byte vector atomic (float4 RED), so a pair
// costs one position gather and one atomic -- half the gathers of the full
// gather.  j-side sums are plain FP32 and their order varies run to run.
template <int G, int U, bool PBC, bool SOA, bool ANISO>
__global__ void __launch_bounds__(256) k_scatter_mixed_u(const Particles P, const Csr C,
                                                         const int4* __restrict__ qfix,
                                                         float4* __restrict__ facc,
                                                         const MixedConsts K0) {
  // Launched as a programmatic dependent of the image pass, which also
  // clears facc: nothing the stream wrote is read before that grid finished.
  asm volatile("griddepcontrol.wait;" ::: "memory");
  const MixedConsts K = PBC ? K0 : frame_consts(K0);
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = t / G;
  const int lane = t & (G - 1);
  const bool valid = i < C.n;
  int cnt = 0;
  int64_t k0 = 0;
  int4 xi = make_int4(0, 0, 0, 0);
  if (valid) {
    cnt = __ldg(C.np + i);
    k0 = row_start(C, i);
    xi = __ldg(qfix + i);
  }
  int cmax = cnt;
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) cmax = max(cmax, __shfl_xor_sync(kFullMask, cmax, off));
  KahanF ax, ay, az;
  ax.init();
  ay.init();
  az.init();
  int jn[U];
#pragma unroll
  for (int u = 0; u < U; u++) {
    const int k = lane + u * G;
    jn[u] = k < cnt ? __ldg(C.list + k0 + k) : 0;
  }
  for (int base = 0; base < cmax; base += G * U) {
    int jj[U];
    bool ok[U];
#pragma unroll
    for (int u = 0; u < U; u++) {
      ok[u] = base + lane + u * G < cnt;
      jj[u] = ok[u] ? jn[u] : 0;
    }
    int4 xj[U];
#pragma unroll
    for (int u = 0; u < U; u++) xj[u] = __ldg(qfix + jj[u]);
#pragma unroll
    for (int u = 0; u < U; u++) {
      const int k = base + G * U + lane + u * G;
      jn[u] = k < cnt ? __ldg(C.list + k0 + k) : 0;
    }
    float sx = 0.f, sy = 0.f, sz = 0.f;
#pragma unroll
    for (int u = 0; u < U; u++) {
      const float3 d = sep_mixed<ANISO>(xi, xj[u], K);
      const float r2 = fmaf(d.z, d.z, fmaf(d.y, d.y, d.x * d.x));
      bool in = ok[u] && r2 <= K.cl2_lo;
      if (ok[u] && r2 > K.cl2_lo && r2 <= K.cl2_hi) {  // rare: decided in FP64
        const double3 d64 = sep_fp64<PBC>(load_q<SOA>(P, i), load_q<SOA>(P, jj[u]), K.f64);
        in = !beyond_cutoff(r2_fp64(d64), K.f64.cl2_bits);
      }
      if (in) {
        const float df = df_mixed<ANISO>(r2, K);
        const float fx = df * d.x, fy = df * d.y, fz = df * d.z;
        sx += fx;
        sy += fy;
        sz += fz;
        atomicAdd(facc + jj[u], make_float4(-fx, -fy, -fz, 0.f));
      }
    }
    ax.add(sx);
    ay.add(sy);
    az.add(sz);
  }
  // the kick may be scheduled once every block is here (it still waits for
  // this grid to finish before reading facc)
  asm volatile("griddepcontrol.launch_dependents;");
  float hx = ax.s, lx = -ax.c, hy = ay.s, ly = -ay.c, hz = az.s, lz = -az.c;
  if (G > 1) {
    group_reduce_comp<G>(hx, lx);
    group_reduce_comp<G>(hy, ly);
    group_reduce_comp<G>(hz, lz);
  }
  if (valid && lane == 0) atomicAdd(facc + i, make_float4(hx + lx, hy + ly, hz + lz, 0.f));
}

// Two-float mixed scatter over the half list (kernel 2 with two-float pair
// terms): the traversal of k_scatter_mixed_u; the i side sums in registers
// as the gather does, the reaction on j goes to two float4 accumulators per
// particle: facc[2 j] takes the leading part of each term snapped to a fixed
// grid (K.snap), whose float sums are exact in any order, and facc[2 j + 1]
// the small remainder.  The j-side sums are therefore as accurate as the
// i-side ones, and the leading sums do not depend on the order of the
// atomics.
template <int G, int U, bool PBC, bool SOA, bool ANISO>
__global__ void __launch_bounds__(256) k_scatter_mixed_ff(const Particles P, const Csr C,
                                                          const int4* __restrict__ qfix,
                                                          float4* __restrict__ facc,
                                                          const MixedConsts K0) {
  // Launched as a programmatic dependent of the image pass, which also
  // clears facc: nothing the stream wrote is read before that grid finished.
  asm volatile("griddepcontrol.wait;" ::: "memory");
  const MixedConsts K = PBC ? K0 : frame_consts(K0);
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = t / G;
  const int lane = t & (G - 1);
  const bool valid = i < C.n;
  int cnt = 0;
  int64_t k0 = 0;
  int4 xi = make_int4(0, 0, 0, 0);
  if (valid) {
    cnt = __ldg(C.np + i);
    k0 = row_start(C, i);
    xi = __ldg(qfix + i);
  }
  int cmax = cnt;
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) cmax = max(cmax, __shfl_xor_sync(kFullMask, cmax, off));
  int li[3];
  image_lo(xi.w, li[0], li[1], li[2]);
  RowSums<true> acc;
  acc.init();
  int jn[U];
#pragma unroll
  for (int u = 0; u < U; u++) {
    const int k = lane + u * G;
    jn[u] = k < cnt ? __ldg(C.list + k0 + k) : 0;
  }
  for (int base = 0; base < cmax; base += G * U) {
    int jj[U];
    bool ok[U];
#pragma unroll
    for (int u = 0; u < U; u++) {
      ok[u] = base + lane + u * G < cnt;
      jj[u] = ok[u] ? jn[u] : 0;
    }
    int4 xj[U];
#pragma unroll
    for (int u = 0; u < U; u++) xj[u] = __ldg(qfix + jj[u]);
#pragma unroll
    for (int u = 0; u < U; u++) {
      const int k = base + G * U + lane + u * G;
      jn[u] = k < cnt ? __ldg(C.list + k0 + k) : 0;
    }
#pragma unroll
    for (int u = 0; u < U; u++) {
      float a[3], b[3], S, s;
      pair_sep_ff<ANISO>(xi, li[0], li[1], li[2], xj[u], K.u_hi, K.u_lo, a, b, S, s);
      bool in = ok[u] && S <= K.cl2_lo;
      if (ok[u] && S > K.cl2_lo && S <= K.cl2_hi) {  // rare: decided in FP64
        const double3 d64 = sep_fp64<PBC>(load_q<SOA>(P, i), load_q<SOA>(P, jj[u]), K.f64);
        in = !beyond_cutoff(r2_fp64(d64), K.f64.cl2_bits);
      }
      if (in) {
        const ff g = pair_g_ff<ANISO>(S, s, K.k_hi, K.k_lo);
        float p[3], e[3], h[3];
#pragma unroll
        for (int d = 0; d < 3; d++) {
          term_parts(g, a[d], b[d], p[d], e[d]);
          h[d] = snap_to_grid(p[d], K.snap);
        }
        acc.x.add_parts(p[0], e[0]);
        acc.y.add_parts(p[1], e[1]);
        acc.z.add_parts(p[2], e[2]);
        float4* fj = facc + 2 * (size_t)jj[u];
        atomicAdd(fj, make_float4(-h[0], -h[1], -h[2], 0.f));
        atomicAdd(fj + 1, make_float4(-__fadd_rn(__fsub_rn(p[0], h[0]), e[0]),
                                      -__fadd_rn(__fsub_rn(p[1], h[1]), e[1]),
                                      -__fadd_rn(__fsub_rn(p[2], h[2]), e[2]), 0.f));
      }
    }
  }
  asm volatile("griddepcontrol.launch_dependents;");
  float hx, lx, hy, ly, hz, lz;
  acc.get(hx, lx, hy, ly, hz, lz);
  if (G > 1) {
    group_reduce_comp<G>(hx, lx);
    group_reduce_comp<G>(hy, ly);
    group_reduce_comp<G>(hz, lz);
  }
  if (valid && lane == 0) {
    const float sx = snap_to_grid(hx, K.snap), sy = snap_to_grid(hy, K.snap),
                sz = snap_to_grid(hz, K.snap);
    float4* fi = facc + 2 * (size_t)i;
    atomicAdd(fi, make_float4(sx, sy, sz, 0.f));
    atomicAdd(fi + 1, make_float4(__fadd_rn(__fsub_rn(hx, sx), lx),
                                  __fadd_rn(__fsub_rn(hy, sy), ly),
                                  __fadd_rn(__fsub_rn(hz, sz), lz), 0.f));
  }
}

// p += F dt from the scatter's per-particle sums: one float4 (FP32 terms) or
// the snapped leading part and the remainder (two-float terms, FF).
template <bool SOA, bool FF = false>
__global__ void __launch_bounds__(256) k_kick_from_scratch(const Particles P, int n,
                                                           const float* __restrict__ facc,
                                                           const MixedConsts K0) {
  // may be launched as a programmatic dependent of the scatter: the sums
  // are read only after that grid has finished
  asm volatile("griddepcontrol.wait;" ::: "memory");
  const MixedConsts K = frame_consts(K0);
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (FF) {
    const float* f = facc + 8 * (size_t)i;
    kick_p<SOA>(P, i, widen_sum<true>(f[0], f[4]), widen_sum<true>(f[1], f[5]),
                widen_sum<true>(f[2], f[6]), K.fscale, K.fexp);
  } else {
    kick_p<SOA>(P, i, widen_f32(facc[4 * (size_t)i]), widen_f32(facc[4 * (size_t)i + 1]),
                widen_f32(facc[4 * (size_t)i + 2]), K.fscale, K.fexp);
  }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
Fp64Consts make_fp64_consts(const Periodic& box, double dt, double cl2) {
  Fp64Consts k{};
  k.c24 = 24.0 * dt;
  k.c48 = 48.0 * dt;
  long long b;
  std::memcpy(&b, &cl2, sizeof b);
  k.cl2_bits = b;
  for (int d = 0; d < 3; d++) {
    k.len[d] = box.on ? box.len[d] : 0.0;
    const double h = box.on ? box.half[d] : 0.0;
    std::memcpy(&b, &h, sizeof b);
    k.half_bits[d] = b;
  }
  return k;
}

void split_float(double v, float& hi, float& lo) {
  hi = (float)v;
  lo = (float)(v - (double)hi);
}

MixedConsts make_mixed_consts(const ForceLaunch& L) {
  MixedConsts k{};
  k.f64 = make_fp64_consts(L.box, L.dt, L.cl2);
  const bool ff = L.precision == LJ_PREC_MIXED;
  // pair units: coarse fixed units (isotropic) or length (anisotropic)
  const double u2 = L.aniso ? 1.0 : L.unit[0] * L.unit[0];
  const double cl2u = L.cl2 / u2;
  // separation error per axis in pair units: the coarse quantum (FP32
  // terms read X >> 10 only) or the fine one (two-float terms)
  const double umax = std::max(L.unit[0], std::max(L.unit[1], L.unit[2]));
  const double q_c = kCoarseQuantumErr * (L.aniso ? umax : 1.0);
  const double q = ff ? q_c / 1024.0 : q_c;
  const double base = ff ? kBandFF : kBandFp32;
  const double band = cutoff_band(std::sqrt(cl2u), q, base);
  k.cl2_lo = (float)(cl2u * (1.0 - band));
  k.cl2_hi = (float)(cl2u * (1.0 + band));
  k.cl2_0 = (float)cl2u;
  k.band_base = (float)base;
  k.qerr = (float)q;
  // FP32 terms of the near/far split: the FP32 band on the coarse image
  const double band32 = cutoff_band(std::sqrt(cl2u), q_c, kBandFp32);
  k.cl2s_lo = (float)(cl2u * (1.0 - band32));
  k.cl2s_hi = (float)(cl2u * (1.0 + band32));
  k.near2 = (float)(kFarCheck * kFarCheck / u2);
  k.near_build2 = (float)(kFarSplit * kFarSplit / u2);
  split_float(L.aniso ? 1.0 : 1.0 / u2, k.k_hi, k.k_lo);
  // two-float terms: 24 moves from the pair term into the kick scale
  const double c = ff ? 24.0 : 1.0;
  for (int d = 0; d < 3; d++) {
    split_float(L.unit[d], k.u_hi[d], k.u_lo[d]);
    k.fscale[d] = L.aniso ? c * L.dt : c * L.unit[d] * L.dt;
  }
  // scatter j-side grid: 2^-10 in force units (|F| below 2^14 sums exactly),
  // expressed in pair units (a pair unit of force is 24 unit of force units)
  const double grid_units = std::ldexp(1.0, -10) / (24.0 * (L.aniso ? 1.0 : L.unit[0]));
  int qe;
  std::frexp(grid_units, &qe);  // grid_units in [2^(qe-1), 2^qe)
  k.snap = (float)std::ldexp(1.5, 23 + qe - 1);
  k.open_frame = L.open_frame;
  return k;
}

// Launches `kfn` as a programmatic dependent of the previous kernel on `s`:
// its blocks may be scheduled while that kernel drains, and the kernel itself
// executes griddepcontrol.wait before reading anything the stream produced.
template <typename... KArgs, typename... Args>
cudaError_t launch_dependent(void (*kfn)(KArgs...), int blocks, int block, cudaStream_t s,
                             Args... args) {
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = dim3(blocks);
  cfg.blockDim = dim3(block);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kfn, args...);
}

template <typename F>
cudaError_t dispatch_lanes(int lanes, F&& f) {
  switch (lanes) {
    case 1: return f(std::integral_constant<int, 1>{});
    case 2: return f(std::integral_constant<int, 2>{});
    case 4: return f(std::integral_constant<int, 4>{});
    case 8: return f(std::integral_constant<int, 8>{});
    case 16: return f(std::integral_constant<int, 16>{});
    case 32: return f(std::integral_constant<int, 32>{});
    default: return cudaErrorInvalidValue;
  }
}

template <bool A, bool B, typename F>
cudaError_t with_bools(F&& f) {
  return f(std::integral_constant<bool, A>{}, std::integral_constant<bool, B>{});
}

template <typename F>
cudaError_t dispatch_bools(bool a, bool b, F&& f) {
  if (a) return b ? with_bools<true, true>(f) : with_bools<true, false>(f);
  return b ? with_bools<false, true>(f) : with_bools<false, false>(f);
}

}  // namespace

// Mixed-precision launchers of the other translation units (the constants
// come from make_mixed_consts of the same launch).
cudaError_t launch_mixed_fp32(const ForceLaunch& L, const MixedConsts& K, cudaStream_t s);
cudaError_t launch_mixed_ff_gather(const ForceLaunch& L, const MixedConsts& K, cudaStream_t s);
cudaError_t launch_mixed_ff_scatter(const ForceLaunch& L, const MixedConsts& K, cudaStream_t s);
cudaError_t launch_mixed_ff_split(const ForceLaunch& L, const MixedConsts& K, cudaStream_t s);

}  // namespace ljg
