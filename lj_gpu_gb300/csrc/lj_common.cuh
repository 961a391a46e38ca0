// lj_common.cuh -- device helpers shared by the force and list kernels.
//
// Arithmetic notes for GB300 (sm_103a):
//   * FP64 runs at ~1/64 of the FP32 rate on this part, and f32<->f64
//     conversions issue at the FP64 rate too.  The FP64 kernels therefore
//     avoid every FP64 instruction that is not arithmetic the reference does:
//     comparisons are done on the IEEE bit patterns with integer compares and
//     the division is a Newton-Raphson reciprocal seeded by the FP32 MUFU.
//   * The mixed kernels never touch FP64 per pair: positions are read from a
//     32-bit fixed-point image (see to_fixed), so the minimum image is plain
//     two's-complement wrap-around and dx is exact before its one rounding to
//     FP32.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace ljg {

constexpr unsigned kFullMask = 0xffffffffu;

// ---------------------------------------------------------------------------
// IEEE-754 double helpers on bit patterns (integer pipe only)
// ---------------------------------------------------------------------------
__device__ __forceinline__ long long dbits(double x) { return __double_as_longlong(x); }

// x > y for finite/inf non-negative y and any non-NaN x: for a positive y the
// ordering of doubles equals the signed ordering of their bit patterns.
__device__ __forceinline__ bool dgt_pos(double x, long long ybits) {
  return dbits(x) > ybits;
}
// x < -y for y >= 0: x negative with magnitude above y.
__device__ __forceinline__ bool dlt_neg(double x, long long ybits) {
  return (unsigned long long)dbits(x) > (0x8000000000000000ull | (unsigned long long)ybits);
}

// Minimum-image shift of one FP64 component: `d > L/2 ? d - L : d < -L/2 ?
// d + L : d`.  The comparisons run on bit patterns and the shift (0, -L or +L)
// is selected with integer moves, so exactly one FP64 add is issued (two
// predicated adds would both occupy the FP64 pipe).  d + (-L) is bitwise
// d - L, so the result equals the branchy form.
__device__ __forceinline__ double min_image_fp64(double d, double len, long long half_bits) {
  const long long lb = dbits(len);
  long long sb = 0;  // +0.0
  if (dgt_pos(d, half_bits)) sb = lb ^ (long long)0x8000000000000000ull;
  if (dlt_neg(d, half_bits)) sb = lb;
  return d + __longlong_as_double(sb);
}

// 1/r2 in FP64.  The seed is the MUFU FP32 reciprocal of the top 20 mantissa
// bits of r2 (rebiased exponent, so no f64->f32 conversion instruction is
// issued); relative error <= 2^-19.  One cubic Newton-Raphson step
//   e = 1 - r2 y0,  y1 = y0 (1 + e + e^2)
// takes the error to O(2^-57), i.e. the result is within an ulp of 1/r2.
// Valid for r2 in [2^-100, 2^100]; callers divide directly outside that
// range (only overlapping particles get there).
__device__ __forceinline__ double rcp_fp64(double r2) {
  const unsigned hi = (unsigned)__double2hiint(r2);
  const unsigned fbits = (hi - (896u << 20)) << 3;  // f32 with 20 mantissa bits of r2
  float y0f;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y0f) : "f"(__uint_as_float(fbits)));
  const unsigned yb = __float_as_uint(y0f);
  const double y0 = __hiloint2double((int)((yb >> 3) + (896u << 20)), 0);
  const double e = fma(-r2, y0, 1.0);
  return fma(y0, fma(e, e, e), y0);
}

// True when r2 may be seeded by rcp_fp64 (2^-100 <= r2 <= 2^100).
__device__ __forceinline__ bool rcp_fp64_in_range(double r2) {
  const long long b = dbits(r2);
  return b >= 0x39B0000000000000ll && b <= 0x4630000000000000ll;
}

// ---------------------------------------------------------------------------
// Fixed-point position frame for the mixed path.
//   periodic: X = floor(x * 2^32 / L) mod 2^32, so (Xj - Xi) as int32 is the
//             minimum-image separation in units of L / 2^32 -- wrap-around
//             int32 arithmetic does the minimum image exactly;
//   open:     X = trunc(x * 2^k), with 2^k chosen on the host from the largest
//             |coordinate| so that every |Xj - Xi| < 2^31 (nothing wraps).
// The conversion is done with integer instructions only: x = m 2^(E-1075),
// scale = mult 2^-sigma with mult in [2^63, 2^64), and X is 32 bits of the
// 128-bit product m * mult taken at bit 1075 + sigma - E.
// ---------------------------------------------------------------------------
struct FixedAxis {
  unsigned long long mult;  // scale mantissa, top bit set
  int sigma;                // scale = mult * 2^-sigma
  int pad;
};

// Open boxes: exponent k of the fixed-point scale 2^k chosen from the largest
// |coordinate| (key: its IEEE bits, as k_max_abs leaves them): |x| < 2^e and
// k = 30 - e keep |X| <= 2^30, so every difference fits in int32.  k is held
// in [-60, 50] so the FP32 pair constants (which scale by 2^2k) stay finite
// and normal.  Must equal the host's choice in make_fixed_frame.
__host__ __device__ __forceinline__ int open_frame_exp(unsigned long long key) {
  const int be = (int)((key >> 52) & 0x7ffull);
  const int e = key == 0ull ? 1 : (be == 0 ? -1021 : be - 1022);  // frexp exponent
  const int k = 30 - e;
  return k < -60 ? -60 : (k > 50 ? 50 : k);
}

// The axis of scale 2^k (mult 2^63, sigma 63 - k).
__host__ __device__ __forceinline__ FixedAxis pow2_axis(int k) {
  FixedAxis a;
  a.mult = 1ull << 63;
  a.sigma = 63 - k;
  a.pad = 0;
  return a;
}

__device__ __forceinline__ int to_fixed(double x, const FixedAxis& ax) {
  const unsigned long long b = (unsigned long long)dbits(x);
  const int e = (int)((b >> 52) & 0x7ffull);
  unsigned long long m = b & 0x000fffffffffffffull;
  if (e != 0) m |= 0x0010000000000000ull;
  const int sh = 1075 + ax.sigma - (e != 0 ? e : 1);
  const unsigned long long lo = m * ax.mult;
  const unsigned long long hi = __umul64hi(m, ax.mult);
  unsigned v;
  if (sh >= 128) v = 0u;
  else if (sh >= 64) v = (unsigned)(hi >> (sh - 64));
  else if (sh > 0) v = (unsigned)((lo >> sh) | (hi << (64 - sh)));
  else if (sh > -32) v = (unsigned)(lo << (-sh));
  else v = 0u;
  return (b >> 63) ? -(int)v : (int)v;
}

// Periodic wrap of a coordinate into [0, len) with one shift and one FP64
// add; the comparisons run on the IEEE bit patterns (integer pipe), since
// FP64 compares issue on the slow FP64 pipe.  x >= len (or +inf) gets -len,
// x < 0 gets +len, anything else (including -0.0) adds +0.0; a result that
// rounds up to len becomes 0; NaN passes through.
__device__ __forceinline__ double wrap_into_box(double x, double len) {
  const unsigned long long b = (unsigned long long)dbits(x);
  const unsigned long long lb = (unsigned long long)dbits(len);
  const unsigned long long mag = b & 0x7fffffffffffffffull;
  const bool nan = mag > 0x7ff0000000000000ull;
  long long sb = 0;
  if ((b >> 63) == 0 && !nan && b >= lb) sb = dbits(-len);
  if ((b >> 63) != 0 && mag != 0 && !nan) sb = (long long)lb;
  const double y = x + __longlong_as_double(sb);
  const unsigned long long by = (unsigned long long)dbits(y);
  return ((by >> 63) == 0 && by <= 0x7ff0000000000000ull && by >= lb) ? 0.0 : y;
}

// int32 difference with wrap-around (no signed-overflow UB)
__device__ __forceinline__ int wrap_sub(int a, int b) {
  return (int)((unsigned)a - (unsigned)b);
}

// ---------------------------------------------------------------------------
// Compensated FP32 accumulation (Kahan 1965): sum + comp carries the exact
// running sum to O(eps^2).
// ---------------------------------------------------------------------------
struct KahanF {
  float s, c;
  __device__ __forceinline__ void init() { s = 0.f; c = 0.f; }
  __device__ __forceinline__ void add(float x) {
    const float y = __fsub_rn(x, c);
    const float t = __fadd_rn(s, y);
    c = __fsub_rn(__fsub_rn(t, s), y);
    s = t;
  }
};

// Knuth's TwoSum: s + e == a + b exactly.
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// Reduce a compensated pair (s, -c) over `width` lanes with xor shuffles,
// keeping the rounding error of every partial sum.  Returns hi + lo with the
// total in lane 0 of each group (all lanes of the group receive it).
template <int W>
__device__ __forceinline__ void group_reduce_comp(float& hi, float& lo) {
#pragma unroll
  for (int off = W / 2; off > 0; off >>= 1) {
    const float oh = __shfl_xor_sync(kFullMask, hi, off);
    const float ol = __shfl_xor_sync(kFullMask, lo, off);
    float s, e;
    two_sum(hi, oh, s, e);
    hi = s;
    lo = __fadd_rn(lo, __fadd_rn(ol, e));
  }
}

template <int W>
__device__ __forceinline__ double group_reduce_fp64(double v) {
#pragma unroll
  for (int off = W / 2; off > 0; off >>= 1) v += __shfl_xor_sync(kFullMask, v, off);
  return v;
}

// Exact f32 -> f64 widening with integer instructions (normal numbers, zero,
// inf and NaN; FP32 denormals, which the FTZ pair math never produces, become
// zero).  Avoids the f32->f64 conversion instruction, which issues at the
// FP64 rate on this part.
__device__ __forceinline__ double widen_f32(float f) {
  const unsigned b = __float_as_uint(f);
  const unsigned e = (b >> 23) & 0xffu;
  if (e == 0u) return 0.0;
  const unsigned ed = (e == 0xffu) ? 0x7ffu : e + 896u;
  const unsigned hi = (b & 0x80000000u) | (ed << 20) | ((b & 0x7fffffu) >> 3);
  const unsigned lo = b << 29;
  return __hiloint2double((int)hi, (int)lo);
}

}  // namespace ljg
