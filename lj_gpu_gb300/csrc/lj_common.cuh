// lj_common.cuh -- device helpers shared by the force and list kernels.
//
// Arithmetic notes for GB300 (sm_103a):
//   * FP64 runs at ~1/64 of the FP32 rate on this part, and f32<->f64
//     conversions issue at the FP64 rate too.  The FP64 kernels therefore
//     avoid every FP64 instruction that is not arithmetic the reference does:
//     comparisons are done on the IEEE bit patterns with integer compares and
//     the division is a Newton-Raphson reciprocal seeded by the FP32 MUFU.
//   * The mixed kernels never touch FP64 per pair: positions are read from a
//     42-bit fixed-point image (see pack_image), so the minimum image is plain
//     two's-complement wrap-around and dx is exact, as an integer, before
//     any floating-point rounding.
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
//
// Every coordinate is held as a 42-bit fixed-point number X (fine units).
// The position image of a particle is one int4:
//   x, y, z: X >> 10 per axis (32-bit "coarse" units), w: the three low
//   10-bit fields, X & 1023 of x in bits 0-9, of y in bits 10-19, of z in
//   bits 20-29.
// Coarse-only consumers (list builders, FP32 screening, the FP32 pair
// kernels) read x, y, z; the two-float pair kernels also read w.
//
//   periodic: X = floor(x * 2^42 / L) mod 2^42, so the coarse difference
//             (Xj - Xi) >> 10 taken as wrapping int32 is the minimum-image
//             separation in units of L / 2^32, and adding the difference of
//             the low fields gives it in units of L / 2^42;
//   open:     X = trunc(x 2^kf) - trunc(o 2^kf) with o the per-axis minimum
//             coordinate and 2^kf chosen from the largest per-axis extent
//             (open_frame_kf), so X stays within [-1, 2^40 + 1] and the
//             quantum follows the system's size, not its distance from the
//             origin.
// The conversion is done with integer instructions only: x = m 2^(E-1075),
// scale = mult 2^-sigma with mult in [2^63, 2^64), and X is 64 bits of the
// 128-bit product m * mult taken at bit 1075 + sigma - E - 10.
// ---------------------------------------------------------------------------
struct FixedAxis {
  unsigned long long mult;  // coarse scale mantissa, top bit set
  int sigma;                // coarse scale = mult * 2^-sigma (fine = coarse * 2^10)
  int pad;
};

constexpr int kFineBits = 10;  // fine units per coarse unit: 2^10

// The coarse axis of scale 2^k (mult 2^63, sigma 63 - k).
__host__ __device__ __forceinline__ FixedAxis pow2_axis(int k) {
  FixedAxis a;
  a.mult = 1ull << 63;
  a.sigma = 63 - k;
  a.pad = 0;
  return a;
}

// 64 bits of the 128-bit product m * mult starting at bit sh (0 beyond it).
__device__ __forceinline__ unsigned long long prod_bits(unsigned long long m,
                                                        unsigned long long mult, int sh) {
  const unsigned long long lo = m * mult;
  const unsigned long long hi = __umul64hi(m, mult);
  if (sh >= 128) return 0ull;
  if (sh >= 64) return hi >> (sh - 64);
  if (sh > 0) return (lo >> sh) | (hi << (64 - sh));
  if (sh > -64) return lo << (-sh);
  return 0ull;
}

// x in fine units, truncated toward zero, as a wrapping 64-bit integer.
__device__ __forceinline__ long long to_fixed_fine(double x, const FixedAxis& ax) {
  const unsigned long long b = (unsigned long long)dbits(x);
  const int e = (int)((b >> 52) & 0x7ffull);
  unsigned long long m = b & 0x000fffffffffffffull;
  if (e != 0) m |= 0x0010000000000000ull;
  const int sh = 1075 + ax.sigma - (e != 0 ? e : 1) - kFineBits;
  const unsigned long long v = prod_bits(m, ax.mult, sh);
  return (b >> 63) ? (long long)(0ull - v) : (long long)v;
}

// The image int4 of three fine coordinates.
__device__ __forceinline__ int4 pack_image(long long X, long long Y, long long Z) {
  const unsigned w = ((unsigned)X & 1023u) | (((unsigned)Y & 1023u) << 10) |
                     (((unsigned)Z & 1023u) << 20);
  return make_int4((int)(X >> kFineBits), (int)(Y >> kFineBits), (int)(Z >> kFineBits), (int)w);
}

// Coarse coordinate only (32 bits of the fine value above the low field).
__device__ __forceinline__ int to_fixed(double x, const FixedAxis& ax) {
  return (int)(to_fixed_fine(x, ax) >> kFineBits);
}

// ---------------------------------------------------------------------------
// Relative half-width of the band around a cutoff (or search) sphere inside
// which an FP32 comparison of r2 is not trusted and the pair is re-decided
// in FP64: `base` (rounding of the FP32 r2 and of the band edges) plus the
// largest r2 error the position quantum allows, |dr2| <= 2 sqrt(3) rc q +
// 3 q^2 for a separation error of at most q per axis, relative to rc^2.
// rc and q are in the same units (coarse fixed units, or lengths).
__host__ __device__ __forceinline__ double cutoff_band(double rc, double q, double base) {
  if (!(rc > 0.0)) return base;
  return base + (3.4641016151377544 * rc * q + 3.0 * q * q) / (rc * rc);
}
constexpr double kBandFp32 = 4e-6;  // FP32 r2 from rounded FP32 separations
constexpr double kBandFF = 6e-7;    // two-float r2 rounded to float vs float edges
// separation error per axis of the coarse image (X >> 10 of both ends), in
// coarse units; the fine image's is kCoarseQuantumErr / 1024
constexpr double kCoarseQuantumErr = 2.0;
// Near/far split of the two-float gathers (lengths, sigma = 1): rows are
// ordered near-first at r < kFarSplit (k_partition_near, or the MD build's
// split rows), and any pair found closer than kFarCheck is evaluated in
// two-float arithmetic wherever it sits in its row.  FP32 terms for every
// pair beyond 2.0 sigma keep the net force of each particle within 2.2e-6
// (108,000 particles, rho 0.5), 1.1e-6 (1M, rho 1, over 1,000 MD steps) and
// 2.4e-6 (8M, rho 1) of FP64, against a bar of 1e-5.  Rows split at 2.1
// sigma: the few rows whose far pairs come inside 2.0 sigma before the next
// rebuild are queued and their close terms added by a second pass
// (k_seg_close_terms, k_batch_close_terms).
constexpr double kFarSplit = 2.1;
constexpr double kFarCheck = 2.0;

// ---------------------------------------------------------------------------
// Open-box frame chosen on the device.  A bounds pass (k_open_bounds) folds
// every coordinate into per-axis min / max keys; its last block turns them
// into the frame below, in the same device words, and re-arms the keys for
// the next call.  Word layout (kOpenFrameWords x 8 bytes):
//   [0..2] min keys, [3..5] max keys (order-preserving u64 of the doubles),
//   [6] blocks done, [8] fine exponent kf, [9..11] origin per axis in fine
//   units (trunc(min_a 2^kf)).
// ---------------------------------------------------------------------------
constexpr int kOpenFrameWords = 16;
constexpr int kOfMin = 0, kOfMax = 3, kOfDone = 6, kOfExp = 8, kOfOrigin = 9;

// Order-preserving map of a double's bits to u64 (and back).
__host__ __device__ __forceinline__ unsigned long long order_key(unsigned long long b) {
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
__host__ __device__ __forceinline__ unsigned long long order_unkey(unsigned long long k) {
  return (k >> 63) ? (k & 0x7fffffffffffffffull) : ~k;
}

// frexp exponent of |v| from its bits (v = f 2^e, f in [0.5, 1)); 1 for zero
// and for non-finite values a large exponent.
__host__ __device__ __forceinline__ int frexp_exp_bits(unsigned long long b) {
  const int be = (int)((b >> 52) & 0x7ffull);
  if ((b & 0x7fffffffffffffffull) == 0ull) return 1;
  if (be == 0x7ff) return 2000;
  return be == 0 ? -1021 : be - 1022;
}

// Fine exponent kf of an open frame from the largest |coordinate| (bits
// amax_bits) and the largest per-axis extent (bits ext_bits, max - min, an
// extent below 2^e_ext).  kf = 40 - e_ext keeps every origin-relative X in
// [-1, 2^40 + 1] after truncation, so coarse differences (X >> 10) stay
// within +-(2^30 + 1) (int32, and exact as floats once their low 8 bits are
// cleared); |x| 2^kf < 2^61 keeps the 64-bit conversion exact.  kf is held
// in [-20, 60] so the FP32 pair constants, which scale by 2^(2 (kf - 10)),
// stay finite and normal.
__host__ __device__ __forceinline__ int open_frame_kf(unsigned long long amax_bits,
                                                      unsigned long long ext_bits) {
  const int e_ext = frexp_exp_bits(ext_bits);
  const int e_abs = frexp_exp_bits(amax_bits);
  int kf = 40 - e_ext;
  if (kf > 61 - e_abs) kf = 61 - e_abs;
  return kf < -20 ? -20 : (kf > 60 ? 60 : kf);
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
