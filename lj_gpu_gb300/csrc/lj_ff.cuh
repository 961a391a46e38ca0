// lj_ff.cuh -- two-float ("float-float") pair arithmetic of the mixed path.
//
// A value is the unevaluated sum h + l of two floats (about 48 significant
// bits).  Products and sums are made error-free with two published
// transformations:
//   * TwoProd by fused multiply-add: p = fl(a b), e = fma(a, b, -p) gives
//     a b = p + e exactly (Dekker 1971's exact product, in its FMA form);
//   * TwoSum (Knuth, TAOCP vol. 2, 4.2.2): s = fl(a + b) and
//     e = (a - (s - b')) + (b - b'), b' = s - a, gives a + b = s + e exactly;
//     when |a| >= |b| the shorter Fast2Sum e = b - (s - a) (Dekker) suffices.
// Only FP32 instructions are issued (GB300 runs FP64 at 1/64 of the FP32
// rate), and every operation is written with the _rn intrinsics so the
// compiler cannot contract or reorder it.
//
// The pair term of the Lennard-Jones kick is evaluated as
//   d = q_j - q_i from the exact 42-bit fixed-point difference,
//   s = 1 / |d|^2, g = s^4 (1 - 2 s^3), f = g d,
// with 24 and dt folded into the FP64 kick scale: the arithmetic of
// cpu_ref/force_aos.cpp:206-218 (df = (24 r^6 - 48) / r^14 dt) rearranged as
// 24 r^-8 (1 - 2 r^-6) dt.  Relative error of a pair term is about 2^-44, so
// the net force of a particle keeps ~1e-9 relative accuracy even where its
// pair terms cancel 1000-fold.
#pragma once

#include "lj_common.cuh"

namespace ljg {

struct ff {
  float h, l;
};

// a * b for two-float a, b (the l * l term is below the result's precision)
__device__ __forceinline__ ff ff_mul(ff a, ff b) {
  const float p = __fmul_rn(a.h, b.h);
  float e = __fmaf_rn(a.h, b.h, -p);
  e = __fmaf_rn(a.h, b.l, e);
  e = __fmaf_rn(a.l, b.h, e);
  return ff{p, e};
}

__device__ __forceinline__ ff ff_sqr(ff a) {
  const float p = __fmul_rn(a.h, a.h);
  float e = __fmaf_rn(a.h, a.h, -p);
  e = __fmaf_rn(__fadd_rn(a.h, a.h), a.l, e);
  return ff{p, e};
}

// Knuth's TwoSum of two floats into a two-float value.
__device__ __forceinline__ ff ff_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return ff{s, e};
}

// The exact coarse-unit separation of one axis as a + b: dh = (Xj - Xi) >> 10
// (wrapping int32: the minimum image for periodic frames) and dlo the
// difference of the low 10-bit fields.  a = dh with its low 8 bits cleared
// has at most 23 significant bits, b = ((dh & 255) 1024 + dlo) / 1024 fewer
// than 18: both conversions are exact, and |b| < 256 <= the lowest set bit
// of a (or a = 0).
__device__ __forceinline__ void sep_axis_ff(int xj, int xi, int dlo, float& a, float& b) {
  const int dh = wrap_sub(xj, xi);
  a = __int2float_rn(dh & ~255);
  b = __fmul_rn(__int2float_rn(((dh & 255) << kFineBits) + dlo), 0.0009765625f);
}

// The three low fields of an image's w word.
__device__ __forceinline__ void image_lo(int w, int& lx, int& ly, int& lz) {
  lx = w & 1023;
  ly = (w >> 10) & 1023;
  lz = (w >> 20) & 1023;
}

// Separation of one pair in pair units: a + b per axis, and |d|^2 as the
// normalised two-float S + s (S = fl(r2), what cutoff decisions compare).
// Before normalisation the cross terms 2 a b -- up to ~1e-4 of r2 when the
// coarse unit is large -- sit in the low part; the reciprocal's one-step
// refinement needs |s| <= ulp(S).
// With ANISO the per-axis unit (two-float uh + ul) is applied, so the pair
// units are lengths; otherwise they are coarse fixed units.
template <bool ANISO>
__device__ __forceinline__ void pair_sep_ff(const int4& xi, int lix, int liy, int liz,
                                            const int4& xj, const float* uh, const float* ul,
                                            float (&a)[3], float (&b)[3], float& S, float& s) {
  int ljx, ljy, ljz;
  image_lo(xj.w, ljx, ljy, ljz);
  sep_axis_ff(xj.x, xi.x, ljx - lix, a[0], b[0]);
  sep_axis_ff(xj.y, xi.y, ljy - liy, a[1], b[1]);
  sep_axis_ff(xj.z, xi.z, ljz - liz, a[2], b[2]);
  float p[3], e[3];
#pragma unroll
  for (int d = 0; d < 3; d++) {
    if (ANISO) {  // (a + b) (uh + ul) as a two-float length
      const float m = __fmul_rn(a[d], uh[d]);
      float t = __fmaf_rn(a[d], uh[d], -m);
      t = __fmaf_rn(b[d], uh[d], t);
      t = __fmaf_rn(a[d], ul[d], t);
      a[d] = m;
      b[d] = t;
    }
    // (a + b)^2 = a^2 + (2a + b) b, a^2 exactly as p + e
    p[d] = __fmul_rn(a[d], a[d]);
    e[d] = __fmaf_rn(a[d], a[d], -p[d]);
    e[d] = __fmaf_rn(__fadd_rn(a[d], a[d]), b[d], e[d]);
    e[d] = __fmaf_rn(b[d], b[d], e[d]);
  }
  const ff s1 = ff_two_sum(p[0], p[1]);
  const ff s2 = ff_two_sum(s1.h, p[2]);
  const float lo = __fadd_rn(__fadd_rn(e[0], e[1]), __fadd_rn(e[2], __fadd_rn(s1.l, s2.l)));
  // Fast2Sum (|s2.h| >= |lo|): S = fl(s2.h + lo), s the exact remainder
  S = __fadd_rn(s2.h, lo);
  s = __fsub_rn(lo, __fsub_rn(S, s2.h));
}

// g = s^4 (1 - 2 s^3) with s = k / (S + s_lo), two-float k the square of the
// pair unit's inverse (1 for lengths).  The reciprocal is the MUFU seed y
// refined once: y (1 + e), e = 1 - (S + s_lo) y, error O(e^2) ~ 2^-44.
template <bool ANISO>
__device__ __forceinline__ ff pair_g_ff(float S, float s_lo, float kh, float kl) {
  float y;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(S));
  float e = __fmaf_rn(-S, y, 1.0f);
  e = __fmaf_rn(-s_lo, y, e);
  ff inv{y, __fmul_rn(y, e)};
  if (!ANISO) inv = ff_mul(inv, ff{kh, kl});
  const ff i2 = ff_sqr(inv);
  const ff i6 = ff_mul(i2, inv);
  // w = 1 - 2 s^3 by TwoSum (1, -2 i6.h) (the product by 2 is exact)
  const float m = __fmul_rn(-2.0f, i6.h);
  ff w = ff_two_sum(1.0f, m);
  w.l = __fmaf_rn(-2.0f, i6.l, w.l);
  return ff_mul(ff_sqr(i2), w);
}

// One axis of a pair term, g (a + b) = p + e: g.h a exactly as p plus its
// rounding error, the small products added to that error.
__device__ __forceinline__ void term_parts(ff g, float a, float b, float& p, float& e) {
  p = __fmul_rn(g.h, a);
  e = __fmaf_rn(g.h, a, -p);
  e = __fmaf_rn(g.h, b, e);
  e = __fmaf_rn(g.l, a, e);
}

// p rounded to the grid of the snap constant (1.5 2^(23+q) rounds |p| <
// 2^(22+q) to a multiple of 2^q): sums of such values are exact in FP32 while
// they stay below 2^(24+q), whatever their order.
__device__ __forceinline__ float snap_to_grid(float p, float snap) {
  return __fsub_rn(__fadd_rn(p, snap), snap);
}

// Compensated accumulation of one axis: the leading part of every term is
// added to hi by TwoSum, whose rounding error joins the small parts in the
// plain sum lo.  TwoSum is exact whatever the magnitudes (Kahan's update is
// exact only while the running sum dominates each term, and the pair terms
// of a particle cancel to a net force far smaller than themselves).
struct AccFF {
  float hi, lo;
  __device__ __forceinline__ void init() { hi = lo = 0.f; }
  // += g (a + b)
  __device__ __forceinline__ void add(ff g, float a, float b) {
    float p, e;
    term_parts(g, a, b, p, e);
    add_parts(p, e);
  }
  __device__ __forceinline__ void add_parts(float p, float e) {
    const ff s = ff_two_sum(hi, p);
    hi = s.h;
    lo = __fadd_rn(lo, __fadd_rn(s.l, e));
  }
  // the sum as a two-float value (hi, lo)
  __device__ __forceinline__ void get(float& h, float& l) const {
    h = hi;
    l = lo;
  }
};

// ---------------------------------------------------------------------------
// Two pair terms at once: packed f32x2 instructions (sm_100 and later) carry
// one pair in each 32-bit half of a 64-bit register.  Every packed operation
// is the scalar code's IEEE operation (round to nearest, no flush) on each
// half, so a pair's bits do not depend on which form evaluated it, and a step
// costs fewer FP32 issue slots.  PTX has no packed negation, so the
// operations with a negated operand stay scalar (f2_fms, f2_nfma).
// ---------------------------------------------------------------------------
typedef unsigned long long f2;  // low half: first pair, high half: second pair

__device__ __forceinline__ f2 f2_pack(float a, float b) {
  f2 r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
  return r;
}
__device__ __forceinline__ void f2_unpack(f2 v, float& a, float& b) {
  asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(v));
}
__device__ __forceinline__ f2 f2_splat(float a) { return f2_pack(a, a); }
__device__ __forceinline__ f2 f2_add(f2 a, f2 b) {
  f2 r;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
__device__ __forceinline__ f2 f2_sub(f2 a, f2 b) {
  f2 r;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
__device__ __forceinline__ f2 f2_mul(f2 a, f2 b) {
  f2 r;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
__device__ __forceinline__ f2 f2_fma(f2 a, f2 b, f2 c) {
  f2 r;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
  return r;
}
// a b - c and c - a b per half: two scalar FMAs, whose negated operand is
// free (a packed negation would cost two integer XORs on the ALU pipe, the
// busiest pipe of the two-float gathers)
__device__ __forceinline__ f2 f2_fms(f2 a, f2 b, f2 c) {
  float a0, a1, b0, b1, c0, c1;
  f2_unpack(a, a0, a1);
  f2_unpack(b, b0, b1);
  f2_unpack(c, c0, c1);
  return f2_pack(__fmaf_rn(a0, b0, -c0), __fmaf_rn(a1, b1, -c1));
}
__device__ __forceinline__ f2 f2_nfma(f2 a, f2 b, f2 c) {
  float a0, a1, b0, b1, c0, c1;
  f2_unpack(a, a0, a1);
  f2_unpack(b, b0, b1);
  f2_unpack(c, c0, c1);
  return f2_pack(__fmaf_rn(-a0, b0, c0), __fmaf_rn(-a1, b1, c1));
}

struct ff2 {
  f2 h, l;
};

__device__ __forceinline__ ff2 ff2_mul(ff2 a, ff2 b) {
  const f2 p = f2_mul(a.h, b.h);
  f2 e = f2_fms(a.h, b.h, p);
  e = f2_fma(a.h, b.l, e);
  e = f2_fma(a.l, b.h, e);
  return ff2{p, e};
}

__device__ __forceinline__ ff2 ff2_sqr(ff2 a) {
  const f2 p = f2_mul(a.h, a.h);
  f2 e = f2_fms(a.h, a.h, p);
  e = f2_fma(f2_add(a.h, a.h), a.l, e);
  return ff2{p, e};
}

__device__ __forceinline__ ff2 ff2_two_sum(f2 a, f2 b) {
  const f2 s = f2_add(a, b);
  const f2 bb = f2_sub(s, a);
  const f2 e = f2_add(f2_sub(a, f2_sub(s, bb)), f2_sub(b, bb));
  return ff2{s, e};
}

// pair_sep_ff of two pairs (i, j0) and (i, j1): a + b per axis and S + s.
template <bool ANISO>
__device__ __forceinline__ void pair_sep_ff2(const int4& xi, int lix, int liy, int liz,
                                             const int4& xj0, const int4& xj1, const float* uh,
                                             const float* ul, f2 (&a)[3], f2 (&b)[3], f2& S,
                                             f2& s) {
  int l0[3], l1[3];
  image_lo(xj0.w, l0[0], l0[1], l0[2]);
  image_lo(xj1.w, l1[0], l1[1], l1[2]);
  const int ci[3] = {xi.x, xi.y, xi.z}, c0[3] = {xj0.x, xj0.y, xj0.z},
            c1[3] = {xj1.x, xj1.y, xj1.z}, li[3] = {lix, liy, liz};
  const f2 fine = f2_splat(0.0009765625f);
  f2 p[3], e[3];
#pragma unroll
  for (int d = 0; d < 3; d++) {
    // sep_axis_ff of both pairs; the scaling of the fine part packed
    const int dh0 = wrap_sub(c0[d], ci[d]), dh1 = wrap_sub(c1[d], ci[d]);
    a[d] = f2_pack(__int2float_rn(dh0 & ~255), __int2float_rn(dh1 & ~255));
    b[d] = f2_mul(f2_pack(__int2float_rn(((dh0 & 255) << kFineBits) + (l0[d] - li[d])),
                          __int2float_rn(((dh1 & 255) << kFineBits) + (l1[d] - li[d]))),
                  fine);
    if (ANISO) {
      const f2 h = f2_splat(uh[d]), l = f2_splat(ul[d]);
      const f2 m = f2_mul(a[d], h);
      f2 t = f2_fms(a[d], h, m);
      t = f2_fma(b[d], h, t);
      t = f2_fma(a[d], l, t);
      a[d] = m;
      b[d] = t;
    }
    p[d] = f2_mul(a[d], a[d]);
    e[d] = f2_fms(a[d], a[d], p[d]);
    e[d] = f2_fma(f2_add(a[d], a[d]), b[d], e[d]);
    e[d] = f2_fma(b[d], b[d], e[d]);
  }
  const ff2 s1 = ff2_two_sum(p[0], p[1]);
  const ff2 s2 = ff2_two_sum(s1.h, p[2]);
  const f2 lo = f2_add(f2_add(e[0], e[1]), f2_add(e[2], f2_add(s1.l, s2.l)));
  S = f2_add(s2.h, lo);
  s = f2_sub(lo, f2_sub(S, s2.h));
}

// pair_g_ff of two pairs (the reciprocal seeds are scalar MUFU operations).
template <bool ANISO>
__device__ __forceinline__ ff2 pair_g_ff2(f2 S, f2 s_lo, float kh, float kl) {
  float S0, S1, y0, y1;
  f2_unpack(S, S0, S1);
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y0) : "f"(S0));
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y1) : "f"(S1));
  const f2 y = f2_pack(y0, y1);
  f2 e = f2_nfma(S, y, f2_splat(1.0f));
  e = f2_nfma(s_lo, y, e);
  ff2 inv{y, f2_mul(y, e)};
  if (!ANISO) inv = ff2_mul(inv, ff2{f2_splat(kh), f2_splat(kl)});
  const ff2 i2 = ff2_sqr(inv);
  const ff2 i6 = ff2_mul(i2, inv);
  const f2 m2 = f2_splat(-2.0f);
  const f2 m = f2_mul(m2, i6.h);
  ff2 w = ff2_two_sum(f2_splat(1.0f), m);
  w.l = f2_fma(m2, i6.l, w.l);
  return ff2_mul(ff2_sqr(i2), w);
}

// term_parts of two pairs for one axis.
__device__ __forceinline__ void term_parts2(ff2 g, f2 a, f2 b, f2& p, f2& e) {
  p = f2_mul(g.h, a);
  e = f2_fms(g.h, a, p);
  e = f2_fma(g.h, b, e);
  e = f2_fma(g.l, a, e);
}

}  // namespace ljg
