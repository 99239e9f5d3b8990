// df32.cuh -- compensated single-precision arithmetic for the shape sums.
//
// A value is carried as an unevaluated sum h + l of two floats ("double-float",
// the error-free transformations of Knuth's TwoSum and the FMA product error;
// Dekker 1971, Ogita-Rump-Oishi 2005).  The pair kernels use it for the
// per-pair terms of the fields whose sums cancel (e+, ex, e++, exx, e+x,
// kappa): their bin sums are orders of magnitude smaller than the sum of the
// terms' magnitudes, so a plain float term (2^-24 relative) would leave errors
// near 1e-6 of the bin value, while h + l carries about 2^-44.
//
// Every function is usable on the host (g++ with -ffp-contract=off, where fmaf
// is the correctly rounded fused multiply-add of the C library) and on the
// device, where the sums and products whose rounding the transformations
// depend on use the _rn intrinsics, which the compiler never contracts into an
// FMA.
#pragma once

#include <math.h>
#include <stdint.h>
#include <string.h>

#ifdef __CUDACC__
#define DF_HD __host__ __device__ __forceinline__
#else
#define DF_HD inline
#endif

namespace cpc {

struct df32 {
  float h, l;  // value h + l
};

DF_HD float rn_add(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fadd_rn(a, b);
#else
  return a + b;
#endif
}
DF_HD float rn_sub(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fsub_rn(a, b);
#else
  return a - b;
#endif
}
DF_HD float rn_mul(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fmul_rn(a, b);
#else
  return a * b;
#endif
}
DF_HD float rn_fma(float a, float b, float c) {
#ifdef __CUDA_ARCH__
  return __fmaf_rn(a, b, c);
#else
  return fmaf(a, b, c);
#endif
}

// s + e == a + b exactly (TwoSum: no condition on the magnitudes)
DF_HD df32 two_sum(float a, float b) {
  const float s = rn_add(a, b);
  const float bb = rn_sub(s, a);
  const float e = rn_add(rn_sub(a, rn_sub(s, bb)), rn_sub(b, bb));
  return {s, e};
}
DF_HD df32 two_diff(float a, float b) { return two_sum(a, -b); }

// p + e == a * b exactly
DF_HD df32 two_prod(float a, float b) {
  const float p = rn_mul(a, b);
  return {p, rn_fma(a, b, -p)};
}

// (a.h + a.l)(b.h + b.l); dropped: a.l b.l and the roundings of the low part
DF_HD df32 df_mul(df32 a, df32 b) {
  const float p = rn_mul(a.h, b.h);
  float e = rn_fma(a.h, b.h, -p);
  e = rn_fma(a.h, b.l, e);
  e = rn_fma(a.l, b.h, e);
  return {p, e};
}
// (a.h + a.l) b for a float b
DF_HD df32 df_mulf(df32 a, float b) {
  const float p = rn_mul(a.h, b);
  float e = rn_fma(a.h, b, -p);
  e = rn_fma(a.l, b, e);
  return {p, e};
}
DF_HD df32 df_add(df32 a, df32 b) {
  const df32 s = two_sum(a.h, b.h);
  return {s.h, rn_add(s.l, rn_add(a.l, b.l))};
}
DF_HD df32 df_sub(df32 a, df32 b) {
  const df32 s = two_sum(a.h, -b.h);
  return {s.h, rn_add(s.l, rn_sub(a.l, b.l))};
}
// (ah + al) - (bh + bl) for two values held as float hi and lo parts (positions
// that are not float32 values), renormalised: close pairs of such positions
// have a lo difference comparable to the hi difference
DF_HD df32 df_diff_hl(float ah, float al, float bh, float bl) {
  const df32 d = two_diff(ah, bh);
  return two_sum(d.h, rn_add(d.l, rn_sub(al, bl)));
}
// exact scaling by a power of two
DF_HD df32 df_scale(df32 a, float p2) { return {rn_mul(a.h, p2), rn_mul(a.l, p2)}; }

// Rotation of the ellipticity (e1, e2) by 2 theta, given c = cos 2theta and
// s = sin 2theta (calcs.cpp:60-64): e+ = c e1 - s e2, ex = s e1 + c e2.
// e1, e2, c and s are double-floats.
DF_HD void df_rotate(df32 c, df32 s, df32 e1, df32 e2, df32 &ep, df32 &ex) {
  const df32 a = two_prod(c.h, e1.h), b = two_prod(s.h, e2.h);
  const df32 p = two_prod(s.h, e1.h), q = two_prod(c.h, e2.h);
  const df32 d = two_diff(a.h, b.h), t = two_sum(p.h, q.h);
  float ld = rn_add(d.l, rn_sub(a.l, b.l));
  ld = rn_fma(c.h, e1.l, ld);
  ld = rn_fma(c.l, e1.h, ld);
  ld = rn_fma(-s.h, e2.l, ld);
  ld = rn_fma(-s.l, e2.h, ld);
  float lt = rn_add(t.l, rn_add(p.l, q.l));
  lt = rn_fma(s.h, e1.l, lt);
  lt = rn_fma(s.l, e1.h, lt);
  lt = rn_fma(c.h, e2.l, lt);
  lt = rn_fma(c.l, e2.h, lt);
  ep = {d.h, ld};
  ex = {t.h, lt};
}

// cos 2theta and sin 2theta of the line joining a pair, theta = atan(dy / dx)
// (angle_orient_axis_PB, calcs.cpp:54-57): c = (dx^2 - dy^2) / q,
// s = 2 dx dy / q, q = dx^2 + dy^2 (exact identities; the quadrant of atan does
// not matter for the doubled angle).  dx, dy are double-floats, q > 0.  The
// quotients start from an approximate reciprocal of q (a few ulps) and are
// completed by one residual step each: c = c0 + (C - c0 q) / q.
DF_HD float approx_rcp(float q) {
#ifdef __CUDA_ARCH__
  return __fdividef(1.0f, q);
#else
  return 1.0f / q;
#endif
}
DF_HD void df_cos_sin_2theta(df32 dx, df32 dy, df32 &c, df32 &s) {
  const float dlx2 = rn_add(dx.l, dx.l), dly2 = rn_add(dy.l, dy.l);
  const float A = rn_mul(dx.h, dx.h);
  const float Al = rn_fma(dx.h, dlx2, rn_fma(dx.h, dx.h, -A));  // dx^2 = A + Al
  const float B = rn_mul(dy.h, dy.h);
  const float Bl = rn_fma(dy.h, dly2, rn_fma(dy.h, dy.h, -B));  // dy^2 = B + Bl
  const float dx2 = rn_add(dx.h, dx.h);
  const float M = rn_mul(dx2, dy.h);                             // 2 dx dy = M + Ml
  float Ml = rn_fma(dx2, dy.h, -M);
  Ml = rn_fma(dx2, dy.l, Ml);
  Ml = rn_fma(dlx2, dy.h, Ml);
  const df32 C = two_diff(A, B), Q = two_sum(A, B);
  const float Cl = rn_add(C.l, rn_sub(Al, Bl)), Ql = rn_add(Q.l, rn_add(Al, Bl));
  const float r = approx_rcp(Q.h);
  const float c0 = rn_mul(C.h, r);
  float rc = rn_add(rn_fma(-c0, Q.h, C.h), Cl);
  rc = rn_fma(-c0, Ql, rc);
  c = {c0, rn_mul(rc, r)};
  const float s0 = rn_mul(M, r);
  float rs = rn_add(rn_fma(-s0, Q.h, M), Ml);
  rs = rn_fma(-s0, Ql, rs);
  s = {s0, rn_mul(rs, r)};
}

// Fixed-point conversion of a double-float term: u = rint((h + l) 2^S), for
// |h + l| 2^S < 2^30 and a normalised-enough pair (|l| 2^S < 2^21); qs = 2^S.
// Only float adds, FMAs and integer ops (no conversion instructions): the
// integer parts are read from the mantissa of x + 1.5 2^23.
DF_HD int magic_int(float x_plus_magic) {
  int32_t i;
#ifdef __CUDA_ARCH__
  i = __float_as_int(x_plus_magic);
#else
  memcpy(&i, &x_plus_magic, 4);
#endif
  return i - 0x4B400000;
}
DF_HD int df_to_int(df32 v, float qs) {
  const float kM = 12582912.0f;  // 1.5 * 2^23
  const float t = rn_mul(v.h, qs);                      // exact (power of two)
  const float a = rn_fma(t, 3.0517578125e-05f, kM);     // t 2^-15 + M: rint(t 2^-15) + M
  const float hf = rn_sub(a, kM);                       // rint(t 2^-15)
  const float lo = rn_fma(hf, -32768.0f, t);            // t - hf 2^15, exact, |lo| <= 2^14
  const float lo2 = rn_fma(v.l, qs, lo);                // + l 2^S
  const float b = rn_add(lo2, kM);
  return magic_int(a) * 32768 + magic_int(b);           // rint((h + l) 2^S)
}
// The same as a 15-bit low word (0 .. 2^15 - 1) and the arithmetic shift
// u >> 15, for |h + l| 2^S < 2^29 - 2^17 (the shared-memory histograms).
DF_HD void df_to_fixed15(df32 v, float qs, unsigned &lo15, unsigned &hi) {
  const int u = df_to_int(v, qs);
  lo15 = (unsigned)u & 0x7FFFu;
  hi = (unsigned)(u >> 15);
}
// the same for a float term (one rounding conversion)
DF_HD void f_to_fixed15(float v, float qs, unsigned &lo15, unsigned &hi) {
#ifdef __CUDA_ARCH__
  const int u = __float2int_rn(v * qs);
#else
  const int u = (int)rintf(v * qs);
#endif
  lo15 = (unsigned)u & 0x7FFFu;
  hi = (unsigned)(u >> 15);
}

}  // namespace cpc
