// pair_sky.cu -- sky pair loop (coordinates 0) on the GPU in double precision.
//
// The reference's sky path (corr.cpp:350-423 with lim_calc_sky and
// do_pair_sorted): for each g1 row a window in redshift, Dec and RA computed
// from the distance table (sky_calcs.cpp:105-196); g2 scanned in redshift
// order from the window's lower edge to its upper edge; Dec then RA tests;
// then corel_bin with Pi = DC2 - DC1 (calcs.cpp:126-132) and
// r_p = acos(sin d1 sin d2 + cos d1 cos d2 cos(a1 - a2)) (DA1 + DA2) / 2
// (sky_calcs.cpp:24-31, 91-96), and the jackknife rule jk_check_sky.
//
// Exactness.  The windows, sin/cos of Dec and the angles in radians are
// computed once per galaxy on the host with the C library (exactly the
// reference's values), so every window test and the Pi bin are exact here.
// Only cos(a1 - a2) and acos come from CUDA's math library, whose results can
// differ from the C library's by a few ulps; near sum = 1 acos amplifies that
// by 1/sin(theta).  Each pair gets a rigorous bound on the r_p difference
// (esum on the cosine sum, propagated through acos and the product) and every
// pair whose r_p lies within that bound of a bin threshold, or whose sum lies
// within esum of the reference's clamp at 0.9999999999, is appended to a host
// queue and binned there with the C library.  All other pairs are binned here
// against the exact host-derived thresholds, so the integer counts equal the
// reference's.  Shape sums use CUDA's atan/cos/sin (within 1e-6).
//
// Two kernels:
//  * sky_fp64_kernel -- the plain FP64 kernel: one thread per g1 row, every
//    window pair through the FP64 path, global atomics (CPC_ENGINE_FP64).
//  * sky_warp_kernel -- the fast kernel (CPC_ENGINE_FAST): one warp per g1 row
//    (dynamic row queue), lanes take consecutive candidates of the row's
//    redshift range, their float views prefetched into per-warp shared stages
//    with asynchronous copies one 32-candidate stage ahead; FP32 definite-in/definite-out
//    window tests (ambiguous ones re-tested in double); FP32 prefilters that
//    reject pairs certainly outside the Pi range or certainly outside
//    [thr_0, thr_nrp) in r_p (the chord |u1 - u2| of float unit vectors with a
//    rigorous error bound); survivors are compacted into a per-warp queue and
//    evaluated 32 at a time with every lane busy: Pi and r_p in FP32 from hi+lo
//    floats with per-pair error bounds, FP32 shape values when both bins are
//    certain, the FP64 path (and behind it the host tier) otherwise.  The main
//    histogram lives in shared memory (FP64 atomics) and is flushed once per
//    block.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <climits>

#include "cpc_device.cuh"
#include "kernels.h"
#include "pair_df.cuh"

namespace cpc {

// number of thresholds thr[0..nrp] that are <= v
__device__ inline int thr_count(const JobDev &J, double v) {
  if (!(v >= J.thr[0])) return 0;
  int lo = 0, hi = J.nrp + 1;  // thr[lo] <= v, thr[hi] > v (hi = nrp+1: none)
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (v >= J.thr[mid]) lo = mid; else hi = mid;
  }
  return lo + 1;
}

__global__ void __launch_bounds__(128)
sky_fp64_kernel(const JobDev *__restrict__ jobp, SkyView a, SkyView b, int2 *hq,
                unsigned long long *hq_n, unsigned long long hq_cap, double esum) {
  const JobDev &J = *jobp;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t n1 = a.d.n, n2 = b.d.n;
  if (i >= n1) return;
  if (J.row_stride > 1 && ((a.d.orig[i] - J.row_offset) % J.row_stride) != 0) return;
  // corels1: the scan from row i + 1 must pass the lower redshift bound (sorted)
  if (J.auto_mode == 2 && !(a.d.aflag[i] & kAutoStart0)) return;
  const int64_t oi = a.d.orig[i];
  const double z_min = a.win[i], z_max = a.win[n1 + i];
  const double ra_min = a.win[2 * n1 + i], ra_max = a.win[3 * n1 + i];
  const double dec_min = a.win[4 * n1 + i], dec_max = a.win[5 * n1 + i];
  const double ra1 = a.d.x[i], dec1 = a.d.y[i];
  const double dc1 = a.dc[i], da1 = a.da[i], sd1 = a.sd[i], cd1 = a.cd[i];
  const double rar1 = a.rar[i], decr1 = a.decr[i];
  // first g2 row with redshift >= z_min
  int64_t lo = 0, hi = n2;
  while (lo < hi) {
    const int64_t mid = (lo + hi) >> 1;
    if (b.d.z[mid] < z_min) lo = mid + 1; else hi = mid;
  }
  const double kClamp = 0.9999999999;        // dA_calc (sky_calcs.cpp:28)
  const double kEps = 2.220446049250313e-16;  // 2^-52
  unsigned long long nwin = 0;
  for (int64_t j = lo; j < n2; j++) {
    const double z2 = b.d.z[j];
    if (z2 > z_max) break;
    if (J.auto_mode && !(b.d.orig[j] > oi)) continue;  // corels1: partners after row i
    const double dec2 = b.d.y[j];
    if (dec2 > dec_max || dec2 < dec_min) continue;
    const double ra2 = b.d.x[j];
    if (ra2 < ra_min || ra2 > ra_max) continue;  // NaN bounds pass, as in the reference
    nwin++;
    // Pi bin (exact)
    const double dP = __dsub_rn(b.dc[j], dc1);
    const double v2 = floor(__ddiv_rn(__dsub_rn(dP, J.pmin), J.ps));
    if (!(v2 >= 0.0) || v2 >= (double)J.npi) continue;
    // great-circle separation
    const double cdel = cos(__dsub_rn(rar1, b.rar[j]));
    const double sum = __dadd_rn(__dmul_rn(sd1, b.sd[j]), __dmul_rn(__dmul_rn(cd1, b.cd[j]), cdel));
    bool amb = fabs(sum - kClamp) <= esum;
    double daR = 0.0, tol = 0.0;
    if (!(sum > kClamp)) {
      const double th = acos(sum);
      daR = __ddiv_rn(__dmul_rn(th, __dadd_rn(da1, b.da[j])), 2.0);
      const double st = sin(th);
      // |d theta| <= esum / sin(theta) + a few ulps of theta (both acos)
      const double rel = esum / fmax(st * th, 1e-300) + 8.0 * kEps;
      tol = 2.0 * daR * rel;
    }
    const int k = thr_count(J, daR);
    if (!amb && tol > 0.0) amb = thr_count(J, daR - tol) != k || thr_count(J, daR + tol) != k;
    if (amb) {
      const unsigned long long q = atomicAdd(hq_n, 1ull);
      if (q < hq_cap) hq[q] = make_int2((int)i, (int)j);
      continue;
    }
    if (k < 1 || k > J.nrp) continue;
    // values (angle_orient_axis_sky, sky_calcs.cpp:13-22) and accumulation
    const double wt = __dmul_rn(a.d.w[i], b.d.w[j]);
    double theta = 0.0;
    if (J.corel != COREL_DD)
      theta = atan((dec2 - dec1) / ((ra2 - ra1) * cos((decr1 + b.decr[j]) / 2.0)));
    double f[kNF];
    pair_values(J.corel, J.gws, wt, theta, PairGal{a.d.e1[i], a.d.e2[i], a.d.phi[i]},
                PairGal{b.d.e1[j], b.d.e2[j], b.d.phi[j]}, f);
    exact_accumulate(J, a.d, i, b.d, j, k - 1, (int)v2, f);
  }
  if (nwin) atomicAdd(&J.counters[1], nwin);
}

// ---------------------------------------------------------------------------
// fast kernel
// ---------------------------------------------------------------------------

constexpr int kSkyThreads = 256;
constexpr int kSkyWarps = kSkyThreads / 32;
constexpr int kSkyQ = 64;
constexpr int kSkyAhead = 1;  // candidate stages copied ahead of the tested one

struct SkyRow {
  int64_t i;
  double ra, dec, dc, da, sd, cd, rar, decr, w, e1, e2, phi;
  int jk, keep;
};

// Jackknife attribution of a sky pair: jk_check_sky (jk.cpp:53-57), each
// region whose galaxy has jk_prob >= 0.5 (same region: g1's only).
__device__ __forceinline__ int sky_regions(int r1, int keep1, int r2, int keep2, int rs[2]) {
  int n = 0;
  if (keep1) rs[n++] = r1;
  if (r2 != r1 && keep2) rs[n++] = r2;
  return n;
}

// FP64 values of a pair from the FP64 path: global FP64 atomics (rare pairs),
// corel_jk1 (jk.cpp:138-171) for the regions.
__device__ __forceinline__ void sky_accumulate_exact(const JobDev &J, int r1, int keep1, int r2,
                                                     int keep2, int64_t cell,
                                                     const double f[kNF]) {
  const int nf = J.corel == COREL_DD ? 1 : kNF;
  atomicAdd(&J.acc_num[cell], 1ull);
  for (int q = 0; q < nf; q++)
    if (f[q] != 0) atomicAdd(&J.acc_sums[cell * kNF + q], f[q]);
  if (!J.do_jk) return;
  const int64_t hstride = (int64_t)J.nrp * J.npi;
  int rs[2];
  const int nr = sky_regions(r1, keep1, r2, keep2, rs);
  for (int t = 0; t < nr; t++) {
    const int64_t hc = (int64_t)(1 + rs[t]) * hstride + cell;
    atomicAdd(&J.acc_num[hc], 1ull);
    double *sj = J.acc_sums + hc * kNF;
    if (f[0] != 0) atomicAdd(&sj[0], f[0]);
    if (J.which_corr == 0 || nf == 1) continue;
    for (int q = 1; q < kNF; q += 2)
      if (f[q] != 0) atomicAdd(&sj[q], f[q]);
  }
}

// Terms of a pair from the mixed-precision path as fixed-point integers
// Add x (a term rint(v 2^S_f), or a block's partial sum of terms) to the
// global fixed-point sum of one bin and field: its low 15 bits (0 .. 2^15 - 1)
// into word lo, its arithmetic shift x >> 15 into word hi.  Terms have
// |x| < 2^30 and a block's partial sum holds fewer than 2^33 of them, so a bin
// takes 2^48 terms before either word can overflow; the value is
// hi 2^15 + lo (fix_to_sums_kernel).
__device__ __forceinline__ void fix_add(unsigned long long *lo, unsigned long long *hi,
                                        long long x) {
  const unsigned long long l = (unsigned long long)x & 0x7FFFull;
  const long long h = x >> 15;
  if (l) atomicAdd(lo, l);
  if (h) atomicAdd(hi, (unsigned long long)h);
}

// rint(v 2^S_f), |v| 2^S_f < 2^30 (S_f from bounds on |v|): the fields whose
// sums cancel from double-float terms vd, the others from float terms v; added
// as 64-bit integers: the main histogram in shared memory (SMEM) or in the
// global fixed-point block, the regions in the global fixed-point block.
// Field 0 (the weight) is skipped when every weight is 1 (wt_num = count).
template <bool SMEM>
__device__ __forceinline__ void sky_accumulate_fixed(const JobDev &J, int r1, int keep1, int r2,
                                                     int keep2, int64_t cell, const float *v,
                                                     const df32 *vd, int nf, const float *s_qs,
                                                     unsigned long long *s_num,
                                                     unsigned long long *s_fix) {
  const int f0 = J.unit_w ? 1 : 0;
  const int corel = J.corel;
  auto fx = [&](int q) {
    return (long long)(df_field(corel, q) ? df_to_int(vd[q], s_qs[q])
                                          : __float2int_rn(v[q] * s_qs[q]));
  };
  auto nz = [&](int q) { return df_field(corel, q) ? vd[q].h != 0.0f : v[q] != 0.0f; };
  atomicAdd(SMEM ? &s_num[cell] : &J.acc_num[cell], 1ull);
#pragma unroll
  for (int q = 0; q < kNF; q++) {  // constant indices: v stays in registers
    if (q < f0 || q >= nf || !nz(q)) continue;
    const int64_t o = cell * kNF + q;
    if (SMEM) atomicAdd(&s_fix[o], (unsigned long long)fx(q));
    else fix_add(&J.acc_fix[o], &J.acc_fixh[o], fx(q));
  }
  if (!J.do_jk) return;
  const int64_t hstride = (int64_t)J.nrp * J.npi;
  int rs[2];
  const int nr = sky_regions(r1, keep1, r2, keep2, rs);
  for (int t = 0; t < nr; t++) {
    const int64_t hc = (int64_t)(1 + rs[t]) * hstride + cell;
    atomicAdd(&J.acc_num[hc], 1ull);
    unsigned long long *sj = J.acc_fix + hc * kNF, *sh = J.acc_fixh + hc * kNF;
    if (f0 == 0 && v[0] != 0.0f) fix_add(&sj[0], &sh[0], fx(0));
    if (J.which_corr == 0 || nf == 1) continue;
#pragma unroll
    for (int q = 1; q < kNF; q += 2)
      if (nz(q)) fix_add(&sj[q], &sh[q], fx(q));
  }
}

// FP64 path of one window pair whose Pi and r_p may fall in the bins: exact
// Pi bin, great-circle r_p, ambiguity test, values and accumulation.
__device__ __noinline__ void sky_pair_fp64(const JobDev &J, int64_t i, int64_t j, int2 *hq,
                                           unsigned long long *hq_n, unsigned long long hq_cap,
                                           double esum) {
  const SkyView &a = J.sky1, &b = J.sky2;
  SkyRow r;
  r.i = i;
  r.ra = a.d.x[i]; r.dec = a.d.y[i]; r.dc = a.dc[i]; r.da = a.da[i];
  r.sd = a.sd[i]; r.cd = a.cd[i]; r.rar = a.rar[i]; r.decr = a.decr[i];
  r.w = a.d.w[i]; r.e1 = a.d.e1[i]; r.e2 = a.d.e2[i]; r.phi = a.d.phi[i];
  r.jk = a.d.jk[i]; r.keep = a.d.keep[i];
  const double dP = __dsub_rn(b.dc[j], r.dc);
  const double v2 = floor(__ddiv_rn(__dsub_rn(dP, J.pmin), J.ps));
  if (!(v2 >= 0.0) || v2 >= (double)J.npi) return;
  const double cdel = cos(__dsub_rn(r.rar, b.rar[j]));
  const double sum = __dadd_rn(__dmul_rn(r.sd, b.sd[j]), __dmul_rn(__dmul_rn(r.cd, b.cd[j]), cdel));
  const double kClamp = 0.9999999999;
  const double kEps = 2.220446049250313e-16;
  bool amb = fabs(sum - kClamp) <= esum;
  double daR = 0.0, tol = 0.0;
  if (!(sum > kClamp)) {
    const double th = acos(sum);
    daR = __ddiv_rn(__dmul_rn(th, __dadd_rn(r.da, b.da[j])), 2.0);
    const double rel = esum / fmax(sin(th) * th, 1e-300) + 8.0 * kEps;
    tol = 2.0 * daR * rel;
  }
  const int k = thr_count(J, daR);
  if (!amb && tol > 0.0) amb = thr_count(J, daR - tol) != k || thr_count(J, daR + tol) != k;
  if (amb) {
    const unsigned long long q = atomicAdd(hq_n, 1ull);
    if (q < hq_cap) hq[q] = make_int2((int)r.i, (int)j);
    return;
  }
  if (k < 1 || k > J.nrp) return;
  const double wt = __dmul_rn(r.w, b.d.w[j]);
  double theta = 0.0;
  if (J.corel != COREL_DD)
    theta = atan((b.d.y[j] - r.dec) / ((b.d.x[j] - r.ra) * cos((r.decr + b.decr[j]) / 2.0)));
  double f[kNF];
  pair_values(J.corel, J.gws, wt, theta, PairGal{r.e1, r.e2, r.phi},
              PairGal{b.d.e1[j], b.d.e2[j], b.d.phi[j]}, f);
  sky_accumulate_exact(J, r.jk, r.keep, b.d.jk[j], b.d.keep[j], (int64_t)(k - 1) * J.npi + (int)v2,
                       f);
}

// the row's float quantities for the mixed-precision path
struct SkyRowF {
  float4 u, ul, w, x, s, h;  // su, sl, sw, sx, ss, sh of the row
  float2 p;                  // sp of the row
};

// estimated bin index confirmed against definite bands: the bin, -1 certainly
// outside, -2 undecided.  band k is [lo_k, hi_k) in the estimate's units.
__device__ __forceinline__ int band_bin(float v, float tol, int est, int n, const float *lo,
                                        const float *hi, float rej_lo, float rej_hi) {
  if (v + tol < rej_lo || v - tol >= rej_hi) return -1;
  est = min(max(est, 0), n - 1);
  for (int d = 0; d < 3; d++) {
    const int k = d == 0 ? est : d == 1 ? est - 1 : est + 1;
    if (k < 0 || k >= n) continue;
    if (v - tol >= lo[k] && v + tol < hi[k]) return k;
  }
  return -2;
}

// Mixed-precision evaluation of a pair that may bin.  Pi from hi+lo float
// comoving distances, r_p = 2 asin(|u1 - u2| / 2) (D_A1 + D_A2) / 2 from hi+lo
// float unit vectors, each with a bound on its difference from the
// reference's double value; when both bins are certain the shape values are
// computed in FP32 and accumulated, otherwise the pair takes the FP64 path.
template <bool SMEM>
__device__ __forceinline__ void sky_pair_mixed(const JobDev &J, const SkyRow &r, const SkyRowF &rf,
                                               const SkyView &b, const SkyFast &fb, int64_t j,
                                               unsigned long long *s_num,
                                               unsigned long long *s_fix, const float *s_qs,
                                               int2 *hq, unsigned long long *hq_n,
                                               unsigned long long hq_cap, double esum,
                                               const float *s_A, const float *s_B,
                                               const float *s_PA, const float *s_PB) {
  const float4 w2 = fb.sw[j], l2 = fb.sl[j], u2 = fb.su[j];
  // every load of the pair issued before the first test: one memory round trip
  // instead of three (most queued pairs bin)
  const float4 x2 = fb.sx[j];
  const int jk2 = b.d.jk[j], keep2 = b.d.keep[j];
  float4 se2 = make_float4(0.f, 0.f, 0.f, 0.f), sh2 = se2;
  float2 sp2 = make_float2(0.f, 0.f);
  if (J.corel != COREL_DD) {
    se2 = fb.ss[j];
    sh2 = fb.sh[j];
    sp2 = fb.sp[j];
  }
  // Pi: (dc2_hi - dc1_hi) + (dc2_lo - dc1_lo); the bands carry the error bound
  const float pf = (w2.w - rf.w.w) + (l2.w - rf.ul.w);
  const int k2 = band_bin(pf, 0.0f, (int)floorf(fmaf(pf, J.inv_ps_f, J.tp0)), J.npi, s_PA, s_PB,
                          J.pi_out_lo, J.pi_out_hi);
  if (k2 == -1) return;
  // chord of the unit vectors, then theta and r_p
  const float dx = (rf.u.x - u2.x) + (rf.ul.x - l2.x);
  const float dy = (rf.u.y - u2.y) + (rf.ul.y - l2.y);
  const float dz = (rf.u.z - u2.z) + (rf.ul.z - l2.z);
  const float c2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
  const float c = sqrtf(c2);
  int k1 = -2;
  if (k2 >= 0 && c > 1.5e-5f) {  // below: near the clamp of dA_calc
    // |rp - rp_ref| / rp: float chord, asinf and D_A sum (< 6e-7), the double
    // unit vectors (3e-16 / c), and the reference's own sum = cos(theta)
    // rounding through acos (< 1.2e-15 / theta^2), each with margin
    const float rp = asinf(0.5f * c) * (rf.u.w + u2.w);
    // (approximate reciprocal: the factor 1.001 covers its few-ulp error)
    const float rc = __fdividef(1.0f, c);
    const float tol = rp * fmaf(4e-15f * rc, rc, fmaf(3e-14f, rc, 1.5e-6f)) * 1.001f;
    const int est = J.lin_bin ? (int)floorf((rp - J.rmin_f) * J.inv_rsize_f)
                              : (int)floorf((__log2f(rp * rp) - J.l2rmin2) * J.inv_lw);
    k1 = band_bin(rp, tol, est, J.nrp, s_A, s_B, J.rej_lo, J.rej_hi);
    if (k1 == -1) return;
  }
  if (k1 < 0 || k2 < 0) {
    sky_pair_fp64(J, r.i, j, hq, hq_n, hq_cap, esum);
    return;
  }
  // values: theta = atan(dDec / (dRA cos(mean Dec))) (sky_calcs.cpp:13-22)
  const float wt = rf.x.w * x2.w;
  const int64_t cell = (int64_t)k1 * J.npi + k2;
  if (J.corel == COREL_DD) {
    const float f0[1] = {wt};
    sky_accumulate_fixed<SMEM>(J, r.jk, r.keep, jk2, keep2, cell, f0, nullptr, 1, s_qs, s_num,
                               s_fix);
  } else {
    // the separation in RA and Dec (hi + lo degrees) and cos of the mean Dec,
    // cos(d1/2 + d2/2), as double-floats; X = dRA cos(mean Dec), Y = dDec
    const df32 dra = df_diff_hl(w2.x, x2.x, rf.w.x, rf.x.x);
    const df32 ddec = df_diff_hl(w2.y, x2.y, rf.w.y, rf.x.y);
    const df32 cm = df_sub(df_mul(df32{rf.h.x, rf.h.y}, df32{sh2.x, sh2.y}),
                           df_mul(df32{rf.h.z, rf.h.w}, df32{sh2.z, sh2.w}));
    const df32 X = df_mul(dra, cm);
    float v[kNF];
    df32 vd[kNF];
    for (int q = 0; q < kNF; q++) {
      v[q] = 0.0f;
      vd[q] = df32{0.0f, 0.0f};
    }
    v[0] = wt;
    if (X.h == 0.0f && ddec.h == 0.0f) {  // coincident on the sky: atan(0/0), the FP64 path
      sky_pair_fp64(J, r.i, j, hq, hq_n, hq_cap, esum);
      return;
    }
    df32 c, sn;
    df_cos_sin_2theta(X, ddec, c, sn);
    const float theta = atanf(__fdividef(ddec.h, X.h));
    const DfGal g1{{rf.s.x, rf.s.z}, {rf.s.y, rf.s.w}, {rf.x.w, rf.p.y}, rf.p.x};
    const DfGal g2{{se2.x, se2.z}, {se2.y, se2.w}, {x2.w, sp2.y}, sp2.x};
    const bool uw = J.unit_w != 0;
    if (J.corel == COREL_SD) df_pair_terms<COREL_SD>(c, sn, theta, g1, g2, J.gws, uw, vd, v);
    else if (J.corel == COREL_SS) df_pair_terms<COREL_SS>(c, sn, theta, g1, g2, J.gws, uw, vd, v);
    else df_pair_terms<COREL_SSA>(c, sn, theta, g1, g2, J.gws, uw, vd, v);
    sky_accumulate_fixed<SMEM>(J, r.jk, r.keep, jk2, keep2, cell, v, vd, kNF, s_qs, s_num,
                               s_fix);
  }
}

// 16-byte asynchronous copy global -> shared (the candidate prefetch below)
__device__ __forceinline__ void cp_async16(void *smem, const void *gmem) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
// all but the newest kSkyAhead groups complete: the current stage has landed
__device__ __forceinline__ void cp_async_wait_prev() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(kSkyAhead) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.wait_group 0;\n" ::: "memory");
}

// window membership of x in [lo, hi] from the float value: 1 in, 0 out,
// -1 undecided (x within a float ulp of a bound, or a NaN bound)
__device__ __forceinline__ int fwin(float x, float lo_ru, float hi_rd, float lo_rd, float hi_ru) {
  if (x > lo_ru && x < hi_rd) return 1;
  if (x < lo_rd || x > hi_ru) return 0;
  return -1;
}

// Rows are dealt in chunks of consecutive rows of one job (a pair type of the
// batch): a block takes a chunk, its warps take the chunk's rows one at a time,
// and the block meets at a barrier between chunks.  The block-private main
// histogram belongs to one job; when the next chunk belongs to another job
// (the chunks are numbered job after job, so a block switches at most
// n_jobs - 1 times) the block adds it to the previous job's global block and
// starts the next from zero.  A job's rows are every row of g1 or, for a row
// sample, the listed rows.
template <bool SMEM, int MINB>
__global__ void __launch_bounds__(kSkyThreads, MINB)
sky_warp_kernel(const JobDev *__restrict__ jobs, const long long *__restrict__ chunk0, int n_jobs,
                int rows_per_chunk, unsigned long long *chunk_ctr, unsigned long long hq_cap,
                double esum, float rp_lo_f, float rp_hi_f, int zero_bin) {
  extern __shared__ __align__(16) unsigned char sky_smem[];
  __shared__ int s_q[kSkyWarps][kSkyQ];
  // per warp, kSkyAhead + 1 stages of 32 candidates' sw and su views: the next
  // kSkyAhead stages are copied asynchronously while the current one is tested
  __shared__ float4 s_pw[kSkyWarps][kSkyAhead + 1][32], s_pu[kSkyWarps][kSkyAhead + 1][32];
  __shared__ SkyRowF s_rowf[kSkyWarps];
  __shared__ float s_A[kMaxRp], s_B[kMaxRp], s_PA[kMaxPi], s_PB[kMaxPi];
  __shared__ float s_qs[kNF];
  __shared__ long long s_chunk;
  __shared__ int s_rowctr, s_xmin, s_xmax;
  __shared__ unsigned long long s_red[kSkyWarps];
  const int ncell = jobs[0].nrp * jobs[0].npi;  // one binning for every job of a launch
  unsigned long long *s_num = reinterpret_cast<unsigned long long *>(sky_smem);
  unsigned long long *s_fix = s_num + ncell;
  const unsigned FULL = 0xffffffffu;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int *q = s_q[warp];
  int cur = -1;                 // the job whose histogram the block holds
  unsigned long long nwin = 0;  // window pairs of this thread's rows of job cur
  for (;;) {
    __syncthreads();  // every warp is done with the previous chunk
    if (threadIdx.x == 0) {
      s_chunk = (long long)atomicAdd(chunk_ctr, 1ull);
      s_rowctr = 0;
      s_xmin = INT_MAX;
      s_xmax = INT_MIN;
    }
    __syncthreads();
    const long long ch = s_chunk;
    int k = 0;
    while (k < n_jobs && ch >= chunk0[k + 1]) k++;  // block-uniform
    if (k != cur) {
      if (cur >= 0) {  // the previous job's window count (its histogram is flushed)
        const JobDev &P = jobs[cur];
        unsigned long long v = nwin;
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(FULL, v, o);
        if (lane == 0 && v) atomicAdd(&P.counters[1], v);
        nwin = 0;
      }
      if (k >= n_jobs) break;
      cur = k;
      const JobDev &N = jobs[k];
      for (int c = threadIdx.x; c < N.nrp; c += blockDim.x) { s_A[c] = N.A[c]; s_B[c] = N.B[c]; }
      for (int c = threadIdx.x; c < N.npi; c += blockDim.x) { s_PA[c] = N.PA[c]; s_PB[c] = N.PB[c]; }
      if (threadIdx.x < kNF) s_qs[threadIdx.x] = N.qscale[threadIdx.x];
      if (SMEM) {
        for (int c = threadIdx.x; c < ncell; c += blockDim.x) s_num[c] = 0ull;
        for (int c = threadIdx.x; c < ncell * kNF; c += blockDim.x) s_fix[c] = 0ull;
      }
      __syncthreads();  // bands, scales, zeroed histogram
    }
    const JobDev &J = jobs[k];
    const SkyView &a = J.sky1, &b = J.sky2;
    const SkyFast &fa = J.sf1, &fb = J.sf2;
    const int64_t n1 = a.d.n, n2 = b.d.n;
    const int64_t n_rows = J.row_list ? J.n_rows : n1;
    const int64_t r0 = (ch - chunk0[k]) * rows_per_chunk;
    const int64_t r1 = min(r0 + (int64_t)rows_per_chunk, n_rows);
    const float pmin_f = (float)J.pmin, pmax_f = (float)J.pmax;
    int2 *hq = J.hq;
    unsigned long long *hq_n = J.hq_n;
    // When every outer row of the chunk lies in one jackknife region xreg and is
    // kept (jk_prob >= 0.5), that region takes every pair the chunk adds to the
    // block histogram (jk_check_sky, jk.cpp:53-57): it receives the histogram
    // when the chunk ends, and the rows' pairs skip their own region update.
    // (The rows are ordered by redshift slab and region, so most chunks are.)
    int xreg = -1;
    if (SMEM && J.do_jk) {
      for (int64_t t = r0 + threadIdx.x; t < r1; t += blockDim.x) {
        const int64_t ii = J.row_list ? J.row_list[t] : t;
        const int reg = a.d.keep[ii] ? a.d.jk[ii] : -1;
        atomicMin(&s_xmin, reg);
        atomicMax(&s_xmax, reg);
      }
      __syncthreads();
      xreg = (s_xmin == s_xmax && s_xmin >= 0) ? s_xmin : -1;
    }
  for (;;) {
    int64_t i = 0;
    if (lane == 0) i = r0 + atomicAdd(&s_rowctr, 1);
    i = __shfl_sync(FULL, i, 0);
    if (i >= r1) break;
    if (J.row_list) i = J.row_list[i];
    if (J.auto_mode == 2 && !(a.d.aflag[i] & kAutoStart0)) continue;  // corels1, sorted
    const int64_t oi = a.d.orig[i];
    // the mixed path reads the row's index, region and keep flag; the FP64 path
    // reloads the rest by index
    SkyRow r;
    r.i = i;
    r.jk = a.d.jk[i];
    r.keep = xreg >= 0 ? 0 : a.d.keep[i];  // xreg: the region takes the chunk's histogram
    const double z_min = a.win[i], z_max = a.win[n1 + i];
    // RA / Dec windows: float bounds rounded both ways here; the exact double
    // bounds are reloaded in the rare undecided case (fewer live registers)
    const double *w_ra_min = a.win + 2 * n1 + i, *w_ra_max = a.win + 3 * n1 + i;
    const double *w_de_min = a.win + 4 * n1 + i, *w_de_max = a.win + 5 * n1 + i;
    const float ra_lru = __double2float_ru(*w_ra_min), ra_hrd = __double2float_rd(*w_ra_max);
    const float ra_lrd = __double2float_rd(*w_ra_min), ra_hru = __double2float_ru(*w_ra_max);
    const float de_lru = __double2float_ru(*w_de_min), de_hrd = __double2float_rd(*w_de_max);
    const float de_lrd = __double2float_rd(*w_de_min), de_hru = __double2float_ru(*w_de_max);
    const float4 u1 = fa.su[i];
    const float dc1f = fa.sw[i].w;
    // the row's float views for the heavy step, in this warp's shared slot
    SkyRowF &rf = s_rowf[warp];
    if (lane == 0) {
      rf.u = u1;
      rf.ul = fa.sl[i];
      rf.w = fa.sw[i];
      rf.x = fa.sx[i];
      rf.s = fa.ss[i];
      rf.h = fa.sh[i];
      rf.p = fa.sp[i];
    }
    __syncwarp();
    // redshift range [lo, hi): z_min <= z <= z_max
    int64_t lo = 0, hi = n2;
    while (lo < hi) {
      const int64_t mid = (lo + hi) >> 1;
      if (b.d.z[mid] < z_min) lo = mid + 1; else hi = mid;
    }
    int64_t end = n2, l2 = lo;
    while (l2 < end) {
      const int64_t mid = (l2 + end) >> 1;
      if (b.d.z[mid] > z_max) end = mid; else l2 = mid + 1;
    }
    int count = 0;
    // each lane prefetches its own candidate slot (no cross-lane reads of the
    // stage buffers): stage 0 now, stage k+1 while stage k is tested
    for (int a0 = 0; a0 < kSkyAhead; a0++) {
      const int64_t jp = lo + 32 * a0 + lane;
      if (jp < end) {
        cp_async16(&s_pw[warp][a0][lane], fb.sw + jp);
        cp_async16(&s_pu[warp][a0][lane], fb.su + jp);
      }
      cp_async_commit();
    }
    int stage = 0;
    for (int64_t base = lo; base < end; base += 32, stage = (stage + 1) % (kSkyAhead + 1)) {
      const int64_t j = base + lane;
      const int64_t jn = j + 32 * kSkyAhead;
      const int sn = (stage + kSkyAhead) % (kSkyAhead + 1);
      if (jn < end) {
        cp_async16(&s_pw[warp][sn][lane], fb.sw + jn);
        cp_async16(&s_pu[warp][sn][lane], fb.su + jn);
      }
      cp_async_commit();
      cp_async_wait_prev();  // this lane's copies of the current stage are done
      bool need = false;
      if (j < end && (!J.auto_mode || b.d.orig[j] > oi)) {  // corels1: partners after i
        const float4 w2 = s_pw[warp][stage][lane];
        int in = fwin(w2.y, de_lru, de_hrd, de_lrd, de_hru);
        if (in < 0) {
          const double d2 = b.d.y[j];
          in = !(d2 > *w_de_max || d2 < *w_de_min);
        }
        if (in) {
          int ir = fwin(w2.x, ra_lru, ra_hrd, ra_lrd, ra_hru);
          if (ir < 0) {
            const double a2 = b.d.x[j];
            ir = !(a2 < *w_ra_min || a2 > *w_ra_max);
          }
          in = ir;
        }
        if (in) {
          nwin++;
          // Pi certainly outside [p_min, p_max): float dc carry <= 1 ulp each
          const float pf = w2.w - dc1f;
          const float pe = 4.0f * 5.96e-8f * (fabsf(w2.w) + fabsf(dc1f)) + 1e-30f;
          const bool pi_out = (pf < pmin_f - pe) || (pf > pmax_f + pe);
          if (!pi_out) {
            // r_p bounds from the chord of float unit vectors
            const float4 u2 = s_pu[warp][stage][lane];
            const float dx = u1.x - u2.x, dy = u1.y - u2.y, dz = u1.z - u2.z;
            const float c2 = dx * dx + dy * dy + dz * dz;
            const float ch = sqrtf(c2);
            const float dsum = 0.5f * (u1.w + u2.w);
            const float ch_lo = fmaxf(ch * (1.0f - 1e-6f) - 4e-7f, 0.0f);
            const float ch_hi = ch * (1.0f + 1e-6f) + 4e-7f;
            const float rlo = ch_lo * dsum * (1.0f - 1e-6f);
            const float rhi = ch_hi * (1.0f + ch_hi * ch_hi * (1.0f / 6.0f)) * dsum * (1.0f + 1e-6f);
            // a clamped pair (theta < 1.41421e-5, r_p = 0) can bin when
            // thr_0 <= 0: never reject it as "above the range" then
            const bool above = rlo >= rp_hi_f && (!zero_bin || ch_lo > 1.5e-5f);
            need = !(above || rhi < rp_lo_f);
          }
        }
      }
      const unsigned m = __ballot_sync(FULL, need);
      if (need) q[count + __popc(m & ((1u << lane) - 1u))] = (int)j;
      count += __popc(m);
      __syncwarp();
      if (count >= 32) {
        sky_pair_mixed<SMEM>(J, r, rf, b, fb, q[lane], s_num, s_fix, s_qs, hq, hq_n, hq_cap, esum, s_A,
                             s_B, s_PA, s_PB);
        __syncwarp();
        if (lane < count - 32) q[lane] = q[lane + 32];
        count -= 32;
        __syncwarp();
      }
    }
    cp_async_wait_all();  // no copy in flight into the stage buffers of the next row
    if (lane < count)
      sky_pair_mixed<SMEM>(J, r, rf, b, fb, q[lane], s_num, s_fix, s_qs, hq, hq_n, hq_cap, esum, s_A,
                           s_B, s_PA, s_PB);
    __syncwarp();
  }  // rows of the chunk
    if (SMEM) {  // the chunk's block histogram into the job's main block (and region xreg)
      __syncthreads();
      const int64_t hx = xreg >= 0 ? (int64_t)(1 + xreg) * ncell : -1;
      const bool regf = J.which_corr != 0 && J.corel != COREL_DD;
      const bool wf = !J.unit_w;
      for (int c = threadIdx.x; c < ncell; c += blockDim.x) {
        const unsigned long long v = s_num[c];
        if (!v) continue;
        s_num[c] = 0ull;
        atomicAdd(&J.acc_num[c], v);
        if (hx >= 0) atomicAdd(&J.acc_num[hx + c], v);
        for (int f = 0; f < kNF; f++) {
          const long long x = (long long)s_fix[c * kNF + f];
          if (x == 0) continue;
          s_fix[c * kNF + f] = 0ull;
          const int64_t o = c * kNF + f, ox = (hx + c) * kNF + f;
          fix_add(&J.acc_fix[o], &J.acc_fixh[o], x);
          if (hx >= 0 && ((f == 0 && wf) || ((f & 1) && regf)))
            fix_add(&J.acc_fix[ox], &J.acc_fixh[ox], x);
        }
      }
    }
  }  // chunks
}

size_t sky_warp_smem_bytes(int nrp, int npi) {
  return (size_t)nrp * npi * (1 + kNF) * sizeof(unsigned long long);
}

// fixed-point block -> FP64 sums: sums[i] += (hi[i] 2^15 + lo[i]) 2^-S_f,
// f = i mod kNF (fix_add)
__global__ void fix_to_sums_kernel(int64_t n, const unsigned long long *__restrict__ lo,
                                   const unsigned long long *__restrict__ hi,
                                   double *__restrict__ sums, const JobDev *__restrict__ jobp) {
  const JobDev &J = *jobp;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const unsigned long long l = lo[i];
    const long long h = (long long)hi[i];
    if (l != 0 || h != 0)
      sums[i] += fma((double)h, 32768.0, (double)l) * J.inv_qscale[i % kNF];
  }
}

cudaError_t launch_fix_to_sums(int64_t n, const unsigned long long *lo,
                               const unsigned long long *hi, double *sums, const JobDev *job,
                               cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  const int64_t blocks = std::min<int64_t>((n + 255) / 256, 4096);
  fix_to_sums_kernel<<<(unsigned)blocks, 256, 0, st>>>(n, lo, hi, sums, job);
  return cudaGetLastError();
}

template <int MINB>
static cudaError_t launch_sky_warp_t(const JobDev *jobs, const long long *chunk0, int n_jobs,
                                     long long n_chunks, int rows_per_chunk,
                                     unsigned long long *chunk_ctr, unsigned long long hq_cap,
                                     double esum, float rp_lo_f, float rp_hi_f, int zero_bin,
                                     size_t smem, bool use_smem, int sm_count, cudaStream_t st) {
  int bps = 0;
  cudaError_t e;
  if (use_smem) {
    e = cudaFuncSetAttribute(sky_warp_kernel<true, MINB>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, sky_warp_kernel<true, MINB>,
                                                      kSkyThreads, smem);
  } else {
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, sky_warp_kernel<false, MINB>,
                                                      kSkyThreads, 0);
  }
  if (e != cudaSuccess) return e;
  if (bps < 1) bps = 1;
  const int grid = (int)std::min<long long>((long long)sm_count * bps, n_chunks);
  if (use_smem)
    sky_warp_kernel<true, MINB><<<grid, kSkyThreads, smem, st>>>(
        jobs, chunk0, n_jobs, rows_per_chunk, chunk_ctr, hq_cap, esum, rp_lo_f, rp_hi_f,
        zero_bin);
  else
    sky_warp_kernel<false, MINB><<<grid, kSkyThreads, 0, st>>>(
        jobs, chunk0, n_jobs, rows_per_chunk, chunk_ctr, hq_cap, esum, rp_lo_f, rp_hi_f,
        zero_bin);
  return cudaGetLastError();
}

cudaError_t launch_sky_warp(const JobDev *jobs, const long long *chunk0, int n_jobs,
                            long long n_chunks, int rows_per_chunk,
                            unsigned long long *chunk_ctr, unsigned long long hq_cap, double esum,
                            float rp_lo_f, float rp_hi_f, int zero_bin, int nrp, int npi,
                            int sm_count, int blocks_per_sm, cudaStream_t st) {
  if (n_jobs <= 0 || n_chunks <= 0) return cudaSuccess;
  const size_t smem = sky_warp_smem_bytes(nrp, npi);
  const bool use_smem = smem <= 100 * 1024;
  if (blocks_per_sm >= 3)  // 80 registers: more warps, a few spills
    return launch_sky_warp_t<3>(jobs, chunk0, n_jobs, n_chunks, rows_per_chunk, chunk_ctr,
                                hq_cap, esum, rp_lo_f, rp_hi_f, zero_bin, smem, use_smem,
                                sm_count, st);
  return launch_sky_warp_t<2>(jobs, chunk0, n_jobs, n_chunks, rows_per_chunk, chunk_ctr, hq_cap,
                              esum, rp_lo_f, rp_hi_f, zero_bin, smem, use_smem, sm_count, st);
}

cudaError_t launch_sky_fp64(const JobDev *job, const SkyView &a, const SkyView &b, int2 *hq,
                            unsigned long long *hq_n, unsigned long long hq_cap, double esum,
                            cudaStream_t st) {
  const int64_t blocks = (a.d.n + 127) / 128;
  if (blocks == 0) return cudaSuccess;
  sky_fp64_kernel<<<(unsigned)blocks, 128, 0, st>>>(job, a, b, hq, hq_n, hq_cap, esum);
  return cudaGetLastError();
}

}  // namespace cpc
