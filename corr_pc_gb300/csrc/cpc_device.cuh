// cpc_device.cuh -- device-side data layout and the exact FP64 pair evaluation.
//
// Data layout in HBM (per uploaded catalogue, "slot"), all in cell-list order
// (sorted by column, jackknife region, then z):
//   pos  float4 (x, y, z, w)          16 B  -- the fast kernel's only hot stream
//   shp  float4 (e1, e2, phi, e3)     16 B  -- ED orientation
//   ewt  float4 (w e1, w e2 hi; lo)   16 B  -- compensated shape terms
//   aux  float4 (x lo, y lo, phi, w lo) 16 B -- read for binned pairs with shapes
//   keep uint8  jk_prob >= 0.5         1 B
//   xd,yd,zd,wd,e1d,e2d,phid double   56 B  -- FP64 edge recheck only
//   jk   int32 region label            4 B
//   orig int64 original row index      8 B  -- row subsampling only
// plus the compact list of non-empty (column, region) buckets.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "pair_values.h"

namespace cpc {

constexpr int kNF = 13;        // wt, d1v, d1e, ..., d6v, d6e
constexpr int kMaxRp = 64;     // r_p bins supported
constexpr int kMaxPi = 128;    // Pi bins supported
constexpr int kMaxSlots = 8;

// corel functions (initialization.cpp:490-538): density_density, shape_density,
// shape_shape (estimator 0 branch / other estimators), density_convergence,
// shape_convergence, ED_corel
enum Corel {
  COREL_DD = 0, COREL_SD = 1, COREL_SS = 2, COREL_SSA = 3,
  COREL_DK = 4, COREL_SK = 5, COREL_ED = 6
};
// the corel uses the orientation angle of the pair (angle_orient_axis)
__host__ __device__ inline bool corel_has_theta(int c) {
  return c == COREL_SD || c == COREL_SS || c == COREL_SSA || c == COREL_SK;
}
static_assert(kNF == kPairFields, "field count");

// double-precision catalogue view (recheck and plain FP64 kernel)
struct DCat {
  int64_t n;
  const double *x, *y, *z, *w, *e1, *e2, *phi;
  const double *e3;      // third orientation component (ED_corel)
  const int32_t *jk;
  const uint8_t *keep;
  const int64_t *orig;
  const uint8_t *aflag;  // corels1 scan starts of this row (kAuto* bits)
};

// single-precision cell-list view (fast kernel)
struct FCat {
  int64_t n;
  const float4 *pos;
  const float4 *shp;  // e1, e2, phi, e3 (ED orientation)
  const float4 *ewt;  // w e1, w e2 as float hi parts, then their lo parts
  const float4 *aux;  // x - (float)x, y - (float)y (non-float32 inputs), phi,
                      // w - (float)w
  const float *zlo;   // z - (float)z (non-float32 inputs)
  const float *zf;
  const uint8_t *keep;
  const uint8_t *aflag;  // corels1 scan starts of this row (kAuto* bits)
  // non-empty buckets (column-major, region-minor)
  const int *bk_start, *bk_end, *bk_region;
  const float *bk_zmin, *bk_zmax;
  const int *col_begin, *col_end;  // per column: range into the bucket list
};

// sky catalogue (coordinates 0) in redshift order: d.x = RA and d.y = Dec in
// degrees, d.z = redshift, plus the per-galaxy quantities the pair loop reads
struct SkyView {
  DCat d;
  const double *dc, *da;     // comoving (Pi) and transverse (r_p) distance
  const double *sd, *cd;     // sin and cos of Dec in radians (host libm)
  const double *rar, *decr;  // RA and Dec in radians (degrees / r2d)
  const double *win;         // per-row windows, 6 blocks of n: z_min, z_max,
                             // ra_min, ra_max, dec_min, dec_max (host libm)
};

// float views of a sky catalogue for the fast kernel (hi = float(v),
// lo = float(v - hi), so hi + lo carries about 48 bits of v)
struct SkyFast {
  const float4 *su;  // unit vector (cos d cos a, cos d sin a, sin d) hi parts, D_A
  const float4 *sl;  // unit vector lo parts, D_C lo part
  const float4 *sw;  // RA, Dec hi parts, redshift, D_C hi part
  const float4 *sx;  // RA, Dec lo parts, Dec in radians, weight
  const float4 *ss;  // w e1, w e2 hi parts, then their lo parts
  const float4 *sh;  // cos(Dec / 2) hi, lo, sin(Dec / 2) hi, lo (Dec in radians)
  const float2 *sp;  // phi, w lo part
};

struct JobDev {
  FCat f1, f2;  // g1 (outer rows) and g2 after the swap rule
  DCat d1, d2;  // same catalogues, FP64, cell order
  int corel, gws, which_corr, estimator, do_jk, n_jk;
  int periodic, coordinates, nrp, npi, wpi, lin_bin;
  int box_same_keep;        // 1 for the box (jk_check_PB), 0 for the sky
  int auto_mode;            // 0 corels2; corels1: 1 unsorted, 2 z-sorted scan
  int has_lo;               // positions are not float32-exact: use hi+lo for theta
  int rmu;                  // coordinates 7: bins of r = |(dx, dy, Pi)| and mu = Pi / r
  int all_exact;            // fast kernel: every window candidate to the FP64 path
                            // (the cell-list FP64 comparison engine)
  int twin;                 // fast kernel: g1 and g2 hold the same galaxies in the
                            // same order (a cross term of a catalogue with itself):
                            // each unordered pair is tested once and adds both
                            // orders (g1 = i, g2 = j) and (g1 = j, g2 = i)
  int ncx, ncy;
  int64_t row_stride, row_offset;
  // ---- fast-path single precision constants ----
  float Lf;
  float xy_in, xy_out;                 // definite window bounds on max(|dx|,|dy|)
  float pi_in_lo, pi_in_hi, pi_out_lo, pi_out_hi;
  float inv_ps_f, tp0;                 // approximate Pi bin: floor(dz*inv_ps + tp0)
  float l2rmin2, inv_lw;               // log2(r_min^2), 1/(log2 width in r^2)
  float rmin_f, inv_rsize_f;           // linear-bin estimate
  float rej_lo, rej_hi;                // definite r^2 rejection bounds
  float mu_rel, mu_abs;                // coordinates 7: mu-bin margin mu_rel r + mu_abs (dz units)
  float qscale[kNF];                   // per-field fixed-point scale 2^S_f
  int qbias;                           // fixed-point bound: |v_f| 2^S_f <= qbias
  int unit_w;                          // every weight is 1: wt_num = count
  float A[kMaxRp], B[kMaxRp];          // definite r^2 band of r_p bin k
  float PA[kMaxPi], PB[kMaxPi];        // definite Pi band of Pi bin k
  // ---- FP64 exact constants ----
  double L, rmin, rmax, pmin, pmax, ps, rsize;
  double wz_lo, wz_hi;                 // z window offsets: p_min, p_max (coordinates 6)
                                       // or -r_max, r_max (coordinates 7)
  double inv_qscale[kNF];
  double thr[kMaxRp + 1];              // exact r_p thresholds (host libm)
  // ---- outputs ----
  unsigned long long *acc_num;         // [n_hist][nrp][npi]
  double *acc_sums;                    // [n_hist][nrp][npi][kNF]
  unsigned long long *counters;        // [0] window (fast), [1] window (recheck), [2] rechecked
  // sky fast path: fixed-point sums in the layout of acc_sums, each as a low
  // word (sum of the terms' low 15 bits) and a high word (sum of term >> 15)
  unsigned long long *acc_fix, *acc_fixh;
  SkyView sky1, sky2;                  // sky catalogues g1, g2 (FP64 path of the fast kernel)
  SkyFast sf1, sf2;                    // their float views (fast sky kernel)
  const int *row_list;                 // sky row sample: the g1 rows counted, else null
  int64_t n_rows;                      // rows in row_list
  int2 *hq;                            // sky host-tier queue of this job
  unsigned long long *hq_n;            // its length
};

// corels1 (corr.cpp:103-216).  The scan of row i starts at j = i + 1 (j = 0 for
// the +1 z image when the data are sorted) and, sorted, stops at its first
// redshift failure: an image contributes nothing when its first scanned row
// already fails the lower bound.  Per row: whether that first row passes, for
// the 0, -1 and +1 z images.
constexpr uint8_t kAutoStart0 = 1, kAutoStartM = 2, kAutoStartP = 4;

// Whether corels1 counts (i, j) in z image sz: auto_mode 1 (unsorted) j > i;
// auto_mode 2 (sorted) the +1 image every j if its scan start passes, the 0
// and -1 images j > i if theirs does.
__host__ __device__ inline bool auto_image_all(int auto_mode, int sz, uint8_t af) {
  return auto_mode == 0 || (auto_mode == 2 && sz == 1 && (af & kAutoStartP));
}
__host__ __device__ inline bool auto_image_gt(int auto_mode, int sz, uint8_t af) {
  if (auto_mode == 1) return true;
  if (auto_mode != 2 || sz == 1) return false;
  return (af & (sz == 0 ? kAutoStart0 : kAutoStartM)) != 0;
}

struct UnitDesc {
  int job;
  int g1_start, g1_count, g1_stride;  // tile rows g1_start + q*g1_stride, q < g1_count
  int region;      // jackknife region of every g1 row in the tile (0 without jk)
  int n2_base;     // first Pi bin of the block-local window
  int cx_lo, cx_hi, cy_lo, cy_hi;  // neighbour columns (may run past the grid: periodic wrap)
  double zlo, zhi; // candidate range of the shifted z2 + L*sz
};

struct QEntry {
  int job, i1, j2, shift;  // shift code: (sx+1) + 3*(sy+1) + 9*(sz+1), | kWindowCounted
};
constexpr int kShiftMask = 31;
constexpr int kWindowCounted = 32;  // the fast path already counted this window pair

__host__ __device__ inline int shift_code(int sx, int sy, int sz) {
  return (sx + 1) + 3 * (sy + 1) + 9 * (sz + 1);
}
__host__ __device__ inline void shift_decode(int c, int &sx, int &sy, int &sz) {
  sx = c % 3 - 1;
  sy = (c / 3) % 3 - 1;
  sz = c / 9 - 1;
}

// ---------------------------------------------------------------------------
// Binning of one window pair with the reference's double arithmetic (no
// contraction into FMA: explicit _rn intrinsics, same operation order):
// corel_bin (corels.cpp:21-46) with pi_calc_PB / rp_calc_PB (PB_calcs.cpp:87-98)
// and, for coordinates 7, r_mu_calc (calcs.cpp:135-140): r = sqrt(r_p^2 + Pi^2)
// from the already rounded r_p, mu = Pi / r in place of Pi.  The r (or r_p) bin
// comes from the host-computed exact thresholds of floor(log10(r/r_min)/r_size).
// Returns 1 for a window pair outside the bins, 2 binned (n1, n2 set).
// ---------------------------------------------------------------------------
__device__ inline int exact_bin(const JobDev &J, double x1, double y1, double z1, double x2s,
                                double y2s, double z2s, int &n1, int &n2) {
  double dP = __dsub_rn(z2s, z1);
  const double t0 = __dsub_rn(x1, x2s), t1 = __dsub_rn(y1, y2s);
  double rp = __dsqrt_rn(__dadd_rn(__dmul_rn(t0, t0), __dmul_rn(t1, t1)));
  if (J.rmu) {
    rp = __dsqrt_rn(__dadd_rn(__dmul_rn(rp, rp), __dmul_rn(dP, dP)));
    dP = __ddiv_rn(dP, rp);
  }
  const double v2 = floor(__ddiv_rn(__dsub_rn(dP, J.pmin), J.ps));
  if (!(v2 >= 0.0) || v2 >= (double)J.npi) return 1;
  int k1;
  if (J.lin_bin) {
    const double v1 = floor(__ddiv_rn(__dsub_rn(rp, J.rmin), J.rsize));
    if (!(v1 >= 0.0) || v1 >= (double)J.nrp) return 1;
    k1 = (int)v1;
  } else {
    if (!(rp >= J.thr[0]) || rp >= J.thr[J.nrp]) return 1;
    int lo = 0, hi = J.nrp;  // thr[lo] <= rp < thr[hi]
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (rp >= J.thr[mid]) lo = mid; else hi = mid;
    }
    k1 = lo;
  }
  n1 = k1;
  n2 = (int)v2;
  return 2;
}

// Exact evaluation of one (g1, g2, image) triple: window predicates of
// PB_calcs.cpp:12-61 (lim_calc_xyz, lim_calc_PB: z window [z1 + p_min, z1 +
// p_max], or [z1 - r_max, z1 + r_max] for coordinates 7) and corr.cpp:67-86,
// then exact_bin.  Returns: 0 not a window pair, 1 window pair outside the
// bins, 2 binned.
__device__ inline int exact_classify(const JobDev &J, const DCat &g1, int64_t i,
                                     const DCat &g2, int64_t j, int sx, int sy, int sz,
                                     int &n1, int &n2) {
  const double x1 = g1.x[i], y1 = g1.y[i], z1 = g1.z[i];
  const double x2 = g2.x[j], y2 = g2.y[j], z2 = g2.z[j];
  // lim_calc_xyz / lim_calc_PB
  const double z_max = __dadd_rn(z1, J.wz_hi), z_min = __dadd_rn(z1, J.wz_lo);
  const double ra_max = __dadd_rn(x1, J.rmax), ra_min = __dsub_rn(x1, J.rmax);
  const double dec_max = __dadd_rn(y1, J.rmax), dec_min = __dsub_rn(y1, J.rmax);
  if (J.periodic) {
    if (sz == 1 && !(z_max > J.L)) return 0;
    if (sz == -1 && !(z_min < 0)) return 0;
    if (sx == 1 && !(ra_max > J.L)) return 0;
    if (sx == -1 && !(ra_min < 0)) return 0;
    if (sy == 1 && !(dec_max > J.L)) return 0;
    if (sy == -1 && !(dec_min < 0)) return 0;
  } else if (sx | sy | sz) {
    return 0;
  }
  const double Lsx = J.L * sx, Lsy = J.L * sy, Lsz = J.L * sz;  // exact (s in -1..1)
  const double z2s = __dadd_rn(z2, Lsz);
  if (z2s > z_max || z2s < z_min) return 0;
  const double y2s = __dadd_rn(y2, Lsy);
  if (y2s > dec_max || y2s < dec_min) return 0;
  const double x2s = __dadd_rn(x2, Lsx);
  if (x2s < ra_min || x2s > ra_max) return 0;
  return exact_bin(J, x1, y1, z1, x2s, y2s, z2s, n1, n2);
}

// Per-pair accumulator values in double (corels.cpp:48-262; calcs.cpp 54-64,
// 97-105; PB_calcs.cpp:101-134) for a binned pair of the box in image (sx, sy,
// sz): theta from the raw, un-shifted positions (angle_orient_axis_PB), the ED
// separation g1 - (g2 + L*shift) (ED_calc_PB).  f[0..12] as in the output
// layout.
__device__ inline void exact_values(const JobDev &J, const DCat &g1, int64_t i, const DCat &g2,
                                    int64_t j, int sx, int sy, int sz, double f[kNF]) {
  const double wt = __dmul_rn(g1.w[i], g2.w[j]);
  double theta = 0.0;
  if (corel_has_theta(J.corel)) theta = atan((g2.y[j] - g1.y[i]) / (g2.x[j] - g1.x[i]));
  double sep[3] = {0.0, 0.0, 0.0};
  if (J.corel == COREL_ED) {
    sep[0] = __dsub_rn(g1.x[i], __dadd_rn(g2.x[j], J.L * sx));
    sep[1] = __dsub_rn(g1.y[i], __dadd_rn(g2.y[j], J.L * sy));
    sep[2] = __dsub_rn(g1.z[i], __dadd_rn(g2.z[j], J.L * sz));
  }
  pair_values(J.corel, J.gws, wt, theta, PairGal{g1.e1[i], g1.e2[i], g1.phi[i], g1.e3[i]},
              PairGal{g2.e1[j], g2.e2[j], g2.phi[j], g2.e3[j]}, f, sep);
}

// Add one binned pair (FP64 values) to the global accumulators, including the
// jackknife attribution of corel_jk (jk.cpp:201-223 with jk_check_PB / _sky).
__device__ inline void exact_accumulate(const JobDev &J, const DCat &g1, int64_t i,
                                        const DCat &g2, int64_t j, int n1, int n2,
                                        const double f[kNF]) {
  const int64_t cell = (int64_t)n1 * J.npi + n2;
  const int64_t hstride = (int64_t)J.nrp * J.npi;
  atomicAdd(&J.acc_num[cell], 1ull);
  double *s = J.acc_sums + cell * kNF;
  for (int q = 0; q < kNF; q++)
    if (f[q] != 0.0) atomicAdd(&s[q], f[q]);
  if (!J.do_jk) return;
  const int r1 = g1.jk[i], r2 = g2.jk[j];
  int k1 = g1.keep[i], k2 = g2.keep[j];
  if (r1 == r2) {
    if (J.box_same_keep) k1 = 1;
    k2 = 0;
  }
  const int rs[2] = {r1, r2};
  const int ks[2] = {k1, k2};
  for (int t = 0; t < 2; t++) {
    if (!ks[t]) continue;
    const int64_t hc = (int64_t)(1 + rs[t]) * hstride + cell;
    atomicAdd(&J.acc_num[hc], 1ull);
    double *sj = J.acc_sums + hc * kNF;
    if (f[0] != 0.0) atomicAdd(&sj[0], f[0]);
    if (J.which_corr == 0) continue;
    for (int q = 1; q < kNF; q += 2)
      if (f[q] != 0.0) atomicAdd(&sj[q], f[q]);
  }
}

}  // namespace cpc
