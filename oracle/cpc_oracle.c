/*
 * cpc_oracle.c -- CPU restatement of corr_pc's pair-counting hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker for the GPU library and
 * the timed CPU baseline: it is imported only by tests/, the smoke check and
 * the CPU-baseline arm of bench.py.  The product never links or calls it.
 *
 * It restates, in plain C and in double precision with the same operation
 * order as the reference, what `corels2` (corr.cpp:219-459) computes for one
 * pair type:
 *   - the swap rule and shape-holder choice   corr.cpp:226-296
 *   - periodic-box windows and image flags    PB_calcs.cpp:12-61
 *   - sky windows                             sky_calcs.cpp:77-81,105-196
 *   - the image loops and z-sorted scan       corr.cpp:350-423, 67-86
 *   - per-pair binning                        corels.cpp:21-46, PB_calcs.cpp:87-98,
 *                                             calcs.cpp:126-132, sky_calcs.cpp:24-31,91-96
 *   - density/shape accumulators              corels.cpp:48-77,122-244, calcs.cpp:54-105
 *   - convergence and ED accumulators         corels.cpp:79-120,246-262, PB_calcs.cpp:101-134
 *   - r-mu binning (coordinates 7)            calcs.cpp:135-140, PB_calcs.cpp:12-28
 *   - jackknife attribution                   jk.cpp:53-71,138-171,201-223
 * with OpenMP threads over the outer rows and thread-private histograms
 * merged at the end (corr.cpp:329-442), as the reference does.
 *
 * Output: RAW per-region sums (before the delete-one conversion
 * final_jk_bins, jk.cpp:74-81, which the caller applies), laid out as
 *   num [h][i_rp][k_pi]                 int64   (p_bin.num)
 *   sums[h][i_rp][k_pi][CPC_NF]         double  (wt_num, data[1..6].val/err)
 * with h = 0 the full sample and h = 1 + r jackknife region r.  The 1-D r_p
 * count b[i].num equals the sum over k of p_bin.num (every binned pair
 * increments both, corels.cpp:67-71, jk.cpp:139-142).
 *
 * Differences from the reference, all documented:
 *   - the z-sorted scan starts at a binary-searched index instead of the
 *     thread's monotone pointer (corr.cpp:361-408).  Identical results
 *     whenever every Pi window holds at least one partner; the reference's
 *     pointer can skip the rest of a thread's rows after an empty window,
 *     which depends on the OpenMP schedule and is not reproduced.
 *   - a galaxy without ellipticities is treated as e = (0, 0) (the reference
 *     reads an uninitialised pointer there, corels.cpp:216-219).
 *   - sig_crit (lensing) and coordinates other than 0, 6 and 7 (periodic) are
 *     rejected.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define CPC_NF 13 /* wt, d1v,d1e, d2v,d2e, d3v,d3e, d4v,d4e, d5v,d5e, d6v,d6e */

enum { ORC_SD = 0, ORC_SRD = 1, ORC_DRS = 2, ORC_RSRD = 3, ORC_RSRS = 4, ORC_SRS = 5, ORC_SS = 6 };
enum { COREL_DD = 0, COREL_SD = 1, COREL_SS = 2, COREL_DK = 4, COREL_SK = 5, COREL_ED = 6 };

typedef struct {
  int64_t n;
  const double *x, *y, *z;   /* box: x y z; sky: ra_deg dec_deg redshift */
  const double *w;           /* NULL: 1 */
  const double *e1, *e2;     /* NULL: no shapes (0) */
  const double *phi;         /* NULL: -10 (read_dat.cpp:269) */
  const int32_t *jk;         /* NULL: -1 */
  const double *jk_prob;     /* NULL: 0 */
  const double *include_prob;/* NULL: 0 */
  const double *dc, *da;     /* sky: comoving / transverse distance per galaxy */
  const double *e3;          /* NULL: 0 (third ED orientation component, e[2]) */
} orc_cat;

typedef struct {
  int which_corr, coordinates, estimator, periodic_box, data_sorted;
  int do_jk, n_jk, lin_bin, n_bins, n_p_bin, sig_crit;
  double bin_r_min, bin_r_max, p_min, p_max, box;
  double include_prob_rr;                 /* include_prob_RR (initialization.cpp:403-405) */
  /* sky */
  double z_max_data, dz, z_sep_max;
  const double *H_z, *dA_z; int64_t n_table;
  int n_threads;
  int64_t row_stride, row_offset;         /* outer-row subsample (1, 0 = all rows) */
} orc_params;

static const double r2d = 180.0 / M_PI;

typedef struct {
  int corel, g_with_shape, swapped;
  double include_prob_max;
} job_t;

/* corr.cpp:226-296 and initialization.cpp:699-752 (choose_corel_func),
 * initialization.cpp:806-808 (include_prob_max). */
static int setup_job(const orc_params *p, int kind, int64_t n1, int64_t n2, job_t *j) {
  int gws = 0;
  switch (kind) {
    case ORC_DRS: gws = 0; if (p->coordinates == 2 || p->coordinates == 4) gws = 1; break;
    case ORC_RSRD: gws = 0; if (p->coordinates == 2 || p->coordinates == 4) gws = 2; break;
    case ORC_RSRS: gws = 0; if (p->coordinates == 2 || p->coordinates == 4) gws = 1; break;
    case ORC_SRD: case ORC_SD: case ORC_SRS: gws = 2; break;
    default: return -1;
  }
  int corel;
  if (kind == ORC_RSRS || kind == ORC_RSRD) corel = COREL_DD;
  else if (p->which_corr == 0) corel = COREL_DD;
  else if (p->which_corr == 1) corel = COREL_SD;
  else if (p->which_corr == 2) corel = (kind == ORC_SD) ? COREL_SS : COREL_SD;
  else if (p->which_corr == 3) corel = COREL_DK;
  else if (p->which_corr == 4) corel = COREL_SK;
  else if (p->which_corr == 5) corel = COREL_ED;
  else return -1;
  j->corel = corel;
  j->swapped = 0;
  if (n2 > n1) { /* corr.cpp:281-296 */
    j->swapped = 1;
    if (gws == 2) gws = 1; else if (gws == 1) gws = 2;
  }
  j->g_with_shape = gws;
  j->include_prob_max = (kind == ORC_RSRS || kind == ORC_RSRD) ? p->include_prob_rr : 1.0;
  return 0;
}

/* per-thread scratch: one full histogram set (like calc_temp.bjk) */
typedef struct {
  int64_t *num;
  double *sums;
  int64_t n_total, n_out;
} hist_t;

typedef struct {
  double z_min, z_max, ra_min, ra_max, dec_min, dec_max;
  int PBx, PBy, PBz;
} window_t;

/* PB_calcs.cpp:12-28 (lim_calc_xyz) and :30-61 (lim_calc_PB) */
static void lim_box(const orc_params *p, double x1, double y1, double z1, window_t *w) {
  w->PBx = w->PBy = w->PBz = 0;
  if (p->coordinates < 3 || p->coordinates == 6) {
    w->z_max = z1 + p->p_max;
    w->z_min = z1 + p->p_min;
  } else {
    w->z_max = z1 + p->bin_r_max;
    w->z_min = z1 - p->bin_r_max;
  }
  w->ra_max = x1 + p->bin_r_max;
  w->ra_min = x1 - p->bin_r_max;
  w->dec_max = y1 + p->bin_r_max;
  w->dec_min = y1 - p->bin_r_max;
  if (!p->periodic_box) return;
  if (w->z_min < 0) w->PBz = -1;
  if (w->z_max > p->box) w->PBz = abs(w->PBz) + 1;
  if (w->ra_min < 0) w->PBx = -1;
  if (w->ra_max > p->box) w->PBx = abs(w->PBx) + 1;
  if (w->dec_min < 0) w->PBy = -1;
  if (w->dec_max > p->box) w->PBy = abs(w->PBy) + 1;
}

/* sky_calcs.cpp:77-81 p_to_dz, :71-75 dAR_to_dA */
static double p_to_dz(const orc_params *p, double pp, double z) {
  int i = (int)floor(z / p->dz);
  return pp * (p->H_z[i] + ((p->H_z[i + 1] - p->H_z[i]) * (z - p->dz * i) / p->dz)) / 300000.0;
}
static double dar_to_da(const orc_params *p, double dar, double z) {
  int i = (int)floor(z / p->dz);
  return dar / (p->dA_z[i] + ((p->dA_z[i + 1] - p->dA_z[i]) * (z - p->dz * i) / p->dz));
}

/* sky_calcs.cpp:150-196 (lim_calc_sky, default case) and :105-145 */
static int lim_sky(const orc_params *p, double ra1, double dec1, double z1, window_t *w) {
  double dec1_rad = dec1 / r2d;
  w->PBx = w->PBy = w->PBz = 0;
  w->z_max = z1 + p->z_sep_max;
  w->z_max = z1 + p_to_dz(p, p->p_max, w->z_max);
  w->z_min = z1 + p_to_dz(p, p->p_min, z1);
  if (w->z_min < 0.001) w->z_min = 0.001;
  if (w->z_min > p->z_max_data) return -1; /* the reference exits here */
  double da_max = dar_to_da(p, p->bin_r_max, w->z_min);
  double ra_lim = acos((pow(cos(da_max), 1) - pow(sin(dec1_rad), 2)) / pow(cos(dec1_rad), 2)) * 1.02 * r2d;
  w->ra_max = ra1 + ra_lim;
  w->ra_min = ra1 - ra_lim;
  if (w->ra_max > 360) { w->ra_min = 0; }
  if (w->ra_min < 0) { w->ra_max = 360; }
  w->dec_max = dec1 + da_max * r2d * 1.05;
  w->dec_min = dec1 - da_max * r2d * 1.05;
  return 0;
}

static inline double absolute(double v) { return v < 0 ? -1 * v : v; }

/* calcs.cpp:97-105 */
static inline double ephi(double phi, double theta) {
  double t = absolute(phi - theta);
  if (t > M_PI / 2.0) t = M_PI - t;
  return t;
}

typedef struct {
  const orc_params *p;
  const job_t *job;
  const orc_cat *g1, *g2;
  double p_size, r_size;
  int n_hist;
} ctx_t;

static inline double cat_w(const orc_cat *c, int64_t i) { return c->w ? c->w[i] : 1.0; }
static inline double cat_e1(const orc_cat *c, int64_t i) { return c->e1 ? c->e1[i] : 0.0; }
static inline double cat_e2(const orc_cat *c, int64_t i) { return c->e2 ? c->e2[i] : 0.0; }
static inline double cat_phi(const orc_cat *c, int64_t i) { return c->phi ? c->phi[i] : -10.0; }
static inline double cat_e3(const orc_cat *c, int64_t i) { return c->e3 ? c->e3[i] : 0.0; }
static inline int cat_jk(const orc_cat *c, int64_t i) { return c->jk ? c->jk[i] : -1; }
static inline double cat_jkp(const orc_cat *c, int64_t i) { return c->jk_prob ? c->jk_prob[i] : 0.0; }

/* one window pair: corel_jk (jk.cpp:201-223) -> corel -> corel_bin.
 * returns 1 when the pair falls outside the bins ("pairs out"). */
static int corel_pair(const ctx_t *c, hist_t *h, int64_t i, int64_t j, int PBx, int PBy, int PBz) {
  const orc_params *p = c->p;
  const orc_cat *g1 = c->g1, *g2 = c->g2;
  double d_P, da_R;
  /* corel_bin corels.cpp:21-46 */
  if (p->coordinates != 0) {
    /* pi_calc_PB / rp_calc_PB, PB_calcs.cpp:87-98 */
    d_P = ((g2->z[j] + p->box * PBz) - g1->z[i]);
    double t0 = g1->x[i] - (g2->x[j] + p->box * PBx);
    double t1 = g1->y[i] - (g2->y[j] + p->box * PBy);
    da_R = sqrt(t0 * t0 + t1 * t1);
    if (p->coordinates == 7) { /* r_mu_calc calcs.cpp:135-140 */
      da_R = sqrt(da_R * da_R + d_P * d_P);
      d_P /= da_R;
    }
  } else {
    /* pi_calc calcs.cpp:126-132; rp_calc_sky sky_calcs.cpp:91-96; dA_calc :24-31 */
    d_P = g2->dc[j] - g1->dc[i];
    double d1 = g1->y[i] / r2d, d2 = g2->y[j] / r2d;
    double a1 = g1->x[i] / r2d, a2 = g2->x[j] / r2d;
    double sum = sin(d1) * sin(d2) + cos(d1) * cos(d2) * cos((a1 - a2));
    double da = (sum > 0.9999999999) ? acos(1.0) : acos(sum);
    da_R = da * (g1->da[i] + g2->da[j]) / 2.;
  }
  double v2 = floor((d_P - p->p_min) / c->p_size);
  if (!(v2 >= 0) || v2 >= p->n_p_bin) return 1;
  double v1;
  if (p->lin_bin) v1 = floor((da_R - p->bin_r_min) / c->r_size);
  else v1 = floor(log10(da_R / p->bin_r_min) / c->r_size);
  if (!(v1 >= 0) || v1 >= p->n_bins) return 1;
  int n1 = (int)v1, n2 = (int)v2;
  double wt = cat_w(g1, i) * cat_w(g2, j);

  double f[CPC_NF];
  memset(f, 0, sizeof f);
  f[0] = wt;
  int corel = c->job->corel, gws = c->job->g_with_shape;
  if (corel == COREL_DK) { /* density_convergence_corel corels.cpp:79-90, sig_crit 1 */
    if (gws == 1) f[1] = wt * cat_e1(g1, i) * 1.0;
    else if (gws == 2) f[1] = wt * cat_e1(g2, j) * 1.0;
  } else if (corel == COREL_ED) { /* ED_corel corels.cpp:246-262, ED_calc_PB PB_calcs.cpp:101-134 */
    double xyz[3];
    xyz[0] = g1->x[i] - (g2->x[j] + p->box * PBx);
    xyz[1] = g1->y[i] - (g2->y[j] + p->box * PBy);
    xyz[2] = g1->z[i] - (g2->z[j] + p->box * PBz);
    double xyz_norm = sqrt(xyz[0] * xyz[0] + xyz[1] * xyz[1] + xyz[2] * xyz[2]);
    double cos_ang;
    if (gws == 2)
      cos_ang = cat_e1(g2, j) * xyz[0] + cat_e2(g2, j) * xyz[1] + cat_e3(g2, j) * xyz[2];
    else
      cos_ang = cat_e1(g1, i) * xyz[0] + cat_e2(g1, i) * xyz[1] + cat_e3(g1, i) * xyz[2];
    cos_ang /= xyz_norm;
    f[11] = cos_ang * cos_ang;
    f[12] = pow(f[11], 2.0);
  } else if (corel != COREL_DD) {
    double theta;
    if (p->coordinates != 0) /* calcs.cpp:54-57 (raw, un-shifted positions) */
      theta = atan((g2->y[j] - g1->y[i]) / (g2->x[j] - g1->x[i]));
    else /* sky_calcs.cpp:13-22 */
      theta = atan((g2->y[j] - g1->y[i]) /
                   ((g2->x[j] - g1->x[i]) * cos((g1->y[i] / r2d + g2->y[j] / r2d) / 2.0)));
    double c2 = cos(2.0 * theta), s2 = sin(2.0 * theta);
    if (corel == COREL_SK) { /* shape_convergence_corel corels.cpp:92-120, sig_crit 1 */
      if (gws == 1 || gws == 2) {
        const orc_cat *gs = (gws == 2) ? g2 : g1, *gk = (gws == 2) ? g1 : g2;
        int64_t is = (gws == 2) ? j : i, ik = (gws == 2) ? i : j;
        double en0 = c2 * cat_e1(gs, is) - s2 * cat_e2(gs, is); /* elip_rotate calcs.cpp:60-64 */
        double en1 = s2 * cat_e1(gs, is) + c2 * cat_e2(gs, is);
        double ep = wt * cat_e1(gk, ik) * 1.0;
        f[1] = ep;
        f[5] = ep * en0;
        f[9] = ep * en1;
      }
    } else if (corel == COREL_SD) { /* corels.cpp:206-244 */
      const orc_cat *gs = (gws == 2) ? g2 : g1;
      int64_t is = (gws == 2) ? j : i;
      double e0 = cat_e1(gs, is), e1 = cat_e2(gs, is);
      double ep = c2 * e0 - s2 * e1, ex = s2 * e0 + c2 * e1; /* calcs.cpp:60-64 */
      f[1] = 1.0 * wt * ep;
      f[2] = pow(wt * ep, 2);
      f[3] = 1.0 * wt * ex;
      f[4] = pow(wt * ex, 2);
      double et = ephi(cat_phi(g1, i), theta);
      f[11] = et;
      f[12] = pow(et, 2.0);
    } else { /* corels.cpp:122-204 */
      double ei0 = c2 * cat_e1(g1, i) - s2 * cat_e2(g1, i);
      double ei1 = s2 * cat_e1(g1, i) + c2 * cat_e2(g1, i);
      double ej0 = c2 * cat_e1(g2, j) - s2 * cat_e2(g2, j);
      double ej1 = s2 * cat_e1(g2, j) + c2 * cat_e2(g2, j);
      if (p->estimator == 0 || p->coordinates == 2 || p->coordinates == 4) {
        if (gws == 2) {
          f[1] = 1.0 * wt * (ej0);
          f[2] = pow(wt * ej0, 2);
          double et = ephi(cat_phi(g2, j), theta);
          f[11] = et;
          f[12] = pow(et, 2.0);
        } else if (gws == 1) {
          f[1] = 1.0 * wt * (ei0);
          f[2] = pow(wt * ei0, 2);
          double et = ephi(cat_phi(g1, i), theta);
          f[11] = et;
          f[12] = pow(et, 2.0);
        }
        /* e-cross stays 0 here (never assigned in this branch) */
      } else {
        f[1] = 1.0 * wt * (ei0 + ej0) / 2.0;
        f[2] = pow(wt * ei0 / 2.0, 2) + pow(wt * ej0 / 2.0, 2);
        f[3] = 1.0 * wt * (ei1 + ej1) / 2.0;
        f[4] = pow(wt * ei1 / 2.0, 2) + pow(wt * ej1 / 2.0, 2);
        double et1 = ephi(cat_phi(g1, i), theta), et2 = ephi(cat_phi(g2, j), theta);
        f[12] = pow(et1, 2.0) + pow(et2, 2.0);
        f[11] = et1 + et2;
      }
      f[5] = 1.0 * wt * (ei0 * ej0);
      f[6] = pow(wt * (ei0 * ej0), 2);
      f[7] = 1.0 * wt * (ei1 * ej1);
      f[8] = pow(wt * (ei1 * ej1), 2);
      f[9] = 1.0 * wt * (ei1 * ej0 + ei0 * ej1) / 2.0;
      f[10] = pow(wt * (ei1 * ej0) / 2.0, 2) + pow(wt * ei0 * ej1 / 2.0, 2);
    }
  }
  int nb = p->n_bins, np = p->n_p_bin;
  int64_t cell = (int64_t)n1 * np + n2;
  h->num[cell]++;
  double *s = h->sums + cell * CPC_NF;
  for (int q = 0; q < CPC_NF; q++) s[q] += f[q];

  if (p->do_jk == 0) return 0;
  /* jk.cpp:201-223 with jk_check_PB (:64-71) or jk_check_sky (:53-57) */
  int r1 = cat_jk(g1, i), r2 = cat_jk(g2, j);
  double q1 = cat_jkp(g1, i), q2 = cat_jkp(g2, j);
  if (r1 == r2) {
    if (p->coordinates != 0) q1 = 1; /* jk_check_PB: periodic box or coordinates 6 */
    q2 = 0;
  }
  int rs[2] = {r1, r2};
  double qs[2] = {q1, q2};
  for (int t = 0; t < 2; t++) {
    if (qs[t] < 0.5) continue;
    int64_t hc = ((int64_t)(1 + rs[t]) * nb * np) + cell;
    h->num[hc]++;
    double *sj = h->sums + hc * CPC_NF;
    sj[0] += wt; /* jk.cpp:138-171: val fields only */
    if (p->which_corr == 0) continue;
    for (int q = 1; q < CPC_NF; q += 2) sj[q] += f[q];
  }
  return 0;
}

/* index of the first g2 row with (z + shift) >= zlo, g2 sorted by z */
static int64_t lower_bound_z(const double *z, int64_t n, double shift, double zlo) {
  int64_t lo = 0, hi = n;
  while (lo < hi) {
    int64_t mid = lo + (hi - lo) / 2;
    if (z[mid] + shift < zlo) lo = mid + 1; else hi = mid;
  }
  return lo;
}

/* corels2 (corr.cpp:219-459).  Returns 0 on success, <0 on invalid input.
 * counters[0] = window pairs ("total pair"), counters[1] = binned ("pairs in"). */
int orc_corels2(const orc_params *p, int kind, const orc_cat *ga, const orc_cat *gb,
                int64_t *num, double *sums, int64_t *counters) {
  if (p->sig_crit != 0) return -2;
  if (p->coordinates != 6 && p->coordinates != 0 && p->coordinates != 7) return -2;
  if (p->coordinates == 0 && p->periodic_box) return -2;
  if (p->coordinates == 7 && !p->periodic_box) return -2;
  if (p->coordinates == 0 && p->which_corr > 2) return -2;
  counters[0] = counters[1] = 0;
  job_t job;
  if (setup_job(p, kind, ga->n, gb->n, &job) != 0) return -1;
  if (ga->n == 0 || gb->n == 0) return 0; /* corr.cpp:273-277 */
  const orc_cat *g1 = job.swapped ? gb : ga, *g2 = job.swapped ? ga : gb;
  int n_hist = 1 + (p->do_jk ? p->n_jk : 0);
  if (p->do_jk) {
    for (int64_t t = 0; t < g1->n; t++) if (!g1->jk || g1->jk[t] < 0 || g1->jk[t] >= p->n_jk) return -3;
    for (int64_t t = 0; t < g2->n; t++) if (!g2->jk || g2->jk[t] < 0 || g2->jk[t] >= p->n_jk) return -3;
  }
  ctx_t c;
  c.p = p; c.job = &job; c.g1 = g1; c.g2 = g2; c.n_hist = n_hist;
  c.p_size = (p->p_max - p->p_min) / (p->n_p_bin); /* initialization.cpp:305 */
  if (p->lin_bin) c.r_size = (p->bin_r_max - p->bin_r_min) / p->n_bins;
  else c.r_size = (log10(p->bin_r_max) - log10(p->bin_r_min)) / p->n_bins;
  int64_t hsize = (int64_t)n_hist * p->n_bins * p->n_p_bin;
  memset(num, 0, sizeof(int64_t) * hsize);
  memset(sums, 0, sizeof(double) * hsize * CPC_NF);
  int64_t stride = p->row_stride > 0 ? p->row_stride : 1, off = p->row_offset;
  int nthr = p->n_threads;
#ifdef _OPENMP
  if (nthr <= 0) nthr = omp_get_num_procs();
#else
  nthr = 1;
#endif
  int err = 0;
  int64_t tot = 0, out = 0;
#ifdef _OPENMP
#pragma omp parallel num_threads(nthr) reduction(+ : tot, out)
#endif
  {
    hist_t h;
    h.num = (int64_t *)calloc(hsize, sizeof(int64_t));
    h.sums = (double *)calloc(hsize * CPC_NF, sizeof(double));
    h.n_total = h.n_out = 0;
    int64_t chunk = g1->n / (nthr * 40);
    if (chunk < 1) chunk = 1;
#ifdef _OPENMP
#pragma omp for schedule(dynamic, chunk)
#endif
    for (int64_t i = 0; i < g1->n; i++) {
      if (((i - off) % stride) != 0) continue;
      if (g1->include_prob && g1->include_prob[i] > job.include_prob_max) continue;
      window_t w;
      if (p->coordinates != 0) lim_box(p, g1->x[i], g1->y[i], g1->z[i], &w);
      else if (lim_sky(p, g1->x[i], g1->y[i], g1->z[i], &w) != 0) { err = 1; continue; }
      int xt = w.PBx, yt = w.PBy, zt = w.PBz;
      int PBy = yt > 0;
      for (int yi = 0; yi <= abs(yt); yi++, PBy--) {
        int PBx = xt > 0;
        for (int xi = 0; xi <= abs(xt); xi++, PBx--) {
          int PBz = zt > 0;
          for (int zi = 0; zi <= abs(zt); zi++, PBz--) {
            double sz = p->box * PBz, sy = p->box * PBy, sx = p->box * PBx;
            if (p->coordinates == 0) sz = sy = sx = 0;
            int64_t j = 0;
            int sorted = p->data_sorted == 1;
            if (sorted && PBz <= 0) j = lower_bound_z(g2->z, g2->n, sz, w.z_min);
            for (; j < g2->n; j++) {
              if (g2->include_prob && g2->include_prob[j] > job.include_prob_max) continue;
              /* do_pair_sorted / do_pair_unsorted corr.cpp:36-86 */
              double zz = g2->z[j] + sz;
              if (zz > w.z_max || zz < w.z_min) { if (sorted) break; continue; }
              double yy = g2->y[j] + sy;
              if (yy > w.dec_max || yy < w.dec_min) continue;
              double xx = g2->x[j] + sx;
              if (xx < w.ra_min || xx > w.ra_max) continue;
              h.n_out += corel_pair(&c, &h, i, j, PBx, PBy, PBz);
              h.n_total++;
            }
          }
        }
      }
    }
#ifdef _OPENMP
#pragma omp critical
#endif
    {
      for (int64_t t = 0; t < hsize; t++) num[t] += h.num[t];
      for (int64_t t = 0; t < hsize * CPC_NF; t++) sums[t] += h.sums[t];
    }
    tot += h.n_total;
    out += h.n_out;
    free(h.num);
    free(h.sums);
  }
  if (err) return -4;
  counters[0] = tot;
  counters[1] = tot - out;
  return 0;
}

/* corels1 (corr.cpp:103-216): pairs within one catalogue, each counted once.
 * For outer row i and each image (lim_calc as in corels2) the scan starts at
 * j = i + 1, except that with data_sorted != 0 the +1 z image starts at j = 0
 * (corr.cpp:171-178); with data_sorted 1 it stops at the first redshift
 * failure (do_pair_sorted, corr.cpp:67-86: ret_z), so an image whose first
 * scanned row already fails the lower redshift bound contributes nothing.
 * g_with_shape = 1 (corr.cpp:112); corel: do_RsRs -> density_density, do_SS ->
 * shape_shape for which_corr 1, 2 (initialization.cpp:490-520).
 * kind: ORC_SS (do_SS) or ORC_RSRS (do_RsRs). */
int orc_corels1(const orc_params *p, int kind, const orc_cat *g, int64_t *num, double *sums,
                int64_t *counters) {
  if (p->sig_crit != 0) return -2;
  if (p->coordinates != 6 && p->coordinates != 0 && p->coordinates != 7) return -2;
  if (p->coordinates == 0 && p->periodic_box) return -2;
  if (p->coordinates == 7 && !p->periodic_box) return -2;
  if (p->coordinates == 0 && p->which_corr > 2) return -2;
  counters[0] = counters[1] = 0;
  job_t job;
  job.swapped = 0;
  job.g_with_shape = 1;
  if (kind == ORC_RSRS) job.corel = COREL_DD;
  else if (kind == ORC_SS)
    job.corel = p->which_corr == 0 ? COREL_DD : p->which_corr <= 2 ? COREL_SS
              : p->which_corr == 3 ? COREL_DK : p->which_corr == 4 ? COREL_SK : COREL_ED;
  else return -1;
  job.include_prob_max = (kind == ORC_RSRS) ? p->include_prob_rr : 1.0;
  if (g->n == 0) return 0;
  int n_hist = 1 + (p->do_jk ? p->n_jk : 0);
  if (p->do_jk)
    for (int64_t t = 0; t < g->n; t++) if (!g->jk || g->jk[t] < 0 || g->jk[t] >= p->n_jk) return -3;
  ctx_t c;
  c.p = p; c.job = &job; c.g1 = g; c.g2 = g; c.n_hist = n_hist;
  c.p_size = (p->p_max - p->p_min) / (p->n_p_bin);
  if (p->lin_bin) c.r_size = (p->bin_r_max - p->bin_r_min) / p->n_bins;
  else c.r_size = (log10(p->bin_r_max) - log10(p->bin_r_min)) / p->n_bins;
  int64_t hsize = (int64_t)n_hist * p->n_bins * p->n_p_bin;
  memset(num, 0, sizeof(int64_t) * hsize);
  memset(sums, 0, sizeof(double) * hsize * CPC_NF);
  int64_t stride = p->row_stride > 0 ? p->row_stride : 1, off = p->row_offset;
  int nthr = p->n_threads;
#ifdef _OPENMP
  if (nthr <= 0) nthr = omp_get_num_procs();
#else
  nthr = 1;
#endif
  int err = 0;
  int64_t tot = 0, out = 0;
  const int64_t n = g->n;
#ifdef _OPENMP
#pragma omp parallel num_threads(nthr) reduction(+ : tot, out)
#endif
  {
    hist_t h;
    h.num = (int64_t *)calloc(hsize, sizeof(int64_t));
    h.sums = (double *)calloc(hsize * CPC_NF, sizeof(double));
    h.n_total = h.n_out = 0;
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 100)
#endif
    for (int64_t i = 0; i < n; i++) {
      if (((i - off) % stride) != 0) continue;
      if (g->include_prob && g->include_prob[i] > job.include_prob_max) continue;
      window_t w;
      if (p->coordinates != 0) lim_box(p, g->x[i], g->y[i], g->z[i], &w);
      else if (lim_sky(p, g->x[i], g->y[i], g->z[i], &w) != 0) { err = 1; continue; }
      int xt = w.PBx, yt = w.PBy, zt = w.PBz;
      int PBx = xt > 0;
      for (int xi = 0; xi <= abs(xt); xi++, PBx--) {
        int PBy = yt > 0;
        for (int yi = 0; yi <= abs(yt); yi++, PBy--) {
          int PBz = zt > 0;
          for (int zi = 0; zi <= abs(zt); zi++, PBz--) {
            double sz = p->box * PBz, sy = p->box * PBy, sx = p->box * PBx;
            if (p->coordinates == 0) sz = sy = sx = 0;
            int64_t j = i + 1;
            if (p->data_sorted != 0 && PBz > 0) j = 0;
            const int sorted = p->data_sorted == 1;
            for (; j < n; j++) {
              if (g->include_prob && g->include_prob[j] > job.include_prob_max) continue;
              double zz = g->z[j] + sz;
              if (zz > w.z_max || zz < w.z_min) { if (sorted) break; continue; }
              double yy = g->y[j] + sy;
              if (yy > w.dec_max || yy < w.dec_min) continue;
              double xx = g->x[j] + sx;
              if (xx < w.ra_min || xx > w.ra_max) continue;
              h.n_out += corel_pair(&c, &h, i, j, PBx, PBy, PBz);
              h.n_total++;
            }
          }
        }
      }
    }
#ifdef _OPENMP
#pragma omp critical
#endif
    {
      for (int64_t t = 0; t < hsize; t++) num[t] += h.num[t];
      for (int64_t t = 0; t < hsize * CPC_NF; t++) sums[t] += h.sums[t];
    }
    tot += h.n_total;
    out += h.n_out;
    free(h.num);
    free(h.sums);
  }
  if (err) return -4;
  counters[0] = tot;
  counters[1] = tot - out;
  return 0;
}

/* glibc random_r TYPE_3 additive-feedback generator, restated from its
 * published description (seed via 16807 LCG, 310 discarded outputs,
 * r[k] = r[k-31] + r[k-3], output r >> 1).  Used for the periodic-box
 * jackknife draws jk_prob = rand()/(RAND_MAX+1.) (read_dat.cpp:243) after
 * srand(124693517) (jk.cpp:40-43). */
void orc_glibc_rand(uint32_t seed, int64_t skip, int64_t n, int32_t *out) {
  int32_t r[34];
  uint32_t ring[34];
  r[0] = (int32_t)seed;
  if (seed == 0) r[0] = 1;
  for (int i = 1; i < 31; i++) {
    int64_t hi = r[i - 1] / 127773, lo = r[i - 1] % 127773;
    int64_t word = 16807 * lo - 2836 * hi;
    if (word < 0) word += 2147483647;
    r[i] = (int32_t)word;
  }
  for (int i = 31; i < 34; i++) r[i] = r[i - 31];
  for (int i = 0; i < 34; i++) ring[i] = (uint32_t)r[i];
  /* ring buffer of the last 34 values; position k holds r[k] */
  int64_t k = 34;
  uint32_t buf[34];
  memcpy(buf, ring, sizeof buf);
  int64_t total = 310 + skip + n;
  for (int64_t t = 0; t < total; t++, k++) {
    uint32_t v = buf[(k - 31) % 34] + buf[(k - 3) % 34];
    buf[k % 34] = v;
    int64_t o = t - 310 - skip;
    if (o >= 0) out[o] = (int32_t)(v >> 1);
  }
}

/* elip_angle (calcs.cpp:35-46, 73-83) with the C library's atan, as the
 * reference calls it: phi = 0.5*arctan(e1, -e2), quadrant-corrected, NaN -> 0. */
void orc_elip_angle(int64_t n, const double *e1, const double *e2, double *phi) {
  for (int64_t i = 0; i < n; i++) {
    const double x = e1[i], y = -1 * e2[i];
    double t = atan(y / x);
    if (x < 0) {
      if (y < 0) t -= M_PI;
      else t += M_PI;
    }
    double p = 0.5 * t;
    if (p != p) p = 0;
    phi[i] = p;
  }
}
