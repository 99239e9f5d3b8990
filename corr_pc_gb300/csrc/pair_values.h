// pair_values.h -- accumulator values of one binned pair, in double precision,
// shared by the device code (CUDA trigonometry) and the host edge tier (the C
// library's trigonometry, as the reference calls it).
//
// Given the orientation angle theta of the line joining the pair
// (angle_orient_axis_PB calcs.cpp:54-57 for the box, angle_orient_axis_sky
// sky_calcs.cpp:13-22 for the sky) and the product weight wt = w1 w2, fill the
// 13 output fields  wt_num, data[1..6].val / data[1..6].err  as
//   shape_density_corel  corels.cpp:206-244  (COREL_SD)
//   shape_shape_corel    corels.cpp:122-204  (COREL_SS: estimator 0 branch,
//                                             e-cross never assigned;
//                                             COREL_SSA: the other estimators)
//   density_convergence_corel corels.cpp:79-90  (COREL_DK: data[1] += w kappa)
//   shape_convergence_corel   corels.cpp:92-120 (COREL_SK: kappa of the other
//                                               galaxy times the rotated e)
//   ED_corel                  corels.cpp:246-262 with ED_calc_PB
//                                               (PB_calcs.cpp:101-134)
// with the rotation of calcs.cpp:60-64 and the folded angle |phi - theta| of
// ephi_calc (calcs.cpp:97-105).  kappa is read into e[0] (read_dat.cpp:300-304),
// so it is e1 here; the ED orientation is (e1, e2, e3), normalised at read
// (read_dat.cpp:282-293).  sep is the shifted separation g1 - (g2 + L*PB)
// that ED_calc_PB projects (ED only).  The convergence weights take the
// reference's default sig_crit = 1 (initialization.cpp:787).
#pragma once

#ifdef __CUDACC__
#define CPC_HD __host__ __device__
#else
#define CPC_HD
#endif

#include <math.h>

namespace cpc {

constexpr int kPairFields = 13;

struct PairGal {
  double e1, e2, phi, e3 = 0.0;
};

CPC_HD inline void pair_values(int corel, int gws, double wt, double theta, const PairGal &g1,
                               const PairGal &g2, double f[kPairFields],
                               const double *sep = nullptr) {
  for (int q = 0; q < kPairFields; q++) f[q] = 0.0;
  f[0] = wt;
  if (corel == 0) return;
  if (corel == 4) {  // only the shape holder's kappa is assigned
    if (gws == 1) f[1] = wt * g1.e1;
    else if (gws == 2) f[1] = wt * g2.e1;
    return;
  }
  if (corel == 6) {  // ED_calc_PB: shape holder g2 if g_with_shape == 2, else g1
    const PairGal &gs = (gws == 2) ? g2 : g1;
    const double norm = sqrt(sep[0] * sep[0] + sep[1] * sep[1] + sep[2] * sep[2]);
    double ca = gs.e1 * sep[0] + gs.e2 * sep[1] + gs.e3 * sep[2];
    ca /= norm;
    f[11] = ca * ca;
    f[12] = f[11] * f[11];
    return;
  }
  const double c2 = cos(2.0 * theta), s2 = sin(2.0 * theta);
  const double kpi = 3.141592653589793;
  auto ephi = [&](double phi) {
    double t = fabs(phi - theta);
    if (t > kpi / 2.0) t = kpi - t;
    return t;
  };
  if (corel == 5) {  // rotate the shape holder's e, weight by the other's kappa
    if (gws != 1 && gws != 2) return;
    const PairGal &gs = (gws == 2) ? g2 : g1, &gk = (gws == 2) ? g1 : g2;
    const double en0 = c2 * gs.e1 - s2 * gs.e2, en1 = s2 * gs.e1 + c2 * gs.e2;
    const double ep = wt * gk.e1;
    f[1] = ep;
    f[5] = ep * en0;
    f[9] = ep * en1;
    return;
  }
  if (corel == 1) {
    const PairGal &gs = (gws == 2) ? g2 : g1;
    const double e0 = gs.e1, e1 = gs.e2;
    const double ep = c2 * e0 - s2 * e1, ex = s2 * e0 + c2 * e1;
    f[1] = wt * ep;
    f[2] = f[1] * f[1];
    f[3] = wt * ex;
    f[4] = f[3] * f[3];
    const double et = ephi(g1.phi);
    f[11] = et;
    f[12] = et * et;
    return;
  }
  const double ei0 = c2 * g1.e1 - s2 * g1.e2, ei1 = s2 * g1.e1 + c2 * g1.e2;
  const double ej0 = c2 * g2.e1 - s2 * g2.e2, ej1 = s2 * g2.e1 + c2 * g2.e2;
  if (corel == 2) {
    if (gws == 2) {
      f[1] = wt * ej0;
      const double et = ephi(g2.phi);
      f[11] = et;
      f[12] = et * et;
    } else if (gws == 1) {
      f[1] = wt * ei0;
      const double et = ephi(g1.phi);
      f[11] = et;
      f[12] = et * et;
    }
    f[2] = f[1] * f[1];
  } else {
    f[1] = wt * (ei0 + ej0) / 2.0;
    f[2] = (wt * ei0 / 2.0) * (wt * ei0 / 2.0) + (wt * ej0 / 2.0) * (wt * ej0 / 2.0);
    f[3] = wt * (ei1 + ej1) / 2.0;
    f[4] = (wt * ei1 / 2.0) * (wt * ei1 / 2.0) + (wt * ej1 / 2.0) * (wt * ej1 / 2.0);
    const double a = ephi(g1.phi), b = ephi(g2.phi);
    f[11] = a + b;
    f[12] = a * a + b * b;
  }
  f[5] = wt * (ei0 * ej0);
  f[6] = f[5] * f[5];
  f[7] = wt * (ei1 * ej1);
  f[8] = f[7] * f[7];
  f[9] = wt * (ei1 * ej0 + ei0 * ej1) / 2.0;
  const double pa = wt * (ei1 * ej0) / 2.0, pb = wt * ei0 * ej1 / 2.0;
  f[10] = pa * pa + pb * pb;
}

}  // namespace cpc
