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
// with the rotation of calcs.cpp:60-64 and the folded angle |phi - theta| of
// ephi_calc (calcs.cpp:97-105).
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
  double e1, e2, phi;
};

CPC_HD inline void pair_values(int corel, int gws, double wt, double theta, const PairGal &g1,
                               const PairGal &g2, double f[kPairFields]) {
  for (int q = 0; q < kPairFields; q++) f[q] = 0.0;
  f[0] = wt;
  if (corel == 0) return;
  const double c2 = cos(2.0 * theta), s2 = sin(2.0 * theta);
  const double kpi = 3.141592653589793;
  auto ephi = [&](double phi) {
    double t = fabs(phi - theta);
    if (t > kpi / 2.0) t = kpi - t;
    return t;
  };
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
