// pair_df.cuh -- per-pair accumulator terms of the mixed-precision kernels.
//
// The fields whose bin sums cancel (the rotated ellipticities e+ and ex, their
// products e++, exx and e+x, and the kappa terms) are computed as double-floats
// (df32.cuh) from exact inputs: the raw separation as a double-float, each
// galaxy's weighted ellipticity w (e1, e2) split into float hi and lo parts on
// the device at upload, and its weight as hi and lo parts.  Those terms carry
// about 2^-44 of their magnitude, so with the 2^-29 fixed-point quantum of the
// histograms every bin sum stays within about 1e-9 of the field bound of the
// reference's double-precision sums.  The fields whose terms cannot cancel
// (weights, squares, the orientation term) are plain floats.
//
// Field definitions follow pair_values.h (the reference's corels.cpp:79-244
// with the rotation of calcs.cpp:60-64); the weight product wt = w1 w2 is
// folded into the weighted ellipticities:
//   wt (c e1_i - s e2_i) = w_j (c w_i e1_i - s w_i e2_i)
//   wt e+_i e+_j        = (rotated w_i e_i)_+ (rotated w_j e_j)_+
#pragma once

#include "df32.cuh"

namespace cpc {

// corel numbering of cpc_device.cuh
constexpr int kDfSD = 1, kDfSS = 2, kDfSSA = 3, kDfDK = 4, kDfSK = 5;

// whether field q of corel C is carried as a double-float
DF_HD constexpr bool df_field(int C, int q) {
  return (C == kDfSD && (q == 1 || q == 3)) ||
         ((C == kDfSS || C == kDfSSA) && (q == 1 || q == 3 || q == 5 || q == 7 || q == 9)) ||
         (C == kDfDK && q == 1) || (C == kDfSK && (q == 1 || q == 5 || q == 9));
}

// The per-galaxy inputs of one side of a pair: its weighted ellipticity
// (w e1, w e2) as hi and lo parts, its weight as hi and lo parts, and phi.
struct DfGal {
  df32 e1, e2;  // w e1, w e2 (kappa: w kappa in e1)
  df32 w;
  float phi;
};

DF_HD float ephi32(float phi, float theta) {  // ephi_calc (calcs.cpp:97-105)
  const float t = fabsf(phi - theta);
  return t > 1.5707963267948966f ? 3.14159265358979f - t : t;
}

// Terms of one binned pair for corel C.  d[q]: double-float terms of the
// fields df_field(C, q); f[q]: float terms of the others (f[0] is set by the
// caller).  c, s: cos 2theta and sin 2theta of the raw separation; theta the
// orientation angle (float, for the phi term only); unit_w: every weight is 1.
// dm, fm (shape_shape estimator 0, when not null): the fields 1, 2, 11 and 12
// of the same pair in the other order (g2, g1), the only ones that differ when
// both galaxies carry the same data in either role (the orientation angle and
// the rotations are those of the pair; the products are symmetric).
template <int C>
DF_HD void df_pair_terms(df32 c, df32 s, float theta, const DfGal &g1, const DfGal &g2, int gws,
                         bool unit_w, df32 *d, float *f, df32 *dm = nullptr,
                         float *fm = nullptr) {
  if (C == kDfDK) {  // density_convergence (corels.cpp:79-90): wt kappa of the shape holder
    const df32 z{0.0f, 0.0f};
    if (gws == 1) d[1] = unit_w ? g1.e1 : df_mul(g2.w, g1.e1);
    else if (gws == 2) d[1] = unit_w ? g2.e1 : df_mul(g1.w, g2.e1);
    else d[1] = z;
    return;
  }
  if (C == kDfSK) {  // shape_convergence (corels.cpp:92-120)
    if (gws != 1 && gws != 2) {
      d[1] = d[5] = d[9] = df32{0.0f, 0.0f};
      return;
    }
    const DfGal &gs = gws == 2 ? g2 : g1, &gk = gws == 2 ? g1 : g2;
    df32 en0, en1;
    df_rotate(c, s, gs.e1, gs.e2, en0, en1);   // w_s * rotated e of the shape holder
    d[1] = unit_w ? gk.e1 : df_mul(gs.w, gk.e1);  // wt kappa_k
    d[5] = df_mul(gk.e1, en0);                   // wt kappa_k e+_s
    d[9] = df_mul(gk.e1, en1);
    return;
  }
  if (C == kDfSD) {  // shape_density (corels.cpp:206-244)
    const DfGal &gs = gws == 2 ? g2 : g1, &go = gws == 2 ? g1 : g2;
    df32 ep, ex;
    df_rotate(c, s, gs.e1, gs.e2, ep, ex);
    d[1] = unit_w ? ep : df_mul(go.w, ep);
    d[3] = unit_w ? ex : df_mul(go.w, ex);
    f[2] = d[1].h * d[1].h;
    f[4] = d[3].h * d[3].h;
    f[11] = ephi32(g1.phi, theta);
    f[12] = f[11] * f[11];
    return;
  }
  // shape_shape (corels.cpp:122-204)
  df32 ei0, ei1, ej0, ej1;
  df_rotate(c, s, g1.e1, g1.e2, ei0, ei1);  // w_1 * rotated e_1
  df_rotate(c, s, g2.e1, g2.e2, ej0, ej1);  // w_2 * rotated e_2
  if (C == kDfSS) {  // estimator 0: e+ and the phi term of the shape holder; ex stays 0
    // the shape holder's terms for the holder in role 2 (g2) and in role 1 (g1);
    // the other order (g2, g1) swaps them
    const df32 e_of2 = unit_w ? ej0 : df_mul(g1.w, ej0), e_of1 = unit_w ? ei0 : df_mul(g2.w, ei0);
    const float t_of2 = ephi32(g2.phi, theta), t_of1 = ephi32(g1.phi, theta);
    if (gws == 2) {
      d[1] = e_of2;
      f[11] = t_of2;
    } else if (gws == 1) {
      d[1] = e_of1;
      f[11] = t_of1;
    } else {
      d[1] = df32{0.0f, 0.0f};
      f[11] = 0.0f;
    }
    f[2] = d[1].h * d[1].h;
    f[12] = f[11] * f[11];
    if (dm) {
      if (gws == 2) {
        dm[1] = e_of1;
        fm[11] = t_of1;
      } else if (gws == 1) {
        dm[1] = e_of2;
        fm[11] = t_of2;
      } else {
        dm[1] = df32{0.0f, 0.0f};
        fm[11] = 0.0f;
      }
      fm[2] = dm[1].h * dm[1].h;
      fm[12] = fm[11] * fm[11];
    }
  } else {  // the other estimators: the pair's mean e+ and ex, both phi terms
    const df32 pa = unit_w ? ei0 : df_mul(g2.w, ei0), pb = unit_w ? ej0 : df_mul(g1.w, ej0);
    const df32 qa = unit_w ? ei1 : df_mul(g2.w, ei1), qb = unit_w ? ej1 : df_mul(g1.w, ej1);
    d[1] = df_scale(df_add(pa, pb), 0.5f);
    d[3] = df_scale(df_add(qa, qb), 0.5f);
    const float ha = 0.5f * pa.h, hb = 0.5f * pb.h, ka = 0.5f * qa.h, kb = 0.5f * qb.h;
    f[2] = ha * ha + hb * hb;
    f[4] = ka * ka + kb * kb;
    const float ta = ephi32(g1.phi, theta), tb = ephi32(g2.phi, theta);
    f[11] = ta + tb;
    f[12] = ta * ta + tb * tb;
  }
  d[5] = df_mul(ei0, ej0);
  f[6] = d[5].h * d[5].h;
  d[7] = df_mul(ei1, ej1);
  f[8] = d[7].h * d[7].h;
  const df32 xa = df_mul(ei1, ej0), xb = df_mul(ei0, ej1);
  d[9] = df_scale(df_add(xa, xb), 0.5f);
  const float ha = 0.5f * xa.h, hb = 0.5f * xb.h;
  f[10] = ha * ha + hb * hb;
}

}  // namespace cpc
