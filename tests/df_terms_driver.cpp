// Host check of the compensated per-pair terms (corr_pc_gb300/csrc/pair_df.cuh)
// against the double-precision terms of pair_values.h, which follow the
// reference's corels.cpp.  Built by tests/test_df_terms.py with g++
// -ffp-contract=off; prints one line per corel: the largest |df - double| of
// each double-float field as a fraction of its bound, the largest fixed-point
// rounding error in quanta, and whether every conversion stayed in range;
// exits 1 when a bound is exceeded.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <initializer_list>

#include "df32.cuh"
#include "pair_df.cuh"
#include "pair_values.h"

using namespace cpc;

static uint64_t g_state = 0x9E3779B97F4A7C15ull;
static double urand() {  // xorshift64*, uniform in [0, 1)
  g_state ^= g_state >> 12;
  g_state ^= g_state << 25;
  g_state ^= g_state >> 27;
  return (double)((g_state * 2685821657736338717ull) >> 11) * (1.0 / 9007199254740992.0);
}
static double nrand() {
  const double u = urand() + 1e-300, v = urand();
  return std::sqrt(-2.0 * std::log(u)) * std::cos(6.283185307179586 * v);
}

static df32 split(double v) {
  const float h = (float)v;
  return {h, (float)(v - (double)h)};
}

int main(int argc, char **argv) {
  const long n = argc > 1 ? std::atol(argv[1]) : 200000;
  const double L = 1000.0;
  int bad = 0;
  for (int corel : {1, 2, 3, 4, 5}) {
    for (int weighted = 0; weighted < 2; weighted++) {
      double maxerr[2] = {0, 0};  // float32 positions, hi + lo positions
      double worst_q = 0.0;
      bool range_ok = true;
      for (long it = 0; it < n; it++) {
        const int gws = 1 + (int)(urand() * 2.0);
        // positions: float32 values or arbitrary doubles (hi + lo floats carry
        // about 48 bits of those); separations from 0.05 (below the smallest
        // r_p bin edge of the configurations, 0.1) to the box (raw, unshifted:
        // wrapped pairs are long)
        const bool f32 = (it & 1) == 0;
        double x1 = urand() * L, y1 = urand() * L;
        const double sc = std::pow(10.0, -1.3 + 4.3 * urand()), ang = 6.283185307179586 * urand();
        double x2 = x1 + sc * std::cos(ang), y2 = y1 + sc * std::sin(ang);
        if (urand() < 0.1) x2 = urand() * L;  // long separations
        if (f32) {
          x1 = (float)x1; y1 = (float)y1; x2 = (float)x2; y2 = (float)y2;
        }
        if (x1 == x2 && y1 == y2) continue;  // coincident: the exact path
        const df32 X1 = split(x1), Y1 = split(y1), X2 = split(x2), Y2 = split(y2);
        // float32 positions: the exact hi difference; others: hi + lo, renormalised
        const df32 dx = f32 ? two_diff(X2.h, X1.h) : df_diff_hl(X2.h, X2.l, X1.h, X1.l);
        const df32 dy = f32 ? two_diff(Y2.h, Y1.h) : df_diff_hl(Y2.h, Y2.l, Y1.h, Y1.l);
        // ellipticities |e| < 1, weights
        double e[2][2], w[2], phi[2];
        for (int g = 0; g < 2; g++) {
          do {
            e[g][0] = 0.5 * nrand();
            e[g][1] = 0.5 * nrand();
          } while (e[g][0] * e[g][0] + e[g][1] * e[g][1] >= 1.0);
          w[g] = weighted ? 0.5 + urand() : 1.0;
          phi[g] = 0.5 * std::atan2(e[g][0], -e[g][1]);
        }
        DfGal G[2];
        for (int g = 0; g < 2; g++) {
          G[g].e1 = split(w[g] * e[g][0]);
          G[g].e2 = split(w[g] * e[g][1]);
          G[g].w = split(w[g]);
          G[g].phi = (float)phi[g];
        }
        // reference terms in double
        const double theta = std::atan((y2 - y1) / (x2 - x1));
        double ref[kPairFields];
        pair_values(corel, gws, w[0] * w[1], theta, PairGal{e[0][0], e[0][1], phi[0]},
                    PairGal{e[1][0], e[1][1], phi[1]}, ref);
        // compensated terms
        df32 c, s;
        df_cos_sin_2theta(dx, dy, c, s);
        df32 d[kPairFields];
        float f[kPairFields];
        for (int q = 0; q < kPairFields; q++) {
          d[q] = df32{0.0f, 0.0f};
          f[q] = 0.0f;
        }
        const bool unit_w = !weighted;
        switch (corel) {
          case 1: df_pair_terms<1>(c, s, (float)theta, G[0], G[1], gws, unit_w, d, f); break;
          case 2: df_pair_terms<2>(c, s, (float)theta, G[0], G[1], gws, unit_w, d, f); break;
          case 3: df_pair_terms<3>(c, s, (float)theta, G[0], G[1], gws, unit_w, d, f); break;
          case 4: df_pair_terms<4>(c, s, (float)theta, G[0], G[1], gws, unit_w, d, f); break;
          default: df_pair_terms<5>(c, s, (float)theta, G[0], G[1], gws, unit_w, d, f); break;
        }
        const double wb = weighted ? 2.25 : 1.0;  // max w1 w2
        for (int q = 1; q < kPairFields; q++) {
          if (!df_field(corel, q)) continue;
          const double bq = wb;  // |e| < 1: every term is at most w1 w2
          const double got = (double)d[q].h + (double)d[q].l;
          const double err = std::fabs(got - ref[q]) / bq;
          if (err > maxerr[f32 ? 0 : 1]) maxerr[f32 ? 0 : 1] = err;
          // fixed point with the kernel's scale rule: |v| 2^S <= 2^29 - 2^17
          const int S = 29 - (int)std::ceil(std::log2(bq * (1.0 + 1.0 / 4096.0)));
          const float qs = std::ldexp(1.0f, S);
          unsigned lo15, hi;
          df_to_fixed15(d[q], qs, lo15, hi);
          const long long u = (long long)(int)hi * 32768ll + (long long)lo15;
          const double exact = ref[q] * std::ldexp(1.0, S);
          const double qe = std::fabs((double)u - exact);
          if (qe > worst_q) worst_q = qe;
          if (lo15 > 0x7FFFu || (int)hi < -16384 || (int)hi > 16383) range_ok = false;
        }
      }
      std::printf("corel %d weighted %d max_err_over_bound f32 %.3e hilo %.3e "
                  "worst_fixed_quanta %.3f range %s\n",
                  corel, weighted, maxerr[0], maxerr[1], worst_q, range_ok ? "ok" : "BAD");
      // float32 positions: the terms' own 2^-44; hi + lo positions (48 bits of a
      // coordinate <= 1000): 2 * sqrt2 * 2^-48 * 1000 / 0.05 rad of 2 theta
      if (maxerr[0] > std::ldexp(1.0, -40) || maxerr[1] > 3e-10 || worst_q > 0.52 || !range_ok)
        bad = 1;
    }
  }
  return bad;
}
