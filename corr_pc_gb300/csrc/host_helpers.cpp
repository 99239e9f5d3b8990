// host_helpers.cpp -- host-side numerics shared by the library and its host
// driver.  Compiled with -ffp-contract=off so every double expression rounds
// exactly as the reference's x86-64 build does.
//
//  * glibc rand() stream (read_dat.cpp:243, 320 after srand in jk.cpp:40-43),
//    restated from glibc's published TYPE_3 additive-feedback generator.
//  * elip_angle (calcs.cpp:35-46, 73-83).
//  * exact bin thresholds: the smallest double at which the reference's own
//    bin expression  floor(log10(r/r_min)/r_size)  (corels.cpp:41-44) or
//    floor((Pi - p_min)/p_size)  (corels.cpp:26) reaches each bin index,
//    found by bisection over the ordered doubles with the host libm -- the
//    same log10 the reference calls.  Comparing a double r_p against these
//    thresholds reproduces the reference's bin index exactly.
//  * sky geometry: per-row windows (lim_calc_sky / lim_calc_ra_dec,
//    sky_calcs.cpp:105-196), the exact bin of a sky pair (corel_bin with
//    pi_calc, rp_calc_sky and dA_calc) and the pair's orientation angle, all
//    with the C library's trigonometry in the reference's operation order.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>

#include "host_helpers.h"

namespace cpc {

void glibc_rand_stream(uint32_t seed, int64_t skip, int64_t n, int32_t *out) {
  uint32_t buf[34];
  int32_t r[34];
  r[0] = (int32_t)(seed == 0 ? 1u : seed);
  for (int i = 1; i < 31; i++) {
    const int64_t hi = r[i - 1] / 127773, lo = r[i - 1] % 127773;
    int64_t word = 16807 * lo - 2836 * hi;
    if (word < 0) word += 2147483647;
    r[i] = (int32_t)word;
  }
  for (int i = 31; i < 34; i++) r[i] = r[i - 31];
  for (int i = 0; i < 34; i++) buf[i] = (uint32_t)r[i];
  const int64_t total = 310 + skip + n;
  int64_t k = 34;
  for (int64_t t = 0; t < total; t++, k++) {
    const uint32_t v = buf[(k - 31) % 34] + buf[(k - 3) % 34];
    buf[k % 34] = v;
    const int64_t o = t - 310 - skip;
    if (o >= 0) out[o] = (int32_t)(v >> 1);
  }
}

double elip_angle(double e0, double e1in) {
  double e1 = -1 * e1in;
  double t = atan(e1 / e0);  // arctan(x, y) with x = e0, y = -e1
  if (e0 < 0) {
    if (e1 < 0) t -= M_PI;
    else t += M_PI;
  }
  double phi = 0.5 * t;
  if (phi != phi) phi = 0;
  return phi;
}

// ordered-integer view of doubles: a monotone bijection double <-> int64
// (+0.0 -> 0, -0.0 -> -1, larger magnitude negatives -> more negative)
static inline int64_t ord_of(double d) {
  uint64_t u;
  std::memcpy(&u, &d, 8);
  if (!(u >> 63)) return (int64_t)u;
  return -1 - (int64_t)(u & 0x7fffffffffffffffull);
}
static inline double dbl_of(int64_t o) {
  uint64_t u = o >= 0 ? (uint64_t)o : (0x8000000000000000ull | (uint64_t)(-1 - o));
  double d;
  std::memcpy(&d, &u, 8);
  return d;
}

// smallest double x in [lo, hi] with bin(x) >= k; bin monotone non-decreasing
template <class F>
static double first_at_least(F bin, int k, double lo_d, double hi_d) {
  int64_t lo = ord_of(lo_d), hi = ord_of(hi_d);
  if (bin(hi_d) < k) return std::numeric_limits<double>::infinity();
  if (bin(lo_d) >= k) return lo_d;
  while ((uint64_t)hi - (uint64_t)lo > 1) {
    const int64_t mid = (int64_t)((uint64_t)lo + ((uint64_t)hi - (uint64_t)lo) / 2);
    if (bin(dbl_of(mid)) >= k) hi = mid; else lo = mid;
  }
  return dbl_of(hi);
}

int rp_thresholds(int lin_bin, int n_bins, double rmin, double rmax, double *thr) {
  if (n_bins <= 0 || !(rmax > rmin)) return -1;
  if (lin_bin) {
    const double r_size = (rmax - rmin) / n_bins;  // initialization.cpp:519
    auto bin = [&](double r) {
      const double v = floor((r - rmin) / r_size);
      return v < -1e9 ? -1000000000 : (v > 1e9 ? 1000000000 : (int)v);
    };
    for (int k = 0; k <= n_bins; k++) thr[k] = first_at_least(bin, k, 0.0, 1e300);
  } else {
    if (!(rmin > 0)) return -1;
    const double r_size = (log10(rmax) - log10(rmin)) / n_bins;  // initialization.cpp:520
    auto bin = [&](double r) {
      const double v = floor(log10(r / rmin) / r_size);
      return !(v > -1e9) ? -1000000000 : (v > 1e9 ? 1000000000 : (int)v);
    };
    for (int k = 0; k <= n_bins; k++) {
      thr[k] = first_at_least(bin, k, 0.0, 1e300);
      // the reference's expression must be monotone around the threshold
      double a = thr[k], b = thr[k];
      for (int m = 0; m < 256; m++) {
        a = nextafter(a, 0.0);
        b = nextafter(b, 1e300);
        if (bin(a) >= k || bin(b) < k) return -2;
      }
    }
  }
  return 0;
}

int pi_thresholds(int n_p_bin, double pmin, double pmax, double *thr) {
  if (n_p_bin <= 0 || !(pmax > pmin)) return -1;
  const double p_size = (pmax - pmin) / (n_p_bin);  // initialization.cpp:514
  auto bin = [&](double p) {
    const double v = floor((p - pmin) / p_size);
    return !(v > -1e9) ? -1000000000 : (v > 1e9 ? 1000000000 : (int)v);
  };
  for (int k = 0; k <= n_p_bin; k++) thr[k] = first_at_least(bin, k, -1e300, 1e300);
  return 0;
}

}  // namespace cpc

namespace cpc {
GlibcRand::GlibcRand(uint32_t seed) {
  int32_t r[34];
  r[0] = (int32_t)(seed == 0 ? 1u : seed);
  for (int i = 1; i < 31; i++) {
    const int64_t hi = r[i - 1] / 127773, lo = r[i - 1] % 127773;
    int64_t word = 16807 * lo - 2836 * hi;
    if (word < 0) word += 2147483647;
    r[i] = (int32_t)word;
  }
  for (int i = 31; i < 34; i++) r[i] = r[i - 31];
  for (int i = 0; i < 34; i++) buf_[i] = (uint32_t)r[i];
  k_ = 34;
  for (int t = 0; t < 310; t++) next();
}
int32_t GlibcRand::next() {
  const uint32_t v = buf_[(k_ - 31) % 34] + buf_[(k_ - 3) % 34];
  buf_[k_ % 34] = v;
  k_++;
  return (int32_t)(v >> 1);
}
}  // namespace cpc

namespace cpc {

static const double kR2d = 180.0 / M_PI;  // sky_calcs.cpp:10, calcs.cpp

void sky_angles(double ra_deg, double dec_deg, double *ra_rad, double *dec_rad, double *sin_dec,
                double *cos_dec) {
  *ra_rad = ra_deg / kR2d;  // angle_deg_to_rad (calcs.cpp:19-22)
  *dec_rad = dec_deg / kR2d;
  *sin_dec = sin(*dec_rad);
  *cos_dec = cos(*dec_rad);
}

// table interpolation of sky_calcs.cpp:71-81 (dAR_to_dA, p_to_dz)
static bool table_row(const SkyParams &p, double z, int *i) {
  const double f = floor(z / p.dz);
  if (!(f >= 0) || f + 1 >= (double)p.n_table) return false;
  *i = (int)f;
  return true;
}

int sky_window(const SkyParams &p, double ra_deg, double dec_deg, double z, double win[6]) {
  const double dec_rad = dec_deg / kR2d;
  int i;
  // lim_calc_sky, default case (sky_calcs.cpp:183-186)
  double z_max = z + p.z_sep_max;
  if (!table_row(p, z_max, &i)) return 2;
  z_max = z + p.p_max * (p.H[i] + ((p.H[i + 1] - p.H[i]) * (z_max - p.dz * i) / p.dz)) / 300000.0;
  if (!table_row(p, z, &i)) return 2;
  double z_min = z + p.p_min * (p.H[i] + ((p.H[i + 1] - p.H[i]) * (z - p.dz * i) / p.dz)) / 300000.0;
  // lim_calc_ra_dec (sky_calcs.cpp:105-145)
  if (z_min < 0.001) z_min = 0.001;
  if (z_min > p.z_max) return 1;
  if (!table_row(p, z_min, &i)) return 2;
  const double da_max =
      p.r_max / (p.dA[i] + ((p.dA[i + 1] - p.dA[i]) * (z_min - p.dz * i) / p.dz));
  double ra_lim = acos((pow(cos(da_max), 1) - pow(sin(dec_rad), 2)) / pow(cos(dec_rad), 2)) *
                  1.02 * kR2d;
  double ra_max = ra_deg + ra_lim;
  double ra_min = ra_deg - ra_lim;
  if (ra_max > 360) {
    ra_min = 0;
    ra_lim = 360;
  }
  if (ra_min < 0) {
    ra_max = 360;
    ra_lim = 360;
  }
  (void)ra_lim;
  win[0] = z_min;
  win[1] = z_max;
  win[2] = ra_min;
  win[3] = ra_max;
  win[4] = dec_deg - da_max * kR2d * 1.05;
  win[5] = dec_deg + da_max * kR2d * 1.05;
  return 0;
}

int sky_bin(const SkyParams &p, double ra1, double dec1, double dc1, double da1, double ra2,
            double dec2, double dc2, double da2, int *n1, int *n2) {
  // pi_calc (calcs.cpp:126-132) then rp_calc_sky (sky_calcs.cpp:91-96)
  const double d_P = dc2 - dc1;
  const double d1 = dec1 / kR2d, d2 = dec2 / kR2d, a1 = ra1 / kR2d, a2 = ra2 / kR2d;
  const double sum = sin(d1) * sin(d2) + cos(d1) * cos(d2) * cos((a1 - a2));
  const double da = (sum > 0.9999999999) ? acos(1.0) : acos(sum);
  const double da_R = da * (da1 + da2) / 2.;
  // corel_bin (corels.cpp:21-46)
  const double v2 = floor((d_P - p.p_min) / p.p_size);
  if (!(v2 >= 0) || v2 >= p.n_p_bin) return 1;
  double v1;
  if (p.lin_bin) v1 = floor((da_R - p.r_min) / p.r_size);
  else v1 = floor(log10(da_R / p.r_min) / p.r_size);
  if (!(v1 >= 0) || v1 >= p.n_bins) return 1;
  *n1 = (int)v1;
  *n2 = (int)v2;
  return 2;
}

double sky_orient(double ra1, double dec1, double ra2, double dec2) {
  return atan((dec2 - dec1) / ((ra2 - ra1) * cos((dec1 / kR2d + dec2 / kR2d) / 2.0)));
}

}  // namespace cpc
