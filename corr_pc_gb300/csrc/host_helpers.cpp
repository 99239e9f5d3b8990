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
