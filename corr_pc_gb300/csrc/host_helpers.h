// host_helpers.h -- host numerics shared by the library and the host driver.
#pragma once
#include <cstdint>

namespace cpc {
// glibc rand() outputs rand_{skip} .. rand_{skip+n-1} after srand(seed).
void glibc_rand_stream(uint32_t seed, int64_t skip, int64_t n, int32_t *out);
// elip_angle (calcs.cpp:73-83): 0.5*arctan(e0, -e1), NaN -> 0.
double elip_angle(double e0, double e1);
// exact r_p thresholds (n_bins + 1 entries); 0 ok, <0 invalid / non-monotone.
int rp_thresholds(int lin_bin, int n_bins, double rmin, double rmax, double *thr);
// exact Pi thresholds (n_p_bin + 1 entries).
int pi_thresholds(int n_p_bin, double pmin, double pmax, double *thr);
}  // namespace cpc

namespace cpc {
// glibc rand() as a running stream (same algorithm as glibc_rand_stream).
class GlibcRand {
 public:
  explicit GlibcRand(uint32_t seed);
  int32_t next();  // the next rand() value, 0 .. RAND_MAX
 private:
  uint32_t buf_[34];
  int64_t k_;
};
}  // namespace cpc
