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

namespace cpc {
// ---- sky geometry (coordinates 0) with the C library's math ----
struct SkyParams {
  const double *H, *dA;  // distance table columns as data_ini stores them
  int64_t n_table;
  double dz, z_max, z_sep_max;
  double p_min, p_max, p_size;
  double r_min, r_max, r_size;
  int lin_bin, n_bins, n_p_bin;
};
// per-galaxy angles: dec_rad = dec/r2d, ra_rad = ra/r2d, sin/cos(dec_rad)
void sky_angles(double ra_deg, double dec_deg, double *ra_rad, double *dec_rad, double *sin_dec,
                double *cos_dec);
// lim_calc_sky + lim_calc_ra_dec for one g1 row: win = z_min, z_max, ra_min,
// ra_max, dec_min, dec_max.  0 ok; 1 z_min > z_max (the reference exits);
// 2 a distance-table index outside the table.
int sky_window(const SkyParams &p, double ra_deg, double dec_deg, double z, double win[6]);
// corel_bin of a sky pair: 2 binned (n1, n2 set), 1 outside the bins.
int sky_bin(const SkyParams &p, double ra1, double dec1, double dc1, double da1, double ra2,
            double dec2, double dc2, double da2, int *n1, int *n2);
// angle_orient_axis_sky
double sky_orient(double ra1, double dec1, double ra2, double dec2);
}  // namespace cpc
