// inp.cpp -- the positional .inp parameter file (initialization.cpp:62-130):
// whitespace-separated "key value" pairs whose keys are ignored; the order is
// the contract (the Gen_inp notebooks write exactly this order).  Plus the
// settings data_ini derives from it for the paths this library implements.
#include <algorithm>
#include <cmath>
#include <fstream>
#include <sstream>

#include "host.h"

namespace cpch {

namespace {
template <class T>
bool next(std::istream &in, T &v) {
  std::string key;
  if (!(in >> key)) return false;
  return static_cast<bool>(in >> v);
}
bool next_bool(std::istream &in, int &v) {
  std::string key;
  int x = 0;
  if (!(in >> key >> x)) return false;
  v = x != 0;
  return true;
}
}  // namespace

int read_inp(const std::string &path, Info &d, std::string &err) {
  std::ifstream in(path);
  if (!in.is_open()) {
    err = "parameter file not open: " + path;
    return 1;
  }
  bool ok = next(in, d.which_corr) && next(in, d.coordinates) && next(in, d.estimator) &&
            next(in, d.data_sorted) && next_bool(in, d.use_comoving) && next(in, d.do_jk) &&
            next(in, d.sig_crit) && next(in, d.shape_pos) && next(in, d.shape_z) &&
            next(in, d.shape_e) && next(in, d.shape_wt) && next(in, d.shape_jk) &&
            next(in, d.shape_patch) && next(in, d.density_pos) && next(in, d.density_z) &&
            next(in, d.density_wt) && next(in, d.density_jk) && next(in, d.density_e) &&
            next(in, d.srand_pos) && next(in, d.srand_z) && next(in, d.srand_wt) &&
            next(in, d.srand_jk) && next(in, d.srand_patch) && next(in, d.drand_pos) &&
            next(in, d.drand_z) && next(in, d.drand_wt) && next(in, d.drand_jk) &&
            next(in, d.distance_file) && next(in, d.patches_file) && next(in, d.out_file) &&
            next(in, d.n_threads) && next(in, d.n_shape) && next(in, d.n_density) &&
            next(in, d.n_shape_rand) && next(in, d.n_density_rand) &&
            next_bool(in, d.rand_subsample) && next(in, d.n_jk_regions) && next(in, d.n_patch) &&
            next(in, d.bin_r_min) && next(in, d.bin_r_max) && next(in, d.n_bins) &&
            next_bool(in, d.lin_bin) && next(in, d.n_p_bin) && next(in, d.p_min) &&
            next(in, d.p_max) && next(in, d.z_min) && next(in, d.z_max) && next(in, d.dz) &&
            next(in, d.z_sep_min) && next(in, d.z_sep_max) && next_bool(in, d.periodic_box) &&
            next(in, d.periodic_box_size);
  if (!ok) {
    err = "parameter file ended early or has a malformed value: " + path;
    return 1;
  }
  return 0;
}

namespace {
// da_Z (initialization.cpp:23-60): rows "z H D_A D_C D_T"; with use_comoving the
// fifth column is stored as the transverse distance, else the third; reads at
// most ceil((z_max+1)/dz)+1 rows and needs at least ceil(z_max/dz)+1.
int read_distances(Info &d, std::string &err) {
  std::ifstream in(d.distance_file);
  if (!in.is_open()) {
    err = "da_Z:: distances file (dA vs Z) not opened: " + d.distance_file;
    return 1;
  }
  const int64_t want = (int64_t)std::ceil((d.z_max + 1) / d.dz) + 1;
  const int64_t need = (int64_t)std::ceil(d.z_max / d.dz) + 1;
  d.H_z.clear();
  d.dA_z.clear();
  d.dC_z.clear();
  double z, h, c3, c4, c5;
  while ((int64_t)d.H_z.size() < want && (in >> z >> h >> c3 >> c4 >> c5)) {
    d.H_z.push_back(h);
    d.dC_z.push_back(c4);
    d.dA_z.push_back(d.use_comoving ? c5 : c3);
  }
  if ((int64_t)d.H_z.size() < need) {
    err = "da_Z:: distances file (dA vs Z) ended unexpectedly";
    return 1;
  }
  return 0;
}
}  // namespace

// data_ini's derived settings (initialization.cpp:349-561).
int derive_info(Info &d, std::string &err) {
  if (d.periodic_box) {
    if (d.coordinates != 6 && d.coordinates != 7) {
      err = "wrong coordinates choice for periodic box";
      return 1;
    }
    d.dz = 0;
    if (d.data_sorted == 2) {
      err = "data_sorted==2 does not work with a periodic box";
      return 1;
    }
  }
  switch (d.estimator) {
    case 0: d.do_cross_corr = 1; d.do_auto_corr = 0; break;
    case 2: d.do_auto_rebin = 1; d.do_auto_corr = 1; d.do_cross_corr = 0; break;
    case 1: d.do_auto_corr = 1; d.do_cross_corr = 0; break;
    case 3: d.do_auto_corr = 1; d.do_cross_corr = 1; d.do_auto_rebin = 1; break;
    default: d.do_cross_corr = 1; d.do_auto_corr = 0; d.do_auto_rebin = 0; break;
  }
  d.RsRd_same = 0;
  if (d.n_density_rand == 0 && d.which_corr <= 2) {
    d.RsRd_same = 1;
    d.n_density_rand = d.n_shape_rand;
  }
  d.include_prob_RR = 1;
  if (d.rand_subsample)
    d.include_prob_RR = std::sqrt(std::sqrt(double(d.n_density) / d.n_density_rand *
                                            double(d.n_shape) / d.n_shape_rand)) * 1.0;
  d.n_jk = d.n_jk_regions;  // jk_initilize (jk.cpp:22-38), do_jk = 1
  if (d.do_jk > 1) d.n_jk = d.n_jk_regions * (d.n_jk_regions + 1) / 2;
  if (d.z_sep_max == 0) d.z_sep_max = 9;
  if (d.dz == 0 && d.periodic_box == 0) {
    err = "dz=0";
    return 1;
  }
  if (!d.periodic_box && read_distances(d, err)) return 1;
  const int64_t z_idx = (int64_t)std::ceil(d.z_max / d.dz);
  if (d.coordinates == 0) {
    if (z_idx >= (int64_t)d.H_z.size()) {
      err = "distances file shorter than z_max / dz";
      return 1;
    }
    d.z_sep_max = d.p_max * d.H_z[z_idx] / 300000.0 + 0.001;
    d.z_sep_min = d.p_min * d.H_z[z_idx] / 300000.0 - 0.001;
  } else if (d.coordinates == 6) {
    d.z_sep_max = d.p_max + 1;
    d.z_sep_min = d.p_min - 1;
  } else if (d.coordinates == 7) {
    d.z_sep_max = d.bin_r_max + 0.1;
    d.z_sep_min = d.z_sep_max * -1;
  }
  if (d.bin_r_max == 0 || d.bin_r_min > d.bin_r_max) {
    err = "Bad Bin limits";
    return 1;
  }
  d.p_size = (d.p_max - d.p_min) / (d.n_p_bin);
  if (d.coordinates == 3 || d.coordinates == 5) d.p_size = 1;
  if (d.lin_bin) d.r_size = (d.bin_r_max - d.bin_r_min) / d.n_bins;
  else d.r_size = (std::log10(d.bin_r_max) - std::log10(d.bin_r_min)) / d.n_bins;
  return 0;
}

cpc_params to_params(const Info &d) {
  cpc_params p{};
  p.which_corr = d.which_corr;
  p.coordinates = d.coordinates;
  p.estimator = d.estimator;
  p.periodic_box = d.periodic_box;
  p.data_sorted = d.data_sorted;
  p.do_jk = d.do_jk;
  p.n_jk = d.n_jk;
  p.sig_crit = d.sig_crit;
  p.rand_subsample = d.rand_subsample;
  p.n_bins = d.n_bins;
  p.lin_bin = d.lin_bin;
  p.n_p_bin = d.n_p_bin;
  p.bin_r_min = d.bin_r_min;
  p.bin_r_max = d.bin_r_max;
  p.p_min = d.p_min;
  p.p_max = d.p_max;
  p.periodic_box_size = d.periodic_box_size;
  p.z_max = d.z_max;
  p.dz = d.dz;
  p.z_sep_max = d.z_sep_max;
  if (!d.periodic_box && !d.H_z.empty()) {
    p.H_z = d.H_z.data();
    p.dA_z = d.dA_z.data();
    p.n_table = (int64_t)std::min(d.H_z.size(), d.dA_z.size());
  }
  return p;
}

}  // namespace cpch
