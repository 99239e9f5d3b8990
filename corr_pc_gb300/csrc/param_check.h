// param_check.h -- the parameter checks every entry point that takes a
// cpc_params applies (cpc_create, cpc_count_fp64_noalloc): the .inp values the
// pair loop reads (initialization.cpp:62-130) restricted to what this library
// computes.  Returns nullptr when the parameters are accepted, else the reason.
#pragma once

#include <cmath>

#include "../../include/corrpc.h"
#include "cpc_device.cuh"

namespace cpc {

inline const char *param_error(const cpc_params &p) {
  if (p.coordinates != 6 && p.coordinates != 7 && p.coordinates != 0)
    return "coordinates: 6 (x,y,z with r_p, Pi), 7 (x,y,z with r, mu) and 0 (sky, r_p and Pi) "
           "are supported";
  if (p.which_corr < 0 || p.which_corr > 5) return "which_corr must be in 0..5";
  // coordinates 7 outside a periodic box takes the sky window (lim_calc_sky,
  // corr.cpp:311-324) in the reference: not a box computation
  if (p.coordinates == 7 && !p.periodic_box) return "coordinates 7 (r, mu) needs a periodic box";
  if (p.sig_crit != 0) return "sig_crit weights are not supported";
  if (p.rand_subsample != 0) return "rand_subsample is not supported";
  if (p.do_jk != 0 && p.do_jk != 1) return "do_jk must be 0 or 1";
  if (p.do_jk && (p.n_jk <= 0 || p.n_jk > 100000)) return "n_jk out of range";
  if (p.n_bins <= 0 || p.n_bins > kMaxRp) return "n_bins must be in 1..64";
  if (p.n_p_bin <= 0 || p.n_p_bin > kMaxPi) return "n_p_bin must be in 1..128";
  if (!(p.bin_r_max > p.bin_r_min) || !(p.bin_r_min >= 0) || (!p.lin_bin && !(p.bin_r_min > 0)))
    return "bad r_p bin limits";
  if (!(p.p_max > p.p_min)) return "bad Pi bin limits";
  if (p.coordinates == 0) {
    if (p.periodic_box) return "coordinates 0 (sky) cannot be periodic";
    if (p.which_corr > 2) return "which_corr 3-5 (kappa, ED) run in x,y,z (coordinates 6, 7)";
    if (!p.H_z || !p.dA_z || p.n_table < 2)
      return "sky runs need the distance table (H_z, dA_z, n_table)";
    if (!(p.dz > 0) || !(p.z_max > 0) || !std::isfinite(p.z_sep_max))
      return "sky runs need dz > 0, z_max > 0 and a finite z_sep_max";
    return nullptr;
  }
  if (!(p.periodic_box_size > 0)) return "box size must be > 0";
  if (p.periodic_box) {
    const double L = p.periodic_box_size;
    const bool rmu = p.coordinates == 7;  // p_min, p_max bound mu there
    if (p.bin_r_max > L || (!rmu && (p.p_max > L || -p.p_min > L)))
      return "bin limits larger than the periodic box";
  }
  return nullptr;
}

}  // namespace cpc
