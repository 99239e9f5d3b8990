// outp.cpp -- the reference's text outputs (outp.cpp:45-162): 1-D and 2-D bin
// tables written with the default ostream formatting (6 significant digits)
// and the same column layout and separators, so the notebooks that read them
// (Process PC data*.ipynb) work unchanged.
#include <fstream>

#include "host.h"

namespace cpch {

int outp_bins(const Bins &b, int h, const std::string &path) {
  std::ofstream w(path);
  if (!w.is_open()) return 1;
  w << "# rp\tnpairs\twgg\twgg_err\twgp\twgp_err\twgx wgx_err\twpp \twpp_err\t\twxx\twxx_err\t\twpx  "
       "wpx_err \ttheta   theta_err   LS_err     wt_npair    rp_low   rp_high sig_crit"
    << std::endl;
  for (int i = 0; i < b.nb; i++) {
    const size_t c = b.bi(h, i);
    w << (b.b_max[i] + b.b_min[i]) / 2 << "\t" << b.bnum[c];
    for (int j = 0; j < 7; j++) {
      const double val = b.bdat[(c * 7 + j) * 2], err = b.bdat[(c * 7 + j) * 2 + 1];
      w << "\t" << val << "\t" << err;
    }
    w << "\t" << b.bls[c] << "   " << b.bwt[c] << "      " << b.b_min[i] << "    " << b.b_max[i]
      << "    " << b.bsig[c] << std::endl;
  }
  return w.good() ? 0 : 1;
}

int outp_2Dbins(const Bins &b, int h, const std::string &path) {
  std::ofstream w(path);
  if (!w.is_open()) return 1;
  w << "# rp     pi   npairs     wgg      wgg_err  wgp     wgp_err  wgx  wgx_err     wpp  wpp_err "
       "   wxx   wxx_err  wpx   wpx_err    theta    theta_err  wt_npairs "
    << std::endl;
  for (int i = 0; i < b.nb; i++)
    for (int k = 0; k < b.np; k++) {
      const size_t c = b.pi(h, i, k);
      w << (b.b_max[i] + b.b_min[i]) / 2 << "        " << (b.p_min[k] + b.p_max[k]) / 2.0
        << "         " << b.pnum[c];
      for (int j = 0; j < 7; j++)
        w << "       " << b.pdat[(c * 7 + j) * 2] << "      " << b.pdat[(c * 7 + j) * 2 + 1];
      w << "   " << b.pwt[c] << std::endl;
    }
  return w.good() ? 0 : 1;
}

int outp_data_info(const Info &d, const std::string &path) {
  std::ofstream w(path);
  if (!w.is_open()) return 1;
  auto line = [&](const char *key, const auto &v) { w << key << v << std::endl; };
  line("do_auto_corr         ", d.do_auto_corr);
  line("do_cross_corr        ", d.do_cross_corr);
  line("data_sorted          ", d.data_sorted);
  line("use_comoving         ", d.use_comoving);
  line("do_auto_rebin        ", d.do_auto_rebin);
  line("do_jk                ", d.do_jk);
  line("shape_pos            ", d.shape_pos);
  line("shape_z              ", d.shape_z);
  line("shape_e              ", d.shape_e);
  line("shape_wt             ", d.shape_wt);
  line("shape_jk             ", d.shape_jk);
  line("density_pos          ", d.density_pos);
  line("density_z            ", d.density_z);
  line("density_wt           ", d.density_wt);
  line("density_jk           ", d.density_jk);
  line("density_e            ", d.density_e);
  line("shape_rand_pos       ", d.srand_pos);
  line("shape_rand_z         ", d.srand_z);
  line("shape_rand_wt        ", d.srand_wt);
  line("shape_rand_jk        ", d.srand_jk);
  line("density_rand_pos     ", d.drand_pos);
  line("density_rand_z       ", d.drand_z);
  line("density_rand_wt      ", d.drand_wt);
  line("density_rand_jk      ", d.drand_jk);
  line("distances            ", d.distance_file);
  line("output               ", d.out_file);
  line("n_threads            ", d.n_threads);
  line("n_shape              ", d.n_shape);
  line("n_density            ", d.n_density);
  line("n_shape_rand         ", d.n_shape_rand);
  line("n_density_rand       ", d.n_density_rand);
  line("n_jk                 ", d.n_jk);
  line("bin_r_min            ", d.bin_r_min);
  line("bin_r_max            ", d.bin_r_max);
  line("n_bins               ", d.n_bins);
  line("lin_bin              ", d.lin_bin);
  line("n_p_bin              ", d.n_p_bin);
  line("p_min                ", d.p_min);
  line("p_max                ", d.p_max);
  line("z_min                ", d.z_min);
  line("z_max                ", d.z_max);
  line("dz                   ", d.dz);
  line("p_bin_siz            ", d.p_size);
  line("z_sep_max            ", d.z_sep_max);
  line("z_sep_min            ", d.z_sep_min);
  line("DD_Wt                ", d.DD_wt);
  line("DRs_wt               ", d.DRs_wt[0]);
  line("SS_wt                ", d.SS_wt);
  line("SRs_wt               ", d.SRs_wt);
  line("SD_wt                ", d.SD_wt[0]);
  line("RsRs_Wt              ", d.RsRs_wt[0]);
  line("RsRd_wt              ", d.RsRd_wt[0]);
  line("S_wt                 ", d.S_wt[0]);
  line("D_wt                 ", d.D_wt[0]);
  line("Rs_wt                ", d.Rs_wt[0]);
  line("Rd_wt                ", d.Rd_wt[0]);
  line("RsRd_same            ", d.RsRd_same);
  return w.good() ? 0 : 1;
}

}  // namespace cpch
