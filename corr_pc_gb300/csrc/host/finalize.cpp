// finalize.cpp -- bin trees and the estimator finalisation of cross and auto
// runs (do_corr.cpp:203-433 with bins_calcs.cpp:30-91, 94-256, 331-530 and the
// analytic periodic-box RR of PB_calcs.cpp:63-85).  Bin edges are formed in
// single precision exactly as the reference's initialisers do
// (initialization.cpp:357-444), because they are printed in the outputs.
#include <atomic>
#include <cmath>
#include <cstdio>
#include <new>
#include <sstream>

#include "host.h"

namespace cpch {

int outp_bins(const Bins &b, int h, const std::string &path);
int outp_2Dbins(const Bins &b, int h, const std::string &path);

void Bins::init(const Info &d, int n_hist) {
  nb = d.n_bins;
  np = d.n_p_bin;
  nh = n_hist;
  b_min.assign(nb, 0); b_max.assign(nb, 0); p_min.assign(np, 0); p_max.assign(np, 0);
  if (d.lin_bin) {  // bin_lin
    const float b_size = (d.bin_r_max - d.bin_r_min) / (float)d.n_bins;
    float temp = d.bin_r_min;
    for (int i = 0; i < nb; i++) {
      b_min[i] = temp;
      temp += b_size;
      b_max[i] = temp;
    }
  } else {  // bin_log
    float lo = std::log10(d.bin_r_min);
    const float hi = std::log10(d.bin_r_max);
    const float b_size = (hi - lo) / (float)d.n_bins;
    for (int i = 0; i < nb; i++) {
      b_min[i] = std::pow(10.0, lo);
      lo += b_size;
      b_max[i] = std::pow(10.0, lo);
    }
  }
  {  // P_bin_ini
    const float ps = d.p_size;
    float temp = d.p_min;
    for (int k = 0; k < np; k++) {
      p_min[k] = temp;
      temp += ps;
      p_max[k] = temp;
    }
  }
  const size_t nbh = (size_t)nh * nb, nph = nbh * np;
  bnum.assign(nbh, 0); bwt.assign(nbh, 0); bdat.assign(nbh * 14, 0); bls.assign(nbh, 0);
  bsig.assign(nbh, 0);
  pnum.assign(nph, 0); pwt.assign(nph, 0); pdat.assign(nph * 14, 0); pls.assign(nph, 0);
}

void add_count(Bins &b, const Info &d, const int64_t *num, const double *sums) {
  for (int h = 0; h < b.nh; h++)
    for (int i = 0; i < b.nb; i++)
      for (int k = 0; k < b.np; k++) {
        const size_t c = b.pi(h, i, k);
        const int64_t n = num[c];
        b.pnum[c] += n;
        b.bnum[b.bi(h, i)] += n;  // b[n1].num++ for every binned pair
        const double *s = sums + c * CPC_NF;
        b.pwt[c] += s[0];
        for (int j = 1; j <= 6; j++) {
          b.pd(h, i, k, j, 0) += s[1 + 2 * (j - 1)];
          b.pd(h, i, k, j, 1) += s[2 + 2 * (j - 1)];
        }
      }
  if (!d.do_jk) return;
  // final_jk_bins: every field of sample r := full - region r
  for (int h = 1; h < b.nh; h++)
    for (int i = 0; i < b.nb; i++) {
      const size_t f = b.bi(0, i), r = b.bi(h, i);
      b.bnum[r] = b.bnum[f] - b.bnum[r];
      b.bwt[r] = b.bwt[f] - b.bwt[r];
      b.bls[r] = b.bls[f] - b.bls[r];
      b.bsig[r] = b.bsig[f] - b.bsig[r];
      for (int j = 0; j < 7; j++)
        for (int e = 0; e < 2; e++) b.bd(h, i, j, e) = b.bd(0, i, j, e) - b.bd(h, i, j, e);
      for (int k = 0; k < b.np; k++) {
        const size_t pf = b.pi(0, i, k), pr = b.pi(h, i, k);
        b.pnum[pr] = b.pnum[pf] - b.pnum[pr];
        b.pwt[pr] = b.pwt[pf] - b.pwt[pr];
        b.pls[pr] = b.pls[pf] - b.pls[pr];
        for (int j = 0; j < 7; j++)
          for (int e = 0; e < 2; e++) b.pd(h, i, k, j, e) = b.pd(0, i, k, j, e) - b.pd(h, i, k, j, e);
      }
    }
}

namespace {

// RR_PB_calc (PB_calcs.cpp:63-85): expected pair fraction per (r_p, Pi) bin in
// a periodic box; per (r, mu) bin for coordinates 7 (shell volume times the
// mu-bin width over 2)
void rr_periodic(Bins &rr, int h, const Info &d) {
  const double total_volume = std::pow(d.periodic_box_size, 3);
  for (int i = 0; i < rr.nb; i++) {
    double area = 0;
    if (d.coordinates == 6) area = M_PI * (rr.b_max[i] * rr.b_max[i] - rr.b_min[i] * rr.b_min[i]);
    else if (d.coordinates == 7)
      area = 4. / 3. * M_PI *
             (rr.b_max[i] * rr.b_max[i] * rr.b_max[i] - rr.b_min[i] * rr.b_min[i] * rr.b_min[i]);
    rr.bnum[rr.bi(h, i)] = 1;
    for (int k = 0; k < rr.np; k++) {
      double volume = 0;
      if (d.coordinates == 6) volume = area * (rr.p_max[k] - rr.p_min[k]);
      else if (d.coordinates == 7) volume = area / 2 * (rr.p_max[k] - rr.p_min[k]);
      rr.pwt[rr.pi(h, i, k)] = volume / total_volume;
      rr.pnum[rr.pi(h, i, k)] = 1;
    }
  }
}

// final_calc_bins (bins_calcs.cpp:94-256) for sample h of each term
void final_bins(Bins &sd, Bins &sr, Bins &dr, Bins &rr, Bins &fin, int h, const Info &d) {
  const double SD_wt = d.SD_wt[0], SR_wt = d.SRd_wt[0], DR_wt = d.DRs_wt[0], RR_wt = d.RsRd_wt[0];
  for (int i = 0; i < sd.nb; i++) {
    for (int k = 0; k < sd.np; k++) {
      const size_t c = sd.pi(h, i, k);
      fin.bnum[fin.bi(h, i)] += sd.pnum[c];
      const double sd_num = (double)sd.pnum[c], sr_num = (double)sr.pnum[c];
      const double rr_num = (double)rr.pnum[c];
      const double sd_w = sd.pwt[c], sr_w = sr.pwt[c], dr_w = dr.pwt[c], rr_w = rr.pwt[c];
      if (rr_num == 0) continue;
      const double sd_rel = (sd_w / rr_w) * (RR_wt / SD_wt);
      const double sr_rel = (sr_w / rr_w) * (RR_wt / SR_wt);
      const double dr_rel = (dr_w / rr_w) * (RR_wt / DR_wt);
      double w = sd_rel - sr_rel - dr_rel + 1.0;  // Landy-Szalay
      if (d.periodic_box) w = sd_rel - 1.0;
      fin.pd(h, i, k, 0, 0) = w;
      sd.pd(h, i, k, 0, 0) = sd_rel;
      sr.pd(h, i, k, 0, 0) = sr_rel;
      dr.pd(h, i, k, 0, 0) = dr_rel;
      rr.pd(h, i, k, 0, 0) = 1.0;
      if (d.which_corr == 0) continue;
      for (int j = 1; j < 7; j++) {
        const double sd_val = sd.pd(h, i, k, j, 0), sr_val = sr.pd(h, i, k, j, 0);
        double sd_norm = 0, sr_norm = 0;
        if (d.which_corr == 5 && j == 6) {  // ED: mean cos^2 minus its isotropic 1/3
          if (sd_num > 0) sd_norm = sd_val / sd_w;
          sd_norm -= 1. / 3;
        } else {
          sd_norm = (sd_val / rr_w) * (RR_wt / SD_wt);
          sr_norm = (sr_val / rr_w) * (RR_wt / SR_wt);
        }
        double val = sd_norm - sr_norm;
        if (sd_num == 0 || sr_num == 0 || rr_num == 0) {
          val = 0;
          if (d.periodic_box) val = sd_norm;
        }
        fin.pd(h, i, k, j, 0) = val;
        sr.pd(h, i, k, j, 0) = sr_norm;  // sd keeps its raw sum
        if (j == 6) {
          sd.pd(h, i, k, j, 0) = sd_num == 0 ? 0.0 : sd_val;
          sr.pd(h, i, k, j, 0) = sr_num == 0 ? 0.0 : sr_val;
        }
      }
    }
  }
}

// int_calc (bins_calcs.cpp:331-357): integrate over Pi
void integrate(Bins &b, int h, const Info &d) {
  const double dC = d.p_size;
  for (int i = 0; i < b.nb; i++) {
    const size_t bi = b.bi(h, i);
    for (int k = 0; k < b.np; k++) {
      const size_t c = b.pi(h, i, k);
      b.bwt[bi] += b.pwt[c];
      for (int j = 0; j < 7; j++) {
        b.bd(h, i, j, 0) += b.pd(h, i, k, j, 0) * dC;
        b.bd(h, i, j, 1) += std::pow(b.pd(h, i, k, j, 1) * dC, 2);
      }
      b.bls[bi] += std::pow(b.pls[c] * dC, 2);
    }
    for (int j = 0; j < 7; j++) b.bd(h, i, j, 1) = std::sqrt(b.bd(h, i, j, 1));
    b.bls[bi] = std::sqrt(b.bls[bi]);
  }
}

// final_calc (6-argument form, bins_calcs.cpp:30-52)
void final_calc(Info &d, Bins &sd, Bins &sr, Bins &dr, Bins &rr, Bins &fin, int h) {
  auto rel = [](const double *w) { return w[1] / std::pow(w[0], 2); };
  d.SD_wt[0] = d.S_wt[0] * d.D_wt[0];
  d.SD_wt[1] = d.SD_wt[0] * std::sqrt(rel(d.S_wt) + rel(d.D_wt));
  d.DRs_wt[0] = d.Rs_wt[0] * d.D_wt[0];
  d.DRs_wt[1] = d.DRs_wt[0] * std::sqrt(rel(d.Rs_wt) + rel(d.D_wt));
  d.SRd_wt[0] = d.S_wt[0] * d.Rd_wt[0];
  d.SRd_wt[1] = d.SRd_wt[0] * std::sqrt(rel(d.S_wt) + rel(d.Rd_wt));
  d.RsRd_wt[0] = d.Rs_wt[0] * d.Rd_wt[0] * d.include_prob_RR * d.include_prob_RR;
  d.RsRd_wt[1] = d.RsRd_wt[0] * std::sqrt(rel(d.Rs_wt) + rel(d.Rd_wt));
  if (d.periodic_box) {
    d.RsRd_wt[0] = 1;
    d.RsRd_wt[1] = 0;
    rr_periodic(rr, h, d);
  }
  final_bins(sd, sr, dr, rr, fin, h, d);
  integrate(sd, h, d);
  integrate(sr, h, d);
  integrate(dr, h, d);
  integrate(rr, h, d);
  integrate(fin, h, d);
}

// jk_final / jk_final2D (bins_calcs.cpp:393-462): value of the full sample,
// error from the spread of the delete-one samples
void jk_final(Bins &out, Bins &fin, const Info &d) {
  const int nj = d.n_jk;
  const double f = (nj - 1.0) / nj;
  for (int i = 0; i < fin.nb; i++) {
    for (int j = 0; j < 7; j++) {
      double mean = 0, var = 0;
      for (int r = 1; r <= nj; r++) mean += fin.bd(r, i, j, 0);
      mean /= nj;
      for (int r = 1; r <= nj; r++) var += std::pow(fin.bd(r, i, j, 0) - mean, 2.0);
      var *= f;
      out.bd(0, i, j, 0) = fin.bd(0, i, j, 0);
      out.bd(0, i, j, 1) = std::sqrt(var);
    }
    for (int k = 0; k < fin.np; k++)
      for (int j = 0; j < 7; j++) {
        double mean = 0, var = 0;
        for (int r = 1; r <= nj; r++) mean += fin.pd(r, i, k, j, 0);
        mean /= nj;
        for (int r = 1; r <= nj; r++) var += std::pow(fin.pd(r, i, k, j, 0) - mean, 2.0);
        var *= f;
        out.pd(0, i, k, j, 0) = fin.pd(0, i, k, j, 0);
        out.pd(0, i, k, j, 1) = std::sqrt(var);
      }
  }
}

// re_bin (bins_calcs.cpp:465-530): fold each negative-Pi bin of sample h onto
// its mirror bin (estimators 2, 3), with the reference's edge checks
void re_bin(Bins &b, int h, const Info &d) {
  if (d.n_p_bin <= 1) return;
  for (int i = 0; i < b.nb; i++) {
    for (int k = 0; k < b.np; k++) {
      if (b.p_min[k] >= 0) break;  // only negative bins move
      const double p_val = 0.0 - (b.p_min[k] + b.p_max[k]) / 2.0;
      int p = (int)std::floor((p_val - d.p_min) / d.p_size);
      bool found = false;
      for (;;) {
        if (p < 0 || p >= d.n_p_bin) break;
        if (p_val < b.p_min[p]) p--;
        else if (p_val > b.p_max[p]) p++;
        else { found = true; break; }
      }
      if (!found) break;  // the reference leaves the Pi loop here
      if (std::fabs(b.p_min[k] + b.p_max[p]) > (d.p_size / 100.) ||
          std::fabs(b.p_max[k] + b.p_min[p]) > (d.p_size / 100.) || b.p_max[p] < 0)
        continue;  // "rebinning problem": bin left in place
      const size_t from = b.pi(h, i, k), to = b.pi(h, i, p);
      b.pnum[to] += b.pnum[from];
      b.pnum[from] = 0;
      b.pwt[to] += b.pwt[from];
      b.pwt[from] = 0;
      b.pls[to] += b.pls[from];
      b.pls[from] = 0;
      for (int j = 0; j < 7; j++)
        for (int e = 0; e < 2; e++) {
          b.pd(h, i, p, j, e) += b.pd(h, i, k, j, e);
          b.pd(h, i, k, j, e) = 0;
        }
    }
  }
}

// final_calc_auto (bins_calcs.cpp:54-91) for sample h: SS normalised by
// S_wt^2 / 2, SR by S_wt Rs_wt, RR by Rs_wt^2 (halved when the randoms pairs
// were counted once by corels1) or the analytic periodic RR
void final_calc_auto(Info &d, Bins &ss, Bins &sr, Bins &rr, Bins &fin, int h) {
  auto rel = [](const double *w) { return w[1] / std::pow(w[0], 2); };
  const double SS_wt = d.S_wt[0] * d.S_wt[0] / 2.0;
  const double SS_err = SS_wt * std::sqrt(rel(d.S_wt) + rel(d.S_wt));
  const double SR_wt = d.S_wt[0] * d.Rs_wt[0];
  const double SR_err = SR_wt * std::sqrt(rel(d.S_wt) + rel(d.Rs_wt));
  double RR_wt = d.Rs_wt[0] * d.Rs_wt[0] * d.include_prob_RR * d.include_prob_RR;
  double RR_err = RR_wt * std::sqrt(rel(d.Rs_wt) + rel(d.Rs_wt));
  if (!d.RsRd_same) {
    RR_wt /= 2.0;
    RR_err /= 2.0;
  }
  if (d.periodic_box) {
    RR_wt = 1;
    RR_err = 0;
    rr_periodic(rr, h, d);
    if (d.do_auto_rebin) re_bin(rr, h, d);
  }
  d.SD_wt[0] = SS_wt; d.SD_wt[1] = SS_err;
  d.SRd_wt[0] = SR_wt; d.SRd_wt[1] = SR_err;
  d.RsRd_wt[0] = RR_wt; d.RsRd_wt[1] = RR_err;
  d.DRs_wt[0] = SR_wt; d.DRs_wt[1] = SR_err;
  final_bins(ss, sr, sr, rr, fin, h, d);  // DR = SR (bins_calcs.cpp:88)
  integrate(ss, h, d);
  integrate(rr, h, d);
  integrate(sr, h, d);
  integrate(fin, h, d);
}

// One output table: sample h of a bin tree, as outp_bins (1-D) or outp_2Dbins.
struct OutTable {
  const Bins *b;
  int h;
  bool two_d;
  std::string path;
};

// Write the tables on the host's cores (each file depends only on its own
// sample, which is final once queued); nonzero if any could not be written.
int write_tables(const std::vector<OutTable> &ts) {
  std::atomic<int> bad{0};
  run_parallel((int64_t)ts.size(), [&](int64_t i) {
    const OutTable &t = ts[i];
    if ((t.two_d ? outp_2Dbins(*t.b, t.h, t.path) : outp_bins(*t.b, t.h, t.path)) != 0) bad = 1;
  });
  return bad.load();
}

}  // namespace

// do_bining's auto part (do_corr.cpp:220-324)
int do_bining_auto(Info &d, Bins &SS, Bins &SRs, Bins &RsRs, std::string &err) {
  const std::string &o = d.out_file;
  int bad = 0;
  std::vector<OutTable> out;
  if (d.do_auto_rebin) {
    re_bin(SS, 0, d);
    re_bin(SRs, 0, d);
    re_bin(RsRs, 0, d);
    bad |= outp_2Dbins(SRs, 0, o + "bins_auto_SR2.temp");
  }
  Bins fin, jk;
  fin.init(d, SS.nh);
  final_calc_auto(d, SS, SRs, RsRs, fin, 0);
  out.push_back({&fin, 0, false, o + "bins_auto_final.dat"});
  out.push_back({&SS, 0, false, o + "bins_auto_SS.dat"});
  out.push_back({&SRs, 0, false, o + "bins_auto_SR.dat"});
  out.push_back({&RsRs, 0, false, o + "bins_auto_RR.dat"});
  out.push_back({&fin, 0, true, o + "bins2D_auto_final.dat"});
  out.push_back({&SS, 0, true, o + "bins2D_auto_SS.dat"});
  out.push_back({&SRs, 0, true, o + "bins2D_auto_SR.dat"});
  out.push_back({&RsRs, 0, true, o + "bins2D_auto_RR.dat"});
  if (d.do_jk) {
    for (int r = 0; r < d.n_jk; r++) {
      const int h = r + 1;
      if (d.do_auto_rebin) {
        re_bin(SS, h, d);
        re_bin(RsRs, h, d);
        re_bin(SRs, h, d);
      }
      final_calc_auto(d, SS, SRs, RsRs, fin, h);
      const std::string s = o + "bins_auto_jk" + std::to_string(r);
      const std::string s2 = o + "bins2D_auto_jk" + std::to_string(r);
      out.push_back({&SS, h, false, s + "_SS.dat"});
      out.push_back({&RsRs, h, false, s + "_RR.dat"});
      out.push_back({&SRs, h, false, s + "_SR.dat"});
      out.push_back({&fin, h, false, s + "_final.dat"});
      out.push_back({&fin, h, true, s2 + "_final.dat"});
      out.push_back({&SS, h, true, s2 + "_SS.dat"});
      out.push_back({&RsRs, h, true, s2 + "_RR.dat"});
      out.push_back({&SRs, h, true, s2 + "_SR.dat"});
    }
    if (d.do_jk == 1) {
      jk.init(d, 1);
      jk_final(jk, fin, d);
      out.push_back({&jk, 0, false, o + "bins_auto_jk_final.dat"});
      out.push_back({&jk, 0, true, o + "bins2D_auto_jk_final.dat"});
    }
  }
  bad |= write_tables(out);
  if (bad) {
    err = "could not write output files with prefix " + o;
    return 1;
  }
  return 0;
}

// add_bins of do_corr.cpp:135-155: b += a over every sample and field
void add_bins(Bins &b, const Bins &a) {
  for (size_t k = 0; k < b.bnum.size(); k++) b.bnum[k] += a.bnum[k];
  for (size_t k = 0; k < b.bwt.size(); k++) b.bwt[k] += a.bwt[k];
  for (size_t k = 0; k < b.bdat.size(); k++) b.bdat[k] += a.bdat[k];
  for (size_t k = 0; k < b.bls.size(); k++) b.bls[k] += a.bls[k];
  for (size_t k = 0; k < b.bsig.size(); k++) b.bsig[k] += a.bsig[k];
  for (size_t k = 0; k < b.pnum.size(); k++) b.pnum[k] += a.pnum[k];
  for (size_t k = 0; k < b.pwt.size(); k++) b.pwt[k] += a.pwt[k];
  for (size_t k = 0; k < b.pdat.size(); k++) b.pdat[k] += a.pdat[k];
  for (size_t k = 0; k < b.pls.size(); k++) b.pls[k] += a.pls[k];
}

// do_bining (do_corr.cpp:203-433): the temporary SR files, then the auto and
// the cross parts as the estimator asks
int do_bining(Info &d, Bins &SS, Bins &SRs, Bins &RsRs, Bins &SD, Bins &SRd, Bins &DRs,
              Bins &RsRd, std::string &err) {
  const std::string &o = d.out_file;
  if (outp_2Dbins(SRs, 0, o + "bins_auto_SR.temp") || outp_2Dbins(SRd, 0, o + "bins_cross_SR.temp")) {
    err = "could not write output files with prefix " + o;
    return 1;
  }
  if (d.do_auto_corr && do_bining_auto(d, SS, SRs, RsRs, err)) return 1;
  if (d.do_cross_corr && do_bining_cross(d, SD, SRd, DRs, RsRd, err)) return 1;
  return 0;
}

int do_bining_cross(Info &d, Bins &SD, Bins &SRd, Bins &DRs, Bins &RsRd, std::string &err) {
  const std::string &o = d.out_file;
  int bad = 0;
  std::vector<OutTable> out;
  Bins fin, jk;
  fin.init(d, SD.nh);
  final_calc(d, SD, SRd, DRs, RsRd, fin, 0);
  out.push_back({&fin, 0, false, o + "bins_cross_final.dat"});
  out.push_back({&fin, 0, true, o + "bins2D_cross_final.dat"});
  out.push_back({&SD, 0, false, o + "bins_cross_SD.dat"});
  out.push_back({&SD, 0, true, o + "bins2D_cross_SD.dat"});
  out.push_back({&SRd, 0, false, o + "bins_cross_SR.dat"});
  out.push_back({&SRd, 0, true, o + "bins2D_cross_SR.dat"});
  out.push_back({&DRs, 0, false, o + "bins_cross_DR.dat"});
  out.push_back({&DRs, 0, true, o + "bins2D_cross_DR.dat"});
  out.push_back({&RsRd, 0, false, o + "bins_cross_RR.dat"});
  out.push_back({&RsRd, 0, true, o + "bins2D_cross_RR.dat"});
  if (d.do_jk) {
    for (int r = 0; r < d.n_jk; r++) {
      const int h = r + 1;
      final_calc(d, SD, SRd, DRs, RsRd, fin, h);
      const std::string s = o + "bins_cross_jk" + std::to_string(r);
      const std::string s2 = o + "bins2D_cross_jk" + std::to_string(r);
      out.push_back({&SD, h, false, s + "_SD.dat"});
      out.push_back({&RsRd, h, false, s + "_RR.dat"});
      out.push_back({&DRs, h, false, s + "_DR.dat"});
      out.push_back({&SRd, h, false, s + "_SR.dat"});
      out.push_back({&fin, h, false, s + "_final.dat"});
      out.push_back({&fin, h, true, s2 + "_final.dat"});
      out.push_back({&SD, h, true, s2 + "_SD.dat"});
      out.push_back({&RsRd, h, true, s2 + "_RR.dat"});
      out.push_back({&DRs, h, true, s2 + "_DR.dat"});
      out.push_back({&SRd, h, true, s2 + "_SR.dat"});
    }
    jk.init(d, 1);
    jk_final(jk, fin, d);
    out.push_back({&jk, 0, false, o + "bins_cross_jk_final.dat"});
    out.push_back({&jk, 0, true, o + "bins2D_cross_jk_final.dat"});
  }
  bad |= write_tables(out);
  if (bad) {
    err = "could not write output files with prefix " + o;
    return 1;
  }
  return 0;
}

}  // namespace cpch

// C ABI: finalisation and output files of a cross run from raw histogram
// blocks (the cpc_count layout), e.g. blocks counted elsewhere or summed over
// several processes.  NULL term arrays are empty terms.
extern "C" cpc_status cpc_host_finalize_cross(const char *inp_path, const int64_t *sd_num,
                                              const double *sd_sums, const int64_t *srd_num,
                                              const double *srd_sums, const int64_t *drs_num,
                                              const double *drs_sums, const int64_t *rsrd_num,
                                              const double *rsrd_sums, const double *weights) try {
  using namespace cpch;
  if (!inp_path || !weights) return CPC_ERR_INVALID;
  Info d;
  std::string err;
  if (read_inp(inp_path, d, err) || derive_info(d, err)) return CPC_ERR_INVALID;
  d.S_wt[0] = weights[0]; d.S_wt[1] = weights[1];
  d.D_wt[0] = weights[2]; d.D_wt[1] = weights[3];
  d.Rs_wt[0] = weights[4]; d.Rs_wt[1] = weights[5];
  d.Rd_wt[0] = weights[6]; d.Rd_wt[1] = weights[7];
  const int nh = 1 + (d.do_jk ? d.n_jk : 0);
  Bins SD, SRd, DRs, RsRd;
  SD.init(d, nh); SRd.init(d, nh); DRs.init(d, nh); RsRd.init(d, nh);
  const int64_t *nums[4] = {sd_num, srd_num, drs_num, rsrd_num};
  const double *sums[4] = {sd_sums, srd_sums, drs_sums, rsrd_sums};
  Bins *terms[4] = {&SD, &SRd, &DRs, &RsRd};
  for (int k = 0; k < 4; k++)
    if (nums[k] && sums[k]) add_count(*terms[k], d, nums[k], sums[k]);
  outp_data_info(d, d.out_file + "inp.info");
  Bins SS, SRs, RsRs;
  SS.init(d, nh); SRs.init(d, nh); RsRs.init(d, nh);
  d.do_auto_corr = 0;
  d.do_cross_corr = 1;
  if (do_bining(d, SS, SRs, RsRs, SD, SRd, DRs, RsRd, err)) return CPC_ERR_INVALID;
  outp_data_info(d, d.out_file + "inp2.info");
  return CPC_OK;
} catch (const std::bad_alloc &) {
  return CPC_ERR_NOMEM;
} catch (...) {
  return CPC_ERR_HOST;
}

// C ABI: finalisation and output files of an auto-correlation run (the auto
// part of do_bining) from RAW histogram blocks of SS (corels1), SRs and RsRs
// (corels1, or corels2 of the randoms with themselves when RsRd_same).
extern "C" cpc_status cpc_host_finalize_auto(const char *inp_path, const int64_t *ss_num,
                                             const double *ss_sums, const int64_t *srs_num,
                                             const double *srs_sums, const int64_t *rsrs_num,
                                             const double *rsrs_sums, const double *weights) try {
  using namespace cpch;
  if (!inp_path || !weights) return CPC_ERR_INVALID;
  Info d;
  std::string err;
  if (read_inp(inp_path, d, err) || derive_info(d, err)) return CPC_ERR_INVALID;
  d.S_wt[0] = weights[0]; d.S_wt[1] = weights[1];
  d.Rs_wt[0] = weights[4]; d.Rs_wt[1] = weights[5];
  const int nh = 1 + (d.do_jk ? d.n_jk : 0);
  Bins SS, SRs, RsRs;
  SS.init(d, nh); SRs.init(d, nh); RsRs.init(d, nh);
  if (ss_num && ss_sums) add_count(SS, d, ss_num, ss_sums);
  if (srs_num && srs_sums) add_count(SRs, d, srs_num, srs_sums);
  if (rsrs_num && rsrs_sums) add_count(RsRs, d, rsrs_num, rsrs_sums);
  outp_data_info(d, d.out_file + "inp.info");
  if (do_bining_auto(d, SS, SRs, RsRs, err)) return CPC_ERR_INVALID;
  outp_data_info(d, d.out_file + "inp2.info");
  return CPC_OK;
} catch (const std::bad_alloc &) {
  return CPC_ERR_NOMEM;
} catch (...) {
  return CPC_ERR_HOST;
}
