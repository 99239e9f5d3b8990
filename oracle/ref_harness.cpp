// Test harness around the UNMODIFIED reference corr_pc sources (compiled from
// the reference tree by oracle/Makefile; nothing of the reference is copied
// here).  It replays the reference driver's sequence for one .inp file and
// dumps every raw pair-count histogram tree (bin_jk) at full precision, so
// the repository's C restatement (oracle/cpc_oracle.c) and the GPU path can
// be pinned against the reference itself.
//
// Sequence followed: main.cpp:27-82 (data_ini, inp.info) and do_corr.cpp:24-161
// (read order S, Rs, D, Rd -- which fixes the glibc rand() stream used for the
// periodic-box jackknife draws -- then the corels2/corels1 calls per estimator,
// then do_bining which writes the reference's own output files).
//
// Usage: ref_harness <file.inp> <dump.txt> [--no-bining] [--drs-wgg]
// Test infrastructure only: the product never links or runs this.
#include <cstdio>
#include <cstring>
#include <iostream>
#include <string>

#include "data_def.h"
#include "initialization.h"
#include "read_dat.h"
#include "corr.h"
#include "jk.h"
#include "outp.h"
#include "bins_calcs.h"
#include "do_corr.h"

static void dump_bin_jk(FILE *f, const char *term, long n_in, bin_jk &bjk,
                        data_info &d) {
  int n_jk = d.do_jk ? d.n_jk : 0;
  std::fprintf(f, "T %s %ld %d %d %d\n", term, n_in, d.n_bins, d.n_p_bin, n_jk);
  for (int h = 0; h <= n_jk; h++) {
    bin *b = (h == 0) ? bjk.b : bjk.jk[h - 1].b;
    for (int i = 0; i < d.n_bins; i++) {
      std::fprintf(f, "B %d %d %ld %.17g", h, i, b[i].num, b[i].wt_num);
      for (int j = 0; j < 7; j++)
        std::fprintf(f, " %.17g %.17g", b[i].data[j].val, b[i].data[j].err);
      std::fprintf(f, "\n");
      for (int k = 0; k < d.n_p_bin; k++) {
        P_bin &p = b[i].p_bin[k];
        std::fprintf(f, "P %d %d %d %ld %.17g", h, i, k, p.num, p.wt_num);
        for (int j = 0; j < 7; j++)
          std::fprintf(f, " %.17g %.17g", p.data[j].val, p.data[j].err);
        std::fprintf(f, "\n");
      }
    }
  }
}

int main(int argc, char **argv) {
  if (argc < 3) {
    std::fprintf(stderr, "usage: %s file.inp dump.txt [--no-bining]\n", argv[0]);
    return 2;
  }
  bool bining = true, drs_wgg = false;
  for (int a = 3; a < argc; a++) {
    if (std::strcmp(argv[a], "--no-bining") == 0) bining = false;
    if (std::strcmp(argv[a], "--drs-wgg") == 0) drs_wgg = true;
  }
  data_info d = data_info();
  if (data_ini(d, argv[1]) != 0) {
    std::printf("Bad initialization!! Bye\n");
    return 1;
  }
  outp_data_info(d, d.out_file + "inp.info");
  FILE *f = std::fopen(argv[2], "w");
  if (!f) return 1;
  std::fprintf(f, "W %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g\n",
               d.S_wt.val, d.S_wt.err, d.D_wt.val, d.D_wt.err, d.Rs_wt.val,
               d.Rs_wt.err, d.Rd_wt.val, d.Rd_wt.err);

  // do_corr.cpp:24-157, replayed step by step so each term can be dumped.
  gal *gshape = 0, *grand_density = 0, *grand_shape = 0, *gdensity = 0;
  int bbye = 0;
  bool RsRd_same = d.RsRd_same;
  bins B;
  bins_ini(B, d);
  d.do_SS = 1;
  gshape = new gal[d.n_shape];
  bbye = read_data(gshape, d);
  d.do_SS = 0;
  if (!d.periodic_box || (d.periodic_box && d.n_jk > 0)) {
    d.do_RsRs = 1;
    grand_shape = new gal[d.n_shape_rand];
    bbye += read_data(grand_shape, d);
    d.do_RsRs = 0;
  }
  if (bbye != 0) return 1;
  long n;
  if (d.do_auto_corr) {
    d.do_SS = 1;
    n = corels1(gshape, B.SS, d);
    d.do_SS = 0;
    dump_bin_jk(f, "SS", n, B.SS, d);
  }
  if ((d.do_auto_corr || RsRd_same) && (!d.periodic_box)) {
    d.do_SRs = 1;
    n = corels2(grand_shape, gshape, B.SRs, d);
    d.do_SRs = 0;
    dump_bin_jk(f, "SRs", n, B.SRs, d);
    d.do_RsRs = 1;
    if (!d.RsRd_same) {
      n = corels1(grand_shape, B.RsRs, d);
      d.do_RsRs = 0;
      dump_bin_jk(f, "RsRs", n, B.RsRs, d);
    } else {
      n = corels2(grand_shape, grand_shape, B.RsRd, d);
      d.do_RsRs = 0;
      dump_bin_jk(f, "RsRd", n, B.RsRd, d);
    }
  }
  if (d.do_cross_corr) {
    d.do_DD = 1;
    gdensity = new gal[d.n_density];
    bbye += read_data(gdensity, d);
    d.do_DD = 0;
    if (!RsRd_same) {
      d.do_RsRd = 1;
      grand_density = new gal[d.n_density_rand];
      bbye += read_data(grand_density, d);
      d.do_RsRd = 0;
      if (bbye != 0) return 1;
      d.do_SRd = 1;
      n = corels2(grand_density, gshape, B.SRd, d);
      d.do_SRd = 0;
      dump_bin_jk(f, "SRd", n, B.SRd, d);
      d.do_RsRd = 1;
      n = corels2(grand_density, grand_shape, B.RsRd, d);
      d.do_RsRd = 0;
      dump_bin_jk(f, "RsRd", n, B.RsRd, d);
    } else {
      grand_density = grand_shape;
    }
    if (bbye != 0) return 1;
    d.do_SD = 1;
    n = corels2(gdensity, gshape, B.SD, d);
    d.do_SD = 0;
    dump_bin_jk(f, "SD", n, B.SD, d);
    if (!d.periodic_box) {
      // --drs-wgg: run this term as a density-density count.  With which_corr
      // 1 the reference's DRs term rotates the ellipticities of randoms that
      // were read without any (an uninitialised pointer, corels.cpp:216-219)
      // and crashes; its counts and weights do not depend on which_corr.
      const int wc = d.which_corr;
      if (drs_wgg) d.which_corr = 0;
      d.do_DRs = 1;
      n = corels2(grand_shape, gdensity, B.DRs, d);
      d.do_DRs = 0;
      d.which_corr = wc;
      dump_bin_jk(f, "DRs", n, B.DRs, d);
    }
  }
  std::fprintf(f, "W %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g\n",
               d.S_wt.val, d.S_wt.err, d.D_wt.val, d.D_wt.err, d.Rs_wt.val,
               d.Rs_wt.err, d.Rd_wt.val, d.Rd_wt.err);
  std::fclose(f);
  if (!bining) return 0;
  // do_corr.cpp:135-161 then main.cpp:79-81: the reference's own finalisation
  // and output files (used for file-level parity of the host finalisation).
  if (RsRd_same && (!d.periodic_box)) {
    bool sub = false;
    add_bins(B.RsRs.b, B.RsRd.b, B.RsRs.b, d, sub);
    add_bins(B.SRd.b, B.SRs.b, B.SRd.b, d, sub);
    d.RsRs_wt.val *= 2.0;
    d.RsRs_wt.err *= 2.0;
    d.Rd_wt.err = d.Rs_wt.err;
    d.Rd_wt.val = d.Rs_wt.val;
    if (d.do_jk)
      for (int i = 0; i < d.n_jk; i++) {
        add_bins(B.RsRs.jk[i].b, B.RsRd.jk[i].b, B.RsRs.jk[i].b, d, sub);
        add_bins(B.SRd.jk[i].b, B.SRs.jk[i].b, B.SRd.jk[i].b, d, sub);
      }
  }
  do_bining(B, d);
  outp_data_info(d, d.out_file + "inp2.info");
  return 0;
}
