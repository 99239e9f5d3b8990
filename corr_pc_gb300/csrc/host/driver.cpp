// driver.cpp -- the corr_pc command line on the GPU pair loop:
//     corr_pc_gb300 <file.inp> [--engine fast|fp64]
// Same argument, same parameter file, same input and output files as the
// reference's corr_pc (main.cpp:27-82).  The sequence follows do_corr for a
// cross-correlation run (do_corr.cpp:24-161): read S, Rs, D, Rd in that order
// (which fixes the glibc rand() jackknife draws), one GPU corels2 per pair
// type (SRd, RsRd, SD, DRs; SD alone in a periodic box), then the finalisation
// and output files.
#include <chrono>
#include <cstdio>
#include <cstring>
#include <iostream>
#include <string>

#include "host.h"

using namespace cpch;

namespace {

struct Ctx {
  cpc_ctx *c = nullptr;
  ~Ctx() { cpc_destroy(c); }
};

int count_term(Ctx &ctx, Info &d, cpc_pair_kind kind, int s1, int s2, Bins &out, cpc_engine eng) {
  int nh, nb, np;
  cpc_accum_shape(ctx.c, &nh, &nb, &np);
  std::vector<int64_t> num((size_t)nh * nb * np);
  std::vector<double> sums(num.size() * CPC_NF);
  cpc_accum acc{};
  acc.num = num.data();
  acc.sums = sums.data();
  const auto t0 = std::chrono::steady_clock::now();
  const cpc_status s = cpc_count(ctx.c, kind, s1, s2, eng, 1, 0, &acc);
  const double dt = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  if (s != CPC_OK) {
    std::cout << "corels2 on the GPU failed: " << cpc_last_error(ctx.c) << std::endl;
    return 1;
  }
  add_count(out, d, num.data(), sums.data());
  std::cout << "corel2 ends::time: " << dt << "  total pair= " << acc.n_window
            << "\tpairs out= " << acc.n_window - acc.n_binned << "   pairs in=" << acc.n_binned
            << "    PB=0" << std::endl;
  return 0;
}

}  // namespace

int main(int argc, char **argv) {
  std::cout << "Beginning corr_pc_gb300 (" << cpc_version() << ")" << std::endl;
  if (argc < 2) {
    std::cout << "no input file given!!" << std::endl << "Bad initialization!! Bye" << std::endl;
    return 1;
  }
  cpc_engine eng = CPC_ENGINE_FAST;
  for (int a = 2; a < argc; a++)
    if (!std::strcmp(argv[a], "--engine") && a + 1 < argc)
      eng = std::strcmp(argv[++a], "fp64") == 0 ? CPC_ENGINE_FP64 : CPC_ENGINE_FAST;
  Info d;
  std::string err;
  if (read_inp(argv[1], d, err) || derive_info(d, err)) {
    std::cout << err << std::endl << "Bad initialization!! Bye" << std::endl;
    return 1;
  }
  outp_data_info(d, d.out_file + "inp.info");
  if ((d.coordinates != 6 && d.coordinates != 0) || d.estimator != 0 || d.which_corr > 2 ||
      d.sig_crit) {
    std::cout << "this build runs cross correlations (estimator 0) of wgg/wg+/w++ in x,y,z "
                 "(coordinates 6) or on the sky (coordinates 0)" << std::endl;
    return 1;
  }
  if (d.RsRd_same && !d.periodic_box) {
    std::cout << "without a periodic box this build needs separate density randoms "
                 "(n_Drand > 0)" << std::endl;
    return 1;
  }
  Ctx ctx;
  cpc_params p = to_params(d);
  if (cpc_create(&ctx.c, &p) != CPC_OK) {
    std::cout << "GPU context: " << cpc_last_error(nullptr) << std::endl;
    return 1;
  }
  // do_corr.cpp:40-96: read order S, Rs, D, Rd; slots 0..3
  int64_t draws = 0;
  Catalog S, Rs, D, Rd;
  if (read_catalog(d, ROLE_S, S, draws, err)) { std::cout << err << std::endl; return 1; }
  if (!d.periodic_box || d.n_jk > 0)
    if (read_catalog(d, ROLE_RS, Rs, draws, err)) { std::cout << err << std::endl; return 1; }
  if (read_catalog(d, ROLE_D, D, draws, err)) { std::cout << err << std::endl; return 1; }
  if (!d.RsRd_same)
    if (read_catalog(d, ROLE_RD, Rd, draws, err)) { std::cout << err << std::endl; return 1; }
  const Catalog *cats[4] = {&S, &Rs, &D, &Rd};
  for (int k = 0; k < 4; k++) {
    if (k == 3 && d.RsRd_same) continue;
    cpc_catalog v = cats[k]->view();
    if (cpc_upload(ctx.c, k, &v) != CPC_OK) {
      std::cout << "upload: " << cpc_last_error(ctx.c) << std::endl;
      return 1;
    }
  }
  const int nh = 1 + (d.do_jk ? d.n_jk : 0);
  Bins SD, SRd, DRs, RsRd;
  SD.init(d, nh); SRd.init(d, nh); DRs.init(d, nh); RsRd.init(d, nh);
  const int rd_slot = d.RsRd_same ? 1 : 3;
  if (!d.RsRd_same) {
    if (count_term(ctx, d, CPC_PAIR_SRD, rd_slot, 0, SRd, eng)) return 1;
    if (count_term(ctx, d, CPC_PAIR_RSRD, rd_slot, 1, RsRd, eng)) return 1;
  }
  if (count_term(ctx, d, CPC_PAIR_SD, 2, 0, SD, eng)) return 1;
  if (!d.periodic_box)
    if (count_term(ctx, d, CPC_PAIR_DRS, 1, 2, DRs, eng)) return 1;
  if (do_bining_cross(d, SD, SRd, DRs, RsRd, err)) {
    std::cout << err << std::endl;
    return 1;
  }
  std::cout << "Binning done" << std::endl;
  outp_data_info(d, d.out_file + "inp2.info");
  return 0;
}
