// driver.cpp -- the corr_pc command line on the GPU pair loop:
//     corr_pc_gb300 <file.inp> [--engine fast|fp64]
//     corr_pc_gb300 --batch <a.inp> <b.inp> ... [--engine fast|fp64]
// Same argument, same parameter file, same input and output files as the
// reference's corr_pc (main.cpp:27-82).  The sequence follows do_corr
// (do_corr.cpp:24-161): read S, Rs, D, Rd in that order (which fixes the glibc
// rand() jackknife draws); the auto pair types (SS by corels1; SRs and RsRs
// without a periodic box) for estimators 1-3; the cross pair types (SRd, RsRd,
// SD, DRs; SD alone in a periodic box) for estimators 0 and 3; then the
// finalisation and output files.
// --batch runs several periodic-box cross runs (e.g. the sub-boxes of one
// simulation, each its own .inp, catalogues and output prefix) as the reference
// would run them one after another, except that their SD terms are counted
// together in one persistent launch (cpc_count_batch); every run still writes
// its own files.
#include <chrono>
#include <cstdio>
#include <cstring>
#include <iostream>
#include <memory>
#include <string>
#include <vector>

#include "host.h"

using namespace cpch;

namespace {

struct Ctx {
  cpc_ctx *c = nullptr;
  ~Ctx() { cpc_destroy(c); }
};

// one counted pair type, for the run record
struct TermRecord {
  std::string name;
  int64_t n_window, n_binned, n_rechecked;
  double wall_s, kernel_ms;
};

const char *term_name(cpc_pair_kind k) {
  static const char *names[] = {"SD", "SRd", "DRs", "RsRd", "RsRs", "SRs", "SS"};
  return (k >= CPC_PAIR_SD && k <= CPC_PAIR_SS) ? names[k] : "?";
}

// <out_file>run.json: the engine and, per pair type, the window and binned
// pairs, the pairs resolved by the FP64 recheck, the wall time of the call, the
// device time of the count and the binned pairs per second of device time
void write_run_record(const Info &d, cpc_engine eng, const std::vector<TermRecord> &g_terms) {
  FILE *f = std::fopen((d.out_file + "run.json").c_str(), "w");
  if (!f) return;
  std::fprintf(f, "{\"library\": \"%s\", \"engine\": \"%s\", \"terms\": [", cpc_version(),
               eng == CPC_ENGINE_FP64 ? "fp64" : "fast");
  for (size_t k = 0; k < g_terms.size(); k++) {
    const TermRecord &t = g_terms[k];
    std::fprintf(f,
                 "%s\n  {\"pair_type\": \"%s\", \"n_window\": %lld, \"n_binned\": %lld, "
                 "\"n_rechecked\": %lld, \"wall_s\": %.6g, \"kernel_ms\": %.6g, "
                 "\"binned_pairs_per_s\": %.6g}",
                 k ? "," : "", t.name.c_str(), (long long)t.n_window, (long long)t.n_binned,
                 (long long)t.n_rechecked, t.wall_s, t.kernel_ms,
                 t.kernel_ms > 0 ? t.n_binned / (t.kernel_ms * 1e-3) : 0.0);
  }
  std::fprintf(f, "\n]}\n");
  std::fclose(f);
}

// the reference's per-term log line (corr.cpp:457-458, 213-214) and the record
void log_term(std::vector<TermRecord> &terms, cpc_pair_kind kind, const cpc_accum &acc,
              double dt, bool auto_pairs) {
  terms.push_back(TermRecord{term_name(kind), acc.n_window, acc.n_binned, acc.n_rechecked, dt,
                             acc.kernel_ms});
  std::cout << (auto_pairs ? "corel 1 ends: time:" : "corel2 ends::time: ") << dt
            << "  total pair= " << acc.n_window
            << "\tpairs out= " << acc.n_window - acc.n_binned << "   pairs in=" << acc.n_binned
            << "    PB=0" << std::endl;
}

int count_term(Ctx &ctx, Info &d, cpc_pair_kind kind, int s1, int s2, Bins &out, cpc_engine eng,
               std::vector<TermRecord> &terms, bool auto_pairs = false) {
  int nh, nb, np;
  cpc_accum_shape(ctx.c, &nh, &nb, &np);
  std::vector<int64_t> num((size_t)nh * nb * np);
  std::vector<double> sums(num.size() * CPC_NF);
  cpc_accum acc{};
  acc.num = num.data();
  acc.sums = sums.data();
  const auto t0 = std::chrono::steady_clock::now();
  const cpc_status s = auto_pairs ? cpc_count_auto(ctx.c, kind, s1, eng, 1, 0, &acc)
                                  : cpc_count(ctx.c, kind, s1, s2, eng, 1, 0, &acc);
  const double dt = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  if (s != CPC_OK) {
    std::cout << "corels2 on the GPU failed: " << cpc_last_error(ctx.c) << std::endl;
    return 1;
  }
  add_count(out, d, num.data(), sums.data());
  log_term(terms, kind, acc, dt, auto_pairs);
  return 0;
}

// One run (one .inp): its parameters, GPU context, bin trees and catalogues.
struct Run {
  Info d;
  Ctx ctx;
  Bins SS, SRs, RsRs, SD, SRd, DRs, RsRd;
  Catalog S, Rs, D, Rd;
  std::vector<TermRecord> terms;
  bool box = false;
};

// Everything of a run up to its SD count (read, upload and count in do_corr's
// order); with defer_sd the SD count is left to the caller, which needs a
// periodic-box cross run (there SD is the last cross term).
int run_prepare(Run &r, const char *inp, cpc_engine eng, bool defer_sd) {
  Info &d = r.d;
  std::string err;
  if (read_inp(inp, d, err) || derive_info(d, err)) {
    std::cout << err << std::endl << "Bad initialization!! Bye" << std::endl;
    return 1;
  }
  outp_data_info(d, d.out_file + "inp.info");
  if ((d.coordinates != 6 && d.coordinates != 7 && d.coordinates != 0) || d.estimator < 0 ||
      d.estimator > 3 || d.which_corr < 0 || d.which_corr > 5 || d.sig_crit ||
      (d.coordinates == 7 && !d.periodic_box) || (d.coordinates == 0 && d.which_corr > 2)) {
    std::cout << "this build runs which_corr 0-5 with estimators 0-3 in x,y,z (coordinates 6; "
                 "7 in a periodic box) and which_corr 0-2 on the sky (coordinates 0)"
              << std::endl;
    return 1;
  }
  r.box = d.periodic_box != 0;
  if (defer_sd && !(r.box && d.do_cross_corr)) {
    std::cout << inp << ": --batch takes periodic-box cross runs (estimator 0 or 3)" << std::endl;
    return 1;
  }
  Ctx &ctx = r.ctx;
  cpc_params p = to_params(d);
  if (cpc_create(&ctx.c, &p) != CPC_OK) {
    std::cout << "GPU context: " << cpc_last_error(nullptr) << std::endl;
    return 1;
  }
  const bool box = r.box;
  const bool read_rs = !box || d.n_jk > 0;
  const int nh = 1 + (d.do_jk ? d.n_jk : 0);
  for (Bins *b : {&r.SS, &r.SRs, &r.RsRs, &r.SD, &r.SRd, &r.DRs, &r.RsRd}) b->init(d, nh);
  // do_corr.cpp:40-52: S, then the shape randoms; slots S 0, Rs 1, D 2, Rd 3
  int64_t draws = 0;
  TextCache files;  // S and D (Rs and Rd) naming the same files parse them once
  auto upload = [&](int slot, const Catalog &c) {
    cpc_catalog v = c.view();
    if (cpc_upload(ctx.c, slot, &v) != CPC_OK) {
      std::cout << "upload: " << cpc_last_error(ctx.c) << std::endl;
      return 1;
    }
    return 0;
  };
  if (read_catalog(d, ROLE_S, r.S, draws, err, &files)) { std::cout << err << std::endl; return 1; }
  if (upload(0, r.S)) return 1;
  if (read_rs) {
    if (read_catalog(d, ROLE_RS, r.Rs, draws, err, &files)) { std::cout << err << std::endl; return 1; }
    if (upload(1, r.Rs)) return 1;
  }
  // do_corr.cpp:56-81: auto pair types
  if (d.do_auto_corr)
    if (count_term(ctx, d, CPC_PAIR_SS, 0, 0, r.SS, eng, r.terms, true)) return 1;
  if ((d.do_auto_corr || d.RsRd_same) && !box) {
    if (count_term(ctx, d, CPC_PAIR_SRS, 1, 0, r.SRs, eng, r.terms)) return 1;
    if (!d.RsRd_same) {
      if (count_term(ctx, d, CPC_PAIR_RSRS, 1, 1, r.RsRs, eng, r.terms, true)) return 1;
    } else {
      if (count_term(ctx, d, CPC_PAIR_RSRS, 1, 1, r.RsRd, eng, r.terms)) return 1;
    }
  }
  // do_corr.cpp:83-133: cross pair types
  if (d.do_cross_corr) {
    if (read_catalog(d, ROLE_D, r.D, draws, err, &files)) { std::cout << err << std::endl; return 1; }
    if (upload(2, r.D)) return 1;
    if (d.RsRd_same) files = TextCache();  // D was the last sample read
    if (!d.RsRd_same) {
      if (read_catalog(d, ROLE_RD, r.Rd, draws, err, &files)) { std::cout << err << std::endl; return 1; }
      files = TextCache();
      if (upload(3, r.Rd)) return 1;
      if (count_term(ctx, d, CPC_PAIR_SRD, 3, 0, r.SRd, eng, r.terms)) return 1;
      if (count_term(ctx, d, CPC_PAIR_RSRD, 3, 1, r.RsRd, eng, r.terms)) return 1;
    }
    if (defer_sd) return 0;
    if (count_term(ctx, d, CPC_PAIR_SD, 2, 0, r.SD, eng, r.terms)) return 1;
    if (!box)
      if (count_term(ctx, d, CPC_PAIR_DRS, 1, 2, r.DRs, eng, r.terms)) return 1;
  }
  return 0;
}

// After the counts: the random-sample merge, finalisation, files, run record.
int run_finish(Run &r, cpc_engine eng) {
  Info &d = r.d;
  std::string err;
  // do_corr.cpp:135-155: with one random sample the auto terms feed the cross ones
  if (d.RsRd_same && !r.box) {
    add_bins(r.RsRs, r.RsRd);
    add_bins(r.SRd, r.SRs);
    d.Rd_wt[0] = d.Rs_wt[0];
    d.Rd_wt[1] = d.Rs_wt[1];
  }
  if (do_bining(d, r.SS, r.SRs, r.RsRs, r.SD, r.SRd, r.DRs, r.RsRd, err)) {
    std::cout << err << std::endl;
    return 1;
  }
  std::cout << "Binning done" << std::endl;
  outp_data_info(d, d.out_file + "inp2.info");
  write_run_record(d, eng, r.terms);
  return 0;
}

// --batch: every run prepared in turn, their SD terms in one cpc_count_batch
// launch (the fast engine; FP64 counts them one by one), then each finished.
int run_batch(const std::vector<const char *> &inps, cpc_engine eng) {
  std::vector<std::unique_ptr<Run>> runs;
  for (const char *inp : inps) {
    runs.emplace_back(new Run());
    if (run_prepare(*runs.back(), inp, eng, true)) return 1;
  }
  const int n = (int)runs.size();
  std::vector<std::vector<int64_t>> nums(n);
  std::vector<std::vector<double>> sums(n);
  std::vector<cpc_accum> outs(n);
  std::vector<cpc_ctx *> ctxs(n);
  for (int k = 0; k < n; k++) {
    int nh, nb, np;
    cpc_accum_shape(runs[k]->ctx.c, &nh, &nb, &np);
    nums[k].resize((size_t)nh * nb * np);
    sums[k].resize(nums[k].size() * CPC_NF);
    outs[k] = cpc_accum{};
    outs[k].num = nums[k].data();
    outs[k].sums = sums[k].data();
    ctxs[k] = runs[k]->ctx.c;
  }
  const auto t0 = std::chrono::steady_clock::now();
  if (eng == CPC_ENGINE_FAST) {
    const std::vector<cpc_pair_kind> kinds(n, CPC_PAIR_SD);
    const std::vector<int> s1(n, 2), s2(n, 0);
    if (cpc_count_batch(n, ctxs.data(), kinds.data(), s1.data(), s2.data(), outs.data()) !=
        CPC_OK) {
      std::cout << "batched corels2 on the GPU failed: " << cpc_last_error(nullptr)
                << std::endl;
      return 1;
    }
  } else {
    for (int k = 0; k < n; k++)
      if (cpc_count(ctxs[k], CPC_PAIR_SD, 2, 0, eng, 1, 0, &outs[k]) != CPC_OK) {
        std::cout << "corels2 on the GPU failed: " << cpc_last_error(ctxs[k]) << std::endl;
        return 1;
      }
  }
  const double dt = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  for (int k = 0; k < n; k++) {
    Run &r = *runs[k];
    add_count(r.SD, r.d, nums[k].data(), sums[k].data());
    log_term(r.terms, CPC_PAIR_SD, outs[k], dt, false);
    if (run_finish(r, eng)) return 1;
  }
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
  std::vector<const char *> inps;
  const bool batch = !std::strcmp(argv[1], "--batch");
  for (int a = batch ? 2 : 1; a < argc; a++) {
    if (!std::strcmp(argv[a], "--engine") && a + 1 < argc)
      eng = std::strcmp(argv[++a], "fp64") == 0 ? CPC_ENGINE_FP64 : CPC_ENGINE_FAST;
    else if (batch || inps.empty())
      inps.push_back(argv[a]);
  }
  if (inps.empty()) {
    std::cout << "no input file given!!" << std::endl << "Bad initialization!! Bye" << std::endl;
    return 1;
  }
  if (batch) return run_batch(inps, eng);
  Run r;
  if (run_prepare(r, inps[0], eng, false)) return 1;
  return run_finish(r, eng);
}
