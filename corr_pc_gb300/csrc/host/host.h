// host.h -- the host side of the drop-in (C++): the reference's parameter
// file, catalogue readers, estimator finalisation and output writers around
// the GPU pair loop of include/corrpc.h.
//
//   inp.cpp      positional .inp reader/writer          (initialization.cpp:62-352)
//   reader.cpp   read_data text formats + derived fields (read_dat.cpp:18-347)
//   finalize.cpp bin trees, final_calc / int_calc / jk_final, analytic RR
//                                                        (bins_calcs.cpp, PB_calcs.cpp:63-85)
//   outp.cpp     outp_bins / outp_2Dbins / outp_data_info (outp.cpp:45-162)
//   driver.cpp   corr_pc command line: main + do_corr    (main.cpp, do_corr.cpp)
#pragma once
#include <algorithm>
#include <atomic>
#include <cstdint>
#include <exception>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <system_error>
#include <thread>
#include <vector>

#include "../../../include/corrpc.h"

namespace cpch {

// Run task(i) for every i in [0, n) on the host's cores: the calling thread and
// up to 63 workers take indices from a shared counter.  When a worker cannot
// be started the others do its share; the first exception a task throws is
// rethrown here once every thread has stopped.
template <class F>
void run_parallel(int64_t n, F &&task) {
  if (n <= 0) return;
  const int64_t hw = std::max(1u, std::thread::hardware_concurrency());
  const int64_t nt = std::min<int64_t>({hw, n, 64});
  std::atomic<int64_t> next{0};
  std::exception_ptr first;
  std::mutex mu;
  auto work = [&] {
    for (int64_t i; (i = next.fetch_add(1)) < n;) {
      try {
        task(i);
      } catch (...) {
        std::lock_guard<std::mutex> lk(mu);
        if (!first) first = std::current_exception();
      }
    }
  };
  std::vector<std::thread> th;
  th.reserve(nt);
  for (int64_t t = 1; t < nt; t++) {
    try {
      th.emplace_back(work);
    } catch (const std::system_error &) {
      break;
    }
  }
  work();
  for (auto &x : th) x.join();
  if (first) std::rethrow_exception(first);
}

// data_info (data_def.h:46-96): the fields read from the .inp plus the values
// data_ini derives.
struct Info {
  int which_corr = 0, coordinates = 6, estimator = 0, data_sorted = 1, use_comoving = 1;
  int do_jk = 0, sig_crit = 0;
  std::string shape_pos, shape_z, shape_e, shape_wt, shape_jk, shape_patch;
  std::string density_pos, density_z, density_wt, density_jk, density_e;
  std::string srand_pos, srand_z, srand_wt, srand_jk, srand_patch;
  std::string drand_pos, drand_z, drand_wt, drand_jk;
  std::string distance_file, patches_file, out_file;
  int n_threads = 0, n_shape = 0, n_density = 0, n_shape_rand = 0, n_density_rand = 0;
  int rand_subsample = 0, n_jk_regions = 0, n_patch = 0;
  double bin_r_min = 0, bin_r_max = 0;
  int n_bins = 0, lin_bin = 0, n_p_bin = 0;
  double p_min = 0, p_max = 0, z_min = 0, z_max = 0, dz = 0, z_sep_min = 0, z_sep_max = 0;
  int periodic_box = 0;
  double periodic_box_size = 0;
  // derived (data_ini)
  int do_auto_corr = 0, do_cross_corr = 0, do_auto_rebin = 0, RsRd_same = 0, n_jk = 0;
  double include_prob_RR = 1, p_size = 0, r_size = 0;
  // weight totals accumulated by read_data (val = sum w, err = sum w^2)
  double S_wt[2] = {0, 0}, D_wt[2] = {0, 0}, Rs_wt[2] = {0, 0}, Rd_wt[2] = {0, 0};
  double SD_wt[2] = {0, 0}, SRd_wt[2] = {0, 0}, DRs_wt[2] = {0, 0}, RsRd_wt[2] = {0, 0};
  double SS_wt = 0, SRs_wt = 0, RsRs_wt[2] = {0, 0}, DD_wt = 0;
  // distance table (da_Z, initialization.cpp:23-60), read when not periodic
  std::vector<double> H_z, dA_z, dC_z;
};

// 0 ok, nonzero: message in err
int read_inp(const std::string &path, Info &d, std::string &err);
// data_ini's derived settings (initialization.cpp:349-561, periodic box / xyz)
int derive_info(Info &d, std::string &err);
cpc_params to_params(const Info &d);

// One catalogue as read_data leaves it (flattened gal[]).
struct Catalog {
  int64_t n = 0;
  std::vector<double> x, y, z, w, e1, e2, e3, phi, jk_prob, include_prob;
  std::vector<double> dc, da;  // table rows at floor(z/dz) (not periodic)
  std::vector<int32_t> jk;
  bool has_e = false;   // e1, e2 hold e (or kappa in e1, e2 = 0)
  bool has_e3 = false;  // the ED orientation's third component
  cpc_catalog view() const;
};
enum Role { ROLE_S = 0, ROLE_D = 1, ROLE_RS = 2, ROLE_RD = 3 };
// The number files of one run, each parsed once: samples that name the same
// file (S and D from one catalogue, as the notebooks write them) share it.
struct TextCache {
  std::map<std::string, std::shared_ptr<const std::vector<double>>> reals;
  std::map<std::string, std::shared_ptr<const std::vector<int32_t>>> ints;
};
// read one sample like read_data; `draws` is the running index into the glibc
// rand() stream (advanced by the draws this sample consumes).  Files already
// in `cache` are not read again; files read are added to it.
int read_catalog(Info &d, Role role, Catalog &c, int64_t &draws, std::string &err,
                 TextCache *cache = nullptr);

// bin tree of one term (bin_jk: full sample + n_jk jackknife samples)
struct Bins {
  int nb = 0, np = 0, nh = 0;  // r_p bins, Pi bins, 1 + n_jk
  // per (h, i): 1-D bin
  std::vector<double> b_min, b_max;  // edges (float arithmetic, like bin_log/bin_lin)
  std::vector<double> p_min, p_max;  // Pi edges (float arithmetic, P_bin_ini)
  std::vector<int64_t> bnum;         // [h][i]
  std::vector<double> bwt;           // [h][i]
  std::vector<double> bdat;          // [h][i][7][2]  (val, err)
  std::vector<double> bls, bsig;     // [h][i]
  // per (h, i, k): 2-D bin
  std::vector<int64_t> pnum;         // [h][i][k]
  std::vector<double> pwt;           // [h][i][k]
  std::vector<double> pdat;          // [h][i][k][7][2]
  std::vector<double> pls;           // [h][i][k]
  void init(const Info &d, int n_hist);
  double &bd(int h, int i, int j, int e) { return bdat[(((size_t)h * nb + i) * 7 + j) * 2 + e]; }
  double &pd(int h, int i, int k, int j, int e) {
    return pdat[((((size_t)h * nb + i) * np + k) * 7 + j) * 2 + e];
  }
  size_t bi(int h, int i) const { return (size_t)h * nb + i; }
  size_t pi(int h, int i, int k) const { return ((size_t)h * nb + i) * np + k; }
};

// corels2's end: add the GPU histogram block (raw region sums) into the tree
// and apply final_jk_bins (jk.cpp:74-81).
void add_count(Bins &b, const Info &d, const int64_t *num, const double *sums);
// do_corr's finalisation and output files (do_corr.cpp:203-433): both parts,
// the cross part, the auto part; and add_bins (b += a, every sample)
int do_bining(Info &d, Bins &SS, Bins &SRs, Bins &RsRs, Bins &SD, Bins &SRd, Bins &DRs,
              Bins &RsRd, std::string &err);
int do_bining_cross(Info &d, Bins &SD, Bins &SRd, Bins &DRs, Bins &RsRd, std::string &err);
int do_bining_auto(Info &d, Bins &SS, Bins &SRs, Bins &RsRs, std::string &err);
void add_bins(Bins &b, const Bins &a);
int outp_data_info(const Info &d, const std::string &path);

}  // namespace cpch
