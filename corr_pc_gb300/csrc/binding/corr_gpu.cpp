// corr_gpu.cpp -- corels2 on the GPU through libcorrpc_gb300
#include <cmath>
#include <iostream>
#include <vector>
#include "corrpc.h"
#include "data_def.h"
#include "jk.h"

namespace {

cpc_ctx *ctx = nullptr;            // do_corr calls corels2 from one host thread
const gal *slot_src[8] = {};       // which gal[] each device slot holds
long slot_n[8] = {};

cpc_params to_params(const data_info &d) {
  cpc_params p = {};
  p.which_corr = d.which_corr;   p.coordinates = d.coordinates;
  p.estimator = d.estimator;     p.periodic_box = d.periodic_box;
  p.data_sorted = d.data_sorted; p.do_jk = d.do_jk;  p.n_jk = d.n_jk;
  p.sig_crit = d.sig_crit;       p.rand_subsample = d.rand_subsample;
  p.n_bins = d.n_bins;           p.lin_bin = d.lin_bin;  p.n_p_bin = d.n_p_bin;
  p.bin_r_min = d.bin_r_min;     p.bin_r_max = d.bin_r_max;
  p.p_min = d.p_min;             p.p_max = d.p_max;
  p.periodic_box_size = d.periodic_box_size;
  // sky runs (coordinates 0): the distance table da_Z read and the derived
  // z_sep_max (initialization.cpp:23-60, 271-276)
  p.z_max = d.z_max; p.dz = d.dz; p.z_sep_max = d.z_sep_max;
  if (!d.periodic_box) {
    p.H_z = d.H_z; p.dA_z = d.dA_z;
    p.n_table = (int64_t)std::ceil((d.z_max + 1) / d.dz) + 1;  // rows da_Z read
  }
  return p;
}

// How many e[] entries read_data filled for a sample (read_dat.cpp:27-150):
// 2 (e1, e2), 1 (kappa, which_corr 3 and the density sample of 4), 3 (the ED
// orientation, which_corr 5) or 0 -- gal::e is left unset otherwise.
int e_count(const data_info &d, bool shape_sample, bool density_sample) {
  if (shape_sample) return d.which_corr == 3 ? 1 : d.which_corr == 5 ? 3 : d.which_corr ? 2 : 0;
  if (density_sample) return d.which_corr == 2 ? 2 : d.which_corr == 4 ? 1 : 0;
  return 0;
}

// Flatten one gal[] (data_def.h:23-44) and upload it into a slot (once per array).
int slot_for(const gal *g, long n, const data_info &d, int ne) {
  for (int s = 0; s < 8; s++)
    if (slot_src[s] == g && slot_n[s] == n) return s;
  int s = 0;
  while (s < 8 && slot_src[s]) s++;
  std::vector<double> x(n), y(n), z(n), w(n), e1(n), e2(n), e3(n), phi(n), prob(n), dc(n), da(n);
  std::vector<int32_t> jk(n);
  for (long i = 0; i < n; i++) {
    x[i] = g[i].ra.val_deg; y[i] = g[i].dec.val_deg; z[i] = g[i].redshift;
    w[i] = g[i].wt; phi[i] = g[i].phi; jk[i] = g[i].jk; prob[i] = g[i].jk_prob;
    e1[i] = ne > 0 ? g[i].e[0] : 0.0;
    e2[i] = ne > 1 ? g[i].e[1] : 0.0;
    e3[i] = ne > 2 ? g[i].e[2] : 0.0;
    dc[i] = g[i].DC; da[i] = g[i].DA;  // read_data's table lookups (sky runs)
  }
  cpc_catalog c = {n, x.data(), y.data(), z.data(), w.data(), e1.data(), e2.data(),
                   phi.data(), d.do_jk ? jk.data() : nullptr, prob.data(),
                   d.periodic_box ? nullptr : dc.data(), d.periodic_box ? nullptr : da.data(),
                   e3.data()};
  if (cpc_upload(ctx, s, &c) != CPC_OK) return -1;
  slot_src[s] = g; slot_n[s] = n;
  return s;
}

// Create the context on first use (do_corr calls the pair loop from one thread).
bool ensure_ctx(const data_info &d) {
  if (ctx) return true;
  cpc_params p = to_params(d);
  if (cpc_create(&ctx, &p) == CPC_OK) return true;
  std::cout << cpc_last_error(nullptr) << std::endl;
  return false;
}

// Add a RAW histogram block into bjk, then corels's delete-one step
// (corr.cpp:445-448 for corels2, :207-210 for corels1).
void add_block(bin_jk &bjk, data_info &d, int nh, int nb, int np,
               const std::vector<int64_t> &num, const std::vector<double> &sums) {
  for (int h = 0; h < nh; h++) {
    bin *b = h == 0 ? bjk.b : bjk.jk[h - 1].b;
    for (int i = 0; i < nb; i++)
      for (int k = 0; k < np; k++) {
        const size_t c = ((size_t)h * nb + i) * np + k;
        const double *s = &sums[c * CPC_NF];
        b[i].num += num[c];
        b[i].p_bin[k].num += num[c];
        b[i].p_bin[k].wt_num += s[0];
        for (int j = 1; j <= 6; j++) {
          b[i].p_bin[k].data[j].val += s[1 + 2 * (j - 1)];
          b[i].p_bin[k].data[j].err += s[2 + 2 * (j - 1)];
        }
      }
  }
  if (d.do_jk == 1) final_jk_bins(bjk, d);
}

}  // namespace

long corels2(gal g1[], gal g2[], bin_jk &bjk, data_info &data_inf) {
  if (!ensure_ctx(data_inf)) return 0;
  cpc_pair_kind kind = data_inf.do_SD ? CPC_PAIR_SD : data_inf.do_SRd ? CPC_PAIR_SRD
                     : data_inf.do_DRs ? CPC_PAIR_DRS : data_inf.do_RsRd ? CPC_PAIR_RSRD
                     : data_inf.do_RsRs ? CPC_PAIR_RSRS : CPC_PAIR_SRS;
  // the array lengths corels2 itself derives from the do_* flags (corr.cpp:226-271)
  long n1 = data_inf.do_SD ? data_inf.n_density : data_inf.do_SRd ? data_inf.n_density_rand
          : data_inf.do_RsRd ? data_inf.n_density_rand : data_inf.n_shape_rand;
  long n2 = data_inf.do_DRs ? data_inf.n_density
          : (data_inf.do_SD || data_inf.do_SRd || data_inf.do_SRs) ? data_inf.n_shape
          : data_inf.n_shape_rand;
  // g1 is the density sample for SD, g2 the shape sample for SD, SRd and SRs
  int s1 = slot_for(g1, n1, data_inf, e_count(data_inf, false, data_inf.do_SD));
  int s2 = slot_for(g2, n2, data_inf,
                    e_count(data_inf, data_inf.do_SD || data_inf.do_SRd || data_inf.do_SRs,
                            data_inf.do_DRs));
  int nh, nb, np;
  cpc_accum_shape(ctx, &nh, &nb, &np);
  std::vector<int64_t> num((size_t)nh * nb * np);
  std::vector<double> sums(num.size() * CPC_NF);
  cpc_accum acc = {num.data(), sums.data()};
  if (s1 < 0 || s2 < 0 ||
      cpc_count(ctx, kind, s1, s2, CPC_ENGINE_FAST, 1, 0, &acc) != CPC_OK) {
    std::cout << "corels2 (GPU): " << cpc_last_error(ctx) << std::endl;
    return 0;
  }
  // data_inf.g_with_shape: the library applied corels2's rule internally; set it the
  // same way if later code reads it (corr.cpp:226-296).
  add_block(bjk, data_inf, nh, nb, np, num, sums);
  std::cout << "corel2 ends:: total pair= " << acc.n_window << "\tpairs in=" << acc.n_binned
            << std::endl;
  return acc.n_binned;
}

// corels1 (corr.cpp:103-216): the auto pairs of one catalogue, SS or RsRs
// (do_corr.cpp:63, 76).
long corels1(gal g1[], bin_jk &bjk, data_info &data_inf) {
  if (!ensure_ctx(data_inf)) return 0;
  const bool ss = data_inf.do_SS;
  long n = ss ? data_inf.n_shape : data_inf.n_shape_rand;
  int s = slot_for(g1, n, data_inf, e_count(data_inf, ss, false));
  int nh, nb, np;
  cpc_accum_shape(ctx, &nh, &nb, &np);
  std::vector<int64_t> num((size_t)nh * nb * np);
  std::vector<double> sums(num.size() * CPC_NF);
  cpc_accum acc = {num.data(), sums.data()};
  if (s < 0 || cpc_count_auto(ctx, ss ? CPC_PAIR_SS : CPC_PAIR_RSRS, s, CPC_ENGINE_FAST, 1, 0,
                              &acc) != CPC_OK) {
    std::cout << "corels1 (GPU): " << cpc_last_error(ctx) << std::endl;
    return 0;
  }
  add_block(bjk, data_inf, nh, nb, np, num, sums);
  std::cout << "corel1 ends:: total pair= " << acc.n_window << "\tpairs in=" << acc.n_binned
            << std::endl;
  return acc.n_binned;
}
