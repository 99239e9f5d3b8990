// host_asan_driver.cpp -- the host side of the corr_pc_gb300 command line for a
// periodic-box cross run, with the SD term's RAW histogram block read from files
// instead of counted on a GPU: the positional .inp, every catalogue in do_corr's
// order (the glibc rand() draws included), the block added into the bin tree with
// the delete-one step, the finalisation and the output files.  tests/test_host.py
// builds it with AddressSanitizer and UndefinedBehaviorSanitizer (no GPU needed).
//
//   host_asan_driver <run.inp> <num.bin (int64)> <sums.bin (float64)>
//   host_asan_driver --dump <run.inp> <out.bin>
//
// The second form reads S and D only and writes, per sample, n (int64), then x,
// y, z, w, phi, jk_prob, e1, e2 (float64) and the labels (int32).
#include <cstdio>
#include <iostream>
#include <string>
#include <vector>

#include "host/host.h"

using namespace cpch;

template <class T>
static bool read_all(const char *path, std::vector<T> &v) {
  FILE *f = std::fopen(path, "rb");
  if (!f) return false;
  T x;
  while (std::fread(&x, sizeof x, 1, f) == 1) v.push_back(x);
  std::fclose(f);
  return true;
}

static int dump(const char *inp, const char *out_path) {
  Info d;
  std::string err;
  if (read_inp(inp, d, err) || derive_info(d, err)) {
    std::cout << err << std::endl;
    return 1;
  }
  int64_t draws = 0;
  TextCache files;
  Catalog S, D;
  if (read_catalog(d, ROLE_S, S, draws, err, &files) ||
      read_catalog(d, ROLE_D, D, draws, err, &files)) {
    std::cout << err << std::endl;
    return 1;
  }
  FILE *f = std::fopen(out_path, "wb");
  if (!f) return 1;
  for (const Catalog *c : {&S, &D}) {
    std::fwrite(&c->n, sizeof c->n, 1, f);
    const std::vector<double> zero(c->n, 0.0);
    for (const std::vector<double> *v : {&c->x, &c->y, &c->z, &c->w, &c->phi, &c->jk_prob,
                                         c->has_e ? &c->e1 : &zero, c->has_e ? &c->e2 : &zero})
      std::fwrite(v->data(), sizeof(double), c->n, f);
    std::vector<int32_t> jk(c->jk);
    jk.resize(c->n, -1);
    std::fwrite(jk.data(), sizeof(int32_t), c->n, f);
  }
  std::fclose(f);
  return 0;
}

int main(int argc, char **argv) {
  if (argc == 4 && std::string(argv[1]) == "--dump") return dump(argv[2], argv[3]);
  if (argc < 4) {
    std::cout << "usage: host_asan_driver run.inp num.bin sums.bin" << std::endl;
    return 2;
  }
  Info d;
  std::string err;
  if (read_inp(argv[1], d, err) || derive_info(d, err)) {
    std::cout << err << std::endl;
    return 1;
  }
  outp_data_info(d, d.out_file + "inp.info");
  const bool box = d.periodic_box != 0;
  if (!box || !d.do_cross_corr || d.do_auto_corr) {
    std::cout << "a periodic-box cross run is expected" << std::endl;
    return 1;
  }
  const int nh = 1 + (d.do_jk ? d.n_jk : 0);
  Bins SS, SRs, RsRs, SD, SRd, DRs, RsRd;
  for (Bins *b : {&SS, &SRs, &RsRs, &SD, &SRd, &DRs, &RsRd}) b->init(d, nh);
  int64_t draws = 0;
  TextCache files;  // S and D naming the same files parse them once
  Catalog S, Rs, D, Rd;
  // do_corr.cpp:40-52 and 83-133: S, the shape randoms, D, the density randoms
  if (read_catalog(d, ROLE_S, S, draws, err, &files)) { std::cout << err << std::endl; return 1; }
  if (d.n_jk > 0 && read_catalog(d, ROLE_RS, Rs, draws, err, &files)) {
    std::cout << err << std::endl;
    return 1;
  }
  if (read_catalog(d, ROLE_D, D, draws, err, &files)) { std::cout << err << std::endl; return 1; }
  if (!d.RsRd_same && read_catalog(d, ROLE_RD, Rd, draws, err, &files)) {
    std::cout << err << std::endl;
    return 1;
  }
  std::vector<int64_t> num;
  std::vector<double> sums;
  if (!read_all(argv[2], num) || !read_all(argv[3], sums) ||
      num.size() != (size_t)nh * SD.nb * SD.np || sums.size() != num.size() * CPC_NF) {
    std::cout << "histogram block files do not match the .inp's bins" << std::endl;
    return 1;
  }
  add_count(SD, d, num.data(), sums.data());
  if (do_bining(d, SS, SRs, RsRs, SD, SRd, DRs, RsRd, err)) {
    std::cout << err << std::endl;
    return 1;
  }
  outp_data_info(d, d.out_file + "inp2.info");
  std::cout << "host pipeline done: " << S.n << " shape and " << D.n << " density galaxies"
            << std::endl;
  return 0;
}
