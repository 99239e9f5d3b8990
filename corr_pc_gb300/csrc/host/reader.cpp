// reader.cpp -- the reference's catalogue input format (read_dat.cpp:18-347):
// <prefix>_pos.dat (two columns), _z.dat, _e.dat (e1 e2; one column of kappa
// or phi, or three of the ED orientation, depending on which_corr and the file
// name), _wt.dat, _jk.dat (integer labels), "0" meaning "absent".  Per galaxy it derives what the pair
// loop reads: jk_prob (glibc rand()/(RAND_MAX+1.) in a periodic box, one draw
// per galaxy in read order after srand(124693517); 1 otherwise, 0 without
// jackknife), phi (elip_angle, or -10 without shapes), include_prob (a second
// draw for random catalogues), the table distances D_C and D_A of a non-periodic
// run, and the weight totals.  Numbers are parsed with
// std::from_chars, which rounds exactly as the reference's istream >> double,
// in chunks on the host's cores.
#include <charconv>
#include <cmath>
#include <cstdio>

#include "../host_helpers.h"
#include "host.h"

namespace cpch {

namespace {

inline bool is_ws(char c) { return c == ' ' || c == '\t' || c == '\n' || c == '\r'; }

// The whole file in one buffer; false if it cannot be opened.
bool slurp(const std::string &path, std::string &buf) {
  FILE *f = std::fopen(path.c_str(), "rb");
  if (!f) return false;
  buf.clear();
  if (std::fseek(f, 0, SEEK_END) == 0) {
    const long sz = std::ftell(f);
    if (sz > 0) buf.reserve((size_t)sz);
    std::rewind(f);
  }
  char tmp[1 << 16];
  size_t k;
  while ((k = std::fread(tmp, 1, sizeof tmp, f)) > 0) buf.append(tmp, k);
  std::fclose(f);
  return true;
}

// Numbers of [b, e) in order, as istream >> reads them one after another:
// whitespace skipped, one leading '+' allowed, each number the longest prefix
// from_chars accepts.  Returns true when it stopped at something that is not a
// number (the numbers after it are never read).
template <class T>
bool parse_span(const char *b, const char *e, std::vector<T> &out) {
  const char *p = b;
  for (;;) {
    while (p < e && is_ws(*p)) p++;
    if (p >= e) return false;
    const char *q = *p == '+' ? p + 1 : p;
    // istream >> double reads no "inf" or "nan" (from_chars would): a letter
    // where the digits start ends the numbers
    const char *d = (q < e && *q == '-') ? q + 1 : q;
    if (d < e && ((*d >= 'a' && *d <= 'z') || (*d >= 'A' && *d <= 'Z'))) return true;
    T v;
    const auto r = std::from_chars(q, e, v);
    if (r.ec != std::errc()) return true;
    out.push_back(v);
    p = r.ptr;
  }
}

// parse_span over a whole file, in chunks of >= 1 MiB on the host's cores.
// Chunks start at whitespace, where the sequential reader always starts a new
// number (no number contains whitespace), so the numbers are the same; the
// list ends at the first chunk that stopped early.
template <class T>
std::vector<T> parse_numbers(const std::string &buf) {
  const size_t n = buf.size();
  const char *b = buf.data();
  const int64_t parts = (int64_t)std::min<size_t>(256, std::max<size_t>(1, n >> 20));
  std::vector<T> out;
  if (parts == 1) {
    parse_span(b, b + n, out);
    return out;
  }
  std::vector<size_t> cut(parts + 1);
  cut[0] = 0;
  cut[parts] = n;
  for (int64_t t = 1; t < parts; t++) {
    size_t c = std::max(cut[t - 1], n * (size_t)t / (size_t)parts);
    while (c < n && !is_ws(b[c])) c++;
    cut[t] = c;
  }
  std::vector<std::vector<T>> piece(parts);
  std::vector<char> stopped(parts, 0);
  run_parallel(parts, [&](int64_t t) {
    piece[t].reserve((cut[t + 1] - cut[t]) / 8);
    stopped[t] = parse_span(b + cut[t], b + cut[t + 1], piece[t]);
  });
  size_t total = 0;
  int64_t last = parts - 1;
  for (int64_t t = 0; t < parts; t++) {
    total += piece[t].size();
    if (stopped[t]) { last = t; break; }
  }
  out.resize(total);
  size_t at = 0;
  for (int64_t t = 0; t <= last; t++) {
    std::copy(piece[t].begin(), piece[t].end(), out.begin() + at);
    at += piece[t].size();
    std::vector<T>().swap(piece[t]);
  }
  return out;
}

// One number file of a sample, read in order by get().
struct TextCols {
  std::shared_ptr<const std::vector<double>> reals;
  std::shared_ptr<const std::vector<int32_t>> ints;
  size_t pos = 0;
  template <class T, class M>
  static bool load(const std::string &path, TextCache *cache, M &map,
                   std::shared_ptr<const std::vector<T>> &dst) {
    if (cache) {
      auto it = map.find(path);
      if (it != map.end()) {
        dst = it->second;
        return true;
      }
    }
    std::string buf;
    if (!slurp(path, buf)) return false;
    dst = std::make_shared<const std::vector<T>>(parse_numbers<T>(buf));
    if (cache) map[path] = dst;
    return true;
  }
  bool open(const std::string &path, TextCache *cache) {
    TextCache local;
    return load(path, cache, cache ? cache->reals : local.reals, reals);
  }
  bool open_ints(const std::string &path, TextCache *cache) {
    TextCache local;
    return load(path, cache, cache ? cache->ints : local.ints, ints);
  }
  bool get(double &v) {
    if (!reals || pos >= reals->size()) return false;
    v = (*reals)[pos++];
    return true;
  }
  bool get(int32_t &v) {
    if (!ints || pos >= ints->size()) return false;
    v = (*ints)[pos++];
    return true;
  }
};

// What a sample reads from its e file (read_dat.cpp:27-205): the which_corr
// switch (case 5 falls through into case 8), the per-sample overrides, then
// the file-name rule ("phi" or "kappa" in the name selects a one-column read).
struct EFlags {
  bool e = false, kappa = false, phi = false, e3 = false;
  std::string file;
  bool any() const { return e || kappa || phi || e3; }
};

EFlags e_flags(const Info &d, Role role) {
  EFlags f;
  f.e = true;
  bool css = false;  // cross_shape_shape: the density sample reads density_e
  switch (d.which_corr) {
    case 0: f.e = false; break;
    case 3: css = false; f.e = false; f.kappa = true; break;
    case 4:
      f.e = role == ROLE_S;
      f.kappa = role != ROLE_S;
      css = true;
      break;
    case 5:
      f.e = false;
      if (role == ROLE_S) f.e3 = true;
      f.kappa = false;  // falls through into case 8
      css = true;
      break;
    case 2: css = true; break;
    default: css = false; break;
  }
  if (role == ROLE_S) {
    f.file = d.shape_e;
    if (d.which_corr == 4) { f.e = true; f.kappa = false; }
  } else if (role == ROLE_D) {
    if (css) f.file = d.density_e;
    else f.e = f.kappa = f.phi = f.e3 = false;
  } else {
    f.e = f.kappa = f.phi = false;
    if (role == ROLE_RS || role == ROLE_RD) f.e3 = false;
  }
  if (f.any()) {
    if (f.file.find("phi") != std::string::npos || f.phi) { f.phi = true; f.e = false; f.kappa = false; }
    if (f.file.find("kappa") != std::string::npos || f.kappa) { f.kappa = true; f.e = false; f.phi = false; }
  }
  return f;
}

}  // namespace

cpc_catalog Catalog::view() const {
  cpc_catalog c{};
  c.n = n;
  c.x = x.data();
  c.y = y.data();
  c.z = z.data();
  c.w = w.data();
  c.e1 = has_e ? e1.data() : nullptr;
  c.e2 = has_e ? e2.data() : nullptr;
  c.e3 = has_e3 ? e3.data() : nullptr;
  c.phi = phi.data();
  c.jk = jk.empty() ? nullptr : jk.data();
  c.jk_prob = jk_prob.data();
  c.dc = dc.empty() ? nullptr : dc.data();
  c.da = da.empty() ? nullptr : da.data();
  return c;
}

int read_catalog(Info &d, Role role, Catalog &c, int64_t &draws, std::string &err,
                 TextCache *cache) {
  const EFlags ef = e_flags(d, role);
  std::string p_f, z_f, w_f, jk_f;
  const std::string &e_f = ef.file;
  double *wt = nullptr;
  int n_gal = 0;
  if (role == ROLE_S) {
    p_f = d.shape_pos; z_f = d.shape_z; w_f = d.shape_wt; jk_f = d.shape_jk;
    n_gal = d.n_shape; wt = d.S_wt;
  } else if (role == ROLE_D) {
    p_f = d.density_pos; z_f = d.density_z; w_f = d.density_wt; jk_f = d.density_jk;
    n_gal = d.n_density; wt = d.D_wt;
  } else if (role == ROLE_RS) {
    p_f = d.srand_pos; z_f = d.srand_z; w_f = d.srand_wt; jk_f = d.srand_jk;
    n_gal = d.n_shape_rand; wt = d.Rs_wt;
  } else {
    p_f = d.drand_pos; z_f = d.drand_z; w_f = d.drand_wt; jk_f = d.drand_jk;
    n_gal = d.n_density_rand; wt = d.Rd_wt;
  }
  c = Catalog();
  if (n_gal == 0) return 0;  // read_dat.cpp:152-156: nothing read, no draws
  const bool randoms = role == ROLE_RS || role == ROLE_RD;
  const bool read_jk = jk_f != "0" && d.do_jk;
  TextCols fp, fz, fe, fw, fj;
  if (!fp.open(p_f, cache)) { err = "pos file not open: " + p_f; return 1; }
  if (!fz.open(z_f, cache)) { err = "z file not open: " + z_f; return 1; }
  if (w_f != "0" && !fw.open(w_f, cache)) { err = "wt file not open: " + w_f; return 1; }
  if (read_jk && !fj.open_ints(jk_f, cache)) { err = "jk file not open: " + jk_f; return 1; }
  if (ef.any() && !fe.open(e_f, cache)) { err = "e file not open: " + e_f; return 1; }
  const uint32_t seed = d.periodic_box ? 124693517u : 1u;  // srand only in a box
  cpc::GlibcRand rng(seed);
  for (int64_t s = 0; s < draws; s++) rng.next();
  c.n = n_gal;
  c.x.resize(n_gal); c.y.resize(n_gal); c.z.resize(n_gal); c.w.assign(n_gal, 1.0);
  c.phi.assign(n_gal, -10.0); c.jk_prob.assign(n_gal, 1.0); c.include_prob.assign(n_gal, 0.0);
  if (read_jk) c.jk.assign(n_gal, -1);
  const bool two = ef.e && !ef.kappa && !ef.phi;     // e1 e2, then elip_angle
  const bool one_phi = !ef.e && ef.phi && !ef.kappa;  // phi
  const bool one_kappa = ef.kappa && !ef.e && !ef.phi;  // kappa into e[0]
  c.has_e = two || ef.e3 || one_kappa;
  c.has_e3 = ef.e3;
  if (!d.periodic_box) { c.dc.resize(n_gal); c.da.resize(n_gal); }
  if (c.has_e) { c.e1.assign(n_gal, 0.0); c.e2.assign(n_gal, 0.0); }
  if (c.has_e3) c.e3.assign(n_gal, 0.0);
  for (int i = 0; i < n_gal; i++) {
    if (!fp.get(c.x[i]) || !fp.get(c.y[i]) || !fz.get(c.z[i])) {
      err = "gal data reading ended unexpectedly at row " + std::to_string(i) + " of " + p_f;
      return 1;
    }
    if (c.z[i] < 0) c.z[i] = 0;
    if (c.z[i] > d.z_max) {
      err = "wrong z at row " + std::to_string(i) + " (above z_max)";
      return 1;
    }
    if (d.periodic_box) {
      c.jk_prob[i] = rng.next() / (2147483647 + 1.);
      draws++;
    } else {  // read_dat.cpp:247-251: table rows, no interpolation
      const int64_t it = (int64_t)std::floor(c.z[i] / d.dz);
      if (it < 0 || it >= (int64_t)d.dC_z.size()) {
        err = "redshift beyond the distances table at row " + std::to_string(i);
        return 1;
      }
      c.dc[i] = d.dC_z[it];
      c.da[i] = d.dA_z[it];
    }
    if (d.do_jk == 0 || d.n_jk == 0) c.jk_prob[i] = 0;
    if (w_f != "0" && !fw.get(c.w[i])) { err = "wt file ended early"; return 1; }
    if (read_jk && !fj.get(c.jk[i])) { err = "jk file ended early"; return 1; }
    if (two) {
      if (!fe.get(c.e1[i]) || !fe.get(c.e2[i])) { err = "e file ended early"; return 1; }
    }
    if (ef.e3) {  // read_dat.cpp:282-293: normalised to unit length when non-zero
      if (!fe.get(c.e1[i]) || !fe.get(c.e2[i]) || !fe.get(c.e3[i])) {
        err = "e file ended early";
        return 1;
      }
      const double en = std::sqrt(c.e1[i] * c.e1[i] + c.e2[i] * c.e2[i] + c.e3[i] * c.e3[i]);
      if (en > 0) {
        c.e1[i] /= en;
        c.e2[i] /= en;
        c.e3[i] /= en;
      }
    }
    if (one_phi && !fe.get(c.phi[i])) { err = "phi file ended early"; return 1; }
    if (one_kappa && !fe.get(c.e1[i])) { err = "kappa file ended early"; return 1; }
    if (randoms) {
      c.include_prob[i] = rng.next() / (2147483647 + 1.);
      draws++;
    }
    wt[0] += c.w[i];
    wt[1] += c.w[i] * c.w[i];
  }
  if (two)  // phi = elip_angle(e1, e2) per galaxy (read_dat.cpp:279), in blocks on the host's cores
    run_parallel((n_gal + 65535) / 65536, [&](int64_t b) {
      const int64_t lo = b * 65536, hi = std::min<int64_t>(n_gal, lo + 65536);
      for (int64_t i = lo; i < hi; i++) c.phi[i] = cpc::elip_angle(c.e1[i], c.e2[i]);
    });
  if (!read_jk && d.do_jk) c.jk.assign(n_gal, -1);
  return 0;
}

}  // namespace cpch
