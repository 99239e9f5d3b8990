// capi.cu -- the C ABI (include/corrpc.h): contexts, catalogue upload with the
// on-device cell list, per-job set-up (the reference's corels2 rules, exact
// thresholds and FP32 guard bands), work-unit construction and launches.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <cstdlib>
#include <exception>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <system_error>
#include <thread>
#include <tuple>
#include <vector>

#include "../../include/corrpc.h"
#include "cpc_device.cuh"
#include "host_helpers.h"
#include "param_check.h"
#include "kernels.h"

using namespace cpc;

// initial capacity of the FP64 edge queue (entries); it grows when a count
// needs more
#ifndef CPC_EDGE_QUEUE_INIT
#define CPC_EDGE_QUEUE_INIT (1ull << 24)
#endif

namespace {

// message of the calling thread's last failing call (entry points without a context)
thread_local std::string g_err;

template <class T>
struct DevBuf {
  T *p = nullptr;
  size_t n = 0;
  DevBuf() = default;
  DevBuf(const DevBuf &) = delete;
  DevBuf &operator=(const DevBuf &) = delete;
  ~DevBuf() { reset(); }
  void reset() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  cudaError_t alloc(size_t count) {
    if (count <= n && p) return cudaSuccess;
    reset();
    if (count == 0) count = 1;
    cudaError_t e = cudaMalloc(&p, sizeof(T) * count);
    if (e != cudaSuccess) {
      p = nullptr;
      return e;
    }
    n = count;
    return cudaSuccess;
  }
};

struct Slot {
  bool valid = false;
  int64_t n = 0;
  bool has_e = false, exact_f32 = true;
  double wmax = 1.0, wmin = 1.0, emax = 0.0, cmax = 0.0, phimax = 0.0;
  uint64_t version = 0;
  // grid this cell list was built with
  int ncx = 0, ncy = 0, n_reg = 1, kcells = 0;
  double cw_x = 0, cw_y = 0;
  // device, cell order
  DevBuf<float4> pos, shp, ewt, aux;
  DevBuf<float> zlo, zf;
  DevBuf<double> x, y, z, w, e1, e2, phi, e3;
  DevBuf<int32_t> jk;
  DevBuf<uint8_t> keep;
  DevBuf<int64_t> orig;
  DevBuf<uint8_t> aflag;  // corels1 scan-start flags of each row (cell order)
  DevBuf<int> bk_start, bk_end, bk_region, col_begin, col_end;
  DevBuf<float> bk_zmin, bk_zmax;
  // host copies used to build work units
  std::vector<float4> h_pos;
  std::vector<int> h_bk_start, h_bk_end, h_bk_region;
  // z-ordered FP64 copy for the plain kernel (built on first use)
  bool zbuilt = false;
  DevBuf<double> zx, zy, zz, zw, ze1, ze2, zphi, ze3;
  DevBuf<int32_t> zjk;
  DevBuf<uint8_t> zkeep, zaflag;
  DevBuf<int64_t> zorig;
  // sky (coordinates 0): x, y, z, w, e1, e2, phi, jk, keep, orig above hold the
  // redshift-ordered catalogue; these the sky-only per-galaxy quantities
  bool sky = false;
  DevBuf<double> dc, da, sd, cd, rar, decr, win;
  DevBuf<float4> sky_su, sky_sl, sky_sw, sky_sx, sky_ss, sky_sh;  // float views (SkyFast)
  DevBuf<float2> sky_sp;
  double dcmax = 0;  // largest |D_C| (error bound of the float Pi)
  // host copies in the same order for the host edge tier
  std::vector<double> hs_ra, hs_dec, hs_dc, hs_da, hs_w, hs_e1, hs_e2, hs_phi;
  std::vector<int32_t> hs_jk;
  std::vector<uint8_t> hs_keep;
  std::vector<int64_t> hs_orig;  // input row of each redshift-ordered row (row samples)
  // the sky kernel's outer-row order: redshift-ordered positions grouped by
  // redshift slab (16 of equal size) and jackknife region, redshift order within
  std::vector<int> hs_rorder;
};

// device buffers of one job of a sky launch: its histogram block, fixed-point
// sums, counters, host-tier queue and row sample
struct SkyJobBufs {
  DevBuf<unsigned long long> num, fix, counters, hq_n;
  DevBuf<double> sums;
  DevBuf<int2> hq;
  DevBuf<int> rows;
};

struct UnitCache {
  uint64_t v1 = 0, v2 = 0;
  int s1 = -1, s2 = -1, wpi = 0, tile = 0, twin = 0;
  std::vector<UnitDesc> units;  // job field filled at launch
};

}  // namespace

namespace {
struct JobPlan;  // one planned count (below)
}  // namespace

struct cpc_ctx {
  cpc_params p{};
  std::vector<double> H, dA;
  std::string err;
  Slot slots[kMaxSlots];
  uint64_t version_ctr = 0;
  double ps = 0, rsize = 0;
  double thr_rp[kMaxRp + 1];
  double thr_pi[kMaxPi + 1];
  int tune_k = 0, tune_wpi = 0, tune_tile = 0;
  int device = 0, sm_count = 152;
  cudaStream_t st = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr, e2 = nullptr;
  cudaEvent_t e_in = nullptr, e_done = nullptr;  // cpc_count_async ordering
  // scratch
  DevBuf<JobDev> d_jobs;
  DevBuf<UnitDesc> d_units;
  DevBuf<unsigned int> d_unit_ctr;
  DevBuf<QEntry> d_queue;
  DevBuf<unsigned long long> d_qcount;
  unsigned long long qcap = 0;
  double q_per_unit = 0;  // most pairs any count queued per work unit (queue sizing)
  size_t last_units = 0;  // work units of the last fast launch
  DevBuf<unsigned long long> d_num;
  DevBuf<double> d_sums;
  DevBuf<unsigned long long> d_counters;
  // sky launches: one buffer set per job of the launch, the chunk table
  std::vector<std::unique_ptr<SkyJobBufs>> sky_bufs;
  DevBuf<long long> d_chunk0;
  DevBuf<unsigned long long> d_chunk_ctr;
  // sort scratch
  DevBuf<uint64_t> d_keys, d_ktmp;
  DevBuf<uint32_t> d_vals, d_vtmp, d_hist, d_bucket;
  DevBuf<unsigned long long> d_census;
  // upload scratch: a catalogue in input order, its checks and statistics
  DevBuf<double> u_x, u_y, u_z, u_w, u_e1, u_e2, u_phi, u_prob, u_e3;
  DevBuf<int32_t> u_jk;
  DevBuf<uint8_t> u_keep, u_flag;
  DevBuf<int64_t> u_orig;
  DevBuf<UploadStats> d_ustats;
  UploadStats h_ustats{};
  // sky: fixed-point sums of the fast kernel, host edge queue
  DevBuf<unsigned long long> d_fix;
  DevBuf<int2> d_hq;
  DevBuf<unsigned long long> d_hq_n;
  std::vector<UnitCache> unit_cache;
  // a count enqueued by cpc_count_async, collected by cpc_count_finish
  int pending = 0;  // 0 none, 1 fast engine, 2 FP64 engine
  std::vector<JobPlan> pending_jobs;
  int64_t launches = 0;  // kernels launched by this context (all entry points)
  // work-unit shard of the fast box engine (cpc_set_shard)
  int shard = 0, n_shards = 1;
  // whether two box slots hold the same galaxies in the same order (twin jobs),
  // for the slot pair and versions last compared; CPC_TWIN=0 turns twin jobs off
  int twin_s1 = -1, twin_s2 = -1;
  uint64_t twin_v1 = 0, twin_v2 = 0;
  bool twin_same = false;
  int twin_on = 1;
  int last_twin = 0;  // the last fast count ran a twin job
  DevBuf<unsigned> d_differ;
  // register bound of the fast sky kernel: 2 or 3 blocks of 256 threads per SM
  // (CPC_SKY_BLOCKS_PER_SM in the environment; the autotuner of a sky context
  // would set it)
  int sky_blocks_per_sm = 2;
  // CUDA graph of the fast engine's device work (zeroing, pair kernels,
  // recheck), replayed while every value baked into it stays the same
  int graph_on = 1;
  cudaGraphExec_t gexec = nullptr;
  std::vector<uint64_t> gkey;
  int64_t graph_captures = 0, graph_replays = 0;
};

namespace {

// Record msg as the context's (and the library's) last error and return s.  A
// message that cannot be stored (out of host memory) leaves the old one.
cpc_status fail(cpc_ctx *c, cpc_status s, const std::string &msg) noexcept {
  try {
    if (c) c->err = msg;
    g_err = msg;
  } catch (...) {
  }
  return s;
}

// The status of a C++ exception that reached an entry point (called from its
// catch block): no exception crosses the C ABI.  A stream capture left open
// by the interrupted call is closed so that the context stays usable.
cpc_status host_exception(cpc_ctx *c) noexcept {
  if (c && c->st) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(c->st, &cs) == cudaSuccess && cs != cudaStreamCaptureStatusNone) {
      cudaGraph_t g = nullptr;
      cudaStreamEndCapture(c->st, &g);
      if (g) cudaGraphDestroy(g);
      cudaGetLastError();
    }
  }
  try {
    throw;
  } catch (const std::bad_alloc &) {
    return fail(c, CPC_ERR_NOMEM, "host allocation failed");
  } catch (const std::length_error &) {
    return fail(c, CPC_ERR_NOMEM, "host allocation too large");
  } catch (const std::exception &e) {
    return fail(c, CPC_ERR_HOST, std::string("host error: ") + e.what());
  } catch (...) {
    return fail(c, CPC_ERR_HOST, "host error");
  }
}

cpc_status cuda_fail(cpc_ctx *c, cudaError_t e, const char *where) {
  std::string m = std::string(where) + ": " + cudaGetErrorString(e);
  if (e == cudaErrorMemoryAllocation) return fail(c, CPC_ERR_NOMEM, m);
  if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return fail(c, CPC_ERR_NODEVICE, m);
  return fail(c, CPC_ERR_CUDA, m);
}

#define CK(expr, where)                              \
  do {                                               \
    cudaError_t _e = (expr);                         \
    if (_e != cudaSuccess) return cuda_fail(c, _e, where); \
  } while (0)

// Run f(begin, end, part) over [0, n) in contiguous chunks on the host's cores
// (one chunk per thread, part < 64, at least min_chunk items each; in the
// calling thread when n is small).  Parts whose thread cannot be started run in
// the calling thread; the first exception thrown by a part is rethrown here
// after every part has finished.
template <class F>
void host_parallel(int64_t n, F &&f, int64_t min_chunk = 16384) {
  const int64_t hw = std::max(1u, std::thread::hardware_concurrency());
  const int T = (int)std::max<int64_t>(1, std::min<int64_t>({hw, 64, n / min_chunk}));
  if (T <= 1) {
    f((int64_t)0, n, 0);
    return;
  }
  std::exception_ptr errs[64];
  auto part = [&f, &errs, n, T](int t) {
    try {
      f(n * t / T, n * (t + 1) / T, t);
    } catch (...) {
      errs[t] = std::current_exception();
    }
  };
  std::vector<std::thread> th;
  th.reserve(T);
  int t = 0;
  for (; t < T; t++) {
    try {
      th.emplace_back(part, t);
    } catch (const std::system_error &) {
      break;
    }
  }
  for (; t < T; t++) part(t);
  for (auto &x : th) x.join();
  for (int k = 0; k < T; k++)
    if (errs[k]) std::rethrow_exception(errs[k]);
}

// float ULP at magnitude v (v > 0)
double ulpf(double v) {
  if (!(v > 0)) return std::ldexp(1.0, -149);
  int ex;
  std::frexp(v, &ex);  // v = m * 2^ex, m in [0.5, 1)
  return std::ldexp(1.0, ex - 1 - 23);
}
float f_up(double v) {
  float f = (float)v;
  if ((double)f < v) f = std::nextafter(f, INFINITY);
  return f;
}
float f_down(double v) {
  float f = (float)v;
  if ((double)f > v) f = std::nextafter(f, -INFINITY);
  return f;
}

cpc_status validate_params(cpc_ctx *c, const cpc_params &p) {
  if (const char *m = param_error(p)) return fail(c, CPC_ERR_INVALID, m);
  return CPC_OK;
}

// corels2's pair-type rules (corr.cpp:226-296) and corel choice
// (initialization.cpp:699-752).
struct JobRule {
  int corel, gws, swapped;
};
int job_rule(const cpc_params &p, cpc_pair_kind kind, int64_t n1, int64_t n2, JobRule &r) {
  int gws = 0;
  switch (kind) {
    case CPC_PAIR_DRS: case CPC_PAIR_RSRD: case CPC_PAIR_RSRS: gws = 0; break;
    case CPC_PAIR_SRD: case CPC_PAIR_SD: case CPC_PAIR_SRS: gws = 2; break;
    default: return -1;
  }
  int corel;
  if (kind == CPC_PAIR_RSRS || kind == CPC_PAIR_RSRD || p.which_corr == 0) corel = COREL_DD;
  else if (p.which_corr == 1) corel = COREL_SD;
  else if (p.which_corr == 2) corel = (kind == CPC_PAIR_SD) ? COREL_SS : COREL_SD;
  else corel = COREL_DK + (p.which_corr - 3);  // 3 DK, 4 SK, 5 ED
  if (corel == COREL_SS && p.estimator != 0) corel = COREL_SSA;
  r.swapped = 0;
  if (n2 > n1) {
    r.swapped = 1;
    if (gws == 2) gws = 1; else if (gws == 1) gws = 2;
  }
  r.corel = corel;
  r.gws = gws;
  return 0;
}

// corels1's rules (corr.cpp:103-216): g_with_shape = 1, no swap; corel by
// choose_corel_func (initialization.cpp:490-520) with do_RsRs or do_SS set.
int job_rule_auto(const cpc_params &p, cpc_pair_kind kind, JobRule &r) {
  int corel;
  if (kind == CPC_PAIR_RSRS) corel = COREL_DD;
  else if (kind == CPC_PAIR_SS)
    corel = p.which_corr == 0 ? COREL_DD : p.which_corr <= 2 ? COREL_SS : COREL_DK + (p.which_corr - 3);
  else return -1;
  if (corel == COREL_SS && p.estimator != 0) corel = COREL_SSA;
  r.swapped = 0;
  r.corel = corel;
  r.gws = 1;
  return 0;
}

void fill_views(Slot &s, FCat &f, DCat &d) {
  f.n = s.n;
  f.pos = s.pos.p;
  f.shp = s.shp.p;
  f.ewt = s.ewt.p;
  f.aux = s.aux.p;
  f.zlo = s.zlo.p;
  f.zf = s.zf.p;
  f.keep = s.keep.p;
  f.aflag = s.aflag.p;
  f.bk_start = s.bk_start.p;
  f.bk_end = s.bk_end.p;
  f.bk_region = s.bk_region.p;
  f.bk_zmin = s.bk_zmin.p;
  f.bk_zmax = s.bk_zmax.p;
  f.col_begin = s.col_begin.p;
  f.col_end = s.col_end.p;
  d.n = s.n;
  d.x = s.x.p; d.y = s.y.p; d.z = s.z.p; d.w = s.w.p;
  d.e1 = s.e1.p; d.e2 = s.e2.p; d.phi = s.phi.p; d.e3 = s.e3.p;
  d.jk = s.jk.p; d.keep = s.keep.p; d.orig = s.orig.p; d.aflag = s.aflag.p;
}

// z window offsets of lim_calc_xyz (PB_calcs.cpp:12-28): [p_min, p_max], or
// [-r_max, r_max] for coordinates 7 (p_min, p_max then bound mu)
double wz_lo(const cpc_params &p) { return p.coordinates == 7 ? -p.bin_r_max : p.p_min; }
double wz_hi(const cpc_params &p) { return p.coordinates == 7 ? p.bin_r_max : p.p_max; }

// error bound (absolute, per coordinate difference) of the FP32 separations
double eps_abs(const cpc_ctx *c, const Slot &a, const Slot &b) {
  const cpc_params &p = c->p;
  const double L = p.periodic_box_size;
  const double cmax = std::max({a.cmax, b.cmax, L});
  double e = 0;
  if (!(a.exact_f32 && b.exact_f32)) e += ulpf(cmax);
  const double wmax = std::max({p.bin_r_max, wz_hi(p), -wz_lo(p)});
  if (p.periodic_box && !(wmax <= 0.45 * L)) e += ulpf(2 * cmax);
  return e;
}

struct JobPlan {
  cpc_ctx *c;
  cpc_pair_kind kind;
  int s1, s2;  // after the swap
  JobRule rule;
  int wpi, tile;
  int64_t row_stride, row_offset;
  cpc_accum *out;
  JobDev jd;
  bool empty;
};

// every weight of both catalogues is 1: the weight sum is the count (the fast
// kernel keeps no words for it)
int unit_weights(const Slot &a, const Slot &b) {
  return (a.wmax == 1.0 && a.wmin == 1.0 && b.wmax == 1.0 && b.wmin == 1.0) ? 1 : 0;
}

// A context's unit shard replaced for the autotuner's trials, restored when the
// trials end (or on any early return).
struct ShardOverride {
  cpc_ctx *c;
  int shard, n_shards;
  bool active = true;
  ShardOverride(cpc_ctx *ctx, int sh, int nsh) : c(ctx), shard(ctx->shard), n_shards(ctx->n_shards) {
    c->shard = sh;
    c->n_shards = nsh;
  }
  void restore() {
    if (!active) return;
    c->shard = shard;
    c->n_shards = n_shards;
    active = false;
  }
  ~ShardOverride() { restore(); }
};

// Whether box slots sa and sb hold the same galaxies in the same (cell) order:
// positions, weights, shapes, orientations, regions and input rows identical
// (the keep flags, drawn from rand() per read, may differ).  A cross term of a
// catalogue with itself, uploaded as two samples, is such a pair.  Compared on
// the device, cached per slot versions.
bool slots_twin(cpc_ctx *c, int sa, int sb) {
  if (sa == sb) return true;
  Slot &A = c->slots[sa], &B = c->slots[sb];
  if (!A.valid || !B.valid || A.sky || B.sky || A.n != B.n || A.has_e != B.has_e ||
      A.kcells != B.kcells || A.ncx != B.ncx || A.ncy != B.ncy || A.n_reg != B.n_reg)
    return false;
  if (c->twin_s1 == sa && c->twin_s2 == sb && c->twin_v1 == A.version && c->twin_v2 == B.version)
    return c->twin_same;
  const int64_t n = A.n;
  bool same = false;
  if (c->d_differ.alloc(1) == cudaSuccess &&
      cudaMemsetAsync(c->d_differ.p, 0, sizeof(unsigned), c->st) == cudaSuccess) {
    const std::pair<const void *, const void *> arr8[] = {
        {A.x.p, B.x.p}, {A.y.p, B.y.p}, {A.z.p, B.z.p}, {A.w.p, B.w.p}, {A.e1.p, B.e1.p},
        {A.e2.p, B.e2.p}, {A.phi.p, B.phi.p}, {A.e3.p, B.e3.p}, {A.orig.p, B.orig.p}};
    bool ok = true;
    for (const auto &ab : arr8)
      ok = ok && launch_bytes_differ(ab.first, ab.second, 8 * n, c->d_differ.p, c->st) ==
                     cudaSuccess;
    ok = ok && launch_bytes_differ(A.jk.p, B.jk.p, 4 * n, c->d_differ.p, c->st) == cudaSuccess;
    unsigned d = 1;
    if (ok && cudaMemcpyAsync(&d, c->d_differ.p, sizeof d, cudaMemcpyDeviceToHost, c->st) ==
                  cudaSuccess &&
        cudaStreamSynchronize(c->st) == cudaSuccess)
      same = d == 0;
    c->launches += ok ? 10 : 0;
  }
  c->twin_s1 = sa;
  c->twin_s2 = sb;
  c->twin_v1 = A.version;
  c->twin_v2 = B.version;
  c->twin_same = same;
  return same;
}

// Whether a box cross term counts as a twin job: the fast engine on every
// outer row (no row sample), coordinates 6, a corel whose other order differs
// only in the fields FieldMap::a lists (density_density, shape_shape), a Pi
// binning symmetric about 0 and twin slots.  Symmetric: the exact thresholds
// satisfy |thr[k] + thr[npi - k]| <= 2^-24 |thr| + 1e-13 L (the reference's
// floor((Pi - p_min) / p_size) leaves them a few ulps from exact symmetry),
// a quarter of the guard of the fast path's Pi bands at most, so the other
// order of every pair the fast path bins has Pi bin npi - 1 - bin.
bool twin_job(cpc_ctx *c, const JobRule &rule, int s1, int s2, int64_t rs, int64_t ro,
              int auto_mode) {
  const cpc_params &p = c->p;
  if (!c->twin_on || auto_mode || rs > 1 || ro != 0 || p.coordinates != 6) return false;
  if (rule.corel != COREL_DD && rule.corel != COREL_SS && rule.corel != COREL_SSA) return false;
  const int npi = p.n_p_bin;
  if (npi < 1 || npi > kMaxPi) return false;
  const double tol_abs = 1e-13 * p.periodic_box_size;
  for (int k = 0; k <= npi; k++) {
    const double a = c->thr_pi[k], b = c->thr_pi[npi - k];
    if (!(std::fabs(a + b) <= std::ldexp(1.0, -24) * std::max(std::fabs(a), std::fabs(b)) + tol_abs))
      return false;
  }
  return slots_twin(c, s1, s2);
}

// allow_twin: false for the cell-list FP64 comparison engine, which counts every
// order and keeps the plain job's window
cpc_status plan_job(cpc_ctx *c, cpc_pair_kind kind, int slot_g1, int slot_g2, int64_t rs,
                    int64_t ro, cpc_accum *out, JobPlan &jp, int auto_mode = 0,
                    bool allow_twin = true) {
  if (slot_g1 < 0 || slot_g1 >= kMaxSlots || slot_g2 < 0 || slot_g2 >= kMaxSlots)
    return fail(c, CPC_ERR_INVALID, "slot out of range");
  Slot &A = c->slots[slot_g1], &B = c->slots[slot_g2];
  if (!A.valid || !B.valid) return fail(c, CPC_ERR_STATE, "count before upload");
  if (!out || !out->num || !out->sums) return fail(c, CPC_ERR_INVALID, "null output arrays");
  const cpc_params &p = c->p;
  jp.c = c;
  jp.kind = kind;
  jp.out = out;
  jp.row_stride = rs > 1 ? rs : 1;
  jp.row_offset = ro;
  if ((auto_mode ? job_rule_auto(p, kind, jp.rule) : job_rule(p, kind, A.n, B.n, jp.rule)) != 0)
    return fail(c, CPC_ERR_INVALID, "bad pair kind");
  jp.s1 = jp.rule.swapped ? slot_g2 : slot_g1;
  jp.s2 = jp.rule.swapped ? slot_g1 : slot_g2;
  Slot &g1 = c->slots[jp.s1], &g2 = c->slots[jp.s2];
  if (g1.ncx != g2.ncx || g1.ncy != g2.ncy || g1.n_reg != g2.n_reg)
    return fail(c, CPC_ERR_STATE, "catalogues were uploaded with different cell grids");
  jp.empty = (A.n == 0 || B.n == 0);
  const int nrp = p.n_bins, npi = p.n_p_bin;
  const int jk = p.do_jk ? 1 : 0;
  // block-local Pi window: as many Pi bins as fit kFastBlocksPerSM blocks per SM.  With
  // coordinates 7 the mu bins have no locality in z: a block holds every mu bin
  // when they fit (else the units are repeated over slices of wpi mu bins)
  const bool rmu = p.coordinates == 7;
  // twin job: each unordered pair once, both orders added (its block holds the
  // other order's histograms too, so the window is narrower; it covers only
  // the pair order with g2 ahead, whose units span half the Pi range)
  const int twin =
      (allow_twin && !jp.empty && twin_job(c, jp.rule, jp.s1, jp.s2, rs, ro, auto_mode)) ? 1 : 0;
  const int wmin = rmu ? 1 : twin ? 5 : 8;
  // Automatic window: the largest that fits 4 blocks per SM when it holds at
  // least 12 Pi bins (or all of them), else the largest for 3 blocks.
  const size_t static_b = fast_static_smem_bytes(twin);
  auto fit = [&](int blocks) {
    const size_t budget = (size_t)(228 * 1024) / blocks - static_b - 1024;
    int w = npi;
    while (w > wmin && fast_smem_bytes(jp.rule.corel, jk, nrp, w, auto_mode,
                                       unit_weights(g1, g2), twin) > budget)
      w--;
    return w;
  };
  int wpi = npi;
  if (c->tune_wpi > 0 && !rmu) {
    wpi = std::min(npi, c->tune_wpi);
  } else {
    wpi = fit(kFastBlocksPerSM);
    if (wpi < npi && wpi < 12) wpi = std::max(wpi, fit(kFastBlocksPerSM - 1));
  }
  if (!rmu && wpi < npi && wpi < wmin) wpi = std::min(npi, wmin);
  jp.wpi = wpi;
  jp.tile = kTileThreads;

  JobDev &J = jp.jd;
  std::memset(&J, 0, sizeof J);
  fill_views(g1, J.f1, J.d1);
  fill_views(g2, J.f2, J.d2);
  J.corel = jp.rule.corel;
  J.gws = jp.rule.gws;
  J.twin = twin;
  J.which_corr = p.which_corr;
  J.estimator = p.estimator;
  J.do_jk = jk;
  J.n_jk = p.n_jk;
  J.periodic = p.periodic_box ? 1 : 0;
  J.coordinates = p.coordinates;
  J.nrp = nrp;
  J.npi = npi;
  J.wpi = wpi;
  J.lin_bin = p.lin_bin ? 1 : 0;
  J.box_same_keep = 1;  // jk_check_PB (jk.cpp:64-71) for coordinates 6
  J.auto_mode = auto_mode;
  J.has_lo = (g1.exact_f32 && g2.exact_f32) ? 0 : 1;
  J.rmu = rmu ? 1 : 0;
  J.ncx = g1.ncx;
  J.ncy = g1.ncy;
  J.row_stride = jp.row_stride;
  J.row_offset = jp.row_offset;
  const double L = p.periodic_box_size;
  J.L = L;
  J.Lf = (float)L;
  J.rmin = p.bin_r_min;
  J.rmax = p.bin_r_max;
  J.pmin = p.p_min;
  J.pmax = p.p_max;
  J.wz_lo = wz_lo(p);
  J.wz_hi = wz_hi(p);
  J.ps = c->ps;
  J.rsize = c->rsize;
  for (int k = 0; k <= nrp; k++) J.thr[k] = c->thr_rp[k];
  // ---- guard bands (see pair_fast.cu): relative 2^-21 per coordinate
  // difference, 2^-20 on r^2, plus the absolute representation/wrap error.
  const double ea = eps_abs(c, g1, g2);
  const double crel = std::ldexp(1.0, -21);
  const double zlo_w = J.wz_lo, zhi_w = J.wz_hi;
  const double dtiny = 1e-12 * (L + std::max({p.bin_r_max, zhi_w, -zlo_w}));
  const double gxy = crel * p.bin_r_max + 2 * ea + dtiny;
  J.xy_in = f_down(p.bin_r_max - gxy);
  J.xy_out = f_up(p.bin_r_max + gxy);
  auto gp = [&](double v) { return crel * std::fabs(v) + 2 * ea + dtiny + 1e-30; };
  J.pi_in_lo = f_up(zlo_w + gp(zlo_w));
  J.pi_out_lo = f_down(zlo_w - gp(zlo_w));
  J.pi_in_hi = f_down(zhi_w - gp(zhi_w));
  J.pi_out_hi = f_up(zhi_w + gp(zhi_w));
  if (!rmu) {
    for (int k = 0; k < npi; k++) {
      const double lo = c->thr_pi[k], hi = c->thr_pi[k + 1];
      J.PA[k] = f_up(lo + gp(lo));
      J.PB[k] = f_down(hi - gp(hi));
    }
  } else {
    // mu bins: the edges themselves (nearest float); a pair is inside bin k when
    // dz - PA[k] r >= mu_rel r + mu_abs and PB[k] r - dz > mu_rel r + mu_abs,
    // which covers the float errors of dz, r, the edge and the products
    for (int k = 0; k < npi; k++) {
      J.PA[k] = (float)c->thr_pi[k];
      J.PB[k] = (float)c->thr_pi[k + 1];
    }
    const double tmax = std::max({1.0, std::fabs(p.p_min), std::fabs(p.p_max)});
    J.mu_rel = (float)(std::ldexp(1.0, -19) * tmax);
    J.mu_abs = (float)(8 * ea * tmax + dtiny + 1e-30);
  }
  J.inv_ps_f = (float)(1.0 / c->ps);
  J.tp0 = (float)(-p.p_min / c->ps);
  // r^2 error bound: two squared differences (r_p), three for coordinates 7 (r)
  const double nterm = rmu ? 3.0 : 2.0;
  auto gr = [&](double T) {
    return std::ldexp(1.0, -20) * T * T + 2.0 * std::sqrt(nterm) * T * ea + nterm * ea * ea +
           1e-12 * T * T;
  };
  for (int k = 0; k < nrp; k++) {
    const double lo = c->thr_rp[k], hi = c->thr_rp[k + 1];
    J.A[k] = f_up(lo * lo + gr(lo));
    J.B[k] = f_down(hi * hi - gr(hi));
  }
  J.rej_lo = f_down(c->thr_rp[0] * c->thr_rp[0] - gr(c->thr_rp[0]));
  J.rej_hi = f_up(c->thr_rp[nrp] * c->thr_rp[nrp] + gr(c->thr_rp[nrp]));
  J.rmin_f = (float)p.bin_r_min;
  J.inv_rsize_f = (float)(1.0 / c->rsize);
  if (p.lin_bin) {  // linear bins: estimate index from r, bands still decide
    J.l2rmin2 = 0.f;
    J.inv_lw = 0.f;
  } else {
    J.l2rmin2 = (float)(2.0 * std::log2(p.bin_r_min));
    J.inv_lw = (float)(1.0 / (2.0 * std::log2(p.bin_r_max / p.bin_r_min) / nrp));
  }
  // fixed-point scales: field f's terms are rint(v 2^S_f) with
  // |v_f| 2^S_f <= 2^29 / (1 + 2^-12) < 2^29 - 2^17 (see pair_fast.cu); S_f
  // from a bound on |v_f| (emax bounds |e|, so every rotated ellipticity)
  {
    const double wm = std::max(g1.wmax, 1e-30) * std::max(g2.wmax, 1e-30);
    const double em = std::max({g1.emax, g2.emax, 1e-30});
    // |phi - theta| folded (calcs.cpp:97-105): phi = -10 for galaxies read
    // without shapes gives values outside [0, pi/2]
    const double tm = std::max(M_PI / 2, std::max(g1.phimax, g2.phimax) + M_PI);
    const double tm2 = (jp.rule.corel == COREL_SSA) ? 2 * tm : tm;
    double vb[kNF];
    vb[0] = wm;
    vb[1] = vb[3] = wm * em;
    vb[2] = vb[4] = wm * wm * em * em;
    vb[5] = vb[7] = vb[9] = wm * em * em;
    vb[6] = vb[8] = vb[10] = wm * wm * em * em * em * em;
    vb[11] = tm2;
    vb[12] = 2 * tm * tm;
    if (jp.rule.corel == COREL_ED) {  // cos^2 <= |e|^2 <= 3 max|e_k|^2
      vb[11] = std::max(1.0, 3 * em * em);
      vb[12] = vb[11] * vb[11];
    }
    for (int f = 0; f < kNF; f++) {
      const double v = std::max(vb[f] * (1.0 + 1.0 / 4096.0), 1e-30);
      int S = 29 - (int)std::ceil(std::log2(v));
      S = std::min(60, std::max(-60, S));
      J.qscale[f] = (float)std::ldexp(1.0, S);
      J.inv_qscale[f] = std::ldexp(1.0, -S);
    }
  }
  J.qbias = 1 << 29;
  J.unit_w = unit_weights(g1, g2);
  return CPC_OK;
}

// tiles of g1 rows and their units (cached per slot versions and window)
const std::vector<UnitDesc> &build_units(JobPlan &jp) {
  cpc_ctx *c = jp.c;
  for (auto &uc : c->unit_cache)
    if (uc.s1 == jp.s1 && uc.s2 == jp.s2 && uc.v1 == c->slots[jp.s1].version &&
        uc.v2 == c->slots[jp.s2].version && uc.wpi == jp.wpi && uc.tile == jp.tile &&
        uc.twin == jp.jd.twin)
      return uc.units;
  if (c->unit_cache.size() >= 8) c->unit_cache.erase(c->unit_cache.begin());
  c->unit_cache.emplace_back();
  UnitCache &uc = c->unit_cache.back();
  uc.s1 = jp.s1;
  uc.s2 = jp.s2;
  uc.v1 = c->slots[jp.s1].version;
  uc.v2 = c->slots[jp.s2].version;
  uc.wpi = jp.wpi;
  uc.tile = jp.tile;
  uc.twin = jp.jd.twin;
  const cpc_params &p = c->p;
  const Slot &g1 = c->slots[jp.s1];
  const double L = p.periodic_box_size;
  const double ps = c->ps;
  const int npi = p.n_p_bin, wpi = jp.wpi;
  const double cmax = std::max(g1.cmax, L);
  const double ea = eps_abs(c, g1, c->slots[jp.s2]);
  const bool rmu = p.coordinates == 7;
  const double zw0 = wz_lo(p), zw1 = wz_hi(p);
  const double guard = 4 * ulpf(2 * cmax) + 2 * ea + std::ldexp(1.0, -20) * (std::fabs(zw0) + std::fabs(zw1) + p.bin_r_max);
  // tile z-extent: wide enough that the 32 lanes of a warp (spread over the
  // tile) see different Pi bins, small enough to fit the block-local window
  double Emax = 0.25 * (zw1 - zw0);
  if (!rmu) {
    if (wpi < npi) Emax = std::min(Emax, (wpi - 6) * ps / 2.0);
    Emax = std::max(Emax, std::min(2.0 * ps, 0.25 * (p.p_max - p.p_min)));
  }
  // sparse buckets: a chunk of extent Emax may hold fewer rows than a warp has
  // lanes (the other lanes then test rows that do not exist); such a chunk grows
  // up to Ehi, the widest extent whose units still fit the window
  // ((wpi - 4) ps - extent >= ps), until it holds 32 rows
  const double Ehi = (!rmu && wpi < npi) ? std::max(Emax, (wpi - 5) * ps) : Emax;
  const int ncx = g1.ncx, ncy = g1.ncy;
  const double inv_cwx = 1.0 / g1.cw_x, inv_cwy = 1.0 / g1.cw_y;
  std::vector<UnitDesc> &units = uc.units;
  units.clear();
  const int nb = (int)g1.h_bk_start.size();
  // buckets are independent: contiguous bucket ranges on the host's cores, each
  // into its own list, concatenated in bucket order (the serial order)
  std::vector<std::vector<UnitDesc>> part_units(64);
  host_parallel(nb, [&](int64_t b_lo, int64_t b_hi, int part) {
    std::vector<UnitDesc> &units = part_units[part];
    for (int b = (int)b_lo; b < (int)b_hi; b++) {
      const int s = g1.h_bk_start[b], e = g1.h_bk_end[b];
      int i = s;
      while (i < e) {
        // z-chunk of extent <= Emax, dealt round-robin into tiles of <= tile rows
        const float z0 = g1.h_pos[i].z;
        int j = i;
        float bx0 = INFINITY, bx1 = -INFINITY, by0 = INFINITY, by1 = -INFINITY;
        while (j < e && ((double)g1.h_pos[j].z - z0 <= Emax ||
                         (j - i < 32 && (double)g1.h_pos[j].z - z0 <= Ehi))) {
          bx0 = std::min(bx0, g1.h_pos[j].x);
          bx1 = std::max(bx1, g1.h_pos[j].x);
          by0 = std::min(by0, g1.h_pos[j].y);
          by1 = std::max(by1, g1.h_pos[j].y);
          j++;
        }
        const int m = j - i;
        const int nt = (m + jp.tile - 1) / jp.tile;
        const double zt0 = g1.h_pos[i].z, zt1 = g1.h_pos[j - 1].z;
        const double rg = p.bin_r_max + guard;
        int cx0 = (int)std::floor((bx0 - rg) * inv_cwx), cx1 = (int)std::floor((bx1 + rg) * inv_cwx);
        int cy0 = (int)std::floor((by0 - rg) * inv_cwy), cy1 = (int)std::floor((by1 + rg) * inv_cwy);
        if (p.periodic_box) {
          cx0 = std::max(cx0, -ncx); cx1 = std::min(cx1, 2 * ncx - 1);
          cy0 = std::max(cy0, -ncy); cy1 = std::min(cy1, 2 * ncy - 1);
        } else {
          cx0 = std::max(cx0, 0); cx1 = std::min(cx1, ncx - 1);
          cy0 = std::max(cy0, 0); cy1 = std::min(cy1, ncy - 1);
        }
        // twin jobs: only candidates ahead of the rows (Pi >= 0; the other order
        // is added with each pair)
        const double Zlo = zt0 + (jp.jd.twin ? 0.0 : zw0) - guard, Zhi = zt1 + zw1 + guard;
        for (int k = 0; k < nt; k++) {
          UnitDesc u;
          std::memset(&u, 0, sizeof u);
          u.g1_start = i + k;
          u.g1_stride = nt;
          u.g1_count = (m - k + nt - 1) / nt;
          u.region = g1.h_bk_region[b];
          u.cx_lo = cx0; u.cx_hi = cx1; u.cy_lo = cy0; u.cy_hi = cy1;
          if (wpi >= npi || rmu) {
            // coordinates 7: one unit per slice of wpi mu bins; each pair is
            // taken by the slice holding its estimated bin (pair_fast.cu)
            u.zlo = Zlo;
            u.zhi = Zhi;
            for (int base = 0; base < npi; base += wpi) {
              u.n2_base = base;
              units.push_back(u);
            }
          } else {
            const double span = std::max(ps, (wpi - 4) * ps - (zt1 - zt0));
            const int U = std::max(1, (int)std::ceil((Zhi - Zlo) / span));
            for (int q = 0; q < U; q++) {
              const double a = (q == 0) ? Zlo : Zlo + (Zhi - Zlo) * q / U;
              const double bnd = (q == U - 1) ? Zhi : Zlo + (Zhi - Zlo) * (q + 1) / U;
              int base = (int)std::floor((a - zt1 - p.p_min) / ps) - 1;
              base = std::max(0, std::min(base, npi - wpi));
              u.n2_base = base;
              u.zlo = a;
              u.zhi = bnd;
              units.push_back(u);
            }
          }
        }
        i = j;
      }
    }
  }, 512);  // a bucket's units take microseconds: threads pay for large catalogues
  size_t total = 0;
  for (const auto &v : part_units) total += v.size();
  units.reserve(total);
  for (const auto &v : part_units) units.insert(units.end(), v.begin(), v.end());
  return units;
}

cpc_status ensure_scratch(cpc_ctx *c, size_t n_units, size_t n_jobs) {
  CK(c->d_units.alloc(n_units), "alloc units");
  CK(c->d_jobs.alloc(n_jobs), "alloc jobs");
  CK(c->d_unit_ctr.alloc(1), "alloc counter");
  CK(c->d_qcount.alloc(1), "alloc queue counter");
  if (!c->d_queue.p) {
    c->qcap = CPC_EDGE_QUEUE_INIT;
    // CPC_EDGE_QUEUE_INIT in the environment (a positive entry count) starts the
    // context with another capacity: tests use a small one to drive the overflow
    // path (grow, count again)
    if (const char *ev = std::getenv("CPC_EDGE_QUEUE_INIT")) {
      const long long v = std::atoll(ev);
      if (v > 0) c->qcap = (unsigned long long)v;
    }
    cudaError_t e = c->d_queue.alloc(c->qcap);
    if (e != cudaSuccess) {
      cudaGetLastError();
      c->qcap = 1ull << 20;
      CK(c->d_queue.alloc(c->qcap), "alloc edge queue");
    }
  }
  return CPC_OK;
}

cpc_status alloc_accum(cpc_ctx *c) {
  const cpc_params &p = c->p;
  const size_t n_hist = 1 + (p.do_jk ? p.n_jk : 0);
  const size_t cells = n_hist * p.n_bins * p.n_p_bin;
  CK(c->d_num.alloc(cells), "alloc accum");
  CK(c->d_sums.alloc(cells * kNF), "alloc accum");
  CK(c->d_counters.alloc(4), "alloc counters");
  return CPC_OK;
}

cpc_status zero_accum(cpc_ctx *c, cudaStream_t st) {
  const cpc_params &p = c->p;
  const size_t n_hist = 1 + (p.do_jk ? p.n_jk : 0);
  const size_t cells = n_hist * p.n_bins * p.n_p_bin;
  CK(cudaMemsetAsync(c->d_num.p, 0, sizeof(unsigned long long) * cells, st), "memset");
  CK(cudaMemsetAsync(c->d_sums.p, 0, sizeof(double) * cells * kNF, st), "memset");
  CK(cudaMemsetAsync(c->d_counters.p, 0, sizeof(unsigned long long) * 4, st), "memset");
  return CPC_OK;
}

// the histogram block and counters in device buffers num / sums / counters
cpc_status fetch_accum_from(cpc_ctx *c, const unsigned long long *num, const double *sums,
                            const unsigned long long *counters, cpc_accum *out, cudaStream_t st,
                            int unit_w) {
  const cpc_params &p = c->p;
  const size_t n_hist = 1 + (p.do_jk ? p.n_jk : 0);
  const size_t cells = n_hist * p.n_bins * p.n_p_bin;
  unsigned long long cnt[4];
  CK(cudaMemcpyAsync(out->num, num, sizeof(int64_t) * cells, cudaMemcpyDeviceToHost, st), "D2H");
  CK(cudaMemcpyAsync(out->sums, sums, sizeof(double) * cells * kNF, cudaMemcpyDeviceToHost, st), "D2H");
  CK(cudaMemcpyAsync(cnt, counters, sizeof cnt, cudaMemcpyDeviceToHost, st), "D2H");
  CK(cudaStreamSynchronize(st), "sync");
  if (unit_w)
    for (size_t k = 0; k < cells; k++) out->sums[k * kNF] = (double)out->num[k];
  out->n_window = (int64_t)(cnt[0] + cnt[1]);
  out->n_rechecked = (int64_t)cnt[2];
  int64_t nb = 0;
  const size_t c0 = (size_t)p.n_bins * p.n_p_bin;
  for (size_t k = 0; k < c0; k++) nb += out->num[k];
  out->n_binned = nb;
  return CPC_OK;
}

cpc_status fetch_accum(cpc_ctx *c, cpc_accum *out, cudaStream_t st, int unit_w) {
  return fetch_accum_from(c, c->d_num.p, c->d_sums.p, c->d_counters.p, out, st, unit_w);
}

cpc_status build_zorder(cpc_ctx *c, Slot &s) {
  if (s.zbuilt) return CPC_OK;
  const int64_t n = s.n;
  cudaStream_t st = c->st;
  CK(c->d_keys.alloc(n), "alloc");
  CK(c->d_ktmp.alloc(n), "alloc");
  CK(c->d_vals.alloc(n), "alloc");
  CK(c->d_vtmp.alloc(n), "alloc");
  CK(c->d_hist.alloc(radix_hist_words(n)), "alloc");
  CK(c->d_census.alloc(8 * 256), "alloc");
  CK(launch_z_keys(n, s.z.p, c->d_keys.p, c->d_vals.p, st), "z keys");
  CK(radix_sort_pairs(n, c->d_keys.p, c->d_vals.p, c->d_ktmp.p, c->d_vtmp.p, c->d_hist.p,
                      c->d_census.p, st, &c->launches), "z sort");
  c->launches += 2;  // z keys + gather
  CK(s.zx.alloc(n), "alloc"); CK(s.zy.alloc(n), "alloc"); CK(s.zz.alloc(n), "alloc");
  CK(s.zw.alloc(n), "alloc"); CK(s.ze1.alloc(n), "alloc"); CK(s.ze2.alloc(n), "alloc");
  CK(s.zphi.alloc(n), "alloc"); CK(s.zjk.alloc(n), "alloc"); CK(s.zkeep.alloc(n), "alloc");
  CK(s.zorig.alloc(n), "alloc"); CK(s.ze3.alloc(n), "alloc");
  GatherIn in{s.x.p, s.y.p, s.z.p, s.w.p, s.e1.p, s.e2.p, s.phi.p, s.jk.p, s.keep.p, s.e3.p};
  GatherOut out{};
  out.x = s.zx.p; out.y = s.zy.p; out.z = s.zz.p; out.w = s.zw.p;
  out.e1 = s.ze1.p; out.e2 = s.ze2.p; out.phi = s.zphi.p; out.e3 = s.ze3.p; out.jk = s.zjk.p;
  out.keep = s.zkeep.p; out.orig = s.zorig.p; out.orig_in = s.orig.p;
  CK(launch_gather(n, c->d_keys.p, c->d_vals.p, in, out, st), "z gather");
  CK(s.zaflag.alloc(n), "alloc");
  CK(launch_gather_u8(n, c->d_vals.p, s.aflag.p, s.zaflag.p, st), "z gather");
  c->launches += 1;
  CK(cudaStreamSynchronize(st), "sync");
  s.zbuilt = true;
  return CPC_OK;
}

DCat zview(Slot &s) {
  DCat d;
  d.n = s.n;
  d.x = s.zx.p; d.y = s.zy.p; d.z = s.zz.p; d.w = s.zw.p;
  d.e1 = s.ze1.p; d.e2 = s.ze2.p; d.phi = s.zphi.p; d.e3 = s.ze3.p;
  d.jk = s.zjk.p; d.keep = s.zkeep.p; d.orig = s.zorig.p; d.aflag = s.zaflag.p;
  return d;
}

// the plain FP64 kernel: enqueue on the context's stream, then fetch
cpc_status enqueue_plain(JobPlan &jp) {
  cpc_ctx *c = jp.c;
  cpc_status s;
  if ((s = alloc_accum(c)) != CPC_OK) return s;
  if ((s = zero_accum(c, c->st)) != CPC_OK) return s;
  CK(cudaEventRecord(c->e0, c->st), "event");
  if (jp.empty) {
    CK(cudaEventRecord(c->e1, c->st), "event");
    return CPC_OK;
  }
  Slot &g1 = c->slots[jp.s1], &g2 = c->slots[jp.s2];
  if ((s = build_zorder(c, g1)) != CPC_OK) return s;
  if ((s = build_zorder(c, g2)) != CPC_OK) return s;
  if ((s = ensure_scratch(c, 1, 1)) != CPC_OK) return s;
  jp.jd.acc_num = c->d_num.p;
  jp.jd.acc_sums = c->d_sums.p;
  jp.jd.counters = c->d_counters.p;
  DCat a = zview(g1), b = zview(g2);
  jp.jd.d1 = a;
  jp.jd.d2 = b;
  CK(cudaMemcpyAsync(c->d_jobs.p, &jp.jd, sizeof(JobDev), cudaMemcpyHostToDevice, c->st), "H2D job");
  CK(launch_plain_fp64(c->d_jobs.p, a, b, c->st), "plain fp64 kernel");
  c->launches += 1;
  CK(cudaEventRecord(c->e1, c->st), "event");
  return CPC_OK;
}

cpc_status finish_plain(JobPlan &jp) {
  cpc_ctx *c = jp.c;
  cpc_status s;
  if ((s = fetch_accum(c, jp.out, c->st, 0)) != CPC_OK) return s;
  float ms = 0;
  CK(cudaEventElapsedTime(&ms, c->e0, c->e1), "event time");
  jp.out->kernel_ms = ms;
  jp.out->pair_kernel_ms = ms;
  return CPC_OK;
}

cpc_status run_plain(JobPlan &jp) {
  const cpc_status s = enqueue_plain(jp);
  return s != CPC_OK ? s : finish_plain(jp);
}

// fast engine over one or more jobs (one persistent launch per corel group):
// enqueue on the first context's stream, then wait, check the edge queue and
// fetch
cpc_status run_fast(std::vector<JobPlan> &jobs, int grow_attempt = 0);

// one persistent launch of the fast kernel over a range of the unit list
struct FastGroup {
  int corel, jk, minb, grid;
  size_t first, n_units, smem;
  FastScales sc;
  int auto_pairs;  // the group holds corels1 jobs (their rules in shared memory)
  int twin;        // the group's jobs are twin jobs (their own kernel)
};

size_t accum_cells(const cpc_ctx *c) {
  const cpc_params &p = c->p;
  return (size_t)(1 + (p.do_jk ? p.n_jk : 0)) * p.n_bins * p.n_p_bin;
}

// The device work of one fast count, in stream order on st: zero every job's
// histogram block and counters, the edge-queue counter, then per group the
// unit counter and the persistent kernel, then the FP64 recheck.  rec_flags
// records the timing events (cudaEventRecordExternal inside a capture, so
// that they become event nodes of the graph).
cpc_status fast_body(cpc_ctx *c0, std::vector<JobPlan> &jobs, const std::vector<FastGroup> &gs,
                     cudaStream_t st, unsigned rec_flags) {
  cpc_ctx *c = c0;
  for (size_t k = 0; k < jobs.size(); k++) {
    const cpc_status s = zero_accum(jobs[k].c, st);
    if (s != CPC_OK) return s;
  }
  CK(cudaMemsetAsync(c0->d_qcount.p, 0, sizeof(unsigned long long), st), "memset");
  CK(cudaEventRecordWithFlags(c0->e0, st, rec_flags), "event");
  for (const FastGroup &g : gs) {
    CK(cudaMemsetAsync(c0->d_unit_ctr.p, 0, sizeof(unsigned int), st), "memset");
    CK(launch_fast(g.corel, g.jk, g.minb, g.twin, c0->d_jobs.p, c0->d_units.p + g.first,
                   (int)g.n_units,
                   c0->d_unit_ctr.p, c0->d_queue.p, c0->d_qcount.p, c0->qcap, g.sc, g.smem,
                   g.grid, g.auto_pairs, st),
       "fast kernel");
  }
  CK(cudaEventRecordWithFlags(c0->e2, st, rec_flags), "event");
  CK(launch_recheck(c0->d_jobs.p, c0->d_queue.p, c0->d_qcount.p, c0->qcap, c0->sm_count * 8, st),
     "recheck kernel");
  CK(cudaEventRecordWithFlags(c0->e1, st, rec_flags), "event");
  return CPC_OK;
}

// Everything fast_body bakes into its launches: buffer addresses and sizes,
// queue capacity, and each group's kernel, unit range, grid and shared memory.
std::vector<uint64_t> fast_graph_key(cpc_ctx *c0, const std::vector<JobPlan> &jobs,
                                     const std::vector<FastGroup> &gs) {
  std::vector<uint64_t> k;
  auto put = [&](uint64_t v) { k.push_back(v); };
  put((uint64_t)(uintptr_t)c0->st);
  put((uint64_t)(uintptr_t)c0->d_jobs.p);
  put((uint64_t)(uintptr_t)c0->d_units.p);
  put((uint64_t)(uintptr_t)c0->d_unit_ctr.p);
  put((uint64_t)(uintptr_t)c0->d_queue.p);
  put((uint64_t)(uintptr_t)c0->d_qcount.p);
  put(c0->qcap);
  put((uint64_t)c0->sm_count);
  put(jobs.size());
  for (const JobPlan &jp : jobs) {
    put((uint64_t)(uintptr_t)jp.c->d_num.p);
    put((uint64_t)(uintptr_t)jp.c->d_sums.p);
    put((uint64_t)(uintptr_t)jp.c->d_counters.p);
    put(accum_cells(jp.c));
  }
  put(gs.size());
  for (const FastGroup &g : gs) {
    put((uint64_t)g.corel);
    put((uint64_t)g.jk);
    put((uint64_t)g.minb);
    put((uint64_t)g.grid);
    put(g.first);
    put(g.n_units);
    put(g.smem);
    put((uint64_t)g.auto_pairs);
    put((uint64_t)g.twin);
    for (int f = 0; f < kNF; f++) {  // the scales are kernel parameters too
      uint32_t b;
      std::memcpy(&b, &g.sc.qs[f], sizeof b);
      put(b);
    }
  }
  return k;
}

void drop_graph(cpc_ctx *c) {
  if (c->gexec) cudaGraphExecDestroy(c->gexec);
  c->gexec = nullptr;
  c->gkey.clear();
}

// Launch the fast count's device work: replay the context's graph when it was
// captured for the same key, else capture it anew (or launch directly when
// graphs are off or the capture fails, which turns graphs off for the context).
cpc_status launch_fast_body(cpc_ctx *c0, std::vector<JobPlan> &jobs,
                            const std::vector<FastGroup> &gs) {
  cpc_ctx *c = c0;
  cudaStream_t st = c0->st;
  const int64_t n_launch = (int64_t)gs.size() + 1;
  if (!c0->graph_on) {
    const cpc_status s = fast_body(c0, jobs, gs, st, cudaEventRecordDefault);
    if (s == CPC_OK) c0->launches += n_launch;
    return s;
  }
  std::vector<uint64_t> key = fast_graph_key(c0, jobs, gs);
  if (!c0->gexec || key != c0->gkey) {
    drop_graph(c0);
    cudaGraph_t g = nullptr;
    CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal), "begin capture");
    const cpc_status s = fast_body(c0, jobs, gs, st, cudaEventRecordExternal);
    const cudaError_t e_end = cudaStreamEndCapture(st, &g);
    cudaGraphExec_t ex = nullptr;
    cudaError_t e_inst = cudaErrorUnknown;
    if (s == CPC_OK && e_end == cudaSuccess && g) e_inst = cudaGraphInstantiate(&ex, g, 0);
    if (g) cudaGraphDestroy(g);
    if (s != CPC_OK || e_end != cudaSuccess || e_inst != cudaSuccess) {
      // capture unavailable here: direct launches from now on
      cudaGetLastError();
      if (ex) cudaGraphExecDestroy(ex);
      c0->graph_on = 0;
      const cpc_status s2 = fast_body(c0, jobs, gs, st, cudaEventRecordDefault);
      if (s2 == CPC_OK) c0->launches += n_launch;
      return s2;
    }
    c0->gexec = ex;
    c0->gkey = std::move(key);
    c0->graph_captures++;
  }
  CK(cudaGraphLaunch(c0->gexec, st), "graph launch");
  c0->graph_replays++;
  c0->launches += n_launch;
  return CPC_OK;
}

cpc_status enqueue_fast(std::vector<JobPlan> &jobs) {
  cpc_ctx *c0 = jobs[0].c;
  cpc_ctx *c = c0;
  cudaStream_t st = c0->st;
  std::vector<UnitDesc> all;
  for (size_t k = 0; k < jobs.size(); k++) {
    cpc_status s;
    if ((s = alloc_accum(jobs[k].c)) != CPC_OK) return s;
    jobs[k].jd.acc_num = jobs[k].c->d_num.p;
    jobs[k].jd.acc_sums = jobs[k].c->d_sums.p;
    jobs[k].jd.counters = jobs[k].c->d_counters.p;
  }
  // group by kernel template
  // group by kernel instantiation: corel, jackknife, twin
  std::map<std::tuple<int, int, int>, std::vector<int>> groups;
  for (size_t k = 0; k < jobs.size(); k++)
    if (!jobs[k].empty)
      groups[std::make_tuple(jobs[k].jd.corel, jobs[k].jd.do_jk, jobs[k].jd.twin)].push_back((int)k);
  size_t total_units = 0;
  std::vector<std::pair<size_t, size_t>> ranges;
  std::vector<std::tuple<int, int, int>> gkeys;
  for (auto &g : groups) {
    const size_t b = all.size();
    for (int k : g.second) {
      const std::vector<UnitDesc> &u = build_units(jobs[k]);
      // this context's shard of the units (cpc_set_shard): every n_shards-th
      // unit from `shard`; the units partition the pairs, so the shards' blocks
      // sum to the whole count
      const int nsh = jobs[k].c->n_shards, sh = jobs[k].c->shard;
      for (size_t ui = (size_t)sh; ui < u.size(); ui += (size_t)nsh) {
        UnitDesc d = u[ui];
        d.job = k;
        const int64_t ncol = (int64_t)(d.cx_hi - d.cx_lo + 1) * (d.cy_hi - d.cy_lo + 1);
        if (ncol < 1 || ncol > kFastMaxCols || d.g1_count < 1 || d.g1_count > kTileThreads)
          return fail(c, CPC_ERR_INVALID, "work unit outside kernel limits (too many neighbour columns)");
        all.push_back(d);
      }
    }
    ranges.push_back({b, all.size()});
    gkeys.push_back(g.first);
  }
  total_units = all.size();
  cpc_status s;
  if ((s = ensure_scratch(c0, std::max<size_t>(1, total_units), jobs.size())) != CPC_OK) return s;
  // size the edge queue from the rate earlier counts of this context queued
  // (per unit): a count whose queue overflows is run again, which a full count
  // after sharded or sampled ones would otherwise pay
  {
    const double need = c0->q_per_unit * (double)total_units * 1.25;
    if (need > (double)c0->qcap && need < 4e9) {
      unsigned long long cap = c0->qcap;
      while ((double)cap < need) cap *= 2;
      c0->d_queue.reset();
      CK(c0->d_queue.alloc(cap), "alloc edge queue");
      c0->qcap = cap;
    }
  }
  c0->last_units = total_units;
  c0->last_twin = 0;
  for (const JobPlan &jp : jobs) c0->last_twin |= jp.jd.twin;
  std::vector<JobDev> jds(jobs.size());
  for (size_t k = 0; k < jobs.size(); k++) jds[k] = jobs[k].jd;
  CK(cudaMemcpyAsync(c0->d_jobs.p, jds.data(), sizeof(JobDev) * jds.size(), cudaMemcpyHostToDevice, st), "H2D jobs");
  if (total_units)
    CK(cudaMemcpyAsync(c0->d_units.p, all.data(), sizeof(UnitDesc) * total_units, cudaMemcpyHostToDevice, st), "H2D units");
  std::vector<FastGroup> gs;
  for (size_t g = 0; g < ranges.size(); g++) {
    const int corel = std::get<0>(gkeys[g]), jk = std::get<1>(gkeys[g]), twin = std::get<2>(gkeys[g]);
    size_t smem = 0;  // the largest any job of the group needs
    FastScales sc;    // per field the smallest scale of the group's jobs
    int auto_pairs = 0;
    for (int f = 0; f < kNF; f++) {
      sc.qs[f] = INFINITY;
      sc.iqs[f] = 0.0;
    }
    for (size_t k = ranges[g].first; k < ranges[g].second; k++)
      auto_pairs |= jobs[all[k].job].jd.auto_mode ? 1 : 0;
    for (size_t k = ranges[g].first; k < ranges[g].second; k++) {
      const JobPlan &jp = jobs[all[k].job];
      smem = std::max(smem, fast_smem_bytes(corel, jk, jp.jd.nrp, jp.wpi, auto_pairs,
                                            jp.jd.unit_w, jp.jd.twin));
      for (int f = 0; f < kNF; f++)
        if (jp.jd.qscale[f] < sc.qs[f]) {
          sc.qs[f] = jp.jd.qscale[f];
          sc.iqs[f] = jp.jd.inv_qscale[f];
        }
    }
    int bps = 0;
    const int minb = fast_variant(corel, jk, smem, &bps,
                                  jobs[all[ranges[g].first].job].jd.all_exact, twin);
    if (bps <= 0) return fail(c, CPC_ERR_INVALID, "fast kernel does not fit on an SM with these bins");
    const size_t n_units = ranges[g].second - ranges[g].first;
    if (n_units == 0) continue;
    const int grid = (int)std::min<int64_t>((int64_t)c0->sm_count * bps, (int64_t)n_units);
    gs.push_back(
        FastGroup{corel, jk, minb, grid, ranges[g].first, n_units, smem, sc, auto_pairs, twin});
  }
  return launch_fast_body(c0, jobs, gs);
}

cpc_status finish_fast(std::vector<JobPlan> &jobs, int grow_attempt) {
  cpc_ctx *c0 = jobs[0].c;
  cpc_ctx *c = c0;
  cudaStream_t st = c0->st;
  cpc_status s;
  CK(cudaStreamSynchronize(st), "fast kernels");
  float ms = 0, pms = 0;
  CK(cudaEventElapsedTime(&ms, c0->e0, c0->e1), "event time");
  CK(cudaEventElapsedTime(&pms, c0->e0, c0->e2), "event time");
  unsigned long long qn = 0;
  CK(cudaMemcpy(&qn, c0->d_qcount.p, sizeof qn, cudaMemcpyDeviceToHost), "D2H");
  if (c0->last_units > 0 && !jobs[0].jd.all_exact)  // (the FP64 comparison queues every pair)
    c0->q_per_unit = std::max(c0->q_per_unit, (double)qn / (double)c0->last_units);
  if (qn > c0->qcap) {
    // the edge queue overflowed: grow it to hold every queued pair and count
    // again (the queued set does not depend on the order of execution)
    if (grow_attempt) return fail(c, CPC_ERR_NOMEM, "edge queue overflow after growing it");
    unsigned long long cap = c0->qcap;
    while (cap < qn) cap *= 2;
    c0->d_queue.reset();
    CK(c0->d_queue.alloc(cap), "alloc edge queue");
    c0->qcap = cap;
    return run_fast(jobs, 1);
  }
  for (size_t k = 0; k < jobs.size(); k++) {
    if ((s = fetch_accum(jobs[k].c, jobs[k].out, st, jobs[k].jd.unit_w)) != CPC_OK) return s;
    jobs[k].out->kernel_ms = ms;
    jobs[k].out->pair_kernel_ms = pms;
  }
  return CPC_OK;
}

cpc_status run_fast(std::vector<JobPlan> &jobs, int grow_attempt) {
  const cpc_status s = enqueue_fast(jobs);
  return s != CPC_OK ? s : finish_fast(jobs, grow_attempt);
}

// Cell list of slot s from a catalogue held in the context's upload buffers
// (u_x .. u_flag; orig_in maps their rows to input rows, null = identity):
// grid of columns r_max / k wide, keys, radix sort, gather into the slot, the
// bucket and column tables.  check_stats: the upload's device checks must pass.
cpc_status build_cells(cpc_ctx *c, Slot &s, int64_t n, int k, const int64_t *orig_in,
                       bool check_stats) {
  const cpc_params &p = c->p;
  const double L = p.periodic_box_size;
  const size_t nn = std::max<int64_t>(n, 1);
  cudaStream_t st = c->st;
  DevBuf<double> &ox = c->u_x, &oy = c->u_y, &oz = c->u_z, &ow = c->u_w, &oe1 = c->u_e1,
                 &oe2 = c->u_e2, &ophi = c->u_phi, &oe3 = c->u_e3;
  DevBuf<int32_t> &ojk = c->u_jk;
  DevBuf<uint8_t> &okeep = c->u_keep, &oflag = c->u_flag;
  // grid: columns of width >= r_max / k over [0, box)
  int nc = (int)std::floor(L / (p.bin_r_max / k));
  nc = std::max(1, std::min(nc, 2048));
  s.ncx = s.ncy = nc;
  s.cw_x = s.cw_y = L / nc;
  s.kcells = k;
  s.n_reg = p.do_jk ? p.n_jk : 1;
  if ((double)nc * nc * s.n_reg >= 4294967295.0) return fail(c, CPC_ERR_INVALID, "too many cell buckets");
  CK(c->d_keys.alloc(nn), "alloc"); CK(c->d_ktmp.alloc(nn), "alloc");
  CK(c->d_vals.alloc(nn), "alloc"); CK(c->d_vtmp.alloc(nn), "alloc");
  CK(c->d_hist.alloc(radix_hist_words(nn)), "alloc");
  CK(c->d_census.alloc(8 * 256), "alloc");
  CK(c->d_bucket.alloc(nn), "alloc");
  CK(s.pos.alloc(nn), "alloc"); CK(s.shp.alloc(nn), "alloc"); CK(s.zf.alloc(nn), "alloc");
  CK(s.ewt.alloc(nn), "alloc"); CK(s.aux.alloc(nn), "alloc"); CK(s.zlo.alloc(nn), "alloc"); CK(s.e3.alloc(nn), "alloc");
  CK(s.x.alloc(nn), "alloc"); CK(s.y.alloc(nn), "alloc"); CK(s.z.alloc(nn), "alloc");
  CK(s.w.alloc(nn), "alloc"); CK(s.e1.alloc(nn), "alloc"); CK(s.e2.alloc(nn), "alloc");
  CK(s.phi.alloc(nn), "alloc"); CK(s.jk.alloc(nn), "alloc"); CK(s.keep.alloc(nn), "alloc");
  CK(s.orig.alloc(nn), "alloc");
  CK(launch_cell_keys(n, ox.p, oy.p, oz.p, ojk.p, 1.0 / s.cw_x, 1.0 / s.cw_y, s.ncx, s.ncy, s.n_reg,
                      c->d_keys.p, c->d_vals.p, st), "cell keys");
  CK(radix_sort_pairs(n, c->d_keys.p, c->d_vals.p, c->d_ktmp.p, c->d_vtmp.p, c->d_hist.p,
                      c->d_census.p, st, &c->launches), "radix sort");
  if (n > 0) c->launches += 2;  // cell keys + gather
  GatherIn in{ox.p, oy.p, oz.p, ow.p, oe1.p, oe2.p, ophi.p, ojk.p, okeep.p, oe3.p};
  GatherOut go{};
  go.pos = s.pos.p; go.shp = s.shp.p; go.ewt = s.ewt.p; go.aux = s.aux.p; go.zlo = s.zlo.p; go.zf = s.zf.p;
  go.bucket = c->d_bucket.p;
  go.x = s.x.p; go.y = s.y.p; go.z = s.z.p; go.w = s.w.p; go.e1 = s.e1.p; go.e2 = s.e2.p;
  go.e3 = s.e3.p;
  go.phi = s.phi.p; go.jk = s.jk.p; go.keep = s.keep.p; go.orig = s.orig.p; go.orig_in = orig_in;
  CK(launch_gather(n, c->d_keys.p, c->d_vals.p, in, go, st), "gather");
  CK(s.aflag.alloc(nn), "alloc");
  if (n > 0) {
    CK(launch_gather_u8(n, c->d_vals.p, oflag.p, s.aflag.p, st), "gather");
    c->launches += 1;
  }
  // buckets on the host
  std::vector<uint32_t> hb(n);
  s.h_pos.resize(n);
  if (n > 0) {
    CK(cudaMemcpyAsync(hb.data(), c->d_bucket.p, 4 * n, cudaMemcpyDeviceToHost, st), "D2H");
    CK(cudaMemcpyAsync(s.h_pos.data(), s.pos.p, sizeof(float4) * n, cudaMemcpyDeviceToHost, st), "D2H");
  }
  CK(cudaStreamSynchronize(st), "upload");
  if (check_stats) {  // the device checks (first failing row of each kind) and statistics
    const UploadStats &u = c->h_ustats;
    static const char *what[4] = {"non-finite position", "position outside [0, box_size]",
                                  "non-finite weight, ellipticity or phi",
                                  "jackknife label out of range"};
    int kind = -1;
    for (int q = 0; q < 4; q++)
      if (u.bad_row[q] != ~0ull && (kind < 0 || u.bad_row[q] < u.bad_row[kind])) kind = q;
    if (kind >= 0)
      return fail(c, CPC_ERR_RANGE,
                  std::string(what[kind]) + " at row " + std::to_string(u.bad_row[kind]));
    double v;
    std::memcpy(&v, &u.cmax_bits, 8); s.cmax = v;
    std::memcpy(&v, &u.wmax_bits, 8); s.wmax = v;
    std::memcpy(&v, &u.emax_bits, 8); s.emax = v;
    std::memcpy(&v, &u.phimax_bits, 8); s.phimax = v;
    s.wmin = n > 0 ? from_orderable_key(u.wmin_key) : 1.0;
    s.exact_f32 = u.not_f32 == 0;
  }
  s.h_bk_start.clear(); s.h_bk_end.clear(); s.h_bk_region.clear();
  std::vector<float> bz0, bz1;
  const int ncol = s.ncx * s.ncy;
  std::vector<int> cb(ncol, 0), ce(ncol, 0);
  // bucket starts (rows whose key differs from the previous row's), found in
  // chunks on the host's cores and concatenated in row order
  std::vector<std::vector<int64_t>> part_starts(64);
  host_parallel(n, [&](int64_t b0, int64_t b1, int part) {
    for (int64_t i = b0; i < b1; i++)
      if (i == 0 || hb[i] != hb[i - 1]) part_starts[part].push_back(i);
  }, 1 << 20);  // a cheap pass: threads only pay for millions of rows
  std::vector<int64_t> starts;
  for (const auto &v : part_starts) starts.insert(starts.end(), v.begin(), v.end());
  for (size_t q = 0; q < starts.size(); q++) {
    const int64_t i = starts[q], j = q + 1 < starts.size() ? starts[q + 1] : n;
    const int b = (int)s.h_bk_start.size();
    const int col = (int)(hb[i] / s.n_reg), reg = (int)(hb[i] % s.n_reg);
    if (ce[col] == 0 && cb[col] == 0) cb[col] = b;
    ce[col] = b + 1;
    s.h_bk_start.push_back((int)i);
    s.h_bk_end.push_back((int)j);
    s.h_bk_region.push_back(reg);
    bz0.push_back(s.h_pos[i].z);
    bz1.push_back(s.h_pos[j - 1].z);
  }
  // columns with no bucket: empty range
  for (int q = 0; q < ncol; q++)
    if (ce[q] == 0) cb[q] = 0;
  const size_t nbk = std::max<size_t>(1, s.h_bk_start.size());
  CK(s.bk_start.alloc(nbk), "alloc"); CK(s.bk_end.alloc(nbk), "alloc");
  CK(s.bk_region.alloc(nbk), "alloc"); CK(s.bk_zmin.alloc(nbk), "alloc");
  CK(s.bk_zmax.alloc(nbk), "alloc"); CK(s.col_begin.alloc(ncol), "alloc");
  CK(s.col_end.alloc(ncol), "alloc");
  const size_t nb = s.h_bk_start.size();
  if (nb) {
    CK(cudaMemcpyAsync(s.bk_start.p, s.h_bk_start.data(), 4 * nb, cudaMemcpyHostToDevice, st), "H2D");
    CK(cudaMemcpyAsync(s.bk_end.p, s.h_bk_end.data(), 4 * nb, cudaMemcpyHostToDevice, st), "H2D");
    CK(cudaMemcpyAsync(s.bk_region.p, s.h_bk_region.data(), 4 * nb, cudaMemcpyHostToDevice, st), "H2D");
    CK(cudaMemcpyAsync(s.bk_zmin.p, bz0.data(), 4 * nb, cudaMemcpyHostToDevice, st), "H2D");
    CK(cudaMemcpyAsync(s.bk_zmax.p, bz1.data(), 4 * nb, cudaMemcpyHostToDevice, st), "H2D");
  }
  CK(cudaMemcpyAsync(s.col_begin.p, cb.data(), 4 * ncol, cudaMemcpyHostToDevice, st), "H2D");
  CK(cudaMemcpyAsync(s.col_end.p, ce.data(), 4 * ncol, cudaMemcpyHostToDevice, st), "H2D");
  CK(cudaStreamSynchronize(st), "upload");
  s.valid = true;
  return CPC_OK;
}

// Rebuild a box slot's cell list with columns r_max / k wide from its own
// device arrays (the autotuner's cell-size candidates).
cpc_status rebuild_cells(cpc_ctx *c, Slot &s, int k) {
  const int64_t n = s.n;
  const size_t nn = std::max<int64_t>(n, 1);
  cudaStream_t st = c->st;
  CK(c->u_x.alloc(nn), "alloc"); CK(c->u_y.alloc(nn), "alloc"); CK(c->u_z.alloc(nn), "alloc");
  CK(c->u_w.alloc(nn), "alloc"); CK(c->u_e1.alloc(nn), "alloc"); CK(c->u_e2.alloc(nn), "alloc");
  CK(c->u_phi.alloc(nn), "alloc"); CK(c->u_jk.alloc(nn), "alloc"); CK(c->u_keep.alloc(nn), "alloc");
  CK(c->u_flag.alloc(nn), "alloc"); CK(c->u_orig.alloc(nn), "alloc"); CK(c->u_e3.alloc(nn), "alloc");
  if (n > 0) {
    auto d2d = [&](void *d, const void *h, size_t bytes) {
      return cudaMemcpyAsync(d, h, bytes, cudaMemcpyDeviceToDevice, st);
    };
    CK(d2d(c->u_x.p, s.x.p, 8 * n), "D2D"); CK(d2d(c->u_y.p, s.y.p, 8 * n), "D2D");
    CK(d2d(c->u_z.p, s.z.p, 8 * n), "D2D"); CK(d2d(c->u_w.p, s.w.p, 8 * n), "D2D");
    CK(d2d(c->u_e1.p, s.e1.p, 8 * n), "D2D"); CK(d2d(c->u_e2.p, s.e2.p, 8 * n), "D2D");
    CK(d2d(c->u_phi.p, s.phi.p, 8 * n), "D2D"); CK(d2d(c->u_jk.p, s.jk.p, 4 * n), "D2D");
    CK(d2d(c->u_keep.p, s.keep.p, n), "D2D"); CK(d2d(c->u_flag.p, s.aflag.p, n), "D2D");
    CK(d2d(c->u_orig.p, s.orig.p, 8 * n), "D2D");
    CK(d2d(c->u_e3.p, s.e3.p, 8 * n), "D2D");
  }
  s.valid = false;
  s.zbuilt = false;
  s.version = ++c->version_ctr;
  return build_cells(c, s, n, k, c->u_orig.p, false);
}

// ---------------------------------------------------------------------------
// sky path (coordinates 0)
// ---------------------------------------------------------------------------

SkyParams sky_params(const cpc_ctx *c) {
  const cpc_params &p = c->p;
  SkyParams sp;
  sp.H = c->H.data();
  sp.dA = c->dA.data();
  sp.n_table = (int64_t)std::min(c->H.size(), c->dA.size());
  sp.dz = p.dz;
  sp.z_max = p.z_max;
  sp.z_sep_max = p.z_sep_max;
  sp.p_min = p.p_min;
  sp.p_max = p.p_max;
  sp.p_size = c->ps;
  sp.r_min = p.bin_r_min;
  sp.r_max = p.bin_r_max;
  sp.r_size = c->rsize;
  sp.lin_bin = p.lin_bin ? 1 : 0;
  sp.n_bins = p.n_bins;
  sp.n_p_bin = p.n_p_bin;
  return sp;
}

// Upload a sky catalogue: per-galaxy windows and angles on the host (C
// library, exactly the reference's values), redshift order from the device
// radix sort, then every array in that order on the device and on the host.
cpc_status sky_upload(cpc_ctx *c, int slot, const cpc_catalog *cat) {
  const cpc_params &p = c->p;
  const int64_t n = cat->n;
  if (n > 0 && (!cat->dc || !cat->da))
    return fail(c, CPC_ERR_INVALID, "sky catalogues need dc and da (distance-table lookups)");
  Slot &s = c->slots[slot];
  s.valid = false;
  s.zbuilt = false;
  s.sky = true;
  s.n = n;
  s.version = ++c->version_ctr;
  const SkyParams sp = sky_params(c);
  std::vector<double> w(n, 1.0), e1(n, 0.0), e2(n, 0.0), phi(n, -10.0);
  std::vector<double> rar(n), decr(n), sd(n), cd(n), win(6 * (size_t)n);
  std::vector<int32_t> jk(n, 0);
  std::vector<uint8_t> keep(n, 0);
  s.has_e = cat->e1 && cat->e2;
  // per row, on the host's cores: the read-path checks (the first failing row
  // in input order is reported), the statistics that size the fixed-point
  // scales, the angles and the lim_calc_sky window with the C library
  struct Part {
    int64_t bad = -1;
    std::string msg;
    double wmax = 0, wmin = 1e300, emax = 0, phimax = 0;
  };
  const int kMaxParts = 64;
  std::vector<Part> parts(kMaxParts);
  host_parallel(n, [&](int64_t b0, int64_t b1, int part) {
    Part &P = parts[part];
    for (int64_t i = b0; i < b1; i++) {
      auto bad = [&](const std::string &m) {
        P.bad = i;
        P.msg = m;
      };
      const double ra = cat->x[i], dec = cat->y[i], z = cat->z[i];
      if (!std::isfinite(ra) || !std::isfinite(dec) || !std::isfinite(z) ||
          !std::isfinite(cat->dc[i]) || !std::isfinite(cat->da[i])) {
        bad("non-finite position or distance at row " + std::to_string(i));
        return;
      }
      if (z < 0 || z > p.z_max) {  // read_dat.cpp:228-234
        bad("redshift outside [0, z_max] at row " + std::to_string(i));
        return;
      }
      if (cat->w) {
        if (!std::isfinite(cat->w[i])) { bad("non-finite weight"); return; }
        w[i] = cat->w[i];
      }
      if (s.has_e) {
        if (!std::isfinite(cat->e1[i]) || !std::isfinite(cat->e2[i])) {
          bad("non-finite ellipticity");
          return;
        }
        e1[i] = cat->e1[i];
        e2[i] = cat->e2[i];
      }
      if (cat->phi) {
        if (!std::isfinite(cat->phi[i])) { bad("non-finite phi"); return; }
        phi[i] = cat->phi[i];
      }
      if (p.do_jk) {
        const int r = cat->jk[i];
        if (r < 0 || r >= p.n_jk) {
          bad("jackknife label out of range at row " + std::to_string(i));
          return;
        }
        jk[i] = r;
      }
      if (cat->jk_prob) keep[i] = cat->jk_prob[i] >= 0.5 ? 1 : 0;
      P.wmax = std::max(P.wmax, std::fabs(w[i]));
      P.wmin = std::min(P.wmin, w[i]);
      P.emax = std::max(P.emax, std::sqrt(e1[i] * e1[i] + e2[i] * e2[i]) * (1.0 + 1e-15));
      P.phimax = std::max(P.phimax, std::fabs(phi[i]));
      sky_angles(ra, dec, &rar[i], &decr[i], &sd[i], &cd[i]);
      double wv[6];
      const int rc = sky_window(sp, ra, dec, z, wv);
      if (rc == 1) {  // lim_calc_ra_dec exits the program here (sky_calcs.cpp:109-113)
        bad("window z_min above z_max at row " + std::to_string(i));
        return;
      }
      if (rc == 2) {
        bad("distance table too short for the window of row " + std::to_string(i));
        return;
      }
      for (int q = 0; q < 6; q++) win[(size_t)q * n + i] = wv[q];
    }
  });
  s.wmax = 0;
  s.wmin = n > 0 ? 1e300 : 1.0;
  s.emax = 0;
  s.phimax = 0;
  for (const Part &P : parts) {  // chunks are in input order: the first bad row
    if (P.bad >= 0) return fail(c, CPC_ERR_RANGE, P.msg);
    s.wmax = std::max(s.wmax, P.wmax);
    s.wmin = std::min(s.wmin, P.wmin);
    s.emax = std::max(s.emax, P.emax);
    s.phimax = std::max(s.phimax, P.phimax);
  }
  // redshift order (stable: ties keep the input order)
  cudaStream_t st = c->st;
  const size_t nn = std::max<int64_t>(n, 1);
  std::vector<uint32_t> perm(n);
  {
    DevBuf<double> oz;
    CK(oz.alloc(nn), "alloc");
    CK(c->d_keys.alloc(nn), "alloc"); CK(c->d_ktmp.alloc(nn), "alloc");
    CK(c->d_vals.alloc(nn), "alloc"); CK(c->d_vtmp.alloc(nn), "alloc");
    CK(c->d_hist.alloc(radix_hist_words(nn)), "alloc");
    CK(c->d_census.alloc(8 * 256), "alloc");
    if (n > 0) {
      CK(cudaMemcpyAsync(oz.p, cat->z, 8 * n, cudaMemcpyHostToDevice, st), "H2D");
      CK(launch_z_keys(n, oz.p, c->d_keys.p, c->d_vals.p, st), "z keys");
      c->launches += 1;
      CK(radix_sort_pairs(n, c->d_keys.p, c->d_vals.p, c->d_ktmp.p, c->d_vtmp.p, c->d_hist.p,
                          c->d_census.p, st, &c->launches), "z sort");
      CK(cudaMemcpyAsync(perm.data(), c->d_vals.p, 4 * n, cudaMemcpyDeviceToHost, st), "D2H");
    }
    CK(cudaStreamSynchronize(st), "sort");
  }
  auto take = [&](const double *src, std::vector<double> &dst) {
    dst.resize(n);
    host_parallel(n, [&](int64_t b0, int64_t b1, int) {
      for (int64_t k = b0; k < b1; k++) dst[k] = src[perm[k]];
    });
  };
  std::vector<double> zs, sds, cds, rars, decrs;
  take(cat->x, s.hs_ra);
  take(cat->y, s.hs_dec);
  take(cat->z, zs);
  take(cat->dc, s.hs_dc);
  take(cat->da, s.hs_da);
  take(w.data(), s.hs_w);
  take(e1.data(), s.hs_e1);
  take(e2.data(), s.hs_e2);
  take(phi.data(), s.hs_phi);
  take(sd.data(), sds);
  take(cd.data(), cds);
  take(rar.data(), rars);
  take(decr.data(), decrs);
  s.hs_jk.resize(n);
  s.hs_keep.resize(n);
  std::vector<int64_t> &orig = s.hs_orig;
  orig.assign(n, 0);
  std::vector<double> wins(6 * (size_t)n);
  std::vector<uint8_t> aflag(n);
  host_parallel(n, [&](int64_t b0, int64_t b1, int) {
    for (int64_t k = b0; k < b1; k++) {
      const uint32_t o = perm[k];
      s.hs_jk[k] = jk[o];
      s.hs_keep[k] = keep[o];
      orig[k] = o;
      for (int q = 0; q < 6; q++) wins[(size_t)q * n + k] = win[(size_t)q * n + o];
      // corels1 scan start: row o + 1 (input order) against z_min of row o
      aflag[k] = (o + 1 < (uint32_t)n && !(cat->z[o + 1] < win[o])) ? kAutoStart0 : 0;
    }
  });
  // outer-row order of the fast sky kernel: (redshift slab, region, redshift),
  // so that a chunk of consecutive rows usually lies in one region
  {
    const int kSlabs = 16;
    const int nreg = p.do_jk ? p.n_jk : 1;
    std::vector<int64_t> start((size_t)kSlabs * nreg + 1, 0);
    auto key = [&](int64_t k) {
      return (int64_t)(k * kSlabs / std::max<int64_t>(n, 1)) * nreg + (p.do_jk ? s.hs_jk[k] : 0);
    };
    for (int64_t k = 0; k < n; k++) start[key(k) + 1]++;
    for (size_t q = 1; q < start.size(); q++) start[q] += start[q - 1];
    s.hs_rorder.assign(n, 0);
    for (int64_t k = 0; k < n; k++) s.hs_rorder[start[key(k)]++] = (int)k;
  }
  auto put = [&](DevBuf<double> &d, const std::vector<double> &h, size_t cnt) -> cudaError_t {
    cudaError_t e = d.alloc(std::max<size_t>(cnt, 1));
    if (e != cudaSuccess || cnt == 0) return e;
    return cudaMemcpyAsync(d.p, h.data(), 8 * cnt, cudaMemcpyHostToDevice, st);
  };
  CK(put(s.x, s.hs_ra, n), "sky upload"); CK(put(s.y, s.hs_dec, n), "sky upload");
  CK(put(s.z, zs, n), "sky upload"); CK(put(s.w, s.hs_w, n), "sky upload");
  CK(put(s.e1, s.hs_e1, n), "sky upload"); CK(put(s.e2, s.hs_e2, n), "sky upload");
  CK(put(s.phi, s.hs_phi, n), "sky upload"); CK(put(s.dc, s.hs_dc, n), "sky upload");
  CK(put(s.da, s.hs_da, n), "sky upload"); CK(put(s.sd, sds, n), "sky upload");
  CK(put(s.cd, cds, n), "sky upload"); CK(put(s.rar, rars, n), "sky upload");
  CK(put(s.decr, decrs, n), "sky upload"); CK(put(s.win, wins, 6 * (size_t)n), "sky upload");
  // float views for the fast kernel: hi parts and the remainders
  std::vector<float4> su(n), sl(n), sw(n), sx(n), ss(n), sh(n);
  std::vector<float2> sph(n);
  auto hi = [](double v) { return (float)v; };
  auto lo = [](double v) { return (float)(v - (double)(float)v); };
  std::vector<double> dcm(kMaxParts, 0.0);
  host_parallel(n, [&](int64_t b0, int64_t b1, int part) {
    for (int64_t k = b0; k < b1; k++) {
      const double ux = cds[k] * std::cos(rars[k]), uy = cds[k] * std::sin(rars[k]), uz = sds[k];
      const double dcv = s.hs_dc[k];
      dcm[part] = std::max(dcm[part], std::fabs(dcv));
      su[k] = make_float4(hi(ux), hi(uy), hi(uz), (float)s.hs_da[k]);
      sl[k] = make_float4(lo(ux), lo(uy), lo(uz), lo(dcv));
      sw[k] = make_float4(hi(s.hs_ra[k]), hi(s.hs_dec[k]), (float)zs[k], hi(dcv));
      sx[k] = make_float4(lo(s.hs_ra[k]), lo(s.hs_dec[k]), (float)decrs[k], (float)s.hs_w[k]);
      // weighted ellipticity and the half Dec angle's cosine and sine as hi +
      // lo parts (the compensated shape terms: cos of the pair's mean Dec is
      // cos(d1/2) cos(d2/2) - sin(d1/2) sin(d2/2))
      const double we1 = s.hs_w[k] * s.hs_e1[k], we2 = s.hs_w[k] * s.hs_e2[k];
      ss[k] = make_float4(hi(we1), hi(we2), lo(we1), lo(we2));
      const double ch = std::cos(decrs[k] / 2.0), sh2 = std::sin(decrs[k] / 2.0);
      sh[k] = make_float4(hi(ch), lo(ch), hi(sh2), lo(sh2));
      sph[k] = make_float2((float)s.hs_phi[k], lo(s.hs_w[k]));
    }
  });
  s.dcmax = 0;
  for (double v : dcm) s.dcmax = std::max(s.dcmax, v);
  DevBuf<float4> *fbufs[6] = {&s.sky_su, &s.sky_sl, &s.sky_sw, &s.sky_sx, &s.sky_ss, &s.sky_sh};
  const std::vector<float4> *fsrc[6] = {&su, &sl, &sw, &sx, &ss, &sh};
  for (int q = 0; q < 6; q++) {
    CK(fbufs[q]->alloc(nn), "alloc");
    if (n > 0)
      CK(cudaMemcpyAsync(fbufs[q]->p, fsrc[q]->data(), sizeof(float4) * n, cudaMemcpyHostToDevice,
                         st), "H2D");
  }
  CK(s.sky_sp.alloc(nn), "alloc");
  if (n > 0)
    CK(cudaMemcpyAsync(s.sky_sp.p, sph.data(), sizeof(float2) * n, cudaMemcpyHostToDevice, st),
       "H2D");
  CK(s.jk.alloc(nn), "alloc"); CK(s.keep.alloc(nn), "alloc"); CK(s.orig.alloc(nn), "alloc");
  CK(s.aflag.alloc(nn), "alloc");
  if (n > 0) {
    CK(cudaMemcpyAsync(s.aflag.p, aflag.data(), n, cudaMemcpyHostToDevice, st), "H2D");
    CK(cudaMemcpyAsync(s.jk.p, s.hs_jk.data(), 4 * n, cudaMemcpyHostToDevice, st), "H2D");
    CK(cudaMemcpyAsync(s.keep.p, s.hs_keep.data(), n, cudaMemcpyHostToDevice, st), "H2D");
    CK(cudaMemcpyAsync(s.orig.p, orig.data(), 8 * n, cudaMemcpyHostToDevice, st), "H2D");
  }
  CK(cudaStreamSynchronize(st), "sky upload");
  s.valid = true;
  return CPC_OK;
}

// One sky corels2 call of a launch (several pair types may share one launch of
// the fast kernel): its job descriptor, device buffers and output.
struct SkyPlan {
  cpc_pair_kind kind;
  int s1, s2;  // slots after the swap rule
  JobRule rule;
  cpc_accum *out;
  JobDev J;
  bool empty;
  size_t cells, n_fix;
};

SkyView sky_view(Slot &s) {
  SkyView v;
  v.d.n = s.n;
  v.d.x = s.x.p; v.d.y = s.y.p; v.d.z = s.z.p; v.d.w = s.w.p;
  v.d.e1 = s.e1.p; v.d.e2 = s.e2.p; v.d.phi = s.phi.p;
  v.d.jk = s.jk.p; v.d.keep = s.keep.p; v.d.orig = s.orig.p; v.d.aflag = s.aflag.p;
  v.dc = s.dc.p; v.da = s.da.p; v.sd = s.sd.p; v.cd = s.cd.p;
  v.rar = s.rar.p; v.decr = s.decr.p; v.win = s.win.p;
  return v;
}

SkyFast sky_fast(Slot &s) {
  return SkyFast{s.sky_su.p, s.sky_sl.p, s.sky_sw.p, s.sky_sx.p, s.sky_ss.p, s.sky_sh.p,
                 s.sky_sp.p};
}

// Plan job k of a sky launch: the corels2 rules, the bands and fixed-point
// scales of the mixed-precision path, zeroed device buffers (set k), the row
// sample as a list of g1 rows.
cpc_status sky_plan(cpc_ctx *c, cpc_pair_kind kind, int slot_g1, int slot_g2, int64_t rs,
                    int64_t ro, cpc_engine engine, cpc_accum *out, int auto_mode, size_t k,
                    SkyPlan &P) {
  if (slot_g1 < 0 || slot_g1 >= kMaxSlots || slot_g2 < 0 || slot_g2 >= kMaxSlots)
    return fail(c, CPC_ERR_INVALID, "slot out of range");
  Slot &A = c->slots[slot_g1], &B = c->slots[slot_g2];
  if (!A.valid || !B.valid || !A.sky || !B.sky) return fail(c, CPC_ERR_STATE, "count before upload");
  if (!out || !out->num || !out->sums) return fail(c, CPC_ERR_INVALID, "null output arrays");
  const cpc_params &p = c->p;
  JobRule rule;
  if ((auto_mode ? job_rule_auto(p, kind, rule) : job_rule(p, kind, A.n, B.n, rule)) != 0)
    return fail(c, CPC_ERR_INVALID, "bad pair kind");
  const int s1 = rule.swapped ? slot_g2 : slot_g1, s2 = rule.swapped ? slot_g1 : slot_g2;
  Slot &g1 = c->slots[s1], &g2 = c->slots[s2];
  P.kind = kind;
  P.s1 = s1;
  P.s2 = s2;
  P.rule = rule;
  P.out = out;
  P.empty = A.n == 0 || B.n == 0;  // corr.cpp:273-277
  P.cells = (size_t)(1 + (p.do_jk ? p.n_jk : 0)) * p.n_bins * p.n_p_bin;
  P.n_fix = P.cells * kNF;
  out->kernel_ms = out->pair_kernel_ms = 0;
  while (c->sky_bufs.size() <= k) c->sky_bufs.emplace_back(new SkyJobBufs());
  SkyJobBufs &Bf = *c->sky_bufs[k];
  cudaStream_t st = c->st;
  CK(Bf.num.alloc(P.cells), "alloc histograms");
  CK(Bf.sums.alloc(P.cells * kNF), "alloc histograms");
  CK(Bf.counters.alloc(4), "alloc counters");
  CK(cudaMemsetAsync(Bf.num.p, 0, sizeof(unsigned long long) * P.cells, st), "memset");
  CK(cudaMemsetAsync(Bf.sums.p, 0, sizeof(double) * P.cells * kNF, st), "memset");
  CK(cudaMemsetAsync(Bf.counters.p, 0, sizeof(unsigned long long) * 4, st), "memset");
  JobDev &J = P.J;
  std::memset(&J, 0, sizeof J);
  J.acc_num = Bf.num.p;
  J.acc_sums = Bf.sums.p;
  J.counters = Bf.counters.p;
  if (P.empty) return CPC_OK;
  J.corel = rule.corel;
  J.gws = rule.gws;
  J.which_corr = p.which_corr;
  J.estimator = p.estimator;
  J.do_jk = p.do_jk ? 1 : 0;
  J.n_jk = p.n_jk;
  J.coordinates = 0;
  J.nrp = p.n_bins;
  J.npi = p.n_p_bin;
  J.lin_bin = p.lin_bin ? 1 : 0;
  J.box_same_keep = 0;  // jk_check_sky (jk.cpp:53-57)
  J.auto_mode = auto_mode;
  J.row_stride = rs > 1 ? rs : 1;
  J.row_offset = ro;
  J.rmin = p.bin_r_min;
  J.rmax = p.bin_r_max;
  J.pmin = p.p_min;
  J.pmax = p.p_max;
  J.ps = c->ps;
  J.rsize = c->rsize;
  for (int q = 0; q <= p.n_bins; q++) J.thr[q] = c->thr_rp[q];
  // float bands of the mixed-precision path.  r_p bin k is certain when
  // [rp - tol, rp + tol] lies inside [A_k, B_k) (the exact thresholds rounded
  // inwards; tol is per pair).  The float Pi differs from the reference's by at
  // most 2^-23 |Pi| + 2^-46 max|D_C|; the Pi bands are shrunk by twice that.
  {
    const int nrp = p.n_bins, npi = p.n_p_bin;
    for (int k = 0; k < nrp; k++) {
      J.A[k] = f_up(c->thr_rp[k]);
      J.B[k] = f_down(c->thr_rp[k + 1]);
    }
    J.rej_lo = f_down(c->thr_rp[0]);
    J.rej_hi = f_up(c->thr_rp[nrp]);
    const double dcm = std::max(g1.dcmax, g2.dcmax);
    auto gp = [&](double v) { return 2.4e-7 * std::fabs(v) + 4e-14 * dcm + 1e-30; };
    for (int k = 0; k < npi; k++) {
      const double lo = c->thr_pi[k], hi = c->thr_pi[k + 1];
      J.PA[k] = f_up(lo + gp(lo));
      J.PB[k] = f_down(hi - gp(hi));
    }
    J.pi_out_lo = f_down(c->thr_pi[0] - gp(c->thr_pi[0]));
    J.pi_out_hi = f_up(c->thr_pi[npi] + gp(c->thr_pi[npi]));
    J.inv_ps_f = (float)(1.0 / c->ps);
    J.tp0 = (float)(-p.p_min / c->ps);
    J.rmin_f = (float)p.bin_r_min;
    J.inv_rsize_f = (float)(1.0 / c->rsize);
    if (!p.lin_bin) {
      J.l2rmin2 = (float)(2.0 * std::log2(p.bin_r_min));
      J.inv_lw = (float)(1.0 / (2.0 * std::log2(p.bin_r_max / p.bin_r_min) / nrp));
    }
  }
  // fixed-point scales of the fast kernel: terms rint(v 2^S_f),
  // |v| 2^S_f <= 2^30 / (1 + 2^-12); the global sums keep a low and a high
  // 64-bit word per bin and field (2^48 terms per bin, checked after the count)
  {
    const double wm = std::max(g1.wmax, 1e-30) * std::max(g2.wmax, 1e-30);
    const double em = std::max({g1.emax, g2.emax, 1e-30});
    const double tm = std::max(M_PI / 2, std::max(g1.phimax, g2.phimax) + M_PI);
    const double tm2 = (rule.corel == COREL_SSA) ? 2 * tm : tm;
    double vb[kNF];
    vb[0] = wm;
    vb[1] = vb[3] = wm * em;
    vb[2] = vb[4] = wm * wm * em * em;
    vb[5] = vb[7] = vb[9] = wm * em * em;
    vb[6] = vb[8] = vb[10] = wm * wm * em * em * em * em;
    vb[11] = tm2;
    vb[12] = 2 * tm * tm;
    for (int f = 0; f < kNF; f++) {
      const double v = std::max(vb[f] * (1.0 + 1.0 / 4096.0), 1e-30);
      int S = 30 - (int)std::ceil(std::log2(v));
      S = std::min(60, std::max(-60, S));
      J.qscale[f] = (float)std::ldexp(1.0, S);
      J.inv_qscale[f] = std::ldexp(1.0, -S);
    }
    J.unit_w = (engine == CPC_ENGINE_FAST && g1.wmax == 1.0 && g1.wmin == 1.0 &&
                g2.wmax == 1.0 && g2.wmin == 1.0) ? 1 : 0;
  }
  CK(Bf.fix.alloc(2 * P.n_fix), "alloc fixed-point sums");  // low words, then high words
  CK(cudaMemsetAsync(Bf.fix.p, 0, sizeof(unsigned long long) * 2 * P.n_fix, st), "memset");
  J.acc_fix = Bf.fix.p;
  J.acc_fixh = Bf.fix.p + P.n_fix;
  J.sky1 = sky_view(g1);
  J.sky2 = sky_view(g2);
  J.sf1 = sky_fast(g1);
  J.sf2 = sky_fast(g2);
  CK(Bf.hq.alloc(kSkyHostQueue), "alloc host queue");
  CK(Bf.hq_n.alloc(1), "alloc");
  CK(cudaMemsetAsync(Bf.hq_n.p, 0, sizeof(unsigned long long), st), "memset");
  J.hq = Bf.hq.p;
  J.hq_n = Bf.hq_n.p;
  // a row sample: the redshift-ordered positions of the g1 rows whose input
  // index i satisfies i % rs == ro (the outer rows corels2 would count); a
  // work shard of the fast engine (cpc_set_shard): the positions k with
  // k % n_shards == shard
  J.row_list = nullptr;
  J.n_rows = g1.n;
  const int W = engine == CPC_ENGINE_FAST ? c->n_shards : 1;
  if (engine == CPC_ENGINE_FAST) {  // the rows in the kernel's order (hs_rorder)
    std::vector<int> rows;
    rows.reserve((size_t)(g1.n / std::max<int64_t>(1, rs) / W + 1));
    for (const int i : g1.hs_rorder)
      if ((W <= 1 || i % W == c->shard) && (rs <= 1 || ((g1.hs_orig[i] - ro) % rs) == 0))
        rows.push_back(i);
    CK(Bf.rows.alloc(std::max<size_t>(rows.size(), 1)), "alloc row sample");
    if (!rows.empty())
      CK(cudaMemcpyAsync(Bf.rows.p, rows.data(), sizeof(int) * rows.size(),
                         cudaMemcpyHostToDevice, st), "H2D");
    CK(cudaStreamSynchronize(st), "sync");  // rows is a host temporary
    J.row_list = Bf.rows.p;
    J.n_rows = (int64_t)rows.size();
  }
  return CPC_OK;
}

// The host edge tier of a finished job: the pairs the GPU queued are binned with
// the C library in the reference's operation order and added to the output.
cpc_status sky_finish(cpc_ctx *c, SkyPlan &P, size_t k, cpc_engine engine, float ms) {
  const cpc_params &p = c->p;
  cpc_accum *out = P.out;
  SkyJobBufs &Bf = *c->sky_bufs[k];
  cpc_status st_;
  if ((st_ = fetch_accum_from(c, Bf.num.p, Bf.sums.p, Bf.counters.p, out, c->st,
                              P.empty ? 0 : P.J.unit_w)) != CPC_OK)
    return st_;
  out->kernel_ms = out->pair_kernel_ms = ms;
  if (P.empty) return CPC_OK;
  if (engine != CPC_ENGINE_FP64) {
    // the low and high fixed-point words hold 2^48 terms of |u| < 2^30 per bin
    for (size_t q = 0; q < P.cells; q++)
      if ((unsigned long long)out->num[q] >= (1ull << 48))
        return fail(c, CPC_ERR_RANGE,
                    "a sky bin holds 2^48 pairs or more: its fixed-point sums may overflow; "
                    "count the term in row samples (row_stride)");
  }
  unsigned long long nq = 0;
  CK(cudaMemcpy(&nq, Bf.hq_n.p, sizeof nq, cudaMemcpyDeviceToHost), "D2H");
  if (nq > kSkyHostQueue)
    return fail(c, CPC_ERR_RANGE, "too many pairs within the trigonometry error bound of a bin edge");
  std::vector<int2> q(nq);
  if (nq) CK(cudaMemcpy(q.data(), Bf.hq.p, sizeof(int2) * nq, cudaMemcpyDeviceToHost), "D2H");
  const JobRule &rule = P.rule;
  Slot &g1 = c->slots[P.s1], &g2 = c->slots[P.s2];
  // host edge tier: the reference's own arithmetic with the C library
  const SkyParams sp = sky_params(c);
  const int nb = p.n_bins, npb = p.n_p_bin;
  const size_t hstride = (size_t)nb * npb;
  for (const int2 &e : q) {
    const int i = e.x, j = e.y;
    int n1, n2;
    if (sky_bin(sp, g1.hs_ra[i], g1.hs_dec[i], g1.hs_dc[i], g1.hs_da[i], g2.hs_ra[j],
                g2.hs_dec[j], g2.hs_dc[j], g2.hs_da[j], &n1, &n2) != 2)
      continue;
    const double wt = g1.hs_w[i] * g2.hs_w[j];
    const double theta = rule.corel == COREL_DD
                             ? 0.0 : sky_orient(g1.hs_ra[i], g1.hs_dec[i], g2.hs_ra[j], g2.hs_dec[j]);
    double f[kNF];
    pair_values(rule.corel, rule.gws, wt, theta, PairGal{g1.hs_e1[i], g1.hs_e2[i], g1.hs_phi[i]},
                PairGal{g2.hs_e1[j], g2.hs_e2[j], g2.hs_phi[j]}, f);
    const size_t cell = (size_t)n1 * npb + n2;
    out->num[cell] += 1;
    for (int k = 0; k < kNF; k++) out->sums[cell * kNF + k] += f[k];
    if (!p.do_jk) continue;
    const int r1 = g1.hs_jk[i], r2 = g2.hs_jk[j];
    int k1 = g1.hs_keep[i], k2 = g2.hs_keep[j];
    if (r1 == r2) k2 = 0;
    const int rr[2] = {r1, r2}, kk[2] = {k1, k2};
    for (int t = 0; t < 2; t++) {
      if (!kk[t]) continue;
      const size_t hc = (size_t)(1 + rr[t]) * hstride + cell;
      out->num[hc] += 1;
      out->sums[hc * kNF] += f[0];
      if (p.which_corr == 0) continue;
      for (int k = 1; k < kNF; k += 2) out->sums[hc * kNF + k] += f[k];
    }
  }
  int64_t nbin = 0;
  for (size_t q2 = 0; q2 < hstride; q2++) nbin += out->num[q2];
  out->n_binned = nbin;
  out->n_rechecked = (int64_t)nq;
  return CPC_OK;
}

// Sky counts (coordinates 0) of one context: the fast engine runs every job in
// one launch of the chunked warp kernel, then the fixed-point blocks are
// converted and each job's host edge tier runs; the FP64 engine runs the plain
// kernel per job.
constexpr int kSkyRowsPerChunk = 64;
cpc_status sky_run(cpc_ctx *c, std::vector<SkyPlan> &plans, cpc_engine engine) {
  const cpc_params &p = c->p;
  cudaStream_t st = c->st;
  cpc_status st_;
  if ((st_ = ensure_scratch(c, 1, plans.size())) != CPC_OK) return st_;
  std::vector<JobDev> jd;
  std::vector<long long> chunk0(1, 0);
  std::vector<size_t> idx;  // plan of each launched job
  for (size_t k = 0; k < plans.size(); k++) {
    if (plans[k].empty) continue;
    jd.push_back(plans[k].J);
    idx.push_back(k);
    const long long nr = plans[k].J.n_rows;
    chunk0.push_back(chunk0.back() + (nr + kSkyRowsPerChunk - 1) / kSkyRowsPerChunk);
  }
  // bound on |sum_gpu - sum_libm|: cos differs by <= 3 ulp (CUDA 2 + C library
  // 1), one more ulp from each of the product and the sum, doubled
  const double esum = 8.0 * std::ldexp(1.0, -52);
  CK(cudaEventRecord(c->e0, st), "event");
  if (!jd.empty()) {
    CK(cudaMemcpyAsync(c->d_jobs.p, jd.data(), sizeof(JobDev) * jd.size(), cudaMemcpyHostToDevice,
                       st), "H2D jobs");
    if (engine == CPC_ENGINE_FP64) {
      for (size_t m = 0; m < jd.size(); m++) {
        Slot &g1 = c->slots[plans[idx[m]].s1], &g2 = c->slots[plans[idx[m]].s2];
        CK(launch_sky_fp64(c->d_jobs.p + m, sky_view(g1), sky_view(g2), jd[m].hq, jd[m].hq_n,
                           kSkyHostQueue, esum, st), "sky kernel");
        c->launches += 1;
      }
    } else {
      CK(c->d_chunk0.alloc(chunk0.size()), "alloc chunk table");
      CK(c->d_chunk_ctr.alloc(1), "alloc");
      CK(cudaMemcpyAsync(c->d_chunk0.p, chunk0.data(), sizeof(long long) * chunk0.size(),
                         cudaMemcpyHostToDevice, st), "H2D");
      CK(cudaMemsetAsync(c->d_chunk_ctr.p, 0, sizeof(unsigned long long), st), "memset");
      const float rp_lo_f = f_down(c->thr_rp[0]), rp_hi_f = f_up(c->thr_rp[p.n_bins]);
      CK(launch_sky_warp(c->d_jobs.p, c->d_chunk0.p, (int)jd.size(), chunk0.back(),
                         kSkyRowsPerChunk, c->d_chunk_ctr.p, kSkyHostQueue, esum, rp_lo_f,
                         rp_hi_f, c->thr_rp[0] <= 0.0 ? 1 : 0, p.n_bins, p.n_p_bin, c->sm_count,
                         c->sky_blocks_per_sm, st), "sky kernel");
      c->launches += 1;
      for (size_t m = 0; m < jd.size(); m++) {
        const SkyPlan &P = plans[idx[m]];
        CK(launch_fix_to_sums((int64_t)P.n_fix, jd[m].acc_fix, jd[m].acc_fixh, jd[m].acc_sums,
                              c->d_jobs.p + m, st), "fixed-point sums");
        c->launches += 1;
      }
    }
  }
  CK(cudaEventRecord(c->e1, st), "event");
  CK(cudaEventSynchronize(c->e1), "sync");
  float ms = 0;
  CK(cudaEventElapsedTime(&ms, c->e0, c->e1), "event time");
  for (size_t k = 0; k < plans.size(); k++)
    if ((st_ = sky_finish(c, plans[k], k, engine, ms)) != CPC_OK) return st_;
  return CPC_OK;
}

// one sky corels2 call
cpc_status sky_count(cpc_ctx *c, cpc_pair_kind kind, int slot_g1, int slot_g2, int64_t rs,
                     int64_t ro, cpc_engine engine, cpc_accum *out, int auto_mode = 0) {
  std::vector<SkyPlan> plans(1);
  cpc_status s = sky_plan(c, kind, slot_g1, slot_g2, rs, ro, engine, out, auto_mode, 0, plans[0]);
  if (s != CPC_OK) return s;
  return sky_run(c, plans, engine);
}

}  // namespace

extern "C" {

const char *cpc_version(void) { return "corr_pc_gb300 0.1 (sm_103a)"; }

const char *cpc_last_error(const cpc_ctx *ctx) {
  if (ctx) return ctx->err.c_str();
  return g_err.c_str();
}

cpc_status cpc_create(cpc_ctx **out, const cpc_params *params) try {
  if (!out || !params) return fail(nullptr, CPC_ERR_INVALID, "null argument");
  *out = nullptr;
  cpc_status s = validate_params(nullptr, *params);
  if (s != CPC_OK) return s;
  std::unique_ptr<cpc_ctx> c(new (std::nothrow) cpc_ctx());
  if (!c) return fail(nullptr, CPC_ERR_NOMEM, "host allocation failed");
  c->p = *params;
  if (params->H_z && params->n_table > 0) {
    c->H.assign(params->H_z, params->H_z + params->n_table);
    c->p.H_z = c->H.data();
  }
  if (params->dA_z && params->n_table > 0) {
    c->dA.assign(params->dA_z, params->dA_z + params->n_table);
    c->p.dA_z = c->dA.data();
  }
  const cpc_params &p = c->p;
  c->ps = (p.p_max - p.p_min) / (p.n_p_bin);
  if (p.lin_bin) c->rsize = (p.bin_r_max - p.bin_r_min) / p.n_bins;
  else c->rsize = (std::log10(p.bin_r_max) - std::log10(p.bin_r_min)) / p.n_bins;
  int rc = rp_thresholds(p.lin_bin, p.n_bins, p.bin_r_min, p.bin_r_max, c->thr_rp);
  if (rc != 0) return fail(nullptr, CPC_ERR_INVALID, "r_p bin thresholds could not be derived (non-monotone bin function)");
  rc = pi_thresholds(p.n_p_bin, p.p_min, p.p_max, c->thr_pi);
  if (rc != 0) return fail(nullptr, CPC_ERR_INVALID, "Pi bin thresholds could not be derived");
  cudaError_t e = cudaGetDevice(&c->device);
  if (e != cudaSuccess) return cuda_fail(nullptr, e, "cudaGetDevice");
  e = cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, c->device);
  if (e != cudaSuccess) return cuda_fail(nullptr, e, "device attribute");
  if (const char *ev = std::getenv("CPC_SKY_BLOCKS_PER_SM"))
    c->sky_blocks_per_sm = std::atoi(ev) >= 3 ? 3 : 2;
  if (const char *ev = std::getenv("CPC_TWIN")) c->twin_on = std::atoi(ev) != 0 ? 1 : 0;
  e = cudaStreamCreateWithFlags(&c->st, cudaStreamNonBlocking);
  if (e != cudaSuccess) return cuda_fail(nullptr, e, "stream");
  e = cudaEventCreate(&c->e0);
  if (e == cudaSuccess) e = cudaEventCreate(&c->e1);
  if (e == cudaSuccess) e = cudaEventCreate(&c->e2);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->e_in, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->e_done, cudaEventDisableTiming);
  if (e != cudaSuccess) return cuda_fail(nullptr, e, "event");
  *out = c.release();
  return CPC_OK;
} catch (...) {
  return host_exception(nullptr);
}

cpc_status cpc_destroy(cpc_ctx *c) try {
  if (!c) return CPC_OK;
  cudaStreamSynchronize(c->st);
  drop_graph(c);
  if (c->e0) cudaEventDestroy(c->e0);
  if (c->e1) cudaEventDestroy(c->e1);
  if (c->e2) cudaEventDestroy(c->e2);
  if (c->e_in) cudaEventDestroy(c->e_in);
  if (c->e_done) cudaEventDestroy(c->e_done);
  if (c->st) cudaStreamDestroy(c->st);
  delete c;
  return CPC_OK;
} catch (...) {
  return host_exception(c);
}

cpc_status cpc_accum_shape(const cpc_ctx *c, int *n_hist, int *n_bins, int *n_p_bin) {
  if (!c) return fail(nullptr, CPC_ERR_INVALID, "null context");
  if (n_hist) *n_hist = 1 + (c->p.do_jk ? c->p.n_jk : 0);
  if (n_bins) *n_bins = c->p.n_bins;
  if (n_p_bin) *n_p_bin = c->p.n_p_bin;
  return CPC_OK;
}

// a count enqueued by cpc_count_async must be collected first
static bool busy(cpc_ctx *c) {
  if (!c || !c->pending) return false;
  fail(c, CPC_ERR_STATE, "a count is pending: call cpc_count_finish first");
  return true;
}

cpc_status cpc_set_tuning(cpc_ctx *c, int cells_per_rmax, int pi_window, int tile) {
  if (!c) return fail(nullptr, CPC_ERR_INVALID, "null context");
  if (busy(c)) return CPC_ERR_STATE;
  if (cells_per_rmax < 0 || cells_per_rmax > kMaxCellsPerRmax || pi_window < 0 ||
      (tile != 0 && tile != kTileThreads))
    return fail(c, CPC_ERR_INVALID, "tuning values out of range");
  c->tune_k = cells_per_rmax;
  c->tune_wpi = pi_window;
  c->tune_tile = tile;
  return CPC_OK;
}

cpc_status cpc_upload(cpc_ctx *c, int slot, const cpc_catalog *cat) try {
  if (!c || !cat) return fail(c, CPC_ERR_INVALID, "null argument");
  if (busy(c)) return CPC_ERR_STATE;
  if (slot < 0 || slot >= kMaxSlots) return fail(c, CPC_ERR_INVALID, "slot out of range");
  const cpc_params &p = c->p;
  const int64_t n = cat->n;
  if (n < 0 || n >= 2147483647LL) return fail(c, CPC_ERR_INVALID, "catalogue size out of range");
  if (n > 0 && (!cat->x || !cat->y || !cat->z)) return fail(c, CPC_ERR_INVALID, "null positions");
  if (p.do_jk && n > 0 && !cat->jk) return fail(c, CPC_ERR_INVALID, "jackknife labels required (do_jk=1)");
  if (p.coordinates == 0) return sky_upload(c, slot, cat);
  Slot &s = c->slots[slot];
  s.sky = false;
  s.valid = false;
  s.zbuilt = false;
  s.n = n;
  s.version = ++c->version_ctr;
  const double L = p.periodic_box_size;
  s.has_e = cat->e1 || cat->e2 || cat->e3;
  cudaStream_t st = c->st;
  // the caller's arrays, in input order, in context buffers reused by every
  // upload; absent optional arrays get the reference's defaults on the device
  // (w 1, e 0, phi -10, region 0)
  const size_t nn = std::max<int64_t>(n, 1);
  DevBuf<double> &ox = c->u_x, &oy = c->u_y, &oz = c->u_z, &ow = c->u_w, &oe1 = c->u_e1,
                 &oe2 = c->u_e2, &ophi = c->u_phi, &oprob = c->u_prob, &oe3 = c->u_e3;
  DevBuf<int32_t> &ojk = c->u_jk;
  DevBuf<uint8_t> &okeep = c->u_keep, &oflag = c->u_flag;
  CK(oe3.alloc(nn), "alloc");
  CK(ox.alloc(nn), "alloc"); CK(oy.alloc(nn), "alloc"); CK(oz.alloc(nn), "alloc");
  CK(ow.alloc(nn), "alloc"); CK(oe1.alloc(nn), "alloc"); CK(oe2.alloc(nn), "alloc");
  CK(ophi.alloc(nn), "alloc"); CK(oprob.alloc(nn), "alloc"); CK(ojk.alloc(nn), "alloc");
  CK(okeep.alloc(nn), "alloc"); CK(oflag.alloc(nn), "alloc");
  CK(c->d_ustats.alloc(1), "alloc");
  UploadStats init;
  for (int q = 0; q < 4; q++) init.bad_row[q] = ~0ull;
  init.cmax_bits = init.wmax_bits = init.emax_bits = init.phimax_bits = 0;
  init.wmin_key = ~0ull;
  init.not_f32 = 0;
  c->h_ustats = init;
  if (n > 0) {
    auto h2d = [&](void *d, const void *h, size_t bytes) {
      return cudaMemcpyAsync(d, h, bytes, cudaMemcpyHostToDevice, st);
    };
    CK(h2d(ox.p, cat->x, 8 * n), "H2D");
    CK(h2d(oy.p, cat->y, 8 * n), "H2D");
    CK(h2d(oz.p, cat->z, 8 * n), "H2D");
    CK(cat->w ? h2d(ow.p, cat->w, 8 * n) : launch_fill_f64(n, 1.0, ow.p, st), "weights");
    // e1 alone carries kappa (which_corr 3, 4)
    CK(cat->e1 ? h2d(oe1.p, cat->e1, 8 * n) : cudaMemsetAsync(oe1.p, 0, 8 * n, st), "e1");
    CK(cat->e2 ? h2d(oe2.p, cat->e2, 8 * n) : cudaMemsetAsync(oe2.p, 0, 8 * n, st), "e2");
    CK(cat->phi ? h2d(ophi.p, cat->phi, 8 * n) : launch_fill_f64(n, -10.0, ophi.p, st), "phi");
    CK(cat->e3 ? h2d(oe3.p, cat->e3, 8 * n) : cudaMemsetAsync(oe3.p, 0, 8 * n, st), "e3");
    CK(p.do_jk ? h2d(ojk.p, cat->jk, 4 * n) : cudaMemsetAsync(ojk.p, 0, 4 * n, st), "labels");
    if (cat->jk_prob) CK(h2d(oprob.p, cat->jk_prob, 8 * n), "H2D");
    CK(h2d(c->d_ustats.p, &c->h_ustats, sizeof(UploadStats)), "H2D");
    PrepIn pin;
    pin.n = n;
    pin.x = ox.p; pin.y = oy.p; pin.z = oz.p; pin.w = cat->w ? ow.p : nullptr;
    pin.e1 = s.has_e ? oe1.p : nullptr; pin.e2 = s.has_e ? oe2.p : nullptr;
    pin.phi = cat->phi ? ophi.p : nullptr; pin.jk_prob = cat->jk_prob ? oprob.p : nullptr;
    pin.jk = p.do_jk ? ojk.p : nullptr;
    pin.e3 = cat->e3 ? oe3.p : nullptr;
    pin.L = L;
    pin.wz_lo = wz_lo(p);
    pin.n_jk = p.n_jk;
    CK(launch_prep_catalog(pin, okeep.p, oflag.p, c->d_ustats.p, st), "catalogue checks");
    c->launches += 1;
    CK(cudaMemcpyAsync(&c->h_ustats, c->d_ustats.p, sizeof(UploadStats), cudaMemcpyDeviceToHost,
                       st), "D2H");
  }
  return build_cells(c, s, n, c->tune_k > 0 ? c->tune_k : 2, nullptr, true);
} catch (...) {
  return host_exception(c);
}

cpc_status cpc_count(cpc_ctx *c, cpc_pair_kind kind, int slot_g1, int slot_g2, cpc_engine engine,
                     int64_t row_stride, int64_t row_offset, cpc_accum *out) try {
  if (!c) return fail(nullptr, CPC_ERR_INVALID, "null context");
  if (busy(c)) return CPC_ERR_STATE;
  if (engine != CPC_ENGINE_FAST && engine != CPC_ENGINE_FP64 && engine != CPC_ENGINE_CELL_FP64)
    return fail(c, CPC_ERR_INVALID, "unknown engine");
  if (kind == CPC_PAIR_SS)
    return fail(c, CPC_ERR_INVALID, "CPC_PAIR_SS pairs one catalogue: use cpc_count_auto");
  // sky: FP32-prefiltered warp kernel (fast) or plain FP64 kernel, both with
  // the FP64 path and the host edge tier for the pairs that can bin
  if (c->p.coordinates == 0) {
    if (engine == CPC_ENGINE_CELL_FP64)
      return fail(c, CPC_ERR_INVALID, "the cell-list FP64 engine counts box pairs only");
    return sky_count(c, kind, slot_g1, slot_g2, row_stride, row_offset, engine, out);
  }
  std::vector<JobPlan> jobs(1);
  cpc_status s = plan_job(c, kind, slot_g1, slot_g2, row_stride, row_offset, out, jobs[0], 0,
                          engine == CPC_ENGINE_FAST);
  if (s != CPC_OK) return s;
  if (engine == CPC_ENGINE_FP64) return run_plain(jobs[0]);
  jobs[0].jd.all_exact = engine == CPC_ENGINE_CELL_FP64 ? 1 : 0;
  return run_fast(jobs);
} catch (...) {
  return host_exception(c);
}

cpc_status cpc_count_async(cpc_ctx *c, cpc_pair_kind kind, int slot_g1, int slot_g2,
                           cpc_engine engine, int64_t row_stride, int64_t row_offset,
                           void *stream) try {
  if (!c) return fail(nullptr, CPC_ERR_INVALID, "null context");
  if (busy(c)) return CPC_ERR_STATE;
  if (engine != CPC_ENGINE_FAST && engine != CPC_ENGINE_FP64)
    return fail(c, CPC_ERR_INVALID, "unknown engine");
  if (kind == CPC_PAIR_SS)
    return fail(c, CPC_ERR_INVALID, "CPC_PAIR_SS pairs one catalogue: use cpc_count_auto");
  if (c->p.coordinates == 0)
    return fail(c, CPC_ERR_INVALID,
                "sky counts finish on the host (edge tier): use cpc_count for coordinates 0");
  cudaStream_t user = reinterpret_cast<cudaStream_t>(stream);
  std::vector<JobPlan> jobs(1);
  cpc_accum placeholder{};  // plan_job checks the output arrays; the real ones come at finish
  int64_t dummy_num = 0;
  double dummy_sums = 0;
  placeholder.num = &dummy_num;
  placeholder.sums = &dummy_sums;
  cpc_status s = plan_job(c, kind, slot_g1, slot_g2, row_stride, row_offset, &placeholder, jobs[0]);
  if (s != CPC_OK) return s;
  jobs[0].out = nullptr;
  // the count follows the caller's earlier work on `stream`
  CK(cudaEventRecord(c->e_in, user), "event");
  CK(cudaStreamWaitEvent(c->st, c->e_in, 0), "stream wait");
  s = engine == CPC_ENGINE_FP64 ? enqueue_plain(jobs[0]) : enqueue_fast(jobs);
  if (s != CPC_OK) return s;
  // and the caller's later work on `stream` follows the count
  CK(cudaEventRecord(c->e_done, c->st), "event");
  CK(cudaStreamWaitEvent(user, c->e_done, 0), "stream wait");
  c->pending = engine == CPC_ENGINE_FP64 ? 2 : 1;
  c->pending_jobs = std::move(jobs);
  return CPC_OK;
} catch (...) {
  return host_exception(c);
}

cpc_status cpc_count_finish(cpc_ctx *c, cpc_accum *out) try {
  if (!c) return fail(nullptr, CPC_ERR_INVALID, "null context");
  if (!c->pending) return fail(c, CPC_ERR_STATE, "no count is pending");
  if (!out || !out->num || !out->sums) return fail(c, CPC_ERR_INVALID, "null output arrays");
  std::vector<JobPlan> jobs = std::move(c->pending_jobs);
  const int mode = c->pending;
  c->pending = 0;
  c->pending_jobs.clear();
  jobs[0].out = out;
  return mode == 2 ? finish_plain(jobs[0]) : finish_fast(jobs, 0);
} catch (...) {
  return host_exception(c);
}

cpc_status cpc_count_auto(cpc_ctx *c, cpc_pair_kind kind, int slot, cpc_engine engine,
                          int64_t row_stride, int64_t row_offset, cpc_accum *out) try {
  if (!c) return fail(nullptr, CPC_ERR_INVALID, "null context");
  if (busy(c)) return CPC_ERR_STATE;
  if (engine != CPC_ENGINE_FAST && engine != CPC_ENGINE_FP64)
    return fail(c, CPC_ERR_INVALID, "unknown engine");
  if (kind != CPC_PAIR_SS && kind != CPC_PAIR_RSRS)
    return fail(c, CPC_ERR_INVALID, "auto pairs: kind must be CPC_PAIR_SS or CPC_PAIR_RSRS");
  if (c->p.data_sorted != 0 && c->p.data_sorted != 1)
    return fail(c, CPC_ERR_INVALID, "auto pairs: data_sorted must be 0 or 1");
  const int mode = c->p.data_sorted == 1 ? 2 : 1;
  if (c->p.coordinates == 0)
    return sky_count(c, kind, slot, slot, row_stride, row_offset, engine, out, mode);
  std::vector<JobPlan> jobs(1);
  cpc_status s = plan_job(c, kind, slot, slot, row_stride, row_offset, out, jobs[0], mode);
  if (s != CPC_OK) return s;
  if (engine == CPC_ENGINE_FP64) return run_plain(jobs[0]);
  return run_fast(jobs);
} catch (...) {
  return host_exception(c);
}

// Pi windows the autotuner tries: for 4, 3 and 2 blocks per SM the largest
// window whose histograms fit, and three quarters of it (more, narrower units).
// With coordinates 7 the mu window is automatic (every mu bin when they fit):
// only the cell width is tuned.
std::vector<int> tune_windows(const cpc_params &p, int corel, int unit_w, int twin) {
  std::vector<int> ws;
  if (p.coordinates == 7) return {0};
  const int wmin = twin ? 5 : 8;
  const int jk = p.do_jk ? 1 : 0, nrp = p.n_bins, npi = p.n_p_bin;
  const size_t static_b = fast_static_smem_bytes(twin);
  for (int b = 4; b >= 2; b--) {
    const size_t budget = (size_t)(228 * 1024) / b - static_b - 1024;
    int w = npi;
    while (w > 1 && fast_smem_bytes(corel, jk, nrp, w, 0, unit_w, twin) > budget) w--;
    if (fast_smem_bytes(corel, jk, nrp, w, 0, unit_w, twin) > budget) continue;
    for (int cand : {w, (3 * w + 3) / 4}) {
      if (cand < std::min(npi, wmin)) continue;
      if (std::find(ws.begin(), ws.end(), cand) == ws.end()) ws.push_back(cand);
    }
    if (w == npi) break;  // every Pi bin fits: fewer blocks gain nothing
  }
  if (ws.empty()) ws.push_back(0);
  return ws;
}

cpc_status cpc_autotune(cpc_ctx *c, cpc_pair_kind kind, int slot_g1, int slot_g2,
                        int64_t sample_stride, int *cells_per_rmax, int *pi_window) try {
  if (!c) return fail(nullptr, CPC_ERR_INVALID, "null context");
  if (busy(c)) return CPC_ERR_STATE;
  const cpc_params &p = c->p;
  if (slot_g1 < 0 || slot_g1 >= kMaxSlots || slot_g2 < 0 || slot_g2 >= kMaxSlots)
    return fail(c, CPC_ERR_INVALID, "slot out of range");
  if (!c->slots[slot_g1].valid || !c->slots[slot_g2].valid)
    return fail(c, CPC_ERR_STATE, "autotune before upload");
  if (c->slots[slot_g1].sky) {  // the sky kernel has no cell or window knobs
    if (cells_per_rmax) *cells_per_rmax = 0;
    if (pi_window) *pi_window = 0;
    return CPC_OK;
  }
  int nh, nb, npb;
  cpc_accum_shape(c, &nh, &nb, &npb);
  std::vector<int64_t> num((size_t)nh * nb * npb);
  std::vector<double> sums(num.size() * kNF);
  cpc_accum acc{};
  acc.num = num.data();
  acc.sums = sums.data();
  const int ks[5] = {2, 3, 4, 5, 6};
  std::vector<int> ws;
  {
    JobRule rule;
    if (job_rule(p, kind, c->slots[slot_g1].n, c->slots[slot_g2].n, rule) != 0)
      return fail(c, CPC_ERR_INVALID, "bad pair kind");
    const int s1 = rule.swapped ? slot_g2 : slot_g1, s2 = rule.swapped ? slot_g1 : slot_g2;
    ws = tune_windows(p, rule.corel, unit_weights(c->slots[slot_g1], c->slots[slot_g2]),
                      twin_job(c, rule, s1, s2, 1, 0, 0) ? 1 : 0);
  }
  // the trials count every sample_stride-th work unit (a unit shard: whole
  // tiles, so each trial's per-unit costs are those of the full count)
  const int64_t stride = std::max<int64_t>(1, sample_stride);
  ShardOverride so(c, 0, (int)std::min<int64_t>(stride, 1 << 30));
  double best = INFINITY;
  int bk = c->slots[slot_g1].kcells, bw = c->tune_wpi;
  for (int k : ks) {
    cpc_status s;
    if (c->slots[slot_g1].kcells != k && (s = rebuild_cells(c, c->slots[slot_g1], k)) != CPC_OK)
      return s;
    if (slot_g2 != slot_g1 && c->slots[slot_g2].kcells != k &&
        (s = rebuild_cells(c, c->slots[slot_g2], k)) != CPC_OK)
      return s;
    for (int w : ws) {
      c->tune_wpi = w;
      // first run builds the work units, the next two are timed (the faster counts)
      if (cpc_count(c, kind, slot_g1, slot_g2, CPC_ENGINE_FAST, 1, 0, &acc) != CPC_OK) continue;
      double t = INFINITY;
      for (int rep = 0; rep < 2; rep++) {
        if (cpc_count(c, kind, slot_g1, slot_g2, CPC_ENGINE_FAST, 1, 0, &acc) != CPC_OK) break;
        t = std::min(t, (double)acc.pair_kernel_ms);
      }
      if (t < best) {
        best = t;
        bk = k;
        bw = w;
      }
    }
  }
  so.restore();
  // keep the best: every box slot on the chosen grid (counts pair slots of one grid)
  c->tune_k = bk;
  c->tune_wpi = bw;
  for (int q = 0; q < kMaxSlots; q++) {
    Slot &sl = c->slots[q];
    if (sl.valid && !sl.sky && sl.kcells != bk) {
      const cpc_status s = rebuild_cells(c, sl, bk);
      if (s != CPC_OK) return s;
    }
  }
  if (cells_per_rmax) *cells_per_rmax = bk;
  if (pi_window) *pi_window = bw;
  return CPC_OK;
} catch (...) {
  return host_exception(c);
}

// The batch of cpc_count_batch on every row_stride-th outer row of each job.
cpc_status count_batch_rows(int n_jobs, cpc_ctx *const *ctxs, const cpc_pair_kind *kinds,
                            const int *slots_g1, const int *slots_g2, cpc_accum *outs,
                            int64_t row_stride) {
  std::vector<JobPlan> jobs(n_jobs);
  for (int k = 0; k < n_jobs; k++) {
    if (ctxs[k]->device != ctxs[0]->device) return fail(ctxs[k], CPC_ERR_INVALID, "batch spans devices");
    cpc_status s = plan_job(ctxs[k], kinds[k], slots_g1[k], slots_g2[k], row_stride, 0, &outs[k],
                            jobs[k]);
    if (s != CPC_OK) return s;
  }
  return run_fast(jobs);
}

cpc_status cpc_autotune_batch(int n_jobs, cpc_ctx *const *ctxs, const cpc_pair_kind *kinds,
                              const int *slots_g1, const int *slots_g2, int64_t sample_stride,
                              int *cells_per_rmax, int *pi_window) try {
  if (n_jobs <= 0 || !ctxs || !kinds || !slots_g1 || !slots_g2)
    return fail(nullptr, CPC_ERR_INVALID, "bad batch arguments");
  for (int k = 0; k < n_jobs; k++) {
    if (!ctxs[k]) return fail(nullptr, CPC_ERR_INVALID, "null context in batch");
    if (busy(ctxs[k])) return CPC_ERR_STATE;
    const cpc_ctx *c = ctxs[k];
    if (slots_g1[k] < 0 || slots_g1[k] >= kMaxSlots || slots_g2[k] < 0 || slots_g2[k] >= kMaxSlots)
      return fail(ctxs[k], CPC_ERR_INVALID, "slot out of range");
    if (!c->slots[slots_g1[k]].valid || !c->slots[slots_g2[k]].valid)
      return fail(ctxs[k], CPC_ERR_STATE, "autotune before upload");
    if (c->slots[slots_g1[k]].sky || c->p.coordinates != ctxs[0]->p.coordinates ||
        c->p.n_bins != ctxs[0]->p.n_bins || c->p.n_p_bin != ctxs[0]->p.n_p_bin ||
        c->p.which_corr != ctxs[0]->p.which_corr)
      return fail(ctxs[k], CPC_ERR_INVALID,
                  "batch autotuning needs box jobs with one binning and which_corr");
  }
  JobRule rule;
  {
    const cpc_ctx *c0 = ctxs[0];
    if (job_rule(c0->p, kinds[0], c0->slots[slots_g1[0]].n, c0->slots[slots_g2[0]].n, rule) != 0)
      return fail(ctxs[0], CPC_ERR_INVALID, "bad pair kind");
  }
  int unit_w = 1, twin = 1;
  for (int k = 0; k < n_jobs; k++) {
    cpc_ctx *c = ctxs[k];
    unit_w &= unit_weights(c->slots[slots_g1[k]], c->slots[slots_g2[k]]);
    JobRule rk;
    if (job_rule(c->p, kinds[k], c->slots[slots_g1[k]].n, c->slots[slots_g2[k]].n, rk) != 0)
      return fail(c, CPC_ERR_INVALID, "bad pair kind");
    const int s1 = rk.swapped ? slots_g2[k] : slots_g1[k], s2 = rk.swapped ? slots_g1[k] : slots_g2[k];
    twin &= twin_job(c, rk, s1, s2, 1, 0, 0) ? 1 : 0;
  }
  const std::vector<int> ws = tune_windows(ctxs[0]->p, rule.corel, unit_w, twin);
  std::vector<std::vector<int64_t>> nums(n_jobs);
  std::vector<std::vector<double>> sums(n_jobs);
  std::vector<cpc_accum> accs(n_jobs);
  for (int k = 0; k < n_jobs; k++) {
    int nh, nb, npb;
    cpc_accum_shape(ctxs[k], &nh, &nb, &npb);
    nums[k].resize((size_t)nh * nb * npb);
    sums[k].resize(nums[k].size() * kNF);
    accs[k] = cpc_accum{};
    accs[k].num = nums[k].data();
    accs[k].sums = sums[k].data();
  }
  // the trials count every sample_stride-th work unit of each context (unit
  // shards: whole tiles, so each trial's per-unit costs are those of the full
  // count)
  const int64_t stride = std::max<int64_t>(1, sample_stride);
  std::vector<std::unique_ptr<ShardOverride>> sos;
  for (int k = 0; k < n_jobs; k++) {
    bool seen = false;
    for (const auto &so : sos) seen = seen || so->c == ctxs[k];
    if (!seen)
      sos.emplace_back(new ShardOverride(ctxs[k], 0, (int)std::min<int64_t>(stride, 1 << 30)));
  }
  // every slot a job reads, on cells r_max / kc
  auto regrid = [&](int kc) -> cpc_status {
    for (int k = 0; k < n_jobs; k++)
      for (int sl : {slots_g1[k], slots_g2[k]}) {
        Slot &s = ctxs[k]->slots[sl];
        if (s.kcells != kc) {
          const cpc_status st = rebuild_cells(ctxs[k], s, kc);
          if (st != CPC_OK) return st;
        }
      }
    return CPC_OK;
  };
  double best = INFINITY;
  int bk = ctxs[0]->slots[slots_g1[0]].kcells, bw = ctxs[0]->tune_wpi;
  for (int kc : {2, 3, 4, 5, 6}) {
    cpc_status s = regrid(kc);
    if (s != CPC_OK) return s;
    for (int w : ws) {
      for (int k = 0; k < n_jobs; k++) ctxs[k]->tune_wpi = w;
      // first run builds the work units, the next two are timed (the faster counts)
      if (count_batch_rows(n_jobs, ctxs, kinds, slots_g1, slots_g2, accs.data(), 1) != CPC_OK)
        continue;
      double t = INFINITY;
      for (int rep = 0; rep < 2; rep++) {
        if (count_batch_rows(n_jobs, ctxs, kinds, slots_g1, slots_g2, accs.data(), 1) != CPC_OK)
          break;
        t = std::min(t, (double)accs[0].pair_kernel_ms);
      }
      if (t < best) {
        best = t;
        bk = kc;
        bw = w;
      }
    }
  }
  sos.clear();  // the contexts' own shards again
  for (int k = 0; k < n_jobs; k++) {
    ctxs[k]->tune_k = bk;
    ctxs[k]->tune_wpi = bw;
  }
  const cpc_status s = regrid(bk);
  if (s != CPC_OK) return s;
  if (cells_per_rmax) *cells_per_rmax = bk;
  if (pi_window) *pi_window = bw;
  return CPC_OK;
} catch (...) {
  return host_exception(n_jobs > 0 && ctxs ? ctxs[0] : nullptr);
}

cpc_status cpc_count_batch(int n_jobs, cpc_ctx *const *ctxs, const cpc_pair_kind *kinds,
                           const int *slots_g1, const int *slots_g2, cpc_accum *outs) try {
  if (n_jobs <= 0 || !ctxs || !kinds || !slots_g1 || !slots_g2 || !outs)
    return fail(nullptr, CPC_ERR_INVALID, "bad batch arguments");
  for (int k = 0; k < n_jobs; k++)
    if (busy(ctxs[k])) return CPC_ERR_STATE;
  for (int k = 0; k < n_jobs; k++)
    if (!ctxs[k]) return fail(nullptr, CPC_ERR_INVALID, "null context in batch");
  for (int k = 0; k < n_jobs; k++)
    if (ctxs[k]->p.coordinates == 0) {
      bool one_ctx = true;
      for (int m = 0; m < n_jobs; m++) one_ctx = one_ctx && ctxs[m] == ctxs[0];
      if (one_ctx) {  // the pair types of one sky run: one launch of the fast kernel
        cpc_ctx *c = ctxs[0];
        std::vector<SkyPlan> plans(n_jobs);
        for (int m = 0; m < n_jobs; m++) {
          const cpc_status s = sky_plan(c, kinds[m], slots_g1[m], slots_g2[m], 1, 0,
                                        CPC_ENGINE_FAST, &outs[m], 0, (size_t)m, plans[m]);
          if (s != CPC_OK) return s;
        }
        return sky_run(c, plans, CPC_ENGINE_FAST);
      }
      for (int m = 0; m < n_jobs; m++) {  // sky jobs of several contexts: one launch each
        const cpc_status s = cpc_count(ctxs[m], kinds[m], slots_g1[m], slots_g2[m],
                                       CPC_ENGINE_FAST, 1, 0, &outs[m]);
        if (s != CPC_OK) return s;
      }
      return CPC_OK;
    }
  return count_batch_rows(n_jobs, ctxs, kinds, slots_g1, slots_g2, outs, 1);
} catch (...) {
  return host_exception(n_jobs > 0 && ctxs ? ctxs[0] : nullptr);
}

cpc_status cpc_host_rand_uniform(uint32_t seed, int64_t skip, int64_t n, double *out) try {
  if (n < 0 || skip < 0 || (n > 0 && !out)) return fail(nullptr, CPC_ERR_INVALID, "bad arguments");
  std::vector<int32_t> r(n);
  glibc_rand_stream(seed, skip, n, r.data());
  for (int64_t i = 0; i < n; i++) out[i] = r[i] / (2147483647 + 1.);
  return CPC_OK;
} catch (...) {
  return host_exception(nullptr);
}

cpc_status cpc_host_elip_angle(int64_t n, const double *e1, const double *e2, double *phi) try {
  if (n < 0 || (n > 0 && (!e1 || !e2 || !phi))) return fail(nullptr, CPC_ERR_INVALID, "bad arguments");
  for (int64_t i = 0; i < n; i++) phi[i] = elip_angle(e1[i], e2[i]);
  return CPC_OK;
} catch (...) {
  return host_exception(nullptr);
}

cpc_status cpc_host_rp_thresholds(const cpc_params *p, double *thr) try {
  if (!p || !thr) return fail(nullptr, CPC_ERR_INVALID, "null argument");
  if (p->n_bins <= 0 || p->n_bins > kMaxRp) return fail(nullptr, CPC_ERR_INVALID, "n_bins out of range");
  const int rc = rp_thresholds(p->lin_bin, p->n_bins, p->bin_r_min, p->bin_r_max, thr);
  return rc == 0 ? CPC_OK : fail(nullptr, CPC_ERR_INVALID, "threshold derivation failed");
} catch (...) {
  return host_exception(nullptr);
}

cpc_status cpc_set_shard(cpc_ctx *c, int shard, int n_shards) {
  if (!c) return fail(nullptr, CPC_ERR_INVALID, "null context");
  if (busy(c)) return CPC_ERR_STATE;
  if (n_shards < 1 || shard < 0 || shard >= n_shards)
    return fail(c, CPC_ERR_INVALID, "shard must satisfy 0 <= shard < n_shards");
  c->shard = shard;
  c->n_shards = n_shards;
  return CPC_OK;
}

cpc_status cpc_set_graph_replay(cpc_ctx *c, int enable) try {
  if (!c) return fail(nullptr, CPC_ERR_INVALID, "null context");
  if (busy(c)) return CPC_ERR_STATE;
  cudaStreamSynchronize(c->st);
  drop_graph(c);
  c->graph_on = enable ? 1 : 0;
  return CPC_OK;
} catch (...) {
  return host_exception(c);
}

cpc_status cpc_graph_stats(const cpc_ctx *c, int64_t *captures, int64_t *replays) {
  if (!c) return fail(nullptr, CPC_ERR_INVALID, "null context");
  if (captures) *captures = c->graph_captures;
  if (replays) *replays = c->graph_replays;
  return CPC_OK;
}

cpc_status cpc_set_twin(cpc_ctx *c, int enable) try {
  if (!c) return fail(nullptr, CPC_ERR_INVALID, "null context");
  if (busy(c)) return CPC_ERR_STATE;
  c->twin_on = enable ? 1 : 0;
  return CPC_OK;
} catch (...) {
  return host_exception(c);
}

cpc_status cpc_last_twin(const cpc_ctx *c, int *twin) {
  if (!c || !twin) return fail(nullptr, CPC_ERR_INVALID, "null argument");
  *twin = c->last_twin;
  return CPC_OK;
}

cpc_status cpc_launch_count(const cpc_ctx *c, int64_t *launches) {
  if (!c || !launches) return fail(nullptr, CPC_ERR_INVALID, "null argument");
  *launches = c->launches;
  return CPC_OK;
}

cpc_status cpc_host_pi_thresholds(const cpc_params *p, double *thr) try {
  if (!p || !thr) return fail(nullptr, CPC_ERR_INVALID, "null argument");
  if (p->n_p_bin <= 0 || p->n_p_bin > kMaxPi) return fail(nullptr, CPC_ERR_INVALID, "n_p_bin out of range");
  const int rc = pi_thresholds(p->n_p_bin, p->p_min, p->p_max, thr);
  return rc == 0 ? CPC_OK : fail(nullptr, CPC_ERR_INVALID, "threshold derivation failed");
} catch (...) {
  return host_exception(nullptr);
}

}  // extern "C"
