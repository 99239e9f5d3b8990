// pair_noalloc.cu -- cpc_count_fp64_noalloc: the plain FP64 pair count for
// callers that cannot allocate GPU memory (for example code running inside a
// host framework that owns every device allocation, or a memory pool that
// forbids cudaMalloc after start-up).  The caller passes device-resident
// inputs and device output buffers; the kernel's own scratch (the job
// descriptor with the exact bin thresholds, the pair counters and an
// input-order flag) lives in one file-scope __device__ array below, so this
// entry point calls no cudaMalloc, cudaFree or allocating library routine.
//
// The array is kNoallocScratchBytes (16 KiB) per device and stays resident on
// every device that loads the library until the process exits.  It is shared
// by every call on that device and keeps the last call's contents, so each
// call rewrites the descriptor and clears the counters before it counts; two
// calls whose work overlaps on the GPU (different streams, or host threads
// racing) would overwrite each other's scratch and must be serialised by the
// caller.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "../../include/corrpc.h"
#include "cpc_device.cuh"
#include "host_helpers.h"
#include "pair_values.h"
#include "param_check.h"

namespace cpc {
namespace {

constexpr size_t kNoallocScratchBytes = 16384;
constexpr size_t kCountersOffset = 4096;  // after the JobDev
static_assert(sizeof(JobDev) <= kCountersOffset, "job descriptor must fit the scratch");
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocScratchBytes];

std::mutex g_noalloc_mu;
unsigned char *g_scratch_ptr[kMaxDevices] = {nullptr};

struct NCat {
  int64_t n;
  const double *x, *y, *z, *w, *e1, *e2, *phi, *jk_prob;
  const int32_t *jk;
};

__device__ __forceinline__ double nc_w(const NCat &c, int64_t i) { return c.w ? c.w[i] : 1.0; }
__device__ __forceinline__ double nc_e1(const NCat &c, int64_t i) { return c.e1 ? c.e1[i] : 0.0; }
__device__ __forceinline__ double nc_e2(const NCat &c, int64_t i) { return c.e2 ? c.e2[i] : 0.0; }
__device__ __forceinline__ double nc_phi(const NCat &c, int64_t i) { return c.phi ? c.phi[i] : -10.0; }
__device__ __forceinline__ int nc_keep(const NCat &c, int64_t i) {
  return c.jk_prob ? (c.jk_prob[i] >= 0.5) : 0;
}

// input checks before counting: bit 0 -- b's z column is not ascending;
// bit 1 -- a jackknife label outside [0, n_jk) (it would index outside the
// caller's output buffers)
__global__ void check_inputs_kernel(NCat a, NCat b, int n_jk, int *flag) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < b.n; i += stride) {
    if (i > 0 && !(b.z[i] >= b.z[i - 1])) atomicOr(flag, 1);
    if (n_jk > 0 && (b.jk[i] < 0 || b.jk[i] >= n_jk)) atomicOr(flag, 2);
  }
  if (n_jk > 0)
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += stride)
      if (a.jk[i] < 0 || a.jk[i] >= n_jk) atomicOr(flag, 2);
}

// the per-pair values of corels.cpp:48-77, 122-244 in double: pair_values.h,
// the function the other FP64 paths use, with the orientation angle of
// angle_orient_axis_PB (calcs.cpp:54-57)
__device__ void noalloc_values(const JobDev &J, const NCat &g1, int64_t i, const NCat &g2,
                               int64_t j, double f[kNF]) {
  const double wt = __dmul_rn(nc_w(g1, i), nc_w(g2, j));
  const double theta =
      J.corel == COREL_DD ? 0.0 : atan((g2.y[j] - g1.y[i]) / (g2.x[j] - g1.x[i]));
  pair_values(J.corel, J.gws, wt, theta, PairGal{nc_e1(g1, i), nc_e2(g1, i), nc_phi(g1, i)},
              PairGal{nc_e1(g2, j), nc_e2(g2, j), nc_phi(g2, j)}, f);
}

// thread per g1 row, z-window binary search in the z-sorted g2, exact FP64
// predicates (exact_classify), global atomics into the caller's buffers
__global__ void __launch_bounds__(256)
noalloc_fp64_kernel(const JobDev *__restrict__ jp, NCat a, NCat b) {
  const JobDev &J = *jp;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  DCat da{}, db{};
  da.n = a.n; da.x = a.x; da.y = a.y; da.z = a.z;
  db.n = b.n; db.x = b.x; db.y = b.y; db.z = b.z;
  const double z1 = a.z[i];
  const double z_max = __dadd_rn(z1, J.pmax), z_min = __dadd_rn(z1, J.pmin);
  unsigned long long nwin = 0, nbin = 0;
  // images the reference visits for this row (lim_calc_PB, PB_calcs.cpp:30-61)
  int zlo = 0, zhi = 0, ylo = 0, yhi = 0, xlo = 0, xhi = 0;
  if (J.periodic) {
    const double x1 = a.x[i], y1 = a.y[i];
    zlo = z_min < 0 ? -1 : 0;
    zhi = z_max > J.L ? 1 : 0;
    xlo = __dsub_rn(x1, J.rmax) < 0 ? -1 : 0;
    xhi = __dadd_rn(x1, J.rmax) > J.L ? 1 : 0;
    ylo = __dsub_rn(y1, J.rmax) < 0 ? -1 : 0;
    yhi = __dadd_rn(y1, J.rmax) > J.L ? 1 : 0;
  }
  for (int sz = zlo; sz <= zhi; sz++)
    for (int sy = ylo; sy <= yhi; sy++)
      for (int sx = xlo; sx <= xhi; sx++) {
        const double Lsz = J.L * sz;
        int64_t lo = 0, hi = b.n;
        while (lo < hi) {
          const int64_t mid = (lo + hi) >> 1;
          if (__dadd_rn(b.z[mid], Lsz) < z_min) lo = mid + 1; else hi = mid;
        }
        for (int64_t j = lo; j < b.n && __dadd_rn(b.z[j], Lsz) <= z_max; j++) {
          int n1, n2;
          const int r = exact_classify(J, da, i, db, j, sx, sy, sz, n1, n2);
          if (r == 0) continue;
          nwin++;
          if (r != 2) continue;
          nbin++;
          double f[kNF];
          noalloc_values(J, a, i, b, j, f);
          const int64_t cell = (int64_t)n1 * J.npi + n2;
          atomicAdd(&J.acc_num[cell], 1ull);
          for (int q = 0; q < kNF; q++)
            if (f[q] != 0.0) atomicAdd(&J.acc_sums[cell * kNF + q], f[q]);
          if (!J.do_jk) continue;
          // corel_jk with jk_check_PB (jk.cpp:64-71, 201-223)
          const int r1 = a.jk[i], r2 = b.jk[j];
          int k1 = nc_keep(a, i), k2 = nc_keep(b, j);
          if (r1 == r2) {
            k1 = 1;
            k2 = 0;
          }
          const int rs[2] = {r1, r2}, ks[2] = {k1, k2};
          for (int t = 0; t < 2; t++) {
            if (!ks[t]) continue;
            const int64_t hc = (int64_t)(1 + rs[t]) * J.nrp * J.npi + cell;
            atomicAdd(&J.acc_num[hc], 1ull);
            double *sj = J.acc_sums + hc * kNF;
            if (f[0] != 0.0) atomicAdd(&sj[0], f[0]);
            if (J.which_corr == 0) continue;
            for (int q = 1; q < kNF; q += 2)
              if (f[q] != 0.0) atomicAdd(&sj[q], f[q]);
          }
        }
      }
  if (nwin) atomicAdd(&J.counters[0], nwin);
  if (nbin) atomicAdd(&J.counters[1], nbin);
}

void put_err(char *buf, size_t len, const char *msg) {
  if (buf && len) std::snprintf(buf, len, "%s", msg);
}

}  // namespace
}  // namespace cpc

using namespace cpc;

static cpc_status count_fp64_noalloc(const cpc_params *p, cpc_pair_kind kind,
                                     const cpc_device_catalog *c1, const cpc_device_catalog *c2,
                                     int64_t *d_num, double *d_sums, int64_t *n_window,
                                     int64_t *n_binned, void *stream, char *err, size_t err_len) {
  if (!p || !c1 || !c2 || !d_num || !d_sums) {
    put_err(err, err_len, "null argument");
    return CPC_ERR_INVALID;
  }
  if (p->coordinates != 6 || p->which_corr < 0 || p->which_corr > 2) {
    put_err(err, err_len, "unsupported parameters (coordinates 6 and which_corr 0-2 only)");
    return CPC_ERR_INVALID;
  }
  // the checks cpc_create applies (bin limits, box, n_bins <= 64 and
  // n_p_bin <= 128 -- also the scratch capacity)
  if (const char *m = param_error(*p)) {
    put_err(err, err_len, m);
    return CPC_ERR_INVALID;
  }
  if (c1->n < 0 || c2->n < 0 || c1->n > 2147483647LL || c2->n > 2147483647LL) {
    put_err(err, err_len, "catalogue size out of range");
    return CPC_ERR_INVALID;
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    put_err(err, err_len, "no usable CUDA device");
    return CPC_ERR_NODEVICE;
  }
  unsigned char *scratch = nullptr;
  {
    // once per device, with that device current: the device address of the array
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_scratch_ptr[dev]) {
      void *ptr = nullptr;
      e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
      if (e != cudaSuccess || !ptr) {
        put_err(err, err_len, "cudaGetSymbolAddress failed for the scratch array");
        return CPC_ERR_CUDA;
      }
      g_scratch_ptr[dev] = static_cast<unsigned char *>(ptr);
    }
    scratch = g_scratch_ptr[dev];
  }
  // corels2's pair-type rules (corr.cpp:226-296, initialization.cpp:699-752)
  int gws = (kind == CPC_PAIR_SRD || kind == CPC_PAIR_SD || kind == CPC_PAIR_SRS) ? 2 : 0;
  if (kind < CPC_PAIR_SD || kind > CPC_PAIR_SRS) {
    put_err(err, err_len, "bad pair kind");
    return CPC_ERR_INVALID;
  }
  int corel;
  if (kind == CPC_PAIR_RSRS || kind == CPC_PAIR_RSRD || p->which_corr == 0) corel = COREL_DD;
  else if (p->which_corr == 1) corel = COREL_SD;
  else corel = (kind == CPC_PAIR_SD) ? (p->estimator != 0 ? COREL_SSA : COREL_SS) : COREL_SD;
  const cpc_device_catalog *g1 = c1, *g2 = c2;
  if (c2->n > c1->n) {
    g1 = c2;
    g2 = c1;
    if (gws == 2) gws = 1; else if (gws == 1) gws = 2;
  }
  if ((g1->n > 0 && (!g1->x || !g1->y || !g1->z)) || (g2->n > 0 && (!g2->x || !g2->y || !g2->z)) ||
      (p->do_jk && ((g1->n > 0 && !g1->jk) || (g2->n > 0 && !g2->jk)))) {
    put_err(err, err_len, "missing device arrays (positions, or jackknife labels with do_jk)");
    return CPC_ERR_INVALID;
  }
  // the box attribution of a cross-region pair reads both galaxies' jk_prob
  // draws (jk_check_PB, jk.cpp:64-71): without them it would be lost
  if (p->do_jk && ((g1->n > 0 && !g1->jk_prob) || (g2->n > 0 && !g2->jk_prob))) {
    put_err(err, err_len, "jk_prob required with do_jk (the jackknife attribution reads it)");
    return CPC_ERR_INVALID;
  }
  JobDev J;
  std::memset(&J, 0, sizeof J);
  J.corel = corel;
  J.gws = gws;
  J.which_corr = p->which_corr;
  J.estimator = p->estimator;
  J.do_jk = p->do_jk;
  J.n_jk = p->n_jk;
  J.periodic = p->periodic_box ? 1 : 0;
  J.coordinates = 6;
  J.nrp = p->n_bins;
  J.npi = p->n_p_bin;
  J.lin_bin = p->lin_bin ? 1 : 0;
  J.box_same_keep = 1;
  J.L = p->periodic_box_size;
  J.rmin = p->bin_r_min;
  J.rmax = p->bin_r_max;
  J.pmin = p->p_min;
  J.pmax = p->p_max;
  J.wz_lo = p->p_min;  // coordinates 6: z window [z + p_min, z + p_max]
  J.wz_hi = p->p_max;
  J.ps = (p->p_max - p->p_min) / (p->n_p_bin);
  J.rsize = p->lin_bin ? (p->bin_r_max - p->bin_r_min) / p->n_bins
                       : (std::log10(p->bin_r_max) - std::log10(p->bin_r_min)) / p->n_bins;
  if (rp_thresholds(J.lin_bin, J.nrp, J.rmin, J.rmax, J.thr) != 0) {
    put_err(err, err_len, "r_p bin thresholds could not be derived");
    return CPC_ERR_INVALID;
  }
  J.acc_num = reinterpret_cast<unsigned long long *>(d_num);
  J.acc_sums = d_sums;
  J.counters = reinterpret_cast<unsigned long long *>(scratch + kCountersOffset);
  int *flag = reinterpret_cast<int *>(scratch + kCountersOffset + 64);
  const size_t cells = (size_t)(1 + (p->do_jk ? p->n_jk : 0)) * p->n_bins * p->n_p_bin;
  NCat a{g1->n, g1->x, g1->y, g1->z, g1->w, g1->e1, g1->e2, g1->phi, g1->jk_prob, g1->jk};
  NCat b{g2->n, g2->x, g2->y, g2->z, g2->w, g2->e1, g2->e2, g2->phi, g2->jk_prob, g2->jk};
  // the scratch keeps the previous call's contents: rewrite and clear it
  int sorted_flag = 0;
  unsigned long long cnt[2] = {0, 0};
  if ((e = cudaMemcpyAsync(scratch, &J, sizeof J, cudaMemcpyHostToDevice, st)) != cudaSuccess ||
      (e = cudaMemsetAsync(scratch + kCountersOffset, 0, 128, st)) != cudaSuccess ||
      (e = cudaMemsetAsync(d_num, 0, sizeof(int64_t) * cells, st)) != cudaSuccess ||
      (e = cudaMemsetAsync(d_sums, 0, sizeof(double) * cells * kNF, st)) != cudaSuccess) {
    put_err(err, err_len, cudaGetErrorString(e));
    return CPC_ERR_CUDA;
  }
  if (a.n > 0 && b.n > 0) {
    check_inputs_kernel<<<152, 256, 0, st>>>(a, b, p->do_jk ? p->n_jk : 0, flag);
    if ((e = cudaMemcpyAsync(&sorted_flag, flag, sizeof(int), cudaMemcpyDeviceToHost, st)) !=
            cudaSuccess ||
        (e = cudaStreamSynchronize(st)) != cudaSuccess) {
      put_err(err, err_len, cudaGetErrorString(e));
      return CPC_ERR_CUDA;
    }
    if (sorted_flag & 2) {
      put_err(err, err_len, "a jackknife label is outside [0, n_jk)");
      return CPC_ERR_RANGE;
    }
    if (sorted_flag & 1) {
      put_err(err, err_len, "the second catalogue scanned (after the swap rule) is not sorted by z");
      return CPC_ERR_INVALID;
    }
    noalloc_fp64_kernel<<<(unsigned)((a.n + 255) / 256), 256, 0, st>>>(
        reinterpret_cast<const JobDev *>(scratch), a, b);
    if ((e = cudaGetLastError()) != cudaSuccess) {
      put_err(err, err_len, cudaGetErrorString(e));
      return CPC_ERR_CUDA;
    }
  }
  if ((e = cudaMemcpyAsync(cnt, scratch + kCountersOffset, sizeof cnt, cudaMemcpyDeviceToHost, st)) !=
          cudaSuccess ||
      (e = cudaStreamSynchronize(st)) != cudaSuccess) {
    put_err(err, err_len, cudaGetErrorString(e));
    return CPC_ERR_CUDA;
  }
  if (n_window) *n_window = (int64_t)cnt[0];
  if (n_binned) *n_binned = (int64_t)cnt[1];
  return CPC_OK;
}

extern "C" cpc_status cpc_count_fp64_noalloc(const cpc_params *p, cpc_pair_kind kind,
                                             const cpc_device_catalog *c1,
                                             const cpc_device_catalog *c2, int64_t *d_num,
                                             double *d_sums, int64_t *n_window,
                                             int64_t *n_binned, void *stream, char *err,
                                             size_t err_len) {
  try {
    return count_fp64_noalloc(p, kind, c1, c2, d_num, d_sums, n_window, n_binned, stream, err,
                              err_len);
  } catch (...) {  // e.g. std::system_error from the mutex: never across the C ABI
    put_err(err, err_len, "host exception in cpc_count_fp64_noalloc");
    return CPC_ERR_HOST;
  }
}
