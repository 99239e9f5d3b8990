// pair_sky.cu -- sky pair loop (coordinates 0) on the GPU in double precision.
//
// The reference's sky path (corr.cpp:350-423 with lim_calc_sky and
// do_pair_sorted): for each g1 row a window in redshift, Dec and RA computed
// from the distance table (sky_calcs.cpp:105-196); g2 scanned in redshift
// order from the window's lower edge to its upper edge; Dec then RA tests;
// then corel_bin with Pi = DC2 - DC1 (calcs.cpp:126-132) and
// r_p = acos(sin d1 sin d2 + cos d1 cos d2 cos(a1 - a2)) (DA1 + DA2) / 2
// (sky_calcs.cpp:24-31, 91-96), and the jackknife rule jk_check_sky.
//
// Exactness.  The windows, sin/cos of Dec and the angles in radians are
// computed once per galaxy on the host with the C library (exactly the
// reference's values), so every window test and the Pi bin are exact here.
// Only cos(a1 - a2) and acos come from CUDA's math library, whose results can
// differ from the C library's by a few ulps; near sum = 1 acos amplifies that
// by 1/sin(theta).  Each pair gets a rigorous bound on the r_p difference
// (esum on the cosine sum, propagated through acos and the product) and every
// pair whose r_p lies within that bound of a bin threshold, or whose sum lies
// within esum of the reference's clamp at 0.9999999999, is appended to a host
// queue and binned there with the C library.  All other pairs are binned here
// against the exact host-derived thresholds, so the integer counts equal the
// reference's.  Shape sums use CUDA's atan/cos/sin (within 1e-6).
#include <cuda_runtime.h>
#include <stdint.h>

#include "cpc_device.cuh"
#include "kernels.h"

namespace cpc {

// number of thresholds thr[0..nrp] that are <= v
__device__ inline int thr_count(const JobDev &J, double v) {
  if (!(v >= J.thr[0])) return 0;
  int lo = 0, hi = J.nrp + 1;  // thr[lo] <= v, thr[hi] > v (hi = nrp+1: none)
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (v >= J.thr[mid]) lo = mid; else hi = mid;
  }
  return lo + 1;
}

__global__ void __launch_bounds__(128)
sky_fp64_kernel(const JobDev *__restrict__ jobp, SkyView a, SkyView b, int2 *hq,
                unsigned long long *hq_n, unsigned long long hq_cap, double esum) {
  const JobDev &J = *jobp;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t n1 = a.d.n, n2 = b.d.n;
  if (i >= n1) return;
  if (J.row_stride > 1 && ((a.d.orig[i] - J.row_offset) % J.row_stride) != 0) return;
  const double z_min = a.win[i], z_max = a.win[n1 + i];
  const double ra_min = a.win[2 * n1 + i], ra_max = a.win[3 * n1 + i];
  const double dec_min = a.win[4 * n1 + i], dec_max = a.win[5 * n1 + i];
  const double ra1 = a.d.x[i], dec1 = a.d.y[i];
  const double dc1 = a.dc[i], da1 = a.da[i], sd1 = a.sd[i], cd1 = a.cd[i];
  const double rar1 = a.rar[i], decr1 = a.decr[i];
  // first g2 row with redshift >= z_min
  int64_t lo = 0, hi = n2;
  while (lo < hi) {
    const int64_t mid = (lo + hi) >> 1;
    if (b.d.z[mid] < z_min) lo = mid + 1; else hi = mid;
  }
  const double kClamp = 0.9999999999;        // dA_calc (sky_calcs.cpp:28)
  const double kEps = 2.220446049250313e-16;  // 2^-52
  unsigned long long nwin = 0;
  for (int64_t j = lo; j < n2; j++) {
    const double z2 = b.d.z[j];
    if (z2 > z_max) break;
    const double dec2 = b.d.y[j];
    if (dec2 > dec_max || dec2 < dec_min) continue;
    const double ra2 = b.d.x[j];
    if (ra2 < ra_min || ra2 > ra_max) continue;  // NaN bounds pass, as in the reference
    nwin++;
    // Pi bin (exact)
    const double dP = __dsub_rn(b.dc[j], dc1);
    const double v2 = floor(__ddiv_rn(__dsub_rn(dP, J.pmin), J.ps));
    if (!(v2 >= 0.0) || v2 >= (double)J.npi) continue;
    // great-circle separation
    const double cdel = cos(__dsub_rn(rar1, b.rar[j]));
    const double sum = __dadd_rn(__dmul_rn(sd1, b.sd[j]), __dmul_rn(__dmul_rn(cd1, b.cd[j]), cdel));
    bool amb = fabs(sum - kClamp) <= esum;
    double daR = 0.0, tol = 0.0;
    if (!(sum > kClamp)) {
      const double th = acos(sum);
      daR = __ddiv_rn(__dmul_rn(th, __dadd_rn(da1, b.da[j])), 2.0);
      const double st = sin(th);
      // |d theta| <= esum / sin(theta) + a few ulps of theta (both acos)
      const double rel = esum / fmax(st * th, 1e-300) + 8.0 * kEps;
      tol = 2.0 * daR * rel;
    }
    const int k = thr_count(J, daR);
    if (!amb && tol > 0.0) amb = thr_count(J, daR - tol) != k || thr_count(J, daR + tol) != k;
    if (amb) {
      const unsigned long long q = atomicAdd(hq_n, 1ull);
      if (q < hq_cap) hq[q] = make_int2((int)i, (int)j);
      continue;
    }
    if (k < 1 || k > J.nrp) continue;
    // values (angle_orient_axis_sky, sky_calcs.cpp:13-22) and accumulation
    const double wt = __dmul_rn(a.d.w[i], b.d.w[j]);
    double theta = 0.0;
    if (J.corel != COREL_DD)
      theta = atan((dec2 - dec1) / ((ra2 - ra1) * cos((decr1 + b.decr[j]) / 2.0)));
    double f[kNF];
    pair_values(J.corel, J.gws, wt, theta, PairGal{a.d.e1[i], a.d.e2[i], a.d.phi[i]},
                PairGal{b.d.e1[j], b.d.e2[j], b.d.phi[j]}, f);
    exact_accumulate(J, a.d, i, b.d, j, k - 1, (int)v2, f);
  }
  if (nwin) atomicAdd(&J.counters[1], nwin);
}

cudaError_t launch_sky_fp64(const JobDev *job, const SkyView &a, const SkyView &b, int2 *hq,
                            unsigned long long *hq_n, unsigned long long hq_cap, double esum,
                            cudaStream_t st) {
  const int64_t blocks = (a.d.n + 127) / 128;
  if (blocks == 0) return cudaSuccess;
  sky_fp64_kernel<<<(unsigned)blocks, 128, 0, st>>>(job, a, b, hq, hq_n, hq_cap, esum);
  return cudaGetLastError();
}

}  // namespace cpc
