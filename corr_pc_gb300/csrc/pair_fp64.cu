// pair_fp64.cu -- the plain all-FP64 GPU kernel (comparison baseline and a
// full-size GPU cross-check of the fast kernel).
//
// One thread per g1 row, z-sorted catalogues, the reference's own predicates
// and arithmetic in double precision (corr.cpp:350-423 and 67-86: the image
// loops, a z-sorted window scan that stops at the first z failure, then the
// y and x windows; corel_jk for each window pair), accumulating straight into
// the global histogram block with atomics.  No cell list, no batching, no
// shared-memory privatisation.
#include <cuda_runtime.h>
#include <stdint.h>

#include "cpc_device.cuh"
#include "kernels.h"

namespace cpc {

__global__ void __launch_bounds__(256)
plain_fp64_kernel(const JobDev *__restrict__ jobp, DCat a, DCat b) {
  const JobDev &J = *jobp;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  if (J.row_stride > 1 && ((a.orig[i] - J.row_offset) % J.row_stride) != 0) return;
  const double x1 = a.x[i], y1 = a.y[i], z1 = a.z[i];
  // lim_calc_xyz / lim_calc_PB (PB_calcs.cpp:12-61)
  const double z_max = __dadd_rn(z1, J.wz_hi), z_min = __dadd_rn(z1, J.wz_lo);
  const double ra_max = __dadd_rn(x1, J.rmax), ra_min = __dsub_rn(x1, J.rmax);
  const double dec_max = __dadd_rn(y1, J.rmax), dec_min = __dsub_rn(y1, J.rmax);
  int PBx = 0, PBy = 0, PBz = 0;
  if (J.periodic) {
    if (z_min < 0) PBz = -1;
    if (z_max > J.L) PBz = abs(PBz) + 1;
    if (ra_min < 0) PBx = -1;
    if (ra_max > J.L) PBx = abs(PBx) + 1;
    if (dec_min < 0) PBy = -1;
    if (dec_max > J.L) PBy = abs(PBy) + 1;
  }
  unsigned long long nwin = 0;
  int sy = PBy > 0;
  for (int yi = 0; yi <= abs(PBy); yi++, sy--) {
    int sx = PBx > 0;
    for (int xi = 0; xi <= abs(PBx); xi++, sx--) {
      int sz = PBz > 0;
      for (int zi = 0; zi <= abs(PBz); zi++, sz--) {
        // corels1 (corr.cpp:165-180): every partner, partners after row i in
        // input order, or none
        const uint8_t af = J.auto_mode ? a.aflag[i] : 0;
        const bool a_all = auto_image_all(J.auto_mode, sz, af);
        const bool a_gt = !a_all && auto_image_gt(J.auto_mode, sz, af);
        if (!a_all && !a_gt) continue;
        const double Lsx = J.L * sx, Lsy = J.L * sy, Lsz = J.L * sz;
        // first b row with z + L*sz >= z_min (b is z-sorted)
        int64_t lo = 0, hi = b.n;
        while (lo < hi) {
          const int64_t mid = (lo + hi) >> 1;
          if (__dadd_rn(b.z[mid], Lsz) < z_min) lo = mid + 1; else hi = mid;
        }
        for (int64_t j = lo; j < b.n; j++) {
          const double z2s = __dadd_rn(b.z[j], Lsz);
          if (z2s > z_max) break;
          if (!a_all && !(b.orig[j] > a.orig[i])) continue;
          const double y2s = __dadd_rn(b.y[j], Lsy);
          if (y2s > dec_max || y2s < dec_min) continue;
          const double x2s = __dadd_rn(b.x[j], Lsx);
          if (x2s < ra_min || x2s > ra_max) continue;
          nwin++;
          // corel_bin (corels.cpp:21-46)
          int n1, n2;
          if (exact_bin(J, x1, y1, z1, x2s, y2s, z2s, n1, n2) != 2) continue;
          double f[kNF];
          exact_values(J, a, i, b, j, sx, sy, sz, f);
          exact_accumulate(J, a, i, b, j, n1, n2, f);
        }
      }
    }
  }
  if (nwin) atomicAdd(&J.counters[1], nwin);
}

cudaError_t launch_plain_fp64(const JobDev *job, const DCat &a, const DCat &b, cudaStream_t st) {
  const int64_t blocks = (a.n + 255) / 256;
  if (blocks == 0) return cudaSuccess;
  plain_fp64_kernel<<<(unsigned)blocks, 256, 0, st>>>(job, a, b);
  return cudaGetLastError();
}

}  // namespace cpc
