// pair_fast.cu -- the mixed-precision pair-counting kernel (sm_103a).
//
// One persistent launch drains a device work queue of "units".  A unit is a
// tile of up to kTile g1 rows from one (column, jackknife region) bucket and
// z-chunk, paired with every g2 candidate of the neighbouring columns inside
// the unit's shifted-z range.  A block of 8 warps keeps the tile's rows in
// shared memory; each warp stages its own batches of up to 32 candidates and
// tests them against every row, in W passes of 32 rows for a tile of up to
// 32 W rows (one row per lane; the lanes of a warp are spread over the tile).
// Candidates are drawn in chunks of a coprime-stride permutation of the
// (partner region, image shift) group, so simultaneous pairs of a warp fall in
// different bins; the block meets at a barrier once per chunk.
//
// Light pass (every candidate): FP32 separations with the image shift applied
// exactly, definite in / definite out tests of the reference's window, r^2
// range test; binned pairs go to a per-warp queue.  Heavy step (32 queued
// pairs, all lanes busy): exact r_p and Pi bins from an estimated index checked
// against definite bands, shape values, histogram updates.
//
// Precision: a pair is resolved on this path only when it is farther than a
// rigorous error bound from every decision boundary (the r_p / Pi window,
// every r_p and Pi bin edge); otherwise it is appended to an edge queue and
// re-evaluated with the reference's exact double-precision arithmetic
// (recheck_kernel), so integer counts are bit-identical with the reference.
//
// Accumulation: block-private histograms over (r_p bin, block-local Pi window)
// in shared memory -- the full sample ("main"), the cross-region pairs that the
// tile's own jackknife region does NOT take ("NX": that region's sums are main
// minus NX, so the pairs it takes, most of them, cost no update of their own) and
// one other region ("Y", the partner's region for cross-region pairs) -- with
// 32-bit counts and fixed-point sums split over two 32-bit words per field
// (exact integer addition, order independent), flushed to the FP64 global
// histogram block when the pairs added since the last flush could overflow a
// word (below) and at the end of the unit.  The terms of the fields whose sums
// cancel (rotated ellipticities and their products, kappa) are computed in
// compensated single precision (pair_df.cuh) and quantised at 2^-29 of their
// bound, so every bin sum matches the reference's double-precision sum to
// about 1e-9 of the field's bound.
#include <cuda_runtime.h>
#include <stdint.h>
#include <climits>

#include "cpc_device.cuh"
#include "kernels.h"
#include "pair_df.cuh"

namespace cpc {

constexpr int kTile = kTileThreads;          // g1 rows per tile
constexpr int kThreads = 256;                 // block size: 8 warps
constexpr int kBatch = kThreads;              // staging slots: 32 per warp
constexpr int kMaxSeg = kFastMaxSeg;
constexpr int kMaxCols = kFastMaxCols;
// candidates of a group per block barrier: a chunk adds at most kTile * kChunk
// = 2^17 terms to any word, so the flush test below runs once per chunk
constexpr int kChunk = 4 * kThreads;

// Per corel: the main fields m(k), k < FM, the jackknife fields j(g), g < FJ, and
// jm(g), the main slot holding jackknife field g (m(jm(g)) == j(g)).  FA, a(i):
// the main slots whose terms differ between the two orders of a pair whose
// galaxies carry the same data in either role (twin jobs); the others are the
// same in both orders.  Twin jobs run the corels with FA = 0 and shape_shape.
struct NoAsym {
  static constexpr int FA = 0;
  __host__ __device__ static constexpr int a(int) { return -1; }
};
template <int C> struct FieldMap;
template <> struct FieldMap<COREL_DD> : NoAsym {
  static constexpr int FM = 1, FJ = 1;
  __host__ __device__ static constexpr int m(int) { return 0; }
  __host__ __device__ static constexpr int j(int) { return 0; }
  __host__ __device__ static constexpr int jm(int) { return 0; }
};
template <> struct FieldMap<COREL_SD> : NoAsym {
  static constexpr int FM = 7, FJ = 4;
  __host__ __device__ static constexpr int m(int k) {
    return k == 0 ? 0 : k == 1 ? 1 : k == 2 ? 2 : k == 3 ? 3 : k == 4 ? 4 : k == 5 ? 11 : 12;
  }
  __host__ __device__ static constexpr int j(int k) { return k == 0 ? 0 : k == 1 ? 1 : k == 2 ? 3 : 11; }
  __host__ __device__ static constexpr int jm(int g) { return g == 0 ? 0 : g == 1 ? 1 : g == 2 ? 3 : 5; }
};
template <> struct FieldMap<COREL_SS> {
  static constexpr int FM = 11, FJ = 6;
  __host__ __device__ static constexpr int m(int k) { return k < 2 ? k : k == 2 ? 2 : k + 2; }
  __host__ __device__ static constexpr int j(int k) { return k == 0 ? 0 : 2 * k - 1 + (k >= 2 ? 2 : 0); }
  __host__ __device__ static constexpr int jm(int g) { return g == 0 ? 0 : 2 * g - 1; }
  // estimator 0: e+ of the shape holder (data[1]) and its square, the phi term
  // (data[6]) and its square: fields 1, 2, 11, 12
  static constexpr int FA = 4;
  __host__ __device__ static constexpr int a(int i) { return i == 0 ? 1 : i == 1 ? 2 : i == 2 ? 9 : 10; }
};
template <> struct FieldMap<COREL_SSA> : NoAsym {
  static constexpr int FM = 13, FJ = 7;
  __host__ __device__ static constexpr int m(int k) { return k; }
  __host__ __device__ static constexpr int j(int k) { return k == 0 ? 0 : 2 * k - 1; }
  __host__ __device__ static constexpr int jm(int g) { return g == 0 ? 0 : 2 * g - 1; }
};
// density_convergence: wt, data[1].val
template <> struct FieldMap<COREL_DK> : NoAsym {
  static constexpr int FM = 2, FJ = 2;
  __host__ __device__ static constexpr int m(int k) { return k; }
  __host__ __device__ static constexpr int j(int k) { return k; }
  __host__ __device__ static constexpr int jm(int g) { return g; }
};
// shape_convergence: wt, data[1].val, data[3].val, data[5].val
template <> struct FieldMap<COREL_SK> : NoAsym {
  static constexpr int FM = 4, FJ = 4;
  __host__ __device__ static constexpr int m(int k) { return k == 0 ? 0 : k == 1 ? 1 : k == 2 ? 5 : 9; }
  __host__ __device__ static constexpr int j(int k) { return k == 0 ? 0 : k == 1 ? 1 : k == 2 ? 5 : 9; }
  __host__ __device__ static constexpr int jm(int g) { return g; }
};
// ED: wt, data[6].val, data[6].err (regions: wt, data[6].val)
template <> struct FieldMap<COREL_ED> : NoAsym {
  static constexpr int FM = 3, FJ = 2;
  __host__ __device__ static constexpr int m(int k) { return k == 0 ? 0 : k == 1 ? 11 : 12; }
  __host__ __device__ static constexpr int j(int k) { return k == 0 ? 0 : 11; }
  __host__ __device__ static constexpr int jm(int g) { return g; }
};

template <class FM, int G = 0>
constexpr bool jm_consistent() {
  if constexpr (G >= FM::FJ) {
    return true;
  } else {
    return FM::m(FM::jm(G)) == FM::j(G) && jm_consistent<FM, G + 1>();
  }
}
// position of main slot k among the order-dependent slots a(i), or -1
template <class FM>
__host__ __device__ constexpr int asym_pos(int k) {
  for (int i = 0; i < FM::FA; i++)
    if (FM::a(i) == k) return i;
  return -1;
}
static_assert(FieldMap<COREL_SS>::m(FieldMap<COREL_SS>::a(0)) == 1 &&
                  FieldMap<COREL_SS>::m(FieldMap<COREL_SS>::a(1)) == 2 &&
                  FieldMap<COREL_SS>::m(FieldMap<COREL_SS>::a(2)) == 11 &&
                  FieldMap<COREL_SS>::m(FieldMap<COREL_SS>::a(3)) == 12,
              "order-dependent shape_shape fields");
static_assert(jm_consistent<FieldMap<COREL_DD>>() && jm_consistent<FieldMap<COREL_SD>>() &&
                  jm_consistent<FieldMap<COREL_SS>>() && jm_consistent<FieldMap<COREL_SSA>>() &&
                  jm_consistent<FieldMap<COREL_DK>>() && jm_consistent<FieldMap<COREL_SK>>() &&
                  jm_consistent<FieldMap<COREL_ED>>(),
              "jackknife fields must map onto main slots");

// Padding that puts the high-word array (FW * NB words after the low words)
// 16 banks away from the low-word array.
__host__ __device__ constexpr int hi_pad(int words) { return (16 - (words & 31) + 32) & 31; }

// Replicas of the hot r_p bins (a build option, off by default).  Most pairs
// fall in the few largest r_p bins (their count grows as r_p^2), so the lanes of
// one heavy-step instruction often add into the same main-histogram bins, and
// same-address shared reductions are serialised.  With CPC_HOT_REP > 1 the top
// kHotBins r_p bins of the main histogram get kHotRep copies each, the copy
// picked by lane bits 1-2 (bit 0 already splits lanes over the low and high
// words), and the flush adds the copies together in exact integer arithmetic.
// Measured on GB300: 4 copies of the top 4 bins gain 2% on the 200k wg+ box and
// lose 3-4% on the kappa and ED workloads (the copies take shared memory from
// the Pi window); on the 2M w++ box 2 copies of the top one or two rows or 4
// of the top row gain nothing (777, 773 and 786 ms against 773 ms), so the
// default is one copy.
#ifndef CPC_HOT_REP
#define CPC_HOT_REP 1
#endif
#ifndef CPC_HOT_BINS
#define CPC_HOT_BINS 4
#endif
constexpr int kHotRep = CPC_HOT_REP, kHotBins = CPC_HOT_BINS;
static_assert(kHotRep == 1 || kHotRep == 2 || kHotRep == 4 || kHotRep == 8, "replicas: 1, 2, 4 or 8");
// main-histogram bins of a block: nrp * wpi, plus the hot bins' extra copies
__host__ __device__ __forceinline__ int hot_rows(int nrp) { return nrp < kHotBins ? nrp : kHotBins; }
__host__ __device__ __forceinline__ int main_bins(int nrp, int wpi) {
  return nrp * wpi + (kHotRep - 1) * hot_rows(nrp) * wpi;
}
// bin of copy r (1 <= r < kHotRep) of hot bin (n1, elk), n1 >= nrp - hot_rows(nrp)
__host__ __device__ __forceinline__ int rep_bin(int r, int n1, int elk, int nrp, int wpi) {
  const int h = hot_rows(nrp);
  return nrp * wpi + ((r - 1) * h + (n1 - (nrp - h))) * wpi + elk;
}

// Dynamic shared memory of the candidate staging: positions, then (for the
// corels with values) the weighted ellipticities or orientation and the aux
// view (x lo, y lo, phi, w lo) of each staged candidate.
__host__ __device__ constexpr size_t stage_bytes(int corel) {
  return sizeof(float4) * (corel == COREL_DD ? 2 : 3) * kBatch +
         (corel == COREL_ED ? sizeof(float) * (kBatch + kTile) : 0);  // ED: z lo parts
}
// Dynamic shared memory of the corels1 (auto pair) rules, after the staging:
// each staged candidate's input index and each row's thresholds per z image.
constexpr size_t kAutoBytes = sizeof(int) * (kBatch + 3 * kTile);

// Shared-memory bytes a block needs for a job with nrp r_p bins and a wpi-bin
// Pi window.  With unit weights (unit_w) field 0 (the weight sum, equal to the
// count) is not accumulated and has no words.  A twin job adds the other
// order's order-dependent main fields and its two region histograms.
size_t fast_smem_bytes(int corel, int do_jk, int nrp, int wpi, int auto_pairs, int unit_w,
                       int twin) {
  const int NB = nrp * wpi, NBm = main_bins(nrp, wpi);
  int FM = 1, FJ = 1;
  if (corel == COREL_SD) { FM = 7; FJ = 4; }
  if (corel == COREL_SS) { FM = 11; FJ = 6; }
  if (corel == COREL_SSA) { FM = 13; FJ = 7; }
  if (corel == COREL_DK) { FM = 2; FJ = 2; }
  if (corel == COREL_SK) { FM = 4; FJ = 4; }
  if (corel == COREL_ED) { FM = 3; FJ = 2; }
  const int FA = corel == COREL_SS ? FieldMap<COREL_SS>::FA : 0;
  const int f0 = unit_w ? 1 : 0;
  FM -= f0;
  FJ -= f0;
  size_t b = stage_bytes(corel) + (auto_pairs ? kAutoBytes : 0);  // staging
  b += 8ull * FM * NBm + 4ull * NBm + 4ull * hi_pad(FM * NBm);
  if (do_jk) b += 2 * (8ull * FJ * NB + 4ull * NB + 4ull * hi_pad(FJ * NB));
  if (twin) {
    b += 8ull * FA * NB + 4ull * hi_pad(FA * NB);
    if (do_jk) b += 2 * (8ull * FJ * NB + 4ull * NB + 4ull * hi_pad(FJ * NB));
  }
  return b;
}

// Fixed-point sums in 32-bit shared words.  A term v of field f becomes the
// integer u = rint(v * 2^S_f), |u| < 2^29 (S_f from a bound on |v|); u is split
// into its low 15 bits (0..32767) and the arithmetic shift u >> 15
// (-2^14..2^14 - 1), each added to its own 32-bit word with a plain reduction
// (no return value: no scoreboard wait; lanes of one instruction that hit the
// same word are serialised, which red_pair halves).  A block counts the pairs
// its warps queued since the last flush and flushes before a chunk that could
// take the count past 2^17 (a chunk adds at most kTile * kChunk = 2^17 pairs),
// so a bin takes at most 2^17 terms between flushes: the low word stays below
// 2^32 and the high word, read as a signed integer, within [-2^31, 2^31).
constexpr unsigned kFlushTerms = 1u << 17;
static_assert((unsigned)kTile * kChunk <= kFlushTerms, "a chunk fits between flushes");
// The two reductions of one term, even lanes taking the low word first and odd
// lanes the high word first: lanes of one instruction that hit the same bin then
// split over two addresses 16 banks apart (same-address shared reductions are
// serialised), halving those collisions.
// wa, wb: the lane's two words in that order (low, high for even lanes).
__device__ __forceinline__ void red_pair(unsigned *lo, unsigned *hi, unsigned wa, unsigned wb,
                                         bool odd) {
  atomicAdd(odd ? hi : lo, wa);
  atomicAdd(odd ? lo : hi, wb);
}
__device__ __forceinline__ double fixed_total(unsigned lw, unsigned hw, double inv_scale) {
  const long long tot = (long long)(int)hw * 32768ll + (long long)lw;
  return (double)tot * inv_scale;
}

__device__ __forceinline__ int gcd_int(int a, int b) {
  while (b) {
    const int r = a % b;
    a = b;
    b = r;
  }
  return a;
}

__device__ __forceinline__ int floordiv(int a, int b) {
  int q = a / b;
  if ((a % b != 0) && ((a < 0) != (b < 0))) --q;
  return q;
}

// first index in [lo, hi) with zf[idx] >= v
__device__ __forceinline__ int lower_bound_f(const float *zf, int lo, int hi, float v) {
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (__ldg(zf + mid) < v) lo = mid + 1; else hi = mid;
  }
  return lo;
}

// Append a pair to the FP64 edge queue.  Entries past the capacity are only
// counted: the host then grows the queue and runs the job again (the set of
// queued pairs is deterministic), so the kernel never needs an inline FP64
// path of its own.
__device__ __forceinline__ void enqueue(int job, int64_t i1, int64_t j2, int code, QEntry *q,
                                        unsigned long long *qcount, unsigned long long qcap) {
  const unsigned long long pos = atomicAdd(qcount, 1ull);
  if (pos < qcap) {
    QEntry e;
    e.job = job;
    e.i1 = (int)i1;
    e.j2 = (int)j2;
    e.shift = code;
    q[pos] = e;
  }
}

// ephi_calc (calcs.cpp:97-105) in FP32
__device__ __forceinline__ float ephi_f(float phi, float theta) {
  float t = fabsf(phi - theta);
  return t > 1.5707963267948966f ? 3.14159265358979f - t : t;
}

// Flush the partner-region histogram (jackknife fields) into the global FP64
// block at histogram index h, and zero it.  mirror: the histogram holds the
// other order of twin pairs, whose Pi bin is npi - 1 - (the window's bin).
template <class FMAP>
__device__ __forceinline__ void flush_region(unsigned *cnt, unsigned *lo, unsigned *hi, int NB,
                                             int wpi, int npi, int nrp, int n2_base, int h, int f0,
                                             const double *s_iqs, const JobDev &J,
                                             bool mirror = false) {
  const int64_t hb = (int64_t)h * nrp * npi;
  for (int lb = threadIdx.x; lb < NB; lb += kThreads) {
    const unsigned n = cnt[lb];
    if (!n) continue;
    const int n2 = n2_base + lb % wpi;
    const int64_t cell = hb + (int64_t)(lb / wpi) * npi + (mirror ? npi - 1 - n2 : n2);
    atomicAdd(&J.acc_num[cell], (unsigned long long)n);
    cnt[lb] = 0u;
#pragma unroll
    for (int g = 0; g < FMAP::FJ; g++) {
      if (g < f0) continue;  // field 0 of unit weights: no words
      const size_t o = (size_t)g * NB + lb;
      const int fld = FMAP::j(g);
      const double v = fixed_total(lo[o], hi[o], s_iqs[fld]);
      if (v != 0.0) atomicAdd(&J.acc_sums[cell * kNF + fld], v);
      lo[o] = 0u;
      hi[o] = 0u;
    }
  }
}

// The histograms of the other order of twin pairs (a twin job's block): its
// order-dependent main fields (FA words per bin, low and high) and its two
// region histograms (the tile's region: the pairs it does not take; the
// partner's region), all indexed by the window bin of the pair's own order.
struct TwinHist {
  bool on;
  unsigned *alo, *ahi;              // order-dependent main fields [FA][NB]
  unsigned *ncnt, *nlo, *nhi;       // tile's region, pairs it does not take
  unsigned *ycnt, *ylo, *yhi;       // partner's region
};

// Flush the main histogram (into h = 0) and the tile's region (into hx): the
// region takes main minus NX, in exact integer arithmetic; zero both.
// Main bins are strided by NBm (main_bins: the hot bins' copies after the NB
// plain bins); the copies of a hot bin are summed into it.  Twin blocks also
// add the other order of each bin's pairs to the mirrored Pi bin
// npi - 1 - n2: the same count and order-independent sums, its own
// order-dependent sums, and its own tile-region exclusions.
template <int FM, int FJ, class FMAP>
__device__ __forceinline__ void flush_main_x(unsigned *mcnt, unsigned *mlo, unsigned *mhi,
                                             unsigned *ncnt, unsigned *nlo, unsigned *nhi, int NB,
                                             int NBm, int wpi, int npi, int nrp, int n2_base,
                                             int hx, bool jk, int f0, const double *s_iqs,
                                             const JobDev &J, const TwinHist &tw) {
  const int64_t hsz = (int64_t)nrp * npi;
  const int hot0 = nrp - hot_rows(nrp);
  constexpr int FA = FMAP::FA > 0 ? FMAP::FA : 1;
  for (int lb = threadIdx.x; lb < NB; lb += kThreads) {
    const int n1 = lb / wpi, elk = lb - n1 * wpi;
    const int nrep = (kHotRep > 1 && n1 >= hot0) ? kHotRep : 1;
    unsigned n = mcnt[lb];
    for (int r = 1; r < nrep; r++) n += mcnt[rep_bin(r, n1, elk, nrp, wpi)];
    if (!n) continue;  // no pair in this bin since the last flush: every word is 0
    const int64_t cell = (int64_t)n1 * npi + n2_base + elk;
    atomicAdd(&J.acc_num[cell], (unsigned long long)n);
    mcnt[lb] = 0u;
    for (int r = 1; r < nrep; r++) mcnt[rep_bin(r, n1, elk, nrp, wpi)] = 0u;
    long long tm[FM];
#pragma unroll
    for (int f = 0; f < FM; f++) {
      tm[f] = 0;
      if (f < f0) continue;  // field 0 of unit weights: no words
      for (int r = 0; r < nrep; r++) {
        const size_t o = (size_t)f * NBm + (r == 0 ? lb : rep_bin(r, n1, elk, nrp, wpi));
        tm[f] += (long long)(int)mhi[o] * 32768ll + (long long)mlo[o];
        mlo[o] = 0u;
        mhi[o] = 0u;
      }
      const int fld = FMAP::m(f);
      if (tm[f] != 0) atomicAdd(&J.acc_sums[cell * kNF + fld], (double)tm[f] * s_iqs[fld]);
    }
    long long ta[FA];
    const int64_t cm = (int64_t)n1 * npi + (npi - 1 - (n2_base + elk));
    if (tw.on) {
      atomicAdd(&J.acc_num[cm], (unsigned long long)n);
#pragma unroll
      for (int i = 0; i < FMAP::FA; i++) {
        const size_t o = (size_t)i * NB + lb;
        ta[i] = (long long)(int)tw.ahi[o] * 32768ll + (long long)tw.alo[o];
        tw.alo[o] = 0u;
        tw.ahi[o] = 0u;
      }
#pragma unroll
      for (int f = 0; f < FM; f++) {
        if (f < f0) continue;
        const int ap = asym_pos<FMAP>(f);
        const long long v = ap >= 0 ? ta[ap] : tm[f];
        const int fld = FMAP::m(f);
        if (v != 0) atomicAdd(&J.acc_sums[cm * kNF + fld], (double)v * s_iqs[fld]);
      }
    }
    if (!jk) continue;
    const int64_t xc = (int64_t)hx * hsz + cell;
    const unsigned nx = ncnt[lb];
    ncnt[lb] = 0u;
    if (n - nx) atomicAdd(&J.acc_num[xc], (unsigned long long)(n - nx));
#pragma unroll
    for (int g = 0; g < FJ; g++) {
      if (g < f0) continue;
      const size_t o = (size_t)g * NB + lb;
      const long long tn = (long long)(int)nhi[o] * 32768ll + (long long)nlo[o];
      nlo[o] = 0u;
      nhi[o] = 0u;
      const long long tx = tm[FMAP::jm(g)] - tn;
      const int fld = FMAP::j(g);
      if (tx != 0) atomicAdd(&J.acc_sums[xc * kNF + fld], (double)tx * s_iqs[fld]);
    }
    if (!tw.on) continue;
    const int64_t xm = (int64_t)hx * hsz + cm;
    const unsigned nxm = tw.ncnt[lb];
    tw.ncnt[lb] = 0u;
    if (n - nxm) atomicAdd(&J.acc_num[xm], (unsigned long long)(n - nxm));
#pragma unroll
    for (int g = 0; g < FJ; g++) {
      if (g < f0) continue;
      const size_t o = (size_t)g * NB + lb;
      const long long tn = (long long)(int)tw.nhi[o] * 32768ll + (long long)tw.nlo[o];
      tw.nlo[o] = 0u;
      tw.nhi[o] = 0u;
      const int ap = asym_pos<FMAP>(FMAP::jm(g));
      const long long tx = (ap >= 0 ? ta[ap] : tm[FMAP::jm(g)]) - tn;
      const int fld = FMAP::j(g);
      if (tx != 0) atomicAdd(&J.acc_sums[xm * kNF + fld], (double)tx * s_iqs[fld]);
    }
  }
}

constexpr int kQCap = 64;  // per-warp ring of binned pairs awaiting the heavy step
constexpr unsigned kEdgeFlag = 0x8000u;  // queue entry: near the window edge

// MINB: blocks per SM the registers are bounded for (4 when the job's
// histograms fit a quarter of shared memory, else 3).  TW: twin jobs (every job
// of the launch), compiled apart so that the other jobs' kernel carries none of
// the twin code.
template <int C, bool JK, int MINB, bool TW>
__global__ void __launch_bounds__(kThreads, MINB == 1 ? 2 : MINB)
fast_pairs_kernel(const JobDev *__restrict__ jobs, const UnitDesc *__restrict__ units,
                  int n_units, unsigned int *__restrict__ unit_ctr, QEntry *__restrict__ queue,
                  unsigned long long *__restrict__ qcount, unsigned long long qcap,
                  const __grid_constant__ FastScales sc, int zero_words, int auto_smem) {
  using F = FieldMap<C>;
  extern __shared__ __align__(16) unsigned char smem[];
  float4 *s_pos = reinterpret_cast<float4 *>(smem);
  float4 *s_shp = s_pos + kBatch;
  float4 *s_aux = s_shp + kBatch;  // x lo, y lo, phi, w lo of each staged candidate
  // ED: z lo parts of the staged candidates and of the tile's rows
  float *s_zlo = reinterpret_cast<float *>(smem + sizeof(float4) * 3 * kBatch);
  float *s_rzlo = s_zlo + kBatch;
  // corels1 rules (launches with auto-pair jobs only): the input index of each
  // staged candidate; per row and z image (index sz + 1) a threshold on the
  // partner's input index: -1 every partner (and every pair outside corels1),
  // the row's own index: partners after it, INT_MAX: none
  int *s_orig = auto_smem ? reinterpret_cast<int *>(smem + stage_bytes(C)) : nullptr;
  int *s_rothr = auto_smem ? s_orig + kBatch : nullptr;
  unsigned char *hist_base = smem + stage_bytes(C) + (auto_smem ? kAutoBytes : 0);
  // the candidate slots of a unit, used only while the staging buffer is idle
  // (between the unit's slot set-up barriers, before any candidate is staged)
  int *s_slot_b = reinterpret_cast<int *>(s_pos);
  int *s_slot_info = s_slot_b + kMaxSeg;
  static_assert(2 * kMaxSeg * sizeof(int) <= kBatch * sizeof(float4), "slot tables fit the staging buffer");

  __shared__ int s_unit;
  __shared__ int s_cnt[kMaxCols + 1];
  __shared__ int s_seg_a[kMaxSeg], s_seg_len[kMaxSeg], s_seg_key[kMaxSeg];
  __shared__ int s_order[kMaxSeg], s_pre[kMaxSeg + 1];
  __shared__ int s_jidx[kBatch];
  __shared__ unsigned char s_keep[kBatch];
  // twin jobs: the other role's keep flag of each staged candidate (g1's) and of
  // each tile row (g2's)
  __shared__ unsigned char s_keep2[TW ? kBatch : 1];
  __shared__ unsigned long long s_red[kThreads / 32];
  __shared__ unsigned s_nbin;  // pairs queued by the block's warps since the last flush
  __shared__ float s_A[kMaxRp], s_B[kMaxRp], s_PA[kMaxPi], s_PB[kMaxPi];
  // the tile's g1 rows, for the heavy step (any lane may process any row)
  // s_rshp / s_shp hold the weighted ellipticities (ewt) for the corels with
  // shape terms and the orientation (shp) for ED
  __shared__ float4 s_rpos[kTile], s_rshp[kTile], s_raux[kTile];
  __shared__ unsigned char s_rkeep[kTile], s_rkeep2[TW ? kTile : 1];
  __shared__ unsigned s_wq[kThreads / 32][kQCap];

  const int t = threadIdx.x, lane = t & 31, wid = t >> 5;
  const unsigned lt_mask = (1u << lane) - 1u;
  {
    unsigned int *z = reinterpret_cast<unsigned int *>(hist_base);
    for (int k = t; k < zero_words; k += kThreads) z[k] = 0u;
    if (t == 0) s_nbin = 0u;
  }
  __syncthreads();

  for (;;) {
    if (t == 0) s_unit = (int)atomicAdd(unit_ctr, 1u);
    __syncthreads();
    const int u = s_unit;
    if (u >= n_units) break;
    const UnitDesc U = units[u];
    const JobDev &J = jobs[U.job];
    const int nrp = J.nrp, wpi = J.wpi, npi = J.npi, NB = nrp * wpi;
    const int NBm = main_bins(nrp, wpi), hot0 = nrp - hot_rows(nrp);
    // per histogram: count[NB], low words [F][NB], high words [F][NB] (main:
    // NBm bins, the hot bins' copies included).  Unit weights: wt_num = count,
    // field 0 is not accumulated and gets no words; the word arrays are indexed
    // by field f >= f0 from a base f0 rows before their first stored row (which
    // then coincides with the count array, never read through it).
    const int f0 = J.unit_w ? 1 : 0;
    const int FMs = F::FM - f0, FJs = F::FJ - f0;  // stored fields
    unsigned *s_mnum = reinterpret_cast<unsigned *>(hist_base);
    // the high words sit hi_pad words after a 32-word-aligned offset from the low
    // words, so the low and high word of one bin are 16 banks apart (red_pair)
    unsigned *s_mlo0 = s_mnum + NBm;
    unsigned *s_mhi0 = s_mlo0 + (size_t)FMs * NBm + hi_pad(FMs * NBm);
    unsigned *s_nxnum = s_mhi0 + (size_t)FMs * NBm;
    unsigned *s_nxlo0 = s_nxnum + NB;
    unsigned *s_nxhi0 = s_nxlo0 + (size_t)FJs * NB + hi_pad(FJs * NB);
    unsigned *s_ynum = s_nxhi0 + (size_t)FJs * NB;
    unsigned *s_ylo0 = s_ynum + NB;
    unsigned *s_yhi0 = s_ylo0 + (size_t)FJs * NB + hi_pad(FJs * NB);
    unsigned *s_mlo = s_mlo0 - (size_t)f0 * NBm, *s_mhi = s_mhi0 - (size_t)f0 * NBm;
    unsigned *s_nxlo = s_nxlo0 - (size_t)f0 * NB, *s_nxhi = s_nxhi0 - (size_t)f0 * NB;
    unsigned *s_ylo = s_ylo0 - (size_t)f0 * NB, *s_yhi = s_yhi0 - (size_t)f0 * NB;
    // twin jobs: the other order's histograms after the region histograms
    constexpr bool twin = TW;
    constexpr int FA = F::FA;
    TwinHist tw;
    {
      unsigned *base = JK ? s_yhi0 + (size_t)FJs * NB : s_nxnum;
      tw.on = twin;
      tw.alo = base;
      tw.ahi = tw.alo + (size_t)FA * NB + hi_pad(FA * NB);
      tw.ncnt = tw.ahi + (size_t)FA * NB;
      unsigned *nlo0 = tw.ncnt + NB;
      unsigned *nhi0 = nlo0 + (size_t)FJs * NB + hi_pad(FJs * NB);
      tw.ycnt = nhi0 + (size_t)FJs * NB;
      unsigned *ylo0 = tw.ycnt + NB;
      unsigned *yhi0 = ylo0 + (size_t)FJs * NB + hi_pad(FJs * NB);
      tw.nlo = nlo0 - (size_t)f0 * NB;
      tw.nhi = nhi0 - (size_t)f0 * NB;
      tw.ylo = ylo0 - (size_t)f0 * NB;
      tw.yhi = yhi0 - (size_t)f0 * NB;
    }

    // ---- the tile's g1 rows, in shared memory.  Row slot tr = s * 32 + l holds
    // tile row q = l * W + s (s < W): a warp holds slots s * 32 .. s * 32 + 31 in
    // its pass s, so its lanes are spread over the whole tile and simultaneous
    // pairs of a warp fall in different Pi bins.  Every warp tests its own
    // candidates against every row, one pass of 32 rows at a time. ----
    const int W = (U.g1_count + 31) >> 5;
    // hi + lo positions for the orientation angle (raw separations) and the ED
    // separation
    constexpr bool kTheta = C == COREL_SD || C == COREL_SS || C == COREL_SSA || C == COREL_SK;
    const bool has_lo = (kTheta || C == COREL_ED) && J.has_lo;
    const int rmu = J.rmu;
    // MINB == 1: the cell-list FP64 comparison engine (CPC_ENGINE_CELL_FP64): every
    // candidate inside the outer window bounds is evaluated by the FP64 path,
    // inline, with global atomics (no FP32 value, no shared histogram)
    constexpr bool all_exact = MINB == 1;
    // jackknife attribution: jk_check_PB (the box's rule; this kernel runs box
    // jobs only)
    const int gws = J.gws, lin_bin = J.lin_bin;
    const float rmin_f = J.rmin_f, inv_rsize_f = J.inv_rsize_f;
    for (int tr = t; tr < 32 * W; tr += kThreads) {
      const int q = (tr & 31) * W + (tr >> 5);
      float4 p = make_float4(0.f, 0.f, 0.f, 0.f);
      unsigned char ok = 0, af = 0;
      int oi = 0;
      if (q < U.g1_count) {
        const int64_t i1 = (int64_t)U.g1_start + (int64_t)q * U.g1_stride;
        p = J.f1.pos[i1];
        ok = 1;
        if (J.auto_mode) {
          oi = (int)J.d1.orig[i1];  // input index (corels1)
          af = J.f1.aflag[i1];      // corels1 scan-start flags
        }
        if (J.row_stride > 1) {
          const int64_t o = J.d1.orig[i1] - J.row_offset;
          ok = (o % J.row_stride) == 0;
        }
        if (C != COREL_DD) {
          s_rshp[tr] = C == COREL_ED ? J.f1.shp[i1] : J.f1.ewt[i1];
          s_raux[tr] = J.f1.aux[i1];
        }
        if (C == COREL_ED && has_lo) s_rzlo[tr] = J.f1.zlo[i1];
        if (JK) s_rkeep[tr] = J.f1.keep[i1];
        if (JK && TW) s_rkeep2[tr] = J.f2.keep[i1];
      }
      // a row that is not counted gets z = NaN: every window test fails
      if (!ok) p.z = __int_as_float(0x7fc00000);
      s_rpos[tr] = p;
      if (auto_smem)
        for (int z = -1; z <= 1; z++)
          s_rothr[(z + 1) * kTile + tr] = auto_image_all(J.auto_mode, z, af) ? -1
                                          : auto_image_gt(J.auto_mode, z, af) ? oi : INT_MAX;
    }
    const float Lf = J.Lf;
    const float xy_in = J.xy_in, xy_out = J.xy_out;
    const float pi_in_lo = J.pi_in_lo, pi_in_hi = J.pi_in_hi;
    const float pi_out_lo = J.pi_out_lo, pi_out_hi = J.pi_out_hi;
    const float inv_ps = J.inv_ps_f, tp0 = J.tp0;
    const float mu_rel = J.mu_rel, mu_abs = J.mu_abs;
    for (int k = t; k < nrp; k += kThreads) { s_A[k] = J.A[k]; s_B[k] = J.B[k]; }
    for (int k = t; k < npi; k += kThreads) { s_PA[k] = J.PA[k]; s_PB[k] = J.PB[k]; }
    const float l2rmin2 = J.l2rmin2, inv_lw = J.inv_lw, rej_lo = J.rej_lo, rej_hi = J.rej_hi;
    const int n2_base = U.n2_base;
    unsigned nwin = 0;  // window pairs of this thread's row in this unit

    // ---- enumerate candidate slots: (column, bucket, sz) overlapping the unit's z range ----
    const int ncxu = U.cx_hi - U.cx_lo + 1;
    const int ncol = ncxu * (U.cy_hi - U.cy_lo + 1);
    const int nsz_lo = J.periodic ? -1 : 0, nsz_hi = J.periodic ? 1 : 0;
    for (int c = t; c < ncol; c += kThreads) {
      const int cx = U.cx_lo + c % ncxu, cy = U.cy_lo + c / ncxu;
      const int sx = J.periodic ? floordiv(cx, J.ncx) : 0, sy = J.periodic ? floordiv(cy, J.ncy) : 0;
      int cnt = 0;
      if (sx >= -1 && sx <= 1 && sy >= -1 && sy <= 1) {
        const int col = (cy - sy * J.ncy) * J.ncx + (cx - sx * J.ncx);
        const int b0 = J.f2.col_begin[col], b1 = J.f2.col_end[col];
        for (int b = b0; b < b1; b++) {
          const float bz0 = J.f2.bk_zmin[b], bz1 = J.f2.bk_zmax[b];
          for (int sz = nsz_lo; sz <= nsz_hi; sz++) {
            const float lo = (float)(U.zlo - J.L * sz), hi = (float)(U.zhi - J.L * sz);
            if (bz1 >= lo && bz0 < hi) cnt++;
          }
        }
      }
      s_cnt[c] = cnt;
    }
    __syncthreads();
    if (t == 0) {
      int run = 0;
      for (int c = 0; c < ncol; c++) {
        const int v = s_cnt[c];
        s_cnt[c] = run;
        run += v;
      }
      s_cnt[ncol] = run;
    }
    __syncthreads();
    const int total_slots = s_cnt[ncol];
    int cur_y = -1;        // region held in the Y histogram
    unsigned wbin = 0;     // pairs this warp queued in its current batch

    for (int chunk0 = 0; chunk0 < total_slots; chunk0 += kMaxSeg) {
      const int nslot = min(kMaxSeg, total_slots - chunk0);
      for (int c = t; c < ncol; c += kThreads) {
        int pos = s_cnt[c];
        if (pos >= chunk0 + kMaxSeg || s_cnt[c + 1] <= chunk0) continue;
        const int cx = U.cx_lo + c % ncxu, cy = U.cy_lo + c / ncxu;
        const int sx = J.periodic ? floordiv(cx, J.ncx) : 0, sy = J.periodic ? floordiv(cy, J.ncy) : 0;
        const int col = (cy - sy * J.ncy) * J.ncx + (cx - sx * J.ncx);
        const int b0 = J.f2.col_begin[col], b1 = J.f2.col_end[col];
        for (int b = b0; b < b1; b++) {
          const float bz0 = J.f2.bk_zmin[b], bz1 = J.f2.bk_zmax[b];
          for (int sz = nsz_lo; sz <= nsz_hi; sz++) {
            const float lo = (float)(U.zlo - J.L * sz), hi = (float)(U.zhi - J.L * sz);
            if (!(bz1 >= lo && bz0 < hi)) continue;
            const int k = pos - chunk0;
            if (k >= 0 && k < kMaxSeg) {
              s_slot_b[k] = b;
              s_slot_info[k] = shift_code(sx, sy, sz);
            }
            pos++;
          }
        }
      }
      __syncthreads();
      for (int k = t; k < nslot; k += kThreads) {
        const int b = s_slot_b[k], code = s_slot_info[k];
        const int sz = code / 9 - 1;
        const float lo = (float)(U.zlo - J.L * sz), hi = (float)(U.zhi - J.L * sz);
        const int bs = J.f2.bk_start[b], be = J.f2.bk_end[b];
        const int a = lower_bound_f(J.f2.zf, bs, be, lo);
        const int e = lower_bound_f(J.f2.zf, a, be, hi);
        s_seg_a[k] = a;
        s_seg_len[k] = e - a;
        s_seg_key[k] = (e > a) ? J.f2.bk_region[b] * 27 + code : INT_MAX;
      }
      __syncthreads();
      for (int k = t; k < nslot; k += kThreads) {  // stable rank sort by key
        const int key = s_seg_key[k];
        int r = 0;
        for (int m = 0; m < nslot; m++) {
          const int km = s_seg_key[m];
          r += (km < key) || (km == key && m < k);
        }
        s_order[r] = k;
      }
      __syncthreads();
      if (t == 0) {
        int run = 0;
        for (int k = 0; k < nslot; k++) {
          s_pre[k] = run;
          run += s_seg_len[s_order[k]];
        }
        s_pre[nslot] = run;
      }
      __syncthreads();

      int k = 0;
      while (k < nslot) {
        const int key = s_seg_key[s_order[k]];
        if (key == INT_MAX) break;
        int g = k + 1;
        while (g < nslot && s_seg_key[s_order[g]] == key) g++;
        const int region2 = key / 27, code = key % 27;
        int sx, sy, sz;
        shift_decode(code, sx, sy, sz);
        const bool same_region = region2 == U.region;
        // twin jobs test each unordered pair once, in the order whose g2 is
        // ahead of g1: z image +1, or image 0 with a larger z (ties: the image
        // shift in y, then x, then the index).  Image -1 candidates are the
        // other order of image +1 pairs of their own tiles.
        if (twin && sz < 0) {
          k = g;
          continue;
        }
        const int tie_dir = sy != 0 ? sy : sx;  // z ties within image 0
        // staging order: position (i * ks) mod N over the group's N candidates,
        // ks coprime with N and ~0.618 N, so a batch is a spread-out sample of
        // the group's columns and z range (decorrelated bins, fewer collisions)
        const int gN = s_pre[g] - s_pre[k];
        int ks = 1;
        if (gN > 2) {
          ks = max(1, (int)(0.6180339887f * gN));
          while (gcd_int(ks, gN) != 1) ks++;
        }
        if (JK && !same_region && cur_y != region2) {
          if (cur_y >= 0) {
            __syncthreads();
            flush_region<F>(s_ynum, s_ylo, s_yhi, NB, wpi, npi, nrp, n2_base,
                                       1 + cur_y, f0, sc.iqs, J);
            if (twin)
              flush_region<F>(tw.ycnt, tw.ylo, tw.yhi, NB, wpi, npi, nrp, n2_base, 1 + cur_y, f0,
                              sc.iqs, J, true);
            __syncthreads();
          }
          cur_y = region2;
        }
        // g2-side shift for -1 images (x2 - L exact for the candidates that can
        // reach the window); the g1-side shift for +1 images (x1 - L exact for
        // x1 >= L/2) is applied per row below
        const float g2sx = sx == -1 ? Lf : 0.f, g2sy = sy == -1 ? Lf : 0.f, g2sz = sz == -1 ? Lf : 0.f;

        for (int base = 0; base < gN; base += kChunk) {
          const int nc = min(kChunk, gN - base);
          // s_nbin is read after a barrier and changed only after the next one
          if (s_nbin + (unsigned)(kTile * nc) > kFlushTerms) {  // keep every word below 2^32
            __syncthreads();
            flush_main_x<F::FM, F::FJ, F>(s_mnum, s_mlo, s_mhi, s_nxnum, s_nxlo, s_nxhi, NB, NBm,
                                          wpi, npi, nrp, n2_base, 1 + U.region, JK, f0, sc.iqs,
                                          J, tw);
            if (JK && cur_y >= 0) {
              flush_region<F>(s_ynum, s_ylo, s_yhi, NB, wpi, npi, nrp, n2_base,
                                         1 + cur_y, f0, sc.iqs, J);
              if (twin)
                flush_region<F>(tw.ycnt, tw.ylo, tw.yhi, NB, wpi, npi, nrp, n2_base, 1 + cur_y,
                                f0, sc.iqs, J, true);
            }
            if (t == 0) s_nbin = 0u;
            __syncthreads();
          }
          // this warp's share of the chunk, positions [wlo, wlo + wlen) (an
          // eighth of it), in nbw batches of at most 32 candidates of even size,
          // staged in the warp's own slots c0 .. c0 + 31 (read by this warp
          // only: no block barrier)
          const int c0 = wid * 32;
          const int wlo = (wid * nc) / (kThreads / 32);
          const int wlen = ((wid + 1) * nc) / (kThreads / 32) - wlo;
          const int nbw = (wlen + 31) >> 5;
          for (int bw = 0; bw < nbw; bw++) {
          const int s0 = wlo + (bw * wlen) / nbw;
          const int nk = wlo + ((bw + 1) * wlen) / nbw - s0;  // 1 .. 32
          if (lane < nk) {
            const int p = s_pre[k] + (int)(((long long)(base + s0 + lane) * ks) % gN);
            int lo = k, hi = g;  // segment s_order[lo] with s_pre[lo] <= p < s_pre[lo+1]
            while (hi - lo > 1) {
              const int mid = (lo + hi) >> 1;
              if (s_pre[mid] <= p) lo = mid; else hi = mid;
            }
            const int sg = s_order[lo];
            const int j2 = s_seg_a[sg] + (p - s_pre[lo]);
            float4 q2 = J.f2.pos[j2];
            q2.x -= g2sx;
            q2.y -= g2sy;
            q2.z -= g2sz;
            s_pos[t] = q2;
            if (C != COREL_DD) {
              s_shp[t] = C == COREL_ED ? J.f2.shp[j2] : J.f2.ewt[j2];
              s_aux[t] = J.f2.aux[j2];
            }
            if (C == COREL_ED && has_lo) s_zlo[t] = J.f2.zlo[j2];
            s_jidx[t] = j2;
            if (auto_smem && J.auto_mode) s_orig[t] = (int)J.d2.orig[j2];
            if (JK) s_keep[t] = J.f2.keep[j2];
            if (JK && twin) s_keep2[t] = J.f1.keep[j2];
          }
          __syncwarp();

          // ---- light pass over the warp's candidates, row pass by row pass;
          // binned pairs are queued per warp and the heavy step runs whenever
          // 32 are queued (all lanes busy).  Lane l at step s takes slot
          // c0 + (s + l) mod nk, so a warp works on 32 different candidates. ----
          // row registers of pass `pass` (row slot pass * 32 + lane): the
          // shifted position and othr, the row's corels1 threshold for this image
          int pass = 0;
          float x1s, y1s, z1s;
          int othr;
#define CPC_SET_ROW()                                                         \
  {                                                                           \
    const int tr_ = pass * 32 + lane;                                         \
    const float4 p1 = s_rpos[tr_];                                            \
    x1s = sx == 1 ? p1.x - Lf : p1.x;                                         \
    y1s = sy == 1 ? p1.y - Lf : p1.y;                                         \
    z1s = sz == 1 ? p1.z - Lf : p1.z;                                         \
    othr = auto_smem ? s_rothr[(sz + 1) * kTile + tr_] : -1;                  \
  }
          CPC_SET_ROW();
          int step = 0;
          int qhead = 0, qtail = 0;
          int cr = lane % nk;  // (step + lane) mod nk, kept incrementally
          for (;;) {
            while (pass < W && (qtail - qhead) < 32) {
              const int c = c0 + cr;
              const float4 p2 = s_pos[c];
              const float dz = p2.z - z1s;
              const float dx = x1s - p2.x;
              const float dy = y1s - p2.y;
              const float m = fmaxf(fabsf(dx), fabsf(dy));
              bool binned = false, edge = false;
              // twin jobs, image 0: the order with g2 ahead of g1 (the sign of a
              // float difference is exact); a pair of a row with itself counts once
              bool canon = true, tself = false;
              if (twin && sz == 0 && !(dz > 0.0f)) {
                canon = false;
                if (dz == 0.0f) {
                  if (tie_dir > 0) {
                    canon = true;
                  } else if (tie_dir == 0) {
                    const int gi = U.g1_start + (lane * W + pass) * U.g1_stride;
                    canon = s_jidx[c] >= gi;
                    tself = s_jidx[c] == gi;
                  }
                }
              }
              if (canon && (othr < 0 || s_orig[c] > othr) && dz >= pi_out_lo &&
                  dz <= pi_out_hi && m <= xy_out) {
                if (all_exact || !(dz >= pi_in_lo && dz <= pi_in_hi && m <= xy_in)) {
                  // near the window edge: queued with a flag, the heavy step hands
                  // it to the exact FP64 evaluation of the whole pair
                  edge = true;
                } else {
                  nwin += (twin && !tself) ? 2u : 1u;
                  // r_p^2, or r^2 = r_p^2 + dz^2 for coordinates 7
                  float r2 = fmaf(dx, dx, dy * dy);
                  if (rmu) r2 = fmaf(dz, dz, r2);
                  binned = r2 >= rej_lo && r2 < rej_hi;
                }
              }
              const bool push = binned || edge;
              const unsigned bm = __ballot_sync(0xffffffffu, push);
              if (push)
                s_wq[wid][(qtail + __popc(bm & lt_mask)) & (kQCap - 1)] =
                    (unsigned)(pass * 32 + lane) | ((unsigned)c << 7) | (edge ? kEdgeFlag : 0u);
              qtail += __popc(bm);
              if (++step == nk) {  // next row pass
                step = 0;
                cr = lane % nk;
                if (++pass < W) CPC_SET_ROW();
              } else {
                cr = (cr + 1 == nk) ? 0 : cr + 1;
              }
            }
            const int avail = qtail - qhead;
            if (avail == 0) break;
            __syncwarp();
            const int take = min(avail, 32);
            if (lane < take) {
              // ---- heavy step for one queued pair ----
              const unsigned e = s_wq[wid][(qhead + lane) & (kQCap - 1)];
              const int er = e & 127, ec = (e >> 7) & 255;
              const bool edge = (e & kEdgeFlag) != 0;
              const float4 r1 = s_rpos[er];
              const float4 p2 = s_pos[ec];
              // exact bins: approximate index confirmed against the definite bands
              const float hdz = p2.z - (sz == 1 ? r1.z - Lf : r1.z);
              const float hdx = (sx == 1 ? r1.x - Lf : r1.x) - p2.x;
              const float hdy = (sy == 1 ? r1.y - Lf : r1.y) - p2.y;
              float r2 = fmaf(hdx, hdx, hdy * hdy);
              bool amb = false, own = true;
              int n2;
              if (!rmu) {
                n2 = (int)floorf(fmaf(hdz, inv_ps, tp0));
                n2 = min(max(n2, 0), npi - 1);
                if (!(hdz >= s_PA[n2] && hdz < s_PB[n2])) {
                  if (n2 > 0 && hdz >= s_PA[n2 - 1] && hdz < s_PB[n2 - 1]) n2--;
                  else if (n2 + 1 < npi && hdz >= s_PA[n2 + 1] && hdz < s_PB[n2 + 1]) n2++;
                  else amb = true;
                }
              } else {
                // coordinates 7: r = |(dx, dy, dz)|, mu = dz / r (r_mu_calc); the
                // mu bin is certain when dz is farther than mu_rel r + mu_abs from
                // both edges scaled by r.  A block holds the mu bins
                // [n2_base, n2_base + wpi): each pair belongs to the unit whose
                // slice holds its estimated bin, the others skip it
                r2 = fmaf(hdz, hdz, r2);
                const float r = sqrtf(r2);
                n2 = r2 > 0.0f ? (int)floorf(fmaf(__fdividef(hdz, r), inv_ps, tp0)) : 0;
                n2 = min(max(n2, 0), npi - 1);
                own = n2 >= n2_base && n2 < n2_base + wpi;
                const float mg = fmaf(r, mu_rel, mu_abs);
                auto in_mu = [&](int k) {
                  return hdz - s_PA[k] * r >= mg && s_PB[k] * r - hdz > mg;
                };
                if (!in_mu(n2)) {
                  if (n2 > 0 && in_mu(n2 - 1)) n2--;
                  else if (n2 + 1 < npi && in_mu(n2 + 1)) n2++;
                  else amb = true;
                }
              }
              int n1 = lin_bin ? (int)floorf((sqrtf(r2) - rmin_f) * inv_rsize_f)
                               : (int)floorf((__log2f(r2) - l2rmin2) * inv_lw);
              n1 = min(max(n1, 0), nrp - 1);
              if (!(r2 >= s_A[n1] && r2 < s_B[n1])) {
                if (n1 > 0 && r2 >= s_A[n1 - 1] && r2 < s_B[n1 - 1]) n1--;
                else if (n1 + 1 < nrp && r2 >= s_A[n1 + 1] && r2 < s_B[n1 + 1]) n1++;
                else amb = true;
              }
              const int elk = n2 - n2_base;
              if ((unsigned)elk >= (unsigned)wpi) amb = true;
              // raw (un-shifted) separation for the orientation angle
              // (angle_orient_axis_PB); coincident positions give atan(0/0) in
              // the reference: those pairs take the exact path
              // The separation is a double-float: the exact difference of the
              // float hi parts, plus the lo parts for inputs that are not
              // float32 values (renormalised); it is zero only when the
              // positions coincide.
              df32 dxr{0.f, 0.f}, dyr{0.f, 0.f};
              if (kTheta) {
                const float x2r = p2.x + g2sx, y2r = p2.y + g2sy;  // x2, y2 restored exactly
                if (has_lo) {
                  const float4 a1 = s_raux[er], a2 = s_aux[ec];
                  dxr = df_diff_hl(x2r, a2.x, r1.x, a1.x);
                  dyr = df_diff_hl(y2r, a2.y, r1.y, a1.y);
                } else {
                  dxr = two_diff(x2r, r1.x);
                  dyr = two_diff(y2r, r1.y);
                }
                if (dxr.h == 0.0f && dyr.h == 0.0f) amb = true;
              }
              // ED: the shifted separation g1 - (g2 + L*PB) (ED_calc_PB) from
              // hi + lo positions; a zero separation gives 0/0 in the reference
              float sxe = 0.f, sye = 0.f, sze = 0.f, see = 1.f;
              if (C == COREL_ED) {
                sxe = hdx;
                sye = hdy;
                sze = -hdz;
                if (has_lo) {
                  const float4 a1 = s_raux[er], a2 = s_aux[ec];
                  sxe += a1.x - a2.x;
                  sye += a1.y - a2.y;
                  sze += s_rzlo[er] - s_zlo[ec];
                }
                see = fmaf(sxe, sxe, fmaf(sye, sye, sze * sze));
                if (!(see > 0.0f)) amb = true;
              }
              // twin jobs: a row paired with itself has no other order; it takes
              // the exact path (its count is not mirrored)
              bool tself = false;
              if (twin && sx == 0 && sy == 0 && sz == 0 && hdz == 0.0f) {
                const int gi = U.g1_start + (((er & 31) * W) + (er >> 5)) * U.g1_stride;
                tself = s_jidx[ec] == gi;
                if (tself) amb = true;
              }
              if (all_exact) {
                // the comparison engine: the reference's double arithmetic for
                // every candidate (window, bins, values), global FP64 atomics.
                // With coordinates 7 every mu slice visits the pair: the window
                // count is kept from slice 0 only, the pair's values go in by the
                // slice that holds its exact mu bin
                const int64_t gi1 = (int64_t)U.g1_start +
                                    (int64_t)(((er & 31) * W) + (er >> 5)) * U.g1_stride;
                const int64_t gj2 = s_jidx[ec];
                int xn1, xn2;
                const int r = exact_classify(J, J.d1, gi1, J.d2, gj2, sx, sy, sz, xn1, xn2);
                if (r >= 1) nwin++;
                if (r == 2 && (!rmu || (xn2 >= n2_base && xn2 < n2_base + wpi))) {
                  double f[kNF];
                  exact_values(J, J.d1, gi1, J.d2, gj2, sx, sy, sz, f);
                  exact_accumulate(J, J.d1, gi1, J.d2, gj2, xn1, xn2, f);
                }
              } else if (!own) {
                // another mu slice's pair
              } else if (amb || edge) {
                // near the window edge (not yet counted) or a bin edge (window
                // counted): exact FP64 evaluation
                const int64_t gi1 = (int64_t)U.g1_start +
                                    (int64_t)(((er & 31) * W) + (er >> 5)) * U.g1_stride;
                enqueue(U.job, gi1, s_jidx[ec], edge ? code : (code | kWindowCounted), queue,
                        qcount, qcap);
                // twin jobs: the other order, (g1 = the candidate, g2 = the row)
                // at the opposite image
                if (twin && !tself) {
                  const int mcode = shift_code(-sx, -sy, -sz);
                  enqueue(U.job, s_jidx[ec], gi1, edge ? mcode : (mcode | kWindowCounted), queue,
                          qcount, qcap);
                }
              } else {
              const int lb = n1 * wpi + elk;
              // per-field terms: v (float) for every field, vd (double-float)
              // for the fields whose sums cancel (df_field)
              float v[kNF];
              df32 vd[kNF];
              // twin jobs: the other order's order-dependent terms (shape_shape)
              constexpr bool kMir = F::FA > 0;
              float vm[kMir ? kNF : 1];
              df32 vdm[kMir ? kNF : 1];
              const float w = r1.w * p2.w;
              v[0] = w;
              if (C == COREL_ED) {
                const float4 es = gws == 2 ? s_shp[ec] : s_rshp[er];
                const float dot = fmaf(es.x, sxe, fmaf(es.y, sye, es.w * sze));
                v[11] = __fdividef(dot * dot, see);
                v[12] = v[11] * v[11];
              } else if (C != COREL_DD) {
                // (w e1, w e2) hi and lo parts, the weight's lo part and phi
                const float4 ea = s_rshp[er], eb = s_shp[ec];
                const float4 xa = s_raux[er], xb = s_aux[ec];
                const DfGal g1{{ea.x, ea.z}, {ea.y, ea.w}, {r1.w, xa.w}, xa.z};
                const DfGal g2{{eb.x, eb.z}, {eb.y, eb.w}, {p2.w, xb.w}, xb.z};
                df32 c2{0.f, 0.f}, s2v{0.f, 0.f};
                float theta = 0.f;
                if (kTheta) {
                  df_cos_sin_2theta(dxr, dyr, c2, s2v);
                  if (C != COREL_SK) theta = atanf(__fdividef(dyr.h, dxr.h));
                }
                if constexpr (kMir)
                  df_pair_terms<C>(c2, s2v, theta, g1, g2, gws, J.unit_w != 0, vd, v,
                                   twin ? vdm : nullptr, twin ? vm : nullptr);
                else
                  df_pair_terms<C>(c2, s2v, theta, g1, g2, gws, J.unit_w != 0, vd, v);
              }
              // fixed-point words of the main fields, in this lane's order (even
              // lanes low word first, odd lanes high word first: red_pair); the
              // region histograms reuse them
              const bool odd_lane = (lane & 1) != 0;
              unsigned wa[F::FM], wb[F::FM];
#pragma unroll
              for (int f = 0; f < F::FM; f++) {
                const int q = F::m(f);
                unsigned lo15, hi;
                if (df_field(C, q)) df_to_fixed15(vd[q], sc.qs[q], lo15, hi);
                else f_to_fixed15(v[q], sc.qs[q], lo15, hi);
                wa[f] = odd_lane ? hi : lo15;
                wb[f] = odd_lane ? lo15 : hi;
              }
              // the main bin, or one of its copies for a hot r_p bin
              const int rep = (lane >> 1) & (kHotRep - 1);
              const int lbm = (kHotRep > 1 && n1 >= hot0 && rep != 0)
                                  ? rep_bin(rep, n1, elk, nrp, wpi) : lb;
              atomicAdd(&s_mnum[lbm], 1u);
#pragma unroll
              for (int f = 0; f < F::FM; f++)
                if (f >= f0)
                  red_pair(&s_mlo[(size_t)f * NBm + lbm], &s_mhi[(size_t)f * NBm + lbm], wa[f],
                           wb[f], odd_lane);
              if (JK) {
                // jk_check_PB (jk.cpp:64-71): the tile's region takes a same-region
                // pair and a cross-region pair whose row is kept (main - NX); the
                // partner's region takes a cross-region pair whose partner is kept
                const bool nxc = !same_region && !s_rkeep[er];
                const bool yc = !same_region && s_keep[ec];
                if (nxc) {
                  atomicAdd(&s_nxnum[lb], 1u);
#pragma unroll
                  for (int g = 0; g < F::FJ; g++)
                    if (g >= f0)
                      red_pair(&s_nxlo[(size_t)g * NB + lb], &s_nxhi[(size_t)g * NB + lb],
                               wa[F::jm(g)], wb[F::jm(g)], odd_lane);
                }
                if (yc) {
                  atomicAdd(&s_ynum[lb], 1u);
#pragma unroll
                  for (int g = 0; g < F::FJ; g++)
                    if (g >= f0)
                      red_pair(&s_ylo[(size_t)g * NB + lb], &s_yhi[(size_t)g * NB + lb],
                               wa[F::jm(g)], wb[F::jm(g)], odd_lane);
                }
              }
              if (twin) {
                // the other order (g1 = the candidate, g2 = the row): the same bin
                // count and order-independent terms (added at the flush), its
                // order-dependent terms here, and its own region attribution:
                // the tile's region takes it when the row is kept in the g2 role,
                // the partner's region when the candidate is kept in the g1 role
                unsigned xa[kMir ? F::FA : 1], xb[kMir ? F::FA : 1];
                if constexpr (kMir) {
#pragma unroll
                  for (int i = 0; i < F::FA; i++) {
                    const int q = F::m(F::a(i));
                    unsigned lo15, hi;
                    if (df_field(C, q)) df_to_fixed15(vdm[q], sc.qs[q], lo15, hi);
                    else f_to_fixed15(vm[q], sc.qs[q], lo15, hi);
                    xa[i] = odd_lane ? hi : lo15;
                    xb[i] = odd_lane ? lo15 : hi;
                    red_pair(&tw.alo[(size_t)i * NB + lb], &tw.ahi[(size_t)i * NB + lb], xa[i],
                             xb[i], odd_lane);
                  }
                }
                if (JK) {
                  const bool nxm = !same_region && !s_rkeep2[er];
                  const bool ym = !same_region && s_keep2[ec];
                  if (nxm) {
                    atomicAdd(&tw.ncnt[lb], 1u);
#pragma unroll
                    for (int g = 0; g < F::FJ; g++) {
                      if (g < f0) continue;
                      const int ap = asym_pos<F>(F::jm(g));
                      red_pair(&tw.nlo[(size_t)g * NB + lb], &tw.nhi[(size_t)g * NB + lb],
                               ap >= 0 ? xa[ap] : wa[F::jm(g)], ap >= 0 ? xb[ap] : wb[F::jm(g)],
                               odd_lane);
                    }
                  }
                  if (ym) {
                    atomicAdd(&tw.ycnt[lb], 1u);
#pragma unroll
                    for (int g = 0; g < F::FJ; g++) {
                      if (g < f0) continue;
                      const int ap = asym_pos<F>(F::jm(g));
                      red_pair(&tw.ylo[(size_t)g * NB + lb], &tw.yhi[(size_t)g * NB + lb],
                               ap >= 0 ? xa[ap] : wa[F::jm(g)], ap >= 0 ? xb[ap] : wb[F::jm(g)],
                               odd_lane);
                    }
                  }
                }
              }
              }
            }
            qhead += take;
            wbin += (unsigned)take;
            __syncwarp();
            if (pass >= W && qtail == qhead) break;
          }
          if (lane == 0 && wbin) atomicAdd(&s_nbin, wbin);
          wbin = 0;
          __syncwarp();  // every lane is done with the staged slots before restaging
          }
#undef CPC_SET_ROW
          // s_nbin complete before the next chunk's flush test
          __syncthreads();
        }
        k = g;
      }
      __syncthreads();
    }

    // ---- flush main, X and the last Y ----
    __syncthreads();
    flush_main_x<F::FM, F::FJ, F>(s_mnum, s_mlo, s_mhi, s_nxnum, s_nxlo, s_nxhi, NB, NBm, wpi, npi,
                                  nrp, n2_base, 1 + U.region, JK, f0, sc.iqs, J, tw);
    if (JK && cur_y >= 0) {
      flush_region<F>(s_ynum, s_ylo, s_yhi, NB, wpi, npi, nrp, n2_base, 1 + cur_y, f0,
                                 sc.iqs, J);
      if (twin)
        flush_region<F>(tw.ycnt, tw.ylo, tw.yhi, NB, wpi, npi, nrp, n2_base, 1 + cur_y, f0,
                        sc.iqs, J, true);
    }
    if (t == 0) s_nbin = 0u;
    // window-pair counter (once per pair: mu slices other than the first skip it)
    {
      unsigned long long v = (rmu && n2_base != 0) ? 0ull : (unsigned long long)nwin;
      for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
      if (lane == 0) s_red[wid] = v;
      __syncthreads();
      if (t == 0) {
        unsigned long long sm = 0;
        for (int w = 0; w < kThreads / 32; w++) sm += s_red[w];
        if (sm) atomicAdd(&J.counters[0], sm);
      }
    }
    __syncthreads();
  }
}

// Exact FP64 re-evaluation of the edge queue.
__global__ void recheck_kernel(const JobDev *__restrict__ jobs, const QEntry *__restrict__ queue,
                               const unsigned long long *__restrict__ qcount,
                               unsigned long long qcap) {
  const unsigned long long n = min(*qcount, qcap);
  for (unsigned long long idx = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; idx < n;
       idx += (unsigned long long)gridDim.x * blockDim.x) {
    const QEntry e = queue[idx];
    const JobDev &J = jobs[e.job];
    int sx, sy, sz, n1, n2;
    shift_decode(e.shift & kShiftMask, sx, sy, sz);
    const int r = exact_classify(J, J.d1, e.i1, J.d2, e.j2, sx, sy, sz, n1, n2);
    atomicAdd(&J.counters[2], 1ull);
    if (r == 0) continue;
    if (!(e.shift & kWindowCounted)) atomicAdd(&J.counters[1], 1ull);
    if (r == 2) {
      double f[kNF];
      exact_values(J, J.d1, e.i1, J.d2, e.j2, sx, sy, sz, f);
      exact_accumulate(J, J.d1, e.i1, J.d2, e.j2, n1, n2, f);
    }
  }
}

// ---- host-side launchers (called from capi.cu) ----
// Calls fn.run<C, JK, MINB>() for the runtime corel, jackknife flag and bound.
template <class Fn>
static auto dispatch(int corel, int jk, int minb, int twin, const Fn &fn)
    -> decltype(fn.template run<0, false, 3, false>()) {
  // twin jobs: density_density and shape_shape, 4 or 3 blocks per SM
#define CPC_TCASE(CC)                                                                 \
  if (corel == CC) {                                                                  \
    if (jk) return minb == 4 ? fn.template run<CC, true, 4, true>()                  \
                             : fn.template run<CC, true, 3, true>();                  \
    return minb == 4 ? fn.template run<CC, false, 4, true>()                          \
                     : fn.template run<CC, false, 3, true>();                         \
  }
  if (twin && minb != 1) {
    CPC_TCASE(COREL_DD)
    CPC_TCASE(COREL_SS)
    CPC_TCASE(COREL_SSA)
  }
#undef CPC_TCASE
#define CPC_CASE(CC)                                                                  \
  if (corel == CC) {                                                                  \
    if (jk) return minb == 4 ? fn.template run<CC, true, 4, false>()                 \
                  : minb == 1 ? fn.template run<CC, true, 1, false>()                 \
                              : fn.template run<CC, true, 3, false>();                \
    return minb == 4 ? fn.template run<CC, false, 4, false>()                         \
           : minb == 1 ? fn.template run<CC, false, 1, false>()                       \
                       : fn.template run<CC, false, 3, false>();                      \
  }
  CPC_CASE(COREL_DD)
  CPC_CASE(COREL_SD)
  CPC_CASE(COREL_SS)
  CPC_CASE(COREL_SSA)
  CPC_CASE(COREL_DK)
  CPC_CASE(COREL_SK)
  CPC_CASE(COREL_ED)
#undef CPC_CASE
  return fn.template run<COREL_DD, false, 3, false>();  // unreachable for valid corels
}

struct LaunchFast {
  const JobDev *jobs;
  const UnitDesc *units;
  int n_units;
  unsigned int *unit_ctr;
  QEntry *q;
  unsigned long long *qcount, qcap;
  const FastScales *sc;
  size_t smem;
  int grid;
  int auto_pairs;
  cudaStream_t st;
  template <int C, bool JK, int MINB, bool TW>
  cudaError_t run() const {
    auto kern = fast_pairs_kernel<C, JK, MINB, TW>;
    cudaError_t err =
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (err != cudaSuccess) return err;
    const int zero_words =
        (int)((smem - stage_bytes(C) - (auto_pairs ? kAutoBytes : 0)) / 4);
    kern<<<grid, kThreads, smem, st>>>(jobs, units, n_units, unit_ctr, q, qcount, qcap, *sc,
                                       zero_words, auto_pairs);
    return cudaGetLastError();
  }
};

struct Occupancy {
  size_t smem;
  template <int C, bool JK, int MINB, bool TW>
  int run() const {
    auto kern = fast_pairs_kernel<C, JK, MINB, TW>;
    int nb = 0;
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
            cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kern, kThreads, smem) != cudaSuccess)
      return 0;
    return nb;
  }
};

cudaError_t launch_fast(int corel, int jk, int minb, int twin, const JobDev *jobs,
                        const UnitDesc *units, int n_units, unsigned int *unit_ctr, QEntry *q,
                        unsigned long long *qcount, unsigned long long qcap,
                        const FastScales &sc, size_t smem, int grid, int auto_pairs,
                        cudaStream_t st) {
  if (corel < COREL_DD || corel > COREL_ED) return cudaErrorInvalidValue;
  return dispatch(corel, jk, minb, twin,
                  LaunchFast{jobs, units, n_units, unit_ctr, q, qcount, qcap, &sc, smem, grid,
                             auto_pairs, st});
}

// The register-bound variant for this shared-memory size and its blocks per SM:
// the 4-block variant when 4 blocks fit, else the 3-block one.
int fast_variant(int corel, int jk, size_t smem, int *blocks_per_sm, int all_exact, int twin) {
  if (corel < COREL_DD || corel > COREL_ED) { *blocks_per_sm = 0; return 3; }
  if (all_exact) {  // the cell-list FP64 comparison engine
    *blocks_per_sm = dispatch(corel, jk, 1, 0, Occupancy{smem});
    return 1;
  }
  const int b4 = dispatch(corel, jk, 4, twin, Occupancy{smem});
  if (b4 >= 4) { *blocks_per_sm = b4; return 4; }
  *blocks_per_sm = dispatch(corel, jk, 3, twin, Occupancy{smem});
  return 3;
}

cudaError_t launch_recheck(const JobDev *jobs, const QEntry *q, const unsigned long long *qcount,
                           unsigned long long qcap, int grid, cudaStream_t st) {
  recheck_kernel<<<grid, 256, 0, st>>>(jobs, q, qcount, qcap);
  return cudaGetLastError();
}

}  // namespace cpc

namespace cpc {
size_t fast_static_smem_bytes(int twin) {
  cudaFuncAttributes a;
  const cudaError_t e = twin ? cudaFuncGetAttributes(&a, fast_pairs_kernel<COREL_SS, true, 4, true>)
                             : cudaFuncGetAttributes(&a, fast_pairs_kernel<COREL_SS, true, 4, false>);
  if (e != cudaSuccess) return 24 * 1024;
  return a.sharedSizeBytes;
}
}  // namespace cpc
