// kernels.h -- host-callable launchers of the device code.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "cpc_device.cuh"

namespace cpc {

struct GatherIn {
  const double *x, *y, *z, *w, *e1, *e2, *phi;
  const int32_t *jk;
  const uint8_t *keep;
  const double *e3;
};
struct GatherOut {
  float4 *pos, *shp;  // null for the z-ordered (FP64) copy; shp = (e1, e2, phi, e3)
  float4 *ewt;        // (w e1, w e2) hi parts, then their lo parts
  float4 *aux;        // x lo, y lo, phi, w lo
  float *zlo;
  float *zf;
  uint32_t *bucket;   // null for the z-ordered copy
  double *x, *y, *z, *w, *e1, *e2, *phi, *e3;
  int32_t *jk;
  uint8_t *keep;
  int64_t *orig;
  const int64_t *orig_in;  // when set, orig[k] = orig_in[perm[k]]
};

// cell_list.cu
cudaError_t radix_sort_pairs(int64_t n, uint64_t *keys, uint32_t *vals, uint64_t *ktmp,
                             uint32_t *vtmp, uint32_t *hist, unsigned long long *census_d,
                             cudaStream_t st, int64_t *launches);
int64_t radix_hist_words(int64_t n);
cudaError_t launch_cell_keys(int64_t n, const double *x, const double *y, const double *z,
                             const int32_t *jk, double inv_cw_x, double inv_cw_y, int ncx, int ncy,
                             int n_reg, uint64_t *keys, uint32_t *vals, cudaStream_t st);
cudaError_t launch_z_keys(int64_t n, const double *z, uint64_t *keys, uint32_t *vals,
                          cudaStream_t st);
cudaError_t launch_gather(int64_t n, const uint64_t *keys, const uint32_t *perm, const GatherIn &in,
                          const GatherOut &out, cudaStream_t st);

cudaError_t launch_gather_u8(int64_t n, const uint32_t *perm, const uint8_t *in, uint8_t *out,
                             cudaStream_t st);
// *differ |= 1 when the n bytes at a and b differ (device memory, 4-byte aligned)
cudaError_t launch_bytes_differ(const void *a, const void *b, int64_t n, unsigned *differ,
                                cudaStream_t st);

// Checks and derived per-row data of a box catalogue (input order), on the
// device: the first failing row of each check, the statistics the error bounds
// and fixed-point scales need, the keep flags and the corels1 scan starts.
struct UploadStats {
  unsigned long long bad_row[4];  // first row: 0 non-finite position, 1 outside
                                  // [0, L], 2 non-finite w/e/phi, 3 label range
  unsigned long long cmax_bits, wmax_bits, emax_bits, phimax_bits;  // non-negative
  unsigned long long wmin_key;    // orderable key of min w
  unsigned int not_f32;           // a position is not a float32 value
};
struct PrepIn {
  int64_t n;
  const double *x, *y, *z, *w, *e1, *e2, *phi, *jk_prob;  // w, e1, e2, phi, jk_prob may be null
  const double *e3;   // may be null
  const int32_t *jk;  // null without jackknife
  double L, wz_lo;    // box size, lower z-window offset (p_min, or -r_max for coordinates 7)
  int n_jk;
};
cudaError_t launch_fill_f64(int64_t n, double v, double *out, cudaStream_t st);
cudaError_t launch_prep_catalog(const PrepIn &in, uint8_t *keep, uint8_t *aflag,
                                UploadStats *stats, cudaStream_t st);
unsigned long long orderable_key(double v);
double from_orderable_key(unsigned long long k);

// pair_fast.cu
constexpr int kTileThreads = 128;  // g1 rows per tile (a warp tests them in passes of 32)
constexpr int kFastBlocksPerSM = 4;  // occupancy target: registers and shared memory sized for it
// Per work unit: at most kFastMaxCols neighbour columns (the host rejects units
// with more; (2k + 3)^2 columns for cells r_max / k wide, so k <= 9) and
// candidate slots taken kFastMaxSeg at a time.
constexpr int kFastMaxCols = 512;
constexpr int kFastMaxSeg = 256;
constexpr int kMaxCellsPerRmax = 9;
// auto_pairs: the launch holds corels1 (auto-pair) jobs, whose rules take
// another kBatch + 3 kTile ints of shared memory
size_t fast_smem_bytes(int corel, int do_jk, int nrp, int wpi, int auto_pairs, int unit_w,
                       int twin);
size_t fast_static_smem_bytes(int twin);
// minb 4 or 3: the register bound (blocks per SM) of the fast kernel; 1: the
// cell-list FP64 comparison engine (all_exact jobs).  twin: the twin kernels
// (density_density and shape_shape jobs whose slots hold the same galaxies)
int fast_variant(int corel, int jk, size_t smem, int *blocks_per_sm, int all_exact, int twin);
// Fixed-point scales of one fast-kernel launch (kernel parameters, read from
// the constant bank): field f's terms are rint(v qs[f]), summed back with
// iqs[f] = 1 / qs[f].  A launch over several jobs takes, per field, the smallest
// of the jobs' scales (all powers of two), which keeps every job's terms within
// their bound.
struct FastScales {
  float qs[kNF];
  double iqs[kNF];
};
cudaError_t launch_fast(int corel, int jk, int minb, int twin, const JobDev *jobs,
                        const UnitDesc *units, int n_units, unsigned int *unit_ctr, QEntry *q,
                        unsigned long long *qcount, unsigned long long qcap,
                        const FastScales &sc, size_t smem, int grid, int auto_pairs,
                        cudaStream_t st);
cudaError_t launch_recheck(const JobDev *jobs, const QEntry *q, const unsigned long long *qcount,
                           unsigned long long qcap, int grid, cudaStream_t st);

// pair_fp64.cu
cudaError_t launch_plain_fp64(const JobDev *job, const DCat &a, const DCat &b, cudaStream_t st);

// pair_sky.cu
// Sky pairs (coordinates 0) in FP64; pairs whose r_p may bin differently with
// the C library's trigonometry are appended to hq (host edge tier).
constexpr unsigned long long kSkyHostQueue = 1ull << 22;
// (SkyFast, the float views of a sky catalogue, is declared in cpc_device.cuh)
// The fast sky kernel over n_jobs jobs (pair types) in one launch: job k's rows
// are dealt in chunks chunk0[k] .. chunk0[k+1]-1 of rows_per_chunk rows;
// chunk_ctr (zeroed) is the chunk queue.  Every job has the same binning.
// blocks_per_sm: the register bound the kernel is compiled for (2 or 3).
cudaError_t launch_sky_warp(const JobDev *jobs, const long long *chunk0, int n_jobs,
                            long long n_chunks, int rows_per_chunk,
                            unsigned long long *chunk_ctr, unsigned long long hq_cap, double esum,
                            float rp_lo_f, float rp_hi_f, int zero_bin, int nrp, int npi,
                            int sm_count, int blocks_per_sm, cudaStream_t st);
cudaError_t launch_fix_to_sums(int64_t n, const unsigned long long *lo,
                               const unsigned long long *hi, double *sums, const JobDev *job,
                               cudaStream_t st);
cudaError_t launch_sky_fp64(const JobDev *job, const SkyView &a, const SkyView &b, int2 *hq,
                            unsigned long long *hq_n, unsigned long long hq_cap, double esum,
                            cudaStream_t st);

}  // namespace cpc
