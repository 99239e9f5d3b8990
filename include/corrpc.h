/*
 * corrpc.h -- C ABI of the GB300 pair-counting library (libcorrpc_gb300.so).
 *
 * Drop-in boundary for corr_pc's pair loop.  The reference runs one pair type
 * per call of
 *     long corels2(gal g1[], gal g2[], bin_jk &bjk, data_info &data_inf)
 *     (corr.cpp:219-459, called from do_corr.cpp:70,78,110,115,125,131)
 * selecting the pair type through data_inf.do_SD/do_SRd/do_DRs/do_RsRd/do_RsRs/
 * do_SRs.  This ABI replaces that body: the caller flattens the two gal[]
 * arrays into plain arrays (cpc_catalog), uploads them once, and calls
 * cpc_count with the same pair-type code; the library applies corels2's own
 * rules (shape-holder choice and g1/g2 swap, corr.cpp:226-296; corel choice,
 * initialization.cpp:699-752), counts on the GPU and returns the histogram
 * block, which the caller scatters into its bin_jk tree followed by the
 * delete-one conversion final_jk_bins (jk.cpp:74-81), exactly as corels2 ends.
 *
 * Conventions: plain pointers and sizes only; every entry point returns a
 * cpc_status and never aborts; cpc_last_error() gives a message.  One context
 * per host thread; a context owns all its device memory.  Host arrays are
 * copied (never aliased after the call returns).
 */
#ifndef CORRPC_H
#define CORRPC_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  CPC_OK = 0,
  CPC_ERR_INVALID = 1,     /* bad argument or unsupported configuration */
  CPC_ERR_CUDA = 2,        /* CUDA runtime error (message in cpc_last_error) */
  CPC_ERR_NOMEM = 3,       /* device or host allocation failed */
  CPC_ERR_TIMEOUT = 4,     /* a bounded device wait gave up */
  CPC_ERR_STATE = 5,       /* call order (e.g. count before upload) */
  CPC_ERR_RANGE = 6,       /* data out of range (jackknife label, NaN position) */
  CPC_ERR_NODEVICE = 7,    /* no CUDA device */
  CPC_ERR_HOST = 8         /* other host-side failure (e.g. a thread could not start) */
} cpc_status;

/* pair type: the data_info.do_* flag set around each corels2 call
 * (do_corr.cpp:61-131) */
typedef enum {
  CPC_PAIR_SD = 0,   /* do_SD   : corels2(gdensity, gshape, ...)        */
  CPC_PAIR_SRD = 1,  /* do_SRd  : corels2(grand_density, gshape, ...)   */
  CPC_PAIR_DRS = 2,  /* do_DRs  : corels2(grand_shape, gdensity, ...)   */
  CPC_PAIR_RSRD = 3, /* do_RsRd : corels2(grand_density, grand_shape)   */
  CPC_PAIR_RSRS = 4, /* do_RsRs : corels2(grand_shape, grand_shape)     */
  CPC_PAIR_SRS = 5,  /* do_SRs  : corels2(grand_shape, gshape, ...)     */
  CPC_PAIR_SS = 6    /* do_SS   : corels1(gshape, ...) (cpc_count_auto only) */
} cpc_pair_kind;

/* which kernel counts the pairs */
typedef enum {
  CPC_ENGINE_FAST = 0,      /* FP32 cell-list kernel with FP64 recheck near edges */
  CPC_ENGINE_FP64 = 1,      /* plain all-FP64 kernel: one thread per g1 row      */
  CPC_ENGINE_CELL_FP64 = 2  /* the fast kernel's cell list and work units, every
                               window candidate evaluated by the FP64 path (box
                               cross counts, cpc_count only): the precision
                               comparison at equal algorithm                     */
} cpc_engine;

/* Parameters: the data_info fields the pair loop reads (data_def.h:46-96),
 * with the values data_ini computes (initialization.cpp:62-352). */
typedef struct {
  int which_corr;    /* 0 wgg, 1 wg+, 2 w++, 3 kappa-density, 4 shape-kappa,
                        5 ED (cos^2 of the 3-D orientation angle); 3-5 box only */
  int coordinates;   /* 6: x,y,z (r_p, Pi); 7: x,y,z (r, mu; periodic box);
                        0: sky ra,dec,z (r_p, Pi) */
  int estimator;     /* 0..3 (affects the shape-shape accumulators only) */
  int periodic_box;  /* 1: periodic images (coordinates 6 only) */
  int data_sorted;   /* 0/1: as in the .inp (results follow set semantics) */
  int do_jk;         /* 0 or 1 (1 = delete-one jackknife) */
  int n_jk;          /* number of jackknife regions (labels 0..n_jk-1) */
  int sig_crit;      /* must be 0 (lensing weights are not supported) */
  int rand_subsample;/* must be 0 */
  int n_bins;        /* r_p bins */
  int lin_bin;       /* 1 linear, 0 log10 */
  int n_p_bin;       /* Pi bins (mu bins for coordinates 7, p_min..p_max in mu) */
  double bin_r_min, bin_r_max;
  double p_min, p_max;
  double periodic_box_size;
  /* sky only (coordinates 0): */
  double z_max, dz, z_sep_max;
  const double *H_z;   /* distance table columns as read by da_Z */
  const double *dA_z;  /* (initialization.cpp:23-60), n_table entries */
  int64_t n_table;
} cpc_params;

/* One catalogue: the gal[] fields the pair loop reads (data_def.h:23-44),
 * flattened.  Box: x,y,z = ra.val_deg, dec.val_deg, redshift.  Sky: x = RA
 * degrees, y = Dec degrees, z = redshift, plus dc/da.  Optional arrays may be
 * NULL: w (weights 1), e1/e2 (no shapes: treated as 0), phi (-10, the
 * reference's value for galaxies read without e), jk (required when do_jk),
 * jk_prob (0), dc/da (sky only), e3 (0).  which_corr 3 and 4 read kappa into
 * e[0] (read_dat.cpp:300-304): pass it as e1 (e2 may be NULL then); which_corr 5
 * reads a 3-D orientation normalised to unit length (read_dat.cpp:282-293):
 * pass it as e1, e2, e3. */
typedef struct {
  int64_t n;
  const double *x, *y, *z;
  const double *w;
  const double *e1, *e2;
  const double *phi;
  const int32_t *jk;
  const double *jk_prob;
  const double *dc, *da;
  const double *e3;
} cpc_catalog;

#define CPC_NF 13 /* wt_num, data[1..6].val, data[1..6].err interleaved */

/* Histogram block written by cpc_count (caller-owned host memory):
 *   num [n_hist][n_bins][n_p_bin]            p_bin.num      (int64)
 *   sums[n_hist][n_bins][n_p_bin][CPC_NF]    p_bin.wt_num, data[j].val/.err
 * field f: 0 wt_num; 1+2(j-1) data[j].val; 2+2(j-1) data[j].err (j = 1..6).
 * h = 0 is the full sample; h = 1+r is the RAW sum over pairs attributed to
 * jackknife region r (jk.cpp:138-171), before the delete-one conversion.
 * n_hist = 1 + (do_jk ? n_jk : 0).  The 1-D r_p count b[i].num is the sum of
 * num over the Pi bins. */
typedef struct {
  int64_t *num;
  double *sums;
  int64_t n_window;   /* corels2 "total pair"  (window pairs) */
  int64_t n_binned;   /* corels2 "pairs in"    (its return value) */
  int64_t n_rechecked;/* pairs resolved on the FP64 edge path (diagnostic) */
  double kernel_ms;   /* device time of the whole count (zeroing, pair kernel, recheck) */
  double pair_kernel_ms; /* device time of the pair-kernel launch(es) alone */
} cpc_accum;

typedef struct cpc_ctx cpc_ctx;

/* Library version string. */
const char *cpc_version(void);

/* Create a context on the current CUDA device.  Validates params. */
cpc_status cpc_create(cpc_ctx **ctx, const cpc_params *params);

/* Destroy a context and free its device memory (NULL is a no-op). */
cpc_status cpc_destroy(cpc_ctx *ctx);

/* Message for the last failing call on ctx, or, for ctx NULL, of the calling
 * thread's last failing call (any entry point).  The pointer stays valid until
 * the next call on ctx (for NULL: the thread's next failing call). */
const char *cpc_last_error(const cpc_ctx *ctx);

/* Copy a catalogue into slot `slot` (0..7) and build its on-device cell list
 * (radix sort by (column, region, z)).  Replaces any previous catalogue in the
 * slot.  Validates labels (0 <= jk < n_jk when do_jk) and finite positions. */
cpc_status cpc_upload(cpc_ctx *ctx, int slot, const cpc_catalog *cat);

/* Count one pair type between the catalogues in slots slot_g1, slot_g2 --
 * the two arrays corels2 receives, in its argument order -- and write the
 * histogram block into *out (arrays sized by the caller, see cpc_accum).
 * row_stride/row_offset > 1 restrict the outer loop to rows whose original
 * index i (after the swap rule) has (i - row_offset) % row_stride == 0
 * (1, 0 = all rows).  Synchronous. */
cpc_status cpc_count(cpc_ctx *ctx, cpc_pair_kind kind, int slot_g1, int slot_g2,
                     cpc_engine engine, int64_t row_stride, int64_t row_offset,
                     cpc_accum *out);

/* Asynchronous form of cpc_count for box runs (coordinates 6 and 7): plans the
 * count and enqueues its kernels after the work already queued on `stream` (a
 * cudaStream_t; NULL is the legacy default stream), makes later work on
 * `stream` wait for it, and returns without waiting.  cpc_count_finish then
 * waits, writes the histogram block into *out and returns the status; no other
 * call on ctx may come in between (they return CPC_ERR_STATE).  Sky counts
 * (coordinates 0) finish on the host and are only available through cpc_count.
 * Extends the reference's synchronous corels2 for callers that overlap the
 * count with their own GPU work. */
cpc_status cpc_count_async(cpc_ctx *ctx, cpc_pair_kind kind, int slot_g1, int slot_g2,
                           cpc_engine engine, int64_t row_stride, int64_t row_offset,
                           void *stream);
cpc_status cpc_count_finish(cpc_ctx *ctx, cpc_accum *out);

/* Auto pairs of one catalogue: the reference's
 *     long corels1(gal g1[], bin_jk &bjk, data_info &data_inf)
 *     (corr.cpp:103-216; do_corr.cpp:63 with do_SS, :76 with do_RsRs)
 * for the catalogue in slot `slot`, kind CPC_PAIR_SS or CPC_PAIR_RSRS.  Each
 * pair is taken once by input order (row i with rows j > i), except that with
 * data_sorted 1 the +1 z image of a periodic box pairs row i with every row,
 * and an image whose first scanned row fails the lower redshift bound adds
 * nothing (the reference's sorted scan).  data_sorted 1 expects input sorted
 * by z, as the reference does.  Same output block as cpc_count. */
cpc_status cpc_count_auto(cpc_ctx *ctx, cpc_pair_kind kind, int slot, cpc_engine engine,
                          int64_t row_stride, int64_t row_offset, cpc_accum *out);

/* Histogram shape for this context: n_hist, n_bins, n_p_bin. */
cpc_status cpc_accum_shape(const cpc_ctx *ctx, int *n_hist, int *n_bins, int *n_p_bin);

/* Batched counting: run n_jobs pair types, possibly on different contexts
 * (e.g. many periodic sub-boxes), in ONE persistent launch of the fast
 * kernel that drains a single device work queue.  ctxs[k], kinds[k],
 * slots_g1[k], slots_g2[k] and outs[k] describe job k.  All contexts must
 * live on the current device.  Sky jobs (coordinates 0) that share one
 * context -- the SRd, RsRd, SD and DRs terms of a sky run, do_corr.cpp:103-131
 * -- run in one launch of the fast sky kernel, whose blocks take chunks of
 * each term's outer rows in turn; sky jobs on several contexts run one launch
 * each.  Synchronous. */
cpc_status cpc_count_batch(int n_jobs, cpc_ctx *const *ctxs, const cpc_pair_kind *kinds,
                           const int *slots_g1, const int *slots_g2, cpc_accum *outs);

/* Tuning knobs of the fast kernel (0 = automatic).  cells_per_rmax: column
 * width = r_max / k, k <= 9; pi_window: Pi bins held per block; tile: g1 rows
 * per block (0 or 128). */
cpc_status cpc_set_tuning(cpc_ctx *ctx, int cells_per_rmax, int pi_window, int tile);

/* Autotuner: times the fast kernel on every `sample_stride`-th work unit (a
 * unit shard: whole tiles of outer rows, so per-unit costs are those of the
 * full count; twin counts run as twins) of this pair type, the faster of two
 * timed runs per candidate, for cell widths r_max / k (k = 2 .. 6; the cell lists are
 * rebuilt on the device) and block-local Pi windows (for 4, 3 and 2 blocks per
 * SM, the largest window that fits and three quarters of it), keeps the
 * fastest for this context (as cpc_set_tuning would) and returns it.  Results
 * never depend on the choice.  With coordinates 7 (r-mu) only the cell width is
 * tuned and pi_window returns 0 (the mu window stays automatic).  Box runs only
 * (sky runs return zeros). */
cpc_status cpc_autotune(cpc_ctx *ctx, cpc_pair_kind kind, int slot_g1, int slot_g2,
                        int64_t sample_stride, int *cells_per_rmax, int *pi_window);

/* Autotuner of a batch (the jobs of cpc_count_batch, box runs with one binning
 * and which_corr): the same cell widths and Pi windows, each trial one batched
 * launch over every `sample_stride`-th work unit of every job; the fastest is
 * kept for every context of the batch and returned.  No counterpart in the
 * reference (its sub-boxes are separate runs, corr.cpp:219). */
cpc_status cpc_autotune_batch(int n_jobs, cpc_ctx *const *ctxs, const cpc_pair_kind *kinds,
                              const int *slots_g1, const int *slots_g2, int64_t sample_stride,
                              int *cells_per_rmax, int *pi_window);

/* Work sharding over GPUs (replaces the reference's division of the outer
 * rows over OpenMP threads, corr.cpp:299-302 and 329-424): later
 * fast-engine box counts on ctx (cpc_count, cpc_count_async, cpc_count_auto,
 * cpc_count_batch) process only the work units i with i % n_shards == shard.
 * A unit is a tile of outer rows against one slice of its candidates, and the
 * units partition the pairs, so the RAW blocks of shards 0 .. n_shards-1 (one
 * per GPU, each on its own context with the same catalogues) sum to the whole
 * count: counts exactly, sums up to the order of FP64 additions.  Unlike
 * row_stride, whose skipped rows still pass through every unit, each shard does
 * about 1/n_shards of the work.  Fast sky counts take the outer rows at
 * redshift-ordered positions k with k % n_shards == shard (the shards again
 * partition the pairs); the FP64 engine shards by rows (row_stride /
 * row_offset), which it skips cheaply.  Default: shard 0 of 1. */
cpc_status cpc_set_shard(cpc_ctx *ctx, int shard, int n_shards);

/* Number of GPU kernels this context has launched so far (all entry points;
 * for a batch, counted on the first job's context). */
cpc_status cpc_launch_count(const cpc_ctx *ctx, int64_t *launches);

/* CUDA graphs of the fast box engine (no counterpart in the reference, whose
 * pair loop is an OpenMP loop on the host).  A fast count -- cpc_count,
 * cpc_count_async, cpc_count_auto, cpc_count_batch (on the first job's
 * context) -- zeroes its histogram blocks, runs one persistent pair-kernel
 * launch per corel group and the FP64 recheck.  The context captures that
 * device work once into a CUDA graph and replays it on later counts whose
 * launches are the same (same buffers, queue capacity, unit ranges, grids and
 * shared memory; the job descriptors and work units are copied in before each
 * replay), capturing again when any of them changes.  Results do not depend on
 * it.  Enabled by default; cpc_set_graph_replay(ctx, 0) launches directly.  If
 * a capture fails the context falls back to direct launches. */
cpc_status cpc_set_graph_replay(cpc_ctx *ctx, int enable);

/* Graph captures and replays of this context's fast counts so far. */
cpc_status cpc_graph_stats(const cpc_ctx *ctx, int64_t *captures, int64_t *replays);

/* Twin counts (no counterpart in the reference; results do not depend on it):
 * a fast box count over every outer row of two slots that hold the same
 * galaxies in the same order -- positions, weights, shapes, regions and input
 * rows equal, as when the S and D samples of a cross term read the same files
 * -- with a density_density or shape_shape accumulator and a Pi binning
 * symmetric about 0, tests each unordered pair once and adds both orders
 * (g1 = i, g2 = j) and (g1 = j, g2 = i), each with its own keep flags and
 * order-dependent terms.  cpc_set_twin(ctx, 0) counts every order separately
 * (default 1; CPC_TWIN=0 in the environment at cpc_create does the same);
 * cpc_last_twin reports whether the context's last fast count ran so. */
cpc_status cpc_set_twin(cpc_ctx *ctx, int enable);
cpc_status cpc_last_twin(const cpc_ctx *ctx, int *twin);

/* ---- host helpers of the reference's read path (no GPU needed) ---- */

/* glibc rand() stream after srand(seed): out[i] = rand_{skip+i}() /
 * (RAND_MAX + 1.) (read_dat.cpp:243, 320; seed 124693517 per jk.cpp:40-43). */
cpc_status cpc_host_rand_uniform(uint32_t seed, int64_t skip, int64_t n, double *out);

/* phi = 0.5 * arctan(e1, -e2) with the reference's quadrant rule, NaN -> 0
 * (elip_angle, calcs.cpp:73-83). */
cpc_status cpc_host_elip_angle(int64_t n, const double *e1, const double *e2, double *phi);

/* The exact r_p bin thresholds the library uses: thr[k] = smallest double r
 * with floor(log10(r/r_min)/r_size) >= k (log bins) or the linear analogue,
 * k = 0..n_bins (corels.cpp:41-44).  thr has n_bins+1 entries. */
cpc_status cpc_host_rp_thresholds(const cpc_params *params, double *thr);

/* The exact Pi bin thresholds: thr[k] = smallest double Pi with
 * floor((Pi - p_min)/p_size) >= k, k = 0..n_p_bin (corels.cpp:26). */
cpc_status cpc_host_pi_thresholds(const cpc_params *params, double *thr);

/* Finalisation of a cross-correlation run (do_corr.cpp:203-433: final_calc,
 * int_calc, jk_final, analytic periodic RR) and its output files, written
 * with the .inp's out_file prefix, from the RAW histogram blocks of the four
 * pair types (cpc_accum layout; NULL = empty term; the delete-one conversion
 * is applied here).  weights: S_wt, S_wt2, D_wt, D_wt2, Rs_wt, Rs_wt2, Rd_wt,
 * Rd_wt2 (sums of w and w^2 per sample, as read_data accumulates them). */
cpc_status cpc_host_finalize_cross(const char *inp_path, const int64_t *sd_num,
                                   const double *sd_sums, const int64_t *srd_num,
                                   const double *srd_sums, const int64_t *drs_num,
                                   const double *drs_sums, const int64_t *rsrd_num,
                                   const double *rsrd_sums, const double *weights);

/* Finalisation of an auto-correlation run (do_corr.cpp:220-324: re_bin for
 * estimators 2 and 3, final_calc_auto, int_calc, jk_final) and its bins_auto_*
 * output files, from the RAW blocks of SS (corels1), SRs and RsRs (NULL = empty
 * term; the delete-one conversion is applied here).  weights as for
 * cpc_host_finalize_cross (S and Rs totals are used). */
cpc_status cpc_host_finalize_auto(const char *inp_path, const int64_t *ss_num,
                                  const double *ss_sums, const int64_t *srs_num,
                                  const double *srs_sums, const int64_t *rsrs_num,
                                  const double *rsrs_sums, const double *weights);

/* ---- counting without any GPU allocation (no counterpart in the reference) ----
 *
 * For callers that cannot allocate GPU memory themselves -- code embedded in a
 * host application or framework that owns every device allocation, runs a
 * memory pool that forbids cudaMalloc after start-up, or must not grow the
 * device footprint -- this entry point counts one pair type with the plain
 * FP64 kernel and allocates nothing: the inputs and outputs are the caller's
 * device buffers, and the kernel's scratch (job descriptor with the exact bin
 * thresholds, pair counters, an input-order flag) lives in a fixed 16 KiB
 * array inside the library, resident on every device that loads it until the
 * process exits.
 *
 *  - g1/g2: device arrays as corels2 receives them (same rules: swap when g2
 *    is larger, shape holder, corel choice); after the swap the scanned
 *    catalogue must be sorted by z (checked; CPC_ERR_INVALID otherwise), as
 *    the reference requires for data_sorted 1.  NULL optional arrays as in
 *    cpc_catalog; jk_prob replaces the host-side keep flags and is required
 *    with do_jk (CPC_ERR_INVALID otherwise).
 *  - d_num / d_sums: device buffers laid out as cpc_accum's num / sums (raw
 *    region sums); zeroed by the call.  n_window / n_binned: host outputs.
 *  - limits: coordinates 6, which_corr 0-2, n_bins <= 64, n_p_bin <= 128 (the
 *    scratch holds the thresholds), catalogue sizes < 2^31, and every check
 *    cpc_create applies; other values are rejected with CPC_ERR_INVALID and a
 *    message.
 *  - the first call on a device looks up the scratch array's device address
 *    (with that device current) and keeps it for later calls; make that first
 *    call before any stream capture.  A device reset (cudaDeviceReset) between
 *    calls is not supported: the kept address would no longer be valid.  The
 *    call synchronises `stream` (a cudaStream_t, NULL = legacy default
 *    stream).
 *  - every call on a device shares the one scratch array and leaves its
 *    contents behind; calls are safe one after another, but calls that overlap
 *    on the GPU race on it and must be serialised by the caller.
 *  - errors: a message is written to err (err_len bytes) if err is not NULL. */
typedef struct {
  int64_t n;
  const double *x, *y, *z;
  const double *w;
  const double *e1, *e2;
  const double *phi;
  const int32_t *jk;
  const double *jk_prob;
} cpc_device_catalog;

#define CPC_NOALLOC_SCRATCH_BYTES 16384

cpc_status cpc_count_fp64_noalloc(const cpc_params *params, cpc_pair_kind kind,
                                  const cpc_device_catalog *g1, const cpc_device_catalog *g2,
                                  int64_t *d_num, double *d_sums, int64_t *n_window,
                                  int64_t *n_binned, void *stream, char *err, size_t err_len);

#ifdef __cplusplus
}
#endif
#endif /* CORRPC_H */
