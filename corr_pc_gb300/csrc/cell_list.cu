// cell_list.cu -- on-device cell list: key computation, LSD radix sort and
// the gather into the cell-ordered structure-of-arrays the pair kernels read.
//
// Key of a point = (bucket << 32) | orderable(float z), bucket = column (x, y
// grid of width ~ r_max / k) * n_regions + jackknife region.  Sorting by this
// key gives every (column, region) bucket as a contiguous, z-sorted range.
//
// The radix sort is a stable least-significant-digit sort with 8-bit digits:
// per-block digit histograms, one exclusive scan over (digit, block), and a
// stable scatter that ranks equal digits inside a block with warp match masks.
// Digit positions whose digit is the same for every key are skipped.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cstring>

#include "kernels.h"

namespace cpc {

constexpr int kSortThreads = 256;
constexpr int kSortItems = 16;  // keys per thread per block
constexpr int kSortBlockKeys = kSortThreads * kSortItems;

__device__ __forceinline__ uint32_t orderable_f32(float f) {
  const uint32_t u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ uint64_t orderable_f64(double d) {
  const uint64_t u = (uint64_t)__double_as_longlong(d);
  return (u & 0x8000000000000000ull) ? ~u : (u | 0x8000000000000000ull);
}

__global__ void cell_keys_kernel(int64_t n, const double *__restrict__ x, const double *__restrict__ y,
                                 const double *__restrict__ z, const int32_t *__restrict__ jk,
                                 double inv_cw_x, double inv_cw_y, int ncx, int ncy, int n_reg,
                                 uint64_t *__restrict__ keys, uint32_t *__restrict__ vals) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int cx = (int)floor(x[i] * inv_cw_x), cy = (int)floor(y[i] * inv_cw_y);
  cx = min(max(cx, 0), ncx - 1);
  cy = min(max(cy, 0), ncy - 1);
  const int r = (n_reg > 1 && jk) ? jk[i] : 0;
  const uint64_t bucket = (uint64_t)(cy * ncx + cx) * (uint64_t)n_reg + (uint64_t)r;
  keys[i] = (bucket << 32) | orderable_f32((float)z[i]);
  vals[i] = (uint32_t)i;
}

__global__ void z_keys_kernel(int64_t n, const double *__restrict__ z, uint64_t *__restrict__ keys,
                              uint32_t *__restrict__ vals) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  keys[i] = orderable_f64(z[i]);
  vals[i] = (uint32_t)i;
}

// all-positions digit histogram: hist8[pos][digit]
__global__ void digit_census_kernel(int64_t n, const uint64_t *__restrict__ keys,
                                    unsigned long long *__restrict__ hist8) {
  __shared__ unsigned int h[8][256];
  for (int k = threadIdx.x; k < 8 * 256; k += blockDim.x) (&h[0][0])[k] = 0u;
  __syncthreads();
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t k = keys[i];
#pragma unroll
    for (int p = 0; p < 8; p++) atomicAdd(&h[p][(k >> (8 * p)) & 0xff], 1u);
  }
  __syncthreads();
  for (int k = threadIdx.x; k < 8 * 256; k += blockDim.x) {
    const unsigned int v = (&h[0][0])[k];
    if (v) atomicAdd(&hist8[k], (unsigned long long)v);
  }
}

__global__ void radix_hist_kernel(int64_t n, const uint64_t *__restrict__ keys, int shift,
                                  uint32_t *__restrict__ hist, int nblocks) {
  __shared__ unsigned int h[256];
  h[threadIdx.x] = 0u;
  __syncthreads();
  const int64_t base = (int64_t)blockIdx.x * kSortBlockKeys;
  for (int r = 0; r < kSortItems; r++) {
    const int64_t i = base + (int64_t)r * kSortThreads + threadIdx.x;
    if (i < n) atomicAdd(&h[(keys[i] >> shift) & 0xff], 1u);
  }
  __syncthreads();
  hist[(int64_t)threadIdx.x * nblocks + blockIdx.x] = h[threadIdx.x];
}

// exclusive scan of `total` uint32 values, single block of 1024 threads
__global__ void scan_kernel(uint32_t *__restrict__ data, int64_t total) {
  __shared__ uint32_t part[1024];
  const int t = threadIdx.x;
  const int64_t per = (total + 1023) / 1024;
  const int64_t b = t * per, e = min(total, b + per);
  uint32_t s = 0;
  for (int64_t i = b; i < e; i++) s += data[i];
  part[t] = s;
  __syncthreads();
  for (int off = 1; off < 1024; off <<= 1) {  // Hillis-Steele inclusive scan
    const uint32_t v = t >= off ? part[t - off] : 0u;
    __syncthreads();
    part[t] += v;
    __syncthreads();
  }
  uint32_t run = t ? part[t - 1] : 0u;
  for (int64_t i = b; i < e; i++) {
    const uint32_t v = data[i];
    data[i] = run;
    run += v;
  }
}

__global__ void radix_scatter_kernel(int64_t n, const uint64_t *__restrict__ kin,
                                     const uint32_t *__restrict__ vin, uint64_t *__restrict__ kout,
                                     uint32_t *__restrict__ vout, int shift,
                                     const uint32_t *__restrict__ hist, int nblocks) {
  __shared__ uint32_t s_base[256], s_tot[256];
  __shared__ uint32_t s_wcnt[kSortThreads / 32][256];
  __shared__ uint32_t s_wpre[kSortThreads / 32][256];
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  s_base[t] = hist[(int64_t)t * nblocks + blockIdx.x];
  for (int w = 0; w < kSortThreads / 32; w++) s_wcnt[w][t] = 0u;
  __syncthreads();
  const unsigned lt_mask = (1u << lane) - 1u;
  const int64_t base = (int64_t)blockIdx.x * kSortBlockKeys;
  for (int r = 0; r < kSortItems; r++) {
    const int64_t i = base + (int64_t)r * kSortThreads + t;
    const bool ok = i < n;
    uint64_t k = 0;
    uint32_t v = 0;
    int d = 256;  // sentinel digit for lanes past the end
    if (ok) {
      k = kin[i];
      v = vin[i];
      d = (int)((k >> shift) & 0xff);
    }
    const unsigned peers = __match_any_sync(0xffffffffu, d);
    const int rank = __popc(peers & lt_mask);
    if (ok && rank == 0) s_wcnt[warp][d] = (uint32_t)__popc(peers);
    __syncthreads();
    {
      uint32_t run = 0;
      for (int w = 0; w < kSortThreads / 32; w++) {
        const uint32_t c = s_wcnt[w][t];
        s_wpre[w][t] = run;
        run += c;
        s_wcnt[w][t] = 0u;
      }
      s_tot[t] = run;
    }
    __syncthreads();
    if (ok) {
      const uint32_t dst = s_base[d] + s_wpre[warp][d] + (uint32_t)rank;
      kout[dst] = k;
      vout[dst] = v;
    }
    __syncthreads();
    s_base[t] += s_tot[t];
    __syncthreads();
  }
}

// Sort (keys, vals) in place (results end in keys/vals).  Scratch: ktmp, vtmp
// (n each), hist (256 * nblocks uint32), census (8*256 u64, device) and a
// host census buffer.
cudaError_t radix_sort_pairs(int64_t n, uint64_t *keys, uint32_t *vals, uint64_t *ktmp,
                             uint32_t *vtmp, uint32_t *hist, unsigned long long *census_d,
                             cudaStream_t st, int64_t *launches) {
  if (n <= 1) return cudaSuccess;
  *launches += 1;
  cudaError_t err = cudaMemsetAsync(census_d, 0, sizeof(unsigned long long) * 8 * 256, st);
  if (err != cudaSuccess) return err;
  digit_census_kernel<<<152 * 4, 256, 0, st>>>(n, keys, census_d);
  unsigned long long census[8 * 256];
  err = cudaMemcpyAsync(census, census_d, sizeof census, cudaMemcpyDeviceToHost, st);
  if (err != cudaSuccess) return err;
  err = cudaStreamSynchronize(st);
  if (err != cudaSuccess) return err;
  const int nblocks = (int)((n + kSortBlockKeys - 1) / kSortBlockKeys);
  uint64_t *ka = keys, *kb = ktmp;
  uint32_t *va = vals, *vb = vtmp;
  for (int p = 0; p < 8; p++) {
    bool uniform = false;
    for (int d = 0; d < 256; d++)
      if (census[p * 256 + d] == (unsigned long long)n) uniform = true;
    if (uniform) continue;
    *launches += 3;
    radix_hist_kernel<<<nblocks, kSortThreads, 0, st>>>(n, ka, 8 * p, hist, nblocks);
    scan_kernel<<<1, 1024, 0, st>>>(hist, (int64_t)256 * nblocks);
    radix_scatter_kernel<<<nblocks, kSortThreads, 0, st>>>(n, ka, va, kb, vb, 8 * p, hist, nblocks);
    uint64_t *tk = ka; ka = kb; kb = tk;
    uint32_t *tv = va; va = vb; vb = tv;
  }
  err = cudaGetLastError();
  if (err != cudaSuccess) return err;
  if (ka != keys) {
    err = cudaMemcpyAsync(keys, ka, sizeof(uint64_t) * n, cudaMemcpyDeviceToDevice, st);
    if (err != cudaSuccess) return err;
    err = cudaMemcpyAsync(vals, va, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, st);
  }
  return err;
}

int64_t radix_hist_words(int64_t n) {
  return 256 * ((n + kSortBlockKeys - 1) / kSortBlockKeys);
}

cudaError_t launch_cell_keys(int64_t n, const double *x, const double *y, const double *z,
                             const int32_t *jk, double inv_cw_x, double inv_cw_y, int ncx, int ncy,
                             int n_reg, uint64_t *keys, uint32_t *vals, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  cell_keys_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(n, x, y, z, jk, inv_cw_x, inv_cw_y,
                                                                ncx, ncy, n_reg, keys, vals);
  return cudaGetLastError();
}

cudaError_t launch_z_keys(int64_t n, const double *z, uint64_t *keys, uint32_t *vals,
                          cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  z_keys_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(n, z, keys, vals);
  return cudaGetLastError();
}

// Gather the cell-ordered (or z-ordered) arrays from the original ones.
__global__ void gather_kernel(int64_t n, const uint64_t *__restrict__ keys,
                              const uint32_t *__restrict__ perm, GatherIn in, GatherOut out) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const uint32_t i = perm[k];
  const double x = in.x[i], y = in.y[i], z = in.z[i], w = in.w[i];
  const double e1 = in.e1[i], e2 = in.e2[i], phi = in.phi[i], e3 = in.e3[i];
  if (out.pos) {
    out.pos[k] = make_float4((float)x, (float)y, (float)z, (float)w);
    out.shp[k] = make_float4((float)e1, (float)e2, (float)phi, (float)e3);
    // the weighted ellipticity w (e1, e2) and the weight as float hi + lo parts
    // (the compensated shape terms of the pair kernel)
    const double we1 = __dmul_rn(w, e1), we2 = __dmul_rn(w, e2);
    const float h1 = (float)we1, h2 = (float)we2;
    out.ewt[k] = make_float4(h1, h2, (float)(we1 - (double)h1), (float)(we2 - (double)h2));
    out.aux[k] = make_float4((float)(x - (double)(float)x), (float)(y - (double)(float)y),
                             (float)phi, (float)(w - (double)(float)w));
    out.zf[k] = (float)z;
    out.zlo[k] = (float)(z - (double)(float)z);
  }
  if (out.bucket) out.bucket[k] = (uint32_t)(keys[k] >> 32);
  out.x[k] = x;
  out.y[k] = y;
  out.z[k] = z;
  out.w[k] = w;
  out.e1[k] = e1;
  out.e2[k] = e2;
  out.phi[k] = phi;
  out.e3[k] = e3;
  out.jk[k] = in.jk[i];
  out.keep[k] = in.keep[i];
  out.orig[k] = out.orig_in ? out.orig_in[i] : (int64_t)i;
}

cudaError_t launch_gather(int64_t n, const uint64_t *keys, const uint32_t *perm, const GatherIn &in,
                          const GatherOut &out, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  gather_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(n, keys, perm, in, out);
  return cudaGetLastError();
}

__global__ void fill_f64_kernel(int64_t n, double v, double *__restrict__ out) {
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n;
       k += (int64_t)gridDim.x * blockDim.x)
    out[k] = v;
}

cudaError_t launch_fill_f64(int64_t n, double v, double *out, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  const int64_t blocks = std::min<int64_t>((n + 255) / 256, 4096);
  fill_f64_kernel<<<(unsigned)blocks, 256, 0, st>>>(n, v, out);
  return cudaGetLastError();
}

unsigned long long orderable_key(double v) {
  unsigned long long u;
  std::memcpy(&u, &v, 8);
  return (u >> 63) ? ~u : (u | 0x8000000000000000ull);
}
double from_orderable_key(unsigned long long k) {
  const unsigned long long u = (k >> 63) ? (k & 0x7fffffffffffffffull) : ~k;
  double v;
  std::memcpy(&v, &u, 8);
  return v;
}

__device__ __forceinline__ unsigned long long warp_max_u64(unsigned long long v) {
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long w = __shfl_xor_sync(0xffffffffu, v, o);
    v = w > v ? w : v;
  }
  return v;
}
__device__ __forceinline__ unsigned long long warp_min_u64(unsigned long long v) {
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long w = __shfl_xor_sync(0xffffffffu, v, o);
    v = w < v ? w : v;
  }
  return v;
}
// bit pattern of a non-negative double: ordered like the values
__device__ __forceinline__ unsigned long long nonneg_bits(double v) {
  return (unsigned long long)__double_as_longlong(v);
}

// One pass over a catalogue in input order (the host checks of the reference's
// read path plus what the pair kernels need): see UploadStats.  The corels1
// scan starts compare, as do_pair_sorted does, z + L*PBz with z_min = z_i + p_min
// (lim_calc_PB; z_i - r_max for coordinates 7): row i + 1 for the 0 and -1
// images, row 0 for the +1 image.
__global__ void prep_catalog_kernel(PrepIn in, uint8_t *__restrict__ keep,
                                    uint8_t *__restrict__ aflag, UploadStats *__restrict__ st) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  unsigned long long cm = 0, wm = 0, em = 0, pm = 0, wk = ~0ull;
  unsigned int nf = 0;
  if (i < in.n) {
    const double x = in.x[i], y = in.y[i], z = in.z[i];
    const double L = in.L;
    if (!isfinite(x) || !isfinite(y) || !isfinite(z)) atomicMin(&st->bad_row[0], (unsigned long long)i);
    else if (x < 0 || y < 0 || z < 0 || x > L || y > L || z > L)
      atomicMin(&st->bad_row[1], (unsigned long long)i);
    if ((double)(float)x != x || (double)(float)y != y || (double)(float)z != z) nf = 1u;
    cm = nonneg_bits(fmax(fmax(fmax(x, y), z), 0.0));
    const double w = in.w ? in.w[i] : 1.0;
    bool bad = !isfinite(w);
    wm = nonneg_bits(fabs(w));
    // orderable key of w for the minimum
    const unsigned long long u = (unsigned long long)__double_as_longlong(w);
    wk = (u >> 63) ? ~u : (u | 0x8000000000000000ull);
    // |e| (with the third ED component): bounds the rotated ellipticities,
    // kappa (read into e1) and the ED cosine alike
    double e2sum = 0.0;
    if (in.e1) {
      const double a = in.e1[i], b = in.e2[i];
      bad |= !isfinite(a) || !isfinite(b);
      e2sum = a * a + b * b;
    }
    if (in.e3) {
      const double c3 = in.e3[i];
      bad |= !isfinite(c3);
      e2sum += c3 * c3;
    }
    if (isfinite(e2sum)) em = nonneg_bits(sqrt(e2sum) * (1.0 + 1e-15));
    const double ph = in.phi ? in.phi[i] : -10.0;
    bad |= !isfinite(ph);
    pm = nonneg_bits(fabs(ph));
    if (bad) atomicMin(&st->bad_row[2], (unsigned long long)i);
    if (in.jk) {
      const int r = in.jk[i];
      if (r < 0 || r >= in.n_jk) atomicMin(&st->bad_row[3], (unsigned long long)i);
    }
    keep[i] = (in.jk_prob && in.jk_prob[i] >= 0.5) ? 1 : 0;
    const double zmin = __dadd_rn(z, in.wz_lo);
    uint8_t f = 0;
    if (i + 1 < in.n) {
      const double zn = in.z[i + 1];
      if (!(__dadd_rn(zn, __dmul_rn(L, 0.0)) < zmin)) f |= kAutoStart0;
      if (!(__dadd_rn(zn, __dmul_rn(L, -1.0)) < zmin)) f |= kAutoStartM;
    }
    if (!(__dadd_rn(in.z[0], __dmul_rn(L, 1.0)) < zmin)) f |= kAutoStartP;
    aflag[i] = f;
  }
  cm = warp_max_u64(cm);
  wm = warp_max_u64(wm);
  em = warp_max_u64(em);
  pm = warp_max_u64(pm);
  wk = warp_min_u64(wk);
  nf = __any_sync(0xffffffffu, nf != 0u) ? 1u : 0u;
  if ((threadIdx.x & 31) == 0) {
    if (cm) atomicMax(&st->cmax_bits, cm);
    if (wm) atomicMax(&st->wmax_bits, wm);
    if (em) atomicMax(&st->emax_bits, em);
    if (pm) atomicMax(&st->phimax_bits, pm);
    if (wk != ~0ull) atomicMin(&st->wmin_key, wk);
    if (nf) atomicOr(&st->not_f32, 1u);
  }
}

cudaError_t launch_prep_catalog(const PrepIn &in, uint8_t *keep, uint8_t *aflag,
                                UploadStats *stats, cudaStream_t st) {
  if (in.n == 0) return cudaSuccess;
  prep_catalog_kernel<<<(unsigned)((in.n + 255) / 256), 256, 0, st>>>(in, keep, aflag, stats);
  return cudaGetLastError();
}

__global__ void gather_u8_kernel(int64_t n, const uint32_t *__restrict__ perm,
                                 const uint8_t *__restrict__ in, uint8_t *__restrict__ out) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) out[k] = in[perm[k]];
}

cudaError_t launch_gather_u8(int64_t n, const uint32_t *perm, const uint8_t *in, uint8_t *out,
                             cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  gather_u8_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(n, perm, in, out);
  return cudaGetLastError();
}

// *differ becomes nonzero when the bytes [0, n) of a and b differ anywhere
// (4-byte words, then the tail bytes)
__global__ void bytes_differ_kernel(const uint8_t *__restrict__ a, const uint8_t *__restrict__ b,
                                    int64_t n, unsigned *__restrict__ differ) {
  const int64_t nw = n / 4;
  const uint32_t *wa = reinterpret_cast<const uint32_t *>(a);
  const uint32_t *wb = reinterpret_cast<const uint32_t *>(b);
  unsigned d = 0;
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < nw;
       k += (int64_t)gridDim.x * blockDim.x)
    d |= wa[k] ^ wb[k];
  if (blockIdx.x == 0 && threadIdx.x < (unsigned)(n - 4 * nw))
    d |= a[4 * nw + threadIdx.x] ^ b[4 * nw + threadIdx.x];
  if (__any_sync(0xffffffffu, d != 0) && (threadIdx.x & 31) == 0) atomicOr(differ, 1u);
}

cudaError_t launch_bytes_differ(const void *a, const void *b, int64_t n, unsigned *differ,
                                cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  const int64_t blocks = std::min<int64_t>((n / 4 + 255) / 256 + 1, 2048);
  bytes_differ_kernel<<<(unsigned)blocks, 256, 0, st>>>(static_cast<const uint8_t *>(a),
                                                       static_cast<const uint8_t *>(b), n, differ);
  return cudaGetLastError();
}

}  // namespace cpc
