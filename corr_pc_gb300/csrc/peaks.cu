// peaks.cu -- micro-benchmarks for the roofline denominators of the pair
// kernel, which is bound neither by HBM nor by tensor cores:
//   * FP32 FMA issue rate (independent FFMA chains, all SMs),
//   * conflict-free shared-memory atomic add throughput (u32, u64, f32, f64),
//   * the same with every lane of a warp on one address (fully conflicted).
// Built as a separate library (libcpc_peaks.so); not part of the C ABI.
#include <cuda_runtime.h>
#include <stdint.h>

namespace {

constexpr int kChains = 8;

__global__ void ffma_kernel(float *out, int iters, float a, float b) {
  float x[kChains];
#pragma unroll
  for (int k = 0; k < kChains; k++) x[k] = threadIdx.x * 0.001f + k;
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int k = 0; k < kChains; k++) x[k] = fmaf(x[k], a, b);
  }
  float s = 0.f;
#pragma unroll
  for (int k = 0; k < kChains; k++) s += x[k];
  if (s == 1234.5678f) out[0] = s;  // keep the work alive
}

template <class T>
__global__ void smem_atomic_ret_kernel(T *out, int iters, int conflict) {
  extern __shared__ __align__(16) unsigned char raw[];
  T *h = reinterpret_cast<T *>(raw);
  const int n = blockDim.x * 4;
  for (int k = threadIdx.x; k < n; k += blockDim.x) h[k] = T(0);
  __syncthreads();
  const int base = conflict ? (threadIdx.x >> 5) * 32 : threadIdx.x;
  T acc = T(0);
  for (int i = 0; i < iters; i++) {
    const int a = (base + (i & 3) * blockDim.x) % n;
    const T old = atomicAdd(&h[a], T(1));
    if (old + T(1) < old) acc += T(1);  // consume the returned value
  }
  __syncthreads();
  if (threadIdx.x == 0 && h[0] == T(-1)) out[0] = h[1] + acc;
}

template <class T>
__global__ void smem_atomic_kernel(T *out, int iters, int conflict) {
  extern __shared__ __align__(16) unsigned char raw[];
  T *h = reinterpret_cast<T *>(raw);
  const int n = blockDim.x * 4;
  for (int k = threadIdx.x; k < n; k += blockDim.x) h[k] = T(0);
  __syncthreads();
  // conflict-free: lane-distinct consecutive words (distinct banks)
  const int base = conflict ? (threadIdx.x >> 5) * 32 : threadIdx.x;
  for (int i = 0; i < iters; i++) {
    const int a = (base + (i & 3) * blockDim.x) % n;
    atomicAdd(&h[a], T(1));
  }
  __syncthreads();
  if (threadIdx.x == 0 && h[0] == T(-1)) out[0] = h[1];
}

}  // namespace

extern "C" {

// which: 0 FFMA (returns FLOP/s), 1 u32, 2 u64, 3 f32, 4 f64 shared atomics
// (returns atomic ops/s), 5 u32 add returning the old value (carry test),
// +8 for the fully conflicted variant.
int cpc_peak(int which, double *result, double *ms_out) {
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 2;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  void *buf = nullptr;
  if (cudaMalloc(&buf, 64) != cudaSuccess) return 3;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  const int threads = 256, blocks = sms * 8;
  double ops = 0;
  const int conflict = which >= 8;
  const int w = which & 7;
  for (int rep = 0; rep < 2; rep++) {  // first repetition warms up
    cudaEventRecord(e0);
    if (w == 0) {
      const int iters = 1 << 14;
      ffma_kernel<<<blocks, threads>>>((float *)buf, iters, 0.9999f, 0.0001f);
      ops = 2.0 * kChains * iters * (double)threads * blocks;
    } else {
      const int iters = conflict ? 1 << 11 : 1 << 14;
      const size_t smem = (size_t)threads * 4 * 8;
      if (w == 1) smem_atomic_kernel<unsigned int><<<blocks, threads, smem>>>((unsigned int *)buf, iters, conflict);
      if (w == 2) smem_atomic_kernel<unsigned long long><<<blocks, threads, smem>>>((unsigned long long *)buf, iters, conflict);
      if (w == 3) smem_atomic_kernel<float><<<blocks, threads, smem>>>((float *)buf, iters, conflict);
      if (w == 4) smem_atomic_kernel<double><<<blocks, threads, smem>>>((double *)buf, iters, conflict);
      if (w == 5) smem_atomic_ret_kernel<unsigned int><<<blocks, threads, smem>>>((unsigned int *)buf, iters, conflict);
      ops = (double)iters * threads * blocks;
    }
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
  }
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaError_t err = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(buf);
  if (err != cudaSuccess) return 2;
  *result = ops / (ms * 1e-3);
  if (ms_out) *ms_out = ms;
  return 0;
}
}
