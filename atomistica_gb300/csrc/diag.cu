// Diagnostics used by the benchmark: a dependent-free FMA-chain microbenchmark
// that measures the FP32 and FP64 pipe peaks of the device (the roofline
// denominators for the SIMT bond-order kernels, which use no tensor cores).

#include <cuda_runtime.h>

#include <algorithm>

#include "internal.h"

namespace gb {
namespace {

template <class T>
__global__ void __launch_bounds__(256) fma_chains(T *out, int iters, T a, T b) {
  T x[8];
#pragma unroll
  for (int q = 0; q < 8; q++) x[q] = (T)(threadIdx.x + q);
  for (int it = 0; it < iters; it++) {
#pragma unroll
    for (int q = 0; q < 8; q++) x[q] = fma(x[q], a, b);
  }
  T s = 0;
#pragma unroll
  for (int q = 0; q < 8; q++) s += x[q];
  if (s == (T)-1.2345e-30) out[blockIdx.x] = s;  // keeps the chains live
}

template <class T>
int measure(double *tflops) {
  int dev = 0, sms = 0;
  GB_CUDA(cudaGetDevice(&dev));
  GB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  T *out = nullptr;
  GB_CUDA(cudaMalloc(&out, sizeof(T) * 65536));
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  const int blocks = sms * 8, threads = 256;
  const int iters = sizeof(T) == 8 ? 2048 : 16384;
  double best = 0.0;
  for (int rep = 0; rep < 6; rep++) {
    cudaEventRecord(e0);
    fma_chains<T><<<blocks, threads>>>(out, iters, (T)0.999999, (T)1e-7);
    note_launch();
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    const double flops = 2.0 * 8.0 * iters * (double)blocks * threads;
    if (rep > 0) best = std::max(best, flops / (ms * 1e-3) / 1e12);
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  GB_CUDA(cudaGetLastError());
  *tflops = best;
  return 0;
}

// sqrt_from_rsqrt against the correctly rounded sqrt for n arguments drawn
// uniformly from [lo, hi] (a counter-based hash, argument k for index k).
__device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
__global__ void sqrt_check(int64_t n, double lo, double hi, unsigned long long *bad) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  unsigned long long mine = 0;
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += stride) {
    const double u = (double)(mix64((uint64_t)k) >> 11) * (1.0 / 9007199254740992.0);
    const double x = lo + (hi - lo) * u;
    mine += sqrt_from_rsqrt(x, rsqrt_refined(x)) != sqrt(x);
  }
  if (mine) atomicAdd(bad, mine);
}

}  // namespace
}  // namespace gb

extern "C" int gb_diag_sqrt_check(int64_t n, double lo, double hi, int64_t *mismatches) {
  gb::clear_error();
  if (!mismatches || n < 0 || !(lo > 0.0) || !(hi >= lo)) return GB_ERROR_ARGUMENT;
  unsigned long long *bad = nullptr;
  GB_CUDA(cudaMalloc(&bad, sizeof(unsigned long long)));
  GB_CUDA(cudaMemset(bad, 0, sizeof(unsigned long long)));
  int dev = 0, sms = 0;
  GB_CUDA(cudaGetDevice(&dev));
  GB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  gb::sqrt_check<<<sms * 8, 256>>>(n, lo, hi, bad);
  gb::note_launch();
  unsigned long long h = 0;
  const cudaError_t e = cudaMemcpy(&h, bad, sizeof(h), cudaMemcpyDeviceToHost);
  cudaFree(bad);
  GB_CUDA(e);
  *mismatches = (int64_t)h;
  return 0;
}

extern "C" int gb_bench_fma_peak(int fp64, double *tflops) {
  gb::clear_error();
  if (!tflops) return GB_ERROR_ARGUMENT;
  return fp64 ? gb::measure<double>(tflops) : gb::measure<float>(tflops);
}
