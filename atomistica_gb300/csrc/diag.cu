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

}  // namespace
}  // namespace gb

extern "C" int gb_bench_fma_peak(int fp64, double *tflops) {
  gb::clear_error();
  if (!tflops) return GB_ERROR_ARGUMENT;
  return fp64 ? gb::measure<double>(tflops) : gb::measure<float>(tflops);
}
