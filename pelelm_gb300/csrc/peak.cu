// FP64 FMA throughput of the current device: the denominator of the reactor's roofline (rate
// evaluation and the BDF are FP64-issue bound on GB300). Eight independent FMA chains per
// thread, a full grid of 512-thread blocks, timed with CUDA events.
#include <cuda_runtime.h>

#include "reactor_registry.cuh"

namespace {

__global__ void dfma_peak_kernel(double* sink, int iters) {
  double a[8];
  const double b = 1.0000000001, c = 1e-12;
#pragma unroll
  for (int i = 0; i < 8; ++i) a[i] = threadIdx.x * 1e-3 + i;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int i = 0; i < 8; ++i) a[i] = fma(a[i], b, c);
  }
  double s = 0.0;
#pragma unroll
  for (int i = 0; i < 8; ++i) s += a[i];
  if (s == 1.2345) sink[0] = s;  // never true; keeps the chains live
}

}  // namespace

extern "C" int pgb_fp64_peak_tflops(int iters, double* tflops) {
  using namespace pgb_host;
  if (!tflops || iters < 1) return set_err("pgb_fp64_peak_tflops: bad arguments");
  int dev = 0, nsm = 0;
  PGB_CUDA(cudaGetDevice(&dev));
  PGB_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  double* sink = nullptr;
  PGB_CUDA(cudaMalloc(&sink, sizeof(double)));
  cudaEvent_t e0, e1;
  PGB_CUDA(cudaEventCreate(&e0));
  PGB_CUDA(cudaEventCreate(&e1));
  const int blocks = nsm * 4, threads = 512;
  dfma_peak_kernel<<<blocks, threads>>>(sink, 64);  // warm-up
  PGB_CUDA(cudaGetLastError());
  float best = 1e30f;
  for (int rep = 0; rep < 3; ++rep) {
    PGB_CUDA(cudaEventRecord(e0));
    dfma_peak_kernel<<<blocks, threads>>>(sink, iters);
    PGB_CUDA(cudaEventRecord(e1));
    PGB_CUDA(cudaEventSynchronize(e1));
    float ms = 0.f;
    PGB_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    best = ms < best ? ms : best;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(sink);
  *tflops = 2.0 * 8.0 * (double)iters * blocks * threads / (best * 1e-3) / 1e12;
  return 0;
}
