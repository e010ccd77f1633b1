// GB300 FP64-pipe microbenchmark (not part of the library): DFMA throughput with 1, 1/2, 1/4
// and 1/32 of the lanes active, FFMA throughput and CUDA's exp(double), each timed with CUDA
// events over a full grid. Numbers in profiles/fp64_pipe_probes_gb300.txt.
//   nvcc -std=c++17 -O3 -gencode arch=compute_103a,code=sm_103a -o fp64_active_lanes \
//        pelelm_gb300/csrc/probes/fp64_active_lanes.cu && ./fp64_active_lanes
#include <cstdio>
#include <cuda_runtime.h>
#define CK(x) do{cudaError_t e=(x); if(e!=cudaSuccess){printf("ERR %s %d: %s\n",__FILE__,__LINE__,cudaGetErrorString(e)); return 1;}}while(0)

template<int ILP>
__global__ void dfma_kernel(double* out, int iters, int active_mod) {
  double a[ILP]; double b = 1.0000001, c = 1e-9;
  for (int i=0;i<ILP;i++) a[i] = threadIdx.x*1e-3 + i;
  int lane = threadIdx.x & 31;
  if ((lane % active_mod) == 0) {
    for (int it=0; it<iters; it++) {
#pragma unroll
      for (int i=0;i<ILP;i++) a[i] = fma(a[i], b, c);
    }
  }
  double s=0; for (int i=0;i<ILP;i++) s+=a[i];
  if (s == 12345.0) out[0]=s;
}
template<int ILP>
__global__ void ffma_kernel(float* out, int iters) {
  float a[ILP]; float b = 1.0000001f, c = 1e-9f;
  for (int i=0;i<ILP;i++) a[i] = threadIdx.x*1e-3f + i;
  for (int it=0; it<iters; it++) {
#pragma unroll
    for (int i=0;i<ILP;i++) a[i] = fmaf(a[i], b, c);
  }
  float s=0; for (int i=0;i<ILP;i++) s+=a[i];
  if (s == 12345.0f) out[0]=s;
}
__global__ void dexp_kernel(double* out, int iters) {
  double x = -5.0 + threadIdx.x*1e-3, s = 0;
  for (int it=0; it<iters; it++) { s += exp(x); x += 1e-7; }
  if (s == 12345.0) out[0]=s;
}
int main(){
  int dev=0; cudaDeviceProp p; CK(cudaGetDeviceProperties(&p,dev));
  printf("name %s SMs %d cc %d.%d smemPerBlockOptin %zu regsPerSM %d L2 %d\n", p.name, p.multiProcessorCount, p.major,p.minor, p.sharedMemPerBlockOptin, p.regsPerMultiprocessor, p.l2CacheSize);
  double* d; CK(cudaMalloc(&d, 64)); float* f; CK(cudaMalloc(&f,64));
  cudaEvent_t e0,e1; cudaEventCreate(&e0); cudaEventCreate(&e1);
  int sms = p.multiProcessorCount;
  int iters = 20000;
  for (int tpb : {128, 256, 512, 1024}) {
    for (int mod : {1, 2, 4, 32}) {
      dfma_kernel<8><<<sms, tpb>>>(d, 100, mod); CK(cudaDeviceSynchronize());
      cudaEventRecord(e0);
      dfma_kernel<8><<<sms, tpb>>>(d, iters, mod);
      cudaEventRecord(e1); CK(cudaEventSynchronize(e1));
      float ms; cudaEventElapsedTime(&ms,e0,e1);
      double active = (double)sms*tpb/mod;
      double fl = active*iters*8*2.0;
      double warp_instr = (double)sms*tpb/32*iters*8;
      printf("DFMA tpb %4d active 1/%2d: %.3f ms  %.3f TFLOP/s (active lanes)  %.3f Gwarpinstr/s\n", tpb, mod, ms, fl/ms/1e9, warp_instr/ms/1e6);
    }
  }
  for (int tpb : {256, 1024}) {
    ffma_kernel<8><<<sms*2, tpb>>>(f, 100); CK(cudaDeviceSynchronize());
    cudaEventRecord(e0);
    ffma_kernel<8><<<sms*2, tpb>>>(f, iters*8);
    cudaEventRecord(e1); CK(cudaEventSynchronize(e1));
    float ms; cudaEventElapsedTime(&ms,e0,e1);
    double fl = (double)sms*2*tpb*iters*8*8*2.0;
    printf("FFMA tpb %4d: %.3f ms %.2f TFLOP/s\n", tpb, ms, fl/ms/1e9);
  }
  for (int tpb : {128, 256, 1024}) {
    int it2 = 2000;
    dexp_kernel<<<sms, tpb>>>(d, 10); CK(cudaDeviceSynchronize());
    cudaEventRecord(e0);
    dexp_kernel<<<sms, tpb>>>(d, it2);
    cudaEventRecord(e1); CK(cudaEventSynchronize(e1));
    float ms; cudaEventElapsedTime(&ms,e0,e1);
    double calls = (double)sms*tpb*it2;
    printf("exp(double) tpb %4d: %.3f ms  %.3f Gexp/s\n", tpb, ms, calls/ms/1e6);
  }
  return 0;
}
