// GB300 FP64-pipe microbenchmark (not part of the library): warp-instruction throughput of
// DFMA, FFMA, double<->float and int<->double converts, DSETP, fmax, IEEE division, __drcp_rn
// and CUDA's log/exp(double), 8 independent chains per thread over a full grid, timed with
// CUDA events. Numbers in profiles/fp64_pipe_probes_gb300.txt.
//   nvcc -std=c++17 -O3 -gencode arch=compute_103a,code=sm_103a -o fp64_op_costs \
//        pelelm_gb300/csrc/probes/fp64_op_costs.cu && ./fp64_op_costs
#include <cstdio>
#include <cuda_runtime.h>
#define CK(x) do{cudaError_t e=(x); if(e!=cudaSuccess){printf("ERR %s %d: %s\n",__FILE__,__LINE__,cudaGetErrorString(e)); return 1;}}while(0)
// Each kernel: 8 independent chains, iters loop. Reports warp-instructions/s of the op.
#define KBODY(INIT, OP, FIN) \
  { INIT; for (int it=0; it<iters; it++) { _Pragma("unroll") for (int i=0;i<8;i++) { OP; } } FIN; }
__global__ void k_f2f_d2f(float* o, int iters){ double d[8]; float f[8]; for(int i=0;i<8;i++){d[i]=threadIdx.x+i; f[i]=0;}
  for(int it=0;it<iters;it++){ _Pragma("unroll") for(int i=0;i<8;i++){ f[i]+= (float)d[i]; d[i]+=1e-30; } }
  float s=0; for(int i=0;i<8;i++) s+=f[i]; if(s==1.2345f) o[0]=s; }
__global__ void k_f2f_f2d(double* o, int iters){ float f[8]; double d[8]; for(int i=0;i<8;i++){f[i]=threadIdx.x+i; d[i]=0;}
  for(int it=0;it<iters;it++){ _Pragma("unroll") for(int i=0;i<8;i++){ d[i] = (double)f[i]; f[i] = f[i]*1.0000001f + (float)(d[i]==3.0); } }
  double s=0; for(int i=0;i<8;i++) s+=d[i]; if(s==1.2345) o[0]=s; }
__global__ void k_dsetp(int* o, int iters){ double d[8]; int c[8]; for(int i=0;i<8;i++){d[i]=threadIdx.x*0.5+i; c[i]=0;}
  for(int it=0;it<iters;it++){ _Pragma("unroll") for(int i=0;i<8;i++){ c[i] += (d[i] < (double)(it&7)) ? 1 : 0; } }
  int s=0; for(int i=0;i<8;i++) s+=c[i]; if(s==12345) o[0]=s; }
__global__ void k_dmnmx(double* o, int iters){ double d[8]; for(int i=0;i<8;i++) d[i]=threadIdx.x+i;
  for(int it=0;it<iters;it++){ _Pragma("unroll") for(int i=0;i<8;i++){ d[i] = fmax(d[i], (double)i); } }
  double s=0; for(int i=0;i<8;i++) s+=d[i]; if(s==1.2345) o[0]=s; }
__global__ void k_ddiv(double* o, int iters){ double d[8]; for(int i=0;i<8;i++) d[i]=threadIdx.x+i+1.5;
  for(int it=0;it<iters;it++){ _Pragma("unroll") for(int i=0;i<8;i++){ d[i] = 3.0 / d[i]; } }
  double s=0; for(int i=0;i<8;i++) s+=d[i]; if(s==1.2345) o[0]=s; }
__global__ void k_drcp(double* o, int iters){ double d[8]; for(int i=0;i<8;i++) d[i]=threadIdx.x+i+1.5;
  for(int it=0;it<iters;it++){ _Pragma("unroll") for(int i=0;i<8;i++){ d[i] = __drcp_rn(d[i]); } }
  double s=0; for(int i=0;i<8;i++) s+=d[i]; if(s==1.2345) o[0]=s; }
__global__ void k_dlog(double* o, int iters){ double d[8]; for(int i=0;i<8;i++) d[i]=threadIdx.x+i+1.5;
  for(int it=0;it<iters;it++){ _Pragma("unroll") for(int i=0;i<8;i++){ d[i] = log(d[i]) + 2.0; } }
  double s=0; for(int i=0;i<8;i++) s+=d[i]; if(s==1.2345) o[0]=s; }
__global__ void k_dexp(double* o, int iters){ double d[8]; for(int i=0;i<8;i++) d[i]=-(threadIdx.x*1e-3+i);
  for(int it=0;it<iters;it++){ _Pragma("unroll") for(int i=0;i<8;i++){ d[i] = exp(d[i]) - 1.0; } }
  double s=0; for(int i=0;i<8;i++) s+=d[i]; if(s==1.2345) o[0]=s; }
__global__ void k_ffma(float* o, int iters){ float d[8]; for(int i=0;i<8;i++) d[i]=threadIdx.x+i;
  for(int it=0;it<iters;it++){ _Pragma("unroll") for(int i=0;i<8;i++){ d[i] = fmaf(d[i],1.0000001f,1e-7f); } }
  float s=0; for(int i=0;i<8;i++) s+=d[i]; if(s==1.2345f) o[0]=s; }
__global__ void k_dfma(double* o, int iters){ double d[8]; for(int i=0;i<8;i++) d[i]=threadIdx.x+i;
  for(int it=0;it<iters;it++){ _Pragma("unroll") for(int i=0;i<8;i++){ d[i] = fma(d[i],1.0000001,1e-7); } }
  double s=0; for(int i=0;i<8;i++) s+=d[i]; if(s==1.2345) o[0]=s; }
__global__ void k_i2d(double* o, int iters){ int a[8]; double d[8]; for(int i=0;i<8;i++){a[i]=threadIdx.x+i; d[i]=0;}
  for(int it=0;it<iters;it++){ _Pragma("unroll") for(int i=0;i<8;i++){ d[i] = (double)a[i]; a[i] += (int)(d[i]==5.0) + 1; } }
  double s=0; for(int i=0;i<8;i++) s+=d[i]; if(s==1.2345) o[0]=s; }
__global__ void k_d2i(int* o, int iters){ double d[8]; int a[8]; for(int i=0;i<8;i++){d[i]=threadIdx.x+i+0.3; a[i]=0;}
  for(int it=0;it<iters;it++){ _Pragma("unroll") for(int i=0;i<8;i++){ a[i] += __double2int_rn(d[i]); d[i] = __longlong_as_double(__double_as_longlong(d[i]) ^ 1); } }
  int s=0; for(int i=0;i<8;i++) s+=a[i]; if(s==12345) o[0]=s; }
template<typename K, typename T> int run(const char* name, K k, T* buf, int iters, int sms){
  cudaEvent_t e0,e1; cudaEventCreate(&e0); cudaEventCreate(&e1);
  k<<<sms, 512>>>(buf, 10); CK(cudaDeviceSynchronize());
  cudaEventRecord(e0); k<<<sms, 512>>>(buf, iters); cudaEventRecord(e1); CK(cudaEventSynchronize(e1));
  float ms; cudaEventElapsedTime(&ms,e0,e1);
  double wi = (double)sms*512/32*iters*8;
  printf("%-12s %8.3f ms  %8.3f G op-warp/s  (%.3f Gop-lane/s)\n", name, ms, wi/ms/1e6, wi*32/ms/1e6);
  return 0;
}
int main(){ cudaDeviceProp p; cudaGetDeviceProperties(&p,0); int sms=p.multiProcessorCount;
  double* d; float* f; int* i; CK(cudaMalloc(&d,64)); CK(cudaMalloc(&f,64)); CK(cudaMalloc(&i,64));
  run("dfma", k_dfma, d, 2000, sms); run("ffma", k_ffma, f, 20000, sms);
  run("cvt d->f", k_f2f_d2f, f, 2000, sms); run("cvt f->d", k_f2f_f2d, d, 2000, sms);
  run("dsetp", k_dsetp, i, 2000, sms); run("dmnmx", k_dmnmx, d, 2000, sms);
  run("i2d", k_i2d, d, 2000, sms); run("d2i", k_d2i, i, 2000, sms);
  run("ddiv", k_ddiv, d, 200, sms); run("drcp_rn", k_drcp, d, 200, sms);
  run("log(d)", k_dlog, d, 200, sms); run("exp(d)", k_dexp, d, 200, sms);
  return 0; }
