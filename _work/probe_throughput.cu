// probe_throughput.cu -- GB300 throughput probe behind the design: FP64 FMA, FP32 FMA, FP64 DMMA
// (mma.sync m8n8k4), dependent-chain FP64 FMA and divide latency, device copy bandwidth.
// Not part of the library. All accesses in bounds, all loops bounded.
#include <cstdio>
#include <cuda_runtime.h>
#define CK(x) do{cudaError_t e=(x); if(e!=cudaSuccess){printf("err %s line %d\n", cudaGetErrorString(e), __LINE__); return 1;}}while(0)

__global__ void fma64(double *out, int iters, double a, double b) {
  double x0=threadIdx.x, x1=x0+1, x2=x0+2, x3=x0+3, x4=x0+4, x5=x0+5, x6=x0+6, x7=x0+7;
  for (int i = 0; i < iters; ++i) {
    x0 = fma(x0,a,b); x1 = fma(x1,a,b); x2 = fma(x2,a,b); x3 = fma(x3,a,b);
    x4 = fma(x4,a,b); x5 = fma(x5,a,b); x6 = fma(x6,a,b); x7 = fma(x7,a,b);
  }
  out[blockIdx.x*blockDim.x+threadIdx.x] = x0+x1+x2+x3+x4+x5+x6+x7;
}
__global__ void fma32(float *out, int iters, float a, float b) {
  float x0=threadIdx.x, x1=x0+1, x2=x0+2, x3=x0+3, x4=x0+4, x5=x0+5, x6=x0+6, x7=x0+7;
  for (int i = 0; i < iters; ++i) {
    x0 = fmaf(x0,a,b); x1 = fmaf(x1,a,b); x2 = fmaf(x2,a,b); x3 = fmaf(x3,a,b);
    x4 = fmaf(x4,a,b); x5 = fmaf(x5,a,b); x6 = fmaf(x6,a,b); x7 = fmaf(x7,a,b);
  }
  out[blockIdx.x*blockDim.x+threadIdx.x] = x0+x1+x2+x3+x4+x5+x6+x7;
}
__global__ void dmma(double *out, int iters) {
  double a = 1.0 + threadIdx.x * 1e-3, b = 0.5;
  double c0=0,c1=0,c2=0,c3=0,c4=0,c5=0,c6=0,c7=0;
  for (int i = 0; i < iters; ++i) {
    asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};" : "+d"(c0), "+d"(c1) : "d"(a), "d"(b));
    asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};" : "+d"(c2), "+d"(c3) : "d"(a), "d"(b));
    asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};" : "+d"(c4), "+d"(c5) : "d"(a), "d"(b));
    asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};" : "+d"(c6), "+d"(c7) : "d"(a), "d"(b));
  }
  out[blockIdx.x*blockDim.x+threadIdx.x] = c0+c1+c2+c3+c4+c5+c6+c7;
}
__global__ void copyk(const double2 *__restrict__ a, double2 *__restrict__ b, size_t n) {
  for (size_t i = blockIdx.x*(size_t)blockDim.x+threadIdx.x; i < n; i += (size_t)gridDim.x*blockDim.x) b[i] = a[i];
}
__global__ void divlat(double *out, int iters, double d) {
  double x = 1.0 + threadIdx.x;
  for (int i = 0; i < iters; ++i) x = d / (x + 1.0);
  out[blockIdx.x*blockDim.x+threadIdx.x] = x;
}
__global__ void fmalat(double *out, int iters, double a, double b) {
  double x = threadIdx.x;
  for (int i = 0; i < iters; ++i) x = fma(x, a, b);
  out[blockIdx.x*blockDim.x+threadIdx.x] = x;
}
int main() {
  int sms; cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0);
  int clk; cudaDeviceGetAttribute(&clk, cudaDevAttrClockRate, 0);
  printf("SMs %d clockKHz %d\n", sms, clk);
  int blocks = sms * 8, threads = 256; size_t nt = (size_t)blocks*threads;
  double *o64; float *o32; CK(cudaMalloc(&o64, nt*8)); CK(cudaMalloc(&o32, nt*4));
  cudaEvent_t e0, e1; cudaEventCreate(&e0); cudaEventCreate(&e1); float ms;
  int it = 4096;
  for (int rep = 0; rep < 2; ++rep) {
  fma64<<<blocks,threads>>>(o64, it, 0.999, 1e-3); CK(cudaDeviceSynchronize());
  cudaEventRecord(e0); fma64<<<blocks,threads>>>(o64, it, 0.999, 1e-3); cudaEventRecord(e1); CK(cudaEventSynchronize(e1));
  cudaEventElapsedTime(&ms, e0, e1); printf("FP64 FMA: %.3f TFLOP/s (%.3f ms)\n", 2.0*8*it*nt/ms/1e9, ms);
  fma32<<<blocks,threads>>>(o32, it*8, 0.999f, 1e-3f); CK(cudaDeviceSynchronize());
  cudaEventRecord(e0); fma32<<<blocks,threads>>>(o32, it*8, 0.999f, 1e-3f); cudaEventRecord(e1); CK(cudaEventSynchronize(e1));
  cudaEventElapsedTime(&ms, e0, e1); printf("FP32 FMA: %.3f TFLOP/s (%.3f ms)\n", 2.0*8*it*8*nt/ms/1e9, ms);
  dmma<<<blocks,threads>>>(o64, it/4); CK(cudaDeviceSynchronize());
  cudaEventRecord(e0); dmma<<<blocks,threads>>>(o64, it/4); cudaEventRecord(e1); CK(cudaEventSynchronize(e1));
  cudaEventElapsedTime(&ms, e0, e1); printf("DMMA m8n8k4: %.3f TFLOP/s (%.3f ms)\n", 2.0*8*8*4*4*(it/4)*(nt/32)/ms/1e9, ms);
  fmalat<<<1,32>>>(o64, 100000, 0.999, 1e-3); CK(cudaDeviceSynchronize());
  cudaEventRecord(e0); fmalat<<<1,32>>>(o64, 100000, 0.999, 1e-3); cudaEventRecord(e1); CK(cudaEventSynchronize(e1));
  cudaEventElapsedTime(&ms, e0, e1); printf("FP64 FMA dep-chain latency: %.1f ns/op\n", ms*1e6/100000);
  divlat<<<1,32>>>(o64, 20000, 0.7); CK(cudaDeviceSynchronize());
  cudaEventRecord(e0); divlat<<<1,32>>>(o64, 20000, 0.7); cudaEventRecord(e1); CK(cudaEventSynchronize(e1));
  cudaEventElapsedTime(&ms, e0, e1); printf("FP64 div dep-chain latency: %.1f ns/op\n", ms*1e6/20000);
  }
  size_t n2 = (size_t)1 << 27; // 2 GiB per buffer in double2
  double2 *a, *b; CK(cudaMalloc(&a, n2*16)); CK(cudaMalloc(&b, n2*16)); CK(cudaMemset(a, 0, n2*16));
  for (int rep = 0; rep < 3; ++rep) {
    cudaEventRecord(e0); copyk<<<sms*4, 512>>>(a, b, n2); cudaEventRecord(e1); CK(cudaEventSynchronize(e1));
    cudaEventElapsedTime(&ms, e0, e1); printf("copy: %.1f GB/s\n", 2.0*n2*16/ms/1e6);
  }
  return 0;
}
