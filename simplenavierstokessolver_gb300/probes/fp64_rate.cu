// FP64 / FP32 / INT32 pipe throughput of this GPU: independent chains saturating each pipe.
#include <cstdio>
#include <cuda_runtime.h>

#define ITERS 4096

__global__ void k_dfma(double *out, double a, double b) {
  double x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0+4, x5=x0+5, x6=x0+6, x7=x0+7;
  for (int i = 0; i < ITERS; i++) {
    x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
    x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}
__global__ void k_dadd(double *out, double a, double b) {
  double x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0+4, x5=x0+5, x6=x0+6, x7=x0+7;
  for (int i = 0; i < ITERS; i++) {
    x0 = __dadd_rn(x0, a); x1 = __dadd_rn(x1, a); x2 = __dadd_rn(x2, a); x3 = __dadd_rn(x3, a);
    x4 = __dadd_rn(x4, b); x5 = __dadd_rn(x5, b); x6 = __dadd_rn(x6, b); x7 = __dadd_rn(x7, b);
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}
__global__ void k_dmul(double *out, double a, double b) {
  double x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0+4, x5=x0+5, x6=x0+6, x7=x0+7;
  for (int i = 0; i < ITERS; i++) {
    x0 = __dmul_rn(x0, a); x1 = __dmul_rn(x1, a); x2 = __dmul_rn(x2, a); x3 = __dmul_rn(x3, a);
    x4 = __dmul_rn(x4, b); x5 = __dmul_rn(x5, b); x6 = __dmul_rn(x6, b); x7 = __dmul_rn(x7, b);
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}
__global__ void k_ddiv(double *out, double a, double b) {
  double x0 = threadIdx.x + 1, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3;
  for (int i = 0; i < ITERS / 8; i++) {
    x0 = a / x0; x1 = b / x1; x2 = a / x2; x3 = b / x3;
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3;
}
__global__ void k_ffma(float *out, float a, float b) {
  float x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0+4, x5=x0+5, x6=x0+6, x7=x0+7;
  for (int i = 0; i < ITERS; i++) {
    x0 = fmaf(x0, a, b); x1 = fmaf(x1, a, b); x2 = fmaf(x2, a, b); x3 = fmaf(x3, a, b);
    x4 = fmaf(x4, a, b); x5 = fmaf(x5, a, b); x6 = fmaf(x6, a, b); x7 = fmaf(x7, a, b);
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}
__global__ void k_imad(unsigned *out, unsigned a, unsigned b) {
  unsigned x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0+4, x5=x0+5, x6=x0+6, x7=x0+7;
  for (int i = 0; i < ITERS; i++) {
    x0 = x0 * a + b; x1 = x1 * a + b; x2 = x2 * a + b; x3 = x3 * a + b;
    x4 = x4 * a + b; x5 = x5 * a + b; x6 = x6 * a + b; x7 = x7 * a + b;
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

int main() {
  int sms; cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0);
  int clk; cudaDeviceGetAttribute(&clk, cudaDevAttrClockRate, 0);
  printf("SMs %d clock(kHz) %d\n", sms, clk);
  const int blocks = sms * 8, threads = 256;
  void *buf; cudaMalloc(&buf, (size_t)blocks * threads * 8);
  cudaEvent_t e0, e1; cudaEventCreate(&e0); cudaEventCreate(&e1);
  float ms;
  double n = (double)blocks * threads * ITERS * 8;
#define RUN(name, launch, opsper) \
  for (int w = 0; w < 2; w++) launch; cudaEventRecord(e0); for (int r = 0; r < 3; r++) launch; cudaEventRecord(e1); \
  cudaEventSynchronize(e1); cudaEventElapsedTime(&ms, e0, e1); \
  printf("%-6s %10.1f Gop/s  (%.2f ops/clk/SM at max clock)\n", name, 3 * n * (opsper) / (ms * 1e-3) / 1e9, 3 * n * (opsper) / (ms * 1e-3) / (sms * clk * 1e3));
  RUN("dfma", (k_dfma<<<blocks, threads>>>((double *)buf, 1.0000001, 1e-7)), 1.0)
  RUN("dadd", (k_dadd<<<blocks, threads>>>((double *)buf, 1e-7, 2e-7)), 1.0)
  RUN("dmul", (k_dmul<<<blocks, threads>>>((double *)buf, 1.0000001, 0.9999999)), 1.0)
  RUN("ddiv", (k_ddiv<<<blocks, threads>>>((double *)buf, 1.0000001, 0.9999999)), 4.0 / 8 / 8)
  RUN("ffma", (k_ffma<<<blocks, threads>>>((float *)buf, 1.0000001f, 1e-7f)), 1.0)
  RUN("imad", (k_imad<<<blocks, threads>>>((unsigned *)buf, 1664525u, 1013904223u)), 1.0)
  cudaError_t err = cudaDeviceSynchronize();
  printf("status %s\n", cudaGetErrorString(err));
  return err == cudaSuccess ? 0 : 1;
}
