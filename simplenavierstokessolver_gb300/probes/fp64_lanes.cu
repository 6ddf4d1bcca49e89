// Does an FP64 warp instruction with few active lanes cost fewer FP64-pipe cycles?
// Each active lane runs a dependent chain (like a Thomas sweep); we vary active lanes per warp
// and the number of warps per SM. All writes in bounds: one store per thread.
#include <cstdio>
#include <cuda_runtime.h>

__global__ void chain(double *out, int active, int iters, double a, double b) {
  const int lane = threadIdx.x & 31;
  double x = threadIdx.x * 1e-3, y = x + 1.0;
  if (lane < active) {
    for (int i = 0; i < iters; i++) {
      x = a * (x - b * y);   // 3 dependent ops like the forward sweep, two chains
      y = a * (y - b * x);
    }
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x + y;
}

int main() {
  int sms;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0);
  double *buf;
  cudaMalloc(&buf, sizeof(double) * 152 * 4 * 32 * 8);
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  const int iters = 4096;
  for (int warps_per_block : {1, 4}) {
    for (int blocks : {17, 152, 608}) {
      for (int active : {1, 2, 4, 8, 16, 32}) {
        if (blocks * warps_per_block > 152 * 4 * 8) continue;
        chain<<<blocks, 32 * warps_per_block>>>(buf, active, 16, 0.999, 0.001);
        cudaEventRecord(e0);
        chain<<<blocks, 32 * warps_per_block>>>(buf, active, iters, 0.999, 0.001);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float ms;
        cudaEventElapsedTime(&ms, e0, e1);
        const double cyc = ms * 1e-3 * 2.0e9 / iters;  // cycles per iteration (6 FP64 ops, 2 chains)
        printf("warps/block %d blocks %4d active %2d : %8.3f ms  %7.1f cycles/iter  chains %d\n", warps_per_block,
               blocks, active, ms, cyc, blocks * warps_per_block * active);
      }
    }
  }
  cudaError_t err = cudaDeviceSynchronize();
  printf("status %s\n", cudaGetErrorString(err));
  return err == cudaSuccess ? 0 : 1;
}
