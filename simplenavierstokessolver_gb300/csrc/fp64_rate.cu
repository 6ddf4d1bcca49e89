// FP64 issue rate of the current GPU: the denominator of the plain path's
// FP64 roofline. The plain FP64 kernels are bound by FP64 instruction issue on
// GB300 (its FP64 pipe runs at about 1/73 of the FP32 rate), so bench.py puts
// their operation counts against this measured rate rather than a constant.
//
// Each thread advances eight independent chains, so the pipe, not the
// dependent-operation latency, sets the pace; the grid covers every SM eight
// blocks deep. Additions and multiplications are timed separately (the plain
// path issues no fused multiply-adds).
#include <cuda_runtime.h>

#include "sns_gpu.h"
#include "sns_internal.h"

namespace sns {
namespace {

constexpr int kRateIters = 4096;
constexpr int kRateThreads = 256;
constexpr int kRateBlocksPerSm = 8;

template <int OP>
__global__ void __launch_bounds__(kRateThreads) k_fp64_rate(double *out, double a, double b) {
  double x[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) x[k] = threadIdx.x + k;
#pragma unroll 4
  for (int i = 0; i < kRateIters; ++i) {
#pragma unroll
    for (int k = 0; k < 8; ++k) x[k] = OP == 0 ? __dadd_rn(x[k], k < 4 ? a : b) : __dmul_rn(x[k], k < 4 ? a : b);
  }
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < 8; ++k) s += x[k];
  out[(size_t)blockIdx.x * blockDim.x + threadIdx.x] = s;
}

}  // namespace
}  // namespace sns

using namespace sns;

extern "C" int sns_fp64_issue_rate(double out[2]) {
  if (!out) {
    record_error("sns_fp64_issue_rate: NULL output");
    return SNS_ERR_ARG;
  }
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) !=
                                                   cudaSuccess) {
    cudaGetLastError();
    record_error("sns_fp64_issue_rate: no CUDA device");
    return SNS_ERR_CUDA;
  }
  const int blocks = sms * kRateBlocksPerSm;
  double *buf = nullptr;
  cudaStream_t st = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int rc = SNS_OK;
  const double ops = (double)blocks * kRateThreads * kRateIters * 8.0;
  auto ok = [&](cudaError_t e) {
    if (e == cudaSuccess) return true;
    record_error(cudaGetErrorString(e));
    rc = SNS_ERR_CUDA;
    return false;
  };
  if (ok(counted_malloc(&buf, sizeof(double) * (size_t)blocks * kRateThreads)) &&
      ok(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking)) && ok(cudaEventCreate(&e0)) &&
      ok(cudaEventCreate(&e1))) {
    for (int op = 0; op < 2 && rc == SNS_OK; ++op) {
      auto launch = [&] {
        if (op == 0)
          k_fp64_rate<0><<<blocks, kRateThreads, 0, st>>>(buf, 1e-7, 2e-7);
        else
          k_fp64_rate<1><<<blocks, kRateThreads, 0, st>>>(buf, 1.0000001, 0.9999999);
        count_launches(1);
      };
      launch();  // warm-up
      launch();
      float ms = 0.f;
      if (!ok(cudaEventRecord(e0, st))) break;
      for (int r = 0; r < 3; ++r) launch();
      if (!ok(cudaEventRecord(e1, st)) || !ok(cudaEventSynchronize(e1)) || !ok(cudaEventElapsedTime(&ms, e0, e1)))
        break;
      out[op] = 3.0 * ops / (ms * 1e-3) / 1e9;
    }
  }
  if (rc == SNS_OK) ok(cudaGetLastError());
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (st) cudaStreamDestroy(st);
  if (buf) cudaFree(buf);
  return rc;
}
