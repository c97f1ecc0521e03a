// probe.cu -- measured binary64 FMA throughput (the ceiling of the FP64 step
// kernel on GB300, whose FP64 rate is a small fraction of its FP32 rate).
#include <cuda_runtime.h>

#include "../../include/fv2d_gpu.h"

namespace {

// 8 independent FMA chains per thread; operands stay in registers.
__global__ void __launch_bounds__(256) dfma_loop(double *out, int iters, double b, double c) {
  double a0 = threadIdx.x * 1e-9, a1 = a0 + 1, a2 = a0 + 2, a3 = a0 + 3, a4 = a0 + 4, a5 = a0 + 5, a6 = a0 + 6,
         a7 = a0 + 7;
  for (int k = 0; k < iters; ++k) {
    a0 = fma(a0, b, c); a1 = fma(a1, b, c); a2 = fma(a2, b, c); a3 = fma(a3, b, c);
    a4 = fma(a4, b, c); a5 = fma(a5, b, c); a6 = fma(a6, b, c); a7 = fma(a7, b, c);
  }
  const double s = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
  if (s == 1.2345) out[blockIdx.x] = s;  // keeps the loop live
}

}  // namespace

extern "C" int fv2d_probe_fp64_peak(int device, double *gflops) {
  if (!gflops) return FV2D_ERR_INVALID;
  if (device >= 0 && cudaSetDevice(device) != cudaSuccess) return FV2D_ERR_CUDA;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  double *out = nullptr;
  if (cudaMalloc(&out, sizeof(double) * 8 * sms) != cudaSuccess) return FV2D_ERR_NOMEM;
  cudaStream_t s;
  cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  const int blocks = 8 * sms, threads = 256, iters = 4096;
  dfma_loop<<<blocks, threads, 0, s>>>(out, iters, 0.999999, 1e-7);  // warm-up
  float best = 1e30f;
  for (int r = 0; r < 5; ++r) {
    cudaEventRecord(e0, s);
    dfma_loop<<<blocks, threads, 0, s>>>(out, iters, 0.999999, 1e-7);
    cudaEventRecord(e1, s);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best) best = ms;
  }
  const cudaError_t err = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaStreamDestroy(s);
  cudaFree(out);
  if (err != cudaSuccess) return FV2D_ERR_CUDA;
  const double flops = 2.0 * 8.0 * (double)iters * (double)blocks * threads;
  *gflops = flops / (best * 1e-3) / 1e9;
  return FV2D_OK;
}
