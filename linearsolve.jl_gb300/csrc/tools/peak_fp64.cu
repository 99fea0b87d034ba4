// FP64 fused-multiply-add throughput of a register-only loop, reported beside
// the FP64 roofline fractions (the FP64 trailing update runs on the FP64 pipe;
// tcgen05 has no FP64 kind).  On GB300 such loops top out near 1.0-1.1
// TFLOP/s, below what a DFMA GEMM reaches, so the fractions use the nominal
// rate.  Registers only; one store per thread.
#include <cuda_runtime.h>
#include <stdint.h>

namespace {
__global__ void dfma_loop(double* out, int iters, double s) {
  double a[8];
  for (int i = 0; i < 8; i++) a[i] = threadIdx.x * 1e-3 + i;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int i = 0; i < 8; i++) a[i] = fma(a[i], s, 1e-7);
  }
  double t = 0;
  for (int i = 0; i < 8; i++) t += a[i];
  out[blockIdx.x * blockDim.x + threadIdx.x] = t;
}
}  // namespace

extern "C" int32_t gblu_tool_peak_fp64(int32_t device, double* tflops) {
  if (!tflops) return 1;
  if (cudaSetDevice(device) != cudaSuccess) return 2;
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  const int blocks = sms * 4, threads = 256, iters = 20000;
  double* d = nullptr;
  if (cudaMalloc(&d, sizeof(double) * blocks * threads) != cudaSuccess) return 3;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  dfma_loop<<<blocks, threads>>>(d, 200, 0.999);
  float best = 1e30f;
  for (int rep = 0; rep < 3; ++rep) {
    cudaEventRecord(e0);
    dfma_loop<<<blocks, threads>>>(d, iters, 0.999);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best) best = ms;
  }
  cudaError_t err = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(d);
  if (err != cudaSuccess) return 4;
  *tflops = 2.0 * 8 * iters * (double)blocks * threads / (best * 1e-3) / 1e12;
  return 0;
}
