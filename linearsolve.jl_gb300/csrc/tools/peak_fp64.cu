// FP64 fused-multiply-add throughput of this GPU, the denominator of the FP64
// roofline fractions (the FP64 trailing update runs on the FP64 pipe; tcgen05
// has no FP64 kind).
//
// Each thread keeps a 4 x 4 block of accumulators and updates it with
// c[i][j] = fma(a[i], b[j], c[i][j]) from eight register operands, the
// instruction mix of the DFMA GEMM's inner loop: 16 independent chains per
// thread, every operand in a register (no constant-bank operands), one store
// per thread at the end.  The launch shape (CTAs per SM x threads) is swept
// and the best event-timed rate kept; every shape keeps at least 8 warps per
// SM so the 64-cycle DFMA latency is covered many times over.
#include <cuda_runtime.h>
#include <stdint.h>

namespace {
__global__ void dfma_block(const double* __restrict__ in, double* __restrict__ out, int iters) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  double a[4], b[4], c[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    a[i] = in[(t + i) & 63];
    b[i] = in[(t + 4 + i) & 63];
  }
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) c[i][j] = 0.0;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) c[i][j] = fma(a[i], b[j], c[i][j]);
  }
  double s = 0.0;
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) s += c[i][j];
  out[t] = s;
}
}  // namespace

// Best FP64 FMA rate (TFLOP/s, 2 flops per FMA) over the swept launch shapes;
// shape_out (may be NULL) receives {CTAs per SM, threads per CTA} of the best.
extern "C" int32_t gblu_tool_peak_fp64_shape(int32_t device, double* tflops, int32_t* shape_out) {
  if (!tflops) return 1;
  if (cudaSetDevice(device) != cudaSuccess) return 2;
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  const int shapes[][2] = {{1, 256}, {2, 256}, {4, 256}, {1, 512}, {2, 512}, {1, 1024}};
  const int iters = 4096;
  const size_t max_threads = (size_t)sms * 4 * 256;
  double *din = nullptr, *dout = nullptr;
  if (cudaMalloc(&din, 64 * sizeof(double)) != cudaSuccess) return 3;
  if (cudaMalloc(&dout, max_threads * sizeof(double)) != cudaSuccess) {
    cudaFree(din);
    return 3;
  }
  double h[64];
  for (int i = 0; i < 64; ++i) h[i] = 1e-3 * (1 + (i % 7));  // c stays O(iters * 1e-5)
  cudaMemcpy(din, h, sizeof(h), cudaMemcpyHostToDevice);
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  double best = 0.0;
  int best_shape[2] = {0, 0};
  for (const auto& sh : shapes) {
    const int blocks = sms * sh[0], threads = sh[1];
    dfma_block<<<blocks, threads>>>(din, dout, 64);  // warm-up
    for (int rep = 0; rep < 3; ++rep) {
      cudaEventRecord(e0);
      dfma_block<<<blocks, threads>>>(din, dout, iters);
      cudaEventRecord(e1);
      cudaEventSynchronize(e1);
      float ms = 0;
      cudaEventElapsedTime(&ms, e0, e1);
      const double tf = 2.0 * 16.0 * iters * (double)blocks * threads / (ms * 1e-3) / 1e12;
      if (ms > 0 && tf > best) {
        best = tf;
        best_shape[0] = sh[0];
        best_shape[1] = sh[1];
      }
    }
  }
  cudaError_t err = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(din);
  cudaFree(dout);
  if (err != cudaSuccess) return 4;
  *tflops = best;
  if (shape_out) {
    shape_out[0] = best_shape[0];
    shape_out[1] = best_shape[1];
  }
  return 0;
}

extern "C" int32_t gblu_tool_peak_fp64(int32_t device, double* tflops) {
  return gblu_tool_peak_fp64_shape(device, tflops, nullptr);
}
