// Self-test of the bounded device waits: one small kernel waits on something
// nothing will ever provide and must give up after the wait limit with the
// expected error code, leaving the context usable.
//   which 0: the cooperative panel's grid barrier (a count nothing reaches)
//   which 1: getrs value polling (a sentinel nothing overwrites)
//   which 2: the register panel's mbarrier wait (a phase nothing completes)
// No trap, no fault, no endless loop: each wait reads %globaltimer and
// returns.
#include <cuda_runtime.h>
#include <stdint.h>

#include <chrono>

#include "../device_util.cuh"
#include "../waits.cuh"

namespace {

__global__ void wait_check_kernel(int which, gblu::DevScratch* scr, const double* sentinel, int* ok_out) {
  __shared__ __align__(8) unsigned long long bar;
  int ok = 1;
  if (which == 0) {
    // one CTA, target 2: the count reaches 1 only
    ok = gblu::grid_barrier(scr, 2u) ? 1 : 0;
  } else if (which == 1) {
    if (threadIdx.x == 0) {
      double v = 0.0;
      ok = gblu::poll_value(sentinel, scr, &v) ? 1 : 0;
    }
  } else {
    if (threadIdx.x == 0) gblu::pan_bar_init(gblu::pan_saddr(&bar));  // count 1, never armed
    __syncthreads();
    if (threadIdx.x == 0) ok = gblu::pan_bar_wait(gblu::pan_saddr(&bar), 0u, &scr->error) ? 1 : 0;
  }
  if (threadIdx.x == 0) *ok_out = ok;
}

}  // namespace

// code: the DEV_* word the wait left (0 = none); gave_up: 1 when the wait
// returned false; seconds: host wall time of the launch.
extern "C" int32_t gblu_tool_waitcheck(int32_t which, int32_t* code, int32_t* gave_up, double* seconds) {
  if (!code || !gave_up || !seconds || which < 0 || which > 2) return 1;
  gblu::DevScratch* scr = nullptr;
  double* sentinel = nullptr;
  int* ok = nullptr;
  if (cudaMalloc(&scr, sizeof(gblu::DevScratch)) != cudaSuccess) return 2;
  if (cudaMalloc(&sentinel, sizeof(double)) != cudaSuccess || cudaMalloc(&ok, sizeof(int)) != cudaSuccess) {
    cudaFree(scr);
    return 2;
  }
  cudaMemset(scr, 0, sizeof(gblu::DevScratch));
  cudaMemset(sentinel, 0xFF, sizeof(double));  // the all-ones sentinel
  cudaMemset(ok, 0xFF, sizeof(int));
  const auto t0 = std::chrono::steady_clock::now();
  wait_check_kernel<<<1, 32>>>(which, scr, sentinel, ok);
  cudaError_t e = cudaDeviceSynchronize();
  const auto t1 = std::chrono::steady_clock::now();
  *seconds = std::chrono::duration<double>(t1 - t0).count();
  gblu::DevScratch hs{};
  int hok = -1;
  if (e == cudaSuccess) e = cudaMemcpy(&hs, scr, sizeof(hs), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(&hok, ok, sizeof(int), cudaMemcpyDeviceToHost);
  cudaFree(scr);
  cudaFree(sentinel);
  cudaFree(ok);
  if (e != cudaSuccess) return 3;
  *code = hs.error;
  *gave_up = hok == 0 ? 1 : 0;
  return 0;
}
