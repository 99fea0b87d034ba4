// Bitwise check of the library's integer FP64 -> FP32 conversion
// (gblu::f64_to_f32_rn, used when the mixed factors convert A) against the
// hardware conversion with round-to-nearest-even, on random doubles: the
// whole exponent range (zeros, subnormals, overflow, infinities and NaNs
// included), exponents around the FP32 normal and subnormal boundaries, and
// fractions at and next to rounding ties.  NaN results compare by NaN-ness.
#include <cuda_runtime.h>
#include <stdint.h>

#include "../device_util.cuh"

namespace {
__device__ __forceinline__ uint64_t mix64(uint64_t x) {
  x ^= x >> 33; x *= 0xff51afd7ed558ccdull; x ^= x >> 33; x *= 0xc4ceb9fe1a85ec53ull; x ^= x >> 33;
  return x;
}

__device__ double make_value(uint64_t h, uint64_t h2) {
  const uint64_t sign = (h >> 63) << 63;
  uint64_t e, m = h2 & ((1ull << 52) - 1);
  switch (h & 7) {
    case 0: case 1: e = (h >> 3) & 0x7FF; break;                   // any exponent
    case 2: case 3: e = 1023 - 160 + ((h >> 3) % 300); break;      // FP32 range and its edges
    case 4: e = 1023 - 150 + ((h >> 3) % 30); break;               // FP32 subnormal range
    default: e = 1023 - 126 + ((h >> 3) % 254); break;             // FP32 normal range
  }
  const int tie = (int)((h >> 20) & 7);                            // rounding-tie fractions
  if (tie == 1) m = (m & ~0x1FFFFFFFull) | 0x10000000ull;
  if (tie == 2) m = (m & ~0x1FFFFFFFull) | 0x0FFFFFFFull;
  if (tie == 3) m = (m & ~0x1FFFFFFFull) | 0x10000001ull;
  if (tie == 4) m = (h >> 30) & 1 ? ((1ull << 52) - 1) : 0;        // all-ones / zero fraction
  return __longlong_as_double((long long)(sign | (e << 52) | m));
}

__global__ void cvtcheck_kernel(uint64_t seed, int64_t n, unsigned long long* mismatches) {
  unsigned long long bad = 0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double d = make_value(mix64(seed ^ (2 * i + 1)), mix64(seed + 0x9e3779b97f4a7c15ull * (i + 3)));
    const float a = gblu::f64_to_f32_rn(d), b = __double2float_rn(d);
    const bool same = __float_as_uint(a) == __float_as_uint(b) || (isnan(a) && isnan(b));
    if (!same) ++bad;
  }
  if (bad) atomicAdd(mismatches, bad);
}
}  // namespace

// Returns the number of doubles (out of n) whose conversions differ.
extern "C" int32_t gblu_tool_cvtcheck(int64_t n, uint64_t seed, uint64_t* mismatches) {
  unsigned long long* d = nullptr;
  if (cudaMalloc(&d, sizeof(unsigned long long)) != cudaSuccess) return 1;
  cudaMemset(d, 0, sizeof(unsigned long long));
  cvtcheck_kernel<<<1024, 256>>>(seed, n, d);
  unsigned long long h = 0;
  cudaError_t e = cudaMemcpy(&h, d, sizeof(h), cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (e != cudaSuccess) return 2;
  *mismatches = h;
  return 0;
}
