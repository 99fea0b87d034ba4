// Bitwise check of the library's Markstein division against the IEEE division
// on random operands (all significands, including the all-ones and power-of-two
// edge cases, and exponents across the range where the fast path is used).
#include <cuda_runtime.h>
#include <stdint.h>

#include "../device_util.cuh"

namespace {
__device__ __forceinline__ uint64_t mix64(uint64_t x) {
  x ^= x >> 33; x *= 0xff51afd7ed558ccdull; x ^= x >> 33; x *= 0xc4ceb9fe1a85ec53ull; x ^= x >> 33;
  return x;
}
template <typename T, typename U>
__device__ T make_operand(uint64_t h, int kind);
template <>
__device__ double make_operand<double, uint64_t>(uint64_t h, int kind) {
  uint64_t mant = h & ((1ull << 52) - 1);
  if (kind == 1) mant = (1ull << 52) - 1;        // all-ones significand
  if (kind == 2) mant = 0;                        // power of two
  if (kind == 3) mant = (h >> 7) & 0xFull;        // just above a power of two
  const uint64_t e = 1023 + (int64_t)((h >> 52) % 800) - 400;  // |x| in [2^-400, 2^400)
  const uint64_t sign = (h >> 63) << 63;
  return __longlong_as_double((long long)(sign | (e << 52) | mant));
}
template <>
__device__ float make_operand<float, uint32_t>(uint64_t h, int kind) {
  uint32_t mant = (uint32_t)h & ((1u << 23) - 1);
  if (kind == 1) mant = (1u << 23) - 1;
  if (kind == 2) mant = 0;
  if (kind == 3) mant = (uint32_t)(h >> 7) & 0xFu;
  const uint32_t e = 127 + (int32_t)((h >> 40) % 80) - 40;
  const uint32_t sign = (uint32_t)(h >> 63) << 31;
  return __uint_as_float(sign | (e << 23) | mant);
}

template <typename T, typename U>
__global__ void divcheck_kernel(uint64_t seed, int64_t n, unsigned long long* mismatches) {
  unsigned long long bad = 0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t h1 = mix64(seed ^ (2 * i + 1)), h2 = mix64(seed + 0x9e3779b97f4a7c15ull * (i + 7));
    const int ka = (int)(h1 & 7) < 4 ? (int)(h1 & 3) : 0, kb = (int)(h2 & 7) < 4 ? (int)(h2 & 3) : 0;
    const T a = make_operand<T, U>(h1, ka), b = make_operand<T, U>(h2, kb);
    const T y = T(1) / b;
    const T q1 = a / b, q2 = gblu::div_markstein(a, b, y);
    if (sizeof(T) == 8) {
      if (__double_as_longlong((double)q1) != __double_as_longlong((double)q2)) ++bad;
    } else {
      if (__float_as_uint((float)q1) != __float_as_uint((float)q2)) ++bad;
    }
  }
  if (bad) atomicAdd(mismatches, bad);
}
}  // namespace

// Returns the number of operand pairs (out of n per type) whose quotients differ.
extern "C" int32_t gblu_tool_divcheck(int64_t n, uint64_t seed, uint64_t* mism_f64, uint64_t* mism_f32) {
  unsigned long long* d = nullptr;
  if (cudaMalloc(&d, 2 * sizeof(unsigned long long)) != cudaSuccess) return 1;
  cudaMemset(d, 0, 2 * sizeof(unsigned long long));
  divcheck_kernel<double, uint64_t><<<1024, 256>>>(seed, n, d);
  divcheck_kernel<float, uint32_t><<<1024, 256>>>(seed ^ 0x5555, n, d + 1);
  unsigned long long h[2] = {0, 0};
  cudaError_t e = cudaMemcpy(h, d, sizeof(h), cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (e != cudaSuccess) return 2;
  *mism_f64 = h[0];
  *mism_f32 = h[1];
  return 0;
}
