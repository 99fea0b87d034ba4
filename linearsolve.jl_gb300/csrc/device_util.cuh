// Device helpers shared by the kernels: bounded waits, coherent loads.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "gblu_internal.h"

namespace gblu {

// Every spin-wait in this library gives up after this many nanoseconds of
// %globaltimer and records an error word instead of hanging the GPU.
constexpr unsigned long long kSpinTimeoutNs = 2000000000ull;  // 2 s

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ int ld_acquire_i32(const int* p) {
  int v;
  asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void st_release_i32(int* p, int v) {
  asm volatile("st.release.gpu.global.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ int ld_volatile_i32(const int* p) {
  return *(volatile const int*)p;
}

// Named CTA barrier `id` (1..15) over `nthreads` threads (a multiple of 32):
// arrive does not wait, sync waits for all nthreads.
__device__ __forceinline__ void named_bar_arrive(int id, int nthreads) {
  asm volatile("bar.arrive %0, %1;" ::"r"(id), "r"(nthreads) : "memory");
}
__device__ __forceinline__ void named_bar_sync(int id, int nthreads) {
  asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(nthreads) : "memory");
}

// Grid-wide barrier for cooperative launches.  Arrival counter is
// s->barrier (zeroed before the launch); `target` = (#barriers so far) * G.
// Returns false (on every thread of the CTA) when the wait timed out or another
// CTA already recorded an error; the caller then leaves the kernel.
__device__ __forceinline__ bool grid_barrier(DevScratch* s, unsigned target) {
  __shared__ int ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    atomicAdd(&s->barrier, 1u);
    int res = 1;
    unsigned long long t0 = 0;
    for (unsigned it = 0;; ++it) {
      if (ld_acquire_u32(&s->barrier) >= target) break;
      if (ld_volatile_i32(&s->error) != 0) { res = 0; break; }
      if ((it & 63u) == 0) {
        unsigned long long now = global_ns();
        if (t0 == 0) t0 = now;
        else if (now - t0 > kSpinTimeoutNs) {
          atomicCAS(&s->error, 0, (int)DEV_TIMEOUT_PANEL);
          res = 0;
          break;
        }
      }
    }
    __threadfence();
    ok = res;
  }
  __syncthreads();
  return ok != 0;
}

// Pivot candidates are compared by integer keys: the bit pattern of |a|, which
// orders non-negative floating-point values like the values themselves, with
// NaN mapped to 0 so it never becomes a candidate (the reference's `v > amax`
// is false for NaN).  This keeps the reductions off the FP64 pipe.
template <typename T>
struct PivKey;
template <>
struct PivKey<double> {
  using K = unsigned long long;
  static __device__ __forceinline__ K of(double x) {
    const K a = (K)__double_as_longlong(x) & 0x7fffffffffffffffull;
    return a > 0x7ff0000000000000ull ? 0ull : a;
  }
  // x != 0 (NaN counts as nonzero, as in `x != 0.0`)
  static __device__ __forceinline__ bool nonzero(double x) {
    return ((K)__double_as_longlong(x) << 1) != 0ull;
  }
};
template <>
struct PivKey<float> {
  using K = unsigned;
  static __device__ __forceinline__ K of(float x) {
    const K a = __float_as_uint(x) & 0x7fffffffu;
    return a > 0x7f800000u ? 0u : a;
  }
  static __device__ __forceinline__ bool nonzero(float x) { return (__float_as_uint(x) << 1) != 0u; }
};

// Warp-wide pivot choice: every lane holds a candidate (key v, row g; g < 0 =
// none); on return every lane holds the winner (largest key, then smallest
// row) and `src` = the lane it came from (-1 when no lane has a candidate).
// Built from the warp reduction instructions: one max per 32-bit half of the
// key (the low half compared only among lanes holding the largest high
// half), one min over the rows holding the largest key, one ballot.  Rows
// are unique across lanes.
template <typename K>
__device__ __forceinline__ void warp_pivot_choice(K& v, int& g, int& src) {
  constexpr unsigned kAll = 0xffffffffu;
  if constexpr (sizeof(K) == 4) {
    const unsigned vm = g >= 0 ? (unsigned)v : 0u;
    const unsigned mk = __reduce_max_sync(kAll, vm);
    const bool mine = g >= 0 && vm == mk;
    const unsigned gmin = __reduce_min_sync(kAll, mine ? (unsigned)g : 0xffffffffu);
    const unsigned who = __ballot_sync(kAll, mine && (unsigned)g == gmin);
    src = who ? __ffs(who) - 1 : -1;
    v = who ? (K)mk : K(0);
    g = who ? (int)gmin : -1;
  } else {
    const unsigned long long vm = g >= 0 ? (unsigned long long)v : 0ull;
    const unsigned hi = (unsigned)(vm >> 32), lo = (unsigned)vm;
    const unsigned mh = __reduce_max_sync(kAll, hi);
    const unsigned ml = __reduce_max_sync(kAll, hi == mh ? lo : 0u);
    const bool mine = g >= 0 && hi == mh && lo == ml;
    const unsigned gmin = __reduce_min_sync(kAll, mine ? (unsigned)g : 0xffffffffu);
    const unsigned who = __ballot_sync(kAll, mine && (unsigned)g == gmin);
    src = who ? __ffs(who) - 1 : -1;
    v = who ? (K)(((unsigned long long)mh << 32) | ml) : K(0);
    g = who ? (int)gmin : -1;
  }
}

// Correctly rounded a / b from y = RN(1/b), following Markstein's division
// (P. Markstein, IBM J. Res. Develop. 34(1):111-119, 1990): q = RN(a*y) is
// within one ulp of a/b, the remainder r = a - b*q is exact with one fused
// multiply-add, and RN(q + r*y) is the correctly rounded quotient.  The
// sequence needs q, y and r*y clear of underflow and overflow; outside that
// range (and for zeros, infinities and NaNs) the IEEE division is used.
// The range test is done on the exponent bits with integer arithmetic: on
// this GPU a floating-point comparison of doubles occupies the FP64 pipe.
// in_range(x): 2^-960 <= |x| < 2^960 (double), 2^-100 <= |x| < 2^100 (float);
// zero, subnormals, infinities and NaN are outside.
template <typename T>
struct DivRange;
template <>
struct DivRange<double> {
  static __device__ __forceinline__ bool in_range(double x) {
    const unsigned e = ((unsigned)(__double_as_longlong(x) >> 52)) & 0x7ffu;  // biased exponent
    return e - (1023u - 960u) < 2u * 960u;  // 1023-960 <= e < 1023+960
  }
};
template <>
struct DivRange<float> {
  static __device__ __forceinline__ bool in_range(float x) {
    const unsigned e = (__float_as_uint(x) >> 23) & 0xffu;
    return e - (127u - 100u) < 2u * 100u;  // 127-100 <= e < 127+100
  }
};

template <typename T>
__device__ __forceinline__ T div_markstein(T a, T b, T y) {
  const T q = a * y;
  if (!(DivRange<T>::in_range(q) && DivRange<T>::in_range(y))) return a / b;
  const T r = fma(-b, q, a);
  return fma(r, y, q);
}

// a[i] / b for N > 1 dividends with one divisor, as N independent chains
// without branches in the common case (so the compiler can interleave them;
// with one dividend the plain div_markstein is faster).  A zero
// dividend gives q = a*y, which is the correctly signed zero a/b; any other
// operand outside the safe range sends all N through the IEEE division.
template <typename T, int N>
__device__ __forceinline__ void div_markstein_n(T (&a)[N], T b, T y) {
  bool bad = !DivRange<T>::in_range(y);
  T res[N];
#pragma unroll
  for (int i = 0; i < N; ++i) {
    const T q = a[i] * y;
    const bool zero = !PivKey<T>::nonzero(a[i]);
    bad |= !zero && !DivRange<T>::in_range(q);
    const T r = fma(-b, q, a[i]);
    res[i] = zero ? q : fma(r, y, q);
  }
  if (bad) {
#pragma unroll
    for (int i = 0; i < N; ++i) res[i] = a[i] / b;
  }
#pragma unroll
  for (int i = 0; i < N; ++i) a[i] = res[i];
}

// IEEE 754 binary64 -> binary32 with round-to-nearest-even, on integer
// operations only (the FP64 pipe of this GPU retires two lanes per cycle per
// SM, so a conversion there costs as much as an FP64 FMA).  The standard's
// narrowing: keep 23 of the 52 fraction bits and round on the other 29
// (ties to even; a carry out of the fraction increments the exponent, and
// past the largest finite value gives infinity); results below the normal
// range are denormalised from the full 53-bit significand; NaN stays NaN
// (quiet, upper payload bits kept).  Checked bitwise against the hardware
// conversion by gblu_tool_cvtcheck.
__device__ __forceinline__ float f64_to_f32_rn(double d) {
  const unsigned long long u = (unsigned long long)__double_as_longlong(d);
  const unsigned sign = (unsigned)(u >> 32) & 0x80000000u;
  const int e = (int)((u >> 52) & 0x7FF);
  const unsigned long long m = u & 0xFFFFFFFFFFFFFull;
  if (e == 0x7FF) return __uint_as_float(sign | 0x7F800000u | (m ? 0x00400000u | (unsigned)(m >> 29) : 0u));
  const int fe = e - 1023 + 127;
  if (fe >= 0xFF) return __uint_as_float(sign | 0x7F800000u);
  if (fe <= 0) {
    const int shift = 926 - e;  // value = (2^52 + m) 2^(e - 1075) = f 2^-149
    if (e == 0 || shift > 54) return __uint_as_float(sign);
    const unsigned long long M = m | (1ull << 52);
    const unsigned long long f = M >> shift, rem = M & ((1ull << shift) - 1), half = 1ull << (shift - 1);
    const unsigned r = (unsigned)f + ((rem > half || (rem == half && (f & 1ull))) ? 1u : 0u);
    return __uint_as_float(sign | r);
  }
  const unsigned long long f = m >> 29, rem = m & 0x1FFFFFFFull;
  unsigned bits = ((unsigned)fe << 23) | (unsigned)f;
  bits += (rem > 0x10000000ull || (rem == 0x10000000ull && (f & 1ull))) ? 1u : 0u;
  return __uint_as_float(sign | bits);
}

template <typename T>
__device__ __forceinline__ T ldcg(const T* p) { return __ldcg(p); }
template <typename T>
__device__ __forceinline__ void stcg(T* p, T v) { __stcg(p, v); }

}  // namespace gblu
