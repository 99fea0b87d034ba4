// Bounded waits on values published by other CTAs and the mbarrier steps of
// the panel exchange, shared by the kernels and the wait self-test.  Every
// wait gives up after kSpinTimeoutNs of %globaltimer, records a DEV_* code in
// the scratch error word and returns false; it never traps or spins forever.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "device_util.cuh"

namespace gblu {

// Published solution values are polled directly: the buffers a sweep's
// dependents read are filled with an all-ones bit pattern (a NaN no
// computation produces, outputs are written with canonical NaNs) before the
// sweep, and each 4/8-byte value is single-copy atomic, so a value that is not
// the sentinel is final.  This saves the flag round trip per tile.
template <typename T>
struct SweepBits;
template <>
struct SweepBits<double> {
  using U = unsigned long long;
  static constexpr U kSentinel = ~0ull;
  static __device__ __forceinline__ U load(const double* p) {
    U v;
    asm volatile("ld.relaxed.gpu.global.b64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
  }
  static __device__ __forceinline__ double as_t(U v) { return __longlong_as_double((long long)v); }
  // NaN -> the canonical quiet NaN, on the integer pipe
  static __device__ __forceinline__ double canon(double v) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(v);
    return (b << 1) > 0xffe0000000000000ull ? __longlong_as_double(0x7ff8000000000000ll) : v;
  }
};
template <>
struct SweepBits<float> {
  using U = unsigned;
  static constexpr U kSentinel = ~0u;
  static __device__ __forceinline__ U load(const float* p) {
    U v;
    asm volatile("ld.relaxed.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
  }
  static __device__ __forceinline__ float as_t(U v) { return __uint_as_float(v); }
  static __device__ __forceinline__ float canon(float v) {
    return (__float_as_uint(v) << 1) > 0xff000000u ? __uint_as_float(0x7fc00000u) : v;
  }
};

// Wait for one published value; false on timeout or when another CTA failed.
template <typename T>
__device__ __forceinline__ bool poll_value(const T* p, DevScratch* scr, T* out) {
  using B = SweepBits<T>;
  unsigned long long t0 = 0;
  for (unsigned it = 0;; ++it) {
    const typename B::U v = B::load(p);
    if (v != B::kSentinel) { *out = B::as_t(v); return true; }
    if ((it & 63u) == 63u) {
      if (ld_volatile_i32(&scr->error) != 0) return false;
      const unsigned long long now = global_ns();
      if (t0 == 0) t0 = now;
      else if (now - t0 > kSpinTimeoutNs) {
        atomicCAS(&scr->error, 0, (int)DEV_TIMEOUT_SOLVE);
        return false;
      }
    }
  }
}

// Shared-memory addresses, cluster mapping, st.async and the mbarrier steps
// of the panel exchange.
__device__ __forceinline__ uint32_t pan_saddr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ uint32_t pan_mapa(uint32_t a, int rank) {
  uint32_t r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(rank));
  return r;
}
__device__ __forceinline__ void pan_st_async(uint32_t raddr, int4 v, uint32_t rbar) {
  asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.v4.b32 [%0], {%1, %2, %3, %4}, [%5];"
               ::"r"(raddr), "r"(v.x), "r"(v.y), "r"(v.z), "r"(v.w), "r"(rbar)
               : "memory");
}
__device__ __forceinline__ void pan_bar_init(uint32_t a) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(a) : "memory");
}
__device__ __forceinline__ void pan_bar_arm(uint32_t a, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(a), "r"(bytes) : "memory");
}
// Bounded wait for the phase of the given parity; false when it gave up
// (the error word is set).
__device__ __forceinline__ bool pan_bar_wait(uint32_t a, uint32_t parity, int* err) {
  unsigned long long t0 = 0;
  for (uint32_t it = 0;; ++it) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(a), "r"(parity)
        : "memory");
    if (ok) return true;
    if ((it & 63u) == 0) {
      const unsigned long long now = global_ns();
      if (t0 == 0) t0 = now;
      else if (now - t0 > kSpinTimeoutNs) {
        atomicCAS(err, 0, (int)DEV_TIMEOUT_PANEL);
        return false;
      }
    }
  }
}

}  // namespace gblu
