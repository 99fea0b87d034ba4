// Trailing update C -= A * B on the 5th-generation tensor cores (tcgen05).
//
// The mixed-precision getrf stores its working matrix in FP32; the trailing
// update -- the one dense contraction of LU (src/blocked_lufact.jl:186-656,
// A22 -= L21 * U12) -- rounds its two operands to BF16 or FP16 and accumulates
// in FP32 in tensor memory:
//
//   1. conversion kernels write A (M x K) and B (K x N) as K-major 16-bit
//      copies (FP16: each column of B scaled by an exact power of two so that
//      its largest entry lies in [2^14, 2^15); |L21| <= 1 needs no scale);
//   2. tc_gemm_kernel, persistent (one CTA per SM walking 128 x 256 output
//      tiles): one warp issues TMA loads (128-byte swizzled boxes of 64 x 128
//      and 64 x 256 elements, 4-stage mbarrier ring running across tile
//      boundaries), one thread issues tcgen05.mma (M=128, N=256, K=16 per
//      instruction) into one of two 256-column FP32 accumulators in TMEM, and
//      four warps read the other accumulator back with tcgen05.ld and apply
//      C -= acc * 2^-s in the epilogue (coalesced along the column-major C),
//      so a tile's epilogue overlaps the next tile's MMAs.
//
// All mbarrier waits are bounded (globaltimer, 2 s); an expired wait records
// DEV_TIMEOUT_GEMM, every CTA then skips to its teardown and frees TMEM.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>
#include <type_traits>

#include "device_util.cuh"
#include "gblu_internal.h"
#include "profile.h"

namespace gblu {
namespace tc {

// Output tiles BM x BN with BN = 256 where the tiles still cover the SMs
// (each 64-deep k slice then moves 48 KB from L2 for 128 x 256 x 64 MMAs, a
// quarter less traffic per flop than 128 x 128; two 256-column FP32
// accumulators fill the 512 TMEM columns), BN = 128 otherwise.
constexpr int BM = 128, BK = 64, THREADS = 192;
constexpr int UMMA_K = 16;
constexpr uint32_t A_BYTES = BM * BK * 2;
template <int BN> struct Tile {
  static constexpr int STAGES = BN == 256 ? 4 : 6;
  static constexpr uint32_t B_BYTES = BN * BK * 2;
  static constexpr uint32_t STAGE_BYTES = A_BYTES + B_BYTES;
  static constexpr uint32_t TMEM_COLS = 2 * BN;  // two accumulators: one drains while the other fills
  static constexpr size_t SMEM_BYTES = (size_t)STAGES * STAGE_BYTES + 1024 + 256;
};

__device__ __forceinline__ uint32_t saddr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint32_t a, uint32_t cnt) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(a), "r"(cnt) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint32_t a) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(a) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t a, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(a), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try(uint32_t a, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(a), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait; false when it gave up (error recorded) or another CTA failed.
__device__ __forceinline__ bool mbar_wait(uint32_t a, uint32_t parity, int* err) {
  unsigned long long t0 = 0;
  for (uint32_t it = 0;; ++it) {
    if (mbar_try(a, parity)) return true;
    if ((it & 127u) == 0) {
      if (ld_volatile_i32(err) != 0) return false;
      const unsigned long long now = global_ns();
      if (t0 == 0) t0 = now;
      else if (now - t0 > kSpinTimeoutNs) {
        atomicCAS(err, 0, (int)DEV_TIMEOUT_GEMM);
        return false;
      }
    }
  }
}
__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, int x, int y,
                                            uint32_t mbar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3}], [%4];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(mbar)
      : "memory");
}
__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tmem_alloc(uint32_t slot, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(slot),
               "r"(ncols)
               : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols)
               : "memory");
}
__device__ __forceinline__ void tc_mma(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc,
                                       uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}
__device__ __forceinline__ void tc_commit(uint32_t mbar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar)
      : "memory");
}
__device__ __forceinline__ void tmem_ld_32cols(uint32_t taddr, uint32_t (&v)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
      "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
      "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
        "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]),
        "=r"(v[14]), "=r"(v[15]), "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]),
        "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]), "=r"(v[24]), "=r"(v[25]),
        "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// Shared-memory matrix descriptor: K-major operand tile whose rows are 128
// bytes (64 16-bit elements) with the 128-byte swizzle; 8-row groups are
// 1024 bytes apart (stride byte offset); the leading byte offset is unused
// for swizzled K-major layouts.
__device__ __forceinline__ uint64_t sdesc_k128(uint32_t a) {
  return (uint64_t)((a & 0x3FFFFu) >> 4) | ((uint64_t)1 << 16) | ((uint64_t)(1024 >> 4) << 32) |
         ((uint64_t)1 << 46) | ((uint64_t)2 << 61);
}

// Instruction descriptor, kind::f16: D = F32, A/B = F16 (fmt 0) or BF16 (fmt 1),
// both K-major, N = BN, M = BM.
template <int BN>
__host__ __device__ constexpr uint32_t idesc_f16(uint32_t fmt) {
  return (1u << 4) | (fmt << 7) | (fmt << 10) | ((uint32_t)(BN >> 3) << 17) |
         ((uint32_t)(BM >> 4) << 24);
}

// Persistent: one CTA per SM walks the output tiles t = blockIdx.x,
// blockIdx.x + gridDim.x, ... (row-tile index fastest, so the CTAs of a wave
// share their B tiles in L2).  The producer's TMA ring runs across tile
// boundaries; the MMA issuer fills TMEM accumulator (i & 1) of the CTA's i-th
// tile while the epilogue warps drain the other one.
//   full[s] / empty[s]      smem stage s loaded / consumed (ring of STAGES)
//   tfull[b] / tempty[b]    accumulator b complete / drained (4 epilogue warps)
template <uint32_t FMT, int BN>
__global__ void __launch_bounds__(THREADS, 1)
tc_gemm_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
               float* __restrict__ C, int64_t ldc, int M, int N, int K,
               const float* __restrict__ inv_scale, int* __restrict__ err) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* smem =
      reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  constexpr int STAGES = Tile<BN>::STAGES;
  constexpr uint32_t STAGE_BYTES = Tile<BN>::STAGE_BYTES, TMEM_COLS = Tile<BN>::TMEM_COLS;
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + STAGES * STAGE_BYTES);
  uint64_t* full = bars;
  uint64_t* empty = bars + STAGES;
  uint64_t* tfull = bars + 2 * STAGES;       // [2]
  uint64_t* tempty = bars + 2 * STAGES + 2;  // [2]
  uint32_t* tslot = reinterpret_cast<uint32_t*>(bars + 2 * STAGES + 4);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int kblocks = (K + BK - 1) / BK;
  const int tiles_m = (M + BM - 1) / BM;
  const int tiles = tiles_m * ((N + BN - 1) / BN);

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(saddr(&full[s]), 1);
      mbar_init(saddr(&empty[s]), 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(saddr(&tfull[b]), 1);
      mbar_init(saddr(&tempty[b]), 4);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    tmem_alloc(saddr(tslot), TMEM_COLS);
    tmem_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tbase = *tslot;

  if (warp == 0 && lane == 0) {
    // TMA producer: k-blocks of every tile of this CTA, one ring
    int it = 0;
    bool ok = true;
    for (int t = blockIdx.x; t < tiles && ok; t += gridDim.x) {
      const int m0 = (t % tiles_m) * BM, n0 = (t / tiles_m) * BN;
      for (int kb = 0; kb < kblocks; ++kb, ++it) {
        const int s = it % STAGES;
        if (it >= STAGES && !mbar_wait(saddr(&empty[s]), ((it / STAGES) & 1) ^ 1, err)) { ok = false; break; }
        const uint32_t a_dst = saddr(smem + s * STAGE_BYTES);
        const uint32_t b_dst = a_dst + A_BYTES;
        mbar_expect_tx(saddr(&full[s]), STAGE_BYTES);
        tma_load_2d(a_dst, &tmA, kb * BK, m0, saddr(&full[s]));
        tma_load_2d(b_dst, &tmB, kb * BK, n0, saddr(&full[s]));
      }
    }
  } else if (warp == 1 && lane == 0) {
    // MMA issuer
    constexpr uint32_t idesc = idesc_f16<BN>(FMT);
    int it = 0, i = 0;
    bool ok = true;
    for (int t = blockIdx.x; t < tiles && ok; t += gridDim.x, ++i) {
      const int b = i & 1;
      // accumulator b is free once the epilogue drained its previous tile
      if (i >= 2 && !mbar_wait(saddr(&tempty[b]), ((i >> 1) & 1) ^ 1, err)) break;
      tc_fence_after();
      const uint32_t acc = tbase + (uint32_t)(b * BN);
      for (int kb = 0; kb < kblocks; ++kb, ++it) {
        const int s = it % STAGES;
        if (!mbar_wait(saddr(&full[s]), (it / STAGES) & 1, err)) { ok = false; break; }
        tc_fence_after();
        const uint32_t a_base = saddr(smem + s * STAGE_BYTES);
        const uint32_t b_base = a_base + A_BYTES;
#pragma unroll
        for (int k = 0; k < BK / UMMA_K; ++k) {
          const uint64_t ad = sdesc_k128(a_base + k * UMMA_K * 2);
          const uint64_t bd = sdesc_k128(b_base + k * UMMA_K * 2);
          tc_mma(acc, ad, bd, idesc, (kb > 0 || k > 0) ? 1u : 0u);
        }
        tc_commit(saddr(&empty[s]));  // stage s is free once these MMAs have read it
      }
      tc_commit(saddr(&tfull[b]));  // accumulator b complete (or abandoned)
    }
  } else if (warp >= 2) {
    // epilogue: TMEM lanes [32*(warp%4), +32) are this warp's rows
    const int q = warp & 3;
    int i = 0;
    for (int t = blockIdx.x; t < tiles; t += gridDim.x, ++i) {
      const int b = i & 1;
      if (!mbar_wait(saddr(&tfull[b]), (i >> 1) & 1, err)) break;
      tc_fence_after();
      const int m0 = (t % tiles_m) * BM, n0 = (t / tiles_m) * BN;
      const int row = m0 + q * 32 + lane;
#pragma unroll 1
      for (int c0 = 0; c0 < BN; c0 += 32) {
        // the 32 C values of this row first (independent loads in flight),
        // then the accumulator columns, then C - acc * 2^-s
        float cv[32];
        const float* crow = C + (int64_t)row + (int64_t)(n0 + c0) * ldc;
#pragma unroll
        for (int j = 0; j < 32; ++j)
          cv[j] = (row < M && n0 + c0 + j < N) ? crow[(int64_t)j * ldc] : 0.f;
        uint32_t v[32];
        tmem_ld_32cols(tbase + ((uint32_t)(q * 32) << 16) + (uint32_t)(b * BN + c0), v);
        if (row < M) {
          float* cw = C + (int64_t)row + (int64_t)(n0 + c0) * ldc;
#pragma unroll
          for (int j = 0; j < 32; ++j) {
            const int col = n0 + c0 + j;
            if (col < N) {
              float a = __uint_as_float(v[j]);
              if (inv_scale) a *= inv_scale[col];
              cw[(int64_t)j * ldc] = cv[j] - a;
            }
          }
        }
      }
      // this warp's reads of accumulator b are complete (tcgen05.wait::ld)
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(saddr(&tempty[b]));
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    tmem_dealloc(tbase, TMEM_COLS);
  }
}

// Four FP32 values rounded to 16 bits, packed into 8 bytes (element 0 lowest).
template <typename H>
__device__ __forceinline__ uint2 pack4(float a, float b, float c, float d) {
  uint32_t lo, hi;
  if constexpr (std::is_same<H, __nv_bfloat16>::value) {
    const __nv_bfloat162 x = __floats2bfloat162_rn(a, b), y = __floats2bfloat162_rn(c, d);
    lo = *reinterpret_cast<const uint32_t*>(&x);
    hi = *reinterpret_cast<const uint32_t*>(&y);
  } else {
    const __half2 x = __floats2half2_rn(a, b), y = __floats2half2_rn(c, d);
    lo = *reinterpret_cast<const uint32_t*>(&x);
    hi = *reinterpret_cast<const uint32_t*>(&y);
  }
  return make_uint2(lo, hi);
}

// A (M x K, column-major, lda) -> Ah (M rows of K, row-major, ldh, ldh a
// multiple of 8): 64 x 64 tiles through shared memory; a warp reads 64
// consecutive rows of a column and each thread writes 4 consecutive k of a
// row as one 8-byte store.
template <typename H>
__global__ void __launch_bounds__(256)
conv_a_kernel(int M, int K, const float* __restrict__ A, int64_t lda, H* __restrict__ Ah, int64_t ldh) {
  __shared__ float t[64][65];  // t[k][m]
  const int k0 = blockIdx.x * 64, m0 = blockIdx.y * 64;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int kk = warp; kk < 64; kk += 8) {
    const int k = k0 + kk, m = m0 + 2 * lane;
    float v0 = 0.f, v1 = 0.f;
    if (k < K) {
      const float* src = A + (int64_t)k * lda;
      if (m < M) v0 = src[m];
      if (m + 1 < M) v1 = src[m + 1];
    }
    t[kk][2 * lane] = v0;
    t[kk][2 * lane + 1] = v1;
  }
  __syncthreads();
  for (int idx = threadIdx.x; idx < 64 * 16; idx += 256) {
    const int mm = idx >> 4, q = idx & 15;  // row of the tile, pack of 4 k
    const int m = m0 + mm, k = k0 + 4 * q;
    if (m < M && k < ldh) {  // k < ldh implies k + 4 <= ldh (both multiples of 4)
      float v[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) v[i] = (k + i < K) ? t[4 * q + i][mm] : 0.f;
      *reinterpret_cast<uint2*>(Ah + (int64_t)m * ldh + k) = pack4<H>(v[0], v[1], v[2], v[3]);
    }
  }
}

// B (K x N, column-major, ldb) -> Bh (N rows of K, ldh a multiple of 8), row n
// scaled by scale[n]: a column of B is a row of Bh, so each thread converts
// 4 consecutive k with one 8-byte store; 4 columns per CTA.
template <typename H>
__global__ void __launch_bounds__(256)
conv_b_kernel(int K, int N, const float* __restrict__ B, int64_t ldb, H* __restrict__ Bh, int64_t ldh,
              const float* __restrict__ scale) {
  const int n = blockIdx.x * 4 + (threadIdx.x >> 6);
  if (n >= N) return;
  const float s = scale ? scale[n] : 1.f;
  const float* col = B + (int64_t)n * ldb;
  for (int64_t k = 4 * (threadIdx.x & 63); k < ldh; k += 256) {
    float v[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) v[i] = (k + i < K) ? col[k + i] * s : 0.f;
    *reinterpret_cast<uint2*>(Bh + (int64_t)n * ldh + k) = pack4<H>(v[0], v[1], v[2], v[3]);
  }
}

// Per-column power-of-two scale for FP16: max |B[:,n]| -> [2^14, 2^15).
__global__ void col_scale_kernel(int K, int N, const float* __restrict__ B, int64_t ldb,
                                 float* __restrict__ scale, float* __restrict__ inv_scale) {
  __shared__ float red[8];
  const int n = blockIdx.x;
  if (n >= N) return;
  float mx = 0.f;
  for (int k = threadIdx.x; k < K; k += blockDim.x) mx = fmaxf(mx, fabsf(B[(int64_t)k + (int64_t)n * ldb]));
  for (int off = 16; off; off >>= 1) mx = fmaxf(mx, __shfl_down_sync(0xffffffffu, mx, off));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = mx;
  __syncthreads();
  if (threadIdx.x == 0) {
    float m = 0.f;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) m = fmaxf(m, red[w]);
    int e = 0;
    if (m > 0.f && isfinite(m)) e = ilogbf(m) - 14;  // m * 2^-e in [2^14, 2^15)
    e = max(-120, min(120, e));
    scale[n] = ldexpf(1.f, -e);
    inv_scale[n] = ldexpf(1.f, e);
  }
}

// ---------------------------------------------------------------------------
// host side

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static std::once_flag once;
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  });
  return fn;
}

// 2D K-major map: rows of `inner` 16-bit elements, `outer` rows, pitch in
// bytes; boxes of BK x box_rows.
bool make_map(CUtensorMap* m, const void* base, uint64_t inner, uint64_t outer, uint64_t pitch_bytes,
              bool bf16, uint32_t box_rows) {
  auto fn = encode_fn();
  if (!fn) return false;
  if ((reinterpret_cast<uintptr_t>(base) & 15) || (pitch_bytes & 15)) return false;
  cuuint64_t dims[2] = {inner, outer};
  cuuint64_t strides[1] = {pitch_bytes};
  cuuint32_t box[2] = {(cuuint32_t)BK, box_rows};
  cuuint32_t es[2] = {1, 1};
  CUresult r = fn(m, bf16 ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2,
                  const_cast<void*>(base), dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
                  CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

}  // namespace tc

size_t tc_work_bytes(int64_t M, int64_t N, int64_t K) {
  const int64_t Kp = ((K + 7) / 8) * 8;
  return (size_t)(M * Kp + N * Kp) * 2 + 2 * (size_t)N * sizeof(float) + 1024;
}

void tc_configure(int /*device*/) {
  cudaFuncSetAttribute(tc::tc_gemm_kernel<0, 128>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)tc::Tile<128>::SMEM_BYTES);
  cudaFuncSetAttribute(tc::tc_gemm_kernel<1, 128>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)tc::Tile<128>::SMEM_BYTES);
  cudaFuncSetAttribute(tc::tc_gemm_kernel<0, 256>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)tc::Tile<256>::SMEM_BYTES);
  cudaFuncSetAttribute(tc::tc_gemm_kernel<1, 256>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)tc::Tile<256>::SMEM_BYTES);
}

// C (M x N, FP32, ldc) -= round16(A) (M x K, FP32 col-major, lda) * round16(B) (K x N, ldb).
// mode: 1 = BF16 operands, 2 = FP16 operands with per-column power-of-two scaling.
// work: tc_work_bytes(M, N, K) bytes of device scratch (256-byte aligned).
cudaError_t tc_gemm_sub(int mode, int64_t M, int64_t N, int64_t K, const float* A, int64_t lda,
                        const float* B, int64_t ldb, float* C, int64_t ldc, void* work, int* err,
                        cudaStream_t s) {
  if (M <= 0 || N <= 0 || K <= 0) return cudaSuccess;
  if (M > INT32_MAX || N > INT32_MAX || K > INT32_MAX) return cudaErrorInvalidValue;
  const bool bf16 = mode == 1;
  const int64_t Kp = ((K + 7) / 8) * 8;
  unsigned char* w = reinterpret_cast<unsigned char*>(work);
  void* Ah = w;
  void* Bh = w + (((size_t)M * Kp * 2 + 255) & ~size_t(255));
  float* scale = reinterpret_cast<float*>(reinterpret_cast<unsigned char*>(Bh) +
                                          (((size_t)N * Kp * 2 + 255) & ~size_t(255)));
  float* inv_scale = scale + N;
  {
    LaunchScope ls(K_GEMM, 0.0, (double)(M * K + K * N) * 6.0, s);
    dim3 ga((unsigned)((Kp + 63) / 64), (unsigned)((M + 63) / 64));
    if (bf16)
      tc::conv_a_kernel<__nv_bfloat16><<<ga, 256, 0, s>>>((int)M, (int)K, A, lda,
                                                          reinterpret_cast<__nv_bfloat16*>(Ah), Kp);
    else
      tc::conv_a_kernel<__half><<<ga, 256, 0, s>>>((int)M, (int)K, A, lda, reinterpret_cast<__half*>(Ah), Kp);
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  {
    LaunchScope ls(K_GEMM, 0.0, (double)(K * N) * 6.0, s);
    if (bf16) {
      tc::conv_b_kernel<__nv_bfloat16><<<(unsigned)((N + 3) / 4), 256, 0, s>>>(
          (int)K, (int)N, B, ldb, reinterpret_cast<__nv_bfloat16*>(Bh), Kp, nullptr);
    } else {
      tc::col_scale_kernel<<<(unsigned)N, 256, 0, s>>>((int)K, (int)N, B, ldb, scale, inv_scale);
      tc::conv_b_kernel<__half><<<(unsigned)((N + 3) / 4), 256, 0, s>>>((int)K, (int)N, B, ldb,
                                                             reinterpret_cast<__half*>(Bh), Kp, scale);
    }
  }
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  // 128 x 256 tiles when they still cover the SMs, else 128 x 128
  int device = 0;
  cudaGetDevice(&device);
  const int sms = device_info(device).num_sms;
  const int64_t tiles_m = (M + tc::BM - 1) / tc::BM;
  const bool wide = tiles_m * ((N + 255) / 256) >= sms;
  const int bn = wide ? 256 : 128;
  CUtensorMap ta, tb;
  if (!tc::make_map(&ta, Ah, (uint64_t)K, (uint64_t)M, (uint64_t)Kp * 2, bf16, tc::BM) ||
      !tc::make_map(&tb, Bh, (uint64_t)K, (uint64_t)N, (uint64_t)Kp * 2, bf16, (uint32_t)bn))
    return cudaErrorInvalidValue;
  // persistent: at most one CTA per SM, each walking its share of the tiles
  const int64_t tiles = tiles_m * ((N + bn - 1) / bn);
  if (tiles > INT32_MAX) return cudaErrorInvalidValue;
  dim3 grid((unsigned)std::min<int64_t>(tiles, sms));
  LaunchScope ls(K_GEMM, 2.0 * M * N * K, (2.0 * M * N + (double)(M + N) * K / 2.0) * 4.0, s);
  const float* isc = bf16 ? nullptr : inv_scale;
  if (wide) {
    if (bf16)
      tc::tc_gemm_kernel<1, 256><<<grid, tc::THREADS, tc::Tile<256>::SMEM_BYTES, s>>>(
          ta, tb, C, ldc, (int)M, (int)N, (int)K, isc, err);
    else
      tc::tc_gemm_kernel<0, 256><<<grid, tc::THREADS, tc::Tile<256>::SMEM_BYTES, s>>>(
          ta, tb, C, ldc, (int)M, (int)N, (int)K, isc, err);
  } else {
    if (bf16)
      tc::tc_gemm_kernel<1, 128><<<grid, tc::THREADS, tc::Tile<128>::SMEM_BYTES, s>>>(
          ta, tb, C, ldc, (int)M, (int)N, (int)K, isc, err);
    else
      tc::tc_gemm_kernel<0, 128><<<grid, tc::THREADS, tc::Tile<128>::SMEM_BYTES, s>>>(
          ta, tb, C, ldc, (int)M, (int)N, (int)K, isc, err);
  }
  return cudaGetLastError();
}

}  // namespace gblu
