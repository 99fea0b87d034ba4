// getrf on the device: recursive right-looking LU with partial pivoting.
//
// Structure (the LAPACK getrf structure the reference states in
// src/blocked_lufact.jl:658-679, arranged recursively as in
// RFLUFactorization's RecursiveFactorization, ext/LinearSolveRecursiveFactorizationExt.jl:15-42):
//
//   rec(c0, w):  if w <= panel width:  panel_kernel   (getf2 on the leaf,
//                                       blocked_lufact.jl:93-122)
//                                       laswp_kernel   (interchanges on every
//                                       other column, :126-141)
//                else  rec(c0, w1)
//                      trsm  U12 := L11 \ A12       (:146-178)
//                      gemm  A22 -= L21 * U12       (:186-656)
//                      rec(c0 + w1, w - w1)
//
// Floating point: each element A[i,j] receives fma(-l_ik, u_kj, a_ij) for
// k ascending, exactly as the reference's muladd loops, and the multipliers
// are a_ik * (1 / u_kk).  Every kernel below keeps that per-element order
// (C is loaded first, then updated k = 0, 1, ...), so the factors and ipiv
// are bit-identical to the reference's blocked LU for any blocking.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <type_traits>
#include <vector>

#include <cooperative_groups.h>

#include "device_util.cuh"
#include "waits.cuh"
#include "gblu_internal.h"
#include "profile.h"

namespace gblu {

constexpr int kPanelThreads = 256;
constexpr int kPanelMaxW = 32;
constexpr int kPanelRowsTarget = 64;

// ---------------------------------------------------------------------------
// Pivot-candidate ordering: larger |a| wins; ties go to the smaller row;
// row -1 means "no candidate" (|a| == 0 or NaN everywhere, blocked_lufact.jl:38-54).
template <typename T>
__device__ __forceinline__ bool cand_better(T v, int64_t g, T bv, int64_t bg) {
  if (g < 0) return false;
  if (bg < 0) return true;
  return (v > bv) || (v == bv && g < bg);
}


// ---------------------------------------------------------------------------
// Cooperative panel kernel: getf2 on rows [c0, m) x columns [c0, c0+w).
// Each CTA holds a contiguous slice of R rows of the panel in shared memory;
// one grid barrier per column exchanges the pivot candidates.
template <typename T>
__global__ void __launch_bounds__(kPanelThreads)
panel_kernel(T* __restrict__ A, int64_t lda, int64_t m, int64_t c0, int w,
             int64_t* __restrict__ ipiv, int64_t* __restrict__ info_out,
             DevScratch* __restrict__ scr, PanelSlots<T> slots, int R) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* tile = reinterpret_cast<T*>(smem_raw);  // column j at tile + j*R
  __shared__ T pivrow[kPanelMaxW];
  __shared__ T diagrow[kPanelMaxW];
  using K = typename PivKey<T>::K;  // pivot candidates compared as integer keys of |a|
  __shared__ K red_v[kPanelThreads / 32];
  __shared__ int64_t red_g[kPanelThreads / 32];
  __shared__ int red_c[kPanelThreads / 32];
  K* cand_key = reinterpret_cast<K*>(slots.cand_val);
  __shared__ int64_t s_best_g;
  __shared__ int s_best_c;

  const int G = gridDim.x;
  const int cta = blockIdx.x;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int64_t base = c0 + (int64_t)cta * R;
  const int nloc = (int)max((int64_t)0, min((int64_t)R, m - base));

  for (int j = 0; j < w; ++j)
    for (int i = tid; i < R; i += blockDim.x)
      tile[(size_t)j * R + i] = (i < nloc) ? A[(base + i) + (c0 + j) * lda] : T(0);
  int64_t info_local = 0;
  __syncthreads();

  for (int k = 0; k < w; ++k) {
    const int64_t d = c0 + k;
    const int buf = k & 1;
    const T* colk = tile + (size_t)k * R;

    // 1. local candidate: first row of max |a| among rows >= d (NaN ignored)
    K bv = 0;
    int64_t bg = -1;
    for (int i = tid; i < nloc; i += blockDim.x) {
      int64_t g = base + i;
      K v = PivKey<T>::of(colk[i]);
      if (g >= d && v > bv) { bv = v; bg = g; }
    }
    for (int off = 16; off; off >>= 1) {
      K ov = __shfl_down_sync(0xffffffffu, bv, off);
      int64_t og = __shfl_down_sync(0xffffffffu, bg, off);
      if (cand_better(ov, og, bv, bg)) { bv = ov; bg = og; }
    }
    if (lane == 0) { red_v[warp] = bv; red_g[warp] = bg; }
    __syncthreads();
    if (warp == 0) {
      bv = lane < (kPanelThreads / 32) ? red_v[lane] : K(0);
      bg = lane < (kPanelThreads / 32) ? red_g[lane] : -1;
      for (int off = 16; off; off >>= 1) {
        K ov = __shfl_down_sync(0xffffffffu, bv, off);
        int64_t og = __shfl_down_sync(0xffffffffu, bg, off);
        if (cand_better(ov, og, bv, bg)) { bv = ov; bg = og; }
      }
      if (lane == 0) {
        stcg(&cand_key[buf * G + cta], bv);
        stcg(&slots.cand_row[buf * G + cta], bg);
        s_best_g = bg;
      }
    }
    __syncthreads();
    // 2. publish the candidate's panel row and, if owned here, the diagonal row
    if (tid < w) {
      if (s_best_g >= 0)
        stcg(&slots.cand_rowvals[((size_t)buf * G + cta) * kPanelMaxW + tid],
             tile[(size_t)tid * R + (s_best_g - base)]);
      if (d >= base && d < base + nloc)
        stcg(&slots.diag_rowvals[buf * kPanelMaxW + tid], tile[(size_t)tid * R + (d - base)]);
    }
    if (!grid_barrier(scr, (unsigned)(k + 1) * (unsigned)G)) return;

    // 3. global winner over the G candidates (same reduction on every CTA)
    bv = 0;
    bg = -1;
    int bc = -1;
    for (int c = tid; c < G; c += blockDim.x) {
      K v = ldcg(&cand_key[buf * G + c]);
      int64_t g = ldcg(&slots.cand_row[buf * G + c]);
      if (cand_better(v, g, bv, bg)) { bv = v; bg = g; bc = c; }
    }
    for (int off = 16; off; off >>= 1) {
      K ov = __shfl_down_sync(0xffffffffu, bv, off);
      int64_t og = __shfl_down_sync(0xffffffffu, bg, off);
      int oc = __shfl_down_sync(0xffffffffu, bc, off);
      if (cand_better(ov, og, bv, bg)) { bv = ov; bg = og; bc = oc; }
    }
    if (lane == 0) { red_v[warp] = bv; red_g[warp] = bg; red_c[warp] = bc; }
    __syncthreads();
    if (warp == 0) {
      bv = lane < (kPanelThreads / 32) ? red_v[lane] : K(0);
      bg = lane < (kPanelThreads / 32) ? red_g[lane] : -1;
      bc = lane < (kPanelThreads / 32) ? red_c[lane] : -1;
      for (int off = 16; off; off >>= 1) {
        K ov = __shfl_down_sync(0xffffffffu, bv, off);
        int64_t og = __shfl_down_sync(0xffffffffu, bg, off);
        int oc = __shfl_down_sync(0xffffffffu, bc, off);
        if (cand_better(ov, og, bv, bg)) { bv = ov; bg = og; bc = oc; }
      }
      if (lane == 0) { s_best_g = bg; s_best_c = bc; }
    }
    __syncthreads();
    const int64_t p = s_best_g < 0 ? d : s_best_g;  // kp = k when amax == 0
    const int pc = s_best_c;
    if (tid < w) {
      T dv = ldcg(&slots.diag_rowvals[buf * kPanelMaxW + tid]);
      diagrow[tid] = dv;
      pivrow[tid] = (p == d) ? dv : ldcg(&slots.cand_rowvals[((size_t)buf * G + pc) * kPanelMaxW + tid]);
    }
    if (cta == 0 && tid == 0) ipiv[d] = p + 1;
    __syncthreads();
    const T piv = pivrow[k];

    // 4. interchange (only when the pivot is nonzero), scale, rank-1 update
    if (piv != T(0)) {
      if (p != d) {
        if (tid < w) {
          if (d >= base && d < base + nloc) tile[(size_t)tid * R + (d - base)] = pivrow[tid];
          if (p >= base && p < base + nloc) tile[(size_t)tid * R + (p - base)] = diagrow[tid];
        }
        __syncthreads();
      }
      const T inv = T(1) / piv;
      for (int i = tid; i < nloc; i += blockDim.x)
        if (base + i > d) tile[(size_t)k * R + i] *= inv;
    } else if (info_local == 0) {
      info_local = d + 1;
    }
    __syncthreads();
    // rank-1 update of this CTA's rows below the diagonal: one row per thread,
    // columns k+1..w-1 in order (per element: one fma, k ascending)
    for (int i = tid; i < nloc; i += blockDim.x) {
      if (base + i <= d) continue;
      const T l = tile[(size_t)k * R + i];
      for (int j = k + 1; j < w; ++j)
        tile[(size_t)j * R + i] = fma(-l, pivrow[j], tile[(size_t)j * R + i]);
    }
    __syncthreads();
  }

  for (int j = 0; j < w; ++j)
    for (int i = tid; i < nloc; i += blockDim.x) A[(base + i) + (c0 + j) * lda] = tile[(size_t)j * R + i];
  if (cta == 0 && tid == 0 && info_local != 0 && *info_out == 0) *info_out = info_local;
}

// ---------------------------------------------------------------------------
// Cluster panel kernel: the same getf2 on rows [c0, m) x columns [c0, c0+w),
// for panels that fit in the shared memory of one thread-block cluster (up to
// 16 CTAs).  Pivot candidates, the candidate rows and the diagonal row live in
// each CTA's shared memory; after the hardware cluster barrier every CTA reads
// the others' slots through distributed shared memory, so a column costs one
// cluster barrier and one round of DSMEM loads instead of a grid barrier and
// two L2 round trips.  The arithmetic per element is the grid kernel's.
template <typename T>
__global__ void __launch_bounds__(kPanelThreads)
panel_cluster_kernel(T* __restrict__ A, int64_t lda, int64_t m, int64_t c0, int w,
                     int64_t* __restrict__ ipiv, int64_t* __restrict__ info_out, int R) {
  namespace cg = cooperative_groups;
  cg::cluster_group cluster = cg::this_cluster();
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* tile = reinterpret_cast<T*>(smem_raw);  // column j at tile + j*R
  __shared__ typename PivKey<T>::K s_cval[2];
  __shared__ int64_t s_crow[2];
  __shared__ T s_crowv[2][kPanelMaxW];
  __shared__ T s_diagv[2][kPanelMaxW];
  __shared__ T pivrow[kPanelMaxW];
  __shared__ T diagrow[kPanelMaxW];
  using K = typename PivKey<T>::K;  // pivot candidates compared as integer keys of |a|
  __shared__ K red_v[kPanelThreads / 32];
  __shared__ int64_t red_g[kPanelThreads / 32];
  __shared__ int64_t s_best_g;
  __shared__ int s_best_c;

  const int G = (int)cluster.num_blocks();
  const int cta = (int)cluster.block_rank();
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int64_t base = c0 + (int64_t)cta * R;
  const int nloc = (int)max((int64_t)0, min((int64_t)R, m - base));

  for (int j = 0; j < w; ++j)
    for (int i = tid; i < R; i += blockDim.x)
      tile[(size_t)j * R + i] = (i < nloc) ? A[(base + i) + (c0 + j) * lda] : T(0);
  int64_t info_local = 0;
  __syncthreads();

  for (int k = 0; k < w; ++k) {
    const int64_t d = c0 + k;
    const int buf = k & 1;
    const T* colk = tile + (size_t)k * R;
    K bv = 0;
    int64_t bg = -1;
    for (int i = tid; i < nloc; i += blockDim.x) {
      int64_t g = base + i;
      K v = PivKey<T>::of(colk[i]);
      if (g >= d && v > bv) { bv = v; bg = g; }
    }
    for (int off = 16; off; off >>= 1) {
      K ov = __shfl_down_sync(0xffffffffu, bv, off);
      int64_t og = __shfl_down_sync(0xffffffffu, bg, off);
      if (cand_better(ov, og, bv, bg)) { bv = ov; bg = og; }
    }
    if (lane == 0) { red_v[warp] = bv; red_g[warp] = bg; }
    __syncthreads();
    if (warp == 0) {
      bv = lane < (kPanelThreads / 32) ? red_v[lane] : K(0);
      bg = lane < (kPanelThreads / 32) ? red_g[lane] : -1;
      for (int off = 16; off; off >>= 1) {
        K ov = __shfl_down_sync(0xffffffffu, bv, off);
        int64_t og = __shfl_down_sync(0xffffffffu, bg, off);
        if (cand_better(ov, og, bv, bg)) { bv = ov; bg = og; }
      }
      if (lane == 0) { s_cval[buf] = bv; s_crow[buf] = bg; s_best_g = bg; }
    }
    __syncthreads();
    if (tid < w) {
      if (s_best_g >= 0) s_crowv[buf][tid] = tile[(size_t)tid * R + (s_best_g - base)];
      if (d >= base && d < base + nloc) s_diagv[buf][tid] = tile[(size_t)tid * R + (d - base)];
    }
    cluster.sync();  // publishes the slots of step k (release/acquire across the cluster)

    // winner over the G candidates, read through distributed shared memory
    bv = 0;
    bg = -1;
    int bc = -1;
    if (tid < G) {
      const K* rv = cluster.map_shared_rank(&s_cval[buf], tid);
      const int64_t* rr = cluster.map_shared_rank(&s_crow[buf], tid);
      bv = *rv;
      bg = *rr;
      bc = bg >= 0 ? tid : -1;
    }
    if (warp == 0) {
      for (int off = 16; off; off >>= 1) {
        K ov = __shfl_down_sync(0xffffffffu, bv, off);
        int64_t og = __shfl_down_sync(0xffffffffu, bg, off);
        int oc = __shfl_down_sync(0xffffffffu, bc, off);
        if (cand_better(ov, og, bv, bg)) { bv = ov; bg = og; bc = oc; }
      }
      if (lane == 0) { s_best_g = bg; s_best_c = bc; }
    }
    __syncthreads();
    const int64_t p = s_best_g < 0 ? d : s_best_g;
    const int pc = s_best_c;
    const int downer = (int)((d - c0) / R);
    if (tid < w) {
      const T dv = *cluster.map_shared_rank(&s_diagv[buf][tid], downer);
      diagrow[tid] = dv;
      pivrow[tid] = (p == d) ? dv : *cluster.map_shared_rank(&s_crowv[buf][tid], pc);
    }
    if (cta == 0 && tid == 0) ipiv[d] = p + 1;
    __syncthreads();
    const T piv = pivrow[k];
    if (piv != T(0)) {
      if (p != d) {
        if (tid < w) {
          if (d >= base && d < base + nloc) tile[(size_t)tid * R + (d - base)] = pivrow[tid];
          if (p >= base && p < base + nloc) tile[(size_t)tid * R + (p - base)] = diagrow[tid];
        }
        __syncthreads();
      }
      const T inv = T(1) / piv;
      for (int i = tid; i < nloc; i += blockDim.x)
        if (base + i > d) tile[(size_t)k * R + i] *= inv;
    } else if (info_local == 0) {
      info_local = d + 1;
    }
    __syncthreads();
    // rank-1 update of this CTA's rows below the diagonal: one row per thread,
    // columns k+1..w-1 in order (per element: one fma, k ascending)
    for (int i = tid; i < nloc; i += blockDim.x) {
      if (base + i <= d) continue;
      const T l = tile[(size_t)k * R + i];
      for (int j = k + 1; j < w; ++j)
        tile[(size_t)j * R + i] = fma(-l, pivrow[j], tile[(size_t)j * R + i]);
    }
    __syncthreads();
  }
  for (int j = 0; j < w; ++j)
    for (int i = tid; i < nloc; i += blockDim.x) A[(base + i) + (c0 + j) * lda] = tile[(size_t)j * R + i];
  if (cta == 0 && tid == 0 && info_local != 0 && *info_out == 0) *info_out = info_local;
  cluster.sync();  // no CTA leaves while another may still read its shared memory
}

template <typename T>
struct Vec16;  // 16-byte vector of T
template <>
struct Vec16<float> {
  using V = float4;
  static constexpr int N = 4;
  static __device__ __forceinline__ float get(const V& v, int e) { return e == 0 ? v.x : e == 1 ? v.y : e == 2 ? v.z : v.w; }
  static __device__ __forceinline__ V make(const float* x) { return make_float4(x[0], x[1], x[2], x[3]); }
};
template <>
struct Vec16<double> {
  using V = double2;
  static constexpr int N = 2;
  static __device__ __forceinline__ double get(const V& v, int e) { return e == 0 ? v.x : v.y; }
  static __device__ __forceinline__ V make(const double* x) { return make_double2(x[0], x[1]); }
};

template <typename T, int W>
__device__ __forceinline__ void row_store(T* dst, const T (&src)[W]) {
  using VT = Vec16<T>;
#pragma unroll
  for (int q = 0; q < W / VT::N; ++q) reinterpret_cast<typename VT::V*>(dst)[q] = VT::make(&src[q * VT::N]);
}

template <typename T, int W>
__device__ __forceinline__ void row_load(T (&dst)[W], const T* src) {
  using VT = Vec16<T>;
#pragma unroll
  for (int q = 0; q < W / VT::N; ++q) {
    const typename VT::V v = reinterpret_cast<const typename VT::V*>(src)[q];
#pragma unroll
    for (int e = 0; e < VT::N; ++e) dst[q * VT::N + e] = VT::get(v, e);
  }
}

// ---------------------------------------------------------------------------
// Register panel kernel: the same getf2 on rows [c0, m) x columns [c0, c0+w)
// with every panel row held in registers by one thread for the whole leaf
// (row base + tid + NT * r of CTA `cta`, r < RPT, the CTA holding R rows).
// The registers rotate by one slot per column, identically in every thread,
// so the current column is always slot 0 and the column loop is a plain loop
// with one small body; rows are exchanged in slot order (16-byte shared
// memory accesses, no index arithmetic).
//
// The CTAs exchange pivot candidates by pushing them: no cluster barrier per
// column.  After the interchange and scaling of column k, each thread
// updates only slot 1 (column k+1); each warp reduces its column-k+1
// candidate and leaves it, with the candidate row and the diagonal row in
// their partly updated form (slot 0 = the multiplier l, slot 1 updated,
// slots 2.. not yet), in shared memory; the pushing warp (the last warp)
// waits for them on a named barrier, reduces them to the CTA's candidate and
// writes candidate, row and (in the diagonal row's CTA) the diagonal row into
// every CTA's receive slots with st.async, each store counted by the
// receiver's mbarrier of that column.  The other warps run the rest of the
// update (slots 2..) meanwhile.  Warp 0 of every CTA waits on its own
// mbarrier (a bounded wait), picks the winner among the G received
// candidates, and finishes the update of the received pivot row and
// diagonal row itself with the same fma(-l, u, a) on the same operands the
// owners use, so they are bit-identical to the owners' registers; warp 1
// computes 1 / |candidate| of every received candidate from its key (the bit
// pattern of |a|) and hands the winner's to warp 0 through a named barrier.
// One CTA barrier hands the pivot row to every thread.
//
// Receive slots are double-buffered by column parity.  A CTA pushes column
// k+1 only after it received every CTA's column k, and each CTA pushes
// column k only after it finished reading its column k-1 slots, so a push
// never overwrites slots still being read.  Warps that hold no rows skip the
// arithmetic (a predicated-off FP64 instruction still occupies the FP64
// pipe).  The per-element arithmetic is panel_kernel's.
constexpr int kRegPanelThreads = 512;

// A CTA's pivot candidate as one 16-byte word: key, row (-1 = none), warp.
template <typename K>
__device__ __forceinline__ int4 cand_pack(K key, int row, int warp) {
  if constexpr (sizeof(K) == 4) return make_int4((int)key, row, warp, 0);
  else return make_int4((int)(unsigned)key, (int)(unsigned)(key >> 32), row, warp);
}
template <typename K>
__device__ __forceinline__ void cand_unpack(const int4& c, K& key, int& row, int& warp) {
  if constexpr (sizeof(K) == 4) { key = (K)(unsigned)c.x; row = c.y; warp = c.z; }
  else { key = ((K)(unsigned)c.y << 32) | (K)(unsigned)c.x; row = c.z; warp = c.w; }
}

// The value whose bit pattern is the key (|a| for a key of a)
template <typename T>
__device__ __forceinline__ T key_magnitude(typename PivKey<T>::K key) {
  if constexpr (sizeof(T) == 4) return __uint_as_float(key);
  else return __longlong_as_double((long long)key);
}

// x with the sign of s (bit operations only)
template <typename T>
__device__ __forceinline__ T with_sign_of(T x, T s) {
  if constexpr (sizeof(T) == 4)
    return __uint_as_float(__float_as_uint(x) ^ (__float_as_uint(s) & 0x80000000u));
  else
    return __longlong_as_double(__double_as_longlong(x) ^
                                (__double_as_longlong(s) & (long long)0x8000000000000000ull));
}

template <typename T, int RPT>
__global__ void __launch_bounds__(kRegPanelThreads, 1)
panel_reg_kernel(T* __restrict__ A, int64_t lda, int64_t m, int64_t c0, int w,
                 int64_t* __restrict__ ipiv, int64_t* __restrict__ info_out, int R,
                 DevScratch* __restrict__ scr) {
  namespace cg = cooperative_groups;
  using K = typename PivKey<T>::K;
  using VT = Vec16<T>;
  constexpr unsigned kAll = 0xffffffffu;
  cg::cluster_group cluster = cg::this_cluster();
  constexpr int NT = kRegPanelThreads, NW = NT / 32, W = kPanelMaxW;
  constexpr int RB = W * (int)sizeof(T) / 16;  // 16-byte chunks per row
  constexpr int kPusher = NW - 1;              // the warp that pushes the CTA's candidate
  // [b]: column k uses buffer k & 1
  __shared__ __align__(16) T s_crowv[2][NW][W];  // each warp's candidate row (published form)
  __shared__ __align__(16) T s_diagv[2][W];      // the diagonal row (owner CTA, published form)
  __shared__ __align__(16) T s_piv[2][W];        // the pivot row of column k, slot order of step k
  __shared__ __align__(16) T s_old[W];           // the old diagonal row, for the pivot row's owner
  __shared__ __align__(16) T r_row[2][16][W];    // received: CTA c's candidate row
  __shared__ __align__(16) T r_diag[2][W];       // received: the diagonal row
  __shared__ __align__(16) int4 r_cand[2][16];   // received: CTA c's candidate (cand_pack)
  __shared__ __align__(8) unsigned long long r_bar[2];  // counts the received bytes of a column
  __shared__ K s_cval[2][NW];
  __shared__ int s_crow[2][NW];
  __shared__ T s_rinv[16];                       // 1 / |candidate| of CTA c's candidate
  __shared__ int s_p;
  __shared__ T s_inv;

  const int G = (int)cluster.num_blocks();
  const int cta = (int)cluster.block_rank();
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int64_t base = c0 + (int64_t)cta * R;
  const int nloc = (int)max((int64_t)0, min((int64_t)R, m - base));
  const bool warp_rows = warp * 32 < nloc;  // this warp holds at least one row
  // bytes received per column: G candidates and rows, one diagonal row
  const uint32_t rx_bytes = (uint32_t)(G * 16 * (1 + RB) + 16 * RB);
  int* const err = &scr->error;
  bool bad = false;  // a wait gave up: stop waiting, finish without hanging

  T pr[RPT][W];  // slot j: column (k + j) mod 32 at step k
#pragma unroll
  for (int r = 0; r < RPT; ++r) {
    const int i = tid + NT * r;
#pragma unroll
    for (int j = 0; j < W; ++j) pr[r][j] = (i < nloc && j < w) ? A[(base + i) + (c0 + j) * lda] : T(0);
  }
  if (tid == 0) {
    pan_bar_init(pan_saddr(&r_bar[0]));
    pan_bar_init(pan_saddr(&r_bar[1]));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    pan_bar_arm(pan_saddr(&r_bar[0]), rx_bytes);  // column 0
    pan_bar_arm(pan_saddr(&r_bar[1]), rx_bytes);  // column 1
  }
  cluster.sync();  // every CTA's mbarriers exist before the first push
  int64_t info_local = 0;

  // Candidates of the column in slot S among rows >= dn into buffer pb: each
  // warp's first row of max |a| (NaN ignored) with its row, and the diagonal
  // row dn; the pushing warp reduces them to the CTA's candidate and writes
  // it into every CTA's receive slots.
  auto publish = [&](auto slot_c, int64_t dn, int pb) {
    constexpr int S = decltype(slot_c)::value;
    K bv = 0;
    int bg = -1;
#pragma unroll
    for (int r = 0; r < RPT; ++r) {
      const int i = tid + NT * r;
      const K v = PivKey<T>::of(pr[r][S]);
      if (i < nloc && base + i >= dn && v > bv) { bv = v; bg = (int)(base + i); }
    }
    {
      int src;
      warp_pivot_choice(bv, bg, src);
    }
    // the stores are issued by the owning warp only (a predicated-off store
    // still occupies the shared-memory pipe)
    if (bg >= 0) {
      const int lw = (int)(bg - base);  // the winner's local row
#pragma unroll
      for (int r = 0; r < RPT; ++r)
        if (lw >= NT * r && lw < NT * (r + 1)) {
          if (tid + NT * r == lw) row_store<T, W>(s_crowv[pb][warp], pr[r]);
        }
    }
    const int64_t ldn = dn - base;
    const bool own_diag = ldn >= 0 && ldn < nloc;
    if (own_diag && (((int)ldn & (NT - 1)) >> 5) == warp) {
#pragma unroll
      for (int r = 0; r < RPT; ++r)
        if (ldn >= NT * r && ldn < NT * (r + 1)) {
          if (tid + NT * r == ldn) row_store<T, W>(s_diagv[pb], pr[r]);
        }
    }
    if (lane == 0) { s_cval[pb][warp] = bv; s_crow[pb][warp] = bg; }
    if (warp != kPusher) {
      named_bar_arrive(2, NT);
      return;
    }
    named_bar_sync(2, NT);  // every warp's candidate and rows are in shared memory
    K v = lane < NW ? s_cval[pb][lane] : K(0);
    int g = lane < NW ? s_crow[pb][lane] : -1;
    int wsrc;
    warp_pivot_choice(v, g, wsrc);
    // lane c writes CTA c's receive slots: the candidate, the candidate row
    // and, from the diagonal row's CTA, the diagonal row (offsets within
    // one mapped array stay in that CTA's shared memory window)
    if (lane < G) {
      const int4 cand = cand_pack<K>(v, g, wsrc);
      const int4* rsrc = reinterpret_cast<const int4*>(s_crowv[pb][wsrc < 0 ? 0 : wsrc]);
      const uint32_t rbar = pan_mapa(pan_saddr(&r_bar[pb]), lane);
      const uint32_t rc = pan_mapa(pan_saddr(&r_cand[pb][cta]), lane);
      const uint32_t rr = pan_mapa(pan_saddr(&r_row[pb][cta][0]), lane);
      pan_st_async(rc, cand, rbar);
#pragma unroll
      for (int q = 0; q < RB; ++q) pan_st_async(rr + 16u * q, rsrc[q], rbar);
      if (own_diag) {
        const int4* dsrc = reinterpret_cast<const int4*>(s_diagv[pb]);
        const uint32_t rd = pan_mapa(pan_saddr(&r_diag[pb][0]), lane);
#pragma unroll
        for (int q = 0; q < RB; ++q) pan_st_async(rd + 16u * q, dsrc[q], rbar);
      }
    }
  };

  publish(std::integral_constant<int, 0>{}, c0, 0);  // column 0: the rows as loaded

  for (int k = 0; k < w; ++k) {
    const int64_t d = c0 + k;
    const int buf = k & 1;
    // 1. warp 0: the winner over the CTAs of the cluster, the pivot row and,
    //    for the pivot row's CTA, the old diagonal row
    if (warp == 0) {
      if (!bad && !pan_bar_wait(pan_saddr(&r_bar[buf]), (uint32_t)(k >> 1) & 1u, err)) bad = true;
      if (lane == 0 && k + 2 < w) pan_bar_arm(pan_saddr(&r_bar[buf]), rx_bytes);  // column k + 2
      K v = 0;
      int g = -1, ew = 0;
      if (lane < G) cand_unpack<K>(r_cand[buf][lane], v, g, ew);
      int ec;  // the winning CTA
      warp_pivot_choice(v, g, ec);
      const int64_t p = g < 0 ? d : (int64_t)g;  // kp = k when amax == 0
      // received rows are in the slot order of step k-1: lane j takes slot
      // j + 1 and finishes its step-(k-1) update (slots 2 .. w-k of step k-1)
      const int js = k > 0 ? ((lane + 1) & (W - 1)) : lane;
      T dv = r_diag[buf][js];
      T pv = p != d ? r_row[buf][ec < 0 ? 0 : ec][js] : dv;
      if (k > 0) {
        const T u = s_piv[buf ^ 1][js];
        const T ld = __shfl_sync(kAll, dv, W - 1);  // slot 0 of step k-1: the multiplier
        const T lp = __shfl_sync(kAll, pv, W - 1);
        if (lane >= 1 && lane < w - k) {
          dv = fma(-ld, u, dv);
          pv = fma(-lp, u, pv);
        }
      }
      // 1 / |pivot| from warp 1
      named_bar_sync(1, 64);
      const T inv_mag = s_rinv[ec < 0 ? 0 : ec];
      s_piv[buf][lane] = pv;
      if (p != d && p >= base && p < base + nloc) s_old[lane] = dv;
      if (lane == 0) {
        s_p = (int)p;
        // no candidate: the pivot is the diagonal entry, zero or NaN
        s_inv = g >= 0 ? with_sign_of(inv_mag, pv) : (PivKey<T>::nonzero(pv) ? T(1) / pv : T(0));
      }
    } else if (warp == 1) {
      // 1 / |candidate| of every received candidate (its key is the bit
      // pattern of |a|), beside warp 0's reduction: the division is a long
      // dependent sequence
      if (!bad && !pan_bar_wait(pan_saddr(&r_bar[buf]), (uint32_t)(k >> 1) & 1u, err)) bad = true;
      K v = 0;
      int g = -1, ew = 0;
      if (lane < G) cand_unpack<K>(r_cand[buf][lane], v, g, ew);
      const T rinv = T(1) / key_magnitude<T>(g >= 0 ? v : K(1));
      if (lane < G) s_rinv[lane] = rinv;
      named_bar_arrive(1, 64);
    }
    __syncthreads();
    const int64_t p = s_p;
    const T piv = s_piv[buf][0];
    const bool nz = PivKey<T>::nonzero(piv);
    if (cta == 0 && tid == 0) {
      ipiv[d] = p + 1;
      if (!nz && info_local == 0) info_local = d + 1;
    }
    // 2. interchange (nonzero pivot only) and scale
    const bool swap = nz && p != d;
    const T inv = s_inv;  // 1 / piv, computed once by warp 0
    const int lim = w - k;  // slots 1..lim-1 hold columns k+1..w-1
    T l[RPT];
    bool upd[RPT];
    if (swap) {
      // only the warps holding row d or row p load
      const int64_t ld = d - base, lp = p - base;
      const bool own_d = ld >= 0 && ld < nloc && (((int)ld & (NT - 1)) >> 5) == warp;
      const bool own_p = lp >= 0 && lp < nloc && (((int)lp & (NT - 1)) >> 5) == warp;
      if (own_d || own_p) {
#pragma unroll
        for (int r = 0; r < RPT; ++r) {
          const int64_t gi = base + tid + NT * r;
          if (gi == d) row_load<T, W>(pr[r], s_piv[buf]);
          else if (gi == p) row_load<T, W>(pr[r], s_old);
        }
      }
    }
#pragma unroll
    for (int r = 0; r < RPT; ++r) {
      const int i = tid + NT * r;
      upd[r] = i < nloc && base + i > d;
      l[r] = pr[r][0];
    }
    if (warp_rows) {
#pragma unroll
      for (int r = 0; r < RPT; ++r) {
        if (upd[r] && nz) l[r] *= inv;
        if (upd[r]) pr[r][0] = l[r];
      }
    }
    if (k + 1 < w) {
      // 3. slot 1 first, publish the candidates of column k + 1, then the
      //    rest of the rank-1 update while the candidates travel
      if (warp_rows) {
        const T u1 = s_piv[buf][1];
#pragma unroll
        for (int r = 0; r < RPT; ++r)
          if (upd[r]) pr[r][1] = fma(-l[r], u1, pr[r][1]);
      }
      publish(std::integral_constant<int, 1>{}, d + 1, buf ^ 1);
      if (warp_rows) {
        if constexpr (sizeof(T) == 4) {
          // FP32: predicated FMAs over all slots (no branches)
#pragma unroll
          for (int q = 0; q < W / VT::N; ++q) {
            const typename VT::V pv = reinterpret_cast<const typename VT::V*>(s_piv[buf])[q];
#pragma unroll
            for (int e = 0; e < VT::N; ++e) {
              const int j = q * VT::N + e;
              if (j >= 2 && j < lim) {
                const T u = VT::get(pv, e);
#pragma unroll
                for (int r = 0; r < RPT; ++r)
                  if (upd[r]) pr[r][j] = fma(-l[r], u, pr[r][j]);
              }
            }
          }
        } else {
          // FP64: stop at the last live slot with a uniform branch, so the FP64
          // pipe only sees the FMAs that do work; the pivot row is read two
          // slots per 16-byte load
#pragma unroll
          for (int j = 2; j < W; j += 2) {
            if (j >= lim) break;
            const typename VT::V u2 = reinterpret_cast<const typename VT::V*>(s_piv[buf])[j / 2];
#pragma unroll
            for (int r = 0; r < RPT; ++r)
              if (upd[r]) pr[r][j] = fma(-l[r], VT::get(u2, 0), pr[r][j]);
            if (j + 1 >= lim) break;
#pragma unroll
            for (int r = 0; r < RPT; ++r)
              if (upd[r]) pr[r][j + 1] = fma(-l[r], VT::get(u2, 1), pr[r][j + 1]);
          }
        }
      }
    }
#pragma unroll
    for (int r = 0; r < RPT; ++r) {
      const T t0 = pr[r][0];
#pragma unroll
      for (int j = 0; j < W - 1; ++j) pr[r][j] = pr[r][j + 1];
      pr[r][W - 1] = t0;
    }
  }
  // after w steps slot j holds column (w + j) mod 32
#pragma unroll
  for (int r = 0; r < RPT; ++r) {
    const int i = tid + NT * r;
    if (i < nloc)
#pragma unroll
      for (int j = 0; j < W; ++j) {
        const int c = (w + j) & (W - 1);
        if (c < w) A[(base + i) + (c0 + c) * lda] = pr[r][j];
      }
  }
  if (cta == 0 && tid == 0 && info_local != 0 && *info_out == 0) *info_out = info_local;
  cluster.sync();  // no CTA exits while a push to it may be in flight
}

// ---------------------------------------------------------------------------
// laswp for one leaf: interchanges ipiv[c0, c0+w) applied to every column
// outside [c0, c0+w) (blocked_lufact.jl:126-141 applies them to [1, j0) and
// (j1, n]).  Warp 0 of every CTA composes the w swaps into at most 2w moves
// "row r receives old row src(r)"; then each warp moves one column at a time.
template <typename T>
__global__ void __launch_bounds__(256)
laswp_leaf_kernel(T* __restrict__ A, int64_t lda, int64_t m, int64_t ncols_total,
                  int64_t c0, int w, const int64_t* __restrict__ ipiv,
                  DevScratch* __restrict__ scr, int32_t* __restrict__ perm) {
  __shared__ int64_t mv_dst[2 * kPanelMaxW];
  __shared__ int64_t mv_src[2 * kPanelMaxW];
  __shared__ int s_nmv;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (warp == 0) {
    // entry 0 of lane k tracks row c0+k; entry 1 tracks target t_k when it lies
    // below the leaf and no earlier lane already tracks it.
    int64_t t = (lane < w) ? ipiv[c0 + lane] - 1 : -1;
    if (lane < w && (t < c0 + lane || t >= m)) atomicCAS(&scr->error, 0, (int)DEV_BAD_PIVOT_INDEX);
    int64_t row0 = (lane < w) ? c0 + lane : -1;
    int64_t src0 = row0;
    bool dup = false;
    for (int j = 0; j < 32; ++j) {
      int64_t tj = __shfl_sync(0xffffffffu, t, j);
      if (j < lane && tj == t) dup = true;
    }
    int64_t row1 = (lane < w && t >= c0 + w && t < m && !dup) ? t : -1;
    int64_t src1 = row1;
    for (int k = 0; k < w; ++k) {
      int64_t a = c0 + k;
      int64_t b = __shfl_sync(0xffffffffu, t, k);
      if (b == a || b < 0) continue;
      unsigned ha0 = __ballot_sync(0xffffffffu, row0 == a), ha1 = __ballot_sync(0xffffffffu, row1 == a);
      unsigned hb0 = __ballot_sync(0xffffffffu, row0 == b), hb1 = __ballot_sync(0xffffffffu, row1 == b);
      if ((ha0 | ha1) == 0 || (hb0 | hb1) == 0) continue;  // corrupt ipiv: flagged above
      int la = ha0 ? __ffs(ha0) - 1 : __ffs(ha1) - 1;
      int lb = hb0 ? __ffs(hb0) - 1 : __ffs(hb1) - 1;
      int64_t sa = ha0 ? __shfl_sync(0xffffffffu, src0, la) : __shfl_sync(0xffffffffu, src1, la);
      int64_t sb = hb0 ? __shfl_sync(0xffffffffu, src0, lb) : __shfl_sync(0xffffffffu, src1, lb);
      if (ha0) { if (lane == la) src0 = sb; } else { if (lane == la) src1 = sb; }
      if (hb0) { if (lane == lb) src0 = sa; } else { if (lane == lb) src1 = sa; }
    }
    bool m0 = row0 >= 0 && src0 != row0, m1 = row1 >= 0 && src1 != row1;
    unsigned b0 = __ballot_sync(0xffffffffu, m0), b1 = __ballot_sync(0xffffffffu, m1);
    int n0 = __popc(b0);
    if (m0) { int pos = __popc(b0 & ((1u << lane) - 1)); mv_dst[pos] = row0; mv_src[pos] = src0; }
    if (m1) { int pos = n0 + __popc(b1 & ((1u << lane) - 1)); mv_dst[pos] = row1; mv_src[pos] = src1; }
    if (lane == 0) s_nmv = n0 + __popc(b1);
  }
  __syncthreads();
  const int nmv = s_nmv;
  if (nmv == 0) return;
  if (perm != nullptr && blockIdx.x == 0 && warp == 0) {
    // the row permutation (original row of each row) moves like one more column
    int32_t p0 = 0, p1 = 0;
    if (lane < nmv) p0 = perm[mv_src[lane]];
    if (lane + 32 < nmv) p1 = perm[mv_src[lane + 32]];
    __syncwarp();
    if (lane < nmv) perm[mv_dst[lane]] = p0;
    if (lane + 32 < nmv) perm[mv_dst[lane + 32]] = p1;
  }
  const int64_t nother = ncols_total - w;
  const int warps = blockDim.x >> 5;
  const int64_t stride = (int64_t)gridDim.x * warps;
  // two columns per pass: all four loads in flight before the stores
  for (int64_t q = (int64_t)blockIdx.x * warps + warp; q < nother; q += 2 * stride) {
    const int64_t q2 = q + stride;
    T* a = A + (q < c0 ? q : q + w) * lda;
    T* b2 = q2 < nother ? A + (q2 < c0 ? q2 : q2 + w) * lda : nullptr;
    T v0 = T(0), v1 = T(0), u0 = T(0), u1 = T(0);
    if (lane < nmv) v0 = a[mv_src[lane]];
    if (lane + 32 < nmv) v1 = a[mv_src[lane + 32]];
    if (b2 && lane < nmv) u0 = b2[mv_src[lane]];
    if (b2 && lane + 32 < nmv) u1 = b2[mv_src[lane + 32]];
    __syncwarp();
    if (lane < nmv) a[mv_dst[lane]] = v0;
    if (lane + 32 < nmv) a[mv_dst[lane + 32]] = v1;
    if (b2 && lane < nmv) b2[mv_dst[lane]] = u0;
    if (b2 && lane + 32 < nmv) b2[mv_dst[lane + 32]] = u1;
  }
}

// ---------------------------------------------------------------------------
// Unit-lower TRSM base case: B[0:k, cols] := L \ B with L = k x k (k <= KM,
// KM = 64 or 128) held in shared memory.  One warp per right-hand-side
// column: lane l holds rows l, l + 32, ... in registers; x_kk is broadcast
// with a shuffle and every row below it is updated, kk ascending
// (blocked_lufact.jl:146-178 order).  Row blocks of 32 that are already
// final are skipped with a warp-uniform branch, so finished rows cost no
// (FP64) instructions.
constexpr int kTrsmMax = 128;
// warps per CTA: one CTA holds the L block; the FP32 128-row variant runs
// more columns per CTA, while FP64 keeps more CTAs (each SM's FP64 pipe is
// the limit, so the columns should spread over as many SMs as possible)
template <typename T, int KM>
__host__ __device__ constexpr int trsm_warps() { return (sizeof(T) == 4 && KM == 128) ? 16 : 8; }

template <typename T, int KM>
__global__ void __launch_bounds__(trsm_warps<T, KM>() * 32)
trsm_lunit_kernel(const T* __restrict__ L, int64_t ldl, int k, T* __restrict__ B,
                  int64_t ldb, int64_t ncols) {
  constexpr int RPL = KM / 32;  // rows per lane
  // warps (columns in flight) of this CTA: chosen per launch for FP64, fixed
  // for FP32 (a compile-time stride keeps its short chain steps lean)
  const int nw = sizeof(T) == 8 ? (int)(blockDim.x >> 5) : trsm_warps<T, KM>();
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T(*sL)[KM + 1] = reinterpret_cast<T(*)[KM + 1]>(smem_raw);  // sL[c][r] = L[r, c]
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if constexpr (sizeof(T) == 8) {
    // the strictly lower triangle of L, copied asynchronously (an FP64 CTA
    // may have a single warp)
    for (int c = warp; c < k; c += nw)
      for (int r = c + 1 + lane; r < k; r += 32) {
        const unsigned d = (unsigned)__cvta_generic_to_shared(&sL[c][r]);
        asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(d), "l"(L + r + (int64_t)c * ldl)
                     : "memory");
      }
    asm volatile("cp.async.wait_all;" ::: "memory");
  } else {
    // asynchronous copies, all in flight at once (a load-store loop waits
    // out one global latency per element); a fixed thread count keeps the
    // index arithmetic compile-time
    constexpr int NT = trsm_warps<T, KM>() * 32;
#pragma unroll
    for (int e = 0; e < KM * KM / NT; ++e) {
      const int idx = e * NT + (int)threadIdx.x, c = idx / KM, r = idx % KM;
      if (c < k && r > c && r < k) {
        const unsigned d = (unsigned)__cvta_generic_to_shared(&sL[c][r]);
        asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(d), "l"(L + r + (int64_t)c * ldl)
                     : "memory");
      }
    }
    asm volatile("cp.async.wait_all;" ::: "memory");
  }
  __syncthreads();
  for (int64_t col = (int64_t)blockIdx.x * nw + warp; col < ncols; col += (int64_t)gridDim.x * nw) {
    T* b = B + col * ldb;
    T v[RPL];
#pragma unroll
    for (int q = 0; q < RPL; ++q) v[q] = lane + 32 * q < k ? b[lane + 32 * q] : T(0);
    for (int kk = 0; kk < k - 1; ++kk) {
      const int qk = kk >> 5;
      T src = v[0];
#pragma unroll
      for (int q = 1; q < RPL; ++q)
        if (qk == q) src = v[q];
      const T xk = __shfl_sync(0xffffffffu, src, kk & 31);
#pragma unroll
      for (int q = 0; q < RPL; ++q) {
        if (q < qk) continue;  // rows 32q..32q+31 are final
        if (sizeof(T) == 8 && 32 * q >= k) break;  // no rows (a predicated-off FP64 FMA still occupies the pipe)
        const int r = lane + 32 * q;
        if (r > kk && r < k) v[q] = fma(-sL[kk][r], xk, v[q]);
      }
    }
#pragma unroll
    for (int q = 0; q < RPL; ++q)
      if (lane + 32 * q < k) b[lane + 32 * q] = v[q];
  }
}

template <typename T, int KM>
constexpr size_t trsm_smem() { return (size_t)KM * (KM + 1) * sizeof(T); }

// ---------------------------------------------------------------------------
// TRSM base blocks of the 16-bit-operand factors (FP32 working matrix; the
// factors are refinement's preconditioner, not the reference's bit pattern):
// X = L^-1 of a unit-lower k x k diagonal block (64 < k <= 128) once per
// getrf, then B := X B as a product, with no dependent chain.
constexpr int kTinvLd = 128;       // leading dimension of a cached inverse
constexpr int kTinvApCols = 32;    // B columns per CTA of the product
constexpr int kTinvApLdB = kTinvLd + 1;

// Warp w of CTA b solves L x = e_j, j = 16 b + w (the TRSM chain, starting
// at row j: the inverse is lower triangular); column j of X, ld 128.
__global__ void __launch_bounds__(512)
trsm_inv_kernel(const float* __restrict__ L, int64_t ldl, int k, float* __restrict__ X) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float(*sL)[kTinvLd + 1] = reinterpret_cast<float(*)[kTinvLd + 1]>(smem_raw);  // sL[c][r] = L[r, c]
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int e = 0; e < kTinvLd * kTinvLd / 512; ++e) {
    const int idx = e * 512 + (int)threadIdx.x, c = idx / kTinvLd, r = idx % kTinvLd;
    if (c < k && r > c && r < k) {
      const unsigned d = (unsigned)__cvta_generic_to_shared(&sL[c][r]);
      asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(d), "l"(L + r + (int64_t)c * ldl) : "memory");
    }
  }
  asm volatile("cp.async.wait_all;" ::: "memory");
  __syncthreads();
  const int j = blockIdx.x * 16 + warp;
  if (j >= k) return;
  float v[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) v[q] = lane + 32 * q == j ? 1.f : 0.f;
  for (int kk = j; kk < k - 1; ++kk) {
    const int qk = kk >> 5;
    float src = v[0];
#pragma unroll
    for (int q = 1; q < 4; ++q)
      if (qk == q) src = v[q];
    const float xk = __shfl_sync(0xffffffffu, src, kk & 31);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      if (q < qk) continue;
      const int r = lane + 32 * q;
      if (r > kk && r < k) v[q] = fmaf(-sL[kk][r], xk, v[q]);
    }
  }
#pragma unroll
  for (int q = 0; q < 4; ++q) X[lane + 32 * q + (int64_t)j * kTinvLd] = lane + 32 * q < k ? v[q] : 0.f;
}

// B (k x ncols, ldb) := X B with X the cached k x k inverse (ld 128), k a
// multiple of 4.  CTA: 128 rows x 32 columns; thread (ty, tx) = 4 rows x 4
// columns, accumulating over the columns kk <= its last row (X is lower
// triangular).  Each CTA reads its columns of B whole before writing them.
__global__ void __launch_bounds__(256)
trsm_inv_apply_kernel(const float* __restrict__ X, int k, float* __restrict__ B, int64_t ldb, int64_t ncols) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float* sX = reinterpret_cast<float*>(smem_raw);  // sX[kk * 128 + r] = X[r, kk]
  float* sB = sX + kTinvLd * kTinvLd;             // sB[c * 129 + kk] = B[kk, cb + c]
  const int tid = threadIdx.x, ty = tid >> 3, tx = tid & 7;
  const int64_t cb = (int64_t)blockIdx.x * kTinvApCols;
  const int nc = (int)min((int64_t)kTinvApCols, ncols - cb);
  for (int i = tid; i < k * (kTinvLd / 4); i += 256) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(sX + 4 * i);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d), "l"(X + 4 * i) : "memory");
  }
  for (int i = tid; i < k * nc; i += 256) {
    const int c = i / k, kk = i % k;
    const unsigned d = (unsigned)__cvta_generic_to_shared(sB + c * kTinvApLdB + kk);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(d), "l"(B + kk + (cb + c) * ldb) : "memory");
  }
  asm volatile("cp.async.wait_all;" ::: "memory");
  __syncthreads();
  float acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int c = 0; c < 4; ++c) acc[i][c] = 0.f;
  const int kend = min(k, 4 * ty + 4);
  const float* bcol = sB + (4 * tx) * kTinvApLdB;
  for (int kk = 0; kk < kend; ++kk) {
    const float4 x0 = *reinterpret_cast<const float4*>(sX + kk * kTinvLd + 4 * ty);
    const float xr[4] = {x0.x, x0.y, x0.z, x0.w};
    float bv[4];
#pragma unroll
    for (int c = 0; c < 4; ++c) bv[c] = bcol[c * kTinvApLdB + kk];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int c = 0; c < 4; ++c) acc[i][c] = fmaf(xr[i], bv[c], acc[i][c]);
  }
  if (4 * ty >= k) return;
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    if (4 * tx + c >= nc) break;
    float* dst = B + 4 * ty + (cb + 4 * tx + c) * ldb;
#pragma unroll
    for (int i = 0; i < 4; ++i)
      if (4 * ty + i < k) dst[i] = acc[i][c];
  }
}

constexpr size_t trsm_inv_smem() { return (size_t)kTinvLd * (kTinvLd + 1) * sizeof(float); }
constexpr size_t trsm_inv_apply_smem() {
  return (size_t)kTinvLd * kTinvLd * sizeof(float) + (size_t)kTinvApCols * kTinvApLdB * sizeof(float);
}

// ---------------------------------------------------------------------------
// SIMT GEMM update C -= A * B (column-major), every C element updated by
// fma(-a_k, b_k, c) for k ascending.  BM x BN tile (64 x 64, 32 x 32 or
// 16 x 16), 16-deep k slices, 256 threads with a (BM/16) x (BN/16) register
// tile each.  The smaller tiles spread short updates over more SMs: one SM
// of this GPU retires two FP64 FMA lanes per cycle, so an update covered by
// a few 64 x 64 tiles would run on a few SMs.
constexpr int kGBK = 16;

template <typename T, int BM, int BN>
__global__ void __launch_bounds__(256, BM == 64 ? 2 : 4)
gemm_sub_kernel(int64_t M, int64_t N, int64_t K, const T* __restrict__ A, int64_t lda,
                const T* __restrict__ B, int64_t ldb, T* __restrict__ C, int64_t ldc) {
  constexpr int TM = BM / 16, TN = BN / 16;
  __shared__ T sA[kGBK][BM];
  __shared__ T sB[kGBK][BN + 1];
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  const int64_t m0 = (int64_t)blockIdx.x * BM, n0 = (int64_t)blockIdx.y * BN;
  T c[TM][TN];
#pragma unroll
  for (int i = 0; i < TM; ++i)
#pragma unroll
    for (int j = 0; j < TN; ++j) {
      int64_t r = m0 + tx + 16 * i, cc = n0 + ty + 16 * j;
      c[i][j] = (r < M && cc < N) ? C[r + cc * ldc] : T(0);
    }
  for (int64_t k0 = 0; k0 < K; k0 += kGBK) {
#pragma unroll
    for (int q = 0; q < (kGBK * BM) / 256; ++q) {
      int idx = tid + 256 * q;
      int kk = idx / BM, i = idx % BM;
      int64_t r = m0 + i, kc = k0 + kk;
      sA[kk][i] = (r < M && kc < K) ? A[r + kc * lda] : T(0);
    }
#pragma unroll
    for (int q = 0; q < (kGBK * BN) / 256; ++q) {
      int idx = tid + 256 * q;
      int kb = idx % kGBK, j = idx / kGBK;
      int64_t kr = k0 + kb, cc = n0 + j;
      sB[kb][j] = (kr < K && cc < N) ? B[kr + cc * ldb] : T(0);
    }
    __syncthreads();
    const int kmax = (int)min((int64_t)kGBK, K - k0);
    for (int kk = 0; kk < kmax; ++kk) {
      T a[TM], b[TN];
#pragma unroll
      for (int i = 0; i < TM; ++i) a[i] = sA[kk][tx + 16 * i];
#pragma unroll
      for (int j = 0; j < TN; ++j) b[j] = sB[kk][ty + 16 * j];
#pragma unroll
      for (int i = 0; i < TM; ++i)
#pragma unroll
        for (int j = 0; j < TN; ++j) c[i][j] = fma(-a[i], b[j], c[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < TM; ++i)
#pragma unroll
    for (int j = 0; j < TN; ++j) {
      int64_t r = m0 + tx + 16 * i, cc = n0 + ty + 16 * j;
      if (r < M && cc < N) C[r + cc * ldc] = c[i][j];
    }
}

// FP32 update with a 128 x 128 tile and an 8 x 8 register block per thread
// (rows tx*4 .. tx*4+3 and 64+tx*4 .. 64+tx*4+3, the same for columns), so
// each k step reads four float4 from shared memory for 64 FMAs; the next
// 8-deep k slice is fetched into registers while the current one is used.
// Every C element is loaded first and updated by fma(-a_k, b_k, c) for k
// ascending, as in gemm_sub_kernel.
constexpr int kRbK = 8;

__global__ void __launch_bounds__(256, 2)
gemm_sub_f32_rb_kernel(int64_t M, int64_t N, int64_t K, const float* __restrict__ A, int64_t lda,
                       const float* __restrict__ B, int64_t ldb, float* __restrict__ C, int64_t ldc) {
  constexpr int BM = 128, BN = 128, BK = kRbK;
  __shared__ __align__(16) float sA[BK][BM];      // sA[k][i] = A[m0 + i, k0 + k]
  __shared__ __align__(16) float sB[BK][BN + 4];  // sB[k][j] = B[k0 + k, n0 + j] (padded: conflict-free stores)
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  const int64_t m0 = (int64_t)blockIdx.x * BM, n0 = (int64_t)blockIdx.y * BN;
  float c[8][8];
#pragma unroll
  for (int i = 0; i < 8; ++i)
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const int64_t r = m0 + tx * 4 + (i & 3) + (i >> 2) * 64, cc = n0 + ty * 4 + (j & 3) + (j >> 2) * 64;
      c[i][j] = (r < M && cc < N) ? C[r + cc * ldc] : 0.f;
    }
  // this thread's share of a k slice: A elements (kk = idx / 128, i = idx % 128)
  // and B elements (kb = idx % 8, j = idx / 8) for idx = tid + 256 q, q < 4
  float pa[4], pb[4];
  auto fetch = [&](int64_t k0) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int idx = tid + 256 * q;
      const int kk = idx >> 7, i = idx & 127;
      const int64_t r = m0 + i, kc = k0 + kk;
      pa[q] = (r < M && kc < K) ? A[r + kc * lda] : 0.f;
      const int kb = idx & 7, j = idx >> 3;
      const int64_t kr = k0 + kb, cc = n0 + j;
      pb[q] = (kr < K && cc < N) ? B[kr + cc * ldb] : 0.f;
    }
  };
  auto stash = [&]() {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int idx = tid + 256 * q;
      sA[idx >> 7][idx & 127] = pa[q];
      sB[idx & 7][idx >> 3] = pb[q];
    }
  };
  fetch(0);
  stash();
  __syncthreads();
  for (int64_t k0 = 0; k0 < K; k0 += BK) {
    const bool more = k0 + BK < K;
    if (more) fetch(k0 + BK);  // in flight while this slice is used
    const int kmax = (int)min((int64_t)BK, K - k0);
    for (int kk = 0; kk < kmax; ++kk) {
      const float4 a0 = *reinterpret_cast<const float4*>(&sA[kk][tx * 4]);
      const float4 a1 = *reinterpret_cast<const float4*>(&sA[kk][64 + tx * 4]);
      const float4 b0 = *reinterpret_cast<const float4*>(&sB[kk][ty * 4]);
      const float4 b1 = *reinterpret_cast<const float4*>(&sB[kk][64 + ty * 4]);
      const float a[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
      const float b[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
#pragma unroll
      for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) c[i][j] = fmaf(-a[i], b[j], c[i][j]);
    }
    __syncthreads();
    if (more) {
      stash();
      __syncthreads();
    }
  }
#pragma unroll
  for (int i = 0; i < 8; ++i)
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const int64_t r = m0 + tx * 4 + (i & 3) + (i >> 2) * 64, cc = n0 + ty * 4 + (j & 3) + (j >> 2) * 64;
      if (r < M && cc < N) C[r + cc * ldc] = c[i][j];
    }
}

// The tile for an M x N update.  FP64: the least work on the busiest SM,
// ceil(tiles / SMs) x BM x BN, ties to the larger tile (the FP64 pipe is the
// bound: timing every update shape of the n = 8192 and 16384 recursions with
// each tile, this rule came within 0.1 % of the best tile per shape, and the
// smaller tiles' extra loads cost nothing measurable).  FP32: the largest of
// 128 x 128 (register-blocked kernel), 64 x 64, 32 x 32 whose tiles cover the
// SMs, else 16 x 16.
inline int gemm_tile_choice(int64_t M, int64_t N, int sms, int elem_size) {
  auto tiles = [&](int b) { return ((M + b - 1) / b) * ((N + b - 1) / b); };
  if (elem_size == 4) {
    if (tiles(128) >= sms) return 128;
    if (tiles(64) >= sms) return 64;
    if (tiles(32) >= sms) return 32;
    return 16;
  }
  const int bm[3] = {64, 32, 16};
  int best = 64;
  int64_t bt = 0;
  for (int q = 0; q < 3; ++q) {
    const int64_t t = (tiles(bm[q]) + sms - 1) / sms * bm[q] * bm[q];
    if (q == 0 || t < bt) { bt = t; best = bm[q]; }
  }
  return best;
}

// GBLU_GEMM_TILE=128|64|32|16 forces the SIMT update's tile (128: FP32 only,
// 64 for FP64; the tiles give
// identical results), so each variant can be tested on small matrices.
int forced_gemm_tile() {
  const char* e = getenv("GBLU_GEMM_TILE");
  if (!e) return 0;
  const int t = atoi(e);
  return (t == 128 || t == 64 || t == 32 || t == 16) ? t : 0;
}

// forced: 0 = gemm_tile_choice, else the tile edge (64, 32 or 16)
template <typename T>
void gemm_sub_launch(int64_t M, int64_t N, int64_t K, const T* A, int64_t lda, const T* B, int64_t ldb,
                     T* C, int64_t ldc, int sms, int forced, cudaStream_t s) {
  int t = forced ? forced : gemm_tile_choice(M, N, sms, (int)sizeof(T));
  if (t == 128 && sizeof(T) != 4) t = 64;
  dim3 grid((unsigned)((M + t - 1) / t), (unsigned)((N + t - 1) / t));
  if constexpr (std::is_same<T, float>::value) {
    if (t == 128) {
      gemm_sub_f32_rb_kernel<<<grid, 256, 0, s>>>(M, N, K, A, lda, B, ldb, C, ldc);
      return;
    }
  }
  if (t == 64) gemm_sub_kernel<T, 64, 64><<<grid, 256, 0, s>>>(M, N, K, A, lda, B, ldb, C, ldc);
  else if (t == 32) gemm_sub_kernel<T, 32, 32><<<grid, 256, 0, s>>>(M, N, K, A, lda, B, ldb, C, ldc);
  else gemm_sub_kernel<T, 16, 16><<<grid, 256, 0, s>>>(M, N, K, A, lda, B, ldb, C, ldc);
}

// ---------------------------------------------------------------------------
// perm from ipiv: (P A)[i] = A[perm[i]].  One CTA; the interchanges are
// inherently sequential, the rest is parallel.
constexpr int kPermSmemMax = 48 * 1024;  // rows held in shared memory
constexpr int kPermChunk = 4096;         // pivots staged in shared memory at a time

__global__ void __launch_bounds__(1024)
perm_from_ipiv_kernel(const int64_t* __restrict__ ipiv, int64_t kmax, int64_t m,
                      int32_t* __restrict__ perm, DevScratch* __restrict__ scr) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const bool in_smem = m <= kPermSmemMax;
  int32_t* st = reinterpret_cast<int32_t*>(smem_raw);  // kPermChunk pivot targets
  int32_t* sp = st + kPermChunk;
  int32_t* p = in_smem ? sp : perm;
  __shared__ int s_bad;
  for (int64_t i = threadIdx.x; i < m; i += blockDim.x) p[i] = (int32_t)i;
  if (threadIdx.x == 0) s_bad = 0;
  for (int64_t k0 = 0; k0 < kmax; k0 += kPermChunk) {
    const int kc = (int)min((int64_t)kPermChunk, kmax - k0);
    __syncthreads();
    for (int i = threadIdx.x; i < kc; i += blockDim.x) {
      const int64_t t = ipiv[k0 + i] - 1;
      st[i] = (t < k0 + i || t >= m) ? -1 : (int32_t)t;
    }
    __syncthreads();
    if (threadIdx.x == 0 && s_bad == 0) {
      for (int k = 0; k < kc; ++k) {  // the swaps in order, in shared memory only
        const int t = st[k];
        if (t < 0) { s_bad = 1; atomicCAS(&scr->error, 0, (int)DEV_BAD_PIVOT_INDEX); break; }
        const int64_t r = k0 + k;
        const int32_t x = p[r];
        p[r] = p[t];
        p[t] = x;
      }
    }
  }
  __syncthreads();
  if (in_smem)
    for (int64_t i = threadIdx.x; i < m; i += blockDim.x) perm[i] = sp[i];
}

__global__ void iota_kernel(int32_t* __restrict__ perm, int64_t m) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x)
    perm[i] = (int32_t)i;
}

// ---------------------------------------------------------------------------
// Host driver

size_t getrf_scratch_bytes(int64_t m, int64_t n, int elem_size, int panel_width,
                           int device) {
  const DeviceInfo& di = device_info(device);
  size_t G = (size_t)di.num_sms * 8;  // upper bound on panel CTAs
  size_t b = 256;                     // DevScratch, aligned
  b += 2 * G * elem_size + 2 * G * sizeof(int64_t);
  b += 2 * G * kPanelMaxW * elem_size + 2 * kPanelMaxW * elem_size;
  return b + 1024;
}

template <typename T>
void getrf_carve(GetrfPlan<T>& p, void* base, size_t bytes, int device) {
  const DeviceInfo& di = device_info(device);
  size_t G = (size_t)di.num_sms * 8;
  char* c = reinterpret_cast<char*>(base);
  auto take = [&](size_t n) { char* r = c; c += (n + 255) & ~size_t(255); return r; };
  p.scratch = reinterpret_cast<DevScratch*>(take(sizeof(DevScratch)));
  p.slots.cand_val = reinterpret_cast<T*>(take(2 * G * sizeof(T)));
  p.slots.cand_row = reinterpret_cast<int64_t*>(take(2 * G * sizeof(int64_t)));
  p.slots.cand_rowvals = reinterpret_cast<T*>(take(2 * G * kPanelMaxW * sizeof(T)));
  p.slots.diag_rowvals = reinterpret_cast<T*>(take(2 * kPanelMaxW * sizeof(T)));
  (void)bytes;
}

namespace {

template <typename T>
int panel_max_blocks(size_t smem, int /*device*/) {
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, panel_kernel<T>, kPanelThreads, smem) !=
      cudaSuccess)
    return 0;
  return nb;
}

template <typename T>
struct Driver {
  const GetrfPlan<T>& p;
  cudaStream_t s;
  int device;
  cudaError_t err = cudaSuccess;
  int forced = 0;  // forced_panel_kind()
  int forced_tile = 0;  // forced_gemm_tile()
  // the TRSM inverse cache of this getrf: slot and order of the inverse kept
  // for the diagonal block starting at row 32 i (-1: none yet)
  std::vector<int> inv_slot, inv_k;
  int inv_next = 0;

  T* at(int64_t r, int64_t c) const { return p.A + r + c * p.lda; }

  void check(cudaError_t e) {
    if (err == cudaSuccess && e != cudaSuccess) err = e;
  }

  // Cluster panel when the whole panel fits in one cluster's shared memory and
  // each CTA's share of the rank-1 updates stays small; 0 if not launchable.
  bool panel_cluster(int64_t c0, int w) {
    const int64_t M = p.m - c0;
    const int64_t rmax = sizeof(T) == 4 ? 1536 : 192;  // rows per CTA
    int cs = (int)std::min<int64_t>(16, std::max<int64_t>(1, (M + 255) / 256));
    int64_t R = (M + cs - 1) / cs;
    if (R > rmax) return false;
    const size_t smem = (size_t)R * w * sizeof(T);
    if (!cluster_ok(cs, smem)) return false;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(cs);
    cfg.blockDim = dim3(kPanelThreads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = cs;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    double fl = 0;
    for (int k = 0; k < w; ++k) fl += (double)(M - k - 1) * (1.0 + 2.0 * (w - k - 1));
    LaunchScope ls(K_PANEL, fl, 2.0 * M * w * sizeof(T), s);
    check(cudaLaunchKernelEx(&cfg, panel_cluster_kernel<T>, p.A, p.lda, p.m, c0, w, p.ipiv, p.info,
                             (int)R));
    return true;
  }

  static bool cluster_ok(int cs, size_t smem) {
    static std::mutex mu;
    static int cache[17][2] = {};  // [cs][T] : 0 unknown, 1 ok, -1 no (per process, one device family)
    std::lock_guard<std::mutex> g(mu);
    int& c = cache[cs][sizeof(T) == 4 ? 0 : 1];
    if (c == 0) {
      cudaLaunchConfig_t cfg = {};
      cfg.gridDim = dim3(cs);
      cfg.blockDim = dim3(kPanelThreads);
      cfg.dynamicSmemBytes = (sizeof(T) == 4 ? 1536 : 192) * kPanelMaxW * sizeof(T);
      cudaLaunchAttribute attr[1];
      attr[0].id = cudaLaunchAttributeClusterDimension;
      attr[0].val.clusterDim.x = cs;
      attr[0].val.clusterDim.y = 1;
      attr[0].val.clusterDim.z = 1;
      cfg.attrs = attr;
      cfg.numAttrs = 1;
      int nclusters = 0;
      cudaError_t e = cudaOccupancyMaxActiveClusters(&nclusters, panel_cluster_kernel<T>, &cfg);
      c = (e == cudaSuccess && nclusters >= 1) ? 1 : -1;
      cudaGetLastError();
    }
    (void)smem;
    return c == 1;
  }

  template <int RPT>
  bool panel_reg_launch(int64_t c0, int w, int cs) {
    const int64_t M = p.m - c0;
    const int64_t R = (M + cs - 1) / cs;
    if (R > (int64_t)kRegPanelThreads * RPT || !reg_cluster_ok<RPT>(cs)) return false;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(cs);
    cfg.blockDim = dim3(kRegPanelThreads);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = cs;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    double fl = 0;
    for (int k = 0; k < w; ++k) fl += (double)(M - k - 1) * (1.0 + 2.0 * (w - k - 1));
    LaunchScope ls(K_PANEL, fl, 2.0 * M * w * sizeof(T), s);
    check(cudaLaunchKernelEx(&cfg, panel_reg_kernel<T, RPT>, p.A, p.lda, p.m, c0, w, p.ipiv, p.info, (int)R,
                             p.scratch));
    return true;
  }

  // Register panel: the rows spread evenly over up to 16 CTAs of one cluster
  // (at least 128 rows each), one or two rows per thread; false when the
  // panel is taller or not launchable.
  bool panel_reg(int64_t c0, int w) {
    const int64_t M = p.m - c0;
    // FP64 leaves above 8192 rows (two rows per thread would not fit the
    // registers) go to the grid kernel
    if (sizeof(T) == 8 && M > 8192) return false;
    const int cs = (int)std::min<int64_t>(16, std::max<int64_t>(1, (M + 127) / 128));
    const int64_t R = (M + cs - 1) / cs;
    if (R <= kRegPanelThreads) return panel_reg_launch<1>(c0, w, cs);
    if constexpr (sizeof(T) == 4) {
      if (R <= 2 * kRegPanelThreads) return panel_reg_launch<2>(c0, w, cs);
    }
    return false;
  }

  template <int RPT>
  static bool reg_cluster_ok(int cs) {
    static std::mutex mu;
    static int cache[17] = {};  // 0 unknown, 1 ok, -1 no (per process and instantiation)
    std::lock_guard<std::mutex> g(mu);
    int& c = cache[cs];
    if (c == 0) {
      cudaLaunchConfig_t cfg = {};
      cfg.gridDim = dim3(cs);
      cfg.blockDim = dim3(kRegPanelThreads);
      cfg.dynamicSmemBytes = 0;
      cudaLaunchAttribute attr[1];
      attr[0].id = cudaLaunchAttributeClusterDimension;
      attr[0].val.clusterDim.x = cs;
      attr[0].val.clusterDim.y = 1;
      attr[0].val.clusterDim.z = 1;
      cfg.attrs = attr;
      cfg.numAttrs = 1;
      int nclusters = 0;
      cudaError_t e = cudaOccupancyMaxActiveClusters(&nclusters, panel_reg_kernel<T, RPT>, &cfg);
      c = (e == cudaSuccess && nclusters >= 1) ? 1 : -1;
      cudaGetLastError();
    }
    return c == 1;
  }

  void panel(int64_t c0, int w) {
    const int64_t M = p.m - c0;
    const DeviceInfo& di = device_info(device);
    if constexpr (std::is_same<T, float>::value) {
      // random-butterfly-transformed factors: no pivot search, no interchanges
      if (p.nopivot && p.tslu_work) {
        check(genp_panel_launch(p.A, p.lda, p.m, c0, w, p.ipiv, p.info, p.tslu_work, s));
        return;
      }
      // low-precision factors: tournament pivoting for the tall leaves
      if (p.tslu && p.tslu_work && M > 512 && tslu_fits(M, w)) {
        check(tslu_panel_launch(p.A, p.lda, p.m, c0, w, p.ipiv, p.info, p.tslu_work, p.scratch, s));
        laswp(c0, w);
        return;
      }
    }
    // forced: 0 automatic, 1 grid kernel only, 2 shared-memory cluster kernel
    // where it fits, 3 register kernel where it fits (falling back in order)
    if (forced != 1 && forced != 2 && p.use_reg_panel && panel_reg(c0, w)) {
      laswp(c0, w);
      return;
    }
    if (forced != 1 && p.use_cluster_panel && panel_cluster(c0, w)) {
      laswp(c0, w);
      return;
    }
    int G = p.panel_ctas > 0 ? p.panel_ctas
                             : (int)std::max<int64_t>(1, (M + kPanelRowsTarget - 1) / kPanelRowsTarget);
    int R = (int)((M + G - 1) / G);
    size_t smem = (size_t)R * w * sizeof(T);
    const size_t smem_cap = std::min<size_t>(di.smem_optin, 200 * 1024);
    if (smem > smem_cap) {  // need more CTAs for this height
      int64_t rmax = (int64_t)(smem_cap / ((size_t)w * sizeof(T)));
      G = (int)((M + rmax - 1) / rmax);
      R = (int)((M + G - 1) / G);
      smem = (size_t)R * w * sizeof(T);
    }
    int per_sm = panel_max_blocks<T>(smem, device);
    int gmax = std::min(per_sm * di.num_sms, di.num_sms * 8);
    if (G > gmax) {
      G = gmax;
      R = (int)((M + G - 1) / G);
      smem = (size_t)R * w * sizeof(T);
      if (smem > smem_cap || G <= 0) { check(cudaErrorInvalidConfiguration); return; }
    }
    check(cudaMemsetAsync(&p.scratch->barrier, 0, sizeof(unsigned), s));
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(G);
    cfg.blockDim = dim3(kPanelThreads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    {
      double fl = 0;  // getf2 flops of the leaf: scale + rank-1 updates
      for (int k = 0; k < w; ++k) fl += (double)(M - k - 1) * (1.0 + 2.0 * (w - k - 1));
      LaunchScope ls(K_PANEL, fl, 2.0 * M * w * sizeof(T), s);
      check(cudaLaunchKernelEx(&cfg, panel_kernel<T>, p.A, p.lda, p.m, c0, w, p.ipiv, p.info,
                               p.scratch, p.slots, R));
    }
    laswp(c0, w);
  }

  // interchanges of the leaf on every other column
  // The leaf's interchanges on every other column, and on the row permutation
  // (so getrs can gather through it without replaying ipiv).
  void laswp(int64_t c0, int w) {
    const DeviceInfo& di = device_info(device);
    const int64_t nother = p.n - w;
    // CTAs per SM (GBLU_LASWP_CTAS_PER_SM overrides): every CTA first turns
    // the leaf's pivots into its row moves, so fewer CTAs walking more
    // columns each pay that once per SM rather than once per 8 columns
    static const int64_t per_sm = [] {
      const char* e = getenv("GBLU_LASWP_CTAS_PER_SM");
      return e ? std::max<int64_t>(1, atoll(e)) : int64_t(4);
    }();
    const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>((nother + 7) / 8, (int64_t)di.num_sms * per_sm));
    LaunchScope ls(K_LASWP, 0.0, 4.0 * w * std::max<int64_t>(nother, 0) * sizeof(T), s);
    laswp_leaf_kernel<T><<<blocks, 256, 0, s>>>(p.A, p.lda, p.m, p.n, c0, w, p.ipiv, p.scratch, p.perm);
    check(cudaGetLastError());
  }

  void gemm(int64_t M, int64_t N, int64_t K, const T* A, int64_t lda, const T* B, int64_t ldb,
            T* C, int64_t ldc) {
    if (M <= 0 || N <= 0 || K <= 0) return;
    if constexpr (std::is_same<T, float>::value) {
      // the tensor-core path costs two conversion launches besides the GEMM:
      // updates with fewer than 256 rows or 128 columns stay on the SIMT
      // kernel (GBLU_TC_MIN_N overrides the column threshold)
      static const int64_t tc_min_n = [] {
        const char* e = getenv("GBLU_TC_MIN_N");
        return e ? std::max<int64_t>(1, atoll(e)) : int64_t(128);
      }();
      if (p.tc_mode != 0 && M >= 256 && N >= tc_min_n && K >= 64 &&
          tc_work_bytes(M, N, K) <= p.tc_work_bytes) {
        check(tc_gemm_sub(p.tc_mode, M, N, K, A, lda, B, ldb, C, ldc, p.tc_work, &p.scratch->error, s));
        return;
      }
    }
    LaunchScope ls(K_GEMM, 2.0 * M * N * K, (2.0 * M * N + (double)M * K + (double)K * N) * sizeof(T), s);
    gemm_sub_launch<T>(M, N, K, A, lda, B, ldb, C, ldc, device_info(device).num_sms, forced_tile, s);
    check(cudaGetLastError());
  }

  // The cached inverse of the k x k diagonal block of L at row r0 (r0 a
  // multiple of 32): computed on first use in this getrf (the block is final
  // once the leaves covering it are done; a later getrf starts a new cache),
  // reused for any order up to k (the leading block of an inverse is the
  // inverse of the leading block).  Returns the slot, or -1 when full.
  int inverse_slot(int64_t r0, int64_t k) {
    if (inv_slot.empty()) {
      inv_slot.assign((size_t)(p.m / 32 + 2), -1);
      inv_k.assign(inv_slot.size(), 0);
    }
    const size_t key = (size_t)(r0 / 32);
    if (key >= inv_slot.size()) return -1;
    if (inv_slot[key] >= 0 && inv_k[key] >= k) return inv_slot[key];
    int slot = inv_slot[key];
    if (slot < 0) {
      if (inv_next >= p.trsm_inv_slots) return -1;
      slot = inv_next++;
    }
    float* X = p.trsm_inv + (size_t)slot * kTinvLd * kTinvLd;
    LaunchScope ls(K_TRSM, (double)k * k * k / 3.0, ((double)k * k / 2 + (double)k * kTinvLd) * 4.0, s);
    trsm_inv_kernel<<<(unsigned)((k + 15) / 16), 512, trsm_inv_smem(), s>>>(
        reinterpret_cast<const float*>(at(r0, r0)), p.lda, (int)k, X);
    check(cudaGetLastError());
    inv_slot[key] = slot;
    inv_k[key] = (int)k;
    return slot;
  }

  // B (k x ncols at (r0, bc0)) := L \ B, L unit lower at (r0, r0) of size k.
  void trsm(int64_t r0, int64_t k, int64_t bc0, int64_t ncols) {
    if (k <= 0 || ncols <= 0) return;
    if constexpr (std::is_same<T, float>::value) {
      if (p.trsm_inv && k > 64 && k <= kTinvLd && k % 4 == 0 && r0 % 32 == 0) {
        const int slot = inverse_slot(r0, k);
        if (slot >= 0) {
          LaunchScope ls(K_TRSM, 2.0 * k * k * ncols / 2.0, (2.0 * k * ncols + (double)k * k) * 4.0, s);
          trsm_inv_apply_kernel<<<(unsigned)((ncols + kTinvApCols - 1) / kTinvApCols), 256,
                                  trsm_inv_apply_smem(), s>>>(p.trsm_inv + (size_t)slot * kTinvLd * kTinvLd,
                                                              (int)k, at(r0, bc0), p.lda, ncols);
          check(cudaGetLastError());
          return;
        }
      }
    }
    if (k <= p.trsm_base && k <= kTrsmMax) {
      const DeviceInfo& di = device_info(device);
      // one column per warp.  FP64: few columns are spread over the SMs one
      // or two warps per CTA (each column is a chain of k dependent steps of
      // 64-cycle FMAs, and the warps of one SM share its FP64 pipe); FP32
      // chains are short and keep full CTAs.
      const int maxw = k <= 64 ? trsm_warps<T, 64>() : trsm_warps<T, 128>();
      const int warps = sizeof(T) == 4 ? maxw
                                       : (int)std::max<int64_t>(1, std::min<int64_t>(maxw, (ncols + di.num_sms - 1) / di.num_sms));
      unsigned blocks = (unsigned)std::min<int64_t>((ncols + warps - 1) / warps, (int64_t)di.num_sms * 8);
      LaunchScope ls(K_TRSM, (double)k * (k - 1) * ncols, (2.0 * k * ncols + (double)k * k) * sizeof(T), s);
      if (k <= 64)
        trsm_lunit_kernel<T, 64><<<blocks, warps * 32, trsm_smem<T, 64>(), s>>>(
            at(r0, r0), p.lda, (int)k, at(r0, bc0), p.lda, ncols);
      else
        trsm_lunit_kernel<T, 128><<<blocks, warps * 32, trsm_smem<T, 128>(), s>>>(
            at(r0, r0), p.lda, (int)k, at(r0, bc0), p.lda, ncols);
      check(cudaGetLastError());
      return;
    }
    int64_t k1 = k / 2;
    if (p.trsm_inv) {  // halves on 32-row boundaries, so cached blocks recur
      const int64_t a = (k1 + 31) / 32 * 32;
      if (a < k) k1 = a;
    }
    trsm(r0, k1, bc0, ncols);
    gemm(k - k1, ncols, k1, at(r0 + k1, r0), p.lda, at(r0, bc0), p.lda, at(r0 + k1, bc0), p.lda);
    trsm(r0 + k1, k - k1, bc0, ncols);
  }

  void rec(int64_t c0, int64_t w) {
    const int wb = p.panel_width;
    if (w <= wb) {
      panel(c0, (int)w);
      return;
    }
    int64_t w1 = ((w / 2 + wb - 1) / wb) * wb;
    if (w1 >= w) w1 = w - wb;
    rec(c0, w1);
    const int64_t c1 = c0 + w1, w2 = w - w1;
    trsm(c0, w1, c1, w2);
    gemm(p.m - c1, w2, w1, at(c1, c0), p.lda, at(c0, c1), p.lda, at(c1, c1), p.lda);
    rec(c1, w2);
  }
};

}  // namespace

cudaError_t simt_gemm_sub_f32(int64_t M, int64_t N, int64_t K, const float* A, int64_t lda,
                              const float* B, int64_t ldb, float* C, int64_t ldc, cudaStream_t s) {
  if (M <= 0 || N <= 0 || K <= 0) return cudaSuccess;
  int device = 0;
  cudaGetDevice(&device);
  LaunchScope ls(K_GEMM, 2.0 * M * N * K, (2.0 * M * N + (double)M * K + (double)K * N) * 4.0, s);
  gemm_sub_launch<float>(M, N, K, A, lda, B, ldb, C, ldc, device_info(device).num_sms, forced_gemm_tile(), s);
  return cudaGetLastError();
}

cudaError_t perm_build_launch(const int64_t* ipiv, int64_t kmax, int64_t m, int32_t* perm,
                              DevScratch* scr, cudaStream_t s) {
  size_t smem = (size_t)kPermChunk * sizeof(int32_t) + (m <= kPermSmemMax ? (size_t)m * sizeof(int32_t) : 0);
  LaunchScope ls(K_PERM, 0.0, 8.0 * kmax + 4.0 * m, s);
  perm_from_ipiv_kernel<<<1, 1024, smem, s>>>(ipiv, kmax, m, perm, scr);
  return cudaGetLastError();
}

int trsm_inv_slot_count(int64_t n) { return (int)(n / 64 + 8); }
size_t trsm_inv_bytes(int64_t n) {
  return (size_t)trsm_inv_slot_count(n) * kTinvLd * kTinvLd * sizeof(float);
}

void getrf_configure(int device) {
  cudaFuncSetAttribute(trsm_inv_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)trsm_inv_smem());
  cudaFuncSetAttribute(trsm_inv_apply_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)trsm_inv_apply_smem());
  const DeviceInfo& di = device_info(device);
  const int cap = (int)std::min<size_t>(di.smem_optin, 200 * 1024);
  cudaFuncSetAttribute(panel_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, cap);
  cudaFuncSetAttribute(panel_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, cap);
  cudaFuncSetAttribute(panel_cluster_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, cap);
  cudaFuncSetAttribute(panel_cluster_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, cap);
  cudaFuncSetAttribute(panel_cluster_kernel<double>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
  cudaFuncSetAttribute(panel_cluster_kernel<float>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
  cudaFuncSetAttribute(panel_reg_kernel<double, 1>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
  cudaFuncSetAttribute(panel_reg_kernel<float, 1>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
  cudaFuncSetAttribute(panel_reg_kernel<float, 2>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
  cudaFuncSetAttribute(trsm_lunit_kernel<double, 128>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)trsm_smem<double, 128>());
  cudaFuncSetAttribute(trsm_lunit_kernel<float, 128>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)trsm_smem<float, 128>());
  cudaFuncSetAttribute(perm_from_ipiv_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (kPermSmemMax + kPermChunk) * (int)sizeof(int32_t));
  getrs_configure(device);
  tc_configure(device);
  tslu_configure(device);
}

// GBLU_PANEL=grid|cluster|reg forces one panel kernel (where the panel fits
// it; the kernels give identical results), so every variant can be tested on
// small matrices.  Read at each factorization.
int forced_panel_kind() {
  const char* e = getenv("GBLU_PANEL");
  if (!e) return 0;
  if (!strcmp(e, "grid")) return 1;
  if (!strcmp(e, "cluster")) return 2;
  if (!strcmp(e, "reg")) return 3;
  return 0;
}

template <typename T>
cudaError_t getrf_launch(const GetrfPlan<T>& p, cudaStream_t stream) {
  int device = 0;
  cudaGetDevice(&device);
  Driver<T> d{p, stream, device};
  d.forced = forced_panel_kind();
  d.forced_tile = forced_gemm_tile();
  const int64_t minmn = std::min(p.m, p.n);
  d.check(cudaMemsetAsync(p.info, 0, sizeof(int64_t), stream));
  if (minmn > 0) {
    {
      LaunchScope ls(K_PERM, 0.0, 4.0 * p.m, stream);
      iota_kernel<<<(unsigned)std::min<int64_t>((p.m + 255) / 256, 1024), 256, 0, stream>>>(p.perm, p.m);
      d.check(cudaGetLastError());
    }
    d.rec(0, minmn);  // each leaf's laswp also permutes p.perm
    if (p.n > p.m) d.trsm(0, p.m, p.m, p.n - p.m);  // wide: U12 := L11 \ A12
  }
  return d.err;
}

template cudaError_t getrf_launch<double>(const GetrfPlan<double>&, cudaStream_t);
template cudaError_t getrf_launch<float>(const GetrfPlan<float>&, cudaStream_t);
template void getrf_carve<double>(GetrfPlan<double>&, void*, size_t, int);
template void getrf_carve<float>(GetrfPlan<float>&, void*, size_t, int);

}  // namespace gblu
