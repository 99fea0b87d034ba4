// Batched uneven LU: thousands of independent square systems A_i x_i = b_i
// (n_i <= 256) factored and solved by one persistent kernel per size bucket,
// all captured in one CUDA graph.
//
// Per system the algorithm is the reference's blocked getrf
// (src/blocked_lufact.jl:658-679: panel getf2, interchanges, unit-lower TRSM,
// Schur update) followed by its back-solve (src/factorization.jl:433-457),
// with the same per-element fused-multiply-add order, so the FP64 results are
// bit-identical to the oracle's per-system getrf + getrs.  A CTA takes the
// next system from a queue ordered by decreasing size (longest first), keeps
// the current panel in registers (one row per thread) and its columns and the
// U12 row block in shared memory, and updates the trailing matrix in global
// memory, where the system's working set stays L2-resident.
//
// The mixed variant factors a FP32 copy with the same code and refines each
// system in FP64 (residual with the FP64 A, per-system backward-error test,
// up to `maxit` corrections); systems that do not converge are flagged and
// re-solved by the FP64 kernel in the same graph.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <new>
#include <vector>

#include "device_util.cuh"
#include "gblu_internal.h"
#include "objects.h"
#include "profile.h"

namespace gblu {

constexpr int kBatchMaxN = 256;

struct BatchDev {
  const int32_t* order;   // systems in processing order (decreasing n)
  const int32_t* sizes;   // n_i
  const int64_t* a_off;   // element offset of A_i in the packed A
  const int64_t* b_off;   // element offset of b_i / x_i / ipiv_i
  int32_t count;          // systems in this bucket's queue
  unsigned* queue;        // next index into order (zeroed before the launch)
  int64_t* info;          // per system: getrf info; refinement failure sets flag
  int32_t* flag;          // per system: 1 = needs the FP64 path
  int32_t* iters;         // per system: refinement iterations, -1 = FP64 re-solve
};

constexpr int kBatchUStride = kBatchMaxN + 8;  // U12 rows, padded for the micro-tile loads

// Shared-memory carve of one system's working set (NB <= 16, NT <= 512).
template <typename T, int NT, int NB>
struct SysSmem {
  static constexpr int NW = NT / 32;
  T* L;      // panel columns: column j of the current panel at L + j*kBatchMaxN (row-indexed)
  T* U;      // U12 rows: row j at U + j*kBatchUStride (indexed by column - c1)
  T* xs;     // solve vector
  typename PivKey<T>::K* cval;  // [2][NW] pivot candidate key per warp (double-buffered by column parity)
  T* crowv;  // [2][NW][NB] candidate row's panel values
  T* diagv;  // [2][NB] current diagonal row's panel values
  int* crow;  // [2][NW] candidate row per warp
  int* perm;  // [kBatchMaxN] row r of the factored matrix holds original row perm[r]
  int* list;  // [32] rows moved by the current panel's interchanges
  int* lsrc;  // [32] row each of them receives its value from
  int* pidx;  // [NB] pivot rows of the current panel (0-based)
  int* cnt;   // entries of list
  double* xd;   // FP64 iterate (mixed kernel)
  double* rd;   // FP64 residual (mixed kernel)
  double* red;  // [64] block reductions

  __host__ __device__ static constexpr size_t al(size_t x) { return (x + 15) & ~size_t(15); }
  __host__ __device__ static constexpr size_t bytes(bool mixed) {
    return al(NB * kBatchMaxN * sizeof(T)) + al(NB * kBatchUStride * sizeof(T)) +
           al(kBatchMaxN * sizeof(T)) + al(2 * NW * sizeof(T)) + al(2 * NW * NB * sizeof(T)) +
           al(2 * NB * sizeof(T)) + al(2 * NW * 4) + al(kBatchMaxN * 4) + 2 * al(32 * 4) + al(NB * 4) +
           al(4) + (mixed ? 2 * al(kBatchMaxN * 8) : 0) + al(64 * 8);
  }
  __device__ explicit SysSmem(unsigned char* p, bool mixed) {
    auto take = [&](size_t b) { unsigned char* q = p; p += al(b); return q; };
    L = reinterpret_cast<T*>(take(NB * kBatchMaxN * sizeof(T)));
    U = reinterpret_cast<T*>(take(NB * kBatchUStride * sizeof(T)));
    xs = reinterpret_cast<T*>(take(kBatchMaxN * sizeof(T)));
    cval = reinterpret_cast<typename PivKey<T>::K*>(take(2 * NW * sizeof(T)));
    crowv = reinterpret_cast<T*>(take(2 * NW * NB * sizeof(T)));
    diagv = reinterpret_cast<T*>(take(2 * NB * sizeof(T)));
    crow = reinterpret_cast<int*>(take(2 * NW * 4));
    perm = reinterpret_cast<int*>(take(kBatchMaxN * 4));
    list = reinterpret_cast<int*>(take(32 * 4));
    lsrc = reinterpret_cast<int*>(take(32 * 4));
    pidx = reinterpret_cast<int*>(take(NB * 4));
    cnt = reinterpret_cast<int*>(take(4));
    xd = rd = nullptr;
    if (mixed) {
      xd = reinterpret_cast<double*>(take(kBatchMaxN * 8));
      rd = reinterpret_cast<double*>(take(kBatchMaxN * 8));
    }
    red = reinterpret_cast<double*>(take(64 * 8));
  }
};


// In-place getrf of one n x n column-major system (ld = n) in global memory,
// blocked by NB columns (src/blocked_lufact.jl:658-679 order):
//   * panel getf2: the row i of the panel lives in registers of thread i % NT;
//     per column each warp publishes its candidate (first row of max |a|),
//     the candidate row's panel values and the diagonal row, one barrier,
//     then every thread picks the winner, interchanges, scales by the
//     reciprocal of the pivot and updates its own rows, columns in order;
//   * interchanges on the other columns: warp 0 composes the panel's
//     interchanges into "row list[m] takes the value of row lsrc[m]" with
//     ballots and shuffles, then each column is one gather (independent loads);
//   * U12 = L11 \ A12 by one thread per column, k ascending;
//   * A22 -= L21 U12 by register micro-tiles, each element j ascending.
// The per-element arithmetic is the reference's, so FP64 results are
// bit-identical to the oracle's getrf.  ipiv: 1-based; sm.perm receives the
// composed row permutation.  Returns info (0 or first zero pivot, 1-based).
template <typename T, int NT, int NB>
__device__ int64_t factor_system(T* __restrict__ A, int n, int32_t* __restrict__ ipiv,
                                 const SysSmem<T, NT, NB>& sm) {
  constexpr int NW = NT / 32;
  constexpr int RPT = (kBatchMaxN + NT - 1) / NT;  // panel rows per thread
  using K = typename PivKey<T>::K;
  static_assert(NB <= 16, "composition warp holds 2*NB rows");
  static_assert(sizeof(K) == sizeof(T), "key and value slots share a size");
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  int64_t info = 0;
  for (int i = tid; i < kBatchMaxN; i += NT) sm.perm[i] = i;
  __syncthreads();
  for (int k0 = 0; k0 < n; k0 += NB) {
    const int kb = min(NB, n - k0);
    const int c1 = k0 + kb;
    T pr[RPT][NB];
#pragma unroll
    for (int m = 0; m < RPT; ++m) {
      const int i = tid + NT * m;
#pragma unroll
      for (int j = 0; j < NB; ++j)
        pr[m][j] = (i >= k0 && i < n && j < kb) ? A[i + (int64_t)(k0 + j) * n] : T(0);
    }
#pragma unroll
    for (int j = 0; j < NB; ++j) {
      if (j >= kb) continue;  // uniform; keeps the loop fully unrolled (pr indexed statically)
      const int col = k0 + j;
      const int buf = j & 1;
      K bv = 0;
      int bg = -1;
#pragma unroll
      for (int m = 0; m < RPT; ++m) {
        const int i = tid + NT * m;
        if (i >= col && i < n) {
          const K v = PivKey<T>::of(pr[m][j]);
          if (v > bv) { bv = v; bg = i; }
        }
      }
      {
        int src;
        warp_pivot_choice(bv, bg, src);
      }
      if (lane == 0) { sm.cval[buf * NW + warp] = bv; sm.crow[buf * NW + warp] = bg; }
      // the owners publish (row tests, not a computed slot index, so pr stays in registers)
#pragma unroll
      for (int m = 0; m < RPT; ++m)
        if (bg == tid + NT * m)
#pragma unroll
          for (int jj = 0; jj < NB; ++jj)
            if (jj < kb) sm.crowv[(buf * NW + warp) * NB + jj] = pr[m][jj];
#pragma unroll
      for (int m = 0; m < RPT; ++m)
        if (col == tid + NT * m)
#pragma unroll
          for (int jj = 0; jj < NB; ++jj)
            if (jj < kb) sm.diagv[buf * NB + jj] = pr[m][jj];
      __syncthreads();
      K wv = lane < NW ? sm.cval[buf * NW + lane] : K(0);
      int wg = lane < NW ? sm.crow[buf * NW + lane] : -1;
      int ww;  // the winning warp (= the lane that held its slot)
      warp_pivot_choice(wv, wg, ww);
      const int p = wg < 0 ? col : wg;  // kp = k when the column is zero below the diagonal
      const T* src = (p == col) ? sm.diagv + buf * NB : sm.crowv + (buf * NW + ww) * NB;
      const T piv = src[j];
      const bool nz = PivKey<T>::nonzero(piv);  // integer test, off the FP64 pipe
      if (tid == 0) { sm.pidx[j] = p; ipiv[col] = p + 1; }
      if (!nz && info == 0) info = col + 1;
      const bool swap = nz && p != col;
      const T inv = nz ? T(1) / piv : T(0);
#pragma unroll
      for (int m = 0; m < RPT; ++m) {
        // row slot m of the CTA holds rows NT*m .. NT*m+NT-1: skip it with a
        // block-uniform branch when all of them lie above the diagonal row (no
        // interchange, no update) or outside the system (predicated-off FP64
        // instructions still occupy the FP64 pipe)
        if (NT * m + NT - 1 < col || NT * m >= n) continue;
        const int i = tid + NT * m;
        if (swap && i == col) {
#pragma unroll
          for (int jj = 0; jj < NB; ++jj)
            if (jj < kb) pr[m][jj] = src[jj];
        } else if (swap && i == p) {
#pragma unroll
          for (int jj = 0; jj < NB; ++jj)
            if (jj < kb) pr[m][jj] = sm.diagv[buf * NB + jj];
        }
        if (i > col && i < n) {
          T l = pr[m][j];
          if (nz) l *= inv;
          pr[m][j] = l;
#pragma unroll
          for (int jj = j + 1; jj < NB; ++jj) {
            if (jj >= kb) break;
            pr[m][jj] = fma(-l, src[jj], pr[m][jj]);
          }
        }
      }
    }
    // panel back to global memory; its columns to shared memory for TRSM and update
#pragma unroll
    for (int m = 0; m < RPT; ++m) {
      const int i = tid + NT * m;
      if (i >= k0 && i < n)
#pragma unroll
        for (int jj = 0; jj < NB; ++jj)
          if (jj < kb) {
            A[i + (int64_t)(k0 + jj) * n] = pr[m][jj];
            sm.L[jj * kBatchMaxN + i] = pr[m][jj];
          }
    }
    if (warp == 0) {
      // rows touched by the panel's interchanges: k0..c1-1 (lanes 0..kb-1) and
      // the pivot rows below the panel (lanes NB.., duplicates dropped)
      int row = -1;
      if (lane < kb) row = k0 + lane;
      else if (lane >= NB && lane - NB < kb) {
        const int pj = sm.pidx[lane - NB];
        if (pj >= c1) row = pj;
      }
      const unsigned same = __match_any_sync(0xffffffffu, row);
      if (row >= 0 && __ffs(same) - 1 != lane) row = -1;
      int from = row;  // original row whose value ends at `row`
      for (int j = 0; j < kb; ++j) {
        const int b = sm.pidx[j];
        if (b != k0 + j) {
          const unsigned hm = __ballot_sync(0xffffffffu, row == b);
          if (hm != 0u) {
            const int hb = __ffs(hm) - 1;
            const int srcl = lane == j ? hb : (lane == hb ? j : lane);
            from = __shfl_sync(0xffffffffu, from, srcl);
          }
        }
      }
      const unsigned vm = __ballot_sync(0xffffffffu, row >= 0);
      const int pos = __popc(vm & ((1u << lane) - 1u));
      const int pv = row >= 0 ? sm.perm[from] : 0;
      __syncwarp();
      if (row >= 0) {
        sm.list[pos] = row;
        sm.lsrc[pos] = from;
        sm.perm[row] = pv;
      }
      if (lane == 0) *sm.cnt = __popc(vm);
    }
    __syncthreads();
    // interchanges on the other columns (list entries 0..kb-1 are rows k0..c1-1
    // in order), fused with U12 := L11 \ A12 for the columns right of the panel
    const int cnt = *sm.cnt;
    for (int c = tid; c < n; c += NT) {
      if (c >= k0 && c < c1) continue;
      T* ac = A + (int64_t)c * n;
      T v[2 * NB];
#pragma unroll
      for (int m = 0; m < 2 * NB; ++m)
        if (m < cnt) v[m] = ac[sm.lsrc[m]];
      if (c >= c1) {
#pragma unroll
        for (int j = 0; j < NB; ++j)
#pragma unroll
          for (int i = j + 1; i < NB; ++i)
            if (i < kb) v[i] = fma(-sm.L[j * kBatchMaxN + k0 + i], v[j], v[i]);
#pragma unroll
        for (int j = 0; j < NB; ++j)
          if (j < kb) sm.U[j * kBatchUStride + (c - c1)] = v[j];
      }
#pragma unroll
      for (int m = 0; m < 2 * NB; ++m)
        if (m < cnt) ac[sm.list[m]] = v[m];
    }
    __syncthreads();
    // A22 -= L21 * U12: warp tiles of 32*RM rows x CN columns, each lane RM x CN
    const int nr = n - c1;
    if (nr > 0) {
      constexpr int RM = 4;
      constexpr int CN = sizeof(T) == 4 ? 8 : 4;
      const int RB = (nr + 32 * RM - 1) / (32 * RM), CB = (nr + CN - 1) / CN;
      for (int t = warp; t < RB * CB; t += NW) {
        const int rb = t % RB, cb = t / RB;
        const int i0 = c1 + rb * 32 * RM;
        const int rg = min(RM, (n - i0 + 31) / 32);  // 32-row groups reaching below n (warp-uniform)
        const int ib = i0 + lane;
        const int cc = cb * CN;  // column offset from c1
        T acc[RM][CN];
#pragma unroll
        for (int r = 0; r < RM; ++r)
#pragma unroll
          for (int q = 0; q < CN; ++q) {
            const int i = ib + 32 * r, c = c1 + cc + q;
            acc[r][q] = (r < rg && i < n && c < n) ? A[i + (int64_t)c * n] : T(0);
          }
#pragma unroll
        for (int jj = 0; jj < NB; ++jj) {
          if (jj >= kb) continue;
          T lv[RM], uv[CN];
#pragma unroll
          for (int r = 0; r < RM; ++r)
            lv[r] = r < rg ? sm.L[jj * kBatchMaxN + min(ib + 32 * r, kBatchMaxN - 1)] : T(0);
#pragma unroll
          for (int q = 0; q < CN; ++q) uv[q] = sm.U[jj * kBatchUStride + cc + q];
#pragma unroll
          for (int r = 0; r < RM; ++r) {
            if (r >= rg) break;  // warp-uniform: row groups below n only
#pragma unroll
            for (int q = 0; q < CN; ++q) acc[r][q] = fma(-lv[r], uv[q], acc[r][q]);
          }
        }
#pragma unroll
        for (int r = 0; r < RM; ++r)
#pragma unroll
          for (int q = 0; q < CN; ++q) {
            const int i = ib + 32 * r, c = c1 + cc + q;
            if (r < rg && i < n && c < n) A[i + (int64_t)c * n] = acc[r][q];
          }
      }
    }
    __syncthreads();
  }
  return info;
}

// xs := U \ (L \ xs) with the factors of factor_system, xs already permuted
// (xs[r] = b[perm[r]]).  Blocks of 32: warp 0 solves the diagonal block with
// shuffles, then every thread applies the block column to its rows.  Per
// element the order is the reference's back-solve (src/factorization.jl:433-457):
// forward j ascending, backward j descending with x[j] / U[j,j] (a correctly
// rounded quotient from the reciprocal, Markstein's method).
template <typename T, int NT>
__device__ void lu_solve_permuted(const T* __restrict__ LU, int n, T* xs) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (int b0 = 0; b0 < n; b0 += 32) {
    const int bw = min(32, n - b0);
    if (warp == 0) {
      T lr[32];
#pragma unroll
      for (int j = 0; j < 32; ++j)
        lr[j] = (j < lane && lane < bw) ? LU[(b0 + lane) + (int64_t)(b0 + j) * n] : T(0);
      T x = lane < bw ? xs[b0 + lane] : T(0);
#pragma unroll
      for (int j = 0; j < 32; ++j) {
        const T xj = __shfl_sync(0xffffffffu, x, j);
        if (j < lane && lane < bw) x = fma(-lr[j], xj, x);
      }
      if (lane < bw) xs[b0 + lane] = x;
    }
    __syncthreads();
    for (int i = b0 + bw + tid; i < n; i += NT) {
      T lr[32];
#pragma unroll
      for (int j = 0; j < 32; ++j) lr[j] = j < bw ? LU[i + (int64_t)(b0 + j) * n] : T(0);
      T acc = xs[i];
#pragma unroll
      for (int j = 0; j < 32; ++j)
        if (j < bw) acc = fma(-lr[j], xs[b0 + j], acc);
      xs[i] = acc;
    }
    __syncthreads();
  }
  for (int b0 = ((n - 1) / 32) * 32; b0 >= 0; b0 -= 32) {
    const int bw = min(32, n - b0);
    if (warp == 0) {
      T ur[32];
#pragma unroll
      for (int j = 0; j < 32; ++j)
        ur[j] = (j > lane && j < bw) ? LU[(b0 + lane) + (int64_t)(b0 + j) * n] : T(0);
      const T d = lane < bw ? LU[(b0 + lane) + (int64_t)(b0 + lane) * n] : T(1);
      const T y = T(1) / d;
      T x = lane < bw ? xs[b0 + lane] : T(0);
#pragma unroll
      for (int j = 31; j >= 0; --j) {
        if (j < bw) {
          if (lane == j) x = div_markstein(x, d, y);
          const T xj = __shfl_sync(0xffffffffu, x, j);
          if (lane < j) x = fma(-ur[j], xj, x);
        }
      }
      if (lane < bw) xs[b0 + lane] = x;
    }
    __syncthreads();
    for (int i = tid; i < b0; i += NT) {
      T ur[32];
#pragma unroll
      for (int j = 0; j < 32; ++j) ur[j] = j < bw ? LU[i + (int64_t)(b0 + j) * n] : T(0);
      T acc = xs[i];
#pragma unroll
      for (int j = 31; j >= 0; --j)
        if (j < bw) acc = fma(-ur[j], xs[b0 + j], acc);
      xs[i] = acc;
    }
    __syncthreads();
  }
}

// NaN-propagating maximum (a NaN residual must not look converged).
__device__ __forceinline__ double nan_max(double a, double b) {
  if (a != a) return a;
  if (b != b) return b;
  return a > b ? a : b;
}

// Block-wide maxima of two values (every thread receives both).
template <int NT>
__device__ __forceinline__ void block_max2(double& a, double& b, double* red) {
  for (int off = 16; off; off >>= 1) {
    a = nan_max(a, __shfl_down_sync(0xffffffffu, a, off));
    b = nan_max(b, __shfl_down_sync(0xffffffffu, b, off));
  }
  if ((threadIdx.x & 31) == 0) { red[threadIdx.x >> 5] = a; red[32 + (threadIdx.x >> 5)] = b; }
  __syncthreads();
  a = 0.0;
  b = 0.0;
  for (int w = 0; w < NT / 32; ++w) { a = nan_max(a, red[w]); b = nan_max(b, red[32 + w]); }
  __syncthreads();
}

template <typename T, int NT, int NB>
__host__ __device__ constexpr size_t batch_smem(bool mixed) {
  return SysSmem<T, NT, NB>::bytes(mixed);
}

// FP64: factor in place and solve; x overwrites b.  With only_flagged, only
// the systems the mixed kernel flagged are processed, each first copied from
// Asrc (the untouched FP64 input) into Awork.
template <int NT, int NB>
__global__ void __launch_bounds__(NT, NT <= 64 ? 8 : NT <= 128 ? (NB <= 8 ? 4 : 3) : (NT <= 256 ? 2 : 1))
batch_fp64_kernel(BatchDev d, double* __restrict__ Awork, const double* __restrict__ Asrc,
                  double* __restrict__ X, int32_t* __restrict__ ipiv_all, int only_flagged) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const SysSmem<double, NT, NB> sm(smem_raw, false);
  __shared__ int s_idx;
  for (;;) {
    if (threadIdx.x == 0) s_idx = (int)atomicAdd(d.queue, 1u);
    __syncthreads();
    const int qi = s_idx;
    __syncthreads();
    if (qi >= d.count) break;
    const int s = d.order[qi];
    if (only_flagged && d.flag[s] == 0) continue;
    const int n = d.sizes[s];
    double* A = Awork + d.a_off[s];
    if (only_flagged) {
      const double* A0 = Asrc + d.a_off[s];
      for (int i = threadIdx.x; i < n * n; i += NT) A[i] = A0[i];
      __syncthreads();
    }
    int32_t* ipiv = ipiv_all + d.b_off[s];
    const int64_t info = factor_system<double, NT, NB>(A, n, ipiv, sm);
    if (threadIdx.x == 0) { d.info[s] = info; if (only_flagged) d.flag[s] = 0; }
    if (info == 0) {
      double* x = X + d.b_off[s];
      for (int i = threadIdx.x; i < n; i += NT) sm.xs[i] = x[sm.perm[i]];
      __syncthreads();
      lu_solve_permuted<double, NT>(A, n, sm.xs);
      for (int i = threadIdx.x; i < n; i += NT) x[i] = sm.xs[i];
    }
    __syncthreads();
  }
}

// Mixed: FP32 factors of each system, FP64 refinement against the FP64 A:
// residual r = b - A x in FP64, correction LU32 \ (r / s) * s with s a power
// of two near ||r||, stop when ||r|| / (||A|| ||x|| + ||b||) <= n eps (infinity
// norms), at stagnation, or after maxit corrections.  Systems that do not
// converge (or whose FP32 factorization hit a zero pivot) are flagged for the
// FP64 kernel that runs after this one in the same graph.
template <int NT, int NB>
__global__ void __launch_bounds__(NT, NT <= 64 ? 8 : NT <= 128 ? (NB <= 8 ? 4 : 3) : (NT <= 256 ? 2 : 1))
batch_mixed_kernel(BatchDev d, const double* __restrict__ A64, float* __restrict__ A32,
                   double* __restrict__ X, const double* __restrict__ Bcopy,
                   int32_t* __restrict__ ipiv_all, int maxit, double tol_per_n) {
  constexpr int RPT = (kBatchMaxN + NT - 1) / NT;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const SysSmem<float, NT, NB> sm(smem_raw, true);
  __shared__ int s_idx;
  for (;;) {
    if (threadIdx.x == 0) s_idx = (int)atomicAdd(d.queue, 1u);
    __syncthreads();
    const int qi = s_idx;
    __syncthreads();
    if (qi >= d.count) break;
    const int s = d.order[qi];
    const int n = d.sizes[s];
    const double* A = A64 + d.a_off[s];
    float* F = A32 + d.a_off[s];
    int32_t* ipiv = ipiv_all + d.b_off[s];
    double* xo = X + d.b_off[s];
    const double* b = Bcopy + d.b_off[s];
    // FP32 copy and FP64 row sums of |A| in one pass (thread i % NT owns row i)
    double rs[RPT];
#pragma unroll
    for (int m = 0; m < RPT; ++m) rs[m] = 0.0;
    for (int j = 0; j < n; ++j) {
#pragma unroll
      for (int m = 0; m < RPT; ++m) {
        if (NT * m >= n) break;  // block-uniform: no rows in this slot
        const int i = threadIdx.x + NT * m;
        if (i < n) {
          const double a = A[i + (int64_t)j * n];
          F[i + (int64_t)j * n] = (float)a;
          rs[m] += fabs(a);
        }
      }
    }
    double ra = 0.0, bm = 0.0;
#pragma unroll
    for (int m = 0; m < RPT; ++m) {
      const int i = threadIdx.x + NT * m;
      if (i < n) {
        ra = nan_max(ra, rs[m]);
        bm = nan_max(bm, fabs(b[i]));
        sm.xd[i] = 0.0;
        sm.rd[i] = b[i];
      }
    }
    block_max2<NT>(ra, bm, sm.red);
    const double anorm = ra, bnorm = bm;
    const int64_t info = factor_system<float, NT, NB>(F, n, ipiv, sm);
    const double tol = tol_per_n * n;
    bool ok = false;
    int iters_done = 0;
    if (info == 0) {
      double prev = INFINITY;
      for (int it = 0; it <= maxit; ++it) {
        iters_done = it;
        if (it > 0) {  // r = b - A x (FP64, row-parallel, column order fixed)
          for (int i = threadIdx.x; i < n; i += NT) {
            double acc = b[i];
            for (int j = 0; j < n; ++j) acc = fma(-A[i + (int64_t)j * n], sm.xd[j], acc);
            sm.rd[i] = acc;
          }
        }
        double rm = 0.0, xm = 0.0;
        for (int i = threadIdx.x; i < n; i += NT) {
          rm = nan_max(rm, fabs(sm.rd[i]));
          xm = nan_max(xm, fabs(sm.xd[i]));
        }
        block_max2<NT>(rm, xm, sm.red);
        const double den = anorm * xm + bnorm;
        const double be = den > 0 ? rm / den : (rm == 0 ? 0.0 : INFINITY);
        if (be <= tol) { ok = true; break; }
        if (!(be < 0.9 * prev) && it >= 2) break;  // stagnation (or NaN)
        prev = be;
        if (it == maxit) break;
        const double sc = rm > 0 && isfinite(rm) ? ldexp(1.0, ilogb(rm)) : 1.0;
        for (int i = threadIdx.x; i < n; i += NT) sm.xs[i] = (float)(sm.rd[sm.perm[i]] / sc);
        __syncthreads();
        lu_solve_permuted<float, NT>(F, n, sm.xs);
        for (int i = threadIdx.x; i < n; i += NT) sm.xd[i] += sc * (double)sm.xs[i];
        __syncthreads();
      }
    }
    if (ok)
      for (int i = threadIdx.x; i < n; i += NT) xo[i] = sm.xd[i];
    if (threadIdx.x == 0) {
      d.info[s] = 0;
      d.flag[s] = ok ? 0 : 1;  // the FP64 kernel re-solves flagged systems from A64
      d.iters[s] = ok ? iters_done : -1;
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// host side

struct BatchBucket {
  int nt = 256;  // threads per CTA
  int nb = 16;   // panel width
  int lo = 1, hi = kBatchMaxN;
  int count = 0;
  int32_t* order = nullptr;  // device slice of the order array
  unsigned* queue = nullptr;
  int ctas = 0;
};

}  // namespace gblu

struct gblu_batch {
  int64_t count = 0;
  int32_t precision = GBLU_FP64;
  int64_t a_total = 0, b_total = 0;
  std::vector<int32_t> sizes;
  void* arena = nullptr;
  size_t bytes = 0;
  // device views
  int32_t* d_sizes = nullptr;
  int32_t* d_order = nullptr;
  int64_t* d_aoff = nullptr;
  int64_t* d_boff = nullptr;
  int64_t* d_info = nullptr;
  int32_t* d_flag = nullptr;
  int32_t* d_iters = nullptr;
  unsigned* d_queues = nullptr;
  double* d_A = nullptr;      // FP64 A (input copy; factored in place by the FP64 path)
  double* d_Awork = nullptr;  // FP64 work for the fallback of the mixed path
  float* d_A32 = nullptr;
  double* d_X = nullptr;
  double* d_B = nullptr;      // copy of b for the mixed path
  int32_t* d_ipiv = nullptr;
  std::vector<gblu::BatchBucket> buckets;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  int maxit = 10;
};

namespace gblu {

namespace {

template <int NT, int NB>
void configure_batch_kernels() {
  cudaFuncSetAttribute(batch_fp64_kernel<NT, NB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)batch_smem<double, NT, NB>(false));
  cudaFuncSetAttribute(batch_mixed_kernel<NT, NB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)batch_smem<float, NT, NB>(true));
}

template <int NT, int NB>
cudaError_t launch_fp64(const BatchDev& d, int ctas, gblu_batch* b, double* Awork, int only_flagged,
                        cudaStream_t s) {
  LaunchScope ls(K_BATCH, 0.0, 0.0, s);
  batch_fp64_kernel<NT, NB><<<ctas, NT, batch_smem<double, NT, NB>(false), s>>>(
      d, Awork, only_flagged ? b->d_A : nullptr, b->d_X, b->d_ipiv, only_flagged);
  return cudaGetLastError();
}

template <int NT, int NB>
cudaError_t launch_mixed(const BatchDev& d, int ctas, gblu_batch* b, cudaStream_t s) {
  LaunchScope ls(K_BATCH, 0.0, 0.0, s);
  batch_mixed_kernel<NT, NB><<<ctas, NT, batch_smem<float, NT, NB>(true), s>>>(
      d, b->d_A, b->d_A32, b->d_X, b->d_B, b->d_ipiv, b->maxit, 2.220446049250313e-16);
  return cudaGetLastError();
}

// Dispatch over the compiled (threads, panel width) variants.
cudaError_t launch_bucket(gblu_batch* b, const BatchBucket& k, bool mixed, int only_flagged,
                          double* Awork, cudaStream_t s) {
  BatchDev d;
  d.order = k.order;
  d.sizes = b->d_sizes;
  d.a_off = b->d_aoff;
  d.b_off = b->d_boff;
  d.count = k.count;
  d.queue = k.queue;
  d.info = b->d_info;
  d.flag = b->d_flag;
  d.iters = b->d_iters;
  const int ctas = std::max(1, k.ctas);
#define GBLU_BATCH_CASE(NT_, NB_)                                                   \
  if (k.nt == NT_ && k.nb == NB_)                                                   \
    return mixed ? launch_mixed<NT_, NB_>(d, ctas, b, s)                           \
                 : launch_fp64<NT_, NB_>(d, ctas, b, Awork, only_flagged, s);
  GBLU_BATCH_CASE(64, 8)
  GBLU_BATCH_CASE(128, 8)
  GBLU_BATCH_CASE(128, 16)
  GBLU_BATCH_CASE(256, 8)
  GBLU_BATCH_CASE(256, 16)
  GBLU_BATCH_CASE(512, 16)
#undef GBLU_BATCH_CASE
  return cudaErrorInvalidValue;
}

}  // namespace

void batch_configure(int /*device*/) {
  configure_batch_kernels<64, 8>();
  configure_batch_kernels<128, 8>();
  configure_batch_kernels<128, 16>();
  configure_batch_kernels<256, 8>();
  configure_batch_kernels<256, 16>();
  configure_batch_kernels<512, 16>();
}

bool batch_config_supported(int nt, int nb) {
  return (nt == 64 && nb == 8) || (nt == 128 && (nb == 8 || nb == 16)) ||
         (nt == 256 && (nb == 8 || nb == 16)) || (nt == 512 && nb == 16);
}

}  // namespace gblu

using namespace gblu;

namespace {

// Arithmetic of the batch: sum of LU flops plus 2 n^2 per solve.
double batch_flops(const gblu_batch* b) {
  double f = 0;
  for (int32_t n : b->sizes) {
    const double m = n;
    f += 2.0 * m * m * m / 3.0 - m * m / 2.0 - m / 6.0 + m * (m - 1) / 2.0 + 2.0 * m * m;
  }
  return f;
}

// Default schedule: three size buckets, CTAs sized to fill the GPU.
void default_buckets(gblu_batch* b, std::vector<BatchBucket>& out, const int32_t* edges,
                     int nedges, const int32_t* nts, const int32_t* nbs, int device) {
  const DeviceInfo& di = device_info(device);
  out.clear();
  int lo = 1;
  for (int e = 0; e <= nedges; ++e) {
    BatchBucket k;
    k.lo = lo;
    k.hi = e < nedges ? edges[e] : kBatchMaxN;
    k.nt = nts ? nts[e] : 256;
    k.nb = nbs ? nbs[e] : 16;
    k.ctas = di.num_sms * (k.nt <= 64 ? 8 : k.nt <= 128 ? 4 : (k.nt <= 256 ? 2 : 1));
    out.push_back(k);
    lo = k.hi + 1;
  }
  (void)b;
}

// The device arena of a batch holding up to `count` systems with a_total / b_total
// packed elements (sets b->arena, b->bytes and the device views).
int32_t batch_alloc(gblu_ctx* ctx, gblu_batch* b, int64_t count, int64_t a_total, int64_t b_total,
                    int32_t precision) {
  const int nbuckets_max = 8;
  size_t bytes = 0;
  auto add = [&](size_t x) { size_t o = bytes; bytes += align256(x); return o; };
  size_t o_sizes = add(count * 4 + 4), o_order = add(count * 4 + 4), o_aoff = add(count * 8 + 8),
         o_boff = add(count * 8 + 8), o_info = add(count * 8 + 8), o_flag = add(count * 4 + 4),
         o_iters = add(count * 4 + 4),
         o_q = add(2 * nbuckets_max * 4), o_A = add(a_total * 8 + 8), o_X = add(b_total * 8 + 8),
         o_ipiv = add(b_total * 4 + 4);
  size_t o_A32 = 0, o_B = 0, o_Aw = 0;
  if (precision != GBLU_FP64) {
    o_A32 = add(a_total * 4 + 4);
    o_B = add(b_total * 8 + 8);
    o_Aw = add(a_total * 8 + 8);
  }
  int32_t st = ctx_alloc(ctx, bytes, &b->arena);
  if (st) return st;
  b->bytes = bytes;
  char* base = reinterpret_cast<char*>(b->arena);
  b->d_sizes = reinterpret_cast<int32_t*>(base + o_sizes);
  b->d_order = reinterpret_cast<int32_t*>(base + o_order);
  b->d_aoff = reinterpret_cast<int64_t*>(base + o_aoff);
  b->d_boff = reinterpret_cast<int64_t*>(base + o_boff);
  b->d_info = reinterpret_cast<int64_t*>(base + o_info);
  b->d_flag = reinterpret_cast<int32_t*>(base + o_flag);
  b->d_iters = reinterpret_cast<int32_t*>(base + o_iters);
  b->d_queues = reinterpret_cast<unsigned*>(base + o_q);
  b->d_A = reinterpret_cast<double*>(base + o_A);
  b->d_X = reinterpret_cast<double*>(base + o_X);
  b->d_ipiv = reinterpret_cast<int32_t*>(base + o_ipiv);
  b->d_A32 = nullptr;
  b->d_B = nullptr;
  b->d_Awork = nullptr;
  if (precision != GBLU_FP64) {
    b->d_A32 = reinterpret_cast<float*>(base + o_A32);
    b->d_B = reinterpret_cast<double*>(base + o_B);
    b->d_Awork = reinterpret_cast<double*>(base + o_Aw);
  }
  return GBLU_OK;
}

int32_t build_graph(gblu_ctx* ctx, gblu_batch* b) {
  if (b->exec) { cudaGraphExecDestroy(b->exec); b->exec = nullptr; }
  if (b->graph) { cudaGraphDestroy(b->graph); b->graph = nullptr; }
  // order: systems sorted by decreasing n, grouped by bucket
  std::vector<int32_t> order(b->count);
  for (int64_t i = 0; i < b->count; ++i) order[i] = (int32_t)i;
  std::stable_sort(order.begin(), order.end(),
                   [&](int32_t x, int32_t y) { return b->sizes[x] > b->sizes[y]; });
  std::vector<int32_t> grouped;
  grouped.reserve(b->count);
  int64_t pos = 0;
  std::vector<int64_t> starts;
  for (auto& k : b->buckets) {
    starts.push_back(pos);
    int c = 0;
    for (int32_t s : order)
      if (b->sizes[s] >= k.lo && b->sizes[s] <= k.hi) { grouped.push_back(s); ++c; }
    k.count = c;
    pos += c;
  }
  GBLU_CK(ctx, cudaMemcpyAsync(b->d_order, grouped.data(), grouped.size() * sizeof(int32_t),
                               cudaMemcpyHostToDevice, ctx->stream), "batch order");
  for (size_t i = 0; i < b->buckets.size(); ++i) {
    b->buckets[i].order = b->d_order + starts[i];
    b->buckets[i].queue = b->d_queues + i;
  }
  GBLU_CK(ctx, cudaStreamSynchronize(ctx->stream), "batch order");
  // capture: reset queues, one persistent kernel per bucket, then (mixed) the FP64 pass
  // over flagged systems.  Buckets run back to back on the stream; each fills the GPU.
  cudaStream_t s = ctx->stream;
  GBLU_CK(ctx, cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal), "begin capture");
  cudaError_t e = cudaMemsetAsync(b->d_queues, 0, 2 * b->buckets.size() * sizeof(unsigned), s);
  const bool mixed = b->precision != GBLU_FP64;
  for (auto& k : b->buckets)
    if (e == cudaSuccess && k.count > 0) e = launch_bucket(b, k, mixed, 0, b->d_A, s);
  if (mixed) {
    for (auto& k : b->buckets) {
      if (e != cudaSuccess || k.count == 0) continue;
      BatchBucket k2 = k;
      k2.queue = b->d_queues + b->buckets.size() + (&k - &b->buckets[0]);
      // fallback: each flagged system is copied from A64 into the work area and
      // factored there (A64 stays intact)
      e = launch_bucket(b, k2, false, 1, b->d_Awork, s);
    }
  }
  cudaGraph_t g = nullptr;
  cudaError_t e2 = cudaStreamEndCapture(s, &g);
  if (e != cudaSuccess) { if (g) cudaGraphDestroy(g); return cuda_fail(ctx, e, "capturing batch"); }
  if (e2 != cudaSuccess) return cuda_fail(ctx, e2, "end capture");
  b->graph = g;
  GBLU_CK(ctx, cudaGraphInstantiate(&b->exec, g, 0), "instantiating batch graph");
  return GBLU_OK;
}

}  // namespace

extern "C" {

int32_t gblu_batch_create(gblu_ctx* ctx, int64_t count, const int64_t* sizes, int32_t precision,
                          gblu_batch** out) {
  if (!ctx || !out || (count > 0 && !sizes)) return fail(ctx, GBLU_EINVAL, "gblu_batch_create: NULL argument");
  *out = nullptr;
  if (count < 0 || count > INT32_MAX) return fail(ctx, GBLU_EINVAL, "gblu_batch_create: bad count");
  if (precision != GBLU_FP64 && precision != GBLU_FP32)
    return fail(ctx, GBLU_EUNSUPPORTED, "gblu_batch_create: precision must be GBLU_FP64 or GBLU_FP32");
  for (int64_t i = 0; i < count; ++i)
    if (sizes[i] < 1 || sizes[i] > kBatchMaxN)
      return fail(ctx, GBLU_EUNSUPPORTED, "gblu_batch_create: system %lld has n = %lld (1..%d supported)",
                  (long long)i, (long long)sizes[i], kBatchMaxN);
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  DeviceGuard g(ctx->device);
  {
    static std::mutex mu;
    static bool done[64] = {false};
    std::lock_guard<std::mutex> l2(mu);
    if (ctx->device < 64 && !done[ctx->device]) { batch_configure(ctx->device); done[ctx->device] = true; }
  }
  gblu_batch* b = new gblu_batch();
  b->count = count;
  b->precision = precision;
  b->sizes.resize(count);
  std::vector<int64_t> aoff(count), boff(count);
  for (int64_t i = 0; i < count; ++i) {
    b->sizes[i] = (int32_t)sizes[i];
    aoff[i] = b->a_total;
    boff[i] = b->b_total;
    b->a_total += sizes[i] * sizes[i];
    b->b_total += sizes[i];
  }
  int32_t st = batch_alloc(ctx, b, count, b->a_total, b->b_total, precision);
  if (st) { delete b; return st; }
  const size_t bytes = b->bytes;
  cudaError_t e = cudaMemsetAsync(b->arena, 0, bytes, ctx->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(b->d_sizes, b->sizes.data(), count * 4, cudaMemcpyHostToDevice, ctx->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(b->d_aoff, aoff.data(), count * 8, cudaMemcpyHostToDevice, ctx->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(b->d_boff, boff.data(), count * 8, cudaMemcpyHostToDevice, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) {
    ctx_free(ctx, b->arena, bytes);
    delete b;
    return cuda_fail(ctx, e, "gblu_batch_create");
  }
  // default schedules: the autotuner's choice for 20,000 systems with n
  // uniform in [8, 256] (128-thread CTAs with 8-column panels throughout)
  if (precision == GBLU_FP64) {
    const int32_t edges[2] = {32, 96};
    const int32_t nts[3] = {128, 128, 128};
    const int32_t nbs[3] = {8, 8, 8};
    default_buckets(b, b->buckets, edges, 2, nts, nbs, ctx->device);
  } else {
    const int32_t edges[3] = {48, 96, 160};
    const int32_t nts[4] = {128, 128, 128, 128};
    const int32_t nbs[4] = {8, 8, 8, 8};
    default_buckets(b, b->buckets, edges, 3, nts, nbs, ctx->device);
  }
  st = count > 0 ? build_graph(ctx, b) : GBLU_OK;
  if (st) {
    ctx_free(ctx, b->arena, bytes);
    delete b;
    return st;
  }
  *out = b;
  return GBLU_OK;
}

int32_t gblu_batch_schedule(gblu_ctx* ctx, gblu_batch* b, int32_t nbuckets, const int32_t* upper,
                            const int32_t* threads, const int32_t* panel, const int32_t* ctas) {
  if (!ctx || !b) return fail(ctx, GBLU_EINVAL, "gblu_batch_schedule: NULL argument");
  if (nbuckets < 1 || nbuckets > 8 || !upper || !threads || !panel)
    return fail(ctx, GBLU_EINVAL, "gblu_batch_schedule: 1..8 buckets with upper/threads/panel arrays");
  int lo = 1;
  for (int i = 0; i < nbuckets; ++i) {
    if (upper[i] < lo || (i == nbuckets - 1 && upper[i] != kBatchMaxN) || upper[i] > kBatchMaxN)
      return fail(ctx, GBLU_EINVAL, "gblu_batch_schedule: bucket edges must increase and end at %d", kBatchMaxN);
    if (!batch_config_supported(threads[i], panel[i]))
      return fail(ctx, GBLU_EUNSUPPORTED, "gblu_batch_schedule: (threads %d, panel %d) not compiled",
                  threads[i], panel[i]);
    lo = upper[i] + 1;
  }
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  DeviceGuard g(ctx->device);
  const DeviceInfo& di = device_info(ctx->device);
  b->buckets.clear();
  lo = 1;
  for (int i = 0; i < nbuckets; ++i) {
    BatchBucket k;
    k.lo = lo;
    k.hi = upper[i];
    k.nt = threads[i];
    k.nb = panel[i];
    k.ctas = (ctas && ctas[i] > 0) ? ctas[i] : di.num_sms * (k.nt <= 64 ? 8 : k.nt <= 128 ? 4 : (k.nt <= 256 ? 2 : 1));
    b->buckets.push_back(k);
    lo = upper[i] + 1;
  }
  return b->count > 0 ? build_graph(ctx, b) : GBLU_OK;
}

int32_t gblu_batch_solve(gblu_ctx* ctx, gblu_batch* b, const double* A, double* B, int32_t loc,
                         int64_t* info_host) {
  if (!ctx || !b) return fail(ctx, GBLU_EINVAL, "gblu_batch_solve: NULL argument");
  if (b->count == 0) return GBLU_OK;
  if (!A || !B) return fail(ctx, GBLU_EINVAL, "gblu_batch_solve: NULL A or B");
  if (loc != GBLU_HOST && loc != GBLU_DEVICE) return fail(ctx, GBLU_EINVAL, "gblu_batch_solve: bad loc");
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  DeviceGuard g(ctx->device);
  ActiveProfiler ap(&ctx->prof);
  cudaStream_t s = ctx->stream;
  const cudaMemcpyKind kin = loc == GBLU_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice;
  const cudaMemcpyKind kout = loc == GBLU_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
  GBLU_CK(ctx, cudaMemcpyAsync(b->d_A, A, b->a_total * 8, kin, s), "batch A");
  GBLU_CK(ctx, cudaMemcpyAsync(b->d_X, B, b->b_total * 8, kin, s), "batch B");
  if (b->precision != GBLU_FP64) {
    GBLU_CK(ctx, cudaMemcpyAsync(b->d_B, b->d_X, b->b_total * 8, cudaMemcpyDeviceToDevice, s), "batch B copy");
  }
  {
    // one graph launch runs every persistent kernel of the schedule; the scope
    // times the whole graph and the counters record each kernel it holds
    int nk = 0;
    for (auto& k : b->buckets) nk += k.count > 0 ? (b->precision != GBLU_FP64 ? 2 : 1) : 0;
    LaunchScope ls(K_BATCH, batch_flops(b), (double)b->a_total * 8.0 * (b->precision != GBLU_FP64 ? 1.5 : 2.0), s);
    if (tl_profiler && nk > 1) {
      tl_profiler->launches += nk - 1;
      tl_profiler->count[K_BATCH] += nk - 1;
    }
    GBLU_CK(ctx, cudaGraphLaunch(b->exec, s), "batch graph launch");
  }
  GBLU_CK(ctx, cudaMemcpyAsync(B, b->d_X, b->b_total * 8, kout, s), "batch X");
  if (info_host)
    GBLU_CK(ctx, cudaMemcpyAsync(info_host, b->d_info, b->count * 8, cudaMemcpyDeviceToHost, s), "batch info");
  GBLU_CK(ctx, cudaStreamSynchronize(s), "batch solve");
  return GBLU_OK;
}

int32_t gblu_batch_iterations(gblu_ctx* ctx, gblu_batch* b, int32_t* iterations_host) {
  if (!ctx || !b || (b->count > 0 && !iterations_host))
    return fail(ctx, GBLU_EINVAL, "gblu_batch_iterations: NULL argument");
  if (b->count == 0) return GBLU_OK;
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  DeviceGuard g(ctx->device);
  GBLU_CK(ctx, cudaMemcpyAsync(iterations_host, b->d_iters, b->count * 4, cudaMemcpyDeviceToHost, ctx->stream),
          "batch iterations");
  GBLU_CK(ctx, cudaStreamSynchronize(ctx->stream), "batch iterations");
  return GBLU_OK;
}

int32_t gblu_batch_destroy(gblu_ctx* ctx, gblu_batch* b) {
  if (!b) return GBLU_OK;
  if (!ctx) return fail(ctx, GBLU_EINVAL, "gblu_batch_destroy: NULL ctx");
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  DeviceGuard g(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  ctx_free(ctx, b->arena, b->bytes);
  delete b;
  return GBLU_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Lane: batches whose system list changes at every call (the serving loop's
// small-system lane).  One bucket [1, 256] of 128-thread CTAs with 8-column
// panels, direct launches instead of a captured graph, device arena and
// pinned staging grown to the largest call and then reused.

namespace gblu {

struct BatchLane {
  gblu_batch b;
  int64_t cap_count = 0, cap_a = 0, cap_b = 0;
  int32_t precision = -1;
  double* hA = nullptr;  // pinned: packed A
  double* hX = nullptr;  // pinned: packed b in, x out
  char* hmeta = nullptr; // pinned: sizes, order, a_off, b_off, info, iters
  size_t hA_cap = 0, hX_cap = 0, hmeta_cap = 0;
};

BatchLane* batch_lane_create() { return new (std::nothrow) BatchLane(); }

void batch_lane_destroy(gblu_ctx* ctx, BatchLane* lane) {
  if (!lane) return;
  if (ctx) {
    DeviceGuard g(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    if (lane->b.arena) ctx_free(ctx, lane->b.arena, lane->b.bytes);
  }
  if (lane->hA) cudaFreeHost(lane->hA);
  if (lane->hX) cudaFreeHost(lane->hX);
  if (lane->hmeta) cudaFreeHost(lane->hmeta);
  delete lane;
}

namespace {
int32_t grow_pinned(gblu_ctx* ctx, void** p, size_t* cap, size_t need) {
  if (*cap >= need) return GBLU_OK;
  if (*p) cudaFreeHost(*p);
  *p = nullptr;
  *cap = 0;
  const size_t sz = std::max<size_t>(need + need / 2, 4096);
  GBLU_CK(ctx, cudaMallocHost(p, sz), "pinned lane staging");
  *cap = sz;
  return GBLU_OK;
}
}  // namespace

int32_t batch_lane_solve(gblu_ctx* ctx, BatchLane* lane, int32_t precision, int count, const int32_t* sizes,
                         const double* const* A, const double* const* bvec, double* const* x, int64_t* info,
                         int32_t* iters) {
  if (count <= 0) return GBLU_OK;
  DeviceGuard g(ctx->device);
  {
    static std::mutex mu;
    static bool done[64] = {false};
    std::lock_guard<std::mutex> l2(mu);
    if (ctx->device < 64 && !done[ctx->device]) { batch_configure(ctx->device); done[ctx->device] = true; }
  }
  cudaStream_t s = ctx->stream;
  int64_t a_total = 0, b_total = 0;
  for (int i = 0; i < count; ++i) {
    if (sizes[i] < 1 || sizes[i] > kBatchMaxN)
      return fail(ctx, GBLU_EUNSUPPORTED, "batch lane: n = %d outside 1..%d", sizes[i], kBatchMaxN);
    a_total += (int64_t)sizes[i] * sizes[i];
    b_total += sizes[i];
  }
  const bool mixed = precision != GBLU_FP64;
  gblu_batch& b = lane->b;
  if (lane->cap_count < count || lane->cap_a < a_total || lane->cap_b < b_total ||
      (mixed && lane->precision == GBLU_FP64) || lane->precision < 0) {
    GBLU_CK(ctx, cudaStreamSynchronize(s), "batch lane");
    if (b.arena) ctx_free(ctx, b.arena, b.bytes);
    b.arena = nullptr;
    const int64_t cc = std::max<int64_t>(count, 2 * lane->cap_count);
    const int64_t ca = std::max<int64_t>(a_total, 2 * lane->cap_a);
    const int64_t cb = std::max<int64_t>(b_total, 2 * lane->cap_b);
    const int32_t prec = mixed ? GBLU_FP32 : GBLU_FP64;
    int32_t st = batch_alloc(ctx, &b, cc, ca, cb, prec);
    if (st) { lane->cap_count = lane->cap_a = lane->cap_b = 0; lane->precision = -1; return st; }
    GBLU_CK(ctx, cudaMemsetAsync(b.arena, 0, b.bytes, s), "batch lane clear");
    lane->cap_count = cc;
    lane->cap_a = ca;
    lane->cap_b = cb;
    lane->precision = prec;
  }
  const size_t meta = (size_t)count * (4 + 4 + 8 + 8 + 8 + 4) + 64;
  int32_t st = grow_pinned(ctx, reinterpret_cast<void**>(&lane->hA), &lane->hA_cap, (size_t)a_total * 8);
  if (!st) st = grow_pinned(ctx, reinterpret_cast<void**>(&lane->hX), &lane->hX_cap, (size_t)b_total * 8);
  if (!st) st = grow_pinned(ctx, reinterpret_cast<void**>(&lane->hmeta), &lane->hmeta_cap, meta);
  if (st) return st;
  int64_t* h_aoff = reinterpret_cast<int64_t*>(lane->hmeta);
  int64_t* h_boff = h_aoff + count;
  int64_t* h_info = h_boff + count;
  int32_t* h_sizes = reinterpret_cast<int32_t*>(h_info + count);
  int32_t* h_order = h_sizes + count;
  int32_t* h_iters = h_order + count;
  int64_t ao = 0, bo = 0;
  for (int i = 0; i < count; ++i) {
    const int n = sizes[i];
    h_sizes[i] = n;
    h_aoff[i] = ao;
    h_boff[i] = bo;
    std::memcpy(lane->hA + ao, A[i], (size_t)n * n * sizeof(double));
    std::memcpy(lane->hX + bo, bvec[i], (size_t)n * sizeof(double));
    ao += (int64_t)n * n;
    bo += n;
    h_order[i] = i;
  }
  std::stable_sort(h_order, h_order + count, [&](int32_t p, int32_t q) { return h_sizes[p] > h_sizes[q]; });
  GBLU_CK(ctx, cudaMemcpyAsync(b.d_sizes, h_sizes, count * 4, cudaMemcpyHostToDevice, s), "lane sizes");
  GBLU_CK(ctx, cudaMemcpyAsync(b.d_order, h_order, count * 4, cudaMemcpyHostToDevice, s), "lane order");
  GBLU_CK(ctx, cudaMemcpyAsync(b.d_aoff, h_aoff, count * 8, cudaMemcpyHostToDevice, s), "lane offsets");
  GBLU_CK(ctx, cudaMemcpyAsync(b.d_boff, h_boff, count * 8, cudaMemcpyHostToDevice, s), "lane offsets");
  GBLU_CK(ctx, cudaMemcpyAsync(b.d_A, lane->hA, a_total * 8, cudaMemcpyHostToDevice, s), "lane A");
  GBLU_CK(ctx, cudaMemcpyAsync(b.d_X, lane->hX, b_total * 8, cudaMemcpyHostToDevice, s), "lane b");
  if (mixed)
    GBLU_CK(ctx, cudaMemcpyAsync(b.d_B, b.d_X, b_total * 8, cudaMemcpyDeviceToDevice, s), "lane b copy");
  GBLU_CK(ctx, cudaMemsetAsync(b.d_queues, 0, 2 * sizeof(unsigned), s), "lane queues");
  GBLU_CK(ctx, cudaMemsetAsync(b.d_flag, 0, count * 4, s), "lane flags");
  GBLU_CK(ctx, cudaMemsetAsync(b.d_iters, 0, count * 4, s), "lane iterations");
  b.precision = mixed ? GBLU_FP32 : GBLU_FP64;
  b.count = count;
  BatchDev d;
  d.order = b.d_order;
  d.sizes = b.d_sizes;
  d.a_off = b.d_aoff;
  d.b_off = b.d_boff;
  d.count = count;
  d.queue = b.d_queues;
  d.info = b.d_info;
  d.flag = b.d_flag;
  d.iters = b.d_iters;
  const int ctas = std::max(1, std::min(count, device_info(ctx->device).num_sms * 4));
  cudaError_t e;
  if (!mixed) {
    e = launch_fp64<128, 8>(d, ctas, &b, b.d_A, 0, s);
  } else {
    e = launch_mixed<128, 8>(d, ctas, &b, s);
    if (e == cudaSuccess) {
      d.queue = b.d_queues + 1;  // FP64 re-solve of the systems refinement flagged
      e = launch_fp64<128, 8>(d, ctas, &b, b.d_Awork, 1, s);
    }
  }
  GBLU_CK(ctx, e, "batch lane launch");
  GBLU_CK(ctx, cudaMemcpyAsync(lane->hX, b.d_X, b_total * 8, cudaMemcpyDeviceToHost, s), "lane x");
  GBLU_CK(ctx, cudaMemcpyAsync(h_info, b.d_info, count * 8, cudaMemcpyDeviceToHost, s), "lane info");
  GBLU_CK(ctx, cudaMemcpyAsync(h_iters, b.d_iters, count * 4, cudaMemcpyDeviceToHost, s), "lane iterations");
  GBLU_CK(ctx, cudaStreamSynchronize(s), "batch lane");
  for (int i = 0; i < count; ++i) {
    std::memcpy(x[i], lane->hX + h_boff[i], (size_t)sizes[i] * sizeof(double));
    if (info) info[i] = h_info[i];
    if (iters) iters[i] = h_iters[i];
  }
  return GBLU_OK;
}

}  // namespace gblu
