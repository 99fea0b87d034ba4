// Tournament-pivoting panel for the low-precision getrf (BF16 / FP16
// trailing updates): the panel of a 32-column leaf picks its pivots in two
// local factorizations instead of one cross-CTA exchange per column.
//
//   1. tslu_local_kernel: the panel rows are cut into P chunks of R rows; one
//      CTA per chunk runs getf2 with partial pivoting on its chunk in shared
//      memory and nominates the chunk's w pivot rows.
//   2. tslu_tree_kernel: one CTA runs getf2 with partial pivoting on the P*w
//      nominated rows (their original values) and keeps the first w: the
//      panel's pivot rows in order, and the packed L11 \ U11 of those rows.
//   3. tslu_moves_kernel: the pivot order as the LAPACK interchange sequence
//      ipiv[c0 .. c0+w) and the at most 2w row moves it implies, with the
//      moved rows' panel values staged.
//   4. tslu_apply_kernel: rows c0 .. c0+w-1 receive L11 \ U11; every other
//      panel row receives l = a U11^{-1} (a: its value after the moves).
// The interchanges reach the other columns through the leaf's laswp, as for
// the partial-pivoting panels.
//
// This is communication-avoiding LU's tall-skinny panel (Grigori, Demmel and
// Xiang, SIAM J. Matrix Anal. Appl. 32(4), 2011), one reduction level.  Its
// pivots differ from partial pivoting's, so the factors are not the
// reference's; they serve only as the preconditioner of FP64 refinement,
// whose result meets the FP64 backward-error bound (and whose pivot-growth
// check and FP64 fallback guard the rare matrix where they are poor).
#include <cuda_runtime.h>

#include <algorithm>

#include "device_util.cuh"
#include "gblu_internal.h"
#include "objects.h"
#include "profile.h"

namespace gblu {

namespace {

constexpr int kTsW = 32;          // panel width
constexpr int kTsMaxCand = 1024;  // nominated rows the tree factors at once
constexpr int kTsLocalThreads = 512;
constexpr int kTsTreeThreads = 1024;

// |a| as an ordered integer key; NaN is never a pivot (key -1).
__device__ __forceinline__ int piv_key(float a) {
  const float v = fabsf(a);
  return isnan(v) ? -1 : __float_as_int(v);
}

// Block-wide (key max, then smallest index) over one candidate per thread.
// Returns the winning index (or -1 when no key >= 0) in every thread.
template <int NT>
__device__ __forceinline__ int block_argmax(int key, int idx, int* s_key, int* s_idx) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int off = 16; off; off >>= 1) {
    const int ok = __shfl_xor_sync(0xffffffffu, key, off);
    const int oi = __shfl_xor_sync(0xffffffffu, idx, off);
    if (ok > key || (ok == key && oi < idx)) { key = ok; idx = oi; }
  }
  if (lane == 0) { s_key[warp] = key; s_idx[warp] = idx; }
  __syncthreads();
  if (warp == 0) {
    key = lane < NT / 32 ? s_key[lane] : -1;
    idx = lane < NT / 32 ? s_idx[lane] : 0x7fffffff;
#pragma unroll
    for (int off = 16; off; off >>= 1) {
      const int ok = __shfl_xor_sync(0xffffffffu, key, off);
      const int oi = __shfl_xor_sync(0xffffffffu, idx, off);
      if (ok > key || (ok == key && oi < idx)) { key = ok; idx = oi; }
    }
    if (lane == 0) s_idx[32] = key >= 0 ? idx : -1;
  }
  __syncthreads();
  const int r = s_idx[32];
  __syncthreads();  // s_key / s_idx are reused by the next call
  return r;
}

// getf2 with partial pivoting on rows [0, nr) x columns [0, w) of the shared
// matrix s (row stride kTsW + 1), rows tid, tid + NT, ...; row indices in sidx
// follow the swaps (rows whose index is negative are padding, never pivots).
// Returns the first column with no usable pivot (-1: none).
template <int NT, int RPT>
__device__ int smem_getf2(float* s, int* sidx, int nr, int w, int* s_key, int* s_idx) {
  constexpr int LD = kTsW + 1;
  int zero_col = -1;
  for (int k = 0; k < w && k < nr; ++k) {
    int key = -1, idx = 0x7fffffff;
#pragma unroll
    for (int t = 0; t < RPT; ++t) {
      const int i = threadIdx.x + NT * t;
      if (i >= k && i < nr && sidx[i] >= 0) {
        const int kk = piv_key(s[i * LD + k]);
        if (kk > key || (kk == key && i < idx)) { key = kk; idx = i; }
      }
    }
    int piv = block_argmax<NT>(key, idx, s_key, s_idx);
    const bool usable = piv >= 0 && s[piv * LD + k] != 0.f;
    if (!usable) {
      if (zero_col < 0) zero_col = k;
      piv = k;
    }
    if (piv != k && threadIdx.x < w) {  // interchange rows k and piv
      const int j = threadIdx.x;
      const float t = s[k * LD + j];
      s[k * LD + j] = s[piv * LD + j];
      s[piv * LD + j] = t;
      if (j == 0) {
        const int ti = sidx[k];
        sidx[k] = sidx[piv];
        sidx[piv] = ti;
      }
    }
    __syncthreads();
    if (usable) {
      const float rp = 1.0f / s[k * LD + k];
#pragma unroll
      for (int t = 0; t < RPT; ++t) {
        const int i = threadIdx.x + NT * t;
        if (i > k && i < nr) {
          float* row = s + i * LD;
          const float l = row[k] * rp;
          row[k] = l;
          for (int j = k + 1; j < w; ++j) row[j] = fmaf(-l, s[k * LD + j], row[j]);
        }
      }
    }
    __syncthreads();
  }
  return zero_col;
}

// 1. one CTA per chunk of R rows (R <= RPT * NT): nominate the chunk's pivot rows.
template <int RPT>
__global__ void __launch_bounds__(kTsLocalThreads)
tslu_local_kernel(const float* __restrict__ A, int64_t lda, int64_t m, int64_t c0, int w, int R,
                  int32_t* __restrict__ cand_rows, float* __restrict__ cand_vals) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float* s = reinterpret_cast<float*>(smem_raw);
  int* sidx = reinterpret_cast<int*>(s + (size_t)R * (kTsW + 1));
  __shared__ int s_key[32], s_idx[33];
  const int p = blockIdx.x;
  const int64_t r0 = c0 + (int64_t)p * R;
  const int nr = (int)min((int64_t)R, m - r0);
  for (int j = 0; j < w; ++j)
    for (int i = threadIdx.x; i < nr; i += kTsLocalThreads) s[i * (kTsW + 1) + j] = A[(r0 + i) + (c0 + j) * lda];
  for (int i = threadIdx.x; i < nr; i += kTsLocalThreads) sidx[i] = (int)(r0 + i);
  __syncthreads();
  smem_getf2<kTsLocalThreads, RPT>(s, sidx, nr, w, s_key, s_idx);
  // nominated rows and their original panel values
  const int cw = min(w, nr);
  for (int idx = threadIdx.x; idx < kTsW * kTsW; idx += kTsLocalThreads) {
    const int k = idx / kTsW, j = idx % kTsW;
    float v = 0.f;
    if (k < cw && j < w) v = A[(int64_t)sidx[k] + (c0 + j) * lda];
    cand_vals[((size_t)p * kTsW + k) * kTsW + j] = v;
  }
  if (threadIdx.x < kTsW) cand_rows[p * kTsW + threadIdx.x] = threadIdx.x < cw ? sidx[threadIdx.x] : -1;
}

// 2. one CTA: the panel's pivot rows from the nominated ones, and L11 \ U11.
__global__ void __launch_bounds__(kTsTreeThreads)
tslu_tree_kernel(int ncand, int w, int64_t c0, const int32_t* __restrict__ cand_rows,
                 const float* __restrict__ cand_vals, int32_t* __restrict__ piv_rows,
                 float* __restrict__ lu11, int64_t* __restrict__ info) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float* s = reinterpret_cast<float*>(smem_raw);
  int* sidx = reinterpret_cast<int*>(s + (size_t)kTsMaxCand * (kTsW + 1));
  __shared__ int s_key[32], s_idx[33];
  for (int idx = threadIdx.x; idx < ncand * kTsW; idx += kTsTreeThreads) {
    const int k = idx / kTsW, j = idx % kTsW;
    s[k * (kTsW + 1) + j] = cand_vals[idx];
  }
  for (int i = threadIdx.x; i < ncand; i += kTsTreeThreads) sidx[i] = cand_rows[i];
  __syncthreads();
  const int zc = smem_getf2<kTsTreeThreads, 1>(s, sidx, ncand, w, s_key, s_idx);
  if (threadIdx.x < kTsW) piv_rows[threadIdx.x] = threadIdx.x < w ? sidx[threadIdx.x] : -1;
  for (int idx = threadIdx.x; idx < kTsW * kTsW; idx += kTsTreeThreads) {
    const int k = idx / kTsW, j = idx % kTsW;
    lu11[idx] = (k < w && j < w) ? s[k * (kTsW + 1) + j] : 0.f;
  }
  if (threadIdx.x == 0 && zc >= 0)
    atomicCAS(reinterpret_cast<unsigned long long*>(info), 0ull, (unsigned long long)(c0 + zc + 1));
}

// 3. one thread: ipiv[c0 + k] (1-based) from the pivot rows, and the row moves
// "position dst receives original row src"; all threads then stage the moved
// rows' panel values.
__global__ void tslu_moves_kernel(const float* __restrict__ A, int64_t lda, int64_t c0, int w,
                                  const int32_t* __restrict__ piv_rows, int64_t* __restrict__ ipiv,
                                  int32_t* __restrict__ moves, float* __restrict__ staged,
                                  DevScratch* __restrict__ scr) {
  __shared__ int pos_s[2 * kTsW], row_s[2 * kTsW];  // touched positions and the row each holds
  __shared__ int cnt_s;
  if (threadIdx.x == 0) {
    int cnt = 0;
    bool bad = false;
    for (int k = 0; k < w; ++k) {
      const int g = piv_rows[k];
      if (g < c0) { bad = true; break; }
      // where row g sits now: a touched position holding it, or its own
      int q = g;
      for (int t = 0; t < cnt; ++t)
        if (row_s[t] == g) { q = pos_s[t]; break; }
      const int target = (int)(c0 + k);
      ipiv[target] = (int64_t)q + 1;
      if (q == target) continue;
      int tt = -1, tq = -1;
      for (int t = 0; t < cnt; ++t) {
        if (pos_s[t] == target) tt = t;
        if (pos_s[t] == q) tq = t;
      }
      const int row_at_target = tt >= 0 ? row_s[tt] : target;
      if (tt < 0) { tt = cnt++; pos_s[tt] = target; }
      row_s[tt] = g;
      if (tq < 0) { tq = cnt++; pos_s[tq] = q; }
      row_s[tq] = row_at_target;
    }
    if (bad) {
      atomicCAS(&scr->error, 0, (int)DEV_BAD_PIVOT_INDEX);
      cnt = 0;
    }
    cnt_s = cnt;
  }
  __syncthreads();
  const int cnt = cnt_s;
  for (int t = threadIdx.x; t < 2 * kTsW; t += blockDim.x) {
    moves[1 + 2 * t] = t < cnt ? pos_s[t] : -1;
    moves[2 + 2 * t] = t < cnt ? row_s[t] : -1;
  }
  if (threadIdx.x == 0) moves[0] = cnt;
  for (int idx = threadIdx.x; idx < cnt * kTsW; idx += blockDim.x) {
    const int t = idx / kTsW, j = idx % kTsW;
    staged[idx] = j < w ? A[(int64_t)row_s[t] + (c0 + j) * lda] : 0.f;
  }
}

// 4. every panel row: L11 \ U11 on top, l = a U11^{-1} below.
__global__ void __launch_bounds__(256)
tslu_apply_kernel(float* __restrict__ A, int64_t lda, int64_t m, int64_t c0, int w,
                  const float* __restrict__ lu11, const int32_t* __restrict__ moves,
                  const float* __restrict__ staged) {
  __shared__ float su[kTsW][kTsW + 1];
  __shared__ float rdiag[kTsW];
  __shared__ int mdst[2 * kTsW];
  __shared__ int ncnt;
  for (int idx = threadIdx.x; idx < kTsW * kTsW; idx += blockDim.x) su[idx / kTsW][idx % kTsW] = lu11[idx];
  if (threadIdx.x == 0) ncnt = moves[0];
  __syncthreads();
  for (int t = threadIdx.x; t < 2 * kTsW; t += blockDim.x) mdst[t] = t < ncnt ? moves[1 + 2 * t] : -1;
  if (threadIdx.x < kTsW) rdiag[threadIdx.x] = 1.0f / su[threadIdx.x][threadIdx.x];
  __syncthreads();
  const int64_t p = c0 + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= m) return;
  if (p < c0 + w) {
    const int k = (int)(p - c0);
    for (int j = 0; j < w; ++j) A[p + (c0 + j) * lda] = su[k][j];
    return;
  }
  int mi = -1;
  for (int t = 0; t < ncnt; ++t)
    if (mdst[t] == p) { mi = t; break; }
  float x[kTsW];
#pragma unroll
  for (int j = 0; j < kTsW; ++j)
    x[j] = j < w ? (mi >= 0 ? staged[mi * kTsW + j] : A[p + (c0 + j) * lda]) : 0.f;
#pragma unroll
  for (int j = 0; j < kTsW; ++j) {
    if (j >= w) break;
    float sacc = x[j];
#pragma unroll
    for (int i = 0; i < j; ++i) sacc = fmaf(-x[i], su[i][j], sacc);
    x[j] = sacc * rdiag[j];
  }
#pragma unroll
  for (int j = 0; j < kTsW; ++j)
    if (j < w) A[p + (c0 + j) * lda] = x[j];
}

size_t local_smem(int R) { return (size_t)R * (kTsW + 1) * sizeof(float) + (size_t)R * sizeof(int); }
size_t tree_smem() { return (size_t)kTsMaxCand * (kTsW + 1) * sizeof(float) + kTsMaxCand * sizeof(int); }

}  // namespace

size_t tslu_work_bytes() {
  return align256(kTsMaxCand * sizeof(int32_t)) + align256((size_t)kTsMaxCand * kTsW * sizeof(float)) +
         align256(kTsW * sizeof(int32_t)) + align256(kTsW * kTsW * sizeof(float)) +
         align256((1 + 4 * kTsW) * sizeof(int32_t)) + align256(2 * kTsW * kTsW * sizeof(float));
}

bool tslu_fits(int64_t rows, int w) {
  // at most kTsMaxCand / kTsW chunks of at most 2 * kTsLocalThreads rows
  return w <= kTsW && rows > 0 && rows <= (int64_t)(kTsMaxCand / kTsW) * 2 * kTsLocalThreads;
}

void tslu_configure(int /*device*/) {
  cudaFuncSetAttribute(tslu_local_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)local_smem(512));
  cudaFuncSetAttribute(tslu_local_kernel<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)local_smem(1024));
  cudaFuncSetAttribute(tslu_tree_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tree_smem());
}

cudaError_t tslu_panel_launch(float* A, int64_t lda, int64_t m, int64_t c0, int w, int64_t* ipiv,
                              int64_t* info, void* work, DevScratch* scr, cudaStream_t s) {
  const int64_t M = m - c0;
  if (!tslu_fits(M, w)) return cudaErrorInvalidValue;
  char* c = reinterpret_cast<char*>(work);
  int32_t* cand_rows = reinterpret_cast<int32_t*>(c);
  c += align256(kTsMaxCand * sizeof(int32_t));
  float* cand_vals = reinterpret_cast<float*>(c);
  c += align256((size_t)kTsMaxCand * kTsW * sizeof(float));
  int32_t* piv_rows = reinterpret_cast<int32_t*>(c);
  c += align256(kTsW * sizeof(int32_t));
  float* lu11 = reinterpret_cast<float*>(c);
  c += align256(kTsW * kTsW * sizeof(float));
  int32_t* moves = reinterpret_cast<int32_t*>(c);
  c += align256((1 + 4 * kTsW) * sizeof(int32_t));
  float* staged = reinterpret_cast<float*>(c);
  // chunks: at most kTsMaxCand / kTsW of them, of at least 512 rows
  const int pmax = kTsMaxCand / kTsW;
  int R = 512;
  if ((M + R - 1) / R > pmax) R = (int)(((M + pmax - 1) / pmax + 31) / 32 * 32);
  const int P = (int)((M + R - 1) / R);
  double fl = 0;
  for (int k = 0; k < w; ++k) fl += (double)(M - k - 1) * (1.0 + 2.0 * (w - k - 1));
  {
    LaunchScope ls(K_PANEL, fl, 2.0 * M * w * sizeof(float), s);
    if (R <= 512)
      tslu_local_kernel<1><<<P, kTsLocalThreads, local_smem(R), s>>>(A, lda, m, c0, w, R, cand_rows, cand_vals);
    else
      tslu_local_kernel<2><<<P, kTsLocalThreads, local_smem(R), s>>>(A, lda, m, c0, w, R, cand_rows, cand_vals);
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  {
    LaunchScope ls(K_PANEL, 0.0, (double)P * kTsW * kTsW * sizeof(float), s);
    tslu_tree_kernel<<<1, kTsTreeThreads, tree_smem(), s>>>(P * kTsW, w, c0, cand_rows, cand_vals, piv_rows, lu11,
                                                            info);
  }
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  {
    LaunchScope ls(K_PANEL, 0.0, 0.0, s);
    tslu_moves_kernel<<<1, 64, 0, s>>>(A, lda, c0, w, piv_rows, ipiv, moves, staged, scr);
  }
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  LaunchScope ls(K_PANEL, (double)M * w * w, 2.0 * M * w * sizeof(float), s);
  tslu_apply_kernel<<<(unsigned)((M + 255) / 256), 256, 0, s>>>(A, lda, m, c0, w, lu11, moves, staged);
  return cudaGetLastError();
}

}  // namespace gblu
