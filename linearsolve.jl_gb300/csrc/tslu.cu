// Tournament-pivoting panel for the low-precision getrf (BF16 / FP16
// trailing updates): the panel of a 32-column leaf picks its pivots in two
// local factorizations instead of one cross-CTA exchange per column.
//
//   1. tslu_select_kernel, every CTA: the panel rows are cut into P <= 32
//      chunks of R rows; one CTA per chunk runs getf2 with partial pivoting
//      on its chunk, rows held in registers, and nominates the chunk's w
//      pivot rows (their original values go to the candidate buffer).
//   2. the same kernel, the CTA that finishes last: getf2 with partial
//      pivoting on the P*w nominated rows keeps the first w -- the panel's
//      pivot rows in order and the packed L11 \ U11 of those rows -- while
//      one warp turns the pivot order into the LAPACK interchange
//      sequence ipiv[c0 .. c0+w) and the at most 2w row moves it implies,
//      and the moved rows' panel values are staged.
//   3. tslu_apply_kernel: rows c0 .. c0+w-1 receive L11 \ U11; every other
//      panel row receives l solving l U11 = a (a: its value after the
//      moves), by substitution in registers.
// The interchanges reach the other columns through the leaf's laswp, as for
// the partial-pivoting panels.
//
// The getf2 keeps each row in registers, with the columns rotating down one
// register per step (the live column is always register 0, so the step loop
// is not unrolled); no row is ever moved: the pivot row of a step leaves the
// active set.  Every warp publishes its best row whole, so one barrier per
// column suffices (double-buffered by column parity).
//
// This is communication-avoiding LU's tall-skinny panel (Grigori, Demmel and
// Xiang, SIAM J. Matrix Anal. Appl. 32(4), 2011), one reduction level.  Its
// pivots differ from partial pivoting's, so the factors are not the
// reference's; they serve only as the preconditioner of FP64 refinement,
// whose result meets the FP64 backward-error bound (and whose pivot-growth
// check and FP64 fallback guard the rare matrix where they are poor).
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>

#include "device_util.cuh"
#include "gblu_internal.h"
#include "objects.h"
#include "profile.h"

namespace gblu {

namespace {

constexpr int kTsW = 32;                        // panel width
constexpr int kTsThreads = 512;                 // threads of a selection CTA
constexpr int kTsWarps = kTsThreads / 32;
constexpr int kTsMaxChunks = 32;                // chunks (CTAs) per panel
constexpr int kTsMaxCand = kTsMaxChunks * kTsW; // nominated rows the tree factors
constexpr int kTsTreeRpt = kTsMaxCand / kTsThreads;

// |a| as an ordered integer key for an active row (NaN ranks with zero);
// -1 marks a row that is no longer a candidate.
__device__ __forceinline__ int piv_key(float a) {
  const float v = fabsf(a);
  return isnan(v) ? 0 : __float_as_int(v);
}

template <int RPT>
__device__ __forceinline__ float pick(const float (&a)[RPT][kTsW], int q, int j) {
  float v = a[0][j];
#pragma unroll
  for (int t = 1; t < RPT; ++t)
    if (q == t) v = a[t][j];
  return v;
}

struct StepShared {
  float cand[2][kTsWarps][kTsW];  // each warp's best row, by column parity
  int key[2][kTsWarps];
  int slot[2][kTsWarps];
  int piv[kTsW];                  // slot of the pivot row of each step
  float U[kTsW][kTsW];            // tree: U row k, shifted (U[k][j] = u_{k,k+j})
};

// getf2 with partial pivoting over the rows in registers: thread t holds
// slots t*RPT + q (q < RPT), a[q][j] = the row's column k + j at step k.
// Records the pivot slot of every step; Tree also keeps the multipliers
// (sl[k * kTsMaxCand + slot]) and the U rows.  Returns the first column with
// no nonzero pivot, or -1.
template <int RPT, bool Tree>
__device__ int reg_getf2(float (&a)[RPT][kTsW], bool (&act)[RPT], int w, StepShared& sh, float* sl) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  int zc = -1;
#pragma unroll 1
  for (int k = 0; k < w; ++k) {
    const int buf = k & 1;
    int key = -1, qb = 0;
#pragma unroll
    for (int q = 0; q < RPT; ++q) {
      const int kq = act[q] ? piv_key(a[q][0]) : -1;
      if (kq > key) { key = kq; qb = q; }
    }
    const int wmax = __reduce_max_sync(0xffffffffu, key);
    const int wl = __ffs(__ballot_sync(0xffffffffu, key == wmax)) - 1;
    if (lane == wl) {
      float4* dst = reinterpret_cast<float4*>(&sh.cand[buf][warp][0]);
#pragma unroll
      for (int j = 0; j < kTsW; j += 4)
        dst[j / 4] = make_float4(pick<RPT>(a, qb, j), pick<RPT>(a, qb, j + 1), pick<RPT>(a, qb, j + 2),
                                 pick<RPT>(a, qb, j + 3));
      sh.key[buf][warp] = wmax;
      sh.slot[buf][warp] = tid * RPT + qb;
    }
    __syncthreads();
    const int kk = lane < kTsWarps ? sh.key[buf][lane] : INT_MIN;
    const int bmax = __reduce_max_sync(0xffffffffu, kk);
    const int ww = __ffs(__ballot_sync(0xffffffffu, kk == bmax)) - 1;
    const int pslot = sh.slot[buf][ww];
    const float4* u4 = reinterpret_cast<const float4*>(&sh.cand[buf][ww][0]);
    if (tid == 0) sh.piv[k] = pslot;
    if (pslot / RPT == tid) {  // the pivot row leaves the active set
      const int pq = pslot - tid * RPT;
#pragma unroll
      for (int q = 0; q < RPT; ++q)
        if (q == pq) act[q] = false;
      if constexpr (Tree) {
#pragma unroll
        for (int j = 0; j < kTsW; ++j) sh.U[k][j] = pick<RPT>(a, pq, j);
      }
    }
    const bool usable = bmax > 0;  // a nonzero, non-NaN pivot
    if (!usable && zc < 0) zc = k;
    float u[kTsW];
#pragma unroll
    for (int j = 0; j < kTsW; j += 4) {
      const float4 v = u4[j / 4];
      u[j] = v.x; u[j + 1] = v.y; u[j + 2] = v.z; u[j + 3] = v.w;
    }
    const float rp = usable ? 1.0f / u[0] : 0.0f;
#pragma unroll
    for (int q = 0; q < RPT; ++q) {
      if (!act[q]) continue;
      const float l = a[q][0] * rp;
      if constexpr (Tree) sl[k * kTsMaxCand + tid * RPT + q] = l;
#pragma unroll
      for (int j = 0; j < kTsW - 1; ++j) a[q][j] = fmaf(-l, u[j + 1], a[q][j + 1]);
      a[q][kTsW - 1] = 0.f;
    }
  }
  __syncthreads();
  return zc;
}

// Steps 1 and 2.  Dynamic shared memory (last CTA only uses it): the tree's
// multipliers, kTsW x kTsMaxCand floats, and the candidates' row numbers.
template <int RPT>
__global__ void __launch_bounds__(kTsThreads, 1)
tslu_select_kernel(const float* __restrict__ A, int64_t lda, int64_t m, int64_t c0, int w, int R,
                   int32_t* __restrict__ cand_rows, float* __restrict__ cand_vals,
                   unsigned* __restrict__ ticket, float* __restrict__ lu11,
                   int32_t* __restrict__ moves, float* __restrict__ staged, int64_t* __restrict__ ipiv,
                   int64_t* __restrict__ info, DevScratch* __restrict__ scr) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float* sl = reinterpret_cast<float*>(smem_raw);
  int* srows = reinterpret_cast<int*>(sl + (size_t)kTsW * kTsMaxCand);
  __shared__ __align__(16) StepShared sh;
  __shared__ int pos_s[2 * kTsW], row_s[2 * kTsW], cnt_s;
  __shared__ bool last_s;
  const int tid = threadIdx.x;
  const int P = gridDim.x;
  const int p = blockIdx.x;
  const int64_t r0 = c0 + (int64_t)p * R;
  const int nr = (int)min((int64_t)R, m - r0);

  // ---- 1. this chunk's nominations
  {
    float a[RPT][kTsW];
    bool act[RPT];
#pragma unroll
    for (int q = 0; q < RPT; ++q) {
      const int i = tid * RPT + q;
      act[q] = i < nr;
#pragma unroll
      for (int j = 0; j < kTsW; ++j) a[q][j] = (act[q] && j < w) ? A[(r0 + i) + (c0 + j) * lda] : 0.f;
    }
    const int cw = min(w, nr);
    reg_getf2<RPT, false>(a, act, cw, sh, nullptr);
    for (int idx = tid; idx < kTsW * kTsW; idx += kTsThreads) {
      const int k = idx / kTsW, j = idx % kTsW;
      float v = 0.f;
      if (k < cw && j < w) v = A[(r0 + sh.piv[k]) + (c0 + j) * lda];
      cand_vals[((size_t)p * kTsW + k) * kTsW + j] = v;
    }
    if (tid < kTsW) cand_rows[p * kTsW + tid] = tid < cw ? (int32_t)(r0 + sh.piv[tid]) : -1;
  }
  // ---- the last CTA to finish runs the tree (no CTA waits for another)
  __threadfence();
  __syncthreads();
  if (tid == 0) last_s = atomicAdd(ticket, 1u) == (unsigned)(P - 1);
  __syncthreads();
  if (!last_s) return;
  __threadfence();
  if (tid == 0) *ticket = 0u;  // ready for the next panel

  // ---- 2. the pivot rows among the nominated ones
  const int ncand = P * kTsW;
  int zc;
  {
    float a[kTsTreeRpt][kTsW];
    bool act[kTsTreeRpt];
#pragma unroll
    for (int q = 0; q < kTsTreeRpt; ++q) {
      const int c = tid * kTsTreeRpt + q;
      const int row = c < ncand ? __ldcg(cand_rows + c) : -1;
      act[q] = row >= 0;
      srows[c] = row;
      const float4* src = reinterpret_cast<const float4*>(cand_vals + (size_t)c * kTsW);
#pragma unroll
      for (int j = 0; j < kTsW; j += 4) {
        const float4 v = act[q] ? __ldcg(src + j / 4) : make_float4(0.f, 0.f, 0.f, 0.f);
        a[q][j] = v.x; a[q][j + 1] = v.y; a[q][j + 2] = v.z; a[q][j + 3] = v.w;
      }
    }
    __syncthreads();
    zc = reg_getf2<kTsTreeRpt, true>(a, act, w, sh, sl);
  }
  if (tid == 0 && zc >= 0)
    atomicCAS(reinterpret_cast<unsigned long long*>(info), 0ull, (unsigned long long)(c0 + zc + 1));
  // the interchange sequence: warp 0, one pivot at a time; position c0 + k
  // receives row g_k, which sits at a touched position or at its own.
  // The other warps write the packed L11 \ U11 of the pivot rows meanwhile.
  if ((tid >> 5) != 0) {
    for (int idx = tid - 32; idx < kTsW * kTsW; idx += kTsThreads - 32) {
      const int k = idx / kTsW, j = idx % kTsW;
      float v = 0.f;
      if (k < w && j < w) v = j < k ? sl[j * kTsMaxCand + sh.piv[k]] : sh.U[k][j - k];
      lu11[idx] = v;
    }
  } else {
    const int lane = tid & 31;
    int cnt = 0;
    bool bad = false;
    for (int k = 0; k < w; ++k) {
      const int g = srows[sh.piv[k]];
      if (g < c0 || g >= m) { bad = true; break; }
      const int target = (int)(c0 + k);
      // entries lane and lane + 32 of the touched list
      const int pa = lane < cnt ? pos_s[lane] : -1, ra = lane < cnt ? row_s[lane] : -1;
      const int pb = lane + 32 < cnt ? pos_s[lane + 32] : -1, rb = lane + 32 < cnt ? row_s[lane + 32] : -1;
      const unsigned ha = __ballot_sync(0xffffffffu, ra == g), hb = __ballot_sync(0xffffffffu, rb == g);
      int q = g;
      if (ha) q = __shfl_sync(0xffffffffu, pa, __ffs(ha) - 1);
      else if (hb) q = __shfl_sync(0xffffffffu, pb, __ffs(hb) - 1);
      if (lane == 0) ipiv[target] = (int64_t)q + 1;
      if (q != target) {
        const unsigned ta = __ballot_sync(0xffffffffu, pa == target), tb = __ballot_sync(0xffffffffu, pb == target);
        const unsigned qa = __ballot_sync(0xffffffffu, pa == q), qb = __ballot_sync(0xffffffffu, pb == q);
        const int tt = ta ? __ffs(ta) - 1 : (tb ? __ffs(tb) - 1 + 32 : -1);
        const int tq = qa ? __ffs(qa) - 1 : (qb ? __ffs(qb) - 1 + 32 : -1);
        // the row now at the target position (the one g displaces)
        const int rta = __shfl_sync(0xffffffffu, ra, tt & 31), rtb = __shfl_sync(0xffffffffu, rb, tt & 31);
        const int rt = tt < 0 ? target : (tt < 32 ? rta : rtb);
        if (lane == 0) {
          int c2 = cnt, t1 = tt, t2 = tq;
          if (t1 < 0) { t1 = c2++; pos_s[t1] = target; }
          row_s[t1] = g;
          if (t2 < 0) { t2 = c2++; pos_s[t2] = q; }
          row_s[t2] = rt;
          cnt = c2;
        }
        cnt = __shfl_sync(0xffffffffu, cnt, 0);
        __syncwarp();
      }
    }
    if (bad) {
      if (lane == 0) atomicCAS(&scr->error, 0, (int)DEV_BAD_PIVOT_INDEX);
      cnt = 0;
    }
    if (lane == 0) cnt_s = cnt;
  }
  __syncthreads();
  const int cnt = cnt_s;
  for (int t = tid; t < 2 * kTsW; t += kTsThreads) {
    moves[1 + 2 * t] = t < cnt ? pos_s[t] : -1;
    moves[2 + 2 * t] = t < cnt ? row_s[t] : -1;
  }
  if (tid == 0) moves[0] = cnt;
  for (int idx = tid; idx < cnt * kTsW; idx += kTsThreads) {
    const int t = idx / kTsW, j = idx % kTsW;
    staged[idx] = j < w ? A[(int64_t)row_s[t] + (c0 + j) * lda] : 0.f;
  }
}

// 3. every panel row: L11 \ U11 on top; below, l with l U11 = a, by
// right-looking substitution (a zero pivot, singular panel with info set,
// divides by 1).
constexpr int kTsApplyThreads = 128;
__global__ void __launch_bounds__(kTsApplyThreads)
tslu_apply_kernel(float* __restrict__ A, int64_t lda, int64_t m, int64_t c0, int w,
                  const float* __restrict__ lu11, const int32_t* __restrict__ moves,
                  const float* __restrict__ staged) {
  __shared__ __align__(16) float su[kTsW][kTsW];  // U11, row-major, zero below the diagonal
  __shared__ float rdiag[kTsW];
  __shared__ int mdst[2 * kTsW];
  __shared__ int ncnt;
  for (int idx = threadIdx.x; idx < kTsW * kTsW; idx += blockDim.x) {
    const int i = idx / kTsW, j = idx % kTsW;
    su[i][j] = j >= i ? lu11[idx] : 0.f;
  }
  if (threadIdx.x == 0) ncnt = moves[0];
  __syncthreads();
  for (int t = threadIdx.x; t < 2 * kTsW; t += blockDim.x) mdst[t] = t < ncnt ? moves[1 + 2 * t] : -1;
  if (threadIdx.x < kTsW) {
    const float d = su[threadIdx.x][threadIdx.x];
    rdiag[threadIdx.x] = d != 0.f ? 1.0f / d : 1.0f;
  }
  __syncthreads();
  const int64_t p = c0 + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= m) return;
  if (p < c0 + w) {
    const int k = (int)(p - c0);
    for (int j = 0; j < w; ++j) A[p + (c0 + j) * lda] = lu11[k * kTsW + j];
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
  for (int i = 0; i < kTsW; ++i) {
    x[i] *= rdiag[i];
    const float4* r4 = reinterpret_cast<const float4*>(&su[i][0]);
#pragma unroll
    for (int j4 = 0; j4 < kTsW / 4; ++j4) {
      if (4 * j4 + 3 <= i) continue;  // columns up to i are final
      const float4 v = r4[j4];
      if (4 * j4 > i) x[4 * j4] = fmaf(-x[i], v.x, x[4 * j4]);
      if (4 * j4 + 1 > i) x[4 * j4 + 1] = fmaf(-x[i], v.y, x[4 * j4 + 1]);
      if (4 * j4 + 2 > i) x[4 * j4 + 2] = fmaf(-x[i], v.z, x[4 * j4 + 2]);
      x[4 * j4 + 3] = fmaf(-x[i], v.w, x[4 * j4 + 3]);
    }
  }
#pragma unroll
  for (int j = 0; j < kTsW; ++j)
    if (j < w) A[p + (c0 + j) * lda] = x[j];
}

// ---------------------------------------------------------------------------
// No-pivot leaf of the random-butterfly-transformed factors: the top w x w
// block is factored without interchanges by warp 0 of every CTA (the same
// arithmetic everywhere, from the values before any CTA writes; lane i holds
// row i in registers, rotating one register per column, and the finished row
// is broadcast with shuffles), then each CTA solves l U11 = a for its 128 rows
// below the block by right-looking substitution; the last CTA to finish
// writes the top block back, the identity interchanges, and info for an
// exactly zero pivot (whose column is then left unscaled, as LAPACK's getf2
// does).
constexpr int kGenpRows = 128;
__global__ void __launch_bounds__(kGenpRows)
genp_panel_kernel(float* __restrict__ A, int64_t lda, int64_t m, int64_t c0, int w, int64_t* __restrict__ ipiv,
                  int64_t* __restrict__ info, unsigned* __restrict__ ticket) {
  __shared__ float U[kTsW][kTsW + 1];   // U[i][j], j >= i
  __shared__ float Lm[kTsW][kTsW + 1];  // multipliers L[i][j], i > j
  __shared__ float rdiag[kTsW];
  __shared__ int zcol;
  __shared__ bool last_s;
  const int tid = threadIdx.x;
  // this thread's row below the block, loaded while warp 0 factors the block
  const int64_t p = c0 + w + (int64_t)blockIdx.x * kGenpRows + tid;
  float x[kTsW];
#pragma unroll
  for (int j = 0; j < kTsW; ++j) x[j] = (p < m && j < w) ? A[p + (c0 + j) * lda] : 0.f;
  if (tid < 32) {
    const int i = tid;
    float r[kTsW];
#pragma unroll
    for (int j = 0; j < kTsW; ++j) r[j] = (i < w && j < w) ? A[(c0 + i) + (c0 + j) * lda] : 0.f;
    int zc = -1;
#pragma unroll 1
    for (int k = 0; k < w; ++k) {
      float u[kTsW];  // row k, columns k, k+1, ... (final)
#pragma unroll
      for (int j = 0; j < kTsW; ++j) u[j] = __shfl_sync(0xffffffffu, r[j], k);
      if (i == k) {
#pragma unroll
        for (int j = 0; j < kTsW; ++j)
          if (k + j < kTsW) U[k][k + j] = r[j];
      }
      if (u[0] == 0.f && zc < 0) zc = k;
      const float rp = u[0] != 0.f ? 1.0f / u[0] : 1.0f;
      if (i > k && i < w) {
        const float l = r[0] * rp;
        Lm[i][k] = l;
#pragma unroll
        for (int j = 0; j < kTsW - 1; ++j) r[j] = fmaf(-l, u[j + 1], r[j + 1]);
        r[kTsW - 1] = 0.f;
      }
    }
    if (i == 0) zcol = zc;
  }
  __syncthreads();
  if (tid < w) rdiag[tid] = U[tid][tid] != 0.f ? 1.0f / U[tid][tid] : 1.0f;
  __syncthreads();
  if (p < m) {
#pragma unroll
    for (int i = 0; i < kTsW; ++i) {
      if (i >= w) break;
      x[i] *= rdiag[i];
#pragma unroll
      for (int j = i + 1; j < kTsW; ++j) x[j] = fmaf(-x[i], U[i][j], x[j]);
    }
#pragma unroll
    for (int j = 0; j < kTsW; ++j)
      if (j < w) A[p + (c0 + j) * lda] = x[j];
  }
  __threadfence();
  __syncthreads();
  if (tid == 0) last_s = atomicAdd(ticket, 1u) == gridDim.x - 1;
  __syncthreads();
  if (!last_s) return;
  __threadfence();
  for (int idx = tid; idx < w * w; idx += kGenpRows) {
    const int j = idx / w, i = idx % w;
    A[(c0 + i) + (c0 + j) * lda] = j >= i ? U[i][j] : Lm[i][j];
  }
  if (tid < w) ipiv[c0 + tid] = c0 + tid + 1;
  if (tid == 0) {
    if (zcol >= 0) atomicCAS(reinterpret_cast<unsigned long long*>(info), 0ull, (unsigned long long)(c0 + zcol + 1));
    *ticket = 0u;  // ready for the next leaf
  }
}

size_t select_smem() { return (size_t)kTsW * kTsMaxCand * sizeof(float) + kTsMaxCand * sizeof(int); }

unsigned* work_ticket(void* work) {
  return reinterpret_cast<unsigned*>(reinterpret_cast<char*>(work) + align256(kTsMaxCand * sizeof(int32_t)) +
                                     align256((size_t)kTsMaxCand * kTsW * sizeof(float)));
}

}  // namespace

size_t tslu_work_bytes() {
  return align256(kTsMaxCand * sizeof(int32_t)) + align256((size_t)kTsMaxCand * kTsW * sizeof(float)) +
         align256(sizeof(unsigned)) + align256(kTsW * kTsW * sizeof(float)) +
         align256((1 + 4 * kTsW) * sizeof(int32_t)) + align256(2 * kTsW * kTsW * sizeof(float));
}

bool tslu_fits(int64_t rows, int w) {
  // at most kTsMaxChunks chunks of at most 2 * kTsThreads rows
  return w <= kTsW && w > 0 && rows > 0 && rows <= (int64_t)kTsMaxChunks * 2 * kTsThreads;
}

void tslu_configure(int /*device*/) {
  cudaFuncSetAttribute(tslu_select_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)select_smem());
  cudaFuncSetAttribute(tslu_select_kernel<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)select_smem());
}

// `work` (tslu_work_bytes(), zeroed when allocated: the ticket must start at 0)
cudaError_t tslu_panel_launch(float* A, int64_t lda, int64_t m, int64_t c0, int w, int64_t* ipiv,
                              int64_t* info, void* work, DevScratch* scr, cudaStream_t s) {
  const int64_t M = m - c0;
  if (!tslu_fits(M, w)) return cudaErrorInvalidValue;
  char* c = reinterpret_cast<char*>(work);
  int32_t* cand_rows = reinterpret_cast<int32_t*>(c);
  c += align256(kTsMaxCand * sizeof(int32_t));
  float* cand_vals = reinterpret_cast<float*>(c);
  c += align256((size_t)kTsMaxCand * kTsW * sizeof(float));
  unsigned* ticket = reinterpret_cast<unsigned*>(c);
  c += align256(sizeof(unsigned));
  if (ticket != work_ticket(work)) return cudaErrorInvalidValue;
  float* lu11 = reinterpret_cast<float*>(c);
  c += align256(kTsW * kTsW * sizeof(float));
  int32_t* moves = reinterpret_cast<int32_t*>(c);
  c += align256((1 + 4 * kTsW) * sizeof(int32_t));
  float* staged = reinterpret_cast<float*>(c);
  // chunks of 512 rows (one per thread), or of up to 1024 when more than
  // kTsMaxChunks would be needed
  int R = kTsThreads;
  if ((M + R - 1) / R > kTsMaxChunks) R = 2 * kTsThreads;
  const int P = (int)((M + R - 1) / R);
  double fl = 0;
  for (int k = 0; k < w; ++k) fl += (double)(M - k - 1) * (1.0 + 2.0 * (w - k - 1));
  {
    LaunchScope ls(K_PANEL, fl, 2.0 * M * w * sizeof(float), s);
    if (R == kTsThreads)
      tslu_select_kernel<1><<<P, kTsThreads, select_smem(), s>>>(A, lda, m, c0, w, R, cand_rows, cand_vals, ticket,
                                                                  lu11, moves, staged, ipiv, info, scr);
    else
      tslu_select_kernel<2><<<P, kTsThreads, select_smem(), s>>>(A, lda, m, c0, w, R, cand_rows, cand_vals, ticket,
                                                                  lu11, moves, staged, ipiv, info, scr);
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  LaunchScope ls(K_PANEL, (double)M * w * w, 2.0 * M * w * sizeof(float), s);
  tslu_apply_kernel<<<(unsigned)((M + kTsApplyThreads - 1) / kTsApplyThreads), kTsApplyThreads, 0, s>>>(
      A, lda, m, c0, w, lu11, moves, staged);
  return cudaGetLastError();
}

cudaError_t genp_panel_launch(float* A, int64_t lda, int64_t m, int64_t c0, int w, int64_t* ipiv,
                              int64_t* info, void* work, cudaStream_t s) {
  if (w <= 0 || w > kTsW || m - c0 < w) return cudaErrorInvalidValue;
  const int64_t below = m - c0 - w;
  const unsigned grid = (unsigned)std::max<int64_t>(1, (below + kGenpRows - 1) / kGenpRows);
  double fl = 0;
  for (int k = 0; k < w; ++k) fl += (double)(m - c0 - k - 1) * (1.0 + 2.0 * (w - k - 1));
  LaunchScope ls(K_PANEL, fl, 2.0 * (m - c0) * w * sizeof(float), s);
  genp_panel_kernel<<<grid, kGenpRows, 0, s>>>(A, lda, m, c0, w, ipiv, info, work_ticket(work));
  return cudaGetLastError();
}

}  // namespace gblu
