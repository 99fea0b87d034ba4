// getrs on the device: P, L and U solves as two wavefront kernels.
//
// Order of operations follows the reference's back-solve
// _naive_lu_ldiv! (src/factorization.jl:433-457), applied per RHS column:
//   b[i] <-> b[ipiv[i]] for i ascending           (here: one gather through perm)
//   for j ascending:   b[i] = fma(-L[i,j], b[j], b[i])   (i > j)
//   for j descending:  b[j] /= U[j,j];  b[i] = fma(-U[i,j], b[j], b[i])  (i < j)
// Each row's value is updated in exactly that sequence, so the result is
// bit-identical to the reference's vector back-solve.  The transposed solve
// (trans = 'T') is U^T y = b, L^T z = y, x = P^T z as LAPACK dgetrs 'T'.
//
// Parallel structure: the matrix is cut into 64-row block rows.  Each CTA takes
// a block row by ticket (tickets are handed out in launch order, so every CTA
// waits only for CTAs already running), streams its off-diagonal tiles in
// order, waiting on a per-block-row flag only right before a tile's
// solution values are needed, then solves its diagonal block and publishes its
// rows with a release flag.  All waits are bounded (DEV_TIMEOUT_SOLVE).
#include <algorithm>

#include "device_util.cuh"
#include "gblu_internal.h"
#include "profile.h"

namespace gblu {

constexpr int kTS = 64;  // block-row height == tile width

// Wait until flags[j] != 0; returns false on timeout/abort (all threads).
__device__ __forceinline__ bool wait_flag(const int32_t* flags, int j, DevScratch* scr) {
  __shared__ int ok;
  if (threadIdx.x == 0) {
    int res = 1;
    unsigned long long t0 = 0;
    for (unsigned it = 0;; ++it) {
      if (ld_acquire_i32(flags + j) != 0) break;
      if (ld_volatile_i32(&scr->error) != 0) { res = 0; break; }
      if ((it & 63u) == 0) {
        unsigned long long now = global_ns();
        if (t0 == 0) t0 = now;
        else if (now - t0 > kSpinTimeoutNs) {
          atomicCAS(&scr->error, 0, (int)DEV_TIMEOUT_SOLVE);
          res = 0;
          break;
        }
      }
    }
    ok = res;
  }
  __syncthreads();
  return ok != 0;
}

// Load tile (rows r0.., cols c0..) of op(LU) into shared memory as t[c][r]
// (element op(LU)[r0 + r, c0 + c]).  trans: op(LU)[i,j] = LU[j,i].
template <typename T, bool TRANS>
__device__ __forceinline__ void load_tile(T (*t)[kTS + 1], const T* __restrict__ LU, int64_t lda,
                                          int64_t n, int64_t r0, int64_t c0, int nr, int nc) {
#pragma unroll 16
  for (int idx = threadIdx.x; idx < kTS * kTS; idx += blockDim.x) {
    int a = idx >> 6, b = idx & 63;  // b fastest -> contiguous in memory
    if (!TRANS) {                    // element (r = b, c = a): LU[r0+b, c0+a]
      t[a][b] = (b < nr && a < nc) ? LU[(r0 + b) + (c0 + a) * lda] : T(0);
    } else {                         // element (r = a, c = b): LU[c0+b, r0+a]
      t[b][a] = (a < nr && b < nc) ? LU[(c0 + b) + (r0 + a) * lda] : T(0);
    }
  }
}

// Forward sweep with a unit-lower (trans 'N': L) or non-unit-lower
// (trans 'T': U^T) triangle.  Input row i of the RHS is In[src(i)] where
// src = perm for 'N' and identity for 'T'; the result goes to Y.
template <typename T, int NR, bool TRANS>
__global__ void __launch_bounds__(kTS)
solve_fwd_kernel(int64_t n, const T* __restrict__ LU, int64_t lda, const int32_t* __restrict__ perm,
                 const T* __restrict__ In, int64_t ldi, T* __restrict__ Y, int64_t ldy, int nrhs,
                 int32_t* __restrict__ flags, DevScratch* __restrict__ scr) {
  __shared__ T tile[kTS][kTS + 1];
  __shared__ T sx[kTS][NR];
  __shared__ int s_blk;
  if (threadIdx.x == 0) s_blk = (int)atomicAdd(&scr->ticket, 1u);
  __syncthreads();
  const int blk = s_blk;
  const int64_t r0 = (int64_t)blk * kTS;
  const int nr = (int)min((int64_t)kTS, n - r0);
  const int r = threadIdx.x;
  const int64_t row = r0 + r;
  const bool valid = r < nr;
  T acc[NR];
#pragma unroll
  for (int q = 0; q < NR; ++q) {
    int64_t src = valid ? (TRANS ? row : (int64_t)perm[row]) : 0;
    acc[q] = (valid && q < nrhs) ? In[src + q * ldi] : T(0);
  }
  for (int j = 0; j < blk; ++j) {
    const int64_t c0 = (int64_t)j * kTS;
    load_tile<T, TRANS>(tile, LU, lda, n, r0, c0, nr, kTS);
    if (!wait_flag(flags, j, scr)) return;
    for (int idx = threadIdx.x; idx < kTS * NR; idx += blockDim.x) {
      int c = idx / NR, q = idx - c * NR;
      sx[c][q] = q < nrhs ? ldcg(&Y[(c0 + c) + q * ldy]) : T(0);
    }
    __syncthreads();
#pragma unroll 8
    for (int c = 0; c < kTS; ++c) {
      const T l = tile[c][r];
#pragma unroll
      for (int q = 0; q < NR; ++q) acc[q] = fma(-l, sx[c][q], acc[q]);
    }
    __syncthreads();
  }
  // diagonal block
  load_tile<T, TRANS>(tile, LU, lda, n, r0, r0, nr, nr);
  __syncthreads();
  for (int c = 0; c < nr; ++c) {
    if (r == c) {
#pragma unroll
      for (int q = 0; q < NR; ++q) {
        if (TRANS) acc[q] = acc[q] / tile[c][c];
        sx[c][q] = acc[q];
      }
    }
    __syncthreads();
    if (r > c && valid) {
      const T l = tile[c][r];
#pragma unroll
      for (int q = 0; q < NR; ++q) acc[q] = fma(-l, sx[c][q], acc[q]);
    }
  }
  if (valid)
#pragma unroll
    for (int q = 0; q < NR; ++q)
      if (q < nrhs) Y[row + q * ldy] = acc[q];
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) st_release_i32(flags + blk, 1);
}

// Backward sweep with a non-unit upper (trans 'N': U) or unit upper
// (trans 'T': L^T) triangle; block rows are taken last-first.  Results go
// to Y (for the other block rows) and to Out[dst(i)] (dst = identity for 'N',
// perm for 'T', i.e. x = P^T z).
template <typename T, int NR, bool TRANS>
__global__ void __launch_bounds__(kTS)
solve_bwd_kernel(int64_t n, const T* __restrict__ LU, int64_t lda, const int32_t* __restrict__ perm,
                 T* __restrict__ Y, int64_t ldy, T* __restrict__ Out, int64_t ldo, int nrhs,
                 int32_t* __restrict__ flags, DevScratch* __restrict__ scr) {
  __shared__ T tile[kTS][kTS + 1];
  __shared__ T sx[kTS][NR];
  __shared__ int s_blk;
  const int nblk = (int)((n + kTS - 1) / kTS);
  if (threadIdx.x == 0) s_blk = nblk - 1 - (int)atomicAdd(&scr->ticket, 1u);
  __syncthreads();
  const int blk = s_blk;
  const int64_t r0 = (int64_t)blk * kTS;
  const int nr = (int)min((int64_t)kTS, n - r0);
  const int r = threadIdx.x;
  const int64_t row = r0 + r;
  const bool valid = r < nr;
  T acc[NR];
#pragma unroll
  for (int q = 0; q < NR; ++q) acc[q] = (valid && q < nrhs) ? Y[row + q * ldy] : T(0);
  for (int j = nblk - 1; j > blk; --j) {
    const int64_t c0 = (int64_t)j * kTS;
    const int nc = (int)min((int64_t)kTS, n - c0);
    load_tile<T, TRANS>(tile, LU, lda, n, r0, c0, nr, nc);
    if (!wait_flag(flags, j, scr)) return;
    for (int idx = threadIdx.x; idx < kTS * NR; idx += blockDim.x) {
      int c = idx / NR, q = idx - c * NR;
      sx[c][q] = (q < nrhs && c < nc) ? ldcg(&Y[(c0 + c) + q * ldy]) : T(0);
    }
    __syncthreads();
    for (int c = nc - 1; c >= 0; --c) {
      const T u = tile[c][r];
#pragma unroll
      for (int q = 0; q < NR; ++q) acc[q] = fma(-u, sx[c][q], acc[q]);
    }
    __syncthreads();
  }
  load_tile<T, TRANS>(tile, LU, lda, n, r0, r0, nr, nr);
  __syncthreads();
  for (int c = nr - 1; c >= 0; --c) {
    if (r == c) {
#pragma unroll
      for (int q = 0; q < NR; ++q) {
        if (!TRANS) acc[q] = acc[q] / tile[c][c];
        sx[c][q] = acc[q];
      }
    }
    __syncthreads();
    if (r < c) {
      const T u = tile[c][r];
#pragma unroll
      for (int q = 0; q < NR; ++q) acc[q] = fma(-u, sx[c][q], acc[q]);
    }
  }
  if (valid) {
    const int64_t dst = TRANS ? (int64_t)perm[row] : row;
#pragma unroll
    for (int q = 0; q < NR; ++q)
      if (q < nrhs) {
        Y[row + q * ldy] = acc[q];
        Out[dst + q * ldo] = acc[q];
      }
  }
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) st_release_i32(flags + blk, 1);
}

size_t getrs_scratch_bytes(int64_t n, int elem_size, int64_t work_cols) {
  int64_t nblk = (n + kTS - 1) / kTS;
  size_t b = 256 + ((2 * nblk * sizeof(int32_t) + 255) & ~size_t(255));
  b += ((size_t)n * work_cols * elem_size + 255) & ~size_t(255);
  return b + 256;
}

template <typename T>
void getrs_carve(GetrsPlan<T>& p, void* base, size_t bytes, int64_t work_cols) {
  char* c = reinterpret_cast<char*>(base);
  auto take = [&](size_t nb) { char* r = c; c += (nb + 255) & ~size_t(255); return r; };
  int64_t nblk = (p.n + kTS - 1) / kTS;
  p.scratch = reinterpret_cast<DevScratch*>(take(sizeof(DevScratch)));
  p.flags = reinterpret_cast<int32_t*>(take(2 * nblk * sizeof(int32_t)));
  p.work = reinterpret_cast<T*>(take((size_t)p.n * work_cols * sizeof(T)));
  p.work_cols = work_cols;
  (void)bytes;
}

namespace {
template <typename T, int NR>
cudaError_t run_chunk(const GetrsPlan<T>& p, char trans, int nr, T* B, int64_t ldb,
                      cudaStream_t s) {
  const int64_t nblk = (p.n + kTS - 1) / kTS;
  int32_t* ffwd = p.flags;
  int32_t* fbwd = p.flags + nblk;
  cudaError_t e = cudaMemsetAsync(p.flags, 0, 2 * nblk * sizeof(int32_t), s);
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(&p.scratch->ticket, 0, sizeof(unsigned), s);
  if (e != cudaSuccess) return e;
  const bool tr = trans == 'T' || trans == 't' || trans == 'C' || trans == 'c';
  // algorithmic work of one sweep: the triangle (n^2/2 elements) read once,
  // n^2 flops per right-hand side
  const double tri_bytes = 0.5 * (double)p.n * (double)p.n * sizeof(T) + 2.0 * p.n * nr * sizeof(T);
  const double sweep_flops = (double)p.n * (double)p.n * nr;
  {
  LaunchScope ls(K_SOLVE, sweep_flops, tri_bytes, s);
  if (!tr)
    solve_fwd_kernel<T, NR, false><<<(unsigned)nblk, kTS, 0, s>>>(
        p.n, p.LU, p.lda, p.perm, B, ldb, p.work, p.n, nr, ffwd, p.scratch);
  else
    solve_fwd_kernel<T, NR, true><<<(unsigned)nblk, kTS, 0, s>>>(
        p.n, p.LU, p.lda, p.perm, B, ldb, p.work, p.n, nr, ffwd, p.scratch);
  }
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(&p.scratch->ticket, 0, sizeof(unsigned), s);
  if (e != cudaSuccess) return e;
  LaunchScope ls(K_SOLVE, sweep_flops, tri_bytes, s);
  if (!tr)
    solve_bwd_kernel<T, NR, false><<<(unsigned)nblk, kTS, 0, s>>>(
        p.n, p.LU, p.lda, p.perm, p.work, p.n, B, ldb, nr, fbwd, p.scratch);
  else
    solve_bwd_kernel<T, NR, true><<<(unsigned)nblk, kTS, 0, s>>>(
        p.n, p.LU, p.lda, p.perm, p.work, p.n, B, ldb, nr, fbwd, p.scratch);
  return cudaGetLastError();
}
}  // namespace

template <typename T>
cudaError_t getrs_launch(const GetrsPlan<T>& p, char trans, int64_t nrhs, T* B, int64_t ldb,
                         uint32_t* /*epoch*/, cudaStream_t s) {
  if (p.n <= 0 || nrhs <= 0) return cudaSuccess;
  const int64_t chunk = std::min<int64_t>(p.work_cols, 8);
  for (int64_t c = 0; c < nrhs; c += chunk) {
    int nr = (int)std::min<int64_t>(chunk, nrhs - c);
    T* Bc = B + c * ldb;
    cudaError_t e;
    if (nr == 1) e = run_chunk<T, 1>(p, trans, nr, Bc, ldb, s);
    else if (nr == 2) e = run_chunk<T, 2>(p, trans, nr, Bc, ldb, s);
    else if (nr <= 4) e = run_chunk<T, 4>(p, trans, nr, Bc, ldb, s);
    else e = run_chunk<T, 8>(p, trans, nr, Bc, ldb, s);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

template cudaError_t getrs_launch<double>(const GetrsPlan<double>&, char, int64_t, double*, int64_t,
                                          uint32_t*, cudaStream_t);
template cudaError_t getrs_launch<float>(const GetrsPlan<float>&, char, int64_t, float*, int64_t,
                                         uint32_t*, cudaStream_t);
template void getrs_carve<double>(GetrsPlan<double>&, void*, size_t, int64_t);
template void getrs_carve<float>(GetrsPlan<float>&, void*, size_t, int64_t);

}  // namespace gblu
