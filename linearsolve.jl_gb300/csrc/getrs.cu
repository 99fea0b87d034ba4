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
#include "waits.cuh"
#include "gblu_internal.h"
#include "profile.h"

namespace gblu {

constexpr int kTS = kGetrsTile;  // block-row height == tile width
// fast-solve matrices per 64-row block b, each 64 x 64 column-major:
// InvL_bb, InvU_bb, InvL_bb L_{b,b-1}, InvU_bb U_{b,b+1}
constexpr int kInvSlots = 4;

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

constexpr int kSweepThreads = 128;  // all issue copies; threads 0..63 own one row each
constexpr int kStages = 3;          // tiles in flight per CTA

template <typename T>
__device__ __forceinline__ void cp_async_elem(T* dst, const T* src, bool valid) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  const int sz = valid ? (int)sizeof(T) : 0;  // 0: zero-fill, nothing read
  if (sizeof(T) == 8)
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;" ::"r"(d), "l"(src), "r"(sz) : "memory");
  else
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(d), "l"(src), "r"(sz) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

// Row stride of a staged tile: 16 bytes of padding keep every column of
// t[c][r] 16-byte aligned (for 16-byte copies) and its reads conflict-free.
template <typename T>
__host__ __device__ constexpr int tile_ld() { return kTS + 16 / (int)sizeof(T); }

// Issue the copies of tile element (r, c) = op(LU)[r0 + r, c0 + c] into t[c][r];
// 'N': LU[r0+r + (c0+c)*lda] (contiguous in r), 'T': LU[c0+c + (r0+r)*lda]
// (contiguous in c).  Elements outside nr x nc are zero-filled.  A full 'N'
// tile of a 16-byte-aligned matrix (vec16) moves in 16-byte copies, each
// thread walking a fixed row slice across every (kSweepThreads / 16-byte
// copies per column)-th column.
template <typename T, bool TRANS>
__device__ __forceinline__ void issue_tile(T (*t)[tile_ld<T>()], const T* __restrict__ LU, int64_t lda,
                                           int64_t r0, int64_t c0, int nr, int nc, bool vec16) {
  if (!TRANS && vec16 && nr == kTS && nc == kTS) {
    constexpr int V = 16 / (int)sizeof(T);    // elements per copy
    constexpr int CPC = kTS / V;              // copies per column
    constexpr int CSTEP = kSweepThreads / CPC;  // columns per pass
    const int cl = (int)threadIdx.x / CPC, rv = ((int)threadIdx.x % CPC) * V;
    const T* src = LU + (r0 + rv) + (c0 + cl) * lda;
#pragma unroll
    for (int c = cl; c < kTS; c += CSTEP, src += CSTEP * lda) {
      const unsigned d = (unsigned)__cvta_generic_to_shared(&t[c][rv]);
      asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d), "l"(src) : "memory");
    }
    return;
  }
#pragma unroll 8
  for (int idx = threadIdx.x; idx < kTS * kTS; idx += kSweepThreads) {
    const int a = idx >> 6, b = idx & 63;  // b runs along the contiguous direction
    const int r = TRANS ? a : b, c = TRANS ? b : a;
    const bool ok = r < nr && c < nc;
    const T* src = ok ? (TRANS ? LU + (c0 + c) + (r0 + r) * lda : LU + (r0 + r) + (c0 + c) * lda) : LU;
    cp_async_elem(&t[c][r], src, ok);
  }
}

// One triangular sweep over 64-row block rows.
//   FWD  : block rows first-to-last, columns ascending; 'N' unit-lower L with
//          the right-hand side gathered through perm, 'T' non-unit U^T.
//   !FWD : block rows last-to-first, columns descending; 'N' non-unit U,
//          'T' unit L^T; results also scattered to Out (through perm for 'T').
// Each row accumulates its updates in exactly the reference's order; the
// diagonal block is solved by warp shuffles (no block barrier per column).
//
// FAST: the same wavefront without the reference's order: each row keeps
// four independent partial sums over the off-diagonal tiles, and the
// diagonal block is applied as a 64 x 64 matrix-vector product with its
// precomputed inverse (inv: [block][L, U][64 x 64], column-major), so a block
// row's critical path is two short product chains instead of 64 dependent
// division / FMA steps.  Backward-error accurate, not bit-exact.
template <typename T, int NR, bool TRANS, bool FWD, bool FAST>
__global__ void __launch_bounds__(kSweepThreads)
solve_sweep_kernel(int64_t n, const T* __restrict__ LU, int64_t lda, const int32_t* __restrict__ perm,
                   const T* __restrict__ In, int64_t ldi, T* __restrict__ Y, int64_t ldy,
                   T* __restrict__ Out, int64_t ldo, int nrhs, int32_t* __restrict__ flags,
                   DevScratch* __restrict__ scr, const T* __restrict__ inv) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T(*tiles)[kTS][tile_ld<T>()] = reinterpret_cast<T(*)[kTS][tile_ld<T>()]>(smem_raw);
  // 16-byte copies need a 16-byte-aligned matrix and column stride
  const bool vec16 = ((reinterpret_cast<uintptr_t>(LU) | (uintptr_t)(lda * (int64_t)sizeof(T))) & 15) == 0;
  __shared__ T sx[kTS][NR];
  __shared__ int s_blk;
  __shared__ int s_fail;
  constexpr bool kUnit = FWD != TRANS;  // fwd 'N' (L) and bwd 'T' (L^T) have unit diagonals
  // FP64: rows are published as soon as they are final and the next block
  // row applies them as they come (its last tile is 64 dependent 64-cycle
  // FMAs per row); FP32 tiles are cheap, so rows are published at the end.
  constexpr bool kEarly = sizeof(T) == 8 && !FAST;
  const int nblk = (int)((n + kTS - 1) / kTS);
  if (threadIdx.x == 0) {
    const int t = (int)atomicAdd(&scr->ticket, 1u);
    s_blk = FWD ? t : nblk - 1 - t;
    s_fail = 0;
  }
  __syncthreads();
  const int blk = s_blk;
  const int64_t r0 = (int64_t)blk * kTS;
  const int nr = (int)min((int64_t)kTS, n - r0);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int r = tid;  // row within the block (threads 0..63)
  const bool valid = r < nr;
  T acc[NR];
#pragma unroll
  for (int q = 0; q < NR; ++q) {
    acc[q] = T(0);
    if (valid && q < nrhs) {
      if (FWD) acc[q] = In[(TRANS ? r0 + r : (int64_t)perm[r0 + r]) + q * ldi];
      else acc[q] = Y[(r0 + r) + q * ldy];
    }
  }
  const int noff = FWD ? blk : nblk - 1 - blk;  // off-diagonal tiles of this block row
  const int ntiles = noff + 1;                  // + the diagonal tile
  auto col_block = [&](int t) -> int { return t < noff ? (FWD ? t : nblk - 1 - t) : blk; };
  auto issue = [&](int t) {
    if (FAST && t == noff) {  // op(inverse of the diagonal block): tile[c][r] = op(Inv)(r, c)
      const T* ib = inv + ((int64_t)blk * kInvSlots + (kUnit ? 0 : 1)) * (kTS * kTS);
      issue_tile<T, TRANS>(tiles[t % kStages], ib, kTS, 0, 0, nr, nr, true);
      return;
    }
    const int cb = col_block(t);
    const int64_t c0 = (int64_t)cb * kTS;
    const int nc = (int)min((int64_t)kTS, n - c0);
    issue_tile<T, TRANS>(tiles[t % kStages], LU, lda, r0, c0, nr, nc, vec16);
  };
  // FAST: three more partial sums per right-hand side (acc is the first)
  T acc2[FAST ? 3 : 1][NR];
#pragma unroll
  for (int j = 0; j < (FAST ? 3 : 1); ++j)
#pragma unroll
    for (int q = 0; q < NR; ++q) acc2[j][q] = T(0);
#pragma unroll
  for (int t = 0; t < kStages - 1; ++t) {
    if (t < ntiles) issue(t);
    cp_async_commit();
  }
  // Solution values of the next off-diagonal tile are fetched one tile ahead
  // (most are published long before they are needed); a value still equal to
  // the sentinel is polled until it arrives.
  using UB = typename SweepBits<T>::U;
  constexpr int KP = (kTS * NR + kSweepThreads - 1) / kSweepThreads;
  UB pre[KP];
  auto src_of = [&](int cb, int c, int q) -> const T* {
    const int64_t c0 = (int64_t)cb * kTS;
    return FWD ? &Y[(c0 + c) + q * ldy] : &Out[(TRANS ? (int64_t)perm[c0 + c] : c0 + c) + q * ldo];
  };
  auto prefetch = [&](int t) {
    const int cb = col_block(t);
    const int nc = (int)min((int64_t)kTS, n - (int64_t)cb * kTS);
#pragma unroll
    for (int k = 0; k < KP; ++k) {
      const int idx = tid + k * kSweepThreads;
      const int c = idx / NR, q = idx - c * NR;
      pre[k] = (idx < kTS * NR && q < nrhs && c < nc) ? SweepBits<T>::load(src_of(cb, c, q)) : UB(0);
    }
  };
  // (FP64: the last off-diagonal tile is consumed as it is published)
  if (noff > (kEarly ? 1 : 0)) prefetch(0);
  // this row's solution values, to the sweep's output (dependents poll them)
  auto publish_row = [&]() {
#pragma unroll
    for (int q = 0; q < NR; ++q)
      if (q < nrhs) {
        const T v = SweepBits<T>::canon(acc[q]);
        if (FWD) Y[(r0 + r) + q * ldy] = v;
        else Out[(TRANS ? (int64_t)perm[r0 + r] : r0 + r) + q * ldo] = v;
      }
  };
  for (int t = 0; t < ntiles; ++t) {
    if (t + kStages - 1 < ntiles) issue(t + kStages - 1);
    cp_async_commit();
    cp_async_wait<kStages - 1>();
    __syncthreads();
    T(*tile)[tile_ld<T>()] = tiles[t % kStages];
    if (kEarly && t == noff - 1) {
      // The tile of the block row just before this one in the sweep: its
      // rows are published one by one while that block solves its diagonal,
      // so it is applied CH columns at a time in sweep order, warp 2 polling
      // the next columns while warps 0-1 apply the previous ones.
      const int cb = col_block(t);
      const int nc = (int)min((int64_t)kTS, n - (int64_t)cb * kTS);
      constexpr int CH = 8, NCH = kTS / CH;
      for (int ch = 0; ch <= NCH; ++ch) {
        if (warp == 2 && ch < NCH) {
          const int cbeg = FWD ? CH * ch : kTS - CH * (ch + 1);
          for (int idx = lane; idx < CH * NR; idx += 32) {
            const int c = cbeg + idx / NR, q = idx % NR;
            T v = T(0);
            if (q < nrhs && c < nc && !poll_value(src_of(cb, c, q), scr, &v)) s_fail = 1;
            sx[c][q] = v;
          }
        }
        if (warp < 3) named_bar_sync(1, 96);
        if (ch > 0 && tid < kTS) {
          const int pc = ch - 1;
          if (FWD) {
#pragma unroll
            for (int c = CH * pc; c < CH * pc + CH; ++c) {
              const T l = tile[c][r];
#pragma unroll
              for (int q = 0; q < NR; ++q) acc[q] = fma(-l, sx[c][q], acc[q]);
            }
          } else {
#pragma unroll
            for (int c = kTS - CH * pc - 1; c >= kTS - CH * (pc + 1); --c) {
              if (c >= nc) continue;
              const T u = tile[c][r];
#pragma unroll
              for (int q = 0; q < NR; ++q) acc[q] = fma(-u, sx[c][q], acc[q]);
            }
          }
        }
      }
      if (!__syncthreads_and(s_fail == 0)) {
        cp_async_wait<0>();  // no copy may land after the CTA has left
        return;
      }
      continue;
    }
    if (t < noff) {
      const int cb = col_block(t);
      const int64_t c0 = (int64_t)cb * kTS;
      const int nc = (int)min((int64_t)kTS, n - c0);
      int ok = 1;
#pragma unroll
      for (int k = 0; k < KP; ++k) {
        const int idx = tid + k * kSweepThreads;
        if (idx >= kTS * NR) continue;
        const int c = idx / NR, q = idx - c * NR;
        T v = T(0);
        if (q < nrhs && c < nc) {
          if (pre[k] != SweepBits<T>::kSentinel) v = SweepBits<T>::as_t(pre[k]);
          else if (!poll_value(src_of(cb, c, q), scr, &v)) ok = 0;
        }
        sx[c][q] = v;
      }
      if (!__syncthreads_and(ok)) {
        cp_async_wait<0>();  // no copy may land after the CTA has left
        return;
      }
      if (t + 1 < noff - (kEarly ? 1 : 0)) prefetch(t + 1);
      if constexpr (FAST) {
        // four independent partial sums (columns c = 4i + j); entries past nc
        // are zero in both the tile and sx
        if (tid < kTS) {
#pragma unroll 4
          for (int c = 0; c < kTS; c += 4) {
            const T l0 = tile[c][r], l1 = tile[c + 1][r], l2 = tile[c + 2][r], l3 = tile[c + 3][r];
#pragma unroll
            for (int q = 0; q < NR; ++q) {
              acc[q] = fma(-l0, sx[c][q], acc[q]);
              acc2[0][q] = fma(-l1, sx[c + 1][q], acc2[0][q]);
              acc2[1][q] = fma(-l2, sx[c + 2][q], acc2[1][q]);
              acc2[2][q] = fma(-l3, sx[c + 3][q], acc2[2][q]);
            }
          }
        }
      } else if (tid < kTS) {
        if (FWD) {
#pragma unroll 8
          for (int c = 0; c < kTS; ++c) {
            const T l = tile[c][r];
#pragma unroll
            for (int q = 0; q < NR; ++q) acc[q] = fma(-l, sx[c][q], acc[q]);
          }
        } else if (nc == kTS) {
#pragma unroll 8
          for (int c = kTS - 1; c >= 0; --c) {
            const T u = tile[c][r];
#pragma unroll
            for (int q = 0; q < NR; ++q) acc[q] = fma(-u, sx[c][q], acc[q]);
          }
        } else {
          for (int c = nc - 1; c >= 0; --c) {
            const T u = tile[c][r];
#pragma unroll
            for (int q = 0; q < NR; ++q) acc[q] = fma(-u, sx[c][q], acc[q]);
          }
        }
      }
      __syncthreads();
      continue;
    }
    if constexpr (FAST) {
      // ---- diagonal block: x = op(Inv) (b - off-diagonal products) ----
      if (tid < kTS) {
#pragma unroll
        for (int q = 0; q < NR; ++q) {
          const T tot = (acc[q] + acc2[0][q]) + (acc2[1][q] + acc2[2][q]);
          sx[r][q] = valid ? tot : T(0);
        }
      }
      __syncthreads();
      if (tid < kTS) {
        T y[4][NR];
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
          for (int q = 0; q < NR; ++q) y[j][q] = T(0);
#pragma unroll 4
        for (int c = 0; c < kTS; c += 4) {
          const T m0 = tile[c][r], m1 = tile[c + 1][r], m2 = tile[c + 2][r], m3 = tile[c + 3][r];
#pragma unroll
          for (int q = 0; q < NR; ++q) {
            y[0][q] = fma(m0, sx[c][q], y[0][q]);
            y[1][q] = fma(m1, sx[c + 1][q], y[1][q]);
            y[2][q] = fma(m2, sx[c + 2][q], y[2][q]);
            y[3][q] = fma(m3, sx[c + 3][q], y[3][q]);
          }
        }
#pragma unroll
        for (int q = 0; q < NR; ++q) acc[q] = (y[0][q] + y[1][q]) + (y[2][q] + y[3][q]);
      }
      continue;
    }
    // ---- diagonal block: warp shuffles within each 32-row half ----

    // reciprocal of this row's diagonal entry, off the dependency chain
    const T yrow = (!kUnit && valid && tid < kTS) ? T(1) / tile[r][r] : T(1);
    const int w_first = FWD ? 0 : 1, w_second = FWD ? 1 : 0;
    const int lo_second = FWD ? 32 : 0;  // first row of the second half
    (void)lo_second;
    // One column of the diagonal chain for all NR right-hand sides: the
    // divisions (lane `src` only, non-unit diagonal), then the broadcasts,
    // then the updates, so the NR chains overlap.
    // keep: the owner also leaves its value in sx for the other warp
    auto chain_step = [&](int c, int src, bool divide_here, bool update, bool keep) {
      if (!kUnit && divide_here) {
        if constexpr (NR == 1) acc[0] = div_markstein(acc[0], tile[c][c], yrow);
        else div_markstein_n<T, NR>(acc, tile[c][c], yrow);
      }
      T xc[NR];
#pragma unroll
      for (int q = 0; q < NR; ++q) xc[q] = __shfl_sync(0xffffffffu, acc[q], src);
      // row c is final: its dependents may start on it (stored while the
      // broadcast is in flight)
      if (kEarly && r == c && valid) {
        publish_row();
        if (keep)
#pragma unroll
          for (int q = 0; q < NR; ++q) sx[c][q] = acc[q];
      }
      if (update) {
        const T a = tile[c][r];
#pragma unroll
        for (int q = 0; q < NR; ++q) acc[q] = fma(-a, xc[q], acc[q]);
      }
    };
    // FP64: the second warp applies the first half's solutions eight
    // columns at a time while the first warp is still solving (one named
    // barrier per group of eight), instead of re-applying all of them as a
    // chain of 64-cycle FMAs afterwards.
    const bool prog = kEarly && nr > 32;
    const int m1 = FWD ? min(nr, 32) : nr - 32;  // columns of the first half
    if (warp == w_first) {
      // columns of the first half, in sweep order
      for (int st = 0; st < m1; ++st) {
        const int c = FWD ? st : nr - 1 - st;
        if (FWD) chain_step(c, c, lane == c, r > c && r < nr, prog);
        else chain_step(c, c - 32, r == c, r < c, prog);
        if (prog && ((st & 7) == 7 || st == m1 - 1)) named_bar_arrive(2 + (st >> 3), 64);
      }
      if (!prog && valid)
#pragma unroll
        for (int q = 0; q < NR; ++q) sx[r][q] = acc[q];
    }
    if (!prog) __syncthreads();
    if (warp == w_second) {
      // the first half's columns applied in sweep order, then this half's chain
      for (int st = 0; st < m1; ++st) {
        if (prog && (st & 7) == 0) named_bar_sync(2 + (st >> 3), 64);
        const int c = FWD ? st : nr - 1 - st;
        if (FWD && nr <= 32) break;
#pragma unroll
        for (int q = 0; q < NR; ++q) acc[q] = fma(-tile[c][r], sx[c][q], acc[q]);
      }
      if (FWD) {
        for (int c = 32; c < nr; ++c) chain_step(c, c - 32, r == c, r > c && r < nr, false);
      } else {
        for (int c = min(nr, 32) - 1; c >= 0; --c) chain_step(c, c, lane == c, r < c, false);
      }
    }
  }
  cp_async_wait<0>();
  if (!kEarly && valid && tid < kTS) publish_row();
  (void)flags;
}

// Fast 'N' sweeps.  Block row i's solution is x_i = d_i - M_i x_p, where x_p
// is the block row just before it in the sweep, M_i its coupling (fold_kernel)
// and d_i = Inv_ii (b_i - the products with every earlier block row but x_p):
// d_i is computed while x_p is still being solved, so only the 64 x 64
// product M_i x_p lies on the wavefront's critical path.  Two threads per
// row, each taking half of every tile's columns with four independent
// partial sums, combined through shared memory.  Tile order per block row:
// the earlier off-diagonal blocks but the last (in sweep order), Inv_ii,
// then M_i.  Backward-error accurate, not bit-exact.
template <typename T, int NR, bool FWD>
__global__ void __launch_bounds__(kSweepThreads)
fast_sweep_kernel(int64_t n, const T* __restrict__ LU, int64_t lda, const int32_t* __restrict__ perm,
                  const T* __restrict__ In, int64_t ldi, T* __restrict__ Y, int64_t ldy,
                  T* __restrict__ Out, int64_t ldo, int nrhs, DevScratch* __restrict__ scr,
                  const T* __restrict__ inv) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T(*tiles)[kTS][tile_ld<T>()] = reinterpret_cast<T(*)[kTS][tile_ld<T>()]>(smem_raw);
  __shared__ T sx[kTS][NR];
  __shared__ T part[2][kTS][NR];
  __shared__ int s_blk;
  const bool vec16 = ((reinterpret_cast<uintptr_t>(LU) | (uintptr_t)(lda * (int64_t)sizeof(T))) & 15) == 0;
  const int nblk = (int)((n + kTS - 1) / kTS);
  if (threadIdx.x == 0) {
    const int t = (int)atomicAdd(&scr->ticket, 1u);
    s_blk = FWD ? t : nblk - 1 - t;
  }
  __syncthreads();
  const int blk = s_blk;
  const int64_t r0 = (int64_t)blk * kTS;
  const int nr = (int)min((int64_t)kTS, n - r0);
  const int tid = threadIdx.x, r = tid & 63, h = tid >> 6;
  const bool valid = r < nr;
  const int noff = FWD ? blk : nblk - 1 - blk;  // block rows before this one in the sweep
  const int nlead = noff > 0 ? noff - 1 : 0;    // off-diagonal tiles before the coupling
  const int ntiles = nlead + 1 + (noff > 0 ? 1 : 0);
  const int pcb = FWD ? blk - 1 : blk + 1;      // the coupled block row (noff > 0)
  const int pnc = noff > 0 ? (int)min((int64_t)kTS, n - (int64_t)pcb * kTS) : 0;
  auto col_block = [&](int t) -> int { return FWD ? t : nblk - 1 - t; };
  auto issue = [&](int t) {
    if (t < nlead) {
      const int64_t c0 = (int64_t)col_block(t) * kTS;
      issue_tile<T, false>(tiles[t % kStages], LU, lda, r0, c0, nr, (int)min((int64_t)kTS, n - c0), vec16);
    } else {
      const bool coupling = t > nlead;
      const int slot = (coupling ? 2 : 0) + (FWD ? 0 : 1);
      issue_tile<T, false>(tiles[t % kStages], inv + ((int64_t)blk * kInvSlots + slot) * (kTS * kTS), kTS, 0, 0,
                           nr, coupling ? pnc : nr, true);
    }
  };
  T a[4][NR];  // partial sums; thread h = 0 starts from the right-hand side
#pragma unroll
  for (int j = 0; j < 4; ++j)
#pragma unroll
    for (int q = 0; q < NR; ++q) a[j][q] = T(0);
  if (h == 0 && valid)
#pragma unroll
    for (int q = 0; q < NR; ++q)
      if (q < nrhs) a[0][q] = FWD ? In[(int64_t)perm[r0 + r] + q * ldi] : Y[(r0 + r) + q * ldy];
  T d[NR];
#pragma unroll
  for (int q = 0; q < NR; ++q) d[q] = T(0);
#pragma unroll
  for (int t = 0; t < kStages - 1; ++t) {
    if (t < ntiles) issue(t);
    cp_async_commit();
  }
  // solution values of the next block needed, fetched one step ahead
  using UB = typename SweepBits<T>::U;
  constexpr int KP = (kTS * NR + kSweepThreads - 1) / kSweepThreads;
  UB pre[KP];
  auto src_of = [&](int cb, int c, int q) -> const T* {
    const int64_t c0 = (int64_t)cb * kTS;
    return FWD ? &Y[(c0 + c) + q * ldy] : &Out[(c0 + c) + q * ldo];
  };
  auto prefetch = [&](int cb) {
    const int nc = (int)min((int64_t)kTS, n - (int64_t)cb * kTS);
#pragma unroll
    for (int k = 0; k < KP; ++k) {
      const int idx = tid + k * kSweepThreads;
      const int c = idx / NR, q = idx - c * NR;
      pre[k] = (idx < kTS * NR && q < nrhs && c < nc) ? SweepBits<T>::load(src_of(cb, c, q)) : UB(0);
    }
  };
  auto fill_sx = [&](int cb) -> int {
    const int nc = (int)min((int64_t)kTS, n - (int64_t)cb * kTS);
    int ok = 1;
#pragma unroll
    for (int k = 0; k < KP; ++k) {
      const int idx = tid + k * kSweepThreads;
      if (idx >= kTS * NR) continue;
      const int c = idx / NR, q = idx - c * NR;
      T v = T(0);
      if (q < nrhs && c < nc) {
        if (pre[k] != SweepBits<T>::kSentinel) v = SweepBits<T>::as_t(pre[k]);
        else if (!poll_value(src_of(cb, c, q), scr, &v)) ok = 0;
      }
      sx[c][q] = v;
    }
    return ok;
  };
  // this thread's half of a tile's columns times sx, added to (sign -1) or
  // into fresh sums (sign +1)
  auto half_product = [&](T(*tile)[tile_ld<T>()], T(&y)[4][NR], T sign) {
#pragma unroll 2
    for (int c = 32 * h; c < 32 * h + 32; c += 4) {
      const T m0 = sign * tile[c][r], m1 = sign * tile[c + 1][r], m2 = sign * tile[c + 2][r],
              m3 = sign * tile[c + 3][r];
#pragma unroll
      for (int q = 0; q < NR; ++q) {
        y[0][q] = fma(m0, sx[c][q], y[0][q]);
        y[1][q] = fma(m1, sx[c + 1][q], y[1][q]);
        y[2][q] = fma(m2, sx[c + 2][q], y[2][q]);
        y[3][q] = fma(m3, sx[c + 3][q], y[3][q]);
      }
    }
  };
  if (nlead > 0) prefetch(col_block(0));
  else if (noff > 0) prefetch(pcb);
  for (int t = 0; t < ntiles; ++t) {
    if (t + kStages - 1 < ntiles) issue(t + kStages - 1);
    cp_async_commit();
    cp_async_wait<kStages - 1>();
    __syncthreads();
    T(*tile)[tile_ld<T>()] = tiles[t % kStages];
    if (t < nlead) {  // an earlier off-diagonal block: b -= L_ij x_j
      const int ok = fill_sx(col_block(t));
      if (!__syncthreads_and(ok)) {
        cp_async_wait<0>();  // no copy may land after the CTA has left
        return;
      }
      prefetch(t + 1 < nlead ? col_block(t + 1) : pcb);
      half_product(tile, a, T(-1));
      continue;
    }
    if (t == nlead) {  // d = Inv_ii (right-hand side so far)
#pragma unroll
      for (int q = 0; q < NR; ++q) part[h][r][q] = (a[0][q] + a[1][q]) + (a[2][q] + a[3][q]);
      __syncthreads();
      if (h == 0)
#pragma unroll
        for (int q = 0; q < NR; ++q) sx[r][q] = valid ? part[0][r][q] + part[1][r][q] : T(0);
      __syncthreads();
      T y[4][NR];
#pragma unroll
      for (int j = 0; j < 4; ++j)
#pragma unroll
        for (int q = 0; q < NR; ++q) y[j][q] = T(0);
      half_product(tile, y, T(1));
#pragma unroll
      for (int q = 0; q < NR; ++q) part[h][r][q] = (y[0][q] + y[1][q]) + (y[2][q] + y[3][q]);
      __syncthreads();
      if (h == 0)
#pragma unroll
        for (int q = 0; q < NR; ++q) d[q] = part[0][r][q] + part[1][r][q];
      continue;
    }
    // the coupling: x = d - M_i x_p
    const int ok = fill_sx(pcb);
    if (!__syncthreads_and(ok)) {
      cp_async_wait<0>();
      return;
    }
    T y[4][NR];
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int q = 0; q < NR; ++q) y[j][q] = T(0);
    half_product(tile, y, T(1));
#pragma unroll
    for (int q = 0; q < NR; ++q) part[h][r][q] = (y[0][q] + y[1][q]) + (y[2][q] + y[3][q]);
    __syncthreads();
    if (h == 0)
#pragma unroll
      for (int q = 0; q < NR; ++q) d[q] -= part[0][r][q] + part[1][r][q];
  }
  cp_async_wait<0>();
  if (h == 0 && valid)
#pragma unroll
    for (int q = 0; q < NR; ++q)
      if (q < nrhs) {
        const T v = SweepBits<T>::canon(d[q]);
        if (FWD) Y[(r0 + r) + q * ldy] = v;
        else Out[(r0 + r) + q * ldo] = v;
      }
}

template <typename T>
constexpr size_t sweep_smem() { return (size_t)kStages * kTS * tile_ld<T>() * sizeof(T); }

// Inverses of the 64 x 64 diagonal blocks for the fast sweeps: CTA (b, 0)
// inverts the unit-lower L_bb, CTA (b, 1) the upper U_bb; thread j computes
// column j of the inverse in registers (substitution against e_j, the block
// in shared memory).  A ragged last block is padded with the identity.
// Output: inv[(b * kInvSlots + which) * 4096 + i + 64 j] = Inv(i, j).
template <typename T>
__global__ void __launch_bounds__(kTS)
diag_inverse_kernel(int64_t n, const T* __restrict__ LU, int64_t lda, T* __restrict__ inv) {
  __shared__ T s[kTS][kTS + 1];  // s[c][r] = block(r, c)
  const int b = blockIdx.x, which = blockIdx.y;
  const int64_t r0 = (int64_t)b * kTS;
  const int nb = (int)min((int64_t)kTS, n - r0);
  const int j = threadIdx.x;
  for (int idx = j; idx < kTS * kTS; idx += kTS) {
    const int c = idx >> 6, r = idx & 63;
    T v = (r < nb && c < nb) ? LU[(r0 + r) + (r0 + c) * lda] : T(0);
    if (r == c && r >= nb) v = T(1);
    s[c][r] = v;
  }
  __syncthreads();
  T x[kTS];
#pragma unroll
  for (int i = 0; i < kTS; ++i) x[i] = (i == j) ? T(1) : T(0);
  if (which == 0) {  // L_bb unit lower: forward substitution
#pragma unroll
    for (int k = 0; k < kTS; ++k)
#pragma unroll
      for (int i = k + 1; i < kTS; ++i) x[i] = fma(-s[k][i], x[k], x[i]);
  } else {  // U_bb upper: backward substitution
#pragma unroll
    for (int k = kTS - 1; k >= 0; --k) {
      x[k] = x[k] / s[k][k];
#pragma unroll
      for (int i = 0; i < k; ++i) x[i] = fma(-s[k][i], x[k], x[i]);
    }
  }
  T* out = inv + ((int64_t)b * kInvSlots + which) * (kTS * kTS) + (int64_t)j * kTS;
#pragma unroll
  for (int i = 0; i < kTS; ++i) out[i] = x[i];
}

// The couplings of the fast 'N' sweeps: slot 2 of block b = InvL_bb L_{b,b-1}
// (b >= 1), slot 3 = InvU_bb U_{b,b+1} (b <= nblk - 2); zero where there is
// no such block and outside ragged edges.  Thread (r, g): row r, columns
// 16 g .. 16 g + 15 of the product.
template <typename T>
__global__ void __launch_bounds__(256)
fold_kernel(int64_t n, const T* __restrict__ LU, int64_t lda, T* __restrict__ inv) {
  __shared__ T sO[kTS][kTS + 1];  // sO[c][k] = O(k, c), O the off-diagonal block
  const int b = blockIdx.x, which = blockIdx.y;
  const int64_t nblk = (n + kTS - 1) / kTS;
  T* out = inv + ((int64_t)b * kInvSlots + 2 + which) * (kTS * kTS);
  const int64_t ob = which == 0 ? (int64_t)b - 1 : (int64_t)b + 1;
  const int tid = threadIdx.x;
  if (ob < 0 || ob >= nblk) {
    for (int idx = tid; idx < kTS * kTS; idx += 256) out[idx] = T(0);
    return;
  }
  const int64_t r0 = (int64_t)b * kTS, c0 = ob * kTS;
  const int nb = (int)min((int64_t)kTS, n - r0), nc = (int)min((int64_t)kTS, n - c0);
  const T* I = inv + ((int64_t)b * kInvSlots + which) * (kTS * kTS);
  for (int idx = tid; idx < kTS * kTS; idx += 256) {
    const int c = idx >> 6, k = idx & 63;
    sO[c][k] = (k < nb && c < nc) ? LU[(r0 + k) + (c0 + c) * lda] : T(0);
  }
  __syncthreads();
  const int r = tid & 63, g = tid >> 6;
  T acc[16];
#pragma unroll
  for (int j = 0; j < 16; ++j) acc[j] = T(0);
  for (int k = 0; k < kTS; ++k) {
    const T a = I[r + k * kTS];  // Inv(r, k), coalesced over r
#pragma unroll
    for (int j = 0; j < 16; ++j) acc[j] = fma(a, sO[16 * g + j][k], acc[j]);
  }
#pragma unroll
  for (int j = 0; j < 16; ++j) out[r + (int64_t)(16 * g + j) * kTS] = r < nb ? acc[j] : T(0);
}

size_t getrs_inverse_bytes(int64_t n, int elem_size) {
  const int64_t nblk = (n + kTS - 1) / kTS;
  return (size_t)std::max<int64_t>(nblk, 1) * kInvSlots * kTS * kTS * elem_size;
}

template <typename T>
cudaError_t getrs_invert_launch(const GetrsPlan<T>& p, cudaStream_t s) {
  if (p.n <= 0) return cudaSuccess;
  if (!p.inv) return cudaErrorInvalidValue;
  const int64_t nblk = (p.n + kTS - 1) / kTS;
  LaunchScope ls(K_SOLVE, (double)nblk * 2.0 * kTS * kTS * kTS / 3.0,
                 (double)nblk * 3.0 * kTS * kTS * sizeof(T), s);
  diag_inverse_kernel<T><<<dim3((unsigned)nblk, 2), kTS, 0, s>>>(p.n, p.LU, p.lda, p.inv);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  LaunchScope ls2(K_SOLVE, (double)nblk * 4.0 * kTS * kTS * kTS, (double)nblk * 6.0 * kTS * kTS * sizeof(T), s);
  fold_kernel<T><<<dim3((unsigned)nblk, 2), 256, 0, s>>>(p.n, p.LU, p.lda, p.inv);
  return cudaGetLastError();
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
template <typename T, int NR, bool FAST>
cudaError_t run_chunk(const GetrsPlan<T>& p, char trans, int nr, T* B, int64_t ldb,
                      cudaStream_t s) {
  const int64_t nblk = (p.n + kTS - 1) / kTS;
  int32_t* ffwd = p.flags;
  int32_t* fbwd = p.flags + nblk;
  // dependents poll Y (forward) and B (backward): fill both with the sentinel
  cudaError_t e = cudaMemsetAsync(p.work, 0xFF, (size_t)p.n * nr * sizeof(T), s);
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(&p.scratch->ticket, 0, sizeof(unsigned), s);
  if (e != cudaSuccess) return e;
  const bool tr = trans == 'T' || trans == 't' || trans == 'C' || trans == 'c';
  // algorithmic work of one sweep: the triangle (n^2/2 elements) read once,
  // n^2 flops per right-hand side
  const double tri_bytes = 0.5 * (double)p.n * (double)p.n * sizeof(T) + 2.0 * p.n * nr * sizeof(T);
  const double sweep_flops = (double)p.n * (double)p.n * nr;
  const size_t smem = sweep_smem<T>();
  {
    LaunchScope ls(K_SOLVE, sweep_flops, tri_bytes, s);
    if (FAST && !tr)
      fast_sweep_kernel<T, NR, true><<<(unsigned)nblk, kSweepThreads, smem, s>>>(
          p.n, p.LU, p.lda, p.perm, B, ldb, p.work, p.n, nullptr, 0, nr, p.scratch, p.inv);
    else if (!tr)
      solve_sweep_kernel<T, NR, false, true, FAST><<<(unsigned)nblk, kSweepThreads, smem, s>>>(
          p.n, p.LU, p.lda, p.perm, B, ldb, p.work, p.n, nullptr, 0, nr, ffwd, p.scratch, p.inv);
    else
      solve_sweep_kernel<T, NR, true, true, FAST><<<(unsigned)nblk, kSweepThreads, smem, s>>>(
          p.n, p.LU, p.lda, p.perm, B, ldb, p.work, p.n, nullptr, 0, nr, ffwd, p.scratch, p.inv);
  }
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(&p.scratch->ticket, 0, sizeof(unsigned), s);
  if (e != cudaSuccess) return e;
  e = cudaMemset2DAsync(B, ldb * sizeof(T), 0xFF, p.n * sizeof(T), nr, s);
  if (e != cudaSuccess) return e;
  LaunchScope ls(K_SOLVE, sweep_flops, tri_bytes, s);
  if (FAST && !tr)
    fast_sweep_kernel<T, NR, false><<<(unsigned)nblk, kSweepThreads, smem, s>>>(
        p.n, p.LU, p.lda, p.perm, nullptr, 0, p.work, p.n, B, ldb, nr, p.scratch, p.inv);
  else if (!tr)
    solve_sweep_kernel<T, NR, false, false, FAST><<<(unsigned)nblk, kSweepThreads, smem, s>>>(
        p.n, p.LU, p.lda, p.perm, nullptr, 0, p.work, p.n, B, ldb, nr, fbwd, p.scratch, p.inv);
  else
    solve_sweep_kernel<T, NR, true, false, FAST><<<(unsigned)nblk, kSweepThreads, smem, s>>>(
        p.n, p.LU, p.lda, p.perm, nullptr, 0, p.work, p.n, B, ldb, nr, fbwd, p.scratch, p.inv);
  return cudaGetLastError();
}

template <typename T, int NR>
cudaError_t run_chunk_mode(const GetrsPlan<T>& p, char trans, int nr, T* B, int64_t ldb, cudaStream_t s) {
  return (p.fast && p.inv) ? run_chunk<T, NR, true>(p, trans, nr, B, ldb, s)
                           : run_chunk<T, NR, false>(p, trans, nr, B, ldb, s);
}
}  // namespace

template <typename T, int NR, bool FAST>
void configure_nr_mode() {
  const int b = (int)sweep_smem<T>();
  cudaFuncSetAttribute(solve_sweep_kernel<T, NR, false, true, FAST>, cudaFuncAttributeMaxDynamicSharedMemorySize, b);
  cudaFuncSetAttribute(solve_sweep_kernel<T, NR, true, true, FAST>, cudaFuncAttributeMaxDynamicSharedMemorySize, b);
  cudaFuncSetAttribute(solve_sweep_kernel<T, NR, false, false, FAST>, cudaFuncAttributeMaxDynamicSharedMemorySize, b);
  cudaFuncSetAttribute(solve_sweep_kernel<T, NR, true, false, FAST>, cudaFuncAttributeMaxDynamicSharedMemorySize, b);
  if (FAST) {
    cudaFuncSetAttribute(fast_sweep_kernel<T, NR, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, b);
    cudaFuncSetAttribute(fast_sweep_kernel<T, NR, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, b);
  }
}

template <typename T, int NR>
void configure_nr() {
  configure_nr_mode<T, NR, false>();
  configure_nr_mode<T, NR, true>();
}

void getrs_configure(int /*device*/) {
  configure_nr<double, 1>(); configure_nr<double, 2>(); configure_nr<double, 4>(); configure_nr<double, 8>();
  configure_nr<float, 1>(); configure_nr<float, 2>(); configure_nr<float, 4>(); configure_nr<float, 8>();
}

template <typename T>
cudaError_t getrs_launch(const GetrsPlan<T>& p, char trans, int64_t nrhs, T* B, int64_t ldb,
                         uint32_t* /*epoch*/, cudaStream_t s) {
  if (p.n <= 0 || nrhs <= 0) return cudaSuccess;
  const int64_t chunk = std::min<int64_t>(p.work_cols, 8);
  for (int64_t c = 0; c < nrhs; c += chunk) {
    int nr = (int)std::min<int64_t>(chunk, nrhs - c);
    T* Bc = B + c * ldb;
    cudaError_t e;
    if (nr == 1) e = run_chunk_mode<T, 1>(p, trans, nr, Bc, ldb, s);
    else if (nr == 2) e = run_chunk_mode<T, 2>(p, trans, nr, Bc, ldb, s);
    else if (nr <= 4) e = run_chunk_mode<T, 4>(p, trans, nr, Bc, ldb, s);
    else e = run_chunk_mode<T, 8>(p, trans, nr, Bc, ldb, s);
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
template cudaError_t getrs_invert_launch<double>(const GetrsPlan<double>&, cudaStream_t);
template cudaError_t getrs_invert_launch<float>(const GetrsPlan<float>&, cudaStream_t);

}  // namespace gblu
