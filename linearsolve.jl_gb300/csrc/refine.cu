// Mixed-precision solve: FP32 factors + FP64 iterative refinement / GMRES-IR.
//
// No counterpart in the reference: LinearSolve.jl's *32Mixed* algorithms
// (src/openblas.jl:461-543, ext/LinearSolveCUDAExt.jl:211-242) factor and
// solve in FP32 and stop.  Here only the residual r = b - A x, the update
// x += d and the convergence test run in FP64; the correction is solved with
// the FP32 factors (IR) or by FP64 GMRES preconditioned by them (GMRES-IR,
// Carson & Higham, SIAM J. Sci. Comput. 40(2), 2018).  Every reduction has a
// fixed order, so a solve's result does not depend on what else runs on the
// device.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "device_util.cuh"
#include "gblu_internal.h"
#include "objects.h"
#include "profile.h"
#include "refine.h"

namespace gblu {

constexpr int kRowsPerCta = 256;
constexpr int kXTile = 128;  // columns of X staged in shared memory at a time
constexpr int kMaxW = 8;

// ---------------------------------------------------------------------------
// kernels

__device__ __forceinline__ void atomic_max_nonneg(unsigned long long* p, double v) {
  // non-negative doubles order like their bit patterns; NaN maps above +inf
  unsigned long long bits = isnan(v) ? 0x7ff8000000000000ull : (unsigned long long)__double_as_longlong(v);
  atomicMax(p, bits);
}

// Block-wide max of non-negative v (NaN wins) folded into *p by thread 0.
__device__ __forceinline__ void block_max_into(double v, unsigned long long* p) {
  __shared__ double red[32];
  for (int off = 16; off; off >>= 1) {
    const double o = __shfl_down_sync(0xffffffffu, v, off);
    v = (o > v || isnan(o)) ? o : v;
  }
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double m = 0.0;
    for (int w = 0; w < (int)((blockDim.x + 31) >> 5); ++w) m = (red[w] > m || isnan(red[w])) ? red[w] : m;
    atomic_max_nonneg(p, m);
  }
}

// One pass over the FP64 matrix before the low-precision getrf: B = float(A),
// P[s][i] = sum of |A_ij| over the columns j of chunk s (kPrepChunks column
// chunks, j ascending), and max |A_ij| into *amax.  A CTA covers 1024
// consecutive rows (4 per thread, 8 KB of a column per step) of one chunk,
// so every column step is one long contiguous read; prepare_reduce_kernel
// adds the chunks in index order.  Only the row sums use the FP64 pipe: the
// conversion, |a| and the maximum (over the bit patterns of |a|, which order
// like the values, NaN above infinity) run on the integer pipe.
constexpr int kPrepChunks = 64;
constexpr int kPrepRows = 1024;

template <bool WRITE>
__global__ void __launch_bounds__(256)
prepare_kernel(int64_t n, const double* __restrict__ A, int64_t lda, float* __restrict__ B, int64_t ldb,
               double* __restrict__ P, unsigned long long* __restrict__ amax) {
  const int s = blockIdx.y;
  const int64_t cs = (n + kPrepChunks - 1) / kPrepChunks;
  const int64_t j0 = s * cs, j1 = min(n, j0 + cs);
  const int64_t i0 = (int64_t)blockIdx.x * kPrepRows + threadIdx.x;
  double acc[4] = {0.0, 0.0, 0.0, 0.0};
  long long mxb = 0;  // bits of the largest |a| so far
  bool ok[4];
#pragma unroll
  for (int r = 0; r < 4; ++r) ok[r] = i0 + 256 * r < n;
#pragma unroll 2
  for (int64_t j = j0; j < j1; ++j) {
    const double* a = A + i0 + j * lda;
    float* b = B + i0 + j * ldb;
    double v[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) v[r] = ok[r] ? a[256 * r] : 0.0;
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      if (WRITE && ok[r]) b[256 * r] = f64_to_f32_rn(v[r]);
      const long long ab = __double_as_longlong(v[r]) & 0x7FFFFFFFFFFFFFFFll;
      acc[r] += __longlong_as_double(ab);
      mxb = ab > mxb ? ab : mxb;
    }
  }
#pragma unroll
  for (int r = 0; r < 4; ++r)
    if (ok[r]) P[(size_t)s * n + i0 + 256 * r] = acc[r];
  block_max_into(__longlong_as_double(mxb), amax);
}

// ---------------------------------------------------------------------------
// Random butterfly transform.  A butterfly of order m is B = [R S; R -S]
// (R, S diagonal of order m/2); the depth-2 transform of one side is
// W = B1 diag(B2a, B2b) (B1 of order n, B2a / B2b of order n/2), with the
// 1/sqrt(2) of each level gathered into one exact 1/2.  Rows i, i + n/4,
// i + n/2, i + 3n/4 (i < n/4) only mix with each other: an orbit.
//   W^T v:  level 1 then level 2 of  v_i, v_{i+h} -> R_i (v_i + v_{i+h}), S_i (v_i - v_{i+h})
//   W v:    level 2 then level 1 of  v_i, v_{i+h} -> R_i v_i + S_i v_{i+h}, R_i v_i - S_i v_{i+h}
// The transformed matrix only feeds the low-precision factorization, so it
// is formed in FP32 (inputs narrowed with the integer-pipe conversion).

struct RbtSide {
  const float *R1, *S1, *R2, *S2;
  __device__ RbtSide(const float* rbt, int64_t n, int side) {
    const float* b = rbt + (size_t)side * 2 * n;
    R1 = b; S1 = b + n / 2; R2 = b + n; S2 = b + 3 * n / 2;
  }
  // x[0..3] = the orbit of a (offsets 0, n/4, n/2, 3n/4): x := W^T x (no 1/2)
  __device__ __forceinline__ void t_form(float (&x)[4], int64_t a, int64_t h2) const {
    const float y0 = R1[a] * (x[0] + x[2]), y2 = S1[a] * (x[0] - x[2]);
    const float y1 = R1[a + h2] * (x[1] + x[3]), y3 = S1[a + h2] * (x[1] - x[3]);
    x[0] = R2[a] * (y0 + y1);
    x[1] = S2[a] * (y0 - y1);
    x[2] = R2[h2 + a] * (y2 + y3);
    x[3] = S2[h2 + a] * (y2 - y3);
  }
  // x := W x (no 1/2)
  __device__ __forceinline__ void n_form(float (&x)[4], int64_t a, int64_t h2) const {
    const float y0 = R2[a] * x[0] + S2[a] * x[1], y1 = R2[a] * x[0] - S2[a] * x[1];
    const float y2 = R2[h2 + a] * x[2] + S2[h2 + a] * x[3], y3 = R2[h2 + a] * x[2] - S2[h2 + a] * x[3];
    x[0] = R1[a] * y0 + S1[a] * y2;
    x[2] = R1[a] * y0 - S1[a] * y2;
    x[1] = R1[a + h2] * y1 + S1[a + h2] * y3;
    x[3] = R1[a + h2] * y1 - S1[a + h2] * y3;
  }
};

// B = U^T A V / 4: thread (a, b) takes the 4 x 4 block of row orbit a and
// column orbit b.  Consecutive threads take consecutive rows (coalesced).
__global__ void __launch_bounds__(128)
rbt_matrix_kernel(int64_t n, const double* __restrict__ A, int64_t lda, float* __restrict__ B, int64_t ldb,
                  const float* __restrict__ rbt) {
  const int64_t h2 = n / 4;
  const int64_t a = (int64_t)blockIdx.x * blockDim.x + threadIdx.x, b = blockIdx.y;
  if (a >= h2) return;
  const RbtSide L(rbt, n, 0), Rt(rbt, n, 1);
  float x[4][4];  // x[i][j]: row orbit member i, column orbit member j
#pragma unroll
  for (int j = 0; j < 4; ++j)
#pragma unroll
    for (int i = 0; i < 4; ++i) x[i][j] = f64_to_f32_rn(A[(a + i * h2) + (b + j * h2) * lda]);
#pragma unroll
  for (int j = 0; j < 4; ++j) {  // rows: U^T
    float c[4] = {x[0][j], x[1][j], x[2][j], x[3][j]};
    L.t_form(c, a, h2);
#pragma unroll
    for (int i = 0; i < 4; ++i) x[i][j] = c[i];
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) Rt.t_form(x[i], b, h2);  // columns: V (A V = (V^T A^T)^T)
#pragma unroll
  for (int j = 0; j < 4; ++j)
#pragma unroll
    for (int i = 0; i < 4; ++i) B[(a + i * h2) + (b + j * h2) * ldb] = 0.25f * x[i][j];
}

// The rows and columns past the butterflies' order n4 (fewer than four of
// each): the transforms are diag(W, I), so the extra rows take the column
// transform only, the extra columns the row transform only, and the corner
// is copied.  blockIdx.y: extra row y (y < r), extra column y - r (y < 2r),
// the corner (y = 2r).
__global__ void __launch_bounds__(128)
rbt_edge_kernel(int64_t n, int64_t n4, const double* __restrict__ A, int64_t lda, float* __restrict__ B,
                int64_t ldb, const float* __restrict__ rbt) {
  const int64_t h2 = n4 / 4, r = n - n4;
  const int64_t y = blockIdx.y;
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (y < r) {
    if (t >= h2) return;
    const RbtSide Rt(rbt, n4, 1);
    const int64_t i = n4 + y;
    float x[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) x[j] = f64_to_f32_rn(A[i + (t + j * h2) * lda]);
    Rt.t_form(x, t, h2);
#pragma unroll
    for (int j = 0; j < 4; ++j) B[i + (t + j * h2) * ldb] = 0.5f * x[j];
  } else if (y < 2 * r) {
    if (t >= h2) return;
    const RbtSide L(rbt, n4, 0);
    const int64_t c = n4 + (y - r);
    float x[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) x[i] = f64_to_f32_rn(A[(t + i * h2) + c * lda]);
    L.t_form(x, t, h2);
#pragma unroll
    for (int i = 0; i < 4; ++i) B[(t + i * h2) + c * ldb] = 0.5f * x[i];
  } else {
    if (t >= r * r) return;
    const int64_t i = n4 + t % r, c = n4 + t / r;
    B[i + c * ldb] = f64_to_f32_rn(A[i + c * lda]);
  }
}

// v := W^T v / 2 or W v / 2, W columns of v.
__global__ void __launch_bounds__(256)
rbt_vec_kernel(int64_t n, int W, float* __restrict__ v, int64_t ldv, const float* __restrict__ rbt, int side,
               int transposed) {
  const int64_t h2 = n / 4;
  const int64_t a = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int q = blockIdx.y;
  if (a >= h2 || q >= W) return;
  const RbtSide S(rbt, n, side);
  float* c = v + (size_t)q * ldv;
  float x[4] = {c[a], c[a + h2], c[a + 2 * h2], c[a + 3 * h2]};
  if (transposed) S.t_form(x, a, h2);
  else S.n_form(x, a, h2);
#pragma unroll
  for (int i = 0; i < 4; ++i) c[a + i * h2] = 0.5f * x[i];
}

// ||A||_inf = max_i sum_s P[s][i] (chunks added in index order) into *anorm.
__global__ void __launch_bounds__(256)
prepare_reduce_kernel(int64_t n, const double* __restrict__ P, unsigned long long* __restrict__ anorm) {
  double mx = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    double sum = 0.0;
    for (int s = 0; s < kPrepChunks; ++s) sum += P[(size_t)s * n + i];
    mx = (sum > mx || isnan(sum)) ? sum : mx;
  }
  block_max_into(mx, anorm);
}

// max |U_ij| over the upper triangle of the n x n FP32 factors: one warp per
// column (rows 0..j, 32 consecutive rows per load), eight columns per CTA.
__global__ void __launch_bounds__(256)
umax_kernel(int64_t n, const float* __restrict__ LU, int64_t ld, unsigned long long* __restrict__ umax) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t j = (int64_t)blockIdx.x * 8 + warp;
  float mx = 0.f;
  if (j < n) {
    const float* col = LU + j * ld;
#pragma unroll 4
    for (int64_t i = lane; i <= j; i += 32) {
      const float v = fabsf(col[i]);
      mx = (v > mx || isnan(v)) ? v : mx;
    }
  }
  block_max_into((double)mx, umax);
}

// P[s][q][i] = sum_{j in chunk s} op(A)[i, j] * X[j, q]
//   'N': op(A)[i,j] = A[i + j*lda], A is rows x cols, i < rows
//   'T': op(A)[i,j] = A[j + i*lda], i < cols (one warp per output row)
// Chunks are fixed by (cols or rows) and kSplit, so the sum order is fixed.
// ABS (|A| x, for the backward error's denominator) is a compile-time
// switch: on this GPU a predicated-off FP64 instruction still occupies the
// FP64 pipe, so a runtime flag would cost the plain residual a fifth more.
template <int W, bool ABS>
__global__ void __launch_bounds__(kRowsPerCta)
gemv_n_partial_kernel(int64_t rows, int64_t cols, const double* __restrict__ A, int64_t lda,
                      const double* __restrict__ X, int64_t ldx, int wreal, double* __restrict__ P) {
  __shared__ double sx[kXTile][W];
  const int s = blockIdx.y;
  const int64_t cs = (cols + kSplit - 1) / kSplit;
  const int64_t j0 = s * cs, j1 = min(cols, j0 + cs);
  const int64_t i = (int64_t)blockIdx.x * kRowsPerCta + threadIdx.x;
  double acc[W];
#pragma unroll
  for (int q = 0; q < W; ++q) acc[q] = 0.0;
  for (int64_t jt = j0; jt < j1; jt += kXTile) {
    const int nt = (int)min((int64_t)kXTile, j1 - jt);
    __syncthreads();
    for (int idx = threadIdx.x; idx < nt * W; idx += blockDim.x) {
      const int jj = idx / W, q = idx - jj * W;
      sx[jj][q] = X ? (q < wreal ? X[(jt + jj) + q * ldx] : 0.0) : 1.0;
    }
    __syncthreads();
    if (i < rows) {
      const double* a = A + i + jt * lda;
#pragma unroll 4
      for (int jj = 0; jj < nt; ++jj) {
        double v = a[jj * lda];
        if constexpr (ABS) v = fabs(v);
#pragma unroll
        for (int q = 0; q < W; ++q) acc[q] = fma(v, sx[jj][q], acc[q]);
      }
    }
  }
  if (i < rows)
#pragma unroll
    for (int q = 0; q < W; ++q) P[((size_t)s * W + q) * rows + i] = acc[q];
}

template <int W>
__global__ void __launch_bounds__(256)
gemv_t_partial_kernel(int64_t rows, int64_t cols, const double* __restrict__ A, int64_t lda,
                      const double* __restrict__ X, int64_t ldx, int wreal, double* __restrict__ P) {
  const int s = blockIdx.y;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t i = (int64_t)blockIdx.x * 8 + warp;  // output index = column of A
  const int64_t cs = (rows + kSplit - 1) / kSplit;
  const int64_t j0 = s * cs, j1 = min(rows, j0 + cs);
  if (i >= cols) return;
  double acc[W];
#pragma unroll
  for (int q = 0; q < W; ++q) acc[q] = 0.0;
  const double* a = A + i * lda;
  for (int64_t j = j0 + lane; j < j1; j += 32) {
    const double v = a[j];
#pragma unroll
    for (int q = 0; q < W; ++q) acc[q] = fma(v, q < wreal ? X[j + q * ldx] : 0.0, acc[q]);
  }
#pragma unroll
  for (int q = 0; q < W; ++q) {
    double v = acc[q];
    for (int off = 16; off; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
    if (lane == 0) P[((size_t)s * W + q) * cols + i] = v;
  }
}

// out[i,q] = beta*C[i,q] + alpha*sum_s P[s][q][i]; optional column max of |out|.
__global__ void gemv_reduce_kernel(int64_t len, int W, int Wp, const double* __restrict__ P, double alpha,
                                   const double* __restrict__ C, int64_t ldc, double beta,
                                   double* __restrict__ out, int64_t ldo,
                                   unsigned long long* __restrict__ colmax) {
  __shared__ double red[256 / 32];
  for (int q = 0; q < W; ++q) {
    double mx = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < len;
         i += (int64_t)gridDim.x * blockDim.x) {
      double sum = 0.0;
      for (int s = 0; s < kSplit; ++s) sum += P[((size_t)s * Wp + q) * len + i];
      double v = alpha * sum;
      if (beta != 0.0) v = fma(beta, C[i + q * ldc], v);
      out[i + q * ldo] = v;
      double av = fabs(v);
      mx = (av > mx || isnan(av)) ? av : mx;
    }
    if (colmax) {
      for (int off = 16; off; off >>= 1) {
        double o = __shfl_down_sync(0xffffffffu, mx, off);
        mx = (o > mx || isnan(o)) ? o : mx;
      }
      if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = mx;
      __syncthreads();
      if (threadIdx.x == 0) {
        double m = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) m = (red[w] > m || isnan(red[w])) ? red[w] : m;
        atomic_max_nonneg(colmax + q, m);
      }
      __syncthreads();
    }
  }
}

__global__ void colmax_kernel(int64_t n, int W, const double* __restrict__ X, int64_t ldx,
                              unsigned long long* __restrict__ colmax) {
  __shared__ double red[256 / 32];
  for (int q = 0; q < W; ++q) {
    double mx = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
      double av = fabs(X[i + q * ldx]);
      mx = (av > mx || isnan(av)) ? av : mx;
    }
    for (int off = 16; off; off >>= 1) {
      double o = __shfl_down_sync(0xffffffffu, mx, off);
      mx = (o > mx || isnan(o)) ? o : mx;
    }
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = mx;
    __syncthreads();
    if (threadIdx.x == 0) {
      double m = 0.0;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) m = (red[w] > m || isnan(red[w])) ? red[w] : m;
      atomic_max_nonneg(colmax + q, m);
    }
    __syncthreads();
  }
}

// Per-column power-of-two scale from the column maxima (bit patterns):
// sc[q] = 1 / 2^ilogb(max), sc[kMaxW + q] = 2^ilogb(max) (1 for a zero or
// non-finite maximum), so the FP32 right-hand side is O(1).
__global__ void pow2_scales_kernel(int W, const unsigned long long* __restrict__ colmax,
                                   double* __restrict__ sc) {
  const int q = threadIdx.x;
  if (q >= W) return;
  const double m = __longlong_as_double((long long)colmax[q]);
  const double scale = (m > 0 && isfinite(m)) ? ldexp(1.0, ilogb(m)) : 1.0;
  sc[q] = 1.0 / scale;
  sc[kMaxW + q] = scale;
}

// D[:,q] = float(R[:,q] * inv_scale[q])
__global__ void scale_to_f32_kernel(int64_t n, int W, const double* __restrict__ R, int64_t ldr,
                                    const double* __restrict__ inv_scale, float* __restrict__ D,
                                    int64_t ldd) {
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < n * W;
       idx += (int64_t)gridDim.x * blockDim.x) {
    int q = (int)(idx / n);
    int64_t i = idx - (int64_t)q * n;
    D[i + q * ldd] = (float)(R[i + q * ldr] * inv_scale[q]);
  }
}

// X[:,q] = beta*X[:,q] + scale[q] * double(D[:,q])
__global__ void update_from_f32_kernel(int64_t n, int W, double* __restrict__ X, int64_t ldx,
                                       const float* __restrict__ D, int64_t ldd,
                                       const double* __restrict__ scale, double beta) {
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < n * W;
       idx += (int64_t)gridDim.x * blockDim.x) {
    int q = (int)(idx / n);
    int64_t i = idx - (int64_t)q * n;
    double d = scale[q] * (double)D[i + q * ldd];
    X[i + q * ldx] = beta == 0.0 ? d : fma(beta, X[i + q * ldx], d);
  }
}

// Sum of squares of each of W columns, in two fixed-order passes: block b of
// column q sums rows b, b + kSumBlocks*256, ... (strided per thread, then a
// shuffle / shared-memory tree) into part[q][b]; sumsq_final adds part[q][*]
// in index order.  The result does not depend on scheduling.
constexpr int kSumBlocks = 64;

__global__ void __launch_bounds__(256)
sumsq_partial_kernel(int64_t n, const double* __restrict__ X, int64_t ldx, double* __restrict__ part) {
  __shared__ double red[8];
  const int q = blockIdx.y;
  double acc = 0.0;
  for (int64_t i = blockIdx.x * 256 + threadIdx.x; i < n; i += (int64_t)kSumBlocks * 256) {
    const double v = X[i + q * ldx];
    acc = fma(v, v, acc);
  }
  for (int off = 16; off; off >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, off);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < 8; ++w) s += red[w];
    part[q * kSumBlocks + blockIdx.x] = s;
  }
}

__global__ void sumsq_final_kernel(int W, const double* __restrict__ part, double* __restrict__ out) {
  const int q = threadIdx.x;
  if (q >= W) return;
  double s = 0.0;
  for (int b = 0; b < kSumBlocks; ++b) s += part[q * kSumBlocks + b];
  out[q] = s;
}

// ---- GMRES(m) bookkeeping on the device, one thread per RHS column ----
// State of column q: gm + q * kGmStride (H, rotations, g, y, beta, 1/norm of
// the newest basis vector); flags gflags[2q] = still extending its basis,
// gflags[2q + 1] = basis size k.  A column that stopped keeps its state and
// gets 1/norm = 0, so its later basis vectors are zero and stay finite.

// beta_q = ||z_q||_2 from the squared norm in hn2[q] (columns outside run_mask
// do not step), g = beta e_1.
__global__ void gmres_begin_kernel(int nc, unsigned run_mask, const double* __restrict__ hn2,
                                   double* __restrict__ gm, int* __restrict__ gflags) {
  const int q = threadIdx.x;
  if (q >= nc) return;
  double* st = gm + (size_t)q * kGmStride;
  int* fl = gflags + 2 * q;
  const double beta = ((run_mask >> q) & 1u) ? sqrt(hn2[q]) : 0.0;
  const bool step = beta > 0 && isfinite(beta);
  for (int i = 0; i <= kGmresRestart; ++i) {
    st[kGmG + i] = 0.0;
    st[kGmY + i] = 0.0;
  }
  st[kGmG] = beta;
  st[kGmBeta] = beta;
  st[kGmInv] = step ? 1.0 / beta : 0.0;
  fl[0] = step ? 1 : 0;
  fl[1] = 0;
}

// V_q(:, j) *= 1/norm_q for the nc bases (column q's basis starts at V + q * ldV).
__global__ void gmres_scale_kernel(int64_t n, int nc, double* __restrict__ V, int64_t ldV, int j,
                                   const double* __restrict__ gm) {
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < n * nc;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int q = (int)(idx / n);
    const int64_t i = idx - (int64_t)q * n;
    double* v = V + (size_t)q * ldV + (size_t)j * n + i;
    *v = gm[(size_t)q * kGmStride + kGmInv] * *v;
  }
}

// Step j of each stepping column: Hessenberg column from the two projection
// passes and the norm (h: [q][pass 0, 1, norm^2][m + 1]), the previous Givens
// rotations, the new rotation, g, the stopping test |g_{j+1}| <= rtol beta.
__global__ void gmres_step_kernel(int nc, int j, int m, const double* __restrict__ h, double rtol,
                                  double* __restrict__ gm, int* __restrict__ gflags) {
  const int q = threadIdx.x;
  if (q >= nc) return;
  double* st = gm + (size_t)q * kGmStride;
  int* fl = gflags + 2 * q;
  if (!fl[0]) {
    st[kGmInv] = 0.0;
    return;
  }
  const int hs = kGmresRestart + 1;
  const double* h1 = h + (size_t)(q * 3) * hs;
  const double* h2 = h1 + hs;
  const double hn = sqrt(h1[2 * hs]);
  double* Hj = st + kGmH + (size_t)j * (m + 1);
  double* cs = st + kGmCs;
  double* sn = st + kGmSn;
  double* g = st + kGmG;
  for (int i = 0; i <= j; ++i) Hj[i] = h1[i] + h2[i];
  Hj[j + 1] = hn;
  for (int i = 0; i < j; ++i) {
    const double a = Hj[i], b = Hj[i + 1];
    Hj[i] = cs[i] * a + sn[i] * b;
    Hj[i + 1] = -sn[i] * a + cs[i] * b;
  }
  const double a = Hj[j], b = Hj[j + 1];
  const double rr = hypot(a, b);
  cs[j] = rr > 0 ? a / rr : 1.0;
  sn[j] = rr > 0 ? b / rr : 0.0;
  Hj[j] = rr;
  Hj[j + 1] = 0.0;
  g[j + 1] = -sn[j] * g[j];
  g[j] = cs[j] * g[j];
  fl[1] = j + 1;
  if (fabs(g[j + 1]) <= rtol * st[kGmBeta] || !(hn > 0) || !isfinite(hn)) {
    fl[0] = 0;
    st[kGmInv] = 0.0;
  } else {
    st[kGmInv] = 1.0 / hn;
  }
}

// y_q = H_q(1:k, 1:k) \ g_q(1:k) by back substitution, into y_out + q * hs.
__global__ void gmres_finish_kernel(int nc, int m, const double* __restrict__ gm,
                                    const int* __restrict__ gflags, double* __restrict__ y_out) {
  const int q = threadIdx.x;
  if (q >= nc) return;
  const int hs = kGmresRestart + 1;
  const double* st = gm + (size_t)q * kGmStride;
  const double* H = st + kGmH;
  const double* g = st + kGmG;
  const int k = gflags[2 * q + 1];
  double* y = y_out + (size_t)q * hs;
  for (int i = 0; i < hs; ++i) y[i] = 0.0;
  for (int i = k - 1; i >= 0; --i) {
    double acc = g[i];
    for (int jj = i + 1; jj < k; ++jj) acc -= H[(size_t)jj * (m + 1) + i] * y[jj];
    const double d = H[(size_t)i * (m + 1) + i];
    y[i] = d != 0 ? acc / d : 0.0;
  }
}

// Y = a*X + b*Y
__global__ void axpby_kernel(int64_t n, double a, const double* __restrict__ X, double b,
                             double* __restrict__ Y) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    Y[i] = b == 0.0 ? a * X[i] : fma(a, X[i], b * Y[i]);
}

// ---------------------------------------------------------------------------
// buffers

size_t refine_bytes(int64_t n, int64_t W) {
  size_t b = 0;
  b += 3 * align256((size_t)n * W * sizeof(double));       // x, r, b
  b += align256((size_t)n * W * sizeof(float));            // d32
  size_t pe = (size_t)kSplit * std::max<int64_t>(n, kGmresRestart + 1) * W;
  b += align256(pe * sizeof(double));                      // partial
  b += align256((size_t)n * (kGmresRestart + 1) * W * sizeof(double));  // V
  b += align256((size_t)n * W * sizeof(double));           // w
  b += align256(3 * (kGmresRestart + 1) * W * sizeof(double));  // h
  b += align256(4 * W * sizeof(unsigned long long));       // colmax
  b += align256((size_t)kDotBlocks * (kGmresRestart + 1) * sizeof(double));
  b += align256(4 * sizeof(double) * kMaxW);               // scales
  b += align256(sizeof(double));                           // anorm
  b += align256(2 * sizeof(unsigned long long));           // growth words
  b += align256((size_t)W * kGmStride * sizeof(double));   // GMRES state
  b += align256((size_t)W * 2 * sizeof(int));              // GMRES flags
  return b + 256;
}

void refine_carve(RefineWork& w, char* base, int64_t n, int64_t W) {
  char* c = base;
  auto take = [&](size_t b) { char* r = c; c += align256(b); return r; };
  w.n = n;
  w.W = W;
  w.restart = kGmresRestart;
  w.x = reinterpret_cast<double*>(take((size_t)n * W * sizeof(double)));
  w.r = reinterpret_cast<double*>(take((size_t)n * W * sizeof(double)));
  w.b = reinterpret_cast<double*>(take((size_t)n * W * sizeof(double)));
  w.d32 = reinterpret_cast<float*>(take((size_t)n * W * sizeof(float)));
  size_t pe = (size_t)kSplit * std::max<int64_t>(n, kGmresRestart + 1) * W;
  w.partial = reinterpret_cast<double*>(take(pe * sizeof(double)));
  w.V = reinterpret_cast<double*>(take((size_t)n * (kGmresRestart + 1) * W * sizeof(double)));
  w.w = reinterpret_cast<double*>(take((size_t)n * W * sizeof(double)));
  w.h = reinterpret_cast<double*>(take(3 * (kGmresRestart + 1) * W * sizeof(double)));
  w.colmax = reinterpret_cast<unsigned long long*>(take(4 * W * sizeof(unsigned long long)));
  w.dots = reinterpret_cast<double*>(take((size_t)kDotBlocks * (kGmresRestart + 1) * sizeof(double)));
  w.anorm_dev = reinterpret_cast<double*>(take(4 * sizeof(double) * kMaxW));
  w.growth_bits = reinterpret_cast<unsigned long long*>(take(2 * sizeof(unsigned long long)));
  w.gm = reinterpret_cast<double*>(take((size_t)W * kGmStride * sizeof(double)));
  w.gflags = reinterpret_cast<int*>(take((size_t)W * 2 * sizeof(int)));
}

namespace {

unsigned grid_for(int64_t n, int threads = 256) {
  int64_t b = (n + threads - 1) / threads;
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>(b, 152 * 8));
}

// out = beta*C + alpha*op(A) X   (op(A): len x k; A stored rows x cols)
cudaError_t gemv(char op, int64_t rows, int64_t cols, const double* A, int64_t lda, const double* X,
                 int64_t ldx, int W, double alpha, const double* C, int64_t ldc, double beta,
                 double* out, int64_t ldo, double* P, unsigned long long* colmax, cudaStream_t s,
                 bool absval = false) {
  int64_t len;
  // the partial-sum layout is P[s][q][i] with the padded width Wp
  const int Wp = W <= 1 ? 1 : W <= 2 ? 2 : W <= 4 ? 4 : 8;
  if (op == 'N') {
    len = rows;
    dim3 grid((unsigned)((rows + kRowsPerCta - 1) / kRowsPerCta), kSplit);
    LaunchScope ls_(K_REFINE, 2.0 * rows * cols * W, 8.0 * rows * cols, s);
    if (absval) {
      if (Wp == 1 || X == nullptr) gemv_n_partial_kernel<1, true><<<grid, kRowsPerCta, 0, s>>>(rows, cols, A, lda, X, ldx, W, P);
      else if (Wp == 2) gemv_n_partial_kernel<2, true><<<grid, kRowsPerCta, 0, s>>>(rows, cols, A, lda, X, ldx, W, P);
      else if (Wp == 4) gemv_n_partial_kernel<4, true><<<grid, kRowsPerCta, 0, s>>>(rows, cols, A, lda, X, ldx, W, P);
      else gemv_n_partial_kernel<8, true><<<grid, kRowsPerCta, 0, s>>>(rows, cols, A, lda, X, ldx, W, P);
    } else {
      if (Wp == 1 || X == nullptr) gemv_n_partial_kernel<1, false><<<grid, kRowsPerCta, 0, s>>>(rows, cols, A, lda, X, ldx, W, P);
      else if (Wp == 2) gemv_n_partial_kernel<2, false><<<grid, kRowsPerCta, 0, s>>>(rows, cols, A, lda, X, ldx, W, P);
      else if (Wp == 4) gemv_n_partial_kernel<4, false><<<grid, kRowsPerCta, 0, s>>>(rows, cols, A, lda, X, ldx, W, P);
      else gemv_n_partial_kernel<8, false><<<grid, kRowsPerCta, 0, s>>>(rows, cols, A, lda, X, ldx, W, P);
    }
  } else {
    len = cols;
    dim3 grid((unsigned)((cols + 7) / 8), kSplit);
    LaunchScope ls_(K_REFINE, 2.0 * rows * cols * W, 8.0 * rows * cols, s);
    if (Wp == 1) gemv_t_partial_kernel<1><<<grid, 256, 0, s>>>(rows, cols, A, lda, X, ldx, W, P);
    else if (Wp == 2) gemv_t_partial_kernel<2><<<grid, 256, 0, s>>>(rows, cols, A, lda, X, ldx, W, P);
    else if (Wp == 4) gemv_t_partial_kernel<4><<<grid, 256, 0, s>>>(rows, cols, A, lda, X, ldx, W, P);
    else gemv_t_partial_kernel<8><<<grid, 256, 0, s>>>(rows, cols, A, lda, X, ldx, W, P);
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  { LaunchScope ls_(K_REFINE, 0.0, 0.0, s);
  const int Wp_used = (op == 'N' && X == nullptr) ? 1 : Wp;
  gemv_reduce_kernel<<<grid_for(len), 256, 0, s>>>(len, W, Wp_used, P, alpha, C, ldc, beta, out, ldo, colmax);
  }
  return cudaGetLastError();
}

double bits_to_double(unsigned long long b) {
  double d;
  std::memcpy(&d, &b, sizeof(d));
  return d;
}

}  // namespace

cudaError_t refine_prepare(RefineWork& w, int64_t n, const double* A, int64_t lda, float* A32,
                           int64_t ld32, cudaStream_t s, bool write_f32) {
  if (n == 0) { w.anorm = 0; w.amax = 0; return cudaSuccess; }
  cudaError_t e = cudaMemsetAsync(w.growth_bits, 0, 2 * sizeof(unsigned long long), s);
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(w.colmax, 0, sizeof(unsigned long long), s);
  if (e != cudaSuccess) return e;
  // FP32 copy, row sums of |A| and max |A| in one pass over A; then
  // ||A||_inf = max_i sum_j |A[i,j]| from the row sums
  {
    LaunchScope ls_(K_REFINE, (double)n * n, (write_f32 ? 12.0 : 8.0) * n * n, s);
    dim3 grid((unsigned)((n + kPrepRows - 1) / kPrepRows), kPrepChunks);
    if (write_f32)
      prepare_kernel<true><<<grid, 256, 0, s>>>(n, A, lda, A32, ld32, w.partial, w.growth_bits);
    else
      prepare_kernel<false><<<grid, 256, 0, s>>>(n, A, lda, A32, ld32, w.partial, w.growth_bits);
  }
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  {
    LaunchScope ls_(K_REFINE, 0.0, 8.0 * kPrepChunks * n, s);
    prepare_reduce_kernel<<<grid_for(n), 256, 0, s>>>(n, w.partial, w.colmax);
  }
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  unsigned long long bits[2] = {0, 0};
  e = cudaMemcpyAsync(&bits[0], w.colmax, sizeof(bits[0]), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(&bits[1], w.growth_bits, sizeof(bits[1]), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  w.anorm = bits_to_double(bits[0]);
  w.amax = bits_to_double(bits[1]);
  return e;
}

cudaError_t rbt_matrix_launch(int64_t n, const double* A, int64_t lda, float* B, int64_t ldb,
                              const float* rbt, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  const int64_t n4 = n - n % 4;
  if (n4 < 4 || n4 / 4 > 65535) return cudaErrorInvalidValue;
  {
    LaunchScope ls_(K_REFINE, 32.0 * n4 * n4 / 16.0 * 2.0, 12.0 * n4 * n4, s);
    dim3 grid((unsigned)((n4 / 4 + 127) / 128), (unsigned)(n4 / 4));
    rbt_matrix_kernel<<<grid, 128, 0, s>>>(n4, A, lda, B, ldb, rbt);
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess || n4 == n) return e;
  LaunchScope ls_(K_REFINE, 0.0, 12.0 * 2.0 * (n - n4) * n, s);
  dim3 grid((unsigned)((n4 / 4 + 127) / 128), (unsigned)(2 * (n - n4) + 1));
  rbt_edge_kernel<<<grid, 128, 0, s>>>(n, n4, A, lda, B, ldb, rbt);
  return cudaGetLastError();
}

cudaError_t rbt_vec_launch(int64_t n, int W, float* v, int64_t ldv, const float* rbt, int side,
                           bool transposed, cudaStream_t s) {
  if (n <= 0 || W <= 0) return cudaSuccess;
  const int64_t n4 = n - n % 4;  // entries past n4 are left as they are (identity)
  if (n4 < 4 || W > 65535) return cudaErrorInvalidValue;
  LaunchScope ls_(K_REFINE, 12.0 * n4 * W, 8.0 * n4 * W, s);
  dim3 grid((unsigned)((n4 / 4 + 255) / 256), (unsigned)W);
  rbt_vec_kernel<<<grid, 256, 0, s>>>(n4, W, v, ldv, rbt, side, transposed ? 1 : 0);
  return cudaGetLastError();
}

void rbt_fill_host(int64_t n, float* out) {
  // splitmix64 stream from a fixed seed: the transform (and so every
  // result) is the same on every run; 4 n4 values, n4 = n - n mod 4
  const int64_t n4 = n - n % 4;
  uint64_t x = 0x5eedb077e4f1ULL;
  for (int64_t i = 0; i < 4 * n4; ++i) {
    x += 0x9e3779b97f4a7c15ULL;
    uint64_t z = x;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    z ^= z >> 31;
    const double u = (double)(z >> 11) * (1.0 / 9007199254740992.0) - 0.5;
    out[i] = (float)std::exp(u / 10.0);
  }
}

cudaError_t refine_growth_launch(RefineWork& w, int64_t n, const float* LU, int64_t ld, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  LaunchScope ls_(K_REFINE, 0.0, 2.0 * n * n, s);
  umax_kernel<<<(unsigned)((n + 7) / 8), 256, 0, s>>>(n, LU, ld, w.growth_bits + 1);
  return cudaGetLastError();
}

double refine_growth(const RefineWork& w, unsigned long long umax_bits) {
  const double umax = bits_to_double(umax_bits);
  if (!(umax <= INFINITY)) return INFINITY;  // NaN in the factors
  if (w.amax > 0) return umax / w.amax;
  return umax > 0 ? INFINITY : 1.0;
}

double growth_limit_default(int32_t precision) {
  // 1 / u of the arithmetic the factors were computed in: FP32 (u = 2^-24),
  // or the 16-bit operands of the tensor-core updates (FP16 2^-11, BF16 2^-8)
  if (precision == GBLU_BF16) return 256.0;
  if (precision == GBLU_FP16) return 2048.0;
  return 16777216.0;
}

gblu_refine_opts refine_default_opts() {
  gblu_refine_opts o;
  o.mode = GBLU_REFINE_IR;
  o.max_iter = 30;
  o.tol = 0.0;
  o.fallback = 1;
  o.gmres_restart = kGmresRestart;
  o.gmres_tol = 1e-10;
  o.growth_limit = 0.0;
  return o;
}

namespace {

struct Solver {
  gblu_ctx* ctx;
  gblu_factor* f;
  RefineWork& w;
  char trans;
  cudaStream_t s;
  int64_t n;

  // out (len n, W cols) <- M^{-1} v using the FP32 factors with a per-column
  // power-of-two scale so the FP32 right-hand side is O(1).  No host sync.
  int32_t precond(const double* v, int64_t ldv, double* out, int64_t ldo, int W) {
    unsigned long long* cm = w.colmax + 3 * w.W;
    double* dsc = w.anorm_dev;  // 2*kMaxW doubles of scale storage
    GBLU_CK(ctx, cudaMemsetAsync(cm, 0, W * sizeof(unsigned long long), s), "memset");
    {
      LaunchScope ls_(K_REFINE, 0.0, 0.0, s);
      colmax_kernel<<<grid_for(n), 256, 0, s>>>(n, W, v, ldv, cm);
    }
    GBLU_CK(ctx, cudaGetLastError(), "colmax");
    {
      LaunchScope ls_(K_REFINE, 0.0, 0.0, s);
      pow2_scales_kernel<<<1, 32, 0, s>>>(W, cm, dsc);
    }
    GBLU_CK(ctx, cudaGetLastError(), "scales");
    {
      LaunchScope ls_(K_REFINE, 0.0, 0.0, s);
      scale_to_f32_kernel<<<grid_for(n * W), 256, 0, s>>>(n, W, v, ldv, dsc, w.d32, n);
    }
    GBLU_CK(ctx, cudaGetLastError(), "scale");
    // RBT factors: d := W1^T d / 2, LU solve, d := W2 d / 2 with (W1, W2) =
    // (U, V) for op = N and (V, U) for op = T
    const bool rbt = f->pivoting == GBLU_PIVOT_RBT;
    const int side_in = trans == 'N' ? 0 : 1;
    if (rbt) GBLU_CK(ctx, rbt_vec_launch(n, W, w.d32, n, f->rbt, side_in, true, s), "butterfly");
    GBLU_CK(ctx, getrs_launch<float>(f->rs32, trans, W, w.d32, n, nullptr, s), "FP32 getrs");
    if (rbt) GBLU_CK(ctx, rbt_vec_launch(n, W, w.d32, n, f->rbt, 1 - side_in, false, s), "butterfly");
    {
      LaunchScope ls_(K_REFINE, 0.0, 0.0, s);
      update_from_f32_kernel<<<grid_for(n * W), 256, 0, s>>>(n, W, out, ldo, w.d32, n, dsc + kMaxW, 0.0);
    }
    GBLU_CK(ctx, cudaGetLastError(), "update");
    return GBLU_OK;
  }

  // r = b - op(A) x for W columns; returns |r|_inf and |x|_inf per column.
  int32_t residual(int W, double* rnorm, double* xnorm) {
    GBLU_CK(ctx, cudaMemsetAsync(w.colmax, 0, 2 * w.W * sizeof(unsigned long long), s), "memset");
    GBLU_CK(ctx, gemv(trans == 'N' ? 'N' : 'T', n, n, f->lu64, f->ld, w.x, n, W, -1.0, w.b, n, 1.0,
                      w.r, n, w.partial, w.colmax, s),
            "residual");
    { LaunchScope ls_(K_REFINE, 0.0, 0.0, s);
    colmax_kernel<<<grid_for(n), 256, 0, s>>>(n, W, w.x, n, w.colmax + w.W);
    }
    GBLU_CK(ctx, cudaGetLastError(), "colmax");
    std::vector<unsigned long long> bits(2 * w.W);
    GBLU_CK(ctx, cudaMemcpyAsync(bits.data(), w.colmax, 2 * w.W * sizeof(unsigned long long),
                                 cudaMemcpyDeviceToHost, s), "readback");
    GBLU_CK(ctx, cudaStreamSynchronize(s), "residual");
    for (int q = 0; q < W; ++q) {
      rnorm[q] = bits_to_double(bits[q]);
      xnorm[q] = bits_to_double(bits[w.W + q]);
    }
    return GBLU_OK;
  }

  // The first residual, x = 0: r = b exactly (b - A 0 adds only zeros), so
  // the product with A is skipped; |r|_inf = |b|_inf, |x|_inf = 0.
  int32_t residual_zero_x(int W, double* rnorm, double* xnorm) {
    GBLU_CK(ctx, cudaMemsetAsync(w.colmax, 0, w.W * sizeof(unsigned long long), s), "memset");
    GBLU_CK(ctx, cudaMemcpyAsync(w.r, w.b, (size_t)n * W * sizeof(double), cudaMemcpyDeviceToDevice, s), "r = b");
    { LaunchScope ls_(K_REFINE, 0.0, 0.0, s);
    colmax_kernel<<<grid_for(n), 256, 0, s>>>(n, W, w.b, n, w.colmax);
    }
    GBLU_CK(ctx, cudaGetLastError(), "colmax");
    std::vector<unsigned long long> bits(w.W);
    GBLU_CK(ctx, cudaMemcpyAsync(bits.data(), w.colmax, w.W * sizeof(unsigned long long),
                                 cudaMemcpyDeviceToHost, s), "readback");
    GBLU_CK(ctx, cudaStreamSynchronize(s), "residual");
    for (int q = 0; q < W; ++q) {
      rnorm[q] = bits_to_double(bits[q]);
      xnorm[q] = 0.0;
    }
    return GBLU_OK;
  }

  // GMRES(m) on op(A) d = r[:,q], left-preconditioned by the FP32 LU, for the
  // columns q < nc with run[q] set, in lockstep: each inner step does one
  // nc-column matvec, one nc-column preconditioner solve and the two
  // Gram-Schmidt passes of every column, while every column keeps its own
  // basis V_q, Hessenberg matrix, rotations and stopping step (device state,
  // gmres_*_kernel), so its result is the one it would have alone.  The host
  // never waits inside a step: it reads the stepping flags of step j - 1 while
  // step j is already queued, and stops when no column steps (a step queued
  // after every column stopped changes nothing).  Adds d_q into x[:,q]; its[q]
  // receives the column's inner iterations.
  int32_t gmres_block(int nc, const std::vector<int>& run, int restart, double rtol, std::vector<int>& its) {
    const int m = std::max(1, std::min(restart, (int)kGmresRestart));
    const int64_t ldV = (int64_t)(kGmresRestart + 1) * n;  // stride between the columns' bases
    const int hs = kGmresRestart + 1;
    double* V = w.V;
    auto Vq = [&](int q, int j) { return V + (size_t)q * ldV + (size_t)j * n; };
    if (!w.gflags_host) {
      void* p = nullptr;
      GBLU_CK(ctx, cudaMallocHost(&p, 4 * kMaxW * sizeof(int)), "pinned GMRES flags");
      w.gflags_host = reinterpret_cast<int*>(p);
    }
    int32_t st = precond(w.r, n, V, ldV, nc);
    if (st) return st;
    unsigned mask = 0;
    for (int q = 0; q < nc; ++q)
      if (run[q]) {
        mask |= 1u << q;
        GBLU_CK(ctx, gemv('T', n, 1, Vq(q, 0), n, Vq(q, 0), n, 1, 1.0, nullptr, 1, 0.0, w.h + q, 1,
                          w.partial, nullptr, s), "norm");
      }
    {
      LaunchScope ls_(K_REFINE, 0.0, 0.0, s);
      gmres_begin_kernel<<<1, 32, 0, s>>>(nc, mask, w.h, w.gm, w.gflags);
    }
    {
      LaunchScope ls_(K_REFINE, 0.0, 16.0 * n * nc, s);
      gmres_scale_kernel<<<grid_for(n * nc), 256, 0, s>>>(n, nc, V, ldV, 0, w.gm);
    }
    GBLU_CK(ctx, cudaGetLastError(), "GMRES start");
    cudaEvent_t ev[2] = {nullptr, nullptr};
    for (auto& e : ev) GBLU_CK(ctx, cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "event");
    auto release = [&]() {
      for (auto& e : ev)
        if (e) cudaEventDestroy(e);
    };
    int32_t rc = GBLU_OK;
    for (int j = 0; j < m && mask && rc == GBLU_OK; ++j) {
      // w = op(A) v_j ; z = M^{-1} w  (all nc columns at once)
      cudaError_t ce = gemv(trans == 'N' ? 'N' : 'T', n, n, f->lu64, f->ld, Vq(0, j), ldV, nc, 1.0, nullptr,
                            1, 0.0, w.w, n, w.partial, nullptr, s);
      if (ce != cudaSuccess) { rc = cuda_fail(ctx, ce, "matvec"); break; }
      rc = precond(w.w, n, Vq(0, j + 1), ldV, nc);
      if (rc) break;
      // classical Gram-Schmidt, twice, and the norm, for every column
      for (int q = 0; q < nc && ce == cudaSuccess; ++q) {
        double* z = Vq(q, j + 1);
        for (int pass = 0; pass < 2 && ce == cudaSuccess; ++pass) {
          double* hq = w.h + (size_t)(q * 3 + pass) * hs;
          ce = gemv('T', n, j + 1, Vq(q, 0), n, z, n, 1, 1.0, nullptr, 1, 0.0, hq, 1, w.partial, nullptr, s);
          if (ce == cudaSuccess)
            ce = gemv('N', n, j + 1, Vq(q, 0), n, hq, j + 1, 1, -1.0, z, n, 1.0, z, n, w.partial, nullptr, s);
        }
        if (ce == cudaSuccess)
          ce = gemv('T', n, 1, z, n, z, n, 1, 1.0, nullptr, 1, 0.0, w.h + (size_t)(q * 3 + 2) * hs, 1, w.partial,
                    nullptr, s);
      }
      if (ce != cudaSuccess) { rc = cuda_fail(ctx, ce, "Gram-Schmidt"); break; }
      {
        LaunchScope ls_(K_REFINE, 0.0, 0.0, s);
        gmres_step_kernel<<<1, 32, 0, s>>>(nc, j, m, w.h, rtol, w.gm, w.gflags);
      }
      {
        LaunchScope ls_(K_REFINE, 0.0, 16.0 * n * nc, s);
        gmres_scale_kernel<<<grid_for(n * nc), 256, 0, s>>>(n, nc, V, ldV, j + 1, w.gm);
      }
      ce = cudaGetLastError();
      // pinned slot j & 1 of 2 * kMaxW ints receives this step's flags
      if (ce == cudaSuccess)
        ce = cudaMemcpyAsync(w.gflags_host + (j & 1) * 2 * kMaxW, w.gflags, 2 * nc * sizeof(int),
                             cudaMemcpyDeviceToHost, s);
      if (ce == cudaSuccess) ce = cudaEventRecord(ev[j & 1], s);
      if (ce == cudaSuccess && j >= 1) {
        ce = cudaEventSynchronize(ev[(j - 1) & 1]);
        if (ce == cudaSuccess) {
          const int* fl = w.gflags_host + ((j - 1) & 1) * 2 * kMaxW;
          bool any = false;
          for (int q = 0; q < nc; ++q) any |= fl[2 * q] != 0;
          if (!any) mask = 0;
        }
      }
      if (ce != cudaSuccess) rc = cuda_fail(ctx, ce, "GMRES step");
    }
    release();
    if (rc) return rc;
    // y_q = H_q(1:k,1:k) \ g_q(1:k); x[:,q] += V_q(:,1:k) y_q
    {
      LaunchScope ls_(K_REFINE, 0.0, 0.0, s);
      gmres_finish_kernel<<<1, 32, 0, s>>>(nc, m, w.gm, w.gflags, w.h);
    }
    GBLU_CK(ctx, cudaGetLastError(), "GMRES finish");
    std::vector<int> fl(2 * nc);
    GBLU_CK(ctx, cudaMemcpyAsync(fl.data(), w.gflags, 2 * nc * sizeof(int), cudaMemcpyDeviceToHost, s),
            "reading GMRES steps");
    GBLU_CK(ctx, cudaStreamSynchronize(s), "GMRES");
    for (int q = 0; q < nc; ++q) {
      its[q] = fl[2 * q + 1];
      if (its[q] == 0) continue;
      double* xq = w.x + (size_t)q * n;
      GBLU_CK(ctx, gemv('N', n, its[q], Vq(q, 0), n, w.h + (size_t)q * hs, its[q], 1, 1.0, xq, n, 1.0, xq, n,
                        w.partial, nullptr, s), "update");
    }
    return GBLU_OK;
  }
};

}  // namespace

int32_t refine_solve(gblu_ctx* ctx, gblu_factor* f, char trans, int64_t nrhs, double* B, int64_t ldb,
                     int32_t b_loc, const gblu_refine_opts* opts_in, gblu_refine_stats* stats) {
  gblu_refine_opts o = opts_in ? *opts_in : refine_default_opts();
  const int64_t n = f->n;
  RefineWork& w = f->refine;
  cudaStream_t s = ctx->stream;
  trans = (trans == 'n') ? 'N' : (trans == 't' || trans == 'c' || trans == 'C') ? 'T' : trans;
  const double tol = o.tol > 0 ? o.tol : (double)std::max<int64_t>(n, 1) * 2.220446049250313e-16;
  const int W = (int)w.W;
  {
    int32_t e = ensure_inverse(ctx, f);  // fast low-precision solves
    if (e) return e;
  }
  gblu_refine_stats st_acc{};
  st_acc.converged = 1;
  st_acc.growth = f->growth;
  Solver S{ctx, f, w, trans, s, n};
  if (stats) *stats = gblu_refine_stats{};
  // Pivot growth (FP64 ratio of the device-computed maxima): factors whose
  // rounding errors reach the size of A's entries go straight to the FP64 LU.
  const double glimit = o.growth_limit > 0 ? o.growth_limit : growth_limit_default(f->precision);
  const bool growth_fb = !f->use_fb && !(f->growth <= glimit);
  if (growth_fb && !o.fallback)
    return fail(ctx, GBLU_ESTALL, "pivot growth %.3e of the low-precision factors exceeds %.3e",
                f->growth, glimit);
  const int fb_reason = f->use_fb ? GBLU_FALLBACK_ZERO_PIVOT
                                  : growth_fb ? GBLU_FALLBACK_GROWTH : GBLU_FALLBACK_STALL;
  for (int64_t c0 = 0; c0 < nrhs; c0 += W) {
    const int nc = (int)std::min<int64_t>(W, nrhs - c0);
    double* Bc = B + c0 * ldb;
    cudaMemcpyKind k_in = b_loc == GBLU_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    cudaMemcpyKind k_out = b_loc == GBLU_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    GBLU_CK(ctx, cudaMemcpy2DAsync(w.b, n * sizeof(double), Bc, ldb * sizeof(double),
                                   n * sizeof(double), nc, k_in, s),
            "copying B");
    // Per-column state: every column's iterate depends only on its own data,
    // so a column's result is the same whatever else is in the chunk.
    enum { ACTIVE = 0, CONVERGED = 1, STALLED = 2 };
    std::vector<int> state(nc, ACTIVE), slow(nc, 0), its_q(nc, 0);
    std::vector<double> rn(nc), xn(nc), bn(nc), prev(nc, INFINITY), be_q(nc, INFINITY);
    bool any_fb = false;
    const bool direct_fb = f->use_fb || growth_fb;  // no refinement at all
    if (direct_fb) {
      for (int q = 0; q < nc; ++q) state[q] = STALLED;
    } else {
      GBLU_CK(ctx, cudaMemsetAsync(w.x, 0, (size_t)n * nc * sizeof(double), s), "x0");  // x0 = 0
      for (int it = 0; it <= o.max_iter; ++it) {
        int32_t e = it == 0 ? S.residual_zero_x(nc, rn.data(), xn.data()) : S.residual(nc, rn.data(), xn.data());
        if (e) return e;
        if (it == 0) bn = rn;  // x = 0: r = b
        bool any_active = false;
        for (int q = 0; q < nc; ++q) {
          if (state[q] != ACTIVE) continue;
          const double den = w.anorm * xn[q] + bn[q];
          const double be = den > 0 ? rn[q] / den : (rn[q] == 0 ? 0.0 : INFINITY);
          be_q[q] = be;
          its_q[q] = it;
          if (be <= tol) { state[q] = CONVERGED; continue; }
          if (!std::isfinite(be) && it > 0) { state[q] = STALLED; continue; }
          if (it >= 2 && be > 0.9 * prev[q]) {
            if (++slow[q] >= 2) { state[q] = STALLED; continue; }
          } else {
            slow[q] = 0;
          }
          prev[q] = be;
          if (it == o.max_iter) { state[q] = STALLED; continue; }
          any_active = true;
        }
        if (!any_active) break;
        if (o.mode == GBLU_REFINE_GMRES) {
          std::vector<int> run(nc), its(nc, 0);
          for (int q = 0; q < nc; ++q) run[q] = state[q] == ACTIVE;
          e = S.gmres_block(nc, run, o.gmres_restart, o.gmres_tol, its);
          if (e) return e;
          for (int q = 0; q < nc; ++q) st_acc.inner_iterations += its[q];
        } else {
          e = S.precond(w.r, n, w.r, n, nc);  // d = M^{-1} r (in place), scaled per column
          if (e) return e;
          for (int q = 0; q < nc; ++q) {
            if (state[q] != ACTIVE) continue;
            LaunchScope ls_(K_REFINE, 0.0, 0.0, s);
            axpby_kernel<<<grid_for(n), 256, 0, s>>>(n, 1.0, w.r + (size_t)q * n, 1.0, w.x + (size_t)q * n);
          }
          GBLU_CK(ctx, cudaGetLastError(), "update");
        }
      }
    }
    for (int q = 0; q < nc; ++q) any_fb |= state[q] == STALLED;
    if (any_fb) {
      if (!o.fallback && !f->use_fb)
        return fail(ctx, GBLU_ESTALL, "refinement stalled (backward error %.3e)",
                    *std::max_element(be_q.begin(), be_q.end()));
      if (!f->fb_valid) {
        int64_t info64 = 0;
        int32_t e = factor_fp64_fallback(ctx, f, &info64);
        if (e) return e;
        if (info64 != 0) return fail(ctx, GBLU_EINVAL, "matrix is singular in FP64 (info = %lld)", (long long)info64);
      }
      // plain FP64 solve of the stalled columns on the FP64 factors
      GBLU_CK(ctx, cudaMemcpyAsync(w.r, w.b, (size_t)n * nc * sizeof(double), cudaMemcpyDeviceToDevice, s),
              "copy b");
      GBLU_CK(ctx, getrs_launch<double>(f->fb_rs, trans, nc, w.r, n, nullptr, s), "FP64 getrs");
      for (int q = 0; q < nc; ++q)
        if (state[q] == STALLED)
          GBLU_CK(ctx, cudaMemcpyAsync(w.x + (size_t)q * n, w.r + (size_t)q * n, n * sizeof(double),
                                       cudaMemcpyDeviceToDevice, s), "fallback column");
      int32_t e = S.residual(nc, rn.data(), xn.data());
      if (e) return e;
      if (direct_fb) {  // ||b|| was not measured yet
        GBLU_CK(ctx, cudaMemsetAsync(w.colmax + 2 * w.W, 0, nc * sizeof(unsigned long long), s), "memset");
        {
          LaunchScope ls_(K_REFINE, 0.0, 0.0, s);
          colmax_kernel<<<grid_for(n), 256, 0, s>>>(n, nc, w.b, n, w.colmax + 2 * w.W);
        }
        std::vector<unsigned long long> bits(nc);
        GBLU_CK(ctx, cudaMemcpyAsync(bits.data(), w.colmax + 2 * w.W, nc * sizeof(unsigned long long),
                                     cudaMemcpyDeviceToHost, s), "readback");
        GBLU_CK(ctx, cudaStreamSynchronize(s), "fallback");
        for (int q = 0; q < nc; ++q) bn[q] = bits_to_double(bits[q]);
      }
      for (int q = 0; q < nc; ++q)
        if (state[q] == STALLED) {
          const double den = w.anorm * xn[q] + bn[q];
          be_q[q] = den > 0 ? rn[q] / den : 0.0;
        }
    }
    GBLU_CK(ctx, cudaMemcpy2DAsync(Bc, ldb * sizeof(double), w.x, n * sizeof(double),
                                   n * sizeof(double), nc, k_out, s),
            "copying X");
    const bool fell_back = any_fb;
    const bool done = !any_fb;
    double berr_final = 0;
    int iters = 0;
    for (int q = 0; q < nc; ++q) {
      berr_final = std::max(berr_final, std::isnan(be_q[q]) ? INFINITY : be_q[q]);
      iters = std::max(iters, its_q[q]);
    }
    GBLU_CK(ctx, cudaStreamSynchronize(s), "refined solve");
    int32_t e = check_device_errors(ctx, {f->rs32.scratch, f->fb_rs.scratch});
    if (e) return e;
    st_acc.iterations = std::max(st_acc.iterations, iters);
    st_acc.fell_back |= fell_back ? 1 : 0;
    if (fell_back && st_acc.fallback_reason == GBLU_FALLBACK_NONE) st_acc.fallback_reason = fb_reason;
    if (!done) st_acc.converged = fell_back ? st_acc.converged : 0;
    st_acc.backward_error = std::max(st_acc.backward_error, berr_final);
  }
  if (stats) *stats = st_acc;
  return GBLU_OK;
}

// ||B - op(A) X||_F and ||B||_F with the FP64 matrix the factor keeps; up to
// kMaxW columns at a time through a lazily allocated work arena.
int32_t residual_norm(gblu_ctx* ctx, gblu_factor* f, char trans, int64_t nrhs, const double* X,
                      int64_t ldx, const double* B, int64_t ldb, int32_t loc, double* res_norm,
                      double* b_norm) {
  const int64_t n = f->n;
  const double* A = f->precision == GBLU_FP64 ? (f->a_keep_valid ? f->a_keep : nullptr) : f->lu64;
  if (!A) return fail(ctx, GBLU_EINVAL, "gblu_residual_norm: the factor keeps no copy of A "
                                        "(gblu_factor_keep_matrix before getrf)");
  cudaStream_t s = ctx->stream;
  const int64_t W = kMaxW;
  const size_t vec = align256((size_t)n * W * sizeof(double));
  const size_t pbytes = align256((size_t)kSplit * n * W * sizeof(double));
  const size_t sbytes = align256((size_t)2 * kSumBlocks * W * sizeof(double)) + align256(2 * W * sizeof(double));
  const size_t need = 3 * vec + pbytes + sbytes;
  if (f->chk_bytes < need) {
    if (f->chk_arena) {
      GBLU_CK(ctx, cudaStreamSynchronize(s), "residual check");
      ctx_free(ctx, f->chk_arena, f->chk_bytes);
      f->chk_arena = nullptr;
      f->chk_bytes = 0;
    }
    int32_t st = ctx_alloc(ctx, need, &f->chk_arena);
    if (st) return st;
    f->chk_bytes = need;
  }
  char* c = reinterpret_cast<char*>(f->chk_arena);
  double* Xd = reinterpret_cast<double*>(c);
  double* Bd = reinterpret_cast<double*>(c + vec);
  double* R = reinterpret_cast<double*>(c + 2 * vec);
  double* P = reinterpret_cast<double*>(c + 3 * vec);
  double* part = reinterpret_cast<double*>(c + 3 * vec + pbytes);
  double* sums = part + 2 * kSumBlocks * W;
  const cudaMemcpyKind kind = loc == GBLU_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
  const char op = (trans == 'N' || trans == 'n') ? 'N' : 'T';
  double rr = 0.0, bb = 0.0;
  for (int64_t c0 = 0; c0 < nrhs; c0 += W) {
    const int nc = (int)std::min<int64_t>(W, nrhs - c0);
    GBLU_CK(ctx, cudaMemcpy2DAsync(Xd, n * sizeof(double), X + c0 * ldx, ldx * sizeof(double),
                                   n * sizeof(double), nc, kind, s), "copying X");
    GBLU_CK(ctx, cudaMemcpy2DAsync(Bd, n * sizeof(double), B + c0 * ldb, ldb * sizeof(double),
                                   n * sizeof(double), nc, kind, s), "copying B");
    GBLU_CK(ctx, gemv(op, n, n, A, f->ld, Xd, n, nc, -1.0, Bd, n, 1.0, R, n, P, nullptr, s), "residual");
    {
      LaunchScope ls_(K_REFINE, 0.0, 8.0 * n * nc, s);
      sumsq_partial_kernel<<<dim3(kSumBlocks, nc), 256, 0, s>>>(n, R, n, part);
    }
    {
      LaunchScope ls_(K_REFINE, 0.0, 8.0 * n * nc, s);
      sumsq_partial_kernel<<<dim3(kSumBlocks, nc), 256, 0, s>>>(n, Bd, n, part + kSumBlocks * W);
    }
    {
      LaunchScope ls_(K_REFINE, 0.0, 0.0, s);
      sumsq_final_kernel<<<1, 2 * W, 0, s>>>(2 * W, part, sums);
    }
    GBLU_CK(ctx, cudaGetLastError(), "residual norms");
    double h[2 * kMaxW];
    GBLU_CK(ctx, cudaMemcpyAsync(h, sums, 2 * W * sizeof(double), cudaMemcpyDeviceToHost, s), "reading norms");
    GBLU_CK(ctx, cudaStreamSynchronize(s), "residual check");
    for (int q = 0; q < nc; ++q) {
      rr += h[q];
      bb += h[W + q];
    }
  }
  *res_norm = std::sqrt(rr);
  *b_norm = std::sqrt(bb);
  return GBLU_OK;
}

}  // namespace gblu

extern "C" {

int32_t gblu_refine_opts_default(gblu_refine_opts* opts) {
  if (!opts) return GBLU_EINVAL;
  *opts = gblu::refine_default_opts();
  return GBLU_OK;
}

int32_t gblu_residual_norm(gblu_ctx* ctx, gblu_factor* f, char trans, int64_t nrhs, const double* X,
                           int64_t ldx, const double* B, int64_t ldb, int32_t loc, double* res_norm,
                           double* b_norm) {
  using namespace gblu;
  if (!ctx || !f || !res_norm || !b_norm) return fail(ctx, GBLU_EINVAL, "gblu_residual_norm: NULL argument");
  if (!(trans == 'N' || trans == 'n' || trans == 'T' || trans == 't' || trans == 'C' || trans == 'c'))
    return fail(ctx, GBLU_EINVAL, "gblu_residual_norm: trans must be 'N' or 'T'");
  if (f->m != f->n) return fail(ctx, GBLU_EINVAL, "gblu_residual_norm: factor is not square");
  if (nrhs < 0) return fail(ctx, GBLU_EINVAL, "gblu_residual_norm: nrhs < 0");
  if (ldx < std::max<int64_t>(1, f->n) || ldb < std::max<int64_t>(1, f->n))
    return fail(ctx, GBLU_EINVAL, "gblu_residual_norm: leading dimension < n");
  if (loc != GBLU_HOST && loc != GBLU_DEVICE) return fail(ctx, GBLU_EINVAL, "gblu_residual_norm: bad loc");
  if (!f->factored) return fail(ctx, GBLU_ENOTFACTORED, "gblu_residual_norm: no factorization");
  *res_norm = 0.0;
  *b_norm = 0.0;
  if (nrhs == 0 || f->n == 0) return GBLU_OK;
  if (!X || !B) return fail(ctx, GBLU_EINVAL, "gblu_residual_norm: X or B is NULL");
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  DeviceGuard g(ctx->device);
  ActiveProfiler ap(&ctx->prof);
  return residual_norm(ctx, f, trans, nrhs, X, ldx, B, ldb, loc, res_norm, b_norm);
}

}  // extern "C"
