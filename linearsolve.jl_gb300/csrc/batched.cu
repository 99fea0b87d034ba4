// Batched uneven LU: thousands of independent square systems A_i x_i = b_i
// (n_i <= 256) factored and solved by one persistent kernel per size bucket,
// all captured in one CUDA graph.
//
// Per system the algorithm is the reference's blocked getrf
// (src/blocked_lufact.jl:658-679: panel getf2, interchanges, unit-lower TRSM,
// Schur update) followed by its back-solve (src/factorization.jl:433-457),
// with the same per-element fused-multiply-add order, so the FP64 results are
// bit-identical to the oracle's per-system getrf + getrs.  A CTA takes the
// next system from a queue ordered by decreasing size (longest first), holds
// the current panel (NB columns) and the U12 row block in shared memory, and
// updates the trailing matrix in global memory, where the system's working
// set stays L2-resident.
//
// The mixed variant factors a FP32 copy with the same code and refines each
// system in FP64 (residual with the FP64 A, per-system backward-error test,
// up to `maxit` corrections); systems that do not converge are flagged and
// re-solved by the FP64 kernel in the same graph.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
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

template <typename T>
struct SysSmem {
  T* P;    // panel: NB columns x n rows (column j at P + j*kBatchMaxN)
  T* U;    // U12 block: NB rows x n columns (row j at U + j*kBatchMaxN)
  T* x;    // solve vector (n)
  T* red_v;
  int* red_i;
};

template <typename T>
__device__ __forceinline__ T babs(T v) { return v < T(0) ? -v : v; }

// Block-wide first-index argmax of |v| over rows [lo, n) of column `col` of P.
template <typename T, int NT>
__device__ int block_argmax(const T* col, int lo, int n, T* red_v, int* red_i, T* amax_out) {
  T bv = T(0);
  int bi = -1;
  for (int i = lo + threadIdx.x; i < n; i += NT) {
    const T a = fabs(col[i]);
    if (a > bv) { bv = a; bi = i; }
  }
  for (int off = 16; off; off >>= 1) {
    const T ov = __shfl_down_sync(0xffffffffu, bv, off);
    const int oi = __shfl_down_sync(0xffffffffu, bi, off);
    if (oi >= 0 && (bi < 0 || ov > bv || (ov == bv && oi < bi))) { bv = ov; bi = oi; }
  }
  if ((threadIdx.x & 31) == 0) { red_v[threadIdx.x >> 5] = bv; red_i[threadIdx.x >> 5] = bi; }
  __syncthreads();
  if (threadIdx.x < 32) {
    bv = threadIdx.x < NT / 32 ? red_v[threadIdx.x] : T(0);
    bi = threadIdx.x < NT / 32 ? red_i[threadIdx.x] : -1;
    for (int off = 16; off; off >>= 1) {
      const T ov = __shfl_down_sync(0xffffffffu, bv, off);
      const int oi = __shfl_down_sync(0xffffffffu, bi, off);
      if (oi >= 0 && (bi < 0 || ov > bv || (ov == bv && oi < bi))) { bv = ov; bi = oi; }
    }
    if (threadIdx.x == 0) { red_v[0] = bv; red_i[0] = bi; }
  }
  __syncthreads();
  const int r = red_i[0];
  *amax_out = red_v[0];
  __syncthreads();
  return r;
}

// In-place getrf of one n x n column-major system (ld = n) in global memory.
// ipiv: 1-based.  Returns info (0 or first zero pivot, 1-based).
template <typename T, int NT, int NB>
__device__ int64_t factor_system(T* __restrict__ A, int n, int32_t* __restrict__ ipiv,
                                 const SysSmem<T>& sm) {
  int64_t info = 0;
  const int tid = threadIdx.x;
  for (int k0 = 0; k0 < n; k0 += NB) {
    const int kb = min(NB, n - k0);
    // panel rows [0, n) of columns k0..k0+kb-1 into shared memory (rows < k0 unused)
    for (int j = 0; j < kb; ++j)
      for (int i = k0 + tid; i < n; i += NT) sm.P[j * kBatchMaxN + i] = A[i + (int64_t)(k0 + j) * n];
    __syncthreads();
    for (int j = 0; j < kb; ++j) {
      const int col = k0 + j;
      T* pc = sm.P + j * kBatchMaxN;
      T amax;
      int p = block_argmax<T, NT>(pc, col, n, sm.red_v, sm.red_i, &amax);
      if (p < 0) p = col;  // amax == 0 (or NaN everywhere): kp = k
      if (tid == 0) ipiv[col] = p + 1;
      const T piv = pc[p];
      if (piv != T(0)) {
        if (p != col && tid < kb) {
          T* q = sm.P + tid * kBatchMaxN;
          const T t = q[col];
          q[col] = q[p];
          q[p] = t;
        }
        __syncthreads();
        const T inv = T(1) / pc[col];
        for (int i = col + 1 + tid; i < n; i += NT) pc[i] *= inv;
      } else if (info == 0) {
        info = col + 1;
      }
      __syncthreads();
      for (int i = col + 1 + tid; i < n; i += NT) {  // one row per thread, columns in order
        const T l = pc[i];
        for (int jj = j + 1; jj < kb; ++jj) {
          T* q = sm.P + jj * kBatchMaxN;
          q[i] = fma(-l, q[col], q[i]);
        }
      }
      __syncthreads();
    }
    for (int j = 0; j < kb; ++j)
      for (int i = k0 + tid; i < n; i += NT) A[i + (int64_t)(k0 + j) * n] = sm.P[j * kBatchMaxN + i];
    // interchanges on the other columns, in order (blocked_lufact.jl:126-141)
    for (int c = tid; c < n; c += NT) {
      if (c >= k0 && c < k0 + kb) continue;
      T* ac = A + (int64_t)c * n;
      for (int j = 0; j < kb; ++j) {
        const int p = ipiv[k0 + j] - 1;
        if (p != k0 + j) {
          const T t = ac[k0 + j];
          ac[k0 + j] = ac[p];
          ac[p] = t;
        }
      }
    }
    __syncthreads();  // ipiv writes and global swaps visible to the whole CTA
    const int c1 = k0 + kb, nc = n - c1;
    if (nc > 0) {
      // U12 := L11 \ A12, one thread per column, k ascending (:146-178)
      for (int c = tid; c < nc; c += NT) {
        T* ac = A + (int64_t)(c1 + c) * n;
        T u[NB];
#pragma unroll
        for (int j = 0; j < NB; ++j) u[j] = j < kb ? ac[k0 + j] : T(0);
#pragma unroll
        for (int j = 0; j < NB; ++j)
#pragma unroll
          for (int i = j + 1; i < NB; ++i)
            if (i < kb) u[i] = fma(-sm.P[j * kBatchMaxN + k0 + i], u[j], u[i]);
#pragma unroll
        for (int j = 0; j < NB; ++j)
          if (j < kb) {
            ac[k0 + j] = u[j];
            sm.U[j * kBatchMaxN + c] = u[j];
          }
      }
      __syncthreads();
      // A22 -= L21 * U12, each element k ascending (:186-656)
      const int nr = n - c1;
      const int lane = tid & 31, warp = tid >> 5;
      for (int c = warp; c < nc; c += NT / 32) {   // a warp per column, lanes down the rows
        T u[NB];
#pragma unroll
        for (int j = 0; j < NB; ++j) u[j] = j < kb ? sm.U[j * kBatchMaxN + c] : T(0);
        T* acol = A + c1 + (int64_t)(c1 + c) * n;
        for (int i = lane; i < nr; i += 32) {
          T v = acol[i];
#pragma unroll
          for (int j = 0; j < NB; ++j)
            if (j < kb) v = fma(-sm.P[j * kBatchMaxN + c1 + i], u[j], v);
          acol[i] = v;
        }
      }
    }
    __syncthreads();
  }
  return info;
}

// x := A \ x with the factors of factor_system (src/factorization.jl:433-457),
// x held in shared memory.
template <typename T, int NT>
__device__ void solve_system(const T* __restrict__ LU, int n, const int32_t* __restrict__ ipiv,
                             T* x) {
  if (threadIdx.x == 0)
    for (int i = 0; i < n; ++i) {
      const int p = ipiv[i] - 1;
      if (p != i) { const T t = x[i]; x[i] = x[p]; x[p] = t; }
    }
  __syncthreads();
  for (int j = 0; j < n; ++j) {
    const T xj = x[j];
    for (int i = j + 1 + threadIdx.x; i < n; i += NT) x[i] = fma(-LU[i + (int64_t)j * n], xj, x[i]);
    __syncthreads();
  }
  for (int j = n - 1; j >= 0; --j) {
    if (threadIdx.x == 0) x[j] = x[j] / LU[j + (int64_t)j * n];
    __syncthreads();
    const T xj = x[j];
    for (int i = threadIdx.x; i < j; i += NT) x[i] = fma(-LU[i + (int64_t)j * n], xj, x[i]);
    __syncthreads();
  }
}

template <int NT>
__device__ __forceinline__ double block_max(double v, double* red) {
  for (int off = 16; off; off >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, off));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  double m = 0;
  for (int w = 0; w < NT / 32; ++w) m = fmax(m, red[w]);
  __syncthreads();
  return m;
}

template <typename T, int NB>
constexpr size_t batch_smem() {
  return (size_t)2 * NB * kBatchMaxN * sizeof(T) + kBatchMaxN * sizeof(double) * 3 + 256;
}

// FP64: factor in place (Awork holds a copy of A) and solve; x overwrites b.
template <int NT, int NB>
__global__ void __launch_bounds__(NT)
batch_fp64_kernel(BatchDev d, double* __restrict__ Awork, double* __restrict__ X,
                  int32_t* __restrict__ ipiv_all, int only_flagged) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  SysSmem<double> sm;
  sm.P = reinterpret_cast<double*>(smem_raw);
  sm.U = sm.P + NB * kBatchMaxN;
  sm.x = sm.U + NB * kBatchMaxN;
  sm.red_v = sm.x + kBatchMaxN;
  sm.red_i = reinterpret_cast<int*>(sm.red_v + 32);
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
    int32_t* ipiv = ipiv_all + d.b_off[s];
    const int64_t info = factor_system<double, NT, NB>(A, n, ipiv, sm);
    if (threadIdx.x == 0) { d.info[s] = info; if (only_flagged) d.flag[s] = 0; }
    if (info == 0) {
      double* x = X + d.b_off[s];
      for (int i = threadIdx.x; i < n; i += NT) sm.x[i] = x[i];
      __syncthreads();
      solve_system<double, NT>(A, n, ipiv, sm.x);
      for (int i = threadIdx.x; i < n; i += NT) x[i] = sm.x[i];
    }
    __syncthreads();
  }
}

// Mixed: FP32 factors of each system, FP64 refinement against the FP64 A.
template <int NT, int NB>
__global__ void __launch_bounds__(NT)
batch_mixed_kernel(BatchDev d, const double* __restrict__ A64, float* __restrict__ A32,
                   double* __restrict__ X, double* __restrict__ Bcopy, int32_t* __restrict__ ipiv_all,
                   int maxit, double tol_per_n) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  SysSmem<float> sm;
  sm.P = reinterpret_cast<float*>(smem_raw);
  sm.U = sm.P + NB * kBatchMaxN;
  sm.x = sm.U + NB * kBatchMaxN;
  double* xd = reinterpret_cast<double*>(sm.x + kBatchMaxN);  // FP64 iterate
  double* rd = xd + kBatchMaxN;                               // FP64 residual
  double* redd = rd + kBatchMaxN;
  sm.red_v = reinterpret_cast<float*>(redd + 32);
  sm.red_i = reinterpret_cast<int*>(sm.red_v + 32);
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
    for (int64_t i = threadIdx.x; i < (int64_t)n * n; i += NT) F[i] = (float)A[i];
    __syncthreads();
    const int64_t info = factor_system<float, NT, NB>(F, n, ipiv, sm);
    // ||A||_inf and ||b||_inf
    double ra = 0, bm = 0;
    for (int i = threadIdx.x; i < n; i += NT) {
      double acc = 0;
      for (int j = 0; j < n; ++j) acc += fabs(A[i + (int64_t)j * n]);
      ra = fmax(ra, acc);
      bm = fmax(bm, fabs(b[i]));
      xd[i] = 0.0;
      rd[i] = b[i];
    }
    const double anorm = block_max<NT>(ra, redd);
    const double bnorm = block_max<NT>(bm, redd);
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
            for (int j = 0; j < n; ++j) acc = fma(-A[i + (int64_t)j * n], xd[j], acc);
            rd[i] = acc;
          }
          __syncthreads();
        }
        double rm = 0, xm = 0;
        for (int i = threadIdx.x; i < n; i += NT) { rm = fmax(rm, fabs(rd[i])); xm = fmax(xm, fabs(xd[i])); }
        const double rn = block_max<NT>(rm, redd);
        const double xn = block_max<NT>(xm, redd);
        const double den = anorm * xn + bnorm;
        const double be = den > 0 ? rn / den : (rn == 0 ? 0.0 : INFINITY);
        if (be <= tol) { ok = true; break; }
        if (!(be < 0.9 * prev) && it >= 2) break;  // stagnation
        prev = be;
        if (it == maxit) break;
        // d = LU32 \ (r / s) * s
        const double sc = rn > 0 && isfinite(rn) ? ldexp(1.0, ilogb(rn)) : 1.0;
        for (int i = threadIdx.x; i < n; i += NT) sm.x[i] = (float)(rd[i] / sc);
        __syncthreads();
        solve_system<float, NT>(F, n, ipiv, sm.x);
        for (int i = threadIdx.x; i < n; i += NT) xd[i] += sc * (double)sm.x[i];
        __syncthreads();
      }
    }
    if (ok)
      for (int i = threadIdx.x; i < n; i += NT) xo[i] = xd[i];
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
                       (int)batch_smem<double, NB>());
  cudaFuncSetAttribute(batch_mixed_kernel<NT, NB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)(batch_smem<float, NB>() + 3 * kBatchMaxN * sizeof(double)));
}

template <int NT, int NB>
cudaError_t launch_fp64(const BatchDev& d, int ctas, gblu_batch* b, double* Awork, int only_flagged,
                        cudaStream_t s) {
  LaunchScope ls(K_BATCH, 0.0, 0.0, s);
  batch_fp64_kernel<NT, NB><<<ctas, NT, batch_smem<double, NB>(), s>>>(d, Awork, b->d_X, b->d_ipiv,
                                                                       only_flagged);
  return cudaGetLastError();
}

template <int NT, int NB>
cudaError_t launch_mixed(const BatchDev& d, int ctas, gblu_batch* b, cudaStream_t s) {
  LaunchScope ls(K_BATCH, 0.0, 0.0, s);
  batch_mixed_kernel<NT, NB><<<ctas, NT, batch_smem<float, NB>() + 3 * kBatchMaxN * sizeof(double), s>>>(
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
  configure_batch_kernels<128, 8>();
  configure_batch_kernels<128, 16>();
  configure_batch_kernels<256, 8>();
  configure_batch_kernels<256, 16>();
  configure_batch_kernels<512, 16>();
}

bool batch_config_supported(int nt, int nb) {
  return (nt == 128 && (nb == 8 || nb == 16)) || (nt == 256 && (nb == 8 || nb == 16)) ||
         (nt == 512 && nb == 16);
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
    k.ctas = di.num_sms * (k.nt <= 128 ? 4 : (k.nt <= 256 ? 2 : 1));
    out.push_back(k);
    lo = k.hi + 1;
  }
  (void)b;
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
      // fallback: copy of A (A64 must stay intact for later solves)
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
  const int nbuckets_max = 8;
  size_t bytes = 0;
  auto add = [&](size_t x) { size_t o = bytes; bytes += align256(x); return o; };
  size_t o_sizes = add(count * 4 + 4), o_order = add(count * 4 + 4), o_aoff = add(count * 8 + 8),
         o_boff = add(count * 8 + 8), o_info = add(count * 8 + 8), o_flag = add(count * 4 + 4),
         o_iters = add(count * 4 + 4),
         o_q = add(2 * nbuckets_max * 4), o_A = add(b->a_total * 8 + 8), o_X = add(b->b_total * 8 + 8),
         o_ipiv = add(b->b_total * 4 + 4);
  size_t o_A32 = 0, o_B = 0, o_Aw = 0;
  if (precision != GBLU_FP64) {
    o_A32 = add(b->a_total * 4 + 4);
    o_B = add(b->b_total * 8 + 8);
    o_Aw = add(b->a_total * 8 + 8);
  }
  int32_t st = ctx_alloc(ctx, bytes, &b->arena);
  if (st) { delete b; return st; }
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
  if (precision != GBLU_FP64) {
    b->d_A32 = reinterpret_cast<float*>(base + o_A32);
    b->d_B = reinterpret_cast<double*>(base + o_B);
    b->d_Awork = reinterpret_cast<double*>(base + o_Aw);
  }
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
  const int32_t edges[2] = {64, 128};
  const int32_t nts[3] = {128, 256, 256};
  const int32_t nbs[3] = {8, 16, 16};
  default_buckets(b, b->buckets, edges, 2, nts, nbs, ctx->device);
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
    k.ctas = (ctas && ctas[i] > 0) ? ctas[i] : di.num_sms * (k.nt <= 128 ? 4 : (k.nt <= 256 ? 2 : 1));
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
    GBLU_CK(ctx, cudaMemcpyAsync(b->d_Awork, b->d_A, b->a_total * 8, cudaMemcpyDeviceToDevice, s), "batch A copy");
  }
  {
    // one graph launch runs every persistent kernel of the schedule; the scope
    // times the whole graph and the counters record each kernel it holds
    int nk = 0;
    for (auto& k : b->buckets) nk += k.count > 0 ? (b->precision != GBLU_FP64 ? 2 : 1) : 0;
    LaunchScope ls(K_BATCH, batch_flops(b), (double)b->a_total * 8.0 * (b->precision != GBLU_FP64 ? 4.0 : 2.0), s);
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
