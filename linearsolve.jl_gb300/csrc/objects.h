// Host objects behind the opaque handles of gblu.h, and the helpers the
// translation units share.
#pragma once
#include <cuda_runtime.h>

#include <initializer_list>
#include <mutex>
#include <string>

#include "gblu_internal.h"
#include "profile.h"
#include "refine.h"

struct gblu_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  uint64_t budget = 0;
  uint64_t in_use = 0;
  std::recursive_mutex mu;
  std::string last_error;
  gblu::Profiler prof;
  // pinned staging for large uploads from pageable host memory: two chunks
  // of stage_chunk bytes, each with the event of the copy that last read it
  char* stage = nullptr;
  size_t stage_chunk = 0;
  cudaEvent_t stage_ev[2] = {nullptr, nullptr};
};

struct gblu_factor {
  int64_t m = 0, n = 0, ld = 0;
  int32_t precision = GBLU_FP64;
  bool factored = false;
  int64_t info = 0;
  uint64_t bytes = 0;
  void* arena = nullptr;
  // views into the arena
  double* lu64 = nullptr;  // FP64 factors (FP64) or FP64 copy of A (mixed)
  float* lu32 = nullptr;   // FP32 factors (mixed)
  int64_t* ipiv = nullptr;
  int32_t* perm = nullptr;
  int64_t* info_dev = nullptr;
  gblu::GetrfPlan<double> rf64;
  gblu::GetrfPlan<float> rf32;
  gblu::GetrsPlan<double> rs64;
  gblu::GetrsPlan<float> rs32;
  double* rhs = nullptr;  // device RHS staging, rhs_cols columns of length ld
  int64_t rhs_cols = 0;
  gblu::RefineWork refine;  // mixed-precision refinement buffers
  // FP64 fallback factorization of a mixed factor (allocated on first use)
  void* fb_arena = nullptr;
  uint64_t fb_bytes = 0;
  double* fb_lu = nullptr;
  int64_t* fb_ipiv = nullptr;
  int32_t* fb_perm = nullptr;
  int64_t* fb_info = nullptr;
  gblu::GetrfPlan<double> fb_rf;
  gblu::GetrsPlan<double> fb_rs;
  bool fb_valid = false;   // fallback factors hold the current A
  bool use_fb = false;     // solves go straight to the fallback factors
  double growth = 0;       // max|U| / max|A| of the last low-precision getrf
  // FP64 copy of A kept by a GBLU_FP64 factor for residual checks
  double* a_keep = nullptr;
  bool a_keep_valid = false;  // a_keep holds the matrix of the last getrf
  // residual-check buffers (allocated on the first gblu_residual_norm)
  void* chk_arena = nullptr;
  uint64_t chk_bytes = 0;
  // fast getrs: inverted diagonal blocks of the factors (rs64 or rs32 .inv)
  void* inv_arena = nullptr;
  uint64_t inv_bytes = 0;
  bool inv_owned = false;  // allocated on its own (else a view into the factor arena)
  bool inv_valid = false;  // inverses belong to the current factors
  // the factorization's launch sequence, captured on its second run and
  // replayed from then on (it depends only on the factor's shape)
  cudaGraphExec_t getrf_exec = nullptr;
  gblu::LaunchCounts getrf_graph_counts;  // the captured sequence's launches
  int getrf_runs = 0;
  bool getrf_graph_failed = false;
  // low-precision pivoting of a mixed factor (GBLU_PIVOT_*); for RBT the
  // butterflies' random diagonals (4 n floats: left then right, each R1 S1
  // R2 S2 of n/2), filled on the first switch to RBT
  int32_t pivoting = 0;
  float* rbt = nullptr;
  bool rbt_ready = false;
};

namespace gblu {

int32_t fail(gblu_ctx* ctx, int32_t code, const char* fmt, ...);
int32_t cuda_fail(gblu_ctx* ctx, cudaError_t e, const char* what);
int32_t ctx_alloc(gblu_ctx* ctx, size_t bytes, void** out);
void ctx_free(gblu_ctx* ctx, void* p, size_t bytes);
int32_t check_device_errors(gblu_ctx* ctx, std::initializer_list<DevScratch*> scr);
int32_t upload_matrix(gblu_ctx* ctx, double* dst, int64_t ld_dst, const double* src,
                      int64_t ld_src, int64_t rows, int64_t cols, int32_t loc);
int32_t ensure_rhs(gblu_ctx* ctx, gblu_factor* f, int64_t cols);
// FP64 factorization of the FP64 copy of A of a mixed factor (fb_* fields).
int32_t factor_fp64_fallback(gblu_ctx* ctx, gblu_factor* f, int64_t* info_out);
// Bytes of the arena gblu_factor_create allocates for these arguments.
size_t factor_arena_bytes(int64_t m, int64_t n, int32_t precision, int device);
// Fast getrs: invert the factors' diagonal blocks if the current factors'
// inverses are not there yet (asynchronous on the context stream).
int32_t ensure_inverse(gblu_ctx* ctx, gblu_factor* f);

// Small uneven systems (n <= 256) solved together by one launch of the
// batched kernels, for a system list that changes at every call (batched.cu;
// the serving loop's small-system lane).  Device and pinned buffers grow to
// the largest call and are reused.  System i: A[i] (n_i x n_i, column-major,
// host) x = b[i] (host), x written to x[i]; info[i] its getrf info; iters[i]
// (mixed precision) its refinement corrections, -1 if re-solved in FP64.
struct BatchLane;
BatchLane* batch_lane_create();
void batch_lane_destroy(gblu_ctx* ctx, BatchLane* lane);
int32_t batch_lane_solve(gblu_ctx* ctx, BatchLane* lane, int32_t precision, int count, const int32_t* sizes,
                         const double* const* A, const double* const* b, double* const* x, int64_t* info,
                         int32_t* iters);

inline size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

struct DeviceGuard {
  int prev = -1;
  explicit DeviceGuard(int dev) {
    cudaGetDevice(&prev);
    if (prev != dev) cudaSetDevice(dev);
  }
  ~DeviceGuard() {
    int cur = -1;
    cudaGetDevice(&cur);
    if (prev >= 0 && cur != prev) cudaSetDevice(prev);
  }
};

#define GBLU_CK(ctx, expr, what)                                   \
  do {                                                             \
    cudaError_t e_ = (expr);                                       \
    if (e_ != cudaSuccess) return ::gblu::cuda_fail(ctx, e_, what); \
  } while (0)

}  // namespace gblu
