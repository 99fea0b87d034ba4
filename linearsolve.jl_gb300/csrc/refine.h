// Mixed-precision refinement: FP32 factors, FP64 residuals and updates.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "gblu_internal.h"

struct gblu_ctx;
struct gblu_factor;

namespace gblu {

// Device buffers of the refinement loop for an n x n factor and up to W
// right-hand sides at a time, plus the GMRES basis.
struct RefineWork {
  int64_t n = 0, W = 0, restart = 0;
  double* x = nullptr;      // n x W   solution iterate
  double* r = nullptr;      // n x W   residual / GMRES work vector
  double* b = nullptr;      // n x W   right-hand sides
  float* d32 = nullptr;     // n x W   low-precision correction
  double* partial = nullptr;  // kSplit x n x W  deterministic partial sums
  double* V = nullptr;      // n x (restart + 1) x W   GMRES bases, one per column
  double* w = nullptr;      // n x W    GMRES work vectors
  double* h = nullptr;      // 3 x (restart + 1) x W   projections and norms
  unsigned long long* colmax = nullptr;  // 4 x W   |.|_inf per column (bit patterns)
  double* dots = nullptr;   // kDotBlocks x (restart + 1)
  double anorm = 0;         // ||A||_inf of the FP64 matrix (host copy)
  double* anorm_dev = nullptr;
  double amax = 0;          // max |A_ij| of the FP64 matrix (host copy)
  unsigned long long* growth_bits = nullptr;  // [0] max|A| (FP64 bits), [1] max|U| (FP32 bits)
  // GMRES state on the device, per column: Hessenberg matrix, rotations,
  // right-hand side g, solution y, and scalars (beta, 1/norm) / flags
  double* gm = nullptr;     // W x kGmStride doubles
  int* gflags = nullptr;    // W x 2 ints: stepping, basis size k
  int* gflags_host = nullptr;  // pinned: 2 slots x 2 x 8 ints, flags read one step behind
};

constexpr int kSplit = 16;       // column chunks of the residual GEMV
constexpr int kDotBlocks = 64;   // blocks of the deterministic dot products
constexpr int kGmresRestart = 30;
// per-column GMRES state: H ((m+1) x m), cs (m), sn (m), g (m+1), y (m+1),
// beta, 1/norm of the newest basis vector
constexpr int kGmH = 0;
constexpr int kGmCs = kGmH + (kGmresRestart + 1) * kGmresRestart;
constexpr int kGmSn = kGmCs + kGmresRestart;
constexpr int kGmG = kGmSn + kGmresRestart;
constexpr int kGmY = kGmG + kGmresRestart + 1;
constexpr int kGmBeta = kGmY + kGmresRestart + 1;
constexpr int kGmInv = kGmBeta + 1;
constexpr int kGmStride = kGmInv + 1;

size_t refine_bytes(int64_t n, int64_t W);
void refine_carve(RefineWork& w, char* base, int64_t n, int64_t W);

// FP64 A (ld) -> FP32 A32 (ld32), ||A||_inf and max |A_ij|, before the FP32
// getrf; write_f32 = false computes the norms only (the RBT path writes A32).
cudaError_t refine_prepare(RefineWork& w, int64_t n, const double* A, int64_t lda, float* A32,
                           int64_t ld32, cudaStream_t s, bool write_f32 = true);

// Random butterfly transform (depth 2, both sides) of the mixed factors'
// GBLU_PIVOT_RBT mode, over the leading n4 = n - n mod 4 rows and columns
// (the transforms are diag(W, I)).  rbt: 4 n4 floats, the left then the
// right butterflies' random diagonals, each R1 S1 R2 S2 of n4/2; n >= 4.
// B (FP32, ldb) = U^T A V for the FP64 A (lda), U = diag(W_L / 2, I),
// V = diag(W_R / 2, I).
cudaError_t rbt_matrix_launch(int64_t n, const double* A, int64_t lda, float* B, int64_t ldb,
                              const float* rbt, cudaStream_t s);
// In place on the W columns of v (FP32, ldv): side 0 = U, 1 = V; transposed:
// v := U^T v (before the triangular solves), else v := V v (after); entries
// past n4 are unchanged.
cudaError_t rbt_vec_launch(int64_t n, int W, float* v, int64_t ldv, const float* rbt, int side,
                           bool transposed, cudaStream_t s);
// The random diagonals (exp(u / 10), u uniform in (-1/2, 1/2), a fixed seed).
void rbt_fill_host(int64_t n, float* out);

// max |U_ij| of the FP32 factors (upper triangle of LU) into w.growth_bits[1];
// asynchronous, read back with refine_growth after the stream synchronises.
cudaError_t refine_growth_launch(RefineWork& w, int64_t n, const float* LU, int64_t ld, cudaStream_t s);
// max|U| / max|A| from the host copy of growth_bits (inf for a non-finite max|U|).
double refine_growth(const RefineWork& w, unsigned long long umax_bits);

// The default growth_limit of a factor precision (GBLU_FP32 / BF16 / FP16).
double growth_limit_default(int32_t precision);

gblu_refine_opts refine_default_opts();

// The refined solve behind gblu_getrs / gblu_solve_refined for a factor.
int32_t refine_solve(gblu_ctx* ctx, gblu_factor* f, char trans, int64_t nrhs, double* B,
                     int64_t ldb, int32_t b_loc, const gblu_refine_opts* opts,
                     gblu_refine_stats* stats);

}  // namespace gblu
