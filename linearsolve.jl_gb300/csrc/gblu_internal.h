// Internal declarations shared by the gblu translation units.
//
// Layout conventions (identical to LAPACK, which is what LinearSolve.jl's
// LUFactorization hands to getrf/getrs, src/openblas.jl:131-154,247-278):
//   * matrices are column-major with a leading dimension `ld` >= rows;
//   * ipiv is int64, 1-based, the row-interchange sequence of getrf;
//   * info is int64: 0 ok, k > 0 first exactly-zero pivot (1-based).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>
#include <string>

#include "../../include/gblu.h"

namespace gblu {

// ---------------------------------------------------------------------------
// Device-side error words.  Every bounded wait in a kernel writes one of these
// into the scratch error word instead of spinning forever.
enum : int32_t {
  DEV_OK = 0,
  DEV_TIMEOUT_PANEL = 1,    // grid barrier in the panel kernel gave up
  DEV_TIMEOUT_SOLVE = 2,    // a getrs block row waited too long for a predecessor
  DEV_BAD_PIVOT_INDEX = 3,  // ipiv entry out of range (corrupt input)
  DEV_TIMEOUT_GEMM = 4,     // tcgen05 GEMM pipeline wait gave up
};

// Scratch words used by the cooperative panel kernel and the wavefront solve.
struct DevScratch {
  unsigned int barrier;  // grid-barrier arrival counter (zeroed per launch)
  int32_t error;         // DEV_* code, sticky
  unsigned int ticket;   // wavefront block-row ticket (zeroed per launch)
  int32_t pad;
};

// Panel-kernel exchange slots: per CTA one pivot candidate and its panel row.
template <typename T>
struct PanelSlots {
  T* cand_val;       // [2][G]       |candidate|
  int64_t* cand_row; // [2][G]       global row index of candidate (-1: none)
  T* cand_rowvals;   // [2][G][W]    candidate's panel row
  T* diag_rowvals;   // [2][W]       current diagonal row
};

// ---------------------------------------------------------------------------
// Host-side helpers

// Per-device launch facts, queried once.
struct DeviceInfo {
  int device = 0;
  int num_sms = 0;
  size_t smem_optin = 0;
  int cc_major = 0, cc_minor = 0;
};

const DeviceInfo& device_info(int device);

// ---------------------------------------------------------------------------
// Kernel launch wrappers (implemented in getrf.cu / getrs.cu / refine.cu).
// All are asynchronous on `stream` and return a cudaError_t from the launch.

template <typename T>
struct GetrfPlan {
  int64_t m = 0, n = 0, lda = 0;
  T* A = nullptr;            // device matrix, factored in place
  int64_t* ipiv = nullptr;   // device, length min(m,n), 1-based
  int64_t* info = nullptr;   // device scalar
  int32_t* perm = nullptr;   // device, length m: (P A)[i] = A[perm[i]]
  DevScratch* scratch = nullptr;
  PanelSlots<T> slots{};
  int panel_width = 32;      // leaf width of the recursion
  int panel_ctas = 0;        // CTAs of the cooperative panel kernel (0: auto)
  int trsm_base = 128;       // base size of the recursive TRSM
  bool use_cluster_panel = true;  // DSMEM cluster panel when the panel fits
  bool use_reg_panel = true;      // register-resident cluster panel when the panel fits
  // FP32 working matrix only: trailing updates on tcgen05 with 16-bit operands
  int tc_mode = 0;           // 0 SIMT FP32, 1 BF16 operands, 2 FP16 operands (scaled)
  void* tc_work = nullptr;   // conversion buffers for the operands
  size_t tc_work_bytes = 0;
  // FP32 working matrix only: tournament pivoting for leaves taller than
  // 512 rows (tslu.cu), instead of partial pivoting
  bool tslu = false;
  void* tslu_work = nullptr; // tslu_work_bytes()
  // FP32 working matrix only: no pivoting (the random-butterfly-transformed
  // factors): each leaf is a no-interchange getf2 of its top block and a
  // parallel solve below it (tslu.cu), with no laswp
  bool nopivot = false;
  // FP32 working matrix of the 16-bit-operand factors only: TRSM base blocks
  // of 65..128 rows solved through inverses of L's diagonal blocks, each
  // computed once per getrf and kept in one of these 128 x 128 slots
  float* trsm_inv = nullptr;
  int trsm_inv_slots = 0;
};

// Slots and bytes of the TRSM inverse cache of an n-column factorization.
int trsm_inv_slot_count(int64_t n);
size_t trsm_inv_bytes(int64_t n);

// Tournament-pivoting panel of the low-precision getrf (tslu.cu).
size_t tslu_work_bytes();
bool tslu_fits(int64_t rows, int w);
void tslu_configure(int device);
cudaError_t tslu_panel_launch(float* A, int64_t lda, int64_t m, int64_t c0, int w, int64_t* ipiv,
                              int64_t* info, void* work, DevScratch* scr, cudaStream_t s);
// No-pivot leaf (GetrfPlan::nopivot); work: the tslu work area (its ticket).
cudaError_t genp_panel_launch(float* A, int64_t lda, int64_t m, int64_t c0, int w, int64_t* ipiv,
                              int64_t* info, void* work, cudaStream_t s);

// FP32 SIMT update C -= A * B in the reference's per-element order (getrf.cu).
cudaError_t simt_gemm_sub_f32(int64_t M, int64_t N, int64_t K, const float* A, int64_t lda,
                              const float* B, int64_t ldb, float* C, int64_t ldc, cudaStream_t s);

// tcgen05 trailing update C -= round16(A) * round16(B) (gemm_tc.cu).
size_t tc_work_bytes(int64_t M, int64_t N, int64_t K);
void tc_configure(int device);
cudaError_t tc_gemm_sub(int mode, int64_t M, int64_t N, int64_t K, const float* A, int64_t lda,
                        const float* B, int64_t ldb, float* C, int64_t ldc, void* work, int* err,
                        cudaStream_t s);

template <typename T>
cudaError_t getrf_launch(const GetrfPlan<T>& p, cudaStream_t stream);

// Per-device kernel attributes (shared-memory opt-in); once per device, outside capture.
void getrf_configure(int device);
void getrs_configure(int device);
cudaError_t perm_build_launch(const int64_t* ipiv, int64_t kmax, int64_t m, int32_t* perm,
                              DevScratch* scr, cudaStream_t s);

// Bytes of device scratch getrf needs for an m x n matrix (slots + scratch).
size_t getrf_scratch_bytes(int64_t m, int64_t n, int elem_size, int panel_width,
                           int device);
template <typename T>
void getrf_carve(GetrfPlan<T>& p, void* base, size_t bytes, int device);

// Block-row height (and tile width) of the getrs sweeps, and the per-block-row
// flag words they use for an n-row solve (callers that lay out getrs scratch
// themselves size it from these).
constexpr int kGetrsTile = 64;
constexpr size_t getrs_flag_bytes(int64_t n) {
  return 2 * (size_t)((n + kGetrsTile - 1) / kGetrsTile) * sizeof(int32_t);
}

template <typename T>
struct GetrsPlan {
  int64_t n = 0, lda = 0;
  const T* LU = nullptr;
  const int32_t* perm = nullptr;
  const int64_t* ipiv = nullptr;
  DevScratch* scratch = nullptr;
  int32_t* flags = nullptr;  // 2 * nblocks
  T* work = nullptr;         // n * nrhs_chunk
  int64_t work_cols = 0;
  // fast mode: diagonal blocks applied through their inverses (not the
  // reference's per-row order; backward-error accurate, not bit-exact)
  bool fast = false;
  T* inv = nullptr;          // getrs_inverse_bytes(n): [block][L, U][64 x 64]
};

// Device bytes of the inverted 64 x 64 diagonal blocks of L and U (fast getrs).
size_t getrs_inverse_bytes(int64_t n, int elem_size);
// Invert the diagonal blocks of the factors of p into p.inv (after each getrf).
template <typename T>
cudaError_t getrs_invert_launch(const GetrsPlan<T>& p, cudaStream_t stream);

// In-place solve op(A) X = B for nrhs columns of B (ldb), trans 'N' or 'T'.
template <typename T>
cudaError_t getrs_launch(const GetrsPlan<T>& p, char trans, int64_t nrhs, T* B,
                         int64_t ldb, uint32_t* epoch, cudaStream_t stream);

size_t getrs_scratch_bytes(int64_t n, int elem_size, int64_t work_cols);
template <typename T>
void getrs_carve(GetrsPlan<T>& p, void* base, size_t bytes, int64_t work_cols);

}  // namespace gblu
