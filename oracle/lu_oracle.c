/*
 * CPU oracle for the dense LU path -- TEST INFRASTRUCTURE ONLY.
 *
 * This file restates, in plain C, the reference's own in-tree getrf and getrs
 * so that the GPU library can be checked against it.  Nothing in the product
 * path links or calls this file: only the test-suite, the smoke check and the
 * CPU-baseline leg of the benchmark load it.
 *
 * What is restated (LinearSolve.jl v5.12.0):
 *   getrf  src/blocked_lufact.jl
 *     - pivot search              _blocked_lu_find_pivot      :38-54
 *     - unblocked LU (minmn <= 8) _blocked_lu_unblocked!      :59-89
 *     - panel getf2               _blocked_lu_panel!          :93-122
 *     - row interchanges (laswp)  _blocked_lu_swap_rows!      :126-141
 *     - unit-lower TRSM           _blocked_lu_trsm_unit_lower! :146-178
 *     - Schur update              _blocked_lu_schur*!         :186-656
 *     - driver                    _blocked_lufact!            :658-679
 *     - entry / panel width       _blocked_generic_lufact!    :715-743, :15
 *   getrs  src/factorization.jl
 *     - '_naive_lu_ldiv!' (vector) :433-457  (permute, unit-L forward, U backward)
 *     - transposed solve follows LAPACK dgetrs 'T' (the operation
 *       adjoint_factorization.jl reaches through ldiv!(adjoint(F), b)).
 *
 * Floating-point contract.  Every update of an element A[i,j] in the
 * reference is `muladd(-A[i,k], A[k,j], A[i,j])` (llvm.fmuladd, a fused
 * multiply-add on FMA hardware), applied for k = 1, 2, ... in ascending order;
 * the blocked kernels only change *when* an element is updated, never the
 * order of its own updates.  The factors are therefore independent of the
 * panel width, and this restatement uses C99 fma() in that same order.  The
 * multipliers are A[i,k] * inv(A[k,k]) with inv(x) = 1/x (blocked_lufact.jl:108).
 */
#include <math.h>
#include <stdint.h>
#include <string.h>

#define ORA_UNBLOCKED_CUTOFF 8 /* blocked_lufact.jl:10 */

#define DEFINE_GETRF(T, P, ABS, FMA)                                                  \
  /* _blocked_lu_find_pivot: NaN-ignoring max, first index of the max (:38-54).       \
   * Indices are 0-based here. */                                                     \
  static int64_t P##find_pivot(const T* A, int64_t lda, int64_t k, int64_t m,        \
                               T* amax_out) {                                         \
    T amax = (T)0;                                                                    \
    for (int64_t i = k; i < m; ++i) {                                                 \
      T a = ABS(A[i + k * lda]);                                                      \
      amax = (a > amax) ? a : amax;                                                   \
    }                                                                                 \
    int64_t kp = k;                                                                   \
    if (amax != (T)0) {                                                               \
      for (int64_t i = k; i < m; ++i)                                                 \
        if (ABS(A[i + k * lda]) == amax) { kp = i; break; }                           \
    }                                                                                 \
    *amax_out = amax;                                                                 \
    return kp;                                                                        \
  }                                                                                   \
  /* _blocked_lu_panel! (:93-122) over columns [j0, j1), rows [j0, m);               \
   * also serves as _blocked_lu_unblocked! (:59-89) when j0 = 0, j1 = n and the      \
   * swap covers all columns. */                                                      \
  static int64_t P##panel(T* A, int64_t lda, int64_t* ipiv, int64_t m, int64_t j0,  \
                          int64_t j1, int64_t sw0, int64_t sw1, int64_t info) {       \
    for (int64_t k = j0; k < j1; ++k) {                                               \
      T amax;                                                                         \
      int64_t kp = P##find_pivot(A, lda, k, m, &amax);                                \
      ipiv[k] = kp + 1;                                                               \
      if (A[kp + k * lda] != (T)0) {                                                  \
        if (k != kp) {                                                                \
          for (int64_t j = sw0; j < sw1; ++j) {                                       \
            T t = A[k + j * lda];                                                     \
            A[k + j * lda] = A[kp + j * lda];                                         \
            A[kp + j * lda] = t;                                                      \
          }                                                                           \
        }                                                                             \
        T inv = (T)1 / A[k + k * lda];                                                \
        for (int64_t i = k + 1; i < m; ++i) A[i + k * lda] *= inv;                    \
      } else if (info == 0) {                                                         \
        info = k + 1;                                                                 \
      }                                                                               \
      for (int64_t j = k + 1; j < j1; ++j) {                                          \
        T akj = A[k + j * lda];                                                       \
        for (int64_t i = k + 1; i < m; ++i)                                           \
          A[i + j * lda] = FMA(-A[i + k * lda], akj, A[i + j * lda]);                 \
      }                                                                               \
    }                                                                                 \
    return info;                                                                      \
  }                                                                                   \
  /* _blocked_lu_swap_rows! (:126-141): interchanges ipiv[k0:k1) on cols [c0,c1). */  \
  static void P##swap_rows(T* A, int64_t lda, const int64_t* ipiv, int64_t k0,       \
                           int64_t k1, int64_t c0, int64_t c1) {                      \
    for (int64_t j = c0; j < c1; ++j)                                                 \
      for (int64_t k = k0; k < k1; ++k) {                                             \
        int64_t kp = ipiv[k] - 1;                                                     \
        if (kp != k) {                                                                \
          T t = A[k + j * lda];                                                       \
          A[k + j * lda] = A[kp + j * lda];                                           \
          A[kp + j * lda] = t;                                                        \
        }                                                                             \
      }                                                                               \
  }                                                                                   \
  /* _blocked_lu_trsm_unit_lower! (:146-178): A[j0:j1, c0:c1] := L11 \ A12. */       \
  static void P##trsm_unit_lower(T* A, int64_t lda, int64_t j0, int64_t j1,          \
                                 int64_t c0, int64_t c1) {                            \
    for (int64_t c = c0; c < c1; ++c)                                                 \
      for (int64_t k = j0; k < j1; ++k) {                                             \
        T bk = A[k + c * lda];                                                        \
        for (int64_t i = k + 1; i < j1; ++i)                                          \
          A[i + c * lda] = FMA(-A[i + k * lda], bk, A[i + c * lda]);                  \
      }                                                                               \
  }                                                                                   \
  /* _blocked_lu_schur!: A[j1:m, c0:c1] -= A[j1:m, j0:j1] * A[j0:j1, c0:c1],          \
   * every element updated by k ascending (:186-293, :513-620). */                   \
  static void P##schur(T* A, int64_t lda, int64_t m, int64_t j0, int64_t j1,         \
                       int64_t c0, int64_t c1) {                                      \
    for (int64_t c = c0; c < c1; ++c)                                                 \
      for (int64_t k = j0; k < j1; ++k) {                                             \
        T bk = A[k + c * lda];                                                        \
        for (int64_t i = j1; i < m; ++i)                                              \
          A[i + c * lda] = FMA(-A[i + k * lda], bk, A[i + c * lda]);                  \
      }                                                                               \
  }                                                                                   \
  /* _blocked_generic_lufact! / _blocked_lufact! (:658-679, :715-743).              \
   * ipiv: 1-based, length min(m,n).  Returns info (0, or first zero pivot). */      \
  int64_t ora_##P##getrf_nb(int64_t m, int64_t n, T* A, int64_t lda, int64_t* ipiv, \
                            int64_t nb) {                                             \
    int64_t minmn = m < n ? m : n;                                                    \
    if (minmn <= 0) return 0;                                                         \
    if (nb < 1) nb = 1;                                                               \
    int64_t info = 0;                                                                 \
    for (int64_t j0 = 0; j0 < minmn; j0 += nb) {                                      \
      int64_t jb = (nb < minmn - j0) ? nb : (minmn - j0);                             \
      int64_t j1 = j0 + jb;                                                           \
      info = P##panel(A, lda, ipiv, m, j0, j1, j0, j1, info);                         \
      P##swap_rows(A, lda, ipiv, j0, j1, 0, j0);                                      \
      if (j1 < n) {                                                                   \
        P##swap_rows(A, lda, ipiv, j0, j1, j1, n);                                    \
        P##trsm_unit_lower(A, lda, j0, j1, j1, n);                                    \
        if (j1 < m) P##schur(A, lda, m, j0, j1, j1, n);                               \
      }                                                                               \
    }                                                                                 \
    return info;                                                                      \
  }

/* The unblocked whole-matrix form (_blocked_lu_unblocked!, :59-89): swaps span
 * all n columns and the rank-1 update runs over every column to the right. */
#define DEFINE_UNBLOCKED(T, P, FMA)                                                   \
  static int64_t P##panel_full(T* A, int64_t lda, int64_t* ipiv, int64_t m,          \
                               int64_t n) {                                           \
    int64_t minmn = m < n ? m : n, info = 0;                                          \
    for (int64_t k = 0; k < minmn; ++k) {                                             \
      T amax;                                                                         \
      int64_t kp = P##find_pivot(A, lda, k, m, &amax);                                \
      ipiv[k] = kp + 1;                                                               \
      if (A[kp + k * lda] != (T)0) {                                                  \
        if (k != kp)                                                                  \
          for (int64_t j = 0; j < n; ++j) {                                           \
            T t = A[k + j * lda];                                                     \
            A[k + j * lda] = A[kp + j * lda];                                         \
            A[kp + j * lda] = t;                                                      \
          }                                                                           \
        T inv = (T)1 / A[k + k * lda];                                                \
        for (int64_t i = k + 1; i < m; ++i) A[i + k * lda] *= inv;                    \
      } else if (info == 0) {                                                         \
        info = k + 1;                                                                 \
      }                                                                               \
      for (int64_t j = k + 1; j < n; ++j) {                                           \
        T akj = A[k + j * lda];                                                       \
        for (int64_t i = k + 1; i < m; ++i)                                           \
          A[i + j * lda] = FMA(-A[i + k * lda], akj, A[i + j * lda]);                 \
      }                                                                               \
    }                                                                                 \
    return info;                                                                      \
  }

/* forward declarations so the blocked driver can name the unblocked form */
static int64_t d_panel_full(double*, int64_t, int64_t*, int64_t, int64_t);
static int64_t s_panel_full(float*, int64_t, int64_t*, int64_t, int64_t);

DEFINE_GETRF(double, d_, fabs, fma)
DEFINE_GETRF(float, s_, fabsf, fmaf)
DEFINE_UNBLOCKED(double, d_, fma)
DEFINE_UNBLOCKED(float, s_, fmaf)

/* The default entry: the panel width and unblocked cutoff of the reference. */
int64_t ora_dgetrf(int64_t m, int64_t n, double* A, int64_t lda, int64_t* ipiv) {
  int64_t minmn = m < n ? m : n;
  if (minmn <= 0) return 0;
  if (minmn <= ORA_UNBLOCKED_CUTOFF) return d_panel_full(A, lda, ipiv, m, n);
  return ora_d_getrf_nb(m, n, A, lda, ipiv, minmn <= 160 ? 8 : 16);
}
int64_t ora_sgetrf(int64_t m, int64_t n, float* A, int64_t lda, int64_t* ipiv) {
  int64_t minmn = m < n ? m : n;
  if (minmn <= 0) return 0;
  if (minmn <= ORA_UNBLOCKED_CUTOFF) return s_panel_full(A, lda, ipiv, m, n);
  return ora_s_getrf_nb(m, n, A, lda, ipiv, minmn <= 160 ? 8 : 16);
}

/*
 * getrs.  trans = 'N': factorization.jl:433-457 applied to each RHS column
 * (swap b[i] <-> b[ipiv[i]] in ascending i, unit-lower forward sweep by
 * columns, then b[j] /= U[j,j] and the upper sweep by columns).
 * trans = 'T': U^T y = b (forward), L^T z = y (backward), then the
 * interchanges in descending order (LAPACK dgetrs 'T').  Inner products in
 * the transposed form run j ascending for U^T and j descending for L^T.
 */
#define DEFINE_GETRS(T, P, FMA)                                                       \
  void ora_##P##getrs(char trans, int64_t n, int64_t nrhs, const T* LU, int64_t lda, \
                      const int64_t* ipiv, T* B, int64_t ldb) {                       \
    for (int64_t c = 0; c < nrhs; ++c) {                                              \
      T* b = B + c * ldb;                                                             \
      if (trans == 'N' || trans == 'n') {                                             \
        for (int64_t i = 0; i < n; ++i) {                                             \
          int64_t p = ipiv[i] - 1;                                                    \
          if (p != i) { T t = b[i]; b[i] = b[p]; b[p] = t; }                          \
        }                                                                             \
        for (int64_t j = 0; j < n; ++j) {                                             \
          T bj = b[j];                                                                \
          for (int64_t i = j + 1; i < n; ++i) b[i] = FMA(-LU[i + j * lda], bj, b[i]); \
        }                                                                             \
        for (int64_t j = n - 1; j >= 0; --j) {                                        \
          b[j] /= LU[j + j * lda];                                                    \
          T bj = b[j];                                                                \
          for (int64_t i = 0; i < j; ++i) b[i] = FMA(-LU[i + j * lda], bj, b[i]);     \
        }                                                                             \
      } else {                                                                        \
        for (int64_t i = 0; i < n; ++i) {                                             \
          T acc = b[i];                                                               \
          for (int64_t j = 0; j < i; ++j) acc = FMA(-LU[j + i * lda], b[j], acc);     \
          b[i] = acc / LU[i + i * lda];                                               \
        }                                                                             \
        for (int64_t i = n - 1; i >= 0; --i) {                                        \
          T acc = b[i];                                                               \
          for (int64_t j = n - 1; j > i; --j) acc = FMA(-LU[j + i * lda], b[j], acc); \
          b[i] = acc;                                                                 \
        }                                                                             \
        for (int64_t i = n - 1; i >= 0; --i) {                                        \
          int64_t p = ipiv[i] - 1;                                                    \
          if (p != i) { T t = b[i]; b[i] = b[p]; b[p] = t; }                          \
        }                                                                             \
      }                                                                               \
    }                                                                                 \
  }

DEFINE_GETRS(double, d, fma)
DEFINE_GETRS(float, s, fmaf)

/* Batched form of the same two routines: `count` independent square systems
 * stored back to back (A_i column-major n_i x n_i at a_off[i], b_i at b_off[i]),
 * one RHS each.  info_out[i] receives each system's getrf info. */
void ora_dgesv_batched(int64_t count, const int64_t* sizes, const int64_t* a_off,
                       const int64_t* b_off, double* A, double* B, int64_t* ipiv_work,
                       int64_t* info_out) {
  for (int64_t s = 0; s < count; ++s) {
    int64_t n = sizes[s];
    double* a = A + a_off[s];
    double* b = B + b_off[s];
    info_out[s] = ora_dgetrf(n, n, a, n, ipiv_work);
    if (info_out[s] == 0) ora_dgetrs('N', n, 1, a, n, ipiv_work, b, n);
  }
}
