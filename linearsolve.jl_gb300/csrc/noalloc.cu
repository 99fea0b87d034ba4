// gblu_dgetrs_noalloc: the FP64 getrs for callers that cannot allocate.
//
// Who cannot allocate, and why:
//  * solver loops that call the back-solve once per step (Newton iterations
//    inside an ODE integrator are the typical LinearSolve.jl caller): a
//    cudaMalloc/cudaFree there synchronises the whole device and stalls the
//    loop, and such callers are held to zero-allocation budgets;
//  * a host that has committed all device memory to a fixed budget up front.
// They already own the factors, pivots and right-hand sides in device memory
// and need the solve to touch no allocator at all.
//
// The scratch the wavefront getrs kernels need (per-block-row flags, the
// ticket and error words, the row permutation and one intermediate vector
// block) lives in one file-scope __device__ array of a fixed size, so every
// GPU that loads this library holds it until the process exits.  Host code
// cannot use the array's name as a device address: the address is looked up
// with cudaGetSymbolAddress once per device, with that device current, on the
// first call made on that device.
#include <cuda_runtime.h>

#include <mutex>

#include "gblu_internal.h"
#include "objects.h"

namespace gblu {
namespace {

constexpr int64_t kNoAllocMaxN = 16384;      // largest n accepted
constexpr int64_t kNoAllocCols = 8;          // right-hand sides per pass (getrs_launch's chunk)
constexpr size_t kOffFlags = 256;
constexpr size_t kOffPerm = kOffFlags + getrs_flag_bytes(kNoAllocMaxN);
constexpr size_t kOffWork = (kOffPerm + kNoAllocMaxN * 4 + 255) & ~size_t(255);
constexpr size_t kScratchBytes = kOffWork + kNoAllocMaxN * kNoAllocCols * sizeof(double);
// the carve below must hold what the sweeps use: the error / ticket words,
// the block-row flags of kGetrsTile-row blocks, the permutation, and one
// n x kNoAllocCols block of intermediate values
static_assert(sizeof(DevScratch) <= kOffFlags, "scratch words overlap the flags");
static_assert(kOffPerm - kOffFlags >= getrs_flag_bytes(kNoAllocMaxN), "flag area too small");
static_assert(kScratchBytes - kOffWork >= (size_t)kNoAllocMaxN * kNoAllocCols * sizeof(double),
              "intermediate block too small");

// ~1.1 MB on every device that loads the library, for the life of the process.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

std::mutex g_setup_mu;
void* g_scratch_addr[64] = {nullptr};

// Once per device, with that device current: the device address of the array.
int32_t scratch_address(int device, void** out) {
  if (device < 0 || device >= 64)
    return fail(nullptr, GBLU_EUNSUPPORTED, "gblu_dgetrs_noalloc: device %d out of range", device);
  std::lock_guard<std::mutex> g(g_setup_mu);
  if (!g_scratch_addr[device]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p)
      return fail(nullptr, GBLU_ECUDA, "gblu_dgetrs_noalloc: cudaGetSymbolAddress: %s",
                  cudaGetErrorString(e));
    g_scratch_addr[device] = p;
    getrf_configure(device);  // shared-memory opt-in of the permutation kernel
  }
  *out = g_scratch_addr[device];
  return GBLU_OK;
}

}  // namespace
}  // namespace gblu

using namespace gblu;

extern "C" int32_t gblu_dgetrs_noalloc(char trans, int64_t n, int64_t nrhs, const double* dLU,
                                       int64_t lda, const int64_t* d_ipiv, double* dB,
                                       int64_t ldb, void* stream) {
  if (!(trans == 'N' || trans == 'n' || trans == 'T' || trans == 't' || trans == 'C' || trans == 'c'))
    return fail(nullptr, GBLU_EINVAL, "gblu_dgetrs_noalloc: trans must be 'N' or 'T'");
  if (n < 0 || nrhs < 0) return fail(nullptr, GBLU_EINVAL, "gblu_dgetrs_noalloc: negative size");
  if (n > kNoAllocMaxN)
    return fail(nullptr, GBLU_EUNSUPPORTED,
                "gblu_dgetrs_noalloc: n = %lld exceeds the fixed scratch limit n <= %lld",
                (long long)n, (long long)kNoAllocMaxN);
  if (lda < (n > 1 ? n : 1) || ldb < (n > 1 ? n : 1))
    return fail(nullptr, GBLU_EINVAL, "gblu_dgetrs_noalloc: leading dimension < n");
  if (n == 0 || nrhs == 0) return GBLU_OK;
  if (!dLU || !d_ipiv || !dB) return fail(nullptr, GBLU_EINVAL, "gblu_dgetrs_noalloc: NULL pointer");
  int device = 0;
  cudaError_t e = cudaGetDevice(&device);
  if (e != cudaSuccess) return cuda_fail(nullptr, e, "gblu_dgetrs_noalloc: cudaGetDevice");
  void* base = nullptr;
  int32_t st = scratch_address(device, &base);
  if (st) return st;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  char* c = reinterpret_cast<char*>(base);
  DevScratch* scr = reinterpret_cast<DevScratch*>(c);
  GetrsPlan<double> p;
  p.n = n;
  p.lda = lda;
  p.LU = dLU;
  p.ipiv = d_ipiv;
  p.perm = reinterpret_cast<int32_t*>(c + kOffPerm);
  p.scratch = scr;
  p.flags = reinterpret_cast<int32_t*>(c + kOffFlags);
  p.work = reinterpret_cast<double*>(c + kOffWork);
  p.work_cols = kNoAllocCols;
  // the array keeps the previous call's contents: start from clean words
  e = cudaMemsetAsync(scr, 0, sizeof(DevScratch), s);
  if (e == cudaSuccess) e = perm_build_launch(d_ipiv, n, n, reinterpret_cast<int32_t*>(c + kOffPerm), scr, s);
  if (e == cudaSuccess) e = getrs_launch<double>(p, trans, nrhs, dB, ldb, nullptr, s);
  int32_t err = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&err, &scr->error, sizeof(err), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_fail(nullptr, e, "gblu_dgetrs_noalloc");
  if (err == DEV_TIMEOUT_SOLVE || err == DEV_TIMEOUT_PANEL)
    return fail(nullptr, GBLU_ETIMEOUT, "gblu_dgetrs_noalloc: device wait timed out");
  if (err != DEV_OK) return fail(nullptr, GBLU_EINVAL, "gblu_dgetrs_noalloc: invalid ipiv");
  return GBLU_OK;
}
