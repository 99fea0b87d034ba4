// The C ABI of libgblu (include/gblu.h): contexts, factor objects, getrf /
// getrs entry points and the LAPACK-shaped host entries.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstdarg>
#include <cstdlib>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "gblu_internal.h"
#include "objects.h"
#include "refine.h"

using namespace gblu;

namespace gblu {

thread_local Profiler* tl_profiler = nullptr;

const DeviceInfo& device_info(int device) {
  static std::mutex mu;
  static DeviceInfo cache[64];
  static bool have[64] = {false};
  if (device < 0 || device >= 64) device = 0;
  std::lock_guard<std::mutex> g(mu);
  if (!have[device]) {
    DeviceInfo d;
    d.device = device;
    cudaDeviceGetAttribute(&d.num_sms, cudaDevAttrMultiProcessorCount, device);
    int optin = 0;
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device);
    d.smem_optin = (size_t)optin;
    cudaDeviceGetAttribute(&d.cc_major, cudaDevAttrComputeCapabilityMajor, device);
    cudaDeviceGetAttribute(&d.cc_minor, cudaDevAttrComputeCapabilityMinor, device);
    if (d.num_sms <= 0) d.num_sms = 1;
    cache[device] = d;
    have[device] = true;
  }
  return cache[device];
}

}  // namespace gblu

namespace {
std::mutex g_err_mu;
std::string g_err;  // errors with no context
}  // namespace

namespace gblu {

int32_t fail(gblu_ctx* ctx, int32_t code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  if (ctx) ctx->last_error = buf;
  else {
    std::lock_guard<std::mutex> g(g_err_mu);
    g_err = buf;
  }
  return code;
}

int32_t cuda_fail(gblu_ctx* ctx, cudaError_t e, const char* what) {
  return fail(ctx, GBLU_ECUDA, "%s: %s", what, cudaGetErrorString(e));
}

#define CK GBLU_CK

int32_t ctx_alloc(gblu_ctx* ctx, size_t bytes, void** out) {
  if (ctx->budget && ctx->in_use + bytes > ctx->budget)
    return fail(ctx, GBLU_ENOMEM, "HBM budget exceeded: %llu in use + %llu requested > %llu",
                (unsigned long long)ctx->in_use, (unsigned long long)bytes,
                (unsigned long long)ctx->budget);
  cudaError_t e = cudaMalloc(out, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(ctx, GBLU_ENOMEM, "cudaMalloc(%llu): %s", (unsigned long long)bytes,
                cudaGetErrorString(e));
  }
  ctx->in_use += bytes;
  return GBLU_OK;
}

void ctx_free(gblu_ctx* ctx, void* p, size_t bytes) {
  if (!p) return;
  cudaFree(p);
  ctx->in_use -= std::min<uint64_t>(ctx->in_use, bytes);
}

// Reads back the sticky device error words of the plans a call used.
int32_t check_device_errors(gblu_ctx* ctx, std::initializer_list<DevScratch*> scr) {
  for (DevScratch* s : scr) {
    if (!s) continue;
    int32_t err = 0;
    cudaError_t e = cudaMemcpyAsync(&err, &s->error, sizeof(err), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "reading device error word");
    if (err != DEV_OK) {
      int32_t zero = 0;
      cudaMemcpyAsync(&s->error, &zero, sizeof(zero), cudaMemcpyHostToDevice, ctx->stream);
      cudaStreamSynchronize(ctx->stream);
      if (err == DEV_TIMEOUT_PANEL || err == DEV_TIMEOUT_SOLVE || err == DEV_TIMEOUT_GEMM)
        return fail(ctx, GBLU_ETIMEOUT, "device wait timed out (code %d)", err);
      return fail(ctx, GBLU_EINVAL, "device detected invalid pivot data (code %d)", err);
    }
  }
  return GBLU_OK;
}

// Bytes and carving of one factorization set (factors, ipiv, perm, info,
// getrf and getrs scratch) for an m x n matrix with leading dimension ld.
template <typename T>
size_t set_bytes(int64_t m, int64_t n, int64_t ld, int device, int64_t work_cols) {
  size_t b = align256((size_t)ld * n * sizeof(T));
  b += align256(std::max<int64_t>(1, std::min(m, n)) * sizeof(int64_t));
  b += align256(std::max<int64_t>(1, m) * sizeof(int32_t));
  b += align256(sizeof(int64_t));
  b += align256(getrf_scratch_bytes(m, n, sizeof(T), 32, device));
  b += align256(getrs_scratch_bytes(std::max<int64_t>(m, 1), sizeof(T), work_cols));
  return b;
}

template <typename T>
char* carve_set(char* c, int64_t m, int64_t n, int64_t ld, int device, int64_t work_cols,
                T** lu, int64_t** ipiv, int32_t** perm, int64_t** info, GetrfPlan<T>& rf,
                GetrsPlan<T>& rs) {
  auto take = [&](size_t b) { char* r = c; c += align256(b); return r; };
  *lu = reinterpret_cast<T*>(take((size_t)ld * n * sizeof(T)));
  *ipiv = reinterpret_cast<int64_t*>(take(std::max<int64_t>(1, std::min(m, n)) * sizeof(int64_t)));
  *perm = reinterpret_cast<int32_t*>(take(std::max<int64_t>(1, m) * sizeof(int32_t)));
  *info = reinterpret_cast<int64_t*>(take(sizeof(int64_t)));
  size_t fb = getrf_scratch_bytes(m, n, sizeof(T), 32, device);
  getrf_carve(rf, take(fb), fb, device);
  size_t sb = getrs_scratch_bytes(std::max<int64_t>(m, 1), sizeof(T), work_cols);
  rs.n = m;  // getrs plans are only used for square factors
  getrs_carve(rs, take(sb), sb, work_cols);
  rf.m = m;
  rf.n = n;
  rf.lda = ld;
  rf.A = *lu;
  rf.ipiv = *ipiv;
  rf.info = *info;
  rf.perm = *perm;
  rs.lda = ld;
  rs.LU = *lu;
  rs.perm = *perm;
  rs.ipiv = *ipiv;
  return c;
}

constexpr int64_t kWorkCols = 8;
constexpr int64_t kWorkColsFb = 8;

int32_t ensure_rhs(gblu_ctx* ctx, gblu_factor* f, int64_t cols) {
  if (f->rhs_cols >= cols) return GBLU_OK;
  if (f->rhs) ctx_free(ctx, f->rhs, (size_t)f->ld * f->rhs_cols * sizeof(double));
  f->rhs = nullptr;
  f->rhs_cols = 0;
  void* p = nullptr;
  int32_t st = ctx_alloc(ctx, (size_t)f->ld * cols * sizeof(double), &p);
  if (st) return st;
  f->rhs = reinterpret_cast<double*>(p);
  f->rhs_cols = cols;
  return GBLU_OK;
}


// Bytes of a factor object's arena (the carve in gblu_factor_create follows
// the same order); the serving loop admits new factorizations with it.
size_t factor_arena_bytes(int64_t m, int64_t n, int32_t precision, int device) {
  const int64_t ld = std::max<int64_t>(32, ((m + 31) / 32) * 32);
  if (precision == GBLU_FP64) return set_bytes<double>(m, n, ld, device, kWorkCols);
  size_t bytes = set_bytes<float>(m, n, ld, device, kWorkCols);
  bytes += align256((size_t)ld * n * sizeof(double));  // FP64 copy of A
  bytes += refine_bytes(m, kWorkCols);
  if (precision == GBLU_BF16 || precision == GBLU_FP16) {
    bytes += align256(tc_work_bytes(n, n / 2 + 64, n / 2 + 64));
    bytes += align256(trsm_inv_bytes(n));
  }
  bytes += align256(tslu_work_bytes());
  if (m == n && n > 0) bytes += align256(getrs_inverse_bytes(n, sizeof(float)));
  if (m == n && n >= 4) bytes += align256((size_t)4 * (n - n % 4) * sizeof(float));  // RBT diagonals
  return bytes;
}
}  // namespace gblu


extern "C" {

int32_t gblu_version(void) { return (1 << 16) | 0; }

int32_t gblu_create(gblu_ctx** out, int32_t device, uint64_t hbm_budget_bytes) {
  if (!out) return fail(nullptr, GBLU_EINVAL, "gblu_create: out is NULL");
  *out = nullptr;
  int count = 0;
  cudaError_t e = cudaGetDeviceCount(&count);
  if (e != cudaSuccess || count == 0) {
    cudaGetLastError();
    return fail(nullptr, GBLU_ENODEVICE, "no CUDA device: %s", cudaGetErrorString(e));
  }
  if (device < 0 || device >= count)
    return fail(nullptr, GBLU_EINVAL, "gblu_create: device %d out of range [0,%d)", device, count);
  DeviceGuard g(device);
  const DeviceInfo& di = device_info(device);
  if (di.cc_major < 10)
    return fail(nullptr, GBLU_EUNSUPPORTED, "device %d is sm_%d%d; libgblu is built for sm_103a",
                device, di.cc_major, di.cc_minor);
  {
    static std::mutex cfg_mu;
    static bool configured[64] = {false};
    std::lock_guard<std::mutex> lk(cfg_mu);
    if (device < 64 && !configured[device]) {
      getrf_configure(device);
      configured[device] = true;
    }
  }
  gblu_ctx* c = new (std::nothrow) gblu_ctx();
  if (!c) return fail(nullptr, GBLU_ENOMEM, "host allocation failed");
  c->device = device;
  c->budget = hbm_budget_bytes;
  e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    delete c;
    return fail(nullptr, GBLU_ECUDA, "cudaStreamCreate: %s", cudaGetErrorString(e));
  }
  *out = c;
  return GBLU_OK;
}

int32_t gblu_destroy(gblu_ctx* ctx) {
  if (!ctx) return GBLU_OK;
  {
    DeviceGuard g(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    cudaStreamDestroy(ctx->stream);
    for (cudaEvent_t& e : ctx->stage_ev)
      if (e) cudaEventDestroy(e);
    if (ctx->stage) cudaFreeHost(ctx->stage);
  }
  delete ctx;
  return GBLU_OK;
}

const char* gblu_last_error(const gblu_ctx* ctx) {
  if (ctx) return ctx->last_error.c_str();
  thread_local std::string copy;
  std::lock_guard<std::mutex> g(g_err_mu);
  copy = g_err;
  return copy.c_str();
}

int32_t gblu_ctx_stream(gblu_ctx* ctx, void** stream_out) {
  if (!ctx || !stream_out) return fail(ctx, GBLU_EINVAL, "gblu_ctx_stream: NULL argument");
  *stream_out = reinterpret_cast<void*>(ctx->stream);
  return GBLU_OK;
}

int32_t gblu_ctx_memory(gblu_ctx* ctx, uint64_t* in_use, uint64_t* budget) {
  if (!ctx) return fail(ctx, GBLU_EINVAL, "gblu_ctx_memory: NULL ctx");
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  if (in_use) *in_use = ctx->in_use;
  if (budget) *budget = ctx->budget;
  return GBLU_OK;
}

int32_t gblu_profile_enable(gblu_ctx* ctx, int32_t enable) {
  if (!ctx) return fail(ctx, GBLU_EINVAL, "gblu_profile_enable: NULL ctx");
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  DeviceGuard g(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  ctx->prof.drain();
  ctx->prof.reset();
  ctx->prof.enabled = enable != 0;
  return GBLU_OK;
}

int32_t gblu_profile_read(gblu_ctx* ctx, gblu_profile* out, int32_t reset) {
  if (!ctx || !out) return fail(ctx, GBLU_EINVAL, "gblu_profile_read: NULL argument");
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  DeviceGuard g(ctx->device);
  GBLU_CK(ctx, cudaStreamSynchronize(ctx->stream), "gblu_profile_read");
  ctx->prof.drain();
  std::memset(out, 0, sizeof(*out));
  out->launches = ctx->prof.launches;
  for (int k = 0; k < K_NKINDS && k < GBLU_PROFILE_KINDS; ++k) {
    out->count[k] = ctx->prof.count[k];
    out->ms[k] = ctx->prof.ms[k];
    out->flops[k] = ctx->prof.flops[k];
    out->bytes[k] = ctx->prof.bytes[k];
  }
  if (reset) ctx->prof.reset();
  return GBLU_OK;
}

int32_t gblu_factor_create(gblu_ctx* ctx, int64_t m, int64_t n, int32_t precision,
                           gblu_factor** out) {
  if (!ctx || !out) return fail(ctx, GBLU_EINVAL, "gblu_factor_create: NULL argument");
  *out = nullptr;
  if (m < 0 || n < 0) return fail(ctx, GBLU_EINVAL, "gblu_factor_create: negative size %lld x %lld",
                                  (long long)m, (long long)n);
  if (precision != GBLU_FP64 && precision != GBLU_FP32 && precision != GBLU_BF16 &&
      precision != GBLU_FP16)
    return fail(ctx, GBLU_EUNSUPPORTED, "gblu_factor_create: unknown precision %d", precision);
  if (m > (int64_t)INT32_MAX || n > (int64_t)INT32_MAX)
    return fail(ctx, GBLU_EUNSUPPORTED, "gblu_factor_create: dimension too large");
  if (precision != GBLU_FP64 && m != n)
    return fail(ctx, GBLU_EUNSUPPORTED, "mixed-precision factors must be square");
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  DeviceGuard g(ctx->device);
  gblu_factor* f = new (std::nothrow) gblu_factor();
  if (!f) return fail(ctx, GBLU_ENOMEM, "host allocation failed");
  f->m = m;
  f->n = n;
  f->precision = precision;
  f->ld = std::max<int64_t>(32, ((m + 31) / 32) * 32);
  const size_t bytes = factor_arena_bytes(m, n, precision, ctx->device);
  const size_t tc_bytes =
      (precision == GBLU_BF16 || precision == GBLU_FP16) ? align256(tc_work_bytes(n, n / 2 + 64, n / 2 + 64)) : 0;
  int32_t st = ctx_alloc(ctx, bytes, &f->arena);
  if (st) {
    delete f;
    return st;
  }
  f->bytes = bytes;
  char* c = reinterpret_cast<char*>(f->arena);
  if (precision == GBLU_FP64) {
    c = carve_set<double>(c, m, n, f->ld, ctx->device, kWorkCols, &f->lu64, &f->ipiv, &f->perm,
                          &f->info_dev, f->rf64, f->rs64);
  } else {
    c = carve_set<float>(c, m, n, f->ld, ctx->device, kWorkCols, &f->lu32, &f->ipiv, &f->perm,
                         &f->info_dev, f->rf32, f->rs32);
    f->lu64 = reinterpret_cast<double*>(c);
    c += align256((size_t)f->ld * n * sizeof(double));
    refine_carve(f->refine, c, m, kWorkCols);
    c += refine_bytes(m, kWorkCols);
    if (tc_bytes) {
      f->rf32.tc_mode = precision == GBLU_BF16 ? 1 : 2;
      f->rf32.tc_work = c;
      f->rf32.tc_work_bytes = tc_bytes;
      c += tc_bytes;
      // TRSM base blocks through cached inverses of L's diagonal blocks
      // (GBLU_TRSM=exact at creation keeps the substitution chain)
      const char* te = getenv("GBLU_TRSM");
      if (!(te && !strcmp(te, "exact"))) {
        f->rf32.trsm_inv = reinterpret_cast<float*>(c);
        f->rf32.trsm_inv_slots = trsm_inv_slot_count(n);
      }
      c += align256(trsm_inv_bytes(n));
    }
    // Panel pivoting of the low-precision factors: partial pivoting (the
    // reference's order) by default; GBLU_PANEL=tournament at creation
    // selects tournament pivoting for leaves taller than 512 rows (slower
    // on this GPU than the register cluster panel: two dependent getf2
    // passes per leaf against one).
    {
      const char* pe = getenv("GBLU_PANEL");
      f->rf32.tslu = pe && !strcmp(pe, "tournament");
      if (f->rf32.tslu) f->pivoting = GBLU_PIVOT_TOURNAMENT;
      f->rf32.tslu_work = c;
      c += align256(tslu_work_bytes());
    }
    // the low-precision solve of a mixed factor is refinement's correction
    // solve: fast (inverted diagonal blocks) by default
    if (m == n && n > 0) {
      f->inv_bytes = getrs_inverse_bytes(n, sizeof(float));
      f->inv_arena = c;
      f->rs32.fast = true;
      f->rs32.inv = reinterpret_cast<float*>(c);
      c += align256(f->inv_bytes);
    }
    if (m == n && n >= 4) {
      f->rbt = reinterpret_cast<float*>(c);
      c += align256((size_t)4 * (n - n % 4) * sizeof(float));
    }
  }
  cudaError_t e = cudaMemsetAsync(f->arena, 0, bytes, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) {
    ctx_free(ctx, f->arena, bytes);
    delete f;
    return cuda_fail(ctx, e, "clearing factor arena");
  }
  *out = f;
  return GBLU_OK;
}

int32_t gblu_factor_destroy(gblu_ctx* ctx, gblu_factor* f) {
  if (!f) return GBLU_OK;
  if (!ctx) return fail(ctx, GBLU_EINVAL, "gblu_factor_destroy: NULL ctx");
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  DeviceGuard g(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  if (f->getrf_exec) cudaGraphExecDestroy(f->getrf_exec);
  ctx_free(ctx, f->arena, f->bytes);
  if (f->rhs) ctx_free(ctx, f->rhs, (size_t)f->ld * f->rhs_cols * sizeof(double));
  if (f->fb_arena) ctx_free(ctx, f->fb_arena, f->fb_bytes);
  if (f->a_keep) ctx_free(ctx, f->a_keep, std::max<size_t>((size_t)f->ld * f->n * sizeof(double), 256));
  if (f->chk_arena) ctx_free(ctx, f->chk_arena, f->chk_bytes);
  if (f->inv_arena && f->inv_owned) ctx_free(ctx, f->inv_arena, f->inv_bytes);
  if (f->refine.gflags_host) cudaFreeHost(f->refine.gflags_host);
  delete f;
  return GBLU_OK;
}

int32_t gblu_factor_set_solve(gblu_ctx* ctx, gblu_factor* f, int32_t mode) {
  if (!ctx || !f) return fail(ctx, GBLU_EINVAL, "gblu_factor_set_solve: NULL argument");
  if (mode != GBLU_SOLVE_EXACT && mode != GBLU_SOLVE_FAST)
    return fail(ctx, GBLU_EINVAL, "gblu_factor_set_solve: unknown mode %d", mode);
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  DeviceGuard g(ctx->device);
  const bool fast = mode == GBLU_SOLVE_FAST;
  if (fast && !f->inv_arena && f->m == f->n) {
    const size_t bytes = getrs_inverse_bytes(f->n, f->precision == GBLU_FP64 ? 8 : 4);
    int32_t st = ctx_alloc(ctx, bytes, &f->inv_arena);
    if (st) return st;
    f->inv_bytes = bytes;
    f->inv_owned = true;
    f->inv_valid = false;
  }
  if (f->precision == GBLU_FP64) {
    f->rs64.fast = fast && f->inv_arena;
    f->rs64.inv = reinterpret_cast<double*>(f->inv_arena);
  } else {
    f->rs32.fast = fast && f->inv_arena;
    f->rs32.inv = reinterpret_cast<float*>(f->inv_arena);
  }
  return GBLU_OK;
}

int32_t gblu_factor_set_pivoting(gblu_ctx* ctx, gblu_factor* f, int32_t mode) {
  if (!ctx || !f) return fail(ctx, GBLU_EINVAL, "gblu_factor_set_pivoting: NULL argument");
  if (mode != GBLU_PIVOT_PARTIAL && mode != GBLU_PIVOT_TOURNAMENT && mode != GBLU_PIVOT_RBT)
    return fail(ctx, GBLU_EINVAL, "gblu_factor_set_pivoting: unknown mode %d", mode);
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  DeviceGuard g(ctx->device);
  if (f->precision == GBLU_FP64) {
    if (mode == GBLU_PIVOT_PARTIAL) return GBLU_OK;
    return fail(ctx, GBLU_EUNSUPPORTED, "gblu_factor_set_pivoting: FP64 factors pivot partially (the reference's LU)");
  }
  if (mode == GBLU_PIVOT_RBT && !f->rbt)
    return fail(ctx, GBLU_EUNSUPPORTED,
                "gblu_factor_set_pivoting: the butterfly transform needs a square factor of order 4 or more "
                "(%lld x %lld)", (long long)f->m, (long long)f->n);
  if (mode == GBLU_PIVOT_RBT && !f->rbt_ready) {
    std::vector<float> h((size_t)4 * (f->n - f->n % 4));
    rbt_fill_host(f->n, h.data());
    CK(ctx, cudaMemcpyAsync(f->rbt, h.data(), h.size() * sizeof(float), cudaMemcpyHostToDevice, ctx->stream),
       "uploading the butterfly diagonals");
    CK(ctx, cudaStreamSynchronize(ctx->stream), "uploading the butterfly diagonals");
    f->rbt_ready = true;
  }
  if (mode != f->pivoting) {
    f->pivoting = mode;
    f->rf32.tslu = mode == GBLU_PIVOT_TOURNAMENT;
    f->rf32.nopivot = mode == GBLU_PIVOT_RBT;
    // the captured launch sequence and the factors belong to the old mode
    if (f->getrf_exec) cudaGraphExecDestroy(f->getrf_exec);
    f->getrf_exec = nullptr;
    f->getrf_runs = 0;
    f->getrf_graph_failed = false;
    f->factored = false;
  }
  return GBLU_OK;
}

int32_t gblu_factor_keep_matrix(gblu_ctx* ctx, gblu_factor* f, int32_t keep) {
  if (!ctx || !f) return fail(ctx, GBLU_EINVAL, "gblu_factor_keep_matrix: NULL argument");
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  DeviceGuard g(ctx->device);
  if (f->precision != GBLU_FP64) return GBLU_OK;  // mixed factors keep A anyway
  const size_t bytes = (size_t)f->ld * f->n * sizeof(double);
  if (keep && !f->a_keep) {
    void* p = nullptr;
    int32_t st = ctx_alloc(ctx, std::max<size_t>(bytes, 256), &p);
    if (st) return st;
    f->a_keep = reinterpret_cast<double*>(p);
    f->a_keep_valid = false;
  } else if (!keep && f->a_keep) {
    cudaStreamSynchronize(ctx->stream);
    ctx_free(ctx, f->a_keep, std::max<size_t>(bytes, 256));
    f->a_keep = nullptr;
    f->a_keep_valid = false;
  }
  return GBLU_OK;
}

}  // extern "C"

namespace gblu {

namespace {

// Uploads from pageable host memory of kStageAlways bytes or more, and of
// kStageMin or more while another such upload is in progress in the
// process, go through pinned staging.  A cudaMemcpyAsync from pageable
// memory has the driver read the caller's pages itself; on GB300 one such
// copy at a time ran at ~170 GB/s in every process measured, but with
// several worker threads copying at once the speed depended on the process:
// fine in the first serving process of a box, 3-8x slower factorization
// service in every later one (a serving stream's p99 at 400 Hz: 13 ms, then
// 70-200 ms).  Staged, the CPU copies column blocks into two pinned chunks
// that the copy engine drains alternately (the host copy of one chunk
// overlaps the transfer of the other): about 14 GB/s per thread and a p99 of
// 24 ms in every process.  A lone mid-size upload keeps the direct copy,
// which is faster than the host copy.  GBLU_HOST_STAGING=0 copies directly.
constexpr size_t kStageMin = size_t(4) << 20;
constexpr size_t kStageAlways = size_t(32) << 20;
constexpr size_t kStageChunk = size_t(16) << 20;
std::atomic<int> g_pageable_uploads{0};  // pageable uploads of kStageMin or more in progress

bool host_staging_on() {
  static const bool on = [] {
    const char* e = getenv("GBLU_HOST_STAGING");
    return !(e && e[0] == '0');
  }();
  return on;
}

bool is_pageable(const void* p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return true;
  }
  return a.type == cudaMemoryTypeUnregistered;
}

// columns [c0, c1) of src (ld_src) packed into out (rows per column)
void pack_columns(double* out, const double* src, int64_t ld_src, int64_t rows, int64_t c0, int64_t c1) {
  for (int64_t c = c0; c < c1; ++c)
    std::memcpy(out + (c - c0) * rows, src + c * ld_src, (size_t)rows * sizeof(double));
}

int32_t upload_staged(gblu_ctx* ctx, double* dst, int64_t ld_dst, const double* src, int64_t ld_src,
                      int64_t rows, int64_t cols) {
  const size_t col_bytes = (size_t)rows * sizeof(double);
  const size_t chunk = std::max(kStageChunk, col_bytes);
  if (!ctx->stage || ctx->stage_chunk < chunk) {
    if (ctx->stage) {
      CK(ctx, cudaStreamSynchronize(ctx->stream), "staging");
      cudaFreeHost(ctx->stage);
      ctx->stage = nullptr;
    }
    void* p = nullptr;
    CK(ctx, cudaMallocHost(&p, 2 * chunk), "allocating pinned staging");
    ctx->stage = static_cast<char*>(p);
    ctx->stage_chunk = chunk;
  }
  for (cudaEvent_t& e : ctx->stage_ev)
    if (!e) CK(ctx, cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "staging event");
  const int64_t per = (int64_t)(ctx->stage_chunk / col_bytes);  // columns per chunk
  int i = 0;
  for (int64_t c = 0; c < cols; c += per, i ^= 1) {
    const int64_t k = std::min(per, cols - c);
    CK(ctx, cudaEventSynchronize(ctx->stage_ev[i]), "staging");  // the chunk's last copy is done
    double* buf = reinterpret_cast<double*>(ctx->stage + (size_t)i * ctx->stage_chunk);
    pack_columns(buf, src + c * ld_src, ld_src, rows, 0, k);
    if (ld_dst == rows)
      CK(ctx, cudaMemcpyAsync(dst + c * ld_dst, buf, col_bytes * k, cudaMemcpyHostToDevice, ctx->stream),
         "copying matrix to device");
    else
      CK(ctx, cudaMemcpy2DAsync(dst + c * ld_dst, ld_dst * sizeof(double), buf, col_bytes, col_bytes, k,
                                cudaMemcpyHostToDevice, ctx->stream),
         "copying matrix to device");
    CK(ctx, cudaEventRecord(ctx->stage_ev[i], ctx->stream), "staging");
  }
  return GBLU_OK;
}

}  // namespace

// One cudaMemcpyAsync / cudaMemcpy2DAsync of the matrix.
int32_t upload_direct(gblu_ctx* ctx, double* dst, int64_t ld_dst, const double* src, int64_t ld_src,
                      int64_t rows, int64_t cols, cudaMemcpyKind kind) {
  if (ld_dst == rows && ld_src == rows)  // both contiguous: one linear copy
    CK(ctx, cudaMemcpyAsync(dst, src, (size_t)rows * cols * sizeof(double), kind, ctx->stream),
       "copying matrix to device");
  else
    CK(ctx, cudaMemcpy2DAsync(dst, ld_dst * sizeof(double), src, ld_src * sizeof(double),
                              rows * sizeof(double), cols, kind, ctx->stream),
       "copying matrix to device");
  return GBLU_OK;
}

// Copy a host or device FP64 matrix (rows x cols, ld_src) into dst (ld_dst).
int32_t upload_matrix(gblu_ctx* ctx, double* dst, int64_t ld_dst, const double* src, int64_t ld_src,
                      int64_t rows, int64_t cols, int32_t loc) {
  if (rows == 0 || cols == 0) return GBLU_OK;
  const size_t bytes = (size_t)rows * cols * sizeof(double);
  if (loc == GBLU_HOST && bytes >= kStageMin && host_staging_on() && is_pageable(src)) {
    const int others = g_pageable_uploads.fetch_add(1);
    const int32_t st = bytes >= kStageAlways || others > 0
                           ? upload_staged(ctx, dst, ld_dst, src, ld_src, rows, cols)
                           : upload_direct(ctx, dst, ld_dst, src, ld_src, rows, cols, cudaMemcpyHostToDevice);
    g_pageable_uploads.fetch_sub(1);
    return st;
  }
  return upload_direct(ctx, dst, ld_dst, src, ld_src, rows, cols,
                       loc == GBLU_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice);
}

// Runs the factor's getrf launch sequence: directly on its first two runs
// (the first also fills the host-side caches the launches consult; a factor
// refactored only once or twice does not pay for a capture) and while
// profiling (per-launch events); from the third run on as one replay of a
// CUDA graph captured from that sequence.  Any capture problem falls back to
// direct launches for good.  GBLU_GRAPHS=0 disables the replay.
template <typename Launch>
cudaError_t run_getrf(gblu_ctx* ctx, gblu_factor* f, Launch&& launch) {
  static const bool off = [] {
    const char* e = getenv("GBLU_GRAPHS");
    return e && e[0] == '0';
  }();
  const bool direct = off || f->getrf_graph_failed || ctx->prof.enabled || f->getrf_runs++ < 2;
  if (direct) return launch();
  if (!f->getrf_exec) {
    cudaGraph_t g = nullptr;
    // the launches counted while capturing are kept with the graph and added
    // at each replay (a replay does not pass through LaunchScope)
    const LaunchCounts before = ctx->prof.counts();
    cudaError_t e = cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
      const cudaError_t le = launch();
      e = cudaStreamEndCapture(ctx->stream, &g);
      if (le != cudaSuccess) e = le;
    }
    f->getrf_graph_counts = Profiler::diff(before, ctx->prof.counts());
    ctx->prof.sub(f->getrf_graph_counts);  // counted again below, per launch
    if (e == cudaSuccess && g) e = cudaGraphInstantiate(&f->getrf_exec, g, 0);
    if (g) cudaGraphDestroy(g);
    if (e != cudaSuccess || !f->getrf_exec) {
      cudaGetLastError();  // clear the capture failure, then launch directly
      f->getrf_exec = nullptr;
      f->getrf_graph_failed = true;
      return launch();
    }
  }
  ctx->prof.add(f->getrf_graph_counts);
  return cudaGraphLaunch(f->getrf_exec, ctx->stream);
}

int32_t ensure_inverse(gblu_ctx* ctx, gblu_factor* f) {
  if (f->inv_valid) return GBLU_OK;
  if (f->precision == GBLU_FP64) {
    if (!f->rs64.fast) return GBLU_OK;
    CK(ctx, getrs_invert_launch<double>(f->rs64, ctx->stream), "inverting diagonal blocks");
  } else {
    if (!f->rs32.fast) return GBLU_OK;
    CK(ctx, getrs_invert_launch<float>(f->rs32, ctx->stream), "inverting diagonal blocks");
  }
  f->inv_valid = true;
  return GBLU_OK;
}

int32_t factor_getrf(gblu_ctx* ctx, gblu_factor* f, const double* A, int64_t lda, int32_t a_loc,
                     int64_t* info) {
  f->factored = false;
  f->fb_valid = false;
  f->inv_valid = false;
  int32_t st;
  if (f->precision == GBLU_FP64) {
    st = upload_matrix(ctx, f->lu64, f->ld, A, lda, f->m, f->n, a_loc);
    if (st) return st;
    f->a_keep_valid = false;
    if (f->a_keep) {  // the copy residual checks read (gblu_factor_keep_matrix)
      CK(ctx, cudaMemcpyAsync(f->a_keep, f->lu64, (size_t)f->ld * f->n * sizeof(double),
                              cudaMemcpyDeviceToDevice, ctx->stream),
         "keeping A");
      f->a_keep_valid = true;
    }
    CK(ctx, run_getrf(ctx, f, [&] { return getrf_launch<double>(f->rf64, ctx->stream); }),
       "launching getrf");
  } else {
    st = upload_matrix(ctx, f->lu64, f->ld, A, lda, f->m, f->n, a_loc);
    if (st) return st;
    const bool rbt = f->pivoting == GBLU_PIVOT_RBT;
    CK(ctx, refine_prepare(f->refine, f->n, f->lu64, f->ld, f->lu32, f->ld, ctx->stream, !rbt),
       "preparing mixed-precision factorization");
    if (rbt)  // the low-precision factors are those of U^T A V / 4
      CK(ctx, rbt_matrix_launch(f->n, f->lu64, f->ld, f->lu32, f->ld, f->rbt, ctx->stream),
         "butterfly transform");
    CK(ctx, run_getrf(ctx, f, [&] { return getrf_launch<float>(f->rf32, ctx->stream); }),
       "launching getrf");
    CK(ctx, refine_growth_launch(f->refine, f->n, f->lu32, f->ld, ctx->stream), "pivot growth");
  }
  int64_t hinfo = 0;
  unsigned long long umax_bits = 0;
  CK(ctx, cudaMemcpyAsync(&hinfo, f->info_dev, sizeof(int64_t), cudaMemcpyDeviceToHost, ctx->stream),
     "reading info");
  if (f->precision != GBLU_FP64)
    CK(ctx, cudaMemcpyAsync(&umax_bits, f->refine.growth_bits + 1, sizeof(umax_bits),
                            cudaMemcpyDeviceToHost, ctx->stream),
       "reading pivot growth");
  CK(ctx, cudaStreamSynchronize(ctx->stream), "getrf");
  st = check_device_errors(ctx, {f->precision == GBLU_FP64 ? f->rf64.scratch : f->rf32.scratch});
  if (st) return st;
  f->info = hinfo;
  f->use_fb = false;
  f->growth = f->precision == GBLU_FP64 ? 0.0 : refine_growth(f->refine, umax_bits);
  if (f->precision != GBLU_FP64 && hinfo != 0) {
    // An exactly zero pivot in the low-precision factors: decide singularity
    // with the FP64 factorization, which then serves every solve.
    int64_t info64 = 0;
    st = factor_fp64_fallback(ctx, f, &info64);
    if (st) return st;
    f->info = info64;
    f->use_fb = f->fb_valid;
  }
  f->factored = true;
  if (info) *info = f->info;
  return GBLU_OK;
}

int32_t factor_fp64_fallback(gblu_ctx* ctx, gblu_factor* f, int64_t* info_out) {
  if (!f->fb_arena) {
    size_t bytes = set_bytes<double>(f->m, f->n, f->ld, ctx->device, kWorkColsFb);
    int32_t st = ctx_alloc(ctx, bytes, &f->fb_arena);
    if (st) return st;
    f->fb_bytes = bytes;
    CK(ctx, cudaMemsetAsync(f->fb_arena, 0, bytes, ctx->stream), "clearing fallback arena");
    carve_set<double>(reinterpret_cast<char*>(f->fb_arena), f->m, f->n, f->ld, ctx->device,
                      kWorkColsFb, &f->fb_lu, &f->fb_ipiv, &f->fb_perm, &f->fb_info, f->fb_rf,
                      f->fb_rs);
  }
  CK(ctx, cudaMemcpyAsync(f->fb_lu, f->lu64, (size_t)f->ld * f->n * sizeof(double),
                          cudaMemcpyDeviceToDevice, ctx->stream),
     "copying A for the FP64 fallback");
  CK(ctx, getrf_launch<double>(f->fb_rf, ctx->stream), "launching fallback getrf");
  int64_t hinfo = 0;
  CK(ctx, cudaMemcpyAsync(&hinfo, f->fb_info, sizeof(int64_t), cudaMemcpyDeviceToHost, ctx->stream),
     "reading fallback info");
  CK(ctx, cudaStreamSynchronize(ctx->stream), "fallback getrf");
  int32_t st = check_device_errors(ctx, {f->fb_rf.scratch});
  if (st) return st;
  f->fb_valid = (hinfo == 0);
  if (info_out) *info_out = hinfo;
  return GBLU_OK;
}

int32_t factor_getrs_plain(gblu_ctx* ctx, gblu_factor* f, char trans, int64_t nrhs, double* dB,
                           int64_t ldb) {
  int32_t st = ensure_inverse(ctx, f);
  if (st) return st;
  CK(ctx, getrs_launch<double>(f->rs64, trans, nrhs, dB, ldb, nullptr, ctx->stream),
     "launching getrs");
  return GBLU_OK;
}

}  // namespace gblu

extern "C" {

int32_t gblu_getrf(gblu_ctx* ctx, gblu_factor* f, const double* A, int64_t lda, int32_t a_loc,
                   int64_t* info) {
  if (!ctx || !f) return fail(ctx, GBLU_EINVAL, "gblu_getrf: NULL argument");
  if (!A && f->m * f->n > 0) return fail(ctx, GBLU_EINVAL, "gblu_getrf: A is NULL");
  if (lda < std::max<int64_t>(1, f->m)) return fail(ctx, GBLU_EINVAL, "gblu_getrf: lda %lld < m %lld",
                                                   (long long)lda, (long long)f->m);
  if (a_loc != GBLU_HOST && a_loc != GBLU_DEVICE) return fail(ctx, GBLU_EINVAL, "gblu_getrf: bad a_loc");
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  DeviceGuard g(ctx->device);
  ActiveProfiler ap(&ctx->prof);
  return factor_getrf(ctx, f, A, lda, a_loc, info);
}

int32_t gblu_getrs(gblu_ctx* ctx, gblu_factor* f, char trans, int64_t nrhs, double* B, int64_t ldb,
                   int32_t b_loc) {
  if (!ctx || !f) return fail(ctx, GBLU_EINVAL, "gblu_getrs: NULL argument");
  if (!(trans == 'N' || trans == 'n' || trans == 'T' || trans == 't' || trans == 'C' || trans == 'c'))
    return fail(ctx, GBLU_EINVAL, "gblu_getrs: trans must be 'N' or 'T'");
  if (f->m != f->n) return fail(ctx, GBLU_EINVAL, "gblu_getrs: factor is not square");
  if (nrhs < 0) return fail(ctx, GBLU_EINVAL, "gblu_getrs: nrhs < 0");
  if (ldb < std::max<int64_t>(1, f->n)) return fail(ctx, GBLU_EINVAL, "gblu_getrs: ldb < n");
  if (b_loc != GBLU_HOST && b_loc != GBLU_DEVICE) return fail(ctx, GBLU_EINVAL, "gblu_getrs: bad b_loc");
  if (!f->factored) return fail(ctx, GBLU_ENOTFACTORED, "gblu_getrs: no factorization");
  if (f->info != 0)
    return fail(ctx, GBLU_EINVAL, "gblu_getrs: factorization is singular (info = %lld)",
                (long long)f->info);
  if (nrhs == 0 || f->n == 0) return GBLU_OK;
  if (!B) return fail(ctx, GBLU_EINVAL, "gblu_getrs: B is NULL");
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  DeviceGuard g(ctx->device);
  ActiveProfiler ap(&ctx->prof);
  if (f->precision != GBLU_FP64) {
    gblu_refine_opts o = refine_default_opts();
    return refine_solve(ctx, f, trans, nrhs, B, ldb, b_loc, &o, nullptr);
  }
  double* dB = B;
  int64_t lddb = ldb;
  int32_t st;
  if (b_loc == GBLU_HOST) {
    st = ensure_rhs(ctx, f, std::max<int64_t>(nrhs, 1));
    if (st) return st;
    dB = f->rhs;
    lddb = f->ld;
    st = upload_matrix(ctx, dB, lddb, B, ldb, f->n, nrhs, GBLU_HOST);
    if (st) return st;
  }
  st = factor_getrs_plain(ctx, f, trans, nrhs, dB, lddb);
  if (st) return st;
  if (b_loc == GBLU_HOST)
    CK(ctx, cudaMemcpy2DAsync(B, ldb * sizeof(double), dB, lddb * sizeof(double),
                              f->n * sizeof(double), nrhs, cudaMemcpyDeviceToHost, ctx->stream),
       "copying solution to host");
  CK(ctx, cudaStreamSynchronize(ctx->stream), "getrs");
  return check_device_errors(ctx, {f->rs64.scratch});
}

int32_t gblu_solve_refined(gblu_ctx* ctx, gblu_factor* f, char trans, int64_t nrhs, double* B,
                           int64_t ldb, int32_t b_loc, const gblu_refine_opts* opts,
                           gblu_refine_stats* stats) {
  if (!ctx || !f) return fail(ctx, GBLU_EINVAL, "gblu_solve_refined: NULL argument");
  if (opts && (opts->mode != GBLU_REFINE_IR && opts->mode != GBLU_REFINE_GMRES))
    return fail(ctx, GBLU_EINVAL, "gblu_solve_refined: unknown mode %d", opts->mode);
  if (opts && (opts->max_iter < 0 || opts->gmres_restart < 1))
    return fail(ctx, GBLU_EINVAL, "gblu_solve_refined: bad iteration limits");
  if (f->precision == GBLU_FP64) {
    int32_t st = gblu_getrs(ctx, f, trans, nrhs, B, ldb, b_loc);
    if (st) return st;
    if (stats) {
      *stats = gblu_refine_stats{};
      stats->converged = 1;
      stats->backward_error = -1.0;  // A is not kept for FP64 factors
    }
    return GBLU_OK;
  }
  if (!(trans == 'N' || trans == 'n' || trans == 'T' || trans == 't' || trans == 'C' || trans == 'c'))
    return fail(ctx, GBLU_EINVAL, "gblu_solve_refined: trans must be 'N' or 'T'");
  if (nrhs < 0) return fail(ctx, GBLU_EINVAL, "gblu_solve_refined: nrhs < 0");
  if (ldb < std::max<int64_t>(1, f->n)) return fail(ctx, GBLU_EINVAL, "gblu_solve_refined: ldb < n");
  if (b_loc != GBLU_HOST && b_loc != GBLU_DEVICE)
    return fail(ctx, GBLU_EINVAL, "gblu_solve_refined: bad b_loc");
  if (!f->factored) return fail(ctx, GBLU_ENOTFACTORED, "gblu_solve_refined: no factorization");
  if (f->info != 0)
    return fail(ctx, GBLU_EINVAL, "gblu_solve_refined: factorization is singular (info = %lld)",
                (long long)f->info);
  if (nrhs == 0 || f->n == 0) {
    if (stats) { *stats = gblu_refine_stats{}; stats->converged = 1; }
    return GBLU_OK;
  }
  if (!B) return fail(ctx, GBLU_EINVAL, "gblu_solve_refined: B is NULL");
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  DeviceGuard g(ctx->device);
  ActiveProfiler ap(&ctx->prof);
  return refine_solve(ctx, f, trans, nrhs, B, ldb, b_loc, opts, stats);
}

int32_t gblu_gemm_update(gblu_ctx* ctx, int32_t precision, int64_t m, int64_t n, int64_t k,
                         const float* A, int64_t lda, const float* B, int64_t ldb, float* C,
                         int64_t ldc, int32_t loc) {
  if (!ctx) return fail(ctx, GBLU_EINVAL, "gblu_gemm_update: NULL ctx");
  if (m < 0 || n < 0 || k < 0) return fail(ctx, GBLU_EINVAL, "gblu_gemm_update: negative size");
  if (lda < std::max<int64_t>(1, m) || ldb < std::max<int64_t>(1, k) || ldc < std::max<int64_t>(1, m))
    return fail(ctx, GBLU_EINVAL, "gblu_gemm_update: leading dimension too small");
  if (precision != GBLU_FP32 && precision != GBLU_BF16 && precision != GBLU_FP16)
    return fail(ctx, GBLU_EUNSUPPORTED, "gblu_gemm_update: precision must be FP32, BF16 or FP16");
  if (loc != GBLU_HOST && loc != GBLU_DEVICE) return fail(ctx, GBLU_EINVAL, "gblu_gemm_update: bad loc");
  if (m == 0 || n == 0 || k == 0) return GBLU_OK;
  if (!A || !B || !C) return fail(ctx, GBLU_EINVAL, "gblu_gemm_update: NULL pointer");
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  DeviceGuard g(ctx->device);
  ActiveProfiler ap(&ctx->prof);
  // device staging for host operands + the conversion buffers + an error word
  const size_t a_b = align256((size_t)m * k * 4), b_b = align256((size_t)k * n * 4),
               c_b = align256((size_t)m * n * 4);
  const size_t w_b = precision == GBLU_FP32 ? 0 : align256(tc_work_bytes(m, n, k));
  const size_t total = (loc == GBLU_HOST ? a_b + b_b + c_b : 0) + w_b + 256;
  void* arena = nullptr;
  int32_t st = ctx_alloc(ctx, total, &arena);
  if (st) return st;
  char* c = reinterpret_cast<char*>(arena);
  int* derr = reinterpret_cast<int*>(c);
  c += 256;
  const float *dA = A, *dB = B;
  float* dC = C;
  int64_t la = lda, lb = ldb, lc = ldc;
  cudaError_t e = cudaMemsetAsync(derr, 0, 256, ctx->stream);
  if (loc == GBLU_HOST) {
    float* pa = reinterpret_cast<float*>(c); c += a_b;
    float* pb = reinterpret_cast<float*>(c); c += b_b;
    float* pc = reinterpret_cast<float*>(c); c += c_b;
    if (e == cudaSuccess) e = cudaMemcpy2DAsync(pa, m * 4, A, lda * 4, m * 4, k, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpy2DAsync(pb, k * 4, B, ldb * 4, k * 4, n, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpy2DAsync(pc, m * 4, C, ldc * 4, m * 4, n, cudaMemcpyHostToDevice, ctx->stream);
    dA = pa; dB = pb; dC = pc; la = m; lb = k; lc = m;
  }
  if (e == cudaSuccess) {
    if (precision == GBLU_FP32) e = simt_gemm_sub_f32(m, n, k, dA, la, dB, lb, dC, lc, ctx->stream);
    else e = tc_gemm_sub(precision == GBLU_BF16 ? 1 : 2, m, n, k, dA, la, dB, lb, dC, lc, c, derr, ctx->stream);
  }
  if (e == cudaSuccess && loc == GBLU_HOST)
    e = cudaMemcpy2DAsync(C, ldc * 4, dC, lc * 4, m * 4, n, cudaMemcpyDeviceToHost, ctx->stream);
  int herr = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&herr, derr, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  ctx_free(ctx, arena, total);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "gblu_gemm_update");
  if (herr) return fail(ctx, GBLU_ETIMEOUT, "gblu_gemm_update: device wait timed out (code %d)", herr);
  return GBLU_OK;
}

int32_t gblu_get_ipiv(gblu_ctx* ctx, gblu_factor* f, int64_t* ipiv_host) {
  if (!ctx || !f || !ipiv_host) return fail(ctx, GBLU_EINVAL, "gblu_get_ipiv: NULL argument");
  if (!f->factored) return fail(ctx, GBLU_ENOTFACTORED, "gblu_get_ipiv: no factorization");
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  DeviceGuard g(ctx->device);
  int64_t k = std::min(f->m, f->n);
  if (k == 0) return GBLU_OK;
  CK(ctx, cudaMemcpyAsync(ipiv_host, f->ipiv, k * sizeof(int64_t), cudaMemcpyDeviceToHost, ctx->stream),
     "copying ipiv");
  CK(ctx, cudaStreamSynchronize(ctx->stream), "copying ipiv");
  return GBLU_OK;
}

int32_t gblu_get_factors(gblu_ctx* ctx, gblu_factor* f, double* host, int64_t ld) {
  if (!ctx || !f || (!host && f->m * f->n > 0))
    return fail(ctx, GBLU_EINVAL, "gblu_get_factors: NULL argument");
  if (ld < std::max<int64_t>(1, f->m)) return fail(ctx, GBLU_EINVAL, "gblu_get_factors: ld < m");
  if (!f->factored) return fail(ctx, GBLU_ENOTFACTORED, "gblu_get_factors: no factorization");
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  DeviceGuard g(ctx->device);
  if (f->m * f->n == 0) return GBLU_OK;
  if (f->precision == GBLU_FP64) {
    CK(ctx, cudaMemcpy2DAsync(host, ld * sizeof(double), f->lu64, f->ld * sizeof(double),
                              f->m * sizeof(double), f->n, cudaMemcpyDeviceToHost, ctx->stream),
       "copying factors");
    CK(ctx, cudaStreamSynchronize(ctx->stream), "copying factors");
  } else {
    std::vector<float> tmp((size_t)f->ld * f->n);
    CK(ctx, cudaMemcpyAsync(tmp.data(), f->lu32, tmp.size() * sizeof(float), cudaMemcpyDeviceToHost,
                            ctx->stream),
       "copying factors");
    CK(ctx, cudaStreamSynchronize(ctx->stream), "copying factors");
    for (int64_t j = 0; j < f->n; ++j)
      for (int64_t i = 0; i < f->m; ++i) host[i + j * ld] = (double)tmp[i + j * f->ld];
  }
  return GBLU_OK;
}

int32_t gblu_get_info(gblu_ctx* ctx, gblu_factor* f, int64_t* info) {
  if (!ctx || !f || !info) return fail(ctx, GBLU_EINVAL, "gblu_get_info: NULL argument");
  if (!f->factored) return fail(ctx, GBLU_ENOTFACTORED, "gblu_get_info: no factorization");
  *info = f->info;
  return GBLU_OK;
}

int32_t gblu_get_growth(gblu_ctx* ctx, gblu_factor* f, double* growth) {
  if (!ctx || !f || !growth) return fail(ctx, GBLU_EINVAL, "gblu_get_growth: NULL argument");
  if (!f->factored) return fail(ctx, GBLU_ENOTFACTORED, "gblu_get_growth: no factorization");
  *growth = f->growth;
  return GBLU_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// LAPACK-shaped host entries on a process-wide default context.

namespace {

std::mutex g_lapack_mu;
gblu_ctx* g_lapack_ctx = nullptr;
gblu_factor* g_lapack_f64 = nullptr;

gblu_ctx* lapack_ctx(int32_t* st) {
  if (!g_lapack_ctx) {
    int dev = 0;
    cudaGetDevice(&dev);
    *st = gblu_create(&g_lapack_ctx, dev, 0);
    if (*st) g_lapack_ctx = nullptr;
  }
  return g_lapack_ctx;
}

gblu_factor* lapack_factor(gblu_ctx* ctx, gblu_factor** slot, int64_t m, int64_t n, int32_t* st) {
  if (*slot && ((*slot)->m != m || (*slot)->n != n)) {
    gblu_factor_destroy(ctx, *slot);
    *slot = nullptr;
  }
  if (!*slot) *st = gblu_factor_create(ctx, m, n, GBLU_FP64, slot);
  return *slot;
}

int64_t lapack_err(int32_t st, gblu_ctx* ctx) {
  if (ctx) fail(nullptr, st, "%s", ctx->last_error.c_str());
  return -1000 - (int64_t)st;
}

}  // namespace

namespace gblu {
int32_t factor_getrf_f32_host(gblu_ctx* ctx, int64_t m, int64_t n, float* A, int64_t lda,
                              int64_t* ipiv, int64_t* info);
int32_t factor_getrs_f32_host(gblu_ctx* ctx, char trans, int64_t n, int64_t nrhs, const float* A,
                              int64_t lda, const int64_t* ipiv, float* B, int64_t ldb);
int32_t factor_getrs_f64_host(gblu_ctx* ctx, gblu_factor* f, char trans, int64_t nrhs,
                              const double* A, int64_t lda, const int64_t* ipiv, double* B,
                              int64_t ldb);
}  // namespace gblu

extern "C" {

void gblu_dgetrf_(const int64_t* m, const int64_t* n, double* A, const int64_t* lda, int64_t* ipiv,
                  int64_t* info) {
  if (!m || !n || !lda || !info) return;
  if (*m < 0) { *info = -1; return; }
  if (*n < 0) { *info = -2; return; }
  if (*lda < std::max<int64_t>(1, *m)) { *info = -4; return; }
  *info = 0;
  if (*m == 0 || *n == 0) return;
  std::lock_guard<std::mutex> g(g_lapack_mu);
  int32_t st = GBLU_OK;
  gblu_ctx* ctx = lapack_ctx(&st);
  if (!ctx) { *info = lapack_err(st, nullptr); return; }
  gblu_factor* f = lapack_factor(ctx, &g_lapack_f64, *m, *n, &st);
  if (!f) { *info = lapack_err(st, ctx); return; }
  int64_t inf = 0;
  st = gblu_getrf(ctx, f, A, *lda, GBLU_HOST, &inf);
  if (st) { *info = lapack_err(st, ctx); return; }
  st = gblu_get_factors(ctx, f, A, *lda);
  if (!st) st = gblu_get_ipiv(ctx, f, ipiv);
  if (st) { *info = lapack_err(st, ctx); return; }
  *info = inf;
}

void gblu_dgetrs_(const char* trans, const int64_t* n, const int64_t* nrhs, const double* A,
                  const int64_t* lda, const int64_t* ipiv, double* B, const int64_t* ldb,
                  int64_t* info, long trans_len) {
  (void)trans_len;
  if (!trans || !n || !nrhs || !lda || !ldb || !info) return;
  char t = *trans;
  if (!(t == 'N' || t == 'n' || t == 'T' || t == 't' || t == 'C' || t == 'c')) { *info = -1; return; }
  if (*n < 0) { *info = -2; return; }
  if (*nrhs < 0) { *info = -3; return; }
  if (*lda < std::max<int64_t>(1, *n)) { *info = -5; return; }
  if (*ldb < std::max<int64_t>(1, *n)) { *info = -8; return; }
  *info = 0;
  if (*n == 0 || *nrhs == 0) return;
  std::lock_guard<std::mutex> g(g_lapack_mu);
  int32_t st = GBLU_OK;
  gblu_ctx* ctx = lapack_ctx(&st);
  if (!ctx) { *info = lapack_err(st, nullptr); return; }
  gblu_factor* f = lapack_factor(ctx, &g_lapack_f64, *n, *n, &st);
  if (!f) { *info = lapack_err(st, ctx); return; }
  st = factor_getrs_f64_host(ctx, f, t, *nrhs, A, *lda, ipiv, B, *ldb);
  if (st) *info = lapack_err(st, ctx);
}

void gblu_sgetrf_(const int64_t* m, const int64_t* n, float* A, const int64_t* lda, int64_t* ipiv,
                  int64_t* info) {
  if (!m || !n || !lda || !info) return;
  if (*m < 0) { *info = -1; return; }
  if (*n < 0) { *info = -2; return; }
  if (*lda < std::max<int64_t>(1, *m)) { *info = -4; return; }
  *info = 0;
  if (*m == 0 || *n == 0) return;
  std::lock_guard<std::mutex> g(g_lapack_mu);
  int32_t st = GBLU_OK;
  gblu_ctx* ctx = lapack_ctx(&st);
  if (!ctx) { *info = lapack_err(st, nullptr); return; }
  int64_t inf = 0;
  st = factor_getrf_f32_host(ctx, *m, *n, A, *lda, ipiv, &inf);
  *info = st ? lapack_err(st, ctx) : inf;
}

void gblu_sgetrs_(const char* trans, const int64_t* n, const int64_t* nrhs, const float* A,
                  const int64_t* lda, const int64_t* ipiv, float* B, const int64_t* ldb,
                  int64_t* info, long trans_len) {
  (void)trans_len;
  if (!trans || !n || !nrhs || !lda || !ldb || !info) return;
  char t = *trans;
  if (!(t == 'N' || t == 'n' || t == 'T' || t == 't' || t == 'C' || t == 'c')) { *info = -1; return; }
  if (*n < 0) { *info = -2; return; }
  if (*nrhs < 0) { *info = -3; return; }
  if (*lda < std::max<int64_t>(1, *n)) { *info = -5; return; }
  if (*ldb < std::max<int64_t>(1, *n)) { *info = -8; return; }
  *info = 0;
  if (*n == 0 || *nrhs == 0) return;
  std::lock_guard<std::mutex> g(g_lapack_mu);
  int32_t st = GBLU_OK;
  gblu_ctx* ctx = lapack_ctx(&st);
  if (!ctx) { *info = lapack_err(st, nullptr); return; }
  st = factor_getrs_f32_host(ctx, t, *n, *nrhs, A, *lda, ipiv, B, *ldb);
  if (st) *info = lapack_err(st, ctx);
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Host-factor paths of the LAPACK-shaped entries.

namespace gblu {

namespace {
__global__ void upload_ipiv_check_kernel(const int64_t* ipiv, int64_t n, DevScratch* scr) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
       k += (int64_t)gridDim.x * blockDim.x) {
    int64_t t = ipiv[k] - 1;
    if (t < k || t >= n) atomicCAS(&scr->error, 0, (int)DEV_BAD_PIVOT_INDEX);
  }
}
}  // namespace

int32_t factor_getrs_f64_host(gblu_ctx* ctx, gblu_factor* f, char trans, int64_t nrhs,
                              const double* A, int64_t lda, const int64_t* ipiv, double* B,
                              int64_t ldb) {
  DeviceGuard g(ctx->device);
  const int64_t n = f->n;
  int32_t st = upload_matrix(ctx, f->lu64, f->ld, A, lda, n, n, GBLU_HOST);
  if (st) return st;
  CK(ctx, cudaMemcpyAsync(f->ipiv, ipiv, n * sizeof(int64_t), cudaMemcpyHostToDevice, ctx->stream),
     "copying ipiv");
  ActiveProfiler ap(&ctx->prof);
  upload_ipiv_check_kernel<<<std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, 1024)), 256, 0,
                             ctx->stream>>>(f->ipiv, n, f->rf64.scratch);
  CK(ctx, cudaGetLastError(), "checking ipiv");
  st = check_device_errors(ctx, {f->rf64.scratch});
  if (st) return st;
  CK(ctx, perm_build_launch(f->ipiv, n, n, f->perm, f->rf64.scratch, ctx->stream), "building perm");
  f->factored = true;
  f->info = 0;
  f->fb_valid = false;
  f->inv_valid = false;
  return gblu_getrs(ctx, f, trans, nrhs, B, ldb, GBLU_HOST);
}

int32_t factor_getrf_f32_host(gblu_ctx* ctx, int64_t m, int64_t n, float* A, int64_t lda,
                              int64_t* ipiv, int64_t* info) {
  DeviceGuard g(ctx->device);
  ActiveProfiler ap(&ctx->prof);
  const int64_t ld = std::max<int64_t>(32, ((m + 31) / 32) * 32);
  size_t bytes = set_bytes<float>(m, n, ld, ctx->device, kWorkCols);
  void* arena = nullptr;
  int32_t st = ctx_alloc(ctx, bytes, &arena);
  if (st) return st;
  GetrfPlan<float> rf;
  GetrsPlan<float> rs;
  float* lu;
  int64_t *dipiv, *dinfo;
  int32_t* perm;
  CK(ctx, cudaMemsetAsync(arena, 0, bytes, ctx->stream), "clearing arena");
  carve_set<float>(reinterpret_cast<char*>(arena), m, n, ld, ctx->device, kWorkCols, &lu, &dipiv,
                   &perm, &dinfo, rf, rs);
  cudaError_t e = cudaMemcpy2DAsync(lu, ld * sizeof(float), A, lda * sizeof(float), m * sizeof(float),
                                    n, cudaMemcpyHostToDevice, ctx->stream);
  if (e == cudaSuccess) e = getrf_launch<float>(rf, ctx->stream);
  if (e == cudaSuccess)
    e = cudaMemcpy2DAsync(A, lda * sizeof(float), lu, ld * sizeof(float), m * sizeof(float), n,
                          cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(ipiv, dipiv, std::min(m, n) * sizeof(int64_t), cudaMemcpyDeviceToHost,
                        ctx->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(info, dinfo, sizeof(int64_t), cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e == cudaSuccess) st = check_device_errors(ctx, {rf.scratch});
  ctx_free(ctx, arena, bytes);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "sgetrf");
  return st;
}

int32_t factor_getrs_f32_host(gblu_ctx* ctx, char trans, int64_t n, int64_t nrhs, const float* A,
                              int64_t lda, const int64_t* ipiv, float* B, int64_t ldb) {
  DeviceGuard g(ctx->device);
  ActiveProfiler ap(&ctx->prof);
  const int64_t ld = std::max<int64_t>(32, ((n + 31) / 32) * 32);
  size_t bytes = set_bytes<float>(n, n, ld, ctx->device, kWorkCols) + align256((size_t)ld * nrhs * 4);
  void* arena = nullptr;
  int32_t st = ctx_alloc(ctx, bytes, &arena);
  if (st) return st;
  GetrfPlan<float> rf;
  GetrsPlan<float> rs;
  float* lu;
  int64_t *dipiv, *dinfo;
  int32_t* perm;
  char* end = carve_set<float>(reinterpret_cast<char*>(arena), n, n, ld, ctx->device, kWorkCols, &lu,
                               &dipiv, &perm, &dinfo, rf, rs);
  float* dB = reinterpret_cast<float*>(end);
  cudaError_t e = cudaMemsetAsync(arena, 0, bytes, ctx->stream);
  if (e == cudaSuccess)
    e = cudaMemcpy2DAsync(lu, ld * sizeof(float), A, lda * sizeof(float), n * sizeof(float), n,
                          cudaMemcpyHostToDevice, ctx->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(dipiv, ipiv, n * sizeof(int64_t), cudaMemcpyHostToDevice, ctx->stream);
  if (e == cudaSuccess) {
    upload_ipiv_check_kernel<<<std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, 1024)), 256, 0,
                               ctx->stream>>>(dipiv, n, rf.scratch);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) {
    e = cudaStreamSynchronize(ctx->stream);
    if (e == cudaSuccess) st = check_device_errors(ctx, {rf.scratch});
  }
  if (e == cudaSuccess && st == GBLU_OK) {
    e = perm_build_launch(dipiv, n, n, perm, rf.scratch, ctx->stream);
    if (e == cudaSuccess)
      e = cudaMemcpy2DAsync(dB, ld * sizeof(float), B, ldb * sizeof(float), n * sizeof(float), nrhs,
                            cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = getrs_launch<float>(rs, trans, nrhs, dB, ld, nullptr, ctx->stream);
    if (e == cudaSuccess)
      e = cudaMemcpy2DAsync(B, ldb * sizeof(float), dB, ld * sizeof(float), n * sizeof(float), nrhs,
                            cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e == cudaSuccess) st = check_device_errors(ctx, {rs.scratch});
  }
  ctx_free(ctx, arena, bytes);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "sgetrs");
  return st;
}

}  // namespace gblu
