// Launch accounting: every kernel launch site in the library goes through a
// LaunchScope, which counts launches and, when the calling context has
// profiling enabled, brackets the launch with CUDA events on its stream so the
// host can read per-kind device time and the algorithmic work of each launch.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

namespace gblu {

enum KernelKind : int {
  K_GEMM = 0,     // trailing-matrix update C -= A B
  K_PANEL = 1,    // cooperative panel getf2
  K_LASWP = 2,    // row interchanges outside the panel
  K_TRSM = 3,     // unit-lower triangular solve of the U12 block
  K_PERM = 4,     // permutation from ipiv
  K_SOLVE = 5,    // getrs wavefront sweeps
  K_REFINE = 6,   // residuals, norms, conversions of the refinement loop
  K_BATCH = 7,    // batched persistent factor+solve
  K_OTHER = 8,
  K_NKINDS = 9,
};

// Launch counts and algorithmic work of a launch sequence (a captured graph
// replays them without passing through a LaunchScope).
struct LaunchCounts {
  uint64_t launches = 0;
  uint64_t count[K_NKINDS] = {};
  double flops[K_NKINDS] = {};
  double bytes[K_NKINDS] = {};
};

struct Profiler {
  bool enabled = false;
  uint64_t launches = 0;
  uint64_t count[K_NKINDS] = {};
  double ms[K_NKINDS] = {};
  double flops[K_NKINDS] = {};
  double bytes[K_NKINDS] = {};

  LaunchCounts counts() const {
    LaunchCounts c;
    c.launches = launches;
    for (int k = 0; k < K_NKINDS; ++k) c.count[k] = count[k], c.flops[k] = flops[k], c.bytes[k] = bytes[k];
    return c;
  }
  static LaunchCounts diff(const LaunchCounts& a, const LaunchCounts& b) {  // b - a
    LaunchCounts c;
    c.launches = b.launches - a.launches;
    for (int k = 0; k < K_NKINDS; ++k)
      c.count[k] = b.count[k] - a.count[k], c.flops[k] = b.flops[k] - a.flops[k],
      c.bytes[k] = b.bytes[k] - a.bytes[k];
    return c;
  }
  void add(const LaunchCounts& c) {
    launches += c.launches;
    for (int k = 0; k < K_NKINDS; ++k) count[k] += c.count[k], flops[k] += c.flops[k], bytes[k] += c.bytes[k];
  }
  void sub(const LaunchCounts& c) {
    launches -= c.launches;
    for (int k = 0; k < K_NKINDS; ++k) count[k] -= c.count[k], flops[k] -= c.flops[k], bytes[k] -= c.bytes[k];
  }
  struct Pending {
    int kind;
    double flops, bytes;
    cudaEvent_t a, b;
  };
  std::vector<Pending> pending;
  std::vector<cudaEvent_t> pool;

  cudaEvent_t get_event() {
    if (!pool.empty()) {
      cudaEvent_t e = pool.back();
      pool.pop_back();
      return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
  }
  // Resolve pending event pairs (the stream must be synchronised first).
  void drain() {
    for (auto& p : pending) {
      float t = 0.f;
      if (cudaEventElapsedTime(&t, p.a, p.b) == cudaSuccess) ms[p.kind] += t;
      pool.push_back(p.a);
      pool.push_back(p.b);
    }
    pending.clear();
    cudaGetLastError();
  }
  void reset() {
    launches = 0;
    for (int k = 0; k < K_NKINDS; ++k) count[k] = 0, ms[k] = flops[k] = bytes[k] = 0;
  }
  ~Profiler() {
    for (auto& p : pending) { cudaEventDestroy(p.a); cudaEventDestroy(p.b); }
    for (auto e : pool) cudaEventDestroy(e);
  }
};

// The profiler of the context whose call is running on this thread.
extern thread_local Profiler* tl_profiler;

struct ActiveProfiler {
  Profiler* prev;
  explicit ActiveProfiler(Profiler* p) : prev(tl_profiler) { tl_profiler = p; }
  ~ActiveProfiler() { tl_profiler = prev; }
};

struct LaunchScope {
  Profiler* p;
  int kind;
  double flops, bytes;
  cudaStream_t s;
  cudaEvent_t a = nullptr;
  LaunchScope(int kind_, double flops_, double bytes_, cudaStream_t s_)
      : p(tl_profiler), kind(kind_), flops(flops_), bytes(bytes_), s(s_) {
    if (p) {
      p->launches++;
      p->count[kind]++;
      p->flops[kind] += flops;
      p->bytes[kind] += bytes;
      if (p->enabled) {
        a = p->get_event();
        cudaEventRecord(a, s);
      }
    }
  }
  ~LaunchScope() {
    if (p && p->enabled && a) {
      cudaEvent_t b = p->get_event();
      cudaEventRecord(b, s);
      p->pending.push_back({kind, flops, bytes, a, b});
    }
  }
};

}  // namespace gblu
