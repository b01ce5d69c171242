// Per-kernel device time of a step launched kernel by kernel (benchmark profiling).
//
// With profiling on, the step runs as direct launches and every launch is
// bracketed by two CUDA events on its stream; once the stream has drained the
// pairs are summed per kernel name (multigrid kernels carry their level, e.g.
// "k_mg_down@1").  After each host read-back inside the step (the mixed solve's
// loop decisions) a short spin kernel keeps the stream busy while the host
// queues the next launches, so that the events bracket kernel execution and not
// host launch latency.  Host code only; one profiled step at a time per handle.
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

namespace pfgb {

struct KProf {
  std::vector<cudaEvent_t> ev;       // event pool, reused across steps (2 per launch)
  std::vector<std::string> name;     // kernel of each recorded pair
  size_t n = 0;                      // pairs recorded since the last clear
  bool ok = true;                    // false once an event could not be created or recorded

  KProf() = default;
  KProf(const KProf&) = delete;
  KProf& operator=(const KProf&) = delete;
  ~KProf() {
    for (cudaEvent_t e : ev) cudaEventDestroy(e);
  }
  void clear() {
    n = 0;
    ok = true;
  }
  bool begin(const char* kernel, int level, cudaStream_t s) {
    if (!ok) return false;
    if (2 * n + 2 > ev.size()) {
      const size_t old = ev.size();
      ev.resize(old ? 2 * old : 512);
      for (size_t k = old; k < ev.size(); ++k)
        if (cudaEventCreate(&ev[k]) != cudaSuccess) {
          ev.resize(k);
          ok = false;
          return false;
        }
    }
    if (name.size() <= n) name.resize(n + 1);
    name[n] = level >= 0 ? std::string(kernel) + "@" + std::to_string(level) : std::string(kernel);
    if (cudaEventRecord(ev[2 * n], s) != cudaSuccess) {
      ok = false;
      return false;
    }
    return true;
  }
  void end(cudaStream_t s) {
    if (cudaEventRecord(ev[2 * n + 1], s) != cudaSuccess) {
      ok = false;
      return;
    }
    ++n;
  }
};

struct KTime {
  std::string name;
  int launches = 0;
  double ms = 0.0;
};

// Sum the recorded pairs per kernel name, in order of first launch (the events must
// have completed: call after the step's stream has been synchronised).
inline cudaError_t kprof_collect(const KProf& kp, std::vector<KTime>& out) {
  out.clear();
  for (size_t k = 0; k < kp.n; ++k) {
    float t = 0.f;
    const cudaError_t e = cudaEventElapsedTime(&t, kp.ev[2 * k], kp.ev[2 * k + 1]);
    if (e != cudaSuccess) return e;
    size_t j = 0;
    while (j < out.size() && out[j].name != kp.name[k]) ++j;
    if (j == out.size()) out.push_back(KTime{kp.name[k], 0, 0.0});
    out[j].launches += 1;
    out[j].ms += t;
  }
  return cudaSuccess;
}

}  // namespace pfgb

// Launch `...` (a kernel launch statement) bracketed by profiling events when kp is set.
#define PFGB_TIMED(kp, kernel, level, s, ...)                                \
  do {                                                                       \
    const bool pfgb_timed_ = (kp) != nullptr && (kp)->begin(kernel, level, s); \
    __VA_ARGS__;                                                             \
    if (pfgb_timed_) (kp)->end(s);                                           \
  } while (0)
