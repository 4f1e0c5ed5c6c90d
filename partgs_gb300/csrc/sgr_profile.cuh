// Optional per-phase CUDA-event timing of the entry points.
#pragma once

#include <cuda_runtime.h>

#include <mutex>
#include <vector>

#include "../../include/sgr.h"

namespace sgr {

class PhaseTimer {
 public:
  static PhaseTimer& get() {
    static PhaseTimer t;
    return t;
  }
  bool enabled() const { return enabled_; }
  void enable(bool on) { enabled_ = on; }

  // Records the start event of `phase` on `st` and returns its slot.
  int begin(int phase, cudaStream_t st) {
    if (!enabled_) return -1;
    std::lock_guard<std::mutex> g(mu_);
    Rec r;
    r.phase = phase;
    cudaEventCreate(&r.a);
    cudaEventCreate(&r.b);
    cudaEventRecord(r.a, st);
    recs_.push_back(r);
    return (int)recs_.size() - 1;
  }
  void end(int slot, cudaStream_t st) {
    if (slot < 0) return;
    std::lock_guard<std::mutex> g(mu_);
    if (slot < (int)recs_.size()) {
      cudaEventRecord(recs_[slot].b, st);
      recs_[slot].closed = true;
    }
  }
  int read(float* ms, int32_t* count) {
    std::lock_guard<std::mutex> g(mu_);
    for (int p = 0; p < SGR_NUM_PHASES; ++p) {
      if (ms) ms[p] = 0.f;
      if (count) count[p] = 0;
    }
    int rc = SGR_OK;
    for (auto& r : recs_) {
      if (r.closed) {
        float t = 0.f;
        if (cudaEventSynchronize(r.b) != cudaSuccess || cudaEventElapsedTime(&t, r.a, r.b) != cudaSuccess)
          rc = SGR_ERR_CUDA;
        if (ms) ms[r.phase] += t;
        if (count) count[r.phase] += 1;
      }
      cudaEventDestroy(r.a);
      cudaEventDestroy(r.b);
    }
    recs_.clear();
    return rc;
  }

 private:
  struct Rec {
    int phase = 0;
    cudaEvent_t a = nullptr, b = nullptr;
    bool closed = false;
  };
  bool enabled_ = false;
  std::mutex mu_;
  std::vector<Rec> recs_;
};

// Scope guard: times the enclosed launches as one phase.
struct PhaseScope {
  int slot;
  cudaStream_t st;
  PhaseScope(int phase, cudaStream_t s) : slot(PhaseTimer::get().begin(phase, s)), st(s) {}
  ~PhaseScope() { PhaseTimer::get().end(slot, st); }
};

}  // namespace sgr
