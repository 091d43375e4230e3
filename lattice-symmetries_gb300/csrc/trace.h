// trace.h -- per-stage timing of the hot path (see trace.cu).
#pragma once

#include <cstddef>

#include <cuda_runtime.h>

namespace lsg {

bool tracing();
void set_tracing(bool on);
// Writes "stage count total_ms host_ms" lines (sorted by stage; total_ms between the stage's CUDA
// events, host_ms the wall time the host spent inside the scope) into buffer (NUL-terminated,
// truncated to size) after waiting for every traced stage; returns the full length.  reset clears
// the totals.
int trace_report(char* buffer, size_t size, bool reset);

// A traced stage: an NVTX range and a CUDA-event pair on `s` around the scope's work, when
// tracing is on; nothing otherwise.  `name` must be a string literal.
class StageScope {
 public:
  StageScope(const char* name, cudaStream_t s);
  ~StageScope();
  StageScope(const StageScope&) = delete;
  StageScope& operator=(const StageScope&) = delete;

 private:
  const char* name_;
  cudaStream_t stream_;
  cudaEvent_t start_ = nullptr, stop_ = nullptr;
  double host_start_ms_ = 0.0;
  bool active_ = false;
};

}  // namespace lsg
