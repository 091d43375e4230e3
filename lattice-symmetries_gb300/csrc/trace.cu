// trace.cu -- per-stage timing of the hot path (the GPU counterpart of the reference's timing
// tree: chapel/src/Utils.chpl:49-144, used around enumeration and each matvec stage at
// BatchedOperator.chpl:104-109, :284-295 and DistributedMatrixVector.chpl:74-89).
//
// Off by default.  When on, every traced stage opens an NVTX range (visible in a profiler
// timeline) and records a pair of CUDA events on the stream the stage runs on; the elapsed times
// are read only when a report is requested, so tracing adds no synchronisation to the stages.
// Do not switch tracing on while a stream is being captured into a CUDA graph (event records
// would become graph nodes that the report cannot read).
#include <nvtx3/nvToolsExt.h>

#include <chrono>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "trace.h"

namespace lsg {
namespace {

struct Pending {
  const char* name;
  cudaEvent_t start, stop;
  double host_ms;  // wall time the host spent inside the scope
};
struct Total {
  int64_t count = 0;
  double ms = 0.0;
  double host_ms = 0.0;
};

double host_now_ms() {
  return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

std::mutex g_trace_mutex;
bool g_tracing = false;
std::vector<Pending> g_pending;
std::vector<cudaEvent_t> g_free_events;
std::map<std::string, Total> g_totals;

cudaEvent_t take_event() {
  if (!g_free_events.empty()) {
    cudaEvent_t e = g_free_events.back();
    g_free_events.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  if (cudaEventCreate(&e) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return e;
}

// Reads every pending event pair into the totals (waits for the stages to finish).
void resolve_locked() {
  for (const Pending& p : g_pending) {
    float ms = 0.f;
    if (cudaEventSynchronize(p.stop) == cudaSuccess && cudaEventElapsedTime(&ms, p.start, p.stop) == cudaSuccess) {
      Total& t = g_totals[p.name];
      t.count += 1;
      t.ms += ms;
      t.host_ms += p.host_ms;
    } else {
      cudaGetLastError();
    }
    g_free_events.push_back(p.start);
    g_free_events.push_back(p.stop);
  }
  g_pending.clear();
}

}  // namespace

bool tracing() {
  std::lock_guard<std::mutex> lock(g_trace_mutex);
  return g_tracing;
}

StageScope::StageScope(const char* name, cudaStream_t s) : name_(name), stream_(s) {
  std::lock_guard<std::mutex> lock(g_trace_mutex);
  if (!g_tracing) return;
  start_ = take_event();
  stop_ = take_event();
  if (start_ == nullptr || stop_ == nullptr) return;
  active_ = true;
  nvtxRangePushA(name);
  cudaEventRecord(start_, stream_);
  host_start_ms_ = host_now_ms();
}

StageScope::~StageScope() {
  if (!active_) return;
  const double host_ms = host_now_ms() - host_start_ms_;
  std::lock_guard<std::mutex> lock(g_trace_mutex);
  cudaEventRecord(stop_, stream_);
  nvtxRangePop();
  g_pending.push_back(Pending{name_, start_, stop_, host_ms});
}

void set_tracing(bool on) {
  std::lock_guard<std::mutex> lock(g_trace_mutex);
  g_tracing = on;
}

int trace_report(char* buffer, size_t size, bool reset) {
  std::lock_guard<std::mutex> lock(g_trace_mutex);
  resolve_locked();
  std::string out;
  char line[256];
  for (const auto& kv : g_totals) {
    snprintf(line, sizeof(line), "%s %lld %.6f %.6f\n", kv.first.c_str(), (long long)kv.second.count, kv.second.ms,
             kv.second.host_ms);
    out += line;
  }
  if (reset) g_totals.clear();
  if (buffer != nullptr && size > 0) {
    const size_t n = std::min(size - 1, out.size());
    memcpy(buffer, out.data(), n);
    buffer[n] = '\0';
  }
  return (int)out.size();
}

}  // namespace lsg
