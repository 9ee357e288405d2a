// Kernel tracing: CUDA events around every kernel launch the library makes,
// for per-kernel durations measured on the launching stream while a real
// workload runs (the benchmark's roofline figures come from these).
//
// Off by default; while off, a trace scope costs one relaxed atomic load.
// Launches recorded into a CUDA graph (stream capture) are never traced.
#include <atomic>
#include <mutex>
#include <vector>

#include "gbp_internal.cuh"

namespace gbp {
namespace {

struct Rec {
  const char* name;
  cudaEvent_t a, b;
};

std::atomic<bool> g_on{false};
std::mutex g_mu;
std::vector<Rec> g_recs;
size_t g_cap = 0;

}  // namespace

TraceScope::TraceScope(const char* name, cudaStream_t s) : slot_(-1), s_(s) {
  if (!g_on.load(std::memory_order_relaxed)) return;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(s, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) {
    cudaGetLastError();
    return;
  }
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_on.load() || g_recs.size() >= g_cap) return;
  Rec r{name, nullptr, nullptr};
  if (cudaEventCreate(&r.a) != cudaSuccess || cudaEventCreate(&r.b) != cudaSuccess) {
    if (r.a) cudaEventDestroy(r.a);
    cudaGetLastError();
    return;
  }
  cudaEventRecord(r.a, s);
  slot_ = (int)g_recs.size();
  g_recs.push_back(r);
}

TraceScope::~TraceScope() {
  if (slot_ < 0) return;
  std::lock_guard<std::mutex> lock(g_mu);
  if ((size_t)slot_ < g_recs.size()) cudaEventRecord(g_recs[slot_].b, s_);
}

}  // namespace gbp

using namespace gbp;

static void clear_records() {
  for (Rec& r : g_recs) {
    cudaEventDestroy(r.a);
    cudaEventDestroy(r.b);
  }
  g_recs.clear();
}

extern "C" int gbp_trace_enable(int capacity) {
  if (capacity < 1) return GBP_ERR_INVALID;
  std::lock_guard<std::mutex> lock(g_mu);
  clear_records();
  g_cap = (size_t)capacity;
  g_recs.reserve(g_cap);
  g_on.store(true);
  return GBP_OK;
}

extern "C" int gbp_trace_collect(gbp_trace_record* out, int max_records, int* n_records) {
  if (!n_records || (max_records > 0 && !out)) return GBP_ERR_INVALID;
  std::lock_guard<std::mutex> lock(g_mu);
  g_on.store(false);
  int n = 0;
  int st = GBP_OK;
  for (Rec& r : g_recs) {
    if (n >= max_records) break;
    float ms = -1.0f;
    if (cudaEventSynchronize(r.b) != cudaSuccess || cudaEventElapsedTime(&ms, r.a, r.b) != cudaSuccess) {
      cudaGetLastError();
      ms = -1.0f;
      st = GBP_ERR_CUDA;
    }
    out[n].kernel = r.name;
    out[n].ms = ms;
    ++n;
  }
  *n_records = n;
  clear_records();
  return st;
}
