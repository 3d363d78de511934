// Kernel timing for diagnostics and the benchmark's roofline figures.
//
// When enabled (gbllt_profile_enable(1)), every kernel launch of the library is bracketed by two
// CUDA events recorded on the launch stream, and tagged with its kernel class and the
// algorithmic flops / bytes of that launch (computed from the launch's shape, not measured).
// gbllt_profile_read() waits for the recorded events and returns per-class launch counts, total
// device time and total algorithmic work.  When disabled, a launch pays one relaxed atomic load.
#include <atomic>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "internal.h"

namespace gbllt {

namespace {
std::atomic<int> g_prof_on{0};
std::mutex g_prof_mu;
struct Rec {
  int kind;
  cudaEvent_t e0, e1;
  double flops, bytes;
  cudaStream_t stream;
};
std::vector<Rec> g_recs;
std::vector<std::string> g_kinds;
std::vector<cudaEvent_t> g_free_events;

cudaEvent_t take_event() {
  if (!g_free_events.empty()) {
    cudaEvent_t e = g_free_events.back();
    g_free_events.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}

int kind_id(const char* kind) {
  for (size_t i = 0; i < g_kinds.size(); ++i)
    if (g_kinds[i] == kind) return (int)i;
  g_kinds.emplace_back(kind);
  return (int)g_kinds.size() - 1;
}
}  // namespace

ProfScope::ProfScope(const char* kind, cudaStream_t s, double flops, double bytes) : slot(-1), stream(s) {
  if (!kind || !g_prof_on.load(std::memory_order_relaxed)) return;
  std::lock_guard<std::mutex> lk(g_prof_mu);
  Rec r;
  r.kind = kind_id(kind);
  r.e0 = take_event();
  r.e1 = take_event();
  r.flops = flops;
  r.bytes = bytes;
  r.stream = s;
  cudaEventRecord(r.e0, s);
  g_recs.push_back(r);
  slot = (int)g_recs.size() - 1;
}

ProfScope::~ProfScope() {
  if (slot < 0) return;
  std::lock_guard<std::mutex> lk(g_prof_mu);
  if (slot < (int)g_recs.size()) cudaEventRecord(g_recs[slot].e1, stream);
}

}  // namespace gbllt

using namespace gbllt;

extern "C" {

int gbllt_profile_enable(int on) {
  std::lock_guard<std::mutex> lk(g_prof_mu);
  for (auto& r : g_recs) {
    cudaEventSynchronize(r.e1);
    g_free_events.push_back(r.e0);
    g_free_events.push_back(r.e1);
  }
  g_recs.clear();
  g_prof_on.store(on ? 1 : 0);
  return GBLLT_SUCCESS;
}

int gbllt_profile_read(gbllt_kernel_stat* out, int max_entries, int* n_entries) {
  if (!out && max_entries > 0) return -1;
  if (!n_entries) return -3;
  std::lock_guard<std::mutex> lk(g_prof_mu);
  std::vector<gbllt_kernel_stat> acc(g_kinds.size());
  for (size_t i = 0; i < g_kinds.size(); ++i) {
    memset(&acc[i], 0, sizeof(gbllt_kernel_stat));
    strncpy(acc[i].name, g_kinds[i].c_str(), sizeof(acc[i].name) - 1);
  }
  for (auto& r : g_recs) {
    if (cudaEventSynchronize(r.e1) != cudaSuccess) {
      cudaGetLastError();
      return GBLLT_ERR_CUDA;
    }
    float ms = 0.f;
    cudaEventElapsedTime(&ms, r.e0, r.e1);
    acc[r.kind].launches += 1;
    acc[r.kind].ms += ms;
    acc[r.kind].flops += r.flops;
    acc[r.kind].bytes += r.bytes;
  }
  int cnt = 0;
  for (auto& a : acc)
    if (a.launches > 0) {
      if (cnt < max_entries) out[cnt] = a;
      ++cnt;
    }
  *n_entries = cnt;
  return GBLLT_SUCCESS;
}

int gbllt_profile_trace(gbllt_launch_record* out, int max_entries, int* n_entries) {
  if (!out && max_entries > 0) return -1;
  if (!n_entries) return -3;
  std::lock_guard<std::mutex> lk(g_prof_mu);
  const int cnt = (int)g_recs.size();
  for (int i = 0; i < cnt && i < max_entries; ++i) {
    const Rec& r = g_recs[i];
    if (cudaEventSynchronize(r.e1) != cudaSuccess) {
      cudaGetLastError();
      return GBLLT_ERR_CUDA;
    }
    gbllt_launch_record& o = out[i];
    memset(&o, 0, sizeof o);
    strncpy(o.name, g_kinds[r.kind].c_str(), sizeof(o.name) - 1);
    o.stream = (uint64_t)(uintptr_t)r.stream;
    float t0 = 0.f, t1 = 0.f;
    cudaEventElapsedTime(&t0, g_recs[0].e0, r.e0);
    cudaEventElapsedTime(&t1, g_recs[0].e0, r.e1);
    o.start_ms = t0;
    o.end_ms = t1;
    o.flops = r.flops;
    o.bytes = r.bytes;
  }
  *n_entries = cnt;
  return GBLLT_SUCCESS;
}

}  // extern "C"
