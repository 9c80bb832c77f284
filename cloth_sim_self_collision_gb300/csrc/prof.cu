// prof.cu -- per-kernel CUDA-event timing (see prof.h).
#include <cstring>
#include <mutex>
#include <vector>

#include "prof.h"

namespace cs {

const char* const kProfNames[PK_COUNT] = {"tri_elements", "slot_reduce", "rhs",     "ilu_factor",
                                          "pcg",          "cg_spmv",     "cg_update", "cg_direction",
                                          "refit",        "traverse",    "narrow",    "impulse",
                                          "mx_spmv",      "mx_update",   "mx_direction", "mx_residual",
                                          "mx_persist",   "narrow_filter", "narrow_fv", "narrow_ee",
                                          "sort",         "narrow_ccd64"};

namespace {
struct Pending {
  int kernel;
  cudaEvent_t a, b;
};
bool g_on = false;
// the serving loop's worker and builder threads may both launch profiled kernels
std::mutex g_mu;
std::vector<Pending> g_pending;
std::vector<cudaEvent_t> g_free;
cudaEvent_t g_open[PK_COUNT];
double g_ms[PK_COUNT];
long long g_n[PK_COUNT];
constexpr int kNumCounts = 9;
const char* const kCountNames[kNumCounts] = {"pairs",       "candidates",  "contacts",    "detections",
                                             "fp64_fv_prx", "fp64_ee_prx", "fp64_fv_ccd", "fp64_ee_ccd",
                                             "persist_bytes"};
long long g_counts[kNumCounts];

cudaEvent_t get_event() {
  if (!g_free.empty()) {
    cudaEvent_t e = g_free.back();
    g_free.pop_back();
    return e;
  }
  cudaEvent_t e;
  cudaEventCreate(&e);
  return e;
}
}  // namespace

bool prof_enabled() { return g_on; }

// prof_collect with the lock held
void collect_locked();

void prof_enable(bool on) { g_on = on; }

void prof_begin(ProfKernel k, cudaStream_t s) {
  if (!g_on) return;
  std::lock_guard<std::mutex> lock(g_mu);
  g_open[k] = get_event();
  cudaEventRecord(g_open[k], s);
}

void prof_end(ProfKernel k, cudaStream_t s) {
  if (!g_on) return;
  std::lock_guard<std::mutex> lock(g_mu);
  cudaEvent_t b = get_event();
  cudaEventRecord(b, s);
  g_pending.push_back({(int)k, g_open[k], b});
  if (g_pending.size() > 4096) collect_locked();
}

void collect_locked() {
  for (Pending& p : g_pending) {
    float ms = 0;
    cudaEventSynchronize(p.b);
    if (cudaEventElapsedTime(&ms, p.a, p.b) == cudaSuccess) {
      g_ms[p.kernel] += ms;
      g_n[p.kernel] += 1;
    }
    g_free.push_back(p.a);
    g_free.push_back(p.b);
  }
  g_pending.clear();
}

void prof_collect() {
  std::lock_guard<std::mutex> lock(g_mu);
  collect_locked();
}

void prof_reset() {
  prof_collect();
  std::memset(g_ms, 0, sizeof(g_ms));
  std::memset(g_n, 0, sizeof(g_n));
  std::memset(g_counts, 0, sizeof(g_counts));
}

void prof_count(const char* name, long long n) {
  if (!g_on) return;
  for (int k = 0; k < kNumCounts; k++)
    if (std::strcmp(name, kCountNames[k]) == 0) g_counts[k] += n;
}

bool prof_read(const char* name, double* total_ms, long long* launches) {
  prof_collect();
  for (int k = 0; k < kNumCounts; k++)
    if (std::strcmp(name, kCountNames[k]) == 0) {
      if (total_ms) *total_ms = 0;
      if (launches) *launches = g_counts[k];
      return true;
    }
  for (int k = 0; k < PK_COUNT; k++)
    if (std::strcmp(name, kProfNames[k]) == 0) {
      if (total_ms) *total_ms = g_ms[k];
      if (launches) *launches = g_n[k];
      return true;
    }
  return false;
}

}  // namespace cs
