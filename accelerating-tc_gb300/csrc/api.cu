// Library-wide entry points: version, status text, per-thread error text, device init,
// the device allocation budget and phase timing.
#include <nvtx3/nvToolsExt.h>

#include <atomic>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <vector>

#include "common.cuh"

namespace atc {

static thread_local char g_err[512] = "";

void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

int sm_count() {
  static thread_local int cached_dev = -1, cached_sms = 0;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 1;
  if (dev != cached_dev) {
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cached_dev = dev;
    cached_sms = sms > 0 ? sms : 1;
  }
  return cached_sms;
}

// ---- device allocation budget ----------------------------------------------------
static std::atomic<int64_t> g_budget{-1};  // bytes left; -1 = unlimited

bool alloc_budget_take(size_t bytes) {
  int64_t left = g_budget.load(std::memory_order_relaxed);
  for (;;) {
    if (left < 0) return true;
    if ((uint64_t)left < bytes) return false;
    if (g_budget.compare_exchange_weak(left, left - (int64_t)bytes, std::memory_order_relaxed)) return true;
  }
}

// ---- phases --------------------------------------------------------------------------
namespace {
struct PhaseRec {
  char name[40];
  int depth;
  cudaEvent_t a, b;  // both null: `ms` holds the time (phase_add)
  float ms;
};
struct PhaseLog {
  bool on = false;
  int depth = 0;
  std::vector<PhaseRec> recs;
  ~PhaseLog() { clear(); }
  void clear() {
    for (auto& r : recs) {
      if (r.a) cudaEventDestroy(r.a);
      if (r.b) cudaEventDestroy(r.b);
    }
    recs.clear();
  }
};
thread_local PhaseLog g_phases;
}  // namespace

bool phase_timing_on() { return g_phases.on; }

void phase_add(const char* name, float ms) {
  PhaseLog& L = g_phases;
  if (!L.on) return;
  PhaseRec r{};
  snprintf(r.name, sizeof(r.name), "%s", name);
  r.depth = L.depth;
  r.ms = ms;
  L.recs.push_back(r);
}

Phase::Phase(const char* name, cudaStream_t s) : s_(s) {
  nvtxRangePushA(name);
  PhaseLog& L = g_phases;
  if (!L.on) return;
  PhaseRec r{};
  snprintf(r.name, sizeof(r.name), "%s", name);
  r.depth = L.depth++;
  if (cudaEventCreate(&r.a) != cudaSuccess || cudaEventCreate(&r.b) != cudaSuccess ||
      cudaEventRecord(r.a, s) != cudaSuccess) {
    if (r.a) cudaEventDestroy(r.a);
    if (r.b) cudaEventDestroy(r.b);
    --L.depth;
    return;
  }
  slot_ = (int)L.recs.size();
  L.recs.push_back(r);
}

Phase::~Phase() {
  PhaseLog& L = g_phases;
  if (slot_ >= 0 && slot_ < (int)L.recs.size()) {
    cudaEventRecord(L.recs[slot_].b, s_);
    --L.depth;
  }
  nvtxRangePop();
}

}  // namespace atc

extern "C" atc_status atc_set_alloc_budget(int64_t bytes) try {
  atc::g_budget.store(bytes < 0 ? -1 : bytes);
  return ATC_OK;
} ATC_CATCH

extern "C" atc_status atc_phase_timing(int32_t enable) try {
  atc::PhaseLog& L = atc::g_phases;
  L.clear();
  L.depth = 0;
  L.on = enable != 0;
  return ATC_OK;
} ATC_CATCH

extern "C" atc_status atc_phase_times(atc_phase_time* out, int32_t cap, int32_t* n) try {
  ATC_CHECK_ARG(n != nullptr && (cap == 0 || out != nullptr) && cap >= 0, "NULL argument");
  atc::PhaseLog& L = atc::g_phases;
  int32_t k = 0;
  for (auto& r : L.recs) {
    if (k >= cap) break;
    float ms = r.ms;
    if (r.a) {
      ATC_CK(cudaEventSynchronize(r.b));
      ATC_CK(cudaEventElapsedTime(&ms, r.a, r.b));
    }
    atc_phase_time& o = out[k++];
    memset(&o, 0, sizeof(o));
    snprintf(o.name, sizeof(o.name), "%s", r.name);
    o.depth = r.depth;
    o.ms = ms;
  }
  *n = (int32_t)L.recs.size();
  L.clear();
  return ATC_OK;
} ATC_CATCH

extern "C" const char* atc_version(void) { return "libatc 0.1 (sm_103a)"; }

extern "C" const char* atc_status_string(atc_status s) {
  switch (s) {
    case ATC_OK: return "ok";
    case ATC_ERR_INVALID: return "invalid argument";
    case ATC_ERR_OOM: return "out of memory";
    case ATC_ERR_CUDA: return "CUDA error";
    case ATC_ERR_TIMEOUT: return "device wait timed out";
    case ATC_ERR_UNSUPPORTED: return "unsupported input";
  }
  return "unknown status";
}

extern "C" const char* atc_last_error(void) { return atc::g_err; }

extern "C" atc_status atc_init(int device) try {
  int count = 0;
  cudaError_t e = cudaGetDeviceCount(&count);
  if (e != cudaSuccess || count == 0) {
    atc::set_error("no CUDA device: %s", cudaGetErrorString(e));
    return ATC_ERR_CUDA;
  }
  ATC_CHECK_ARG(device >= -1 && device < count, "device index out of range");
  if (device >= 0) ATC_CK(cudaSetDevice(device));  // -1: keep the caller's current device
  ATC_CK(cudaFree(nullptr));
  return ATC_OK;
} ATC_CATCH
