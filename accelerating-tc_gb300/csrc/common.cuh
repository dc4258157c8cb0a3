// Internal helpers shared by the libatc translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdio>
#include <exception>
#include <new>
#include <string>

#include "atc.h"

namespace atc {

// Per-thread last-error text (atc_last_error).
void set_error(const char* fmt, ...);

// Status plumbing: every CUDA call on a product path goes through CK/CKS.
#define ATC_CK(call)                                                                  \
  do {                                                                                \
    cudaError_t e_ = (call);                                                          \
    if (e_ != cudaSuccess) {                                                          \
      ::atc::set_error("%s at %s:%d: %s", #call, __FILE__, __LINE__,                  \
                       cudaGetErrorString(e_));                                       \
      return e_ == cudaErrorMemoryAllocation ? ATC_ERR_OOM : ATC_ERR_CUDA;            \
    }                                                                                 \
  } while (0)

// Closes a function-try-block around an entry point's body: a host allocation that fails
// (std::bad_alloc), any other C++ exception, and any exception of a type outside the
// std::exception hierarchy become a status, never an exception crossing the C ABI.
#define ATC_CATCH                                                       \
  catch (const std::bad_alloc&) {                                       \
    ::atc::set_error("out of host memory");                             \
    return ATC_ERR_OOM;                                                 \
  }                                                                     \
  catch (const std::exception& ex_) {                                   \
    ::atc::set_error("%s", ex_.what());                                 \
    return ATC_ERR_INVALID;                                             \
  }                                                                     \
  catch (...) {                                                         \
    ::atc::set_error("unknown C++ exception");                          \
    return ATC_ERR_INVALID;                                             \
  }

#define ATC_TRY(expr)                         \
  do {                                        \
    atc_status s_ = (expr);                   \
    if (s_ != ATC_OK) return s_;              \
  } while (0)

#define ATC_CHECK_ARG(cond, msg)                                 \
  do {                                                           \
    if (!(cond)) {                                               \
      ::atc::set_error("invalid argument: %s", msg);             \
      return ATC_ERR_INVALID;                                    \
    }                                                            \
  } while (0)

inline cudaStream_t as_stream(atc_stream s) { return reinterpret_cast<cudaStream_t>(s); }

// Number of SMs of the current device (cached per device).
int sm_count();

// Device allocation budget (atc_set_alloc_budget): takes `bytes` from the budget and
// returns true, or returns false (and takes nothing) when the budget would go below zero.
// Unlimited unless a budget was set.
bool alloc_budget_take(size_t bytes);

// Phase timing on for the calling thread (atc_phase_timing).
bool phase_timing_on();
// Records a phase whose device time was measured elsewhere (stages of a CUDA-graph replay,
// timed by event nodes inside the graph), nested in the phases open on the calling thread.
void phase_add(const char* name, float ms);

// A named phase of a call: an NVTX range (visible to Nsight tools and ncu's NVTX filters)
// and, when phase timing is on for the calling thread (atc_phase_timing), a pair of CUDA
// events on the phase's stream, read back by atc_phase_times.  Phases nest; a phase is
// recorded with its nesting depth.
class Phase {
 public:
  Phase(const char* name, cudaStream_t s);
  ~Phase();
  Phase(const Phase&) = delete;
  Phase& operator=(const Phase&) = delete;

 private:
  int slot_ = -1;
  cudaStream_t s_ = nullptr;
};

// Stream-ordered device buffer: allocated with cudaMallocAsync on the call's stream
// and released on the same stream when it goes out of scope.
template <class T>
struct DevBuf {
  T* p = nullptr;
  size_t n = 0;
  cudaStream_t s = nullptr;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  DevBuf(DevBuf&& o) noexcept : p(o.p), n(o.n), s(o.s) { o.p = nullptr; o.n = 0; }
  DevBuf& operator=(DevBuf&& o) noexcept {
    if (this != &o) { release(); p = o.p; n = o.n; s = o.s; o.p = nullptr; o.n = 0; }
    return *this;
  }
  ~DevBuf() { release(); }
  atc_status alloc(size_t count, cudaStream_t stream) {
    release();
    s = stream;
    n = count;
    if (count == 0) return ATC_OK;
    if (!alloc_budget_take(sizeof(T) * count)) {
      n = 0;
      set_error("device allocation of %zu bytes refused: the allocation budget (atc_set_alloc_budget) is spent",
                sizeof(T) * count);
      return ATC_ERR_OOM;
    }
    cudaError_t e = cudaMallocAsync(reinterpret_cast<void**>(&p), sizeof(T) * count, stream);
    if (e != cudaSuccess) {
      p = nullptr;
      n = 0;
      set_error("cudaMallocAsync(%zu bytes): %s", sizeof(T) * count, cudaGetErrorString(e));
      return e == cudaErrorMemoryAllocation ? ATC_ERR_OOM : ATC_ERR_CUDA;
    }
    return ATC_OK;
  }
  void release() {
    if (p) cudaFreeAsync(p, s);
    p = nullptr;
    n = 0;
  }
  T* detach() { T* q = p; p = nullptr; n = 0; return q; }
};

inline unsigned grid_for(int64_t work, int block, int per_sm = 8) {
  int64_t g = (work + block - 1) / block;
  int64_t cap = (int64_t)sm_count() * per_sm;
  if (g > cap) g = cap;
  if (g < 1) g = 1;
  return (unsigned)g;
}

// splitmix64 finalizer (Steele, Lea, Flood 2014): the counter-based random source of
// every generator here, identical on host and device.
__host__ __device__ inline uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
constexpr uint64_t kGolden = 0x9E3779B97F4A7C15ull;

// R-MAT sample i: `scale` levels, one 32-bit draw per level, quadrant thresholds
// t1 < t2 < t3 on [0, 2^32).  Bits are chosen most-significant first.
__host__ __device__ inline void rmat_sample(uint64_t s0, uint32_t scale, uint64_t i, uint32_t t1,
                                            uint32_t t2, uint32_t t3, int32_t* u, int32_t* v) {
  uint32_t a = 0, b = 0;
  uint64_t r = 0;
  for (uint32_t l = 0; l < scale; ++l) {
    if ((l & 1) == 0) r = mix64(s0 + (i * 16 + (l >> 1) + 1) * kGolden);
    uint32_t x = (l & 1) ? (uint32_t)(r >> 32) : (uint32_t)r;
    uint32_t row = x >= t2;             // quadrants c, d
    uint32_t col = (x >= t1 && x < t2) || x >= t3;  // quadrants b, d
    a = (a << 1) | row;
    b = (b << 1) | col;
  }
  *u = (int32_t)a;
  *v = (int32_t)b;
}

// Stream-ordered timing helper: events recorded on the call's stream.
struct EventTimer {
  cudaEvent_t a = nullptr, b = nullptr;
  EventTimer() { cudaEventCreate(&a); cudaEventCreate(&b); }
  ~EventTimer() { if (a) cudaEventDestroy(a); if (b) cudaEventDestroy(b); }
  void start(cudaStream_t s) { cudaEventRecord(a, s); }
  void stop(cudaStream_t s) { cudaEventRecord(b, s); }
  float ms() { float t = 0; cudaEventSynchronize(b); cudaEventElapsedTime(&t, a, b); return t; }
};

}  // namespace atc
