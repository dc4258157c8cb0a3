// Library-wide entry points: version, status text, per-thread error text, device init.
#include <cstdarg>
#include <cstdio>

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

}  // namespace atc

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
  ATC_CHECK_ARG(device >= 0 && device < count, "device index out of range");
  ATC_CK(cudaSetDevice(device));
  ATC_CK(cudaFree(nullptr));
  return ATC_OK;
} ATC_CATCH
