// Orientation-cost figures of tools/costFuncCal.cpp and tools/verification.cpp.
//
// The per-vertex degree arrays (raw degree, out-degree under id / degree / as-given
// orientation) are built on the device with atomics.  The tools print float sums
// accumulated vertex by vertex in index order; a float sum's value depends on that
// order, so the final accumulation is the same sequential loop on the host over the
// downloaded integer arrays.
#include <cmath>
#include <vector>

#include "internal.cuh"

namespace atc {
namespace {

// costFuncCal.cpp:44-61: raw degree, as-given out-degree, id-based and degree-based
// out-degrees (degree rule: src has the smaller degree, ties to the smaller id).
__global__ void cost_deg_kernel(const int2* p, uint64_t np, int32_t* deg, int32_t* lp) {
  uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < np; i += stride) {
    int2 e = p[i];
    atomicAdd(&deg[e.x], 1);
    atomicAdd(&deg[e.y], 1);
    atomicAdd(&lp[e.x], 1);
  }
}

__global__ void cost_orient_kernel(const int2* p, uint64_t np, const int32_t* deg, int32_t* idd, int32_t* dd) {
  uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < np; i += stride) {
    int s = p[i].x, d = p[i].y;
    atomicAdd(&idd[s < d ? s : d], 1);
    bool src = deg[s] < deg[d] || (deg[s] == deg[d] && s < d);
    atomicAdd(&dd[src ? s : d], 1);
  }
}

// verification.cpp:48-61: degree rule of A-order (src has the smaller degree, ties to
// the larger id).
__global__ void verif_rt_kernel(const int2* p, uint64_t np, const int32_t* deg, int32_t* rt) {
  uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < np; i += stride) {
    int s = p[i].x, d = p[i].y;
    if (deg[s] > deg[d] || (deg[s] == deg[d] && s < d)) atomicAdd(&rt[d], 1);
    else atomicAdd(&rt[s], 1);
  }
}

atc_status upload_pairs(const int32_t* pairs, uint64_t np, DevBuf<int2>* d, int* maxid, cudaStream_t s) {
  int mx = 0;
  for (uint64_t i = 0; i < 2 * np; ++i) {
    ATC_CHECK_ARG(pairs[i] >= 0, "negative vertex id");
    mx = pairs[i] > mx ? pairs[i] : mx;
  }
  *maxid = mx;
  ATC_TRY(d->alloc(np, s));
  if (np) ATC_CK(cudaMemcpyAsync(d->p, pairs, sizeof(int2) * np, cudaMemcpyHostToDevice, s));
  return ATC_OK;
}

}  // namespace
}  // namespace atc

using namespace atc;

extern "C" atc_status atc_costfunc(const int32_t* pairs, uint64_t np, int32_t k, float* out, atc_stream st) try {
  ATC_CHECK_ARG(out != nullptr, "out is NULL");
  ATC_CHECK_ARG(np == 0 || pairs != nullptr, "pairs is NULL");
  cudaStream_t s = as_stream(st);
  DevBuf<int2> d;
  int maxid = 0;
  ATC_TRY(upload_pairs(pairs, np, &d, &maxid, s));
  int64_t n = (int64_t)maxid + 1;
  DevBuf<int32_t> arr;  // deg | lp | idd | dd
  ATC_TRY(arr.alloc(4 * n, s));
  ATC_CK(cudaMemsetAsync(arr.p, 0, sizeof(int32_t) * 4 * n, s));
  int32_t *deg = arr.p, *lp = arr.p + n, *idd = arr.p + 2 * n, *dd = arr.p + 3 * n;
  if (np) {
    cost_deg_kernel<<<grid_for(np, 256), 256, 0, s>>>(d.p, np, deg, lp);
    cost_orient_kernel<<<grid_for(np, 256), 256, 0, s>>>(d.p, np, deg, idd, dd);
    ATC_CK(cudaGetLastError());
  }
  std::vector<int32_t> h(3 * n);
  ATC_CK(cudaMemcpyAsync(h.data(), lp, sizeof(int32_t) * 3 * n, cudaMemcpyDeviceToHost, s));
  ATC_CK(cudaStreamSynchronize(s));
  const int32_t *hlp = h.data(), *hid = h.data() + n, *hdd = h.data() + 2 * n;
  // costFuncCal.cpp:34,63-82 — float arithmetic in vertex order
  unsigned edgeNum = (unsigned)np;
  unsigned nodeNum = (unsigned)n;
  float avg = (float)edgeNum / nodeNum;
  float thr = k * avg;
  float idPart = 0, dPart = 0, lpPart = 0;
  auto fab = [](float a) { return a > 0 ? a : -a; };
  for (int64_t i = 0; i < n; ++i) {
    float c = fab(hid[i] - avg);
    if (hid[i] - avg > thr) idPart += c;
    c = fab(hdd[i] - avg);
    if (hdd[i] - avg > thr) dPart += c;
    c = fab(hlp[i] - avg);
    if (hlp[i] - avg > thr) lpPart += c;
  }
  out[0] = idPart;
  out[1] = dPart;
  out[2] = lpPart;
  return ATC_OK;
} ATC_CATCH

extern "C" atc_status atc_verification(const int32_t* pairs, uint64_t np, float* out, atc_stream st) try {
  ATC_CHECK_ARG(out != nullptr, "out is NULL");
  ATC_CHECK_ARG(np == 0 || pairs != nullptr, "pairs is NULL");
  cudaStream_t s = as_stream(st);
  DevBuf<int2> d;
  int maxid = 0;
  ATC_TRY(upload_pairs(pairs, np, &d, &maxid, s));
  int64_t n = (int64_t)maxid + 1;
  DevBuf<int32_t> arr;  // deg | lp | rt
  ATC_TRY(arr.alloc(3 * n, s));
  ATC_CK(cudaMemsetAsync(arr.p, 0, sizeof(int32_t) * 3 * n, s));
  int32_t *deg = arr.p, *lp = arr.p + n, *rt = arr.p + 2 * n;
  if (np) {
    cost_deg_kernel<<<grid_for(np, 256), 256, 0, s>>>(d.p, np, deg, lp);
    verif_rt_kernel<<<grid_for(np, 256), 256, 0, s>>>(d.p, np, deg, rt);
    ATC_CK(cudaGetLastError());
  }
  std::vector<int32_t> h(2 * n);
  ATC_CK(cudaMemcpyAsync(h.data(), lp, sizeof(int32_t) * 2 * n, cudaMemcpyDeviceToHost, s));
  ATC_CK(cudaStreamSynchronize(s));
  // verification.cpp:25-60
  float dAve = (float)np / n;
  float f_lp = 0;
  for (int64_t i = 0; i < n; ++i) f_lp += std::abs(dAve - h[i]);
  float f_deg = 0;
  for (int64_t i = 0; i + 1 < n; ++i) f_deg += std::abs(h[n + i] - dAve);  // skips the last vertex (:58)
  out[0] = f_lp;
  out[1] = f_deg;
  return ATC_OK;
} ATC_CATCH
