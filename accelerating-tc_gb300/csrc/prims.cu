// Device-wide sort / unique / scan used by preTC.  These are plain library
// primitives (CUB, shipped with the CUDA toolkit), in the role thrust::sort /
// thrust::unique / thrust::exclusive_scan play in the reference preprocessing
// (Hu/preTC.cu:208-212, tricount_gpu.cu:172-174, kcl.cu:197).
#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>
#include <cub/device/device_select.cuh>
#include <thrust/iterator/transform_iterator.h>

#include "internal.cuh"

namespace atc {

atc_status sort_keys_u64(uint64_t*& keys, uint64_t*& alt, size_t n, int begin_bit, int end_bit, cudaStream_t s) {
  if (n <= 1) return ATC_OK;
  cub::DoubleBuffer<uint64_t> db(keys, alt);
  size_t tmp = 0;
  ATC_CK(cub::DeviceRadixSort::SortKeys(nullptr, tmp, db, (int64_t)n, begin_bit, end_bit, s));
  DevBuf<char> t;
  ATC_TRY(t.alloc(tmp, s));
  ATC_CK(cub::DeviceRadixSort::SortKeys(t.p, tmp, db, (int64_t)n, begin_bit, end_bit, s));
  if (db.Current() != keys) {
    alt = keys;
    keys = db.Current();
  }
  return ATC_OK;
}

atc_status sort_pairs_u64_i32(uint64_t*& keys, uint64_t*& kalt, int32_t*& vals, int32_t*& valt, size_t n, int begin_bit,
                             int end_bit, cudaStream_t s) {
  if (n <= 1) return ATC_OK;
  cub::DoubleBuffer<uint64_t> dk(keys, kalt);
  cub::DoubleBuffer<int32_t> dv(vals, valt);
  size_t tmp = 0;
  ATC_CK(cub::DeviceRadixSort::SortPairs(nullptr, tmp, dk, dv, (int64_t)n, begin_bit, end_bit, s));
  DevBuf<char> t;
  ATC_TRY(t.alloc(tmp, s));
  ATC_CK(cub::DeviceRadixSort::SortPairs(t.p, tmp, dk, dv, (int64_t)n, begin_bit, end_bit, s));
  if (dk.Current() != keys) {
    kalt = keys;
    keys = dk.Current();
  }
  if (dv.Current() != vals) {
    valt = vals;
    vals = dv.Current();
  }
  return ATC_OK;
}

atc_status unique_u64(const uint64_t* in, uint64_t* out, size_t n, size_t* n_out, cudaStream_t s) {
  if (n == 0) { *n_out = 0; return ATC_OK; }
  DevBuf<int64_t> cnt;
  ATC_TRY(cnt.alloc(1, s));
  size_t tmp = 0;
  ATC_CK(cub::DeviceSelect::Unique(nullptr, tmp, in, out, cnt.p, (int64_t)n, s));
  DevBuf<char> t;
  ATC_TRY(t.alloc(tmp, s));
  ATC_CK(cub::DeviceSelect::Unique(t.p, tmp, in, out, cnt.p, (int64_t)n, s));
  int64_t h = 0;
  ATC_CK(cudaMemcpyAsync(&h, cnt.p, sizeof(h), cudaMemcpyDeviceToHost, s));
  ATC_CK(cudaStreamSynchronize(s));
  *n_out = (size_t)h;
  return ATC_OK;
}

atc_status exclusive_scan_i64(const int64_t* in, int64_t* out, size_t n, cudaStream_t s) {
  if (n == 0) return ATC_OK;
  size_t tmp = 0;
  ATC_CK(cub::DeviceScan::ExclusiveSum(nullptr, tmp, in, out, (int64_t)n, s));
  DevBuf<char> t;
  ATC_TRY(t.alloc(tmp, s));
  ATC_CK(cub::DeviceScan::ExclusiveSum(t.p, tmp, in, out, (int64_t)n, s));
  return ATC_OK;
}

struct I32ToI64 {
  __host__ __device__ int64_t operator()(int32_t x) const { return (int64_t)x; }
};

atc_status exclusive_scan_i32_to_i64(const int32_t* in, int64_t* out, size_t n, cudaStream_t s) {
  if (n == 0) return ATC_OK;
  thrust::transform_iterator<I32ToI64, const int32_t*, int64_t> it(in, I32ToI64());
  size_t tmp = 0;
  ATC_CK(cub::DeviceScan::ExclusiveSum(nullptr, tmp, it, out, (int64_t)n, s));
  DevBuf<char> t;
  ATC_TRY(t.alloc(tmp, s));
  ATC_CK(cub::DeviceScan::ExclusiveSum(t.p, tmp, it, out, (int64_t)n, s));
  return ATC_OK;
}

// The same scan with caller-provided temporary storage (no allocation, so it can be
// recorded into a CUDA graph).  tmp == nullptr: *bytes receives the size needed.
atc_status exclusive_scan_i32_to_i64_tmp(void* tmp, size_t* bytes, const int32_t* in, int64_t* out, size_t n,
                                         cudaStream_t s) {
  thrust::transform_iterator<I32ToI64, const int32_t*, int64_t> it(in, I32ToI64());
  ATC_CK(cub::DeviceScan::ExclusiveSum(tmp, *bytes, it, out, (int64_t)n, s));
  return ATC_OK;
}

}  // namespace atc
