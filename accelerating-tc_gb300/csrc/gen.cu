// Synthetic inputs: seeded R-MAT samples (host and device produce the same bytes)
// and the host simplifier that turns raw samples into the symmetrised, loop-free,
// duplicate-free edge lists the benchmarks feed to every program.
#include <algorithm>
#include <thread>
#include <vector>

#include "common.cuh"

namespace atc {

static bool rmat_thresholds(uint32_t a, uint32_t b, uint32_t c, uint32_t* t1, uint32_t* t2, uint32_t* t3) {
  uint64_t sa = a, sb = sa + b, sc = sb + c;
  if (sc > 1000000ull) return false;
  *t1 = (uint32_t)((sa << 32) / 1000000ull);
  *t2 = (uint32_t)((sb << 32) / 1000000ull);
  *t3 = sc == 1000000ull ? 0xFFFFFFFFu : (uint32_t)((sc << 32) / 1000000ull);
  return true;
}

__global__ void rmat_kernel(uint64_t s0, uint32_t scale, uint64_t count, uint32_t t1, uint32_t t2,
                            uint32_t t3, int2* out) {
  uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < count; i += stride) {
    int32_t u, v;
    rmat_sample(s0, scale, i, t1, t2, t3, &u, &v);
    out[i] = make_int2(u, v);
  }
}

}  // namespace atc

using namespace atc;

extern "C" atc_status atc_gen_rmat_host(uint32_t scale, uint32_t edge_factor, uint32_t a_ppm, uint32_t b_ppm,
                                        uint32_t c_ppm, uint64_t seed, int32_t* out, int nthreads) {
  ATC_CHECK_ARG(out != nullptr, "out_pairs is NULL");
  ATC_CHECK_ARG(scale >= 1 && scale <= 30, "scale must be in [1,30]");
  uint32_t t1, t2, t3;
  ATC_CHECK_ARG(rmat_thresholds(a_ppm, b_ppm, c_ppm, &t1, &t2, &t3), "a+b+c exceeds 1e6 ppm");
  uint64_t count = (uint64_t)edge_factor << scale;
  uint64_t s0 = mix64(seed);
  if (nthreads < 1) nthreads = 1;
  std::vector<std::thread> th;
  for (int t = 0; t < nthreads; ++t)
    th.emplace_back([=] {
      uint64_t b = count * t / nthreads, e = count * (t + 1) / nthreads;
      for (uint64_t i = b; i < e; ++i) rmat_sample(s0, scale, i, t1, t2, t3, out + 2 * i, out + 2 * i + 1);
    });
  for (auto& x : th) x.join();
  return ATC_OK;
}

extern "C" atc_status atc_gen_rmat_device(uint32_t scale, uint32_t edge_factor, uint32_t a_ppm, uint32_t b_ppm,
                                          uint32_t c_ppm, uint64_t seed, int32_t* out, atc_stream s) {
  ATC_CHECK_ARG(out != nullptr, "out_pairs_dev is NULL");
  ATC_CHECK_ARG(scale >= 1 && scale <= 30, "scale must be in [1,30]");
  uint32_t t1, t2, t3;
  ATC_CHECK_ARG(rmat_thresholds(a_ppm, b_ppm, c_ppm, &t1, &t2, &t3), "a+b+c exceeds 1e6 ppm");
  uint64_t count = (uint64_t)edge_factor << scale;
  if (count == 0) return ATC_OK;
  rmat_kernel<<<grid_for(count, 256, 16), 256, 0, as_stream(s)>>>(mix64(seed), scale, count, t1, t2, t3,
                                                                  reinterpret_cast<int2*>(out));
  ATC_CK(cudaGetLastError());
  ATC_CK(cudaStreamSynchronize(as_stream(s)));
  return ATC_OK;
}

extern "C" atc_status atc_simplify_host(const int32_t* pairs, uint64_t np, int symmetric, int32_t* out,
                                        uint64_t* n_out) {
  ATC_CHECK_ARG(n_out != nullptr, "n_out is NULL");
  ATC_CHECK_ARG(np == 0 || (pairs != nullptr && out != nullptr), "NULL array");
  std::vector<uint64_t> k;
  k.reserve(np * (symmetric ? 2 : 1));
  for (uint64_t i = 0; i < np; ++i) {
    int32_t a = pairs[2 * i], b = pairs[2 * i + 1];
    ATC_CHECK_ARG(a >= 0 && b >= 0, "negative vertex id");
    if (a == b) continue;
    uint32_t lo = (uint32_t)std::min(a, b), hi = (uint32_t)std::max(a, b);
    k.push_back(((uint64_t)lo << 32) | hi);
    if (symmetric) k.push_back(((uint64_t)hi << 32) | lo);
  }
  std::sort(k.begin(), k.end());
  k.erase(std::unique(k.begin(), k.end()), k.end());
  for (size_t i = 0; i < k.size(); ++i) {
    out[2 * i] = (int32_t)(k[i] >> 32);
    out[2 * i + 1] = (int32_t)(k[i] & 0xffffffffu);
  }
  *n_out = k.size();
  return ATC_OK;
}
