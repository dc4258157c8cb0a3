// Synthetic inputs: seeded R-MAT samples (host and device produce the same bytes)
// and the host simplifier that turns raw samples into the symmetrised, loop-free,
// duplicate-free edge lists the benchmarks feed to every program.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <thread>
#include <vector>

#include "internal.cuh"

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

// ---- 2-D random geometric graph ------------------------------------------------------
// Point i has 31-bit fixed-point coordinates drawn from one splitmix64 value; vertices
// i < j are adjacent iff (dx^2 + dy^2) <= R^2 in 64-bit integers, R = radius * 2^31.
// Integer arithmetic only, so host and device (and x86 / Arm) give the same edge set.
__host__ __device__ inline void rgg_point(uint64_t s0, uint64_t i, uint32_t* x, uint32_t* y) {
  uint64_t r = mix64(s0 + (i + 1) * kGolden);
  *x = (uint32_t)(r & 0x7fffffffu);
  *y = (uint32_t)((r >> 32) & 0x7fffffffu);
}

struct RggGrid {
  uint64_t R2;      // squared radius
  uint32_t cell;    // cell side (>= R)
  uint32_t G;       // cells per side
};

static bool rgg_grid(uint32_t n, double mean_degree, RggGrid* g) {
  if (n < 2 || !(mean_degree > 0)) return false;
  double r = std::sqrt(mean_degree / (3.141592653589793 * (double)n));
  if (!(r < 0.5)) return false;
  uint64_t R = (uint64_t)(r * 2147483648.0);
  if (R < 1) R = 1;
  g->R2 = R * R;
  g->cell = (uint32_t)R;
  g->G = (uint32_t)((2147483648ull + R - 1) / R);
  return true;
}

__global__ void rgg_keys_kernel(uint64_t s0, uint32_t n, RggGrid gr, uint64_t* keys) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    uint32_t x, y;
    rgg_point(s0, i, &x, &y);
    uint64_t c = (uint64_t)(y / gr.cell) * gr.G + x / gr.cell;
    keys[i] = (c << 32) | i;
  }
}

__global__ void rgg_cells_kernel(const uint64_t* keys, uint32_t n, uint64_t ncell, uint32_t* cstart) {
  for (uint64_t c = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; c <= ncell; c += (uint64_t)gridDim.x * blockDim.x) {
    uint64_t lo = 0, hi = n;
    while (lo < hi) {
      uint64_t mid = (lo + hi) >> 1;
      if ((keys[mid] >> 32) < c) lo = mid + 1; else hi = mid;
    }
    cstart[c] = (uint32_t)lo;
  }
}

// One thread per point: scans the 3x3 cells around it and emits (i, j) for j > i.
__global__ void rgg_edges_kernel(uint64_t s0, uint32_t n, RggGrid gr, const uint64_t* keys, const uint32_t* cstart,
                                 int2* out, unsigned long long cap, unsigned long long* count) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    uint32_t x, y;
    rgg_point(s0, i, &x, &y);
    int64_t cx = x / gr.cell, cy = y / gr.cell;
    for (int64_t yy = cy - 1; yy <= cy + 1; ++yy) {
      if (yy < 0 || yy >= gr.G) continue;
      for (int64_t xx = cx - 1; xx <= cx + 1; ++xx) {
        if (xx < 0 || xx >= gr.G) continue;
        uint64_t c = (uint64_t)yy * gr.G + (uint64_t)xx;
        for (uint32_t k = cstart[c]; k < cstart[c + 1]; ++k) {
          uint32_t j = (uint32_t)(keys[k] & 0xffffffffu);
          if (j <= i) continue;
          uint32_t xj, yj;
          rgg_point(s0, j, &xj, &yj);
          int64_t dx = (int64_t)xj - (int64_t)x, dy = (int64_t)yj - (int64_t)y;
          if ((uint64_t)(dx * dx) + (uint64_t)(dy * dy) <= gr.R2) {
            unsigned long long at = atomicAdd(count, 1ull);
            if (at < cap) out[at] = make_int2((int32_t)i, (int32_t)j);
          }
        }
      }
    }
  }
}

// ---- Chung-Lu graphs (expected-degree model) ------------------------------------------
// Vertex i has weight w_i = C (i+1)^(-1/(gamma-1)), capped at sqrt(n d) so that every edge
// probability min(1, w_u w_v / S) (S = sum of weights = n d) is a probability; C is set
// from the integral approximation of sum_i (i+1)^(-alpha).  Edges are drawn with the
// O(n + m) skip method of Miller & Hagberg (2011): weights decrease with the index, so
// for each u the candidates v > u are visited by geometric skips at the current
// probability bound and accepted with ratio q / p.  A thread per u; its uniform draws
// come from a counter-based generator, so the counting pass and the writing pass see
// the same sequence.
struct ChungLu {
  double C, alpha, cap, S;
  uint64_t s0;
  uint32_t n;
};

// Arithmetic through round-to-nearest intrinsics: the counting and the writing pass
// must produce the same values, so no operation may be contracted differently.
__device__ __forceinline__ double cl_weight(const ChungLu& c, uint32_t i) {
  double w = __dmul_rn(c.C, pow(__dadd_rn((double)i, 1.0), -c.alpha));
  return w < c.cap ? w : c.cap;
}

__device__ __forceinline__ double cl_uniform(const ChungLu& c, uint32_t u, uint32_t t) {
  uint64_t r = mix64(c.s0 + (((uint64_t)u << 32) | t) * kGolden + 0x5851F42D4C957F2Dull);
  return __dmul_rn(__dadd_rn((double)(r >> 11), 1.0), 1.0 / 9007199254740992.0);  // (0, 1]
}

__device__ __forceinline__ double cl_prob(const ChungLu& c, double wu, uint32_t v) {
  return fmin(__ddiv_rn(__dmul_rn(wu, cl_weight(c, v)), c.S), 1.0);
}

// Edges (u, v > u) of row u; writes at most `limit` of them when out != nullptr.
__device__ __forceinline__ uint32_t cl_row(const ChungLu& c, uint32_t u, int2* out, uint32_t limit) {
  uint32_t found = 0, t = 0;
  const double wu = cl_weight(c, u);
  uint32_t v = u + 1;
  if (v >= c.n) return 0;
  double p = cl_prob(c, wu, v);
  while (v < c.n && p > 0.0) {
    if (p < 1.0) {
      double r = cl_uniform(c, u, t++);
      double skip = floor(__ddiv_rn(log(r), log1p(-p)));
      if (skip >= (double)(c.n - v)) break;
      v += (uint32_t)skip;
    }
    if (v >= c.n) break;
    double q = cl_prob(c, wu, v);
    double r = cl_uniform(c, u, t++);
    if (__dmul_rn(r, p) < q || q >= 1.0) {
      if (out && found < limit) out[found] = make_int2((int32_t)u, (int32_t)v);
      ++found;
    }
    p = q;
    ++v;
  }
  return found;
}

__global__ void cl_count_kernel(ChungLu c, uint32_t* rowcnt) {
  for (uint64_t u = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; u < c.n; u += (uint64_t)gridDim.x * blockDim.x)
    rowcnt[u] = cl_row(c, (uint32_t)u, nullptr, 0);
}

__global__ void cl_write_kernel(ChungLu c, const int64_t* rowoff, const uint32_t* rowcnt, int2* out) {
  for (uint64_t u = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; u < c.n; u += (uint64_t)gridDim.x * blockDim.x)
    cl_row(c, (uint32_t)u, out + rowoff[u], rowcnt[u]);
}

static bool chunglu_params(uint32_t n, double gamma, double mean_degree, uint64_t seed, ChungLu* c) {
  if (n < 2 || !(gamma > 1.05) || !(mean_degree > 0) || mean_degree >= (double)n) return false;
  c->alpha = 1.0 / (gamma - 1.0);
  c->S = (double)n * mean_degree;
  c->cap = std::sqrt(c->S);
  // sum_{i=1..n} i^-alpha ~ integral_1^{n} x^-alpha dx + (1 + n^-alpha) / 2
  double a = c->alpha, nn = (double)n;
  double integral = std::fabs(a - 1.0) < 1e-12 ? std::log(nn) : (std::pow(nn, 1.0 - a) - 1.0) / (1.0 - a);
  double h = integral + 0.5 * (1.0 + std::pow(nn, -a));
  c->C = c->S / h;
  c->s0 = mix64(seed);
  c->n = n;
  return true;
}

}  // namespace atc

using namespace atc;

extern "C" atc_status atc_gen_chunglu_device(uint32_t n, double gamma, double mean_degree, uint64_t seed,
                                             int32_t* out_dev, uint64_t capacity, uint64_t* n_out, atc_stream st) try {
  ATC_CHECK_ARG(n_out != nullptr, "n_out is NULL");
  ChungLu c;
  ATC_CHECK_ARG(chunglu_params(n, gamma, mean_degree, seed, &c), "need n >= 2, gamma > 1.05, 0 < mean degree < n");
  cudaStream_t s = as_stream(st);
  DevBuf<uint32_t> cnt;
  DevBuf<int64_t> off;
  ATC_TRY(cnt.alloc(n + 1, s));
  ATC_TRY(off.alloc(n + 1, s));
  ATC_CK(cudaMemsetAsync(cnt.p + n, 0, sizeof(uint32_t), s));
  cl_count_kernel<<<grid_for(n, 128, 16), 128, 0, s>>>(c, cnt.p);
  ATC_CK(cudaGetLastError());
  ATC_TRY(exclusive_scan_i32_to_i64(reinterpret_cast<const int32_t*>(cnt.p), off.p, (size_t)n + 1, s));
  int64_t total = 0;
  ATC_CK(cudaMemcpyAsync(&total, off.p + n, sizeof(total), cudaMemcpyDeviceToHost, s));
  ATC_CK(cudaStreamSynchronize(s));
  *n_out = (uint64_t)total;
  if (!out_dev) return ATC_OK;
  if ((uint64_t)total > capacity) {
    set_error("Chung-Lu graph has %lld edges, capacity %llu", (long long)total, (unsigned long long)capacity);
    return ATC_ERR_INVALID;
  }
  cl_write_kernel<<<grid_for(n, 128, 16), 128, 0, s>>>(c, off.p, cnt.p, reinterpret_cast<int2*>(out_dev));
  ATC_CK(cudaGetLastError());
  ATC_CK(cudaStreamSynchronize(s));
  return ATC_OK;
} ATC_CATCH

extern "C" atc_status atc_gen_rgg_host(uint32_t n, double mean_degree, uint64_t seed, int32_t* out,
                                       uint64_t capacity, uint64_t* n_out, int nthreads) try {
  ATC_CHECK_ARG(n_out != nullptr, "n_out is NULL");
  RggGrid gr;
  ATC_CHECK_ARG(rgg_grid(n, mean_degree, &gr), "need n >= 2 and 0 < mean degree with radius < 0.5");
  uint64_t s0 = mix64(seed);
  std::vector<uint32_t> xs(n), ys(n);
  for (uint64_t i = 0; i < n; ++i) rgg_point(s0, i, &xs[i], &ys[i]);
  uint64_t ncell = (uint64_t)gr.G * gr.G;
  std::vector<uint32_t> cnt(ncell + 1, 0), order(n);
  auto cell_of = [&](uint64_t i) { return (uint64_t)(ys[i] / gr.cell) * gr.G + xs[i] / gr.cell; };
  for (uint64_t i = 0; i < n; ++i) cnt[cell_of(i) + 1]++;
  for (uint64_t c = 0; c < ncell; ++c) cnt[c + 1] += cnt[c];
  std::vector<uint32_t> cur(cnt.begin(), cnt.end() - 1);
  for (uint64_t i = 0; i < n; ++i) order[cur[cell_of(i)]++] = (uint32_t)i;  // ids ascending within a cell
  if (nthreads < 1) nthreads = 1;
  std::vector<std::vector<std::pair<int32_t, int32_t>>> part(nthreads);
  std::vector<std::thread> th;
  for (int t = 0; t < nthreads; ++t)
    th.emplace_back([&, t] {
      uint64_t b = (uint64_t)n * t / nthreads, e = (uint64_t)n * (t + 1) / nthreads;
      for (uint64_t i = b; i < e; ++i) {
        int64_t cx = xs[i] / gr.cell, cy = ys[i] / gr.cell;
        for (int64_t yy = cy - 1; yy <= cy + 1; ++yy) {
          if (yy < 0 || yy >= gr.G) continue;
          for (int64_t xx = cx - 1; xx <= cx + 1; ++xx) {
            if (xx < 0 || xx >= gr.G) continue;
            uint64_t c = (uint64_t)yy * gr.G + (uint64_t)xx;
            for (uint32_t k = cnt[c]; k < cnt[c + 1]; ++k) {
              uint32_t j = order[k];
              if (j <= i) continue;
              int64_t dx = (int64_t)xs[j] - (int64_t)xs[i], dy = (int64_t)ys[j] - (int64_t)ys[i];
              if ((uint64_t)(dx * dx) + (uint64_t)(dy * dy) <= gr.R2) part[t].emplace_back((int32_t)i, (int32_t)j);
            }
          }
        }
      }
    });
  for (auto& x : th) x.join();
  uint64_t total = 0;
  for (auto& p : part) total += p.size();
  *n_out = total;
  if (!out) return ATC_OK;
  if (total > capacity) {
    set_error("RGG has %llu edges, capacity %llu", (unsigned long long)total, (unsigned long long)capacity);
    return ATC_ERR_INVALID;
  }
  std::vector<std::pair<int32_t, int32_t>> all;
  all.reserve(total);
  for (auto& p : part) all.insert(all.end(), p.begin(), p.end());
  std::sort(all.begin(), all.end());
  for (uint64_t k = 0; k < total; ++k) {
    out[2 * k] = all[k].first;
    out[2 * k + 1] = all[k].second;
  }
  return ATC_OK;
} ATC_CATCH

extern "C" atc_status atc_gen_rgg_device(uint32_t n, double mean_degree, uint64_t seed, int32_t* out_dev,
                                         uint64_t capacity, uint64_t* n_out, atc_stream st) try {
  ATC_CHECK_ARG(n_out != nullptr, "n_out is NULL");
  RggGrid gr;
  ATC_CHECK_ARG(rgg_grid(n, mean_degree, &gr), "need n >= 2 and 0 < mean degree with radius < 0.5");
  cudaStream_t s = as_stream(st);
  uint64_t s0 = mix64(seed);
  uint64_t ncell = (uint64_t)gr.G * gr.G;
  DevBuf<uint64_t> ka, kb;
  DevBuf<uint32_t> cstart;
  DevBuf<unsigned long long> cnt;
  ATC_TRY(ka.alloc(n, s));
  ATC_TRY(kb.alloc(n, s));
  ATC_TRY(cstart.alloc(ncell + 1, s));
  ATC_TRY(cnt.alloc(1, s));
  ATC_CK(cudaMemsetAsync(cnt.p, 0, sizeof(unsigned long long), s));
  rgg_keys_kernel<<<grid_for(n, 256), 256, 0, s>>>(s0, n, gr, ka.p);
  ATC_CK(cudaGetLastError());
  uint64_t* a = ka.p;
  uint64_t* b = kb.p;
  int cb = 1;
  while ((1ull << cb) < ncell + 1) ++cb;
  ATC_TRY(sort_keys_u64(a, b, n, 0, 32 + cb, s));
  rgg_cells_kernel<<<grid_for(ncell + 1, 256), 256, 0, s>>>(a, n, ncell, cstart.p);
  rgg_edges_kernel<<<grid_for(n, 256), 256, 0, s>>>(s0, n, gr, a, cstart.p, reinterpret_cast<int2*>(out_dev),
                                                    out_dev ? capacity : 0, cnt.p);
  ATC_CK(cudaGetLastError());
  unsigned long long h = 0;
  ATC_CK(cudaMemcpyAsync(&h, cnt.p, sizeof(h), cudaMemcpyDeviceToHost, s));
  ATC_CK(cudaStreamSynchronize(s));
  *n_out = h;
  if (out_dev && h > capacity) {
    set_error("RGG has %llu edges, capacity %llu", h, (unsigned long long)capacity);
    return ATC_ERR_INVALID;
  }
  return ATC_OK;
} ATC_CATCH

extern "C" atc_status atc_gen_rmat_host(uint32_t scale, uint32_t edge_factor, uint32_t a_ppm, uint32_t b_ppm,
                                        uint32_t c_ppm, uint64_t seed, int32_t* out, int nthreads) try {
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
} ATC_CATCH

extern "C" atc_status atc_gen_rmat_device(uint32_t scale, uint32_t edge_factor, uint32_t a_ppm, uint32_t b_ppm,
                                          uint32_t c_ppm, uint64_t seed, int32_t* out, atc_stream s) try {
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
} ATC_CATCH

extern "C" atc_status atc_simplify_host(const int32_t* pairs, uint64_t np, int symmetric, int32_t* out,
                                        uint64_t* n_out) try {
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
} ATC_CATCH
