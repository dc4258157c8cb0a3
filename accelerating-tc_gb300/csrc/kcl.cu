// k-clique counting on an oriented CSR (k >= 3), exact in uint64.
//
// The reference (k-clique/kcl.cu:147-215, Pangolin) materialises every level of the
// embedding list in HBM: per level it counts extensions (extend_alloc, :16-50), scans
// them (thrust::exclusive_scan, :197) and writes the next level (extend_insert,
// :115-145), counting instead of writing at level k-2.  Here each warp walks the
// search tree of one oriented edge (u, v) depth first, so nothing but a small stack of
// candidate sets is ever stored:
//
//   C0 = N+(u) ∩ N+(v);  C(l+1) = C(l) ∩ N+(w) for the w chosen from C(l);
//   with k-1 vertices chosen, every element of the current candidate set completes a
//   k-clique, so the last level is counted, never stored.
// When |C0| <= 64 (every RGG edge, most R-MAT edges) the warp instead builds the 64-bit
// successor masks of the DAG induced on C0 with one ballot per member, and each lane
// counts the remaining (k-2)-cliques of its first member with AND / popc on registers.
// From k = 5 on, edges with 64 < |C0| <= 1024 go to a second kernel, a CTA per edge, that
// counts the (k-2)-cliques of C0 from bitmap rows in shared memory (kcl_dense_kernel).
//
// Orientation is acyclic, so every k-clique is found once, from its first two vertices
// in orientation order — the same count kcl_gpu_solver accumulates.  Intersections:
// lanes take the elements of the candidate set (a subset of N+(u)), binary-search each
// in N+(w), and ballot/popc compact the hits in order into the next level, which lives
// in the warp's slice of a scratch buffer ((k-2) x max out-degree ints per warp).
#include <algorithm>

#include "internal.cuh"

namespace atc {

namespace {

__device__ __forceinline__ bool kc_has(const int32_t* a, int64_t n, int32_t x) {
  int64_t lo = 0, hi = n;
  while (lo < hi) {
    int64_t mid = (lo + hi) >> 1;
    if (a[mid] < x) lo = mid + 1; else hi = mid;
  }
  return lo < n && a[lo] == x;
}

// Writes P ∩ L (P given, L sorted) into out in P's order; returns the size (all lanes).
__device__ __forceinline__ int warp_intersect(const int32_t* P, int np, const int32_t* L, int64_t nl, int32_t* out,
                                              int lane) {
  int total = 0;
  for (int base = 0; base < np; base += 32) {
    int j = base + lane;
    bool hit = j < np && kc_has(L, nl, P[j]);
    unsigned mask = __ballot_sync(0xffffffffu, hit);
    if (hit && out) out[total + __popc(mask & ((1u << lane) - 1))] = P[j];
    total += __popc(mask);
  }
  __syncwarp();
  return total;
}

constexpr int kKcWarps = 8;
constexpr int kMaxK = 16;
constexpr int kMaskMax = 64;     // candidate sets up to this size use the warp's bitmask path
constexpr int kDenseMax = 1024;  // larger ones up to this size: a CTA per edge, bitmaps in shared memory
constexpr int kDenseWords = kDenseMax / 64;
constexpr int kDenseThreads = 1024;  // 256: R-MAT s20 k = 6 4.84 s; 512: 3.81 s; 1024: 3.70 s

// d-cliques inside `mask` of the DAG whose successor sets (within C0) are adj[]:
// cliq(1, M) = |M|, cliq(d, M) = sum_{i in M} cliq(d-1, M & adj[i]).  Iterative, one
// lane, an explicit stack of (remaining mask, candidate mask) per depth.
__device__ __forceinline__ unsigned long long mask_cliques(const unsigned long long* adj, unsigned long long mask,
                                                           int d) {
  if (d <= 0) return 1ull;
  if (d == 1) return (unsigned long long)__popcll(mask);
  unsigned long long total = 0;
  unsigned long long rem[kMaxK], cand[kMaxK];
  int top = 0;
  rem[0] = mask;
  cand[0] = mask;
  while (top >= 0) {
    if (rem[top] == 0) {
      --top;
      continue;
    }
    int i = __ffsll(rem[top]) - 1;
    rem[top] &= rem[top] - 1;
    unsigned long long nm = cand[top] & adj[i];
    int left = d - 1 - top;  // vertices still to choose after i
    if (left == 1) {
      total += (unsigned long long)__popcll(nm);
    } else if (__popcll(nm) >= left) {
      ++top;
      rem[top] = nm;
      cand[top] = nm;
    }
  }
  return total;
}

// dense (nullable): edges whose C0 has kMaskMax < |C0| <= kDenseMax are appended to
// dense[1 + ...] (count in dense[0]) for kcl_dense_kernel instead of being walked here.
__global__ void __launch_bounds__(kKcWarps * 32) kcl_kernel(const int64_t* off, const int32_t* cols, const int32_t* esrc,
                                                          int64_t e0, int64_t e1, int k, int cap, int32_t* scratch,
                                                          unsigned long long* dense, unsigned long long* out) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int64_t gw = (int64_t)blockIdx.x * kKcWarps + w;
  const int64_t warps = (int64_t)gridDim.x * kKcWarps;
  const int levels = k - 2;
  int32_t* buf = scratch + gw * (int64_t)levels * cap;
  __shared__ unsigned long long adjm[kKcWarps][kMaskMax];
  unsigned long long cnt = 0, bytes = 0;
  int size[kMaxK];
  int idx[kMaxK];
  for (int64_t e = e0 + gw; e < e1; e += warps) {
    int32_t u = esrc[e], v = cols[e];
    int64_t ub = off[u], ud = off[u + 1] - ub;
    int64_t vb = off[v], vd = off[v + 1] - vb;
    bytes += 4ull * (unsigned long long)vd;
    // C0 = N+(u) ∩ N+(v), in the order of N+(u)
    int c0 = warp_intersect(cols + ub, (int)ud, cols + vb, vd, levels > 1 ? buf : nullptr, lane);
    if (levels == 1) {
      cnt += c0;
      continue;
    }
    if (c0 < levels) continue;  // not enough candidates for k-2 more vertices
    if (dense && c0 > kMaskMax && c0 <= kDenseMax) {
      if (lane == 0) dense[1 + atomicAdd(dense, 1ull)] = (unsigned long long)e;
      bytes -= 4ull * (unsigned long long)vd;  // the dense kernel reads N+(v) again and counts it
      continue;
    }
    if (c0 <= kMaskMax) {
      // bitmask path: adjm[w][i] = members of C0 that are successors of C0[i]
      for (int i = 0; i < c0; ++i) {
        int32_t x = buf[i];
        int64_t xb = off[x], xd = off[x + 1] - xb;
        bytes += 4ull * (unsigned long long)xd;
        bool h0 = lane < c0 && kc_has(cols + xb, xd, buf[lane]);
        bool h1 = lane + 32 < c0 && kc_has(cols + xb, xd, buf[lane + 32]);
        unsigned lo = __ballot_sync(0xffffffffu, h0), hi = __ballot_sync(0xffffffffu, h1);
        if (lane == 0) adjm[w][i] = ((unsigned long long)hi << 32) | lo;
      }
      __syncwarp();
      // (k-2)-cliques of the DAG on C0: lane i takes the ones whose first vertex is C0[i]
      unsigned long long part = 0;
      for (int i = lane; i < c0; i += 32) part += mask_cliques(adjm[w], adjm[w][i], levels - 1);
      for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
      cnt += part;
      __syncwarp();
      continue;
    }
    size[0] = c0;
    idx[0] = 0;
    int l = 0;  // level whose candidates are being chosen from
    while (l >= 0) {
      if (idx[l] >= size[l]) {
        --l;
        if (l >= 0) ++idx[l];
        continue;
      }
      // choose x from C(l); the next level is all of C(l) ∩ N+(x) (lists are sorted by
      // id, not by orientation order, so no prefix of C(l) can be skipped)
      int32_t x = buf[(int64_t)l * cap + idx[l]];
      int64_t xb = off[x], xd = off[x + 1] - xb;
      bytes += 4ull * (unsigned long long)xd;
      const int32_t* P = buf + (int64_t)l * cap;
      if (l == levels - 2) {
        cnt += warp_intersect(P, size[l], cols + xb, xd, nullptr, lane);  // k-th vertices
        ++idx[l];
      } else {
        int c = warp_intersect(P, size[l], cols + xb, xd, buf + (int64_t)(l + 1) * cap, lane);
        if (c >= levels - 1 - l) {
          ++l;
          size[l] = c;
          idx[l] = 0;
        } else {
          ++idx[l];
        }
      }
    }
  }
  if (lane != 0) { cnt = 0; bytes = 0; }
  for (int o = 16; o > 0; o >>= 1) {
    cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
    bytes += __shfl_xor_sync(0xffffffffu, bytes, o);
  }
  if (lane == 0) {
    if (cnt) atomicAdd(out, cnt);
    if (bytes) atomicAdd(out + 1, bytes);
  }
}

// Position of the r-th (from 0) set bit of x; x has more than r set bits.
__device__ __forceinline__ int select_bit(unsigned long long x, int r) {
  int pos = 0;
#pragma unroll
  for (int s = 32; s > 0; s >>= 1) {
    const int c = __popcll(x & ((1ull << s) - 1));
    if (r >= c) {
      r -= c;
      x >>= s;
      pos += s;
    }
  }
  return pos;
}

// d-cliques (d >= 1) among the common higher neighbours of members i < j of C0, in the
// graph whose rows U (`words` uint64 each) hold every member's higher-indexed neighbours:
// cliq(1, M) = |M|, cliq(d, M) = sum_{x in M} cliq(d-1, M & U[x]).  Every set below holds
// members above the last one chosen only, so the word loops start at that member's word.
// One thread, an explicit stack of candidate sets.
__device__ unsigned long long pair_cliques(const unsigned long long* U, int words, int i, int j, int d) {
  const unsigned long long* Ri = U + (size_t)i * words;
  const unsigned long long* Rj = U + (size_t)j * words;
  const int w0 = (j + 1) >> 6;
  if (d == 1) {
    unsigned long long c = 0;
    for (int w = w0; w < words; ++w) c += __popcll(Ri[w] & Rj[w]);
    return c;
  }
  unsigned long long st[kMaxK - 4][kDenseWords];
  int pos[kMaxK - 4];
  int n0 = 0;
  for (int w = w0; w < words; ++w) {
    st[0][w] = Ri[w] & Rj[w];
    n0 += __popcll(st[0][w]);
  }
  if (n0 < d) return 0;
  pos[0] = j + 1;
  int top = 0;
  unsigned long long total = 0;
  const int nbits = words * 64;
  while (top >= 0) {
    // next member x >= pos[top] of st[top]
    int x = -1;
    for (int b = pos[top]; b < nbits;) {
      const unsigned long long word = st[top][b >> 6] >> (b & 63);
      if (word) {
        x = b + __ffsll(word) - 1;
        break;
      }
      b = (b | 63) + 1;
    }
    if (x < 0) {
      --top;
      continue;
    }
    pos[top] = x + 1;
    const unsigned long long* Rx = U + (size_t)x * words;
    const int wx = (x + 1) >> 6;
    const int left = d - 1 - top;  // members still to choose after x
    if (left == 1) {
      for (int w = wx; w < words; ++w) total += __popcll(st[top][w] & Rx[w]);
    } else {
      int c = 0;
      for (int w = wx; w < words; ++w) {
        st[top + 1][w] = st[top][w] & Rx[w];
        c += __popcll(st[top + 1][w]);
      }
      if (c >= left) {
        ++top;
        pos[top] = x + 1;
      }
    }
  }
  return total;
}

// Edges whose C0 = N+(u) ∩ N+(v) holds kMaskMax < |C0| <= kDenseMax members, a CTA per
// edge.  C0 goes to shared memory (sorted by id, as N+(u) is) and the graph induced on it
// to bitmap rows: row i = the members above i adjacent to C0[i] (each oriented edge
// x -> y inside C0 found by a binary search of y in C0, recorded at the lower index of the
// two).  A (k-2)-clique of C0 is then counted once, from its two lowest members i < j:
// the CTA deals the adjacent pairs (i, j) over its threads by a prefix sum of the row
// popcounts, and each thread counts the (k-4)-cliques of row i AND row j with AND / popc
// over 64-member words.  The pairs, not the rows, are the unit, so a dense core's few
// heavy rows are spread over every thread.
constexpr int kDenseRows = kDenseMax / kDenseThreads;  // rows a thread sums in the row scan
static_assert(kDenseRows * kDenseThreads == kDenseMax, "the row scan covers kDenseMax rows");
__global__ void __launch_bounds__(kDenseThreads) kcl_dense_kernel(const int64_t* off, const int32_t* cols,
                                                                  const int32_t* esrc, const unsigned long long* dense,
                                                                  int k, int cmax, unsigned long long* next,
                                                                  unsigned long long* out) {
  extern __shared__ unsigned long long dsm[];  // rows: cmax * words
  __shared__ int32_t C[kDenseMax];
  __shared__ int pre[kDenseMax + 1];
  __shared__ int wcount[kDenseThreads / 32];
  __shared__ int csize;
  __shared__ unsigned long long item;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = kDenseThreads / 32;
  const unsigned long long nitems = dense[0];
  unsigned long long cnt = 0, bytes = 0;
  for (;;) {
    if (threadIdx.x == 0) item = atomicAdd(next, 1ull);
    __syncthreads();
    const unsigned long long it = item;
    if (it >= nitems) break;
    const int64_t e = (int64_t)dense[1 + it];
    const int32_t u = esrc[e], v = cols[e];
    const int64_t ub = off[u], ud = off[u + 1] - ub, vb = off[v], vd = off[v + 1] - vb;
    if (threadIdx.x == 0) {
      csize = 0;
      bytes += 4ull * (unsigned long long)vd;
    }
    __syncthreads();
    // C0 in the order of N+(u): block-wide compaction of the hits, chunk by chunk
    for (int64_t base = 0; base < ud; base += kDenseThreads) {
      const int64_t j = base + threadIdx.x;
      const int32_t x = j < ud ? cols[ub + j] : 0;
      const bool hit = j < ud && kc_has(cols + vb, vd, x);
      const unsigned b = __ballot_sync(0xffffffffu, hit);
      if (lane == 0) wcount[w] = __popc(b);
      __syncthreads();
      int before = csize;
      for (int q = 0; q < w; ++q) before += wcount[q];
      if (hit) C[before + __popc(b & ((1u << lane) - 1))] = x;
      __syncthreads();
      if (threadIdx.x == 0) {
        int t = csize;
        for (int q = 0; q < nw; ++q) t += wcount[q];
        csize = t;
      }
      __syncthreads();
    }
    const int c = csize;
    const int words = (c + 63) >> 6;
    for (int t = threadIdx.x; t < c * words; t += kDenseThreads) dsm[t] = 0ull;
    __syncthreads();
    // the edges inside C0: a warp per member x = C[i], lanes over N+(x)
    for (int i = w; i < c; i += nw) {
      const int64_t xb = off[C[i]], xd = off[C[i] + 1] - xb;
      if (lane == 0) bytes += 4ull * (unsigned long long)xd;
      for (int64_t j = lane; j < xd; j += 32) {
        const int32_t y = cols[xb + j];
        int lo = 0, hi = c;  // y's position in C, if any
        while (lo < hi) {
          const int mid = (lo + hi) >> 1;
          if (C[mid] < y) lo = mid + 1; else hi = mid;
        }
        if (lo < c && C[lo] == y) {
          const int a = min(i, lo), z = max(i, lo);
          atomicOr(&dsm[(size_t)a * words + (z >> 6)], 1ull << (z & 63));
        }
      }
    }
    __syncthreads();
    // pre[i] = adjacent pairs in rows below i: kDenseRows rows a thread, a warp scan, warp sums
    int rc[kDenseRows], mine = 0;
#pragma unroll
    for (int q = 0; q < kDenseRows; ++q) {
      const int i = kDenseRows * threadIdx.x + q;
      rc[q] = 0;
      if (i < c)
        for (int x = (i + 1) >> 6; x < words; ++x) rc[q] += __popcll(dsm[(size_t)i * words + x]);
      mine += rc[q];
    }
    int incl = mine;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += y;
    }
    if (lane == 31) wcount[w] = incl;
    __syncthreads();
    int run = incl - mine;
    for (int q = 0; q < w; ++q) run += wcount[q];
#pragma unroll
    for (int q = 0; q < kDenseRows; ++q) {
      const int i = kDenseRows * threadIdx.x + q;
      if (i < c) pre[i] = run;
      run += rc[q];
    }
    if (threadIdx.x == kDenseThreads - 1) pre[c] = run;  // every pair
    __syncthreads();
    const int npairs = pre[c];
    for (int p = threadIdx.x; p < npairs; p += kDenseThreads) {
      // row i: the last with pre[i] <= p (pre[c] > p); j = its (p - pre[i])-th member
      int lo = 0, hi = c;
      while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (pre[mid] <= p) lo = mid; else hi = mid;
      }
      const int i = lo;
      const unsigned long long* Ri = dsm + (size_t)i * words;
      int r = p - pre[i];
      int x = (i + 1) >> 6;
      for (;; ++x) {
        const int pc = __popcll(Ri[x]);
        if (r < pc) break;
        r -= pc;
      }
      const int j = x * 64 + select_bit(Ri[x], r);
      cnt += pair_cliques(dsm, words, i, j, k - 4);
    }
    __syncthreads();
  }
  for (int o = 16; o > 0; o >>= 1) {
    cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
    bytes += __shfl_xor_sync(0xffffffffu, bytes, o);
  }
  if (lane == 0) {
    if (cnt) atomicAdd(out, cnt);
    if (bytes) atomicAdd(out + 1, bytes);
  }
}

}  // namespace

}  // namespace atc

using namespace atc;

// k-cliques whose first two vertices (in orientation order) form an edge of [e0, e1).
static atc_status kcl_window(const atc_csr* csr, uint32_t k, int64_t e0, int64_t e1, uint64_t* count, atc_stats* stats,
                             cudaStream_t s, bool allow_dense = true) {
  *count = 0;
  unsigned long long h[2] = {0, 0};
  EventTimer tm;
  int launches = 0;
  if (e1 > e0) {
    CsrPriv* pv = static_cast<CsrPriv*>(csr->priv);
    int cap = std::max(csr->max_outdeg, 1);
    int levels = (int)k - 2;
    int bps = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, kcl_kernel, kKcWarps * 32, 0);
    if (bps < 1) bps = 1;
    int64_t grid = (int64_t)sm_count() * bps;
    // keep the scratch within 4 GiB
    int64_t per_warp = (int64_t)levels * cap * 4;
    while (grid > sm_count() && grid * kKcWarps * per_warp > (4ll << 30)) grid /= 2;
    DevBuf<int32_t> scratch;
    ATC_TRY(scratch.alloc((size_t)grid * kKcWarps * levels * cap, s));
    // edges with mid-sized C0 go to the dense kernel from k = 5 on (at k = 4 the count is
    // one intersection per member of C0, which the warp path does as fast: R-MAT scale 20
    // took 562 ms dense, 422 ms without)
    const bool use_dense = allow_dense && k >= 5 && cap > kMaskMax;
    DevBuf<unsigned long long> dense;
    if (use_dense) ATC_TRY(dense.alloc((size_t)csr->m + 2, s));
    tm.start(s);
    ATC_CK(cudaMemsetAsync(pv->counter, 0, 2 * sizeof(unsigned long long), s));
    if (use_dense) ATC_CK(cudaMemsetAsync(dense.p, 0, 2 * sizeof(unsigned long long), s));
    kcl_kernel<<<(unsigned)grid, kKcWarps * 32, 0, s>>>(csr->offsets, csr->cols, pv->esrc, e0, e1, (int)k, cap,
                                                         scratch.p, use_dense ? dense.p + 1 : nullptr, pv->counter);
    ATC_CK(cudaGetLastError());
    launches = 1;
    if (use_dense) {
      // rows for the largest C0 this graph can have
      const int cmax = std::min(cap, kDenseMax);
      const size_t smem = sizeof(unsigned long long) * (size_t)cmax * ((cmax + 63) / 64);
      ATC_CK(cudaFuncSetAttribute((const void*)kcl_dense_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)smem));
      int dbps = 0;
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&dbps, kcl_dense_kernel, kDenseThreads, smem);
      if (dbps < 1) dbps = 1;
      kcl_dense_kernel<<<(unsigned)(sm_count() * dbps), kDenseThreads, smem, s>>>(
          csr->offsets, csr->cols, pv->esrc, dense.p + 1, (int)k, cmax, dense.p, pv->counter);
      ATC_CK(cudaGetLastError());
      launches = 2;
    }
    tm.stop(s);
    ATC_CK(cudaMemcpyAsync(h, pv->counter, sizeof(h), cudaMemcpyDeviceToHost, s));
    ATC_CK(cudaStreamSynchronize(s));
    *count = h[0];
  }
  if (stats) {
    stats->kernel_ms = e1 > e0 ? tm.ms() : 0.0f;
    stats->total_ms = stats->kernel_ms;
    stats->alg_bytes = h[1];
    stats->wedges = (uint64_t)csr->wedges;
    stats->alg_bytes_min = h[1];
    stats->kernel_used = 0;
    stats->launches = launches;
  }
  return ATC_OK;
}

extern "C" atc_status atc_kcl(const atc_csr* csr, uint32_t k, uint64_t* count, atc_stats* stats, atc_stream st) try {
  ATC_CHECK_ARG(csr != nullptr && count != nullptr, "NULL argument");
  ATC_CHECK_ARG(k >= 3 && k <= (uint32_t)kMaxK, "k must be in [3, 16]");
  ATC_CHECK_ARG(csr->priv != nullptr || csr->m == 0, "csr was not built by atc_pretc");
  Phase ph("kcl", as_stream(st));
  return kcl_window(csr, k, 0, csr->m, count, stats, as_stream(st));
} ATC_CATCH

extern "C" atc_status atc_kcl_part(const atc_csr* csr, uint32_t k, uint32_t part, uint32_t nparts, uint64_t* count,
                                   int64_t* edge_range, atc_stats* stats, atc_stream st) try {
  return atc_kcl_part_tuned(csr, k, nullptr, part, nparts, count, edge_range, stats, st);
} ATC_CATCH

extern "C" atc_status atc_kcl_part_tuned(const atc_csr* csr, uint32_t k, const atc_tuning* tuning, uint32_t part,
                                         uint32_t nparts, uint64_t* count, int64_t* edge_range, atc_stats* stats,
                                         atc_stream st) try {
  ATC_CHECK_ARG(csr != nullptr && count != nullptr, "NULL argument");
  ATC_CHECK_ARG(k >= 3 && k <= (uint32_t)kMaxK, "k must be in [3, 16]");
  ATC_CHECK_ARG(csr->priv != nullptr || csr->m == 0, "csr was not built by atc_pretc");
  ATC_CHECK_ARG(nparts >= 1 && part < nparts, "part must be in [0, nparts)");
  cudaStream_t s = as_stream(st);
  *count = 0;
  int64_t b[2];
  ATC_TRY(part_edge_range(csr, part, nparts, b, s));
  if (edge_range) {
    edge_range[0] = b[0];
    edge_range[1] = b[1];
  }
  ATC_CHECK_ARG(!tuning || tuning->kcl_dense == 0 || tuning->kcl_dense == -1, "kcl_dense must be 0 or -1");
  Phase ph("kcl", s);
  return kcl_window(csr, k, b[0], b[1], count, stats, s, !(tuning && tuning->kcl_dense == -1));
} ATC_CATCH
