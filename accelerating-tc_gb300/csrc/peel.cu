// A-direction peel on the GPU, level-synchronous.
//
// The reference peels serially (edge_directing/A-direction-seri.cpp:35-153): each outer
// step admits every unpeeled vertex whose runtime degree rt (twice its remaining degree)
// is <= a float threshold, then repeats waves in which every frontier vertex lowers rt of
// each unpeeled neighbour by 2 and a neighbour that reaches the threshold joins the next
// wave with the next priority.  Which vertices cross in a wave depends only on the set
// of frontier vertices (rt falls by exactly 2 per frontier neighbour until it crosses),
// never on the order the serial loop visits them, and the rt of already-peeled vertices
// (changed by the tie rule at :99-103) never feeds back into a priority.  A wave is
// therefore one parallel pass: atomicSub(rt[y], 2) on each unpeeled neighbour; the one
// subtraction that takes rt from above the threshold to at or below it admits y.  The
// float threshold arithmetic runs on the host exactly as in the reference (:37, :77, :127).
#include <climits>
#include <vector>

#include "internal.cuh"

namespace atc {

namespace {

// Symmetric adjacency from the sorted keys (a < b).  Keys of one smaller endpoint are
// contiguous, so a warp reserves each run's slots with one atomic (the loop is padded to
// whole warps for __match_any_sync); the larger endpoints are scattered one by one.
__global__ void sym_scatter_kernel(const uint64_t* keys, int64_t m, int B, unsigned long long* cur, int32_t* adj) {
  const uint64_t mask = (1ull << B) - 1;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const int64_t m_pad = (m + 31) & ~31ll;
  const int lane = threadIdx.x & 31;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m_pad; i += stride) {
    int64_t a = -1;
    int32_t b = 0;
    if (i < m) {
      const uint64_t k = keys[i];
      a = (int64_t)(k >> B);
      b = (int32_t)(k & mask);
      adj[atomicAdd(&cur[b], 1ull)] = (int32_t)a;
    }
    const unsigned same = __match_any_sync(0xffffffffu, a);
    const int lead = __ffs(same) - 1;
    unsigned long long base = 0;
    if (a >= 0 && lane == lead) base = atomicAdd(&cur[a], (unsigned long long)__popc(same));
    base = __shfl_sync(0xffffffffu, base, lead);
    if (a >= 0) adj[base + __popc(same & ((1u << lane) - 1))] = b;
  }
}

__global__ void peel_init_kernel(const int32_t* deg, int64_t n, int32_t* rt, int32_t* prio) {
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n; v += stride) {
    rt[v] = 2 * deg[v];
    prio[v] = -1;
  }
}

// Outer step (A-direction-seri.cpp:83-89): admit every unpeeled v with rt[v] <= thr.
__global__ void peel_scan_kernel(const int32_t* rt, int32_t* prio, int64_t n, float thr, int32_t p,
                                 int32_t* frontier, int* count) {
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n; v += stride) {
    if (prio[v] == -1 && (float)rt[v] <= thr) {
      prio[v] = p;
      frontier[atomicAdd(count, 1)] = (int32_t)v;
    }
  }
}

// One wave (A-direction-seri.cpp:92-121): a warp per frontier vertex, lanes over its
// neighbours.  prio[y] only ever moves from -1 to a value, so a stale -1 read costs at
// most a harmless extra decrement of an already-admitted vertex.
__global__ void peel_wave_kernel(const int32_t* frontier, int nf, const int64_t* off, const int32_t* adj,
                                 int32_t* rt, int32_t* prio, float thr, int32_t p, int32_t* next, int* count) {
  int lane = threadIdx.x & 31;
  int warps = (gridDim.x * blockDim.x) >> 5;
  for (int f = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; f < nf; f += warps) {
    int32_t x = frontier[f];
    int64_t b = off[x], e = off[x + 1];
    for (int64_t j = b + lane; j < e; j += 32) {
      int32_t y = adj[j];
      if (*(volatile int32_t*)&prio[y] != -1) continue;
      int32_t old = atomicSub(&rt[y], 2);
      if ((float)old > thr && (float)(old - 2) <= thr) {
        prio[y] = p;
        next[atomicAdd(count, 1)] = y;
      }
    }
  }
}

}  // namespace

atc_status peel_priorities(const SimpleEdges& e, const int32_t* deg, int32_t* prio, int* waves_out, cudaStream_t s) {
  Phase ph("peel", s);
  int64_t n = e.n_in, m = e.m;
  *waves_out = 0;
  if (n == 0) return ATC_OK;
  // symmetric adjacency (lists unsorted: the peel only needs neighbour sets)
  DevBuf<int64_t> off;
  DevBuf<unsigned long long> cur;
  DevBuf<int32_t> adj, rt, fa, fb;
  DevBuf<int> cnt;
  ATC_TRY(off.alloc(n + 1, s));
  ATC_TRY(exclusive_scan_i32_to_i64(deg, off.p, n, s));
  int64_t total = 2 * m;
  ATC_CK(cudaMemcpyAsync(off.p + n, &total, sizeof(total), cudaMemcpyHostToDevice, s));
  ATC_TRY(cur.alloc(n, s));
  ATC_CK(cudaMemcpyAsync(cur.p, off.p, sizeof(int64_t) * n, cudaMemcpyDeviceToDevice, s));
  ATC_TRY(adj.alloc(total, s));
  if (m) sym_scatter_kernel<<<grid_for(m, 256), 256, 0, s>>>(e.keys.p, m, e.bits, cur.p, adj.p);
  ATC_CK(cudaGetLastError());
  cur.release();
  ATC_TRY(rt.alloc(n, s));
  ATC_TRY(fa.alloc(n, s));
  ATC_TRY(fb.alloc(n, s));
  ATC_TRY(cnt.alloc(1, s));
  peel_init_kernel<<<grid_for(n, 256), 256, 0, s>>>(deg, n, rt.p, prio);
  ATC_CK(cudaGetLastError());

  // Host-side threshold arithmetic, as A-direction-seri.cpp:37,77,127 (edgeNum = 2m as
  // unsigned, nodeNum = max id + 1 as int).
  unsigned edgeNum = (unsigned)total;
  int nodeNum = (int)n;
  float threshold = ((float)edgeNum) / nodeNum + 1;
  int threshold_old = threshold;
  int32_t p = 0;
  int64_t peeled = 0;
  int waves = 0;
  int32_t* F = fa.p;
  int32_t* N = fb.p;
  int hcnt = 0;
  for (;;) {
    ATC_CK(cudaMemsetAsync(cnt.p, 0, sizeof(int), s));
    peel_scan_kernel<<<grid_for(n, 256), 256, 0, s>>>(rt.p, prio, n, threshold, p, F, cnt.p);
    ATC_CK(cudaGetLastError());
    ATC_CK(cudaMemcpyAsync(&hcnt, cnt.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    ATC_CK(cudaStreamSynchronize(s));
    int nf = hcnt;
    peeled += nf;
    ++p;
    while (nf > 0) {
      ATC_CK(cudaMemsetAsync(cnt.p, 0, sizeof(int), s));
      peel_wave_kernel<<<grid_for((int64_t)nf * 32, 256), 256, 0, s>>>(F, nf, off.p, adj.p, rt.p, prio, threshold, p,
                                                                      N, cnt.p);
      ATC_CK(cudaGetLastError());
      ATC_CK(cudaMemcpyAsync(&hcnt, cnt.p, sizeof(int), cudaMemcpyDeviceToHost, s));
      ATC_CK(cudaStreamSynchronize(s));
      std::swap(F, N);
      nf = hcnt;
      peeled += nf;
      ++p;
      ++waves;
    }
    if (peeled >= n) break;
    float grown = threshold + threshold_old;
    if (!(grown > threshold)) {
      // float addition no longer moves the threshold: the serial reference would loop
      // forever here (runtime degrees above 2^24 are needed to get this far)
      set_error("A-direction threshold stopped growing at %g with %lld vertices unpeeled", (double)threshold,
                (long long)(n - peeled));
      return ATC_ERR_UNSUPPORTED;
    }
    threshold = grown;
  }
  *waves_out = waves;
  return ATC_OK;
}

// ---- Bisson's A-direction relabelling (Bisson/A-direction.cpp:43-163, 283-292) ----------
// The program peels serially over a doubled adjacency list and numbers the outer selection
// and every wave with one priority each (:91-126); the new ids sort the vertices by
// (priority, degreeRecord, id) and reverse the rank (:283-292).  degreeRecord is written at
// the selected vertex in the outer scan but at the frontier POSITION in the waves (:118),
// so it depends on the order in which the serial loop admits vertices.  That order is
// rebuilt here wave by wave, in parallel:
//   - the list of x (allEdges, :69-80) holds N(x) ∩ [0, x), then N(x), then N(x) ∩ (x, n),
//     each ascending, so a neighbour y sits at two known entries of it (first, second);
//   - an unpeeled y loses 1 per entry processed and is admitted at its k-th loss,
//     k = rt(y) - floor(threshold) (rt > threshold while unpeeled, so the loss that crosses
//     leaves rt exactly at the floor): that is entry (k odd ? first : second) of its
//     ceil(k/2)-th frontier neighbour in frontier order;
//   - the next frontier lists the admitted vertices by (position of that neighbour, entry);
//   - every admission writes degreeRecord[position] = floor(threshold); writes happen in
//     program order across waves, so the last one wins as in the serial program.
// Pairs (y, position of an adjacent frontier vertex) are radix-sorted per wave to find
// each y's ceil(k/2)-th frontier neighbour.
namespace {

__global__ void both_dir_keys_kernel(const uint64_t* keys, int64_t m, int B, uint64_t* out) {
  const uint64_t mask = (1ull << B) - 1;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m; i += stride) {
    const uint64_t k = keys[i], a = k >> B, b = k & mask;
    out[2 * i] = (a << B) | b;
    out[2 * i + 1] = (b << B) | a;
  }
}

// adj[j] = the low half of the sorted both-direction keys; nlow[x] = |N(x) ∩ [0, x)|.
__global__ void sorted_adj_kernel(const uint64_t* sk, int64_t m2, int B, int32_t* adj) {
  const uint64_t mask = (1ull << B) - 1;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m2; i += stride)
    adj[i] = (int32_t)(sk[i] & mask);
}

__global__ void nlow_kernel(const int64_t* off, const int32_t* adj, int64_t n, int32_t* nlow) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t x = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; x < n; x += stride) {
    int64_t lo = off[x], hi = off[x + 1];
    const int64_t b = lo;
    while (lo < hi) {
      const int64_t mid = (lo + hi) >> 1;
      if (adj[mid] < (int32_t)x) lo = mid + 1; else hi = mid;
    }
    nlow[x] = (int32_t)(lo - b);
  }
}

__global__ void bis_init_kernel(const int32_t* deg, int64_t n, int32_t* rt, int32_t* prio, int32_t* drec) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n; v += stride) {
    rt[v] = 2 * deg[v];
    prio[v] = -1;
    drec[v] = 0;
  }
}

// Outer selection (:89-98), in id order: flag, then (after a scan) place.
__global__ void bis_flag_kernel(const int32_t* rt, const int32_t* prio, int64_t n, float thr, int32_t* flag) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n; v += stride)
    flag[v] = prio[v] == -1 && (float)rt[v] <= thr;
}

__global__ void bis_place_kernel(const int32_t* flag, const int64_t* pos, const int32_t* rt, int64_t n, int32_t P,
                                 int32_t* prio, int32_t* drec, int32_t* F) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n; v += stride)
    if (flag[v]) {
      F[pos[v]] = (int32_t)v;
      prio[v] = P;
      drec[v] = rt[v];
    }
}

__global__ void bis_fdeg_kernel(const int32_t* F, int64_t nf, const int32_t* deg, int32_t* fd) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < nf; p += stride) fd[p] = deg[F[p]];
}

// (y << 32 | position, rank of y in N(x)) for every unpeeled neighbour y of frontier
// position p; peeled neighbours get the all-ones key, which sorts last.
__global__ void bis_emit_kernel(const int32_t* F, int64_t nf, const int64_t* fstart, const int64_t* off,
                                const int32_t* adj, const int32_t* prio, uint64_t* keys, int32_t* vals) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t p = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; p < nf; p += warps) {
    const int32_t x = F[p];
    const int64_t b = off[x], d = off[x + 1] - b, at = fstart[p];
    for (int64_t j = lane; j < d; j += 32) {
      const int32_t y = adj[b + j];
      keys[at + j] = prio[y] == -1 ? (((uint64_t)(uint32_t)y << 32) | (uint64_t)p) : ~0ull;
      vals[at + j] = (int32_t)j;
    }
  }
}

// One thread per segment start of the sorted pairs: admit y at its k-th loss, or take
// away 2 per adjacent frontier vertex.  cand gets (position << 32 | entry, y).
__global__ void bis_admit_kernel(const uint64_t* keys, const int32_t* vals, int64_t total, const int32_t* F,
                                 const int32_t* deg, const int32_t* nlow, int32_t T, int32_t P, int32_t* rt,
                                 int32_t* prio, int32_t* drec, uint64_t* ckeys, int32_t* cvals, int* ccount) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += stride) {
    const uint64_t key = keys[i];
    if (key == ~0ull) continue;
    const uint32_t y = (uint32_t)(key >> 32);
    if (i > 0 && (uint32_t)(keys[i - 1] >> 32) == y) continue;  // not a segment start
    int64_t lo = i + 1, hi = total;  // first pair of another vertex (the sentinels too)
    while (lo < hi) {
      const int64_t mid = (lo + hi) >> 1;
      if (keys[mid] != ~0ull && (uint32_t)(keys[mid] >> 32) == y) lo = mid + 1; else hi = mid;
    }
    const int64_t c = lo - i;
    const int32_t k = rt[y] - T;  // >= 1
    if (2 * c >= (int64_t)k) {
      const int64_t cross = i + (k + 1) / 2 - 1;
      const uint32_t p = (uint32_t)(keys[cross] & 0xffffffffull);
      const int32_t r = vals[cross];
      const int32_t x = F[p];
      const int32_t nl = nlow[x];
      const int32_t entry = (k & 1) ? ((int32_t)y < x ? r : nl + r) : ((int32_t)y < x ? nl + r : deg[x] + r);
      prio[y] = P;
      rt[y] = T;
      drec[p] = T;  // :118 writes at the frontier position
      const int at = atomicAdd(ccount, 1);
      ckeys[at] = ((uint64_t)p << 32) | (uint32_t)entry;
      cvals[at] = (int32_t)y;
    } else {
      rt[y] -= (int32_t)(2 * c);
    }
  }
}

__global__ void bis_rank_keys_kernel(const int32_t* prio, const int32_t* drec, int64_t n, uint64_t* keys, int32_t* ids) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n; v += stride) {
    keys[v] = ((uint64_t)(uint32_t)prio[v] << 32) | (uint32_t)drec[v];
    ids[v] = (int32_t)v;
  }
}

__global__ void bis_lookup_kernel(const int32_t* ids, int64_t n, int32_t* lookup) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += stride)
    lookup[ids[i]] = (int32_t)(n - 1 - i);
}

}  // namespace

atc_status bisson_adirection_lookup(const SimpleEdges& e, const int32_t* deg, int32_t* lookup, cudaStream_t s) {
  Phase ph("bisson_adirection", s);
  const int64_t n = e.n_in, m = e.m, m2 = 2 * m;
  if (n == 0) return ATC_OK;
  DevBuf<int64_t> off, fstart, pos;
  DevBuf<int32_t> adj, nlow, rt, prio, drec, fa, fb, flag, fd, va, vb, cva, cvb;
  DevBuf<uint64_t> ka, kb, cka, ckb;
  DevBuf<int> cnt;
  // sorted symmetric adjacency
  ATC_TRY(off.alloc(n + 1, s));
  ATC_TRY(exclusive_scan_i32_to_i64(deg, off.p, n, s));
  ATC_CK(cudaMemcpyAsync(off.p + n, &m2, sizeof(m2), cudaMemcpyHostToDevice, s));
  // ka/kb/va/vb: the both-direction keys, each wave's (y, position) pairs (at most 2m) and
  // the final (priority, degreeRecord) keys of all n vertices
  const int64_t cap = std::max(m2, n) + 1;
  ATC_TRY(adj.alloc(m2 + 1, s));
  ATC_TRY(ka.alloc(cap, s));
  ATC_TRY(kb.alloc(cap, s));
  if (m) {
    both_dir_keys_kernel<<<grid_for(m, 256), 256, 0, s>>>(e.keys.p, m, e.bits, ka.p);
    ATC_CK(cudaGetLastError());
    uint64_t* k0 = ka.p;
    uint64_t* k1 = kb.p;
    ATC_TRY(sort_keys_u64(k0, k1, m2, 0, 2 * e.bits, s));
    sorted_adj_kernel<<<grid_for(m2, 256), 256, 0, s>>>(k0, m2, e.bits, adj.p);
    ATC_CK(cudaGetLastError());
  }
  ATC_TRY(nlow.alloc(n, s));
  nlow_kernel<<<grid_for(n, 256), 256, 0, s>>>(off.p, adj.p, n, nlow.p);
  ATC_TRY(rt.alloc(n, s));
  ATC_TRY(prio.alloc(n, s));
  ATC_TRY(drec.alloc(n, s));
  bis_init_kernel<<<grid_for(n, 256), 256, 0, s>>>(deg, n, rt.p, prio.p, drec.p);
  ATC_CK(cudaGetLastError());
  ATC_TRY(fa.alloc(n + 1, s));
  ATC_TRY(fb.alloc(n + 1, s));
  ATC_TRY(flag.alloc(n + 1, s));
  ATC_TRY(pos.alloc(n + 1, s));
  ATC_TRY(fd.alloc(n + 1, s));
  ATC_TRY(fstart.alloc(n + 1, s));
  ATC_TRY(va.alloc(cap, s));
  ATC_TRY(vb.alloc(cap, s));
  ATC_TRY(cka.alloc(n + 1, s));
  ATC_TRY(ckb.alloc(n + 1, s));
  ATC_TRY(cva.alloc(n + 1, s));
  ATC_TRY(cvb.alloc(n + 1, s));
  ATC_TRY(cnt.alloc(1, s));

  // threshold arithmetic of :45, :83, :138 on the host (edgeNum = 2m, nodeNum = max id + 1)
  const unsigned edgeNum = (unsigned)m2;
  const int nodeNum = (int)n;
  float threshold = ((float)edgeNum) / nodeNum + 1;
  const int threshold_old = threshold;
  int32_t P = 0;
  int64_t peeled = 0;
  int32_t* F = fa.p;
  int32_t* N = fb.p;
  for (;;) {
    // outer selection in id order
    ATC_CK(cudaMemsetAsync(flag.p + n, 0, sizeof(int32_t), s));
    bis_flag_kernel<<<grid_for(n, 256), 256, 0, s>>>(rt.p, prio.p, n, threshold, flag.p);
    ATC_CK(cudaGetLastError());
    ATC_TRY(exclusive_scan_i32_to_i64(flag.p, pos.p, n + 1, s));
    bis_place_kernel<<<grid_for(n, 256), 256, 0, s>>>(flag.p, pos.p, rt.p, n, P, prio.p, drec.p, F);
    ATC_CK(cudaGetLastError());
    int64_t nf = 0;
    ATC_CK(cudaMemcpyAsync(&nf, pos.p + n, sizeof(nf), cudaMemcpyDeviceToHost, s));
    ATC_CK(cudaStreamSynchronize(s));
    peeled += nf;
    ++P;
    const int32_t T = (int32_t)floorf(threshold);
    while (nf > 0) {
      // pairs (y, position) of the unpeeled neighbours of the frontier
      bis_fdeg_kernel<<<grid_for(nf, 256), 256, 0, s>>>(F, nf, deg, fd.p);
      ATC_CK(cudaMemsetAsync(fd.p + nf, 0, sizeof(int32_t), s));
      ATC_CK(cudaGetLastError());
      ATC_TRY(exclusive_scan_i32_to_i64(fd.p, fstart.p, nf + 1, s));
      int64_t total = 0;
      ATC_CK(cudaMemcpyAsync(&total, fstart.p + nf, sizeof(total), cudaMemcpyDeviceToHost, s));
      ATC_CK(cudaStreamSynchronize(s));
      ATC_CK(cudaMemsetAsync(cnt.p, 0, sizeof(int), s));
      if (total > 0) {
        bis_emit_kernel<<<grid_for(nf * 32, 256), 256, 0, s>>>(F, nf, fstart.p, off.p, adj.p, prio.p, ka.p, va.p);
        ATC_CK(cudaGetLastError());
        uint64_t* k0 = ka.p;
        uint64_t* k1 = kb.p;
        int32_t* v0 = va.p;
        int32_t* v1 = vb.p;
        ATC_TRY(sort_pairs_u64_i32(k0, k1, v0, v1, total, 0, 64, s));
        bis_admit_kernel<<<grid_for(total, 256), 256, 0, s>>>(k0, v0, total, F, deg, nlow.p, T, P, rt.p, prio.p,
                                                              drec.p, cka.p, cva.p, cnt.p);
        ATC_CK(cudaGetLastError());
      }
      int hc = 0;
      ATC_CK(cudaMemcpyAsync(&hc, cnt.p, sizeof(int), cudaMemcpyDeviceToHost, s));
      ATC_CK(cudaStreamSynchronize(s));
      // the next frontier in admission order
      uint64_t* c0 = cka.p;
      uint64_t* c1 = ckb.p;
      int32_t* w0 = cva.p;
      int32_t* w1 = cvb.p;
      ATC_TRY(sort_pairs_u64_i32(c0, c1, w0, w1, (size_t)hc, 0, 64, s));
      if (hc) ATC_CK(cudaMemcpyAsync(N, w0, sizeof(int32_t) * hc, cudaMemcpyDeviceToDevice, s));
      std::swap(F, N);
      nf = hc;
      peeled += nf;
      ++P;
    }
    if (peeled >= n) break;
    const float grown = threshold + threshold_old;
    if (!(grown > threshold)) {
      set_error("Bisson A-direction threshold stopped growing at %g with %lld vertices unpeeled", (double)threshold,
                (long long)(n - peeled));
      return ATC_ERR_UNSUPPORTED;
    }
    threshold = grown;
  }
  // new id = nodeNum - 1 - rank of (priority, degreeRecord, id)
  {
    uint64_t* k0 = ka.p;
    uint64_t* k1 = kb.p;
    int32_t* v0 = va.p;
    int32_t* v1 = vb.p;
    bis_rank_keys_kernel<<<grid_for(n, 256), 256, 0, s>>>(prio.p, drec.p, n, k0, v0);
    ATC_CK(cudaGetLastError());
    ATC_TRY(sort_pairs_u64_i32(k0, k1, v0, v1, n, 0, 64, s));
    bis_lookup_kernel<<<grid_for(n, 256), 256, 0, s>>>(v0, n, lookup);
    ATC_CK(cudaGetLastError());
  }
  ATC_CK(cudaStreamSynchronize(s));
  return ATC_OK;
}

// ---- k-core numbers (for the k-core direction, edge_directing/kcore_direction.cpp:91-146) ----
// Level-synchronous peeling: at level k every vertex whose remaining degree is <= k
// leaves with core number k, each leaving vertex lowers its remaining neighbours by 1,
// and the level repeats until nothing more leaves; k then jumps to the smallest
// remaining degree.  Which vertices leave at a level does not depend on the order, so
// the core numbers equal the sequential Batagelj-Zaversnik result.  (The reference tool
// counts degrees over the first node_num edges only, :35-38; this uses the true degrees.)
namespace {

__global__ void core_scan_kernel(const int32_t* rt, int32_t* core, int64_t n, int32_t k, int32_t* frontier, int* count) {
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n; v += stride)
    if (core[v] == -1 && rt[v] <= k) {
      core[v] = k;
      frontier[atomicAdd(count, 1)] = (int32_t)v;
    }
}

__global__ void core_wave_kernel(const int32_t* frontier, int nf, const int64_t* off, const int32_t* adj, int32_t* rt,
                                 int32_t* core, int32_t k, int32_t* next, int* count) {
  int lane = threadIdx.x & 31;
  int warps = (gridDim.x * blockDim.x) >> 5;
  for (int f = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; f < nf; f += warps) {
    int32_t x = frontier[f];
    for (int64_t j = off[x] + lane; j < off[x + 1]; j += 32) {
      int32_t y = adj[j];
      if (*(volatile int32_t*)&core[y] != -1) continue;
      int32_t old = atomicSub(&rt[y], 1);
      if (old == k + 1) {  // the one decrement that takes rt from k+1 to k
        core[y] = k;
        next[atomicAdd(count, 1)] = y;
      }
    }
  }
}

__global__ void core_min_kernel(const int32_t* rt, const int32_t* core, int64_t n, int* mn) {
  int best = INT_MAX;
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n; v += stride)
    if (core[v] == -1) best = min(best, rt[v]);
  for (int o = 16; o > 0; o >>= 1) best = min(best, __shfl_xor_sync(0xffffffffu, best, o));
  if ((threadIdx.x & 31) == 0) atomicMin(mn, best);
}

}  // namespace

atc_status core_numbers(const SimpleEdges& e, const int32_t* deg, int32_t* core, cudaStream_t s) {
  const int64_t n = e.n_in, m = e.m;
  if (n == 0) return ATC_OK;
  DevBuf<int64_t> off;
  DevBuf<unsigned long long> cur;
  DevBuf<int32_t> adj, rt, fa, fb;
  DevBuf<int> cnt;
  ATC_TRY(off.alloc(n + 1, s));
  ATC_TRY(exclusive_scan_i32_to_i64(deg, off.p, n, s));
  int64_t total = 2 * m;
  ATC_CK(cudaMemcpyAsync(off.p + n, &total, sizeof(total), cudaMemcpyHostToDevice, s));
  ATC_TRY(cur.alloc(n, s));
  ATC_CK(cudaMemcpyAsync(cur.p, off.p, sizeof(int64_t) * n, cudaMemcpyDeviceToDevice, s));
  ATC_TRY(adj.alloc(total, s));
  if (m) sym_scatter_kernel<<<grid_for(m, 256), 256, 0, s>>>(e.keys.p, m, e.bits, cur.p, adj.p);
  ATC_CK(cudaGetLastError());
  cur.release();
  ATC_TRY(rt.alloc(n, s));
  ATC_TRY(fa.alloc(n, s));
  ATC_TRY(fb.alloc(n, s));
  ATC_TRY(cnt.alloc(1, s));
  ATC_CK(cudaMemcpyAsync(rt.p, deg, sizeof(int32_t) * n, cudaMemcpyDeviceToDevice, s));
  ATC_CK(cudaMemsetAsync(core, 0xff, sizeof(int32_t) * n, s));
  int32_t k = 0;
  int64_t removed = 0;
  int hcnt = 0;
  int32_t* F = fa.p;
  int32_t* N = fb.p;
  for (;;) {
    ATC_CK(cudaMemsetAsync(cnt.p, 0, sizeof(int), s));
    core_scan_kernel<<<grid_for(n, 256), 256, 0, s>>>(rt.p, core, n, k, F, cnt.p);
    ATC_CK(cudaGetLastError());
    ATC_CK(cudaMemcpyAsync(&hcnt, cnt.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    ATC_CK(cudaStreamSynchronize(s));
    int nf = hcnt;
    removed += nf;
    while (nf > 0) {
      ATC_CK(cudaMemsetAsync(cnt.p, 0, sizeof(int), s));
      core_wave_kernel<<<grid_for((int64_t)nf * 32, 256), 256, 0, s>>>(F, nf, off.p, adj.p, rt.p, core, k, N, cnt.p);
      ATC_CK(cudaGetLastError());
      ATC_CK(cudaMemcpyAsync(&hcnt, cnt.p, sizeof(int), cudaMemcpyDeviceToHost, s));
      ATC_CK(cudaStreamSynchronize(s));
      std::swap(F, N);
      nf = hcnt;
      removed += nf;
    }
    if (removed >= n) break;
    int init = INT_MAX;
    ATC_CK(cudaMemcpyAsync(cnt.p, &init, sizeof(int), cudaMemcpyHostToDevice, s));
    core_min_kernel<<<grid_for(n, 256), 256, 0, s>>>(rt.p, core, n, cnt.p);
    ATC_CK(cudaGetLastError());
    ATC_CK(cudaMemcpyAsync(&hcnt, cnt.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    ATC_CK(cudaStreamSynchronize(s));
    if (hcnt <= k) {  // cannot happen: every remaining degree is above k
      set_error("k-core peel made no progress at level %d", k);
      return ATC_ERR_CUDA;
    }
    k = hcnt;
  }
  return ATC_OK;
}

// ---- approximate parallel peel (edge_directing/A-direction-parallel/peel.cu:130-317) ----
// Frontier-synchronous: a frontier is every unpeeled vertex whose runtime degree (simple
// degree minus peeled neighbours, uint32) is <= a limit; it gets the iteration number as
// its major priority and its runtime degree as minor priority.  The limit starts at
// (uint32)(m / n) and grows by that step when a frontier comes out empty or small
// (peel.cu:239-246, 255); the loop stops at 90 % of the vertices, depth 255 or 50
// iterations (:217), and the vertices left keep flag 0xFFFFFFFF and their simple degree.
// Which vertices join a frontier depends only on the set of the previous frontier, so
// the atomic order inside a pass does not matter.
namespace {

constexpr uint32_t kUnpeeled = 0xFFFFFFFFu;

__global__ void apeel_init_kernel(const int32_t* deg, int64_t n, uint32_t* rd, uint32_t* flags, uint32_t* minor) {
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x) {
    rd[v] = (uint32_t)deg[v];
    minor[v] = (uint32_t)deg[v];
    flags[v] = kUnpeeled;
  }
}

// peel.cu:95-117 (advance + back_nbr_count): every unpeeled neighbour w of a frontier
// vertex loses one runtime degree per frontier neighbour.  The lists are symmetric and
// duplicate-free, so counting from the frontier side gives the same sums.
__global__ void apeel_lower_kernel(const int32_t* frontier, int nf, const int64_t* off, const int32_t* adj,
                                   const uint32_t* flags, uint32_t* rd) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t i = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; i < nf; i += warps) {
    const int32_t u = frontier[i];
    for (int64_t j = off[u] + lane; j < off[u + 1]; j += 32) {
      const int32_t w = adj[j];
      if (flags[w] == kUnpeeled) atomicSub(&rd[w], 1u);
    }
  }
}

// peel.cu:239-262: frontier = {v : rd[v] <= limit} (peeled vertices hold rd = 0xFFFFFFFF);
// each member takes flag `it`, minor = rd, rd = 0xFFFFFFFF.  Counts only when `assign` is 0.
// Whole warps step through the ids together so the ballot covers all 32 lanes.
__global__ void apeel_select_kernel(uint32_t* rd, uint32_t* flags, uint32_t* minor, int64_t n, uint32_t limit,
                                    uint32_t it, int assign, int32_t* frontier, int* count) {
  const int lane = threadIdx.x & 31;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t v0 = blockIdx.x * (int64_t)blockDim.x + threadIdx.x - lane; v0 < n; v0 += stride) {
    const int64_t v = v0 + lane;
    const uint32_t r = v < n ? rd[v] : 0u;
    const bool in = v < n && r <= limit;
    const unsigned ballot = __ballot_sync(0xffffffffu, in);
    if (!ballot) continue;
    int base = 0;
    if (lane == 0) base = atomicAdd(count, __popc(ballot));
    base = __shfl_sync(0xffffffffu, base, 0);
    if (in && assign) {
      frontier[base + __popc(ballot & ((1u << lane) - 1))] = (int32_t)v;
      flags[v] = it;
      minor[v] = r;
      rd[v] = kUnpeeled;
    }
  }
}

}  // namespace

atc_status approx_peel(const SimpleEdges& e, const int32_t* deg, uint32_t* flags, uint32_t* minor, int* iters_out,
                       cudaStream_t s) {
  const int64_t n = e.n_in, m = e.m;
  if (iters_out) *iters_out = 0;
  if (n == 0) return ATC_OK;
  DevBuf<int64_t> off;
  DevBuf<unsigned long long> cur;
  DevBuf<int32_t> adj, fr;
  DevBuf<uint32_t> rd;
  DevBuf<int> cnt;
  ATC_TRY(off.alloc(n + 1, s));
  ATC_TRY(exclusive_scan_i32_to_i64(deg, off.p, n, s));
  int64_t total = 2 * m;
  ATC_CK(cudaMemcpyAsync(off.p + n, &total, sizeof(total), cudaMemcpyHostToDevice, s));
  ATC_TRY(cur.alloc(n, s));
  ATC_CK(cudaMemcpyAsync(cur.p, off.p, sizeof(int64_t) * n, cudaMemcpyDeviceToDevice, s));
  ATC_TRY(adj.alloc(total, s));
  if (m) sym_scatter_kernel<<<grid_for(m, 256), 256, 0, s>>>(e.keys.p, m, e.bits, cur.p, adj.p);
  ATC_CK(cudaGetLastError());
  cur.release();
  ATC_TRY(rd.alloc(n, s));
  ATC_TRY(fr.alloc(n, s));
  ATC_TRY(cnt.alloc(1, s));
  apeel_init_kernel<<<grid_for(n, 256), 256, 0, s>>>(deg, n, rd.p, flags, minor);
  ATC_CK(cudaGetLastError());

  // host arithmetic in the reference's types: float threshold, uint32 limits and counts
  const uint32_t node_num = (uint32_t)n, edge_num = (uint32_t)(2 * m);
  const float deg_thre = (float)edge_num / 2 / node_num;
  const uint32_t step = (uint32_t)deg_thre;
  const uint32_t stop_at = node_num * 9 / 10;
  int hcnt = 0;
  auto select = [&](uint32_t limit, uint32_t it, int assign, int* nf) -> atc_status {
    ATC_CK(cudaMemsetAsync(cnt.p, 0, sizeof(int), s));
    apeel_select_kernel<<<grid_for(n, 256), 256, 0, s>>>(rd.p, flags, minor, n, limit, it, assign, fr.p, cnt.p);
    ATC_CK(cudaGetLastError());
    ATC_CK(cudaMemcpyAsync(&hcnt, cnt.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    ATC_CK(cudaStreamSynchronize(s));
    *nf = hcnt;
    return ATC_OK;
  };
  int f_size = 0;
  ATC_TRY(select(step, 1, 1, &f_size));
  uint32_t visited = (uint32_t)f_size;
  uint32_t depth = 1, it = 1;
  while (visited < stop_at && depth < 0xFF && it < 50) {
    ++it;
    if (f_size)
      apeel_lower_kernel<<<grid_for((int64_t)f_size * 32, 256), 256, 0, s>>>(fr.p, f_size, off.p, adj.p, flags, rd.p);
    ATC_CK(cudaGetLastError());
    int cand = 0;
    ATC_TRY(select(step * depth, it, 0, &cand));
    while (cand == 0 && depth < 0xFF && visited < stop_at) {
      ++depth;
      ATC_TRY(select(step * depth, it, 0, &cand));
    }
    ATC_TRY(select(step * depth, it, 1, &f_size));
    visited += (uint32_t)f_size;
    if ((uint32_t)f_size <= node_num / 500) ++depth;
  }
  if (iters_out) *iters_out = (int)it;
  return ATC_OK;
}

}  // namespace atc
