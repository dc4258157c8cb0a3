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
