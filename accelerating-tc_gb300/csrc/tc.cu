// Triangle counting on an oriented CSR: the four kernel families of the reference,
// re-designed for sm_103a.  All count sum_u sum_{v in N+(u)} |N+(u) ∩ N+(v)| exactly in
// uint64; every warp reduces its lanes with shuffles and adds once to a 64-bit counter.
//
//   Hu-style      Hu/tc.cu:22-201       wedge walk: N+(u) staged in shared memory once
//                                        per work item (chunk of N+(u)), every N+(v),
//                                        v in N+(u), streamed through it (W tests);
//                                        sorted copy + branch-free search for short
//                                        N+(u), hash table above.
//   Bisson-style  Bisson/tc.cu:18-104   every edge handed to the endpoint h with the
//                                        longer list (grouping passes); N+(h) as a hash
//                                        table, bitmap or sorted copy in shared memory,
//                                        the partner's shorter list streamed through it
//                                        (sum of min(d+u, d+v) tests).  Kernels in
//                                        bisson.cuh.
//   Fox-style     Fox/tc.cu:18-125,     per-edge work min*log2(max+2); edges binned on
//                 316-384                the device into 1,2,4,...,32 threads per edge;
//                                        each thread searches a slice of the shorter list
//                                        in the longer one.
//   TriCore-style tricount_gpu.cu:215-290  warp per edge; 32 pivots of the longer list
//                                        in shared memory bracket each element of the
//                                        shorter list, then a binary search inside the
//                                        bracket.
#include <cmath>
#include <mutex>
#include <vector>

#include "bisson.cuh"

namespace atc {


namespace {


// ============================== part split ===========================================
// Work of edge e for cutting the edges into parts: the shorter list it streams, plus one.
// work[m] = 0, so that an exclusive scan of m + 1 entries ends with the total.
__global__ void edge_work_kernel(CsrView g, int64_t* work) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e <= g.m; e += stride) {
    int64_t w = 0;
    if (e < g.m) {
      const int32_t u = g.esrc[e], v = g.cols[e];
      const int64_t du = g.off[u + 1] - g.off[u], dv = g.off[v + 1] - g.off[v];
      w = (du < dv ? du : dv) + 1;
    }
    work[e] = w;
  }
}

// bounds[t] (t = 0, 1) = the first edge whose work prefix reaches total * (part + t) / nparts.
__global__ void part_bounds_kernel(const int64_t* prefix, int64_t m, uint32_t part, uint32_t nparts, int64_t* bounds) {
  const int t = threadIdx.x;
  if (t > 1) return;
  const uint32_t k = part + t;
  if (k == 0 || k >= nparts) {
    bounds[t] = k == 0 ? 0 : m;
    return;
  }
  const int64_t target = (int64_t)((__int128)prefix[m] * k / nparts);
  int64_t lo = 0, hi = m;
  while (lo < hi) {
    const int64_t mid = (lo + hi) >> 1;
    if (prefix[mid] < target) lo = mid + 1; else hi = mid;
  }
  bounds[t] = lo;
}

// ============================== TriCore-style ======================================
constexpr int kTriWarps = 8;

__global__ void __launch_bounds__(kTriWarps * 32) tricore_kernel(CsrView g, unsigned long long* out) {
  __shared__ int32_t piv[kTriWarps][32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  unsigned long long cnt = 0;
  const int64_t warps = (int64_t)gridDim.x * kTriWarps;
  for (int64_t e = g.e0 + (int64_t)blockIdx.x * kTriWarps + w; e < g.e1; e += warps) {
    int32_t u = g.esrc[e], v = g.cols[e];
    int64_t au = g.off[u], du = g.off[u + 1] - au;
    int64_t av = g.off[v], dv = g.off[v + 1] - av;
    const int32_t* A = g.cols + (du >= dv ? au : av);
    const int32_t* Bl = g.cols + (du >= dv ? av : au);
    int64_t da = du >= dv ? du : dv, db = du >= dv ? dv : du;
    if (db == 0) continue;
    piv[w][lane] = A[(int64_t)lane * da / 32];
    __syncwarp();
    // a lane's elements ascend: `prev` = where its previous element's search ended, a
    // lower bound for the next one inside any bracket
    int64_t prev = 0;
    for (int64_t j = lane; j < db; j += 32) {
      int32_t x = __ldg(Bl + j);
      // k = number of pivots <= x
      int lo = 0, hi = 32;
      while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (piv[w][mid] <= x) lo = mid + 1; else hi = mid;
      }
      if (lo == 0) continue;                 // x < A[0]
      if (piv[w][lo - 1] == x) { ++cnt; continue; }
      int64_t b = (int64_t)(lo - 1) * da / 32 + 1;  // strictly inside the bracket
      int64_t e2 = lo == 32 ? da : (int64_t)lo * da / 32;
      if (prev > b) b = prev;
      while (b < e2) {  // lower bound of x in A[b, e2)
        const int64_t mid = (b + e2) >> 1;
        if (__ldg(A + mid) < x) b = mid + 1; else e2 = mid;
      }
      cnt += b < da && __ldg(A + b) == x;
      prev = b;
    }
    __syncwarp();
  }
  warp_add_count(cnt, out);
}

// ============================== Fox-style ==========================================
// Work of an edge (Fox/tc.cu:22-31): min(d+u, d+v) * log2(max + 2), as an int.
__device__ __forceinline__ int fox_work(int64_t du, int64_t dv) {
  int64_t big = du > dv ? du : dv, small = du > dv ? dv : du;
  double wv = (double)small * log2((double)big + 2.0);
  return wv > 2147483647.0 ? 2147483647 : (int)wv;
}

__global__ void fox_maxwork_kernel(CsrView g, int* maxw) {
  int best = 0;
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t e = g.e0 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < g.e1; e += stride) {
    int32_t u = g.esrc[e], v = g.cols[e];
    best = max(best, fox_work(g.off[u + 1] - g.off[u], g.off[v + 1] - g.off[v]));
  }
  for (int o = 16; o > 0; o >>= 1) best = max(best, __shfl_xor_sync(0xffffffffu, best, o));
  if ((threadIdx.x & 31) == 0) atomicMax(maxw, best);
}

struct FoxBins {
  int bound[7];  // work thresholds: bin b holds work in [bound[b], bound[b+1])
};

__device__ __forceinline__ int fox_bin(const FoxBins& fb, int wk) {
  int b = 0;
#pragma unroll
  for (int i = 1; i < 6; ++i) b += wk >= fb.bound[i];
  return b;
}

__global__ void fox_hist_kernel(CsrView g, FoxBins fb, unsigned long long* hist) {
  __shared__ unsigned int h[6];
  if (threadIdx.x < 6) h[threadIdx.x] = 0;
  __syncthreads();
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t e = g.e0 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < g.e1; e += stride) {
    int32_t u = g.esrc[e], v = g.cols[e];
    atomicAdd(&h[fox_bin(fb, fox_work(g.off[u + 1] - g.off[u], g.off[v + 1] - g.off[v]))], 1u);
  }
  __syncthreads();
  if (threadIdx.x < 6 && h[threadIdx.x]) atomicAdd(&hist[threadIdx.x], (unsigned long long)h[threadIdx.x]);
}

// Edges into their bins; the lanes of a warp that share a bin reserve their slots with one
// atomic (six cursors taken by every edge would serialise on a handful of addresses).  The
// loop is padded to whole warps for __match_any_sync.
__global__ void fox_scatter_kernel(CsrView g, FoxBins fb, unsigned long long* cursor, int64_t* list) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const int64_t w_pad = (g.e1 - g.e0 + 31) & ~31ll;
  const int lane = threadIdx.x & 31;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < w_pad; i += stride) {
    const int64_t e = g.e0 + i;
    int b = -1;
    if (e < g.e1) {
      const int32_t u = g.esrc[e], v = g.cols[e];
      b = fox_bin(fb, fox_work(g.off[u + 1] - g.off[u], g.off[v + 1] - g.off[v]));
    }
    const unsigned same = __match_any_sync(0xffffffffu, b);
    const int lead = __ffs(same) - 1;
    unsigned long long base = 0;
    if (b >= 0 && lane == lead) base = atomicAdd(&cursor[b], (unsigned long long)__popc(same));
    base = __shfl_sync(0xffffffffu, base, lead);
    if (b >= 0) list[base + __popc(same & ((1u << lane) - 1))] = e;
  }
}

// T threads per edge (Fox/tc.cu:64-125): each thread takes every T-th element of the
// shorter list and searches it in the longer list (exponential search from the previous
// element's position, then binary search).
template <int T>
__global__ void __launch_bounds__(256) fox_kernel(CsrView g, const int64_t* list, int64_t cnt_edges,
                                                  unsigned long long* out) {
  unsigned long long cnt = 0;
  const int64_t gid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int sub = (int)(gid % T);
  const int64_t groups = (int64_t)gridDim.x * blockDim.x / T;
  for (int64_t i = gid / T; i < cnt_edges; i += groups) {
    int64_t e = list[i];
    int32_t u = g.esrc[e], v = g.cols[e];
    int64_t au = g.off[u], du = g.off[u + 1] - au;
    int64_t av = g.off[v], dv = g.off[v + 1] - av;
    const int32_t* L = g.cols + (du >= dv ? au : av);   // longer
    const int32_t* S = g.cols + (du >= dv ? av : au);   // shorter
    int64_t dl = du >= dv ? du : dv, ds = du >= dv ? dv : du;
    // a thread's elements ascend, so each search resumes where the previous one ended:
    // gallop forward from there, then binary-search the last step
    int64_t lo = 0;
    for (int64_t j = sub; j < ds; j += T) {
      const int32_t x = __ldg(S + j);
      int64_t a = lo, b = lo, step = 1;  // every L[i], i < a, is < x
      while (b < dl && __ldg(L + b) < x) {
        a = b + 1;
        b = a + step;
        step <<= 1;
      }
      if (b > dl) b = dl;
      while (a < b) {  // L[b] >= x or b == dl
        const int64_t mid = (a + b) >> 1;
        if (__ldg(L + mid) < x) a = mid + 1; else b = mid;
      }
      cnt += a < dl && __ldg(L + a) == x;
      lo = a;
    }
  }
  warp_add_count(cnt, out);
}

// Fox's interleave (Fox/tc.cu:127-183): a bin's edges are sorted by the length of
// their longer list, cut into groups of 32 and dealt round-robin over `nblk` blocks, so
// every block gets a mix of long and short edges.  Group g = sec*nblk + first moves to
// rank first*q + min(first, r) + sec (q, r = ngroups / nblk, ngroups % nblk): a
// bijection on the groups; the tail of fewer than 32 edges stays in place.
__global__ void fox_lenkey_kernel(CsrView g, const int64_t* list, int64_t nb, uint64_t* keys) {
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nb; i += stride) {
    int64_t e = list[i];
    int32_t u = g.esrc[e], v = g.cols[e];
    int64_t du = g.off[u + 1] - g.off[u], dv = g.off[v + 1] - g.off[v];
    uint64_t mx = (uint64_t)(du > dv ? du : dv);
    if (mx > 0x7fffffffull) mx = 0x7fffffffull;
    keys[i] = (mx << 32) | (uint64_t)i;
  }
}

__global__ void fox_deal_kernel(const uint64_t* keys, const int64_t* list, int64_t nb, int64_t nblk, int64_t* out) {
  int64_t ngroups = nb / 32;
  int64_t q = nblk > 0 ? ngroups / nblk : 0, r = nblk > 0 ? ngroups % nblk : 0;
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nb; i += stride) {
    int64_t src = list[keys[i] & 0xffffffffull];
    int64_t grp = i / 32, dst = i;
    if (grp < ngroups && nblk > 1) {
      int64_t first = grp % nblk, sec = grp / nblk;
      dst = (first * q + (first < r ? first : r) + sec) * 32 + (i % 32);
    }
    out[dst] = src;
  }
}

// ============================== sorted-copy searches ===============================
// TriCore-style and Fox-style counts on the Bisson-style grouping: every edge goes to its
// endpoint h with the longer list and the partner's shorter list is streamed (sum of
// min(d+u, d+v) searches).  N+(h), the longer list of every edge of an item, is staged once
// per item as a sorted copy in shared memory, and every streamed element is searched in
// it.  The reference kernels search the longer list in global memory, one dependent load
// per step, per edge; here only lists too long for shared memory are searched there.
//   KIND 0, TriCore-style (tricount_gpu.cu:215-290): 32 samples of the longer list (the
//     reference's per-warp pivot cache) sit contiguous in shared memory, so the first five
//     levels of every search touch 32 distinct banks; the sample bracket holding the
//     element is then binary-searched.  Every bracket of a list holds at most ceil(d/32)
//     elements, so the bracket search is a fixed run of halving steps, the same number on
//     every lane, without a loop test or a bound test per step (a read past the list is
//     clamped to its last element, which is not below the element searched).
//   KIND 1, Fox-style (Fox/tc.cu:64-125): a lane's successive elements of a list ascend, so
//     each search gallops forward from where the lane's previous one ended (restarting
//     when the element is smaller than the previous one), then binary-searches the last
//     step.
constexpr int kLiftMax = 11;  // the unrolled bracket search covers brackets of up to 4095

template <int KIND>
struct SortedProber {
  const int32_t* T;    // sorted N+(h) (shared memory, or global for lists beyond it)
  const int32_t* piv;  // 32 samples piv[i] = T[i * d / 32] (shared memory)
  int d;
  int32_t hi;    // T[d - 1]
  int prev;      // Fox: lower bound of the lane's previous element
  int32_t last;  // Fox: the lane's previous element
  int gap;       // Fox: how far the lane's previous forward search moved
  int lg = -1;   // TriCore: floor(log2(ceil(d/32))), the first halving step of the bracket search
                 // (the same for the whole list); -1: the bracket is searched by a loop
  __device__ __forceinline__ unsigned probe(int32_t x, bool valid) {
    if (!valid) return 0u;
    if (x > hi) return 0u;  // above the longer list: no search
    if constexpr (KIND == 0) {
      int k = 0;  // number of samples <= x: five fixed steps, then the last sample
#pragma unroll
      for (int step = 16; step > 0; step >>= 1)
        if (piv[k + step - 1] <= x) k += step;
      if (piv[k] <= x) ++k;
      if (k == 0) return 0u;  // x < T[0]
      if (piv[k - 1] == x) return 1u;
      int b = (int)(((int64_t)(k - 1) * d) >> 5) + 1;  // strictly inside the bracket
      int e = k == 32 ? d : (int)(((int64_t)k * d) >> 5);
      if (lg >= 0 && lg <= kLiftMax) {
        // the last index below x: T[b-1] (the sample) is below x, and 2^(lg+1) - 1 steps cover
        // the bracket; T[e] (the next sample, or past the list) is not below x
        int lo = b - 1;
#define ATC_LIFT(t) \
  case t: {        \
    const int c = lo + (1 << t); \
    if (T[min(c, d - 1)] < x) lo = c; \
  }
        switch (lg) {  // enters at the first step and falls through the rest
          ATC_LIFT(11) [[fallthrough]];
          ATC_LIFT(10) [[fallthrough]];
          ATC_LIFT(9) [[fallthrough]];
          ATC_LIFT(8) [[fallthrough]];
          ATC_LIFT(7) [[fallthrough]];
          ATC_LIFT(6) [[fallthrough]];
          ATC_LIFT(5) [[fallthrough]];
          ATC_LIFT(4) [[fallthrough]];
          ATC_LIFT(3) [[fallthrough]];
          ATC_LIFT(2) [[fallthrough]];
          ATC_LIFT(1) [[fallthrough]];
          ATC_LIFT(0)
        }
#undef ATC_LIFT
        return lo + 1 < d && T[lo + 1] == x;
      }
      while (b < e) {
        const int mid = (b + e) >> 1;
        if (T[mid] < x) b = mid + 1; else e = mid;
      }
      return b < d && T[b] == x;
    } else {
      if (x < last) {
        // a new list (or an earlier element): its lower bound lies in [0, prev]
        int a = 0, b = prev;
        while (a < b) {
          const int mid = (a + b) >> 1;
          if (T[mid] < x) a = mid + 1; else b = mid;
        }
        prev = a;
        last = x;
        return a < d && T[a] == x;
      }
      last = x;
      // every T[i], i < a, is < x; the first step is half the lane's previous move, so a
      // lane walking one list at a steady stride settles in about log2(stride) steps
      int a = prev, step = gap > 1 ? gap >> 1 : 1;
      int b = a + step - 1;
      while (b < d && T[b] < x) {
        a = b + 1;
        step <<= 1;
        b = a + step - 1;
      }
      if (b > d) b = d;
      while (a < b) {  // T[b] >= x, or b == d
        const int mid = (a + b) >> 1;
        if (T[mid] < x) a = mid + 1; else b = mid;
      }
      gap = a - prev;
      prev = a;
      return a < d && T[a] == x;
    }
  }
  __device__ __forceinline__ unsigned finish() { return 0u; }
};

// ---- 1-D bulk copies into shared memory (the TMA unit's untiled mode) -------------
// One thread issues cp.async.bulk of a whole list; its completion is counted in bytes on an
// mbarrier that every thread of the copy's group waits on.  Source and destination start on
// 16-byte boundaries and the size is a multiple of 16 bytes: a list is copied from the
// 16-byte boundary at or below its first element to the one at or above its end (the CSR's
// cols carry 16 ints of padding, so the rounded end stays inside the allocation), and read
// from the offset of its first element.  Every wait is bounded in time: a wait that runs out
// records an error for the host (ATC_ERR_TIMEOUT) and the kernel stops counting.
constexpr uint64_t kBulkWaitNs = 1000000000ull;  // one second without the copy landing

__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(bar)) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
}

// Issued by one thread: the byte count the barrier's current phase waits for, then the copy.
// The proxy fence orders the group's earlier ordinary reads of `dst` before the async write.
__device__ __forceinline__ void bulk_list_to_smem(int32_t* dst, const int32_t* src, uint32_t bytes, uint64_t* bar) {
  asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(
                   smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}

// Waits for phase `parity` of the barrier to complete; false if it did not within limit_ns.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, uint64_t limit_ns = kBulkWaitNs) {
  const uint64_t t0 = global_ns();
  for (;;) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    if (done) return true;
    if (global_ns() - t0 > limit_ns) return false;
  }
}

// The bounded wait's failure path, for tests: a barrier whose phase announces 16 bytes that
// no copy delivers (one arrival, its transaction count never reached), waited on with
// limit_ns.  err = 1 when the wait gave up, as it must; nothing is in flight at exit.
__global__ void wait_timeout_check_kernel(uint64_t limit_ns, int* err) {
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar);
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_u32(&bar)), "r"(16u)
                 : "memory");
  }
  __syncthreads();
  const bool ok = mbar_wait(&bar, 0, limit_ns);
  if (!ok && threadIdx.x == 0) *err = 1;
}

// The 16-byte-aligned window [a0, a1) of cols holding the list [hb, hb + dh).
__device__ __forceinline__ void bulk_window(int64_t hb, int64_t dh, int64_t* a0, uint32_t* bytes) {
  *a0 = hb & ~3ll;
  *bytes = (uint32_t)(((hb + dh + 3) & ~3ll) - *a0) * 4u;
}

// bulk: stage N+(h) with bulk copies (device-resident cols); otherwise with loads (cols in
// mapped host memory).  err: set to 1 when a bulk wait runs out.
template <int KIND>
__global__ void __launch_bounds__(kBgWarps * 32) sorted_warp_kernel(CsrView g, const int32_t* __restrict__ plist,
                                                                    const GroupItem* __restrict__ items, int nitems,
                                                                    int* next, bool bulk, int* err,
                                                                    unsigned long long* out) {
  __shared__ __align__(16) int32_t T[kBgWarps][kWarpMax + 8];
  __shared__ int32_t piv[kBgWarps][32];
  __shared__ __align__(8) uint64_t bar[kBgWarps];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) mbar_init(&bar[w]);
  __syncwarp();
  uint32_t phase = 0;
  unsigned long long total = 0;
  for (;;) {
    int it = 0;
    if (lane == 0) it = atomicAdd(next, 1);
    it = __shfl_sync(0xffffffffu, it, 0);
    if (it >= nitems) break;
    const GroupItem gi = items[it];
    const int64_t hb = g.off[gi.h];
    const int dh = (int)(g.off[gi.h + 1] - hb);  // 1 .. kWarpMax
    const int32_t* L = T[w];
    if (bulk) {
      int64_t a0;
      uint32_t bytes;
      bulk_window(hb, dh, &a0, &bytes);
      if (lane == 0) bulk_list_to_smem(T[w], g.cols + a0, bytes, &bar[w]);
      const bool ok = mbar_wait(&bar[w], phase);
      phase ^= 1u;
      if (!__all_sync(0xffffffffu, ok)) {
        if (lane == 0) atomicExch(err, 1);
        mbar_wait(&bar[w], phase ^ 1u);  // once more for the copy in flight, then stop
        break;
      }
      L = T[w] + (hb - a0);
    } else {
      for (int j = lane; j < dh; j += 32) T[w][j] = __ldg(g.cols + hb + j);
      __syncwarp();
    }
    piv[w][lane] = L[(lane * dh) >> 5];
    __syncwarp();
    int64_t cur = gi.b;
    auto nb = [&]() { int64_t r = cur; cur += 32; return r; };
    SortedProber<KIND> pr{L, piv[w], dh, L[dh - 1], 0, INT32_MIN, 16, 31 - __clz((dh + 31) >> 5)};
    total += stream_partners(g, plist, gi.e, lane, nb, pr);
    __syncwarp();  // the next item overwrites the copy
  }
  warp_add_count(total, out);
}

template <int KIND>
__global__ void __launch_bounds__(kBgWarps * 32) sorted_block_kernel(CsrView g, const int32_t* __restrict__ plist,
                                                                     const GroupItem* __restrict__ items, int nitems,
                                                                     int* next, uint32_t tab_words, bool bulk,
                                                                     int* err, unsigned long long* out) {
  extern __shared__ __align__(16) int32_t T[];  // tab_words + 8
  __shared__ int32_t piv[32];
  __shared__ int cur_item;
  __shared__ unsigned long long bnext;
  __shared__ __align__(8) uint64_t bar;
  const int lane = threadIdx.x & 31;
  if (threadIdx.x == 0) mbar_init(&bar);
  __syncthreads();
  uint32_t phase = 0;
  unsigned long long total = 0;
  for (;;) {
    if (threadIdx.x == 0) {
      cur_item = atomicAdd(next, 1);
      bnext = 0;
    }
    __syncthreads();
    const int it = cur_item;
    if (it >= nitems) break;
    const GroupItem gi = items[it];
    const int64_t hb = g.off[gi.h];
    const int64_t dh = g.off[gi.h + 1] - hb;
    const bool staged = dh <= (int64_t)tab_words;
    const int32_t* L = g.cols + hb;
    if (staged && bulk) {
      int64_t a0;
      uint32_t bytes;
      bulk_window(hb, dh, &a0, &bytes);
      if (threadIdx.x == 0) bulk_list_to_smem(T, g.cols + a0, bytes, &bar);
      const bool ok = __syncthreads_and(mbar_wait(&bar, phase));
      phase ^= 1u;
      if (!ok) {
        if (threadIdx.x == 0) atomicExch(err, 1);
        mbar_wait(&bar, phase ^ 1u);  // once more for the copy in flight, then stop
        break;
      }
      L = T + (hb - a0);
    } else if (staged) {
      for (int64_t j = threadIdx.x; j < dh; j += blockDim.x) T[j] = __ldg(g.cols + hb + j);
      L = T;
    }
    if (threadIdx.x < 32) piv[threadIdx.x] = __ldg(g.cols + hb + (((int64_t)threadIdx.x * dh) >> 5));
    __syncthreads();
    auto nb = [&]() {
      unsigned long long r = 0;
      if (lane == 0) r = atomicAdd(&bnext, 32ull);
      return gi.b + (int64_t)__shfl_sync(0xffffffffu, r, 0);
    };
    SortedProber<KIND> pr{L, piv, (int)dh, __ldg(g.cols + hb + dh - 1), 0, INT32_MIN, 16,
                          31 - __clz((int)((dh + 31) >> 5))};
    total += stream_partners(g, plist, gi.e, lane, nb, pr);
    __syncthreads();  // the next item overwrites the copy
  }
  warp_add_count(total, out);
}

}  // namespace

// ---- family drivers ----------------------------------------------------------------
static atc_status run_tricore(const CsrView& g, const atc_tuning* t, unsigned long long* ctr, cudaStream_t s,
                              int* launches) {
  Phase ph("tc.count", s);
  int grid = t && t->tricore_blocks > 0 ? t->tricore_blocks
                                        : sm_count() * blocks_per_sm((const void*)tricore_kernel, kTriWarps * 32, 0);
  tricore_kernel<<<grid, kTriWarps * 32, 0, s>>>(g, ctr);
  ATC_CK(cudaGetLastError());
  *launches += 1;
  return ATC_OK;
}

static atc_status run_fox(const CsrView& g, const atc_tuning* t, unsigned long long* ctr, cudaStream_t s,
                          int* launches) {
  DevBuf<int> mx;
  DevBuf<unsigned long long> hist, cursor;
  std::optional<Phase> ph;
  ph.emplace("tc.bins", s);
  ATC_TRY(mx.alloc(1, s));
  ATC_TRY(hist.alloc(6, s));
  ATC_TRY(cursor.alloc(6, s));
  ATC_CK(cudaMemsetAsync(mx.p, 0, sizeof(int), s));
  ATC_CK(cudaMemsetAsync(hist.p, 0, sizeof(unsigned long long) * 6, s));
  fox_maxwork_kernel<<<grid_for(g.e1 - g.e0, 256), 256, 0, s>>>(g, mx.p);
  ATC_CK(cudaGetLastError());
  int maxw = 0;
  ATC_CK(cudaMemcpyAsync(&maxw, mx.p, sizeof(int), cudaMemcpyDeviceToHost, s));
  ATC_CK(cudaStreamSynchronize(s));
  // Bin boundaries of Fox/tc.cu:318-331: partition points 8^((log8(max)-1)(i-1)/32 + 1)
  // for i = 2, 4, ..., 32; bin i threads holds work in [pp(i), pp(2i)).
  int wpt = t && t->fox_work_per_thread > 1 ? t->fox_work_per_thread : 8;
  FoxBins fb;
  fb.bound[0] = INT32_MIN;
  double maxPow = maxw > 0 ? std::log((double)maxw) / std::log((double)wpt) : 0.0;
  int k = 1;
  for (int i = 2; i <= 32; i *= 2, ++k) {
    double index = (maxPow - 1) * (i - 1) / 32.0 + 1;
    long double pp = powl((long double)wpt, (long double)index);
    fb.bound[k] = pp > 2147483647.0L ? 2147483647 : (int)pp;
  }
  fb.bound[6] = INT32_MAX;
  fox_hist_kernel<<<grid_for(g.e1 - g.e0, 256), 256, 0, s>>>(g, fb, hist.p);
  ATC_CK(cudaGetLastError());
  unsigned long long h[6];
  ATC_CK(cudaMemcpyAsync(h, hist.p, sizeof(h), cudaMemcpyDeviceToHost, s));
  ATC_CK(cudaStreamSynchronize(s));
  unsigned long long start[7];
  start[0] = 0;
  for (int b = 0; b < 6; ++b) start[b + 1] = start[b] + h[b];
  ATC_CK(cudaMemcpyAsync(cursor.p, start, sizeof(unsigned long long) * 6, cudaMemcpyHostToDevice, s));
  DevBuf<int64_t> list, list2;
  ATC_TRY(list.alloc(g.e1 - g.e0, s));
  fox_scatter_kernel<<<grid_for(g.e1 - g.e0, 256), 256, 0, s>>>(g, fb, cursor.p, list.p);
  ATC_CK(cudaGetLastError());
  *launches += 3;
  const int64_t* L = list.p;
  if (t && t->fox_rearrange) {
    ATC_TRY(list2.alloc(g.e1 - g.e0, s));
    for (int b = 0; b < 6; ++b) {
      int64_t nb = (int64_t)h[b];
      if (nb == 0) continue;
      DevBuf<uint64_t> k1, k2;
      ATC_TRY(k1.alloc(nb, s));
      ATC_TRY(k2.alloc(nb, s));
      fox_lenkey_kernel<<<grid_for(nb, 256), 256, 0, s>>>(g, list.p + start[b], nb, k1.p);
      ATC_CK(cudaGetLastError());
      uint64_t* ka = k1.p;
      uint64_t* kb = k2.p;
      ATC_TRY(sort_keys_u64(ka, kb, nb, 0, 63, s));
      int64_t edges_per_block = 256 >> b;
      int64_t nblk = nb / edges_per_block;
      fox_deal_kernel<<<grid_for(nb, 256), 256, 0, s>>>(ka, list.p + start[b], nb, nblk, list2.p + start[b]);
      ATC_CK(cudaGetLastError());
      *launches += 2;
    }
    L = list2.p;
  }
  ph.reset();
  ph.emplace("tc.count", s);
  int sms = sm_count();
  for (int b = 0; b < 6; ++b) {
    int64_t nb = (int64_t)h[b];
    if (nb == 0) continue;
    const int64_t* Lb = L + start[b];
    int64_t threads = nb << b;
    unsigned grid = (unsigned)std::min<int64_t>((threads + 255) / 256, (int64_t)sms * 8);
    switch (b) {
      case 0: fox_kernel<1><<<grid, 256, 0, s>>>(g, Lb, nb, ctr); break;
      case 1: fox_kernel<2><<<grid, 256, 0, s>>>(g, Lb, nb, ctr); break;
      case 2: fox_kernel<4><<<grid, 256, 0, s>>>(g, Lb, nb, ctr); break;
      case 3: fox_kernel<8><<<grid, 256, 0, s>>>(g, Lb, nb, ctr); break;
      case 4: fox_kernel<16><<<grid, 256, 0, s>>>(g, Lb, nb, ctr); break;
      default: fox_kernel<32><<<grid, 256, 0, s>>>(g, Lb, nb, ctr); break;
    }
    ATC_CK(cudaGetLastError());
    *launches += 1;
  }
  ATC_CK(cudaStreamSynchronize(s));  // `start` / `h` live on this frame
  return ATC_OK;
}

// Launches the block and warp kernels over work items; S = hash slots per bucket.
// hc = {warp items, block items, -, longest hashed block list}.
template <int S>
static atc_status launch_bisson(const CsrView& g, const int32_t* plist, const GroupItem* witems,
                                const GroupItem* bitems, const int* hc, int* counters, unsigned long long* ctr,
                                cudaStream_t s, int* launches) {
  if (hc[1]) {
    // block table: enough slots for the longest hashed list at load factor 1/4, or the
    // full bitmap when some list needs it
    uint32_t words = 64;
    while (words < 4u * (uint32_t)hc[3]) words <<= 1;
    if (words > (uint32_t)kTabWords) words = kTabWords;
    size_t smem = sizeof(int32_t) * words;
    ATC_CK(cudaFuncSetAttribute((const void*)bisson_block_kernel<FullItems, S>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int bps = blocks_per_sm((const void*)bisson_block_kernel<FullItems, S>, kBgWarps * 32, smem);
    int grid = std::min(hc[1], sm_count() * bps);
    bisson_block_kernel<FullItems, S><<<grid, kBgWarps * 32, smem, s>>>(
        g, plist, FullItems{bitems}, hc[1], nullptr, counters + 5, words, GraphTags{nullptr, 0, nullptr}, ctr);
    ATC_CK(cudaGetLastError());
    *launches += 1;
  }
  if (hc[0]) {
    int bps = blocks_per_sm((const void*)bisson_warp_kernel<FullItems, S>, kBgWarps * 32, 0);
    int grid = (int)std::min<int64_t>((hc[0] + kBgWarps - 1) / kBgWarps, (int64_t)sm_count() * bps);
    bisson_warp_kernel<FullItems, S><<<grid, kBgWarps * 32, 0, s>>>(g, plist, FullItems{witems}, hc[0], nullptr,
                                                                   counters + 4, GraphTags{nullptr, 0, nullptr}, ctr);
    ATC_CK(cudaGetLastError());
    *launches += 1;
  }
  return ATC_OK;
}

static atc_status launch_slots(int slots, const CsrView& g, const int32_t* plist, const GroupItem* witems,
                               const GroupItem* bitems, const int* hc, int* counters, unsigned long long* ctr,
                               cudaStream_t s, int* launches) {
  if (slots == 1) return launch_bisson<1>(g, plist, witems, bitems, hc, counters, ctr, s, launches);
  if (slots == 2) return launch_bisson<2>(g, plist, witems, bitems, hc, counters, ctr, s, launches);
  return launch_bisson<4>(g, plist, witems, bitems, hc, counters, ctr, s, launches);
}

// Item shape: the defaults, overridden field by field by the tuning (chunks >= 32 partners).
static atc_status item_shape(const atc_tuning* t, ItemShape* sh, int* slots) {
  *sh = default_shape(32);
  *slots = kDefaultSlots;
  if (!t) return ATC_OK;
  ATC_CHECK_ARG(t->bisson_slots == 0 || t->bisson_slots == 1 || t->bisson_slots == 2 || t->bisson_slots == 4,
                "bisson_slots must be 0, 1, 2 or 4");
  if (t->bisson_cutover > 0) sh->cutover = std::min(t->bisson_cutover, kWarpMax);
  if (t->bisson_warp_max > 0) sh->warp_max = std::min(t->bisson_warp_max, kWarpHashMax);
  if (t->bisson_warp_chunk > 0) sh->warp_chunk = std::max(t->bisson_warp_chunk, 32);
  if (t->bisson_block_chunk > 0) sh->block_chunk = std::max(t->bisson_block_chunk, 32);
  if (t->bisson_slots > 0) *slots = t->bisson_slots;
  return ATC_OK;
}

// Hu-style (Hu/tc.cu:69-201): every wedge u -> v -> w is tested against N+(u), which a
// work item stages in shared memory once and which every N+(v), v in N+(u), streams
// through: W tests in all.  The reference binary-searches a sorted run of N+(u); here the
// staged set is the sorted copy searched branch-free for d+(u) <= 32 and a hash table
// above (the Bisson-style kernels' sets).  The reference's 30 000 vertex ranges of equal
// wedge work (Hu/tc.cu:22-67,263-301) become chunks of N+(u) drained from a device queue,
// which balances dynamically.  No grouping pass: the items index the CSR itself.
static atc_status run_hu(const CsrView& g, const atc_tuning* t, unsigned long long* ctr, cudaStream_t s,
                         int* launches) {
  ItemShape sh;
  int slots;
  ATC_TRY(item_shape(t, &sh, &slots));
  // the sorted copy only for N+(u) of at most 8 (every N+(v) is searched in it; the hash
  // takes one probe): 4 % faster than 32 at R-MAT scale 24
  if (!t || t->bisson_cutover <= 0) sh.cutover = 8;
  std::optional<Phase> ph;
  ph.emplace("tc.items", s);
  DevBuf<int> counters;  // warp items, block items, (unused), longest block list, warp next, block next
  ATC_TRY(counters.alloc(8, s));
  ATC_CK(cudaMemsetAsync(counters.p, 0, sizeof(int) * 8, s));
  const int64_t mi = max_items(g.n, g.e1 - g.e0, std::min(sh.warp_chunk, sh.block_chunk));
  DevBuf<GroupItem> witems, bitems;
  ATC_TRY(witems.alloc(mi, s));
  ATC_TRY(bitems.alloc(mi, s));
  // the partner range of u is its own CSR row
  group_items_kernel<<<grid_for(g.n, 256), 256, 0, s>>>(g, g.off, witems.p, bitems.p, counters.p, sh, g.e0, g.e1);
  ATC_CK(cudaGetLastError());
  int hc[4];
  ATC_CK(cudaMemcpyAsync(hc, counters.p, sizeof(hc), cudaMemcpyDeviceToHost, s));
  ATC_CK(cudaStreamSynchronize(s));
  *launches += 1;
  ph.reset();
  ph.emplace("tc.count", s);
  return launch_slots(slots, g, g.cols, witems.p, bitems.p, hc, counters.p, ctr, s, launches);
}

// The Bisson-style grouping of the edges of [e0, e1): every edge {u, v} at its endpoint h
// with the longer list, the partners of each h contiguous in plist, cut into warp and block
// items.  hc = {warp items, block items, -, longest hashed block list}.
struct Grouping {
  DevBuf<int32_t> cnt, cur, plist, deg;
  DevBuf<int64_t> gstart;
  DevBuf<int> counters;  // warp items, block items, (unused), longest block list, warp next, block next
  DevBuf<GroupItem> witems, bitems;
  int hc[4] = {0, 0, 0, 0};
};

static atc_status group_edges(const CsrView& g, const ItemShape& sh, Grouping* gr, cudaStream_t s, int* launches) {
  ATC_TRY(gr->cnt.alloc(g.n + 1, s));
  ATC_TRY(gr->cur.alloc(g.n, s));
  ATC_TRY(gr->gstart.alloc(g.n + 1, s));
  ATC_TRY(gr->counters.alloc(8, s));
  ATC_CK(cudaMemsetAsync(gr->cnt.p, 0, sizeof(int32_t) * (g.n + 1), s));
  ATC_CK(cudaMemsetAsync(gr->cur.p, 0, sizeof(int32_t) * g.n, s));
  ATC_CK(cudaMemsetAsync(gr->counters.p, 0, sizeof(int) * 8, s));
  ATC_TRY(gr->deg.alloc(g.n + 1, s));
  csr_outdeg_kernel<<<grid_for(g.n, 256), 256, 0, s>>>(g, gr->deg.p);
  ATC_CK(cudaGetLastError());
  group_count_kernel<<<grid_for(g.e1 - g.e0, 256), 256, 0, s>>>(g, gr->cnt.p, gr->deg.p);
  ATC_CK(cudaGetLastError());
  ATC_TRY(exclusive_scan_i32_to_i64(gr->cnt.p, gr->gstart.p, g.n + 1, s));
  int64_t total = 0;
  ATC_CK(cudaMemcpyAsync(&total, gr->gstart.p + g.n, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
  ATC_CK(cudaStreamSynchronize(s));
  ATC_TRY(gr->plist.alloc(total + 32, s));
  group_scatter_kernel<<<grid_for(g.e1 - g.e0, 256), 256, 0, s>>>(g, gr->gstart.p, gr->cur.p, gr->plist.p,
                                                                   gr->deg.p);
  ATC_CK(cudaGetLastError());
  // items: at most one per group plus one per chunk boundary
  int64_t max_items = g.n + total / std::min(sh.warp_chunk, sh.block_chunk) + 1;
  ATC_TRY(gr->witems.alloc(max_items, s));
  ATC_TRY(gr->bitems.alloc(max_items, s));
  group_items_kernel<<<grid_for(g.n, 256), 256, 0, s>>>(g, gr->gstart.p, gr->witems.p, gr->bitems.p,
                                                         gr->counters.p, sh, 0, INT64_MAX);
  ATC_CK(cudaGetLastError());
  ATC_CK(cudaMemcpyAsync(gr->hc, gr->counters.p, sizeof(gr->hc), cudaMemcpyDeviceToHost, s));
  ATC_CK(cudaStreamSynchronize(s));
  *launches += 5;
  return ATC_OK;
}

static atc_status run_bisson(const CsrView& g, const atc_tuning* t, unsigned long long* ctr, cudaStream_t s,
                             int* launches) {
  ItemShape sh;
  int slots;
  ATC_TRY(item_shape(t, &sh, &slots));
  std::optional<Phase> ph;
  ph.emplace("tc.group", s);
  Grouping gr;
  ATC_TRY(group_edges(g, sh, &gr, s, launches));
  ph.reset();
  ph.emplace("tc.count", s);
  return launch_slots(slots, g, gr.plist.p, gr.witems.p, gr.bitems.p, gr.hc, gr.counters.p, ctr, s, launches);
}

// TriCore-style (KIND 0) and Fox-style (KIND 1) searches of the staged longer lists.
// max_outdeg sizes the block kernels' shared copy (lists above kTabWords stay in global).
// bulk: the lists are staged by TMA bulk copies (cols in device memory); with cols in mapped
// host memory they are staged with loads.
template <int KIND>
static atc_status run_sorted(const CsrView& g, int max_outdeg, bool bulk, unsigned long long* ctr, cudaStream_t s,
                             int* launches) {
  ItemShape sh = default_shape(kWarpMax);
  std::optional<Phase> ph;
  ph.emplace("tc.group", s);
  Grouping gr;
  ATC_TRY(group_edges(g, sh, &gr, s, launches));
  ph.reset();
  ph.emplace("tc.count", s);
  if (gr.hc[1]) {
    uint32_t words = (uint32_t)std::min(std::max(max_outdeg, kWarpMax + 1), kTabWords);
    words = (words + 31) & ~31u;
    const size_t smem = sizeof(int32_t) * (words + 8);  // + the bulk window's rounding
    ATC_CK(cudaFuncSetAttribute((const void*)sorted_block_kernel<KIND>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)smem));
    const int bps = blocks_per_sm((const void*)sorted_block_kernel<KIND>, kBgWarps * 32, smem);
    const int grid = std::min(gr.hc[1], sm_count() * bps);
    sorted_block_kernel<KIND><<<grid, kBgWarps * 32, smem, s>>>(g, gr.plist.p, gr.bitems.p, gr.hc[1],
                                                                 gr.counters.p + 5, words, bulk, gr.counters.p + 7,
                                                                 ctr);
    ATC_CK(cudaGetLastError());
    *launches += 1;
  }
  if (gr.hc[0]) {
    const int bps = blocks_per_sm((const void*)sorted_warp_kernel<KIND>, kBgWarps * 32, 0);
    const int grid = (int)std::min<int64_t>((gr.hc[0] + kBgWarps - 1) / kBgWarps, (int64_t)sm_count() * bps);
    sorted_warp_kernel<KIND><<<grid, kBgWarps * 32, 0, s>>>(g, gr.plist.p, gr.witems.p, gr.hc[0],
                                                            gr.counters.p + 4, bulk, gr.counters.p + 7, ctr);
    ATC_CK(cudaGetLastError());
    *launches += 1;
  }
  int err = 0;
  ATC_CK(cudaMemcpyAsync(&err, gr.counters.p + 7, sizeof(int), cudaMemcpyDeviceToHost, s));
  ATC_CK(cudaStreamSynchronize(s));
  if (err) {
    set_error("a bulk copy into shared memory did not complete within its wait limit");
    return ATC_ERR_TIMEOUT;
  }
  return ATC_OK;
}

// ---- counting without device allocation ------------------------------------------
// Some callers cannot call cudaMalloc: a host whose device memory is all owned by
// another allocator or runtime (a framework's caching pool, a memory manager that
// reserves the device up front), or a real-time loop that must not block in the
// driver's allocator.  atc_tc_noalloc runs the Bisson-style count above with every
// scratch buffer (edge sources, group counts, grouped partner list, work items,
// counters) carved out of one file-scope device array of kNoAllocBytes, fixed in size,
// which every GPU that loads this library keeps until the process exits.  Graphs above
// kNoAllocMaxN vertices or kNoAllocMaxM edges are refused.  The call synchronises its
// stream: it reads the CSR check, the item counts and the count back to the host.  All
// calls share the one array: calls that overlap on the GPU (concurrent streams or host
// threads on one device) race and must be serialised by the caller.
constexpr int64_t kNoAllocMaxN = 1 << 17;  // 131072 vertices
constexpr int64_t kNoAllocMaxM = 1 << 20;  // 1048576 oriented edges
constexpr int64_t kNoAllocItems = kNoAllocMaxN + kNoAllocMaxM / kWarpChunk + 1;

constexpr size_t align256(size_t x) { return (x + 255) & ~size_t(255); }
constexpr size_t kNaEsrc = 0;
constexpr size_t kNaCnt = kNaEsrc + align256(sizeof(int32_t) * (kNoAllocMaxM + 32));
constexpr size_t kNaCur = kNaCnt + align256(sizeof(int32_t) * (kNoAllocMaxN + 1));
constexpr size_t kNaGstart = kNaCur + align256(sizeof(int32_t) * kNoAllocMaxN);
constexpr size_t kNaPlist = kNaGstart + align256(sizeof(int64_t) * (kNoAllocMaxN + 1));
constexpr size_t kNaWitems = kNaPlist + align256(sizeof(int32_t) * (kNoAllocMaxM + 32));
constexpr size_t kNaBitems = kNaWitems + align256(sizeof(GroupItem) * kNoAllocItems);
constexpr size_t kNaCounters = kNaBitems + align256(sizeof(GroupItem) * kNoAllocItems);
constexpr size_t kNaCount = kNaCounters + align256(sizeof(int) * 8);
constexpr size_t kNoAllocBytes = kNaCount + align256(sizeof(unsigned long long));

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

namespace {

// Device address of g_noalloc_scratch for each device, looked up once per device (with
// that device current) and kept for the life of the process.  cudaDeviceReset destroys
// the context that holds the array, so after a reset of a device this entry point must
// not be called on it again in the same process.
atc_status noalloc_scratch(unsigned char** out) {
  static std::mutex mu;
  static unsigned char* addr[64] = {};
  int dev = 0;
  ATC_CK(cudaGetDevice(&dev));
  ATC_CHECK_ARG(dev >= 0 && dev < 64, "device index above 63");
  std::lock_guard<std::mutex> lock(mu);
  if (!addr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) {
      set_error("cudaGetSymbolAddress(g_noalloc_scratch): %s", cudaGetErrorString(e));
      return ATC_ERR_CUDA;
    }
    addr[dev] = static_cast<unsigned char*>(p);
  }
  *out = addr[dev];
  return ATC_OK;
}

// Checks a caller's CSR before any kernel indexes with it: offsets start at 0, end at m
// and never decrease; every row is strictly increasing with ids in [0, n).  Sets
// *bad = 1 on the first violation found by each warp.
__global__ void csr_check_kernel(const int64_t* off, const int32_t* cols, int64_t n, int64_t m, int* bad) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  if (blockIdx.x == 0 && threadIdx.x == 0 && (off[0] != 0 || off[n] != m)) *bad = 1;
  for (int64_t u = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; u < n; u += warps) {
    int64_t b = off[u], e = off[u + 1];
    bool ok = b <= e && b >= 0 && e <= m;
    if (ok) {
      for (int64_t j = b + lane; j < e; j += 32) {
        int32_t x = cols[j];
        if (x < 0 || x >= n || (j + 1 < e && cols[j + 1] <= x)) ok = false;
      }
    }
    if (__any_sync(0xffffffffu, !ok) && lane == 0) *bad = 1;
  }
}

__global__ void esrc_fill_kernel(const int64_t* off, int64_t n, int32_t* esrc) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t u = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; u < n; u += warps)
    for (int64_t j = off[u] + lane; j < off[u + 1]; j += 32) esrc[j] = (int32_t)u;
}

// Exclusive scan of cnt[0, len) into out (int64), one block of 1024 threads, no
// temporary storage: each thread scans a contiguous slice, slices are combined in
// shared memory.
__global__ void __launch_bounds__(1024) scan_one_block_kernel(const int32_t* cnt, int64_t len, int64_t* out) {
  __shared__ int64_t part[1024];
  const int t = threadIdx.x;
  const int64_t per = (len + 1023) / 1024;
  const int64_t b = t * per, e = b + per < len ? b + per : len;
  int64_t s = 0;
  for (int64_t i = b; i < e; ++i) s += cnt[i];
  part[t] = s;
  __syncthreads();
  for (int o = 1; o < 1024; o <<= 1) {
    int64_t y = t >= o ? part[t - o] : 0;
    __syncthreads();
    part[t] += y;
    __syncthreads();
  }
  int64_t run = part[t] - s;
  for (int64_t i = b; i < e; ++i) {
    out[i] = run;
    run += cnt[i];
  }
}

}  // namespace

static atc_status tc_noalloc_impl(const int64_t* off, const int32_t* cols, int64_t n, int64_t m, uint64_t* count,
                                  cudaStream_t s) {
  unsigned char* base = nullptr;
  ATC_TRY(noalloc_scratch(&base));
  int32_t* esrc = reinterpret_cast<int32_t*>(base + kNaEsrc);
  int32_t* cnt = reinterpret_cast<int32_t*>(base + kNaCnt);
  int32_t* cur = reinterpret_cast<int32_t*>(base + kNaCur);
  int64_t* gstart = reinterpret_cast<int64_t*>(base + kNaGstart);
  int32_t* plist = reinterpret_cast<int32_t*>(base + kNaPlist);
  GroupItem* witems = reinterpret_cast<GroupItem*>(base + kNaWitems);
  GroupItem* bitems = reinterpret_cast<GroupItem*>(base + kNaBitems);
  int* counters = reinterpret_cast<int*>(base + kNaCounters);
  unsigned long long* total_ctr = reinterpret_cast<unsigned long long*>(base + kNaCount);
  // what the kernels accumulate into starts at zero; the rest is overwritten
  ATC_CK(cudaMemsetAsync(cnt, 0, sizeof(int32_t) * (n + 1), s));
  ATC_CK(cudaMemsetAsync(cur, 0, sizeof(int32_t) * n, s));
  ATC_CK(cudaMemsetAsync(counters, 0, sizeof(int) * 8, s));
  ATC_CK(cudaMemsetAsync(total_ctr, 0, sizeof(unsigned long long), s));
  csr_check_kernel<<<grid_for(n * 32, 256), 256, 0, s>>>(off, cols, n, m, counters + 6);
  ATC_CK(cudaGetLastError());
  int bad = 0;
  ATC_CK(cudaMemcpyAsync(&bad, counters + 6, sizeof(int), cudaMemcpyDeviceToHost, s));
  ATC_CK(cudaStreamSynchronize(s));
  if (bad) {
    set_error("atc_tc_noalloc: offsets/cols are not an oriented CSR with sorted rows of ids in [0, n)");
    return ATC_ERR_INVALID;
  }
  esrc_fill_kernel<<<grid_for(n * 32, 256), 256, 0, s>>>(off, n, esrc);
  ATC_CK(cudaGetLastError());
  CsrView g = csr_view(off, cols, esrc, n, m);
  group_count_kernel<<<grid_for(m, 256), 256, 0, s>>>(g, cnt, nullptr);
  scan_one_block_kernel<<<1, 1024, 0, s>>>(cnt, n + 1, gstart);
  group_scatter_kernel<<<grid_for(m, 256), 256, 0, s>>>(g, gstart, cur, plist, nullptr);
  group_items_kernel<<<grid_for(n, 256), 256, 0, s>>>(g, gstart, witems, bitems, counters, default_shape(32), 0,
                                                       INT64_MAX);
  ATC_CK(cudaGetLastError());
  int hc[4];
  ATC_CK(cudaMemcpyAsync(hc, counters, sizeof(hc), cudaMemcpyDeviceToHost, s));
  ATC_CK(cudaStreamSynchronize(s));
  int launches = 0;
  ATC_TRY(launch_bisson<kDefaultSlots>(g, plist, witems, bitems, hc, counters, total_ctr, s, &launches));
  unsigned long long h = 0;
  ATC_CK(cudaMemcpyAsync(&h, total_ctr, sizeof(h), cudaMemcpyDeviceToHost, s));
  ATC_CK(cudaStreamSynchronize(s));
  *count = h;
  return ATC_OK;
}

}  // namespace atc

using namespace atc;

atc_status atc::part_edge_range(const atc_csr* csr, uint32_t part, uint32_t nparts, int64_t* range, cudaStream_t s) {
  range[0] = 0;
  range[1] = csr->m;
  if (nparts <= 1 || csr->m == 0) return ATC_OK;
  CsrPriv* pv = static_cast<CsrPriv*>(csr->priv);
  CsrView g = csr_view(csr->offsets, csr->cols, pv->esrc, csr->n, csr->m);
  DevBuf<int64_t> work, prefix, bounds;
  ATC_TRY(work.alloc(csr->m + 1, s));
  ATC_TRY(prefix.alloc(csr->m + 1, s));
  ATC_TRY(bounds.alloc(2, s));
  edge_work_kernel<<<grid_for(csr->m + 1, 256), 256, 0, s>>>(g, work.p);
  ATC_CK(cudaGetLastError());
  ATC_TRY(exclusive_scan_i64(work.p, prefix.p, csr->m + 1, s));
  part_bounds_kernel<<<1, 32, 0, s>>>(prefix.p, csr->m, part, nparts, bounds.p);
  ATC_CK(cudaGetLastError());
  ATC_CK(cudaMemcpyAsync(range, bounds.p, 2 * sizeof(int64_t), cudaMemcpyDeviceToHost, s));
  ATC_CK(cudaStreamSynchronize(s));
  return ATC_OK;
}

// Counts the edges [e0, e1) of the CSR (every edge for the whole count).
// ATC_KERNEL_AUTO: the Bisson-style or the Hu-style count, whichever this cost model of
// their GB300 times predicts is faster for the CSR.  Bisson-style: 1.232 ps per probe of the
// shorter lists (W_min) + 117.5 ps per edge (grouping, items) + 0.3 ms per call (two more
// passes and one more host synchronisation); Hu-style: 1.097 ps per wedge (W) + 103.5 ps per
// edge.  Fitted to R-MAT scale 24 (117 / 231 ms) and Chung-Lu graphs of 4M-46M edges; the
// learned selector (atc_select) chooses among all kernels and pipelines instead.
static atc_kernel auto_kernel(const atc_csr* csr) {
  const double m = (double)csr->m, w = (double)csr->wedges, wmin = (double)csr->wedges_min;
  const double bisson_ps = 1.232 * wmin + 117.5 * m + 3.0e8;
  const double hu_ps = 1.097 * w + 103.5 * m;
  return hu_ps < bisson_ps ? ATC_KERNEL_HU : ATC_KERNEL_BISSON;
}

static atc_status tc_window(const atc_csr* csr, atc_kernel kernel, const atc_tuning* tuning, int64_t e0, int64_t e1,
                            uint64_t* count, atc_stats* stats, cudaStream_t s) {
  if (kernel == ATC_KERNEL_AUTO) kernel = auto_kernel(csr);
  CsrPriv* pv = static_cast<CsrPriv*>(csr->priv);
  int launches = 0;
  EventTimer tm;
  if (e1 > e0) {
    CsrView g = csr_view(csr->offsets, csr->cols, pv->esrc, csr->n, csr->m);
    g.e0 = e0;
    g.e1 = e1;
    unsigned long long* ctr = pv->counter;
    Phase ph("tc", s);
    tm.start(s);
    ATC_CK(cudaMemsetAsync(ctr, 0, sizeof(unsigned long long), s));
    switch (kernel) {
      case ATC_KERNEL_HU: ATC_TRY(run_hu(g, tuning, ctr, s, &launches)); break;
      case ATC_KERNEL_BISSON: ATC_TRY(run_bisson(g, tuning, ctr, s, &launches)); break;
      case ATC_KERNEL_FOX:
        if (tuning && tuning->edge_kernels) ATC_TRY(run_fox(g, tuning, ctr, s, &launches));
        else ATC_TRY(run_sorted<1>(g, csr->max_outdeg, pv->host_cols == nullptr, ctr, s, &launches));
        break;
      default:
        if (tuning && tuning->edge_kernels) ATC_TRY(run_tricore(g, tuning, ctr, s, &launches));
        else ATC_TRY(run_sorted<0>(g, csr->max_outdeg, pv->host_cols == nullptr, ctr, s, &launches));
        break;
    }
    tm.stop(s);
    unsigned long long h = 0;
    {
      Phase ph_rb("tc.readback", s);
      ATC_CK(cudaMemcpyAsync(&h, ctr, sizeof(h), cudaMemcpyDeviceToHost, s));
    }
    ATC_CK(cudaStreamSynchronize(s));
    *count = h;
  }
  if (stats) {
    stats->kernel_ms = e1 > e0 ? tm.ms() : 0.0f;
    stats->total_ms = stats->kernel_ms;
    stats->wedges = (uint64_t)csr->wedges;
    stats->alg_bytes = 4ull * (uint64_t)(csr->n + 1) + 4ull * (uint64_t)csr->m + 4ull * (uint64_t)csr->wedges + 8ull;
    stats->alg_bytes_min =
        4ull * (uint64_t)(csr->n + 1) + 4ull * (uint64_t)csr->m + 4ull * (uint64_t)csr->wedges_min + 8ull;
    stats->kernel_used = (int32_t)kernel;
    stats->launches = launches;
  }
  return ATC_OK;
}

extern "C" atc_status atc_tc(const atc_csr* csr, atc_kernel kernel, const atc_tuning* tuning, uint64_t* count,
                             atc_stats* stats, atc_stream st) try {
  ATC_CHECK_ARG(csr != nullptr && count != nullptr, "NULL argument");
  ATC_CHECK_ARG(csr->priv != nullptr || csr->m == 0, "csr was not built by atc_pretc");
  ATC_CHECK_ARG(kernel >= ATC_KERNEL_AUTO && kernel <= ATC_KERNEL_TRICORE, "unknown atc_kernel");
  *count = 0;
  return tc_window(csr, kernel, tuning, 0, csr->m, count, stats, as_stream(st));
} ATC_CATCH

extern "C" atc_status atc_tc_part(const atc_csr* csr, atc_kernel kernel, const atc_tuning* tuning, uint32_t part,
                                  uint32_t nparts, uint64_t* count, int64_t* edge_range, atc_stats* stats,
                                  atc_stream st) try {
  ATC_CHECK_ARG(csr != nullptr && count != nullptr, "NULL argument");
  ATC_CHECK_ARG(csr->priv != nullptr || csr->m == 0, "csr was not built by atc_pretc");
  ATC_CHECK_ARG(kernel >= ATC_KERNEL_AUTO && kernel <= ATC_KERNEL_TRICORE, "unknown atc_kernel");
  ATC_CHECK_ARG(nparts >= 1 && part < nparts, "part must be in [0, nparts)");
  cudaStream_t s = as_stream(st);
  *count = 0;
  int64_t b[2];
  ATC_TRY(part_edge_range(csr, part, nparts, b, s));
  if (edge_range) {
    edge_range[0] = b[0];
    edge_range[1] = b[1];
  }
  return tc_window(csr, kernel, tuning, b[0], b[1], count, stats, s);
} ATC_CATCH

extern "C" atc_status atc_tc_noalloc(const int64_t* offsets, const int32_t* cols, int64_t n, int64_t m,
                                     uint64_t* count, atc_stream st) try {
  ATC_CHECK_ARG(count != nullptr, "count is NULL");
  ATC_CHECK_ARG(n >= 0 && m >= 0, "negative size");
  if (n > kNoAllocMaxN || m > kNoAllocMaxM) {
    set_error("graph too large for atc_tc_noalloc: n=%lld m=%lld, limits n<=%lld m<=%lld (scratch %zu bytes)",
              (long long)n, (long long)m, (long long)kNoAllocMaxN, (long long)kNoAllocMaxM, kNoAllocBytes);
    return ATC_ERR_INVALID;
  }
  *count = 0;
  if (m == 0 || n == 0) return ATC_OK;
  ATC_CHECK_ARG(offsets != nullptr && cols != nullptr, "NULL CSR array");
  return tc_noalloc_impl(offsets, cols, n, m, count, as_stream(st));
} ATC_CATCH

extern "C" atc_status atc_check_wait_timeout(atc_stream st) try {
  cudaStream_t s = as_stream(st);
  DevBuf<int> err;
  ATC_TRY(err.alloc(1, s));
  ATC_CK(cudaMemsetAsync(err.p, 0, sizeof(int), s));
  atc::wait_timeout_check_kernel<<<1, 32, 0, s>>>(1000000ull, err.p);  // a 1 ms limit
  ATC_CK(cudaGetLastError());
  int h = 0;
  ATC_CK(cudaMemcpyAsync(&h, err.p, sizeof(int), cudaMemcpyDeviceToHost, s));
  ATC_CK(cudaStreamSynchronize(s));
  if (h) {
    atc::set_error("a bulk-copy wait gave up after its time limit (the check's barrier never completes)");
    return ATC_ERR_TIMEOUT;
  }
  return ATC_OK;
} ATC_CATCH
