// Bisson-style grouped counting kernels, shared by the single-graph count (tc.cu), the
// allocation-free count (tc.cu) and the batched count (batch.cu).  Internal header:
// every includer gets its own copy of the kernels.
#pragma once

#include "internal.cuh"

namespace atc {

struct CsrView {
  const int64_t* off;
  const int32_t* cols;
  const int32_t* esrc;
  int64_t n, m;
  int64_t e0, e1;  // edge window [e0, e1) of the per-edge passes (0, m: every edge)
};

inline CsrView csr_view(const int64_t* off, const int32_t* cols, const int32_t* esrc, int64_t n, int64_t m) {
  return CsrView{off, cols, esrc, n, m, 0, m};
}

namespace {

__device__ __forceinline__ void warp_add_count(unsigned long long c, unsigned long long* out) {
  for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
  if ((threadIdx.x & 31) == 0 && c) atomicAdd(out, c);
}

int blocks_per_sm(const void* kernel, int block, size_t smem) {
  int b = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, kernel, block, smem) != cudaSuccess || b < 1) b = 1;
  return b;
}

// ============================== Bisson-style =======================================
// The reference keeps a bitmap of N+(u) for rows longer than 32 and streams every N+(v),
// v in N+(u), through it (Bisson/tc.cu:36-62): one bit test per directed wedge, W tests
// in all.  Here every edge {u, v} is handed to its endpoint h with the longer list; N+(h)
// becomes a set in shared memory and the shorter list of the partner is streamed
// through it.  That tests sum_edges min(d+u, d+v) elements instead of W.
//   warp items (d+h <= kWarpMax): a warp per chunk of partners, no block barriers; N+(h)
//     either copied sorted into the warp's slot and binary-searched (d+h <= cutover, the
//     reference's <=32 branch, Bisson/tc.cu:63-87) or inserted into a warp-private hash
//     table of kWarpSlots slots (load factor <= 1/4);
//   block items (d+h > kWarpMax): a CTA per chunk of partners; N+(h) as a block hash
//     table sized to the largest such list, or a bitmap over [min, max] of the list, or
//     (lists too long for both) binary search in global memory.
// Chunks come from device work counters (one atomicAdd per chunk; nothing waits on them).
constexpr int kBgWarps = 8;
constexpr int kWarpMax = 256;       // longest N+(h) handled by one warp unless tuned
constexpr int kWarpSlots = 1024;    // warp-private hash slots (4 KB)
constexpr int kWarpHashMax = kWarpSlots / 2;  // longest N+(h) a warp item can hash (load 1/2)
constexpr int kWarpChunk = 512;     // partners per warp item
constexpr int kBlockChunk = 2048;   // partners per block item
constexpr int kTabWords = 16384;    // block table limit: 64 KB of slots or bitmap words
constexpr int kHashMax = kTabWords / 4;
constexpr int kBlockSmallList = 2048;  // batches: block items of lists up to this length run in
                                       // tables of at most 32 KB (six CTAs per SM), longer ones in
                                       // a launch of their own with the 64 KB table (three)
constexpr int kWarpGrab = 4;     // warp items taken per atomic
constexpr int kDefaultSlots = 4;  // hash slots per bucket unless tuned (one 16-byte shared load)

struct GroupItem {
  int32_t h;
  int32_t mode;  // warp: 0 sorted copy, 1 hash; block: 0 hash, 1 bitmap, 2 global search
  int64_t b, e;  // partner range in the grouped list
};

__device__ __forceinline__ bool longer_is_u(int32_t u, int32_t v, int64_t du, int64_t dv) {
  return du > dv || (du == dv && u < v);
}

// Out-degrees as int32: the grouping passes read a random vertex's degree with one 4-byte
// load from an array half the size of the offsets (it stays in L2 at R-MAT scale 24).
__global__ void csr_outdeg_kernel(CsrView g, int32_t* deg) {
  for (int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; u < g.n; u += (int64_t)gridDim.x * blockDim.x)
    deg[u] = (int32_t)(g.off[u + 1] - g.off[u]);
}

__device__ __forceinline__ int64_t degree_of(const CsrView& g, const int32_t* deg, int32_t v) {
  return deg ? (int64_t)__ldg(deg + v) : g.off[v + 1] - g.off[v];
}

// Pass 1: partners per group, with warp-aggregated atomics (edges of one source are
// contiguous, so runs of one h are common).  deg (nullable): the out-degrees.
__global__ void group_count_kernel(CsrView g, int32_t* cnt, const int32_t* deg) {
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  int64_t w_pad = (g.e1 - g.e0 + 31) & ~31ll;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < w_pad; i += stride) {
    const int64_t e = g.e0 + i;
    int32_t h = -1;
    if (e < g.e1) {
      int32_t u = g.esrc[e], v = g.cols[e];
      int64_t du = degree_of(g, deg, u), dv = degree_of(g, deg, v);
      if (du > 0 && dv > 0) h = longer_is_u(u, v, du, dv) ? u : v;
    }
    unsigned same = __match_any_sync(0xffffffffu, h);
    int lead = __ffs(same) - 1;
    if (h >= 0 && (int)(threadIdx.x & 31) == lead) atomicAdd(&cnt[h], __popc(same));
  }
}

// Pass 2: scatter partners into their group (order inside a group is irrelevant).
__global__ void group_scatter_kernel(CsrView g, const int64_t* gstart, int32_t* cur, int32_t* plist,
                                     const int32_t* deg) {
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  int64_t w_pad = (g.e1 - g.e0 + 31) & ~31ll;
  const int lane = threadIdx.x & 31;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < w_pad; i += stride) {
    const int64_t e = g.e0 + i;
    int32_t h = -1, p = 0;
    if (e < g.e1) {
      int32_t u = g.esrc[e], v = g.cols[e];
      int64_t du = degree_of(g, deg, u), dv = degree_of(g, deg, v);
      if (du > 0 && dv > 0) {
        bool hu = longer_is_u(u, v, du, dv);
        h = hu ? u : v;
        p = hu ? v : u;
      }
    }
    unsigned same = __match_any_sync(0xffffffffu, h);
    int lead = __ffs(same) - 1;
    int base = 0;
    if (h >= 0 && lane == lead) base = atomicAdd(&cur[h], __popc(same));
    base = __shfl_sync(0xffffffffu, base, lead);
    if (h >= 0) plist[gstart[h] + base + __popc(same & ((1u << lane) - 1))] = p;
  }
}

// Pass 3: cut every group into work items; counters[0] = warp items, [1] = block items,
// [3] = longest N+(h) among block items.
// Runtime shape of the work items: lists up to warp_max (<= kWarpHashMax) go to warp
// items of warp_chunk partners, longer ones to block items of block_chunk partners.
struct ItemShape {
  int cutover;      // warp items: sorted copy up to this length, hash above
  int warp_max;
  int warp_chunk;
  int block_chunk;
  int by_source;    // batches: 1 = every edge at its source (h = u, partners = its row: the
                    // Hu-style wedge walk, no grouping passes), 0 = at the longer endpoint,
                    // 2 = chosen per graph by the cost model (batch.cu)
};

__host__ __device__ inline ItemShape default_shape(int cutover) {
  return ItemShape{cutover, kWarpMax, kWarpChunk, kBlockChunk, 0};
}

// Upper bound on the items of either kind for a graph with n vertices, `partners`
// grouped partners and chunks of at least min_chunk partners.
__host__ __device__ inline int64_t max_items(int64_t n, int64_t partners, int min_chunk) {
  return n + partners / min_chunk + 1;
}

// Reserves k slots of counter `*ctr` for every lane of the warp with one atomic: returns
// this lane's first slot.  All 32 lanes call it (k may be 0).
__device__ __forceinline__ int warp_reserve(int* ctr, int k) {
  const int lane = threadIdx.x & 31;
  int incl = k;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += y;
  }
  int total = __shfl_sync(0xffffffffu, incl, 31);
  int base = 0;
  if (lane == 31 && total) base = atomicAdd(ctr, total);
  base = __shfl_sync(0xffffffffu, base, 31);
  return base + incl - k;
}

// One lane per vertex h; the loop bound is padded to whole warps so that every lane of a
// warp takes part in warp_reserve.
// The partner range of h is [gstart[h], gstart[h+1]) clipped to [clip0, clip1).
__global__ void group_items_kernel(CsrView g, const int64_t* gstart, GroupItem* witems, GroupItem* bitems,
                                   int* counters, ItemShape sh, int64_t clip0, int64_t clip1) {
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  int64_t n_pad = (g.n + 31) & ~31ll;
  for (int64_t h = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; h < n_pad; h += stride) {
    int64_t b = 0, e = 0, hb = 0, dh = 0;
    if (h < g.n) {
      b = max(gstart[h], clip0);
      e = min(gstart[h + 1], clip1);
      hb = g.off[h];
      dh = g.off[h + 1] - hb;
    }
    const bool any = e > b;
    const bool warp = dh <= sh.warp_max;
    const int kw = any && warp ? (int)((e - b + sh.warp_chunk - 1) / sh.warp_chunk) : 0;
    const int kb = any && !warp ? (int)((e - b + sh.block_chunk - 1) / sh.block_chunk) : 0;
    const int atw = warp_reserve(&counters[0], kw);
    const int atb = warp_reserve(&counters[1], kb);
    if (kw) {
      int32_t mode = dh <= sh.cutover ? 0 : 1;
      for (int c = 0; c < kw; ++c)
        witems[atw + c] = GroupItem{(int32_t)h, mode, b + c * (int64_t)sh.warp_chunk,
                                    min(e, b + (c + 1) * (int64_t)sh.warp_chunk)};
    }
    if (kb) {
      int32_t span = g.cols[hb + dh - 1] - g.cols[hb];
      int32_t mode = dh <= kHashMax ? 0 : (span < kTabWords * 32 ? 1 : 2);
      atomicMax(&counters[3], mode == 0 ? (int)dh : kHashMax);
      for (int c = 0; c < kb; ++c)
        bitems[atb + c] = GroupItem{(int32_t)h, mode, b + c * (int64_t)sh.block_chunk,
                                    min(e, b + (c + 1) * (int64_t)sh.block_chunk)};
    }
  }
}

// Where the counting kernels read their work items from.  FullItems: the explicit
// items of the single-graph path.  CompactItems (batches): 8-byte (h, chunk) pairs,
// warp items from the front of one array and block items from its back, decoded with
// the group starts and the item shape.
struct FullItems {
  static constexpr bool kBatch = false;  // one graph: counts go to the kernel's counter
  static constexpr int kMinBlocks = 0;  // no occupancy hint (the register choice measured fastest)
  const GroupItem* p;
  __device__ __forceinline__ GroupItem get(const CsrView&, int i) const { return p[i]; }
};

struct CompactItems {
  static constexpr bool kBatch = true;  // a batch: counts go to each item's graph
  static constexpr int kMinBlocks = 6;    // 40 registers: 6 CTAs of 256 threads per SM
  const int2* p;
  const int64_t* gstart;
  int64_t cap;
  bool from_back;  // items stored from the back of p (the block items of lists up to kBlockSmallList)
  bool block;      // block items
  ItemShape sh;
  __device__ __forceinline__ GroupItem get(const CsrView& g, int i) const {
    int2 c = from_back ? p[cap - 1 - i] : p[i];
    int64_t b0 = gstart[c.x], e0 = gstart[c.x + 1];
    int64_t chunk = block ? sh.block_chunk : sh.warp_chunk;
    int64_t b = b0 + (int64_t)c.y * chunk, e = min(e0, b + chunk);
    int64_t hb = g.off[c.x], dh = g.off[c.x + 1] - hb;
    int32_t mode;
    if (!block) {
      mode = dh <= sh.cutover ? 0 : 1;
    } else {
      int32_t span = g.cols[hb + dh - 1] - g.cols[hb];
      mode = dh <= kHashMax ? 0 : (span < kTabWords * 32 ? 1 : 2);
    }
    return GroupItem{c.x, mode, b, e};
  }
};

// Grouping passes for a CSR without the per-edge source array.  A warp takes a block of
// 32 consecutive rows, whose edges are contiguous in cols, and deals them 32 per round;
// each lane finds the row of its edge by a 5-step search over the lanes' row starts,
// done with shuffles.  Every lane has an edge in every round but the last, whatever the
// row lengths (a warp per row would leave most lanes idle on short rows).  Same grouping
// rule as the per-edge passes.  f(u, v, du, dv, valid) is called by all 32 lanes.
// skip (nullable): rows u with skip[u] != 0 are passed over; a block of 32 such rows is not
// read at all (the graphs of a batch are contiguous vertex ranges).
// queue (nullable, zeroed): row blocks are handed out in order from this counter,
// kRowGrab at a time, instead of by a grid stride.  Over a union of many graphs the warps
// of a grid stride drift apart by many graphs' worth of rows, and the random reads of
// degrees and group counters then spread over all of them; the queue keeps every warp
// within a few graphs.
constexpr int kRowGrab = 4;
template <class F>
__device__ __forceinline__ void for_row_block_edges(const CsrView& g, F f, const uint8_t* skip = nullptr,
                                                    int* queue = nullptr) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const int64_t blocks = (g.n + 31) >> 5;
  int64_t rb = queue ? 0 : (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5, lim = 0;
  for (;; rb = queue ? rb + 1 : rb + warps) {
    if (queue && rb >= lim) {
      int base = 0;
      if (lane == 0) base = atomicAdd(queue, kRowGrab);
      rb = __shfl_sync(0xffffffffu, base, 0);
      lim = rb + kRowGrab;
    }
    if (rb >= blocks) break;
    const int64_t u0 = rb << 5;
    const int64_t row = u0 + lane;
    const int64_t last = min(u0 + 32, g.n);
    if (skip && __all_sync(0xffffffffu, row >= last || skip[row])) continue;
    const int64_t start = __ldg(g.off + min(row, last));  // rows past the end start at the block's end
    const int64_t stop = __shfl_sync(0xffffffffu, __ldg(g.off + last), 0);
    const int64_t first = __shfl_sync(0xffffffffu, start, 0);
    for (int64_t t0 = first; t0 < stop; t0 += 32) {
      const int64_t e = t0 + lane;
      // k = the last lane whose row starts at or before e
      int k = 0;
#pragma unroll
      for (int step = 16; step > 0; step >>= 1) {
        const int64_t sk = __shfl_sync(0xffffffffu, start, k + step);
        if (sk <= e) k += step;
      }
      const int64_t su = __shfl_sync(0xffffffffu, start, k);
      const int64_t eu = __shfl_sync(0xffffffffu, start, (k + 1) & 31);
      const bool valid = e < stop;
      int32_t u = (int32_t)(u0 + k), v = 0;
      int64_t du = (k == 31 ? stop : eu) - su, dv = 0;
      if (valid) {
        v = __ldg(g.cols + e);
        dv = __ldg(g.off + v + 1) - __ldg(g.off + v);
      }
      f(u, v, du, dv, valid && du > 0 && dv > 0);
    }
  }
}

// skip (nullable): rows u with skip[u] != 0 are not grouped (their graph counts by rows).
__global__ void group_count_vc_kernel(CsrView g, int32_t* cnt, const uint8_t* skip, int* queue) {
  for_row_block_edges(g, [&](int32_t u, int32_t v, int64_t du, int64_t dv, bool ok) {
    if (skip && ok) ok = !skip[u];
    const int32_t h = ok ? (longer_is_u(u, v, du, dv) ? u : v) : -1;
    const unsigned same = __match_any_sync(0xffffffffu, h);
    if (h >= 0 && (int)(threadIdx.x & 31) == __ffs(same) - 1) atomicAdd(&cnt[h], __popc(same));
  }, skip, queue);
}

__global__ void group_scatter_vc_kernel(CsrView g, const int64_t* gstart, int32_t* cur, int32_t* plist,
                                        const uint8_t* skip, int* queue) {
  const int lane = threadIdx.x & 31;
  for_row_block_edges(g, [&](int32_t u, int32_t v, int64_t du, int64_t dv, bool ok) {
    if (skip && ok) ok = !skip[u];
    int32_t h = -1, p = 0;
    if (ok) {
      const bool hu = longer_is_u(u, v, du, dv);
      h = hu ? u : v;
      p = hu ? v : u;
    }
    const unsigned same = __match_any_sync(0xffffffffu, h);
    const int lead = __ffs(same) - 1;
    int at = 0;
    if (h >= 0 && lane == lead) at = atomicAdd(&cur[h], __popc(same));
    at = __shfl_sync(0xffffffffu, at, lead);
    if (h >= 0) plist[gstart[h] + at + __popc(same & ((1u << lane) - 1))] = p;
  }, skip, queue);
}

// Compact items: counters[0] warp items (front of `items`), counters[1] block items of lists
// up to kBlockSmallList (back of `items`), counters[2] block items of longer lists (front of
// `big`), counters[3] longest list among the block items in `items`.  sel (nullable): only
// vertices h with sel[h] == want get items.
__global__ void group_items_compact_kernel(CsrView g, const int64_t* gstart, int2* items, int64_t cap, int2* big,
                                           int* counters, ItemShape sh, const uint8_t* sel, uint8_t want) {
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  int64_t n_pad = (g.n + 31) & ~31ll;
  for (int64_t h = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; h < n_pad; h += stride) {
    int64_t b = 0, e = 0, dh = 0;
    if (h < g.n && (!sel || sel[h] == want)) {
      b = gstart[h];
      e = gstart[h + 1];
      dh = g.off[h + 1] - g.off[h];
    }
    const bool any = e > b;
    const bool warp = dh <= sh.warp_max;
    const int kw = any && warp ? (int)((e - b + sh.warp_chunk - 1) / sh.warp_chunk) : 0;
    const int kb = any && !warp ? (int)((e - b + sh.block_chunk - 1) / sh.block_chunk) : 0;
    const bool large = dh > kBlockSmallList;
    const int atw = warp_reserve(&counters[0], kw);
    const int atb = warp_reserve(&counters[1], large ? 0 : kb);
    const int atl = warp_reserve(&counters[2], large ? kb : 0);
    for (int c = 0; c < kw; ++c) items[(int64_t)atw + c] = make_int2((int32_t)h, c);
    if (kb && !large) atomicMax(&counters[3], (int)dh);
    for (int c = 0; c < kb; ++c) {
      if (large) big[(int64_t)atl + c] = make_int2((int32_t)h, c);
      else items[cap - 1 - ((int64_t)atb + c)] = make_int2((int32_t)h, c);
    }
  }
}

// Per-graph attribution for a batch of graphs stored as one disjoint union: vertex
// ranges [vbase[g], vbase[g+1]) belong to graph g; counts[g] receives its triangles.
// counts == nullptr: a single graph, everything goes to the kernel's `out` counter.
struct GraphTags {
  const int64_t* vbase;
  int ngraphs;
  unsigned long long* counts;
};

__device__ __forceinline__ int graph_of(const GraphTags& t, int64_t v) {
  int lo = 0, hi = t.ngraphs;  // last g with vbase[g] <= v
  while (hi - lo > 1) {
    int mid = (lo + hi) >> 1;
    if (t.vbase[mid] <= v) lo = mid; else hi = mid;
  }
  return lo;
}

// Per-warp attribution of counts to the graphs of a batch.  The warp keeps the graph of
// its last item, that graph's vertex range and its running count in shared memory (no
// registers held across the item), and flushes the count (one atomic) only when an item
// of another graph comes or the kernel ends.  A warp takes items in increasing index
// order, which is vertex order, so the graph lookup (a binary search over the graph
// starts) runs about once per graph instead of once per item.  All 32 lanes call add and
// flush; h is the same on every lane.
struct GraphAccSlot {
  int g;
  int32_t lo, hi;
  unsigned long long part;
};
__device__ __forceinline__ void graph_acc_init(GraphAccSlot* a) {
  if ((threadIdx.x & 31) == 0) *a = GraphAccSlot{-1, 0, 0, 0ull};
  __syncwarp();
}
__device__ __forceinline__ void graph_acc_flush(const GraphTags& t, GraphAccSlot* a) {
  if ((threadIdx.x & 31) == 0 && a->part && a->g >= 0) atomicAdd(&t.counts[a->g], a->part);
  __syncwarp();
}
__device__ __forceinline__ void graph_acc_add(const GraphTags& t, GraphAccSlot* a, int64_t h, unsigned c) {
  unsigned long long w = c;
  for (int o = 16; o > 0; o >>= 1) w += __shfl_xor_sync(0xffffffffu, w, o);
  if ((threadIdx.x & 31) == 0) {
    if (h < a->lo || h >= a->hi) {
      if (a->part && a->g >= 0) atomicAdd(&t.counts[a->g], a->part);
      const int g = graph_of(t, h);
      *a = GraphAccSlot{g, (int32_t)t.vbase[g], (int32_t)t.vbase[g + 1], 0ull};
    }
    a->part += w;
  }
  __syncwarp();
}


// Hash tables of N+(h): linear probing over buckets of S slots (S = 1, 2 or 4; 4-, 8- or
// 16-byte aligned), empty slots hold -1.  The home bucket of x is given by Fibonacci
// hashing: the top log2(buckets) bits of x * 2^32/phi.  The low bits of that product
// depend only on the low bits of x, and neighbour ids after relabelling share low-bit
// patterns, which clustered the tables (22 % of the hits at R-MAT scale 24 were not in
// their home slot); the top bits mix all of x.
//
// A key goes into the first empty slot at or after the first slot of its home bucket
// (slots in order, wrapping), so within a bucket the slots fill in order and the last
// slot of a bucket is empty only if no key ever passed over the bucket.  A lookup reads
// a whole bucket with one shared load and is settled by a match or by an empty last
// slot; otherwise it goes on with the next bucket.  Keys are only emptied after every
// lookup of an item is done.
template <int S>
__device__ __forceinline__ uint32_t hash_home(int32_t x, uint32_t mask) {
  constexpr int kLogS = S == 1 ? 0 : (S == 2 ? 1 : 2);
  return (((uint32_t)x * 0x9E3779B1u) >> (32 - (__popc(mask) - kLogS))) * S;
}

// Inserts x (not yet present); concurrent inserters use atomicCAS.
template <int S>
__device__ __forceinline__ void hash_insert(int32_t* tab, uint32_t mask, int32_t x) {
  uint32_t s = hash_home<S>(x, mask);
  for (uint32_t n = 0; n <= mask; ++n) {
    if (atomicCAS(&tab[s], -1, x) == -1) return;
    s = (s + 1) & mask;
  }
}

// Empties the slot holding x (x present); keys are cleared only by the thread that
// inserted them, so the walk always reaches x.
template <int S>
__device__ __forceinline__ void hash_erase(int32_t* tab, uint32_t mask, int32_t x) {
  uint32_t s = hash_home<S>(x, mask);
  for (uint32_t n = 0; n <= mask; ++n) {
    if (tab[s] == x) { tab[s] = -1; return; }
    s = (s + 1) & mask;
  }
}

// Reads the bucket at slot `at`: returns whether x is in it; *stop = its last slot is empty.
template <int S>
__device__ __forceinline__ bool bucket_has(const int32_t* tab, uint32_t at, int32_t x, bool* stop) {
  if constexpr (S == 1) {
    const int32_t y = tab[at];
    *stop = y == -1;
    return y == x;
  } else if constexpr (S == 2) {
    const int2 y = *reinterpret_cast<const int2*>(tab + at);
    *stop = y.y == -1;
    return (y.x == x) | (y.y == x);
  } else {
    const int4 y = *reinterpret_cast<const int4*>(tab + at);
    *stop = y.w == -1;
    return (y.x == x) | (y.y == x) | (y.z == x) | (y.w == x);
  }
}

// Probers: what stream_partners does with each element.  probe(x, valid) is called by
// all 32 lanes together (valid = false on lanes without an element) and returns this
// lane's hits; finish() returns hits still pending when an item ends.
template <class F>
struct DirectProber {  // a branch-light test per element (sorted search, bitmap)
  F f;
  __device__ __forceinline__ unsigned probe(int32_t x, bool valid) { return valid ? f(x) : 0u; }
  __device__ __forceinline__ unsigned finish() { return 0u; }
};
template <class F>
__device__ __forceinline__ DirectProber<F> direct_prober(F f) { return DirectProber<F>{f}; }

// Hash lookups with the chains taken out of the warp's lockstep.  Every key reads its
// home bucket; a key that is neither there nor stopped by an empty last slot is queued
// (key, next bucket, steps) in the warp's 64-entry shared queue, and whenever 32 are
// queued the warp advances all of them one bucket together.  A lookup loop per lane
// would make the whole warp wait for its longest chain.
template <int S>
struct HashQueueProber {
  const int32_t* tab;
  uint32_t mask;
  int32_t* qx;   // 64 keys
  uint32_t* qs;  // 64 (next slot | steps << 16)
  int n;         // queued entries, the same on every lane
  int lane;
  __device__ __forceinline__ void push(bool pend, int32_t x, uint32_t next) {
    const unsigned pm = __ballot_sync(0xffffffffu, pend);
    if (pm) {
      if (pend) {
        const int pos = n + __popc(pm & ((1u << lane) - 1));
        qx[pos] = x;
        qs[pos] = next;
      }
      n += __popc(pm);
    }
  }
  // one bucket further for up to 32 queued keys (the newest); unresolved ones go back
  __device__ __forceinline__ unsigned step() {
    const int take = n < 32 ? n : 32;
    const int base = n - take;
    __syncwarp();
    const bool v = lane < take;
    int32_t x = 0;
    uint32_t q = 0;
    if (v) {
      x = qx[base + lane];
      q = qs[base + lane];
    }
    __syncwarp();
    n = base;
    unsigned hit = 0;
    bool pend = false;
    const uint32_t slot = q & 0xffffu, steps = q >> 16;
    if (v) {
      bool stop;
      hit = bucket_has<S>(tab, slot, x, &stop);
      // a key that walked every bucket is absent (cannot happen below load 1)
      pend = !hit && !stop && steps * S < mask;
    }
    push(pend, x, ((slot + S) & mask) | ((steps + 1) << 16));
    return hit;
  }
  __device__ __forceinline__ unsigned probe(int32_t x, bool valid) {
    unsigned hit = 0;
    bool pend = false;
    uint32_t s = 0;
    if (valid) {
      s = hash_home<S>(x, mask);
      bool stop;
      hit = bucket_has<S>(tab, s, x, &stop);
      pend = !hit && !stop;
    }
    push(pend, x, ((s + S) & mask) | (1u << 16));
    while (n >= 32) hit += step();
    return hit;
  }
  __device__ __forceinline__ unsigned finish() {
    unsigned hit = 0;
    while (n > 0) hit += step();
    __syncwarp();
    return hit;
  }
};

// Streams the lists of the partners plist[base, base+32) for every batch start `base`
// that `next_batch()` hands out (until it reaches i1) through the prober, and returns
// the hits.  Lists of 32 or more elements are walked by the whole warp, one list at a
// time, four coalesced loads in flight per lane.  Shorter lists are laid end to end by
// a warp prefix sum of their lengths and dealt 32 elements per round; each lane finds
// the list holding its element by a 5-step binary search over the lanes' start offsets,
// done with shuffles so that every lane runs the same steps.  Every probe call is made
// by all 32 lanes together.
template <class NextBatch, class Prober>
__device__ __forceinline__ unsigned stream_partners(const CsrView& g, const int32_t* __restrict__ plist, int64_t i1,
                                                    int lane, NextBatch next_batch, Prober& pr) {
  unsigned cnt = 0;
  for (int64_t base = next_batch(); base < i1; base = next_batch()) {
    int64_t i = base + lane;
    int len = 0;
    int64_t pb = 0;
    if (i < i1) {
      int32_t p = __ldg(plist + i);
      pb = __ldg(g.off + p);
      len = (int)(__ldg(g.off + p + 1) - pb);
    }
    unsigned longm = __ballot_sync(0xffffffffu, len >= 32);
    while (longm) {
      const int k = __ffs(longm) - 1;
      longm &= longm - 1;
      const int32_t* P = g.cols + __shfl_sync(0xffffffffu, pb, k);
      const int ln = __shfl_sync(0xffffffffu, len, k);
      int j0 = 0;
      for (; j0 + 128 <= ln; j0 += 128) {
        const int32_t x0 = __ldg(P + j0 + lane), x1 = __ldg(P + j0 + 32 + lane), x2 = __ldg(P + j0 + 64 + lane),
                      x3 = __ldg(P + j0 + 96 + lane);
        cnt += pr.probe(x0, true);
        cnt += pr.probe(x1, true);
        cnt += pr.probe(x2, true);
        cnt += pr.probe(x3, true);
      }
      for (; j0 < ln; j0 += 32) {
        const bool v = j0 + lane < ln;
        cnt += pr.probe(v ? __ldg(P + j0 + lane) : 0, v);
      }
    }
    const int slen = len < 32 ? len : 0;
    int incl = slen;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int y = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += y;
    }
    const int total = __shfl_sync(0xffffffffu, incl, 31);
    const int start = incl - slen;
    for (int t0 = 0; t0 < total; t0 += 32) {
      const int t = t0 + lane;
      // k = the last lane whose start is <= t: a lane with a non-empty short list
      int k = 0;
#pragma unroll
      for (int step = 16; step > 0; step >>= 1) {
        const int sk = __shfl_sync(0xffffffffu, start, k + step);
        if (sk <= t) k += step;
      }
      const int64_t kp = __shfl_sync(0xffffffffu, pb, k);
      const int kx = __shfl_sync(0xffffffffu, start, k);
      const bool v = t < total;
      cnt += pr.probe(v ? __ldg(g.cols + kp + (t - kx)) : 0, v);
    }
  }
  cnt += pr.finish();
  return cnt;
}

// nitems_dev (nullable): the item count read from device memory instead of `nitems`.
template <class Items, int S = 1>
__global__ void __launch_bounds__(kBgWarps * 32, Items::kMinBlocks) bisson_warp_kernel(CsrView g, const int32_t* __restrict__ plist,
                                                                  Items items, int nitems,
                                                                  const int* nitems_dev, int* next, GraphTags tags,
                                                                  unsigned long long* out) {
  __shared__ __align__(16) int32_t tab[kBgWarps][kWarpSlots];
  __shared__ int32_t qx[kBgWarps][64];
  __shared__ uint32_t qs[kBgWarps][64];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int j = lane; j < kWarpSlots; j += 32) tab[w][j] = -1;
  __syncwarp();
  unsigned long long total = 0;
  __shared__ GraphAccSlot acc[kBgWarps];
  if constexpr (Items::kBatch) graph_acc_init(&acc[w]);
  int32_t* T = tab[w];
  if (nitems_dev) nitems = *nitems_dev;
  // batch items are taken kWarpGrab at a time (one atomic): most of them are tiny
  constexpr int grab = Items::kBatch ? kWarpGrab : 1;
  int it = 0, it_end = 0;
  for (;;) {
    if (it == it_end) {
      int first = 0;
      if (lane == 0) first = atomicAdd(next, grab);
      it = __shfl_sync(0xffffffffu, first, 0);
      it_end = min(it + grab, nitems);
    }
    if (it >= nitems) break;
    const GroupItem gi = items.get(g, it++);
    const int64_t hb = g.off[gi.h];
    const int dh = (int)(g.off[gi.h + 1] - hb);
    int64_t cur = gi.b;
    auto nb = [&]() { int64_t r = cur; cur += 32; return r; };
    unsigned cnt;
    if (gi.mode == 0) {
      for (int j = lane; j < dh; j += 32) T[j] = __ldg(g.cols + hb + j);
      __syncwarp();
      auto pr = direct_prober([&](int32_t x) -> unsigned {
        int lo = 0, n = dh;
        while (n > 1) {  // branch-free lower bound over the sorted copy
          int half = n >> 1;
          lo = T[lo + half - 1] < x ? lo + half : lo;
          n -= half;
        }
        return T[lo] == x;
      });
      cnt = stream_partners(g, plist, gi.e, lane, nb, pr);
      __syncwarp();
      for (int j = lane; j < dh; j += 32) T[j] = -1;
    } else {
      uint32_t cap = 64;  // load 1/4, or up to 1/2 for lists longer than kWarpSlots / 4
      while (cap < 4u * (uint32_t)dh && cap < (uint32_t)kWarpSlots) cap <<= 1;
      const uint32_t mask = cap - 1;
      for (int j = lane; j < dh; j += 32) hash_insert<S>(T, mask, __ldg(g.cols + hb + j));
      __syncwarp();
      HashQueueProber<S> pr{T, mask, qx[w], qs[w], 0, lane};
      cnt = stream_partners(g, plist, gi.e, lane, nb, pr);
      __syncwarp();
      for (int j = lane; j < dh; j += 32) hash_erase<S>(T, mask, __ldg(g.cols + hb + j));
    }
    __syncwarp();
    if constexpr (Items::kBatch) graph_acc_add(tags, &acc[w], gi.h, cnt);
    else total += cnt;
  }
  if constexpr (Items::kBatch) graph_acc_flush(tags, &acc[w]);
  warp_add_count(total, out);
}

template <class Items, int S = 1>
__global__ void __launch_bounds__(kBgWarps * 32, Items::kMinBlocks) bisson_block_kernel(CsrView g, const int32_t* __restrict__ plist,
                                                                   Items items, int nitems,
                                                                   const int* nitems_dev, int* next, uint32_t tab_words,
                                                                   GraphTags tags, unsigned long long* out) {
  extern __shared__ __align__(16) int32_t tab[];  // tab_words
  __shared__ int32_t qx[kBgWarps][64];
  __shared__ uint32_t qs[kBgWarps][64];
  __shared__ int cur_item;
  __shared__ unsigned long long bnext;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (uint32_t j = threadIdx.x; j < tab_words; j += blockDim.x) tab[j] = -1;
  unsigned long long total = 0;
  __shared__ GraphAccSlot acc[kBgWarps];
  if constexpr (Items::kBatch) graph_acc_init(&acc[w]);
  if (nitems_dev) nitems = *nitems_dev;
  for (;;) {
    if (threadIdx.x == 0) {
      cur_item = atomicAdd(next, 1);
      bnext = 0;
    }
    __syncthreads();
    const int it = cur_item;
    if (it >= nitems) break;
    const GroupItem gi = items.get(g, it);
    const int64_t hb = g.off[gi.h];
    const int64_t dh = g.off[gi.h + 1] - hb;
    const int32_t* Nh = g.cols + hb;
    // partner batches of 32 handed out to the warps as they finish
    auto nb = [&]() {
      unsigned long long r = 0;
      if (lane == 0) r = atomicAdd(&bnext, 32ull);
      return gi.b + (int64_t)__shfl_sync(0xffffffffu, r, 0);
    };
    unsigned cnt = 0;
    if (gi.mode == 0) {
      uint32_t cap = 64;
      while (cap < 4u * (uint32_t)dh) cap <<= 1;
      const uint32_t mask = cap - 1;
      for (int64_t j = threadIdx.x; j < dh; j += blockDim.x) hash_insert<S>(tab, mask, Nh[j]);
      __syncthreads();
      HashQueueProber<S> pr{tab, mask, qx[w], qs[w], 0, lane};
      cnt = stream_partners(g, plist, gi.e, lane, nb, pr);
      __syncthreads();
      for (int64_t j = threadIdx.x; j < dh; j += blockDim.x) hash_erase<S>(tab, mask, Nh[j]);
    } else if (gi.mode == 1) {
      const int32_t lo = Nh[0], hi = Nh[dh - 1];
      const int words = ((hi - lo) >> 5) + 1;
      uint32_t* bits = reinterpret_cast<uint32_t*>(tab);
      for (int j = threadIdx.x; j < words; j += blockDim.x) bits[j] = 0u;
      __syncthreads();
      for (int64_t j = threadIdx.x; j < dh; j += blockDim.x) {
        int32_t x = Nh[j] - lo;
        atomicOr(&bits[x >> 5], 1u << (x & 31));
      }
      __syncthreads();
      auto pr = direct_prober([&](int32_t x) -> unsigned {
        if (x < lo || x > hi) return 0u;
        x -= lo;
        return (bits[x >> 5] >> (x & 31)) & 1u;
      });
      cnt = stream_partners(g, plist, gi.e, lane, nb, pr);
      __syncthreads();
      for (int j = threadIdx.x; j < words; j += blockDim.x) bits[j] = 0xffffffffu;  // back to empty slots (-1)
    } else {
      auto pr = direct_prober([&](int32_t x) -> unsigned {
        int64_t lo = 0, hi = dh;
        while (lo < hi) {
          int64_t mid = (lo + hi) >> 1;
          if (Nh[mid] < x) lo = mid + 1; else hi = mid;
        }
        return lo < dh && Nh[lo] == x;
      });
      cnt = stream_partners(g, plist, gi.e, lane, nb, pr);
    }
    __syncthreads();
    if constexpr (Items::kBatch) graph_acc_add(tags, &acc[w], gi.h, cnt);
    else total += cnt;
  }
  if constexpr (Items::kBatch) graph_acc_flush(tags, &acc[w]);
  warp_add_count(total, out);
}

}  // namespace

}  // namespace atc
