// preTC on the GPU: raw int32 pairs -> simple graph -> [A-order relabel] -> orientation
// -> [degree<=1 pruning] -> oriented CSR resident in HBM.
//
// Stands in for preProcess() of Hu/Bisson/Fox (Hu/preTC.cu:64-296, Bisson/preTC.cu:77-293,
// Fox/preTC.cu:64-208) and TriCore's cal_degree / redirect_edges / split
// (tricore/src/tricount_gpu.cu:49-203).  Where the reference sorts edges in host buckets
// and merges them into CSR on one CPU thread, everything here stays on the device:
// 64-bit (src << B | dst) keys are radix-sorted once and the CSR offsets are read off
// the sorted keys.
#include <climits>
#include <cstdio>
#include <cstring>
#include <exception>
#include <vector>

#include "internal.cuh"

namespace atc {

namespace {

constexpr uint64_t kSentinel = ~0ull;

__global__ void minmax_kernel(const int2* p, uint64_t np, int* mn, int* mx) {
  int lo = INT_MAX, hi = INT_MIN;
  uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < np; i += stride) {
    int2 e = p[i];
    lo = min(lo, min(e.x, e.y));
    hi = max(hi, max(e.x, e.y));
  }
  for (int o = 16; o > 0; o >>= 1) {
    lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMin(mn, lo);
    atomicMax(mx, hi);
  }
}

__global__ void canon_kernel(const int2* p, uint64_t np, int B, uint64_t* keys) {
  uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < np; i += stride) {
    int2 e = p[i];
    if (e.x == e.y) {
      keys[i] = kSentinel;
    } else {
      uint64_t lo = (uint32_t)min(e.x, e.y), hi = (uint32_t)max(e.x, e.y);
      keys[i] = (lo << B) | hi;
    }
  }
}

// Degrees of the simple graph from its sorted keys.  Keys of one smaller endpoint are
// contiguous, so a warp adds each run of them with one atomic (the loop is padded to whole
// warps for __match_any_sync); the larger endpoints are scattered.
__global__ void degree_kernel(const uint64_t* keys, int64_t m, int B, int32_t* deg) {
  const uint64_t mask = (1ull << B) - 1;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const int64_t m_pad = (m + 31) & ~31ll;
  const int lane = threadIdx.x & 31;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m_pad; i += stride) {
    int64_t lo = -1;
    if (i < m) {
      const uint64_t k = keys[i];
      lo = (int64_t)(k >> B);
      atomicAdd(&deg[k & mask], 1);
    }
    const unsigned same = __match_any_sync(0xffffffffu, lo);
    if (lo >= 0 && lane == __ffs(same) - 1) atomicAdd(&deg[lo], __popc(same));
  }
}

// Both directions of every simple edge (a < b): (a, b) at 2i, (b, a) at 2i+1.
__global__ void both_directions_kernel(const uint64_t* keys, int64_t m, int B, int2* out) {
  const uint64_t mask = (1ull << B) - 1;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
    const int32_t a = (int32_t)(keys[i] >> B), b = (int32_t)(keys[i] & mask);
    out[2 * i] = make_int2(a, b);
    out[2 * i + 1] = make_int2(b, a);
  }
}

struct OrientArgs {
  const int32_t* deg;   // simple degree, by input id
  const int32_t* prio;  // A-direction priority / core number / peel flag, by input id
  const uint32_t* minor;  // approximate peel's minor priority (ADIRECTION_PAR only)
  const int32_t* perm;  // new id of every input id (A-order), or null
  const int32_t* cmap;  // compacted id of every (new) id when pruning, or null
  int dir;
  int bin;              // B of the input keys
  int bout;             // B of the output keys
};

// Orientation rules (each decides src for the edge {x, y}; input ids x, y, new ids xn, yn):
//   ID            src = larger id                       Bisson/preTC.cu:135-144, Fox/preTC.cu:94-98
//   DEGREE        lower degree; tie -> larger id        Hu/preTC.cu:125-133, A-order.cpp:91-96
//   DEGREE_LOWID  lower degree; tie -> smaller id       tricount_gpu.cu:76-78
//   ADIRECTION    lower priority; tie -> smaller id     A-direction-seri.cpp:259-261
//   KCORE         lower core number; tie -> smaller id  kcore_direction.cpp:137-143
// The first three are the counting programs' own rules, applied to the ids they read (the
// relabelled ones, xn/yn).  The direction programs (ADIRECTION, KCORE, ADIRECTION_PAR) orient
// their input before any relabelling, so their ties use the input ids x/y: the relabelled
// graph is then exactly the program's output file relabelled by the ordering.
__global__ void orient_kernel(const uint64_t* ek, int64_t m, OrientArgs a, uint64_t* out,
                              unsigned long long* dropped) {
  uint64_t mask = (1ull << a.bin) - 1;
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  unsigned long long drop = 0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m; i += stride) {
    uint64_t k = ek[i];
    int32_t x = (int32_t)(k >> a.bin), y = (int32_t)(k & mask);
    int32_t dx = a.deg[x], dy = a.deg[y];
    if (a.cmap && (dx <= 1 || dy <= 1)) {
      out[i] = kSentinel;
      ++drop;
      continue;
    }
    int32_t xn = a.perm ? a.perm[x] : x, yn = a.perm ? a.perm[y] : y;
    bool x_src;
    switch (a.dir) {
      case ATC_DIR_ID: x_src = xn > yn; break;
      case ATC_DIR_DEGREE: x_src = dx < dy || (dx == dy && xn > yn); break;
      case ATC_DIR_DEGREE_LOWID: x_src = dx < dy || (dx == dy && xn < yn); break;
      case ATC_DIR_KCORE: {
        int32_t cx = a.prio[x], cy = a.prio[y];
        x_src = cx < cy || (cx == cy && x < y);
        break;
      }
      case ATC_DIR_ADIRECTION_PAR: {  // flags compare as int32 (0xFFFFFFFF = -1)
        int32_t fx = a.prio[x], fy = a.prio[y];
        int32_t mx = (int32_t)a.minor[x], my = (int32_t)a.minor[y];
        x_src = fx < fy || (fx == fy && (mx < my || (mx == my && x < y)));
        break;
      }
      default: {
        int32_t px = a.prio[x], py = a.prio[y];
        x_src = py > px || (py == px && x < y);
      }
    }
    int32_t s = x_src ? xn : yn, d = x_src ? yn : xn;
    if (a.cmap) {
      s = a.cmap[s];
      d = a.cmap[d];
    }
    out[i] = ((uint64_t)(uint32_t)s << a.bout) | (uint32_t)d;
  }
  for (int o = 16; o > 0; o >>= 1) drop += __shfl_xor_sync(0xffffffffu, drop, o);
  if ((threadIdx.x & 31) == 0 && drop) atomicAdd(dropped, drop);
}

// offsets[v] = first index whose source is >= v, for v in [0, n]; sentinels sort last.
__global__ void offsets_kernel(const uint64_t* k, int64_t m, int B, int64_t n, int64_t* off) {
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v <= n; v += stride) {
    int64_t lo = 0, hi = m;
    while (lo < hi) {
      int64_t mid = (lo + hi) >> 1;
      if ((int64_t)(k[mid] >> B) < v) lo = mid + 1; else hi = mid;
    }
    off[v] = lo;
  }
}

__global__ void split_kernel(const uint64_t* k, int64_t m, int B, int32_t* cols, int32_t* esrc) {
  uint64_t mask = (1ull << B) - 1;
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m; i += stride) {
    uint64_t x = k[i];
    cols[i] = (int32_t)(x & mask);
    esrc[i] = (int32_t)(x >> B);
  }
}

__global__ void indeg_kernel(const int32_t* cols, int64_t m, int32_t* indeg) {
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m; i += stride) atomicAdd(&indeg[cols[i]], 1);
}

__global__ void wedge_kernel(const int64_t* off, const int32_t* indeg, int64_t n, unsigned long long* w,
                             int* maxout) {
  unsigned long long s = 0;
  int mo = 0;
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n; v += stride) {
    int64_t d = off[v + 1] - off[v];
    s += (unsigned long long)indeg[v] * (unsigned long long)d;
    mo = max(mo, (int)d);
  }
  for (int o = 16; o > 0; o >>= 1) {
    s += __shfl_xor_sync(0xffffffffu, s, o);
    mo = max(mo, __shfl_xor_sync(0xffffffffu, mo, o));
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(w, s);
    atomicMax(maxout, mo);
  }
}

// sum over edges of min(outdeg(u), outdeg(v)): the elements a shorter-list-probing
// kernel must stream.
__global__ void wedge_min_kernel(const int64_t* off, const int32_t* cols, const int32_t* esrc, int64_t m,
                                 unsigned long long* out) {
  unsigned long long s = 0;
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m; i += stride) {
    int32_t u = esrc[i], v = cols[i];
    int64_t du = off[u + 1] - off[u], dv = off[v + 1] - off[v];
    s += (unsigned long long)(du < dv ? du : dv);
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(out, s);
}

__global__ void keep_kernel(const int32_t* deg, const int32_t* perm, int64_t n, int32_t* keep) {
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n; v += stride) {
    int32_t nv = perm ? perm[v] : (int32_t)v;
    keep[nv] = deg[v] >= 2 ? 1 : 0;
  }
}

__global__ void i64_to_i32_kernel(const int64_t* in, int64_t n, int32_t* out) {
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += stride) out[i] = (int32_t)in[i];
}

__global__ void iota_kernel(int32_t* p, int64_t n) {
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += stride) p[i] = (int32_t)i;
}

__global__ void keys_to_pairs_kernel(const uint64_t* k, int64_t m, int B, int2* out) {
  uint64_t mask = (1ull << B) - 1;
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m; i += stride)
    out[i] = make_int2((int32_t)(k[i] >> B), (int32_t)(k[i] & mask));
}

// Largest "hi" endpoint over canonical keys: the largest id that has an edge.
__global__ void max_hi_kernel(const uint64_t* k, int64_t m, int B, int* mx) {
  uint64_t mask = (1ull << B) - 1;
  int best = 0;
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m; i += stride)
    best = max(best, (int)(k[i] & mask));
  for (int o = 16; o > 0; o >>= 1) best = max(best, __shfl_xor_sync(0xffffffffu, best, o));
  if ((threadIdx.x & 31) == 0) atomicMax(mx, best);
}

void keep_pool() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return;
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, dev) != cudaSuccess) return;
  uint64_t thr = UINT64_MAX;
  cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
}

// Copies the input pairs from pinned host memory to the device with the SMs: every thread
// moves 16-byte pieces (two pairs) through the device's mapping of the host buffer over
// NVLink-C2C.  The copy engines, which cudaMemcpyAsync uses, were measured to slow down
// intermittently to ~20 GB/s on the GPU hosts after other processes had used and freed
// much of the device memory, while SM reads of the same pinned buffer kept their speed
// (about 200 GB/s, as a fast copy-engine transfer).
__global__ void copy_pairs_kernel(const int2* __restrict__ src, uint64_t np, int2* __restrict__ dst) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  const uint64_t i0 = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  const bool vec = ((reinterpret_cast<uintptr_t>(src) | reinterpret_cast<uintptr_t>(dst)) & 15) == 0;
  if (vec) {
    const uint64_t nq = np >> 1;
    const int4* s4 = reinterpret_cast<const int4*>(src);
    int4* d4 = reinterpret_cast<int4*>(dst);
    for (uint64_t i = i0; i < nq; i += stride) d4[i] = s4[i];
    if (i0 == 0 && (np & 1)) dst[np - 1] = src[np - 1];
  } else {
    for (uint64_t i = i0; i < np; i += stride) dst[i] = src[i];
  }
}

}  // namespace

atc_status build_simple_edges(const int2* pairs, uint64_t np, SimpleEdges* out, cudaStream_t s) {
  keep_pool();
  out->m = 0;
  out->n_in = 0;
  out->bits = 1;
  if (np == 0) return ATC_OK;
  DevBuf<int> mm;
  ATC_TRY(mm.alloc(2, s));
  int init[2] = {INT_MAX, INT_MIN};
  ATC_CK(cudaMemcpyAsync(mm.p, init, sizeof(init), cudaMemcpyHostToDevice, s));
  minmax_kernel<<<grid_for(np, 256), 256, 0, s>>>(pairs, np, mm.p, mm.p + 1);
  ATC_CK(cudaGetLastError());
  int h[2];
  ATC_CK(cudaMemcpyAsync(h, mm.p, sizeof(h), cudaMemcpyDeviceToHost, s));
  ATC_CK(cudaStreamSynchronize(s));
  if (h[0] < 0) {
    set_error("negative vertex id %d in the input pairs", h[0]);
    return ATC_ERR_INVALID;
  }
  out->n_in = (int64_t)h[1] + 1;
  out->bits = id_bits(out->n_in);
  DevBuf<uint64_t> a, b;
  ATC_TRY(a.alloc(np, s));
  ATC_TRY(b.alloc(np, s));
  canon_kernel<<<grid_for(np, 256), 256, 0, s>>>(pairs, np, out->bits, a.p);
  ATC_CK(cudaGetLastError());
  uint64_t* ka = a.p;
  uint64_t* kb = b.p;
  ATC_TRY(sort_keys_u64(ka, kb, np, 0, 2 * out->bits, s));
  size_t nu = 0;
  ATC_TRY(unique_u64(ka, kb, np, &nu, s));
  uint64_t last = 0;
  if (nu) {
    ATC_CK(cudaMemcpyAsync(&last, kb + nu - 1, sizeof(last), cudaMemcpyDeviceToHost, s));
    ATC_CK(cudaStreamSynchronize(s));
  }
  out->m = (int64_t)nu - (nu && last == kSentinel ? 1 : 0);
  // keep whichever buffer holds the unique keys
  if (kb == b.p) { out->keys = std::move(b); } else { out->keys = std::move(a); }
  return ATC_OK;
}

atc_status simple_degrees(const SimpleEdges& e, int32_t* deg, cudaStream_t s) {
  ATC_CK(cudaMemsetAsync(deg, 0, sizeof(int32_t) * e.n_in, s));
  if (e.m) degree_kernel<<<grid_for(e.m, 256), 256, 0, s>>>(e.keys.p, e.m, e.bits, deg);
  ATC_CK(cudaGetLastError());
  return ATC_OK;
}

static atc_status pretc_impl(const int2* pairs, uint64_t np, atc_dir dir, atc_order order, const atc_tuning* t,
                             atc_csr* out, int32_t* perm_out, cudaStream_t s) {
  ATC_CHECK_ARG(out != nullptr, "out is NULL");
  ATC_CHECK_ARG(dir >= ATC_DIR_ID && dir <= ATC_DIR_ADIRECTION_PAR, "unknown atc_dir");
  ATC_CHECK_ARG(order >= ATC_ORDER_NONE && order <= ATC_ORDER_RANDOM, "unknown atc_order");
  *out = atc_csr{};
  bool prune = t && t->prune_deg1;
  SimpleEdges e;
  std::optional<Phase> ph;
  ph.emplace("pretc.dedup", s);
  ATC_TRY(build_simple_edges(pairs, np, &e, s));
  ph.reset();
  int64_t n_in = e.n_in;
  DevBuf<int32_t> deg, prio, perm, cmap;
  DevBuf<uint32_t> minor;
  bool peeled = false;  // A-direction priorities computed already
  ph.emplace("pretc.degrees", s);
  ATC_TRY(deg.alloc(n_in, s));
  ATC_TRY(simple_degrees(e, deg.p, s));
  ph.reset();
  if (order != ATC_ORDER_NONE) {
    ph.emplace(order == ATC_ORDER_AORDER && dir == ATC_DIR_ADIRECTION ? "pretc.order+peel" : "pretc.order", s);
    // The relabelling programs see the simple graph with each edge once, as when they
    // read the output of A-direction-seri; their id range ends at the largest id that
    // has an edge.
    ATC_TRY(perm.alloc(n_in, s));
    iota_kernel<<<grid_for(n_in, 256), 256, 0, s>>>(perm.p, n_in);
    ATC_CK(cudaGetLastError());
    int64_t n_v = 0;
    if (e.m) {
      DevBuf<int> mx;
      ATC_TRY(mx.alloc(1, s));
      ATC_CK(cudaMemsetAsync(mx.p, 0, sizeof(int), s));
      max_hi_kernel<<<grid_for(e.m, 256), 256, 0, s>>>(e.keys.p, e.m, e.bits, mx.p);
      ATC_CK(cudaGetLastError());
      int h = 0;
      ATC_CK(cudaMemcpyAsync(&h, mx.p, sizeof(int), cudaMemcpyDeviceToHost, s));
      ATC_CK(cudaStreamSynchronize(s));
      n_v = (int64_t)h + 1;
    }
    if (order == ATC_ORDER_AORDER && dir == ATC_DIR_ADIRECTION) {
      // the peel does not depend on the relabelling: it runs on the device while the
      // host part of A-order runs
      ATC_TRY(prio.alloc(n_in, s));
      int waves = 0;
      const std::function<atc_status()> peel = [&] { return peel_priorities(e, deg.p, prio.p, &waves, s); };
      ATC_TRY(aorder_lookup(nullptr, e.keys.p, e.bits, (uint64_t)e.m, n_v, perm.p, nullptr, s, deg.p, &peel));
      peeled = true;
    } else if (order == ATC_ORDER_AORDER) {
      ATC_TRY(aorder_lookup(nullptr, e.keys.p, e.bits, (uint64_t)e.m, n_v, perm.p, nullptr, s, deg.p));
    } else if (order == ATC_ORDER_ADIRECTION_BISSON) {
      // the program numbers every id up to the largest one in its input (:213-219)
      ATC_TRY(bisson_adirection_lookup(e, deg.p, perm.p, s));
    } else if (order == ATC_ORDER_GRO) {
      // GRO of the undirected graph: both directions of every simple edge
      DevBuf<int2> sym;
      ATC_TRY(sym.alloc(2 * (size_t)e.m + 1, s));
      if (e.m) {
        both_directions_kernel<<<grid_for(e.m, 256), 256, 0, s>>>(e.keys.p, e.m, e.bits, sym.p);
        ATC_CK(cudaGetLastError());
      }
      ATC_TRY(gro_lookup(sym.p, 2 * (uint64_t)e.m, n_v, perm.p, s));
    } else {
      const int kind = order == ATC_ORDER_DEGREE_DESC    ? ATC_RELABEL_DEGREE_DESC
                       : order == ATC_ORDER_AORDER_V2    ? ATC_RELABEL_AORDER_V2
                       : order == ATC_ORDER_NAIVE_SHUFFLED ? ATC_RELABEL_NAIVE_SHUFFLED
                                                           : ATC_RELABEL_RANDOM;
      ATC_TRY(relabel_lookup(nullptr, e.keys.p, e.bits, (uint64_t)e.m, n_v, kind, perm.p, nullptr, s));
    }
    ph.reset();
  }
  ph.emplace("pretc.direction", s);
  if (dir == ATC_DIR_ADIRECTION && !peeled) {
    ATC_TRY(prio.alloc(n_in, s));
    int waves = 0;
    ATC_TRY(peel_priorities(e, deg.p, prio.p, &waves, s));
  } else if (dir == ATC_DIR_KCORE) {
    ATC_TRY(prio.alloc(n_in, s));
    ATC_TRY(core_numbers(e, deg.p, prio.p, s));
  } else if (dir == ATC_DIR_ADIRECTION_PAR) {
    ATC_TRY(prio.alloc(n_in, s));
    ATC_TRY(minor.alloc(n_in, s));
    ATC_TRY(approx_peel(e, deg.p, reinterpret_cast<uint32_t*>(prio.p), minor.p, nullptr, s));
  }
  ph.reset();
  int64_t n = n_in;
  if (prune) {
    ph.emplace("pretc.prune", s);
    DevBuf<int32_t> keep;
    DevBuf<int64_t> pre;
    ATC_TRY(keep.alloc(n_in + 1, s));
    ATC_TRY(pre.alloc(n_in + 1, s));
    ATC_CK(cudaMemsetAsync(keep.p, 0, sizeof(int32_t) * (n_in + 1), s));
    keep_kernel<<<grid_for(n_in, 256), 256, 0, s>>>(deg.p, perm.p, n_in, keep.p);
    ATC_CK(cudaGetLastError());
    ATC_TRY(exclusive_scan_i32_to_i64(keep.p, pre.p, n_in + 1, s));
    ATC_TRY(cmap.alloc(n_in + 1, s));
    i64_to_i32_kernel<<<grid_for(n_in + 1, 256), 256, 0, s>>>(pre.p, n_in + 1, cmap.p);
    ATC_CK(cudaGetLastError());
    int64_t kept = 0;
    ATC_CK(cudaMemcpyAsync(&kept, pre.p + n_in, sizeof(kept), cudaMemcpyDeviceToHost, s));
    ATC_CK(cudaStreamSynchronize(s));
    n = kept;
    ph.reset();
  }
  ph.emplace("pretc.orient+sort", s);
  int bout = id_bits(n);
  DevBuf<uint64_t> k1, k2;
  DevBuf<unsigned long long> dropped;
  ATC_TRY(k1.alloc(e.m, s));
  ATC_TRY(k2.alloc(e.m, s));
  ATC_TRY(dropped.alloc(1, s));
  ATC_CK(cudaMemsetAsync(dropped.p, 0, sizeof(unsigned long long), s));
  OrientArgs oa{deg.p, prio.p, minor.p, perm.p, cmap.p, (int)dir, e.bits, bout};
  if (e.m) orient_kernel<<<grid_for(e.m, 256), 256, 0, s>>>(e.keys.p, e.m, oa, k1.p, dropped.p);
  ATC_CK(cudaGetLastError());
  e.keys.release();
  uint64_t* ka = k1.p;
  uint64_t* kb = k2.p;
  ATC_TRY(sort_keys_u64(ka, kb, e.m, 0, 2 * bout, s));
  unsigned long long hdrop = 0;
  ATC_CK(cudaMemcpyAsync(&hdrop, dropped.p, sizeof(hdrop), cudaMemcpyDeviceToHost, s));
  ATC_CK(cudaStreamSynchronize(s));
  int64_t m = e.m - (int64_t)hdrop;
  ph.reset();
  ph.emplace("pretc.csr", s);

  // Own buffers of the CSR.  cols gets 16 ints of padding so that 16-byte-rounded bulk
  // copies of any list stay inside the allocation.
  DevBuf<int64_t> off;
  DevBuf<int32_t> cols, esrc, indeg;
  DevBuf<unsigned long long> counter;
  ATC_TRY(off.alloc(n + 1, s));
  ATC_TRY(cols.alloc(m + 16, s));
  ATC_TRY(esrc.alloc(m + 16, s));
  ATC_TRY(counter.alloc(4, s));
  ATC_CK(cudaMemsetAsync(cols.p + m, 0, sizeof(int32_t) * 16, s));
  offsets_kernel<<<grid_for(n + 1, 256), 256, 0, s>>>(ka, m, bout, n, off.p);
  ATC_CK(cudaGetLastError());
  if (m) split_kernel<<<grid_for(m, 256), 256, 0, s>>>(ka, m, bout, cols.p, esrc.p);
  ATC_CK(cudaGetLastError());
  // W = sum_v indeg(v) * outdeg(v) and the largest out-degree
  ATC_TRY(indeg.alloc(n + 1, s));
  ATC_CK(cudaMemsetAsync(indeg.p, 0, sizeof(int32_t) * (n + 1), s));
  ATC_CK(cudaMemsetAsync(counter.p, 0, sizeof(unsigned long long) * 4, s));
  if (m) indeg_kernel<<<grid_for(m, 256), 256, 0, s>>>(cols.p, m, indeg.p);
  if (n) wedge_kernel<<<grid_for(n, 256), 256, 0, s>>>(off.p, indeg.p, n, counter.p, (int*)(counter.p + 1));
  if (m) wedge_min_kernel<<<grid_for(m, 256), 256, 0, s>>>(off.p, cols.p, esrc.p, m, counter.p + 2);
  ATC_CK(cudaGetLastError());
  unsigned long long hw[3] = {0, 0, 0};
  ATC_CK(cudaMemcpyAsync(hw, counter.p, sizeof(hw), cudaMemcpyDeviceToHost, s));
  if (perm_out && order != ATC_ORDER_NONE && n_in)
    ATC_CK(cudaMemcpyAsync(perm_out, perm.p, sizeof(int32_t) * n_in, cudaMemcpyDeviceToHost, s));
  else if (perm_out && n_in) {
    std::vector<int32_t> id(n_in);
    for (int64_t i = 0; i < n_in; ++i) id[i] = (int32_t)i;
    std::copy(id.begin(), id.end(), perm_out);
  }
  ATC_CK(cudaStreamSynchronize(s));
  ph.reset();

  CsrPriv* pv = new CsrPriv();
  pv->esrc = esrc.detach();
  pv->counter = counter.detach();
  pv->bits = bout;
  out->n = n;
  out->m = m;
  out->offsets = off.detach();
  out->cols = cols.detach();
  out->n_input = n_in;
  out->wedges = (int64_t)hw[0];
  out->dir = (int32_t)dir;
  out->order = (int32_t)order;
  out->pruned = prune ? 1 : 0;
  out->max_outdeg = (int32_t)(hw[1] & 0xffffffffu);
  out->wedges_min = (int64_t)hw[2];
  out->priv = pv;
  return ATC_OK;
}

}  // namespace atc

using namespace atc;

extern "C" atc_status atc_pretc_device(const int32_t* pairs_dev, uint64_t np, atc_dir dir, atc_order order,
                                       const atc_tuning* t, atc_csr* out, int32_t* perm_out, atc_stream s) try {
  ATC_CHECK_ARG(np == 0 || pairs_dev != nullptr, "pairs_dev is NULL");
  Phase ph("pretc", as_stream(s));
  return pretc_impl(reinterpret_cast<const int2*>(pairs_dev), np, dir, order, t, out, perm_out, as_stream(s));
} ATC_CATCH

extern "C" atc_status atc_pretc(const int32_t* pairs, uint64_t np, atc_dir dir, atc_order order,
                                const atc_tuning* t, atc_csr* out, int32_t* perm_out, atc_stream s) try {
  ATC_CHECK_ARG(np == 0 || pairs != nullptr, "pairs is NULL");
  cudaStream_t st = as_stream(s);
  keep_pool();
  Phase ph("pretc", st);
  DevBuf<int2> d;
  {
    Phase ph_alloc("pretc.alloc", st);
    ATC_TRY(d.alloc(np, st));
  }
  {
    Phase ph_copy("pretc.h2d", st);
    // pinned (page-locked) host memory has a device mapping: the SMs copy it; pageable memory
    // goes through cudaMemcpyAsync
    cudaPointerAttributes attr{};
    const void* mapped = nullptr;
    if (np && cudaPointerGetAttributes(&attr, pairs) == cudaSuccess && attr.type == cudaMemoryTypeHost)
      mapped = attr.devicePointer;
    cudaGetLastError();  // a failed query only selects the copy path
    if (mapped) {
      copy_pairs_kernel<<<grid_for((int64_t)(np >> 1) + 1, 256, 16), 256, 0, st>>>(
          static_cast<const int2*>(mapped), np, d.p);
      ATC_CK(cudaGetLastError());
    } else if (np) {
      ATC_CK(cudaMemcpyAsync(d.p, pairs, sizeof(int2) * np, cudaMemcpyHostToDevice, st));
    }
  }
  return pretc_impl(d.p, np, dir, order, t, out, perm_out, st);
} ATC_CATCH

extern "C" atc_status atc_csr_to_host(const atc_csr* csr, int64_t* offsets, int32_t* cols, atc_stream s) try {
  ATC_CHECK_ARG(csr != nullptr && offsets != nullptr && cols != nullptr, "NULL argument");
  cudaStream_t st = as_stream(s);
  ATC_CK(cudaMemcpyAsync(offsets, csr->offsets, sizeof(int64_t) * (csr->n + 1), cudaMemcpyDeviceToHost, st));
  if (csr->m) ATC_CK(cudaMemcpyAsync(cols, csr->cols, sizeof(int32_t) * csr->m, cudaMemcpyDefault, st));
  ATC_CK(cudaStreamSynchronize(st));
  return ATC_OK;
} ATC_CATCH

extern "C" atc_status atc_csr_free(atc_csr* csr) try {
  if (!csr) return ATC_OK;
  CsrPriv* pv = static_cast<CsrPriv*>(csr->priv);
  const bool host = pv && pv->host_cols;
  if (csr->offsets) cudaFree(csr->offsets);
  if (host) {
    cudaFreeHost(pv->host_cols);
    if (pv->host_esrc) cudaFreeHost(pv->host_esrc);
  } else {
    if (csr->cols) cudaFree(csr->cols);
    if (pv && pv->esrc) cudaFree(pv->esrc);
  }
  if (pv) {
    if (pv->counter) cudaFree(pv->counter);
    delete pv;
  }
  *csr = atc_csr{};
  return ATC_OK;
} ATC_CATCH

// A-direction-seri as a library call: orient the simple graph by peel priority and emit
// the edges sorted by (src, dst) — the byte order of lpBasedGraph.bin (A-direction-seri.cpp:254-273).
extern "C" atc_status atc_adirection(const int32_t* pairs, uint64_t np, int32_t* oriented_out, uint64_t* n_out,
                                     int32_t* prio_out, atc_stream st) try {
  ATC_CHECK_ARG(n_out != nullptr, "n_out is NULL");
  ATC_CHECK_ARG(np == 0 || (pairs != nullptr && oriented_out != nullptr), "NULL array");
  cudaStream_t s = as_stream(st);
  keep_pool();
  *n_out = 0;
  DevBuf<int2> d;
  ATC_TRY(d.alloc(np, s));
  if (np) ATC_CK(cudaMemcpyAsync(d.p, pairs, sizeof(int2) * np, cudaMemcpyHostToDevice, s));
  SimpleEdges e;
  ATC_TRY(build_simple_edges(d.p, np, &e, s));
  d.release();
  if (e.n_in == 0) return ATC_OK;
  DevBuf<int32_t> deg, prio;
  ATC_TRY(deg.alloc(e.n_in, s));
  ATC_TRY(prio.alloc(e.n_in, s));
  ATC_TRY(simple_degrees(e, deg.p, s));
  int waves = 0;
  ATC_TRY(peel_priorities(e, deg.p, prio.p, &waves, s));
  DevBuf<uint64_t> k1, k2;
  DevBuf<unsigned long long> dropped;
  ATC_TRY(k1.alloc(e.m, s));
  ATC_TRY(k2.alloc(e.m, s));
  ATC_TRY(dropped.alloc(1, s));
  OrientArgs oa{deg.p, prio.p, nullptr, nullptr, nullptr, ATC_DIR_ADIRECTION, e.bits, e.bits};
  if (e.m) orient_kernel<<<grid_for(e.m, 256), 256, 0, s>>>(e.keys.p, e.m, oa, k1.p, dropped.p);
  ATC_CK(cudaGetLastError());
  uint64_t* ka = k1.p;
  uint64_t* kb = k2.p;
  ATC_TRY(sort_keys_u64(ka, kb, e.m, 0, 2 * e.bits, s));
  DevBuf<int2> o;
  ATC_TRY(o.alloc(e.m, s));
  if (e.m) keys_to_pairs_kernel<<<grid_for(e.m, 256), 256, 0, s>>>(ka, e.m, e.bits, o.p);
  ATC_CK(cudaGetLastError());
  if (e.m) ATC_CK(cudaMemcpyAsync(oriented_out, o.p, sizeof(int2) * e.m, cudaMemcpyDeviceToHost, s));
  if (prio_out) ATC_CK(cudaMemcpyAsync(prio_out, prio.p, sizeof(int32_t) * e.n_in, cudaMemcpyDeviceToHost, s));
  ATC_CK(cudaStreamSynchronize(s));
  *n_out = (uint64_t)e.m;
  return ATC_OK;
} ATC_CATCH

// ---- k-core direction (edge_directing/kcore_direction.cpp:12-146) -------------------
namespace atc {
__global__ void unpack_u64_pairs_kernel(const uint64_t* e, int64_t ne, int2* out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < ne; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = make_int2((int32_t)(uint32_t)(e[i] >> 32), (int32_t)(uint32_t)e[i]);
}
// One output per input edge, in input order: src = the endpoint of smaller core number,
// the smaller id on a tie (kcore_direction.cpp:133-141).
__global__ void kcore_orient_kernel(const int2* p, int64_t ne, const int32_t* core, uint64_t* out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < ne; i += (int64_t)gridDim.x * blockDim.x) {
    int32_t a = p[i].x, b = p[i].y;
    const int32_t ca = core[a], cb = core[b];
    if (ca > cb || (ca == cb && a > b)) {
      const int32_t t = a;
      a = b;
      b = t;
    }
    out[i] = ((uint64_t)(uint32_t)a << 32) | (uint32_t)b;
  }
}
}  // namespace atc

extern "C" atc_status atc_kcore_direction(const uint64_t* edges, uint64_t ne, uint64_t* oriented_out,
                                          int32_t* core_out, uint64_t* n_vertices, atc_stream st) try {
  ATC_CHECK_ARG(ne == 0 || (edges != nullptr && oriented_out != nullptr), "NULL array");
  cudaStream_t s = as_stream(st);
  keep_pool();
  if (n_vertices) *n_vertices = 0;
  if (ne == 0) return ATC_OK;
  DevBuf<uint64_t> de;
  DevBuf<int2> d;
  ATC_TRY(de.alloc(ne, s));
  ATC_TRY(d.alloc(ne, s));
  ATC_CK(cudaMemcpyAsync(de.p, edges, sizeof(uint64_t) * ne, cudaMemcpyHostToDevice, s));
  atc::unpack_u64_pairs_kernel<<<grid_for(ne, 256), 256, 0, s>>>(de.p, ne, d.p);
  ATC_CK(cudaGetLastError());
  SimpleEdges e;
  ATC_TRY(build_simple_edges(d.p, ne, &e, s));
  DevBuf<int32_t> deg, core;
  ATC_TRY(deg.alloc(e.n_in, s));
  ATC_TRY(core.alloc(e.n_in, s));
  ATC_TRY(simple_degrees(e, deg.p, s));
  ATC_TRY(core_numbers(e, deg.p, core.p, s));
  atc::kcore_orient_kernel<<<grid_for(ne, 256), 256, 0, s>>>(d.p, ne, core.p, de.p);
  ATC_CK(cudaGetLastError());
  ATC_CK(cudaMemcpyAsync(oriented_out, de.p, sizeof(uint64_t) * ne, cudaMemcpyDeviceToHost, s));
  if (core_out) ATC_CK(cudaMemcpyAsync(core_out, core.p, sizeof(int32_t) * e.n_in, cudaMemcpyDeviceToHost, s));
  ATC_CK(cudaStreamSynchronize(s));
  if (n_vertices) *n_vertices = (uint64_t)e.n_in;
  return ATC_OK;
} ATC_CATCH

// ---- approximate parallel A-direction (edge_directing/A-direction-parallel/peel.cu) -----
namespace atc {
// peel.cu:44-59: swap iff flag_d > 0, or flag_d == 0 and minor_d > 0, or both 0 and
// src > dst, with flag_d = (int)(flag[src] - flag[dst]) and minor_d = (int)(minor[src] -
// (compat ? flag[dst] : minor[dst])) in wrapping 32-bit arithmetic.
__global__ void apeel_orient_kernel(const int2* p, int64_t ne, const uint32_t* flags, const uint32_t* minor,
                                    int compat, uint64_t* out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < ne; i += (int64_t)gridDim.x * blockDim.x) {
    uint32_t a = (uint32_t)p[i].x, b = (uint32_t)p[i].y;
    const int32_t flag_d = (int32_t)(flags[a] - flags[b]);
    const int32_t minor_d = (int32_t)(minor[a] - (compat ? flags[b] : minor[b]));
    if (flag_d > 0 || (flag_d == 0 && minor_d > 0) || (flag_d == 0 && minor_d == 0 && a > b)) {
      const uint32_t t = a;
      a = b;
      b = t;
    }
    out[i] = ((uint64_t)a << 32) | b;
  }
}
}  // namespace atc

extern "C" atc_status atc_adirection_par(const uint64_t* edges, uint64_t ne, int compat, uint64_t* oriented_out,
                                         uint32_t* flags_out, uint32_t* minor_out, uint64_t* n_vertices,
                                         int32_t* iterations, atc_stream st) try {
  ATC_CHECK_ARG(ne == 0 || (edges != nullptr && oriented_out != nullptr), "NULL array");
  cudaStream_t s = as_stream(st);
  keep_pool();
  if (n_vertices) *n_vertices = 0;
  if (iterations) *iterations = 0;
  if (ne == 0) return ATC_OK;
  DevBuf<uint64_t> de;
  DevBuf<int2> d;
  ATC_TRY(de.alloc(ne, s));
  ATC_TRY(d.alloc(ne, s));
  ATC_CK(cudaMemcpyAsync(de.p, edges, sizeof(uint64_t) * ne, cudaMemcpyHostToDevice, s));
  atc::unpack_u64_pairs_kernel<<<grid_for(ne, 256), 256, 0, s>>>(de.p, ne, d.p);
  ATC_CK(cudaGetLastError());
  SimpleEdges e;
  ATC_TRY(build_simple_edges(d.p, ne, &e, s));
  DevBuf<int32_t> deg;
  DevBuf<uint32_t> flags, minor;
  ATC_TRY(deg.alloc(e.n_in, s));
  ATC_TRY(flags.alloc(e.n_in, s));
  ATC_TRY(minor.alloc(e.n_in, s));
  ATC_TRY(simple_degrees(e, deg.p, s));
  int iters = 0;
  ATC_TRY(approx_peel(e, deg.p, flags.p, minor.p, &iters, s));
  atc::apeel_orient_kernel<<<grid_for(ne, 256), 256, 0, s>>>(d.p, ne, flags.p, minor.p, compat, de.p);
  ATC_CK(cudaGetLastError());
  ATC_CK(cudaMemcpyAsync(oriented_out, de.p, sizeof(uint64_t) * ne, cudaMemcpyDeviceToHost, s));
  if (flags_out) ATC_CK(cudaMemcpyAsync(flags_out, flags.p, sizeof(uint32_t) * e.n_in, cudaMemcpyDeviceToHost, s));
  if (minor_out) ATC_CK(cudaMemcpyAsync(minor_out, minor.p, sizeof(uint32_t) * e.n_in, cudaMemcpyDeviceToHost, s));
  ATC_CK(cudaStreamSynchronize(s));
  if (n_vertices) *n_vertices = (uint64_t)e.n_in;
  if (iterations) *iterations = iters;
  return ATC_OK;
} ATC_CATCH

// ---- binary CSR cache -----------------------------------------------------------------
// File: "ATCCSR01", then int64 n, m, n_input, wedges, wedges_min, int32 dir, order,
// pruned, max_outdeg, then offsets (n+1 int64) and cols (m int32), little-endian.
namespace atc {
__global__ void csr_fill_esrc_kernel(const int64_t* off, int64_t n, int32_t* esrc) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t u = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; u < n; u += warps)
    for (int64_t j = off[u] + lane; j < off[u + 1]; j += 32) esrc[j] = (int32_t)u;
}
static const char kCsrMagic[8] = {'A', 'T', 'C', 'C', 'S', 'R', '0', '1'};

// int32 array in pinned host memory mapped into the device's address space: `host` for
// the CPU, `dev` for kernels (the same address under unified addressing).
struct HostMapped {
  int32_t* host = nullptr;
  int32_t* dev = nullptr;
  atc_status alloc(int64_t count) {
    void* p = nullptr;
    cudaError_t e = cudaHostAlloc(&p, sizeof(int32_t) * (size_t)std::max<int64_t>(count, 1),
                                  cudaHostAllocMapped | cudaHostAllocPortable);
    if (e != cudaSuccess) {
      set_error("cudaHostAlloc of %lld ints: %s", (long long)count, cudaGetErrorString(e));
      return ATC_ERR_OOM;
    }
    host = static_cast<int32_t*>(p);
    void* d = nullptr;
    e = cudaHostGetDevicePointer(&d, p, 0);
    if (e != cudaSuccess) {
      set_error("cudaHostGetDevicePointer: %s", cudaGetErrorString(e));
      return ATC_ERR_CUDA;
    }
    dev = static_cast<int32_t*>(d);
    return ATC_OK;
  }
  int32_t* release() {
    int32_t* p = host;
    host = dev = nullptr;
    return p;
  }
  ~HostMapped() {
    if (host) cudaFreeHost(host);
  }
};
}  // namespace atc

extern "C" atc_status atc_csr_save(const atc_csr* csr, const char* path, atc_stream st) try {
  ATC_CHECK_ARG(csr != nullptr && path != nullptr, "NULL argument");
  std::vector<int64_t> off(csr->n + 1);
  std::vector<int32_t> cols(csr->m);
  ATC_TRY(atc_csr_to_host(csr, off.data(), cols.data(), st));
  FILE* f = fopen(path, "wb");
  if (!f) {
    set_error("cannot open %s for writing", path);
    return ATC_ERR_INVALID;
  }
  int64_t h64[5] = {csr->n, csr->m, csr->n_input, csr->wedges, csr->wedges_min};
  int32_t h32[4] = {csr->dir, csr->order, csr->pruned, csr->max_outdeg};
  bool ok = fwrite(atc::kCsrMagic, 1, 8, f) == 8 && fwrite(h64, 8, 5, f) == 5 && fwrite(h32, 4, 4, f) == 4 &&
            fwrite(off.data(), 8, off.size(), f) == off.size() &&
            (cols.empty() || fwrite(cols.data(), 4, cols.size(), f) == cols.size());
  ok = (fclose(f) == 0) && ok;
  if (!ok) {
    set_error("short write to %s", path);
    return ATC_ERR_INVALID;
  }
  return ATC_OK;
} ATC_CATCH

static atc_status csr_load_impl(const char* path, bool host_resident, atc_csr* out, cudaStream_t s) {
  ATC_CHECK_ARG(path != nullptr && out != nullptr, "NULL argument");
  *out = atc_csr{};
  FILE* f = fopen(path, "rb");
  if (!f) {
    set_error("cannot open %s", path);
    return ATC_ERR_INVALID;
  }
  fseek(f, 0, SEEK_END);
  const long fsize = ftell(f);
  fseek(f, 0, SEEK_SET);
  char magic[8];
  int64_t h64[5];
  int32_t h32[4];
  bool ok = fread(magic, 1, 8, f) == 8 && memcmp(magic, atc::kCsrMagic, 8) == 0 && fread(h64, 8, 5, f) == 5 &&
            fread(h32, 4, 4, f) == 4 && h64[0] >= 0 && h64[1] >= 0 && h64[0] < (int64_t)INT32_MAX;
  // the header's n and m must fit the file (64-byte header, n+1 offsets, m targets), checked
  // by division so that a forged count cannot wrap or reach the allocations below
  const int64_t body = (int64_t)fsize - 64;
  if (ok) ok = body >= 8 * (h64[0] + 1) && h64[1] <= (body - 8 * (h64[0] + 1)) / 4;
  std::vector<int64_t> off;
  std::vector<int32_t> cols;
  if (ok) {
    try {
      off.resize(h64[0] + 1);
      cols.resize(h64[1]);
    } catch (const std::exception&) {
      fclose(f);
      set_error("out of host memory reading %s", path);
      return ATC_ERR_OOM;
    }
    ok = fread(off.data(), 8, off.size(), f) == off.size() &&
         (cols.empty() || fread(cols.data(), 4, cols.size(), f) == cols.size());
  }
  fclose(f);
  // the arrays must form a CSR: offsets from 0 to m, non-decreasing, rows strictly
  // increasing ids in [0, n)
  const int64_t n = ok ? h64[0] : 0, m = ok ? h64[1] : 0;
  if (ok) ok = off[0] == 0 && off[n] == m;
  for (int64_t u = 0; ok && u < n; ++u) {
    if (off[u + 1] < off[u]) ok = false;
    for (int64_t j = off[u]; ok && j < off[u + 1]; ++j)
      if (cols[j] < 0 || cols[j] >= n || (j > off[u] && cols[j] <= cols[j - 1])) ok = false;
  }
  if (!ok) {
    set_error("%s is not an ATCCSR01 file holding a valid CSR", path);
    return ATC_ERR_INVALID;
  }
  DevBuf<int64_t> doff;
  DevBuf<int32_t> dcols, desrc;
  DevBuf<unsigned long long> counter;
  HostMapped hcols, hesrc;
  ATC_TRY(doff.alloc(n + 1, s));
  ATC_TRY(counter.alloc(4, s));
  ATC_CK(cudaMemcpyAsync(doff.p, off.data(), sizeof(int64_t) * (n + 1), cudaMemcpyHostToDevice, s));
  int32_t* cols_dev;
  int32_t* esrc_dev;
  if (host_resident) {
    ATC_TRY(hcols.alloc(m + 16));
    ATC_TRY(hesrc.alloc(m + 16));
    std::copy(cols.begin(), cols.end(), hcols.host);
    std::fill(hcols.host + m, hcols.host + m + 16, 0);
    cols_dev = hcols.dev;
    esrc_dev = hesrc.dev;
  } else {
    ATC_TRY(dcols.alloc(m + 16, s));
    ATC_TRY(desrc.alloc(m + 16, s));
    ATC_CK(cudaMemsetAsync(dcols.p + m, 0, sizeof(int32_t) * 16, s));
    if (m) ATC_CK(cudaMemcpyAsync(dcols.p, cols.data(), sizeof(int32_t) * m, cudaMemcpyHostToDevice, s));
    cols_dev = dcols.p;
    esrc_dev = desrc.p;
  }
  if (n) atc::csr_fill_esrc_kernel<<<grid_for(n * 32, 256), 256, 0, s>>>(doff.p, n, esrc_dev);
  ATC_CK(cudaGetLastError());
  ATC_CK(cudaStreamSynchronize(s));
  CsrPriv* pv = new CsrPriv();
  if (host_resident) {
    pv->host_cols = hcols.release();
    pv->host_esrc = hesrc.release();
    pv->esrc = esrc_dev;
    out->cols = cols_dev;
  } else {
    pv->esrc = desrc.detach();
    out->cols = dcols.detach();
  }
  pv->counter = counter.detach();
  pv->bits = id_bits(n);
  out->n = n;
  out->m = m;
  out->offsets = doff.detach();
  out->n_input = h64[2];
  out->wedges = h64[3];
  out->wedges_min = h64[4];
  out->dir = h32[0];
  out->order = h32[1];
  out->pruned = h32[2];
  out->max_outdeg = h32[3];
  out->priv = pv;
  return ATC_OK;
}

extern "C" atc_status atc_csr_load(const char* path, atc_csr* out, atc_stream st) try {
  return csr_load_impl(path, false, out, as_stream(st));
} ATC_CATCH

extern "C" atc_status atc_csr_load_host(const char* path, atc_csr* out, atc_stream st) try {
  return csr_load_impl(path, true, out, as_stream(st));
} ATC_CATCH

extern "C" atc_status atc_csr_host_resident(atc_csr* csr, atc_stream st) try {
  ATC_CHECK_ARG(csr != nullptr, "csr is NULL");
  ATC_CHECK_ARG(csr->priv != nullptr, "csr was not built by atc_pretc or atc_csr_load");
  CsrPriv* pv = static_cast<CsrPriv*>(csr->priv);
  if (pv->host_cols) return ATC_OK;
  cudaStream_t s = as_stream(st);
  const int64_t m = csr->m;
  HostMapped hcols, hesrc;
  ATC_TRY(hcols.alloc(m + 16));
  ATC_TRY(hesrc.alloc(m + 16));
  ATC_CK(cudaMemcpyAsync(hcols.host, csr->cols, sizeof(int32_t) * (m + 16), cudaMemcpyDeviceToHost, s));
  ATC_CK(cudaMemcpyAsync(hesrc.host, pv->esrc, sizeof(int32_t) * m, cudaMemcpyDeviceToHost, s));
  ATC_CK(cudaStreamSynchronize(s));
  cudaFree(csr->cols);
  cudaFree(pv->esrc);
  csr->cols = hcols.dev;
  pv->esrc = hesrc.dev;
  pv->host_cols = hcols.release();
  pv->host_esrc = hesrc.release();
  return ATC_OK;
} ATC_CATCH
