// A-order vertex relabelling (vertex_ordering/A-order/A-order.cpp:62-247).
//
// GPU part: degrees (repeats counted), degree orientation and runtime degree rt (the
// out-degree it gives), the histogram of rt, the (rt, id) order of all vertices, and
// the final lookup table.  Host part: the bucket heap of A-order.cpp:123-181, which is
// sequential by definition — its result is fixed by the order in which libstdc++'s
// make_heap / pop_heap / push_heap / sort_heap move elements, so it calls those same
// functions on the same keys.  The heap only needs each position's rt, which the rt
// histogram gives, so no vertex list crosses to the host; the bucket contents go back
// to the device as positions into the (rt, id) order.
#include <algorithm>
#include <cmath>
#include <vector>

#include "internal.cuh"

namespace atc {

namespace {

constexpr int kBucket = 40;  // BUCKETSIZE, A-order.cpp:14

// Lookup tables of A-order.cpp:20-36 (float results; pow in double, sqrt in float).
const float kBwTab[10] = {0, 0, 271, 310, 399, 419, 458, 478, 524, 539};
const float kLamTab[10] = {0, 0, 145.51, 121.98, 53.26, 23.92, 16, 14, 12.94, 10.24};

float bandwidth_of(int len) {
  if (len < 10) return kBwTab[len];
  return 384.1 * std::pow(len, 0.1491);
}

float equal_bandwidth_of(int len) {
  if (len < 10) return kLamTab[len] * std::sqrt(bandwidth_of(len)) / std::sqrt((float)len);
  return 12 * std::sqrt(bandwidth_of(len)) / std::sqrt((float)len);
}

struct HeapItem {
  int id;
  float sup;   // memory superiority
  int slot;    // member block of this bucket
};
struct ByLess {
  bool operator()(const HeapItem& a, const HeapItem& b) const { return a.sup < b.sup || (a.sup == b.sup && a.id < b.id); }
};
struct ByGreat {
  bool operator()(const HeapItem& a, const HeapItem& b) const { return a.sup > b.sup || (a.sup == b.sup && a.id > b.id); }
};
struct ByIdDesc {
  bool operator()(const HeapItem& a, const HeapItem& b) const { return a.id > b.id; }
};

__global__ void deg_pairs_kernel(const int2* p, uint64_t ne, int32_t* deg) {
  uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < ne; i += stride) {
    int2 e = p[i];
    atomicAdd(&deg[e.x], 1);
    atomicAdd(&deg[e.y], 1);
  }
}

__global__ void deg_keys_kernel(const uint64_t* k, uint64_t ne, int B, int32_t* deg) {
  uint64_t mask = (1ull << B) - 1;
  uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < ne; i += stride) {
    atomicAdd(&deg[k[i] >> B], 1);
    atomicAdd(&deg[k[i] & mask], 1);
  }
}

// Degree orientation of A-order.cpp:88-99: the pair is flipped when src has the larger
// degree, or equal degree and the smaller id; rt counts the resulting sources.
__global__ void rt_kernel(const int2* p, const uint64_t* k, int B, uint64_t ne, const int32_t* deg, int32_t* rt,
                          int2* oriented) {
  uint64_t mask = (1ull << B) - 1;
  uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < ne; i += stride) {
    int32_t s, d;
    if (p) { s = p[i].x; d = p[i].y; } else { s = (int32_t)(k[i] >> B); d = (int32_t)(k[i] & mask); }
    if (deg[s] > deg[d] || (deg[s] == deg[d] && s < d)) {
      int32_t t = s; s = d; d = t;
    }
    atomicAdd(&rt[s], 1);
    if (oriented) oriented[i] = make_int2(s, d);
  }
}

// rt = out-degree of the pairs as given (relabel4lpOut.cpp:27-31); oriented = the input.
__global__ void outdeg_kernel(const int2* p, uint64_t ne, int32_t* rt, int2* oriented) {
  uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < ne; i += stride) {
    atomicAdd(&rt[p[i].x], 1);
    if (oriented) oriented[i] = p[i];
  }
}

// Rank lookups over the ascending (rt, id) order of all n vertices; q = n - 1 - rank is
// the position in the reversed (descending) list.
//   DEGREE_DESC: new id = q (goodLookUpTable, A-order-v2.cpp:67-74).
//   AORDER_V2:   the descending list dealt into 40 columns of chunk = n / 40 rows,
//                position i + 40 j <- q = i * chunk + j; the last n % 40 stay in place
//                (A-order-v2.cpp:102-146, the mix without shuffle or reversal).
__global__ void rank_lookup_kernel(const uint64_t* sorted, int B, int64_t n, int kind, int32_t* lookup) {
  const uint64_t mask = (1ull << B) - 1;
  const int64_t chunk = n / 40;
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
    const int64_t q = n - 1 - r;
    int64_t pos = q;
    if (kind == ATC_RELABEL_AORDER_V2 && q < 40 * chunk) pos = q / chunk + 40 * (q % chunk);
    lookup[sorted[r] & mask] = (int32_t)pos;
  }
}

__global__ void rt_hist_kernel(const int32_t* rt, int64_t n, int32_t* hist, int* maxrt) {
  int best = 0;
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n; v += stride) {
    int r = rt[v];
    if (hist) atomicAdd(&hist[r], 1);
    best = max(best, r);
  }
  if (!hist) {
    for (int o = 16; o > 0; o >>= 1) best = max(best, __shfl_xor_sync(0xffffffffu, best, o));
    if ((threadIdx.x & 31) == 0) atomicMax(maxrt, best);
  }
}

__global__ void rtid_keys_kernel(const int32_t* rt, int64_t n, int B, uint64_t* keys) {
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n; v += stride)
    keys[v] = ((uint64_t)rt[v] << B) | (uint64_t)v;
}

// Final relabelling (A-order.cpp:186-210): positions [0, 40*nb) come from the buckets,
// then the rest of the rt>=2 list, then rt==1, then rt==0 vertices, each by id.
__global__ void lookup_kernel(const uint64_t* sorted, int B, int64_t n, int64_t c0, int64_t c1, int64_t S,
                              int64_t nbk, const int32_t* bucket_pos, int32_t* lookup) {
  uint64_t mask = (1ull << B) - 1;
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += stride) {
    int64_t src;
    if (q < nbk) src = c0 + c1 + bucket_pos[q];
    else if (q < S) src = c0 + c1 + q;
    else if (q < S + c1) src = c0 + (q - S);
    else src = q - S - c1;
    lookup[sorted[src] & mask] = (int32_t)q;
  }
}

__global__ void relabel_pairs_kernel(const int2* in, uint64_t ne, const int32_t* lookup, int2* out) {
  uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < ne; i += stride)
    out[i] = make_int2(lookup[in[i].x], lookup[in[i].y]);
}

// The bucket heap of A-order.cpp:123-181 over positions of the rt>=2 list.  `cum[r]` =
// first position of runtime degree r in that list (r >= 2).  Fills `pos` (40*nb ints)
// with list positions in final bucket order.
void bucket_heap(const std::vector<int64_t>& hist, int maxrt, int64_t S, int64_t mdp, std::vector<int32_t>& pos) {
  int64_t nb = S / kBucket;
  std::vector<float> bw(maxrt + 1), ebw(maxrt + 1);
  for (int r = 0; r <= maxrt; ++r) {
    bw[r] = bandwidth_of(r);
    ebw[r] = equal_bandwidth_of(r);
  }
  std::vector<HeapItem> heap(nb);
  for (int64_t i = 0; i < nb; ++i) heap[i] = HeapItem{(int)i, 0.0f, (int)i};
  std::vector<int32_t> members((size_t)nb * kBucket);
  std::vector<int32_t> fill(nb, 0);
  std::make_heap(heap.begin(), heap.end(), ByGreat());
  // rt of list position i: positions are in rt order, so a cursor over the histogram
  // gives it; [lo_hi, lo_hi + hist[r_hi]) are the positions of runtime degree r_hi.
  int r_hi = maxrt;
  int64_t lo_hi = S - hist[maxrt];
  int64_t finished = 0;
  for (int64_t i = nb * kBucket - 1; i >= mdp; --i) {  // phase 1, :144-157
    while (i < lo_hi) {
      --r_hi;
      lo_hi -= hist[r_hi];
    }
    int d = r_hi;
    std::pop_heap(heap.begin(), heap.end() - finished, ByGreat());
    HeapItem& b = *(heap.rbegin() + finished);
    members[(size_t)b.slot * kBucket + fill[b.slot]++] = (int32_t)i;
    b.sup += (bw[d] - ebw[d]) / kBucket;
    if (fill[b.slot] >= kBucket) ++finished;
    else std::push_heap(heap.begin(), heap.end() - finished, ByGreat());
  }
  std::make_heap(heap.begin(), heap.end() - finished, ByLess());  // :163
  int r_lo = 2;
  int64_t hi_lo = hist.size() > 2 ? hist[2] : 0;  // end of rt r_lo
  for (int64_t i = 0; i < mdp; ++i) {  // phase 2, :165-177
    while (i >= hi_lo) {
      ++r_lo;
      hi_lo += hist[r_lo];
    }
    int d = r_lo;
    std::pop_heap(heap.begin(), heap.end() - finished, ByLess());
    HeapItem& b = *(heap.rbegin() + finished);
    members[(size_t)b.slot * kBucket + fill[b.slot]++] = (int32_t)i;
    b.sup -= (ebw[d] - bw[d]) / kBucket;
    if (fill[b.slot] >= kBucket) ++finished;
    else std::push_heap(heap.begin(), heap.end() - finished, ByLess());
  }
  std::sort_heap(heap.begin(), heap.end(), ByIdDesc());  // :181, on a sequence that is not a heap
  pos.resize((size_t)nb * kBucket);
  size_t q = 0;
  for (int64_t i = 0; i < nb; ++i)
    for (int j = 0; j < kBucket; ++j) pos[q++] = members[(size_t)heap[i].slot * kBucket + j];
}

}  // namespace

atc_status relabel_lookup(const int2* pairs, const uint64_t* keys, int bits, uint64_t ne, int64_t n_v, int kind,
                          int32_t* lookup, int2* oriented, cudaStream_t s) {
  if (n_v <= 0) return ATC_OK;
  ATC_CHECK_ARG(kind != ATC_RELABEL_OUTDEG_DESC || pairs != nullptr, "OUTDEG_DESC needs pairs");
  DevBuf<int32_t> deg, rt;
  DevBuf<int> mx;
  ATC_TRY(rt.alloc(n_v, s));
  ATC_TRY(mx.alloc(1, s));
  ATC_CK(cudaMemsetAsync(rt.p, 0, sizeof(int32_t) * n_v, s));
  ATC_CK(cudaMemsetAsync(mx.p, 0, sizeof(int), s));
  if (ne && kind == ATC_RELABEL_OUTDEG_DESC) {
    outdeg_kernel<<<grid_for(ne, 256), 256, 0, s>>>(pairs, ne, rt.p, oriented);
  } else if (ne) {
    ATC_TRY(deg.alloc(n_v, s));
    ATC_CK(cudaMemsetAsync(deg.p, 0, sizeof(int32_t) * n_v, s));
    if (pairs) deg_pairs_kernel<<<grid_for(ne, 256), 256, 0, s>>>(pairs, ne, deg.p);
    else deg_keys_kernel<<<grid_for(ne, 256), 256, 0, s>>>(keys, ne, bits, deg.p);
    ATC_CK(cudaGetLastError());
    rt_kernel<<<grid_for(ne, 256), 256, 0, s>>>(pairs, keys, bits, ne, deg.p, rt.p, oriented);
  }
  ATC_CK(cudaGetLastError());
  rt_hist_kernel<<<grid_for(n_v, 256), 256, 0, s>>>(rt.p, n_v, nullptr, mx.p);
  ATC_CK(cudaGetLastError());
  int maxrt = 0;
  ATC_CK(cudaMemcpyAsync(&maxrt, mx.p, sizeof(int), cudaMemcpyDeviceToHost, s));
  ATC_CK(cudaStreamSynchronize(s));
  const int B = id_bits(n_v), rb = id_bits((int64_t)maxrt + 1);
  DevBuf<uint64_t> ka, kb;
  ATC_TRY(ka.alloc(n_v, s));
  ATC_TRY(kb.alloc(n_v, s));
  rtid_keys_kernel<<<grid_for(n_v, 256), 256, 0, s>>>(rt.p, n_v, B, ka.p);
  ATC_CK(cudaGetLastError());
  uint64_t* a = ka.p;
  uint64_t* b = kb.p;
  ATC_TRY(sort_keys_u64(a, b, n_v, 0, B + rb, s));
  rank_lookup_kernel<<<grid_for(n_v, 256), 256, 0, s>>>(a, B, n_v, kind, lookup);
  ATC_CK(cudaGetLastError());
  return ATC_OK;
}

atc_status aorder_lookup(const int2* pairs, const uint64_t* keys, int bits, uint64_t ne, int64_t n_v, int32_t* lookup,
                         int2* oriented, cudaStream_t s) {
  if (n_v <= 0) {
    set_error("A-order needs at least one edge");
    return ATC_ERR_UNSUPPORTED;
  }
  DevBuf<int32_t> deg, rt;
  DevBuf<int> mx;
  ATC_TRY(deg.alloc(n_v, s));
  ATC_TRY(rt.alloc(n_v, s));
  ATC_TRY(mx.alloc(1, s));
  ATC_CK(cudaMemsetAsync(deg.p, 0, sizeof(int32_t) * n_v, s));
  ATC_CK(cudaMemsetAsync(rt.p, 0, sizeof(int32_t) * n_v, s));
  ATC_CK(cudaMemsetAsync(mx.p, 0, sizeof(int), s));
  if (ne) {
    if (pairs) deg_pairs_kernel<<<grid_for(ne, 256), 256, 0, s>>>(pairs, ne, deg.p);
    else deg_keys_kernel<<<grid_for(ne, 256), 256, 0, s>>>(keys, ne, bits, deg.p);
    ATC_CK(cudaGetLastError());
    rt_kernel<<<grid_for(ne, 256), 256, 0, s>>>(pairs, keys, bits, ne, deg.p, rt.p, oriented);
    ATC_CK(cudaGetLastError());
  }
  rt_hist_kernel<<<grid_for(n_v, 256), 256, 0, s>>>(rt.p, n_v, nullptr, mx.p);
  ATC_CK(cudaGetLastError());
  int maxrt = 0;
  ATC_CK(cudaMemcpyAsync(&maxrt, mx.p, sizeof(int), cudaMemcpyDeviceToHost, s));
  ATC_CK(cudaStreamSynchronize(s));
  DevBuf<int32_t> dh;
  ATC_TRY(dh.alloc(maxrt + 1, s));
  ATC_CK(cudaMemsetAsync(dh.p, 0, sizeof(int32_t) * (maxrt + 1), s));
  rt_hist_kernel<<<grid_for(n_v, 256), 256, 0, s>>>(rt.p, n_v, dh.p, nullptr);
  ATC_CK(cudaGetLastError());
  std::vector<int32_t> h32(maxrt + 1);
  ATC_CK(cudaMemcpyAsync(h32.data(), dh.p, sizeof(int32_t) * (maxrt + 1), cudaMemcpyDeviceToHost, s));
  ATC_CK(cudaStreamSynchronize(s));
  std::vector<int64_t> hist(h32.begin(), h32.end());

  // id_rtDegree (A-order.cpp:110-119): vertices with rt >= 2; memoryDominatePos = the
  // number with rt in [2,4], recorded only once rt 5 is reached.
  int64_t c0 = hist[0], c1 = maxrt >= 1 ? hist[1] : 0;
  int64_t S = n_v - c0 - c1;
  int64_t mdp = 0;
  if (maxrt >= 5) mdp = hist[2] + hist[3] + hist[4];
  int64_t nb = S / kBucket;
  if (mdp == 0 || mdp > nb * kBucket) {
    set_error("A-order undefined on this graph: %lld vertices of runtime degree 2..4, %lld buckets of %d, max "
              "runtime degree %d",
              (long long)mdp, (long long)nb, kBucket, maxrt);
    return ATC_ERR_UNSUPPORTED;
  }
  std::vector<int32_t> pos;
  bucket_heap(hist, maxrt, S, mdp, pos);

  int B = id_bits(n_v);
  int rb = id_bits((int64_t)maxrt + 1);
  DevBuf<uint64_t> ka, kb;
  DevBuf<int32_t> dpos;
  ATC_TRY(ka.alloc(n_v, s));
  ATC_TRY(kb.alloc(n_v, s));
  ATC_TRY(dpos.alloc(pos.size() + 1, s));
  rtid_keys_kernel<<<grid_for(n_v, 256), 256, 0, s>>>(rt.p, n_v, B, ka.p);
  ATC_CK(cudaGetLastError());
  uint64_t* a = ka.p;
  uint64_t* b = kb.p;
  ATC_TRY(sort_keys_u64(a, b, n_v, 0, B + rb, s));
  if (!pos.empty())
    ATC_CK(cudaMemcpyAsync(dpos.p, pos.data(), sizeof(int32_t) * pos.size(), cudaMemcpyHostToDevice, s));
  lookup_kernel<<<grid_for(n_v, 256), 256, 0, s>>>(a, B, n_v, c0, c1, S, nb * kBucket, dpos.p, lookup);
  ATC_CK(cudaGetLastError());
  ATC_CK(cudaStreamSynchronize(s));  // `pos` is pageable host memory read by the copy above
  return ATC_OK;
}

}  // namespace atc

using namespace atc;

extern "C" atc_status atc_aorder(const int32_t* pairs, uint64_t np, int32_t* lookup, int32_t* normal,
                                 int32_t* reordered, atc_stream st) {
  ATC_CHECK_ARG(lookup != nullptr, "lookup is NULL");
  ATC_CHECK_ARG(np == 0 || pairs != nullptr, "pairs is NULL");
  cudaStream_t s = as_stream(st);
  int64_t n_v = 1;  // A-order.cpp:65: maxNodeId starts at 0
  int maxid = 0;
  for (uint64_t i = 0; i < 2 * np; ++i) {
    ATC_CHECK_ARG(pairs[i] >= 0, "negative vertex id");
    maxid = std::max(maxid, (int)pairs[i]);
  }
  n_v = (int64_t)maxid + 1;
  if (np == 0) {
    set_error("A-order undefined on an empty edge list");
    return ATC_ERR_UNSUPPORTED;
  }
  DevBuf<int2> d, o, r;
  DevBuf<int32_t> lk;
  ATC_TRY(d.alloc(np, s));
  ATC_TRY(o.alloc(np, s));
  ATC_TRY(lk.alloc(n_v, s));
  ATC_CK(cudaMemcpyAsync(d.p, pairs, sizeof(int2) * np, cudaMemcpyHostToDevice, s));
  ATC_TRY(aorder_lookup(d.p, nullptr, 1, np, n_v, lk.p, o.p, s));
  ATC_CK(cudaMemcpyAsync(lookup, lk.p, sizeof(int32_t) * n_v, cudaMemcpyDeviceToHost, s));
  if (normal) ATC_CK(cudaMemcpyAsync(normal, o.p, sizeof(int2) * np, cudaMemcpyDeviceToHost, s));
  if (reordered) {
    ATC_TRY(r.alloc(np, s));
    relabel_pairs_kernel<<<grid_for(np, 256), 256, 0, s>>>(o.p, np, lk.p, r.p);
    ATC_CK(cudaGetLastError());
    ATC_CK(cudaMemcpyAsync(reordered, r.p, sizeof(int2) * np, cudaMemcpyDeviceToHost, s));
  }
  ATC_CK(cudaStreamSynchronize(s));
  return ATC_OK;
}

extern "C" atc_status atc_relabel(const int32_t* pairs, uint64_t np, atc_relabel_kind kind, int32_t* lookup,
                                  int32_t* normal, int32_t* relabeled, atc_stream st) {
  ATC_CHECK_ARG(lookup != nullptr, "lookup is NULL");
  ATC_CHECK_ARG(np == 0 || pairs != nullptr, "pairs is NULL");
  ATC_CHECK_ARG(kind >= ATC_RELABEL_DEGREE_DESC && kind <= ATC_RELABEL_OUTDEG_DESC, "unknown atc_relabel_kind");
  cudaStream_t s = as_stream(st);
  int maxid = 0;  // the programs start maxNodeId at 0, so an empty list has one vertex
  for (uint64_t i = 0; i < 2 * np; ++i) {
    ATC_CHECK_ARG(pairs[i] >= 0, "negative vertex id");
    maxid = std::max(maxid, (int)pairs[i]);
  }
  const int64_t n_v = (int64_t)maxid + 1;
  DevBuf<int2> d, o, r;
  DevBuf<int32_t> lk;
  ATC_TRY(d.alloc(np + 1, s));
  ATC_TRY(o.alloc(np + 1, s));
  ATC_TRY(lk.alloc(n_v, s));
  if (np) ATC_CK(cudaMemcpyAsync(d.p, pairs, sizeof(int2) * np, cudaMemcpyHostToDevice, s));
  ATC_TRY(relabel_lookup(d.p, nullptr, 1, np, n_v, kind, lk.p, o.p, s));
  ATC_CK(cudaMemcpyAsync(lookup, lk.p, sizeof(int32_t) * n_v, cudaMemcpyDeviceToHost, s));
  if (normal && np) ATC_CK(cudaMemcpyAsync(normal, o.p, sizeof(int2) * np, cudaMemcpyDeviceToHost, s));
  if (relabeled && np) {
    ATC_TRY(r.alloc(np, s));
    relabel_pairs_kernel<<<grid_for(np, 256), 256, 0, s>>>(o.p, np, lk.p, r.p);
    ATC_CK(cudaGetLastError());
    ATC_CK(cudaMemcpyAsync(relabeled, r.p, sizeof(int2) * np, cudaMemcpyDeviceToHost, s));
  }
  ATC_CK(cudaStreamSynchronize(s));
  return ATC_OK;
}
