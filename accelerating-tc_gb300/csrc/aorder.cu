// A-order vertex relabelling (vertex_ordering/A-order/A-order.cpp:62-247).
//
// GPU part: degrees (repeats counted), degree orientation and runtime degree rt (the
// out-degree it gives), the histogram of rt, the (rt, id) order of all vertices, and
// the final lookup table.  Host part: the bucket heap of A-order.cpp:123-181, which is
// sequential by definition.  Its result is fixed by which bucket each pop takes (the
// extreme key; keys are unique) and by the array that the final sort_heap reorders
// (the buckets in reverse order of filling), so a faster queue with the same pops
// replaces the heap and std::sort_heap is applied to the same array (bucket_heap).  The
// heap only needs each position's rt, which the rt histogram gives, so no vertex list
// crosses to the host; the pops go back to the device, which scatters them into the
// bucket order of positions in the (rt, id) order.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <optional>
#include <thread>
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

// Bucket keys of the heap as one integer: the float memory superiority mapped to an
// order-preserving uint32 (high half), then the bucket id << 6 | its fill count (low
// half).  Bucket ids are unique, so (superiority, id) decides every comparison exactly as
// the reference's comparators (A-order.cpp:40-60) do and the fill count only rides along.
// Superiorities are never NaN; -0 is folded into +0 so that the two compare equal, as
// floats do.
inline uint32_t order_bits(float f) {
  f += 0.0f;
  uint32_t u;
  std::memcpy(&u, &f, 4);
  return (u >> 31) ? ~u : (u | 0x80000000u);
}
inline float from_order_bits(uint32_t o) {
  uint32_t u = (o >> 31) ? (o & 0x7fffffffu) : ~o;
  float f;
  std::memcpy(&f, &u, 4);
  return f;
}
inline uint64_t bucket_key(float sup, uint32_t id_fill) { return ((uint64_t)order_bits(sup) << 32) | id_fill; }

// The priority queue of the bucket heap.  Keys leave in ascending order (Up) or descending
// order (!Up).  Between two changes of the runtime degree d every popped bucket goes back
// with sup + delta(d) for one fixed delta, and float addition is monotone, so the keys put
// back during one run of equal d arrive already in pop order (keys of equal sup can
// arrive out of id order; push() moves them into place from the back).  Each run's keys
// therefore form a sorted sequence: the queue keeps one sequence per run and pops the
// first of their fronts.  A closed sequence is merged into the one before it when it holds
// at least half as many keys, which keeps the number of sequences logarithmic.
template <bool Up>
struct RunQueue {
  static bool first(uint64_t x, uint64_t y) { return Up ? x < y : x > y; }
  std::vector<std::vector<uint64_t>> seq;  // closed runs, each in pop order
  std::vector<size_t> head;                // next key of each closed run
  std::vector<uint64_t> open;              // keys put back during the current run
  size_t open_head = 0;

  void close_run() {
    if (open_head < open.size()) {
      seq.emplace_back(open.begin() + open_head, open.end());
      head.push_back(0);
    }
    open.clear();
    open_head = 0;
    while (seq.size() >= 2) {
      const size_t l = seq.size() - 1;
      const size_t nl = seq[l].size() - head[l], np = seq[l - 1].size() - head[l - 1];
      if (2 * nl < np) break;
      std::vector<uint64_t> out(nl + np);
      const uint64_t* a = seq[l - 1].data() + head[l - 1];
      const uint64_t* b = seq[l].data() + head[l];
      size_t i = 0, j = 0, k = 0;
      while (i < np && j < nl) out[k++] = first(b[j], a[i]) ? b[j++] : a[i++];
      while (i < np) out[k++] = a[i++];
      while (j < nl) out[k++] = b[j++];
      seq.pop_back();
      head.pop_back();
      seq.back().swap(out);
      head.back() = 0;
    }
  }
  uint64_t pop() {  // the queue is not empty
    int best = -1;
    uint64_t bk = 0;
    for (size_t r = 0; r < seq.size(); ++r)
      if (head[r] < seq[r].size() && (best < 0 || first(seq[r][head[r]], bk))) {
        best = (int)r;
        bk = seq[r][head[r]];
      }
    if (open_head < open.size() && (best < 0 || first(open[open_head], bk))) return open[open_head++];
    ++head[best];
    return bk;
  }
  void push(uint64_t k) {
    open.push_back(k);
    size_t i = open.size() - 1;
    while (i > open_head && first(k, open[i - 1])) {
      open[i] = open[i - 1];
      --i;
    }
    open[i] = k;
  }
  std::vector<uint64_t> drain() {  // every key left, in no particular order
    close_run();
    std::vector<uint64_t> all;
    for (size_t r = 0; r < seq.size(); ++r) all.insert(all.end(), seq[r].begin() + head[r], seq[r].end());
    seq.clear();
    head.clear();
    return all;
  }
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

// The shuffled relabellings' deal (relabel-naive.cpp:102-150 with mix = 64,
// relabel4lpOut.cpp:82-110 with mix = 40): entry q of the descending list goes to position
// i + mix*j of column i = q / chunk (chunk = n / mix), j = q mod chunk in the even columns
// and chunk-1 - (q mod chunk) in the odd ones, which are read backwards; entries from
// mix*chunk on keep their place.  dealt[position] = id.
__global__ void mix_deal_kernel(const uint64_t* sorted, int B, int64_t n, int mix, int32_t* dealt) {
  const uint64_t mask = (1ull << B) - 1;
  const int64_t chunk = n / mix;
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
    const int64_t q = n - 1 - r;
    int64_t pos = q;
    if (q < mix * chunk) {
      const int64_t i = q / chunk, jj = q - i * chunk;
      pos = i + mix * ((i & 1) ? chunk - 1 - jj : jj);
    }
    dealt[pos] = (int32_t)(sorted[r] & mask);
  }
}

// inv[perm[p]] = p (badLookUpTable, relabel-naive.cpp:154-158)
__global__ void inverse_kernel(const int32_t* perm, int64_t n, int32_t* inv) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x)
    inv[perm[p]] = (int32_t)p;
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

// Scatters the pops of the bucket heap into the bucket order: pop t filled slot `fill` of
// bucket `id` (log[t] = id * 40 + fill) with list position total-1-t (phase 1, the first
// n1 pops) or t-n1 (phase 2); the bucket's place in the output is rank[id].
__global__ void bucket_scatter_kernel(const uint32_t* log, const uint32_t* rank, int64_t total, int64_t n1,
                                      int32_t* bucket_pos) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t v = log[t];
    const uint32_t id = v / kBucket, f = v - id * kBucket;
    bucket_pos[(int64_t)rank[id] * kBucket + f] = (int32_t)(t < n1 ? total - 1 - t : t - n1);
  }
}

// The bucket heap of A-order.cpp:123-181 over positions of the rt>=2 list, `hist[r]` =
// number of vertices of runtime degree r.  Output: log[t] = id * 40 + fill of the bucket
// that pop t filled, and rank[id] = the bucket's place after the final sort_heap.
//
// The reference's result depends on two things only.  (1) Which bucket each pop takes:
// keys are unique, so that is the extreme key, whatever the heap's internal layout.
// (2) The array that sort_heap(idSort) (:181) reorders: every pop fills one slot and the
// two phases make exactly 40 * nb pops, so at the end every bucket is full and has left
// the heap range; pop_heap left each one at the back of the shrinking range when it
// filled, so the array holds the buckets in reverse order of filling.  The queue below
// reproduces (1), and std::sort_heap with the reference's comparator is applied to the
// array of (2).
void bucket_heap(const std::vector<int64_t>& hist, int maxrt, int64_t S, int64_t mdp, std::vector<uint32_t>& log,
                 std::vector<uint32_t>& rank) {
  const int64_t nb = S / kBucket, total = nb * kBucket;
  std::vector<float> bw(maxrt + 1), ebw(maxrt + 1);
  for (int r = 0; r <= maxrt; ++r) {
    bw[r] = bandwidth_of(r);
    ebw[r] = equal_bandwidth_of(r);
  }
  // ids < 2^26 and id * 40 + fill < 2^32 hold because S <= 2^31 (int32 vertex ids)
  std::vector<int32_t> filled;  // bucket ids in the order they filled
  filled.reserve(nb);
  log.resize(total);
  int64_t t = 0;
  RunQueue<true> up;  // phase 1 pops the smallest (greatCmp heap, :144-157)
  up.open.resize(nb);
  for (int64_t i = 0; i < nb; ++i) up.open[i] = bucket_key(0.0f, (uint32_t)i << 6);
  // rt of list position i: positions are in rt order; [lo, lo + hist[r]) holds rt r
  int r_hi = maxrt;
  int64_t lo_hi = S - hist[maxrt];
  for (int64_t i = total - 1; i >= mdp;) {
    while (i < lo_hi) lo_hi -= hist[--r_hi];
    const int d = r_hi;
    const float delta = (bw[d] - ebw[d]) / kBucket;  // :151
    up.close_run();
    for (const int64_t stop = lo_hi > mdp ? lo_hi : mdp; i >= stop; --i) {
      const uint64_t k = up.pop();
      const uint32_t low = (uint32_t)k, id = low >> 6, fill = low & 63;
      log[t++] = id * kBucket + fill;
      if (fill + 1 >= (uint32_t)kBucket) {
        filled.push_back((int32_t)id);
        continue;
      }
      float sup = from_order_bits((uint32_t)(k >> 32));
      sup += delta;
      up.push(bucket_key(sup, low + 1));
    }
  }
  RunQueue<false> dn;  // phase 2 pops the largest (lessCmp heap, :163-177)
  dn.open = up.drain();
  std::sort(dn.open.begin(), dn.open.end(), [](uint64_t a, uint64_t b) { return a > b; });
  int r_lo = 2;
  int64_t hi_lo = hist.size() > 2 ? hist[2] : 0;  // end of rt r_lo
  for (int64_t i = 0; i < mdp;) {
    while (i >= hi_lo) hi_lo += hist[++r_lo];
    const int d = r_lo;
    const float eps = (ebw[d] - bw[d]) / kBucket;  // :171
    dn.close_run();
    for (const int64_t stop = hi_lo < mdp ? hi_lo : mdp; i < stop; ++i) {
      const uint64_t k = dn.pop();
      const uint32_t low = (uint32_t)k, id = low >> 6, fill = low & 63;
      log[t++] = id * kBucket + fill;
      if (fill + 1 >= (uint32_t)kBucket) {
        filled.push_back((int32_t)id);
        continue;
      }
      float sup = from_order_bits((uint32_t)(k >> 32));
      sup -= eps;
      dn.push(bucket_key(sup, low + 1));
    }
  }
  // the heap array at :181 (reverse filling order), sorted as the reference sorts it;
  // sort_heap's moves depend only on the comparisons, here of the ids alone (idSort)
  std::vector<int32_t> arr(nb);
  for (int64_t k = 0; k < nb; ++k) arr[nb - 1 - k] = filled[k];
  std::sort_heap(arr.begin(), arr.end(), [](int32_t a, int32_t b) { return a > b; });
  rank.resize(nb);
  for (int64_t r = 0; r < nb; ++r) rank[arr[r]] = (uint32_t)r;
}

}  // namespace

atc_status relabel_lookup(const int2* pairs, const uint64_t* keys, int bits, uint64_t ne, int64_t n_v, int kind,
                          int32_t* lookup, int2* oriented, cudaStream_t s) {
  if (n_v <= 0) return ATC_OK;
  const bool as_given = kind == ATC_RELABEL_OUTDEG_DESC || kind == ATC_RELABEL_OUTDEG_SHUFFLED;
  ATC_CHECK_ARG(!as_given || pairs != nullptr, "OUTDEG_DESC / OUTDEG_SHUFFLED need pairs");
  if (kind == ATC_RELABEL_RANDOM) {  // the degree list plays no part (relabel-random.cpp:77-89)
    DevBuf<int32_t> perm;
    ATC_TRY(perm.alloc(n_v, s));
    ATC_TRY(shuffle_ids(perm.p, n_v, s));
    inverse_kernel<<<grid_for(n_v, 256), 256, 0, s>>>(perm.p, n_v, lookup);
    ATC_CK(cudaGetLastError());
    if (!oriented || ne == 0) return ATC_OK;  // else the degree-oriented pairs below
  }
  DevBuf<int32_t> deg, rt;
  DevBuf<int> mx;
  ATC_TRY(rt.alloc(n_v, s));
  ATC_TRY(mx.alloc(1, s));
  ATC_CK(cudaMemsetAsync(rt.p, 0, sizeof(int32_t) * n_v, s));
  ATC_CK(cudaMemsetAsync(mx.p, 0, sizeof(int), s));
  if (ne && as_given) {
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
  if (kind == ATC_RELABEL_RANDOM) return ATC_OK;
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
  if (kind == ATC_RELABEL_NAIVE_SHUFFLED || kind == ATC_RELABEL_OUTDEG_SHUFFLED) {
    const int mix = kind == ATC_RELABEL_NAIVE_SHUFFLED ? 64 : 40;
    DevBuf<int32_t> dealt;
    ATC_TRY(dealt.alloc(n_v, s));
    mix_deal_kernel<<<grid_for(n_v, 256), 256, 0, s>>>(a, B, n_v, mix, dealt.p);
    ATC_CK(cudaGetLastError());
    ATC_TRY(shuffle_blocks(dealt.p, n_v / mix, mix, s));
    inverse_kernel<<<grid_for(n_v, 256), 256, 0, s>>>(dealt.p, n_v, lookup);
    ATC_CK(cudaGetLastError());
    return ATC_OK;
  }
  rank_lookup_kernel<<<grid_for(n_v, 256), 256, 0, s>>>(a, B, n_v, kind, lookup);
  ATC_CK(cudaGetLastError());
  return ATC_OK;
}

atc_status aorder_lookup(const int2* pairs, const uint64_t* keys, int bits, uint64_t ne, int64_t n_v, int32_t* lookup,
                         int2* oriented, cudaStream_t s, const int32_t* known_deg,
                         const std::function<atc_status()>* overlap) {
  if (n_v <= 0) {
    set_error("A-order needs at least one edge");
    return ATC_ERR_UNSUPPORTED;
  }
  DevBuf<int32_t> deg, rt;
  DevBuf<int> mx;
  std::optional<Phase> ph;
  ph.emplace("aorder.device", s);
  ATC_TRY(rt.alloc(n_v, s));
  ATC_TRY(mx.alloc(1, s));
  ATC_CK(cudaMemsetAsync(rt.p, 0, sizeof(int32_t) * n_v, s));
  ATC_CK(cudaMemsetAsync(mx.p, 0, sizeof(int), s));
  const int32_t* degp = known_deg;
  if (!degp) {
    ATC_TRY(deg.alloc(n_v, s));
    ATC_CK(cudaMemsetAsync(deg.p, 0, sizeof(int32_t) * n_v, s));
    if (ne) {
      if (pairs) deg_pairs_kernel<<<grid_for(ne, 256), 256, 0, s>>>(pairs, ne, deg.p);
      else deg_keys_kernel<<<grid_for(ne, 256), 256, 0, s>>>(keys, ne, bits, deg.p);
      ATC_CK(cudaGetLastError());
    }
    degp = deg.p;
  }
  if (ne) {
    rt_kernel<<<grid_for(ne, 256), 256, 0, s>>>(pairs, keys, bits, ne, degp, rt.p, oriented);
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
  // the (rt, id) order of all vertices is sorted on the device while the host runs the
  // bucket heap
  int B = id_bits(n_v);
  int rb = id_bits((int64_t)maxrt + 1);
  DevBuf<uint64_t> ka, kb;
  ATC_TRY(ka.alloc(n_v, s));
  ATC_TRY(kb.alloc(n_v, s));
  rtid_keys_kernel<<<grid_for(n_v, 256), 256, 0, s>>>(rt.p, n_v, B, ka.p);
  ATC_CK(cudaGetLastError());
  uint64_t* a = ka.p;
  uint64_t* b = kb.p;
  ATC_TRY(sort_keys_u64(a, b, n_v, 0, B + rb, s));

  std::vector<uint32_t> log, rank;
  ph.reset();
  ph.emplace(overlap ? "aorder.heap||peel" : "aorder.heap", s);
  if (overlap) {
    bool heap_ok = true;
    std::thread heap([&] {
      try {
        bucket_heap(hist, maxrt, S, mdp, log, rank);
      } catch (const std::bad_alloc&) {
        heap_ok = false;
      }
    });
    const atc_status st = (*overlap)();
    heap.join();
    ATC_TRY(st);
    if (!heap_ok) {
      set_error("A-order: host allocation failed");
      return ATC_ERR_OOM;
    }
  } else {
    bucket_heap(hist, maxrt, S, mdp, log, rank);
  }
  ph.reset();
  ph.emplace("aorder.scatter", s);
  const int64_t total = nb * kBucket;
  DevBuf<uint32_t> dlog, drank;
  DevBuf<int32_t> dpos;
  ATC_TRY(dlog.alloc(total, s));
  ATC_TRY(drank.alloc(nb, s));
  ATC_TRY(dpos.alloc(total + 1, s));
  ATC_CK(cudaMemcpyAsync(dlog.p, log.data(), sizeof(uint32_t) * total, cudaMemcpyHostToDevice, s));
  ATC_CK(cudaMemcpyAsync(drank.p, rank.data(), sizeof(uint32_t) * nb, cudaMemcpyHostToDevice, s));
  bucket_scatter_kernel<<<grid_for(total, 256), 256, 0, s>>>(dlog.p, drank.p, total, total - mdp, dpos.p);
  ATC_CK(cudaGetLastError());
  lookup_kernel<<<grid_for(n_v, 256), 256, 0, s>>>(a, B, n_v, c0, c1, S, total, dpos.p, lookup);
  ATC_CK(cudaGetLastError());
  ATC_CK(cudaStreamSynchronize(s));  // `log` and `rank` are pageable host memory read by the copies above
  return ATC_OK;
}

}  // namespace atc

using namespace atc;

extern "C" atc_status atc_aorder(const int32_t* pairs, uint64_t np, int32_t* lookup, int32_t* normal,
                                 int32_t* reordered, atc_stream st) try {
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
} ATC_CATCH

extern "C" atc_status atc_relabel(const int32_t* pairs, uint64_t np, atc_relabel_kind kind, int32_t* lookup,
                                  int32_t* normal, int32_t* relabeled, atc_stream st) try {
  ATC_CHECK_ARG(lookup != nullptr, "lookup is NULL");
  ATC_CHECK_ARG(np == 0 || pairs != nullptr, "pairs is NULL");
  ATC_CHECK_ARG(kind >= ATC_RELABEL_DEGREE_DESC && kind <= ATC_RELABEL_RANDOM, "unknown atc_relabel_kind");
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
  if (kind == ATC_RELABEL_GRO) {
    ATC_TRY(gro_lookup(d.p, np, n_v, lk.p, s));
    if (np) ATC_CK(cudaMemcpyAsync(o.p, d.p, sizeof(int2) * np, cudaMemcpyDeviceToDevice, s));
  } else if (kind == ATC_RELABEL_ADIRECTION_BISSON) {
    SimpleEdges e;
    ATC_TRY(build_simple_edges(d.p, np, &e, s));
    DevBuf<int32_t> deg;
    ATC_TRY(deg.alloc(n_v, s));
    if (np == 0) {
      ATC_CK(cudaMemsetAsync(deg.p, 0, sizeof(int32_t) * n_v, s));
      e.n_in = n_v;  // the programs number vertex 0 even for an empty file
    } else {
      ATC_TRY(simple_degrees(e, deg.p, s));
    }
    ATC_TRY(bisson_adirection_lookup(e, deg.p, lk.p, s));
    if (np) ATC_CK(cudaMemcpyAsync(o.p, d.p, sizeof(int2) * np, cudaMemcpyDeviceToDevice, s));
  } else {
    ATC_TRY(relabel_lookup(d.p, nullptr, 1, np, n_v, kind, lk.p, o.p, s));
  }
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
} ATC_CATCH
