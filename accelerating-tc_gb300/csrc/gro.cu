// GRO vertex order of the reference's other_order library
// (vertex_ordering/other_order/porder.cpp:141-226, POrder::greedy_mheap).
//
// Vertices are numbered in windows of 32 (PACK_WIDTH, util.hpp:21-27).  A window opens with
// the first unnumbered vertex in (degree desc, id asc) order; every next vertex is the
// unnumbered one with the largest gain, where numbering u adds one to the gain of each
// unnumbered w reached as u <- v -> w or u -> v <- w (each neighbour v once per window).
// Which vertex of equal gain comes first is fixed by the reference's gain list
// (linkedlist_heap.cpp: keys in one linked list ordered by gain, a header per gain value,
// changes applied in the order they were recorded), so that list is rebuilt here with the
// same moves.
//
// GPU part: the out- and in-adjacency (edges sorted by (source, target) and by (target,
// source), repeats kept, as POrder::build, porder.cpp:94-123, fills them) and the degree
// order.  Host part: the greedy loop, sequential by definition.
#include <algorithm>
#include <vector>

#include "internal.cuh"

namespace atc {

namespace {

__global__ void gro_keys_kernel(const int2* p, uint64_t ne, int B, uint64_t* out_keys, uint64_t* in_keys) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < ne; i += stride) {
    const uint64_t a = (uint64_t)p[i].x, b = (uint64_t)p[i].y;
    out_keys[i] = (a << B) | b;
    in_keys[i] = (b << B) | a;
  }
}

// start[v] = first sorted key whose high part is >= v (v in [0, n]); list[i] = low part.
__global__ void gro_csr_kernel(const uint64_t* keys, uint64_t ne, int B, int64_t n, int32_t* start,
                               int32_t* list) {
  const uint64_t mask = (1ull << B) - 1;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t <= n || t < (int64_t)ne; t += stride) {
    if (t <= n) {
      uint64_t lo = 0, hi = ne;
      const uint64_t key = (uint64_t)t << B;
      while (lo < hi) {
        const uint64_t mid = (lo + hi) >> 1;
        if (keys[mid] < key) lo = mid + 1; else hi = mid;
      }
      start[t] = (int32_t)lo;
    }
    if (t < (int64_t)ne) list[t] = (int32_t)(keys[t] & mask);
  }
}

// Degree order keys: (max_deg - deg) << B | v sorts by degree desc, then id asc.
__global__ void gro_degree_keys_kernel(const int32_t* os, const int32_t* is, int64_t n, int B, uint64_t* keys) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n; v += stride) {
    const uint64_t deg = (uint64_t)(os[v + 1] - os[v]) + (uint64_t)(is[v + 1] - is[v]);
    keys[v] = ((0xffffffffull - deg) << B) | (uint64_t)v;
  }
}

// The gain list (linkedlist_heap.cpp): a doubly linked list of keys in non-increasing
// gain; slot g of `first_/last_/stamp_` marks the keys of gain g in the current window.
// A key's gain is stale when its window stamp is old, and then reads as 0.
class GainList {
 public:
  explicit GainList(int n)
      : gain_(n, 0), stamp_of_(n, 0), prev_(n), next_(n), first_(2 * (size_t)n + 2, -1), last_(2 * (size_t)n + 2, -1),
        slot_stamp_(2 * (size_t)n + 2, 0) {
    for (int i = 0; i < n; ++i) {
      prev_[i] = i - 1;
      next_[i] = i + 1 < n ? i + 1 : -1;
    }
    if (n > 0) {
      head_ = 0;
      tail_ = n - 1;
      first_[0] = 0;
      last_[0] = n - 1;
    }
  }
  bool present(int k) const { return gain_[k] != -1; }
  void bump(int k) {  // inc()
    if ((stamp_of_[k] & kStampMask) != window_) {
      gain_[k] = 0;
      stamp_of_[k] = window_;
    }
    ++gain_[k];
    if (!(stamp_of_[k] & kQueued)) {
      queued_.push_back({k, gain_[k] - 1});
      stamp_of_[k] |= kQueued;
    }
  }
  int take_top() {  // pop()
    settle();
    const int k = head_;
    const int g = live_gain(k);
    gain_[k] = -1;
    head_ = next_[k];
    if (head_ == -1) tail_ = -1;
    else prev_[head_] = -1;
    if (first_[g] == last_[g]) first_[g] = last_[g] = -1;
    else first_[g] = head_;
    return k;
  }
  void remove(int k) {  // del()
    settle();
    if (gain_[k] == -1) return;
    const int g = live_gain(k);
    gain_[k] = -1;
    cut(k);
    if (first_[g] == last_[g]) first_[g] = last_[g] = -1;
    else if (first_[g] == k) first_[g] = next_[k];
    else if (last_[g] == k) last_[g] = prev_[k];
  }
  void new_window() {  // reset()
    ++window_;
    queued_.clear();
    first_[0] = head_;
    last_[0] = tail_;
    slot_stamp_[0] = window_;
  }

 private:
  static constexpr int kStampMask = 0x7fffffff;
  static constexpr int kQueued = (int)0x80000000u;
  std::vector<int> gain_, stamp_of_, prev_, next_, first_, last_, slot_stamp_;
  std::vector<std::pair<int, int>> queued_;  // (key, gain before its first bump)
  int window_ = 0, head_ = -1, tail_ = -1;

  int live_gain(int k) const { return stamp_of_[k] != window_ ? 0 : gain_[k]; }
  void cut(int k) {
    if (prev_[k] == -1) head_ = next_[k];
    else next_[prev_[k]] = next_[k];
    if (next_[k] == -1) tail_ = prev_[k];
    else prev_[next_[k]] = prev_[k];
  }
  bool slot_empty(int g) const { return slot_stamp_[g] != window_ || first_[g] == -1; }
  void settle() {  // adjust(): move the bumped keys in the order they were first bumped
    for (const auto& q : queued_) move_up(q.first, q.second);
    queued_.clear();
  }
  void move_up(int k, int old_g) {  // up()
    if (first_[old_g] == last_[old_g]) first_[old_g] = last_[old_g] = -1;
    else if (first_[old_g] == k) first_[old_g] = next_[k];
    else if (last_[old_g] == k) last_[old_g] = prev_[k];
    cut(k);
    const int g = gain_[k];
    if (slot_empty(g)) {
      first_[g] = last_[g] = k;
      slot_stamp_[g] = window_;
      int r = g - 1;  // the next lower gain with keys, no lower than old_g
      while (r > old_g && slot_empty(r)) --r;
      if (first_[r] == -1) {  // relink where it was
        if (prev_[k] == -1) head_ = k;
        else next_[prev_[k]] = k;
        if (next_[k] == -1) tail_ = k;
        else prev_[next_[k]] = k;
      } else {  // in front of gain r's first key
        const int right = first_[r], left = prev_[right];
        prev_[k] = left;
        next_[k] = right;
        if (left == -1) head_ = k;
        else next_[left] = k;
        prev_[right] = k;
      }
    } else {  // behind gain g's last key
      const int left = last_[g], right = next_[left];
      prev_[k] = left;
      next_[k] = right;
      next_[left] = k;
      if (right == -1) tail_ = k;
      else prev_[right] = k;
      last_[g] = k;
    }
    stamp_of_[k] -= kQueued;
  }
};

}  // namespace

atc_status gro_lookup(const int2* pairs, uint64_t ne, int64_t n_v, int32_t* lookup, cudaStream_t s) {
  if (n_v <= 0) return ATC_OK;
  ATC_CHECK_ARG(n_v < (int64_t)INT32_MAX && ne < (uint64_t)INT32_MAX, "graph too large for the GRO order");
  const int B = id_bits(n_v + 1);
  DevBuf<uint64_t> ko, ki, alt;
  DevBuf<int32_t> os, oe, is, ie;
  ATC_TRY(ko.alloc(ne + 1, s));
  ATC_TRY(ki.alloc(ne + 1, s));
  ATC_TRY(alt.alloc(std::max<uint64_t>(ne, (uint64_t)n_v) + 1, s));
  ATC_TRY(os.alloc(n_v + 1, s));
  ATC_TRY(is.alloc(n_v + 1, s));
  ATC_TRY(oe.alloc(ne + 1, s));
  ATC_TRY(ie.alloc(ne + 1, s));
  if (ne) {
    gro_keys_kernel<<<grid_for(ne, 256), 256, 0, s>>>(pairs, ne, B, ko.p, ki.p);
    ATC_CK(cudaGetLastError());
  }
  for (int side = 0; side < 2; ++side) {
    uint64_t* k = side ? ki.p : ko.p;
    uint64_t* a = alt.p;
    if (ne) ATC_TRY(sort_keys_u64(k, a, ne, 0, 2 * B, s));
    gro_csr_kernel<<<grid_for(std::max<int64_t>(n_v + 1, (int64_t)ne), 256), 256, 0, s>>>(
        k, ne, B, n_v, side ? is.p : os.p, side ? ie.p : oe.p);
    ATC_CK(cudaGetLastError());
  }
  // degree order, sorted on the device
  DevBuf<uint64_t> dk;
  ATC_TRY(dk.alloc(n_v, s));
  gro_degree_keys_kernel<<<grid_for(n_v, 256), 256, 0, s>>>(os.p, is.p, n_v, B, dk.p);
  ATC_CK(cudaGetLastError());
  uint64_t* dkp = dk.p;
  uint64_t* dap = alt.p;
  ATC_TRY(sort_keys_u64(dkp, dap, n_v, 0, 32 + B, s));
  std::vector<int32_t> hos(n_v + 1), his(n_v + 1), hoe(ne), hie(ne);
  std::vector<uint64_t> hdk(n_v);
  ATC_CK(cudaMemcpyAsync(hos.data(), os.p, sizeof(int32_t) * (n_v + 1), cudaMemcpyDeviceToHost, s));
  ATC_CK(cudaMemcpyAsync(his.data(), is.p, sizeof(int32_t) * (n_v + 1), cudaMemcpyDeviceToHost, s));
  if (ne) {
    ATC_CK(cudaMemcpyAsync(hoe.data(), oe.p, sizeof(int32_t) * ne, cudaMemcpyDeviceToHost, s));
    ATC_CK(cudaMemcpyAsync(hie.data(), ie.p, sizeof(int32_t) * ne, cudaMemcpyDeviceToHost, s));
  }
  ATC_CK(cudaMemcpyAsync(hdk.data(), dkp, sizeof(uint64_t) * n_v, cudaMemcpyDeviceToHost, s));
  ATC_CK(cudaStreamSynchronize(s));

  const int n = (int)n_v;
  const uint64_t vmask = (1ull << B) - 1;
  std::vector<int32_t> order(n_v);
  for (int64_t i = 0; i < n_v; ++i) order[i] = (int32_t)(hdk[i] & vmask);
  std::vector<int32_t> new_id(n_v, -1);
  std::vector<int32_t> via_out(n_v, -1), via_in(n_v, -1);  // window in which v was expanded
  GainList gains(n);
  size_t next_fresh = 0;  // first vertex of `order` possibly unnumbered
  constexpr int kWindow = 32;
  int window = -1;
  for (int idx = 0; idx < n; ++idx) {
    int u;
    if (idx % kWindow == 0) {
      while (new_id[order[next_fresh]] != -1) ++next_fresh;
      u = order[next_fresh];
      gains.new_window();
      gains.remove(u);
      ++window;
    } else {
      u = gains.take_top();
    }
    new_id[u] = idx;
    for (int j = his[u]; j < his[u + 1]; ++j) {  // u <- v, then v -> w
      const int v = hie[j];
      if (via_out[v] == window) continue;
      via_out[v] = window;
      for (int t = hos[v]; t < hos[v + 1]; ++t)
        if (gains.present(hoe[t])) gains.bump(hoe[t]);
    }
    for (int j = hos[u]; j < hos[u + 1]; ++j) {  // u -> v, then v <- w
      const int v = hoe[j];
      if (via_in[v] == window) continue;
      via_in[v] = window;
      for (int t = his[v]; t < his[v + 1]; ++t)
        if (gains.present(hie[t])) gains.bump(hie[t]);
    }
  }
  ATC_CK(cudaMemcpyAsync(lookup, new_id.data(), sizeof(int32_t) * n_v, cudaMemcpyHostToDevice, s));
  ATC_CK(cudaStreamSynchronize(s));  // new_id is pageable host memory read by the copy
  return ATC_OK;
}

}  // namespace atc
