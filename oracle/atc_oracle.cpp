// CPU ORACLE — TEST INFRASTRUCTURE ONLY.
//
// A plain C++ restatement of the reference's algorithms on the triangle-counting
// path.  tests/, __graft_entry__.smoke() and bench.py's cpu_baseline / reference leg
// load it as the checker; the product library never links, loads or calls it.
//
// Pinning: tests/golden/golden.json holds the outputs of the reference's own CPU
// programs (A-direction-seri, A-order, costFuncCal, verification and the other_order
// OrgTriangleCount), compiled from their unmodified sources by oracle/Makefile and
// run on seeded graphs by tests/golden/make_golden.py.  tests/test_oracle_golden.py
// checks every function below against those fixtures.
//
// Every function cites the reference file:line it restates (paths are relative to
// the pkumod/accelerating-TC tree).
//
// Build: g++ -O2 -std=c++17 -fPIC -shared -ffp-contract=off -pthread
// (-ffp-contract=off keeps float arithmetic identical on x86-64 and aarch64.)

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <iterator>
#include <thread>
#include <vector>

namespace {

// ---------------------------------------------------------------------------
// Simple undirected graph: symmetric adjacency, each list sorted ascending,
// duplicates and self-loops removed.  Vertex count = max id + 1 over all pairs
// (self-loop-only vertices included), as every reference reader computes it
// (Hu/preTC.cu:90-113, A-direction-seri.cpp:187-192, A-order.cpp:68-74).
// ---------------------------------------------------------------------------
struct Adj {
  int64_t n = 0;
  std::vector<int64_t> off;  // n + 1
  std::vector<int32_t> nbr;  // off[n]
};

int64_t max_id(const int32_t* p, uint64_t np) {
  int64_t mx = -1;
  for (uint64_t i = 0; i < 2 * np; ++i) mx = std::max<int64_t>(mx, p[i]);
  return mx;
}

Adj build_adj(const int32_t* p, uint64_t np) {
  Adj g;
  g.n = max_id(p, np) + 1;
  std::vector<int64_t> cnt(g.n + 1, 0);
  for (uint64_t i = 0; i < np; ++i) {
    int32_t s = p[2 * i], d = p[2 * i + 1];
    if (s == d) continue;
    cnt[s + 1]++;
    cnt[d + 1]++;
  }
  for (int64_t v = 0; v < g.n; ++v) cnt[v + 1] += cnt[v];
  std::vector<int32_t> tmp(cnt[g.n]);
  std::vector<int64_t> cur(cnt.begin(), cnt.end() - 1);
  for (uint64_t i = 0; i < np; ++i) {
    int32_t s = p[2 * i], d = p[2 * i + 1];
    if (s == d) continue;
    tmp[cur[s]++] = d;
    tmp[cur[d]++] = s;
  }
  g.off.assign(g.n + 1, 0);
  g.nbr.clear();
  g.nbr.reserve(tmp.size());
  for (int64_t v = 0; v < g.n; ++v) {
    auto b = tmp.begin() + cnt[v], e = tmp.begin() + cnt[v + 1];
    std::sort(b, e);
    e = std::unique(b, e);
    g.nbr.insert(g.nbr.end(), b, e);
    g.off[v + 1] = (int64_t)g.nbr.size();
  }
  return g;
}

// Scalar merge count: other_order/set_operation.cpp:129-144 (intersect_count),
// widened to 64 bits.
inline uint64_t intersect_count(const int32_t* a, int64_t na, const int32_t* b, int64_t nb) {
  int64_t i = 0, j = 0;
  uint64_t r = 0;
  while (i < na && j < nb) {
    if (a[i] == b[j]) {
      ++r; ++i; ++j;
    } else if (a[i] < b[j]) {
      ++i;
    } else {
      ++j;
    }
  }
  return r;
}

template <class F>
void parallel_for(int64_t n, int nthreads, int64_t chunk, F&& body) {
  if (nthreads <= 1 || n <= chunk) {
    for (int64_t i = 0; i < n; ++i) body(i, 0);
    return;
  }
  std::atomic<int64_t> next(0);
  std::vector<std::thread> th;
  for (int t = 0; t < nthreads; ++t)
    th.emplace_back([&, t] {
      for (;;) {
        int64_t b = next.fetch_add(chunk);
        if (b >= n) break;
        int64_t e = std::min(n, b + chunk);
        for (int64_t i = b; i < e; ++i) body(i, t);
      }
    });
  for (auto& x : th) x.join();
}

// Length of the prefix of v's sorted list holding neighbours smaller than v:
// the N-(v) lists OrgTriangleCount::build keeps (org_triangle_count.cpp:15-50).
inline int64_t lower_len(const Adj& g, int64_t v) {
  const int32_t* b = g.nbr.data() + g.off[v];
  const int32_t* e = g.nbr.data() + g.off[v + 1];
  return std::lower_bound(b, e, (int32_t)v) - b;
}

// ---------------------------------------------------------------------------
// A-direction (edge_directing/A-direction-seri.cpp:35-153), restated with the
// reference's own data layout: every neighbour listed twice, degrees doubled,
// float threshold, frontier vectors.
// ---------------------------------------------------------------------------
std::vector<int> seri_peel(const std::vector<std::pair<int, int>>& edges, unsigned edgeNum, int nodeNum) {
  float threshold = ((float)edgeNum) / nodeNum + 1;             // :37
  std::vector<int> priority(nodeNum, -1);                          // :38-39
  std::vector<int> frontier, next;
  std::vector<int> degree(nodeNum, 0);
  for (unsigned i = 0; i < edgeNum; ++i) {                         // :44-47
    degree[edges[i].first]++;
    degree[edges[i].second]++;
  }
  std::vector<int> rt(degree);                                     // :48-49
  std::vector<long long> off(nodeNum, 0);                          // :50-54
  for (int i = 0; i + 1 < nodeNum; ++i) off[i + 1] = off[i] + degree[i];
  std::vector<int> all((size_t)edgeNum * 2);                       // :59-73
  std::vector<long long> cur(off);
  for (unsigned i = 0; i < edgeNum; ++i) {
    int s = edges[i].first, d = edges[i].second;
    all[cur[s]++] = d;
    all[cur[d]++] = s;
  }
  int priorityNum = 0;
  int threshold_old = threshold;                                   // :77
  int peeled = 0;
  for (;;) {                                                       // :79
    frontier.clear();
    next.clear();
    for (int i = 0; i < nodeNum; ++i)                              // :83-89
      if (rt[i] <= threshold && priority[i] == -1) {
        frontier.push_back(i);
        ++peeled;
        priority[i] = priorityNum;
      }
    ++priorityNum;
    while (!frontier.empty()) {                                    // :92-121
      for (size_t f = 0; f < frontier.size(); ++f) {
        int c = frontier[f];
        const int* lst = all.data() + off[c];
        for (int j = 0; j < degree[c]; ++j) {
          int v = lst[j];
          if (priority[v] != -1) {
            if (priority[v] == priority[c] &&
                (rt[v] > rt[c] || (rt[v] == rt[c] && v > c)))
              rt[v]--;
          } else {
            rt[v]--;
            if (rt[v] <= threshold) {
              next.push_back(v);
              ++peeled;
              priority[v] = priorityNum;
            }
          }
        }
      }
      std::swap(frontier, next);
      next.clear();
      ++priorityNum;
    }
    if (peeled >= nodeNum) break;                                  // :125-126
    threshold += threshold_old;                                    // :127
  }
  return priority;
}

// ---------------------------------------------------------------------------
// A-order tables (vertex_ordering/A-order/A-order.cpp:20-36).
// ---------------------------------------------------------------------------
const float kBw[10] = {0, 0, 271, 310, 399, 419, 458, 478, 524, 539};
const float kLambda[10] = {0, 0, 145.51, 121.98, 53.26, 23.92, 16, 14, 12.94, 10.24};  // double literals narrowed, as in the reference

float get_bandwidth(int len) {
  if (len < 10) return kBw[len];
  return 384.1 * std::pow(len, 0.1491);  // double product, narrowed to float on return
}

float get_equal_bandwidth(int len) {
  if (len < 10) return kLambda[len] * std::sqrt(get_bandwidth(len)) / std::sqrt((float)len);
  return 12 * std::sqrt(get_bandwidth(len)) / std::sqrt((float)len);
}

struct Bucket {
  int id;
  float ms;   // memorySuperiority
  int slot;   // index of this bucket's member list (the reference keeps a vector pointer)
};
struct LessCmp {   // A-order.cpp:44-49
  bool operator()(const Bucket& a, const Bucket& b) const {
    return a.ms < b.ms || (a.ms == b.ms && a.id < b.id);
  }
};
struct GreatCmp {  // A-order.cpp:50-55
  bool operator()(const Bucket& a, const Bucket& b) const {
    return a.ms > b.ms || (a.ms == b.ms && a.id > b.id);
  }
};
struct IdSort {    // A-order.cpp:56-60
  bool operator()(const Bucket& a, const Bucket& b) const { return a.id > b.id; }
};

}  // namespace

// ---------------------------------------------------------------------------
// GRO's gain list (vertex_ordering/other_order/linkedlist_heap.cpp:3-254), restated:
// every key sits in one doubly linked list ordered by non-increasing gain; per gain
// value a header marks the first and last key with that gain.  Gains from an earlier
// window are stale (their state label differs) and read as 0.  inc() only records the
// key's first change since the last adjust(); adjust() then moves the recorded keys in
// recording order (up()), which fixes how keys of equal gain are ordered.
// ---------------------------------------------------------------------------
class GroGainList {
 public:
  explicit GroGainList(int cap) : nodes_(cap), heads_(2 * (size_t)cap + 2, Head{-1, -1, 0}), pend_() {
    for (int i = 0; i < cap; ++i) nodes_[i] = Node{0, 0, i - 1, i + 1};
    if (cap) {
      nodes_[cap - 1].next = -1;
      heads_[0] = Head{0, cap - 1, 0};
      head_ = 0;
      tail_ = cap - 1;
    }
  }
  bool has(int key) const { return nodes_[key].val != -1; }  // :141-144
  int max_gain() const { return max_gain_; }
  void inc(int key) {                                         // :25-41
    Node& x = nodes_[key];
    if ((x.state & kLabelMask) != label_) {
      x.val = 0;
      x.state = label_;
    }
    ++x.val;
    if (x.val > max_gain_) max_gain_ = x.val;
    if ((x.state & kPending) == 0) {
      pend_.push_back({key, x.val - 1});
      x.state |= kPending;
    }
  }
  int pop() {  // :49-71
    adjust();
    Node& x = nodes_[head_];
    const int val = x.state != label_ ? 0 : x.val;
    const int key = head_;
    x.val = -1;
    head_ = x.next;
    if (x.next == -1) tail_ = -1;
    else nodes_[x.next].prev = -1;
    Head& h = heads_[val];
    if (h.first == h.last) h.first = h.last = -1;
    else h.first = head_;
    return key;
  }
  void del(int key) {  // :73-98
    adjust();
    Node& x = nodes_[key];
    if (x.val == -1) return;
    const int val = x.state != label_ ? 0 : x.val;
    x.val = -1;
    unlink(key);
    Head& h = heads_[val];
    if (h.first == h.last) h.first = h.last = -1;
    else if (h.first == key) h.first = x.next;
    else if (h.last == key) h.last = x.prev;
  }
  void reset() {  // :100-105
    ++label_;
    pend_.clear();
    heads_[0] = Head{head_, tail_, label_};
  }

 private:
  static constexpr int kLabelMask = 0x7fffffff;
  static constexpr int kPending = (int)0x80000000u;
  struct Node { int state, val, prev, next; };
  struct Head { int first, last, label; };
  std::vector<Node> nodes_;
  std::vector<Head> heads_;
  std::vector<std::pair<int, int>> pend_;  // (key, gain before its first change)
  int label_ = 0, head_ = -1, tail_ = -1, max_gain_ = 0;

  void unlink(int key) {
    const Node& x = nodes_[key];
    if (x.prev == -1) head_ = x.next;
    else nodes_[x.prev].next = x.next;
    if (x.next == -1) tail_ = x.prev;
    else nodes_[x.next].prev = x.prev;
  }
  void adjust() {  // :107-113
    for (const auto& p : pend_) up(p.first, p.second);
    pend_.clear();
  }
  void up(int key, int old_val) {  // :162-216
    Node& x = nodes_[key];
    Head& oh = heads_[old_val];
    if (oh.first == oh.last) oh.first = oh.last = -1;
    else if (oh.first == key) oh.first = x.next;
    else if (oh.last == key) oh.last = x.prev;
    unlink(key);
    Head& nh = heads_[x.val];
    if (nh.label != label_ || nh.first == -1) {  // no key has this gain yet
      nh.first = nh.last = key;
      nh.label = label_;
      int r = x.val - 1;  // the nearest smaller gain that has keys, down to old_val
      while (r > old_val && (heads_[r].label != label_ || heads_[r].first == -1)) --r;
      const Head& rh = heads_[r];
      if (rh.first == -1) {  // back into its old place
        if (x.prev == -1) head_ = key;
        else nodes_[x.prev].next = key;
        if (x.next == -1) tail_ = key;
        else nodes_[x.next].prev = key;
      } else {  // just before the first key of gain r
        const int right = rh.first, left = nodes_[right].prev;
        x.prev = left;
        x.next = right;
        if (left == -1) head_ = key;
        else nodes_[left].next = key;
        nodes_[right].prev = key;
      }
    } else {  // after the last key with this gain
      const int left = nh.last, right = nodes_[left].next;
      x.prev = left;
      x.next = right;
      nodes_[left].next = key;
      if (right == -1) tail_ = key;
      else nodes_[right].prev = key;
      nh.last = key;
    }
    x.state -= kPending;
  }
};

extern "C" {

// Status codes shared by the oracle entry points.
enum { ORC_OK = 0, ORC_UNSUPPORTED = 5 };

// Number of distinct undirected non-loop edges and the vertex count.
void orc_simple_stats(const int32_t* pairs, uint64_t np, int64_t* n_out, int64_t* m_out) {
  Adj g = build_adj(pairs, np);
  *n_out = g.n;
  *m_out = (int64_t)g.nbr.size() / 2;
}

// Triangle count of the simple graph underlying `pairs`: Σ_u Σ_{v∈N-(u)} |N-(u) ∩ N-(v)|
// over the "smaller neighbour" lists, as OrgTriangleCount::triangle_count does
// (other_order/org_triangle_count.cpp:57-79 with set_operation.cpp:129-144), in uint64.
uint64_t orc_tc_count(const int32_t* pairs, uint64_t np, int nthreads) {
  Adj g = build_adj(pairs, np);
  std::vector<int64_t> low(g.n);
  for (int64_t v = 0; v < g.n; ++v) low[v] = lower_len(g, v);
  std::vector<uint64_t> part(std::max(1, nthreads), 0);
  parallel_for(g.n, nthreads, 256, [&](int64_t u, int t) {
    const int32_t* a = g.nbr.data() + g.off[u];
    uint64_t s = 0;
    for (int64_t k = 0; k < low[u]; ++k) {
      int32_t v = a[k];
      s += intersect_count(a, low[u], g.nbr.data() + g.off[v], low[v]);
    }
    part[t] += s;
  });
  uint64_t r = 0;
  for (auto x : part) r += x;
  return r;
}

// Lower CSR of the simple graph: for every vertex u the sorted, duplicate-free list of
// its smaller neighbours (the N-(u) lists of OrgTriangleCount::build,
// org_triangle_count.cpp:15-50).  Threaded.  Call with off == nullptr to size it.
void orc_lower_csr(const int32_t* p, uint64_t np, int64_t* off, int32_t* nbr, int64_t* n_out, int64_t* nnz_out,
                   int nthreads) {
  int64_t n = max_id(p, np) + 1;
  std::vector<int64_t> cnt(n + 1, 0);
  for (uint64_t i = 0; i < np; ++i) {
    int32_t a = p[2 * i], b = p[2 * i + 1];
    if (a != b) cnt[std::max(a, b) + 1]++;
  }
  for (int64_t v = 0; v < n; ++v) cnt[v + 1] += cnt[v];
  std::vector<int32_t> tmp(cnt[n]);
  std::vector<int64_t> cur(cnt.begin(), cnt.end() - 1);
  for (uint64_t i = 0; i < np; ++i) {
    int32_t a = p[2 * i], b = p[2 * i + 1];
    if (a != b) tmp[cur[std::max(a, b)]++] = std::min(a, b);
  }
  std::vector<int64_t> len(n, 0);
  parallel_for(n, nthreads, 4096, [&](int64_t v, int) {
    auto b = tmp.begin() + cnt[v], e = tmp.begin() + cnt[v + 1];
    std::sort(b, e);
    len[v] = std::unique(b, e) - b;
  });
  *n_out = n;
  int64_t total = 0;
  for (int64_t v = 0; v < n; ++v) total += len[v];
  *nnz_out = total;
  if (!off) return;
  off[0] = 0;
  for (int64_t v = 0; v < n; ++v) off[v + 1] = off[v] + len[v];
  parallel_for(n, nthreads, 4096, [&](int64_t v, int) {
    std::memcpy(nbr + off[v], tmp.data() + cnt[v], sizeof(int32_t) * len[v]);
  });
}

// Triangle count over a lower CSR restricted to the vertices u = phase + i*stride (the
// bounded sample the CPU baseline times): Σ_u Σ_{v∈N-(u)} |N-(u) ∩ N-(v)| with the
// scalar merge of set_operation.cpp:129-144.  *edges_out = Σ|N-(u)| over the sample.
uint64_t orc_tc_count_lower_sample(const int64_t* off, const int32_t* nbr, int64_t n, int64_t stride,
                                   int64_t phase, int nthreads, int64_t* edges_out) {
  int64_t nsamp = phase < n ? (n - phase + stride - 1) / stride : 0;
  std::vector<uint64_t> part(std::max(1, nthreads), 0);
  std::vector<int64_t> epart(std::max(1, nthreads), 0);
  parallel_for(nsamp, nthreads, 16, [&](int64_t i, int t) {
    int64_t u = phase + i * stride;
    const int32_t* a = nbr + off[u];
    int64_t lu = off[u + 1] - off[u];
    uint64_t s = 0;
    for (int64_t k = 0; k < lu; ++k) {
      int32_t v = a[k];
      s += intersect_count(a, lu, nbr + off[v], off[v + 1] - off[v]);
    }
    part[t] += s;
    epart[t] += lu;
  });
  uint64_t r = 0;
  int64_t e = 0;
  for (size_t t = 0; t < part.size(); ++t) { r += part[t]; e += epart[t]; }
  *edges_out = e;
  return r;
}

// Symmetric simple CSR (int64 offsets, sorted lists): used by bench.py's CPU leg.
// Call once with off == nullptr to get sizes (n_out, nnz_out), then with buffers.
void orc_symmetric_csr(const int32_t* pairs, uint64_t np, int64_t* off, int32_t* nbr,
                       int64_t* n_out, int64_t* nnz_out) {
  Adj g = build_adj(pairs, np);
  *n_out = g.n;
  *nnz_out = (int64_t)g.nbr.size();
  if (!off) return;
  std::memcpy(off, g.off.data(), sizeof(int64_t) * (g.n + 1));
  std::memcpy(nbr, g.nbr.data(), sizeof(int32_t) * g.nbr.size());
}

// A-direction-seri (edge_directing/A-direction-seri.cpp:170-288): reads pairs as the
// READFROMFILE path does, peels, and writes the oriented edge list (the bytes of
// lpBasedGraph.bin) into `out` (capacity 2*np ints).  `prio_out` (nullable, n ints)
// receives the peel priorities.  Returns the number of oriented edges.
int64_t orc_adirection(const int32_t* pairs, uint64_t np, int32_t* out, int32_t* prio_out) {
  int nodeNum = 0;                                                  // :174
  for (uint64_t i = 0; i < np; ++i) {                               // :188-191
    if (pairs[2 * i] > nodeNum) nodeNum = pairs[2 * i];
    if (pairs[2 * i + 1] > nodeNum) nodeNum = pairs[2 * i + 1];
  }
  nodeNum++;                                                        // :192
  std::vector<std::vector<int>> nb(nodeNum);                        // :199
  for (uint64_t i = 0; i < np; ++i) {                               // :215-221
    int s = pairs[2 * i], e = pairs[2 * i + 1];
    if (s == e) continue;
    nb[s].push_back(e);
    nb[e].push_back(s);
  }
  int totalEdge = 0;                                                // :197
  for (int i = 0; i < nodeNum; ++i) {                               // :225-229
    std::sort(nb[i].begin(), nb[i].end());
    nb[i].erase(std::unique(nb[i].begin(), nb[i].end()), nb[i].end());
    totalEdge += (int)nb[i].size();
  }
  std::vector<std::pair<int, int>> origin;                          // :242-248
  origin.reserve(totalEdge);
  for (int i = 0; i < nodeNum; ++i)
    for (int x : nb[i]) origin.emplace_back(i, x);
  std::vector<int> prio = seri_peel(origin, (unsigned)totalEdge, nodeNum);   // :252
  int64_t k = 0;
  for (int i = 0; i < nodeNum; ++i)                                 // :254-273
    for (int c : nb[i])
      if (prio[c] > prio[i] || (prio[c] == prio[i] && i < c)) {
        out[2 * k] = i;
        out[2 * k + 1] = c;
        ++k;
      }
  if (prio_out) std::memcpy(prio_out, prio.data(), sizeof(int) * nodeNum);
  return k;
}

// Bisson's A-direction relabelling (Bisson/A-direction.cpp:43-163, 196-304): the same
// symmetric, duplicate-free reading as A-direction-seri (:221-239), a serial peel over the
// doubled adjacency list (allEdges, :63-80) whose priorities number the outer selection and
// each wave (:91-126), then new id = nodeNum-1 - rank of (priority, degreeRecord, id)
// (:29-35,283-292).  degreeRecord is written at the selected vertex in the outer scan (:97)
// but at the frontier POSITION in the waves (:118, `degreeRecord[i]`); that quirk makes
// the secondary key depend on the serial visiting order, reproduced here statement by
// statement.  Fills `lookup` (nodeNum ints) and, when `out` is not null, the bytes of
// lpBasedGraph.bin: every (i, neighbour) of the symmetric lists relabelled (:293-300).
// Returns nodeNum (0 for an empty graph, with no output), or -1 where the serial program
// would loop forever (the float threshold stops growing).
int64_t orc_adirection_bisson(const int32_t* pairs, uint64_t np, int32_t* lookup, int32_t* out) {
  int nodeNum = 0;                                                  // :213-219
  for (uint64_t i = 0; i < np; ++i) {
    if (pairs[2 * i] > nodeNum) nodeNum = pairs[2 * i];
    if (pairs[2 * i + 1] > nodeNum) nodeNum = pairs[2 * i + 1];
  }
  nodeNum++;
  std::vector<std::vector<int>> nb(nodeNum);                        // :224-239
  for (uint64_t i = 0; i < np; ++i) {
    int s = pairs[2 * i], e = pairs[2 * i + 1];
    if (s == e) continue;
    nb[s].push_back(e);
    nb[e].push_back(s);
  }
  int totalEdge = 0;                                                // :242-246
  for (int i = 0; i < nodeNum; ++i) {
    std::sort(nb[i].begin(), nb[i].end());
    nb[i].erase(std::unique(nb[i].begin(), nb[i].end()), nb[i].end());
    totalEdge += (int)nb[i].size();
  }
  // peel (:43-163) on originEdges = every (i, neighbour) in list order (:263-268)
  const unsigned edgeNum = (unsigned)totalEdge;
  float threshold = ((float)edgeNum) / nodeNum + 1;                 // :45
  std::vector<int> priority(nodeNum, -1), degree(nodeNum, 0);
  for (int i = 0; i < nodeNum; ++i)                                 // :53-56
    for (int x : nb[i]) { degree[i]++; degree[x]++; }
  std::vector<int> rt(degree);                                      // :57-58
  std::vector<long long> off(nodeNum + 1, 0);                       // :59-63
  for (int i = 0; i < nodeNum - 1; ++i) off[i + 1] = off[i] + degree[i];
  std::vector<int> all((size_t)edgeNum * 2);                        // :69-80
  {
    std::vector<long long> cur(off.begin(), off.end() - 1);
    for (int i = 0; i < nodeNum; ++i)
      for (int x : nb[i]) {
        all[cur[i]++] = x;
        all[cur[x]++] = i;
      }
  }
  std::vector<int> degreeRecord(nodeNum, 0);
  std::vector<int> F, Fn;
  int priorityNum = 0;
  const int threshold_old = threshold;                              // :83
  int peeled = 0;
  for (;;) {                                                        // :85
    F.clear();
    Fn.clear();
    for (int i = 0; i < nodeNum; ++i)                               // :89-98
      if (rt[i] <= threshold && priority[i] == -1) {
        F.push_back(i);
        peeled++;
        priority[i] = priorityNum;
        degreeRecord[i] = rt[i];
      }
    priorityNum++;
    while (!F.empty()) {                                            // :101-131
      for (size_t i = 0; i < F.size(); ++i) {
        const int cur = F[i];
        const int* co = all.data() + off[cur];
        for (int j = 0; j < degree[cur]; ++j) {
          const int node = co[j];
          if (priority[node] != -1) {
            if (priority[node] == priority[cur] && (rt[node] > rt[cur] || (rt[node] == rt[cur] && node > cur)))
              rt[node]--;
          } else {
            rt[node]--;
            if (rt[node] <= threshold) {
              Fn.push_back(node);
              degreeRecord[i] = rt[node];                           // :118, indexed by position
              peeled++;
              priority[node] = priorityNum;
            }
          }
        }
      }
      std::swap(F, Fn);
      Fn.clear();
      priorityNum++;
    }
    if (peeled >= nodeNum) break;                                   // :137-139
    const float grown = threshold + threshold_old;
    if (!(grown > threshold)) return -1;
    threshold = grown;
  }
  std::vector<int> order(nodeNum);                                  // :283-292
  for (int i = 0; i < nodeNum; ++i) order[i] = i;
  std::sort(order.begin(), order.end(), [&](int a, int b) {
    if (priority[a] != priority[b]) return priority[a] < priority[b];
    if (degreeRecord[a] != degreeRecord[b]) return degreeRecord[a] < degreeRecord[b];
    return a < b;
  });
  for (int i = 0; i < nodeNum; ++i) lookup[order[i]] = nodeNum - 1 - i;
  if (out) {                                                        // :293-300
    int64_t k = 0;
    for (int i = 0; i < nodeNum; ++i)
      for (int x : nb[i]) {
        out[2 * k] = lookup[i];
        out[2 * k + 1] = lookup[x];
        ++k;
      }
  }
  return np ? nodeNum : 0;
}

// A-order (vertex_ordering/A-order/A-order.cpp:62-247).  Fills `lookup`
// (maxNodeId+1 ints: badLookUpTable, the new id of every old id), `normal` and
// `reordered` (2*np ints each: the bytes of the two output files).  Returns ORC_OK,
// or ORC_UNSUPPORTED where the reference indexes outside its arrays (no vertex with
// runtime degree in [2,4] or none >= 5, so memoryDominatePos == 0; or more such
// vertices than whole buckets can hold).
int orc_aorder(const int32_t* pairs, uint64_t np, int32_t* lookup, int32_t* normal, int32_t* reordered) {
  const int BUCKETSIZE = 40;                                        // :14
  int maxNodeId = 0;                                                // :65-74
  std::vector<std::pair<int, int>> e(np);
  for (uint64_t i = 0; i < np; ++i) {
    int s = pairs[2 * i], d = pairs[2 * i + 1];
    maxNodeId = s > maxNodeId ? s : maxNodeId;
    maxNodeId = d > maxNodeId ? d : maxNodeId;
    e[i] = {s, d};
  }
  std::vector<int> degree(maxNodeId + 1, 0);                        // :78-83
  for (auto& x : e) { degree[x.first]++; degree[x.second]++; }
  std::vector<int> rt(maxNodeId + 1, 0);                            // :86-99
  for (auto& x : e) {
    int s = x.first, d = x.second;
    if (degree[s] > degree[d] || (degree[s] == degree[d] && s < d)) {
      x.first = d;
      x.second = s;
      rt[d]++;
    } else {
      rt[s]++;
    }
  }
  int maxRt = 0;                                                    // :100-104
  for (int i = 0; i <= maxNodeId; ++i) maxRt = std::max(maxRt, rt[i]);
  std::vector<std::vector<int>> bucket(maxRt + 1);                  // :106-109
  for (int i = 0; i <= maxNodeId; ++i) bucket[rt[i]].push_back(i);
  std::vector<std::pair<int, int>> idrt;                            // :110-119
  unsigned memoryDominatePos = 0;
  for (int i = 2; i <= maxRt; ++i) {
    if (i == 5) memoryDominatePos = (unsigned)idrt.size();
    for (int v : bucket[i]) idrt.emplace_back(v, i);
  }
  int totalBucketNum = (int)idrt.size() / BUCKETSIZE;               // :123
  if (memoryDominatePos == 0 || memoryDominatePos > (unsigned)(BUCKETSIZE * totalBucketNum))
    return ORC_UNSUPPORTED;
  std::vector<Bucket> all(totalBucketNum);                          // :126-132
  std::vector<std::vector<int>> members(totalBucketNum);
  for (int i = 0; i < totalBucketNum; ++i) all[i] = Bucket{i, 0.0f, i};
  std::make_heap(all.begin(), all.end(), GreatCmp());
  std::vector<float> bw(maxRt + 1), ebw(maxRt + 1);                 // :134-139
  for (int i = 0; i < maxRt + 1; ++i) {
    bw[i] = get_bandwidth(i);
    ebw[i] = get_equal_bandwidth(i);
  }
  int finished = 0;
  for (int i = BUCKETSIZE * totalBucketNum - 1; i >= (int)memoryDominatePos; --i) {   // :144-157
    std::pop_heap(all.begin(), all.end() - finished, GreatCmp());
    Bucket& cb = *(all.rbegin() + finished);
    int d = idrt[i].second;
    members[cb.slot].push_back(idrt[i].first);
    cb.ms += (bw[d] - ebw[d]) / BUCKETSIZE;
    if ((int)members[cb.slot].size() >= BUCKETSIZE) ++finished;
    else std::push_heap(all.begin(), all.end() - finished, GreatCmp());
  }
  std::make_heap(all.begin(), all.end() - finished, LessCmp());     // :163
  for (unsigned i = 0; i < memoryDominatePos; ++i) {                // :165-177
    std::pop_heap(all.begin(), all.end() - finished, LessCmp());
    Bucket& cb = *(all.rbegin() + finished);
    int d = idrt[i].second;
    members[cb.slot].push_back(idrt[i].first);
    cb.ms -= (ebw[d] - bw[d]) / BUCKETSIZE;
    if ((int)members[cb.slot].size() >= BUCKETSIZE) ++finished;
    else std::push_heap(all.begin(), all.end() - finished, LessCmp());
  }
  std::sort_heap(all.begin(), all.end(), IdSort());                 // :181 (not a heap under IdSort)
  std::vector<int> order;                                           // :186-198
  order.reserve(maxNodeId + 1);
  for (int i = 0; i < totalBucketNum; ++i)
    for (int v : members[all[i].slot]) order.push_back(v);
  for (size_t i = (size_t)totalBucketNum * BUCKETSIZE; i < idrt.size(); ++i) order.push_back(idrt[i].first);
  if (maxRt >= 1) for (int v : bucket[1]) order.push_back(v);
  for (int v : bucket[0]) order.push_back(v);
  for (int i = 0; i <= maxNodeId; ++i) lookup[order[i]] = i;        // :206-210
  for (uint64_t i = 0; i < np; ++i) {                               // :219-228
    normal[2 * i] = e[i].first;
    normal[2 * i + 1] = e[i].second;
    reordered[2 * i] = lookup[e[i].first];
    reordered[2 * i + 1] = lookup[e[i].second];
  }
  return ORC_OK;
}

// k-cliques (k >= 3) of the simple graph, the quantity kcl_gpu_solver accumulates
// (k-clique/kcl.cu:147-215): embeddings of a DAG extended level by level by vertices
// adjacent to every member (is_all_connected_dag), counted at level k-2.  Restated as
// a depth-first intersection over a degree-ranked DAG (rank by (degree, id); N+(r) =
// higher-ranked neighbours), which keeps hub candidate sets small; the count does not
// depend on the acyclic orientation.
namespace {

struct RankDag {
  int64_t n = 0;
  std::vector<int64_t> off;
  std::vector<int32_t> nbr;  // per rank, higher ranks, sorted
};

RankDag rank_dag(const Adj& g, int nthreads) {
  RankDag d;
  d.n = g.n;
  std::vector<int32_t> order(g.n), rank(g.n);
  for (int64_t v = 0; v < g.n; ++v) order[v] = (int32_t)v;
  std::sort(order.begin(), order.end(), [&](int32_t a, int32_t b) {
    int64_t da = g.off[a + 1] - g.off[a], db = g.off[b + 1] - g.off[b];
    return da < db || (da == db && a < b);
  });
  for (int64_t r = 0; r < g.n; ++r) rank[order[r]] = (int32_t)r;
  std::vector<int64_t> len(g.n + 1, 0);
  for (int64_t v = 0; v < g.n; ++v)
    for (int64_t j = g.off[v]; j < g.off[v + 1]; ++j)
      if (rank[g.nbr[j]] > rank[v]) len[rank[v] + 1]++;
  d.off.assign(g.n + 1, 0);
  for (int64_t r = 0; r < g.n; ++r) d.off[r + 1] = d.off[r] + len[r + 1];
  d.nbr.resize(d.off[g.n]);
  parallel_for(g.n, nthreads, 1024, [&](int64_t v, int) {
    int32_t r = rank[v];
    int64_t at = d.off[r];
    for (int64_t j = g.off[v]; j < g.off[v + 1]; ++j)
      if (rank[g.nbr[j]] > r) d.nbr[at++] = rank[g.nbr[j]];
    std::sort(d.nbr.begin() + d.off[r], d.nbr.begin() + d.off[r + 1]);
  });
  return d;
}

// k-cliques whose lowest-ranked vertex is r.
uint64_t cliques_from(const RankDag& d, int64_t r, int k) {
  std::vector<std::vector<int32_t>> lv(k);
  lv[0].assign(d.nbr.begin() + d.off[r], d.nbr.begin() + d.off[r + 1]);
  struct Rec {
    const RankDag& d; std::vector<std::vector<int32_t>>& lv; int k;
    uint64_t go(int depth) {  // depth chosen vertices; candidates lv[depth-1]
      const auto& c = lv[depth - 1];
      if (depth == k - 1) return c.size();
      uint64_t s = 0;
      for (int32_t v : c) {
        auto& nxt = lv[depth];
        nxt.clear();
        std::set_intersection(c.begin(), c.end(), d.nbr.begin() + d.off[v], d.nbr.begin() + d.off[v + 1],
                              std::back_inserter(nxt));
        if ((int)nxt.size() >= k - 1 - depth) s += go(depth + 1);
      }
      return s;
    }
  } rec{d, lv, k};
  return rec.go(1);
}

}  // namespace

uint64_t orc_kclique(const int32_t* pairs, uint64_t np, int k, int nthreads) {
  Adj g = build_adj(pairs, np);
  if (k < 1) return 0;
  if (k == 1) return (uint64_t)g.n;
  if (k == 2) return (uint64_t)g.nbr.size() / 2;
  RankDag d = rank_dag(g, nthreads);
  std::vector<uint64_t> part(std::max(1, nthreads), 0);
  parallel_for(d.n, nthreads, 64, [&](int64_t r, int t) { part[t] += cliques_from(d, r, k); });
  uint64_t total = 0;
  for (auto x : part) total += x;
  return total;
}

// The same count restricted to cliques whose lowest-ranked vertex has rank r with
// r % stride == phase: the bounded sample the CPU baseline times.  *edges_out = edges
// out of the sampled ranks.
uint64_t orc_kclique_sample(const int32_t* pairs, uint64_t np, int k, int64_t stride, int64_t phase, int nthreads,
                            int64_t* edges_out) {
  Adj g = build_adj(pairs, np);
  RankDag d = rank_dag(g, nthreads);
  int64_t nsamp = phase < d.n ? (d.n - phase + stride - 1) / stride : 0;
  std::vector<uint64_t> part(std::max(1, nthreads), 0);
  std::vector<int64_t> epart(std::max(1, nthreads), 0);
  parallel_for(nsamp, nthreads, 16, [&](int64_t i, int t) {
    int64_t r = phase + i * stride;
    epart[t] += d.off[r + 1] - d.off[r];
    part[t] += k >= 3 ? cliques_from(d, r, k) : 0;
  });
  uint64_t total = 0;
  int64_t e = 0;
  for (size_t t = 0; t < part.size(); ++t) { total += part[t]; e += epart[t]; }
  *edges_out = e;
  return total;
}

// costFuncCal (tools/costFuncCal.cpp:15-88): out = {idPartCost, degreePartCost, lpPartCost}.
void orc_costfunc(const int32_t* pairs, uint64_t np, int k, float* out) {
  unsigned edgeNum = (unsigned)np;
  unsigned maxNode = 0;
  for (unsigned i = 0; i < edgeNum; ++i) {                          // :27-31
    unsigned s = (unsigned)pairs[2 * i], d = (unsigned)pairs[2 * i + 1];
    maxNode = s > maxNode ? s : maxNode;
    maxNode = d > maxNode ? d : maxNode;
  }
  unsigned nodeNum = maxNode + 1;
  float avg = (float)edgeNum / nodeNum;                             // :34
  std::vector<int> deg(nodeNum, 0), idd(nodeNum, 0), dd(nodeNum, 0), lp(nodeNum, 0);
  for (unsigned i = 0; i < edgeNum; ++i) {                          // :44-49
    deg[pairs[2 * i]]++;
    deg[pairs[2 * i + 1]]++;
    lp[pairs[2 * i]]++;
  }
  for (unsigned i = 0; i < edgeNum; ++i) {                          // :50-61
    int s = pairs[2 * i], d = pairs[2 * i + 1];
    if (s < d) idd[s]++; else idd[d]++;
    if (deg[s] < deg[d] || (deg[s] == deg[d] && s < d)) dd[s]++; else dd[d]++;
  }
  auto fabs_ = [](float a) { return a > 0 ? a : -a; };              // :11-13
  float idPart = 0, dPart = 0, lpPart = 0;
  float thr = k * avg;                                              // :66
  for (int i = 0; i < (int)nodeNum; ++i) {                          // :67-82
    float c = fabs_(idd[i] - avg);
    if (idd[i] - avg > thr) idPart += c;
    c = fabs_(dd[i] - avg);
    if (dd[i] - avg > thr) dPart += c;
    c = fabs_(lp[i] - avg);
    if (lp[i] - avg > thr) lpPart += c;
  }
  out[0] = idPart;
  out[1] = dPart;
  out[2] = lpPart;
}

// verification (tools/verification.cpp:11-61, a text-input tool; the caller parses
// the text): out = {f_lp, f_degree}.  The degree sum skips the last vertex (:58).
void orc_verification(const int32_t* pairs, uint64_t np, float* out) {
  int maxNodeId = 0;
  for (uint64_t i = 0; i < np; ++i) {
    maxNodeId = pairs[2 * i] > maxNodeId ? pairs[2 * i] : maxNodeId;
    maxNodeId = pairs[2 * i + 1] > maxNodeId ? pairs[2 * i + 1] : maxNodeId;
  }
  float dAve = (float)np / (maxNodeId + 1);
  std::vector<int> lpd(maxNodeId + 1, 0), deg(maxNodeId + 1, 0), rt(maxNodeId + 1, 0);
  for (uint64_t i = 0; i < np; ++i) {
    lpd[pairs[2 * i]]++;
    deg[pairs[2 * i]]++;
    deg[pairs[2 * i + 1]]++;
  }
  float f_lp = 0;
  for (int i = 0; i <= maxNodeId; ++i) f_lp += std::abs(dAve - lpd[i]);
  for (uint64_t i = 0; i < np; ++i) {
    int s = pairs[2 * i], d = pairs[2 * i + 1];
    if (deg[s] > deg[d] || (deg[s] == deg[d] && s < d)) rt[d]++;
    else rt[s]++;
  }
  float f_deg = 0;
  for (int i = 0; i < maxNodeId; ++i) f_deg += std::abs(rt[i] - dAve);
  out[0] = f_lp;
  out[1] = f_deg;
}

// Hu preTC CSR (Hu/preTC.cu:64-296): degree orientation over the raw pairs (src =
// lower degree, ties to the larger id as src, :125-133), vertices of degree <= 1
// dropped and ids compacted by prefix (:135-169), edges sorted by (src,dst) and merged
// into CSR skipping self-loops and repeats (:186-284).  Outputs the CSR without the
// kernel's sentinels: offsets (n+1 uint32), cols (m int32).  Returns n; *m_out = m.
// Call with offsets == nullptr first to size the buffers.
int64_t orc_hu_csr(const int32_t* pairs, uint64_t np, uint32_t* offsets, int32_t* cols, int64_t* m_out) {
  int64_t mx = max_id(pairs, np);
  int64_t nodeNum = mx + 1;
  std::vector<int> deg(nodeNum, 0);
  for (uint64_t i = 0; i < np; ++i) { deg[pairs[2 * i]]++; deg[pairs[2 * i + 1]]++; }
  std::vector<int64_t> mini(nodeNum, 0);
  int64_t tot = 0;
  for (int64_t i = 0; i < nodeNum; ++i) { if (deg[i] <= 1) ++tot; mini[i] = tot; }
  std::vector<uint64_t> keys;
  keys.reserve(np);
  for (uint64_t i = 0; i < np; ++i) {
    uint32_t s = (uint32_t)pairs[2 * i], d = (uint32_t)pairs[2 * i + 1];
    if (deg[s] > deg[d] || (deg[s] == deg[d] && s < d)) std::swap(s, d);
    if (deg[s] <= 1 || deg[d] <= 1) continue;
    if (s > 0) s -= (uint32_t)mini[s - 1];
    if (d > 0) d -= (uint32_t)mini[d - 1];
    if (s == d) continue;
    keys.push_back(((uint64_t)s << 32) | d);
  }
  std::sort(keys.begin(), keys.end());
  keys.erase(std::unique(keys.begin(), keys.end()), keys.end());
  int64_t n = nodeNum - tot;
  *m_out = (int64_t)keys.size();
  if (!offsets) return n;
  std::fill(offsets, offsets + n + 1, 0u);
  for (auto k : keys) offsets[(k >> 32) + 1]++;
  for (int64_t i = 0; i < n; ++i) offsets[i + 1] += offsets[i];
  for (size_t i = 0; i < keys.size(); ++i) cols[i] = (int32_t)(keys[i] & 0xffffffffu);
  return n;
}

// Directed-wedge count W = Σ_v d-(v)·d+(v) of an oriented CSR (offsets int64, n+1).
uint64_t orc_wedges(const int64_t* off, const int32_t* cols, int64_t n) {
  std::vector<uint64_t> indeg(n, 0);
  for (int64_t i = 0; i < off[n]; ++i) indeg[cols[i]]++;
  uint64_t w = 0;
  for (int64_t v = 0; v < n; ++v) w += indeg[v] * (uint64_t)(off[v + 1] - off[v]);
  return w;
}

// Core numbers of the simple graph by the Batagelj-Zaversnik bucket algorithm, the
// intent of edge_directing/kcore_direction.cpp:91-146 (which counts degrees over only
// the first node_num edges, :35-38).  core (n ints).
void orc_core_numbers(const int32_t* pairs, uint64_t np, int32_t* core) {
  Adj g = build_adj(pairs, np);
  int64_t n = g.n;
  std::vector<int64_t> deg(n), pos(n), vert(n);
  int64_t md = 0;
  for (int64_t v = 0; v < n; ++v) { deg[v] = g.off[v + 1] - g.off[v]; md = std::max(md, deg[v]); }
  std::vector<int64_t> bin(md + 2, 0);
  for (int64_t v = 0; v < n; ++v) bin[deg[v]]++;
  int64_t start = 0;
  for (int64_t d = 0; d <= md; ++d) { int64_t c = bin[d]; bin[d] = start; start += c; }
  for (int64_t v = 0; v < n; ++v) { pos[v] = bin[deg[v]]++; vert[pos[v]] = v; }
  for (int64_t d = md; d >= 1; --d) bin[d] = bin[d - 1];
  bin[0] = 0;
  for (int64_t i = 0; i < n; ++i) {
    int64_t v = vert[i];
    for (int64_t j = g.off[v]; j < g.off[v + 1]; ++j) {
      int64_t u = g.nbr[j];
      if (deg[u] > deg[v]) {
        int64_t du = deg[u], pu = pos[u], pw = bin[du], w = vert[pw];
        if (u != w) { pos[u] = pw; vert[pu] = w; pos[w] = pu; vert[pw] = u; }
        bin[du]++;
        deg[u]--;
      }
    }
  }
  for (int64_t v = 0; v < n; ++v) core[v] = (int32_t)deg[v];
}

// The approximate parallel A-direction program, step for step
// (edge_directing/A-direction-parallel/peel.cu:130-317, buildCSR.cu:75-201): the simple
// symmetric CSR of the input (loops and repeats dropped), the float threshold
// (float)edgeNum/2/nodeNum over directed entries, frontiers collected in id order
// (thrust::copy_if), advance marking unpeeled neighbours (:77-95), back_nbr_count from the
// reached side (:96-117), the depth / 90 % / 50-iteration stopping rules (:217-262) and the
// per-edge output comparison (:44-59).  Input: packed uint64 edges (src = x >> 32).
// Outputs: flags, minor (n each), oriented (ne), iterations.
void orc_adirection_par(const uint64_t* edges, uint64_t ne, int compat, uint64_t* oriented, uint32_t* flags_out,
                        uint32_t* minor_out, int32_t* iterations) {
  std::vector<int32_t> pairs(2 * ne);
  for (uint64_t i = 0; i < ne; ++i) {
    pairs[2 * i] = (int32_t)(uint32_t)(edges[i] >> 32);
    pairs[2 * i + 1] = (int32_t)(uint32_t)edges[i];
  }
  Adj g = build_adj(pairs.data(), ne);
  const uint32_t node_num = (uint32_t)g.n;
  const uint32_t edge_num = (uint32_t)g.off[g.n];
  const uint32_t MAXV = 0xFFFFFFFFu;
  std::vector<uint32_t> flags(node_num, MAXV), rd(node_num), minor(node_num);
  for (uint32_t v = 0; v < node_num; ++v) rd[v] = minor[v] = (uint32_t)(g.off[v + 1] - g.off[v]);
  const float deg_thre = (float)edge_num / 2 / node_num;
  auto collect = [&](uint32_t limit) {
    std::vector<uint32_t> f;
    for (uint32_t v = 0; v < node_num; ++v)
      if (rd[v] <= limit) f.push_back(v);
    return f;
  };
  auto take = [&](const std::vector<uint32_t>& f, uint32_t it) {
    for (uint32_t v : f) flags[v] = it;
    for (uint32_t v : f) minor[v] = rd[v];
    for (uint32_t v : f) rd[v] = MAXV;
  };
  std::vector<uint32_t> F = collect((uint32_t)deg_thre);
  uint32_t visited = (uint32_t)F.size();
  take(F, 1);
  uint32_t depth = 1, it = 1;
  std::vector<uint8_t> reached(node_num), last(node_num);
  while (visited < node_num * 9 / 10 && depth < 0xFF && it < 50) {
    ++it;
    std::fill(reached.begin(), reached.end(), 0);
    for (uint32_t u : F)
      for (int64_t j = g.off[u]; j < g.off[u + 1]; ++j)
        if (flags[g.nbr[j]] == MAXV) reached[g.nbr[j]] = 1;
    std::fill(last.begin(), last.end(), 0);
    for (uint32_t u : F) last[u] = 1;
    for (uint32_t w = 0; w < node_num; ++w) {
      if (!reached[w]) continue;
      uint32_t sum = 0;
      for (int64_t j = g.off[w]; j < g.off[w + 1]; ++j) sum += last[g.nbr[j]] != 0;
      rd[w] -= sum;
    }
    F = collect((uint32_t)deg_thre * depth);
    while (F.empty() && depth < 0xFF && visited < 9 * node_num / 10) {
      ++depth;
      F = collect((uint32_t)deg_thre * depth);
    }
    visited += (uint32_t)F.size();
    take(F, it);
    if (F.size() <= node_num / 500) ++depth;
  }
  for (uint64_t i = 0; i < ne; ++i) {
    uint32_t a = (uint32_t)(edges[i] >> 32), b = (uint32_t)edges[i];
    int flag_d = (int)flags[a] - flags[b];
    int minor_d = (int)minor[a] - (compat ? flags[b] : minor[b]);
    if (flag_d > 0 || (flag_d == 0 && minor_d > 0) || (flag_d == 0 && minor_d == 0 && a > b)) std::swap(a, b);
    oriented[i] = ((uint64_t)a << 32) | b;
  }
  if (flags_out) std::copy(flags.begin(), flags.end(), flags_out);
  if (minor_out) std::copy(minor.begin(), minor.end(), minor_out);
  if (iterations) *iterations = (int32_t)it;
}

// std::random_shuffle(first, first + len) as libstdc++ writes it (bits/stl_algo.h): for
// i = 1 .. len-1, swap a[i] with a[rand() % (i + 1)], rand() being the C library's.
static void orc_random_shuffle(int* a, int64_t len) {
  for (int64_t i = 1; i < len; ++i) {
    const int64_t j = std::rand() % (i + 1);
    if (i != j) std::swap(a[i], a[j]);
  }
}

// Rank relabellings of vertex_ordering/A-order: kind 0 = "good" of relabel-naive.cpp /
// relabel-random.cpp (:29-74), kind 1 = "naive" of A-order-v2.cpp (:29-160), kind 2 =
// "good" of relabel4lpOut.cpp (:27-54, out-degree as given), kind 5 = "naive" of
// relabel-naive.cpp (:77-177: 64 columns, odd ones backwards, blocks of 64 shuffled),
// kind 6 = "bad" of relabel4lpOut.cpp (:57-136: the same with 40 and out-degree as given),
// kind 7 = "bad" of relabel-random.cpp (:76-108: every id shuffled).  The shuffles use the
// C library's rand() from its seed-1 state (srand(1) here; the programs never seed it).
// Degrees count repeats; the degree orientation flips a pair when src has the larger
// degree or equal degree and the smaller id.  lookup: maxNodeId + 1 ints (maxNodeId starts
// at 0); normal: np pairs.
void orc_relabel(const int32_t* pairs, uint64_t np, int kind, int32_t* lookup, int32_t* normal) {
  int max_node = 0;
  for (uint64_t i = 0; i < 2 * np; ++i) max_node = std::max(max_node, pairs[i]);
  const int n = max_node + 1;
  const bool as_given = kind == 2 || kind == 6;
  std::vector<int> degree(n, 0), rt(n, 0);
  for (uint64_t i = 0; i < np; ++i) {
    degree[pairs[2 * i]]++;
    if (!as_given) degree[pairs[2 * i + 1]]++;
  }
  for (uint64_t i = 0; i < np; ++i) {
    int src = pairs[2 * i], dst = pairs[2 * i + 1];
    if (!as_given && (degree[src] > degree[dst] || (degree[src] == degree[dst] && src < dst))) std::swap(src, dst);
    normal[2 * i] = src;
    normal[2 * i + 1] = dst;
    rt[src]++;
  }
  if (as_given) rt = degree;
  if (kind == 7) {
    std::vector<int> bad(n);
    for (int i = 0; i < n; ++i) bad[i] = i;
    std::srand(1);
    orc_random_shuffle(bad.data(), n);
    for (int i = 0; i < n; ++i) lookup[bad[i]] = i;
    return;
  }
  int max_rt = 0;
  for (int v = 0; v < n; ++v) max_rt = std::max(max_rt, rt[v]);
  std::vector<std::vector<int>> bucket(max_rt + 1);
  for (int v = 0; v < n; ++v) bucket[rt[v]].push_back(v);
  std::vector<int> order;  // ascending (rt, id)
  for (int r = 0; r <= max_rt; ++r) order.insert(order.end(), bucket[r].begin(), bucket[r].end());
  if (kind == 0 || kind == 2) {
    for (int i = 0; i < n; ++i) lookup[order[i]] = n - 1 - i;
    return;
  }
  std::reverse(order.begin(), order.end());
  const bool shuffled = kind == 5 || kind == 6;
  const int mix = kind == 5 ? 64 : 40, chunk = n / mix;
  std::vector<int> distri(n, 0);
  for (int i = 0; i < mix; ++i) {
    const bool backwards = shuffled && (i & 1);
    for (int j = 0; j < chunk; ++j)
      distri[i + j * mix] = backwards ? order[(i + 1) * chunk - 1 - j] : order[i * chunk + j];
  }
  if (shuffled) {
    std::srand(1);
    for (int i = 0; i < chunk; ++i) orc_random_shuffle(distri.data() + (int64_t)i * mix, mix);
  }
  for (int i = n - n % mix; i < n; ++i) distri[i] = order[i];
  for (int i = 0; i < n; ++i) lookup[distri[i]] = i;
}

// Masked-MSE loss and gradients of the selector MLP in double precision: the checker for
// the library's FP32 training kernels.  Same parameter layout (W1[I][H] b1 W2[H][H] b2
// W3[H][O] b3), ReLU hidden layers, inputs standardised with (mean, std) first.
void orc_mlp_grad(const float* params, int I, int H, int O, const float* mean, const float* stdv, const float* x,
                  const float* t, const float* mask, int B, double* grads, double* loss) {
  const float* W1 = params;
  const float* b1 = W1 + (int64_t)I * H;
  const float* W2 = b1 + H;
  const float* b2 = W2 + (int64_t)H * H;
  const float* W3 = b2 + H;
  const float* b3 = W3 + (int64_t)H * O;
  int64_t np = (int64_t)I * H + H + (int64_t)H * H + H + (int64_t)H * O + O;
  std::fill(grads, grads + np, 0.0);
  double* gW1 = grads;
  double* gb1 = gW1 + (int64_t)I * H;
  double* gW2 = gb1 + H;
  double* gb2 = gW2 + (int64_t)H * H;
  double* gW3 = gb2 + H;
  double* gb3 = gW3 + (int64_t)H * O;
  double msum = 0;
  for (int64_t k = 0; k < (int64_t)B * O; ++k) msum += mask ? mask[k] : 1.0;
  if (msum <= 0) msum = 1;
  double L = 0;
  std::vector<double> xs(I), a1(H), a2(H), y(O), dy(O), d2(H), d1(H);
  for (int b = 0; b < B; ++b) {
    for (int i = 0; i < I; ++i) xs[i] = ((double)x[(int64_t)b * I + i] - mean[i]) / (stdv[i] > 0 ? stdv[i] : 1.0);
    for (int j = 0; j < H; ++j) {
      double z = b1[j];
      for (int i = 0; i < I; ++i) z += xs[i] * W1[(int64_t)i * H + j];
      a1[j] = z > 0 ? z : 0;
    }
    for (int j = 0; j < H; ++j) {
      double z = b2[j];
      for (int i = 0; i < H; ++i) z += a1[i] * W2[(int64_t)i * H + j];
      a2[j] = z > 0 ? z : 0;
    }
    for (int o = 0; o < O; ++o) {
      double z = b3[o];
      for (int i = 0; i < H; ++i) z += a2[i] * W3[(int64_t)i * O + o];
      y[o] = z;
      double mk = mask ? mask[(int64_t)b * O + o] : 1.0;
      double d = z - t[(int64_t)b * O + o];
      L += mk * d * d;
      dy[o] = mk * d / msum;
    }
    for (int o = 0; o < O; ++o) {
      gb3[o] += dy[o];
      for (int i = 0; i < H; ++i) gW3[(int64_t)i * O + o] += a2[i] * dy[o];
    }
    for (int i = 0; i < H; ++i) {
      double acc = 0;
      for (int o = 0; o < O; ++o) acc += dy[o] * W3[(int64_t)i * O + o];
      d2[i] = a2[i] > 0 ? acc : 0;
    }
    for (int j = 0; j < H; ++j) {
      gb2[j] += d2[j];
      for (int i = 0; i < H; ++i) gW2[(int64_t)i * H + j] += a1[i] * d2[j];
    }
    for (int i = 0; i < H; ++i) {
      double acc = 0;
      for (int j = 0; j < H; ++j) acc += d2[j] * W2[(int64_t)i * H + j];
      d1[i] = a1[i] > 0 ? acc : 0;
    }
    for (int j = 0; j < H; ++j) {
      gb1[j] += d1[j];
      for (int i = 0; i < I; ++i) gW1[(int64_t)i * H + j] += xs[i] * d1[j];
    }
  }
  *loss = 0.5 * L / msum;
}


// GRO order (vertex_ordering/other_order/porder.cpp:141-226, POrder::greedy_mheap) of the
// directed edges `edges` (uint64 words, source in the high half: util.cpp:56-67).  Edges
// are sorted as POrder::build sorts them (porder.cpp:94-123, repeats kept); vertices are
// taken in windows of 32 (PACK_WIDTH, util.hpp:21-27): a window opens with the first
// unplaced vertex in (degree desc, id asc) order, and each next vertex is the head of
// the gain list, where every placed u adds one to each unplaced w that shares an
// in-neighbour's out-list or an out-neighbour's in-list with u (each neighbour once per
// window).  new_id (v_num = max id + 1 ints) receives the order: org2newid of the
// program's _GRO_newID.txt.  Returns v_num.  *max_gain (nullable) = the largest gain any
// key reached: the program's gain headers hold 2 * v_num entries of which only the first
// v_num are initialised (linkedlist_heap.cpp:9-18), so its output is defined only while
// max_gain < v_num.
int32_t orc_gro(const uint64_t* edges, uint64_t ne, int32_t* new_id, int32_t* max_gain) {
  std::vector<std::pair<int, int>> ev(ne);
  int vn = 0;
  for (uint64_t i = 0; i < ne; ++i) {
    ev[i] = {(int)(edges[i] >> 32), (int)(edges[i] & 0xffffffffu)};
    vn = std::max(vn, std::max(ev[i].first, ev[i].second));
  }
  if (ne == 0) return 0;
  ++vn;
  if (!new_id) return vn;
  std::sort(ev.begin(), ev.end());
  std::vector<int> od(vn, 0), id(vn, 0), os(vn + 1, 0), is(vn + 1, 0), oe(ne), ie(ne);
  for (const auto& e : ev) {
    ++od[e.first];
    ++id[e.second];
  }
  for (int v = 0; v < vn; ++v) {
    os[v + 1] = os[v] + od[v];
    is[v + 1] = is[v] + id[v];
  }
  std::vector<int> ipos(is.begin(), is.end() - 1);
  for (uint64_t i = 0; i < ne; ++i) {
    oe[i] = ev[i].second;
    ie[ipos[ev[i].second]++] = ev[i].first;
  }
  std::vector<int> by_deg(vn);
  for (int v = 0; v < vn; ++v) by_deg[v] = v;
  std::sort(by_deg.begin(), by_deg.end(), [&](int a, int b) {
    const int da = od[a] + id[a], db = od[b] + id[b];
    return da == db ? a < b : da > db;
  });
  std::vector<char> placed(vn, 0);
  size_t cursor = 0;  // the first vertex of by_deg not yet placed (doublelinked_list.cpp pop_head)
  GroGainList gains(vn);
  std::vector<int> out_mark(vn, -1), in_mark(vn, -1);
  const int kWindow = 32;
  int window = -1;
  for (int idx = 0; idx < vn; ++idx) {
    int u;
    if (idx % kWindow == 0) {
      while (placed[by_deg[cursor]]) ++cursor;
      u = by_deg[cursor];
      gains.reset();
      gains.del(u);
      ++window;
    } else {
      u = gains.pop();
    }
    placed[u] = 1;
    new_id[u] = idx;
    for (int j = is[u]; j < is[u + 1]; ++j) {
      const int v = ie[j];
      if (out_mark[v] == window) continue;
      out_mark[v] = window;
      for (int k = os[v]; k < os[v + 1]; ++k)
        if (gains.has(oe[k])) gains.inc(oe[k]);
    }
    for (int j = os[u]; j < os[u + 1]; ++j) {
      const int v = oe[j];
      if (in_mark[v] == window) continue;
      in_mark[v] = window;
      for (int k = is[v]; k < is[v + 1]; ++k)
        if (gains.has(ie[k])) gains.inc(ie[k]);
    }
  }
  if (max_gain) *max_gain = gains.max_gain();
  return vn;
}


// Seeded R-MAT samples of the benchmark workloads, written independently of libatc so that
// the CPU arm of the benchmark builds its input without loading the product library.  The
// generator is the benchmark's own (no reference counterpart: the reference reads dataset
// files): splitmix64 (Steele, Lea, Flood 2014) over a counter, two 32-bit draws per 64-bit
// output, one draw per recursion level, quadrant thresholds a, a+b, a+b+c in parts per
// million scaled to 2^32, row bit then column bit chosen most-significant first.  A CPU test
// checks that the bytes equal atc_gen_rmat_host's.
static uint64_t orc_splitmix(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

int orc_gen_rmat(uint32_t scale, uint32_t edge_factor, uint32_t a_ppm, uint32_t b_ppm, uint32_t c_ppm, uint64_t seed,
                 int32_t* out, int nthreads) {
  const uint64_t sa = a_ppm, sb = sa + b_ppm, sc = sb + c_ppm;
  if (sc > 1000000ull || scale < 1 || scale > 30) return 1;
  const uint32_t t1 = (uint32_t)((sa << 32) / 1000000ull), t2 = (uint32_t)((sb << 32) / 1000000ull);
  const uint32_t t3 = sc == 1000000ull ? 0xFFFFFFFFu : (uint32_t)((sc << 32) / 1000000ull);
  const uint64_t count = (uint64_t)edge_factor << scale;
  const uint64_t golden = 0x9E3779B97F4A7C15ull, s0 = orc_splitmix(seed);
  parallel_for((int64_t)count, nthreads, 1 << 16, [&](int64_t i, int) {
    uint32_t row = 0, col = 0;
    uint64_t r = 0;
    for (uint32_t l = 0; l < scale; ++l) {
      if ((l & 1) == 0) r = orc_splitmix(s0 + ((uint64_t)i * 16 + (l >> 1) + 1) * golden);
      const uint32_t x = (l & 1) ? (uint32_t)(r >> 32) : (uint32_t)r;
      row = (row << 1) | (uint32_t)(x >= t2);
      col = (col << 1) | (uint32_t)((x >= t1 && x < t2) || x >= t3);
    }
    out[2 * i] = (int32_t)row;
    out[2 * i + 1] = (int32_t)col;
  });
  return 0;
}

}  // extern "C"
