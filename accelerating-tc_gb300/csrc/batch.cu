// Batched triangle counting: many graphs of uneven sizes counted together.
//
// The reference runs one program per graph.  Here the graphs of a batch are kept as one
// disjoint union on the device (graph g owns vertices [vbase[g], vbase[g+1])), and one
// replay of a CUDA graph counts all of them: the Bisson-style grouping passes run once
// over the union, the persistent counting kernels drain its work items from device
// counters, and every item adds its triangles to its own graph's counter.  Nothing in
// the replay waits on the host, so small graphs cost no launch or synchronisation of
// their own — the overhead a per-graph loop pays 4096 times.
//
// Memory, per union vertex / edge: offsets 8 B, cols 4 B, group count / cursor 8 B,
// group starts 8 B, grouped partner list <= 4 B per edge, work items 8 B each.  No
// per-edge source array is kept (the grouping passes walk rows).
#include <algorithm>
#include <cstring>
#include <vector>

#include "bisson.cuh"

struct atc_batch {
  int64_t n = 0, m = 0;        // vertices / edges held
  int64_t vcap = 0, ecap = 0;  // allocated
  int64_t* off = nullptr;      // vcap + 1
  int32_t* cols = nullptr;     // ecap + 16
  std::vector<int64_t> vbase{0};
  std::vector<int64_t> gm, gw, gwmin;  // per graph: edges, W, sum of min(d+u, d+v)
  int32_t max_outdeg = 0;
  bool dirty = true;
  int rows_graphs = 0;  // graphs of the last built pipeline counted by rows
  int launches = 0;     // kernel launches of one replay of the built pipeline
  atc::ItemShape shape = atc::default_shape(32);
  // counting pipeline, sized for the union when built
  int32_t* cnt = nullptr;
  int32_t* cur = nullptr;
  int64_t* gstart = nullptr;
  int32_t* plist = nullptr;
  int2* items = nullptr;
  int* counters = nullptr;
  int2* items_r = nullptr;   // mode 2: the rows items of the graphs counted by rows
  int* counters_r = nullptr;
  int2* big = nullptr;       // block items of lists longer than kBlockSmallList
  int2* big_r = nullptr;     // the same for the rows items
  int64_t big_cap = 0;
  uint8_t* vrows = nullptr;  // mode 2: 1 for the vertices of graphs counted by rows
  int64_t* vbase_d = nullptr;
  unsigned long long* gcounts = nullptr;
  void* scan_tmp = nullptr;
  int64_t built_n = -1, built_m = -1, items_cap = 0;
  int built_graphs = -1;
  atc::ItemShape built_shape{};
  cudaStream_t cap_stream = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  // event nodes of the replay: stage k runs from stage_ev[k] to stage_ev[k + 1]
  std::vector<cudaEvent_t> stage_ev;
  std::vector<const char*> stage_name;
};

namespace atc {
namespace {

// counters of one replay: [0] warp items, [1] block items, [2] block items of long lists,
// [3] longest list among [1], [4..6] the counting kernels' item cursors, [8], [9] the
// grouping passes' row-block queues
constexpr int kBatchCounters = 16;

__global__ void batch_copy_kernel(const int64_t* off_g, const int32_t* cols_g, int64_t n_g, int64_t m_g,
                                  int64_t vbase, int64_t ebase, int64_t* off_u, int32_t* cols_u) {
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n_g || i < m_g; i += stride) {
    if (i < n_g) off_u[vbase + i] = off_g[i] + ebase;
    if (i < m_g) cols_u[ebase + i] = cols_g[i] + (int32_t)vbase;
  }
}

void free_pipeline(atc_batch* b) {
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  b->exec = nullptr;
  b->graph = nullptr;
  void* bufs[] = {b->cnt, b->cur, b->gstart, b->plist, b->items, b->counters, b->vbase_d, b->gcounts, b->scan_tmp,
                  b->items_r, b->counters_r, b->vrows, b->big, b->big_r};
  for (void* p : bufs)
    if (p) cudaFree(p);
  b->cnt = b->cur = b->plist = nullptr;
  b->gstart = b->vbase_d = nullptr;
  b->items = nullptr;
  b->counters = nullptr;
  b->items_r = nullptr;
  b->counters_r = nullptr;
  b->vrows = nullptr;
  b->big = b->big_r = nullptr;
  b->big_cap = 0;
  b->gcounts = nullptr;
  b->scan_tmp = nullptr;
  b->built_n = b->built_m = -1;
  b->built_graphs = -1;
}

template <class T>
atc_status dev_alloc(T** p, size_t count) {
  if (!alloc_budget_take(sizeof(T) * (count ? count : 1))) {
    *p = nullptr;
    set_error("device allocation of %zu bytes for the batch refused: the allocation budget (atc_set_alloc_budget) "
              "is spent", sizeof(T) * count);
    return ATC_ERR_OOM;
  }
  cudaError_t e = cudaMalloc(reinterpret_cast<void**>(p), sizeof(T) * (count ? count : 1));
  if (e != cudaSuccess) {
    *p = nullptr;
    set_error("cudaMalloc(%zu bytes) for the batch: %s", sizeof(T) * count, cudaGetErrorString(e));
    return e == cudaErrorMemoryAllocation ? ATC_ERR_OOM : ATC_ERR_CUDA;
  }
  return ATC_OK;
}

// Grows the union arrays to hold n vertices and m edges (keeping the contents).
atc_status ensure_union(atc_batch* b, int64_t n, int64_t m, cudaStream_t s) {
  if (n <= b->vcap && m <= b->ecap) return ATC_OK;
  int64_t vcap = std::max(n, b->vcap ? 2 * b->vcap : n);
  int64_t ecap = std::max(m, b->ecap ? 2 * b->ecap : m);
  int64_t* off = nullptr;
  int32_t* cols = nullptr;
  ATC_TRY(dev_alloc(&off, (size_t)vcap + 1));
  atc_status st = dev_alloc(&cols, (size_t)ecap + 16);
  if (st != ATC_OK) {
    cudaFree(off);
    return st;
  }
  ATC_CK(cudaMemsetAsync(cols + ecap, 0, sizeof(int32_t) * 16, s));
  if (b->n) ATC_CK(cudaMemcpyAsync(off, b->off, sizeof(int64_t) * b->n, cudaMemcpyDeviceToDevice, s));
  if (b->m) ATC_CK(cudaMemcpyAsync(cols, b->cols, sizeof(int32_t) * b->m, cudaMemcpyDeviceToDevice, s));
  ATC_CK(cudaStreamSynchronize(s));
  if (b->off) cudaFree(b->off);
  if (b->cols) cudaFree(b->cols);
  b->off = off;
  b->cols = cols;
  b->vcap = vcap;
  b->ecap = ecap;
  return ATC_OK;
}

}  // namespace
}  // namespace atc

using namespace atc;

extern "C" atc_status atc_batch_create(atc_batch** out) try {
  ATC_CHECK_ARG(out != nullptr, "out is NULL");
  *out = new atc_batch();
  return ATC_OK;
} ATC_CATCH

extern "C" atc_status atc_batch_reserve(atc_batch* b, int64_t n, int64_t m, atc_stream s) try {
  ATC_CHECK_ARG(b != nullptr && n >= 0 && m >= 0, "bad argument");
  return ensure_union(b, n, m, as_stream(s));
} ATC_CATCH

extern "C" atc_status atc_batch_add(atc_batch* b, const atc_csr* csr, int32_t* index, atc_stream st) try {
  ATC_CHECK_ARG(b != nullptr && csr != nullptr, "NULL argument");
  ATC_CHECK_ARG(b->n + csr->n < (int64_t)INT32_MAX, "batch would exceed 2^31 vertices");
  cudaStream_t s = as_stream(st);
  ATC_TRY(ensure_union(b, b->n + csr->n, b->m + csr->m, s));
  int64_t work = std::max(csr->n, csr->m);
  if (work > 0) {
    batch_copy_kernel<<<grid_for(work, 256), 256, 0, s>>>(csr->offsets, csr->cols, csr->n, csr->m, b->n, b->m,
                                                          b->off, b->cols);
    ATC_CK(cudaGetLastError());
  }
  ATC_CK(cudaStreamSynchronize(s));
  if (index) *index = (int32_t)(b->vbase.size() - 1);
  b->n += csr->n;
  b->m += csr->m;
  b->vbase.push_back(b->n);
  b->gm.push_back(csr->m);
  b->gw.push_back(csr->wedges);
  b->gwmin.push_back(csr->wedges_min);
  b->max_outdeg = std::max(b->max_outdeg, csr->max_outdeg);
  b->dirty = true;
  return ATC_OK;
} ATC_CATCH

extern "C" atc_status atc_batch_info(const atc_batch* b, int32_t* graphs, int64_t* n, int64_t* m) try {
  ATC_CHECK_ARG(b != nullptr, "NULL batch");
  if (graphs) *graphs = (int32_t)(b->vbase.size() - 1);
  if (n) *n = b->n;
  if (m) *m = b->m;
  return ATC_OK;
} ATC_CATCH

extern "C" atc_status atc_batch_destroy(atc_batch* b) try {
  if (!b) return ATC_OK;
  free_pipeline(b);
  if (b->off) cudaFree(b->off);
  if (b->cols) cudaFree(b->cols);
  if (b->cap_stream) cudaStreamDestroy(b->cap_stream);
  for (cudaEvent_t e : b->stage_ev) cudaEventDestroy(e);
  delete b;
  return ATC_OK;
} ATC_CATCH

namespace atc {
namespace {

bool same_shape(const ItemShape& a, const ItemShape& b) {
  return a.cutover == b.cutover && a.warp_max == b.warp_max && a.warp_chunk == b.warp_chunk &&
         a.block_chunk == b.block_chunk && a.by_source == b.by_source;
}

ItemShape shape_from(const atc_tuning* t, const ItemShape& base) {
  ItemShape sh = base;
  if (!t) return sh;
  if (t->bisson_cutover > 0) sh.cutover = std::min(t->bisson_cutover, kWarpMax);
  if (t->bisson_warp_max > 0) sh.warp_max = std::min(t->bisson_warp_max, kWarpHashMax);
  if (t->bisson_warp_chunk > 0) sh.warp_chunk = t->bisson_warp_chunk;
  if (t->bisson_block_chunk > 0) sh.block_chunk = t->bisson_block_chunk;
  if (t->group_by_source > 0) sh.by_source = t->group_by_source >= 2 ? 2 : 1;
  if (sh.cutover > sh.warp_max) sh.cutover = sh.warp_max;
  return sh;
}

// Sizes the scratch for the union and records the counting pipeline into a CUDA graph
// on the batch's own stream (capture is not allowed on the legacy default stream).
atc_status build_pipeline(atc_batch* b, const ItemShape& sh, cudaStream_t s) {
  const int64_t n = b->n, m = b->m;
  const int ng = (int)(b->vbase.size() - 1);
  const int64_t cap_items = max_items(n, m, std::min(sh.warp_chunk, sh.block_chunk));
  // block items of lists longer than kBlockSmallList: one per such list (at most
  // m / (kBlockSmallList + 1) of them) plus one per chunk boundary
  const int64_t big_cap = m / (kBlockSmallList + 1) + m / sh.block_chunk + 1;
  if (b->built_n != n || b->built_m != m || b->built_graphs != ng || b->items_cap < cap_items ||
      b->big_cap < big_cap) {
    free_pipeline(b);
    ATC_TRY(dev_alloc(&b->cnt, (size_t)n + 1));
    ATC_TRY(dev_alloc(&b->cur, (size_t)n + 1));
    ATC_TRY(dev_alloc(&b->gstart, (size_t)n + 1));
    ATC_TRY(dev_alloc(&b->plist, (size_t)m + 32));
    ATC_TRY(dev_alloc(&b->items, (size_t)cap_items));
    ATC_TRY(dev_alloc(&b->counters, kBatchCounters));
    ATC_TRY(dev_alloc(&b->items_r, (size_t)cap_items));
    ATC_TRY(dev_alloc(&b->counters_r, 8));
    ATC_TRY(dev_alloc(&b->vrows, (size_t)n + 1));
    ATC_TRY(dev_alloc(&b->big, (size_t)big_cap));
    ATC_TRY(dev_alloc(&b->big_r, (size_t)big_cap));
    ATC_TRY(dev_alloc(&b->vbase_d, (size_t)ng + 1));
    ATC_TRY(dev_alloc(&b->gcounts, (size_t)ng));
    size_t bytes = 0;
    ATC_TRY(exclusive_scan_i32_to_i64_tmp(nullptr, &bytes, b->cnt, b->gstart, (size_t)n + 1, s));
    ATC_TRY(dev_alloc(reinterpret_cast<char**>(&b->scan_tmp), bytes));
    ATC_CK(cudaMemcpyAsync(b->vbase_d, b->vbase.data(), sizeof(int64_t) * (ng + 1), cudaMemcpyHostToDevice, s));
    b->built_n = n;
    b->built_m = m;
    b->built_graphs = ng;
    b->items_cap = cap_items;
    b->big_cap = big_cap;
  } else if (b->exec) {
    cudaGraphExecDestroy(b->exec);
    cudaGraphDestroy(b->graph);
    b->exec = nullptr;
    b->graph = nullptr;
  }
  ATC_CK(cudaMemcpyAsync(b->off + n, &b->m, sizeof(int64_t), cudaMemcpyHostToDevice, s));
  ATC_CK(cudaStreamSynchronize(s));
  if (!b->cap_stream) ATC_CK(cudaStreamCreateWithFlags(&b->cap_stream, cudaStreamNonBlocking));

  // block tables: lists up to kBlockSmallList at load factor 1/4 (at most 32 KB), and the
  // full 64 KB table for the longer lists, launched apart so that the short lists' CTAs are
  // not held to the occupancy of the largest table
  const void* kblock = (const void*)bisson_block_kernel<CompactItems, kDefaultSlots>;
  uint32_t words = 64;
  const uint32_t want = 4u * (uint32_t)std::min(std::max(b->max_outdeg, 1), kBlockSmallList);
  while (words < want) words <<= 1;
  const bool any_big = b->max_outdeg > kBlockSmallList;
  const uint32_t words_big = kTabWords;
  const size_t smem = sizeof(int32_t) * words, smem_big = sizeof(int32_t) * words_big;
  ATC_CK(cudaFuncSetAttribute(kblock, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)(any_big ? smem_big : smem)));
  const int grid_block = sm_count() * blocks_per_sm(kblock, kBgWarps * 32, smem);
  const int grid_big = sm_count() * blocks_per_sm(kblock, kBgWarps * 32, smem_big);
  const int grid_warp = sm_count() * blocks_per_sm((const void*)bisson_warp_kernel<CompactItems, kDefaultSlots>, kBgWarps * 32, 0);

  CsrView g = csr_view(b->off, b->cols, nullptr, n, m);
  GraphTags tags{b->vbase_d, ng, b->gcounts};
  // grouped at the source, a vertex's partners are its own row: the items index the CSR
  // itself and the grouping passes are skipped
  const int64_t* gstart = sh.by_source == 1 ? b->off : b->gstart;
  const int32_t* plist = sh.by_source == 1 ? b->cols : b->plist;
  CompactItems witems{b->items, gstart, cap_items, false, false, sh};
  CompactItems bitems{b->items, gstart, cap_items, true, true, sh};
  CompactItems litems{b->big, gstart, big_cap, false, true, sh};
  // mode 2: each graph counts by rows (every wedge tested at its source, W tests, no grouping)
  // or grouped at the longer endpoint (sum of min(d+u, d+v) tests plus the grouping passes),
  // whichever the per-graph cost model of the two kernels predicts faster (the per-call terms
  // of the single-graph model do not apply inside one replay)
  const bool mixed = sh.by_source == 2;
  ItemShape shr = sh;
  shr.by_source = 1;
  shr.cutover = std::min(sh.cutover, 8);  // the rows items' sorted copy, as the single-graph Hu count
  CompactItems witems_r{b->items_r, b->off, cap_items, false, false, shr};
  CompactItems bitems_r{b->items_r, b->off, cap_items, true, true, shr};
  CompactItems litems_r{b->big_r, b->off, big_cap, false, true, shr};
  int nrows = 0;
  if (mixed) {
    ATC_CK(cudaMemsetAsync(b->vrows, 0, (size_t)n + 1, s));
    for (int q = 0; q < ng; ++q) {
      const double m_q = (double)b->gm[q];
      const bool rows = 1.097 * (double)b->gw[q] + 103.5 * m_q < 1.232 * (double)b->gwmin[q] + 117.5 * m_q;
      if (rows && b->vbase[q + 1] > b->vbase[q]) {
        ATC_CK(cudaMemsetAsync(b->vrows + b->vbase[q], 1, (size_t)(b->vbase[q + 1] - b->vbase[q]), s));
        ++nrows;
      }
    }
    ATC_CK(cudaStreamSynchronize(s));
  }
  b->rows_graphs = mixed ? nrows : (sh.by_source == 1 ? ng : 0);
  const uint8_t* skip = mixed ? b->vrows : nullptr;
  cudaStream_t c = b->cap_stream;
  size_t bytes = 0;
  ATC_TRY(exclusive_scan_i32_to_i64_tmp(nullptr, &bytes, b->cnt, b->gstart, (size_t)n + 1, s));

  // event nodes between the stages (read by atc_phase_times after a replay)
  constexpr int kMaxStages = 12;
  while (b->stage_ev.size() < (size_t)kMaxStages + 1) {
    cudaEvent_t e = nullptr;
    ATC_CK(cudaEventCreate(&e));
    b->stage_ev.push_back(e);
  }
  b->stage_name.clear();
  int kernels = 0;
  auto stage = [&](const char* name) {
    b->stage_name.push_back(name);
    cudaEventRecordWithFlags(b->stage_ev[b->stage_name.size()], c, cudaEventRecordExternal);
  };

  ATC_CK(cudaStreamBeginCapture(c, cudaStreamCaptureModeThreadLocal));
  cudaEventRecordWithFlags(b->stage_ev[0], c, cudaEventRecordExternal);
  cudaMemsetAsync(b->cnt, 0, sizeof(int32_t) * (n + 1), c);
  cudaMemsetAsync(b->cur, 0, sizeof(int32_t) * (n + 1), c);
  cudaMemsetAsync(b->counters, 0, sizeof(int) * kBatchCounters, c);
  cudaMemsetAsync(b->gcounts, 0, sizeof(unsigned long long) * ng, c);
  stage("batch.reset");
  if (sh.by_source != 1) {
    group_count_vc_kernel<<<grid_for(n * 32, 256), 256, 0, c>>>(g, b->cnt, skip, b->counters + 8);
    exclusive_scan_i32_to_i64_tmp(b->scan_tmp, &bytes, b->cnt, b->gstart, (size_t)n + 1, c);
    group_scatter_vc_kernel<<<grid_for(n * 32, 256), 256, 0, c>>>(g, b->gstart, b->cur, b->plist, skip,
                                                                 b->counters + 9);
    kernels += 4;  // two grouping passes and the scan's two kernels
    stage("batch.group");
  }
  group_items_compact_kernel<<<grid_for(n, 256), 256, 0, c>>>(g, gstart, b->items, cap_items, b->big, b->counters, sh,
                                                              skip, 0);
  kernels += 3;  // items, block, warp
  stage("batch.items");
  bisson_block_kernel<CompactItems, kDefaultSlots><<<grid_block, kBgWarps * 32, smem, c>>>(g, plist, bitems, 0, b->counters + 1,
                                                                            b->counters + 5, words, tags, b->gcounts);
  stage("batch.block");
  if (any_big) {
    bisson_block_kernel<CompactItems, kDefaultSlots><<<grid_big, kBgWarps * 32, smem_big, c>>>(
        g, plist, litems, 0, b->counters + 2, b->counters + 6, words_big, tags, b->gcounts);
    kernels += 1;
    stage("batch.block.long");
  }
  bisson_warp_kernel<CompactItems, kDefaultSlots><<<grid_warp, kBgWarps * 32, 0, c>>>(g, plist, witems, 0, b->counters,
                                                                       b->counters + 4, tags, b->gcounts);
  stage("batch.warp");
  if (mixed && nrows > 0) {
    cudaMemsetAsync(b->counters_r, 0, sizeof(int) * 8, c);
    group_items_compact_kernel<<<grid_for(n, 256), 256, 0, c>>>(g, b->off, b->items_r, cap_items, b->big_r,
                                                                b->counters_r, shr, b->vrows, 1);
    kernels += 3;
    stage("batch.rows.items");
    bisson_block_kernel<CompactItems, kDefaultSlots><<<grid_block, kBgWarps * 32, smem, c>>>(
        g, b->cols, bitems_r, 0, b->counters_r + 1, b->counters_r + 5, words, tags, b->gcounts);
    stage("batch.rows.block");
    if (any_big) {
      bisson_block_kernel<CompactItems, kDefaultSlots><<<grid_big, kBgWarps * 32, smem_big, c>>>(
          g, b->cols, litems_r, 0, b->counters_r + 2, b->counters_r + 6, words_big, tags, b->gcounts);
      kernels += 1;
      stage("batch.rows.block.long");
    }
    bisson_warp_kernel<CompactItems, kDefaultSlots><<<grid_warp, kBgWarps * 32, 0, c>>>(
        g, b->cols, witems_r, 0, b->counters_r, b->counters_r + 4, tags, b->gcounts);
    stage("batch.rows.warp");
  }
  cudaError_t launch_err = cudaGetLastError();
  cudaError_t end_err = cudaStreamEndCapture(c, &b->graph);
  if (launch_err != cudaSuccess || end_err != cudaSuccess) {
    set_error("capturing the batch pipeline: %s", cudaGetErrorString(launch_err != cudaSuccess ? launch_err : end_err));
    if (b->graph) cudaGraphDestroy(b->graph);
    b->graph = nullptr;
    return ATC_ERR_CUDA;
  }
  ATC_CK(cudaGraphInstantiate(&b->exec, b->graph, 0));
  b->built_shape = sh;
  b->launches = kernels;
  b->dirty = false;
  return ATC_OK;
}

atc_status run_once(atc_batch* b, const ItemShape& sh, uint64_t* counts, float* ms, cudaStream_t s) {
  if (b->dirty || !b->exec || !same_shape(sh, b->built_shape)) ATC_TRY(build_pipeline(b, sh, s));
  EventTimer tm;
  tm.start(s);
  ATC_CK(cudaGraphLaunch(b->exec, s));
  tm.stop(s);
  const int ng = (int)(b->vbase.size() - 1);
  if (counts && ng) ATC_CK(cudaMemcpyAsync(counts, b->gcounts, sizeof(uint64_t) * ng, cudaMemcpyDeviceToHost, s));
  ATC_CK(cudaStreamSynchronize(s));
  if (ms) *ms = tm.ms();
  if (phase_timing_on()) {
    for (size_t k = 0; k < b->stage_name.size(); ++k) {
      float t = 0.f;
      ATC_CK(cudaEventElapsedTime(&t, b->stage_ev[k], b->stage_ev[k + 1]));
      phase_add(b->stage_name[k], t);
    }
  }
  return ATC_OK;
}

}  // namespace
}  // namespace atc

extern "C" atc_status atc_batch_run(atc_batch* b, const atc_tuning* t, uint64_t* counts, atc_stats* stats,
                                    atc_stream st) try {
  ATC_CHECK_ARG(b != nullptr, "NULL batch");
  const int ng = (int)(b->vbase.size() - 1);
  ATC_CHECK_ARG(counts != nullptr || ng == 0, "counts is NULL");
  if (ng == 0 || b->m == 0) {
    for (int i = 0; i < ng; ++i) counts[i] = 0;
    if (stats) memset(stats, 0, sizeof(*stats));
    return ATC_OK;
  }
  atc::ItemShape sh = atc::shape_from(t, b->shape);
  float ms = 0;
  atc::Phase ph("batch", as_stream(st));
  ATC_TRY(atc::run_once(b, sh, counts, &ms, as_stream(st)));
  if (stats) {
    memset(stats, 0, sizeof(*stats));
    stats->kernel_ms = ms;
    stats->total_ms = ms;
    stats->kernel_used = sh.by_source ? ATC_KERNEL_HU : ATC_KERNEL_BISSON;
    stats->launches = b->launches;
  }
  return ATC_OK;
} ATC_CATCH

extern "C" atc_status atc_batch_tune(atc_batch* b, const atc_tuning* cands, int32_t ncand, int32_t* best, float* ms,
                                     atc_stream st) try {
  ATC_CHECK_ARG(b != nullptr && cands != nullptr && ncand > 0 && best != nullptr, "bad argument");
  cudaStream_t s = as_stream(st);
  const int ng = (int)(b->vbase.size() - 1);
  if (ng == 0 || b->m == 0) {
    *best = 0;
    return ATC_OK;
  }
  std::vector<uint64_t> scratch(ng);
  float best_ms = 0;
  *best = 0;
  for (int i = 0; i < ncand; ++i) {
    atc::ItemShape sh = atc::shape_from(&cands[i], atc::default_shape(32));
    float t0 = 0, t1 = 0;
    ATC_TRY(atc::run_once(b, sh, scratch.data(), &t0, s));  // builds and warms
    ATC_TRY(atc::run_once(b, sh, scratch.data(), &t0, s));
    ATC_TRY(atc::run_once(b, sh, scratch.data(), &t1, s));
    float avg = 0.5f * (t0 + t1);
    if (ms) ms[i] = avg;
    if (i == 0 || avg < best_ms) {
      best_ms = avg;
      *best = i;
    }
  }
  b->shape = atc::shape_from(&cands[*best], atc::default_shape(32));
  return ATC_OK;
} ATC_CATCH
