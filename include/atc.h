/*
 * atc.h — C ABI of libatc, the GB300 (sm_103a) triangle-counting library.
 *
 * The reference (pkumod/accelerating-TC) ships stand-alone programs whose in-process
 * interfaces are process globals filled by `preProcess` and `__constant__` pointer
 * symbols read by the kernels.  This header replaces them with reentrant calls on
 * plain pointers and sizes; each declaration names the reference interface it stands
 * for.  All entry points return an atc_status and never abort the process.
 *
 * Ownership: the library owns every device buffer reachable from an atc_csr and frees
 * it in atc_csr_free.  Callers own their input arrays.  Host pointers are plain
 * pageable or pinned memory; "_device" variants take device pointers.  Streams are
 * cudaStream_t values passed as void* (NULL = the legacy default stream); every call
 * that returns a host result synchronises its stream before returning.
 *
 * Vertex ids are int32 >= 0; an input pair is two consecutive int32 {src, dst}, the
 * little-endian layout of the reference's binary edge files (Hu/preTC.cu:29-32,84).
 */
#ifndef ATC_H_
#define ATC_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef void* atc_stream; /* a cudaStream_t */

typedef enum atc_status {
  ATC_OK = 0,
  ATC_ERR_INVALID = 1,     /* bad argument: negative id, NULL pointer, bad enum, ... */
  ATC_ERR_OOM = 2,         /* device or host allocation failed */
  ATC_ERR_CUDA = 3,        /* a CUDA runtime call failed (message: atc_last_error) */
  ATC_ERR_TIMEOUT = 4,     /* a bounded device wait ran out */
  ATC_ERR_UNSUPPORTED = 5  /* input outside what the algorithm defines (see the call) */
} atc_status;

/* Edge orientation.  Every rule is acyclic, so the count is the same for all. */
typedef enum atc_dir {
  /* u -> v iff u > v: N+(u) holds the smaller ids (Bisson/preTC.cu:135-144, chooseIndex 0;
     Fox/preTC.cu:92-101). */
  ATC_DIR_ID = 0,
  /* lower degree -> higher degree; equal degrees: the larger id is the source
     (Hu/preTC.cu:125-133; A-order.cpp:88-99). */
  ATC_DIR_DEGREE = 1,
  /* lower degree -> higher degree; equal degrees: the smaller id is the source
     (tricore/src/tricount_gpu.cu:69-80). */
  ATC_DIR_DEGREE_LOWID = 2,
  /* A-direction: peel priorities, u -> v iff prio[v] > prio[u] or (equal and u < v)
     (edge_directing/A-direction-seri.cpp:35-153, 254-273). */
  ATC_DIR_ADIRECTION = 3,
  /* k-core: lower core number first; equal cores: the smaller id is the source
     (edge_directing/kcore_direction.cpp:91-146, with true degrees; see atc_pretc). */
  ATC_DIR_KCORE = 4,
  /* approximate parallel A-direction: per vertex a peel iteration `flag` (0xFFFFFFFF for
     vertices never peeled, which compare as -1, i.e. first) and a minor priority; the
     source is the endpoint with the smaller (flag, minor, id)
     (edge_directing/A-direction-parallel/peel.cu:44-59, 130-262; see atc_adirection_par). */
  ATC_DIR_ADIRECTION_PAR = 5
} atc_dir;

typedef enum atc_order {
  ATC_ORDER_NONE = 0,
  /* A-order relabelling (vertex_ordering/A-order/A-order.cpp:62-247). */
  ATC_ORDER_AORDER = 1,
  /* descending degree-orientation out-degree, larger id first on a tie: the "good"
     relabelling of vertex_ordering/A-order/relabel-naive.cpp:67-74 (ATC_RELABEL_DEGREE_DESC) */
  ATC_ORDER_DEGREE_DESC = 2,
  /* A-order-v2's 40-column mix of that list (A-order-v2.cpp:102-146, ATC_RELABEL_AORDER_V2) */
  ATC_ORDER_AORDER_V2 = 3,
  /* other_order's GRO order of the simple graph, both directions of every edge
     (vertex_ordering/other_order/porder.cpp:141-226, ATC_RELABEL_GRO) */
  ATC_ORDER_GRO = 4,
  /* Bisson's A-direction relabelling of the simple graph (Bisson/A-direction.cpp,
     ATC_RELABEL_ADIRECTION_BISSON); with ATC_DIR_ID it is the program's A-direction
     pipeline for Bisson and Fox */
  ATC_ORDER_ADIRECTION_BISSON = 5,
  /* relabel-naive's shuffled 64-column mix of the DEGREE_DESC list (ATC_RELABEL_NAIVE_SHUFFLED) */
  ATC_ORDER_NAIVE_SHUFFLED = 6,
  /* relabel-random's random relabelling (ATC_RELABEL_RANDOM) */
  ATC_ORDER_RANDOM = 7
} atc_order;

/* Rank relabellings of vertex_ordering/A-order (atc_relabel). */
typedef enum atc_relabel_kind {
  /* rt = out-degree after the degree orientation (src = lower degree, larger id on a
     tie; A-order-v2.cpp:38-50); new id = position in the (rt, id)-descending list of all
     ids 0..max (relabel-naive.cpp:67-74,165-172 writes it as "degreeOrder";
     relabel-random.cpp:67-74 as "good"). */
  ATC_RELABEL_DEGREE_DESC = 0,
  /* the same list dealt into 40 columns (A-order-v2.cpp:102-146, output file "naive") */
  ATC_RELABEL_AORDER_V2 = 1,
  /* rt = out-degree of the pairs as given ("good" of relabel4lpOut.cpp:27-54, whose
     input is already oriented) */
  ATC_RELABEL_OUTDEG_DESC = 2,
  /* GRO order of the other_order library on the pairs as directed edges, repeats kept
     (vertex_ordering/other_order/porder.cpp:141-226 with linkedlist_heap.cpp, the
     _GRO_newID.txt of its reorder program); `normal` = the pairs as given.  The program
     reads uninitialised memory once a vertex's gain reaches the vertex count; this
     build reads those gains as unset. */
  ATC_RELABEL_GRO = 3,
  /* Bisson's A-direction relabelling (Bisson/A-direction.cpp:43-163,283-304): the serial
     peel's priorities, then new id = n-1 - rank of (priority, degreeRecord, id), with the
     program's position-indexed degreeRecord (:118) reproduced.  Counting the relabelled
     graph with ATC_DIR_ID realises the A-direction orientation as an id order, which is
     how the program feeds Bisson's kernel.  `normal` = the pairs as given. */
  ATC_RELABEL_ADIRECTION_BISSON = 4,
  /* relabel-naive's "naive" (vertex_ordering/A-order/relabel-naive.cpp:77-177): the
     DEGREE_DESC list dealt into 64 columns of chunk = n/64 positions (position i + 64 j of
     column i takes entry i*chunk + j; odd columns are read backwards), then every block of
     64 positions shuffled by std::random_shuffle with the C library's rand() in its seed-1
     state (the program never seeds it); the last n % 64 positions keep the list's order. */
  ATC_RELABEL_NAIVE_SHUFFLED = 5,
  /* relabel4lpOut's "bad" (relabel4lpOut.cpp:57-136): the OUTDEG_DESC list dealt into 40
     columns the same way and its blocks of 40 shuffled; `normal` = the pairs as given. */
  ATC_RELABEL_OUTDEG_SHUFFLED = 6,
  /* relabel-random's "bad" (relabel-random.cpp:76-108): std::random_shuffle of the ids
     0..max with the C library's rand() in its seed-1 state; `normal` = the degree-oriented
     pairs, as for DEGREE_DESC. */
  ATC_RELABEL_RANDOM = 7
} atc_relabel_kind;

typedef enum atc_kernel {
  ATC_KERNEL_AUTO = 0,    /* Bisson- or Hu-style, whichever a cost model of their GB300 times
                             (W, W_min and m of the CSR) predicts is faster */
  ATC_KERNEL_HU = 1,      /* wedge walk, N+(u) staged in shared memory (Hu/tc.cu:69-201) */
  ATC_KERNEL_BISSON = 2,  /* bitmap for large N+(u), search otherwise (Bisson/tc.cu:18-104) */
  ATC_KERNEL_FOX = 3,     /* edge bins with 1..32 threads per edge (Fox/tc.cu:64-125,316-384) */
  ATC_KERNEL_TRICORE = 4  /* warp per edge, 32 pivots + binary search (tricount_gpu.cu:215-290) */
} atc_kernel;

/* Tuning knobs; zero means "library default".  The reference hard-codes these as
   #defines (Hu/tc.cu:6-8, Bisson/tc.cu:5-6, Fox/tc.cu:318-319, tricount_gpu.cu:24-25). */
typedef struct atc_tuning {
  int32_t prune_deg1;        /* drop degree<=1 vertices, compact ids (Hu/preTC.cu:135-169) */
  int32_t hu_blocks;         /* unused: the Hu-style kernel drains a work queue (layout kept) */
  int32_t hu_stage_ints;     /* unused: N+(u) is staged per work item (layout kept) */
  int32_t bisson_cutover;    /* warp items: sorted copy up to this out-degree, hash above (32) */
  int32_t fox_rearrange;     /* interleave each bin's edges (Fox/tc.cu:127-183) */
  int32_t fox_work_per_thread; /* bin base of the threads-per-edge bins (8) */
  int32_t tricore_blocks;    /* CTAs of the TriCore-style kernel (0: auto) */
  int32_t bisson_warp_max;   /* longest list a warp item handles, <= 512 (256) */
  int32_t bisson_warp_chunk; /* partners per warp item (512) */
  int32_t bisson_block_chunk; /* partners per block item (2048) */
  int32_t bisson_slots;      /* hash slots per bucket of the tables: 1, 2 or 4 (0: default) */
  /* the bisson_* item shape applies to the Hu-style kernel too */
  int32_t group_by_source;   /* batches: 1 = every edge at its source, the items index the
                                CSR rows (Hu-style wedge tests, no grouping passes); 0 = at
                                the endpoint with the longer list (Bisson-style); 2 = each
                                graph the way the Hu/Bisson cost model predicts faster */
  int32_t kcl_dense;         /* k-cliques (atc_kcl_part_tuned): 0 = candidate sets of 65..1024
                                members on the dense kernel from k = 5 on; -1 = every edge on
                                the warp search */
  int32_t edge_kernels;      /* TriCore- and Fox-style: 1 = per-edge kernels searching the longer
                                list in global memory, as the reference kernels do (a warp per
                                edge with 32 pivots; 1..32 threads per edge in work bins);
                                0 = the longer lists staged in shared memory per group item */
  int32_t reserved[2];
} atc_tuning;

/* Oriented CSR on the device (the reference's edgeOffset/edgeRow/adjLength globals,
   Hu/preTC.cu:59-62).  Lists are sorted ascending and duplicate-free. */
typedef struct atc_csr {
  int64_t n;            /* vertices of the counted graph */
  int64_t m;            /* oriented edges */
  int64_t* offsets;     /* device, n+1 */
  int32_t* cols;        /* device, m */
  int64_t n_input;      /* max input id + 1 */
  int64_t wedges;       /* W = sum_v indeg(v) * outdeg(v) */
  int32_t dir;          /* atc_dir used */
  int32_t order;        /* atc_order used */
  int32_t pruned;       /* 1 when degree<=1 vertices were removed */
  int32_t max_outdeg;
  int64_t wedges_min;   /* sum over edges (u,v) of min(outdeg(u), outdeg(v)) */
  void* priv;           /* library-internal */
} atc_csr;

typedef struct atc_stats {
  float kernel_ms;       /* device time of the counting kernels (events on the stream) */
  float total_ms;        /* device time of the whole call */
  uint64_t alg_bytes;    /* 4(n+1) + 4m + 4W + 8: every candidate N+(v), v in N+(u), read once */
  uint64_t wedges;       /* W of the counted CSR */
  uint64_t alg_bytes_min; /* 4(n+1) + 4m + 4*wedges_min + 8: only the shorter list of each edge read */
  int32_t kernel_used;   /* atc_kernel actually run */
  int32_t launches;      /* kernel launches made by the call */
} atc_stats;

/* ---- library ---------------------------------------------------------------- */
const char* atc_version(void);
const char* atc_status_string(atc_status s);
/* Text of the last error on the calling thread (CUDA message or argument check). */
const char* atc_last_error(void);
/* Device allocation budget, for capacity tests and memory-capped hosts: after
   atc_set_alloc_budget(b) with b >= 0, the library's stream-ordered device allocations take
   their size from a budget of b bytes (never returned), and an allocation that the budget
   cannot cover fails with ATC_ERR_OOM before any device call.  b < 0 removes the budget
   (the default).  No counterpart in the reference, which aborts on a failed cudaMalloc. */
atc_status atc_set_alloc_budget(int64_t bytes);
/* Phase timing, for profiling: with atc_phase_timing(1) the library records its named phases
   (preTC stages, counting passes) on the calling thread as CUDA events on each call's
   stream; atc_phase_times copies up to `cap` recorded phases, in the order they began, sets
   *n to the number recorded, waits for their end events, and clears the record.
   atc_phase_timing(0) stops recording.  Every phase is also an NVTX range. */
typedef struct atc_phase_time {
  char name[40];
  int32_t depth; /* nesting depth: 0 = a phase of its own, 1 = inside a depth-0 phase, ... */
  float ms;      /* device time between the phase's start and end events */
} atc_phase_time;
atc_status atc_phase_timing(int32_t enable);
atc_status atc_phase_times(atc_phase_time* out, int32_t cap, int32_t* n);
/* The bounded-wait failure path, for tests: the counting kernels that stage lists with bulk
   copies wait on an mbarrier for at most one second, then stop and report ATC_ERR_TIMEOUT.
   This runs a one-CTA kernel whose barrier can never complete (bytes announced, no copy
   issued) with a 1 ms limit: it returns ATC_ERR_TIMEOUT when the wait gave up, as it must,
   ATC_OK if it did not, and leaves the device usable.  No counterpart in the reference. */
atc_status atc_check_wait_timeout(atc_stream s);
/* Makes `device` current on the calling thread and initialises its context.  device = -1
   initialises the calling thread's current device and leaves the current device as it is. */
atc_status atc_init(int device);

/* ---- synthetic inputs (deterministic, integer-only; no GPU needed for _host) --- */
/* R-MAT, 2^scale vertices, edge_factor*2^scale samples, quadrant probabilities in
   parts per million (Graph500: 570000, 190000, 190000).  Writes the raw samples. */
atc_status atc_gen_rmat_host(uint32_t scale, uint32_t edge_factor, uint32_t a_ppm, uint32_t b_ppm,
                             uint32_t c_ppm, uint64_t seed, int32_t* out_pairs, int nthreads);
atc_status atc_gen_rmat_device(uint32_t scale, uint32_t edge_factor, uint32_t a_ppm, uint32_t b_ppm,
                               uint32_t c_ppm, uint64_t seed, int32_t* out_pairs_dev, atc_stream s);
/* 2-D random geometric graph: n points with 31-bit fixed-point coordinates in the unit
   square, i and j adjacent iff their distance is <= sqrt(mean_degree / (pi n)) (integer
   test).  Writes each edge once as (i, j), i < j: sorted on the host; in no particular
   order on the device.  *n_out = the number of edges; with out == NULL only counts.
   ATC_ERR_INVALID if it exceeds `capacity` (pairs). */
atc_status atc_gen_rgg_host(uint32_t n, double mean_degree, uint64_t seed, int32_t* out_pairs, uint64_t capacity,
                            uint64_t* n_out, int nthreads);
atc_status atc_gen_rgg_device(uint32_t n, double mean_degree, uint64_t seed, int32_t* out_pairs_dev,
                              uint64_t capacity, uint64_t* n_out, atc_stream s);
/* Chung-Lu (expected-degree) graph on the device: n vertices, power-law weights with
   exponent gamma (> 1.05) and mean degree mean_degree, each edge once as (u, v), u < v,
   in row order.  *n_out = edges; with out == NULL only counts.  ATC_ERR_INVALID above
   `capacity` pairs.  Deterministic for one device type (floating-point weights). */
atc_status atc_gen_chunglu_device(uint32_t n, double gamma, double mean_degree, uint64_t seed, int32_t* out_pairs_dev,
                                  uint64_t capacity, uint64_t* n_out, atc_stream s);
/* Drops self-loops and repeats; writes each undirected edge once as (min,max) sorted,
   or, with symmetric != 0, both directions sorted by (src,dst).  Capacity of `out`:
   2*n_pairs pairs when symmetric, else n_pairs. */
atc_status atc_simplify_host(const int32_t* pairs, uint64_t n_pairs, int symmetric,
                             int32_t* out, uint64_t* n_out);

/* ---- preTC: edge list -> oriented CSR on the device -----------------------------
   Replaces bool preProcess(const char*, unsigned& edgeNum, unsigned& nodeNum[, ...])
   (Hu/preTC.cu:64, Bisson/preTC.cu:77, Fox/preTC.cu:64) and TriCore's cal_degree /
   redirect_edges / split (tricore/include/tricount.h:9-15).  Self-loops and repeated
   pairs are dropped; degrees are those of the resulting simple graph.  With
   ATC_ORDER_AORDER the vertices are relabelled by A-order computed on the simple
   graph; the counting programs' rules (ATC_DIR_ID, DEGREE, DEGREE_LOWID) then orient on
   the new ids, while the direction programs' orientations (ADIRECTION, KCORE,
   ADIRECTION_PAR) are decided on the input ids and relabelled, as when A-order reads
   their output file; `perm_out` (nullable, n_input
   ints) receives the new id of every input id.  Returns ATC_ERR_UNSUPPORTED when
   A-order is asked for on a graph where the reference A-order indexes outside its
   arrays (see atc_aorder). */
atc_status atc_pretc(const int32_t* pairs, uint64_t n_pairs, atc_dir dir, atc_order order,
                     const atc_tuning* tuning, atc_csr* out, int32_t* perm_out, atc_stream s);
atc_status atc_pretc_device(const int32_t* pairs_dev, uint64_t n_pairs, atc_dir dir, atc_order order,
                            const atc_tuning* tuning, atc_csr* out, int32_t* perm_out, atc_stream s);
/* Copies the CSR to host arrays (n+1 int64, m int32). */
atc_status atc_csr_to_host(const atc_csr* csr, int64_t* offsets, int32_t* cols, atc_stream s);
atc_status atc_csr_free(atc_csr* csr);
/* Edge-file reader (host only, no GPU): "*.gr" is read as a Galois binary graph
   (versions 1 and 2; the k-clique program's input, k-clique/README.md:12-15), any
   other name as {int32 src, int32 dst} pairs (Hu/preTC.cu:29-32,84).  Two-call
   pattern: with pairs == NULL only *n_out (edge count) is written; then pass a
   buffer of cap >= *n_out pairs.  ATC_ERR_INVALID for an unreadable or malformed file. */
atc_status atc_read_edges(const char* path, int32_t* pairs, uint64_t cap, uint64_t* n_out);

/* Binary CSR cache (no counterpart in the reference, whose programs hand over
   intermediate edge files): writes / reads the oriented CSR with its statistics
   ("ATCCSR01", little-endian), so a graph's preTC can be done once and reloaded.
   atc_csr_load validates the arrays (ATC_ERR_INVALID for a file that is not a CSR). */
atc_status atc_csr_save(const atc_csr* csr, const char* path, atc_stream s);
atc_status atc_csr_load(const char* path, atc_csr* out, atc_stream s);
/* Graphs larger than device memory (TriCore's out-of-core parts,
   tricore/src/tricount_gpu.cu:337-408, copy vertex-range parts of the CSR to the device
   pair by pair).  Here the CSR's edge arrays (cols and the per-edge source array, 8 bytes
   per edge) move into pinned host memory mapped into the device's address space, only the
   offsets stay on the device, and every kernel reads the lists over the CPU-GPU link
   (NVLink-C2C on Grace-Blackwell) in place; atc_tc_part bounds the counting scratch.
   atc_csr_host_resident moves a CSR built on the device; atc_csr_load_host loads a cache
   file straight into host memory.  atc_csr_free releases either kind. */
atc_status atc_csr_host_resident(atc_csr* csr, atc_stream s);
atc_status atc_csr_load_host(const char* path, atc_csr* out, atc_stream s);

/* ---- orientation and ordering as drop-ins for the reference programs ------------ */
/* A-direction-seri <file> (edge_directing/A-direction-seri.cpp:170-288): writes the
   oriented edge list (the bytes of lpBasedGraph.bin; capacity 2*n_pairs pairs) and,
   if non-NULL, the peel priorities (max id + 1 ints). */
atc_status atc_adirection(const int32_t* pairs, uint64_t n_pairs, int32_t* oriented_out,
                          uint64_t* n_out, int32_t* prio_out, atc_stream s);
/* kcore_direction <in> <out> (edge_directing/kcore_direction.cpp:12-146): edges packed
   as uint64 (src = x >> 32, dst = low 32 bits, the program's byte order); writes one
   packed edge per input edge, in input order, directed from the smaller core number to
   the larger, the smaller id first on a tie.  Core numbers are those of the simple graph
   (repeats and loops dropped); `core_out` (nullable) receives them, *n_vertices (nullable)
   = max id + 1.  Ids must be < 2^31 (ATC_ERR_INVALID otherwise).  The reference counts
   degrees over the first node_num edges (:35-38) instead of all edges; this function
   counts all of them. */
atc_status atc_kcore_direction(const uint64_t* edges, uint64_t n_edges, uint64_t* oriented_out,
                               int32_t* core_out, uint64_t* n_vertices, atc_stream s);
/* Peel <in> <out> (edge_directing/A-direction-parallel/peel.cu:130-317): edges packed as
   uint64 (src = x >> 32); writes one packed edge per input edge, in input order, directed
   by the approximate parallel peel's (flag, minor, id) ranking.  compat != 0 reproduces
   the program's comparison exactly, including its minor term minor[src] - flag[dst]
   (peel.cu:49, where minor[dst] is meant); compat == 0 compares minor[src] - minor[dst].
   flags_out / minor_out (nullable, max id + 1 entries each) receive the two priorities,
   *n_vertices (nullable) = max id + 1, *iterations (nullable) the program's final
   itera_times.  Ids must be < 2^31. */
atc_status atc_adirection_par(const uint64_t* edges, uint64_t n_edges, int compat, uint64_t* oriented_out,
                              uint32_t* flags_out, uint32_t* minor_out, uint64_t* n_vertices, int32_t* iterations,
                              atc_stream s);
/* A-order-v2 / relabel-naive / relabel4lpOut on raw pairs, repeats included: `lookup`
   (max id + 1 ints, at least 1) = new id of every id; `normal` (n_pairs pairs, nullable)
   = the degree-oriented pairs (the input as given for OUTDEG_DESC); `relabeled`
   (nullable) = lookup applied to `normal` (the "naive" / "good" output file).  The
   programs' shuffled "bad" outputs depend on the C library's rand() and are not built. */
atc_status atc_relabel(const int32_t* pairs, uint64_t n_pairs, atc_relabel_kind kind, int32_t* lookup,
                       int32_t* normal, int32_t* relabeled, atc_stream s);
/* A-order <file> (vertex_ordering/A-order/A-order.cpp:62-247) on the raw pairs,
   repeats included: `lookup` (max id + 1 ints) = new id of every id (badLookUpTable);
   `normal` / `reordered` (n_pairs pairs each, nullable) = the two output files.
   ATC_ERR_UNSUPPORTED where the reference reads outside its arrays: no vertex of
   runtime degree 2..4 or none of 5 or more (memoryDominatePos == 0, :111-119,144), or
   more degree-2..4 vertices than the whole 40-vertex buckets hold (:165-177). */
atc_status atc_aorder(const int32_t* pairs, uint64_t n_pairs, int32_t* lookup, int32_t* normal,
                      int32_t* reordered, atc_stream s);

/* ---- counting --------------------------------------------------------------------
   Triangle count of the oriented CSR: sum_u sum_{v in N+(u)} |N+(u) ∩ N+(v)|, exact in
   uint64.  Replaces the kernels' launch + host reduction in Hu/tc.cu:317-323,
   Bisson/tc.cu:198-204, Fox/tc.cu:334-384, tricount_gpu.cu:337-408. */
atc_status atc_tc(const atc_csr* csr, atc_kernel kernel, const atc_tuning* tuning,
                  uint64_t* count, atc_stats* stats, atc_stream s);
/* One part of the triangle count: the edges of the CSR are cut into `nparts` contiguous
   ranges of equal work (sum over the edges of min(outdeg u, outdeg v) + 1) and this call
   counts the triangles sum_{(u,v) in part} |N+(u) ∩ N+(v)| of range `part`, so the counts
   of parts 0..nparts-1 add up to atc_tc's.  It is the sharding unit of a count spread over
   several GPUs (each holding the CSR, one uint64 sum at the end), the partitioned
   counting the reference leaves to TriCore's vertex-range parts
   (tricore/src/tricount_gpu.cu:347-406).  edge_range (nullable, 2 entries) receives
   [first, last) edge of the part.  stats describe the whole CSR except kernel_ms. */
atc_status atc_tc_part(const atc_csr* csr, atc_kernel kernel, const atc_tuning* tuning, uint32_t part,
                       uint32_t nparts, uint64_t* count, int64_t* edge_range, atc_stats* stats, atc_stream s);
/* Triangle count of an oriented CSR given as plain device arrays, computed without
   allocating any device memory.  No counterpart in the reference: it is for callers
   that cannot call cudaMalloc, such as a host whose device memory is all owned by
   another allocator or runtime, or a real-time loop that must not block in the
   driver's allocator.  Runs the ATC_KERNEL_BISSON count with all scratch in one fixed
   device array of the library (about 17 MiB, held by every device that loads the
   library until exit).  Limits: n <= 131072 vertices and m <= 1048576 edges, else
   ATC_ERR_INVALID; offsets (n+1, int64) and cols (m) must form a CSR whose rows are
   strictly increasing ids in [0, n) (checked on the device first; ATC_ERR_INVALID
   otherwise).  The call synchronises `s` (it reads results back to the host).  The
   first call on a device looks up the array's device address, so make it before any
   stream capture; after cudaDeviceReset of a device, do not call it on that device
   again in the same process.  All calls share the array: calls that overlap on the
   GPU race. */
atc_status atc_tc_noalloc(const int64_t* offsets_dev, const int32_t* cols_dev, int64_t n, int64_t m,
                          uint64_t* count, atc_stream s);
/* atc_kcl_part with tuning (nullable; tuning->kcl_dense selects the kernels). */
atc_status atc_kcl_part_tuned(const atc_csr* csr, uint32_t k, const atc_tuning* tuning, uint32_t part,
                              uint32_t nparts, uint64_t* count, int64_t* edge_range, atc_stats* stats,
                              atc_stream s);
/* k-clique count (k >= 3) of the oriented CSR, exact in uint64.  Replaces
   kcl_gpu_solver(std::string, unsigned k, AccType& total, size_t) (k-clique/kcl.h:6-7). */
atc_status atc_kcl(const atc_csr* csr, uint32_t k, uint64_t* count, atc_stats* stats, atc_stream s);
/* One part of the k-clique count: the cliques whose first two vertices (in orientation order)
   form an edge of part `part` of the work-balanced edge ranges of atc_tc_part; the counts of
   parts 0..nparts-1 add up to atc_kcl's (sharding by the clique's first edge). */
atc_status atc_kcl_part(const atc_csr* csr, uint32_t k, uint32_t part, uint32_t nparts, uint64_t* count,
                        int64_t* edge_range, atc_stats* stats, atc_stream s);

/* ---- batched counting --------------------------------------------------------------
   Many graphs of uneven sizes counted together.  No counterpart in the reference, which
   runs one program per graph.  The batch keeps the graphs as one disjoint union on the
   device (vertex and edge ranges per graph); atc_batch_run counts every graph in one
   replay of a CUDA graph that holds the whole Bisson-style pipeline (grouping passes and
   the persistent, work-queue-driven counting kernels), with per-graph counters.  The
   captured graph is rebuilt when the batch or the item shape changes. */
typedef struct atc_batch atc_batch;
atc_status atc_batch_create(atc_batch** out);
/* Optional: preallocates room for `n` vertices and `m` edges in total, so that adding
   graphs never regrows the union (regrowth briefly needs the old and the new arrays). */
atc_status atc_batch_reserve(atc_batch* b, int64_t n, int64_t m, atc_stream s);
/* Appends a copy of `csr` (device to device; the caller keeps and frees its csr).
   *index (nullable) receives the graph's position in the batch. */
atc_status atc_batch_add(atc_batch* b, const atc_csr* csr, int32_t* index, atc_stream s);
/* Counts every graph; counts (host, one per graph).  `tuning` (nullable) sets the item
   shape (bisson_cutover, bisson_warp_max, bisson_warp_chunk, bisson_block_chunk). */
atc_status atc_batch_run(atc_batch* b, const atc_tuning* tuning, uint64_t* counts, atc_stats* stats, atc_stream s);
/* Autotuner: runs each of `n` candidate tunings (two timed replays each), keeps the
   fastest as the batch's shape.  *best = its index; ms (nullable, n floats) = times. */
atc_status atc_batch_tune(atc_batch* b, const atc_tuning* candidates, int32_t n, int32_t* best, float* ms,
                          atc_stream s);
/* Graphs, vertices and edges held. */
atc_status atc_batch_info(const atc_batch* b, int32_t* graphs, int64_t* n, int64_t* m);
atc_status atc_batch_destroy(atc_batch* b);

/* ---- learned (direction, ordering, kernel) selection --------------------------------
   No counterpart in the reference.  A small FP32 MLP (n_in -> hidden ReLU -> hidden ReLU
   -> n_out), trained and evaluated on the GPU by the library's own kernels; the
   selector reads graph statistics and predicts one log-time per candidate triple. */
typedef struct atc_mlp atc_mlp;
/* He-uniform weights from `seed`, zero biases. */
atc_status atc_mlp_create(int32_t n_in, int32_t hidden, int32_t n_out, uint64_t seed, atc_mlp** out);
atc_status atc_mlp_destroy(atc_mlp* net);
/* Parameter vector (layout W1[in][h] b1 W2[h][h] b2 W3[h][out] b3): copied out to `get`
   and / or in from `set` (each nullable); *count = its length. */
atc_status atc_mlp_params(atc_mlp* net, float* get, const float* set, int64_t* count);
/* Input standardisation (mean, std per input): read and / or set (each nullable). */
atc_status atc_mlp_scaling(atc_mlp* net, float* get_mean, float* get_std, const float* set_mean, const float* set_std);
/* y[rows][n_out] = net(x[rows][n_in]) (x raw; standardised inside). */
atc_status atc_mlp_forward(atc_mlp* net, const float* x, int32_t rows, float* y, atc_stream s);
/* Masked MSE loss  sum M (y - t)^2 / (2 sum M)  and its gradient w.r.t. every parameter
   (mask nullable = all ones). */
atc_status atc_mlp_gradients(atc_mlp* net, const float* x, const float* t, const float* mask, int32_t rows,
                             float* grads, float* loss, atc_stream s);
/* Adam training (fits the standardisation to x first); final mini-batch loss out. */
atc_status atc_mlp_train(atc_mlp* net, const float* x, const float* t, const float* mask, int32_t rows, int32_t epochs,
                         int32_t batch, float lr, uint64_t seed, float* final_loss, atc_stream s);
/* Six graph statistics of device pairs, log1p-scaled: vertices, edges, mean, variance
   and maximum degree, and the costFuncCal tail cost (tools/costFuncCal.cpp:66-81) of
   the degree orientation (vertices whose out-degree exceeds twice the mean). */
atc_status atc_graph_features(const int32_t* pairs_dev, uint64_t n_pairs, float* features, atc_stream s);
/* The triple the network predicts fastest: *choice = argmin of its outputs;
   predicted (nullable, n_out floats) = the outputs. */
atc_status atc_select(atc_mlp* net, const float* features, int32_t* choice, float* predicted, atc_stream s);

/* ---- orientation-cost figures ----------------------------------------------------- */
/* costFuncCal <file> <k> (tools/costFuncCal.cpp:15-88): out = {idPartCost,
   degreePartCost, lpPartCost}, float sums in vertex order as the tool prints them. */
atc_status atc_costfunc(const int32_t* pairs, uint64_t n_pairs, int32_t k, float* out, atc_stream s);
/* verification <text file> (tools/verification.cpp:11-61) on already-parsed pairs:
   out = {f_lp, f_degree}. */
atc_status atc_verification(const int32_t* pairs, uint64_t n_pairs, float* out, atc_stream s);

#ifdef __cplusplus
}
#endif
#endif /* ATC_H_ */
