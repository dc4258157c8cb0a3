// Declarations shared between libatc translation units (not part of the ABI).
#pragma once

#include <functional>
#include <optional>

#include "common.cuh"

namespace atc {

// ---- device primitives (prims.cu; CUB radix sort / scan / select) ----------------
// Sorts n keys on bits [begin_bit, end_bit).  `keys` and `alt` are two buffers of n
// elements; on return `keys` points at the sorted data (the two may be swapped).
atc_status sort_keys_u64(uint64_t*& keys, uint64_t*& alt, size_t n, int begin_bit, int end_bit, cudaStream_t s);
// Stable sort of n (key, value) pairs on key bits [begin_bit, end_bit); on return `keys` /
// `vals` point at the sorted data (each may be swapped with its alternate buffer).
atc_status sort_pairs_u64_i32(uint64_t*& keys, uint64_t*& kalt, int32_t*& vals, int32_t*& valt, size_t n, int begin_bit,
                             int end_bit, cudaStream_t s);
// Unique over sorted keys; *n_out (host) receives the count.
atc_status unique_u64(const uint64_t* in, uint64_t* out, size_t n, size_t* n_out, cudaStream_t s);
// out[i] = sum_{j<i} in[j], for n elements.
atc_status exclusive_scan_i64(const int64_t* in, int64_t* out, size_t n, cudaStream_t s);
atc_status exclusive_scan_i32_to_i64(const int32_t* in, int64_t* out, size_t n, cudaStream_t s);
atc_status exclusive_scan_i32_to_i64_tmp(void* tmp, size_t* bytes, const int32_t* in, int64_t* out, size_t n,
                                         cudaStream_t s);

// Bits needed to hold ids in [0, n): at least 1.
inline int id_bits(int64_t n) {
  int b = 1;
  while (b < 62 && (int64_t(1) << b) < n) ++b;
  return b;
}

// Canonical simple edge list on the device: keys (a << B) | b with a < b, sorted,
// duplicate-free, self-loops removed.
struct SimpleEdges {
  DevBuf<uint64_t> keys;   // m
  int64_t m = 0;
  int64_t n_in = 0;        // max input id + 1
  int bits = 1;            // B
};

// Validates ids (>= 0), finds n_in and builds the canonical simple edge list.
atc_status build_simple_edges(const int2* pairs, uint64_t np, SimpleEdges* out, cudaStream_t s);
// Simple degree of every vertex (n_in ints) from canonical keys.
atc_status simple_degrees(const SimpleEdges& e, int32_t* deg, cudaStream_t s);

// A-direction peel priorities (edge_directing/A-direction-seri.cpp:35-153) of the simple
// graph given by canonical keys: prio (n_in ints, device).  stats: number of waves.
atc_status peel_priorities(const SimpleEdges& e, const int32_t* deg, int32_t* prio, int* waves_out,
                           cudaStream_t s);

// Bisson's A-direction relabelling (Bisson/A-direction.cpp:43-163,283-292) of the simple
// graph given by canonical keys: lookup (n_in ints, device) = the new id of every vertex.
// ATC_ERR_UNSUPPORTED where the serial program would not terminate.
atc_status bisson_adirection_lookup(const SimpleEdges& e, const int32_t* deg, int32_t* lookup, cudaStream_t s);

// Core numbers (n_in ints, device) of the simple graph given by canonical keys.
atc_status core_numbers(const SimpleEdges& e, const int32_t* deg, int32_t* core, cudaStream_t s);

// Approximate parallel A-direction peel (edge_directing/A-direction-parallel/peel.cu:130-262)
// of the simple graph: flags (major priority, 0xFFFFFFFF = never peeled) and minor
// priority (n_in each, device).  iters_out: the reference's itera_times at exit.
atc_status approx_peel(const SimpleEdges& e, const int32_t* deg, uint32_t* flags, uint32_t* minor, int* iters_out,
                       cudaStream_t s);

// A-order lookup (vertex_ordering/A-order/A-order.cpp:62-210) of an edge list with
// repeats counted.  Edges come either as int2 pairs or as canonical keys (exactly one
// non-null).  n_v = max id + 1 over the edges.  lookup: n_v ints (device).  If
// oriented != nullptr (pairs input only) it receives the degree-oriented pairs (the
// "normal" file).  Returns ATC_ERR_UNSUPPORTED where the reference reads outside its
// arrays.  deg (nullable, device): the degrees of the edges when the caller has them.
// overlap (nullable): device work that does not depend on the lookup, run on the calling
// thread while the host part of A-order runs on another.
atc_status aorder_lookup(const int2* pairs, const uint64_t* keys, int bits, uint64_t ne, int64_t n_v,
                         int32_t* lookup, int2* oriented, cudaStream_t s, const int32_t* deg = nullptr,
                         const std::function<atc_status()>* overlap = nullptr);

// Rank relabellings (vertex_ordering/A-order/A-order-v2.cpp, relabel-naive.cpp,
// relabel4lpOut.cpp) of an edge list with repeats counted: lookup (n_v ints, device);
// oriented (nullable) = the degree-oriented pairs (or the input, for OUTDEG_DESC).
atc_status relabel_lookup(const int2* pairs, const uint64_t* keys, int bits, uint64_t ne, int64_t n_v, int kind,
                          int32_t* lookup, int2* oriented, cudaStream_t s);

// The C library's rand() stream in its seed-1 state and std::random_shuffle over it
// (csrc/shuffle.cu).  rand_stream: out[k] = the value of call k, k < count (device).
// shuffle_blocks: random_shuffle of each block [b*width, (b+1)*width) of a, b < nblocks, in
// block order, one stream (width <= kMaxShuffleWidth).  shuffle_ids: out[p] = the id at
// position p after random_shuffle of the ids 0..n-1.
constexpr int kMaxShuffleWidth = 64;
atc_status rand_stream(uint32_t* out, int64_t count, cudaStream_t s);
atc_status shuffle_blocks(int32_t* a, int64_t nblocks, int width, cudaStream_t s);
atc_status shuffle_ids(int32_t* out, int64_t n, cudaStream_t s);

// Edge range [range[0], range[1]) of part `part` of `nparts` contiguous ranges of equal work
// (sum over the edges of min(outdeg u, outdeg v) + 1) of a CSR built by the library.
atc_status part_edge_range(const atc_csr* csr, uint32_t part, uint32_t nparts, int64_t* range, cudaStream_t s);

// GRO order (vertex_ordering/other_order/porder.cpp:141-226) of the directed pairs (device):
// lookup (n_v ints, device) = new id of every id in [0, n_v).
atc_status gro_lookup(const int2* pairs, uint64_t ne, int64_t n_v, int32_t* lookup, cudaStream_t s);

// Private part of an atc_csr.
struct CsrPriv {
  int32_t* esrc = nullptr;       // m: source vertex of every edge, in edge order
  unsigned long long* counter = nullptr;  // 2 x u64 scratch for counting kernels
  int bits = 1;
  // cols and esrc live in pinned host memory mapped into the device's address space
  // (atc_csr_host_resident / atc_csr_load_host); these are the host allocations
  int32_t* host_cols = nullptr;
  int32_t* host_esrc = nullptr;
};

}  // namespace atc
