// Drop-in command lines for the reference's orientation / ordering / cost tools:
//
//   a_direction_seri <edges.bin>     edge_directing/A-direction-seri.cpp:170-288
//        writes lpBasedGraph (text "src dst") and lpBasedGraph.bin in the working directory
//   bisson_a_direction <edges.bin>   Bisson/A-direction.cpp:196-336 (READFROMFILE, EDGEBINARY)
//        writes lpBasedGraph.bin (every edge in both directions, relabelled by the peel
//        order) and the empty lpBasedGraph the program also creates
//   a_order <edges.bin>              vertex_ordering/A-order/A-order.cpp:62-247
//        writes normal and reordered in the working directory
//   a_order_v2 <edges.bin>           vertex_ordering/A-order/A-order-v2.cpp:14-193
//        writes naive (and the empty degreeOrder) in the working directory
//   relabel_naive <edges.bin>        vertex_ordering/A-order/relabel-naive.cpp:14-193
//        writes naive (the shuffled 64-column mix) and degreeOrder
//   relabel4lp_out <edges.txt>       vertex_ordering/A-order/relabel4lpOut.cpp:13-151 ("src dst"
//        text lines, e.g. A-direction-seri's lpBasedGraph); writes normal, bad and good
//   relabel_random <edges.bin>       vertex_ordering/A-order/relabel-random.cpp:13-124
//        writes normal, bad (every id shuffled) and good; prints the runtime degree of the
//        vertex at each position of the shuffle but the last
//   cost_func_cal <edges.bin> <k>    tools/costFuncCal.cpp:15-95 (prints the three costs)
//   Peel <in> <out> [--compat]       edge_directing/A-direction-parallel/peel.cu:130-317 (uint64
//        edges, src = x >> 32; --compat keeps the program's minor-priority term, peel.cu:49)
//   kcore_direction <in> <out>       edge_directing/kcore_direction.cpp:12-146 (uint64 edges,
//        src = x >> 32; writes the oriented uint64 edges to <out>)
//   reorder <edges.u64>              vertex_ordering/other_order/reorder.cpp:6-97, its default
//        GRO order (uint64 edges, src = x >> 32); writes <name>_GRO.txt (the edges sorted,
//        relabelled, "src dst" lines) and <name>_GRO_newID.txt ("old new" lines)
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <string>
#include <utility>
#include <vector>

#include "atc.h"

static int fail(const char* what, atc_status s) {
  fprintf(stderr, "%s failed: %s: %s\n", what, atc_status_string(s), atc_last_error());
  return 1;
}

static bool read_pairs(const char* path, std::vector<int32_t>& pairs) {
  FILE* f = fopen(path, "rb");
  if (!f) return false;
  fseek(f, 0, SEEK_END);
  long sz = ftell(f);
  fseek(f, 0, SEEK_SET);
  size_t n = sz > 0 ? (size_t)sz / 8 : 0;
  pairs.resize(2 * n);
  size_t got = n ? fread(pairs.data(), 8, n, f) : 0;
  fclose(f);
  return got == n;
}

// "src dst" text lines, read until the first line that does not parse (relabel4lpOut.cpp:20)
static bool read_text_pairs(const char* path, std::vector<int32_t>& pairs) {
  FILE* f = fopen(path, "r");
  if (!f) return false;
  int a = 0, b = 0;
  while (fscanf(f, "%d %d", &a, &b) == 2) {
    pairs.push_back(a);
    pairs.push_back(b);
  }
  fclose(f);
  return true;
}

static bool write_pairs(const char* path, const int32_t* p, size_t n) {
  FILE* f = fopen(path, "wb");
  if (!f) return false;
  size_t w = n ? fwrite(p, 8, n, f) : 0;
  fclose(f);
  return w == n;
}

// Arguments of each program, as its reference counterpart takes them.
#if defined(ATC_PROGRAM_COST_FUNC_CAL)
static const char* const kArgs = "<edges.bin> <k>";
static const int kMinArgc = 3;
#elif defined(ATC_PROGRAM_PEEL)
static const char* const kArgs = "inputFileName outFileName [--compat]";
static const int kMinArgc = 3;
#elif defined(ATC_PROGRAM_KCORE_DIRECTION)
static const char* const kArgs = "<in.u64> <out.u64>";
static const int kMinArgc = 3;
#elif defined(ATC_PROGRAM_REORDER)
static const char* const kArgs = "<graph.u64>";
static const int kMinArgc = 2;
#elif defined(ATC_PROGRAM_RELABEL4LP_OUT)
static const char* const kArgs = "<edges.txt>";
static const int kMinArgc = 2;
#else
static const char* const kArgs = "<edges.bin>";
static const int kMinArgc = 2;
#endif

int main(int argc, char** argv) {
  if (argc < kMinArgc) { fprintf(stderr, "usage: %s %s\n", argv[0], kArgs); return 2; }
  std::vector<int32_t> pairs;
#if defined(ATC_PROGRAM_RELABEL4LP_OUT)
  const bool read_ok = read_text_pairs(argv[1], pairs);
#else
  const bool read_ok = read_pairs(argv[1], pairs);
#endif
  if (!read_ok) { fprintf(stderr, "cannot read %s\n", argv[1]); return 1; }
  uint64_t np = pairs.size() / 2;
  atc_status s = atc_init(0);
  if (s != ATC_OK) return fail("atc_init", s);
#if defined(ATC_PROGRAM_A_DIRECTION_SERI)
  std::vector<int32_t> out(2 * (np ? np : 1));
  uint64_t n_out = 0;
  s = atc_adirection(pairs.data(), np, out.data(), &n_out, nullptr, nullptr);
  if (s != ATC_OK) return fail("atc_adirection", s);
  FILE* t = fopen("lpBasedGraph", "w");
  if (!t) return 1;
  for (uint64_t i = 0; i < n_out; ++i) fprintf(t, "%d %d\n", out[2 * i], out[2 * i + 1]);
  fclose(t);
  if (!write_pairs("lpBasedGraph.bin", out.data(), n_out)) return 1;
  std::cout << "we have dealed with " << n_out << " edges up to now" << std::endl;
#elif defined(ATC_PROGRAM_BISSON_A_DIRECTION)
  int32_t mx = 0;
  for (int32_t x : pairs) mx = x > mx ? x : mx;
  std::vector<int32_t> lookup((size_t)mx + 1);
  s = atc_relabel(pairs.data(), np, ATC_RELABEL_ADIRECTION_BISSON, lookup.data(), nullptr, nullptr, nullptr);
  if (s != ATC_OK) return fail("atc_relabel", s);
  // the program writes each vertex's sorted, duplicate-free neighbours (:293-300)
  std::vector<int32_t> sym(4 * (np ? np : 1));
  uint64_t ns = 0;
  s = atc_simplify_host(pairs.data(), np, 1, sym.data(), &ns);
  if (s != ATC_OK) return fail("atc_simplify_host", s);
  for (uint64_t i = 0; i < 2 * ns; ++i) sym[i] = lookup[sym[i]];
  FILE* t = fopen("lpBasedGraph", "w");  // created empty, as the program leaves it
  if (!t) return 1;
  fclose(t);
  if (!write_pairs("lpBasedGraph.bin", sym.data(), ns)) return 1;
  std::cout << "we have dealed with 0 edges up to now" << std::endl;  // the program's count stays 0
#elif defined(ATC_PROGRAM_A_ORDER)
  int32_t mx = 0;
  for (int32_t x : pairs) mx = x > mx ? x : mx;
  std::vector<int32_t> lookup((size_t)mx + 1), normal(pairs.size()), reordered(pairs.size());
  s = atc_aorder(pairs.data(), np, lookup.data(), normal.data(), reordered.data(), nullptr);
  if (s != ATC_OK) return fail("atc_aorder", s);
  if (!write_pairs("normal", normal.data(), np) || !write_pairs("reordered", reordered.data(), np)) return 1;
#elif defined(ATC_PROGRAM_A_ORDER_V2)
  int32_t mx = 0;
  for (int32_t x : pairs) mx = x > mx ? x : mx;
  std::vector<int32_t> lookup((size_t)mx + 1), naive(pairs.size() + 2);
  s = atc_relabel(pairs.data(), np, ATC_RELABEL_AORDER_V2, lookup.data(), nullptr, naive.data(), nullptr);
  if (s != ATC_OK) return fail("atc_relabel", s);
  if (!write_pairs("naive", naive.data(), np) || !write_pairs("degreeOrder", naive.data(), 0)) return 1;
#elif defined(ATC_PROGRAM_RELABEL_NAIVE) || defined(ATC_PROGRAM_RELABEL4LP_OUT) || defined(ATC_PROGRAM_RELABEL_RANDOM)
#if defined(ATC_PROGRAM_RELABEL_NAIVE)
  const atc_relabel_kind good_kind = ATC_RELABEL_DEGREE_DESC, bad_kind = ATC_RELABEL_NAIVE_SHUFFLED;
#elif defined(ATC_PROGRAM_RELABEL4LP_OUT)
  const atc_relabel_kind good_kind = ATC_RELABEL_OUTDEG_DESC, bad_kind = ATC_RELABEL_OUTDEG_SHUFFLED;
#else
  const atc_relabel_kind good_kind = ATC_RELABEL_DEGREE_DESC, bad_kind = ATC_RELABEL_RANDOM;
#endif
  int32_t mx = 0;
  for (int32_t x : pairs) mx = x > mx ? x : mx;
  const size_t nv = (size_t)mx + 1;
  std::vector<int32_t> good_lookup(nv), bad_lookup(nv), normal(pairs.size() + 2), good(pairs.size() + 2),
      bad(pairs.size() + 2);
  s = atc_relabel(pairs.data(), np, good_kind, good_lookup.data(), nullptr, good.data(), nullptr);
  if (s != ATC_OK) return fail("atc_relabel", s);
  s = atc_relabel(pairs.data(), np, bad_kind, bad_lookup.data(), normal.data(), bad.data(), nullptr);
  if (s != ATC_OK) return fail("atc_relabel", s);
  // the runtime degree: out-degree of the (oriented) pairs
  std::vector<int32_t> rt(nv, 0);
  for (uint64_t i = 0; i < np; ++i) rt[normal[2 * i]]++;
  std::cout << "the max runtime degree is " << *std::max_element(rt.begin(), rt.end()) << std::endl;
#if defined(ATC_PROGRAM_RELABEL_NAIVE)
  std::cout << "the reorder time is 0 s." << std::endl;
  if (!write_pairs("naive", bad.data(), np) || !write_pairs("degreeOrder", good.data(), np)) return 1;
#else
#if defined(ATC_PROGRAM_RELABEL_RANDOM)
  std::vector<int32_t> at(nv);  // the vertex at each position of the shuffle
  for (size_t v = 0; v < nv; ++v) at[bad_lookup[v]] = (int32_t)v;
  for (size_t i = 0; i + 1 < nv; ++i) std::cout << rt[at[i]] << "\n";
  std::cout.flush();
#endif
  if (!write_pairs("normal", normal.data(), np) || !write_pairs("bad", bad.data(), np) ||
      !write_pairs("good", good.data(), np))
    return 1;
#endif
#elif defined(ATC_PROGRAM_COST_FUNC_CAL)
  float c[3];
  s = atc_costfunc(pairs.data(), np, atoi(argv[2]), c, nullptr);
  if (s != ATC_OK) return fail("atc_costfunc", s);
  std::cout << "idPartCost: " << c[0] << std::endl;
  std::cout << "degreePartCost: " << c[1] << std::endl;
  std::cout << "lpPartCost: " << c[2] << std::endl;
#elif defined(ATC_PROGRAM_PEEL)
  const int compat = argc > 3 && strcmp(argv[3], "--compat") == 0;
  std::vector<uint64_t> packed(np), out(np ? np : 1);
  if (np) memcpy(packed.data(), pairs.data(), 8 * np);
  uint64_t nv = 0;
  int32_t iters = 0;
  s = atc_adirection_par(packed.data(), np, compat, out.data(), nullptr, nullptr, &nv, &iters, nullptr);
  if (s != ATC_OK) return fail("atc_adirection_par", s);
  std::cout << "the node num is " << nv << ", and the edgeNum is " << np << std::endl;
  std::cout << "iterations " << iters << std::endl;
  if (!write_pairs(argv[2], reinterpret_cast<const int32_t*>(out.data()), np)) return 1;
#elif defined(ATC_PROGRAM_KCORE_DIRECTION)
  // the file's bytes read as little-endian uint64 edges
  std::vector<uint64_t> packed(np), out(np ? np : 1);
  if (np) memcpy(packed.data(), pairs.data(), 8 * np);
  uint64_t nv = 0;
  s = atc_kcore_direction(packed.data(), np, out.data(), nullptr, &nv, nullptr);
  if (s != ATC_OK) return fail("atc_kcore_direction", s);
  std::cout << "the edge num is " << np << std::endl;
  std::cout << "the node num is " << nv << std::endl;
  if (!write_pairs(argv[2], reinterpret_cast<const int32_t*>(out.data()), np)) return 1;
#elif defined(ATC_PROGRAM_REORDER)
  // the file's uint64 words hold the source in the high half (other_order/util.cpp:56-67)
  std::vector<int32_t> directed(pairs.size());
  int32_t mx = -1;
  for (uint64_t i = 0; i < np; ++i) {
    directed[2 * i] = pairs[2 * i + 1];
    directed[2 * i + 1] = pairs[2 * i];
    mx = std::max(mx, std::max(directed[2 * i], directed[2 * i + 1]));
  }
  std::vector<int32_t> lookup((size_t)std::max(mx, 0) + 1);
  s = atc_relabel(directed.data(), np, ATC_RELABEL_GRO, lookup.data(), nullptr, nullptr, nullptr);
  if (s != ATC_OK) return fail("atc_relabel", s);
  std::string name(argv[1]);
  size_t slash = name.find_last_of('/');
  if (slash != std::string::npos) name = name.substr(slash + 1);
  size_t dot = name.find_last_of('.');
  if (dot != std::string::npos) name = name.substr(0, dot);
  std::vector<std::pair<int32_t, int32_t>> sorted(np);
  for (uint64_t i = 0; i < np; ++i) sorted[i] = {directed[2 * i], directed[2 * i + 1]};
  std::sort(sorted.begin(), sorted.end());
  FILE* g = fopen((name + "_GRO.txt").c_str(), "w");
  FILE* ids = fopen((name + "_GRO_newID.txt").c_str(), "w");
  if (!g || !ids) return 1;
  for (const auto& e : sorted) fprintf(g, "%d %d\n", lookup[e.first], lookup[e.second]);
  const int32_t nv = std::max(mx, 0) + 1;  // the program counts one vertex for an empty list
  for (int32_t i = 0; i < nv; ++i) fprintf(ids, "%d %d\n", i, lookup[i]);
  fclose(g);
  fclose(ids);
  printf("order_algo=gro graph_file=%s\n", name.c_str());
#else
#error "define one ATC_PROGRAM_*"
#endif
  return 0;
}
