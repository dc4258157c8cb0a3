// Drop-in for the k-clique program (k-clique/kcl_gpu.cpp:13-32, kcl.cu:147-215):
//   kcl [-symmetricGraph] [-simpleGraph] <graph.gr | edges.bin> -k=K
// Reads a Galois .gr file (the reference's input) or an int32 pair file, orients by
// A-direction and prints the reference's result line "total_num_cliques = N".
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "atc.h"

int main(int argc, char** argv) {
  const char* path = nullptr;
  unsigned k = 3;
  for (int i = 1; i < argc; ++i) {
    if (strncmp(argv[i], "-k=", 3) == 0) k = (unsigned)atoi(argv[i] + 3);
    else if (argv[i][0] != '-') path = argv[i];
  }
  if (!path) {
    fprintf(stderr, "usage: %s <graph.gr | edges.bin> -k=K\n", argv[0]);
    return 2;
  }
  uint64_t np = 0;
  std::vector<int32_t> pairs;
  atc_status s = atc_read_edges(path, nullptr, 0, &np);
  if (s == ATC_OK) {
    pairs.resize(2 * np);
    s = atc_read_edges(path, pairs.data(), np, &np);
  }
  if (s != ATC_OK) {
    fprintf(stderr, "%s\n", atc_last_error());
    return 1;
  }
  s = atc_init(0);
  atc_csr csr;
  if (s == ATC_OK)
    s = atc_pretc(pairs.data(), pairs.size() / 2, ATC_DIR_ADIRECTION, ATC_ORDER_NONE, nullptr, &csr, nullptr, nullptr);
  uint64_t total = 0;
  atc_stats st;
  if (s == ATC_OK) {
    s = atc_kcl(&csr, k, &total, &st, nullptr);
    atc_csr_free(&csr);
  }
  if (s != ATC_OK) {
    fprintf(stderr, "kcl failed: %s: %s\n", atc_status_string(s), atc_last_error());
    return 1;
  }
  printf("\n\ttotal_num_cliques = %llu\n\n", (unsigned long long)total);
  return 0;
}
