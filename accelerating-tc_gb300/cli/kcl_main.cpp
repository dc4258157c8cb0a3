// Drop-in for the k-clique program (k-clique/kcl_gpu.cpp:13-32, kcl.cu:147-215):
//   kcl <edges.bin> -k=K
// The reference reads a Galois .gr file through Galois/Pangolin (not part of the
// reference tree); this program reads the int32 pair files of the other tools, orients
// by A-direction and prints the reference's result line "total_num_cliques = N".
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "atc.h"

int main(int argc, char** argv) {
  const char* path = nullptr;
  unsigned k = 3;
  for (int i = 1; i < argc; ++i) {
    if (strncmp(argv[i], "-k=", 3) == 0) k = (unsigned)atoi(argv[i] + 3);
    else if (argv[i][0] != '-') path = argv[i];
  }
  if (!path) { fprintf(stderr, "usage: %s <edges.bin> -k=K\n", argv[0]); return 2; }
  FILE* f = fopen(path, "rb");
  if (!f) { fprintf(stderr, "cannot read %s\n", path); return 1; }
  fseek(f, 0, SEEK_END);
  long sz = ftell(f);
  fseek(f, 0, SEEK_SET);
  size_t n = sz > 0 ? (size_t)sz / 8 : 0;
  std::vector<int32_t> pairs(2 * n);
  size_t got = n ? fread(pairs.data(), 8, n, f) : 0;
  fclose(f);
  if (got != n) return 1;
  atc_status s = atc_init(0);
  atc_csr csr;
  if (s == ATC_OK) s = atc_pretc(pairs.data(), n, ATC_DIR_ADIRECTION, ATC_ORDER_NONE, nullptr, &csr, nullptr, nullptr);
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
