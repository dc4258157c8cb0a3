// Drop-in command lines for the reference's triangle-counting programs, on libatc.
// One source, four programs (selected by -DATC_PROGRAM_*):
//
//   tc_hu     -f <edges.bin>               Hu/tc.cu:202-341        (degree orientation, Hu kernel)
//   tc_bisson -f <edges.bin> <chooseIndex> Bisson/tc.cu:105-231    (0: id orientation, 1: degree)
//   tc_fox    -f <edges.bin> <rearrange>   Fox/tc.cu:184-407       (id orientation, Fox kernel)
//   tric_gpu  -f <edges.u64> [debug]       tricore/src/main.cpp:14-100 (packed uint64 edges)
//
// Each prints the reference's result line "There are N triangles in the input graph."
// Unlike the reference, failures exit non-zero with the library's message on stderr.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "atc.h"

static int fail(const char* what, atc_status s) {
  fprintf(stderr, "%s failed: %s: %s\n", what, atc_status_string(s), atc_last_error());
  return 1;
}

static bool read_file(const char* path, std::vector<char>& buf) {
  FILE* f = fopen(path, "rb");
  if (!f) return false;
  fseek(f, 0, SEEK_END);
  long sz = ftell(f);
  fseek(f, 0, SEEK_SET);
  buf.resize(sz > 0 ? (size_t)sz : 0);
  size_t got = sz > 0 ? fread(buf.data(), 1, (size_t)sz, f) : 0;
  fclose(f);
  return got == buf.size();
}

int main(int argc, char** argv) {
  atc_tuning tune;
  memset(&tune, 0, sizeof(tune));
  atc_dir dir = ATC_DIR_DEGREE;
  atc_kernel kernel = ATC_KERNEL_HU;
  bool packed_u64 = false;
#if defined(ATC_PROGRAM_TC_HU)
  if (argc != 3) { printf("Usage: ./TC -f inputFileName\n"); return 2; }
  tune.prune_deg1 = 1;  // Hu/preTC.cu:135-169
#elif defined(ATC_PROGRAM_TC_BISSON)
  if (argc != 4) { printf("Usage: ./TC -f inputFileName chooseindex\n"); return 2; }
  dir = atoi(argv[3]) == 0 ? ATC_DIR_ID : ATC_DIR_DEGREE;
  kernel = ATC_KERNEL_BISSON;
#elif defined(ATC_PROGRAM_TC_FOX)
  if (argc != 4) { printf("Usage: ./TC -f inputFileName\n"); return 2; }
  dir = ATC_DIR_ID;
  kernel = ATC_KERNEL_FOX;
  tune.fox_rearrange = atoi(argv[3]) != 0;
#elif defined(ATC_PROGRAM_TRIC_GPU)
  if (argc < 3) { printf("usage: %s -f graph_name\n", argv[0]); return 2; }
  dir = ATC_DIR_DEGREE_LOWID;
  kernel = ATC_KERNEL_TRICORE;
  packed_u64 = true;
#else
#error "define one ATC_PROGRAM_*"
#endif
  std::vector<char> raw;
  if (!read_file(argv[2], raw)) { fprintf(stderr, "cannot read %s\n", argv[2]); return 1; }
  std::vector<int32_t> pairs;
  if (packed_u64) {
    if (raw.size() % 8) { fprintf(stderr, "file size error: cannot be divided by 8\n"); return 1; }
    size_t n = raw.size() / 8;
    pairs.resize(2 * n);
    for (size_t i = 0; i < n; ++i) {
      uint64_t x;
      memcpy(&x, raw.data() + 8 * i, 8);
      pairs[2 * i] = (int32_t)(uint32_t)(x >> 32);        // FIRST (tricore/include/util.h:14)
      pairs[2 * i + 1] = (int32_t)(uint32_t)(x & 0xffffffffu);  // SECOND
    }
  } else {
    size_t n = raw.size() / 8;  // Hu/preTC.cu:74: whole pairs only
    pairs.resize(2 * n);
    if (n) memcpy(pairs.data(), raw.data(), 8 * n);
  }
  atc_status s = atc_init(0);
  if (s != ATC_OK) return fail("atc_init", s);
  atc_csr csr;
  s = atc_pretc(pairs.data(), pairs.size() / 2, dir, ATC_ORDER_NONE, &tune, &csr, nullptr, nullptr);
  if (s != ATC_OK) return fail("atc_pretc", s);
  uint64_t count = 0;
  atc_stats st;
  s = atc_tc(&csr, kernel, &tune, &count, &st, nullptr);
  atc_csr_free(&csr);
  if (s != ATC_OK) return fail("atc_tc", s);
  printf("There are %llu triangles in the input graph.\n", (unsigned long long)count);
  printf("kernel use %f s.\n", st.kernel_ms / 1000.0);
  return 0;
}
