// Edge-file readers (host only): atc_read_edges.
//   int32 pair files: {int32 src, int32 dst} per edge (Hu/preTC.cu:29-32,84);
//   Galois .gr files (the k-clique program's input, k-clique/README.md:12-15; the format is Galois's (not vendored)): header
//   {u64 version, u64 edge-data size, u64 nodes, u64 edges}, u64 end offset per node,
//   then the targets as u32 (version 1, padded to 8 bytes) or u64 (version 2).

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <exception>
#include <new>
#include <string>
#include <vector>

#include "common.cuh"

namespace atc {

static bool read_file_bytes(const char* path, std::vector<char>& buf) {
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

static bool ends_with(const std::string& s, const char* suf) {
  size_t n = strlen(suf);
  return s.size() >= n && s.compare(s.size() - n, n, suf) == 0;
}

// Whole pairs only, as the reference readers take size / 8 pairs.
static bool read_pairs_file(const char* path, std::vector<int32_t>& pairs) {
  std::vector<char> raw;
  if (!read_file_bytes(path, raw)) return false;
  size_t n = raw.size() / 8;
  pairs.resize(2 * n);
  if (n) memcpy(pairs.data(), raw.data(), 8 * n);
  return true;
}

// Galois .gr (versions 1 and 2) to int32 pairs (one per stored edge).  Returns false on
// a truncated or malformed file or ids beyond int32.
static bool read_gr_file(const char* path, std::vector<int32_t>& pairs) {
  std::vector<char> raw;
  if (!read_file_bytes(path, raw) || raw.size() < 32) return false;
  uint64_t hdr[4];
  memcpy(hdr, raw.data(), 32);
  const uint64_t version = hdr[0], nodes = hdr[2], edges = hdr[3];
  if ((version != 1 && version != 2) || nodes > 0x7fffffffull) return false;
  const size_t idx_at = 32, dst_at = idx_at + 8 * nodes;
  const size_t dst_size = version == 1 ? 4 : 8;
  // the header's counts must fit the file (checked by division: a forged count cannot wrap)
  if (raw.size() < dst_at || edges > (raw.size() - dst_at) / dst_size) return false;
  pairs.resize(2 * edges);
  uint64_t prev = 0;
  for (uint64_t u = 0; u < nodes; ++u) {
    uint64_t end;
    memcpy(&end, raw.data() + idx_at + 8 * u, 8);
    if (end < prev || end > edges) return false;
    for (uint64_t j = prev; j < end; ++j) {
      uint64_t v;
      if (version == 1) {
        uint32_t v32;
        memcpy(&v32, raw.data() + dst_at + 4 * j, 4);
        v = v32;
      } else {
        memcpy(&v, raw.data() + dst_at + 8 * j, 8);
      }
      if (v >= nodes) return false;
      pairs[2 * j] = (int32_t)u;
      pairs[2 * j + 1] = (int32_t)v;
    }
    prev = end;
  }
  return prev == edges;
}

}  // namespace atc

using namespace atc;

// Two-call pattern: with pairs == nullptr only *n_out is written.
extern "C" atc_status atc_read_edges(const char* path, int32_t* pairs, uint64_t cap, uint64_t* n_out) try {
  ATC_CHECK_ARG(path != nullptr && n_out != nullptr, "NULL argument");
  std::vector<int32_t> buf;
  bool ok;
  try {
    ok = ends_with(path, ".gr") ? read_gr_file(path, buf) : read_pairs_file(path, buf);
  } catch (const std::bad_alloc&) {
    atc::set_error("out of host memory reading %s", path);
    return ATC_ERR_OOM;
  } catch (const std::exception&) {
    atc::set_error("cannot read %s", path);
    return ATC_ERR_INVALID;
  }
  if (!ok) {
    atc::set_error("cannot read %s as %s", path, ends_with(path, ".gr") ? "a Galois .gr file" : "int32 pairs");
    return ATC_ERR_INVALID;
  }
  const uint64_t n = buf.size() / 2;
  *n_out = n;
  if (pairs == nullptr) return ATC_OK;
  ATC_CHECK_ARG(cap >= n, "pairs buffer smaller than the file's edge count");
  if (n) memcpy(pairs, buf.data(), 8 * n);
  return ATC_OK;
} ATC_CATCH
