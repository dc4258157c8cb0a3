/* Source-level drop-in for the reference's k-clique entry point,
     void kcl_gpu_solver(std::string filename, unsigned k, AccType& total, size_t N_CHUNK = 1);
   (k-clique/kcl.h:6-7, defined in k-clique/kcl.cu:147-215).  A caller of the solver (such as
   k-clique/kcl_gpu.cpp:28-29) includes this header instead of kcl.h and links libatc instead
   of Pangolin's solver.

   Same name and argument meaning: the graph file (a Galois .gr file, the reference's input, or
   an int32 pair file), k, and an accumulator to which the number of k-cliques is ADDED, as the
   reference adds each chunk's count to `total`.  N_CHUNK, the reference's split of the
   embedding list into chunks, is accepted and has no effect: no level of the search is
   materialised here.  The graph is oriented by A-direction on the device; the count does not
   depend on the orientation.  The count runs on the calling thread's current CUDA device, which
   the call does not change (the reference solver never selects a device either).

   Errors: the reference aborts the process from inside the solver (CUDA_SAFE_CALL).  Here the
   solver throws std::runtime_error carrying libatc's message, and `total` is left unchanged. */
#pragma once

#include <cstddef>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "atc.h"

namespace atc_compat {

inline void kcl_fail(atc_status s, const char* what) {
  throw std::runtime_error(std::string("kcl_gpu_solver: ") + what + ": " + atc_status_string(s) + ": " +
                           atc_last_error());
}

}  // namespace atc_compat

// AccType is the caller's accumulator (an unsigned 64-bit integer in the reference).
template <class AccType>
inline void kcl_gpu_solver(std::string filename, unsigned k, AccType& total, size_t N_CHUNK = 1) {
  (void)N_CHUNK;
  uint64_t np = 0;
  atc_status s = atc_read_edges(filename.c_str(), nullptr, 0, &np);
  if (s != ATC_OK) atc_compat::kcl_fail(s, "reading the graph");
  std::vector<int32_t> pairs(2 * (size_t)np);
  s = atc_read_edges(filename.c_str(), pairs.data(), np, &np);
  if (s != ATC_OK) atc_compat::kcl_fail(s, "reading the graph");
  s = atc_init(-1);  // the caller's current device, as the reference solver uses it
  if (s != ATC_OK) atc_compat::kcl_fail(s, "device");
  atc_csr csr;
  s = atc_pretc(pairs.data(), np, ATC_DIR_ADIRECTION, ATC_ORDER_NONE, nullptr, &csr, nullptr, nullptr);
  if (s != ATC_OK) atc_compat::kcl_fail(s, "orienting the graph");
  uint64_t count = 0;
  s = atc_kcl(&csr, k, &count, nullptr, nullptr);
  atc_csr_free(&csr);
  if (s != ATC_OK) atc_compat::kcl_fail(s, "counting");
  total += (AccType)count;
}
