// Links the reference's other_order reorder program without METIS: the GRO order it is
// built for never calls these; a METIS order request fails loudly instead.
#include <cstdio>
#include <cstdlib>

#include "metis.h"

int METIS_PartGraphRecursive(idx_t*, idx_t*, idx_t*, idx_t*, idx_t*, idx_t*, idx_t*, idx_t*, real_t*, real_t*,
                             idx_t*, idx_t*, idx_t*) {
  std::fprintf(stderr, "METIS is not available in this build\n");
  std::abort();
}

int METIS_SetDefaultOptions(idx_t*) { return METIS_OK; }
