// Driver for the reference's CPU triangle counter (vertex_ordering/other_order:
// OrgTriangleCount in org_triangle_count.cpp with set_operation.cpp / util.cpp).
// Test infrastructure: compiled by oracle/Makefile into oracle/_ref/orgtc on x86
// hosts only (the reference's util.hpp includes <x86intrin.h>).
// Usage: orgtc <edges.u64>   (packed uint64, u = high half, both directions)
#include "org_triangle_count.hpp"
int main(int argc, char** argv) {
  if (argc < 2) return 2;
  EdgeVector ev = load_graph(argv[1]);
  OrgTriangleCount tc;
  tc.build(ev);
  printf("triangles=%d\n", tc.triangle_count());
  return 0;
}
