// Minimal stand-in for the Boost.Graph names that edge_directing/A-direction-seri.cpp
// mentions in typedefs only (lines 28-31).  Its READFROMFILE build path never
// instantiates them, so empty declarations are enough to compile the file unchanged.
#pragma once
namespace boost {
struct vecS {};
struct undirectedS {};
template <class OutEdgeList, class VertexList, class Directed>
class adjacency_list {};
}  // namespace boost
