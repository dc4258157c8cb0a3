// Stand-in: see adjacency_list.hpp in this folder.
#pragma once
namespace boost {
template <class RandomGenerator, class Graph>
class plod_iterator {};
}  // namespace boost
