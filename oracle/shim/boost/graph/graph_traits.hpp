// Stand-in: see adjacency_list.hpp in this folder.
#pragma once
namespace boost {
template <class G>
struct graph_traits {};
}  // namespace boost
