// Stand-in: see ../graph/adjacency_list.hpp.
#pragma once
namespace boost {
class minstd_rand {};
}  // namespace boost
