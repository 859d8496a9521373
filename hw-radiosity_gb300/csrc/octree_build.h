// A built octree before flattening, shared by the host build (octree.cpp) and
// the device build (rad_octree_dev.cu): nodes with 8 children or a leaf, each
// leaf's box and triangle list.  finish_octree turns it into the Octree the
// solver uploads (leaf tables, cell thresholds, cell-to-leaf table).
#pragma once
#include <cstdint>
#include <vector>

#include "rad_host.h"

namespace radgb {

template <typename T>
struct Box { T g0[3], g1[3]; };

struct Node { int32_t child[8]; int32_t leaf; };

template <typename T>
struct Part {
    std::vector<Node> nodes;            // node 0 is the root
    std::vector<Box<T>> leaf_box;
    std::vector<int32_t> leaf_begin;    // into entries
    std::vector<int32_t> entries;       // each leaf's list, ascending triangle id
    int64_t n_list = 0;                 // sum of (list length + 1), the reference's list slots
    T min_edge;                         // smallest leaf edge along x
};

template <typename T>
void finish_octree(const Scene<T>& s, Part<T>& P, Octree<T>& o);

}  // namespace radgb
