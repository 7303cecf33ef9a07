// Acceleration-structure builders.
//
//  * build_ref_tree: a replica of the reference BVH build (BVH::Build / _build /
//    splitByEqualCount / createLeaf / createInternal, src/Accelerators/BVH.cpp:45-54,156-188,
//    269-279,327-355): max-extent axis of the union box, std::nth_element on the box centre at
//    l + (r-l)/2, leaves of at most two objects, nodes numbered from 1 in creation (pre-)order.
//    The object order it leaves behind is the reference's primitive order bit for bit, and the
//    node array is identical; both are parity-tested against the reference.
//  * build_sah_tree: a binned-SAH builder for performance (the reference's SAH variant at
//    BVH.cpp:281-325 sorts by the wrong axis and is not reproduced).  It emits the compact
//    two-children-per-node layout (WideNode) the fast traversal kernels use.
#pragma once
#include <vector>

#include "../c2g_types.h"
#include "scene.h"

namespace c2g {

struct RefTree {
    std::vector<int> order;       // BVH::_objects as scene indices
    std::vector<RefNode> nodes;   // index 0 unused, 1.._tot valid (root = 1)
    int tot = 0;
};

struct SahTree {
    std::vector<int> order;       // prim order (scene indices)
    std::vector<WideNode> nodes;  // root = 0
    std::vector<Node4> nodes4;    // the same tree collapsed to four-wide nodes, root = 0
    int max_depth = 0;
    int leaf_count = 0;
};

void build_ref_tree(const HostScene& s, RefTree& out);
void build_sah_tree(const HostScene& s, SahTree& out, int max_leaf = 4);
// Collapse the binary SAH tree into four-wide nodes: every node absorbs the children of its
// largest-area inner children until it holds four (Node4; boxes and leaves unchanged).
void collapse_bvh4(SahTree& t);

// Prim records for an object order (traversal order).
void make_prims(const HostScene& s, const std::vector<int>& order, std::vector<Prim>& prims);

}  // namespace c2g
