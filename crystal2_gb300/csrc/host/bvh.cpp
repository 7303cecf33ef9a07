#include "bvh.h"

#include "../../../include/c2g.h"

#include <algorithm>
#include <climits>
#include <cmath>
#include <exception>
#include <limits>
#include <thread>
#include <vector>

namespace c2g {

namespace {

struct Box {
    float mn[3], mx[3];
};

inline Box box_union(const Box& a, const Box& b) {
    // glm::min / glm::max per component (Geometry.h:67-72)
    Box r;
    for (int k = 0; k < 3; k++) {
        r.mn[k] = std::min(a.mn[k], b.mn[k]);
        r.mx[k] = std::max(a.mx[k], b.mx[k]);
    }
    return r;
}

// BoundingBox::MaxExtent (Geometry.h:88-102)
inline int max_extent(const Box& b) {
    float v[3] = {b.mx[0] - b.mn[0], b.mx[1] - b.mn[1], b.mx[2] - b.mn[2]};
    int axis = 0;
    float d = std::abs(v[0]);
    for (int i = 1; i < 3; i++) {
        if (std::abs(v[i]) > d) { d = std::abs(v[i]); axis = i; }
    }
    return axis;
}

struct RefBuilder {
    const std::vector<Box>& boxes;
    const std::vector<float>& centers;  // 3 per object: GetCenter() = (min + max) / 2
    std::vector<int>& objs;
    std::vector<RefNode>& nodes;
    int tot = 0;

    void leaf(int& p, int l, int r) {
        Box b = boxes[objs[l]];
        for (int i = l + 1; i <= r; i++) b = box_union(b, boxes[objs[i]]);
        p = ++tot;
        RefNode& n = nodes[tot];
        for (int k = 0; k < 3; k++) { n.mn[k] = b.mn[k]; n.mx[k] = b.mx[k]; }
        n.a = l;
        n.b = (r - l + 1) | (3 << 28);
    }

    // BVH::_build: node ids are assigned before the children are built (pre-order), and the
    // child slots are filled through the reference as in the reference.
    void build(int& p, int l, int r) {
        if (r - l + 1 <= 2) { leaf(p, l, r); return; }
        Box b = boxes[objs[l]];
        for (int i = l + 1; i <= r; i++) b = box_union(b, boxes[objs[i]]);
        int axis = max_extent(b);
        int split = l + (r - l) / 2;
        const float* c = centers.data();
        std::nth_element(objs.begin() + l, objs.begin() + split, objs.begin() + r + 1,
                         [c, axis](int x, int y) { return c[3 * x + axis] < c[3 * y + axis]; });
        int self = ++tot;
        RefNode& n = nodes[self];
        for (int k = 0; k < 3; k++) { n.mn[k] = b.mn[k]; n.mx[k] = b.mx[k]; }
        int c0 = 0, c1 = 0;
        p = self;
        build(c0, l, split);
        build(c1, split + 1, r);
        nodes[self].a = c0;
        nodes[self].b = c1 | (axis << 28);
    }
};

void object_boxes(const HostScene& s, std::vector<Box>& boxes, std::vector<float>& centers) {
    size_t n = s.num_objects();
    boxes.resize(n);
    centers.resize(3 * n);
    for (size_t i = 0; i < n; i++) {
        float b[6];
        s.object_box((int)i, b);
        for (int k = 0; k < 3; k++) {
            boxes[i].mn[k] = b[k];
            boxes[i].mx[k] = b[3 + k];
            centers[3 * i + k] = (b[k] + b[3 + k]) / 2.f;
        }
    }
}

// ---- binned SAH ---------------------------------------------------------------------------

constexpr int kBins = 16;

inline float half_area(const Box& b) {
    float dx = b.mx[0] - b.mn[0], dy = b.mx[1] - b.mn[1], dz = b.mx[2] - b.mn[2];
    return dx * dy + dy * dz + dz * dx;
}

inline Box empty_box() {
    Box b;
    for (int k = 0; k < 3; k++) { b.mn[k] = std::numeric_limits<float>::infinity(); b.mx[k] = -std::numeric_limits<float>::infinity(); }
    return b;
}

struct ChildRef {
    Box box;
    int index;   // node index (internal) or first prim (leaf)
    int count;   // 0 internal, else prim count
};

// Subtrees of at least this many objects above depth par_depth are built on their own thread.
constexpr int kParallelMin = 4096;

struct SahBuilder {
    const std::vector<Box>& boxes;
    const std::vector<float>& centers;
    std::vector<int>& objs;
    std::vector<WideNode>& nodes;
    int max_leaf;
    int par_depth = 0;   // 2^par_depth threads at most
    int max_depth = 0;
    int leaves = 0;

    ChildRef build(int begin, int end, int depth) {
        max_depth = std::max(max_depth, depth);
        Box bb = empty_box(), cb = empty_box();
        for (int i = begin; i < end; i++) {
            const Box& b = boxes[objs[i]];
            bb = box_union(bb, b);
            for (int k = 0; k < 3; k++) {
                float c = centers[3 * objs[i] + k];
                cb.mn[k] = std::min(cb.mn[k], c);
                cb.mx[k] = std::max(cb.mx[k], c);
            }
        }
        int n = end - begin;
        if (n <= max_leaf) { leaves++; return ChildRef{bb, begin, n}; }
        // Best binned split over the three axes.
        float best_cost = std::numeric_limits<float>::infinity();
        int best_axis = -1, best_bin = -1;
        for (int axis = 0; axis < 3; axis++) {
            float lo = cb.mn[axis], hi = cb.mx[axis];
            if (!(hi > lo)) continue;
            float scale = kBins / (hi - lo);
            Box bin_box[kBins];
            int bin_cnt[kBins] = {0};
            for (int b = 0; b < kBins; b++) bin_box[b] = empty_box();
            for (int i = begin; i < end; i++) {
                int o = objs[i];
                int b = std::min(kBins - 1, (int)((centers[3 * o + axis] - lo) * scale));
                bin_cnt[b]++;
                bin_box[b] = box_union(bin_box[b], boxes[o]);
            }
            float right_area[kBins];
            int right_cnt[kBins];
            Box acc = empty_box();
            int cnt = 0;
            for (int b = kBins - 1; b > 0; b--) {
                acc = box_union(acc, bin_box[b]);
                cnt += bin_cnt[b];
                right_area[b] = cnt ? half_area(acc) : 0.f;
                right_cnt[b] = cnt;
            }
            acc = empty_box();
            cnt = 0;
            for (int b = 0; b < kBins - 1; b++) {
                acc = box_union(acc, bin_box[b]);
                cnt += bin_cnt[b];
                if (cnt == 0 || right_cnt[b + 1] == 0) continue;
                float cost = half_area(acc) * cnt + right_area[b + 1] * right_cnt[b + 1];
                if (cost < best_cost) { best_cost = cost; best_axis = axis; best_bin = b; }
            }
        }
        int mid;
        if (best_axis < 0) {
            // All centroids coincide: split by count.
            mid = begin + n / 2;
        } else {
            float lo = cb.mn[best_axis], hi = cb.mx[best_axis];
            float scale = kBins / (hi - lo);
            const float* c = centers.data();
            int ax = best_axis, bb_ = best_bin;
            auto it = std::partition(objs.begin() + begin, objs.begin() + end, [&](int o) {
                int b = std::min(kBins - 1, (int)((c[3 * o + ax] - lo) * scale));
                return b <= bb_;
            });
            mid = (int)(it - objs.begin());
            if (mid == begin || mid == end) mid = begin + n / 2;
        }
        int self = (int)nodes.size();
        nodes.emplace_back();
        ChildRef L, R;
        if (depth < par_depth && n >= kParallelMin) {
            // The right subtree is built on another thread into its own node array and appended
            // after the left one, renumbered: the same depth-first node order, so the same tree
            // as the sequential build.
            std::vector<WideNode> rnodes;
            SahBuilder rb{boxes, centers, objs, rnodes, max_leaf, par_depth};
            ChildRef Rr;
            std::exception_ptr r_err;
            std::thread t([&] {
                try {
                    Rr = rb.build(mid, end, depth + 1);
                } catch (...) {
                    r_err = std::current_exception();
                }
            });
            // the thread is joined on every way out of this block (a failed left build included),
            // so an exception reaches the caller instead of std::terminate
            try {
                L = build(begin, mid, depth + 1);
            } catch (...) {
                t.join();
                throw;
            }
            t.join();
            if (r_err) std::rethrow_exception(r_err);
            const int off = (int)nodes.size();
            for (WideNode& w : rnodes) {
                if (w.n0 == 0) w.c0 += off;
                if (w.n1 == 0) w.c1 += off;
            }
            nodes.insert(nodes.end(), rnodes.begin(), rnodes.end());
            R = Rr;
            if (R.count == 0) R.index += off;
            leaves += rb.leaves;
            max_depth = std::max(max_depth, rb.max_depth);
        } else {
            L = build(begin, mid, depth + 1);
            R = build(mid, end, depth + 1);
        }
        WideNode& w = nodes[self];
        for (int k = 0; k < 3; k++) {
            w.lo0[k] = L.box.mn[k]; w.hi0[k] = L.box.mx[k];
            w.lo1[k] = R.box.mn[k]; w.hi1[k] = R.box.mx[k];
        }
        w.c0 = L.index; w.n0 = L.count;
        w.c1 = R.index; w.n1 = R.count;
        return ChildRef{bb, self, 0};
    }
};

}  // namespace

void build_ref_tree(const HostScene& s, RefTree& out) {
    std::vector<Box> boxes;
    std::vector<float> centers;
    object_boxes(s, boxes, centers);
    size_t n = boxes.size();
    out.order.resize(n);
    for (size_t i = 0; i < n; i++) out.order[i] = (int)i;
    out.nodes.assign(2 * n + 1, RefNode{});
    RefBuilder b{boxes, centers, out.order, out.nodes};
    int root = 0;
    b.build(root, 0, (int)n - 1);
    out.tot = b.tot;
    out.nodes.resize(b.tot + 1);
}

void build_sah_tree(const HostScene& s, SahTree& out, int max_leaf) {
    // traversal packs a leaf as (first prim << 3 | count): counts up to 7, first prim below 2^27
    if (max_leaf > 7) max_leaf = 7;
    if (s.num_objects() >= (size_t(1) << 27)) throw SceneError(C2G_ERR_INVALID, "scene exceeds 2^27 primitives");
    std::vector<Box> boxes;
    std::vector<float> centers;
    object_boxes(s, boxes, centers);
    size_t n = boxes.size();
    out.order.resize(n);
    for (size_t i = 0; i < n; i++) out.order[i] = (int)i;
    out.nodes.clear();
    out.nodes.reserve(n);
    // parallel depth: log2 of the hardware threads (at most 8) plus one, so at most 16 threads
    int par_depth = 0;
    for (unsigned t = std::max(1u, std::min(8u, std::thread::hardware_concurrency())); t > 1; t >>= 1) par_depth++;
    SahBuilder b{boxes, centers, out.order, out.nodes, std::max(1, max_leaf), par_depth + 1};
    if ((int)n <= b.max_leaf) {
        // Single leaf: child 1 is an empty box that never intersects.
        Box bb = empty_box();
        for (size_t i = 0; i < n; i++) bb = box_union(bb, boxes[i]);
        WideNode w{};
        for (int k = 0; k < 3; k++) {
            w.lo0[k] = bb.mn[k]; w.hi0[k] = bb.mx[k];
            w.lo1[k] = std::numeric_limits<float>::infinity(); w.hi1[k] = -std::numeric_limits<float>::infinity();
        }
        w.c0 = 0; w.n0 = (int)n; w.c1 = 0; w.n1 = 0;
        out.nodes.push_back(w);
        out.max_depth = 1;
        out.leaf_count = 1;
        return;
    }
    b.build(0, (int)n, 1);
    out.max_depth = b.max_depth;
    out.leaf_count = b.leaves;
}

namespace {
struct Slot {
    float mn[3], mx[3];
    int wide;          // >= 0: binary inner node; -1: leaf
    int first, count;  // leaf range
};

float slot_area(const Slot& c) {
    float d[3];
    for (int k = 0; k < 3; k++) d[k] = std::max(0.f, c.mx[k] - c.mn[k]);
    return d[0] * d[1] + d[1] * d[2] + d[2] * d[0];
}

void wide_children(const WideNode& w, Slot out[2]) {
    for (int k = 0; k < 3; k++) {
        out[0].mn[k] = w.lo0[k]; out[0].mx[k] = w.hi0[k];
        out[1].mn[k] = w.lo1[k]; out[1].mx[k] = w.hi1[k];
    }
    out[0].wide = w.n0 > 0 ? -1 : w.c0; out[0].first = w.c0; out[0].count = w.n0;
    out[1].wide = w.n1 > 0 ? -1 : w.c1; out[1].first = w.c1; out[1].count = w.n1;
    for (int i = 0; i < 2; i++)
        if (!(out[i].mn[0] <= out[i].mx[0])) { out[i].wide = -1; out[i].count = 0; }  // empty box: no child
}

int emit4(const std::vector<WideNode>& bin, int wide, std::vector<Node4>& out) {
    Slot c[4];
    int n = 0;
    wide_children(bin[wide], c);
    n = 2;
    // an empty child (single-leaf tree) stays a leaf of count 0 and is dropped below
    while (n < 4) {
        int best = -1;
        float best_a = -1.f;
        for (int i = 0; i < n; i++)
            if (c[i].wide >= 0 && slot_area(c[i]) > best_a) { best_a = slot_area(c[i]); best = i; }
        if (best < 0) break;
        Slot two[2];
        wide_children(bin[c[best].wide], two);
        c[best] = two[0];
        c[n++] = two[1];
    }
    const int self = (int)out.size();
    out.emplace_back();
    int child[4];
    for (int i = 0; i < 4; i++) {
        if (i >= n || (c[i].wide < 0 && c[i].count == 0)) { child[i] = INT_MIN; continue; }
        child[i] = c[i].wide >= 0 ? emit4(bin, c[i].wide, out) : -1 - ((c[i].first << 3) | c[i].count);
    }
    Node4& d = out[self];
    const float inf = std::numeric_limits<float>::infinity();
    for (int i = 0; i < 4; i++) {
        const bool used = child[i] != INT_MIN;
        d.lox[i] = used ? c[i].mn[0] : inf; d.hix[i] = used ? c[i].mx[0] : -inf;
        d.loy[i] = used ? c[i].mn[1] : inf; d.hiy[i] = used ? c[i].mx[1] : -inf;
        d.loz[i] = used ? c[i].mn[2] : inf; d.hiz[i] = used ? c[i].mx[2] : -inf;
        d.child[i] = child[i];
        d.pad[i] = 0;
    }
    return self;
}
}  // namespace

void collapse_bvh4(SahTree& t) {
    t.nodes4.clear();
    if (t.nodes.empty()) return;
    t.nodes4.reserve(t.nodes.size() / 2 + 1);
    emit4(t.nodes, 0, t.nodes4);
}

void make_prims(const HostScene& s, const std::vector<int>& order, std::vector<Prim>& prims) {
    prims.resize(order.size());
    for (size_t i = 0; i < order.size(); i++) {
        int obj = order[i];
        const ObjInfo& o = s.objs[obj];
        Prim p{};
        p.objtype = obj | (o.type << 30);
        if (o.type == SHAPE_TRI) {
            const fm::V3* v = &s.tri_pos[3 * o.shape];
            p.v0[0] = v[0].x; p.v0[1] = v[0].y; p.v0[2] = v[0].z;
            p.v1[0] = v[1].x; p.v1[1] = v[1].y; p.v1[2] = v[1].z;
            p.v2[0] = v[2].x; p.v2[1] = v[2].y; p.v2[2] = v[2].z;
            p.aux = o.shape;
        } else {
            const float* b = &s.quad_box[6 * o.shape];
            const Quadric& q = s.quads[o.shape];
            p.v0[0] = q.c[0]; p.v0[1] = q.c[1]; p.v0[2] = q.c[2];
            p.v1[0] = b[0]; p.v1[1] = b[1]; p.v1[2] = b[2];
            p.v2[0] = b[3]; p.v2[1] = b[4]; p.v2[2] = b[5];
            p.aux = o.shape;
        }
        prims[i] = p;
    }
}

}  // namespace c2g
