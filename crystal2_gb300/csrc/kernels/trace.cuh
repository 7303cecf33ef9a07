// Ray/shape intersection and BVH traversal with the reference's semantics.
//
// Triangle hits are solved exactly as Triangle::Intersect/IntersectTest do
// (src/Shapes/Triangle.cpp:32-93): res = inverse(mat3(v1-v0, v2-v0, -d)) * (o - v0) with glm's
// cofactor inverse (glm/detail/func_matrix.inl compute_inverse<3,3>) and every operation
// rounded separately, and the object box test is RayBoxTest (src/Core/Geometry.h:136-157) with
// the same rounding.  Bit-identical arithmetic matters here because the BVH shadow query hands
// the object-box-clipped interval [t1, t2] to the triangle test (BVH.cpp:132-134): for an
// axis-aligned triangle t1 == t2 and the test passes only when both computations agree to the
// last bit, which makes such triangles partly transparent to shadow rays in the reference.
#pragma once
#include <climits>

#include "dev_common.cuh"

namespace c2g {

struct RayQ {
    float3 o, d, inv;
    int neg[3];
};

__device__ __forceinline__ RayQ make_rayq(float3 o, float3 d) {
    RayQ r;
    r.o = o;
    r.d = d;
    r.inv = f3(__frcp_rn(d.x), __frcp_rn(d.y), __frcp_rn(d.z));
    r.neg[0] = r.inv.x < 0.f;
    r.neg[1] = r.inv.y < 0.f;
    r.neg[2] = r.inv.z < 0.f;
    return r;
}

// RayBoxTest(ray, inv, invD, box, tMin, tMax): updates t0/t1 like the reference.
__device__ __forceinline__ bool box_test(const RayQ& r, const float* mn, const float* mx, float& t0, float& t1) {
#pragma unroll
    for (int k = 0; k < 3; k++) {
        float o = k == 0 ? r.o.x : (k == 1 ? r.o.y : r.o.z);
        float iv = k == 0 ? r.inv.x : (k == 1 ? r.inv.y : r.inv.z);
        float a = __fmul_rn(__fsub_rn(mn[k], o), iv);
        float b = __fmul_rn(__fsub_rn(mx[k], o), iv);
        if (r.neg[k]) { float t = a; a = b; b = t; }
        t0 = smax(t0, a);
        t1 = smin(t1, b);
        if (t1 < t0) return false;
    }
    return true;
}

// Solve for res (see file comment).  Returns false as soon as a component is rejected.
// mode 0: Intersect acceptance (u+v <= 1 + EPS); mode 1: IntersectTest acceptance (u+v <= 1).
template <int MODE>
__device__ __forceinline__ bool tri_solve(float3 v0, float3 v1, float3 v2, const RayQ& r, float& rx, float& ry, float& rz) {
    const float m00 = __fsub_rn(v1.x, v0.x), m01 = __fsub_rn(v1.y, v0.y), m02 = __fsub_rn(v1.z, v0.z);
    const float m10 = __fsub_rn(v2.x, v0.x), m11 = __fsub_rn(v2.y, v0.y), m12 = __fsub_rn(v2.z, v0.z);
    const float m20 = -r.d.x, m21 = -r.d.y, m22 = -r.d.z;
    const float px = __fsub_rn(r.o.x, v0.x), py = __fsub_rn(r.o.y, v0.y), pz = __fsub_rn(r.o.z, v0.z);
    const float c00 = __fsub_rn(__fmul_rn(m11, m22), __fmul_rn(m21, m12));
    const float c01 = __fsub_rn(__fmul_rn(m01, m22), __fmul_rn(m21, m02));
    const float c02 = __fsub_rn(__fmul_rn(m01, m12), __fmul_rn(m11, m02));
    const float det = __fadd_rn(__fsub_rn(__fmul_rn(m00, c00), __fmul_rn(m10, c01)), __fmul_rn(m20, c02));
    const float ood = __frcp_rn(det);
    // row 0 of the inverse -> res.x
    const float i00 = __fmul_rn(c00, ood);
    const float i10 = __fmul_rn(-__fsub_rn(__fmul_rn(m10, m22), __fmul_rn(m20, m12)), ood);
    const float i20 = __fmul_rn(__fsub_rn(__fmul_rn(m10, m21), __fmul_rn(m20, m11)), ood);
    rx = __fadd_rn(__fadd_rn(__fmul_rn(i00, px), __fmul_rn(i10, py)), __fmul_rn(i20, pz));
    if (!(rx >= 0.f && rx <= 1.f)) return false;  // also rejects NaN
    const float i01 = __fmul_rn(-c01, ood);
    const float i11 = __fmul_rn(__fsub_rn(__fmul_rn(m00, m22), __fmul_rn(m20, m02)), ood);
    const float i21 = __fmul_rn(-__fsub_rn(__fmul_rn(m00, m21), __fmul_rn(m20, m01)), ood);
    ry = __fadd_rn(__fadd_rn(__fmul_rn(i01, px), __fmul_rn(i11, py)), __fmul_rn(i21, pz));
    if (!(ry >= 0.f && ry <= 1.f)) return false;
    const float i02 = __fmul_rn(c02, ood);
    const float i12 = __fmul_rn(-__fsub_rn(__fmul_rn(m00, m12), __fmul_rn(m10, m02)), ood);
    const float i22 = __fmul_rn(__fsub_rn(__fmul_rn(m00, m11), __fmul_rn(m10, m01)), ood);
    rz = __fadd_rn(__fadd_rn(__fmul_rn(i02, px), __fmul_rn(i12, py)), __fmul_rn(i22, pz));
    if (rz != rz) return false;
    const float uv = __fadd_rn(rx, ry);
    if (MODE == 0) {
        if (uv > 1.0f + kEpsTri) return false;
    } else {
        if (uv > 1.0f) return false;
    }
    return !(rz < 0.f);
}

// Sphere quadratic (Sphere.cpp:39-91).  Returns the hit distance of Intersect semantics,
// or -1 on a miss.  For IntersectTest semantics use sphere_test.
__device__ __forceinline__ void quadric_local(const Quadric& q, const RayQ& r, float3& P, float3& d) {
    float3 c = f3(q.c[0], q.c[1], q.c[2]);
    float3 rel = r.o - c;
    // _world2Local * v: column-major mat3 times vector
    P = f3(q.w2l[0] * rel.x + q.w2l[4] * rel.y + q.w2l[8] * rel.z,
           q.w2l[1] * rel.x + q.w2l[5] * rel.y + q.w2l[9] * rel.z,
           q.w2l[2] * rel.x + q.w2l[6] * rel.y + q.w2l[10] * rel.z);
    d = f3(q.w2l[0] * r.d.x + q.w2l[4] * r.d.y + q.w2l[8] * r.d.z,
           q.w2l[1] * r.d.x + q.w2l[5] * r.d.y + q.w2l[9] * r.d.z,
           q.w2l[2] * r.d.x + q.w2l[6] * r.d.y + q.w2l[10] * r.d.z);
}

__device__ __forceinline__ bool sphere_roots(const Quadric& q, const RayQ& r, float& t1, float& t2) {
    float3 P, d;
    quadric_local(q, r, P, d);
    float rad = q.c[3];
    float a = dot(d, d);
    float b = 2 * dot(d, P);
    float c = dot(P, P) - rad * rad;
    float disc = b * b - 4 * a * c;
    if (disc < 0) return false;
    disc = sqrtf(disc);
    t1 = (-b + disc) / (2 * a);
    t2 = (-b - disc) / (2 * a);
    return true;
}

__device__ __forceinline__ float sphere_hit(const Quadric& q, const RayQ& r) {
    float t1, t2;
    if (!sphere_roots(q, r, t1, t2)) return -1.f;
    if (t1 > t2) { float t = t1; t1 = t2; t2 = t; }
    float t = t1;
    if (isnan(t1) || t1 < 0) t = t2;
    if (isnan(t) || t < 0) return -1.f;
    return t;
}

__device__ __forceinline__ bool sphere_test(const Quadric& q, const RayQ& r, float tmin, float tmax) {
    if (tmin > tmax) return false;
    float t1, t2;
    if (!sphere_roots(q, r, t1, t2)) return false;
    return (t1 >= tmin && t1 <= tmax) || (t2 >= tmin && t2 <= tmax);
}

// Disk (Disk.cpp:45-78)
__device__ __forceinline__ float disk_hit(const Quadric& q, const RayQ& r, float tmin, float tmax, bool test) {
    float3 P, d;
    quadric_local(q, r, P, d);
    if (d.y == 0.f) return -1.f;
    float t = -P.y / d.y;
    if (test) {
        if (t < tmin || t > tmax) return -1.f;
    } else if (t < 0) {
        return -1.f;
    }
    float3 h = P + d * t;
    if (dot(h, h) > q.c[3] * q.c[3]) return -1.f;
    return t;
}

// Object box of a prim (IIntersectable::GetBoundingBox): triangle vertex min/max or stored box.
__device__ __forceinline__ void prim_box(const float4& a, const float4& b, const float4& c, int type, float* mn, float* mx) {
    if (type == SHAPE_TRI) {
        mn[0] = fminf(fminf(a.x, b.x), c.x); mn[1] = fminf(fminf(a.y, b.y), c.y); mn[2] = fminf(fminf(a.z, b.z), c.z);
        mx[0] = fmaxf(fmaxf(a.x, b.x), c.x); mx[1] = fmaxf(fmaxf(a.y, b.y), c.y); mx[2] = fmaxf(fmaxf(a.z, b.z), c.z);
    } else {
        mn[0] = b.x; mn[1] = b.y; mn[2] = b.z;
        mx[0] = c.x; mx[1] = c.y; mx[2] = c.z;
    }
}

struct Hit {
    float t, u, v;
    int obj;
};

struct TraceCounters {
    unsigned nodes, prims;
};

// Closest-hit test of one prim (the leaf body of BVH::Intersect, BVH.cpp:73-90).
__device__ __forceinline__ void closest_prim(const DevScene& S, int pi, const RayQ& r, float tmax, Hit& h) {
    const float4* P = reinterpret_cast<const float4*>(S.prims + pi);
    float4 a = __ldg(P), b = __ldg(P + 1), c = __ldg(P + 2);
    int ot = __float_as_int(a.w);
    int type = prim_type(ot);
    if (S.closest_box) {
        float mn[3], mx[3];
        prim_box(a, b, c, type, mn, mx);
        float t0 = 0.f, t1 = smin(tmax, h.t);
        if (!box_test(r, mn, mx, t0, t1)) return;
    }
    float dis;
    float u = 0.f, v = 0.f;
    if (type == SHAPE_TRI) {
        float rz;
        if (!tri_solve<0>(f3(a), f3(b), f3(c), r, u, v, rz)) return;
        dis = rz;
    } else {
        const Quadric& q = S.quads[__float_as_int(b.w)];
        dis = type == SHAPE_SPHERE ? sphere_hit(q, r) : disk_hit(q, r, 0.f, 0.f, false);
        if (dis < 0.f) return;
    }
    if (dis < h.t) {
        h.t = dis;
        h.u = u;
        h.v = v;
        h.obj = prim_obj(ot);
    }
}

// Any-hit test of one prim (leaf body of BVH::IntersectTest, BVH.cpp:127-136).
__device__ __forceinline__ bool anyhit_prim(const DevScene& S, int pi, const RayQ& r, float tmin, float tmax, int ignore) {
    const float4* P = reinterpret_cast<const float4*>(S.prims + pi);
    float4 a = __ldg(P), b = __ldg(P + 1), c = __ldg(P + 2);
    int ot = __float_as_int(a.w);
    if (prim_obj(ot) == ignore) return false;
    int type = prim_type(ot);
    float t0 = tmin, t1 = tmax;
    if (S.anyhit_clip) {
        float mn[3], mx[3];
        prim_box(a, b, c, type, mn, mx);
        if (!box_test(r, mn, mx, t0, t1)) return false;
    }
    if (type == SHAPE_TRI) {
        if (t0 > t1) return false;
        float rx, ry, rz;
        if (!tri_solve<1>(f3(a), f3(b), f3(c), r, rx, ry, rz)) return false;
        return rz >= t0 && rz <= t1;
    }
    const Quadric& q = S.quads[__float_as_int(b.w)];
    if (type == SHAPE_SPHERE) return sphere_test(q, r, t0, t1);
    return disk_hit(q, r, t0, t1, true) >= 0.f;
}

constexpr int kStack = 64;

// BVH::Intersect over the reference tree (BVH.cpp:56-108): near child by the sign of the ray
// on the split axis, node box clipped by the current closest distance.
template <bool COUNT>
__device__ __forceinline__ Hit trace_closest_ref(const DevScene& S, const RayQ& r, float tmax, TraceCounters* cnt) {
    Hit h{INFINITY, 0.f, 0.f, -1};
    int stack[kStack];
    int top = 0;
    int cur = 1;
    while (true) {
        const float4* N = reinterpret_cast<const float4*>(S.ref_nodes + cur);
        float4 A = __ldg(N), B = __ldg(N + 1);
        if (COUNT) cnt->nodes++;
        float mn[3] = {A.x, A.y, A.z}, mx[3] = {B.x, B.y, B.z};
        float t0 = 0.f, t1 = smin(tmax, h.t);
        bool ok = box_test(r, mn, mx, t0, t1);
        int a = __float_as_int(A.w), b = __float_as_int(B.w);
        int axis = (b >> 28) & 3;
        if (ok && axis == 3) {
            int cnt_ = b & 0x0fffffff;
            for (int i = 0; i < cnt_; i++) {
                if (COUNT) cnt->prims++;
                closest_prim(S, a + i, r, tmax, h);
            }
        } else if (ok) {
            int c1 = b & 0x0fffffff;
            int neg = axis == 0 ? r.neg[0] : (axis == 1 ? r.neg[1] : r.neg[2]);
            if (top >= kStack) { dev_flag_error(S.err, DEVERR_STACK); break; }
            stack[top++] = neg ? a : c1;
            cur = neg ? c1 : a;
            continue;
        }
        if (!top) break;
        cur = stack[--top];
    }
    return h;
}

template <bool COUNT>
__device__ __forceinline__ bool trace_any_ref(const DevScene& S, const RayQ& r, float tmin, float tmax, int ignore, TraceCounters* cnt) {
    int stack[kStack];
    int top = 0;
    int cur = 1;
    while (true) {
        const float4* N = reinterpret_cast<const float4*>(S.ref_nodes + cur);
        float4 A = __ldg(N), B = __ldg(N + 1);
        if (COUNT) cnt->nodes++;
        float mn[3] = {A.x, A.y, A.z}, mx[3] = {B.x, B.y, B.z};
        float t0 = tmin, t1 = tmax;
        bool ok = box_test(r, mn, mx, t0, t1);
        int a = __float_as_int(A.w), b = __float_as_int(B.w);
        int axis = (b >> 28) & 3;
        if (ok && axis == 3) {
            int cnt_ = b & 0x0fffffff;
            for (int i = 0; i < cnt_; i++) {
                if (COUNT) cnt->prims++;
                if (anyhit_prim(S, a + i, r, tmin, tmax, ignore)) return true;
            }
        } else if (ok) {
            int c1 = b & 0x0fffffff;
            int neg = axis == 0 ? r.neg[0] : (axis == 1 ? r.neg[1] : r.neg[2]);
            if (top >= kStack) { dev_flag_error(S.err, DEVERR_STACK); return false; }
            stack[top++] = neg ? a : c1;
            cur = neg ? c1 : a;
            continue;
        }
        if (!top) break;
        cur = stack[--top];
    }
    return false;
}

// Compact SAH tree traversal ("while-while" with leaf postponing).  Both child boxes live in the
// parent node; a child is an inner-node index or a leaf (first prim, count) packed into a negative
// reference.  Each lane walks inner nodes until it has found a leaf, then keeps walking while other
// lanes of the warp still search; the leaves are intersected together once every active lane has
// one, so the expensive exact triangle tests run with most lanes active.  Closest-hit pushes carry
// the entry distance so that subtrees beyond the current hit are dropped on pop.
constexpr int kNoRef = INT_MIN;
__device__ __forceinline__ int leaf_ref(int first, int count) { return -1 - ((first << 3) | count); }
__device__ __forceinline__ bool is_leaf(int ref) { return ref < 0 && ref != kNoRef; }
__device__ __forceinline__ void leaf_range(int ref, int& first, int& count) {
    int v = -1 - ref;
    first = v >> 3;
    count = v & 7;
}

template <bool COUNT>
__device__ __forceinline__ Hit trace_closest_sah(const DevScene& S, const RayQ& r, float tmax, TraceCounters* cnt) {
    Hit h{INFINITY, 0.f, 0.f, -1};
    int stack[kStack];
    float stack_t[kStack];
    int top = 0;
    int ref = 0, leaf = kNoRef;
    auto pop = [&]() -> int {
        while (top > 0) {
            --top;
            if (stack_t[top] <= h.t) return stack[top];
        }
        return kNoRef;
    };
    while (ref != kNoRef || leaf != kNoRef) {
        while (ref >= 0) {
            const float4* N = reinterpret_cast<const float4*>(S.wide_nodes + ref);
            float4 L0 = __ldg(N), H0 = __ldg(N + 1), L1 = __ldg(N + 2), H1 = __ldg(N + 3);
            if (COUNT) cnt->nodes++;
            float lim = smin(tmax, h.t);
            float mn0[3] = {L0.x, L0.y, L0.z}, mx0[3] = {H0.x, H0.y, H0.z};
            float mn1[3] = {L1.x, L1.y, L1.z}, mx1[3] = {H1.x, H1.y, H1.z};
            float a0 = 0.f, b0 = lim, a1 = 0.f, b1 = lim;
            bool hit0 = box_test(r, mn0, mx0, a0, b0);
            bool hit1 = box_test(r, mn1, mx1, a1, b1);
            int n0 = __float_as_int(H0.w), n1 = __float_as_int(H1.w);
            int r0 = n0 > 0 ? leaf_ref(__float_as_int(L0.w), n0) : __float_as_int(L0.w);
            int r1 = n1 > 0 ? leaf_ref(__float_as_int(L1.w), n1) : __float_as_int(L1.w);
            if (hit0 && hit1) {
                bool swap = a1 < a0;
                int nr = swap ? r1 : r0, fr = swap ? r0 : r1;
                float ft = swap ? a0 : a1;
                if (top >= kStack) { dev_flag_error(S.err, DEVERR_STACK); return h; }
                stack[top] = fr;
                stack_t[top] = ft;
                top++;
                ref = nr;
            } else if (hit0) {
                ref = r0;
            } else if (hit1) {
                ref = r1;
            } else {
                ref = pop();
            }
            if (is_leaf(ref) && leaf == kNoRef) {
                leaf = ref;
                ref = pop();
            }
            if (!__any_sync(__activemask(), leaf == kNoRef)) break;
        }
        while (leaf != kNoRef) {
            int first, count;
            leaf_range(leaf, first, count);
            for (int i = 0; i < count; i++) {
                if (COUNT) cnt->prims++;
                closest_prim(S, first + i, r, tmax, h);
            }
            leaf = kNoRef;
            if (is_leaf(ref)) {
                leaf = ref;
                ref = pop();
            }
        }
    }
    return h;
}

template <bool COUNT>
__device__ __forceinline__ bool trace_any_sah(const DevScene& S, const RayQ& r, float tmin, float tmax, int ignore, TraceCounters* cnt) {
    int stack[kStack];
    int top = 0;
    int ref = 0, leaf = kNoRef;
    while (ref != kNoRef || leaf != kNoRef) {
        while (ref >= 0) {
            const float4* N = reinterpret_cast<const float4*>(S.wide_nodes + ref);
            float4 L0 = __ldg(N), H0 = __ldg(N + 1), L1 = __ldg(N + 2), H1 = __ldg(N + 3);
            if (COUNT) cnt->nodes++;
            float mn0[3] = {L0.x, L0.y, L0.z}, mx0[3] = {H0.x, H0.y, H0.z};
            float mn1[3] = {L1.x, L1.y, L1.z}, mx1[3] = {H1.x, H1.y, H1.z};
            float a0 = tmin, b0 = tmax, a1 = tmin, b1 = tmax;
            bool hit0 = box_test(r, mn0, mx0, a0, b0);
            bool hit1 = box_test(r, mn1, mx1, a1, b1);
            int n0 = __float_as_int(H0.w), n1 = __float_as_int(H1.w);
            int r0 = n0 > 0 ? leaf_ref(__float_as_int(L0.w), n0) : __float_as_int(L0.w);
            int r1 = n1 > 0 ? leaf_ref(__float_as_int(L1.w), n1) : __float_as_int(L1.w);
            if (hit0 && hit1) {
                if (top >= kStack) { dev_flag_error(S.err, DEVERR_STACK); return false; }
                stack[top++] = r1;
                ref = r0;
            } else if (hit0) {
                ref = r0;
            } else if (hit1) {
                ref = r1;
            } else {
                ref = top ? stack[--top] : kNoRef;
            }
            if (is_leaf(ref) && leaf == kNoRef) {
                leaf = ref;
                ref = top ? stack[--top] : kNoRef;
            }
            if (!__any_sync(__activemask(), leaf == kNoRef)) break;
        }
        while (leaf != kNoRef) {
            int first, count;
            leaf_range(leaf, first, count);
            for (int i = 0; i < count; i++) {
                if (COUNT) cnt->prims++;
                if (anyhit_prim(S, first + i, r, tmin, tmax, ignore)) return true;
            }
            leaf = kNoRef;
            if (is_leaf(ref)) {
                leaf = ref;
                ref = top ? stack[--top] : kNoRef;
            }
        }
    }
    return false;
}

// ---- four-wide SAH traversal --------------------------------------------------------------------
// The per-axis slab distances are computed with the exact operations of box_test (subtract, then
// multiply, each rounded) and combined with fmaxf/fminf, which ignore NaN exactly as the
// reference's std::max/std::min argument order does; so a child is hit here exactly when box_test
// would accept it, and the leaves reached are those of the binary traversal.
constexpr int kStack4 = 128;

__device__ __forceinline__ bool slab4(const RayQ& r, float lx, float hx, float ly, float hy, float lz, float hz,
                                      float t0, float t1, float& tent) {
    float ax = __fmul_rn(__fsub_rn(lx, r.o.x), r.inv.x), bx = __fmul_rn(__fsub_rn(hx, r.o.x), r.inv.x);
    float ay = __fmul_rn(__fsub_rn(ly, r.o.y), r.inv.y), by = __fmul_rn(__fsub_rn(hy, r.o.y), r.inv.y);
    float az = __fmul_rn(__fsub_rn(lz, r.o.z), r.inv.z), bz = __fmul_rn(__fsub_rn(hz, r.o.z), r.inv.z);
    const float nx = r.neg[0] ? bx : ax, fx = r.neg[0] ? ax : bx;
    const float ny = r.neg[1] ? by : ay, fy = r.neg[1] ? ay : by;
    const float nz = r.neg[2] ? bz : az, fz = r.neg[2] ? az : bz;
    const float tn = fmaxf(fmaxf(nx, ny), fmaxf(nz, t0));
    const float tf = fminf(fminf(fx, fy), fminf(fz, t1));
    tent = tn;
    return tn <= tf;
}

// Near/far-ordered node loads: the ray's direction signs pick, per axis, which of a Node4's lo / hi
// plane words holds the near planes, so the slab test needs no per-child swap (six selects per
// child fewer; 1080p many-material step 605 -> 609 Mpaths/s).  slab_nf on the ordered planes
// computes exactly what slab4 computes on (lo, hi).  C2G_NEARFAR=0 restores the plain loads.
#ifndef C2G_NEARFAR
#define C2G_NEARFAR 1
#endif
struct Node4Planes {
    float4 nx, fx, ny, fy, nz, fz;
    int4 ch;
};
__device__ __forceinline__ Node4Planes load_node4(const Node4* nodes, int ref, const RayQ& r) {
    const float4* N = reinterpret_cast<const float4*>(nodes + ref);
    Node4Planes p;
#if C2G_NEARFAR
    p.nx = __ldg(N + r.neg[0]);
    p.fx = __ldg(N + (r.neg[0] ^ 1));
    p.ny = __ldg(N + 2 + r.neg[1]);
    p.fy = __ldg(N + 2 + (r.neg[1] ^ 1));
    p.nz = __ldg(N + 4 + r.neg[2]);
    p.fz = __ldg(N + 4 + (r.neg[2] ^ 1));
#else
    p.nx = __ldg(N);
    p.fx = __ldg(N + 1);
    p.ny = __ldg(N + 2);
    p.fy = __ldg(N + 3);
    p.nz = __ldg(N + 4);
    p.fz = __ldg(N + 5);
#endif
    p.ch = __ldg(reinterpret_cast<const int4*>(N + 6));
    return p;
}
__device__ __forceinline__ bool slab_nf(const RayQ& r, float nx, float fx, float ny, float fy, float nz, float fz, float t0,
                                        float t1, float& tent) {
#if C2G_NEARFAR
    const float ax = __fmul_rn(__fsub_rn(nx, r.o.x), r.inv.x), bx = __fmul_rn(__fsub_rn(fx, r.o.x), r.inv.x);
    const float ay = __fmul_rn(__fsub_rn(ny, r.o.y), r.inv.y), by = __fmul_rn(__fsub_rn(fy, r.o.y), r.inv.y);
    const float az = __fmul_rn(__fsub_rn(nz, r.o.z), r.inv.z), bz = __fmul_rn(__fsub_rn(fz, r.o.z), r.inv.z);
    const float tn = fmaxf(fmaxf(ax, ay), fmaxf(az, t0));
    const float tf = fminf(fminf(bx, by), fminf(bz, t1));
    tent = tn;
    return tn <= tf;
#else
    return slab4(r, nx, fx, ny, fy, nz, fz, t0, t1, tent);
#endif
}

__device__ __forceinline__ void cswap(float& ta, int& ca, float& tb, int& cb) {
    if (tb < ta) {
        float t = ta; ta = tb; tb = t;
        int c = ca; ca = cb; cb = c;
    }
}

template <bool COUNT>
__device__ __forceinline__ Hit trace_closest_bvh4(const DevScene& S, const RayQ& r, float tmax, TraceCounters* cnt) {
    Hit h{INFINITY, 0.f, 0.f, -1};
    int stack[kStack4];
    float stack_t[kStack4];
    int top = 0;
    int ref = 0, leaf = kNoRef;
    auto pop = [&]() -> int {
        while (top > 0) {
            --top;
            if (stack_t[top] <= h.t) return stack[top];
        }
        return kNoRef;
    };
    while (ref != kNoRef || leaf != kNoRef) {
        while (ref >= 0) {
            const Node4Planes P = load_node4(S.nodes4, ref, r);
            const int4 ch = P.ch;
            if (COUNT) cnt->nodes++;
            const float lim = smin(tmax, h.t);
            float t[4];
            int c[4] = {ch.x, ch.y, ch.z, ch.w};
            if (!slab_nf(r, P.nx.x, P.fx.x, P.ny.x, P.fy.x, P.nz.x, P.fz.x, 0.f, lim, t[0])) { t[0] = INFINITY; c[0] = kNoRef; }
            if (!slab_nf(r, P.nx.y, P.fx.y, P.ny.y, P.fy.y, P.nz.y, P.fz.y, 0.f, lim, t[1])) { t[1] = INFINITY; c[1] = kNoRef; }
            if (!slab_nf(r, P.nx.z, P.fx.z, P.ny.z, P.fy.z, P.nz.z, P.fz.z, 0.f, lim, t[2])) { t[2] = INFINITY; c[2] = kNoRef; }
            if (!slab_nf(r, P.nx.w, P.fx.w, P.ny.w, P.fy.w, P.nz.w, P.fz.w, 0.f, lim, t[3])) { t[3] = INFINITY; c[3] = kNoRef; }
            // nearest first: sort the four (entry, child) pairs, push the far ones far-to-near
            cswap(t[0], c[0], t[1], c[1]);
            cswap(t[2], c[2], t[3], c[3]);
            cswap(t[0], c[0], t[2], c[2]);
            cswap(t[1], c[1], t[3], c[3]);
            cswap(t[1], c[1], t[2], c[2]);
            if (top + 3 > kStack4) { dev_flag_error(S.err, DEVERR_STACK); return h; }
#pragma unroll
            for (int k = 3; k >= 1; k--)
                if (c[k] != kNoRef) { stack[top] = c[k]; stack_t[top] = t[k]; top++; }
            ref = c[0] != kNoRef ? c[0] : pop();
            if (is_leaf(ref) && leaf == kNoRef) {
                leaf = ref;
                ref = pop();
            }
            if (!__any_sync(__activemask(), leaf == kNoRef)) break;
        }
        while (leaf != kNoRef) {
            int first, count;
            leaf_range(leaf, first, count);
            for (int i = 0; i < count; i++) {
                if (COUNT) cnt->prims++;
                closest_prim(S, first + i, r, tmax, h);
            }
            leaf = kNoRef;
            if (is_leaf(ref)) {
                leaf = ref;
                ref = pop();
            }
        }
    }
    return h;
}

template <bool COUNT>
__device__ __forceinline__ bool trace_any_bvh4(const DevScene& S, const RayQ& r, float tmin, float tmax, int ignore, TraceCounters* cnt) {
    int stack[kStack4];
    int top = 0;
    int ref = 0, leaf = kNoRef;
    while (ref != kNoRef || leaf != kNoRef) {
        while (ref >= 0) {
            const Node4Planes P = load_node4(S.nodes4, ref, r);
            const int4 ch = P.ch;
            if (COUNT) cnt->nodes++;
            float te;
            const bool h0 = slab_nf(r, P.nx.x, P.fx.x, P.ny.x, P.fy.x, P.nz.x, P.fz.x, tmin, tmax, te);
            const bool h1 = slab_nf(r, P.nx.y, P.fx.y, P.ny.y, P.fy.y, P.nz.y, P.fz.y, tmin, tmax, te);
            const bool h2 = slab_nf(r, P.nx.z, P.fx.z, P.ny.z, P.fy.z, P.nz.z, P.fz.z, tmin, tmax, te);
            const bool h3 = slab_nf(r, P.nx.w, P.fx.w, P.ny.w, P.fy.w, P.nz.w, P.fz.w, tmin, tmax, te);
            if (top + 3 > kStack4) { dev_flag_error(S.err, DEVERR_STACK); return false; }
            int next = kNoRef;
            if (h3) next = ch.w;
            if (h2) { if (next != kNoRef) stack[top++] = next; next = ch.z; }
            if (h1) { if (next != kNoRef) stack[top++] = next; next = ch.y; }
            if (h0) { if (next != kNoRef) stack[top++] = next; next = ch.x; }
            ref = next != kNoRef ? next : (top ? stack[--top] : kNoRef);
            if (is_leaf(ref) && leaf == kNoRef) {
                leaf = ref;
                ref = top ? stack[--top] : kNoRef;
            }
            if (!__any_sync(__activemask(), leaf == kNoRef)) break;
        }
        while (leaf != kNoRef) {
            int first, count;
            leaf_range(leaf, first, count);
            for (int i = 0; i < count; i++) {
                if (COUNT) cnt->prims++;
                if (anyhit_prim(S, first + i, r, tmin, tmax, ignore)) return true;
            }
            leaf = kNoRef;
            if (is_leaf(ref)) {
                leaf = ref;
                ref = top ? stack[--top] : kNoRef;
            }
        }
    }
    return false;
}

// ---- resumable four-wide traversal rounds (dynamic ray fetch) ----------------------------------
// One while-while round of the traversal above: inner nodes until every active lane of the warp
// holds a leaf, then the leaves.  The state survives between rounds, so a kernel can hand a lane a
// new ray as soon as its previous one is done (see k_shadow_fetch / k_extend_fetch).
struct Bvh4AnyState {       // any hit: no entry distances
    int stack[kStack4];
    int top, ref, leaf;
};
struct Bvh4State {          // closest hit: entry distance per stacked subtree
    int stack[kStack4];
    float stack_t[kStack4];
    int top, ref, leaf;
};

template <class St>
__device__ __forceinline__ void bvh4_begin(St& st) {
    st.top = 0;
    st.ref = 0;
    st.leaf = kNoRef;
}

// Any hit in (tmin, tmax); returns true when the ray is finished (occluded or exhausted).
template <bool COUNT>
__device__ __forceinline__ bool bvh4_any_round(const DevScene& S, const RayQ& r, float tmin, float tmax, int ignore,
                                               Bvh4AnyState& st, TraceCounters* cnt, bool& occluded) {
    occluded = false;
    int top = st.top, ref = st.ref, leaf = st.leaf;
    while (ref >= 0) {
        const Node4Planes P = load_node4(S.nodes4, ref, r);
        const int4 ch = P.ch;
        if (COUNT) cnt->nodes++;
        float te;
        const bool h0 = slab_nf(r, P.nx.x, P.fx.x, P.ny.x, P.fy.x, P.nz.x, P.fz.x, tmin, tmax, te);
        const bool h1 = slab_nf(r, P.nx.y, P.fx.y, P.ny.y, P.fy.y, P.nz.y, P.fz.y, tmin, tmax, te);
        const bool h2 = slab_nf(r, P.nx.z, P.fx.z, P.ny.z, P.fy.z, P.nz.z, P.fz.z, tmin, tmax, te);
        const bool h3 = slab_nf(r, P.nx.w, P.fx.w, P.ny.w, P.fy.w, P.nz.w, P.fz.w, tmin, tmax, te);
        if (top + 3 > kStack4) { dev_flag_error(S.err, DEVERR_STACK); top = 0; ref = kNoRef; leaf = kNoRef; break; }
        int next = kNoRef;
        if (h3) next = ch.w;
        if (h2) { if (next != kNoRef) st.stack[top++] = next; next = ch.z; }
        if (h1) { if (next != kNoRef) st.stack[top++] = next; next = ch.y; }
        if (h0) { if (next != kNoRef) st.stack[top++] = next; next = ch.x; }
        ref = next != kNoRef ? next : (top ? st.stack[--top] : kNoRef);
        if (is_leaf(ref) && leaf == kNoRef) {
            leaf = ref;
            ref = top ? st.stack[--top] : kNoRef;
        }
        if (!__any_sync(__activemask(), leaf == kNoRef)) break;
    }
    while (leaf != kNoRef && !occluded) {
        int first, count;
        leaf_range(leaf, first, count);
        for (int k = 0; k < count; k++) {
            if (COUNT) cnt->prims++;
            if (anyhit_prim(S, first + k, r, tmin, tmax, ignore)) { occluded = true; break; }
        }
        leaf = kNoRef;
        if (!occluded && is_leaf(ref)) {
            leaf = ref;
            ref = top ? st.stack[--top] : kNoRef;
        }
    }
    st.top = top;
    st.ref = ref;
    st.leaf = leaf;
    return occluded || (ref == kNoRef && leaf == kNoRef);
}

// Closest hit (h carries the running result); returns true when the ray is finished.
template <bool COUNT>
__device__ __forceinline__ bool bvh4_closest_round(const DevScene& S, const RayQ& r, float tmax, Hit& h, Bvh4State& st,
                                                   TraceCounters* cnt) {
    int top = st.top, ref = st.ref, leaf = st.leaf;
    auto pop = [&]() -> int {
        while (top > 0) {
            --top;
            if (st.stack_t[top] <= h.t) return st.stack[top];
        }
        return kNoRef;
    };
    while (ref >= 0) {
        const Node4Planes P = load_node4(S.nodes4, ref, r);
        const int4 ch = P.ch;
        if (COUNT) cnt->nodes++;
        const float lim = smin(tmax, h.t);
        float t[4];
        int c[4] = {ch.x, ch.y, ch.z, ch.w};
        if (!slab_nf(r, P.nx.x, P.fx.x, P.ny.x, P.fy.x, P.nz.x, P.fz.x, 0.f, lim, t[0])) { t[0] = INFINITY; c[0] = kNoRef; }
        if (!slab_nf(r, P.nx.y, P.fx.y, P.ny.y, P.fy.y, P.nz.y, P.fz.y, 0.f, lim, t[1])) { t[1] = INFINITY; c[1] = kNoRef; }
        if (!slab_nf(r, P.nx.z, P.fx.z, P.ny.z, P.fy.z, P.nz.z, P.fz.z, 0.f, lim, t[2])) { t[2] = INFINITY; c[2] = kNoRef; }
        if (!slab_nf(r, P.nx.w, P.fx.w, P.ny.w, P.fy.w, P.nz.w, P.fz.w, 0.f, lim, t[3])) { t[3] = INFINITY; c[3] = kNoRef; }
        cswap(t[0], c[0], t[1], c[1]);
        cswap(t[2], c[2], t[3], c[3]);
        cswap(t[0], c[0], t[2], c[2]);
        cswap(t[1], c[1], t[3], c[3]);
        cswap(t[1], c[1], t[2], c[2]);
        if (top + 3 > kStack4) { dev_flag_error(S.err, DEVERR_STACK); top = 0; ref = kNoRef; leaf = kNoRef; break; }
#pragma unroll
        for (int k = 3; k >= 1; k--)
            if (c[k] != kNoRef) { st.stack[top] = c[k]; st.stack_t[top] = t[k]; top++; }
        ref = c[0] != kNoRef ? c[0] : pop();
        if (is_leaf(ref) && leaf == kNoRef) {
            leaf = ref;
            ref = pop();
        }
        if (!__any_sync(__activemask(), leaf == kNoRef)) break;
    }
    while (leaf != kNoRef) {
        int first, count;
        leaf_range(leaf, first, count);
        for (int k = 0; k < count; k++) {
            if (COUNT) cnt->prims++;
            closest_prim(S, first + k, r, tmax, h);
        }
        leaf = kNoRef;
        if (is_leaf(ref)) {
            leaf = ref;
            ref = pop();
        }
    }
    st.top = top;
    st.ref = ref;
    st.leaf = leaf;
    return ref == kNoRef && leaf == kNoRef;
}

// Warp-wide refill: lanes that need a ray take consecutive indices from *fetch.  Returns the index
// for this lane (-1: none left) and must be called by all 32 lanes.
__device__ __forceinline__ int warp_fetch(int* fetch, bool need, int n) {
    const int lane = threadIdx.x & 31;
    const unsigned m = __ballot_sync(0xffffffffu, need);
    if (!m) return -1;
    const int leader = __ffs(m) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(fetch, __popc(m));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (!need) return -1;
    const int idx = base + __popc(m & ((1u << lane) - 1u));
    return idx < n ? idx : -1;
}

// Brute semantics (Brute.cpp:19-55): every object, no box tests.
__device__ __forceinline__ Hit trace_closest_brute(const DevScene& S, const RayQ& r) {
    Hit h{INFINITY, 0.f, 0.f, -1};
    for (int i = 0; i < S.n_prims; i++) closest_prim(S, i, r, INFINITY, h);
    return h;
}
__device__ __forceinline__ bool trace_any_brute(const DevScene& S, const RayQ& r, float tmin, float tmax, int ignore) {
    for (int i = 0; i < S.n_prims; i++)
        if (anyhit_prim(S, i, r, tmin, tmax, ignore)) return true;
    return false;
}

template <bool COUNT>
__device__ __forceinline__ Hit trace_closest(const DevScene& S, float3 o, float3 d, TraceCounters* cnt) {
    RayQ r = make_rayq(o, d);
    if (S.tree == 1) return S.sah_width == 4 ? trace_closest_bvh4<COUNT>(S, r, INFINITY, cnt) : trace_closest_sah<COUNT>(S, r, INFINITY, cnt);
    return trace_closest_ref<COUNT>(S, r, INFINITY, cnt);
}

template <bool COUNT>
__device__ __forceinline__ bool trace_any(const DevScene& S, float3 o, float3 d, float tmin, float tmax, int ignore, TraceCounters* cnt) {
    RayQ r = make_rayq(o, d);
    if (S.tree == 1) return S.sah_width == 4 ? trace_any_bvh4<COUNT>(S, r, tmin, tmax, ignore, cnt) : trace_any_sah<COUNT>(S, r, tmin, tmax, ignore, cnt);
    return trace_any_ref<COUNT>(S, r, tmin, tmax, ignore, cnt);
}

}  // namespace c2g
