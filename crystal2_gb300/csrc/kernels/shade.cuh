// Surface interaction, emission and light sampling (the per-hit work of
// PathTracingIntegrator::Evaluate / EsimateDirect, PathTracingIntegrator.cpp:28-278).
#pragma once
#include "bsdf.cuh"
#include "trace.cuh"

namespace c2g {

struct Surface {
    float3 pos;     // hit position (ray.start + ray.dir * t)
    float3 N;       // shading normal, flipped to face the incoming ray
    float3 dpdu, dpdv;
    bool front;     // front_face
    int obj;
    int mat;
    int light;
};

__device__ __forceinline__ float3 m3mul(const float* m, float3 v) {  // column-major mat3 (3 float4 columns)
    return f3(m[0] * v.x + m[4] * v.y + m[8] * v.z, m[1] * v.x + m[5] * v.y + m[9] * v.z, m[2] * v.x + m[6] * v.y + m[10] * v.z);
}

// Interpolated (unflipped) triangle normal at barycentrics (1-u-v, u, v) (Triangle.cpp:41-53).
__device__ __forceinline__ float3 tri_normal(const TriShade& ts, float u, float v) {
    float b0 = 1 - u - v;
    float3 n = f3(ts.n0) * b0 + f3(ts.n1) * u + f3(ts.n2) * v;
    return normalize(n);
}

// Triangle surface from a hit (Triangle::Intersect, Triangle.cpp:41-74).
__device__ __forceinline__ void tri_surface(const DevScene& S, int shape, float3 d, float u, float v, Surface& s) {
    const TriShade ts = S.tri_shade[shape];
    float3 N = tri_normal(ts, u, v);
    s.front = dot(d, N) < 0;
    N = s.front ? N : -N;
    float3 dpdu = f3(ts.n0[3], ts.n1[3], ts.n2[3]);
    if (is_zero(dpdu)) {
        // No UV tangent: the first axis whose cross product with N is non-zero (Triangle.cpp:59-72)
#pragma unroll
        for (int i = 0; i < 3; i++) {
            float3 e = f3(i == 0 ? 1.f : 0.f, i == 1 ? 1.f : 0.f, i == 2 ? 1.f : 0.f);
            float3 t = cross(e, N);
            if (!is_zero(t)) { dpdu = normalize(t); break; }
        }
    }
    s.N = N;
    s.dpdu = dpdu;
    s.dpdv = cross(N, dpdu);
}

__device__ __forceinline__ void sphere_surface(const Quadric& q, float3 o, float3 d, float t, Surface& s) {
    RayQ r;
    r.o = o;
    r.d = d;
    float3 P, dl;
    quadric_local(q, r, P, dl);
    float3 hp = P + dl * t;
    float3 N = normalize(hp);
    s.front = dot(dl, N) < 0;
    N = s.front ? N : -N;
    s.pos = m3mul(q.l2w, hp) + f3(q.c[0], q.c[1], q.c[2]);
    s.dpdu = normalize(m3mul(q.l2w, f3(-N.z, 0.f, N.x)));
    s.N = m3mul(q.l2w, N);
    s.dpdv = cross(s.N, s.dpdu);
}

__device__ __forceinline__ void disk_surface(const Quadric& q, float3 o, float3 d, float t, Surface& s) {
    RayQ r;
    r.o = o;
    r.d = d;
    float3 P, dl;
    quadric_local(q, r, P, dl);
    float3 hit = P + dl * t;
    float3 N = m3mul(q.l2w, f3(0.f, 1.f, 0.f));
    s.front = dl.y <= 0;
    N = s.front ? N : -N;
    s.pos = m3mul(q.l2w, hit) + f3(q.c[0], q.c[1], q.c[2]);
    s.N = N;
    s.dpdu = normalize(f3(q.c[0], q.c[1], q.c[2]) - s.pos);
    s.dpdv = cross(N, s.dpdu);
}

__device__ __forceinline__ void make_surface(const DevScene& S, float3 o, float3 d, const Hit& h, Surface& s) {
    const ObjInfo oi = S.objs[h.obj];
    s.obj = h.obj;
    s.mat = oi.material;
    s.light = oi.light;
    if (oi.type == SHAPE_TRI) {
        s.pos = o + d * h.t;
        tri_surface(S, oi.shape, d, h.u, h.v, s);
    } else if (oi.type == SHAPE_SPHERE) {
        sphere_surface(S.quads[oi.shape], o, d, h.t, s);
    } else {
        disk_surface(S.quads[oi.shape], o, d, h.t, s);
    }
}

// ---- textures (Texel.cpp:15-19, UVTexture.h, CubemapTexture.cpp:17-57) ------------------------
// ImageTexels::GetTexel: uv clamped to [0, 0.99999], nearest texel, v measured from the last row.
__device__ __forceinline__ float3 tex_lookup(const DevScene& S, int tex, float2 uv) {
    const int4 ti = __ldg(S.tex_info + tex);
    const float u = fminf(fmaxf(uv.x, 0.f), .99999f), v = fminf(fmaxf(uv.y, 0.f), .99999f);
    const int x = (int)__fmul_rn(u, (float)ti.x), y = ti.y - (int)__fmul_rn(v, (float)ti.y) - 1;
    const float* p = S.texels + ti.z + 3 * ((size_t)y * ti.x + x);
    return f3(__ldg(p), __ldg(p + 1), __ldg(p + 2));
}

// ImageCubemapTexture::Evaluate(dir): face by the dominant axis, face uv in [0, 1].
__device__ __forceinline__ float3 sky_lookup(const DevScene& S, float3 p) {
    const float ax = fabsf(p.x), ay = fabsf(p.y), az = fabsf(p.z);
    int id;
    float2 uv;
    if (ax >= ay && ax >= az) { id = p.x >= 0 ? 0 : 1; uv = make_float2(__fdiv_rn(-p.z, p.x), __fdiv_rn(p.y, ax)); }
    else if (ay >= az) { id = p.y >= 0 ? 2 : 3; uv = make_float2(__fdiv_rn(p.x, ay), __fdiv_rn(-p.z, p.y)); }
    else { id = p.z >= 0 ? 4 : 5; uv = make_float2(__fdiv_rn(p.x, p.z), __fdiv_rn(p.y, az)); }
    uv.x = __fadd_rn(__fmul_rn(uv.x, 0.5f), 0.5f);
    uv.y = __fadd_rn(__fmul_rn(uv.y, 0.5f), 0.5f);
    return tex_lookup(S, S.sky[id], uv);
}

// Texture coordinates of a hit: triangles interpolate the vertex uvs at (1-u-v, u, v)
// (Triangle.cpp:9-16,43), spheres use (atan2(-z, x) / pi, acos(y / r) / pi + 1) of the local hit
// (Sphere.cpp:55-59), disks (|hit| / r, (atan2(-z, x) + pi) / 2pi) (Disk.cpp:61-62).
__device__ __forceinline__ float2 surface_uv(const DevScene& S, float3 o, float3 d, const Hit& h) {
    const ObjInfo oi = S.objs[h.obj];
    if (oi.type == SHAPE_TRI) {
        const float2* t = S.tri_uv + 3 * oi.shape;
        const float2 t0 = __ldg(t), t1 = __ldg(t + 1), t2 = __ldg(t + 2);
        const float b0 = __fsub_rn(__fsub_rn(1.f, h.u), h.v), b1 = h.u, b2 = h.v;
        return make_float2(__fadd_rn(__fadd_rn(__fmul_rn(b0, t0.x), __fmul_rn(b1, t1.x)), __fmul_rn(b2, t2.x)),
                           __fadd_rn(__fadd_rn(__fmul_rn(b0, t0.y), __fmul_rn(b1, t1.y)), __fmul_rn(b2, t2.y)));
    }
    const Quadric& q = S.quads[oi.shape];
    RayQ r;
    r.o = o;
    r.d = d;
    float3 P, dl;
    quadric_local(q, r, P, dl);
    const float3 hp = P + dl * h.t;
    if (oi.type == SHAPE_SPHERE)
        return make_float2(atan2f(-hp.z, hp.x) / kPiF, acosf(hp.y / q.c[3]) / kPiF + 1.0f);
    return make_float2(length(hp) / q.c[3], (atan2f(-hp.z, hp.x) + kPiF) / kTwoPiF);
}

// SurfaceInteraction::SpawnRay / SpawnRayTo (SurfaceInteraction.cpp:12-22)
__device__ __forceinline__ float3 spawn_origin(const Surface& s, float3 dir) {
    bool back = dot(dir, s.N) < 0;
    return s.pos + (back ? -s.N : s.N) * kSpawnEps;
}

// DiffusedAreaLight::EvalEmitRadiance with the surface's actual (unflipped) normal.
__device__ __forceinline__ float3 area_Le(const Light& L, float3 n_actual, float3 w) {
    if (dot(n_actual, w) < 0) return f3(0.f, 0.f, 0.f);
    return f3(L.Le[0], L.Le[1], L.Le[2]);
}

// Intersect the light's own shape (Shape::PdfLight, Shape.cpp:4-12) and return the solid-angle
// pdf, 0 on a miss.  The ray leaves pos + N * 1e-4 along wi (SurfaceInfo::SpawnRay, no side test).
__device__ __forceinline__ float light_pdf(const DevScene& S, const Light& L, float3 pos, float3 N, float3 wi) {
    float3 o = pos + N * kSpawnEps;
    RayQ r = make_rayq(o, wi);
    float3 hp, Nh;
    if (L.shape_type == SHAPE_TRI) {
        const float4* v = S.tri_pos + 3 * L.shape_idx;
        float u, vv, t;
        if (!tri_solve<0>(f3(v[0]), f3(v[1]), f3(v[2]), r, u, vv, t)) return 0.f;
        hp = o + wi * t;
        Nh = tri_normal(S.tri_shade[L.shape_idx], u, vv);
        Nh = dot(wi, Nh) < 0 ? Nh : -Nh;
    } else {
        const Quadric& q = S.quads[L.shape_idx];
        float t = L.shape_type == SHAPE_SPHERE ? sphere_hit(q, r) : disk_hit(q, r, 0.f, 0.f, false);
        if (t < 0.f) return 0.f;
        Surface s;
        if (L.shape_type == SHAPE_SPHERE) sphere_surface(q, o, wi, t, s);
        else disk_surface(q, o, wi, t, s);
        hp = s.pos;
        Nh = s.N;
    }
    float3 dv = pos - hp;
    return dot(dv, dv) / (fmaxf(0.f, dot(-normalize(wi), Nh)) * L.area);
}

// Shape::SampleSurface of the light's shape: position and (unflipped) normal.
__device__ __forceinline__ void light_sample_surface(const DevScene& S, const Light& L, float2 u, float3& p, float3& n) {
    if (L.shape_type == SHAPE_TRI) {  // Triangle.cpp:100-125
        const float4* v = S.tri_pos + 3 * L.shape_idx;
        float su = sqrtf(u.x);
        float bu = 1 - su;
        float bv = u.y * su;
        float b0 = 1.f - bu - bv;
        p = b0 * f3(v[0]) + bu * f3(v[1]) + bv * f3(v[2]);
        const TriShade ts = S.tri_shade[L.shape_idx];
        n = normalize(f3(ts.n0) * b0 + f3(ts.n1) * bu + f3(ts.n2) * bv);
    } else if (L.shape_type == SHAPE_SPHERE) {  // NextUnitSphere (Utils.h:138-149)
        const Quadric& q = S.quads[L.shape_idx];
        float y = 2.f * u.x - 1.f;
        float phi = u.y * kTwoPiF;
        float r = sqrtf(1 - y * y);
        float s, c;
        sincosf(phi, &s, &c);
        float3 dir = f3(r * c, y, r * s);
        p = f3(q.c[0], q.c[1], q.c[2]) + dir * q.c[3];
        n = dir;
    } else {  // Disk::SampleSurface (Disk.cpp:85-93)
        const Quadric& q = S.quads[L.shape_idx];
        float r = sqrtf(u.x);
        float phi = u.y * kTwoPiF;
        float s, c;
        sincosf(phi, &s, &c);
        float3 dw = m3mul(q.l2w, f3(c * r * q.c[3], 0.f, -s * r * q.c[3]));
        p = f3(q.c[0], q.c[1], q.c[2]) + dw;
        n = m3mul(q.l2w, f3(0.f, 1.f, 0.f));
    }
}

// Light::Sample_Li (DiffusedAreaLight.cpp:25-34, PointLight.cpp:13-19).
__device__ __forceinline__ float3 light_sample_li(const DevScene& S, const Light& L, float3 pos, float3 N, float2 u,
                                                  float3& endpoint, float& pdf) {
    if (L.type == LIGHT_POINT) {
        endpoint = f3(L.pos[0], L.pos[1], L.pos[2]);
        pdf = 1.0f;
        float3 I = f3(L.Le[0], L.Le[1], L.Le[2]) / (4 * kPiF);
        float3 dv = endpoint - pos;
        return I / dot(dv, dv);
    }
    float3 lp, ln;
    light_sample_surface(S, L, u, lp, ln);
    endpoint = lp;
    float3 dir = lp - pos;
    pdf = light_pdf(S, L, pos, N, dir);
    return area_Le(L, ln, -dir);
}

// PowerHeuristic(1, f, 1, g) (Utils.h:168-172)
__device__ __forceinline__ float power_heuristic(float fPdf, float gPdf) {
    float f = fPdf, g = gPdf;
    return (f * f) / (f * f + g * g);
}

}  // namespace c2g
