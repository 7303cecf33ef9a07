// Plain data shared by the host library and the CUDA kernels: the flattened scene, the two
// tree layouts and the wavefront buffers.  Everything here is POD so it can cross the C ABI
// and be copied to the device verbatim.
#pragma once
#include <stdint.h>

#ifdef __CUDACC__
#define C2G_HD __host__ __device__ __forceinline__
#else
#define C2G_HD inline
#endif

namespace c2g {

// ---- constants shared with the reference ------------------------------------------------
constexpr float kEpsTri = 1e-5f;          // Core/Utils.h:7 (EPS): triangle u+v slack, shadow tMax = 1 - EPS
constexpr float kSpawnEps = 1e-4f;        // Core/SurfaceInteraction.cpp:6 (EPS): spawn offset along N
constexpr float kOneMinusEps = 0x1.fffffep-1f;  // Core/Utils.h:10
constexpr int kHaltonDims = 100;          // dims with permutation tables (HaltonSampler.cpp:210)
constexpr int kMaxResolution = 128;       // HaltonSampler.cpp:8
constexpr int kPermTotal = 24133;         // sum of the first 100 primes (table entries)

// BxDF flags (BSDFs/BSDF.h:4-11)
enum : int {
    BXDF_REFLECTION = 1, BXDF_TRANSMISSION = 2, BXDF_GLOSSY = 4, BXDF_SPECULAR = 8, BXDF_DIFFUSE = 16,
    BXDF_ALL = 0x1F,
};

enum ShapeType : int { SHAPE_TRI = 0, SHAPE_SPHERE = 1, SHAPE_DISK = 2 };

// Materials (Materials/Material.cpp:22-126).  Each hit gets one BxDF except Plastic (two).
enum MatType : int {
    MAT_NONE = -1,        // no "Material" key: pass-through (PathTracingIntegrator.cpp:64-68)
    MAT_DIFFUSE = 0,      // Lambertain
    MAT_MIRROR = 1,       // SpecularReflection + FresnelNoOp
    MAT_GLASS_ROUGH = 2,  // MicrofacetBlend(GGX) + FresnelDielectric
    MAT_GLASS_SMOOTH = 3, // SpecularFresnel + FresnelDielectric
    MAT_MICRO_GGX = 4,    // MicrofacetReflection(GGX) + FresnelSchlick(0.99)
    MAT_MICRO_BECKMANN = 5,
    MAT_PLASTIC_GGX = 6,  // Lambertain(kd) + MicrofacetReflection(ks) (Plastic.cpp)
    MAT_PLASTIC_BECKMANN = 7,
    MAT_ORENNAYAR = 8,    // OrenNayarReflection (Reflections.cpp); A, B precomputed in ax, ay, sigma in ior
    MAT_BLINNPHONG = 9,   // BlinnPhongReflection (BlinnPhongReflection.cpp); exponent K in ior
};

struct alignas(16) Material {
    int type;
    float ior;
    float ax, ay;          // roughness used directly as alpha (MicrofacetMaterial.cpp:18-42)
    float color[4];        // Color / Kd
    float ks[4];           // Ks (Plastic)
    int tex;               // Kd texture (UVTexture) index, -1: the constant color
    int pad[3];
};

enum LightType : int { LIGHT_AREA = 0, LIGHT_POINT = 1 };

struct alignas(16) Light {
    int type;
    int obj;               // scene object carrying the light (area lights), -1 for point lights
    int shape_type;
    int shape_idx;
    float Le[4];           // emitted radiance (area) / Flux (point)
    float pos[4];          // point light position
    float area;            // Shape::SurfaceArea()
    float flux_zero;       // 1 when Flux() == 0 (skipped by UniformSampleAllLights)
    float pad[2];
};

// Sphere / disk with their rotation (Sphere.cpp:17-28, Disk.cpp:19-29).
struct alignas(16) Quadric {
    float c[4];            // center xyz, radius
    float w2l[12];         // world2Local, column-major mat3 in 3 float4 (w unused)
    float l2w[12];         // local2World
};

// Per-object info, scene order (Scene::_sceneObjects).
struct alignas(16) ObjInfo {
    int type;              // ShapeType
    int shape;             // index into tris / quadrics
    int material;          // index or -1
    int light;             // area light index or -1
};

// Triangle shading data, per triangle (scene triangle index).
struct alignas(16) TriShade {
    float n0[4];           // n0.xyz, dpdu.x
    float n1[4];           // n1.xyz, dpdu.y
    float n2[4];           // n2.xyz, dpdu.z   (dpdu == 0 -> fallback tangent, Triangle.cpp:57-72)
};

// Reference-tree node (BVH.cpp:18-33 field meaning, 32 B): a = ch0 or leaf start,
// b = ch1 | axis << 28, or count | 3 << 28 for a leaf.
struct alignas(16) RefNode {
    float mn[3]; int a;
    float mx[3]; int b;
};

// Compact binary node: both children's boxes in the parent (64 B).  Child index c:
// c >= 0 internal node index; c < 0 leaf with first prim ~c>>4... see kernels for encoding.
struct alignas(16) WideNode {
    float lo0[3]; int c0;
    float hi0[3]; int n0;   // n0 > 0: leaf prim count of child 0; 0: internal
    float lo1[3]; int c1;
    float hi1[3]; int n1;
};

// Four-wide SAH node (128 B): the boxes of up to four children as SoA lanes, then the children:
// >= 0 an inner Node4 index, < 0 a leaf -1 - (first prim << 3 | count), INT_MIN an empty slot
// (its box is empty and never hit).  Collapsed from the binary SAH tree: same boxes, same leaves.
struct alignas(16) Node4 {
    float lox[4], hix[4], loy[4], hiy[4], loz[4], hiz[4];
    int child[4];
    int pad[4];
};

// Prim record in traversal order (48 B).  Triangles: v0, v1, v2 (w of v0 = obj | type << 30).
// Spheres/disks: v0 = (unused, obj | type << 30), v1 = box min (w = quadric index), v2 = box max.
struct alignas(16) Prim {
    float v0[3]; int objtype;
    float v1[3]; int aux;
    float v2[3]; int pad;
};

C2G_HD int prim_obj(int objtype) { return objtype & 0x3fffffff; }
C2G_HD int prim_type(int objtype) { return (objtype >> 30) & 3; }

struct alignas(16) Camera {
    float eye[4];
    float look[4];         // normalized
    float up[4];           // orthogonalised, normalized (PerspCamera.cpp:8-12)
    float right[4];        // normalize(cross(look, up))
    float W, H, zNear, pad;
};

// Halton sampler constants (HaltonSampler.cpp:204-229).
struct HaltonParams {
    int baseScales[2];
    int baseExponents[2];
    int sampleStride;
    int multInverse[2];
    int pad;
};

}  // namespace c2g
