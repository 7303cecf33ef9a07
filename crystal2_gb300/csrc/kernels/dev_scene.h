// Device scene view passed by value to the kernels, and the shading bucket ids.  Host-safe: the
// C++ host code holds these structures too.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../c2g_types.h"

namespace c2g {

// ---- device scene view -------------------------------------------------------------------
struct DevScene {
    const ObjInfo* objs;
    const TriShade* tri_shade;
    const float4* tri_pos;        // 3 float4 per scene triangle (v0, v1, v2)
    const Quadric* quads;
    const Material* mats;
    const Light* lights;
    int n_lights;
    int n_objs;
    const Prim* prims;            // traversal order
    int n_prims;
    int tree;                     // C2G_TREE_*
    const RefNode* ref_nodes;     // tree == REF: nodes 1..n, root 1
    const WideNode* wide_nodes;   // tree == SAH: root 0
    const Node4* nodes4;          // tree == SAH: the same tree four-wide, root 0
    int sah_width;                // SAH traversal variant: 2 (WideNode) or 4 (Node4)
    int anyhit_clip;              // 1: BVH semantics (object-box-clipped shadow interval)
    int closest_box;              // 1: per-object box prefilter on closest hits
    Camera cam;
    HaltonParams hp;
    const uint16_t* perm;         // 100 concatenated permutation tables
    const int* perm_off;          // table offsets
    uint64_t seed;
    int sampler;                  // SAMPLER_HALTON / SAMPLER_DEFAULT / SAMPLER_STRATIFIED
    int spp;                      // SamplesPerPixel (the stratified sampler's strata per dimension)
    int strata_side;              // sqrt(spp): the 2D strata grid of the stratified sampler
    int* err;                     // device error word (C2G_DEVERR_*)
    const float2* tri_uv;         // 3 texture coordinates per scene triangle
    const float* texels;          // RGB float texels of every texture, back to back
    const int4* tex_info;         // per texture: width, height, first texel (float index), 0
    int sky[6];                   // cubemap skybox faces (+x, -x, +y, -y, +z, -z), -1: none
};

enum : int { SAMPLER_HALTON = 0, SAMPLER_DEFAULT = 1, SAMPLER_STRATIFIED = 2 };

// Shading buckets: 0..9 = MatType of the hit's material, 10 = no material, 11 = miss.
constexpr int kBuckets = 12;
constexpr int kBucketNone = 10;
constexpr int kBucketMiss = 11;

enum : int {
    DEVERR_STACK = 1,             // traversal stack overflow
    DEVERR_QUEUE = 2,             // queue capacity exceeded
    DEVERR_WAIT = 4,              // a bounded wait on a tensor-core completion barrier ran out
};

}  // namespace c2g
