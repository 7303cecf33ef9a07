// Host-side scene: the reference's JSON/OBJ inputs parsed and flattened into the POD arrays of
// c2g_types.h.  Mirrors RayTracer's construction (src/Core/RayTracer.cpp:11-22):
// ConfigLoader::LoadConfigInfo, Scene::CreateScene, Camera::CreateCamera, Integrator and
// Sampler factories.
#pragma once
#include <memory>
#include <stdexcept>
#include <map>
#include <string>
#include <vector>

#include "../c2g_types.h"
#include "fmath.h"
#include "json.h"

namespace c2g {

struct SceneError : std::runtime_error {
    int code;
    SceneError(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

struct HostConfig {
    int width = 0, height = 0, spp = 0, threads = 1;
    std::string accel;            // "BVH" | "Brute" | "KDTree"
    std::string integrator;       // "PathTracer" | "DirectLight" | "GuidedPathTracer"
    int depth = 0;
    std::string sampler;          // "Halton" | "Default" | "Stratified"
    long long seed = 0;
};

struct HostScene {
    HostConfig cfg;
    Camera cam{};
    std::vector<ObjInfo> objs;         // scene order
    std::vector<fm::V3> tri_pos;       // 3 per triangle
    std::vector<TriShade> tri_shade;   // per triangle
    std::vector<Quadric> quads;        // spheres and disks
    std::vector<float> quad_box;       // 6 per quadric (GetBoundingBox)
    std::vector<Material> mats;
    std::vector<Light> lights;         // Scene::_lights order
    std::vector<float> tri_uv;         // 6 per triangle: texture coordinates of its vertices
    std::vector<float> texels;         // RGB float texels of every texture (ImageTexels)
    std::vector<int> tex_info;         // 4 per texture: width, height, first texel (float index), 0
    std::map<std::string, int> tex_names;
    int sky[6] = {-1, -1, -1, -1, -1, -1};  // skybox faces: +x, -x, +y, -y, +z, -z

    size_t num_objects() const { return objs.size(); }
    // Object bounding box (IIntersectable::GetBoundingBox) as min xyz, max xyz.
    void object_box(int obj, float out[6]) const;
};

// Decoded 8-bit RGB images the caller registered by path (c2g_register_image); scene texture and
// skybox paths are looked up here before the file system.
struct Image {
    int width = 0, height = 0;
    std::vector<unsigned char> rgb;
};
using ImageRegistry = std::map<std::string, Image>;

// Parse config + scene JSON (already loaded as text).  Throws SceneError / JsonError.
void load_scene(HostScene& s, const std::string& config_text, const std::string& scene_text,
                const ImageRegistry* images = nullptr);
std::string read_text_file(const std::string& path);  // throws SceneError(C2G_ERR_IO)

// Halton sampler tables (HaltonSampler.cpp:164-229).
HaltonParams halton_params(int width, int height);
// 100 permutation tables from one default-seeded std::mt19937 and std::shuffle, concatenated in
// prime order (24133 entries), plus each table's start offset.
void halton_perm_tables(std::vector<uint16_t>& perm, std::vector<int>& offset);
// Radical-inverse primes of dims 0..99.
const int* halton_primes();

}  // namespace c2g
