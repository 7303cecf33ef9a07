#include "scene.h"
#include <cstdlib>
#include <cmath>
#include <map>
#include <cctype>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <limits>
#include <random>
#include <sstream>

#include "../../../include/c2g.h"

namespace c2g {

using fm::V3;
using fm::V4;

std::string read_text_file(const std::string& path) {
    std::ifstream f(path, std::ios::binary);
    if (!f) throw SceneError(C2G_ERR_IO, "cannot open file " + path);
    std::stringstream ss;
    ss << f.rdbuf();
    return ss.str();
}

namespace {

V3 parse_vec3(const Json& n) {
    // loader::parse_vec3 (JsonLoader.h:12-18): three GetFloat() narrowed to float
    return V3((float)n.at(0).as_float(), (float)n.at(1).as_float(), (float)n.at(2).as_float());
}
void parse_vec2(const Json& n, float& x, float& y) {
    x = (float)n.at(0).as_float();
    y = (float)n.at(1).as_float();
}

struct ObjVertex {
    V3 pos, nrm;
    float uv[2] = {0, 0};
};

// Wavefront OBJ as ObjLoader::process reads it (ObjLoader.cpp:90-149): v / vt / vn lines and
// triangular faces "a", "a/b", "a//c", "a/b/c"; every face gets three fresh vertices.
void load_obj(const std::string& path, std::vector<ObjVertex>& verts) {
    FILE* f = std::fopen(path.c_str(), "r");
    if (!f) throw SceneError(C2G_ERR_IO, "cannot open OBJ file " + path);
    std::vector<V3> P, N;
    std::vector<std::pair<float, float>> T;
    std::vector<char> line(1 << 17);
    int lineno = 0;
    auto read_int = [](const char* s, int& idx, int& num) {
        num = 0;
        while (s[idx] == ' ') idx++;
        bool neg = false;
        if (s[idx] == '-') { neg = true; idx++; } else if (s[idx] == '+') idx++;
        while (s[idx] >= '0' && s[idx] <= '9') { num = num * 10 + (s[idx] - '0'); idx++; }
        if (neg) num = -num;
    };
    while (std::fgets(line.data(), (int)line.size(), f)) {
        lineno++;
        char tok[16] = {0};
        int consumed = 0;
        if (std::sscanf(line.data(), "%15s%n", tok, &consumed) != 1) continue;
        const char* rest = line.data() + consumed;
        if (!std::strcmp(tok, "v")) {
            double x, y, z;
            if (std::sscanf(rest, "%lf%lf%lf", &x, &y, &z) != 3) { std::fclose(f); throw SceneError(C2G_ERR_PARSE, path + ": bad v line " + std::to_string(lineno)); }
            P.push_back(V3((float)x, (float)y, (float)z));
        } else if (!std::strcmp(tok, "vn")) {
            double x, y, z;
            if (std::sscanf(rest, "%lf%lf%lf", &x, &y, &z) != 3) { std::fclose(f); throw SceneError(C2G_ERR_PARSE, path + ": bad vn line " + std::to_string(lineno)); }
            N.push_back(V3((float)x, (float)y, (float)z));
        } else if (!std::strcmp(tok, "vt")) {
            double x, y;
            if (std::sscanf(rest, "%lf%lf", &x, &y) != 2) { std::fclose(f); throw SceneError(C2G_ERR_PARSE, path + ": bad vt line " + std::to_string(lineno)); }
            T.push_back({(float)x, (float)y});
        } else if (!std::strcmp(tok, "f")) {
            int vd[3] = {0, 0, 0}, vt[3] = {0, 0, 0}, vn[3] = {0, 0, 0};
            int count = 0;
            const char* p = rest;
            char fv[128];
            int used = 0;
            while (std::sscanf(p, "%127s%n", fv, &used) == 1) {
                if (count >= 3) { std::fclose(f); throw SceneError(C2G_ERR_PARSE, path + ": non-triangular face at line " + std::to_string(lineno)); }
                int id = 0;
                read_int(fv, id, vd[count]);
                id++;
                if (id <= (int)std::strlen(fv)) read_int(fv, id, vt[count]);
                id++;
                if (id <= (int)std::strlen(fv)) read_int(fv, id, vn[count]);
                count++;
                p += used;
            }
            if (count != 3) { std::fclose(f); throw SceneError(C2G_ERR_PARSE, path + ": face with fewer than 3 vertices at line " + std::to_string(lineno)); }
            for (int k = 0; k < 3; k++) {
                ObjVertex v;
                if (vd[k] < 1 || vd[k] > (int)P.size()) { std::fclose(f); throw SceneError(C2G_ERR_PARSE, path + ": vertex index out of range at line " + std::to_string(lineno)); }
                v.pos = P[vd[k] - 1];
                if (vn[0] != 0) {
                    if (vn[k] < 1 || vn[k] > (int)N.size()) { std::fclose(f); throw SceneError(C2G_ERR_PARSE, path + ": normal index out of range at line " + std::to_string(lineno)); }
                    v.nrm = N[vn[k] - 1];
                }
                if (vt[0] != 0) {
                    if (vt[k] < 1 || vt[k] > (int)T.size()) { std::fclose(f); throw SceneError(C2G_ERR_PARSE, path + ": uv index out of range at line " + std::to_string(lineno)); }
                    v.uv[0] = T[vt[k] - 1].first;
                    v.uv[1] = T[vt[k] - 1].second;
                }
                verts.push_back(v);
            }
        }
    }
    std::fclose(f);
}

// Sphere / Disk rotation (Sphere.cpp:17-28, Disk.cpp:19-29): X then Y then Z, degrees.
void quadric_rotation(V3 rot, fm::M3& l2w, fm::M3& w2l) {
    fm::M4 m = fm::identity4();
    m = fm::rotate(m, rot.x / 180.f * fm::kPi, V3(1, 0, 0));
    m = fm::rotate(m, rot.y / 180.f * fm::kPi, V3(0, 1, 0));
    m = fm::rotate(m, rot.z / 180.f * fm::kPi, V3(0, 0, 1));
    l2w = fm::mat3_of(m);
    w2l = fm::transpose(l2w);
}

void store_m3(float* dst, const fm::M3& m) {
    for (int c = 0; c < 3; c++) {
        dst[4 * c] = m[c].x; dst[4 * c + 1] = m[c].y; dst[4 * c + 2] = m[c].z; dst[4 * c + 3] = 0.f;
    }
}

// An 8-bit RGB image: a registered decode, else a binary PPM (P6, maxval 255) file.  stb_image, which
// the reference uses (Texel.cpp:4-13), detects the format from the content; this loader reads PPM
// content under any file name and leaves other formats to the caller's registry.
Image load_image(const std::string& path, const ImageRegistry* reg) {
    if (reg) {
        auto it = reg->find(path);
        if (it != reg->end()) return it->second;
    }
    std::string data = read_text_file(path);
    Image im;
    size_t pos = 0;
    auto token = [&]() -> std::string {
        while (pos < data.size()) {
            char ch = data[pos];
            if (ch == '#') { while (pos < data.size() && data[pos] != '\n') pos++; }
            else if (std::isspace((unsigned char)ch)) pos++;
            else break;
        }
        size_t b = pos;
        while (pos < data.size() && !std::isspace((unsigned char)data[pos])) pos++;
        return data.substr(b, pos - b);
    };
    if (data.size() < 2 || data[0] != 'P' || data[1] != '6')
        throw SceneError(C2G_ERR_UNSUPPORTED, "Failed to load image: " + path +
                                                 " (binary PPM only; register other formats decoded with c2g_register_image)");
    pos = 2;
    im.width = std::atoi(token().c_str());
    im.height = std::atoi(token().c_str());
    int maxval = std::atoi(token().c_str());
    pos++;  // the single whitespace byte before the raster
    size_t need = (size_t)im.width * im.height * 3;
    if (im.width <= 0 || im.height <= 0 || maxval != 255 || data.size() < pos + need)
        throw SceneError(C2G_ERR_PARSE, "Failed to load image: " + path);
    im.rgb.assign(data.begin() + pos, data.begin() + pos + need);
    return im;
}

struct Loader {
    HostScene& s;
    const ImageRegistry* images = nullptr;
    // OBJ files parsed so far in this load, by path: a scene that instances one mesh many times
    // (the reference reads the file again for every object) parses it once
    std::map<std::string, std::vector<ObjVertex>> objs_read;
    explicit Loader(HostScene& sc, const ImageRegistry* reg = nullptr) : s(sc), images(reg) {}

    const std::vector<ObjVertex>& obj_vertices(const std::string& path) {
        auto it = objs_read.find(path);
        if (it != objs_read.end()) return it->second;
        std::vector<ObjVertex> v;
        load_obj(path, v);
        return objs_read.emplace(path, std::move(v)).first->second;
    }

    // ImageTexels::CreateImageTexels (Texel.cpp:4-38): texel = (byte / 255)^2.2 in float.
    int add_texture(const std::string& path) {
        Image im = load_image(path, images);
        int idx = (int)s.tex_info.size() / 4;
        s.tex_info.push_back(im.width);
        s.tex_info.push_back(im.height);
        s.tex_info.push_back((int)s.texels.size());
        s.tex_info.push_back(0);
        for (size_t i = 0; i < im.rgb.size(); i++) s.texels.push_back(std::pow((float)im.rgb[i] / 255.f, 2.2f));
        return idx;
    }
    int texture_by_name(const std::string& name) {  // Scene::GetTextureByName (Scene.cpp:69-77)
        auto it = s.tex_names.find(name);
        if (it == s.tex_names.end()) throw SceneError(C2G_ERR_INVALID, "Texture name doesn't exist");
        return it->second;
    }

    int add_material(const Json& n) {
        Material m{};
        const std::string& type = n.at("Type").as_string();
        auto color = [&](const char* key) {
            V3 c = parse_vec3(n.at(key));
            m.color[0] = c.x; m.color[1] = c.y; m.color[2] = c.z; m.color[3] = 0.f;
        };
        m.tex = -1;
        if (type == "Diffuse") {
            m.type = MAT_DIFFUSE;
            if (n.has("Kd")) m.tex = texture_by_name(n.at("Kd").as_string());  // UVTexture Kd
            else color("Color");
        } else if (type == "Mirror") {
            m.type = MAT_MIRROR;
            color("Color");
        } else if (type == "Glass") {
            color("Color");
            parse_vec2(n.at("Roughness"), m.ax, m.ay);
            m.ior = (float)n.at("IOR").as_float();
            m.type = (m.ax == 0.f && m.ay == 0.f) ? MAT_GLASS_SMOOTH : MAT_GLASS_ROUGH;  // Glass.cpp:23-31
        } else if (type == "Micro") {
            color("Color");
            parse_vec2(n.at("Roughness"), m.ax, m.ay);
            m.ior = (float)n.at("IOR").as_float();
            const std::string& ndf = n.at("NDF").as_string();
            if (ndf == "GGX") m.type = MAT_MICRO_GGX;
            else if (ndf == "Beckmann") m.type = MAT_MICRO_BECKMANN;
            else throw SceneError(C2G_ERR_INVALID, "Cannot find NDF Type: " + ndf);
        } else if (type == "Plastic") {
            color("Kd");
            V3 ks = parse_vec3(n.at("Ks"));
            m.ks[0] = ks.x; m.ks[1] = ks.y; m.ks[2] = ks.z;
            parse_vec2(n.at("Roughness"), m.ax, m.ay);
            const std::string& ndf = n.at("NDF").as_string();
            if (ndf == "GGX") m.type = MAT_PLASTIC_GGX;
            else if (ndf == "Beckmann") m.type = MAT_PLASTIC_BECKMANN;
            else throw SceneError(C2G_ERR_INVALID, "Cannot find NDF Type: " + ndf);
        } else if (type == "Phong") {
            // PhongMaterial -> BlinnPhongReflection(color, K) (Material.cpp:86-99, PhongMaterial.cpp:11-19)
            m.type = MAT_BLINNPHONG;
            if (n.has("Kd")) m.tex = texture_by_name(n.at("Kd").as_string());
            else color("Color");
            m.ior = (float)n.at("K").as_int();
        } else if (type == "OrenNayar") {
            // OrenNayarMaterial -> OrenNayarReflection(color, sigma) (Material.cpp:100-121); the
            // constructor's A and B (Reflections.cpp:20-26) in float, as the reference computes them
            if (n.has("Kd")) throw SceneError(C2G_ERR_UNSUPPORTED, "Not implemented");
            m.type = MAT_ORENNAYAR;
            color("Color");
            const float sigma = (float)n.at("Sigma").as_float();
            const float s2 = sigma * sigma;
            m.ior = sigma;
            m.ax = 1.f - s2 / (2 * (s2 + 0.33f));
            m.ay = (0.45f * s2) / (s2 + 0.09f);
        } else {
            throw SceneError(C2G_ERR_INVALID, "Invalid material name");
        }
        s.mats.push_back(m);
        return (int)s.mats.size() - 1;
    }

    // Shapes of one Geometry object (Scene.cpp:145-179), as (type, shape index) pairs.
    std::vector<std::pair<int, int>> add_shapes(const Json& n) {
        std::vector<std::pair<int, int>> out;
        const std::string& type = n.at("Type").as_string();
        if (type == "Sphere" || type == "Disk") {
            V3 pos = parse_vec3(n.at("Position"));
            float r = (float)n.at("Radius").as_float();
            V3 rot(0, 0, 0);
            if (n.has("Rotation")) rot = parse_vec3(n.at("Rotation"));
            fm::M3 l2w, w2l;
            quadric_rotation(rot, l2w, w2l);
            Quadric q{};
            q.c[0] = pos.x; q.c[1] = pos.y; q.c[2] = pos.z; q.c[3] = r;
            store_m3(q.w2l, w2l);
            store_m3(q.l2w, l2w);
            float box[6];
            if (type == "Sphere") {
                // Sphere::GetBoundingBox (Sphere.cpp:30-32): pos -/+ radius
                V3 lo = pos - r, hi = pos + r;
                box[0] = lo.x; box[1] = lo.y; box[2] = lo.z; box[3] = hi.x; box[4] = hi.y; box[5] = hi.z;
            } else {
                // Disk::GetBoundingBox (Disk.cpp:34-43)
                V3 wn = fm::mul(l2w, V3(0, 1, 0));
                float sinT = std::sqrt(1.f - wn.y * wn.y);
                V3 off(r, r * sinT, r);
                V3 lo = pos - off, hi = pos + off;
                box[0] = lo.x; box[1] = lo.y; box[2] = lo.z; box[3] = hi.x; box[4] = hi.y; box[5] = hi.z;
            }
            s.quads.push_back(q);
            s.quad_box.insert(s.quad_box.end(), box, box + 6);
            out.push_back({type == "Sphere" ? SHAPE_SPHERE : SHAPE_DISK, (int)s.quads.size() - 1});
        } else if (type == "TriangleMesh") {
            std::vector<ObjVertex> verts = obj_vertices(n.at("ObjFile").as_string());
            // TriangleMesh::CreateTriangleMesh (TriangleMesh.cpp:9-27)
            V3 pos = parse_vec3(n.at("Translation"));
            V3 scl = parse_vec3(n.at("Scale"));
            V3 rot = parse_vec3(n.at("Rotation")) * 0.01745329251994329576923690768489f;
            fm::M4 M = fm::identity4();
            M = fm::translate(M, pos);
            M = fm::rotate(M, rot.x, V3(1, 0, 0));
            M = fm::rotate(M, rot.y, V3(0, 1, 0));
            M = fm::rotate(M, rot.z, V3(0, 0, 1));
            M = fm::scale(M, scl);
            fm::M4 NT = fm::transpose(fm::inverse(M));
            for (auto& v : verts) {  // TriangleMesh.cpp:29-43
                V4 p = fm::mul(M, V4(v.pos.x, v.pos.y, v.pos.z, 1.0f));
                v.pos = V3(p.x, p.y, p.z);
                V4 q = fm::mul(NT, V4(v.nrm.x, v.nrm.y, v.nrm.z, 0.0f));
                v.nrm = fm::normalize(V3(q.x, q.y, q.z));
            }
            for (size_t f = 0; f + 2 < verts.size(); f += 3) {
                const ObjVertex& a = verts[f];
                const ObjVertex& b = verts[f + 1];
                const ObjVertex& c = verts[f + 2];
                s.tri_pos.push_back(a.pos);
                s.tri_pos.push_back(b.pos);
                s.tri_pos.push_back(c.pos);
                // Triangle::calculateDerivative (Triangle.cpp:100-135): tangent from UVs
                fm::M2 A;
                A.m[0][0] = a.uv[0] - c.uv[0]; A.m[0][1] = a.uv[1] - c.uv[1];
                A.m[1][0] = b.uv[0] - c.uv[0]; A.m[1][1] = b.uv[1] - c.uv[1];
                A = fm::inverse(A);
                V3 dpdu(0, 0, 0);
                bool bad = std::isinf(A.m[0][0]) || std::isinf(A.m[0][1]) || std::isnan(A.m[0][0]) ||
                           std::isnan(A.m[0][1]) || std::isnan(A.m[1][0]) || std::isnan(A.m[1][1]);
                if (!bad) {
                    V3 e0 = a.pos - c.pos, e1 = b.pos - c.pos;
                    float r00 = A.m[0][0] * e0.x + A.m[1][0] * e1.x;
                    float r10 = A.m[0][0] * e0.y + A.m[1][0] * e1.y;
                    float r20 = A.m[0][0] * e0.z + A.m[1][0] * e1.z;
                    dpdu = fm::normalize(V3(r00, r10, r20));
                }
                TriShade ts{};
                ts.n0[0] = a.nrm.x; ts.n0[1] = a.nrm.y; ts.n0[2] = a.nrm.z; ts.n0[3] = dpdu.x;
                ts.n1[0] = b.nrm.x; ts.n1[1] = b.nrm.y; ts.n1[2] = b.nrm.z; ts.n1[3] = dpdu.y;
                ts.n2[0] = c.nrm.x; ts.n2[1] = c.nrm.y; ts.n2[2] = c.nrm.z; ts.n2[3] = dpdu.z;
                s.tri_shade.push_back(ts);
                for (const ObjVertex* v : {&a, &b, &c}) { s.tri_uv.push_back(v->uv[0]); s.tri_uv.push_back(v->uv[1]); }
                out.push_back({SHAPE_TRI, (int)s.tri_shade.size() - 1});
            }
        } else {
            throw SceneError(C2G_ERR_INVALID, "Invalid Shape Type!");
        }
        return out;
    }

    float shape_area(int type, int idx) const {
        if (type == SHAPE_TRI) {
            V3 a = s.tri_pos[3 * idx], b = s.tri_pos[3 * idx + 1], c = s.tri_pos[3 * idx + 2];
            return fm::length(fm::cross(b - a, c - a)) / 2.f;  // Triangle.cpp:95-98
        }
        float r = s.quads[idx].c[3];
        if (type == SHAPE_SPHERE) return 4 * fm::kPi * r * r;  // Sphere.cpp:96-99
        return fm::kPi * r * r;                                // Disk.cpp:80-83
    }

    int add_area_light(const Json& n, int type, int idx, int obj) {
        const std::string& lt = n.at("Type").as_string();
        if (lt != "Diffused") throw SceneError(C2G_ERR_INVALID, "Invalid area light name");
        V3 le = parse_vec3(n.at("Lemit"));
        (void)n.at("Samples").as_int();
        Light L{};
        L.type = LIGHT_AREA;
        L.obj = obj;
        L.shape_type = type;
        L.shape_idx = idx;
        L.Le[0] = le.x; L.Le[1] = le.y; L.Le[2] = le.z;
        L.area = shape_area(type, idx);
        // Flux() = Le * pi * area (DiffusedAreaLight.cpp:41-44); zero flux skips the light
        V3 flux = le * fm::kPi * L.area;
        L.flux_zero = (flux.x == 0.f && flux.y == 0.f && flux.z == 0.f) ? 1.f : 0.f;
        s.lights.push_back(L);
        return (int)s.lights.size() - 1;
    }

    void load_objects(const Json& arr) {
        if (arr.kind != Json::ARRAY) throw SceneError(C2G_ERR_INVALID, "Objects must be an array");
        for (size_t i = 0; i < arr.size(); i++) {
            const Json& node = arr.at(i);
            const std::string& type = node.at("Type").as_string();
            if (type == "Geometry") {
                auto shapes = add_shapes(node.at("Shape"));
                int mat = -1;
                if (node.has("Material")) mat = add_material(node.at("Material"));
                bool has_light = node.has("AreaLight");
                for (auto& sh : shapes) {
                    int obj = (int)s.objs.size();
                    int light = has_light ? add_area_light(node.at("AreaLight"), sh.first, sh.second, obj) : -1;
                    s.objs.push_back(ObjInfo{sh.first, sh.second, mat, light});
                }
            } else if (type == "Light") {
                const std::string& lt = node.at("LightType").as_string();
                if (lt != "Point") throw SceneError(C2G_ERR_INVALID, "Invalid light name");
                V3 pos = parse_vec3(node.at("Position"));
                V3 flux = parse_vec3(node.at("Flux"));
                Light L{};
                L.type = LIGHT_POINT;
                L.obj = -1;
                L.shape_type = -1;
                L.shape_idx = -1;
                L.Le[0] = flux.x; L.Le[1] = flux.y; L.Le[2] = flux.z;
                L.pos[0] = pos.x; L.pos[1] = pos.y; L.pos[2] = pos.z;
                L.flux_zero = (flux.x == 0.f && flux.y == 0.f && flux.z == 0.f) ? 1.f : 0.f;
                s.lights.push_back(L);
            } else {
                throw SceneError(C2G_ERR_INVALID, "Invalid Object Type!");
            }
        }
    }
};

}  // namespace

void HostScene::object_box(int obj, float out[6]) const {
    const ObjInfo& o = objs[obj];
    if (o.type == SHAPE_TRI) {
        // Triangle bbox: per-axis min/max of the three vertices (Triangle.cpp:136-147)
        const V3& a = tri_pos[3 * o.shape];
        V3 mn = a, mx = a;
        for (int k = 1; k < 3; k++) {
            const V3& v = tri_pos[3 * o.shape + k];
            mn.x = std::min(mn.x, v.x); mn.y = std::min(mn.y, v.y); mn.z = std::min(mn.z, v.z);
            mx.x = std::max(mx.x, v.x); mx.y = std::max(mx.y, v.y); mx.z = std::max(mx.z, v.z);
        }
        out[0] = mn.x; out[1] = mn.y; out[2] = mn.z; out[3] = mx.x; out[4] = mx.y; out[5] = mx.z;
    } else {
        for (int k = 0; k < 6; k++) out[k] = quad_box[6 * o.shape + k];
    }
}

void load_scene(HostScene& s, const std::string& config_text, const std::string& scene_text, const ImageRegistry* images) {
    s = HostScene();
    auto cfgp = Json::parse(config_text);
    auto scnp = Json::parse(scene_text);
    const Json& cfg = *cfgp;
    const Json& scn = *scnp;
    // ConfigLoader::LoadConfigInfo (ConfigLoader.cpp:9-18)
    s.cfg.width = (int)cfg.at("Width").as_int();
    s.cfg.height = (int)cfg.at("Height").as_int();
    s.cfg.spp = (int)cfg.at("SamplesPerPixel").as_int();
    s.cfg.accel = cfg.at("Acceleration").as_string();
    s.cfg.threads = (int)cfg.at("Threads").as_int();
    if (s.cfg.width <= 0 || s.cfg.height <= 0 || s.cfg.spp <= 0)
        throw SceneError(C2G_ERR_INVALID, "Width, Height and SamplesPerPixel must be positive");
    if (s.cfg.accel != "BVH" && s.cfg.accel != "Brute" && s.cfg.accel != "KDTree")
        throw SceneError(C2G_ERR_INVALID, "No such accelerator!");
    // Integrator::LoadIntegrator / Sampler::LoadSampler (Integrator.cpp:14-47, Sampler.cpp:10-53)
    const Json& integ = cfg.at("Integrator");
    s.cfg.integrator = integ.at("Type").as_string();
    const Json& smp = integ.at("Sampler");
    s.cfg.sampler = smp.at("Type").as_string();
    s.cfg.seed = smp.at("Seed").as_int();
    // "GPUPathTracer" is the key under which a reference build registers this library's path
    // tracer in its own factory; here it selects the same integrator as "PathTracer".
    if (s.cfg.integrator != "PathTracer" && s.cfg.integrator != "DirectLight" && s.cfg.integrator != "GuidedPathTracer" &&
        s.cfg.integrator != "GPUPathTracer")
        throw SceneError(C2G_ERR_INVALID, "Invalid Integrator Type!");
    s.cfg.depth = (int)integ.at("Depth").as_int();
    if (s.cfg.sampler != "Halton" && s.cfg.sampler != "Default" && s.cfg.sampler != "Stratified")
        throw SceneError(C2G_ERR_INVALID, "Invalid Sampler Type!");
    if (s.cfg.sampler == "Stratified") {  // Sampler.cpp:21-40: a square sample count
        bool square = false;
        for (long long i = 1; i * i <= s.cfg.spp; i++) square |= i * i == s.cfg.spp;
        if (!square) throw SceneError(C2G_ERR_INVALID, "Stratified sampler should have a square number of SamplesPerPixel");
    }
    // Scene::CreateScene (Scene.cpp:23-45)
    const Json& sc = scn.at("Scene");
    Loader ld(s, images);
    // Scene::loadTextures (Scene.cpp:84-92): name -> UVTexture over the image's texels
    const Json& tex = sc.at("Textures");
    if (tex.kind != Json::OBJECT) throw SceneError(C2G_ERR_INVALID, "Textures must be an object");
    for (const auto& kv : tex.obj) s.tex_names[kv.first] = ld.add_texture(kv.second->at("Path").as_string());
    ld.load_objects(sc.at("Objects"));
    // Scene::loadSkybox (Scene.cpp:128-144): six faces <Path>/{pos,neg}{x,y,z}.jpg
    if (sc.has("Skybox") && sc.at("Skybox").kind != Json::NUL) {
        const std::string dir = sc.at("Skybox").at("Path").as_string();
        const char* face[6] = {"posx.jpg", "negx.jpg", "posy.jpg", "negy.jpg", "posz.jpg", "negz.jpg"};
        for (int k = 0; k < 6; k++) s.sky[k] = ld.add_texture(dir + "/" + face[k]);
    }
    // Camera::CreateCamera (Camera.cpp:7-22) + PerspCamera ctor (PerspCamera.cpp:3-13)
    const Json& cam = scn.at("Camera");
    if (cam.at("Type").as_string() != "Normal") throw SceneError(C2G_ERR_INVALID, "Invalid Camera Type!");
    V3 lookAt = parse_vec3(cam.at("LookAt"));
    V3 up = parse_vec3(cam.at("Up"));
    float fov = (float)(cam.at("FOV").as_float() / 180.f * fm::kPi);  // double arithmetic, then narrowed
    V3 eye = parse_vec3(cam.at("Position"));
    float aspect = (float)s.cfg.width / s.cfg.height;
    float zNear = 1.0f;
    float H = zNear * std::tan(fov / 2);
    float W = H * aspect;
    V3 look = fm::normalize(lookAt - eye);
    V3 p = fm::dot(up, look) * look;
    V3 up2 = fm::normalize(up - p);
    V3 right = fm::normalize(fm::cross(look, up));
    Camera& c = s.cam;
    c.eye[0] = eye.x; c.eye[1] = eye.y; c.eye[2] = eye.z;
    c.look[0] = look.x; c.look[1] = look.y; c.look[2] = look.z;
    c.up[0] = up2.x; c.up[1] = up2.y; c.up[2] = up2.z;
    c.right[0] = right.x; c.right[1] = right.y; c.right[2] = right.z;
    c.W = W; c.H = H; c.zNear = zNear;
    if (s.objs.empty()) throw SceneError(C2G_ERR_INVALID, "scene has no objects");
}

// ---- Halton tables ------------------------------------------------------------------------

const int* halton_primes() {
    static int primes[kHaltonDims] = {0};
    if (primes[0] == 0) {
        int n = 0;
        for (int v = 2; n < kHaltonDims; v++) {
            bool is_prime = true;
            for (int d = 2; d * d <= v; d++)
                if (v % d == 0) { is_prime = false; break; }
            if (is_prime) primes[n++] = v;
        }
    }
    return primes;
}

namespace {
void extgcd(uint64_t a, uint64_t b, uint64_t& d, uint64_t& x, uint64_t& y) {
    if (!b) { d = a; x = 1; y = 0; }
    else { extgcd(b, a % b, d, y, x); y -= x * (a / b); }
}
uint64_t mod_inverse(uint64_t A, uint64_t M) {
    uint64_t d, x, y;
    extgcd(A, M, d, x, y);
    return d == 1 ? (x + M) % M : (uint64_t)-1;
}
}  // namespace

HaltonParams halton_params(int width, int height) {
    HaltonParams hp{};
    int res[2] = {width, height};
    for (int i = 0; i < 2; i++) {
        int base = i == 0 ? 2 : 3;
        int scale = 1, exp = 0;
        while (scale < std::min(res[i], kMaxResolution)) { scale *= base; ++exp; }
        hp.baseScales[i] = scale;
        hp.baseExponents[i] = exp;
    }
    hp.sampleStride = hp.baseScales[0] * hp.baseScales[1];
    hp.multInverse[0] = (int)mod_inverse(hp.baseScales[1], hp.baseScales[0]);
    hp.multInverse[1] = (int)mod_inverse(hp.baseScales[0], hp.baseScales[1]);
    return hp;
}

void halton_perm_tables(std::vector<uint16_t>& perm, std::vector<int>& offset) {
    const int* primes = halton_primes();
    std::mt19937 mt;  // default seed, as the reference's file-static generator
    perm.clear();
    offset.clear();
    std::vector<int> t;
    for (int i = 0; i < kHaltonDims; i++) {
        t.resize(primes[i]);
        for (int j = 0; j < primes[i]; j++) t[j] = j;
        std::shuffle(t.begin(), t.end(), mt);
        offset.push_back((int)perm.size());
        for (int v : t) perm.push_back((uint16_t)v);
    }
}

}  // namespace c2g
