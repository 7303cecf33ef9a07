// c2_oracle.cpp - CPU restatement of the Crystal2 path-tracing hot path.
//
// TEST INFRASTRUCTURE ONLY.  This file is the oracle the parity tests, smoke() and the bench's
// CPU baseline compare against; no product code links or calls it.  It restates, in plain
// scalar C++ float arithmetic and in the reference's operation order, the algorithms of the
// reference renderer (paths relative to the reference project):
//   JSON numbers         deps/TREngine/deps/SJson/SJson.cpp:81-231
//   OBJ reader           src/Loaders/ObjLoader.cpp:90-149
//   scene / materials    src/Core/Scene.cpp:23-199, src/Materials/*.cpp, src/Lights/*.cpp
//   mesh transform       src/Shapes/TriangleMesh.cpp:9-43 (glm translate/rotate/scale/inverse)
//   camera               src/Cameras/PerspCamera.cpp:3-29, src/Cameras/Camera.cpp:7-22
//   Halton sampler       src/Samplers/HaltonSampler.cpp:118-291, GlobalSampler.cpp:10-69
//   BVH build/traversal  src/Accelerators/BVH.cpp:45-355, src/Core/Geometry.h:136-157
//   shapes               src/Shapes/Triangle.cpp:32-125, Sphere.cpp:39-99, Disk.cpp:34-98, Shape.cpp:4-12
//   BSDFs                src/BSDFs/BSDF.cpp:25-130, Lambertain.cpp, Microfacet.cpp, FresnelBlend.cpp,
//                        SpecularReflection.cpp, SpecularFresnel.cpp, Models/*.cpp
//   integrator           src/Integrators/PathTracingIntegrator.cpp:28-278, SamplerIntegrator.cpp:17-72
//   film                 src/Core/FrameBuffer.cpp:20-32
// Halton dims >= 100 come from the reference's shared std::mt19937 there (not reproducible);
// here they come from the same counter hash the GPU kernels use, so the two can be compared
// sample by sample.  Build: g++ -O2 -std=c++17 -ffp-contract=off -shared (oracle/build_oracle.py).
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <limits>
#include <map>
#include <memory>
#include <random>
#include <sstream>
#include <string>
#include <thread>
#include <vector>

namespace orc {

// ---------------------------------------------------------------- math (glm operation order)
struct V3 {
    float x = 0, y = 0, z = 0;
    V3() = default;
    V3(float a, float b, float c) : x(a), y(b), z(c) {}
    float operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
    float& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
};
static inline V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
static inline V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
static inline V3 operator-(V3 a) { return {-a.x, -a.y, -a.z}; }
static inline V3 operator*(V3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
static inline V3 operator*(float s, V3 a) { return {s * a.x, s * a.y, s * a.z}; }
static inline V3 operator*(V3 a, V3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
static inline V3 operator/(V3 a, float s) { return {a.x / s, a.y / s, a.z / s}; }
static inline V3 operator-(V3 a, float s) { return {a.x - s, a.y - s, a.z - s}; }
static inline V3 operator+(V3 a, float s) { return {a.x + s, a.y + s, a.z + s}; }
static inline float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline V3 cross(V3 a, V3 b) { return {a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y}; }
static inline V3 normalize(V3 v) { return v * (1.0f / std::sqrt(dot(v, v))); }
static inline float length(V3 v) { return std::sqrt(dot(v, v)); }
static inline bool zero(V3 v) { return v.x == 0.f && v.y == 0.f && v.z == 0.f; }
static inline bool bad(V3 v) { return !std::isfinite(v.x) || !std::isfinite(v.y) || !std::isfinite(v.z); }
static inline V3 clampv(V3 v) {
    return {std::min(std::max(v.x, -1.f), 1.f), std::min(std::max(v.y, -1.f), 1.f), std::min(std::max(v.z, -1.f), 1.f)};
}
constexpr float PI = 3.14159265358979323846264338327950288f;
constexpr float TWO_PI = 6.28318530717958647692528676655900576f;
constexpr float HALF_PI = 1.57079632679489661923132169163975144f;
constexpr float OME = 0x1.fffffep-1f;

struct M3 { V3 c[3]; };  // column-major
static inline V3 mul(const M3& m, V3 v) {
    return {m.c[0].x * v.x + m.c[1].x * v.y + m.c[2].x * v.z, m.c[0].y * v.x + m.c[1].y * v.y + m.c[2].y * v.z,
            m.c[0].z * v.x + m.c[1].z * v.y + m.c[2].z * v.z};
}
static inline M3 transpose(const M3& m) {
    M3 r;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) r.c[i][j] = m.c[j][i];
    return r;
}
struct V4 { float v[4]; };
struct M4 { V4 c[4]; };
static inline V4 v4add(V4 a, V4 b) { return {{a.v[0] + b.v[0], a.v[1] + b.v[1], a.v[2] + b.v[2], a.v[3] + b.v[3]}}; }
static inline V4 v4sub(V4 a, V4 b) { return {{a.v[0] - b.v[0], a.v[1] - b.v[1], a.v[2] - b.v[2], a.v[3] - b.v[3]}}; }
static inline V4 v4mul(V4 a, float s) { return {{a.v[0] * s, a.v[1] * s, a.v[2] * s, a.v[3] * s}}; }
static inline V4 v4mulv(V4 a, V4 b) { return {{a.v[0] * b.v[0], a.v[1] * b.v[1], a.v[2] * b.v[2], a.v[3] * b.v[3]}}; }
static M4 ident4() {
    M4 m{};
    for (int i = 0; i < 4; i++) m.c[i].v[i] = 1.f;
    return m;
}
static M4 translate4(const M4& m, V3 t) {
    M4 r = m;
    r.c[3] = v4add(v4add(v4add(v4mul(m.c[0], t.x), v4mul(m.c[1], t.y)), v4mul(m.c[2], t.z)), m.c[3]);
    return r;
}
static M4 rotate4(const M4& m, float a, V3 v) {
    float c = std::cos(a), s = std::sin(a);
    V3 ax = normalize(v);
    V3 t = (1.0f - c) * ax;
    float R[3][3] = {{c + t[0] * ax[0], t[0] * ax[1] + s * ax[2], t[0] * ax[2] - s * ax[1]},
                     {t[1] * ax[0] - s * ax[2], c + t[1] * ax[1], t[1] * ax[2] + s * ax[0]},
                     {t[2] * ax[0] + s * ax[1], t[2] * ax[1] - s * ax[0], c + t[2] * ax[2]}};
    M4 r;
    for (int i = 0; i < 3; i++) r.c[i] = v4add(v4add(v4mul(m.c[0], R[i][0]), v4mul(m.c[1], R[i][1])), v4mul(m.c[2], R[i][2]));
    r.c[3] = m.c[3];
    return r;
}
static M4 scale4(const M4& m, V3 s) {
    M4 r;
    r.c[0] = v4mul(m.c[0], s.x); r.c[1] = v4mul(m.c[1], s.y); r.c[2] = v4mul(m.c[2], s.z); r.c[3] = m.c[3];
    return r;
}
static V4 mul4(const M4& m, V4 v) {
    return v4add(v4add(v4mul(m.c[0], v.v[0]), v4mul(m.c[1], v.v[1])), v4add(v4mul(m.c[2], v.v[2]), v4mul(m.c[3], v.v[3])));
}
static M4 transpose4(const M4& m) {
    M4 r;
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) r.c[i].v[j] = m.c[j].v[i];
    return r;
}
static M4 inverse4(const M4& M) {  // glm compute_inverse<4,4>
    auto m = [&](int c, int r) { return M.c[c].v[r]; };
    float c00 = m(2, 2) * m(3, 3) - m(3, 2) * m(2, 3), c02 = m(1, 2) * m(3, 3) - m(3, 2) * m(1, 3), c03 = m(1, 2) * m(2, 3) - m(2, 2) * m(1, 3);
    float c04 = m(2, 1) * m(3, 3) - m(3, 1) * m(2, 3), c06 = m(1, 1) * m(3, 3) - m(3, 1) * m(1, 3), c07 = m(1, 1) * m(2, 3) - m(2, 1) * m(1, 3);
    float c08 = m(2, 1) * m(3, 2) - m(3, 1) * m(2, 2), c10 = m(1, 1) * m(3, 2) - m(3, 1) * m(1, 2), c11 = m(1, 1) * m(2, 2) - m(2, 1) * m(1, 2);
    float c12 = m(2, 0) * m(3, 3) - m(3, 0) * m(2, 3), c14 = m(1, 0) * m(3, 3) - m(3, 0) * m(1, 3), c15 = m(1, 0) * m(2, 3) - m(2, 0) * m(1, 3);
    float c16 = m(2, 0) * m(3, 2) - m(3, 0) * m(2, 2), c18 = m(1, 0) * m(3, 2) - m(3, 0) * m(1, 2), c19 = m(1, 0) * m(2, 2) - m(2, 0) * m(1, 2);
    float c20 = m(2, 0) * m(3, 1) - m(3, 0) * m(2, 1), c22 = m(1, 0) * m(3, 1) - m(3, 0) * m(1, 1), c23 = m(1, 0) * m(2, 1) - m(2, 0) * m(1, 1);
    V4 f0{{c00, c00, c02, c03}}, f1{{c04, c04, c06, c07}}, f2{{c08, c08, c10, c11}};
    V4 f3{{c12, c12, c14, c15}}, f4{{c16, c16, c18, c19}}, f5{{c20, c20, c22, c23}};
    V4 a0{{m(1, 0), m(0, 0), m(0, 0), m(0, 0)}}, a1{{m(1, 1), m(0, 1), m(0, 1), m(0, 1)}};
    V4 a2{{m(1, 2), m(0, 2), m(0, 2), m(0, 2)}}, a3{{m(1, 3), m(0, 3), m(0, 3), m(0, 3)}};
    V4 i0 = v4add(v4sub(v4mulv(a1, f0), v4mulv(a2, f1)), v4mulv(a3, f2));
    V4 i1 = v4add(v4sub(v4mulv(a0, f0), v4mulv(a2, f3)), v4mulv(a3, f4));
    V4 i2 = v4add(v4sub(v4mulv(a0, f1), v4mulv(a1, f3)), v4mulv(a3, f5));
    V4 i3 = v4add(v4sub(v4mulv(a0, f2), v4mulv(a1, f4)), v4mulv(a2, f5));
    V4 sa{{1, -1, 1, -1}}, sb{{-1, 1, -1, 1}};
    M4 inv;
    inv.c[0] = v4mulv(i0, sa); inv.c[1] = v4mulv(i1, sb); inv.c[2] = v4mulv(i2, sa); inv.c[3] = v4mulv(i3, sb);
    V4 row0{{inv.c[0].v[0], inv.c[1].v[0], inv.c[2].v[0], inv.c[3].v[0]}};
    V4 d0 = v4mulv(M.c[0], row0);
    float ood = 1.0f / ((d0.v[0] + d0.v[1]) + (d0.v[2] + d0.v[3]));
    M4 r;
    for (int i = 0; i < 4; i++) r.c[i] = v4mul(inv.c[i], ood);
    return r;
}

// ---------------------------------------------------------------- JSON (SJson number rules)
struct JNode {
    enum K { NUL, BOOL, INT, FLT, STR, ARR, OBJ } k = NUL;
    long long i = 0;
    double f = 0;
    bool b = false;
    std::string s;
    std::vector<std::shared_ptr<JNode>> a;
    std::map<std::string, std::shared_ptr<JNode>> o;
    const JNode& m(const char* key) const {
        auto it = o.find(key);
        if (it == o.end()) throw std::runtime_error(std::string("missing member ") + key);
        return *it->second;
    }
    bool has(const char* key) const { return o.count(key) != 0; }
    double F() const { return k == INT ? (double)i : f; }
    long long I() const { return k == FLT ? (long long)f : i; }
};
struct JP {
    const std::string& t;
    size_t p = 0;
    void ws() { while (p < t.size() && isspace((unsigned char)t[p])) p++; }
    std::shared_ptr<JNode> val() {
        ws();
        if (p >= t.size()) throw std::runtime_error("json: end");
        auto n = std::make_shared<JNode>();
        char c = t[p];
        if (c == '{') {
            n->k = JNode::OBJ; p++; ws();
            if (t[p] == '}') { p++; return n; }
            while (true) {
                ws(); std::string key = str(); ws();
                if (t[p] != ':') throw std::runtime_error("json: ':'");
                p++;
                auto v = val();
                n->o.insert({key, v});
                ws();
                if (t[p] == ',') { p++; continue; }
                if (t[p] == '}') { p++; return n; }
                throw std::runtime_error("json: object");
            }
        }
        if (c == '[') {
            n->k = JNode::ARR; p++; ws();
            if (t[p] == ']') { p++; return n; }
            while (true) {
                n->a.push_back(val()); ws();
                if (t[p] == ',') { p++; continue; }
                if (t[p] == ']') { p++; return n; }
                throw std::runtime_error("json: array");
            }
        }
        if (c == '"') { n->k = JNode::STR; n->s = str(); return n; }
        if (t.compare(p, 4, "true") == 0) { p += 4; n->k = JNode::BOOL; n->b = true; return n; }
        if (t.compare(p, 5, "false") == 0) { p += 5; n->k = JNode::BOOL; return n; }
        if (t.compare(p, 4, "null") == 0) { p += 4; return n; }
        bool neg = false;
        if (t[p] == '-') { neg = true; p++; }
        std::string ip, fp, ep;
        bool eneg = false;
        while (p < t.size() && isdigit((unsigned char)t[p])) ip += t[p++];
        if (p < t.size() && t[p] == '.') { p++; while (p < t.size() && isdigit((unsigned char)t[p])) fp += t[p++]; }
        if (p < t.size() && (t[p] == 'e' || t[p] == 'E')) {
            p++;
            if (t[p] == '-') { eneg = true; p++; } else if (t[p] == '+') p++;
            while (p < t.size() && isdigit((unsigned char)t[p])) ep += t[p++];
        }
        if (!ip.empty() && fp.empty() && ep.empty()) {
            long long v = 0;
            for (char d : ip) v = v * 10 + (d - '0');
            n->k = JNode::INT; n->i = neg ? -v : v;
            return n;
        }
        double v = 0;
        for (char d : ip) { v *= 10.0; v += d - '0'; }
        double tt = 10;
        for (char d : fp) { v += (d - '0') / tt; tt *= 10; }
        if (!ep.empty()) {
            long long e = 0;
            for (char d : ep) e = e * 10 + (d - '0');
            v *= std::pow(10.0, (double)(eneg ? -e : e));
        }
        n->k = JNode::FLT; n->f = neg ? -v : v;
        return n;
    }
    std::string str() {
        p++;
        std::string r;
        while (p < t.size() && t[p] != '"') {
            if (t[p] == '\\') { p++; r += t[p++]; continue; }
            r += t[p++];
        }
        p++;
        return r;
    }
};
static std::shared_ptr<JNode> parse_file(const std::string& path) {
    std::ifstream f(path);
    if (!f) throw std::runtime_error("cannot open " + path);
    std::stringstream ss;
    ss << f.rdbuf();
    std::string s = ss.str();
    JP jp{s};
    return jp.val();
}
static V3 vec3(const JNode& n) { return V3((float)n.a.at(0)->F(), (float)n.a.at(1)->F(), (float)n.a.at(2)->F()); }

// ---------------------------------------------------------------- scene
enum { TRI = 0, SPH = 1, DSK = 2 };
enum { M_DIFF, M_MIRROR, M_GLASS_R, M_GLASS_S, M_MICRO_GGX, M_MICRO_BECK, M_PLAST_GGX, M_PLAST_BECK, M_OREN, M_PHONG };
struct Mat { int type; V3 R, S; float ax = 0, ay = 0, ior = 1; int tex = -1; };
struct Tri { V3 p[3], n[3]; V3 dpdu; float uv[6]; };
struct Tex { int w, h; std::vector<V3> texels; };  // ImageTexels (Texel.cpp)
struct Quad { V3 pos; float r; M3 l2w, w2l; };
struct Obj { int type, shape, mat, light; };
struct Light { int type; int obj; int st, si; V3 Le, pos; float area; bool zero; };
struct Box { V3 mn, mx; };
struct Node { Box b; int a, c; int axis; };  // internal: a=ch0, c=ch1; leaf: a=start, c=count

struct Scene {
    int W, H, spp, depth;
    bool direct = false;  // Integrator.Type == "DirectLight"
    int sampler = 0;      // Sampler.Type: 0 Halton, 1 Default, 2 Stratified (Sampler.cpp:10-53)
    int side = 0;         // Stratified: sqrt(SamplesPerPixel)
    bool counter = false; // Default / Stratified drawn per (pixel, sample, dim) as the library does
    bool anyclip = true, closest_box = true;
    V3 eye, look, up, right;
    float CW, CH;
    std::vector<Tri> tris;
    std::vector<Quad> quads;
    std::vector<Mat> mats;
    std::vector<Obj> objs;
    std::vector<Light> lights;
    std::vector<Tex> texs;
    std::map<std::string, int> tex_names;
    int sky[6] = {-1, -1, -1, -1, -1, -1};
    std::vector<Box> boxes;
    std::vector<int> order;
    std::vector<Node> nodes;
    int tot = 0;
    // Halton
    int scales[2], exps[2], stride, minv[2];
};

static void read_obj(const std::string& path, std::vector<V3>& pos, std::vector<V3>& nrm, std::vector<float>& uv) {
    FILE* f = fopen(path.c_str(), "r");
    if (!f) throw std::runtime_error("cannot open " + path);
    std::vector<V3> P, N;
    std::vector<std::pair<float, float>> T;
    char line[8192];
    while (fgets(line, sizeof line, f)) {
        char tok[16];
        int used = 0;
        if (sscanf(line, "%15s%n", tok, &used) != 1) continue;
        const char* r = line + used;
        double x, y, z;
        if (!strcmp(tok, "v") && sscanf(r, "%lf%lf%lf", &x, &y, &z) == 3) P.push_back(V3((float)x, (float)y, (float)z));
        else if (!strcmp(tok, "vn") && sscanf(r, "%lf%lf%lf", &x, &y, &z) == 3) N.push_back(V3((float)x, (float)y, (float)z));
        else if (!strcmp(tok, "vt") && sscanf(r, "%lf%lf", &x, &y) == 2) T.push_back({(float)x, (float)y});
        else if (!strcmp(tok, "f")) {
            int vd[3] = {0}, vt[3] = {0}, vn[3] = {0}, k = 0;
            char fv[128];
            int u2 = 0;
            while (k < 3 && sscanf(r, "%127s%n", fv, &u2) == 1) {
                int a = 0, b = 0, c = 0;
                char* q = fv;
                a = (int)strtol(q, &q, 10);
                if (*q == '/') { q++; if (*q != '/') b = (int)strtol(q, &q, 10); if (*q == '/') { q++; c = (int)strtol(q, &q, 10); } }
                vd[k] = a; vt[k] = b; vn[k] = c;
                k++;
                r += u2;
            }
            for (int i = 0; i < 3; i++) {
                pos.push_back(P.at(vd[i] - 1));
                nrm.push_back(vn[0] ? N.at(vn[i] - 1) : V3());
                uv.push_back(vt[0] ? T.at(vt[i] - 1).first : 0.f);
                uv.push_back(vt[0] ? T.at(vt[i] - 1).second : 0.f);
            }
        }
    }
    fclose(f);
}

// ImageTexels::CreateImageTexels + ImageTexels ctor (Texel.cpp:4-38).  The reference decodes with
// stb_image, which picks the format from the content; the restatement reads binary PPM (P6, 255).
static int add_tex(Scene& s, const std::string& path) {
    FILE* f = fopen(path.c_str(), "rb");
    if (!f) throw std::runtime_error("Failed to load image: " + path);
    std::string d;
    char buf[65536];
    size_t k;
    while ((k = fread(buf, 1, sizeof buf, f)) > 0) d.append(buf, k);
    fclose(f);
    if (d.size() < 2 || d[0] != 'P' || d[1] != '6') throw std::runtime_error("not a binary PPM: " + path);
    size_t pos = 2;
    int hdr[3];
    for (int i = 0; i < 3; i++) {
        for (;;) {
            while (pos < d.size() && isspace((unsigned char)d[pos])) pos++;
            if (pos < d.size() && d[pos] == '#') { while (pos < d.size() && d[pos] != '\n') pos++; continue; }
            break;
        }
        hdr[i] = 0;
        while (pos < d.size() && isdigit((unsigned char)d[pos])) hdr[i] = hdr[i] * 10 + (d[pos++] - '0');
    }
    pos++;
    Tex t;
    t.w = hdr[0]; t.h = hdr[1];
    if (t.w <= 0 || t.h <= 0 || hdr[2] != 255 || d.size() < pos + (size_t)t.w * t.h * 3)
        throw std::runtime_error("bad PPM: " + path);
    for (size_t i = 0; i < (size_t)t.w * t.h; i++) {
        V3 c;
        c.x = std::pow((float)(unsigned char)d[pos + 3 * i] / 255.f, 2.2f);
        c.y = std::pow((float)(unsigned char)d[pos + 3 * i + 1] / 255.f, 2.2f);
        c.z = std::pow((float)(unsigned char)d[pos + 3 * i + 2] / 255.f, 2.2f);
        t.texels.push_back(c);
    }
    s.texs.push_back(t);
    return (int)s.texs.size() - 1;
}

// ImageTexels::GetTexel (Texel.cpp:15-19): nearest texel, uv clamped to [0, .99999], v flipped.
static V3 texel(const Scene& s, int tex, float u, float v) {
    const Tex& t = s.texs[tex];
    u = std::min(std::max(u, 0.f), .99999f);
    v = std::min(std::max(v, 0.f), .99999f);
    int x = (int)(u * t.w), y = t.h - (int)(v * t.h) - 1;
    return t.texels[(size_t)y * t.w + x];
}

// ImageCubemapTexture::Evaluate via XYZ2CubeUV (CubemapTexture.cpp:24-58)
static V3 sky(const Scene& s, V3 p) {
    float ax = std::fabs(p.x), ay = std::fabs(p.y), az = std::fabs(p.z);
    int id;
    float u, v;
    if (ax >= ay && ax >= az) { id = p.x >= 0 ? 0 : 1; u = -p.z / p.x; v = p.y / ax; }
    else if (ay >= az) { id = p.y >= 0 ? 2 : 3; u = p.x / ay; v = -p.z / p.y; }
    else { id = p.z >= 0 ? 4 : 5; u = p.x / p.z; v = p.y / az; }
    return texel(s, s.sky[id], u * 0.5f + 0.5f, v * 0.5f + 0.5f);
}

static int tex_by_name(const Scene& s, const std::string& name) {  // Scene::GetTextureByName
    auto it = s.tex_names.find(name);
    if (it == s.tex_names.end()) throw std::runtime_error("Texture name doesn't exist");
    return it->second;
}

static int add_mat(Scene& s, const JNode& n) {
    Mat m;
    std::string t = n.m("Type").s;
    if (t == "Diffuse") {
        m.type = M_DIFF;
        if (n.has("Kd")) m.tex = tex_by_name(s, n.m("Kd").s);
        else m.R = vec3(n.m("Color"));
    }
    else if (t == "Mirror") { m.type = M_MIRROR; m.R = vec3(n.m("Color")); }
    else if (t == "Glass") {
        m.R = vec3(n.m("Color"));
        m.ax = (float)n.m("Roughness").a[0]->F(); m.ay = (float)n.m("Roughness").a[1]->F();
        m.ior = (float)n.m("IOR").F();
        m.type = (m.ax == 0.f && m.ay == 0.f) ? M_GLASS_S : M_GLASS_R;
    } else if (t == "Micro") {
        m.R = vec3(n.m("Color"));
        m.ax = (float)n.m("Roughness").a[0]->F(); m.ay = (float)n.m("Roughness").a[1]->F();
        m.ior = (float)n.m("IOR").F();
        m.type = n.m("NDF").s == "GGX" ? M_MICRO_GGX : M_MICRO_BECK;
    } else if (t == "Plastic") {
        m.R = vec3(n.m("Kd")); m.S = vec3(n.m("Ks"));
        m.ax = (float)n.m("Roughness").a[0]->F(); m.ay = (float)n.m("Roughness").a[1]->F();
        m.type = n.m("NDF").s == "GGX" ? M_PLAST_GGX : M_PLAST_BECK;
    } else if (t == "OrenNayar") {  // Material.cpp:100-121 -> OrenNayarReflection(color, sigma)
        m.type = M_OREN;
        m.R = vec3(n.m("Color"));
        m.ior = (float)n.m("Sigma").F();
    } else if (t == "Phong") {      // Material.cpp:86-99 -> BlinnPhongReflection(color, K)
        m.type = M_PHONG;
        if (n.has("Kd")) m.tex = tex_by_name(s, n.m("Kd").s);
        else m.R = vec3(n.m("Color"));
        m.ior = (float)n.m("K").I();
    } else throw std::runtime_error("material " + t + " not restated");
    s.mats.push_back(m);
    return (int)s.mats.size() - 1;
}

static float shape_area(const Scene& s, int type, int idx) {
    if (type == TRI) { const Tri& t = s.tris[idx]; return length(cross(t.p[1] - t.p[0], t.p[2] - t.p[0])) / 2.f; }
    float r = s.quads[idx].r;
    return type == SPH ? 4 * PI * r * r : PI * r * r;
}

static void quad_rot(V3 rot, Quad& q) {
    M4 m = ident4();
    m = rotate4(m, rot.x / 180.f * PI, V3(1, 0, 0));
    m = rotate4(m, rot.y / 180.f * PI, V3(0, 1, 0));
    m = rotate4(m, rot.z / 180.f * PI, V3(0, 0, 1));
    for (int i = 0; i < 3; i++) q.l2w.c[i] = V3(m.c[i].v[0], m.c[i].v[1], m.c[i].v[2]);
    q.w2l = transpose(q.l2w);
}

static void load(Scene& s, const std::string& cfgp, const std::string& scnp) {
    auto cfg = parse_file(cfgp);
    auto scn = parse_file(scnp);
    s.W = (int)cfg->m("Width").I(); s.H = (int)cfg->m("Height").I(); s.spp = (int)cfg->m("SamplesPerPixel").I();
    std::string acc = cfg->m("Acceleration").s;
    s.anyclip = acc == "BVH";
    s.closest_box = acc != "Brute";
    s.depth = (int)cfg->m("Integrator").m("Depth").I();
    s.direct = cfg->m("Integrator").m("Type").s == "DirectLight";
    {
        const std::string st = cfg->m("Integrator").m("Sampler").m("Type").s;
        if (st == "Halton") s.sampler = 0;
        else if (st == "Default") s.sampler = 1;
        else if (st == "Stratified") {
            s.sampler = 2;
            for (int i = 1; (long long)i * i <= s.spp; i++) if (i * i == s.spp) s.side = i;
            if (!s.side) throw std::runtime_error("Stratified sampler should have a square number of SamplesPerPixel");
        } else throw std::runtime_error("Invalid Sampler Type!");
    }
    // Scene::CreateScene (Scene.cpp:23-45): textures, objects, then the skybox
    const JNode& texn = scn->m("Scene").m("Textures");
    for (auto& kv : texn.o) s.tex_names[kv.first] = add_tex(s, kv.second->m("Path").s);
    const JNode& objs = scn->m("Scene").m("Objects");
    for (auto& np : objs.a) {
        const JNode& n = *np;
        std::string type = n.m("Type").s;
        if (type == "Light") {
            Light L{};
            L.type = 1; L.obj = -1; L.st = -1; L.si = -1;
            L.pos = vec3(n.m("Position")); L.Le = vec3(n.m("Flux"));
            L.zero = zero(L.Le);
            s.lights.push_back(L);
            continue;
        }
        const JNode& sh = n.m("Shape");
        std::string st = sh.m("Type").s;
        std::vector<std::pair<int, int>> shapes;
        if (st == "Sphere" || st == "Disk") {
            Quad q;
            q.pos = vec3(sh.m("Position")); q.r = (float)sh.m("Radius").F();
            quad_rot(sh.has("Rotation") ? vec3(sh.m("Rotation")) : V3(), q);
            s.quads.push_back(q);
            int qi = (int)s.quads.size() - 1;
            shapes.push_back({st == "Sphere" ? SPH : DSK, qi});
        } else {
            std::vector<V3> P, Nn;
            std::vector<float> UV;
            read_obj(sh.m("ObjFile").s, P, Nn, UV);
            V3 tr = vec3(sh.m("Translation")), sc = vec3(sh.m("Scale")), rot = vec3(sh.m("Rotation")) * 0.01745329251994329576923690768489f;
            M4 M = ident4();
            M = translate4(M, tr);
            M = rotate4(M, rot.x, V3(1, 0, 0)); M = rotate4(M, rot.y, V3(0, 1, 0)); M = rotate4(M, rot.z, V3(0, 0, 1));
            M = scale4(M, sc);
            M4 NT = transpose4(inverse4(M));
            for (size_t i = 0; i < P.size(); i++) {
                V4 p = mul4(M, V4{{P[i].x, P[i].y, P[i].z, 1.f}});
                P[i] = V3(p.v[0], p.v[1], p.v[2]);
                V4 q = mul4(NT, V4{{Nn[i].x, Nn[i].y, Nn[i].z, 0.f}});
                Nn[i] = normalize(V3(q.v[0], q.v[1], q.v[2]));
            }
            for (size_t f = 0; f + 2 < P.size(); f += 3) {
                Tri t;
                for (int k = 0; k < 3; k++) { t.p[k] = P[f + k]; t.n[k] = Nn[f + k]; }
                const float* u = &UV[2 * f];
                for (int k = 0; k < 6; k++) t.uv[k] = u[k];
                float a00 = u[0] - u[4], a01 = u[1] - u[5], a10 = u[2] - u[4], a11 = u[3] - u[5];
                float ood = 1.0f / (a00 * a11 - a10 * a01);
                float i00 = a11 * ood, i01 = -a01 * ood, i10 = -a10 * ood, i11 = a00 * ood;
                t.dpdu = V3();
                if (!(std::isinf(i00) || std::isinf(i01) || std::isnan(i00) || std::isnan(i01) || std::isnan(i10) || std::isnan(i11))) {
                    V3 e0 = t.p[0] - t.p[2], e1 = t.p[1] - t.p[2];
                    t.dpdu = normalize(V3(i00 * e0.x + i10 * e1.x, i00 * e0.y + i10 * e1.y, i00 * e0.z + i10 * e1.z));
                }
                s.tris.push_back(t);
                shapes.push_back({TRI, (int)s.tris.size() - 1});
            }
        }
        int mat = n.has("Material") ? add_mat(s, n.m("Material")) : -1;
        for (auto& shp : shapes) {
            int obj = (int)s.objs.size();
            int li = -1;
            if (n.has("AreaLight")) {
                Light L{};
                L.type = 0; L.obj = obj; L.st = shp.first; L.si = shp.second;
                L.Le = vec3(n.m("AreaLight").m("Lemit"));
                L.area = shape_area(s, shp.first, shp.second);
                L.zero = zero(L.Le * PI * L.area);
                s.lights.push_back(L);
                li = (int)s.lights.size() - 1;
            }
            s.objs.push_back(Obj{shp.first, shp.second, mat, li});
        }
    }
    // camera
    // Scene::loadSkybox (Scene.cpp:128-144)
    if (scn->m("Scene").has("Skybox") && scn->m("Scene").m("Skybox").k != JNode::NUL) {
        const std::string dir = scn->m("Scene").m("Skybox").m("Path").s;
        const char* face[6] = {"posx.jpg", "negx.jpg", "posy.jpg", "negy.jpg", "posz.jpg", "negz.jpg"};
        for (int k = 0; k < 6; k++) s.sky[k] = add_tex(s, dir + "/" + face[k]);
    }
    const JNode& cam = scn->m("Camera");
    V3 la = vec3(cam.m("LookAt")), up = vec3(cam.m("Up")), eye = vec3(cam.m("Position"));
    float fov = (float)(cam.m("FOV").F() / 180.f * PI);
    float aspect = (float)s.W / s.H;
    s.CH = 1.0f * std::tan(fov / 2);
    s.CW = s.CH * aspect;
    s.eye = eye;
    s.look = normalize(la - eye);
    V3 p = dot(up, s.look) * s.look;
    s.up = normalize(up - p);
    s.right = normalize(cross(s.look, up));
    // object boxes
    for (auto& o : s.objs) {
        Box b;
        if (o.type == TRI) {
            const Tri& t = s.tris[o.shape];
            b.mn = b.mx = t.p[0];
            for (int k = 1; k < 3; k++)
                for (int a = 0; a < 3; a++) { b.mn[a] = std::min(b.mn[a], t.p[k][a]); b.mx[a] = std::max(b.mx[a], t.p[k][a]); }
        } else if (o.type == SPH) {
            const Quad& q = s.quads[o.shape];
            b.mn = q.pos - q.r; b.mx = q.pos + q.r;
        } else {
            const Quad& q = s.quads[o.shape];
            V3 wn = mul(q.l2w, V3(0, 1, 0));
            float st = std::sqrt(1.f - wn.y * wn.y);
            V3 off(q.r, q.r * st, q.r);
            b.mn = q.pos - off; b.mx = q.pos + off;
        }
        s.boxes.push_back(b);
    }
}

// ---------------------------------------------------------------- BVH (equal counts)
static void bvh_build(Scene& s, int& p, int l, int r) {
    auto uni = [&](int l0, int r0) {
        Box b = s.boxes[s.order[l0]];
        for (int i = l0 + 1; i <= r0; i++)
            for (int a = 0; a < 3; a++) {
                b.mn[a] = std::min(b.mn[a], s.boxes[s.order[i]].mn[a]);
                b.mx[a] = std::max(b.mx[a], s.boxes[s.order[i]].mx[a]);
            }
        return b;
    };
    if (r - l + 1 <= 2) {
        p = ++s.tot;
        s.nodes[p] = Node{uni(l, r), l, r - l + 1, -1};
        return;
    }
    Box b = uni(l, r);
    V3 ext = b.mx - b.mn;
    int axis = 0;
    float d = std::abs(ext[0]);
    for (int i = 1; i < 3; i++) if (std::abs(ext[i]) > d) { d = std::abs(ext[i]); axis = i; }
    int split = l + (r - l) / 2;
    std::nth_element(s.order.begin() + l, s.order.begin() + split, s.order.begin() + r + 1, [&](int x, int y) {
        return (s.boxes[x].mn[axis] + s.boxes[x].mx[axis]) / 2.f < (s.boxes[y].mn[axis] + s.boxes[y].mx[axis]) / 2.f;
    });
    int self = ++s.tot;
    s.nodes[self] = Node{b, 0, 0, axis};
    p = self;
    int c0 = 0, c1 = 0;
    bvh_build(s, c0, l, split);
    bvh_build(s, c1, split + 1, r);
    s.nodes[self].a = c0;
    s.nodes[self].c = c1;
}

static void build_tree(Scene& s) {
    int n = (int)s.objs.size();
    // the reference's build dereferences the missing objects of an empty scene; refuse it here
    if (n == 0) throw std::runtime_error("scene has no objects");
    s.order.resize(n);
    for (int i = 0; i < n; i++) s.order[i] = i;
    s.nodes.assign(2 * n + 1, Node{});
    s.tot = 0;
    int root = 0;
    bvh_build(s, root, 0, n - 1);
}

// ---------------------------------------------------------------- Halton
// Both tables are built once by a thread-safe static initialiser (render threads may race to the
// first call).
static int prime(int i) {
    static const std::vector<int> P = [] {
        std::vector<int> p;
        for (int v = 2; (int)p.size() < 100; v++) {
            bool ok = true;
            for (int d = 2; d * d <= v; d++) if (v % d == 0) { ok = false; break; }
            if (ok) p.push_back(v);
        }
        return p;
    }();
    return P[i];
}
static const std::vector<std::vector<int>>& perm_tables() {
    static const std::vector<std::vector<int>> T = [] {
        std::vector<std::vector<int>> tabs;
        std::mt19937 mt;
        for (int i = 0; i < 100; i++) {
            std::vector<int> t(prime(i));
            for (int j = 0; j < prime(i); j++) t[j] = j;
            std::shuffle(t.begin(), t.end(), mt);
            tabs.push_back(t);
        }
        return tabs;
    }();
    return T;
}
static void extgcd(uint64_t a, uint64_t b, uint64_t& d, uint64_t& x, uint64_t& y) {
    if (!b) { d = a; x = 1; y = 0; } else { extgcd(b, a % b, d, y, x); y -= x * (a / b); }
}
static void halton_setup(Scene& s, int W, int H) {
    int res[2] = {W, H};
    for (int i = 0; i < 2; i++) {
        int base = i == 0 ? 2 : 3, sc = 1, e = 0;
        while (sc < std::min(res[i], 128)) { sc *= base; ++e; }
        s.scales[i] = sc; s.exps[i] = e;
    }
    s.stride = s.scales[0] * s.scales[1];
    for (int i = 0; i < 2; i++) {
        uint64_t d, x, y;
        uint64_t A = s.scales[!i], M = s.scales[i];
        extgcd(A, M, d, x, y);
        s.minv[i] = (int)(d == 1 ? (x + M) % M : (uint64_t)-1);
    }
}
static int halton_index(const Scene& s, int px, int py, int sample) {
    int64_t off = 0;
    if (s.stride > 1) {
        int pm[2] = {px % 128, py % 128};
        for (int i = 0; i < 2; i++) {
            uint64_t v = (uint64_t)(int64_t)pm[i], r = 0;
            int base = i == 0 ? 2 : 3;
            for (int k = 0; k < s.exps[i]; k++) { r = r * base + (v % base); v /= base; }
            off += (int64_t)(r * (uint64_t)(int64_t)s.scales[!i] * (uint64_t)(int64_t)s.minv[i]);
        }
    }
    return (int)(off + (int64_t)(sample * s.stride));
}
static uint64_t rev64(uint64_t n) {
    uint64_t r = 0;
    for (int i = 0; i < 64; i++) { r = (r << 1) | (n & 1); n >>= 1; }
    return r;
}
static inline uint32_t h32(uint32_t x) { x ^= x >> 16; x *= 0x7feb352dU; x ^= x >> 15; x *= 0x846ca68bU; x ^= x >> 16; return x; }
static float hash_u(uint32_t pixel, uint32_t sample, uint32_t dim, uint64_t seed) {
    uint32_t h = h32(pixel ^ h32(sample * 0x9E3779B9U ^ h32(dim + 0x632BE5ABU * (uint32_t)seed) ^ (uint32_t)(seed >> 32)));
    float u = (float)(h >> 8) * 0x1p-24f;
    return std::min(u, OME);
}
// The library's parallel realisation of the Default and Stratified samplers (the reference's
// tile-sequential std::mt19937 streams cannot be split across parallel paths): uniform draws
// hash_u(pixel, sample, dim); stratified draws visit the strata of each dimension in the order of
// a keyed four-round Feistel permutation (cycle-walked into [0, spp)) and jitter inside them.
// Restated here so the tests can compare the GPU with it draw for draw.
static uint32_t permute_index(uint32_t i, uint32_t n, uint32_t key) {
    if (n <= 1) return 0;
    int bits = 32 - __builtin_clz(n - 1);
    bits = bits < 2 ? 2 : bits + (bits & 1);
    if (bits > 30) return i;
    const int half = bits >> 1;
    const uint32_t hmask = (1u << half) - 1u;
    uint32_t rk[4];
    for (uint32_t r = 0; r < 4; r++) rk[r] = h32(key ^ r);
    uint32_t x = i;
    for (uint32_t it = 0; it < (1u << bits); it++) {
        uint32_t L = x >> half, R = x & hmask;
        for (uint32_t r = 0; r < 4; r++) {
            const uint32_t F = h32(R * 0x27d4eb2dU ^ rk[r]) & hmask;
            const uint32_t t = L ^ F;
            L = R;
            R = t;
        }
        x = (L << half) | R;
        if (x < n) break;
    }
    return x;
}
static uint32_t strata_key(uint32_t pixel, uint32_t block, uint32_t dim, uint64_t seed) {
    return h32(pixel * 0x9E3779B9U ^ h32(dim * 0x632BE5ABU ^ h32(block ^ (uint32_t)seed)));
}
static float counter_1d(const Scene& s, int dim, uint32_t pixel, uint32_t sample, uint64_t seed) {
    const float j = hash_u(pixel, sample, (uint32_t)dim, seed);
    if (s.sampler == 1) return j;
    const uint32_t n = (uint32_t)s.spp, k = sample % n;
    const uint32_t cell = permute_index(k, n, strata_key(pixel, sample / n, (uint32_t)dim, seed));
    return std::min((1.0f / (float)n) * ((float)cell + j), OME);
}
static void counter_2d(const Scene& s, int dim, uint32_t pixel, uint32_t sample, uint64_t seed, float& x, float& y) {
    const float jx = hash_u(pixel, sample, (uint32_t)dim, seed), jy = hash_u(pixel, sample, (uint32_t)dim + 1u, seed);
    if (s.sampler == 1) { x = jx; y = jy; return; }
    const uint32_t n = (uint32_t)s.spp, k = sample % n, side = (uint32_t)s.side;
    const uint32_t cell = permute_index(k, n, strata_key(pixel, sample / n, (uint32_t)dim, seed));
    const uint32_t row = cell / side, col = cell - row * side;
    const float inv = 1.0f / (float)side;
    x = std::min(inv * ((float)col + jx), OME);
    y = std::min(inv * ((float)row + jy), OME);
}

static float halton_value(const Scene& s, int vidx, int dim, uint32_t pixel, uint32_t sample, uint64_t seed) {
    if (dim == 0) return (float)((double)rev64((uint64_t)(int64_t)(vidx >> s.exps[0])) * 0x1p-64);
    if (dim == 1) {
        uint64_t v = (uint64_t)(int64_t)(vidx / s.scales[1]);
        float inv = 1.f / 3, res = 0, invN = 1.0f;
        while (v) { uint64_t dg = v % 3; res = res * 3 + dg; invN *= inv; v /= 3; }
        return std::min(res * invN, OME);
    }
    if (dim < 100) {
        const std::vector<int>& T = perm_tables()[dim];
        int base = prime(dim);
        float inv = 1.f / base, res = 0, invN = 1.0f;
        uint64_t v = (uint64_t)(int64_t)vidx;
        while (v) { uint64_t dg = T[v % base]; res = res * base + dg; invN *= inv; v /= base; }
        return std::min((res + inv * T[0] / (1 - inv)) * invN, OME);
    }
    return hash_u(pixel, sample, (uint32_t)dim, seed);
}

// ---------------------------------------------------------------- ray / shapes
struct Ray { V3 o, d; };
static bool box_test(const Ray& r, const bool neg[3], V3 inv, const Box& b, float& t0, float& t1) {
    V3 mn = (b.mn - r.o) * inv, mx = (b.mx - r.o) * inv;
    for (int a = 0; a < 3; a++) {
        float lo = mn[a], hi = mx[a];
        if (neg[a]) std::swap(lo, hi);
        t0 = std::max(t0, lo);
        t1 = std::min(t1, hi);
        if (t1 < t0) return false;
    }
    return true;
}
static bool tri_solve(const Tri& t, const Ray& r, V3& res) {
    V3 c0 = t.p[1] - t.p[0], c1 = t.p[2] - t.p[0], c2 = -r.d;
    float m00 = c0.x, m01 = c0.y, m02 = c0.z, m10 = c1.x, m11 = c1.y, m12 = c1.z, m20 = c2.x, m21 = c2.y, m22 = c2.z;
    float ood = 1.f / (+m00 * (m11 * m22 - m21 * m12) - m10 * (m01 * m22 - m21 * m02) + m20 * (m01 * m12 - m11 * m02));
    float i00 = +(m11 * m22 - m21 * m12) * ood, i10 = -(m10 * m22 - m20 * m12) * ood, i20 = +(m10 * m21 - m20 * m11) * ood;
    float i01 = -(m01 * m22 - m21 * m02) * ood, i11 = +(m00 * m22 - m20 * m02) * ood, i21 = -(m00 * m21 - m20 * m01) * ood;
    float i02 = +(m01 * m12 - m11 * m02) * ood, i12 = -(m00 * m12 - m10 * m02) * ood, i22 = +(m00 * m11 - m10 * m01) * ood;
    V3 P = r.o - t.p[0];
    res = V3(i00 * P.x + i10 * P.y + i20 * P.z, i01 * P.x + i11 * P.y + i21 * P.z, i02 * P.x + i12 * P.y + i22 * P.z);
    return !(std::isnan(res.x) || std::isnan(res.y) || std::isnan(res.z));
}
struct Hit {
    float t = std::numeric_limits<float>::infinity();
    int obj = -1;
    V3 pos, N, dpdu, dpdv;
    bool front = false;
    float u = 0, v = 0;  // texture coordinates (SurfaceInteraction UV)
};
static V3 tri_normal(const Tri& t, float u, float v) {
    V3 b(1 - u - v, u, v);
    return normalize(b.x * t.n[0] + b.y * t.n[1] + b.z * t.n[2]);
}
static bool shape_intersect(const Scene& s, int type, int idx, const Ray& r, Hit& h) {
    if (type == TRI) {
        const Tri& t = s.tris[idx];
        V3 res;
        if (!tri_solve(t, r, res)) return false;
        if (res.x < 0.f || res.x > 1.f || res.y < 0.f || res.y > 1.f || res.x + res.y > 1.0f + 1e-5f || res.z < 0.f) return false;
        V3 N = tri_normal(t, res.x, res.y);
        h.front = dot(r.d, N) < 0;
        N = h.front ? N : -N;
        V3 dpdu = t.dpdu;
        if (zero(dpdu))
            for (int i = 0; i < 3; i++) {
                V3 e(i == 0, i == 1, i == 2);
                V3 tt = cross(e, N);
                if (!zero(tt)) { dpdu = normalize(tt); break; }
            }
        h.t = res.z; h.pos = r.o + r.d * res.z; h.N = N; h.dpdu = dpdu; h.dpdv = cross(N, dpdu);
        // bary_interp (Triangle.cpp:13-16, 43)
        float b0 = 1 - res.x - res.y, b1 = res.x, b2 = res.y;
        h.u = b0 * t.uv[0] + b1 * t.uv[2] + b2 * t.uv[4];
        h.v = b0 * t.uv[1] + b1 * t.uv[3] + b2 * t.uv[5];
        return true;
    }
    const Quad& q = s.quads[idx];
    V3 P = mul(q.w2l, r.o - q.pos), d = mul(q.w2l, r.d);
    if (type == SPH) {
        float a = dot(d, d), b = 2 * dot(d, P), c = dot(P, P) - q.r * q.r;
        float disc = b * b - 4 * a * c;
        if (disc < 0) return false;
        disc = std::sqrt(disc);
        float t1 = (-b + disc) / (2 * a), t2 = (-b - disc) / (2 * a);
        if (t1 > t2) std::swap(t1, t2);
        float t = t1;
        if (std::isnan(t1) || t1 < 0) t = t2;
        if (std::isnan(t) || t < 0) return false;
        V3 hp = P + d * t;
        V3 N = normalize(hp);
        h.front = dot(d, N) < 0;
        N = h.front ? N : -N;
        h.pos = mul(q.l2w, hp) + q.pos;
        h.dpdu = normalize(mul(q.l2w, V3(-N.z, 0, N.x)));
        h.N = mul(q.l2w, N);
        h.dpdv = cross(h.N, h.dpdu);
        h.t = t;
        h.u = std::atan2(-hp.z, hp.x) / PI;  // Sphere.cpp:57-58
        h.v = std::acos(hp.y / q.r) / PI + 1.0f;
        return true;
    }
    if (d.y == 0.f) return false;
    float t = -P.y / d.y;
    if (t < 0) return false;
    V3 hit = P + d * t;
    if (dot(hit, hit) > q.r * q.r) return false;
    V3 N = mul(q.l2w, V3(0, 1, 0));
    h.front = d.y <= 0;
    N = h.front ? N : -N;
    h.pos = mul(q.l2w, hit) + q.pos;
    h.N = N;
    h.dpdu = normalize(q.pos - h.pos);
    h.dpdv = cross(N, h.dpdu);
    h.u = length(hit) / q.r;  // Disk.cpp:61-62
    h.v = (std::atan2(-hit.z, hit.x) + PI) / TWO_PI;
    h.t = t;
    return true;
}
static bool shape_test(const Scene& s, int type, int idx, const Ray& r, float t0, float t1) {
    if (type == TRI) {
        if (t0 > t1) return false;
        V3 res;
        if (!tri_solve(s.tris[idx], r, res)) return false;
        if (res.x < 0 || res.x > 1 || res.y < 0 || res.y > 1 || res.x + res.y > 1 || res.z < 0) return false;
        return res.z >= t0 && res.z <= t1;
    }
    const Quad& q = s.quads[idx];
    V3 P = mul(q.w2l, r.o - q.pos), d = mul(q.w2l, r.d);
    if (type == SPH) {
        if (t0 > t1) return false;
        float a = dot(d, d), b = 2 * dot(d, P), c = dot(P, P) - q.r * q.r;
        float disc = b * b - 4 * a * c;
        if (disc < 0) return false;
        disc = std::sqrt(disc);
        float ta = (-b + disc) / (2 * a), tb = (-b - disc) / (2 * a);
        return (ta >= t0 && ta <= t1) || (tb >= t0 && tb <= t1);
    }
    if (d.y == 0.f) return false;
    float t = -P.y / d.y;
    if (t < t0 || t > t1) return false;
    V3 hit = P + d * t;
    return !(dot(hit, hit) > q.r * q.r);
}
// BVH::Intersect
static bool intersect(const Scene& s, const Ray& r, Hit& best) {
    V3 inv(1.f / r.d.x, 1.f / r.d.y, 1.f / r.d.z);
    bool neg[3] = {inv.x < 0, inv.y < 0, inv.z < 0};
    int stack[64], top = 0, cur = 1;
    bool hit = false;
    while (true) {
        const Node& n = s.nodes[cur];
        float t0 = 0, t1 = std::min(std::numeric_limits<float>::infinity(), best.t);
        if (box_test(r, neg, inv, n.b, t0, t1)) {
            if (n.axis == -1) {
                for (int i = 0; i < n.c; i++) {
                    int o = s.order[n.a + i];
                    t0 = 0; t1 = std::min(std::numeric_limits<float>::infinity(), best.t);
                    if (s.closest_box && !box_test(r, neg, inv, s.boxes[o], t0, t1)) continue;
                    Hit h;
                    if (!shape_intersect(s, s.objs[o].type, s.objs[o].shape, r, h)) continue;
                    if (h.t < std::numeric_limits<float>::infinity()) hit = true;
                    if (h.t < best.t) { best = h; best.obj = o; }
                }
                if (!top) break;
                cur = stack[--top];
            } else {
                int init = neg[n.axis] ? 1 : 0;
                int ch[2] = {n.a, n.c};
                stack[top++] = ch[!init];
                cur = ch[init];
            }
        } else {
            if (!top) break;
            cur = stack[--top];
        }
    }
    return hit;
}
// BVH::IntersectTest
static bool intersect_test(const Scene& s, const Ray& r, float tmin, float tmax, int ignore) {
    V3 inv(1.f / r.d.x, 1.f / r.d.y, 1.f / r.d.z);
    bool neg[3] = {inv.x < 0, inv.y < 0, inv.z < 0};
    int stack[64], top = 0, cur = 1;
    while (true) {
        const Node& n = s.nodes[cur];
        float t0 = tmin, t1 = tmax;
        if (box_test(r, neg, inv, n.b, t0, t1)) {
            if (n.axis == -1) {
                for (int i = 0; i < n.c; i++) {
                    int o = s.order[n.a + i];
                    if (o == ignore) continue;
                    t0 = tmin; t1 = tmax;
                    if (s.anyclip && !box_test(r, neg, inv, s.boxes[o], t0, t1)) continue;
                    if (!shape_test(s, s.objs[o].type, s.objs[o].shape, r, s.anyclip ? t0 : tmin, s.anyclip ? t1 : tmax)) continue;
                    return true;
                }
                if (!top) break;
                cur = stack[--top];
            } else {
                int init = neg[n.axis] ? 1 : 0;
                int ch[2] = {n.a, n.c};
                stack[top++] = ch[!init];
                cur = ch[init];
            }
        } else {
            if (!top) break;
            cur = stack[--top];
        }
    }
    return false;
}

// ---------------------------------------------------------------- BSDFs
enum { BR = 1, BT = 2, BG = 4, BS = 8, BD = 16, BALL = 0x1F };
struct BxDF { int mt, flags; V3 R, S; float ax, ay, etaA, etaB; };
static int mflags(int mt) {
    switch (mt) {
        case M_DIFF: return BD | BR;
        case M_OREN: return BD | BR;
        case M_MIRROR: return BS | BR;
        case M_GLASS_R: return BT | BR | BG;
        case M_GLASS_S: return BT | BR | BS;
        default: return BR | BG;
    }
}
static BxDF make_bxdf(const Mat& m, bool front) {
    BxDF b{m.type, mflags(m.type), m.R, m.S, m.ax, m.ay, 1.f, 1.f};
    if (m.type == M_OREN) {
        // OrenNayarReflection constructor (Reflections.cpp:20-26): A, B from sigma
        float s2 = m.ior * m.ior;
        b.ax = 1.f - s2 / (2 * (s2 + 0.33f));
        b.ay = (0.45f * s2) / (s2 + 0.09f);
    } else if (m.type == M_PHONG) {
        b.ax = m.ior;  // exponent K
    } else if (m.type != M_MIRROR && m.type != M_DIFF) {
        b.etaB = m.ior;
        if (!front) std::swap(b.etaA, b.etaB);
    }
    return b;
}
static float sqf(float x) { return x * x; }
static float fr_diel(float eA, float eB, float cI) {
    float sI = std::sqrt(std::max(0.f, 1.f - cI * cI)), sT = eA / eB * sI;
    if (sT >= 1.f) return 1.f;
    float cT = std::sqrt(std::max(0.f, 1.f - sT * sT));
    float a = ((eB * cI) - (eA * cT)) / ((eB * cI) + (eA * cT)), b = ((eA * cI) - (eB * cT)) / ((eA * cI) + (eB * cT));
    return (a * a + b * b) / 2;
}
static float fr_schlick(float r0, float eA, float eB, float cI) {
    float sI = std::sqrt(std::max(0.f, 1.f - cI * cI)), sT = eA / eB * sI;
    if (sT >= 1.f) return 1.f;
    return r0 + (1.f - r0) * std::pow(1.f - cI, 5.f);
}
static float fres(const BxDF& b, float c) { return (b.mt == M_MICRO_GGX || b.mt == M_MICRO_BECK) ? fr_schlick(0.99f, b.etaA, b.etaB, c) : fr_diel(b.etaA, b.etaB, c); }
static bool beck(int mt) { return mt == M_MICRO_BECK || mt == M_PLAST_BECK; }
static void csphi(V3 w, float st, float& c, float& s) {
    if (st == 0.f) { c = 1.f; s = 0.f; return; }
    c = std::min(std::max(w.x / st, -1.f), 1.f);
    s = std::min(std::max(-w.z / st, -1.f), 1.f);
}
static float D(const BxDF& b, V3 wh) {
    float c2 = wh.y * wh.y;
    if (!beck(b.mt)) {
        float s2 = std::max(0.f, 1.f - c2), c, s;
        csphi(wh, std::sqrt(s2), c, s);
        float A = sqf(c) / sqf(b.ax) + sqf(s) / sqf(b.ay);
        return 1.f / (PI * b.ax * b.ay * sqf(A - c2 * (A - 1)));
    }
    float s2 = 1.f - c2, t2 = s2 / c2;
    if (std::isinf(t2)) return 0.f;
    float c, s;
    csphi(wh, std::sqrt(s2), c, s);
    return std::exp(-t2 * (sqf(c) / sqf(b.ax) + sqf(s) / sqf(b.ay))) / (PI * b.ax * b.ay * (c2 * c2));
}
static float lambda(const BxDF& b, V3 w) {
    if (!beck(b.mt)) {
        float c2 = w.y * w.y, s2 = 1.f - c2, t2 = s2 / c2;
        if (std::isinf(t2)) return 0.f;
        float c, s;
        csphi(w, std::sqrt(s2), c, s);
        float a2 = sqf(c) * sqf(b.ax) + sqf(s) * sqf(b.ay);
        return (-1 + std::sqrt(1 + a2 * t2)) / 2;
    }
    float ct = w.y, st = std::sqrt(1.f - ct * ct), tt = std::abs(st / ct);
    if (std::isinf(tt)) return 0.f;
    float c, s;
    csphi(w, st, c, s);
    float al = std::sqrt(sqf(c) * sqf(b.ax) + sqf(s) * sqf(b.ay));
    float a = 1.f / (tt * al);
    if (a >= 1.6f) return 0.f;
    return (1 - 1.259f * a + 0.396f * a * a) / (3.535f * a + 2.181f * a * a);
}
static float G(const BxDF& b, V3 o, V3 i) { return 1.f / (1.f + lambda(b, o) + lambda(b, i)); }
static float ndfpdf(const BxDF& b, V3 wh) { return D(b, wh) * std::abs(wh.y); }
static V3 ucos(float ct, float phi) { float r = std::sqrt(1 - ct * ct); return V3(r * std::cos(phi), ct, -r * std::sin(phi)); }
static V3 sample_wh(const BxDF& b, float ux, float uy) {
    float ct, phi;
    if (!beck(b.mt)) {
        if (b.ax == b.ay) { ct = std::sqrt((1 - ux) / (ux * (b.ax * b.ax - 1) + 1)); phi = TWO_PI * uy; }
        else {
            phi = std::atan(b.ay / b.ax * std::tan(TWO_PI * uy + HALF_PI));
            if (uy > 0.5) phi += PI;
            float sp = std::sin(phi), cp = std::cos(phi);
            float A = sqf(cp) / sqf(b.ax) + sqf(sp) / sqf(b.ay);
            ct = std::sqrt(A * (ux - 1) / (ux * (A - 1) - A));
        }
        return ucos(ct, phi);
    }
    float ls = std::log(1.f - ux);
    if (std::isinf(ls)) ls = 0;
    float t2;
    if (b.ax == b.ay) { t2 = -sqf(b.ax) * ls; phi = uy * TWO_PI; }
    else {
        phi = std::atan(b.ay / b.ax * std::tan(TWO_PI * uy + HALF_PI));
        if (uy > 0.5) phi += PI;
        float sp = std::sin(phi), cp = std::cos(phi);
        t2 = -ls / (cp * cp / sqf(b.ax) + sp * sp / sqf(b.ay));
    }
    return ucos(1.f / std::sqrt(1.f + t2), phi);
}
static V3 reflectv(V3 I, V3 N) { return I - N * dot(N, I) * 2.f; }
// OrenNayarReflection::DistributionFunction (Reflections.cpp:36-58)
static V3 onf(const BxDF& b, V3 o, V3 i) {
    float sO = std::sqrt(std::max(0.f, 1.f - o.y * o.y)), sI = std::sqrt(std::max(0.f, 1.f - i.y * i.y));
    float sa, tb;
    if (o.y < i.y) { sa = sI; tb = sO / o.y; }
    else { sa = sO; tb = sI / i.y; }
    float dc = 0.f;
    if (sI > 1e-5f && sO > 1e-5f) {
        float ci, si_, co, so;
        csphi(i, sI, ci, si_);
        csphi(o, sO, co, so);
        dc = std::max(0.f, ci * co + si_ * so);
    }
    return b.R / PI * (b.ax + b.ay * (dc * sa * tb));
}
// BlinnPhongReflection::Pdf / DistributionFunction (BlinnPhongReflection.cpp:14-27); std::pow of a
// float and an int is evaluated in double
static float bppdf(const BxDF& b, V3 o, V3 i) {
    V3 wh = normalize(o + i);
    return (float)((double)((b.ax + 2.f) / TWO_PI) * std::pow((double)std::max(0.f, wh.y), (double)(b.ax + 1.f)));
}
static V3 bpf(const BxDF& b, V3 o, V3 i) {
    V3 wh = normalize(o + i);
    float s = (float)std::pow((double)std::max(0.f, wh.y), (double)b.ax) * (b.ax + 2.f) / TWO_PI;
    return b.R * s / (4.f * std::max(0.f, i.y) * std::max(0.f, o.y));
}
// Redraw after a rejected half vector: a hash of the rejected pair and the attempt (the reference
// redraws from a shared static std::mt19937, BlinnPhongReflection.cpp:33-56); at most 64 draws.
static uint32_t bph(uint32_t x) { x ^= x >> 16; x *= 0x7feb352dU; x ^= x >> 15; x *= 0x846ca68bU; x ^= x >> 16; return x; }
static void phong_redraw(float& ux, float& uy, int attempt) {
    uint32_t bx, by;
    std::memcpy(&bx, &ux, 4);
    std::memcpy(&by, &uy, 4);
    uint32_t h = bph(bx ^ bph(by + 0x9E3779B9u * (uint32_t)(attempt + 1)));
    uint32_t g = bph(h ^ 0x85EBCA6Bu);
    ux = (float)(h >> 8) * 0x1p-24f;
    uy = (float)(g >> 8) * 0x1p-24f;
}
static bool refractv(V3 wo, V3 wh, float eta, V3& wt) {
    float co = std::min(std::max(dot(wo, wh), -1.f), 1.f), s2o = std::max(0.f, 1.f - co * co), s2i = eta * eta * s2o;
    if (s2i > 1.f) return false;
    float ci = std::sqrt(1.f - s2i);
    wt = eta * -wo + (eta * co - ci) * wh;
    return true;
}
static float rpdf(const BxDF& b, V3 o, V3 i) { V3 H = normalize(o + i); return ndfpdf(b, H) / (4 * dot(o, H)); }
static V3 rf(const BxDF& b, V3 o, V3 i) {
    if (o.y * i.y < 0) return V3();
    V3 H = normalize(o + i);
    float F = fres(b, std::max(0.f, dot(o, H)));
    return b.R * D(b, H) * G(b, o, i) * F / (4 * std::max(0.f, i.y) * std::max(0.f, o.y));
}
static float tpdf(const BxDF& b, V3 o, V3 i) {
    if (o.y * i.y > 0) return 0.f;
    float eta = b.etaB / b.etaA;
    V3 H = normalize(o + i * eta);
    return ndfpdf(b, H) * (eta * eta * std::abs(dot(H, i)) / sqf(dot(o, H) + eta * dot(i, H)));
}
static V3 tf(const BxDF& b, V3 o, V3 i) {
    if (i.y * o.y > 0 || o.y == 0.f) return V3();
    float eta = b.etaB / b.etaA;
    V3 H = normalize(o + i * eta);
    if (H.y < 0) H = -H;
    float bot = sqf(dot(o, H) + eta * dot(i, H));
    float F = 1.f - fres(b, std::max(0.f, dot(o, H)));
    return b.R * D(b, H) * G(b, o, i) * F * std::abs(dot(H, o)) * std::abs(dot(H, i)) / (bot * std::max(0.f, -i.y) * std::max(0.f, o.y));
}
static float fbpdf(const BxDF& b, V3 o, V3 i) { V3 H = normalize(o + i); return 0.5f * (std::max(0.f, i.y) / PI + ndfpdf(b, H) / (4 * dot(o, H))); }
static V3 fbf(const BxDF& b, V3 o, V3 i) {
    float ci = std::max(0.f, i.y), co = std::max(0.f, o.y);
    V3 one(1, 1, 1);
    V3 diff = (28.f / (23.f * PI)) * b.R * (one - b.S) * (1.f - (float)std::pow(1.f - 0.5f * co, 5)) * (1.f - (float)std::pow(1.f - 0.5f * ci, 5));
    V3 H = normalize(o + i);
    float wh = dot(i, H);
    V3 sch = b.S + (one - b.S) * std::pow(1.f - wh, 5.f);
    return diff + D(b, H) / (4 * wh * std::max(ci, co)) * sch;
}
static V3 bxf(const BxDF& b, V3 o, V3 i) {
    switch (b.mt) {
        case M_DIFF: return b.R / PI;
        case M_MICRO_GGX: case M_MICRO_BECK: return rf(b, o, i);
        case M_GLASS_R: return o.y * i.y < 0 ? tf(b, o, i) : rf(b, o, i);
        case M_PLAST_GGX: case M_PLAST_BECK: return fbf(b, o, i);
        case M_OREN: return onf(b, o, i);
        case M_PHONG: return bpf(b, o, i);
    }
    return V3();
}
static float bxpdf(const BxDF& b, V3 o, V3 i) {
    switch (b.mt) {
        case M_DIFF: return std::max(0.f, i.y) / PI;
        case M_MICRO_GGX: case M_MICRO_BECK: return rpdf(b, o, i);
        case M_GLASS_R: return o.y * i.y < 0 ? tpdf(b, o, i) : rpdf(b, o, i);
        case M_PLAST_GGX: case M_PLAST_BECK: return fbpdf(b, o, i);
        case M_OREN: return std::max(0.f, i.y) / PI;
        case M_PHONG: return bppdf(b, o, i);
    }
    return 0.f;
}
static V3 cosine_hemi(float ux, float uy, float& pdf) {
    float r = std::sqrt(ux), phi = uy * TWO_PI;
    V3 w(r * std::cos(phi), std::sqrt(1.0f - r * r), r * std::sin(phi));
    pdf = w.y / PI;
    return w;
}
static V3 bxsample(const BxDF& b, float ux, float uy, V3 o, V3& i, float& pdf, int& st) {
    switch (b.mt) {
        case M_DIFF: i = cosine_hemi(ux, uy, pdf); return b.R / PI;
        case M_MIRROR: i = V3(-o.x, o.y, -o.z); pdf = 1.f; return b.R;
        case M_GLASS_S: {
            float fr = fr_diel(b.etaA, b.etaB, o.y);
            if (ux < fr) { st = BR | BS; i = V3(-o.x, o.y, -o.z); pdf = fr; return fr * b.R; }
            st = BT | BS; refractv(o, V3(0, 1, 0), b.etaA / b.etaB, i); pdf = 1.f - fr; return (1.f - fr) * b.R;
        }
        case M_MICRO_GGX: case M_MICRO_BECK: {
            V3 wh = sample_wh(b, ux, uy);
            if (dot(o, wh) <= 0) return V3();
            i = reflectv(-o, wh); pdf = rpdf(b, o, i); i = clampv(i);
            return rf(b, o, i);
        }
        case M_GLASS_R: {
            V3 wh = sample_wh(b, ux, uy);
            if (dot(o, wh) <= 0) return V3();
            float fr = fr_diel(b.etaA, b.etaB, dot(o, wh));
            if (ux < fr) { st = BR | BG; i = reflectv(-o, wh); pdf = bxpdf(b, o, i) * fr; i = clampv(i); return rf(b, o, i); }
            V3 t;
            if (refractv(o, wh, b.etaA / b.etaB, t)) { st = BT | BG; i = t; pdf = bxpdf(b, o, i) * (1 - fr); i = clampv(i); return tf(b, o, i); }
            st = BR | BG; i = reflectv(-o, wh); pdf = bxpdf(b, o, i) * (1 - fr); i = clampv(i); return rf(b, o, i);
        }
        case M_PLAST_GGX: case M_PLAST_BECK: {
            if (ux < 0.5) { i = cosine_hemi(ux * 2.f, uy, pdf); }
            else {
                V3 wh = sample_wh(b, (ux - 0.5f) * 2.f, uy);
                V3 L = reflectv(-o, wh);
                if (L.y * o.y <= 0) return V3();
                i = clampv(L);
            }
            pdf = fbpdf(b, o, i);
            return fbf(b, o, i);
        }
        case M_OREN: i = cosine_hemi(ux, uy, pdf); return onf(b, o, i);
        case M_PHONG: {
            for (int attempt = 0; attempt < 64; attempt++) {
                float ct = (float)std::pow((double)ux, 1.0 / (double)(b.ax + 2.f));
                V3 N = ucos(ct, TWO_PI * uy);
                if (dot(N, o) < 0) { phong_redraw(ux, uy, attempt); continue; }
                V3 w = reflectv(-o, N);
                if (w.y < 0) { phong_redraw(ux, uy, attempt); continue; }
                i = w;
                pdf = bppdf(b, o, i);
                return bpf(b, o, i);
            }
            return V3();
        }
    }
    return V3();
}
struct Frame { V3 T, N, B; };
static V3 loc(const Frame& f, V3 w) { return clampv(V3(dot(f.T, w), dot(f.N, w), dot(f.B, w))); }
static V3 wld(const Frame& f, V3 w) { return clampv(f.T * w.x + f.N * w.y + f.B * w.z); }
static V3 bsdf_f(const BxDF& b, const Frame& fr, V3 wo, V3 wi) {
    V3 o = loc(fr, wo), i = loc(fr, wi);
    bool refl = i.y * o.y > 0;
    if ((refl && (b.flags & BR)) || (!refl && (b.flags & BT))) return bxf(b, o, i);
    return V3();
}
static float bsdf_pdf(const BxDF& b, const Frame& fr, V3 wo, V3 wi, int flags) {
    V3 o = loc(fr, wo), i = loc(fr, wi);
    bool refl = i.y * o.y > 0;
    bool m = (b.flags & flags) == b.flags;
    if ((m && refl && (b.flags & BR)) || (!refl && (b.flags & BT))) return bxpdf(b, o, i);
    return 0.f;
}
static V3 bsdf_sample(const BxDF& b, const Frame& fr, float u1, float ux, float uy, V3 wo, V3& wi, float& pdf, int flags, int& st) {
    (void)u1;
    if ((b.flags & flags) != b.flags) return V3();
    st = b.flags;
    V3 o = loc(fr, wo), i;
    V3 L = bxsample(b, ux, uy, o, i, pdf, st);
    if (zero(L) || pdf == 0.f) return V3();
    wi = wld(fr, i);
    return L;
}

// ---------------------------------------------------------------- lights
static float light_pdf(const Scene& s, const Light& L, V3 pos, V3 N, V3 wi) {
    Ray r{pos + N * 1e-4f, wi};
    Hit h;
    if (!shape_intersect(s, L.st, L.si, r, h)) return 0.f;
    V3 dv = pos - h.pos;
    return dot(dv, dv) / (std::max(0.f, dot(-normalize(wi), h.N)) * L.area);
}
static V3 light_sample(const Scene& s, const Light& L, V3 pos, V3 N, float ux, float uy, V3& ep, float& pdf) {
    if (L.type == 1) {
        ep = L.pos; pdf = 1.0f;
        V3 I = L.Le / (4 * PI);
        V3 dv = ep - pos;
        return I / dot(dv, dv);
    }
    V3 p, n;
    if (L.st == TRI) {
        const Tri& t = s.tris[L.si];
        float u = 1 - std::sqrt(ux), v = uy * std::sqrt(ux);
        V3 b(1.f - u - v, u, v);
        p = b.x * t.p[0] + b.y * t.p[1] + b.z * t.p[2];
        n = normalize(b.x * t.n[0] + b.y * t.n[1] + b.z * t.n[2]);
    } else if (L.st == SPH) {
        const Quad& q = s.quads[L.si];
        float y = 2.f * ux - 1.f, phi = uy * TWO_PI, r = std::sqrt(1 - y * y);
        V3 dir(r * std::cos(phi), y, r * std::sin(phi));
        p = q.pos + dir * q.r; n = dir;
    } else {
        const Quad& q = s.quads[L.si];
        float r = std::sqrt(ux), phi = uy * TWO_PI;
        p = q.pos + mul(q.l2w, V3(std::cos(phi) * r * q.r, 0.f, -std::sin(phi) * r * q.r));
        n = mul(q.l2w, V3(0, 1, 0));
    }
    ep = p;
    V3 dir = p - pos;
    pdf = light_pdf(s, L, pos, N, dir);
    return dot(n, -dir) < 0 ? V3() : L.Le;
}
static float ph(float f, float g) { return (f * f) / (f * f + g * g); }
static V3 spawn(const Hit& h, V3 dir) { bool back = dot(dir, h.N) < 0; return h.pos + (back ? -h.N : h.N) * 1e-4f; }

// ---------------------------------------------------------------- integrator
// DefaultSampler / StratifiedSampler (DefaultSampler.cpp:13-29, StratifiedSampler.cpp:22-100,
// PixelSampler.cpp:14-40): a std::mt19937 per 32 x 32 tile, seeded with the tile index by Clone
// (SamplerIntegrator.cpp:40); every draw is min(1 - 2^-24, mt() * 2^-32) in float (Utils.h:12-15).
// A two-float draw takes the y value first: g++ evaluates the two calls in Point2f(a(), b()) from
// right to left.  The stratified sampler fills 18 one-dimensional and 18 two-dimensional tables of
// SamplesPerPixel entries at StartPixel (jittered strata, then std::shuffle with the same engine);
// requests past the 18th of a kind fall back to plain draws.  The stream is shared by every path of
// the tile, so a value depends on everything the tile traced before it.
struct PixelRng {
    static constexpr int kDims = 18;
    std::mt19937 mt;
    int kind = 1, spp = 1, side = 1;
    int cur = 0, d1 = 0, d2 = 0;
    std::vector<float> t1[kDims];
    std::vector<std::pair<float, float>> t2[kDims];
    PixelRng(int kind_, int spp_, int side_, unsigned tile) : mt(tile), kind(kind_), spp(spp_), side(side_) {
        if (kind == 2)
            for (int i = 0; i < kDims; i++) { t1[i].resize(spp); t2[i].resize(spp); }
    }
    float uni() { return std::min(0x1.fffffep-1f, (float)mt() * 2.3283064365386963e-10f); }
    void pair(float& x, float& y) { y = uni(); x = uni(); }
    void start_pixel() {
        cur = d1 = d2 = 0;
        if (kind != 2) return;
        for (int i = 0; i < kDims; i++) {
            const float inv = 1.f / spp;
            for (int k = 0; k < spp; k++) t1[i][k] = std::min(0x1.fffffep-1f, inv * (k + uni()));
            std::shuffle(t1[i].begin(), t1[i].begin() + spp, mt);
        }
        for (int i = 0; i < kDims; i++) {
            const float inv = 1.f / side;
            int k = 0;
            for (int r = 0; r < side; r++)
                for (int c = 0; c < side; c++, k++) {
                    t2[i][k].first = std::min(0x1.fffffep-1f, inv * (c + uni()));
                    t2[i][k].second = std::min(0x1.fffffep-1f, inv * (r + uni()));
                }
            std::shuffle(t2[i].begin(), t2[i].begin() + spp, mt);
        }
    }
    bool next_sample() { d1 = d2 = 0; return ++cur < spp; }
    float get1() { return (kind == 2 && d1 < kDims) ? t1[d1++][cur] : uni(); }
    void get2(float& x, float& y) {
        if (kind == 2 && d2 < kDims) { x = t2[d2][cur].first; y = t2[d2][cur].second; d2++; }
        else pair(x, y);
    }
};

struct Sampler {
    const Scene& s;
    int vidx;
    uint32_t pixel, sample;
    uint64_t seed;
    int dim = 0;
    PixelRng* pr = nullptr;  // the reference's Default / Stratified stream; else per-draw values
    float get1() {
        if (pr) return pr->get1();
        if (s.sampler != 0) return counter_1d(s, dim++, pixel, sample, seed);
        return halton_value(s, vidx, dim++, pixel, sample, seed);
    }
    void get2(float& x, float& y) {
        if (pr) { pr->get2(x, y); return; }
        if (s.sampler != 0) { counter_2d(s, dim, pixel, sample, seed, x, y); dim += 2; return; }
        x = halton_value(s, vidx, dim++, pixel, sample, seed);
        y = halton_value(s, vidx, dim++, pixel, sample, seed);
    }
};

static V3 evaluate(const Scene& s, Ray ray, Sampler& smp) {
    bool lightPath = true;
    V3 beta(1, 1, 1), L(0, 0, 0);
    for (int bounce = 0; bounce < s.depth; bounce++) {
        Hit h;
        if (!intersect(s, ray, h)) {
            if (s.sky[0] >= 0) L = L + beta * sky(s, ray.d);  // PathTracingIntegrator.cpp:39-46
            break;
        }
        const Obj& ob = s.objs[h.obj];
        if (lightPath && ob.light >= 0) {
            V3 na = h.front ? h.N : -h.N;
            if (!(dot(na, -ray.d) < 0)) L = L + beta * s.lights[ob.light].Le;
        }
        if (ob.mat < 0) { ray = Ray{spawn(h, ray.d), ray.d}; continue; }
        BxDF b = make_bxdf(s.mats[ob.mat], h.front);
        if (s.mats[ob.mat].tex >= 0) b.R = texel(s, s.mats[ob.mat].tex, h.u, h.v);  // UVTexture Kd
        Frame fr{h.dpdu, h.N, h.dpdv};
        V3 wo = -ray.d;
        // UniformSampleAllLights
        float lx, ly, bx, by;
        smp.get2(lx, ly);
        smp.get2(bx, by);
        V3 Ld(0, 0, 0);
        const int ns = BALL & ~BS;
        for (int li = 0; li < (int)s.lights.size(); li++) {
            const Light& Lg = s.lights[li];
            if (Lg.zero || li == ob.light) continue;
            V3 Le(0, 0, 0);
            V3 ep;
            float pl;
            V3 Li = light_sample(s, Lg, h.pos, h.N, lx, ly, ep, pl);
            V3 wi = normalize(ep - h.pos);
            if (pl != 0.f && !zero(Li)) {
                V3 f = bsdf_f(b, fr, wo, wi) * std::max(0.f, dot(h.N, wi));
                float pb = bsdf_pdf(b, fr, wo, wi, ns);
                if (!zero(f)) {
                    bool back = dot(ep - h.pos, h.N) < 0;
                    V3 org = h.pos + (back ? -h.N : h.N) * 1e-4f;
                    if (intersect_test(s, Ray{org, ep - org}, 0, 1 - 1e-5f, Lg.type == 0 ? Lg.obj : -1)) Li = V3();
                    if (!zero(Li)) Le = Le + (Lg.type == 1 ? f * Li / pl : f * Li * ph(pl, pb) / pl);
                }
            }
            if (Lg.type != 1) {
                float u1 = smp.get1();
                V3 wi2;
                float pb2 = 0;
                int st = 0;
                V3 f = bsdf_sample(b, fr, u1, bx, by, wo, wi2, pb2, ns, st);
                if (!zero(f)) {
                    float w = 1.f;
                    bool ok = true;
                    if (!(st & BS)) {
                        f = f * std::max(0.f, dot(h.N, wi2));
                        float pl2 = light_pdf(s, Lg, h.pos, h.N, wi2);
                        if (pl2 == 0.f) ok = false;
                        else w = ph(pb2, pl2);
                    }
                    if (ok) {
                        Hit lh;
                        V3 Li2(0, 0, 0);
                        if (intersect(s, Ray{spawn(h, wi2), wi2}, lh)) {
                            if (s.objs[lh.obj].light == li) {
                                V3 na = lh.front ? lh.N : -lh.N;
                                if (!(dot(na, -wi2) < 0)) Li2 = Lg.Le;
                            }
                        }
                        if (!zero(Li2)) Le = Le + f * Li2 * w / pb2;
                    }
                }
            }
            Ld = Ld + Le;
        }
        L = L + beta * Ld;
        // continuation: SampleDirection(Get1D(), Get2D(), ...) evaluates Get2D first
        float cx, cy;
        smp.get2(cx, cy);
        float c1 = smp.get1();
        V3 wi;
        float pdf = 0;
        int st = 0;
        V3 f = bsdf_sample(b, fr, c1, cx, cy, wo, wi, pdf, BALL, st);
        if (std::abs(pdf) == 0.f || zero(f)) break;
        bool spec = (st & BS) != 0;
        float cosv = spec ? 1.0f : std::max(0.f, (st & BT) ? dot(-h.N, wi) : dot(h.N, wi));
        lightPath = spec || (st & BT);
        ray = Ray{spawn(h, wi), wi};
        beta = beta * (f * cosv / pdf);
        if (bounce > 3) {
            float q = std::max(.05f, 1.f - length(beta));
            if (smp.get1() < q) break;
            beta = beta / (1 - q);
        }
    }
    return L;
}

// DirectLightingIntegrator::eval_rec (DirectLightingIntegrator.cpp:27-156): emission at every hit,
// pass-through at the same level, one round of UniformSampleAllLights (own light included).
static V3 evaluate_direct(const Scene& s, Ray ray, Sampler& smp) {
    V3 L(0, 0, 0);
    if (s.depth <= 0) return L;
    for (int hop = 0; hop < 1 << 20; hop++) {
        Hit h;
        if (!intersect(s, ray, h)) return s.sky[0] >= 0 ? L + sky(s, ray.d) : L;  // DirectLightingIntegrator.cpp:34-38
        const Obj& ob = s.objs[h.obj];
        if (ob.light >= 0) {
            V3 na = h.front ? h.N : -h.N;
            if (!(dot(na, -ray.d) < 0)) L = L + s.lights[ob.light].Le;
        }
        if (ob.mat < 0) {
            if (ob.light >= 0) return L;
            ray = Ray{spawn(h, ray.d), ray.d};
            continue;
        }
        BxDF b = make_bxdf(s.mats[ob.mat], h.front);
        if (s.mats[ob.mat].tex >= 0) b.R = texel(s, s.mats[ob.mat].tex, h.u, h.v);  // UVTexture Kd
        Frame fr{h.dpdu, h.N, h.dpdv};
        V3 wo = -ray.d;
        float lx, ly, bx, by;
        smp.get2(lx, ly);
        smp.get2(bx, by);
        V3 Ld(0, 0, 0);
        const int ns = BALL & ~BS;
        for (int li = 0; li < (int)s.lights.size(); li++) {
            const Light& Lg = s.lights[li];
            if (Lg.zero) continue;
            V3 Le(0, 0, 0), ep;
            float pl;
            V3 Li = light_sample(s, Lg, h.pos, h.N, lx, ly, ep, pl);
            V3 wi = normalize(ep - h.pos);
            if (pl != 0.f && !zero(Li)) {
                V3 f = bsdf_f(b, fr, wo, wi) * std::max(0.f, dot(h.N, wi));
                float pb = bsdf_pdf(b, fr, wo, wi, ns);
                if (!zero(f)) {
                    bool back = dot(ep - h.pos, h.N) < 0;
                    V3 org = h.pos + (back ? -h.N : h.N) * 1e-4f;
                    if (intersect_test(s, Ray{org, ep - org}, 0, 1.f - 1e-5f, Lg.type == 0 ? Lg.obj : -1)) Li = V3();
                    if (!zero(Li)) Le = Le + (Lg.type == 1 ? f * Li / pl : f * Li * ph(pl, pb) / pl);
                }
            }
            if (Lg.type != 1) {
                float u1 = smp.get1();
                V3 wi2;
                float pb2 = 0;
                int st = 0;
                V3 f = bsdf_sample(b, fr, u1, bx, by, wo, wi2, pb2, ns, st);
                bool spec = (st & BS) != 0;
                float w = 1.f;
                bool ok = true;
                if (!spec) {
                    f = f * std::max(0.f, dot(h.N, wi2));
                    float pl2 = light_pdf(s, Lg, h.pos, h.N, wi2);
                    if (pl2 == 0.f) ok = false;
                    else w = ph(pb2, pl2);
                }
                if (ok) {
                    Hit lh;
                    V3 Li2(0, 0, 0);
                    if (intersect(s, Ray{spawn(h, wi2), wi2}, lh) && s.objs[lh.obj].light == li) {
                        V3 na = lh.front ? lh.N : -lh.N;
                        if (!(dot(na, -wi2) < 0)) Li2 = Lg.Le;
                    }
                    if (!zero(Li2)) Le = Le + f * Li2 * w / pb2;
                }
            }
            Ld = Ld + Le;
        }
        return L + Ld;
    }
    return L;
}

static Ray camera_ray(const Scene& s, float px, float py) {
    px = px * 2 - 1; py = py * 2 - 1;
    px *= s.CW; py *= s.CH;
    return Ray{s.eye, normalize(s.right * px + s.up * py + s.look * 1.0f)};
}

}  // namespace orc

using namespace orc;

// One camera sample of pixel (x, y): the sampler's first 2D draw jitters the pixel
// (SamplerIntegrator.cpp:49-55), then the integrator's Evaluate.
static V3 trace_sample(const Scene& s, Sampler& smp, int x, int y) {
    float sx, sy;
    smp.get2(sx, sy);
    Ray cr = camera_ray(s, ((float)x + sx) / s.W, ((float)y + sy) / s.H);
    return s.direct ? evaluate_direct(s, cr, smp) : evaluate(s, cr, smp);
}

// Every sample of one 32 x 32 tile in SamplerIntegrator::Render's order (SamplerIntegrator.cpp:25-69):
// columns outer, rows inner, samples innermost, one sampler clone per tile.  f(x, y, sample, L).
template <class F>
static void run_tile(const Scene& s, int tx, int ty, F&& f) {
    const int nty = (s.H + 31) / 32;
    PixelRng pr(s.sampler, s.spp, s.side, (unsigned)(tx * nty + ty));
    const int x0 = 32 * tx, x1 = std::min(x0 + 32, s.W), y0 = 32 * ty, y1 = std::min(y0 + 32, s.H);
    for (int x = x0; x < x1; x++)
        for (int y = y0; y < y1; y++) {
            pr.start_pixel();
            do {
                Sampler smp{s, 0, (uint32_t)(y * s.W + x), (uint32_t)pr.cur, 0};
                smp.pr = &pr;
                f(x, y, pr.cur, trace_sample(s, smp, x, y));
            } while (pr.next_sample());
        }
}

// Runs `task(i)` for i in [0, n) on `threads` workers.
template <class F>
static void parallel_for(int n, int threads, F&& task) {
    std::atomic<int> next{0};
    std::vector<std::thread> th;
    for (int k = 0; k < std::max(1, threads); k++)
        th.emplace_back([&]() { for (int i; (i = next.fetch_add(1)) < n;) task(i); });
    for (auto& t : th) t.join();
}

extern "C" {

void* orc_open(const char* cfg, const char* scn, char* err, int errlen) {
    try {
        auto* s = new Scene();
        load(*s, cfg, scn);
        halton_setup(*s, s->W, s->H);
        build_tree(*s);
        return s;
    } catch (const std::exception& e) {
        if (err && errlen > 0) snprintf(err, errlen, "%s", e.what());
    }
    return nullptr;
}
void orc_close(void* h) { delete static_cast<Scene*>(h); }
int orc_num_objects(void* h) { return (int)static_cast<Scene*>(h)->objs.size(); }
int orc_num_lights(void* h) { return (int)static_cast<Scene*>(h)->lights.size(); }
void orc_bvh_order(void* h, int* out) { auto* s = static_cast<Scene*>(h); for (size_t i = 0; i < s->order.size(); i++) out[i] = s->order[i]; }
int orc_bvh_nodes(void* h, float* bounds, int* a, int* axis) {
    auto* s = static_cast<Scene*>(h);
    if (bounds)
        for (int i = 1; i <= s->tot; i++) {
            const Node& n = s->nodes[i];
            for (int k = 0; k < 3; k++) { bounds[6 * (i - 1) + k] = n.b.mn[k]; bounds[6 * (i - 1) + 3 + k] = n.b.mx[k]; }
            a[2 * (i - 1)] = n.a; a[2 * (i - 1) + 1] = n.c; axis[i - 1] = n.axis;
        }
    return s->tot;
}
void orc_halton(int W, int H, int n, const int* px, const int* py, const int* sample, int ndim, float* out) {
    Scene s;
    halton_setup(s, W, H);
    for (int i = 0; i < n; i++) {
        int v = halton_index(s, px[i], py[i], sample[i]);
        for (int d = 0; d < ndim; d++) out[(size_t)i * ndim + d] = halton_value(s, v, d, (uint32_t)(py[i] * W + px[i]), (uint32_t)sample[i], 0);
    }
}
void orc_camera(void* h, int n, const float* pos2, float* o, float* d) {
    auto* s = static_cast<Scene*>(h);
    for (int i = 0; i < n; i++) {
        Ray r = camera_ray(*s, pos2[2 * i], pos2[2 * i + 1]);
        for (int k = 0; k < 3; k++) { o[3 * i + k] = r.o[k]; d[3 * i + k] = r.d[k]; }
    }
}
void orc_intersect(void* h, int n, const float* o, const float* d, int* obj, float* t) {
    auto* s = static_cast<Scene*>(h);
    for (int i = 0; i < n; i++) {
        Hit hh;
        bool hit = intersect(*s, Ray{V3(o[3 * i], o[3 * i + 1], o[3 * i + 2]), V3(d[3 * i], d[3 * i + 1], d[3 * i + 2])}, hh);
        obj[i] = hit ? hh.obj : -1;
        t[i] = hit ? hh.t : std::numeric_limits<float>::infinity();
    }
}
void orc_intersect_test(void* h, int n, const float* o, const float* d, const float* tmin, const float* tmax, const int* ign, int* occ) {
    auto* s = static_cast<Scene*>(h);
    for (int i = 0; i < n; i++)
        occ[i] = intersect_test(*s, Ray{V3(o[3 * i], o[3 * i + 1], o[3 * i + 2]), V3(d[3 * i], d[3 * i + 1], d[3 * i + 2])},
                                tmin[i], tmax[i], ign ? ign[i] : -1) ? 1 : 0;
}
// Per-pixel sum and sum of squares over [x0,x1)x[y0,y1) at samples [s0, s0+ns) (NaN/Inf -> 0).
// Default / Stratified samplers run whole tiles (the stream of a tile is sequential) and need
// s0 = 0, ns = spp; returns -1 otherwise.
double orc_render_region(void* h, int threads, int x0, int y0, int x1, int y1, int s0, int ns, unsigned long long seed,
                         double* sum, double* sumsq) {
    auto* s = static_cast<Scene*>(h);
    int rw = x1 - x0;
    auto t0 = std::chrono::steady_clock::now();
    if (s->sampler != 0 && !s->counter) {
        if (s0 != 0 || ns != s->spp) return -1.0;
        std::memset(sum, 0, sizeof(double) * 3 * (size_t)rw * (y1 - y0));
        std::memset(sumsq, 0, sizeof(double) * 3 * (size_t)rw * (y1 - y0));
        const int ntx = (s->W + 31) / 32, nty = (s->H + 31) / 32;
        parallel_for(ntx * nty, threads, [&](int t) {
            const int tx = t / nty, ty = t % nty;
            if (32 * tx >= x1 || 32 * tx + 32 <= x0 || 32 * ty >= y1 || 32 * ty + 32 <= y0) return;
            run_tile(*s, tx, ty, [&](int x, int y, int, V3 c) {
                if (x < x0 || x >= x1 || y < y0 || y >= y1) return;
                if (bad(c)) c = V3();
                size_t idx = (size_t)(y - y0) * rw + (x - x0);
                for (int j = 0; j < 3; j++) { sum[3 * idx + j] += c[j]; sumsq[3 * idx + j] += (double)c[j] * c[j]; }
            });
        });
        return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
    parallel_for(y1 - y0, threads, [&](int r) {
        const int y = y0 + r;
        for (int x = x0; x < x1; x++) {
            double a[3] = {0, 0, 0}, q[3] = {0, 0, 0};
            for (int k = 0; k < ns; k++) {
                int sample = s0 + k;
                Sampler smp{*s, halton_index(*s, x, y, sample), (uint32_t)(y * s->W + x), (uint32_t)sample, seed};
                V3 c = trace_sample(*s, smp, x, y);
                if (bad(c)) c = V3();
                for (int j = 0; j < 3; j++) { a[j] += c[j]; q[j] += (double)c[j] * c[j]; }
            }
            size_t idx = (size_t)r * rw + (x - x0);
            for (int j = 0; j < 3; j++) { sum[3 * idx + j] = a[j]; sumsq[3 * idx + j] = q[j]; }
        }
    });
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

// The whole frame as FrameBuffer holds it (FrameBuffer.cpp:20-32): per pixel a float sum of the
// samples in sampling order (NaN/Inf -> 0) and a float weight; rgbw[4 * (y * W + x) + c].
void orc_render_frame(void* h, int threads, float* rgbw) {
    auto* s = static_cast<Scene*>(h);
    std::memset(rgbw, 0, sizeof(float) * 4 * (size_t)s->W * s->H);
    auto add = [&](int x, int y, V3 c) {
        if (bad(c)) c = V3();
        float* p = rgbw + 4 * ((size_t)y * s->W + x);
        p[0] += c.x; p[1] += c.y; p[2] += c.z; p[3] += 1.f;
    };
    const int ntx = (s->W + 31) / 32, nty = (s->H + 31) / 32;
    parallel_for(ntx * nty, threads, [&](int t) {
        const int tx = t / nty, ty = t % nty;
        if (s->sampler != 0 && !s->counter) { run_tile(*s, tx, ty, [&](int x, int y, int, V3 c) { add(x, y, c); }); return; }
        for (int x = 32 * tx; x < std::min(32 * tx + 32, s->W); x++)
            for (int y = 32 * ty; y < std::min(32 * ty + 32, s->H); y++)
                for (int k = 0; k < s->spp; k++) {
                    Sampler smp{*s, halton_index(*s, x, y, k), (uint32_t)(y * s->W + x), (uint32_t)k, 0};
                    add(x, y, trace_sample(*s, smp, x, y));
                }
    });
}

// 0: Default / Stratified follow the reference's tile streams; 1: the library's per-draw values.
void orc_set_counter_sampler(void* h, int on) { static_cast<Scene*>(h)->counter = on != 0; }

// Per-sample radiance of pixels (px, py) for samples 0..spp-1: out[(p*spp+s)*3+c].
void orc_render_samples(void* h, int n, const int* px, const int* py, int spp, unsigned long long seed, float* out) {
    auto* s = static_cast<Scene*>(h);
    if (s->sampler != 0 && !s->counter) {
        const int nty = (s->H + 31) / 32;
        std::map<int, std::vector<int>> tiles;  // tile -> requested pixel slots
        for (int p = 0; p < n; p++) tiles[(px[p] / 32) * nty + py[p] / 32].push_back(p);
        for (auto& kv : tiles)
            run_tile(*s, kv.first / nty, kv.first % nty, [&](int x, int y, int k, V3 c) {
                for (int p : kv.second)
                    if (px[p] == x && py[p] == y && k < spp)
                        for (int j = 0; j < 3; j++) out[((size_t)p * spp + k) * 3 + j] = c[j];
            });
        return;
    }
    for (int p = 0; p < n; p++)
        for (int k = 0; k < spp; k++) {
            Sampler smp{*s, halton_index(*s, px[p], py[p], k), (uint32_t)(py[p] * s->W + px[p]), (uint32_t)k, seed};
            V3 c = trace_sample(*s, smp, px[p], py[p]);
            for (int j = 0; j < 3; j++) out[((size_t)p * spp + k) * 3 + j] = c[j];
        }
}
int orc_bsdf(const char* kind, const float* params, int front, const float* frame, int n, const float* wo, const float* wi,
             const float* u3, int flags, float* f_eval, float* pdf_eval, float* f_samp, float* wi_samp, float* pdf_samp, int* type_samp) {
    // params: color(3), ks(3), ax, ay, ior
    Mat m;
    std::string k = kind;
    if (k == "Diffuse") m.type = M_DIFF;
    else if (k == "Mirror") m.type = M_MIRROR;
    else if (k == "GlassRough") m.type = M_GLASS_R;
    else if (k == "GlassSmooth") m.type = M_GLASS_S;
    else if (k == "MicroGGX") m.type = M_MICRO_GGX;
    else if (k == "MicroBeckmann") m.type = M_MICRO_BECK;
    else if (k == "PlasticGGX") m.type = M_PLAST_GGX;
    else if (k == "PlasticBeckmann") m.type = M_PLAST_BECK;
    else if (k == "OrenNayar") m.type = M_OREN;
    else if (k == "Phong") m.type = M_PHONG;
    else return -1;
    m.R = V3(params[0], params[1], params[2]); m.S = V3(params[3], params[4], params[5]);
    m.ax = params[6]; m.ay = params[7]; m.ior = params[8];
    BxDF b = make_bxdf(m, front != 0);
    Frame fr{V3(frame[3], frame[4], frame[5]), V3(frame[0], frame[1], frame[2]), V3(frame[6], frame[7], frame[8])};
    for (int i = 0; i < n; i++) {
        V3 o(wo[3 * i], wo[3 * i + 1], wo[3 * i + 2]), w(wi[3 * i], wi[3 * i + 1], wi[3 * i + 2]);
        V3 f = bsdf_f(b, fr, o, w);
        for (int j = 0; j < 3; j++) f_eval[3 * i + j] = f[j];
        pdf_eval[i] = bsdf_pdf(b, fr, o, w, flags);
        V3 ws;
        float pdf = 0;
        int st = 0;
        V3 fs = bsdf_sample(b, fr, u3[3 * i], u3[3 * i + 1], u3[3 * i + 2], o, ws, pdf, flags, st);
        for (int j = 0; j < 3; j++) { f_samp[3 * i + j] = fs[j]; wi_samp[3 * i + j] = ws[j]; }
        pdf_samp[i] = pdf;
        type_samp[i] = st;
    }
    return 1;
}

}  // extern "C"
