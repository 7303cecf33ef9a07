// Small float vector/matrix helpers for the host side of the scene build.
//
// Scene preprocessing (mesh transforms, normals, camera basis, quadric rotations) must produce
// the same float bits as the reference, which does this work with glm 0.9.9.8.  Every helper
// below therefore performs its arithmetic in the operation order glm uses (noted per function);
// the host library is compiled with -ffp-contract=off so no FMA changes the rounding.
#pragma once
#include <cmath>

namespace c2g {
namespace fm {

constexpr float kPi = 3.14159265358979323846264338327950288f;
constexpr float kTwoPi = 6.28318530717958647692528676655900576f;
constexpr float kHalfPi = 1.57079632679489661923132169163975144f;

struct V3 {
    float x = 0, y = 0, z = 0;
    V3() = default;
    V3(float a, float b, float c) : x(a), y(b), z(c) {}
    float& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
    float operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};
struct V4 {
    float x = 0, y = 0, z = 0, w = 0;
    V4() = default;
    V4(float a, float b, float c, float d) : x(a), y(b), z(c), w(d) {}
    float& operator[](int i) { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }
    float operator[](int i) const { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }
};

inline V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 operator-(V3 a) { return {-a.x, -a.y, -a.z}; }
inline V3 operator*(V3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
inline V3 operator*(float s, V3 a) { return {s * a.x, s * a.y, s * a.z}; }
inline V3 operator*(V3 a, V3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
inline V3 operator/(V3 a, float s) { return {a.x / s, a.y / s, a.z / s}; }
inline V3 operator-(V3 a, float s) { return {a.x - s, a.y - s, a.z - s}; }
inline V3 operator+(V3 a, float s) { return {a.x + s, a.y + s, a.z + s}; }
inline V4 operator+(V4 a, V4 b) { return {a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w}; }
inline V4 operator-(V4 a, V4 b) { return {a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w}; }
inline V4 operator*(V4 a, float s) { return {a.x * s, a.y * s, a.z * s, a.w * s}; }
inline V4 operator*(V4 a, V4 b) { return {a.x * b.x, a.y * b.y, a.z * b.z, a.w * b.w}; }

// glm dot: (x*x' + y*y') + z*z' (func_geometric.inl compute_dot via a component product)
inline float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cross(V3 a, V3 b) {
    return {a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y};
}
// glm normalize: v * (1 / sqrt(dot(v, v)))
inline V3 normalize(V3 v) {
    float inv = 1.0f / std::sqrt(dot(v, v));
    return v * inv;
}
inline float length(V3 v) { return std::sqrt(dot(v, v)); }
inline bool is_zero(V3 v) { return v.x == 0.f && v.y == 0.f && v.z == 0.f; }

// Column-major 3x3 / 4x4 (m[c] is column c), like glm::mat.
struct M3 {
    V3 c[3];
    V3& operator[](int i) { return c[i]; }
    const V3& operator[](int i) const { return c[i]; }
};
struct M4 {
    V4 c[4];
    V4& operator[](int i) { return c[i]; }
    const V4& operator[](int i) const { return c[i]; }
};

inline M4 identity4() {
    M4 m;
    m[0] = {1, 0, 0, 0}; m[1] = {0, 1, 0, 0}; m[2] = {0, 0, 1, 0}; m[3] = {0, 0, 0, 1};
    return m;
}

// glm::translate: Result[3] = m[0]*v[0] + m[1]*v[1] + m[2]*v[2] + m[3] (left to right)
inline M4 translate(const M4& m, V3 v) {
    M4 r = m;
    r[3] = m[0] * v.x + m[1] * v.y + m[2] * v.z + m[3];
    return r;
}
// glm::rotate (ext/matrix_transform.inl)
inline M4 rotate(const M4& m, float angle, V3 v) {
    float c = std::cos(angle), s = std::sin(angle);
    V3 axis = normalize(v);
    V3 temp = (1.0f - c) * axis;
    float R[3][3];
    R[0][0] = c + temp[0] * axis[0];
    R[0][1] = temp[0] * axis[1] + s * axis[2];
    R[0][2] = temp[0] * axis[2] - s * axis[1];
    R[1][0] = temp[1] * axis[0] - s * axis[2];
    R[1][1] = c + temp[1] * axis[1];
    R[1][2] = temp[1] * axis[2] + s * axis[0];
    R[2][0] = temp[2] * axis[0] + s * axis[1];
    R[2][1] = temp[2] * axis[1] - s * axis[0];
    R[2][2] = c + temp[2] * axis[2];
    M4 r;
    r[0] = m[0] * R[0][0] + m[1] * R[0][1] + m[2] * R[0][2];
    r[1] = m[0] * R[1][0] + m[1] * R[1][1] + m[2] * R[1][2];
    r[2] = m[0] * R[2][0] + m[1] * R[2][1] + m[2] * R[2][2];
    r[3] = m[3];
    return r;
}
inline M4 scale(const M4& m, V3 v) {
    M4 r;
    r[0] = m[0] * v.x; r[1] = m[1] * v.y; r[2] = m[2] * v.z; r[3] = m[3];
    return r;
}
// glm mat4 * vec4: (m0*v0 + m1*v1) + (m2*v2 + m3*v3)
inline V4 mul(const M4& m, V4 v) {
    V4 a0 = m[0] * v.x + m[1] * v.y;
    V4 a1 = m[2] * v.z + m[3] * v.w;
    return a0 + a1;
}
// glm mat3 * vec3: per row, left to right
inline V3 mul(const M3& m, V3 v) {
    return {m[0][0] * v.x + m[1][0] * v.y + m[2][0] * v.z,
            m[0][1] * v.x + m[1][1] * v.y + m[2][1] * v.z,
            m[0][2] * v.x + m[1][2] * v.y + m[2][2] * v.z};
}
inline M3 mat3_of(const M4& m) {
    M3 r;
    for (int i = 0; i < 3; i++) r[i] = {m[i].x, m[i].y, m[i].z};
    return r;
}
inline M3 transpose(const M3& m) {
    M3 r;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) r[i][j] = m[j][i];
    return r;
}
inline M4 transpose(const M4& m) {
    M4 r;
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) r[i][j] = m[j][i];
    return r;
}
// glm::inverse(mat4): cofactor expansion (detail/func_matrix.inl compute_inverse<4,4>).
inline M4 inverse(const M4& m) {
    float c00 = m[2][2] * m[3][3] - m[3][2] * m[2][3];
    float c02 = m[1][2] * m[3][3] - m[3][2] * m[1][3];
    float c03 = m[1][2] * m[2][3] - m[2][2] * m[1][3];
    float c04 = m[2][1] * m[3][3] - m[3][1] * m[2][3];
    float c06 = m[1][1] * m[3][3] - m[3][1] * m[1][3];
    float c07 = m[1][1] * m[2][3] - m[2][1] * m[1][3];
    float c08 = m[2][1] * m[3][2] - m[3][1] * m[2][2];
    float c10 = m[1][1] * m[3][2] - m[3][1] * m[1][2];
    float c11 = m[1][1] * m[2][2] - m[2][1] * m[1][2];
    float c12 = m[2][0] * m[3][3] - m[3][0] * m[2][3];
    float c14 = m[1][0] * m[3][3] - m[3][0] * m[1][3];
    float c15 = m[1][0] * m[2][3] - m[2][0] * m[1][3];
    float c16 = m[2][0] * m[3][2] - m[3][0] * m[2][2];
    float c18 = m[1][0] * m[3][2] - m[3][0] * m[1][2];
    float c19 = m[1][0] * m[2][2] - m[2][0] * m[1][2];
    float c20 = m[2][0] * m[3][1] - m[3][0] * m[2][1];
    float c22 = m[1][0] * m[3][1] - m[3][0] * m[1][1];
    float c23 = m[1][0] * m[2][1] - m[2][0] * m[1][1];
    V4 f0(c00, c00, c02, c03), f1(c04, c04, c06, c07), f2(c08, c08, c10, c11);
    V4 f3(c12, c12, c14, c15), f4(c16, c16, c18, c19), f5(c20, c20, c22, c23);
    V4 v0(m[1][0], m[0][0], m[0][0], m[0][0]);
    V4 v1(m[1][1], m[0][1], m[0][1], m[0][1]);
    V4 v2(m[1][2], m[0][2], m[0][2], m[0][2]);
    V4 v3(m[1][3], m[0][3], m[0][3], m[0][3]);
    V4 i0 = v1 * f0 - v2 * f1 + v3 * f2;
    V4 i1 = v0 * f0 - v2 * f3 + v3 * f4;
    V4 i2 = v0 * f1 - v1 * f3 + v3 * f5;
    V4 i3 = v0 * f2 - v1 * f4 + v2 * f5;
    V4 sa(1, -1, 1, -1), sb(-1, 1, -1, 1);
    M4 inv;
    inv[0] = i0 * sa; inv[1] = i1 * sb; inv[2] = i2 * sa; inv[3] = i3 * sb;
    V4 row0(inv[0][0], inv[1][0], inv[2][0], inv[3][0]);
    V4 d0 = m[0] * row0;
    float d1 = (d0.x + d0.y) + (d0.z + d0.w);
    float ood = 1.0f / d1;
    M4 r;
    for (int i = 0; i < 4; i++) r[i] = inv[i] * ood;
    return r;
}
// glm::inverse(mat2) (compute_inverse<2,2>): OneOverDeterminant = 1 / (m00*m11 - m10*m01)
struct M2 { float m[2][2]; };
inline M2 inverse(const M2& a) {
    float ood = 1.0f / (a.m[0][0] * a.m[1][1] - a.m[1][0] * a.m[0][1]);
    M2 r;
    r.m[0][0] = +a.m[1][1] * ood;
    r.m[0][1] = -a.m[0][1] * ood;
    r.m[1][0] = -a.m[1][0] * ood;
    r.m[1][1] = +a.m[0][0] * ood;
    return r;
}

}  // namespace fm
}  // namespace c2g
