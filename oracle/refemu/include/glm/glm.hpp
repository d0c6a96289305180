// The subset of glm (the header-only vector library the reference solver is written
// against) that Velvet/VtClothSolverGPU.cu, Velvet/VtClothSolverGPU.cuh and
// Velvet/SpatialHashGPU.cu use — TEST INFRASTRUCTURE for compiling those files on the
// CPU.  glm itself is not in this image and the reference pins no version of it; this is
// our own code with glm's documented semantics: component-wise float arithmetic,
// column-major matrices, and glm's evaluation order —
//   dot(a, b)        (a.x*b.x + a.y*b.y) + a.z*b.z
//   length(v)        sqrt(dot(v, v));  normalize(v) = v * (1 / sqrt(dot(v, v)))
//   mat4 * vec4      (c0*x + c1*y) + (c2*z + c3*w)
//   mat3 * vec3      (c0*x + c1*y) + c2*z
//   mat4 * mat4      column j = ((A0*B[j].x + A1*B[j].y) + A2*B[j].z) + A3*B[j].w
//   clamp(x, lo, hi) min(max(x, lo), hi), max(a, b) = (a < b) ? b : a, min(a, b) = (b < a) ? b : a
// These are the orders the oracle assumes too, so glm's own arithmetic stays unpinned.
#pragma once

#include <cmath>

namespace glm {

struct vec4;

struct vec3 {
    float x, y, z;
    vec3() : x(0), y(0), z(0) {}
    explicit vec3(float s) : x(s), y(s), z(s) {}
    vec3(float a, float b, float c) : x(a), y(b), z(c) {}
    vec3(const vec4& v);  // glm converts vec4 -> vec3 implicitly (drops w)
    float& operator[](int i) { return (&x)[i]; }
    const float& operator[](int i) const { return (&x)[i]; }
    vec3& operator+=(const vec3& b) { x = x + b.x; y = y + b.y; z = z + b.z; return *this; }
    vec3& operator-=(const vec3& b) { x = x - b.x; y = y - b.y; z = z - b.z; return *this; }
    vec3& operator*=(float s) { x = x * s; y = y * s; z = z * s; return *this; }
    vec3& operator/=(float s) { x = x / s; y = y / s; z = z / s; return *this; }
};

struct vec4 {
    float x, y, z, w;
    vec4() : x(0), y(0), z(0), w(0) {}
    explicit vec4(float s) : x(s), y(s), z(s), w(s) {}
    vec4(float a, float b, float c, float d) : x(a), y(b), z(c), w(d) {}
    vec4(const vec3& v, float d) : x(v.x), y(v.y), z(v.z), w(d) {}
    float& operator[](int i) { return (&x)[i]; }
    const float& operator[](int i) const { return (&x)[i]; }
};

inline vec3::vec3(const vec4& v) : x(v.x), y(v.y), z(v.z) {}

inline vec3 operator+(const vec3& a, const vec3& b) { return vec3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline vec3 operator-(const vec3& a, const vec3& b) { return vec3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline vec3 operator-(const vec3& a) { return vec3(-a.x, -a.y, -a.z); }
inline vec3 operator*(const vec3& a, const vec3& b) { return vec3(a.x * b.x, a.y * b.y, a.z * b.z); }
inline vec3 operator*(const vec3& a, float s) { return vec3(a.x * s, a.y * s, a.z * s); }
inline vec3 operator*(float s, const vec3& a) { return vec3(s * a.x, s * a.y, s * a.z); }
inline vec3 operator/(const vec3& a, float s) { return vec3(a.x / s, a.y / s, a.z / s); }
inline vec3 operator/(float s, const vec3& a) { return vec3(s / a.x, s / a.y, s / a.z); }

// column-major: c[j] is column j
struct mat3 {
    vec3 c[3];
    vec3& operator[](int j) { return c[j]; }
    const vec3& operator[](int j) const { return c[j]; }
};
struct mat4 {
    vec4 c[4];
    vec4& operator[](int j) { return c[j]; }
    const vec4& operator[](int j) const { return c[j]; }
};

inline float dot(const vec3& a, const vec3& b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
inline vec3 cross(const vec3& a, const vec3& b)
{
    return vec3(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}
inline float length(const vec3& v) { return std::sqrt(dot(v, v)); }
inline float inversesqrt(float x) { return 1.0f / std::sqrt(x); }
inline vec3 normalize(const vec3& v) { return v * inversesqrt(dot(v, v)); }
inline float max(float a, float b) { return (a < b) ? b : a; }
inline float min(float a, float b) { return (b < a) ? b : a; }
inline float clamp(float x, float lo, float hi) { return min(max(x, lo), hi); }
inline vec3 abs(const vec3& v) { return vec3(std::fabs(v.x), std::fabs(v.y), std::fabs(v.z)); }

inline vec4 operator*(const mat4& m, const vec4& v)
{
    vec4 r;
    for (int i = 0; i < 4; ++i)
        r[i] = (m.c[0][i] * v.x + m.c[1][i] * v.y) + (m.c[2][i] * v.z + m.c[3][i] * v.w);
    return r;
}
inline mat4 operator*(const mat4& a, const mat4& b)
{
    mat4 r;
    for (int j = 0; j < 4; ++j)
        for (int i = 0; i < 4; ++i)
            r.c[j][i] = ((a.c[0][i] * b.c[j].x + a.c[1][i] * b.c[j].y) + a.c[2][i] * b.c[j].z) + a.c[3][i] * b.c[j].w;
    return r;
}
inline mat3 operator*(const mat3& m, float s)
{
    mat3 r;
    for (int j = 0; j < 3; ++j) r.c[j] = m.c[j] * s;
    return r;
}
inline vec3 operator*(const mat3& m, const vec3& v)
{
    vec3 r;
    for (int i = 0; i < 3; ++i) r[i] = (m.c[0][i] * v.x + m.c[1][i] * v.y) + m.c[2][i] * v.z;
    return r;
}

}  // namespace glm
