// glsl_shim.hpp -- TEST INFRASTRUCTURE.  Just enough of GLSL 4.30's types and built-in functions, in
// C++, for the reference's compute shaders (voxelShared.comp, voxelLighting.comp, voxelDraw.comp) to be
// compiled as C++ after oracle/ref/glsl_to_cpp.py has rewritten their few non-C++ constructs.
//
// Semantics follow the GLSL specification where it defines them, and the choices of the CPU oracle
// where it leaves them to the implementation:
//   * float literals and arithmetic are single precision, each operation rounded on its own (the
//     translation units are compiled with -ffp-contract=off);
//   * min(x, y) = y < x ? y : x, max(x, y) = x < y ? y : x, clamp = min(max(x, lo), hi),
//     mix(x, y, a) = x*(1-a) + y*a, normalize(v) = v / sqrt(dot(v, v)), reflect / refract by their
//     specification formulas, fract(x) = x - floor(x);
//   * float -> int conversion truncates, saturates, and maps NaN to 0;
//   * sin() is the oracle's deterministic sine (dno_sin), the one the oracle's reference-RNG mode uses;
//   * matrix products sum over k in ascending order.
// Swizzles are member functions (.xyz() instead of .xyz); the translator rewrites them.
#pragma once
#include <cmath>
#include <cstdint>
#include <climits>
#include <cstring>

extern "C" float dno_sin(float x);

namespace glsl {

typedef unsigned int uint;

inline int f2i(float x)
{
    if (x != x) return 0;
    if (x >= 2147483648.0f) return INT_MAX;
    if (x < -2147483648.0f) return INT_MIN;
    return (int)x;
}
inline uint f2u(float x) { return (uint)f2i(x); }

struct vec2; struct vec3; struct vec4; struct ivec2; struct ivec3; struct uvec2; struct uvec3; struct uvec4;
struct bvec3;

struct bvec3 { bool x, y, z; };

struct uvec2 { uint x, y; uvec2() : x(0), y(0) {} uvec2(uint a, uint b) : x(a), y(b) {} };

struct ivec2 {
    int x, y;
    ivec2() : x(0), y(0) {}
    ivec2(int a, int b) : x(a), y(b) {}
    explicit ivec2(const uvec2& v) : x((int)v.x), y((int)v.y) {}
};

struct uvec3 {
    uint x, y, z;
    uvec3() : x(0), y(0), z(0) {}
    uvec3(uint a, uint b, uint c) : x(a), y(b), z(c) {}
    explicit uvec3(const vec3& v);
    uvec2 xy() const { return uvec2(x, y); }
};

struct ivec3 {
    int x, y, z;
    ivec3() : x(0), y(0), z(0) {}
    ivec3(int a, int b, int c) : x(a), y(b), z(c) {}
    explicit ivec3(const vec3& v);
    explicit ivec3(const bvec3& b) : x(b.x), y(b.y), z(b.z) {}
    ivec3 xyz() const { return *this; }
    ivec3& operator+=(const ivec3& o) { x += o.x; y += o.y; z += o.z; return *this; }
};
inline ivec3 operator+(const ivec3& a, const ivec3& b) { return ivec3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline ivec3 operator*(const ivec3& a, const ivec3& b) { return ivec3(a.x * b.x, a.y * b.y, a.z * b.z); }
inline ivec3 operator-(const ivec3& a) { return ivec3(-a.x, -a.y, -a.z); }

struct uvec4 {
    uint x, y, z, w;
    uvec4() : x(0), y(0), z(0), w(0) {}
    uvec4(uint a, uint b, uint c, uint d) : x(a), y(b), z(c), w(d) {}
    uvec4(const vec3& v, float d);
    uvec4(const vec2& v, uint c, uint d);
    uvec3 yzw() const { return uvec3(y, z, w); }
    uvec3 xyz() const { return uvec3(x, y, z); }
    uvec2 xy() const { return uvec2(x, y); }
};
inline uvec4 operator&(const uvec4& a, uint m) { return uvec4(a.x & m, a.y & m, a.z & m, a.w & m); }
inline uvec3 operator<<(const uvec3& a, int s) { return uvec3(a.x << s, a.y << s, a.z << s); }
inline uvec3 operator|(const uvec3& a, const uvec3& b) { return uvec3(a.x | b.x, a.y | b.y, a.z | b.z); }
inline uvec3 operator&(const uvec3& a, uint m) { return uvec3(a.x & m, a.y & m, a.z & m); }
inline uvec3 operator>>(const uvec3& a, int s) { return uvec3(a.x >> s, a.y >> s, a.z >> s); }

struct vec2 {
    float x, y;
    vec2() : x(0), y(0) {}
    vec2(float a, float b) : x(a), y(b) {}
    explicit vec2(float a) : x(a), y(a) {}
    vec2(const ivec2& v) : x((float)v.x), y((float)v.y) {}
    vec2(const uvec2& v) : x((float)v.x), y((float)v.y) {}
};
inline vec2 operator/(const vec2& a, const vec2& b) { return vec2(a.x / b.x, a.y / b.y); }
inline vec2 operator*(const vec2& a, float s) { return vec2(a.x * s, a.y * s); }
inline vec2 operator-(const vec2& a, float s) { return vec2(a.x - s, a.y - s); }

struct vec3 {
    float x, y, z;
    vec3() : x(0), y(0), z(0) {}
    vec3(float a, float b, float c) : x(a), y(b), z(c) {}
    explicit vec3(float a) : x(a), y(a), z(a) {}
    vec3(const ivec3& v) : x((float)v.x), y((float)v.y), z((float)v.z) {}
    vec3(const uvec3& v) : x((float)v.x), y((float)v.y), z((float)v.z) {}
    explicit vec3(const bvec3& b) : x(b.x ? 1.0f : 0.0f), y(b.y ? 1.0f : 0.0f), z(b.z ? 1.0f : 0.0f) {}
    vec3(float a, const vec2& v) : x(a), y(v.x), z(v.y) {}
    vec3(uint a, const uvec2& v) : x((float)a), y((float)v.x), z((float)v.y) {}
    vec3 xyz() const { return *this; }
    vec3 yzx() const { return vec3(y, z, x); }
    vec3 zxy() const { return vec3(z, x, y); }
    vec2 yz() const { return vec2(y, z); }
    vec2 xy() const { return vec2(x, y); }
    vec3& operator+=(const vec3& o) { x = x + o.x; y = y + o.y; z = z + o.z; return *this; }
    vec3& operator*=(const vec3& o) { x = x * o.x; y = y * o.y; z = z * o.z; return *this; }
    vec3& operator*=(float s) { x = x * s; y = y * s; z = z * s; return *this; }
    vec3& operator/=(float s) { x = x / s; y = y / s; z = z / s; return *this; }
};
inline vec3 operator+(const vec3& a, const vec3& b) { return vec3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline vec3 operator-(const vec3& a, const vec3& b) { return vec3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline vec3 operator*(const vec3& a, const vec3& b) { return vec3(a.x * b.x, a.y * b.y, a.z * b.z); }
inline vec3 operator/(const vec3& a, const vec3& b) { return vec3(a.x / b.x, a.y / b.y, a.z / b.z); }
inline vec3 operator+(const vec3& a, float s) { return vec3(a.x + s, a.y + s, a.z + s); }
inline vec3 operator-(const vec3& a, float s) { return vec3(a.x - s, a.y - s, a.z - s); }
inline vec3 operator*(const vec3& a, float s) { return vec3(a.x * s, a.y * s, a.z * s); }
inline vec3 operator*(float s, const vec3& a) { return vec3(s * a.x, s * a.y, s * a.z); }
inline vec3 operator/(const vec3& a, float s) { return vec3(a.x / s, a.y / s, a.z / s); }
inline vec3 operator/(float s, const vec3& a) { return vec3(s / a.x, s / a.y, s / a.z); }
inline vec3 operator-(const vec3& a) { return vec3(-a.x, -a.y, -a.z); }
inline bool operator==(const vec3& a, const vec3& b) { return a.x == b.x && a.y == b.y && a.z == b.z; }

inline ivec3::ivec3(const vec3& v) : x(f2i(v.x)), y(f2i(v.y)), z(f2i(v.z)) {}
inline uvec3::uvec3(const vec3& v) : x(f2u(v.x)), y(f2u(v.y)), z(f2u(v.z)) {}

struct vec4 {
    float x, y, z, w;
    vec4() : x(0), y(0), z(0), w(0) {}
    vec4(float a, float b, float c, float d) : x(a), y(b), z(c), w(d) {}
    vec4(const vec3& v, float d) : x(v.x), y(v.y), z(v.z), w(d) {}
    vec4(const vec2& v, float c, float d) : x(v.x), y(v.y), z(c), w(d) {}
    vec3 xyz() const { return vec3(x, y, z); }
    vec4& operator/=(float s) { x = x / s; y = y / s; z = z / s; w = w / s; return *this; }
};

inline uvec4::uvec4(const vec3& v, float d) : x(f2u(v.x)), y(f2u(v.y)), z(f2u(v.z)), w(f2u(d)) {}
inline uvec4::uvec4(const vec2& v, uint c, uint d) : x(f2u(v.x)), y(f2u(v.y)), z(c), w(d) {}

struct mat4 {
    float m[4][4];   // column-major m[col][row]
};
inline mat4 operator*(const mat4& a, const mat4& b)
{
    mat4 r;
    for (int c = 0; c < 4; c++)
        for (int row = 0; row < 4; row++)
            r.m[c][row] = a.m[0][row] * b.m[c][0] + a.m[1][row] * b.m[c][1] + a.m[2][row] * b.m[c][2] + a.m[3][row] * b.m[c][3];
    return r;
}
inline vec4 operator*(const mat4& a, const vec4& v)
{
    float o[4];
    for (int row = 0; row < 4; row++) o[row] = a.m[0][row] * v.x + a.m[1][row] * v.y + a.m[2][row] * v.z + a.m[3][row] * v.w;
    return vec4(o[0], o[1], o[2], o[3]);
}

// ---- built-in functions
inline float min(float a, float b) { return (b < a) ? b : a; }
inline float max(float a, float b) { return (a < b) ? b : a; }
inline uint min(uint a, uint b) { return (b < a) ? b : a; }
inline vec3 min(const vec3& a, const vec3& b) { return vec3(min(a.x, b.x), min(a.y, b.y), min(a.z, b.z)); }
inline vec3 max(const vec3& a, const vec3& b) { return vec3(max(a.x, b.x), max(a.y, b.y), max(a.z, b.z)); }
inline vec3 clamp(const vec3& v, const vec3& lo, const vec3& hi) { return min(max(v, lo), hi); }
inline float dot(const vec3& a, const vec3& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline float length(const vec3& v) { return std::sqrt(dot(v, v)); }
inline float distance(const vec3& a, const vec3& b) { return length(a - b); }
inline vec3 normalize(const vec3& v) { return v / std::sqrt(dot(v, v)); }
inline vec3 reflect(const vec3& i, const vec3& n) { return i - n * (2.0f * dot(n, i)); }
inline vec3 refract(const vec3& i, const vec3& n, float eta)
{
    float d = dot(n, i);
    float k = 1.0f - eta * eta * (1.0f - d * d);
    if (k < 0.0f) return vec3(0.0f);
    return i * eta - n * (eta * d + std::sqrt(k));
}
inline float sgn1(float x) { return x > 0.0f ? 1.0f : (x < 0.0f ? -1.0f : 0.0f); }
inline vec3 sign(const vec3& v) { return vec3(sgn1(v.x), sgn1(v.y), sgn1(v.z)); }
inline vec3 abs(const vec3& v) { return vec3(std::fabs(v.x), std::fabs(v.y), std::fabs(v.z)); }
inline vec3 floor(const vec3& v) { return vec3(std::floor(v.x), std::floor(v.y), std::floor(v.z)); }
inline vec3 trunc(const vec3& v) { return vec3(std::trunc(v.x), std::trunc(v.y), std::trunc(v.z)); }
inline vec3 round(const vec3& v) { return vec3(std::round(v.x), std::round(v.y), std::round(v.z)); }
inline vec2 round(const vec2& v) { return vec2(std::round(v.x), std::round(v.y)); }
inline float round(float v) { return std::round(v); }
inline float fract(float x) { return x - std::floor(x); }
inline float sin(float x) { return dno_sin(x); }
inline vec3 pow(const vec3& a, const vec3& b) { return vec3(powf(a.x, b.x), powf(a.y, b.y), powf(a.z, b.z)); }
inline vec3 mix(const vec3& a, const vec3& b, float t) { return vec3(a.x * (1.0f - t) + b.x * t, a.y * (1.0f - t) + b.y * t, a.z * (1.0f - t) + b.z * t); }
inline bvec3 lessThanEqual(const vec3& a, const vec3& b) { return bvec3{a.x <= b.x, a.y <= b.y, a.z <= b.z}; }
inline uint bitCount(uint v) { return (uint)__builtin_popcount(v); }

// ---- buffers, images and samplers
template <class T> struct gbuf {
    T* p = nullptr;
    size_t n = 0;
    T dummy{};
    T& operator[](size_t i) { if (i < n) return p[i]; dummy = T{}; return dummy; }
};
struct image2D { vec4* px = nullptr; int w = 0, h = 0; };
struct sampler2D { int unused = 0; };
struct samplerCube { int unused = 0; };
inline ivec2 imageSize(const image2D& im) { return ivec2(im.w, im.h); }
inline void imageStore(image2D& im, const ivec2& c, const vec4& v)
{
    if (c.x >= 0 && c.y >= 0 && c.x < im.w && c.y < im.h) im.px[(size_t)c.y * im.w + c.x] = v;
}
inline ivec2 textureSize(const sampler2D&, int) { return ivec2(1, 1); }
inline vec4 texture(const sampler2D&, const vec2&) { return vec4(0.0f, 0.0f, 0.0f, 1.0f); }
inline vec4 texture(const samplerCube&, const vec3&) { return vec4(0.0f, 0.0f, 0.0f, 1.0f); }

}  // namespace glsl
