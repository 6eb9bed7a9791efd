// toon_shim.hpp -- enough GLSL 4.40 to compile the reference's particle fragment shader
// (NPR-SPH/toon_fs.glsl) as C++ on the CPU. TEST INFRASTRUCTURE ONLY.
//
// The shader text is #included inside a struct body (ref_toon.cpp), as with the compute
// shaders: its uniforms, its `in` block and `out` variable become members that the host sets
// before calling one of its functions, and its functions become member functions. A uniform
// block becomes a nested struct type (SceneUniformsBlock, MaterialUniformsBlock) and the
// shader instance declares the block's fields as its own members, under the same names. The recipe blanks the first line
// (`#version 440`) and the three forward declarations of its functions (class scope does not
// allow a member function to be declared twice); every other line is as is, in place.
//
// Arithmetic is FP32 throughout (operators on float vectors; the shader's double literals are
// converted to float where they meet a float operand or a built-in's float parameter), built
// with -ffp-contract=off. Built-ins follow the GLSL 4.40 definitions:
//   dot = left-to-right sum of products; length(x) = sqrt(dot(x, x)); normalize(x) = x / length(x);
//   reflect(I, N) = I - 2.0 * dot(N, I) * N; distance(a, b) = length(a - b);
//   pow(x, y): x * x for the literal exponent 2.0, else powf(x, y) for x >= 0 and NaN for x < 0
//   (see pow below); mix(x, y, a) = x * (1 - a) + y * a.
// `discard` throws glslref::Discard. texelFetch reads a 3 x 3 neighbourhood the host sets.
#pragma once

#include <math.h>

namespace glslref {

struct Discard {};

struct v2 { float x, y; };
struct v3 { float x, y, z; };
// The vector types are trivially default-constructible; the host value-initialises a shader
// instance, which zeroes them.

struct vec2 {
    union {
        struct { float x, y; };
        v2 xy;
    };
    vec2() = default;
    explicit vec2(float s) : x(s), y(s) {}
    vec2(float a, float b) : x(a), y(b) {}
    vec2(const v2& v) : x(v.x), y(v.y) {}
};

struct vec3 {
    union {
        struct { float x, y, z; };
        struct { float r, g, b; };
        v3 xyz;
        float e[3];
    };
    vec3() = default;
    explicit vec3(float s) : x(s), y(s), z(s) {}
    vec3(float a, float b, float c) : x(a), y(b), z(c) {}
    vec3(const vec2& p, float c) : x(p.x), y(p.y), z(c) {}
    vec3(const v3& v) : x(v.x), y(v.y), z(v.z) {}
    float& operator[](int i) { return e[i]; }
    float operator[](int i) const { return e[i]; }
};

struct vec4 {
    union {
        struct { float x, y, z, w; };
        struct { float r, g, b, a; };
        v3 xyz;
        v3 rgb;
        v2 xy;
        float e[4];
    };
    vec4() = default;
    explicit vec4(float s) : x(s), y(s), z(s), w(s) {}
    vec4(float a, float b, float c, float d) : x(a), y(b), z(c), w(d) {}
    vec4(const vec3& v, float d) : x(v.x), y(v.y), z(v.z), w(d) {}
};

struct ivec2 {
    int x, y;
    ivec2(int a, int b) : x(a), y(b) {}
    explicit ivec2(const vec4& v) : x((int)v.x), y((int)v.y) {}
};
inline ivec2 operator+(ivec2 a, ivec2 b) { return ivec2(a.x + b.x, a.y + b.y); }

// mat3 of nine floats: column-major, m[i] is column i.
struct mat3 {
    vec3 c[3];
    mat3() = default;
    mat3(float a0, float a1, float a2, float b0, float b1, float b2, float c0, float c1, float c2)
        : c{vec3(a0, a1, a2), vec3(b0, b1, b2), vec3(c0, c1, c2)} {}
    vec3& operator[](int i) { return c[i]; }
    const vec3& operator[](int i) const { return c[i]; }
};
struct mat4 { vec4 c[4]; };
struct sampler2D { int unit; };

inline vec2 operator*(float s, vec2 a) { return vec2(s * a.x, s * a.y); }
inline vec2 operator-(vec2 a, vec2 b) { return vec2(a.x - b.x, a.y - b.y); }
inline vec3 operator+(vec3 a, vec3 b) { return vec3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline vec3 operator-(vec3 a, vec3 b) { return vec3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline vec3 operator-(vec3 a) { return vec3(-a.x, -a.y, -a.z); }
inline vec3 operator-(float s, vec3 a) { return vec3(s - a.x, s - a.y, s - a.z); }
inline vec3 operator*(float s, vec3 a) { return vec3(s * a.x, s * a.y, s * a.z); }
inline vec3 operator*(vec3 a, float s) { return vec3(a.x * s, a.y * s, a.z * s); }
inline vec3 operator*(vec3 a, vec3 b) { return vec3(a.x * b.x, a.y * b.y, a.z * b.z); }
inline vec3 operator/(vec3 a, float s) { return vec3(a.x / s, a.y / s, a.z / s); }
inline vec4 operator+(vec4 a, vec4 b) { return vec4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
inline vec4 operator*(float s, vec4 a) { return vec4(s * a.x, s * a.y, s * a.z, s * a.w); }
inline vec4 operator*(vec4 a, float s) { return vec4(a.x * s, a.y * s, a.z * s, a.w * s); }

inline float dot(vec2 a, vec2 b) { return a.x * b.x + a.y * b.y; }
inline float dot(vec3 a, vec3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline float sqrt(float x) { return sqrtf(x); }
inline float length(vec3 a) { return sqrtf(dot(a, a)); }
inline vec3 normalize(vec3 a) { return a / length(a); }
inline float distance(vec3 a, vec3 b) { return length(a - b); }
inline vec3 reflect(vec3 i, vec3 n) { return i - 2.0f * dot(n, i) * n; }
// GLSL leaves pow(x, y) undefined for x < 0. GPU shader compilers expand a literal integer
// exponent into multiplications (pow(gx, 2.0) is gx * gx, defined for every gx) and evaluate
// any other exponent as exp2(y * log2(x)), which is NaN for x < 0 (C's powf would instead return
// a real power for an integer y). The shim follows the GPUs; the two cases differ in the shader
// text by the exponent's type: a double literal (2.0) or a float uniform (shininess).
inline float pow(float x, float y) { return x < 0.0f ? NAN : powf(x, y); }
inline float pow(float x, double literal) {
    if (literal == 2.0) return x * x;
    return pow(x, (float)literal);
}
inline float max(float x, float y) { return x < y ? y : x; }
inline vec4 mix(vec4 x, vec4 y, float a) { return x * (1.0f - a) + y * a; }

}  // namespace glslref

// Qualifier keywords and block names of the shader text.
#define layout(...)
#define uniform
#define in
#define out
#define SceneUniforms struct SceneUniformsBlock
#define MaterialUniforms struct MaterialUniformsBlock
#define VertexData struct
#define discard throw ::glslref::Discard()
