// glsl_shim.hpp -- just enough GLSL 4.40 to compile the reference's three SPH
// compute shaders (NPR-SPH/rho_pres_comp.glsl, force_comp.glsl,
// integrate_comp.glsl) as C++ on the CPU. TEST INFRASTRUCTURE ONLY.
//
// Each shader's text is #included inside a struct body (ref_shader.cpp), so
//   - its `struct Particle` becomes a nested type,
//   - its interface blocks (`buffer PARTICLES {...}`, `uniform X {...}`) become
//     anonymous struct members (a GNU extension) that the host fills in,
//   - its `void main()` becomes a member function run once per invocation.
// The only edit to the shader text is blanking its first line (`#version 440`),
// which a C preprocessor rejects; line numbers are kept.
//
// Built-ins follow the GLSL 4.40 definitions:
//   length(x) = sqrt(dot(x, x)), dot = x.x*y.x + x.y*y.y + x.z*y.z (left to right)
//   normalize(x) = x / length(x) (component-wise division)
//   max(x, y) = (x < y) ? y : x
//   pow(x, y) = powf(x, y)
// compiled with -ffp-contract=off and no fast-math.
#pragma once

#include <math.h>
#include <stdint.h>

namespace glslref {

typedef unsigned int uint;

struct uvec3 { uint x, y, z; };

// Storage of a vec3 inside a vec4 (the .xyz swizzle). It has no constructor,
// so vec4 stays a trivial type that may sit in an interface block.
struct vec3raw { float x, y, z; };

struct vec3 : vec3raw {
    vec3() = default;
    constexpr explicit vec3(float s) : vec3raw{s, s, s} {}
    constexpr vec3(float a, float b, float c) : vec3raw{a, b, c} {}
    constexpr vec3(const vec3raw& r) : vec3raw(r) {}
};
inline vec3 operator+(vec3 a, vec3 b) { return vec3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline vec3 operator-(vec3 a, vec3 b) { return vec3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline vec3 operator*(float s, vec3 a) { return vec3(s * a.x, s * a.y, s * a.z); }
inline vec3 operator*(vec3 a, float s) { return vec3(a.x * s, a.y * s, a.z * s); }
inline vec3 operator/(vec3 a, float s) { return vec3(a.x / s, a.y / s, a.z / s); }
inline vec3& operator+=(vec3& a, vec3 b) { a = a + b; return a; }
inline vec3& operator-=(vec3& a, vec3 b) { a = a - b; return a; }
inline vec3& operator*=(vec3& a, float s) { a = a * s; return a; }

struct vec4 {
    union {
        struct { float x, y, z, w; };
        vec3raw xyz;
        float e[4];
    };
    float& operator[](uint i) { return e[i]; }
    float operator[](uint i) const { return e[i]; }
};

struct mat4 { vec4 c[4]; };

inline float dot(vec3 a, vec3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline float length(vec3 a) { return sqrtf(dot(a, a)); }
inline vec3 normalize(vec3 a) { return a / length(a); }
inline float max(float x, float y) { return x < y ? y : x; }
inline float pow(float x, float y) { return powf(x, y); }

// Per-invocation built-in inputs.
struct ShaderEnv {
    uvec3 gl_GlobalInvocationID;
};

}  // namespace glslref

// Qualifier keywords of the shader text.
#define layout(...)
#define in
#define buffer struct
#define uniform struct
#define PARTICLES
#define ConstantsUniform
#define BoundaryUniform
// `Particle particles[];` becomes a pointer to the host's particle array.
#define particles (*particles_ptr_)
