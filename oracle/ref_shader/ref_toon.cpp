// ref_toon.cpp -- the reference's particle fragment shader (NPR-SPH/toon_fs.glsl), compiled as
// C++ through toon_shim.hpp. TEST INFRASTRUCTURE ONLY: it pins the render restatement
// (render_oracle.cpp) to the reference's own shading code. Built by `make -C oracle ref` into
// oracle/_ref/ from the shader file in the reference tree; nothing of the reference is committed.
//
// Exposed per fragment:
//   ref_toon_cel      celshading() of SPH mode (mode = 1: the sphere-impostor normal from
//                     gl_PointCoord): which of dark / midtone / highlight it returns, or that
//                     it discards the fragment
//   ref_toon_outline  outline() of a 3 x 3 neighbourhood of the pass-0 texture's green channel:
//                     1 where the Sobel gradient makes an outline (its returned fill is 0)
#include "toon_shim.hpp"

namespace glslref {

struct ToonShader {
    // the fields of the shader's uniform blocks SceneUniforms and MaterialUniforms (toon_fs.glsl:11-26)
    mat4 P, V;
    vec4 eye_w, light_w;
    vec4 dark, midtone, highlight, outline_color;
    float shininess;
    vec4 gl_FragCoord;
    vec2 gl_PointCoord;
    float texel_green[3][3];  // the pass-0 texture around the fragment: [i][j] at (x + i - 1, y + j - 1)

    vec4 texelFetch(sampler2D, ivec2 p, int) const {
        const int i = p.x - (int)gl_FragCoord.x + 1, j = p.y - (int)gl_FragCoord.y + 1;
        return vec4(0.0f, texel_green[i][j], 0.0f, 1.0f);
    }

#include "toon_fs.inc"
};

}  // namespace glslref

extern "C" {

// pw, eye, light: world-space fragment, eye and light positions; pc: gl_PointCoord; colors
// dark / midtone / highlight are set to distinct markers. Returns 0 dark, 1 midtone,
// 2 highlight, -1 discarded.
int ref_toon_cel(const float pw[3], const float eye[3], const float light[3], const float pc[2], float shininess) {
    using namespace glslref;
    ToonShader sh{};
    sh.mode = 1;
    sh.inData.pw = vec3(pw[0], pw[1], pw[2]);
    sh.inData.nw = vec3(0.0f, 0.0f, 1.0f);
    sh.eye_w = vec4(eye[0], eye[1], eye[2], 1.0f);
    sh.light_w = vec4(light[0], light[1], light[2], 1.0f);
    sh.gl_PointCoord = vec2(pc[0], pc[1]);
    sh.dark = vec4(0.0f, 0.0f, 0.0f, 1.0f);
    sh.midtone = vec4(1.0f, 0.0f, 0.0f, 1.0f);
    sh.highlight = vec4(2.0f, 0.0f, 0.0f, 1.0f);
    sh.shininess = shininess;
    try {
        const vec4 c = sh.celshading();
        return (int)c.x;
    } catch (const Discard&) {
        return -1;
    }
}

// green: the 3 x 3 texel greens, green[3 * i + j] at (x + i - 1, y + j - 1); x, y: the fragment.
int ref_toon_outline(const float green[9], int x, int y) {
    using namespace glslref;
    ToonShader sh{};
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) sh.texel_green[i][j] = green[3 * i + j];
    sh.gl_FragCoord = vec4((float)x + 0.5f, (float)y + 0.5f, 0.5f, 1.0f);
    const vec4 fill = sh.outline();
    return fill.x == 0.0f ? 1 : 0;
}

}  // extern "C"
