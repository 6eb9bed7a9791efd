// render_oracle.cpp -- CPU restatement of the reference's SPH-mode particle draw.
// TEST INFRASTRUCTURE ONLY: tests/ load it to check sph_render; the product never links it.
//
// NPR-SPH draws the particles as GL point sprites (Main.cpp:311-337, SPH mode) through
// toon_vs.glsl and toon_fs.glsl in two passes:
//   vertex    gl_Position = P V M pos (toon_vs.glsl:32), pw = M pos (:33), size sim_rad (:47)
//   pass 0    coverage texture: green = flat depth 1.0 for every drawn fragment (:44;
//             toon_fs.glsl:71-77)
//   pass 1    cel shading of the front-most fragment (toon_fs.glsl:90-124) mixed with the
//             Sobel outline of the coverage texture (:126-153; :79-84)
// This restatement follows GL's draw order literally: particles in record order, every
// fragment tested with GL_LESS against a 24-bit depth buffer cleared to 1.0 (equal depths:
// the first drawn stays). The arithmetic is FP32 with round-to-nearest operations (built
// with -ffp-contract=off), in the operation order stated in include/sph_gb300.h for
// sph_render; normalize(v) is v / sqrt(dot(v, v)) and pow(x, s) > 0.95 is x > 0.95^(1/s).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "../include/sph_gb300.h"

namespace {

inline float row4(const float* r, float x, float y, float z) { return ((r[0] * x + r[1] * y) + r[2] * z) + r[3]; }
inline float dot3(const float* a, const float* b) { return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2]; }
inline void normalize3(float* v) {
    const float len = std::sqrt(dot3(v, v));
    for (int k = 0; k < 3; ++k) v[k] = v[k] / len;
}

uint32_t rgba8(const float* c) {
    uint32_t out = 0;
    for (int k = 0; k < 4; ++k) {
        const double v = k < 3 ? (double)c[k] : 1.0;
        const double cl = v < 0.0 ? 0.0 : (v > 1.0 ? 1.0 : v);
        out |= (uint32_t)std::floor(cl * 255.0 + 0.5) << (8 * k);
    }
    return out;
}

struct View {
    float pvm[16], m[12], eye[3], light[3], half_w, half_h, hs, thr;
    int W, H;
};

View prepare(const sph_view* v) {
    View V{};
    auto at = [](const float* m, int r, int c) { return (double)m[4 * c + r]; };
    double pv[16], pvm[16];
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) {
            double a = 0.0;
            for (int k = 0; k < 4; ++k) a += at(v->proj, r, k) * at(v->view, k, c);
            pv[4 * r + c] = a;
        }
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) {
            double a = 0.0;
            for (int k = 0; k < 4; ++k) a += pv[4 * r + k] * at(v->model, k, c);
            pvm[4 * r + c] = a;
        }
    for (int i = 0; i < 16; ++i) V.pvm[i] = (float)pvm[i];
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 4; ++c) V.m[4 * r + c] = v->model[4 * c + r];
    for (int k = 0; k < 3; ++k) {
        V.eye[k] = v->eye_w[k];
        V.light[k] = v->light_w[k];
    }
    V.W = v->width;
    V.H = v->height;
    V.half_w = (float)(0.5 * v->width);
    V.half_h = (float)(0.5 * v->height);
    V.hs = 0.5f * v->point_size;
    V.thr = v->shininess > 0.0f ? (float)std::pow(0.95, 1.0 / (double)v->shininess) : 0.0f;
    return V;
}

// Vertex stage + viewport: window position and 24-bit depth; false when clipped.
bool vertex(const View& V, const float* p, float& xw, float& yw, uint32_t& d24) {
    const float cx = row4(V.pvm, p[0], p[1], p[2]), cy = row4(V.pvm + 4, p[0], p[1], p[2]);
    const float cz = row4(V.pvm + 8, p[0], p[1], p[2]), cw = row4(V.pvm + 12, p[0], p[1], p[2]);
    if (!(cw > 0.0f) || !(std::fabs(cx) <= cw) || !(std::fabs(cy) <= cw) || !(std::fabs(cz) <= cw)) return false;
    xw = (cx / cw + 1.0f) * V.half_w;
    yw = (cy / cw + 1.0f) * V.half_h;
    const float zw = (cz / cw + 1.0f) * 0.5f;
    const float d = zw * 16777215.0f + 0.5f;
    d24 = (uint32_t)d < 16777215u ? (uint32_t)d : 16777215u;
    return true;
}

// 2 gl_PointCoord - 1 at pixel (x, y) (toon_fs.glsl:97), returns |p|^2.
float sprite(const View& V, int x, float xw, int y, float yw, float& px, float& py) {
    px = (((float)x + 0.5f) - xw) / V.hs;
    py = -((((float)y + 0.5f) - yw) / V.hs);
    return px * px + py * py;
}

// Cel shading of one fragment of particle-space position pw (toon_fs.glsl:90-124, SPH mode):
// (px, py) = 2 gl_PointCoord - 1, the sphere impostor's normal (px, py, sqrt(1 - |p|^2)),
// light and view vectors from pw, the reflection of -l about n. Returns -1 (discard: |p|^2 > 1),
// 0 dark (n.l < 0), 1 midtone, 2 highlight (r.v > 0 and r.v > thr, thr = 0.95^(1/shininess):
// the shader's pow(r.v, shininess) > 0.95); *rv_out gets r.v.
int cel_choice(const float* pw, const float* eye, const float* light, float px, float py, float thr, float* rv_out) {
    const float mag = px * px + py * py;
    if (mag > 1.0f) return -1;
    float n3[3] = {px, py, std::sqrt(1.0f - mag)};
    normalize3(n3);
    float l[3] = {light[0] - pw[0], light[1] - pw[1], light[2] - pw[2]};
    normalize3(l);
    float vv[3] = {eye[0] - pw[0], eye[1] - pw[1], eye[2] - pw[2]};
    normalize3(vv);
    const float ml[3] = {-l[0], -l[1], -l[2]};
    const float d2 = 2.0f * dot3(n3, ml);
    float r[3] = {ml[0] - d2 * n3[0], ml[1] - d2 * n3[1], ml[2] - d2 * n3[2]};
    normalize3(r);
    const float nl = dot3(n3, l), rv = dot3(r, vv);
    if (rv_out) *rv_out = rv;
    int c = nl < 0.0f ? 0 : 1;
    if (rv > 0.0f && rv > thr) c = 2;
    return c;
}

// Sobel outline of the pass-0 coverage around a fragment (toon_fs.glsl:126-153): cov[3 i + j]
// is 1 where pixel (x + i - 1, y + j - 1) is covered. gx = column x-1 minus column x+1, gy =
// row y-1 minus row y+1 (weights 1, 2, 1); an outline where sqrt(gx^2 + gy^2) > 0.1.
int outline_choice(const int* cov) {
    auto c = [&](int i, int j) { return cov[3 * i + j]; };
    const int gx = (c(0, 0) + 2 * c(0, 1) + c(0, 2)) - (c(2, 0) + 2 * c(2, 1) + c(2, 2));
    const int gy = (c(0, 0) + 2 * c(1, 0) + c(2, 0)) - (c(0, 2) + 2 * c(1, 2) + c(2, 2));
    const double g = std::sqrt((double)gx * gx + (double)gy * gy);
    return g > 0.1 ? 1 : 0;
}

}  // namespace

extern "C" int oracle_toon_cel(const float pw[3], const float eye[3], const float light[3], float px, float py,
                               float thr, float* rv) {
    return cel_choice(pw, eye, light, px, py, thr, rv);
}

extern "C" int oracle_toon_outline(const int cov[9]) { return outline_choice(cov); }

extern "C" int oracle_render(const sph_view* v, const float* pos4, int64_t n, uint8_t* rgba) {
    if (!v || !rgba || v->width <= 0 || v->height <= 0 || (n > 0 && !pos4)) return -1;
    const View V = prepare(v);
    const int W = V.W, H = V.H;
    std::vector<uint32_t> depth((size_t)W * H, 16777215u);  // cleared to 1.0
    std::vector<int64_t> owner((size_t)W * H, -1);
    for (int64_t i = 0; i < n; ++i) {  // draw order
        const float* p = pos4 + 4 * i;
        float xw, yw;
        uint32_t d24;
        if (!vertex(V, p, xw, yw, d24)) continue;
        // a conservative pixel box (one pixel wider on every side); the exact test follows
        const int ya = std::max(0, (int)std::floor(yw - V.hs) - 1), yb = std::min(H - 1, (int)std::ceil(yw + V.hs) + 1);
        const int xa = std::max(0, (int)std::floor(xw - V.hs) - 1), xb = std::min(W - 1, (int)std::ceil(xw + V.hs) + 1);
        for (int y = ya; y <= yb; ++y) {
            const float cy = (float)y + 0.5f;
            if (!(cy >= yw - V.hs && cy < yw + V.hs)) continue;
            for (int x = xa; x <= xb; ++x) {
                const float cx = (float)x + 0.5f;
                if (!(cx >= xw - V.hs && cx < xw + V.hs)) continue;
                float px, py;
                if (sprite(V, x, xw, y, yw, px, py) > 1.0f) continue;  // discard (toon_fs.glsl:99)
                const size_t k = (size_t)y * W + x;
                if (d24 < depth[k]) {  // GL_LESS
                    depth[k] = d24;
                    owner[k] = i;
                }
            }
        }
    }
    auto cov = [&](int x, int y) { return (x >= 0 && x < W && y >= 0 && y < H && owner[(size_t)y * W + x] >= 0) ? 1 : 0; };
    const uint32_t c_dark = rgba8(v->dark), c_mid = rgba8(v->midtone), c_hi = rgba8(v->highlight);
    const uint32_t c_out = rgba8(v->outline), c_clear = rgba8(v->clear_color);
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            const size_t k = (size_t)y * W + x;
            uint32_t c = c_clear;
            if (owner[k] >= 0) {
                int nb[9];
                for (int i = 0; i < 3; ++i)
                    for (int j = 0; j < 3; ++j) nb[3 * i + j] = cov(x + i - 1, y + j - 1);
                if (outline_choice(nb)) {
                    c = c_out;
                } else {
                    const float* p = pos4 + 4 * owner[k];
                    float xw, yw;
                    uint32_t d24;
                    vertex(V, p, xw, yw, d24);
                    float px, py;
                    sprite(V, x, xw, y, yw, px, py);
                    const float pw[3] = {row4(V.m, p[0], p[1], p[2]), row4(V.m + 4, p[0], p[1], p[2]),
                                         row4(V.m + 8, p[0], p[1], p[2])};
                    const int choice = cel_choice(pw, V.eye, V.light, px, py, V.thr, nullptr);
                    c = choice == 2 ? c_hi : (choice == 0 ? c_dark : c_mid);
                }
            }
            std::memcpy(rgba + 4 * k, &c, 4);
        }
    return 0;
}
