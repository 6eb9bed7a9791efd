// sph_render.cu -- headless toon rendering of the particles: the reference's
// SPH-mode draw (Main.cpp:311-337: toon_vs.glsl, toon_fs.glsl, two passes) as
// three CUDA kernels into an RGBA8 buffer. The restated pipeline is stated in
// include/sph_gb300.h (sph_render); here:
//
//   k_pos_by_id  positions in record order (= the GL draw order)
//   k_splat      one thread per particle: projection (toon_vs.glsl:32), the
//                point sprite's pixels (gl_PointSize = sim_rad, :47), the disc
//                test of toon_fs.glsl:97-99, and the depth test as an atomicMin
//                of (24-bit depth << 32 | record index) per pixel: GL_LESS keeps
//                the first drawn of equal depths, the smallest index
//   k_shade      one thread per pixel: the winning particle's cel colour
//                (toon_fs.glsl:90-124) or the outline colour where the Sobel
//                gradient of the coverage is non-zero (:126-153, pass 0's green
//                channel is a flat 1.0 for every covered pixel, toon_vs.glsl:44)
//
// All arithmetic is FP32 with explicit round-to-nearest operations (no FMA
// contraction), so a CPU restatement reproduces the image byte for byte.
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "sph_ctx.h"
#include "sph_device.cuh"

using namespace sphgb;
using sphgb::engine::fail;

namespace {

constexpr unsigned long long kEmpty = ~0ull;

struct ViewDev {
    float pvm[16];  // (P V M) rows: pvm[4 r + c]
    float m[12];    // M rows 0..2
    float eye[3], light[3];
    float half_w, half_h, hs;  // W/2, H/2, point_size/2
    float thr;                 // highlight when dot(r, v) > thr (and > 0)
    int W, H;
    uint32_t c_dark, c_mid, c_hi, c_out, c_clear;  // RGBA8 (little-endian: r in the low byte)
};

__device__ __forceinline__ float row4(const float* r, float x, float y, float z) {
    return __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(r[0], x), __fmul_rn(r[1], y)), __fmul_rn(r[2], z)), r[3]);
}
__device__ __forceinline__ float dot3(float ax, float ay, float az, float bx, float by, float bz) {
    return __fadd_rn(__fadd_rn(__fmul_rn(ax, bx), __fmul_rn(ay, by)), __fmul_rn(az, bz));
}
__device__ __forceinline__ void normalize3(float& x, float& y, float& z) {
    const float len = __fsqrt_rn(dot3(x, y, z, x, y, z));
    x = __fdiv_rn(x, len);
    y = __fdiv_rn(y, len);
    z = __fdiv_rn(z, len);
}

// Clip test, window position and 24-bit depth of a particle (toon_vs.glsl:32; viewport and
// depth range [0, 1]).
__device__ __forceinline__ bool project(const ViewDev& V, float4 p, float& xw, float& yw, uint32_t& d24) {
    const float cx = row4(V.pvm + 0, p.x, p.y, p.z), cy = row4(V.pvm + 4, p.x, p.y, p.z);
    const float cz = row4(V.pvm + 8, p.x, p.y, p.z), cw = row4(V.pvm + 12, p.x, p.y, p.z);
    if (!(cw > 0.0f) || !(fabsf(cx) <= cw) || !(fabsf(cy) <= cw) || !(fabsf(cz) <= cw)) return false;
    xw = __fmul_rn(__fadd_rn(__fdiv_rn(cx, cw), 1.0f), V.half_w);
    yw = __fmul_rn(__fadd_rn(__fdiv_rn(cy, cw), 1.0f), V.half_h);
    const float zw = __fmul_rn(__fadd_rn(__fdiv_rn(cz, cw), 1.0f), 0.5f);
    const float d = __fadd_rn(__fmul_rn(zw, 16777215.0f), 0.5f);
    d24 = min((uint32_t)d, 16777215u);
    return d24 < 16777215u;  // the depth buffer is cleared to 1.0: GL_LESS fails there
}

// gl_PointCoord mapped to [-1, 1]^2 (toon_fs.glsl:97) at pixel (x, y); returns |p|^2.
__device__ __forceinline__ float sprite_p(const ViewDev& V, int x, float xw, int y, float yw, float& px, float& py) {
    px = __fdiv_rn(__fsub_rn((float)x + 0.5f, xw), V.hs);
    py = -__fdiv_rn(__fsub_rn((float)y + 0.5f, yw), V.hs);
    return __fadd_rn(__fmul_rn(px, px), __fmul_rn(py, py));
}

__global__ void __launch_bounds__(256) k_pos_by_id(const float4* __restrict__ pos, const float4* __restrict__ vel,
                                                   int n, float4* __restrict__ out) {
    const int s = blockIdx.x * 256 + threadIdx.x;
    if (s >= n) return;
    const int id = id_of(vel[s]);
    if (id >= 0 && id < n) out[id] = pos[s];
}

__global__ void __launch_bounds__(256) k_clear_keys(unsigned long long* __restrict__ keys, int npix) {
    for (int i = blockIdx.x * 256 + threadIdx.x; i < npix; i += gridDim.x * 256) keys[i] = kEmpty;
}

__global__ void __launch_bounds__(256) k_splat(const float4* __restrict__ pos_id, int first, int count, ViewDev V,
                                               unsigned long long* __restrict__ keys) {
    for (int k = blockIdx.x * 256 + threadIdx.x; k < count; k += gridDim.x * 256) {
        const float4 p = pos_id[first + k];
        float xw, yw;
        uint32_t d24;
        if (!project(V, p, xw, yw, d24)) continue;
        const unsigned long long key = ((unsigned long long)d24 << 32) | (unsigned)k;
        // pixel centres c with x_w - s/2 <= c < x_w + s/2
        const int x0 = max((int)ceilf(__fsub_rn(__fsub_rn(xw, V.hs), 0.5f)), 0);
        const int x1 = min((int)ceilf(__fsub_rn(__fadd_rn(xw, V.hs), 0.5f)) - 1, V.W - 1);
        const int y0 = max((int)ceilf(__fsub_rn(__fsub_rn(yw, V.hs), 0.5f)), 0);
        const int y1 = min((int)ceilf(__fsub_rn(__fadd_rn(yw, V.hs), 0.5f)) - 1, V.H - 1);
        for (int y = y0; y <= y1; ++y)
            for (int x = x0; x <= x1; ++x) {
                float px, py;
                if (!(sprite_p(V, x, xw, y, yw, px, py) <= 1.0f)) continue;  // toon_fs.glsl:99 discard
                unsigned long long* slot = keys + (size_t)y * V.W + x;
                if (key < *slot) atomicMin(slot, key);
            }
    }
}

__device__ __forceinline__ int covered(const unsigned long long* keys, int W, int H, int x, int y) {
    return (x >= 0 && x < W && y >= 0 && y < H && keys[(size_t)y * W + x] != kEmpty) ? 1 : 0;
}

__global__ void __launch_bounds__(256) k_shade(const float4* __restrict__ pos_id, int first,
                                               const unsigned long long* __restrict__ keys, ViewDev V,
                                               uint32_t* __restrict__ rgba) {
    const int x = blockIdx.x * 16 + (threadIdx.x & 15), y = blockIdx.y * 16 + (threadIdx.x >> 4);
    if (x >= V.W || y >= V.H) return;
    const unsigned long long key = keys[(size_t)y * V.W + x];
    uint32_t c = V.c_clear;
    if (key != kEmpty) {
        const int W = V.W, H = V.H;
        const int gx = (covered(keys, W, H, x - 1, y - 1) + 2 * covered(keys, W, H, x - 1, y) +
                        covered(keys, W, H, x - 1, y + 1)) -
                       (covered(keys, W, H, x + 1, y - 1) + 2 * covered(keys, W, H, x + 1, y) +
                        covered(keys, W, H, x + 1, y + 1));
        const int gy = (covered(keys, W, H, x - 1, y - 1) + 2 * covered(keys, W, H, x, y - 1) +
                        covered(keys, W, H, x + 1, y - 1)) -
                       (covered(keys, W, H, x - 1, y + 1) + 2 * covered(keys, W, H, x, y + 1) +
                        covered(keys, W, H, x + 1, y + 1));
        if (gx != 0 || gy != 0) {
            c = V.c_out;  // sqrt(gx^2 + gy^2) > 0.1 for any non-zero integer gradient
        } else {
            const float4 p = pos_id[first + (int)(key & 0xffffffffu)];
            float xw, yw;
            uint32_t d24;
            project(V, p, xw, yw, d24);
            float nx, ny;
            const float mag = sprite_p(V, x, xw, y, yw, nx, ny);
            float nz = __fsqrt_rn(__fsub_rn(1.0f, mag));
            normalize3(nx, ny, nz);
            const float wx = row4(V.m + 0, p.x, p.y, p.z), wy = row4(V.m + 4, p.x, p.y, p.z);
            const float wz = row4(V.m + 8, p.x, p.y, p.z);
            float lx = __fsub_rn(V.light[0], wx), ly = __fsub_rn(V.light[1], wy), lz = __fsub_rn(V.light[2], wz);
            normalize3(lx, ly, lz);
            float vx = __fsub_rn(V.eye[0], wx), vy = __fsub_rn(V.eye[1], wy), vz = __fsub_rn(V.eye[2], wz);
            normalize3(vx, vy, vz);
            // r = normalize(reflect(-l, n)) = normalize(-l - 2 dot(n, -l) n)
            const float d2 = __fmul_rn(2.0f, -dot3(nx, ny, nz, lx, ly, lz));
            float rx = __fsub_rn(-lx, __fmul_rn(d2, nx)), ry = __fsub_rn(-ly, __fmul_rn(d2, ny));
            float rz = __fsub_rn(-lz, __fmul_rn(d2, nz));
            normalize3(rx, ry, rz);
            const float nl = dot3(nx, ny, nz, lx, ly, lz);
            const float rv = dot3(rx, ry, rz, vx, vy, vz);
            c = nl < 0.0f ? V.c_dark : V.c_mid;
            if (rv > 0.0f && rv > V.thr) c = V.c_hi;
        }
    }
    rgba[(size_t)y * V.W + x] = c;
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

}  // namespace

extern "C" sph_status sph_render(sph_ctx* ctx, const sph_view* v, uint32_t scene, uint8_t* rgba,
                                 int32_t rgba_on_device) {
    if (!ctx || !v || !rgba) return SPH_ERR_INVALID_ARG;
    if (!ctx->have_state) return fail(ctx, SPH_ERR_NOT_READY, "no particles uploaded");
    if (v->width <= 0 || v->height <= 0 || v->width > 16384 || v->height > 16384)
        return fail(ctx, SPH_ERR_INVALID_ARG, "image size out of [1, 16384]");
    if (!(v->point_size > 0.0f && v->point_size <= 1024.0f))
        return fail(ctx, SPH_ERR_INVALID_ARG, "point size out of (0, 1024]");
    if (!(v->shininess >= 0.0f)) return fail(ctx, SPH_ERR_INVALID_ARG, "negative shininess");
    if (scene >= ctx->counts.size()) return fail(ctx, SPH_ERR_INVALID_ARG, "no such scene");
    try {
        cudaSetDevice(ctx->device);
        int first = 0;
        for (uint32_t s = 0; s < scene; ++s) first += (int)ctx->counts[s];
        const int count = (int)ctx->counts[scene];
        const int n = ctx->b.n;
        // host-side view constants: P V M in FP64, rounded once to FP32
        ViewDev V{};
        double pv[16], pvm[16];
        auto at = [](const float* m, int r, int c) { return (double)m[4 * c + r]; };  // column-major
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
        // pow(x, s) > 0.95 <=> x > 0.95^(1/s) for x > 0; s = 0: pow = 1 > 0.95 for every x > 0
        V.thr = v->shininess > 0.0f ? (float)std::pow(0.95, 1.0 / (double)v->shininess) : 0.0f;
        V.c_dark = rgba8(v->dark);
        V.c_mid = rgba8(v->midtone);
        V.c_hi = rgba8(v->highlight);
        V.c_out = rgba8(v->outline);
        V.c_clear = rgba8(v->clear_color);
        const size_t npix = (size_t)v->width * v->height;
        const size_t need = npix * 8 + (size_t)n * 16 + (rgba_on_device ? 0 : npix * 4) + 256;
        if (need > ctx->render_cap) {
            if (ctx->render_buf) cudaFree(ctx->render_buf);
            ctx->render_buf = nullptr;
            ctx->render_cap = 0;
            if (cudaMalloc(&ctx->render_buf, need) != cudaSuccess)
                return fail(ctx, SPH_ERR_OUT_OF_MEMORY, "render scratch");
            ctx->render_cap = need;
        }
        char* base = static_cast<char*>(ctx->render_buf);
        unsigned long long* keys = reinterpret_cast<unsigned long long*>(base);
        float4* pos_id = reinterpret_cast<float4*>(base + npix * 8);
        uint32_t* img = rgba_on_device ? reinterpret_cast<uint32_t*>(rgba)
                                       : reinterpret_cast<uint32_t*>(base + npix * 8 + (size_t)n * 16);
        cudaStream_t st = ctx->stream;
        const int sms = device_sm_count();
        k_pos_by_id<<<(n + 255) / 256, 256, 0, st>>>(ctx->b.pos, ctx->b.vel, n, pos_id);
        k_clear_keys<<<std::min((int)((npix + 255) / 256), sms * 8), 256, 0, st>>>(keys, (int)npix);
        if (count > 0)
            k_splat<<<std::min((count + 255) / 256, sms * 16), 256, 0, st>>>(pos_id, first, count, V, keys);
        const dim3 grid((v->width + 15) / 16, (v->height + 15) / 16);
        k_shade<<<grid, 256, 0, st>>>(pos_id, first, keys, V, img);
        cudaError_t e = cudaGetLastError();
        if (e == cudaSuccess && !rgba_on_device)
            e = cudaMemcpyAsync(rgba, img, npix * 4, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess && !rgba_on_device) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) return fail(ctx, SPH_ERR_CUDA, std::string("render: ") + cudaGetErrorString(e));
        return SPH_OK;
    } catch (const std::bad_alloc&) {
        return fail(ctx, SPH_ERR_OUT_OF_MEMORY, "host allocation failed");
    }
}
