// sph_device.cuh -- device helpers shared by the SPH kernels.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "sph_internal.h"

namespace sphgb {

// Scene index / particle id carried in the w lanes as int bits.
__device__ __forceinline__ int scene_of(float4 p) { return __float_as_int(p.w); }
__device__ __forceinline__ int id_of(float4 v) { return __float_as_int(v.w); }

// The FP32 pair distance of the shaders' `length(pos_i - pos_j)`
// (rho_pres_comp.glsl:48-49) before its square root: dx*dx + dy*dy + dz*dz
// summed left to right, every operation rounded on its own (no FMA), so the
// neighbour predicate d2 < cut_d2 is the same bit for bit in every kernel,
// in the brute-force check and in the CPU oracle.
__device__ __forceinline__ float canon_d2(float xi, float yi, float zi, float xj, float yj, float zj,
                                          float& dx, float& dy, float& dz) {
    dx = __fsub_rn(xi, xj);
    dy = __fsub_rn(yi, yj);
    dz = __fsub_rn(zi, zj);
    return __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
}

// Cell coordinate along one axis: floor((x - lo) / edge), clamped into the box
// (positions on the upper wall, or outside it before the first step, land in
// the edge cells; clamping only shrinks distances, so no pair is lost).
__device__ __forceinline__ int cell_coord(float x, float lo, float inv_edge, int dim) {
    float t = __fmul_rn(__fsub_rn(x, lo), inv_edge);
    int c = (t == t) ? (int)floorf(t) : 0;  // NaN -> cell 0; +-inf saturate, then clamp
    return min(max(c, 0), dim - 1);
}

__device__ __forceinline__ int cell_key(const SceneDev& s, float x, float y, float z) {
    int cx = cell_coord(x, s.lo[0], s.inv_edge, s.dim[0]);
    int cy = cell_coord(y, s.lo[1], s.inv_edge, s.dim[1]);
    int cz = cell_coord(z, s.lo[2], s.inv_edge, s.dim[2]);
    return s.cell_base + cx + s.dim[0] * (cy + s.dim[1] * cz);
}

// splitmix64 finaliser of (j + golden gamma): the neighbour digest term.
__device__ __forceinline__ unsigned long long mix64(unsigned long long z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// Scene constants of a particle: the kernel argument for a single scene, the
// scene table entry (L1-cached) for a batch.
template <bool BATCHED>
__device__ __forceinline__ const SceneDev& scene_params(const SceneDev& s0, const SceneDev* __restrict__ table,
                                                        int sc) {
    if constexpr (BATCHED) return table[sc];
    else return s0;
}

__device__ __forceinline__ void raise_err(uint32_t* err, uint32_t bit) { atomicOr(err, bit); }

// Static obstacle at (x, y, z): phi, the trilinear interpolant of the signed distance samples,
// and g, the trilinear interpolant of the samples' central-difference gradients (one-sided on
// the grid's faces). g is continuous across cells, unlike the interpolant's own gradient,
// which is one-sided on every sample plane. False outside the sampled box or for a NaN
// position.
__device__ __forceinline__ bool sdf_sample(const SceneDev& S, float x, float y, float z, float& phi, float (&g)[3]) {
    const float u = (x - S.sorg[0]) * S.sinv, v = (y - S.sorg[1]) * S.sinv, w = (z - S.sorg[2]) * S.sinv;
    if (!(u >= 0.0f && v >= 0.0f && w >= 0.0f && u <= (float)(S.sdim[0] - 1) && v <= (float)(S.sdim[1] - 1) &&
          w <= (float)(S.sdim[2] - 1)))
        return false;
    const int c[3] = {min((int)u, S.sdim[0] - 2), min((int)v, S.sdim[1] - 2), min((int)w, S.sdim[2] - 2)};
    const float t[3] = {u - (float)c[0], v - (float)c[1], w - (float)c[2]};
    const size_t st[3] = {1, (size_t)S.sdim[0], (size_t)S.sdim[0] * S.sdim[1]};
    phi = 0.0f;
    g[0] = g[1] = g[2] = 0.0f;
#pragma unroll
    for (int corner = 0; corner < 8; ++corner) {
        const int o[3] = {corner & 1, (corner >> 1) & 1, (corner >> 2) & 1};
        float wgt = 1.0f;
        int q[3];
        size_t at = 0;
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            wgt *= o[a] ? t[a] : 1.0f - t[a];
            q[a] = c[a] + o[a];
            at += (size_t)q[a] * st[a];
        }
        phi += wgt * __ldg(S.sdf + at);
#pragma unroll
        for (int a = 0; a < 3; ++a) {  // central difference along a at this corner
            const int lo = max(q[a] - 1, 0), hi = min(q[a] + 1, S.sdim[a] - 1);
            const float d = __ldg(S.sdf + at + (size_t)(hi - q[a]) * st[a]) - __ldg(S.sdf + at - (size_t)(q[a] - lo) * st[a]);
            g[a] += wgt * d / (float)(hi - lo);
        }
    }
#pragma unroll
    for (int a = 0; a < 3; ++a) g[a] *= S.sinv;
    return true;
}

// The obstacle's collision rule after the wall clamp: a particle inside (phi < 0) moves out
// along the normal by its depth, a velocity into the surface keeps -damping of its normal
// component (the walls' rule of integrate_comp.glsl:45-77 along n), and the position is
// clamped into the box again.
__device__ __forceinline__ void obstacle_response(const SceneDev& S, float (&np)[3], float (&nv)[3]) {
    if (!S.sdf) return;
    float phi, g[3];
    if (!sdf_sample(S, np[0], np[1], np[2], phi, g) || !(phi < 0.0f)) return;
    const float gl = sqrtf(g[0] * g[0] + g[1] * g[1] + g[2] * g[2]);
    if (!(gl > 0.0f)) return;
    const float n[3] = {g[0] / gl, g[1] / gl, g[2] / gl};
    const float vn = nv[0] * n[0] + nv[1] * n[1] + nv[2] * n[2];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        np[a] -= phi * n[a];
        if (vn < 0.0f) nv[a] -= (1.0f + S.damp) * vn * n[a];
        np[a] = fminf(fmaxf(np[a], S.lo[a]), S.up[a]);
    }
}

}  // namespace sphgb
