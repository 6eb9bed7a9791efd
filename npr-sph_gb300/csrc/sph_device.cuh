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

}  // namespace sphgb
