// sph_step.cu -- the two pair passes of the SPH step over the cell-sorted state.
//
//   density          rho_pres_comp.glsl:35-59   rho_i = m*315/(64*pi*h^9) * sum_{j: r<h} (h^2 - r^2)^3
//                                               (self included), p_i = max(k*(rho_i - rho0), 0)
//   force+integrate  force_comp.glsl:35-67      spiky pressure + Laplacian viscosity over j != i, r < h,
//                                               viscosity * mu, gravity rho_i*G
//                    integrate_comp.glsl:35-82  a = F/rho; v += dt*a; x += dt*v; per-axis wall clamp,
//                                               v *= -damping
//                    + the cell hash of the new position for the next step's sort.
//
// One thread per particle in cell-sorted order: the threads of a warp walk the
// same few cells, so their candidate loads hit L1. Each thread visits the
// (2R+1)^2 rows of (2R+1) contiguous cells around its own cell (cell edge h/R).
//
// Two phases per thread, so that the warp never runs the interaction code for
// a minority of lanes (with ~15% of candidates inside r < h, some lane almost
// always would):
//   1. candidate scan: the canonical FP32 predicate on every candidate; the
//      passing ones are appended to a per-thread list in shared memory
//      (density keeps d2, force keeps the slot j),
//   2. interaction loop over the list, all lanes busy.
// The list holds kNbCap entries; a longer neighbourhood is processed in chunks.
// Neighbours are visited in candidate order either way, so results are
// deterministic and independent of the chunking.
//
// The (dx, dy) part of the predicate runs as one packed FP32x2 subtraction and
// one packed multiplication (sub.rn.f32x2 / mul.rn.f32x2): each lane is
// rounded on its own, exactly like __fsub_rn / __fmul_rn, so the neighbour
// predicate stays bit-exact.
//
// Numerics: the density sum is compensated (Kahan) in FP32; the force sums are
// plain FP32 with contraction allowed (only the predicate is pinned bit-exact).
// For i != j at r == 0 the pressure term is skipped (the shader's
// normalize(0) is NaN, force_comp.glsl:59); the viscosity term is kept.
#include <type_traits>

#include "sph_device.cuh"

namespace sphgb {

namespace {

constexpr int kNbCap = 32;  // shared-memory neighbour list entries per thread

// (px - ox, py - oy) and their squares, each lane rounded separately.
__device__ __forceinline__ void sub_sq_xy(float px, float py, float ox, float oy, float& dx, float& dy, float& sx,
                                          float& sy) {
    asm("{\n\t.reg .b64 a, b, d, s;\n\t"
        "mov.b64 a, {%4, %5};\n\t"
        "mov.b64 b, {%6, %7};\n\t"
        "sub.rn.f32x2 d, a, b;\n\t"
        "mul.rn.f32x2 s, d, d;\n\t"
        "mov.b64 {%0, %1}, d;\n\t"
        "mov.b64 {%2, %3}, s;\n\t}"
        : "=f"(dx), "=f"(dy), "=f"(sx), "=f"(sy)
        : "f"(px), "f"(py), "f"(ox), "f"(oy));
}

// canon_d2 (sph_device.cuh) with the x/y lanes packed.
__device__ __forceinline__ float canon_d2_pk(float px, float py, float pz, float4 o, float& dx, float& dy, float& dz) {
    float sx, sy;
    sub_sq_xy(px, py, o.x, o.y, dx, dy, sx, sy);
    dz = __fsub_rn(pz, o.z);
    return __fadd_rn(__fadd_rn(sx, sy), __fmul_rn(dz, dz));
}

// Iterate the stencil rows around cell (cx, cy, cz): calls fn(a, b) with the
// contiguous sorted-slot range [a, b) of cells cx-R..cx+R of each row.
template <int R, class Fn>
__device__ __forceinline__ void for_rows(const SceneDev& S, const int* __restrict__ start, int n, int cx, int cy,
                                         int cz, Fn fn) {
    const int x0 = max(cx - R, 0), x1 = min(cx + R, S.dim[0] - 1);
    const int z0 = max(cz - R, 0), z1 = min(cz + R, S.dim[2] - 1);
    const int y0 = max(cy - R, 0), y1 = min(cy + R, S.dim[1] - 1);
    for (int z = z0; z <= z1; ++z) {
        for (int y = y0; y <= y1; ++y) {
            const int row = S.cell_base + S.dim[0] * (y + S.dim[1] * z);
            const int a = max(__ldg(start + row + x0), 0);
            const int b = min(__ldg(start + row + x1 + 1), n);
            fn(a, b);
        }
    }
}

template <bool BATCHED, int R, int BLOCK>
__global__ void __launch_bounds__(BLOCK) k_density(const float4* __restrict__ pos_s, const int* __restrict__ start,
                                                   SceneDev s0, const SceneDev* __restrict__ scenes, int nscene,
                                                   float2* __restrict__ rhop, int n) {
    extern __shared__ float s_d2[];  // [kNbCap][BLOCK]
    float* lst = s_d2 + threadIdx.x;
    for (int t = blockIdx.x * BLOCK + threadIdx.x; t < n; t += gridDim.x * BLOCK) {
        const float4 p = pos_s[t];
        int sc = 0;
        if constexpr (BATCHED) sc = min(max(scene_of(p), 0), nscene - 1);
        const SceneDev& S = scene_params<BATCHED>(s0, scenes, sc);
        const float cut = S.cut_d2, h2 = S.h2;
        const int cx = cell_coord(p.x, S.lo[0], S.inv_edge, S.dim[0]);
        const int cy = cell_coord(p.y, S.lo[1], S.inv_edge, S.dim[1]);
        const int cz = cell_coord(p.z, S.lo[2], S.inv_edge, S.dim[2]);
        float sum = 0.0f, comp = 0.0f;
        int cnt = 0;
        auto flush = [&]() {
            for (int k = 0; k < cnt; ++k) {
                const float w = h2 - lst[k * BLOCK];
                const float yk = w * w * w - comp;  // Kahan step
                const float tk = sum + yk;
                comp = (tk - sum) - yk;
                sum = tk;
            }
            cnt = 0;
        };
        for_rows<R>(S, start, n, cx, cy, cz, [&](int a, int b) {
#pragma unroll 4
            for (int j = a; j < b; ++j) {
                const float4 o = __ldg(pos_s + j);
                float dx, dy, dz;
                const float d2 = canon_d2_pk(p.x, p.y, p.z, o, dx, dy, dz);
                if (d2 < cut) {
                    lst[cnt * BLOCK] = d2;
                    if (++cnt == kNbCap) flush();
                }
            }
        });
        flush();
        const float rho = S.poly6c * sum;
        const float pr = S.gas_k * (rho - S.rho0);
        rhop[t] = make_float2(rho, pr < 0.0f ? 0.0f : pr);  // GLSL max(x, 0): NaN stays NaN
    }
}

template <bool BATCHED, int R, int BLOCK>
__global__ void __launch_bounds__(BLOCK) k_force_integrate(const float4* __restrict__ pos_s, const float4* __restrict__ vel_s,
                                                           const float2* __restrict__ rhop, const int* __restrict__ start,
                                                           SceneDev s0, const SceneDev* __restrict__ scenes, int nscene,
                                                           float4* __restrict__ pos_out, float4* __restrict__ vel_out,
                                                           float4* __restrict__ force_out, int* __restrict__ key_out,
                                                           int* __restrict__ rank_out, int* __restrict__ count, int n) {
    extern __shared__ int s_nb[];  // [kNbCap][BLOCK]
    int* lst = s_nb + threadIdx.x;
    for (int t = blockIdx.x * BLOCK + threadIdx.x; t < n; t += gridDim.x * BLOCK) {
        const float4 p = pos_s[t];
        const float4 v = vel_s[t];
        const float2 rp = rhop[t];
        int sc = 0;
        if constexpr (BATCHED) sc = min(max(scene_of(p), 0), nscene - 1);
        const SceneDev& S = scene_params<BATCHED>(s0, scenes, sc);
        const float cut = S.cut_d2, h = S.h;
        const int cx = cell_coord(p.x, S.lo[0], S.inv_edge, S.dim[0]);
        const int cy = cell_coord(p.y, S.lo[1], S.inv_edge, S.dim[1]);
        const int cz = cell_coord(p.z, S.lo[2], S.inv_edge, S.dim[2]);
        float fpx = 0.f, fpy = 0.f, fpz = 0.f, fvx = 0.f, fvy = 0.f, fvz = 0.f;
        int cnt = 0;
        auto flush = [&]() {
            for (int k = 0; k < cnt; ++k) {
                const int j = lst[k * BLOCK];
                const float4 o = __ldg(pos_s + j);
                const float2 rj = __ldg(rhop + j);
                const float4 vj = __ldg(vel_s + j);
                const float dx = p.x - o.x, dy = p.y - o.y, dz = p.z - o.z;
                const float d2 = dx * dx + dy * dy + dz * dz;
                const float irho = __fdividef(1.0f, rj.x);
                const float inv_r = rsqrtf(d2);
                const float r = d2 > 0.0f ? d2 * inv_r : 0.0f;
                const float hr = h - r;
                const float s = d2 > 0.0f ? (rp.y + rj.y) * irho * hr * hr * inv_r : 0.0f;  // :59 spiky gradient
                fpx += s * dx; fpy += s * dy; fpz += s * dz;
                const float c = irho * hr;                                                // :60 Laplacian
                fvx += c * (vj.x - v.x); fvy += c * (vj.y - v.y); fvz += c * (vj.z - v.z);
            }
            cnt = 0;
        };
        for_rows<R>(S, start, n, cx, cy, cz, [&](int a, int b) {
#pragma unroll 4
            for (int j = a; j < b; ++j) {
                const float4 o = __ldg(pos_s + j);
                float dx, dy, dz;
                const float d2 = canon_d2_pk(p.x, p.y, p.z, o, dx, dy, dz);
                if (d2 < cut && j != t) {  // force_comp.glsl:50-57
                    lst[cnt * BLOCK] = j;
                    if (++cnt == kNbCap) flush();
                }
            }
        });
        flush();
        // :63-66 F = f_p + mu*f_v + rho_i*G (constants folded into pres_c, visc_c)
        const float Fx = S.pres_c * fpx + S.visc_c * fvx + rp.x * S.g[0];
        const float Fy = S.pres_c * fpy + S.visc_c * fvy + rp.x * S.g[1];
        const float Fz = S.pres_c * fpz + S.visc_c * fvz + rp.x * S.g[2];
        // integrate_comp.glsl:41-77
        const float ir = 1.0f / rp.x;
        float nv[3] = {v.x + S.dt * (Fx * ir), v.y + S.dt * (Fy * ir), v.z + S.dt * (Fz * ir)};
        float np[3] = {p.x + S.dt * nv[0], p.y + S.dt * nv[1], p.z + S.dt * nv[2]};
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            if (np[a] < S.lo[a]) { np[a] = S.lo[a]; nv[a] *= -S.damp; }
            else if (np[a] > S.up[a]) { np[a] = S.up[a]; nv[a] *= -S.damp; }
        }
        pos_out[t] = make_float4(np[0], np[1], np[2], p.w);
        vel_out[t] = make_float4(nv[0], nv[1], nv[2], v.w);
        if (force_out) force_out[t] = make_float4(Fx, Fy, Fz, 0.0f);
        // Hash of the new position: the next step's sort starts from here.
        const int c = cell_key(S, np[0], np[1], np[2]);
        key_out[t] = c;
        rank_out[t] = atomicAdd(&count[c], 1);
    }
}

template <class K>
int grid_size(K kernel, int block, size_t smem, int n) {
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, block, smem);
    if (per_sm < 1) per_sm = 1;
    long long need = ((long long)n + block - 1) / block;
    long long cap = (long long)per_sm * device_sm_count();
    return (int)(need < cap ? (need < 1 ? 1 : need) : cap);
}

template <int BLOCK>
constexpr size_t list_bytes() { return (size_t)kNbCap * BLOCK * 4; }

template <bool B, int R, int BLOCK>
void density_impl(const Buffers& b, const SceneDev& s0, cudaStream_t st) {
    auto k = k_density<B, R, BLOCK>;
    const size_t sm = list_bytes<BLOCK>();
    k<<<grid_size(k, BLOCK, sm, b.n), BLOCK, sm, st>>>(b.pos_s, b.start, s0, b.scenes, b.nscene, b.rhop, b.n);
}

template <bool B, int R, int BLOCK>
void force_impl(const Buffers& b, const SceneDev& s0, float4* force_out, cudaStream_t st) {
    auto k = k_force_integrate<B, R, BLOCK>;
    const size_t sm = list_bytes<BLOCK>();
    k<<<grid_size(k, BLOCK, sm, b.n), BLOCK, sm, st>>>(b.pos_s, b.vel_s, b.rhop, b.start, s0, b.scenes, b.nscene,
                                                       b.pos, b.vel, force_out, b.key, b.rank, b.count, b.n);
}

template <bool B, int R>
void set_attrs() {
    cudaFuncSetAttribute(k_density<B, R, 512>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)list_bytes<512>());
    cudaFuncSetAttribute(k_force_integrate<B, R, 512>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)list_bytes<512>());
}

// Calls f(integral_constant<R>, integral_constant<BLOCK>) for the runtime (block, stencil).
template <class F>
void dispatch(int block, int stencil, F f) {
    auto by_block = [&](auto rc) {
        if (block == 128) f(rc, std::integral_constant<int, 128>{});
        else if (block == 512) f(rc, std::integral_constant<int, 512>{});
        else f(rc, std::integral_constant<int, 256>{});
    };
    if (stencil == 2) by_block(std::integral_constant<int, 2>{});
    else by_block(std::integral_constant<int, 1>{});
}

}  // namespace

void init_step_kernels() {
    set_attrs<false, 1>();
    set_attrs<false, 2>();
    set_attrs<true, 1>();
    set_attrs<true, 2>();
}

void launch_density(const Buffers& b, const SceneDev& s0, bool batched, const LaunchCfg& c, cudaStream_t st) {
    if (b.n <= 0) return;
    if (batched)
        dispatch(c.block, c.stencil, [&](auto R, auto BL) { density_impl<true, R.value, BL.value>(b, s0, st); });
    else
        dispatch(c.block, c.stencil, [&](auto R, auto BL) { density_impl<false, R.value, BL.value>(b, s0, st); });
}

void launch_force_integrate(const Buffers& b, const SceneDev& s0, bool batched, const LaunchCfg& c,
                            cudaStream_t st) {
    if (b.n <= 0) return;
    float4* f = s0.keep_force ? b.force_s : nullptr;
    if (batched)
        dispatch(c.block, c.stencil, [&](auto R, auto BL) { force_impl<true, R.value, BL.value>(b, s0, f, st); });
    else
        dispatch(c.block, c.stencil, [&](auto R, auto BL) { force_impl<false, R.value, BL.value>(b, s0, f, st); });
}

}  // namespace sphgb
