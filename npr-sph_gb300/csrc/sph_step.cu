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
// Work decomposition: a CTA takes a chunk of BLOCK consecutive sorted slots
// (one target particle per thread). Consecutive slots share a cell row
// (y, z) -- or a few rows, or several small scenes. For every distinct row of
// the chunk the CTA stages the (2R+1)^2 neighbour-row segments it needs (cells
// x_first-R .. x_last+R of each neighbour row) into shared memory as SoA
// x/y/z arrays, padded to even length with a sentinel that fails every test.
// Each thread then scans the sub-range of each segment that covers its own
// cells cx-R..cx+R, two candidates at a time: one 8-byte shared load per
// coordinate and packed FP32x2 arithmetic (__fadd2_rn / __fmul2_rn, each lane
// rounded on its own, so the neighbour predicate is the canonical FP32
// expression bit for bit). Rounding a sub-range out to even bounds only adds
// candidates from cells two cells away (never within h: cell edge >= h/R with
// margin) or the sentinel.
//
// Density accumulates every candidate branch-free (its weight is zero outside
// r < h). With stencil 1 it also records the predicate r < h of every
// candidate: per segment, two 32-bit masks (even and odd candidates), shifted
// in as it goes and stored column-major (kPairMaskWords coalesced words per
// particle). The force pass then tests nothing: it makes the same chunk plan
// (the same segments and staged offsets, without staging positions), decodes
// the masks into a per-thread list in shared memory and reads the neighbours'
// position, velocity and (rho, p) from global memory. Without a staged tile it
// needs ~37 KB of shared memory per CTA of 256 (~20 per CTA of 128) instead of
// ~80, so more warps hide the gathers' latency and L1 has room for them. A
// segment longer than 32 pairs (a pile-up) is tested by the force pass itself,
// and so is every segment of a chunk on the global-memory path; the particle's
// own bit is dropped (force_comp.glsl:50 skips j == i).
//
// Force processes its list in a second loop in which all lanes are busy: with
// ~15% of candidates inside r < h, testing and interacting in one loop would
// run the ~35-instruction interaction for a minority of lanes almost every
// iteration. The list holds kNbCapForce entries; a longer neighbourhood is
// processed in chunks, in candidate order, so results are deterministic
// either way. With stencil 2 force stages x/y/z like density and tests the
// candidates itself.
//
// A chunk with more distinct rows or more staged candidates than the tile
// holds (heavy pile-ups) takes a global-memory path with the same arithmetic.
//
// Numerics: the density sum is compensated in FP32, by blocks: a plain sum over
// each neighbour-row segment (at most ~30 terms per lane at the densest), then
// a Kahan sum of the segment sums and of the two lanes (relative error a few
// 1e-7 against the FP64 oracle; the global-memory path compensates every term).
// The force sums are plain FP32 with contraction allowed (only the predicate is
// pinned bit-exact).
// For i != j at r == 0 the pressure term is skipped (the shader's
// normalize(0) is NaN, force_comp.glsl:59); the viscosity term is kept.
#include <algorithm>
#include <climits>
#include <type_traits>

#include "sph_device.cuh"

namespace sphgb {

namespace {

// BLOCK threads per CTA = target particles per chunk (256 by default, or 128; autotuned).
// A chunk stages about (2R+1)^2 * (BLOCK + 2R * cell occupancy * rows in the chunk)
// candidates: at most 9.6 * BLOCK (mean 9.4) over the chunks of the 1M dam break's 0.5h
// lattice, its densest state. 12 * BLOCK leaves room for compression and for chunks that
// straddle rows, and keeps the density tile small enough for 5 CTAs of 256 per SM (10 or 11 *
// BLOCK sends many more chunks to the global-memory path); a chunk that needs more takes it.
// With R = 2 (cells of h/2, 25 neighbour rows) a chunk stages ~26 * BLOCK.
template <int R, int BLOCK> constexpr int stage_cap() { return (R == 1 ? 12 : 30) * BLOCK; }
constexpr int kNbCapForce = 48;         // force list entries per thread (u16)
constexpr int kNbCapNb = 42;            // neighbour-list pass entries per thread (u16): three CTAs of
                                        // 256 per SM with the staged tile
constexpr float kSentinel = 1e30f;      // staged padding: its distance to any particle is +inf

template <int R>
struct TileGeom {
    static constexpr int kSide = 2 * R + 1;
    static constexpr int kSegPerRow = kSide * kSide;
    static constexpr int kMaxRows = 16;  // cell rows per chunk tile (more: the global-memory path)
    static constexpr int kMaxSeg = kMaxRows * kSegPerRow;
};

template <int R, int BLOCK>
struct TileShared {
    static constexpr int kWarps = BLOCK / 32;
    int rowid[BLOCK];
    int row_scene[TileGeom<R>::kMaxRows], row_y[TileGeom<R>::kMaxRows], row_z[TileGeom<R>::kMaxRows];
    int row_xa[TileGeom<R>::kMaxRows], row_xb[TileGeom<R>::kMaxRows];
    int seg_gbeg[TileGeom<R>::kMaxSeg], seg_len[TileGeom<R>::kMaxSeg], seg_nrow[TileGeom<R>::kMaxSeg];
    int seg_off[TileGeom<R>::kMaxSeg + 1];
    int warp_cnt[kWarps];
};

struct Staged {
    float* x;
    float* y;
    float* z;
    int* slot;  // global slot of each staged candidate (force only)
};

// Plan and stage one chunk [c0, c0 + BLOCK). Every thread of the CTA calls it.
// Returns false (for the whole CTA) when the chunk does not fit the tile. Without STAGE only
// the plan is made (the same plan and the same decision as with it), and st is not used.
// On return each live thread has its position p, scene sc, cell cx and local row lrow.
template <bool BATCHED, int R, int BLOCK, bool STAGE = true>
__device__ bool stage_chunk(TileShared<R, BLOCK>& T, const Staged& st, int c0, int n, const float4* __restrict__ pos_s,
                            const int* __restrict__ start, const SceneDev& s0, const SceneDev* __restrict__ scenes,
                            int nscene, float4& p, int& sc, int& cx, int& lrow) {
    using G = TileGeom<R>;
    constexpr int kWarps = BLOCK / 32;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int t = c0 + tid;
    const bool live = t < n;
    int cy = 0, cz = 0, rowid = INT_MAX;
    sc = 0;
    cx = 0;
    if (live) {
        p = pos_s[t];
        if constexpr (BATCHED) sc = min(max(scene_of(p), 0), nscene - 1);
        const SceneDev& S = scene_params<BATCHED>(s0, scenes, sc);
        cx = cell_coord(p.x, S.lo[0], S.inv_edge, S.dim[0]);
        cy = cell_coord(p.y, S.lo[1], S.inv_edge, S.dim[1]);
        cz = cell_coord(p.z, S.lo[2], S.inv_edge, S.dim[2]);
        rowid = S.row_base + cy + S.dim[1] * cz;
    }
    T.rowid[tid] = rowid;
    __syncthreads();
    const bool first = live && (tid == 0 || T.rowid[tid - 1] != rowid);
    const bool last = live && (tid == BLOCK - 1 || T.rowid[tid + 1] != rowid);
    const unsigned fb = __ballot_sync(0xffffffffu, first);
    if (lane == 0) T.warp_cnt[warp] = __popc(fb);
    __syncthreads();
    int before = 0, nrows = 0;
#pragma unroll
    for (int w = 0; w < kWarps; ++w) {
        const int c = T.warp_cnt[w];
        before += w < warp ? c : 0;
        nrows += c;
    }
    if (nrows > G::kMaxRows) return false;  // uniform
    lrow = before + __popc(fb & ((1u << lane) - 1)) + (first ? 1 : 0) - 1;
    if (first) {
        T.row_scene[lrow] = sc;
        T.row_y[lrow] = cy;
        T.row_z[lrow] = cz;
        T.row_xa[lrow] = cx;
    }
    if (last) T.row_xb[lrow] = cx;
    __syncthreads();
    const int nseg = nrows * G::kSegPerRow;
    for (int s = tid; s < nseg; s += BLOCK) {
        const int m = s / G::kSegPerRow, r = s % G::kSegPerRow;
        const int dz = r / G::kSide - R, dy = r % G::kSide - R;
        const SceneDev& S = scene_params<BATCHED>(s0, scenes, T.row_scene[m]);
        const int yy = T.row_y[m] + dy, zz = T.row_z[m] + dz;
        int gbeg = 0, len = 0, nrow = 0;
        if (yy >= 0 && yy < S.dim[1] && zz >= 0 && zz < S.dim[2]) {
            nrow = S.cell_base + S.dim[0] * (yy + S.dim[1] * zz);
            const int xa = max(T.row_xa[m] - R, 0), xb = min(T.row_xb[m] + R, S.dim[0] - 1);
            gbeg = min(max(__ldg(start + nrow + xa), 0), n);
            const int gend = min(max(__ldg(start + nrow + xb + 1), 0), n);
            len = max(gend - gbeg, 0);
        }
        T.seg_gbeg[s] = gbeg;
        T.seg_len[s] = len;
        T.seg_nrow[s] = nrow;
    }
    __syncthreads();
    if (warp == 0) {  // exclusive scan of the even-padded segment lengths
        const int per = (nseg + 31) / 32, lo = lane * per, hi = min(lo + per, nseg);
        int local = 0;
        for (int i = lo; i < hi; ++i) local += (T.seg_len[i] + 1) & ~1;
        int incl = local;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int v = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += v;
        }
        int run = incl - local;
        for (int i = lo; i < hi; ++i) {
            T.seg_off[i] = run;
            run += (T.seg_len[i] + 1) & ~1;
        }
        if (lane == 31) T.seg_off[nseg] = incl;
    }
    __syncthreads();
    if (T.seg_off[nseg] > stage_cap<R, BLOCK>()) return false;  // uniform
    if constexpr (STAGE) {  // without it: the plan only (segment table and staged offsets)
        for (int s = warp; s < nseg; s += kWarps) {
            const int gbeg = T.seg_gbeg[s], len = T.seg_len[s], off = T.seg_off[s];
            const int plen = (len + 1) & ~1;
            for (int k = lane; k < plen; k += 32) {
                float x = kSentinel, y = kSentinel, z = kSentinel;
                if (k < len) {
                    const float4 o = __ldg(pos_s + gbeg + k);
                    x = o.x; y = o.y; z = o.z;
                }
                st.x[off + k] = x;
                st.y[off + k] = y;
                st.z[off + k] = z;
                if (st.slot) st.slot[off + k] = k < len ? gbeg + k : 0;
            }
        }
        __syncthreads();
    }
    return true;
}

// Staged sub-range of segment s that covers cells cx-R..cx+R of its row, rounded out to even.
template <int R, int BLOCK>
__device__ __forceinline__ void seg_range(const TileShared<R, BLOCK>& T, int s, int cx, int dimx,
                                          const int* __restrict__ start, int& a, int& b) {
    const int len = T.seg_len[s];
    if (len == 0) { a = b = 0; return; }
    const int nrow = T.seg_nrow[s], gbeg = T.seg_gbeg[s], off = T.seg_off[s];
    const int ga = __ldg(start + nrow + max(cx - R, 0));
    const int gb = __ldg(start + nrow + min(cx + R, dimx - 1) + 1);
    a = off + min(max(ga - gbeg, 0), len);
    b = off + min(max(gb - gbeg, 0), len);
    a &= ~1;
}

// d2 of two staged candidates j, j+1 against (px, py, pz), given as npx = (-px, -px) etc.:
// (x_j - px)^2 + ... is the canonical d2 (the sign of a difference does not change its square).
__device__ __forceinline__ float2 pair_d2(const Staged& st, int j, float2 npx, float2 npy, float2 npz) {
    const float2 X = *reinterpret_cast<const float2*>(st.x + j);
    const float2 Y = *reinterpret_cast<const float2*>(st.y + j);
    const float2 Z = *reinterpret_cast<const float2*>(st.z + j);
    const float2 dx = __fadd2_rn(X, npx), dy = __fadd2_rn(Y, npy), dz = __fadd2_rn(Z, npz);
    return __fadd2_rn(__fadd2_rn(__fmul2_rn(dx, dx), __fmul2_rn(dy, dy)), __fmul2_rn(dz, dz));
}

// Stencil rows around cell (cx, cy, cz) over global memory (the fallback path).
template <int R, class Fn>
__device__ __forceinline__ void for_rows_global(const SceneDev& S, const int* __restrict__ start, int n, int cx, int cy,
                                                int cz, Fn fn) {
    const int x0 = max(cx - R, 0), x1 = min(cx + R, S.dim[0] - 1);
    for (int z = max(cz - R, 0); z <= min(cz + R, S.dim[2] - 1); ++z)
        for (int y = max(cy - R, 0); y <= min(cy + R, S.dim[1] - 1); ++y) {
            const int row = S.cell_base + S.dim[0] * (y + S.dim[1] * z);
            fn(max(__ldg(start + row + x0), 0), min(__ldg(start + row + x1 + 1), n));
        }
}

__device__ __forceinline__ void kahan_add(float& sum, float& comp, float x) {
    const float y = x - comp;
    const float t = sum + y;
    comp = (t - sum) - y;
    sum = t;
}

template <int R, int BLOCK>
constexpr size_t density_smem() { return (size_t)3 * stage_cap<R, BLOCK>() * 4; }
// Stencil 1: the list plus, per thread and segment, the global slot of the segment's first
// staged candidate (the force pass reads neighbours from global memory). Stencil 2: the staged
// tile x, y, z, slot plus the list.
template <int R, int BLOCK>
constexpr size_t force_smem() {
    return R == 1 ? (size_t)kNbCapForce * BLOCK * 2 + (size_t)TileGeom<R>::kSegPerRow * BLOCK * 4
                  : (size_t)4 * stage_cap<R, BLOCK>() * 4 + (size_t)kNbCapForce * BLOCK * 2;
}
template <int R, int BLOCK>
constexpr size_t nb_smem() { return (size_t)4 * stage_cap<R, BLOCK>() * 4 + (size_t)kNbCapNb * BLOCK * 2; }
static_assert(stage_cap<2, 256>() < 65536, "staged indices are 16-bit");
static_assert(kNbCapNb >= kNbList + 2, "the nearest-kNbList pruning runs when two more entries could overflow");

// REC (stencil 1): also the force pass's neighbour records (position, p, velocity, 1/rho).
template <bool BATCHED, int R, int BLOCK, bool REC>
__global__ void __launch_bounds__(BLOCK) k_density(const float4* __restrict__ pos_s, const float4* __restrict__ vel_s,
                                                   const int* __restrict__ start, SceneDev s0,
                                                   const SceneDev* __restrict__ scenes, int nscene,
                                                   float2* __restrict__ rhop, uint32_t* __restrict__ pmask,
                                                   float4* __restrict__ rec, int n, uint32_t* __restrict__ stats) {
    using G = TileGeom<R>;
    constexpr int kCap = stage_cap<R, BLOCK>();
    constexpr bool kMask = R == 1;  // pair masks for the force pass (kPairMaskWords words per particle)
    static_assert(!kMask || 2 * G::kSegPerRow == kPairMaskWords, "two mask words per segment");
    static_assert(!REC || kMask, "neighbour records are written for stencil 1");
    __shared__ TileShared<R, BLOCK> T;
    extern __shared__ float4 dyn_d[];
    float* base = reinterpret_cast<float*>(dyn_d);
    const Staged st{base, base + kCap, base + 2 * kCap, nullptr};
    for (int c0 = blockIdx.x * BLOCK; c0 < n; c0 += gridDim.x * BLOCK) {
        float4 p = make_float4(0.f, 0.f, 0.f, 0.f);
        int sc = 0, cx = 0, lrow = 0;
        const bool tiled =
            stage_chunk<BATCHED, R, BLOCK>(T, st, c0, n, pos_s, start, s0, scenes, nscene, p, sc, cx, lrow);
        const int t = c0 + threadIdx.x;
        if (t < n) {
            if (!tiled) p = pos_s[t];
            if constexpr (BATCHED) sc = min(max(scene_of(p), 0), nscene - 1);
            const SceneDev& S = scene_params<BATCHED>(s0, scenes, sc);
            const float cut = S.cut_d2;
            float sum = 0.0f, comp = 0.0f;
            if (tiled) {
                // Branch-free: every candidate adds max(cut - d2, 0)^3, two per step in packed
                // lanes, each lane its own blocked compensated sum. cut - d2 is the negated
                // difference the neighbour masks take their sign from, so the weight is zero
                // exactly where the predicate d2 < cut fails; it differs from h^2 - d2 by at most
                // the ulp between cut and h^2 (a relative density change below 1e-7).
                const float2 npx = make_float2(-p.x, -p.x), npy = make_float2(-p.y, -p.y);
                const float2 npz = make_float2(-p.z, -p.z);
                const float2 ncut = make_float2(-cut, -cut);
                float2 s2 = make_float2(0.f, 0.f), c2 = make_float2(0.f, 0.f);
#pragma unroll
                for (int r = 0; r < G::kSegPerRow; ++r) {
                    int a, b;
                    seg_range<R, BLOCK>(T, lrow * G::kSegPerRow + r, cx, S.dim[0], start, a, b);
                    uint32_t mx = 0, my = 0;
                    float2 seg = make_float2(0.f, 0.f);
#pragma unroll 2
                    for (int j = a; j < b; j += 2) {
                        const float2 d2 = pair_d2(st, j, npx, npy, npz);
                        // d2 - cut is negative exactly when d2 < cut (a difference of two distinct
                        // floats is never zero; +inf and NaN are positive): its sign bit is the
                        // force pass's predicate, shifted in as the masks' new lowest bit
                        const float2 e = __fadd2_rn(d2, ncut);
                        const float2 w = make_float2(fmaxf(-e.x, 0.0f), fmaxf(-e.y, 0.0f));
                        seg = __ffma2_rn(__fmul2_rn(w, w), w, seg);
                        if constexpr (kMask) {
                            mx = __funnelshift_l(__float_as_uint(e.x), mx, 1);
                            my = __funnelshift_l(__float_as_uint(e.y), my, 1);
                        }
                    }
                    {  // Kahan, per lane, of the segment's sum
                        const float2 y = __fadd2_rn(seg, make_float2(-c2.x, -c2.y));
                        const float2 tt = __fadd2_rn(s2, y);
                        const float2 lost = __fadd2_rn(tt, make_float2(-s2.x, -s2.y));
                        c2 = __fadd2_rn(lost, make_float2(-y.x, -y.y));
                        s2 = tt;
                    }
                    if constexpr (kMask) {
                        pmask[(size_t)(2 * r) * n + t] = mx;
                        pmask[(size_t)(2 * r + 1) * n + t] = my;
                    }
                }
                // combine the two lanes: (s.x - c.x) + (s.y - c.y) with a compensated add
                kahan_add(sum, comp, s2.x);
                kahan_add(sum, comp, -c2.x);
                kahan_add(sum, comp, s2.y);
                kahan_add(sum, comp, -c2.y);
            } else {
                const int gx = cell_coord(p.x, S.lo[0], S.inv_edge, S.dim[0]);
                const int gy = cell_coord(p.y, S.lo[1], S.inv_edge, S.dim[1]);
                const int gz = cell_coord(p.z, S.lo[2], S.inv_edge, S.dim[2]);
                for_rows_global<R>(S, start, n, gx, gy, gz, [&](int a, int b) {
                    for (int j = a; j < b; ++j) {
                        const float4 o = __ldg(pos_s + j);
                        float dx, dy, dz;
                        const float d2 = canon_d2(p.x, p.y, p.z, o.x, o.y, o.z, dx, dy, dz);
                        if (d2 < cut) {
                            const float w = cut - d2;
                            kahan_add(sum, comp, w * w * w);
                        }
                    }
                });
            }
            const float rho = S.poly6c * sum;
            const float pr = S.gas_k * (rho - S.rho0);
            const float prc = pr < 0.0f ? 0.0f : pr;  // GLSL max(x, 0): NaN stays NaN
            rhop[t] = make_float2(rho, prc);
            if constexpr (REC) {  // the force pass's neighbour record: one 32-byte load per neighbour
                const float4 v = vel_s[t];
                rec[2 * (size_t)t] = make_float4(p.x, p.y, p.z, prc);
                rec[2 * (size_t)t + 1] = make_float4(v.x, v.y, v.z, __fdividef(1.0f, rho));
            }
        }
        if (!tiled && threadIdx.x == 0 && stats) atomicAdd(&stats[0], 1u);
        __syncthreads();  // the next chunk reuses the tile
    }
}

// One 32-byte record (two float4) in a single 256-bit read-only load; r is 32-byte aligned.
__device__ __forceinline__ void ld_record(const float4* r, float4& a, float4& b) {
    asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
        : "=f"(a.x), "=f"(a.y), "=f"(a.z), "=f"(a.w), "=f"(b.x), "=f"(b.y), "=f"(b.z), "=f"(b.w)
        : "l"(r));
}

struct ForceAcc {
    float2 fp_xy = make_float2(0.f, 0.f), fv_xy = make_float2(0.f, 0.f);
    float fpz = 0.f, fvz = 0.f;
    // force_comp.glsl:59-60 for one neighbour j at offset (dx, dy, dz) = x_i - x_j; the x/y
    // lanes of the two vector sums run as packed FP32x2 operations.
    __device__ __forceinline__ void add(float dx, float dy, float dz, float h, float pi, float4 v, float2 rj,
                                        float4 vj) {
        add(dx, dy, dz, h, pi, v, rj.y, __fdividef(1.0f, rj.x), vj);
    }
    // The same with the neighbour's pressure pj and 1/rho_j (as __fdividef(1, rho_j)) given.
    __device__ __forceinline__ void add(float dx, float dy, float dz, float h, float pi, float4 v, float pj, float irho,
                                        float4 vj) {
        const float d2 = dx * dx + dy * dy + dz * dz;
        const float inv_r = rsqrtf(d2);
        const float r = d2 > 0.0f ? d2 * inv_r : 0.0f;
        const float hr = h - r;
        const float s = d2 > 0.0f ? (pi + pj) * irho * hr * hr * inv_r : 0.0f;  // spiky gradient
        fp_xy = __ffma2_rn(make_float2(s, s), make_float2(dx, dy), fp_xy);
        fpz = fmaf(s, dz, fpz);
        const float c = irho * hr;                                                // Laplacian
        const float2 dv = __fadd2_rn(make_float2(vj.x, vj.y), make_float2(-v.x, -v.y));
        fv_xy = __ffma2_rn(make_float2(c, c), dv, fv_xy);
        fvz = fmaf(c, vj.z - v.z, fvz);
    }
};

// DIGEST (stencil 1): also the count (self included) and the digest sum mix64(id) of the
// neighbours each particle interacted with, per sorted slot, as sph_neighbor_digest reports them.
// REC (stencil 1): each neighbour is read as the density pass's 32-byte record, otherwise from
// the state arrays; the interactions are the same either way.
template <bool BATCHED, int R, int BLOCK, bool DIGEST, bool REC>
__global__ void __launch_bounds__(BLOCK) k_force_integrate(const float4* __restrict__ pos_s, const float4* __restrict__ vel_s,
                                                           const float2* __restrict__ rhop, const int* __restrict__ start,
                                                           SceneDev s0, const SceneDev* __restrict__ scenes, int nscene,
                                                           float4* __restrict__ pos_out, float4* __restrict__ vel_out,
                                                           float4* __restrict__ force_out, int* __restrict__ key_out,
                                                           int* __restrict__ rank_out, int* __restrict__ count,
                                                           const uint32_t* __restrict__ pmask,
                                                           const float4* __restrict__ rec, int n,
                                                           uint32_t* __restrict__ stats, uint32_t* __restrict__ dig_cnt,
                                                           unsigned long long* __restrict__ dig_sum) {
    using G = TileGeom<R>;
    constexpr int kCap = stage_cap<R, BLOCK>();
    constexpr bool kMask = R == 1;  // the density pass's pair masks replace the candidate tests
    static_assert(!DIGEST || kMask, "the neighbour digest of the force pass is for stencil 1");
    static_assert(!REC || kMask, "neighbour records are written for stencil 1");
    __shared__ TileShared<R, BLOCK> T;
    extern __shared__ float4 dyn_f[];
    float* base = reinterpret_cast<float*>(dyn_f);
    // Stencil 1: [kNbCapForce][BLOCK] list entries (segment * 4096 + candidate offset), then
    // [kSegPerRow][BLOCK] global slots of the segments' first candidates. Stencil 2: the staged
    // tile, then [kNbCapForce][BLOCK] list entries (staged indices).
    const Staged st = kMask ? Staged{nullptr, nullptr, nullptr, nullptr}
                            : Staged{base, base + kCap, base + 2 * kCap, reinterpret_cast<int*>(base + 3 * kCap)};
    unsigned short* lst = reinterpret_cast<unsigned short*>(kMask ? base : base + 4 * kCap) + threadIdx.x;
    int* seg_slot = reinterpret_cast<int*>(base) + (kNbCapForce * BLOCK) / 2 + threadIdx.x;  // stencil 1 only
    for (int c0 = blockIdx.x * BLOCK; c0 < n; c0 += gridDim.x * BLOCK) {
        float4 p = make_float4(0.f, 0.f, 0.f, 0.f);
        int sc = 0, cx = 0, lrow = 0;
        const bool tiled = stage_chunk<BATCHED, R, BLOCK, !kMask>(T, st, c0, n, pos_s, start, s0, scenes, nscene, p,
                                                                  sc, cx, lrow);
        const int t = c0 + threadIdx.x;
        if (t < n) {
            if (!tiled) p = pos_s[t];
            if constexpr (BATCHED) sc = min(max(scene_of(p), 0), nscene - 1);
            const SceneDev& S = scene_params<BATCHED>(s0, scenes, sc);
            const float4 v = vel_s[t];
            const float2 rp = rhop[t];
            const float cut = S.cut_d2, h = S.h;
            ForceAcc acc;
            // Stencil 2 keeps the particle itself in the list (force_comp.glsl:50-53 skips j == i):
            // its offset and relative velocity are exactly zero, so its pressure term is skipped
            // (d2 == 0) and its viscosity term adds zeros. Stencil 1 leaves it out.
            int cnt = 0;
            uint32_t dcount = 1;                                                 // DIGEST: self
            unsigned long long dsum = mix64((unsigned long long)id_of(v));
            // Stencil 1: neighbours come from global memory: the density pass's 32-byte record
            // (position, p_j, velocity, 1/rho_j) in one load when this step has records, else
            // position, velocity and (rho, p) from the state arrays. List entry e is candidate
            // e & 4095 of row segment e >> 12, whose first candidate is global slot seg_slot[segment].
            auto interact = [&](int g) {
                float4 q, vj;
                if constexpr (REC) {
                    ld_record(rec + 2 * (size_t)g, q, vj);
                    acc.add(p.x - q.x, p.y - q.y, p.z - q.z, h, rp.y, v, q.w, vj.w, vj);
                } else {
                    q = __ldg(pos_s + g);
                    vj = __ldg(vel_s + g);
                    acc.add(p.x - q.x, p.y - q.y, p.z - q.z, h, rp.y, v, __ldg(rhop + g), vj);
                }
                if constexpr (DIGEST) {
                    ++dcount;
                    dsum += mix64((unsigned long long)id_of(__ldg(vel_s + g)));
                }
            };
            auto flush_slots = [&]() {
                for (int k = 0; k < cnt; ++k) {
                    const int e = lst[BLOCK * k];
                    interact(seg_slot[BLOCK * (e >> 12)] + (e & 4095));
                }
                cnt = 0;
            };
            // Test candidates [g0, g1) of row segment r from global memory; the passing ones join
            // the list (a candidate beyond 4095 of its segment, in a pile-up, interacts at once).
            auto test_row = [&](int r, int g0, int g1) {
                seg_slot[BLOCK * r] = g0;
                for (int g = g0; g < g1; ++g) {
                    const float4 q = __ldg(pos_s + g);
                    float dx, dy, dz;
                    const float d2 = canon_d2(p.x, p.y, p.z, q.x, q.y, q.z, dx, dy, dz);
                    if (d2 < cut && g != t) {  // :50-57
                        if (g - g0 < 4096) {
                            lst[BLOCK * cnt++] = (unsigned short)(r * 4096 + (g - g0));
                            if (cnt == kNbCapForce) flush_slots();
                        } else {
                            interact(g);
                        }
                    }
                }
            };
            if (tiled) {
                if constexpr (kMask) {
                    // All masks are loaded up front (one coalesced word per segment and parity).
                    // Pair k of a segment's staged [a, b) is bit np-1-k of its masks when the
                    // segment has np <= 32 pairs; a longer segment lost its first bits and is
                    // tested here, from global memory.
                    uint32_t m[kPairMaskWords];
#pragma unroll
                    for (int w = 0; w < kPairMaskWords; ++w) m[w] = __ldg(pmask + (size_t)w * n + t);
#pragma unroll
                    for (int r = 0; r < G::kSegPerRow; ++r) {
                        const int sg = lrow * G::kSegPerRow + r;
                        int a, b;
                        seg_range<R, BLOCK>(T, sg, cx, S.dim[0], start, a, b);
                        const int np = (b - a + 1) >> 1;
                        const int g0 = T.seg_gbeg[sg] + (a - T.seg_off[sg]);  // global slot of staged a
                        if (np > 32) {
                            test_row(r, g0, g0 + (b - a));
                            continue;
                        }
                        seg_slot[BLOCK * r] = g0;
                        if (r == R * G::kSide + R) {  // the particle's own row: drop its own bit (j == i)
                            const int o = t - g0;    // in [0, 2 np): the row holds the particle's cell
                            if (o >= 0 && o < 2 * np) {
                                const uint32_t bit = 1u << (np - 1 - (o >> 1));
                                m[2 * r] &= (o & 1) ? ~0u : ~bit;
                                m[2 * r + 1] &= (o & 1) ? ~bit : ~0u;
                            }
                        }
#pragma unroll
                        for (int par = 0; par < 2; ++par) {
                            uint32_t mk = m[2 * r + par];
                            while (mk) {  // highest bit first: candidate order
                                const int bit = 31 - __clz(mk);
                                mk ^= 1u << bit;
                                lst[BLOCK * cnt++] = (unsigned short)(r * 4096 + 2 * (np - 1 - bit) + par);
                                if (cnt == kNbCapForce) flush_slots();
                            }
                        }
                    }
                    flush_slots();
                } else {
                    auto flush = [&]() {
                        for (int k = 0; k < cnt; ++k) {
                            const int j = lst[BLOCK * k];
                            const int g = st.slot[j];
                            acc.add(p.x - st.x[j], p.y - st.y[j], p.z - st.z[j], h, rp.y, v, __ldg(rhop + g),
                                    __ldg(vel_s + g));
                        }
                        cnt = 0;
                    };
                    const float2 npx = make_float2(-p.x, -p.x), npy = make_float2(-p.y, -p.y);
                    const float2 npz = make_float2(-p.z, -p.z);
#pragma unroll 1
                    for (int r = 0; r < G::kSegPerRow; ++r) {
                        int a, b;
                        seg_range<R, BLOCK>(T, lrow * G::kSegPerRow + r, cx, S.dim[0], start, a, b);
#pragma unroll 2
                        for (int j = a; j < b; j += 2) {
                            const float2 d2 = pair_d2(st, j, npx, npy, npz);
                            if (d2.x < cut) lst[BLOCK * cnt++] = (unsigned short)j;  // :57
                            if (d2.y < cut) lst[BLOCK * cnt++] = (unsigned short)(j + 1);
                            if (cnt > kNbCapForce - 2) flush();
                        }
                    }
                    flush();
                }
            } else {
                const int gx = cell_coord(p.x, S.lo[0], S.inv_edge, S.dim[0]);
                const int gy = cell_coord(p.y, S.lo[1], S.inv_edge, S.dim[1]);
                const int gz = cell_coord(p.z, S.lo[2], S.inv_edge, S.dim[2]);
                if constexpr (kMask) {  // the same list, rows tested from global memory
                    const int x0 = max(gx - 1, 0), x1 = min(gx + 1, S.dim[0] - 1);
                    int r = 0;
                    for (int z = max(gz - 1, 0); z <= min(gz + 1, S.dim[2] - 1); ++z)
                        for (int y = max(gy - 1, 0); y <= min(gy + 1, S.dim[1] - 1); ++y, ++r) {
                            const int row = S.cell_base + S.dim[0] * (y + S.dim[1] * z);
                            test_row(r, max(__ldg(start + row + x0), 0), min(__ldg(start + row + x1 + 1), n));
                        }
                    flush_slots();
                } else {
                    for_rows_global<R>(S, start, n, gx, gy, gz, [&](int a, int b) {
                        for (int j = a; j < b; ++j) {
                            const float4 o = __ldg(pos_s + j);
                            float dx, dy, dz;
                            const float d2 = canon_d2(p.x, p.y, p.z, o.x, o.y, o.z, dx, dy, dz);
                            if (d2 < cut && j != t)
                                acc.add(dx, dy, dz, h, rp.y, v, __ldg(rhop + j), __ldg(vel_s + j));
                        }
                    });
                }
            }
            // :63-66 F = f_p + mu*f_v + rho_i*G (constants folded into pres_c, visc_c)
            const float Fx = S.pres_c * acc.fp_xy.x + S.visc_c * acc.fv_xy.x + rp.x * S.g[0];
            const float Fy = S.pres_c * acc.fp_xy.y + S.visc_c * acc.fv_xy.y + rp.x * S.g[1];
            const float Fz = S.pres_c * acc.fpz + S.visc_c * acc.fvz + rp.x * S.g[2];
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
            if constexpr (DIGEST) {
                dig_cnt[t] = dcount;
                dig_sum[t] = dsum;
            }
            if (force_out) force_out[t] = make_float4(Fx, Fy, Fz, 0.0f);
            // Hash of the new position: the next step's sort starts from here (with an obstacle,
            // k_obstacle_hash hashes after moving the particles out of it).
            if (key_out) {
                const int c = cell_key(S, np[0], np[1], np[2]);
                key_out[t] = c;
                rank_out[t] = atomicAdd(&count[c], 1);
            }
        }
        if (!tiled && threadIdx.x == 0 && stats) atomicAdd(&stats[1], 1u);
        __syncthreads();  // the next chunk reuses the tile
    }
}

// ---- density + nearest-neighbour lists (the learned macro-step's input) ---------------------

// Keep the kNbList nearest entries of a per-thread list of staged indices (stride BLOCK in
// shared memory): the farthest entry is removed until kNbList remain (ties: the later entry).
template <int BLOCK>
__device__ __forceinline__ void prune_nearest(unsigned short* lst, int& cnt, const Staged& st, float px, float py,
                                              float pz) {
    while (cnt > kNbList) {
        float worst = -1.0f;
        int wk = 0;
        for (int k = 0; k < cnt; ++k) {
            const int j = lst[BLOCK * k];
            const float dx = st.x[j] - px, dy = st.y[j] - py, dz = st.z[j] - pz;
            const float d2 = __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
            if (d2 >= worst) { worst = d2; wk = k; }
        }
        lst[BLOCK * wk] = lst[BLOCK * (cnt - 1)];
        --cnt;
    }
}

template <bool BATCHED, int R, int BLOCK>
// 64 registers at most (shared memory holds it to fewer CTAs per SM than that allows).
__global__ void __launch_bounds__(BLOCK, 1024 / BLOCK) k_density_nb(const float4* __restrict__ pos_s, const int* __restrict__ start,
                                                      SceneDev s0, const SceneDev* __restrict__ scenes, int nscene,
                                                      float2* __restrict__ rhop, int* __restrict__ nb,
                                                      int* __restrict__ nbc, int n, uint32_t* __restrict__ stats) {
    using G = TileGeom<R>;
    constexpr int kCap = stage_cap<R, BLOCK>();
    __shared__ TileShared<R, BLOCK> T;
    extern __shared__ float4 dyn_n[];
    float* base = reinterpret_cast<float*>(dyn_n);
    const Staged st{base, base + kCap, base + 2 * kCap, reinterpret_cast<int*>(base + 3 * kCap)};
    unsigned short* lst = reinterpret_cast<unsigned short*>(base + 4 * kCap) + threadIdx.x;  // [kNbCapNb][BLOCK]
    for (int c0 = blockIdx.x * BLOCK; c0 < n; c0 += gridDim.x * BLOCK) {
        float4 p = make_float4(0.f, 0.f, 0.f, 0.f);
        int sc = 0, cx = 0, lrow = 0;
        const bool tiled =
            stage_chunk<BATCHED, R, BLOCK>(T, st, c0, n, pos_s, start, s0, scenes, nscene, p, sc, cx, lrow);
        const int t = c0 + threadIdx.x;
        int c = 0;
        if (t < n) {
            if (!tiled) p = pos_s[t];
            if constexpr (BATCHED) sc = min(max(scene_of(p), 0), nscene - 1);
            const SceneDev& S = scene_params<BATCHED>(s0, scenes, sc);
            const float cut = S.cut_d2;
            float sum = 0.0f, comp = 0.0f;
            int* out = nb + (size_t)t * kNbList;
            if (tiled) {
                // density: the arithmetic of k_density, candidate for candidate; list: the passing
                // candidates other than the particle itself, pruned to the nearest kNbList
                const float2 npx = make_float2(-p.x, -p.x), npy = make_float2(-p.y, -p.y);
                const float2 npz = make_float2(-p.z, -p.z);
                const float2 ncut = make_float2(-cut, -cut);
                float2 s2 = make_float2(0.f, 0.f), c2 = make_float2(0.f, 0.f);
                // the particle's own staged index: its row's centre segment (dy = dz = 0) holds it
                const int cseg = lrow * G::kSegPerRow + R * G::kSide + R;
                const int self_j = T.seg_off[cseg] + (t - T.seg_gbeg[cseg]);
#pragma unroll 1
                for (int r = 0; r < G::kSegPerRow; ++r) {
                    int a, b;
                    seg_range<R, BLOCK>(T, lrow * G::kSegPerRow + r, cx, S.dim[0], start, a, b);
                    float2 seg = make_float2(0.f, 0.f);
                    uint32_t mx = 0, my = 0;  // the predicates, as in k_density: pair k at bit np-1-k
#pragma unroll 2
                    for (int j = a; j < b; j += 2) {
                        const float2 d2 = pair_d2(st, j, npx, npy, npz);
                        const float2 e = __fadd2_rn(d2, ncut);
                        const float2 w = make_float2(fmaxf(-e.x, 0.0f), fmaxf(-e.y, 0.0f));
                        seg = __ffma2_rn(__fmul2_rn(w, w), w, seg);
                        mx = __funnelshift_l(__float_as_uint(e.x), mx, 1);
                        my = __funnelshift_l(__float_as_uint(e.y), my, 1);
                    }
                    // The segment's neighbours into the list, from the masks (a segment of more
                    // than 32 pairs lost its first bits and is tested again). d2 < cut exactly
                    // where the sign bit of d2 - cut is set.
                    const int np = (b - a + 1) >> 1;
                    if (np <= 32) {
#pragma unroll
                        for (int par = 0; par < 2; ++par) {
                            uint32_t mk = par ? my : mx;
                            while (mk) {
                                const int bit = 31 - __clz(mk);
                                mk ^= 1u << bit;
                                const int j = a + 2 * (np - 1 - bit) + par;
                                if (j == self_j) continue;
                                lst[BLOCK * c++] = (unsigned short)j;
                                if (c > kNbCapNb - 2) prune_nearest<BLOCK>(lst, c, st, p.x, p.y, p.z);
                            }
                        }
                    } else {
                        for (int j = a; j < b; j += 2) {
                            const float2 d2 = pair_d2(st, j, npx, npy, npz);
                            if (d2.x < cut && j != self_j) lst[BLOCK * c++] = (unsigned short)j;
                            if (d2.y < cut && j + 1 != self_j) lst[BLOCK * c++] = (unsigned short)(j + 1);
                            if (c > kNbCapNb - 2) prune_nearest<BLOCK>(lst, c, st, p.x, p.y, p.z);
                        }
                    }
                    {  // Kahan, per lane, of the segment's sum
                        const float2 y = __fadd2_rn(seg, make_float2(-c2.x, -c2.y));
                        const float2 tt = __fadd2_rn(s2, y);
                        const float2 lost = __fadd2_rn(tt, make_float2(-s2.x, -s2.y));
                        c2 = __fadd2_rn(lost, make_float2(-y.x, -y.y));
                        s2 = tt;
                    }
                }
                kahan_add(sum, comp, s2.x);
                kahan_add(sum, comp, -c2.x);
                kahan_add(sum, comp, s2.y);
                kahan_add(sum, comp, -c2.y);
                prune_nearest<BLOCK>(lst, c, st, p.x, p.y, p.z);
                c = min(c, kNbList);  // the rows are written below, a warp at a time
            } else {
                // global-memory path: the list lives in the output row itself
                float worst = -1.0f;
                int wpos = 0;
                const int gx = cell_coord(p.x, S.lo[0], S.inv_edge, S.dim[0]);
                const int gy = cell_coord(p.y, S.lo[1], S.inv_edge, S.dim[1]);
                const int gz = cell_coord(p.z, S.lo[2], S.inv_edge, S.dim[2]);
                for_rows_global<R>(S, start, n, gx, gy, gz, [&](int a, int b) {
                    for (int j = a; j < b; ++j) {
                        const float4 o = __ldg(pos_s + j);
                        float dx, dy, dz;
                        const float d2 = canon_d2(p.x, p.y, p.z, o.x, o.y, o.z, dx, dy, dz);
                        if (!(d2 < cut)) continue;
                        const float wgt = cut - d2;
                        kahan_add(sum, comp, wgt * wgt * wgt);
                        if (j == t) continue;
                        if (c < kNbList) {
                            out[c] = j;
                            if (d2 >= worst) { worst = d2; wpos = c; }
                            ++c;
                        } else if (d2 < worst) {
                            out[wpos] = j;
                            worst = -1.0f;
                            for (int k = 0; k < kNbList; ++k) {
                                const float4 q = __ldg(pos_s + out[k]);
                                float ex, ey, ez;
                                const float e2 = canon_d2(p.x, p.y, p.z, q.x, q.y, q.z, ex, ey, ez);
                                if (e2 >= worst) { worst = e2; wpos = k; }
                            }
                        }
                    }
                });
                for (int k = c; k < kNbList; ++k) out[k] = -1;
            }
            nbc[t] = min(c, kNbList);
            const float rho = S.poly6c * sum;
            const float pr = S.gas_k * (rho - S.rho0);
            rhop[t] = make_float2(rho, pr < 0.0f ? 0.0f : pr);
        }
        if (tiled) {  // uniform: the warp writes its 32 particles' rows, one 128-byte row per store
            const int lane = threadIdx.x & 31, w0 = threadIdx.x - lane;
            const unsigned short* lst0 = reinterpret_cast<const unsigned short*>(base + 4 * kCap);
#pragma unroll 1
            for (int r = 0; r < 32; ++r) {
                const int cr = __shfl_sync(0xffffffffu, c, r);
                const int tr = c0 + w0 + r;
                if (tr < n) nb[(size_t)tr * kNbList + lane] = lane < cr ? st.slot[lst0[BLOCK * lane + w0 + r]] : -1;
            }
        }
        if (!tiled && threadIdx.x == 0 && stats) atomicAdd(&stats[0], 1u);
        __syncthreads();
    }
}

// One CTA per chunk: the block scheduler hands the next chunk to whichever SM frees a slot,
// which balances chunks of uneven cost (dense pile-ups, empty rows, scenes of different sizes)
// better than a persistent grid of resident CTAs looping over a fixed share of the chunks
// (measured 3% faster on the 1M dam break, 9% on 256 batched scenes). The kernels keep their
// chunk loops, so any grid is correct.
template <class K>
int grid_size(K, int block, size_t, int n) {
    const long long need = ((long long)n + block - 1) / block;
    return (int)(need < 1 ? 1 : need);
}

template <bool B, int R, int BLOCK>
void density_impl(const Buffers& b, const SceneDev& s0, bool rec, cudaStream_t st) {
    constexpr size_t sm = density_smem<R, BLOCK>();
    auto launch = [&](auto k) {
        k<<<grid_size(k, BLOCK, sm, b.n), BLOCK, sm, st>>>(b.pos_s, b.vel_s, b.start, s0, b.scenes, b.nscene, b.rhop,
                                                           b.pmask, b.rec, b.n, b.tile_stats);
    };
    if constexpr (R == 1) {
        if (rec) {
            launch(k_density<B, R, BLOCK, true>);
            return;
        }
    }
    launch(k_density<B, R, BLOCK, false>);
}

template <bool B, int R, int BLOCK>
void force_impl(const Buffers& b, const SceneDev& s0, bool rec, float4* force_out, uint32_t* dig_cnt,
                unsigned long long* dig_sum, cudaStream_t st) {
    constexpr size_t sm = force_smem<R, BLOCK>();
    auto launch = [&](auto k) {
        k<<<grid_size(k, BLOCK, sm, b.n), BLOCK, sm, st>>>(b.pos_s, b.vel_s, b.rhop, b.start, s0, b.scenes, b.nscene,
                                                           b.pos, b.vel, force_out, s0.sdf ? nullptr : b.key, b.rank,
                                                           b.count, b.pmask, b.rec, b.n, b.tile_stats,
                                                           dig_cnt, dig_sum);
    };
    if constexpr (R == 1) {
        if (dig_cnt) {  // the digest pass runs without records
            launch(k_force_integrate<B, R, BLOCK, true, false>);
            return;
        }
        if (rec) {
            launch(k_force_integrate<B, R, BLOCK, false, true>);
            return;
        }
    }
    launch(k_force_integrate<B, R, BLOCK, false, false>);
}

// The static obstacle's rule (sph_set_obstacle) on the integrated state, then the cell hash of
// the final positions (the force kernel leaves the hash to this kernel when there is an
// obstacle). One thread per slot.
template <bool BATCHED>
__global__ void __launch_bounds__(256) k_obstacle_hash(float4* __restrict__ pos, float4* __restrict__ vel, SceneDev s0,
                                                       const SceneDev* __restrict__ scenes, int nscene,
                                                       int* __restrict__ key_out, int* __restrict__ rank_out,
                                                       int* __restrict__ count, int n) {
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        const float4 p = pos[t], v = vel[t];
        int sc = 0;
        if constexpr (BATCHED) sc = min(max(scene_of(p), 0), nscene - 1);
        const SceneDev& S = scene_params<BATCHED>(s0, scenes, sc);
        float x[3] = {p.x, p.y, p.z}, u[3] = {v.x, v.y, v.z};
        obstacle_response(S, x, u);
        if (x[0] != p.x || x[1] != p.y || x[2] != p.z || u[0] != v.x || u[1] != v.y || u[2] != v.z) {
            pos[t] = make_float4(x[0], x[1], x[2], p.w);
            vel[t] = make_float4(u[0], u[1], u[2], v.w);
        }
        const int c = cell_key(S, x[0], x[1], x[2]);
        key_out[t] = c;
        rank_out[t] = atomicAdd(&count[c], 1);
    }
}

template <bool B, int R, int BLOCK>
void density_nb_impl(const Buffers& b, const SceneDev& s0, int* nb, int* cnt, cudaStream_t st) {
    auto k = k_density_nb<B, R, BLOCK>;
    constexpr size_t sm = nb_smem<R, BLOCK>();
    k<<<grid_size(k, BLOCK, sm, b.n), BLOCK, sm, st>>>(b.pos_s, b.start, s0, b.scenes, b.nscene, b.rhop, nb, cnt, b.n,
                                                   b.tile_stats);
}

template <bool B, int R, int BLOCK>
void set_attrs() {
    cudaFuncSetAttribute(k_density<B, R, BLOCK, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)density_smem<R, BLOCK>());
    cudaFuncSetAttribute(k_force_integrate<B, R, BLOCK, false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)force_smem<R, BLOCK>());
    if constexpr (R == 1) {
        cudaFuncSetAttribute(k_density<B, R, BLOCK, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)density_smem<R, BLOCK>());
        cudaFuncSetAttribute(k_force_integrate<B, R, BLOCK, true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)force_smem<R, BLOCK>());
        cudaFuncSetAttribute(k_force_integrate<B, R, BLOCK, false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)force_smem<R, BLOCK>());
    }
    cudaFuncSetAttribute(k_density_nb<B, R, BLOCK>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)nb_smem<R, BLOCK>());
}

// Calls f(integral_constant<R>, integral_constant<BLOCK>) for the runtime (block, stencil).
template <class F>
void dispatch(int block, int stencil, F f) {
    auto by_block = [&](auto rc) {
        if (block == 128) f(rc, std::integral_constant<int, 128>{});
        else f(rc, std::integral_constant<int, 256>{});
    };
    if (stencil == 2) by_block(std::integral_constant<int, 2>{});
    else by_block(std::integral_constant<int, 1>{});
}

}  // namespace

void init_step_kernels() {
    set_attrs<false, 1, 128>();
    set_attrs<false, 1, 256>();
    set_attrs<false, 2, 128>();
    set_attrs<false, 2, 256>();
    set_attrs<true, 1, 128>();
    set_attrs<true, 1, 256>();
    set_attrs<true, 2, 128>();
    set_attrs<true, 2, 256>();
}

void launch_density(const Buffers& b, const SceneDev& s0, bool batched, const LaunchCfg& c, bool rec, cudaStream_t st) {
    if (b.n <= 0) return;
    if (batched)
        dispatch(c.block, c.stencil, [&](auto R, auto BL) { density_impl<true, R.value, BL.value>(b, s0, rec, st); });
    else
        dispatch(c.block, c.stencil, [&](auto R, auto BL) { density_impl<false, R.value, BL.value>(b, s0, rec, st); });
}

void launch_force_integrate(const Buffers& b, const SceneDev& s0, bool batched, const LaunchCfg& c, bool rec,
                            cudaStream_t st, uint32_t* dig_cnt, unsigned long long* dig_sum) {
    if (b.n <= 0) return;
    float4* f = s0.keep_force ? b.force_s : nullptr;
    if (batched)
        dispatch(c.block, c.stencil,
                 [&](auto R, auto BL) { force_impl<true, R.value, BL.value>(b, s0, rec, f, dig_cnt, dig_sum, st); });
    else
        dispatch(c.block, c.stencil,
                 [&](auto R, auto BL) { force_impl<false, R.value, BL.value>(b, s0, rec, f, dig_cnt, dig_sum, st); });
    if (s0.sdf) {
        const int blocks = std::min((b.n + 255) / 256, device_sm_count() * 8);
        if (batched)
            k_obstacle_hash<true><<<blocks, 256, 0, st>>>(b.pos, b.vel, s0, b.scenes, b.nscene, b.key, b.rank, b.count,
                                                          b.n);
        else
            k_obstacle_hash<false><<<blocks, 256, 0, st>>>(b.pos, b.vel, s0, b.scenes, 1, b.key, b.rank, b.count, b.n);
    }
}

void launch_density_nb(const Buffers& b, const SceneDev& s0, bool batched, const LaunchCfg& c, int* nb, int* cnt,
                       cudaStream_t st) {
    if (b.n <= 0) return;
    // the launch shape of launch_density, so that the densities agree bit for bit
    if (batched)
        dispatch(c.block, c.stencil, [&](auto R, auto BL) { density_nb_impl<true, R.value, BL.value>(b, s0, nb, cnt, st); });
    else
        dispatch(c.block, c.stencil, [&](auto R, auto BL) { density_nb_impl<false, R.value, BL.value>(b, s0, nb, cnt, st); });
}

}  // namespace sphgb
