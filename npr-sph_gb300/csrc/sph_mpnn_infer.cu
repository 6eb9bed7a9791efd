// sph_mpnn_infer.cu -- inference of the learned macro-step network on BF16
// tensor cores (mma.sync m16n8k16, FP32 accumulate), the path that runs at
// scale. The network is the one of sph_mpnn.h; the FP32 kernels of
// sph_mpnn.cu are its reference.
//
// Two kernels, one warp per tile of 16 particles (sorted order):
//   k_infer_r1  per particle: edge features of its <= 32 neighbours, built
//               once per edge into a shared buffer and loaded as B fragments
//               with ldmatrix, the round-1 edge layer as Z^T = We1^T E^T
//               (features on the MMA M side, 4 tiles of 16; edges on N, 4
//               tiles of 8), relu and the edge sum inside the lane -> M1 in a
//               shared tile; per 16 particles: H1 = relu([M1 n 1] Wn1'),
//               P = H1 Wp (H1 is reused from the accumulator registers as the
//               A operand).
//   k_infer_r2  round 2 likewise, with the gathered P_j as the accumulator's
//               initial value; per 16 particles: H2 = relu([M2 H1 1] Wn2'),
//               O = H2 Wo + bo (both heads), then the macro-step update and cell hash.
// Biases ride on a constant-1 feature column, so padded edges (all features
// zero) contribute exactly zero, as in the reference.
// P is stored permuted: for particle j, lane group g reads the 8 features
// {16 m + g + 8 r} it needs as one 16-byte load.
#include <cuda_bf16.h>

#include "sph_device.cuh"
#include "sph_mpnn.h"

namespace sphgb {
namespace mpnn {

namespace {

constexpr int kWarps = 4;
constexpr int kThreads = kWarps * 32;
constexpr int kTile = 16;         // particles per warp tile
constexpr int kLd1 = 88;          // X1 tile row stride (80 used), bf16
constexpr int kLd2 = 152;         // X2 tile row stride (144 used), bf16
constexpr int kK1 = 80, kK2 = 144; // padded K of the two node layers (bias column at W+FN / 128)
// Row stride (ints) of a warp's staged neighbour lists: 4 banks apart per particle, so the edge
// build (lanes of 8 particles x 4 slots) and the P_j index reads (lanes of 4 particles) hit 32
// and 4 distinct banks instead of one.
constexpr int kNbRow = K + 4;
constexpr int kBias1 = W + FN;     // bias column of the round-1 node layer
static_assert(kBias1 < kK1, "round-1 node input does not fit its padded K");
static_assert(2 * W + 16 == kK2, "round-2 node input: [M2 H1], bias column, padding");
static_assert(FO <= 8, "the output layer is one n-tile of 8 columns");

// Fragment-ordered weights (u32 = 2 x bf16), built by k_prep_frags.
constexpr int kFragWe1 = 0;                          // [4 mt][32 lanes][4]
constexpr int kFragWe2 = kFragWe1 + 4 * 32 * 4;      // [4 mt][32][4]
constexpr int kFragWn1 = kFragWe2 + 4 * 32 * 4;      // [5 kt][8 nt][32][2]
constexpr int kFragWp = kFragWn1 + 5 * 8 * 32 * 2;   // [4 kt][8 nt][32][2]
constexpr int kFragWn2 = kFragWp + 4 * 8 * 32 * 2;   // [9 kt][8 nt][32][2]
constexpr int kFragWo = kFragWn2 + 9 * 8 * 32 * 2;   // [4 kt][32][2]
constexpr int kFragTotal = kFragWo + 4 * 32 * 2;

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t*>(&v);
}
__device__ __forceinline__ float bf16_lo(uint32_t u) { return __uint_as_float(u << 16); }
__device__ __forceinline__ float bf16_hi(uint32_t u) { return __uint_as_float(u & 0xffff0000u); }

__device__ __forceinline__ void mma(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// Weight matrix element (row k, column o) of a layer with a bias row at `brow`, zero padded.
__device__ __forceinline__ float wel(const float* Wm, int kin, int nout, const float* b, int brow, int k, int o) {
    if (o >= nout) return 0.0f;
    if (k < kin) return Wm[k * nout + o];
    if (k == brow && b) return b[o];
    return 0.0f;
}

__global__ void k_prep_frags(const float* __restrict__ prm, uint32_t* __restrict__ fr) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= kFragTotal) return;
    int r = t;
    if (r < kFragWn1) {  // edge layers, transposed: A[o][k] = W[k][o]; bias row FE
        const bool second = r >= kFragWe2;
        if (second) r -= kFragWe2;
        const float* Wm = prm + (second ? kWe2 : kWe1);
        const float* b = prm + (second ? kBe2 : kBe1);
        const int mt = r / 128, lane = (r / 4) % 32, q = r % 4;
        const int g = lane >> 2, tq = lane & 3;
        const int o = mt * 16 + g + ((q & 1) ? 8 : 0);
        const int k = 2 * tq + ((q & 2) ? 8 : 0);
        fr[t] = pack_bf16(wel(Wm, FE, W, b, FE, k, o), wel(Wm, FE, W, b, FE, k + 1, o));
        return;
    }
    // node layers: B[k][o], b0 rows k0, k0+1; b1 rows k0+8, k0+9
    const float *Wm, *b;
    int kin, nout, brow, base;
    if (r < kFragWp) { Wm = prm + kWn1; b = prm + kBn1; kin = W + FN; nout = W; brow = kBias1; base = kFragWn1; }
    else if (r < kFragWn2) { Wm = prm + kWp; b = nullptr; kin = W; nout = W; brow = -1; base = kFragWp; }
    else if (r < kFragWo) { Wm = prm + kWn2; b = prm + kBn2; kin = 2 * W; nout = W; brow = 128; base = kFragWn2; }
    else { Wm = prm + kWo; b = nullptr; kin = W; nout = FO; brow = -1; base = kFragWo; }
    r -= base;
    const int ntiles = (base == kFragWo) ? 1 : 8;
    const int q = r % 2, lane = (r / 2) % 32, nt = (r / 64) % ntiles, kt = r / (64 * ntiles);
    const int g = lane >> 2, tq = lane & 3;
    const int o = nt * 8 + g;
    const int k = kt * 16 + 2 * tq + (q ? 8 : 0);
    fr[t] = pack_bf16(wel(Wm, kin, nout, b, brow, k, o), wel(Wm, kin, nout, b, brow, k + 1, o));
}

struct EdgeFrags {
    uint32_t a[4][4];  // [mt][reg]
};

// Feature buffer of one warp: 4 edge slots x 8 particles x kFRow bf16 (48-byte rows, so the
// 8 rows an ldmatrix reads fall on distinct banks).
constexpr int kFRow = 24;
constexpr int kFBuf = 4 * 8 * kFRow;
static_assert(8 * kLd2 + kFBuf <= kTile * kLd2, "round 2 keeps the feature buffer in X rows 8-15");

__device__ __forceinline__ void ldmatrix_x2(uint32_t& r0, uint32_t& r1, const __nv_bfloat16* p) {
    const uint32_t a = static_cast<uint32_t>(__cvta_generic_to_shared(p));
    asm volatile("ldmatrix.sync.aligned.m8n8.x2.shared.b16 {%0, %1}, [%2];\n" : "=r"(r0), "=r"(r1) : "r"(a));
}

// The 16 features of edge (i -> j) as 8 bf16 pairs, in the k order of the edge-layer
// fragments: d (3), u (3), r/h, q, q^2 d/(r/h) (3), q u (3), the bias column 1, and 0.
__device__ __forceinline__ void edge_features(float4 pi, float4 vi, float4 pj, float4 vj, float ih, float ic,
                                              uint4& w0, uint4& w1) {
    const float dx = (pj.x - pi.x) * ih, dy = (pj.y - pi.y) * ih, dz = (pj.z - pi.z) * ih;
    const float ux = (vj.x - vi.x) * ic, uy = (vj.y - vi.y) * ic, uz = (vj.z - vi.z) * ic;
    const float r = sqrtf(dx * dx + dy * dy + dz * dz);
    const float q = 1.0f - r;
    const float sg = r > 0.0f ? q * q / r : 0.0f;
    w0 = make_uint4(pack_bf16(dx, dy), pack_bf16(dz, ux), pack_bf16(uy, uz), pack_bf16(r, q));
    w1 = make_uint4(pack_bf16(sg * dx, sg * dy), pack_bf16(sg * dz, q * ux), pack_bf16(q * uy, q * uz),
                    pack_bf16(1.0f, 0.0f));
}

// Round-1/2 edge layer of a tile of 16 particles (rows of X), two groups of 8. An MMA n-tile
// holds the same edge slot e of the group's 8 particles (column c = particle c). The features
// of each edge are built once: per step of 4 slots, lane L builds those of particle L & 7's
// slot e0 + L / 8 into the warp's buffer E, and each slot's B fragment is one ldmatrix (matrix
// 0: features 0-7 of the 8 particles, matrix 1: features 8-15). Lane (g, tq) accumulates
// relu(Z) for features (16 mt + g, 16 mt + g + 8) of particles 2 tq and 2 tq + 1; padded edges
// have all-zero features (bias included), so they add exactly zero. The sums / K go to
// X[:, 0:64].
template <bool ROUND2>
__device__ __forceinline__ void edge_tile(const EdgeFrags& A, int base, int n, const float4* __restrict__ pos,
                                          const float4* __restrict__ vel, const int* nb_s, const int* cnt_s,
                                          float ih, float ic, const uint4* __restrict__ Pperm,
                                          __nv_bfloat16* X, int ld, __nv_bfloat16* E) {
    const int lane = threadIdx.x & 31, g = lane >> 2, tq = lane & 3;
    const int fp = lane & 7, fs = lane >> 3;  // the edge this lane builds: particle fp, slot e0 + fs
    const __nv_bfloat16* lrow = E + (lane & 7) * kFRow + ((lane >> 3) & 1) * 8;  // ldmatrix row address
#pragma unroll 1
    for (int grp = 0; grp < 2; ++grp) {
        const int pb = grp * 8 + fp, ib = base + pb;
        const float4 pi = ib < n ? pos[ib] : make_float4(0.f, 0.f, 0.f, 0.f);
        const float4 vi = ib < n ? vel[ib] : make_float4(0.f, 0.f, 0.f, 0.f);
        const int cb = cnt_s[pb];
        const int c0 = cnt_s[grp * 8 + 2 * tq], c1 = cnt_s[grp * 8 + 2 * tq + 1];
        int emax = cb;
#pragma unroll
        for (int o = 1; o <= 4; o <<= 1) emax = max(emax, __shfl_xor_sync(0xffffffffu, emax, o));
        float s[4][2][2];
#pragma unroll
        for (int mt = 0; mt < 4; ++mt) s[mt][0][0] = s[mt][0][1] = s[mt][1][0] = s[mt][1][1] = 0.0f;
#pragma unroll 1
        for (int e0 = 0; e0 < emax; e0 += 4) {
            {
                const int e = e0 + fs;
                uint4 w0 = make_uint4(0u, 0u, 0u, 0u), w1 = w0;
                if (e < cb) {
                    const int j = nb_s[pb * kNbRow + e];
                    edge_features(pi, vi, pos[j], vel[j], ih, ic, w0, w1);
                }
                uint4* dst = reinterpret_cast<uint4*>(E + (fs * 8 + fp) * kFRow);
                dst[0] = w0;
                dst[1] = w1;
            }
            __syncwarp();
            const int nsl = min(4, emax - e0);
            auto slot = [&](int sl) {
                const int e = e0 + sl;
                uint32_t b0, b1;
                ldmatrix_x2(b0, b1, lrow + sl * 8 * kFRow);
                float c[4][4];
                if constexpr (ROUND2) {
                    // accumulators start at P_j of the two column particles 2 tq, 2 tq + 1
                    uint4 p0 = make_uint4(0, 0, 0, 0), p1 = make_uint4(0, 0, 0, 0);
                    if (e < c0) p0 = Pperm[(size_t)nb_s[(grp * 8 + 2 * tq) * kNbRow + e] * 8 + g];
                    if (e < c1) p1 = Pperm[(size_t)nb_s[(grp * 8 + 2 * tq + 1) * kNbRow + e] * 8 + g];
                    const uint32_t q0[4] = {p0.x, p0.y, p0.z, p0.w}, q1[4] = {p1.x, p1.y, p1.z, p1.w};
#pragma unroll
                    for (int mt = 0; mt < 4; ++mt) {  // word mt holds features (16 mt + g, 16 mt + g + 8)
                        c[mt][0] = bf16_lo(q0[mt]);
                        c[mt][1] = bf16_lo(q1[mt]);
                        c[mt][2] = bf16_hi(q0[mt]);
                        c[mt][3] = bf16_hi(q1[mt]);
                    }
                } else {
#pragma unroll
                    for (int mt = 0; mt < 4; ++mt) c[mt][0] = c[mt][1] = c[mt][2] = c[mt][3] = 0.0f;
                }
#pragma unroll
                for (int mt = 0; mt < 4; ++mt) {
                    mma(c[mt], A.a[mt], b0, b1);
                    s[mt][0][0] += fmaxf(c[mt][0], 0.0f);
                    s[mt][0][1] += fmaxf(c[mt][1], 0.0f);
                    s[mt][1][0] += fmaxf(c[mt][2], 0.0f);
                    s[mt][1][1] += fmaxf(c[mt][3], 0.0f);
                }
            };
            if constexpr (ROUND2) {  // unrolled: later slots' P_j loads are issued early
#pragma unroll
                for (int sl = 0; sl < 4; ++sl) {
                    if (sl >= nsl) break;
                    slot(sl);
                }
            } else {  // round 1 spills when unrolled
#pragma unroll 1
                for (int sl = 0; sl < nsl; ++sl) slot(sl);
            }
            __syncwarp();
        }
        const float sc = 1.0f / K;
#pragma unroll
        for (int mt = 0; mt < 4; ++mt)
#pragma unroll
            for (int r = 0; r < 2; ++r)
#pragma unroll
                for (int cc = 0; cc < 2; ++cc)
                    X[(grp * 8 + 2 * tq + cc) * ld + mt * 16 + g + 8 * r] = __float2bfloat16_rn(s[mt][r][cc] * sc);
    }
}

// Neighbour lists and counts of a tile into the warp's shared memory (rows past n: none).
__device__ __forceinline__ void stage_tile_lists(int base, int n, const int* __restrict__ nb,
                                                 const int* __restrict__ cnt, int* nb_s, int* cnt_s) {
    const int lane = threadIdx.x & 31;
#pragma unroll 4
    for (int q = lane; q < kTile * K; q += 32) {
        const int i = base + q / K;
        nb_s[(q / K) * kNbRow + q % K] = i < n ? nb[(size_t)base * K + q] : 0;
    }
    if (lane < kTile) {
        const int i = base + lane;
        cnt_s[lane] = i < n ? min(max(cnt[i], 0), K) : 0;
    }
    __syncwarp();
}

// A fragment of k-tile kt from a bf16 smem tile with row stride ld (16 rows).
__device__ __forceinline__ void load_a(const __nv_bfloat16* X, int ld, int kt, uint32_t (&a)[4]) {
    const int lane = threadIdx.x & 31, g = lane >> 2, tq = lane & 3;
    const uint32_t* r0 = reinterpret_cast<const uint32_t*>(X + g * ld + kt * 16 + 2 * tq);
    const uint32_t* r1 = reinterpret_cast<const uint32_t*>(X + (g + 8) * ld + kt * 16 + 2 * tq);
    a[0] = r0[0];
    a[1] = r1[0];
    a[2] = r0[4];
    a[3] = r1[4];
}

// D[16 x 64] = X (16 x 16*KT, smem) * B (frags) ; d[nt][4]
template <int KT>
__device__ __forceinline__ void node_gemm(const __nv_bfloat16* X, int ld, const uint2* __restrict__ Bf, float (&d)[8][4]) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) d[nt][0] = d[nt][1] = d[nt][2] = d[nt][3] = 0.0f;
#pragma unroll
    for (int kt = 0; kt < KT; ++kt) {
        uint32_t a[4];
        load_a(X, ld, kt, a);
#pragma unroll
        for (int nt = 0; nt < 8; ++nt) {
            const uint2 b = __ldg(Bf + (kt * 8 + nt) * 32 + lane);
            mma(d[nt], a, b.x, b.y);
        }
    }
}

__device__ __forceinline__ void load_edge_frags(const uint32_t* __restrict__ fr, int base, EdgeFrags& A) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int mt = 0; mt < 4; ++mt) {
        const uint4 v = __ldg(reinterpret_cast<const uint4*>(fr + base) + mt * 32 + lane);
        A.a[mt][0] = v.x; A.a[mt][1] = v.y; A.a[mt][2] = v.z; A.a[mt][3] = v.w;
    }
}

// 8 CTAs of 4 warps per SM (at most 64 registers): the edge loops wait on neighbour gathers,
// and 32 warps per SM hide that latency better than 16 (with features built in every lane
// of a quad, the macro-step took 2.68 instead of 3.25 ms on the 1M dam break; 6 CTAs per SM,
// 80 registers, took 3.55 ms). Building each edge's features once: 2.20 ms.
__global__ void __launch_bounds__(kThreads, 8) k_infer_r1(const float4* __restrict__ pos, const float4* __restrict__ vel,
                                                      const float2* __restrict__ rhop, const int* __restrict__ nb,
                                                      const int* __restrict__ cnt, FrameConst fc, int n,
                                                      const uint32_t* __restrict__ fr,
                                                      __nv_bfloat16* __restrict__ H1out, uint16_t* __restrict__ Pperm) {
    __shared__ __align__(16) __nv_bfloat16 xs[kWarps][kTile * kLd1];
    __shared__ __align__(16) __nv_bfloat16 es[kWarps][kFBuf];
    __shared__ int nbs[kWarps][kTile * kNbRow];
    __shared__ int cns[kWarps][kTile];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, tq = lane & 3;
    __nv_bfloat16* X = xs[warp];
    EdgeFrags A;
    load_edge_frags(fr, kFragWe1, A);
    const float ih = 1.0f / fc.h, ic = 1.0f / fc.c;
    const int ntiles = (n + kTile - 1) / kTile;
    for (int tile = blockIdx.x * kWarps + warp; tile < ntiles; tile += gridDim.x * kWarps) {
        const int base = tile * kTile;
        stage_tile_lists(base, n, nb, cnt, nbs[warp], cns[warp]);
        edge_tile<false>(A, base, n, pos, vel, nbs[warp], cns[warp], ih, ic, nullptr, X, kLd1, es[warp]);
        // node features, bias column and padding (columns 64 .. 79) of the 16 rows
        for (int q = lane; q < kTile * 16; q += 32) {
            const int p = q >> 4, col = q & 15, i = base + p;
            float v = 0.0f;
            if (i < n) {
                switch (col) {
                    case 0: v = vel[i].x * ic; break;
                    case 1: v = vel[i].y * ic; break;
                    case 2: v = vel[i].z * ic; break;
                    case 3: v = rhop[i].x / fc.rho_self - 1.0f; break;
                    case 4: v = (rhop[i].x - fc.rho0) / fc.rho_self; break;
                    case 5: v = fc.log_mu; break;
                    case 6: v = (float)cns[warp][p] / K; break;
                    case 7: v = 1.0f; break;
                    case 8: v = fc.courant; break;
                    case kBias1 - W: v = 1.0f; break;  // bias column
                    default: v = 0.0f;
                }
            }
            X[p * kLd1 + 64 + col] = __float2bfloat16_rn(v);
        }
        __syncwarp();
        float d[8][4];
        node_gemm<5>(X, kLd1, reinterpret_cast<const uint2*>(fr + kFragWn1), d);
        // H1 = relu(Y1): store, and reuse as the A operand of P = H1 Wp
        uint32_t ha[4][4];
#pragma unroll
        for (int nt = 0; nt < 8; ++nt) {
            const float h0 = fmaxf(d[nt][0], 0.f), h1 = fmaxf(d[nt][1], 0.f), h2 = fmaxf(d[nt][2], 0.f),
                        h3 = fmaxf(d[nt][3], 0.f);
            const uint32_t lo = pack_bf16(h0, h1), hi = pack_bf16(h2, h3);
            const int kt = nt >> 1, half = nt & 1;
            ha[kt][half ? 2 : 0] = lo;
            ha[kt][half ? 3 : 1] = hi;
            const int r0 = base + g, r1 = base + g + 8, col = nt * 8 + 2 * tq;
            if (r0 < n) *reinterpret_cast<uint32_t*>(H1out + (size_t)r0 * W + col) = lo;
            if (r1 < n) *reinterpret_cast<uint32_t*>(H1out + (size_t)r1 * W + col) = hi;
        }
        float pd[8][4];
#pragma unroll
        for (int nt = 0; nt < 8; ++nt) pd[nt][0] = pd[nt][1] = pd[nt][2] = pd[nt][3] = 0.0f;
#pragma unroll
        for (int kt = 0; kt < 4; ++kt)
#pragma unroll
            for (int nt = 0; nt < 8; ++nt) {
                const uint2 b = __ldg(reinterpret_cast<const uint2*>(fr + kFragWp) + (kt * 8 + nt) * 32 + lane);
                mma(pd[nt], ha[kt], b.x, b.y);
            }
        // P permuted: feature f = 16 m + gg + 8 r  ->  P[j][gg][m][r]
#pragma unroll
        for (int nt = 0; nt < 8; ++nt)
#pragma unroll
            for (int q = 0; q < 2; ++q) {
                const int f = nt * 8 + 2 * tq + q;
                const int gg = f & 7, m = f >> 4, rr = (f >> 3) & 1;
                const int slot = gg * 8 + m * 2 + rr;
                const int r0 = base + g, r1 = base + g + 8;
                if (r0 < n) Pperm[(size_t)r0 * W + slot] = __bfloat16_as_ushort(__float2bfloat16_rn(pd[nt][q]));
                if (r1 < n) Pperm[(size_t)r1 * W + slot] = __bfloat16_as_ushort(__float2bfloat16_rn(pd[nt][2 + q]));
            }
        __syncwarp();
    }
}

// Round 2 runs 6 CTAs per SM (80 registers): fewer spills, and the L1 left beside the CTAs'
// shared memory holds more of the gathered P_j rows (2.13 ms per macro-step against 2.20 ms
// at 8 CTAs per SM, 2.25 ms at 4).
__global__ void __launch_bounds__(kThreads, 6) k_infer_r2(const float4* __restrict__ pos, const float4* __restrict__ vel,
                                                      const int* __restrict__ nb, const int* __restrict__ cnt,
                                                      FrameConst fc, int n, const uint32_t* __restrict__ fr,
                                                      const float* __restrict__ prm,
                                                      const __nv_bfloat16* __restrict__ H1,
                                                      const uint4* __restrict__ Pperm, SceneDev S,
                                                      float4* __restrict__ pos_out, float4* __restrict__ vel_out,
                                                      float* __restrict__ out, int* __restrict__ key_out,
                                                      int* __restrict__ rank_out, int* __restrict__ count,
                                                      int integrate) {
    __shared__ __align__(16) __nv_bfloat16 xs[kWarps][kTile * kLd2];
    __shared__ int nbs[kWarps][kTile * kNbRow];
    __shared__ int cns[kWarps][kTile];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, tq = lane & 3;
    __nv_bfloat16* X = xs[warp];
    EdgeFrags A;
    load_edge_frags(fr, kFragWe2, A);
    const float ih = 1.0f / fc.h, ic = 1.0f / fc.c;
    static_assert(FO == 6, "the output gather below is written for two heads of 3");
    float bo[FO];
#pragma unroll
    for (int q = 0; q < FO; ++q) bo[q] = prm[kBo + q];
    const int ntiles = (n + kTile - 1) / kTile;
    for (int tile = blockIdx.x * kWarps + warp; tile < ntiles; tile += gridDim.x * kWarps) {
        const int base = tile * kTile;
        stage_tile_lists(base, n, nb, cnt, nbs[warp], cns[warp]);
        // the feature buffer lives in X rows 8-15, which only group 1's sums (written after its
        // last use) overwrite
        edge_tile<true>(A, base, n, pos, vel, nbs[warp], cns[warp], ih, ic, Pperm, X, kLd2, X + 8 * kLd2);
        // H1 rows (columns 64 .. 127), bias column 128, padding to 143
        for (int p = 0; p < kTile; ++p) {
            const int i = base + p;
            reinterpret_cast<uint32_t*>(X + p * kLd2 + 64)[lane] =
                i < n ? reinterpret_cast<const uint32_t*>(H1 + (size_t)i * W)[lane] : 0u;
            if (lane < 16) X[p * kLd2 + 128 + lane] = __float2bfloat16_rn(lane == 0 && i < n ? 1.0f : 0.0f);
        }
        __syncwarp();
        float d[8][4];
        node_gemm<9>(X, kLd2, reinterpret_cast<const uint2*>(fr + kFragWn2), d);
        uint32_t ha[4][4];
#pragma unroll
        for (int nt = 0; nt < 8; ++nt) {
            const int kt = nt >> 1, half = nt & 1;
            ha[kt][half ? 2 : 0] = pack_bf16(fmaxf(d[nt][0], 0.f), fmaxf(d[nt][1], 0.f));
            ha[kt][half ? 3 : 1] = pack_bf16(fmaxf(d[nt][2], 0.f), fmaxf(d[nt][3], 0.f));
        }
        float o[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
        for (int kt = 0; kt < 4; ++kt) {
            const uint2 b = __ldg(reinterpret_cast<const uint2*>(fr + kFragWo) + kt * 32 + lane);
            mma(o, ha[kt], b.x, b.y);
        }
        // O rows g (o[0], o[1]) and g + 8 (o[2], o[3]), columns 2 tq, 2 tq + 1: lane tq == 0 of each
        // quad gathers the 6 columns of both rows from tq = 1 (columns 2, 3) and tq = 2 (4, 5).
        // col[r][c]: row g + 8 r, column c
        const float c10 = __shfl_sync(0xffffffffu, o[0], (lane & ~3) | 1);
        const float c11 = __shfl_sync(0xffffffffu, o[1], (lane & ~3) | 1);
        const float c12 = __shfl_sync(0xffffffffu, o[2], (lane & ~3) | 1);
        const float c13 = __shfl_sync(0xffffffffu, o[3], (lane & ~3) | 1);
        const float c20 = __shfl_sync(0xffffffffu, o[0], (lane & ~3) | 2);
        const float c21 = __shfl_sync(0xffffffffu, o[1], (lane & ~3) | 2);
        const float c22 = __shfl_sync(0xffffffffu, o[2], (lane & ~3) | 2);
        const float c23 = __shfl_sync(0xffffffffu, o[3], (lane & ~3) | 2);
        if (tq == 0) {
#pragma unroll
            for (int rr = 0; rr < 2; ++rr) {
                const int i = base + g + rr * 8;
                if (i >= n) continue;
                const float O0 = (rr ? o[2] : o[0]) + bo[0], O1 = (rr ? o[3] : o[1]) + bo[1];
                const float O2 = (rr ? c12 : c10) + bo[2], O3 = (rr ? c13 : c11) + bo[3];
                const float O4 = (rr ? c22 : c20) + bo[4], O5 = (rr ? c23 : c21) + bo[5];
                if (out) {
                    float4* orow = reinterpret_cast<float4*>(out + (size_t)i * kOS);
                    orow[0] = make_float4(O0, O1, O2, O3);
                    orow[1] = make_float4(O4, O5, 0.0f, 0.0f);
                }
                if (!integrate) continue;
                float4 np, nv;
                macro_update(S, O0, O1, O2, O3, O4, O5, pos[i], vel[i], np, nv);
                pos_out[i] = np;
                vel_out[i] = nv;
                const int k = cell_key(S, np.x, np.y, np.z);
                key_out[i] = k;
                rank_out[i] = atomicAdd(&count[k], 1);
            }
        }
        __syncwarp();
    }
}

}  // namespace

int infer_frag_words() { return kFragTotal; }

void infer_prep(const float* prm, uint32_t* frags, cudaStream_t st) {
    k_prep_frags<<<(kFragTotal + 255) / 256, 256, 0, st>>>(prm, frags);
}

// Grid of a tile-stride inference kernel: at most the CTAs that fit on the GPU at once.
// One warp per tile of particles (the kernels keep their tile loops, so any grid is correct):
// the block scheduler balances the tiles, which beats a resident grid looping over fixed shares.
static int infer_grid(int n) {
    const int tiles = (n + kTile - 1) / kTile;
    const int blocks = (tiles + kWarps - 1) / kWarps;
    return blocks < 1 ? 1 : blocks;
}

void infer_round1(const Frame& f, const uint32_t* frags, __nv_bfloat16* H1, uint16_t* Pperm, cudaStream_t st) {
    k_infer_r1<<<infer_grid(f.n), kThreads, 0, st>>>(f.pos, f.vel, f.rhop, f.nb, f.cnt, f.fc, f.n, frags, H1, Pperm);
}

void infer_round2(const Frame& f, const uint32_t* frags, const float* prm, const __nv_bfloat16* H1,
                  const uint16_t* Pperm, const SceneDev& S, float4* pos_out, float4* vel_out, float* out, int* key,
                  int* rank, int* count, bool integrate, cudaStream_t st) {
    k_infer_r2<<<infer_grid(f.n), kThreads, 0, st>>>(f.pos, f.vel, f.nb, f.cnt, f.fc, f.n, frags, prm, H1,
                                                     reinterpret_cast<const uint4*>(Pperm), S, pos_out, vel_out, out,
                                                     key, rank, count, integrate ? 1 : 0);
}

}  // namespace mpnn
}  // namespace sphgb
