// sph_mpnn_tc.cu -- inference of the learned macro-step network (sph_mpnn.h) on the sm_103a
// tensor cores: tcgen05 MMAs of BF16 operands staged in shared memory, FP32 accumulators in
// tensor memory (TMEM), every wait bounded (sph_tc.cuh).
//
// One CTA of 128 threads per tile of 128 consecutive particles (sorted order), persistent over
// the tiles. Per tile:
//   edge layer   32 sub-tiles of 4 particles x 32 edge slots = 128 edges (the MMA's M): thread
//                t builds the 16 features of edge t (d, u, r/h, q, the spiky and Laplacian
//                shapes, the constant-1 bias column, a zero) into the A tile, one thread issues
//                Z = E [128 x 16] * We^T (N = 64, K = 16) into one of two TMEM buffers, and
//                while the tensor core runs the next sub-tile is built; warp w then drains
//                particle w of the sub-tile: its 32 edges are its 32 lanes, each lane loads its
//                edge's 64 outputs from TMEM (round 2 adds the neighbour's P_j), applies the ReLU
//                while packing pairs to f16x2, and a butterfly of shuffles (reduce-scatter, f16x2
//                adds) leaves lane l with the sum over the edges of features 2l, 2l+1:
//                M = sum relu(.) / K, written as bf16 into the node tile. Padded edge slots have
//                all-zero features and no P_j, so they add exactly zero. The neighbour gathers of
//                sub-tile s + 1 (and the neighbour lists of s + 2) are issued before sub-tile s - 1
//                is drained, and in round 2 each thread loads its edge's P_j right after building
//                the edge (the thread that builds edge t also drains TMEM lane t).
//   node layers  M = 128 particles: round 1 H1 = relu([M1 n 1] Wn1'), P = H1 Wp (H1 stored,
//                and staged again as the A operand of P); round 2 H2 = relu([M2 H1 1] Wn2'),
//                O = [H2 1] Wo' (N = 16, the 6 outputs in the first columns). Biases ride on a
//                constant-1 column of the activations.
// P is stored as f16 [n][64] (round 2 adds it to the f16x2-packed pre-activations).
// Weights live in one global array of bf16 images already in the canonical layout of
// sph_tc.cuh (built by tc_infer_prep), copied into shared memory once per CTA.
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "sph_device.cuh"
#include "sph_mpnn.h"
#include "sph_tc.cuh"

namespace sphgb {
namespace mpnn {

namespace {

using tc::smem_desc;
using tc::smem_u32;
using tc::tile_off;

constexpr int kThr = 128;
constexpr int kTP = 128;          // particles per tile (the node layers' M)
constexpr int kEP = 4;            // particles per edge MMA: 4 x 32 edges = M 128
constexpr int kSub = kTP / kEP;   // edge sub-tiles per tile (even: each TMEM buffer's barrier
                                  // completes an even number of phases per tile)
constexpr int kKE = 16;           // edge features (14) + bias + zero
constexpr int kKX1 = 80;          // [M1 (64) | node features (9) | bias | 0 ...]
constexpr int kKX2 = 144;         // [M2 (64) | H1 (64) | bias | 0 ...]
constexpr int kKH1 = 64;          // H1 as the A operand of P = H1 Wp
constexpr int kKH2 = 80;          // [H2 (64) | bias | 0 ...]
constexpr int kNO = 16;           // output layer N (6 used)
constexpr uint32_t kCols = 128;   // TMEM columns: two edge accumulators of 64
static_assert(kSub % 2 == 0, "barrier phases must restart with every tile");
static_assert(K == 32 && W == 64 && FE == 14, "the tile shapes assume K = 32, W = 64, 14 edge features");

// Weight images [N][Kpad], bf16, canonical layout, one after the other.
constexpr int kImgWe1 = 0;
constexpr int kImgWn1 = kImgWe1 + W * kKE;
constexpr int kImgWp = kImgWn1 + W * kKX1;
constexpr int kImgWe2 = kImgWp + W * kKH1;
constexpr int kImgWn2 = kImgWe2 + W * kKE;
constexpr int kImgWo = kImgWn2 + W * kKX2;
constexpr int kImgAE1 = kImgWo + kNO * kKH2;  // round 1 with the features on the TMEM lanes:
constexpr int kKA = 32;                          // [128][32], rows 0..63 [We1' | 0], rows 64..127 [0 | We1']
constexpr int kImgTotal = kImgAE1 + 128 * kKA;

__host__ __device__ constexpr uint32_t sbo(int kc) { return (uint32_t)kc * 16u; }

// Element (o, k) of an image with padded K kc, as an element index.
__device__ __forceinline__ int img_at(int o, int k, int kc) { return (int)(tile_off(o, k >> 3, kc) >> 1) + (k & 7); }

// Weight (row k of the input, column o of the output) of a layer with its bias at input row
// `brow` (-1: none), zero elsewhere.
__device__ __forceinline__ float wv(const float* prm, int woff, int boff, int kin, int nout, int brow, int o, int k) {
    if (o >= nout) return 0.0f;
    if (k < kin) return prm[woff + k * nout + o];
    if (k == brow && boff >= 0) return prm[boff + o];
    return 0.0f;
}

__global__ void k_tc_infer_prep(const float* __restrict__ prm, __nv_bfloat16* __restrict__ img) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= kImgTotal) return;
    if (t >= kImgAE1) {  // the block-diagonal edge weights of round 1 (two sub-tiles stacked along K)
        const int r = t - kImgAE1, m = r / kKA, k = r % kKA, half = m >> 6;
        const float v = (k >> 4) == half ? wv(prm, kWe1, kBe1, FE, W, FE, m & 63, k & 15) : 0.0f;
        img[kImgAE1 + img_at(m, k, kKA)] = __float2bfloat16_rn(v);
        return;
    }
    int base, kc, woff, boff, kin, nout, brow;
    if (t < kImgWn1) { base = kImgWe1; kc = kKE; woff = kWe1; boff = kBe1; kin = FE; nout = W; brow = FE; }
    else if (t < kImgWp) { base = kImgWn1; kc = kKX1; woff = kWn1; boff = kBn1; kin = W + FN; nout = W; brow = W + FN; }
    else if (t < kImgWe2) { base = kImgWp; kc = kKH1; woff = kWp; boff = -1; kin = W; nout = W; brow = -1; }
    else if (t < kImgWn2) { base = kImgWe2; kc = kKE; woff = kWe2; boff = kBe2; kin = FE; nout = W; brow = FE; }
    else if (t < kImgWo) { base = kImgWn2; kc = kKX2; woff = kWn2; boff = kBn2; kin = 2 * W; nout = W; brow = 2 * W; }
    else { base = kImgWo; kc = kKH2; woff = kWo; boff = kBo; kin = W; nout = FO; brow = W; }
    const int r = t - base, o = r / kc, k = r % kc;
    img[base + img_at(o, k, kc)] = __float2bfloat16_rn(wv(prm, woff, boff, kin, nout, brow, o, k));
}

__device__ __forceinline__ uint32_t pk_bf16(float lo, float hi) {
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t*>(&v);
}

// relu of two floats packed as f16x2 (lo in the low half).
__device__ __forceinline__ uint32_t relu_f16x2(float lo, float hi) {
    uint32_t d;
    asm("cvt.rn.relu.f16x2.f32 %0, %1, %2;\n" : "=r"(d) : "f"(hi), "f"(lo));
    return d;
}
__device__ __forceinline__ uint32_t to_f16x2(float lo, float hi) {
    uint32_t d;
    asm("cvt.rn.f16x2.f32 %0, %1, %2;\n" : "=r"(d) : "f"(hi), "f"(lo));
    return d;
}
__device__ __forceinline__ uint32_t hadd2(uint32_t a, uint32_t b) {
    __half2 x = *reinterpret_cast<__half2*>(&a), y = *reinterpret_cast<__half2*>(&b);
    __half2 s = __hadd2(x, y);
    return *reinterpret_cast<uint32_t*>(&s);
}
__device__ __forceinline__ uint32_t hrelu2(uint32_t a) {
    __half2 x = *reinterpret_cast<__half2*>(&a);
    __half2 s = __hmax2(x, __float2half2_rn(0.0f));
    return *reinterpret_cast<uint32_t*>(&s);
}

// The 16 features of edge (i -> j) in the order of the edge layer's input rows: d (3), u (3),
// r/h, q = 1 - r/h, q^2 d / (r/h) (3), q u (3), the bias column 1, and 0.
__device__ __forceinline__ void edge_feat16(float4 pi, float4 vi, float4 pj, float4 vj, float ih, float ic, uint4& w0,
                                            uint4& w1) {
    const float dx = (pj.x - pi.x) * ih, dy = (pj.y - pi.y) * ih, dz = (pj.z - pi.z) * ih;
    const float ux = (vj.x - vi.x) * ic, uy = (vj.y - vi.y) * ic, uz = (vj.z - vi.z) * ic;
    const float r = sqrtf(dx * dx + dy * dy + dz * dz);
    const float q = 1.0f - r;
    const float sg = r > 0.0f ? q * q / r : 0.0f;
    w0 = make_uint4(pk_bf16(dx, dy), pk_bf16(dz, ux), pk_bf16(uy, uz), pk_bf16(r, q));
    w1 = make_uint4(pk_bf16(sg * dx, sg * dy), pk_bf16(sg * dz, q * ux), pk_bf16(q * uy, q * uz), pk_bf16(1.0f, 0.0f));
}

// Shared memory of one CTA (dynamic, carved in this order).
template <bool ROUND2>
struct Smem {
    static constexpr int kWe = (ROUND2 ? kImgWe2 : kImgWe1);
    static constexpr int kImgBegin = kWe;
    static constexpr int kImgEnd = ROUND2 ? kImgTotal : kImgWe2;  // the images this round copies
    static constexpr int kImgBytes = (kImgEnd - kImgBegin) * 2;
    static constexpr int kKX = ROUND2 ? kKX2 : kKX1;
    static constexpr int kOffImg = 0;
    static constexpr int kOffA = kOffImg + kImgBytes;          // two edge A tiles [128][16]
    static constexpr int kOffX = kOffA + 2 * kTP * kKE * 2;    // node tile [128][kKX]
    static constexpr int kBytes = kOffX + kTP * kKX * 2;
};

// Drain of edge sub-tile s (all 128 threads): warp w reduces the 32 edges of particle 4 s + w
// (its lanes) to M = sum relu(Z [+ P_j]) / K, written into row 4 s + w of the node tile. pj: this
// lane's P_j (f16, zero for a padded slot), round 2 only.
template <bool ROUND2>
__device__ __forceinline__ void drain_edges(uint32_t tmem_d, int s, const uint4 (&pj)[8], uint8_t* X, int kx) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float z[64];
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        float v[16];
        tc::tmem_ld16(tmem_d + ((uint32_t)(32 * warp) << 16) + (uint32_t)(16 * c), v);
#pragma unroll
        for (int j = 0; j < 16; ++j) z[16 * c + j] = v[j];
    }
    tc::tmem_wait_ld();
    uint32_t h[32];
    if constexpr (ROUND2) {
#pragma unroll
        for (int c = 0; c < 8; ++c) {
            const uint32_t q[4] = {pj[c].x, pj[c].y, pj[c].z, pj[c].w};
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int k = 4 * c + u;
                h[k] = hrelu2(hadd2(to_f16x2(z[2 * k], z[2 * k + 1]), q[u]));
            }
        }
    } else {
#pragma unroll
        for (int k = 0; k < 32; ++k) h[k] = relu_f16x2(z[2 * k], z[2 * k + 1]);
    }
    // reduce-scatter over the 32 lanes: at the step of width w, lanes with bit w set keep the
    // upper half of their words and send the lower half to lane ^ w, and vice versa
#pragma unroll
    for (int w = 16; w >= 1; w >>= 1) {
        const bool up = (lane & w) != 0;
#pragma unroll
        for (int k = 0; k < w; ++k) {
            const uint32_t send = up ? h[k] : h[k + w];
            const uint32_t keep = up ? h[k + w] : h[k];
            h[k] = hadd2(keep, __shfl_xor_sync(0xffffffffu, send, w));
        }
    }
    const __half2 sum = *reinterpret_cast<__half2*>(&h[0]);
    const float2 f = __half22float2(sum);
    const float sc = 1.0f / K;
    const int prow = kEP * s + warp, k = 2 * lane;
    *reinterpret_cast<uint32_t*>(X + tile_off(prow, k >> 3, kx) + (k & 7) * 2) = pk_bf16(f.x * sc, f.y * sc);
}

// The gather of one edge slot: neighbour index j (-1: none), then positions and velocities.
struct EdgeIn {
    float4 pi, vi, pj, vj;
    int j;  // -1: a padded slot
};

__device__ __forceinline__ int edge_j(int p, int e, int n, const int* __restrict__ nb, const int* __restrict__ cnt) {
    if (p >= n) return -1;
    const int cp = min(max(__ldg(cnt + p), 0), K);
    const int j = e < cp ? __ldg(nb + (size_t)p * K + e) : -1;
    return (j >= 0 && j < n) ? j : -1;
}

__device__ __forceinline__ EdgeIn edge_load(int p, int j, const float4* __restrict__ pos, const float4* __restrict__ vel) {
    EdgeIn r;
    r.j = j;
    const int jj = j >= 0 ? j : 0, pp = j >= 0 ? p : 0;
    r.pi = __ldg(pos + pp);
    r.vi = __ldg(vel + pp);
    r.pj = __ldg(pos + jj);
    r.vj = __ldg(vel + jj);
    return r;
}

template <bool ROUND2>
__global__ void __launch_bounds__(kThr) k_tc_round(const float4* __restrict__ pos, const float4* __restrict__ vel,
                                                   const float2* __restrict__ rhop, const int* __restrict__ nb,
                                                   const int* __restrict__ cnt, FrameConst fc, int n,
                                                   const __nv_bfloat16* __restrict__ img,
                                                   __nv_bfloat16* __restrict__ H1, __half* __restrict__ P,
                                                   float* __restrict__ out, uint32_t* __restrict__ err) {
    using L = Smem<ROUND2>;
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ __align__(8) uint64_t mbar[3];
    __shared__ uint32_t tmem_slot;
    __shared__ int bad;
    uint8_t* const sA = smem + L::kOffA;
    uint8_t* const sX = smem + L::kOffX;
    const int tid = threadIdx.x, warp = tid >> 5;
    // weights for this round, once per CTA
    {
        const uint4* src = reinterpret_cast<const uint4*>(img + L::kImgBegin);
        uint4* dst = reinterpret_cast<uint4*>(smem + L::kOffImg);
        for (int i = tid; i < L::kImgBytes / 16; i += kThr) dst[i] = __ldg(src + i);
    }
    if (tid == 0) {
        tc::mbar_init(&mbar[0], 1);
        tc::mbar_init(&mbar[1], 1);
        tc::mbar_init(&mbar[2], 1);
        tc::mbar_init_fence();
        bad = 0;
    }
    if (warp == 0) tc::tmem_alloc(&tmem_slot, kCols);
    tc::fence_smem_to_async();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = tmem_slot;
    const uint32_t sw = smem_u32(smem + L::kOffImg);
    const uint32_t we_desc_addr = sw;  // the round's edge weights come first
    const uint32_t wn_addr = sw + (uint32_t)((ROUND2 ? kImgWn2 - kImgWe2 : kImgWn1 - kImgWe1) * 2);
    const uint32_t w3_addr = sw + (uint32_t)((ROUND2 ? kImgWo - kImgWe2 : kImgWp - kImgWe1) * 2);
    const uint32_t sa = smem_u32(sA), sx = smem_u32(sX);
    const uint32_t id_e = tc::idesc_bf16_f32(128, W);
    const float ih = 1.0f / fc.h, ic = 1.0f / fc.c;
    const int ntiles = (n + kTP - 1) / kTP;

    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int tile0 = tile * kTP;
        // node tile: the columns that do not come from the edge layer, for particle tid
        {
            const int p = tile0 + tid;
            if constexpr (!ROUND2) {
                float v[16];
#pragma unroll
                for (int c = 0; c < 16; ++c) v[c] = 0.0f;
                if (p < n) {
                    const float4 vi = vel[p];
                    const float rho = rhop[p].x;
                    v[0] = vi.x * ic; v[1] = vi.y * ic; v[2] = vi.z * ic;
                    v[3] = rho / fc.rho_self - 1.0f;
                    v[4] = (rho - fc.rho0) / fc.rho_self;
                    v[5] = fc.log_mu;
                    v[6] = (float)min(max(cnt[p], 0), K) / K;
                    v[7] = 1.0f;
                    v[8] = fc.courant;
                    v[9] = 1.0f;  // the bias column (W + FN)
                }
#pragma unroll
                for (int c = 0; c < 2; ++c)
                    *reinterpret_cast<uint4*>(sX + tile_off(tid, 8 + c, kKX1)) =
                        make_uint4(pk_bf16(v[8 * c], v[8 * c + 1]), pk_bf16(v[8 * c + 2], v[8 * c + 3]),
                                   pk_bf16(v[8 * c + 4], v[8 * c + 5]), pk_bf16(v[8 * c + 6], v[8 * c + 7]));
            } else {
                const uint4* src = reinterpret_cast<const uint4*>(H1 + (size_t)p * W);
#pragma unroll
                for (int c = 0; c < 8; ++c)
                    *reinterpret_cast<uint4*>(sX + tile_off(tid, 8 + c, kKX2)) =
                        p < n ? __ldg(src + c) : make_uint4(0u, 0u, 0u, 0u);
                *reinterpret_cast<uint4*>(sX + tile_off(tid, 16, kKX2)) =
                    make_uint4(p < n ? pk_bf16(1.0f, 0.0f) : 0u, 0u, 0u, 0u);  // the bias column (2W)
                *reinterpret_cast<uint4*>(sX + tile_off(tid, 17, kKX2)) = make_uint4(0u, 0u, 0u, 0u);
            }
        }
        // edge layer, pipelined over two A tiles and two TMEM accumulators; thread tid always
        // handles edge slot e of particle q of a sub-tile (and drains TMEM lane tid)
        const int q = tid >> 5, e = tid & 31;
        int j_next = edge_j(tile0 + q, e, n, nb, cnt);                 // sub-tile 0
        EdgeIn in = edge_load(tile0 + q, j_next, pos, vel);
        j_next = edge_j(tile0 + kEP + q, e, n, nb, cnt);               // sub-tile 1
        uint4 pj[8];
#pragma unroll
        for (int c = 0; c < 8; ++c) pj[c] = make_uint4(0u, 0u, 0u, 0u);
        bool quit = false;
        for (int s = 0; s <= kSub; ++s) {
            int j_cur = -1;
            if (s < kSub) {
                const int b = s & 1;
                uint4 w0 = make_uint4(0u, 0u, 0u, 0u), w1 = w0;
                if (in.j >= 0) edge_feat16(in.pi, in.vi, in.pj, in.vj, ih, ic, w0, w1);
                j_cur = in.j;
                uint8_t* A = sA + b * (kTP * kKE * 2);
                *reinterpret_cast<uint4*>(A + tile_off(tid, 0, kKE)) = w0;
                *reinterpret_cast<uint4*>(A + tile_off(tid, 1, kKE)) = w1;
                tc::fence_smem_to_async();
            }
            tc::fence_before_sync();
            if (__syncthreads_or(bad)) { quit = true; break; }
            if (s < kSub && tid == 0) {
                const int b = s & 1;
                tc::fence_after_sync();
                tc::mma_bf16(tmem + (uint32_t)(b * W),
                             smem_desc(sa + (uint32_t)(b * kTP * kKE * 2), 128u, sbo(kKE)),
                             smem_desc(we_desc_addr, 128u, sbo(kKE)), id_e, 0u);
                tc::mma_commit(&mbar[b]);
            }
            // gathers of sub-tile s + 1 (its neighbour index was loaded one iteration ago) and the
            // neighbour index of sub-tile s + 2, in flight while sub-tile s - 1 drains
            const int jn = j_next;
            EdgeIn nxt{};
            if (s + 1 < kSub) {
                nxt = edge_load(tile0 + kEP * (s + 1) + q, jn, pos, vel);
                j_next = s + 2 < kSub ? edge_j(tile0 + kEP * (s + 2) + q, e, n, nb, cnt) : -1;
            }
            if (s >= 1) {
                const int sp = s - 1;
                if (!tc::mbar_wait(&mbar[sp & 1], (sp >> 1) & 1)) bad = 1;
                if (__syncthreads_or(bad)) { quit = true; break; }
                tc::fence_after_sync();
                drain_edges<ROUND2>(tmem + (uint32_t)((sp & 1) * W), sp, pj, sX, ROUND2 ? kKX2 : kKX1);
            }
            if constexpr (ROUND2) {  // P_j of the edge this thread built at s (drained at s + 1)
                if (s < kSub) {
#pragma unroll
                    for (int c = 0; c < 8; ++c)
                        pj[c] = j_cur >= 0 ? __ldg(reinterpret_cast<const uint4*>(P + (size_t)j_cur * W) + c)
                                           : make_uint4(0u, 0u, 0u, 0u);
                }
            }
            if (s + 1 < kSub) in = nxt;
        }
        if (quit) break;
        // node layers
        tc::fence_smem_to_async();
        tc::fence_before_sync();
        if (__syncthreads_or(bad)) break;
        constexpr int kKX = ROUND2 ? kKX2 : kKX1;
        if (tid == 0) {
            tc::fence_after_sync();
            for (int k = 0; k < kKX / 16; ++k)
                tc::mma_bf16(tmem, smem_desc(sx + 256u * k, 128u, sbo(kKX)), smem_desc(wn_addr + 256u * k, 128u, sbo(kKX)),
                             id_e, k > 0 ? 1u : 0u);
            tc::mma_commit(&mbar[2]);
        }
        if (!tc::mbar_wait(&mbar[2], 0)) bad = 1;
        if (__syncthreads_or(bad)) break;
        tc::fence_after_sync();
        const int p = tile0 + tid;
        {
            float hv[64];
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                float v[16];
                tc::tmem_ld16(tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)(16 * c), v);
#pragma unroll
                for (int j = 0; j < 16; ++j) hv[16 * c + j] = fmaxf(v[j], 0.0f);
            }
            tc::tmem_wait_ld();
            // the node tile is free (its MMA has completed): stage the hidden vector as the next A operand
            constexpr int kKN = ROUND2 ? kKH2 : kKH1;
#pragma unroll
            for (int c = 0; c < 8; ++c) {
                const uint4 w = make_uint4(pk_bf16(hv[8 * c], hv[8 * c + 1]), pk_bf16(hv[8 * c + 2], hv[8 * c + 3]),
                                           pk_bf16(hv[8 * c + 4], hv[8 * c + 5]), pk_bf16(hv[8 * c + 6], hv[8 * c + 7]));
                *reinterpret_cast<uint4*>(sX + tile_off(tid, c, kKN)) = w;
                if (!ROUND2 && p < n) reinterpret_cast<uint4*>(H1 + (size_t)p * W)[c] = w;
            }
            if constexpr (ROUND2) {
                *reinterpret_cast<uint4*>(sX + tile_off(tid, 8, kKH2)) = make_uint4(pk_bf16(1.0f, 0.0f), 0u, 0u, 0u);
                *reinterpret_cast<uint4*>(sX + tile_off(tid, 9, kKH2)) = make_uint4(0u, 0u, 0u, 0u);
            }
        }
        tc::fence_smem_to_async();
        tc::fence_before_sync();
        if (__syncthreads_or(bad)) break;
        constexpr int kKN = ROUND2 ? kKH2 : kKH1;
        constexpr int kN3 = ROUND2 ? kNO : W;
        if (tid == 0) {
            tc::fence_after_sync();
            const uint32_t id3 = tc::idesc_bf16_f32(128, kN3);
            for (int k = 0; k < kKN / 16; ++k)
                tc::mma_bf16(tmem + (uint32_t)W, smem_desc(sx + 256u * k, 128u, sbo(kKN)),
                             smem_desc(w3_addr + 256u * k, 128u, sbo(kKN)), id3, k > 0 ? 1u : 0u);
            tc::mma_commit(&mbar[2]);
        }
        if (!tc::mbar_wait(&mbar[2], 1)) bad = 1;
        if (__syncthreads_or(bad)) break;
        tc::fence_after_sync();
        if constexpr (!ROUND2) {  // P = H1 Wp, f16
            float pv[64];
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                float v[16];
                tc::tmem_ld16(tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)(W + 16 * c), v);
#pragma unroll
                for (int j = 0; j < 16; ++j) pv[16 * c + j] = v[j];
            }
            tc::tmem_wait_ld();
            if (p < n) {
                uint4* dst = reinterpret_cast<uint4*>(P + (size_t)p * W);
#pragma unroll
                for (int c = 0; c < 8; ++c)
                    dst[c] = make_uint4(to_f16x2(pv[8 * c], pv[8 * c + 1]), to_f16x2(pv[8 * c + 2], pv[8 * c + 3]),
                                        to_f16x2(pv[8 * c + 4], pv[8 * c + 5]), to_f16x2(pv[8 * c + 6], pv[8 * c + 7]));
            }
        } else {  // O = [H2 1] Wo'
            float v[16];
            tc::tmem_ld16(tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)W, v);
            tc::tmem_wait_ld();
            if (p < n) {
                float4* dst = reinterpret_cast<float4*>(out + (size_t)p * kOS);
                dst[0] = make_float4(v[0], v[1], v[2], v[3]);
                dst[1] = make_float4(v[4], v[5], 0.0f, 0.0f);
            }
        }
        tc::fence_before_sync();
        __syncthreads();  // the next tile rewrites the node tile and the TMEM accumulators
    }
    tc::fence_before_sync();
    __syncthreads();
    if (bad && tid == 0 && err) atomicOr(err, 1u);
    if (warp == 0) tc::tmem_dealloc(tmem, kCols);
}

// ---- round 1 with the features on the TMEM lanes -------------------------------------------
// The edge MMA of k_tc_round puts the edges on the TMEM lanes, so the sum over a particle's 32
// edges crosses the lanes of a warp. Here the 64 features are the lanes and the edges the
// columns: D [128 x 128] = A [128 x 32] * B [128 x 32]^T where B's row n holds edge n of two
// 4-particle sub-tiles X and Y side by side ([e_X(n) | e_Y(n)], 16 features each) and A is
// block-diagonal ([We1' | 0] for rows 0..63, [0 | We1'] for rows 64..127), so rows 0..63 of D
// are sub-tile X's pre-activations and rows 64..127 sub-tile Y's. Thread t drains TMEM lane t
// (feature t % 64 of sub-tile t / 64): for each of the 4 particles, 32 consecutive columns =
// its 32 edges, ReLU-packed to f16x2 and summed by a tree inside the thread. One MMA covers 8
// particles; a 128-particle tile is 16 MMAs, then the node layers as in k_tc_round. P is
// written in the permuted BF16 layout that the mma.sync round 2 (sph_mpnn_infer.cu) reads.
constexpr int kLanesMma = kTP / 8;  // edge MMAs per tile (even: the barrier's phases restart)
static_assert(kLanesMma % 2 == 0, "barrier phases must restart with every tile");
// The node tile's first 64 columns (M1, then H1) keep the K-major core-matrix layout with a
// K stride of 144 bytes instead of 128: a row's eight 16-byte chunks then fall on eight
// different bank groups, and the drain, whose warp stores 32 features of one row, stores without
// bank conflicts. Its last 16 columns (node features, bias, padding) are a separate tile.
constexpr int kLboM = 144;                 // K stride of the M1 / H1 core matrices
constexpr int kSboM = 8 * kLboM - 16;      // row-group stride: 8 core matrices, no trailing pad
__host__ __device__ constexpr uint32_t m_off(int r, int k8) {
    return (uint32_t)((r >> 3) * kSboM + k8 * kLboM + (r & 7) * 16);
}
struct SmemLanes {
    static constexpr int kOffAE = 0;                          // [128][32] block-diagonal We1'
    static constexpr int kOffWn = kOffAE + 128 * kKA * 2;     // Wn1' [64][80] then Wp [64][64]
    static constexpr int kOffB = kOffWn + (kImgWe2 - kImgWn1) * 2;  // edge tile [128][32]
    static constexpr int kOffM = kOffB + 128 * kKA * 2;       // M1 / H1 tile [128][64] (m_off)
    static constexpr int kOffXN = kOffM + (kTP / 8) * kSboM;  // node features [128][16]
    static constexpr int kBytes = kOffXN + kTP * 16 * 2;
};
static_assert(m_off(kTP - 1, 7) + 16 <= SmemLanes::kOffXN - SmemLanes::kOffM, "M1 tile inside its region");
static_assert(SmemLanes::kOffM % 16 == 0 && SmemLanes::kOffXN % 16 == 0, "16-byte aligned operand tiles");

// 256 threads: warps w and w + 4 reach the same 32 TMEM lanes and split the work of a lane
// group (the columns of the edge accumulator, the halves of a node row), so twice the warps
// hide the neighbour gathers. Thread t builds edge column t % 128 of sub-tile t / 128.
constexpr int kThrL = 256;

__global__ void __launch_bounds__(kThrL, 4) k_tc_r1_lanes(const float4* __restrict__ pos, const float4* __restrict__ vel,
                                                       const float2* __restrict__ rhop, const int* __restrict__ nb,
                                                       const int* __restrict__ cnt, FrameConst fc, int n,
                                                       const __nv_bfloat16* __restrict__ img,
                                                       __nv_bfloat16* __restrict__ H1, uint4* __restrict__ Pperm,
                                                       uint32_t* __restrict__ err) {
    using L = SmemLanes;
    extern __shared__ __align__(128) uint8_t smem[];  // no-swizzle operands: 16-byte alignment
    __shared__ __align__(8) uint64_t mbar[2];
    __shared__ uint32_t tmem_slot;
    __shared__ int bad;
    uint8_t* const sB = smem + L::kOffB;
    uint8_t* const sM = smem + L::kOffM;
    uint8_t* const sXN = smem + L::kOffXN;
    const int tid = threadIdx.x, warp = tid >> 5;
    {
        const uint4* a = reinterpret_cast<const uint4*>(img + kImgAE1);
        uint4* da = reinterpret_cast<uint4*>(smem + L::kOffAE);
        for (int i = tid; i < 128 * kKA * 2 / 16; i += kThrL) da[i] = __ldg(a + i);
        const uint4* w = reinterpret_cast<const uint4*>(img + kImgWn1);
        uint4* dw = reinterpret_cast<uint4*>(smem + L::kOffWn);
        for (int i = tid; i < (kImgWe2 - kImgWn1) * 2 / 16; i += kThrL) dw[i] = __ldg(w + i);
    }
    if (tid == 0) {
        tc::mbar_init(&mbar[0], 1);
        tc::mbar_init(&mbar[1], 1);
        tc::mbar_init_fence();
        bad = 0;
    }
    if (warp == 0) tc::tmem_alloc(&tmem_slot, kCols);
    tc::fence_smem_to_async();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = tmem_slot;
    const uint32_t s_ae = smem_u32(smem + L::kOffAE), s_wn = smem_u32(smem + L::kOffWn);
    const uint32_t s_wp = s_wn + (uint32_t)((kImgWp - kImgWn1) * 2);
    const uint32_t sb = smem_u32(sB), sm = smem_u32(sM), sxn = smem_u32(sXN);
    const uint32_t id_e = tc::idesc_bf16_f32(128, 128), id_n = tc::idesc_bf16_f32(128, W);
    const float ih = 1.0f / fc.h, ic = 1.0f / fc.c;
    const int ntiles = (n + kTP - 1) / kTP;
    const int lane_t = tid & 127;                  // the TMEM lane (and node row) this thread serves
    const int grp = tid >> 7;                      // which half of that lane's work it does
    const int col = tid & 127, sub = tid >> 7;     // the edge it builds: column col of sub-tile sub
    const int q = col >> 5, e = col & 31;          //   = particle q of the sub-tile, slot e
    const int f = lane_t & 63, half = lane_t >> 6; // the lane it drains: feature f of sub-tile half
    const uint32_t lane_base = (uint32_t)(32 * (warp & 3)) << 16;

    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int tile0 = tile * kTP;
        if (grp == 0) {  // node features, bias column and padding (columns 64 .. 79) of particle lane_t
            const int p = tile0 + lane_t;
            float v[16];
#pragma unroll
            for (int c = 0; c < 16; ++c) v[c] = 0.0f;
            if (p < n) {
                const float4 vi = vel[p];
                const float rho = rhop[p].x;
                v[0] = vi.x * ic; v[1] = vi.y * ic; v[2] = vi.z * ic;
                v[3] = rho / fc.rho_self - 1.0f;
                v[4] = (rho - fc.rho0) / fc.rho_self;
                v[5] = fc.log_mu;
                v[6] = (float)min(max(cnt[p], 0), K) / K;
                v[7] = 1.0f;
                v[8] = fc.courant;
                v[9] = 1.0f;
            }
#pragma unroll
            for (int c = 0; c < 2; ++c)
                *reinterpret_cast<uint4*>(sXN + tile_off(lane_t, c, 16)) =
                    make_uint4(pk_bf16(v[8 * c], v[8 * c + 1]), pk_bf16(v[8 * c + 2], v[8 * c + 3]),
                               pk_bf16(v[8 * c + 4], v[8 * c + 5]), pk_bf16(v[8 * c + 6], v[8 * c + 7]));
        }
        // edge phase: MMA i takes sub-tile 0 = particles 8 i .. 8 i + 3, sub-tile 1 = 8 i + 4 .. 8 i + 7
        int jn = edge_j(tile0 + 4 * sub + q, e, n, nb, cnt);
        EdgeIn in = edge_load(tile0 + 4 * sub + q, jn, pos, vel);
        jn = edge_j(tile0 + 8 + 4 * sub + q, e, n, nb, cnt);
        bool quit = false;
        for (int i = 0; i < kLanesMma; ++i) {
            {
                uint4 w0 = make_uint4(0u, 0u, 0u, 0u), w1 = w0;
                if (in.j >= 0) edge_feat16(in.pi, in.vi, in.pj, in.vj, ih, ic, w0, w1);
                *reinterpret_cast<uint4*>(sB + tile_off(col, 2 * sub, kKA)) = w0;
                *reinterpret_cast<uint4*>(sB + tile_off(col, 2 * sub + 1, kKA)) = w1;
            }
            tc::fence_smem_to_async();
            tc::fence_before_sync();
            if (__syncthreads_or(bad)) { quit = true; break; }
            if (tid == 0) {
                tc::fence_after_sync();
                for (int k = 0; k < kKA / 16; ++k)
                    tc::mma_bf16(tmem, smem_desc(s_ae + 256u * k, 128u, sbo(kKA)), smem_desc(sb + 256u * k, 128u, sbo(kKA)),
                                 id_e, k > 0 ? 1u : 0u);
                tc::mma_commit(&mbar[0]);
            }
            if (i + 1 < kLanesMma) {  // gathers of MMA i + 1, neighbour index of MMA i + 2, in flight
                const int b1 = tile0 + 8 * (i + 1) + 4 * sub + q;
                in = edge_load(b1, jn, pos, vel);
                jn = i + 2 < kLanesMma ? edge_j(b1 + 8, e, n, nb, cnt) : -1;
            }
            if (!tc::mbar_wait(&mbar[0], i & 1)) bad = 1;
            if (__syncthreads_or(bad)) { quit = true; break; }
            tc::fence_after_sync();
#pragma unroll 1
            for (int k = 0; k < 2; ++k) {  // this thread's two particles of the lane's sub-tile
                const int pq = 2 * grp + k;
                uint32_t r[32];
                tc::tmem_ld32(tmem + lane_base + (uint32_t)(32 * pq), r);
                tc::tmem_wait_ld();
                uint32_t h[16];
#pragma unroll
                for (int u = 0; u < 16; ++u) h[u] = relu_f16x2(__uint_as_float(r[2 * u]), __uint_as_float(r[2 * u + 1]));
#pragma unroll
                for (int w = 8; w >= 1; w >>= 1)
#pragma unroll
                    for (int u = 0; u < w; ++u) h[u] = hadd2(h[u], h[u + w]);
                const float2 s2 = __half22float2(*reinterpret_cast<__half2*>(&h[0]));
                const int row = 8 * i + 4 * half + pq;
                *reinterpret_cast<__nv_bfloat16*>(sM + m_off(row, f >> 3) + (f & 7) * 2) =
                    __float2bfloat16_rn((s2.x + s2.y) * (1.0f / K));
            }
            tc::fence_before_sync();  // the next MMA overwrites the accumulator
        }
        if (quit) break;
        // node layers: H1 = relu([M1 n 1] Wn1'), then P = H1 Wp; node row lane_t, columns 32 grp ..
        tc::fence_smem_to_async();
        tc::fence_before_sync();
        if (__syncthreads_or(bad)) break;
        if (tid == 0) {
            tc::fence_after_sync();
            for (int k = 0; k < W / 16; ++k)  // K 0 .. 63: M1
                tc::mma_bf16(tmem, smem_desc(sm + 2u * kLboM * k, (uint32_t)kLboM, (uint32_t)kSboM),
                             smem_desc(s_wn + 256u * k, 128u, sbo(kKX1)), id_n, k > 0 ? 1u : 0u);
            // K 64 .. 79: node features, bias, padding
            tc::mma_bf16(tmem, smem_desc(sxn, 128u, sbo(16)), smem_desc(s_wn + 256u * (W / 16), 128u, sbo(kKX1)),
                         id_n, 1u);
            tc::mma_commit(&mbar[1]);
        }
        if (!tc::mbar_wait(&mbar[1], 0)) bad = 1;
        if (__syncthreads_or(bad)) break;
        tc::fence_after_sync();
        const int p = tile0 + lane_t;
        {  // the X tile is no longer read (its MMA completed): H1 goes over it
            float hv[32];
#pragma unroll
            for (int c = 0; c < 2; ++c) {
                float v[16];
                tc::tmem_ld16(tmem + lane_base + (uint32_t)(32 * grp + 16 * c), v);
#pragma unroll
                for (int j = 0; j < 16; ++j) hv[16 * c + j] = fmaxf(v[j], 0.0f);
            }
            tc::tmem_wait_ld();
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                const uint4 w = make_uint4(pk_bf16(hv[8 * c], hv[8 * c + 1]), pk_bf16(hv[8 * c + 2], hv[8 * c + 3]),
                                           pk_bf16(hv[8 * c + 4], hv[8 * c + 5]), pk_bf16(hv[8 * c + 6], hv[8 * c + 7]));
                *reinterpret_cast<uint4*>(sM + m_off(lane_t, 4 * grp + c)) = w;
                if (p < n) reinterpret_cast<uint4*>(H1 + (size_t)p * W)[4 * grp + c] = w;
            }
        }
        tc::fence_smem_to_async();
        tc::fence_before_sync();
        if (__syncthreads_or(bad)) break;
        if (tid == 0) {
            tc::fence_after_sync();
            for (int k = 0; k < kKH1 / 16; ++k)
                tc::mma_bf16(tmem + (uint32_t)W, smem_desc(sm + 2u * kLboM * k, (uint32_t)kLboM, (uint32_t)kSboM),
                             smem_desc(s_wp + 256u * k, 128u, sbo(kKH1)), id_n, k > 0 ? 1u : 0u);
            tc::mma_commit(&mbar[1]);
        }
        if (!tc::mbar_wait(&mbar[1], 1)) bad = 1;
        if (__syncthreads_or(bad)) break;
        tc::fence_after_sync();
        {
            float pv[32];  // features 32 grp .. 32 grp + 31
#pragma unroll
            for (int c = 0; c < 2; ++c) {
                float v[16];
                tc::tmem_ld16(tmem + lane_base + (uint32_t)(W + 32 * grp + 16 * c), v);
#pragma unroll
                for (int j = 0; j < 16; ++j) pv[16 * c + j] = v[j];
            }
            tc::tmem_wait_ld();
            if (p < n) {  // words 2 grp, 2 grp + 1 of lane group g: features (16 mt + g, 16 mt + g + 8)
                uint2* dst = reinterpret_cast<uint2*>(Pperm + (size_t)p * 8);
#pragma unroll
                for (int g = 0; g < 8; ++g)
                    dst[2 * g + grp] = make_uint2(pk_bf16(pv[g], pv[g + 8]), pk_bf16(pv[16 + g], pv[24 + g]));
            }
        }
        tc::fence_before_sync();
        __syncthreads();
    }
    tc::fence_before_sync();
    __syncthreads();
    if (bad && tid == 0 && err) atomicOr(err, 1u);
    if (warp == 0) tc::tmem_dealloc(tmem, kCols);
}

int lanes_grid(int n) {
    static int per_sm = 0;
    if (!per_sm) {
        cudaFuncSetAttribute(k_tc_r1_lanes, cudaFuncAttributeMaxDynamicSharedMemorySize, SmemLanes::kBytes);
        int dev = 0, smem_sm = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
        cudaFuncAttributes fa{};
        cudaFuncGetAttributes(&fa, k_tc_r1_lanes);
        per_sm = smem_sm / (SmemLanes::kBytes + (int)fa.sharedSizeBytes + 1024);
        if (per_sm < 1) per_sm = 1;
        if (per_sm > 4) per_sm = 4;
    }
    const int ntiles = (n + kTP - 1) / kTP;
    const int cap = device_sm_count() * per_sm;
    return ntiles < cap ? ntiles : cap;
}

// Resident CTAs per SM: shared memory (dynamic + static + the 1 KB the hardware reserves per
// CTA) and TMEM (4 x 128 columns) decide; the persistent grid holds that many per SM.
template <bool ROUND2>
int tc_grid(int n) {
    static int per_sm = 0;
    auto k = k_tc_round<ROUND2>;
    if (!per_sm) {
        cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, Smem<ROUND2>::kBytes);
        int dev = 0, smem_sm = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
        cudaFuncAttributes fa{};
        cudaFuncGetAttributes(&fa, k);
        const int per = Smem<ROUND2>::kBytes + (int)fa.sharedSizeBytes + 1024;
        per_sm = smem_sm / per;
        if (per_sm < 1) per_sm = 1;
        if (per_sm > 4) per_sm = 4;
    }
    const int ntiles = (n + kTP - 1) / kTP;
    const int cap = device_sm_count() * per_sm;
    return ntiles < cap ? ntiles : cap;
}

}  // namespace

int tc_infer_words() { return kImgTotal; }

void tc_infer_prep(const float* prm, __nv_bfloat16* img, cudaStream_t st) {
    k_tc_infer_prep<<<(kImgTotal + 255) / 256, 256, 0, st>>>(prm, img);
}

void tc_infer_round1(const Frame& f, const __nv_bfloat16* img, __nv_bfloat16* H1, __half* P, uint32_t* err,
                     cudaStream_t st) {
    if (f.n <= 0) return;
    const int g = tc_grid<false>(f.n);
    k_tc_round<false><<<g, kThr, Smem<false>::kBytes, st>>>(f.pos, f.vel, f.rhop, f.nb, f.cnt, f.fc, f.n, img, H1, P,
                                                            nullptr, err);
}

void tc_infer_round1_lanes(const Frame& f, const __nv_bfloat16* img, __nv_bfloat16* H1, uint16_t* Pperm, uint32_t* err,
                           cudaStream_t st) {
    if (f.n <= 0) return;
    const int g = lanes_grid(f.n);
    k_tc_r1_lanes<<<g, kThrL, SmemLanes::kBytes, st>>>(f.pos, f.vel, f.rhop, f.nb, f.cnt, f.fc, f.n, img, H1,
                                                     reinterpret_cast<uint4*>(Pperm), err);
}

void tc_infer_round2(const Frame& f, const __nv_bfloat16* img, const __nv_bfloat16* H1, const __half* P, float* out,
                     uint32_t* err, cudaStream_t st) {
    if (f.n <= 0) return;
    const int g = tc_grid<true>(f.n);
    k_tc_round<true><<<g, kThr, Smem<true>::kBytes, st>>>(f.pos, f.vel, f.rhop, f.nb, f.cnt, f.fc, f.n, img,
                                                          const_cast<__nv_bfloat16*>(H1), const_cast<__half*>(P), out,
                                                          err);
}

}  // namespace mpnn
}  // namespace sphgb
