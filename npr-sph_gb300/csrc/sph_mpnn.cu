// sph_mpnn.cu -- training of the learned macro-step network on the GPU:
// FP32 forward and backward kernels and Adam, over frames the SPH step itself
// recorded. (Inference at scale runs on BF16 tensor cores in
// sph_mpnn_infer.cu; this file is the exact FP32 reference for it.)
//
// The forward pass is split into small kernels that each do one thing:
//   k_edge1_fwd   edge features e_ij (stored), round-1 edge layer, mean -> M1, node features
//   k_dense_fwd   [M1 n] Wn1 -> H1, H1 Wp -> P, [M2 H1] Wn2 -> H2, H2 Wo -> O
//   k_edge2_fwd   round-2 edge layer with the gathered P_j, mean -> M2
// and the backward pass mirrors it: dense data/weight gradients, per-edge
// gradients of round 2 (materialised), the reverse-edge gather that returns
// dP_j to the sending particle, and the round-1 edge weight gradient. Weight
// gradients are reduced in fixed-order partials, and the reverse-edge lists are
// sorted by edge before the gather, so training is deterministic.
#include <cmath>
#include <cstring>
#include <vector>

#include "sph_mpnn.h"
#include "sph_internal.h"
#include "sph_tc.h"

namespace sphgb {
namespace mpnn {

namespace {

constexpr int kT = 128;  // threads per CTA

inline int nblk(long long n, int t = kT) { return (int)((n + t - 1) / t); }

// Edge and node features (the header of sph_mpnn.h states them).
__device__ __forceinline__ void edge_feat(float4 pi, float4 vi, float4 pj, float4 vj, const FrameConst& fc,
                                          float* e) {
    const float ih = 1.0f / fc.h, ic = 1.0f / fc.c;
    const float dx = (pj.x - pi.x) * ih, dy = (pj.y - pi.y) * ih, dz = (pj.z - pi.z) * ih;
    const float ux = (vj.x - vi.x) * ic, uy = (vj.y - vi.y) * ic, uz = (vj.z - vi.z) * ic;
    const float r = sqrtf(dx * dx + dy * dy + dz * dz);
    const float q = 1.0f - r;
    const float sg = r > 0.0f ? q * q / r : 0.0f;
    e[0] = dx; e[1] = dy; e[2] = dz;
    e[3] = ux; e[4] = uy; e[5] = uz;
    e[6] = r;
    e[7] = q;
    e[8] = sg * dx; e[9] = sg * dy; e[10] = sg * dz;
    e[11] = q * ux; e[12] = q * uy; e[13] = q * uz;
}

__device__ __forceinline__ void node_feat(float4 vi, float rho, int cnt, const FrameConst& fc, float* nf) {
    const float ic = 1.0f / fc.c;
    nf[0] = vi.x * ic; nf[1] = vi.y * ic; nf[2] = vi.z * ic;
    nf[3] = rho / fc.rho_self - 1.0f;
    nf[4] = (rho - fc.rho0) / fc.rho_self;
    nf[5] = fc.log_mu;
    nf[6] = (float)cnt / K;
    nf[7] = 1.0f;
    nf[8] = fc.courant;
}

// The edge layers run four threads per particle, each owning 16 of the 64 outputs (kGrp
// groups): 16 accumulators per thread, four times the threads of a thread per particle. Each
// output is summed over the edges in the same order as with one thread per particle.
constexpr int kGrp = 4, kGW = W / kGrp;

// Round 1 edge layer: E (stored, by group 0), relu masks (16 bits per group), X1 = [M1, n].
__global__ void __launch_bounds__(kT) k_edge1_fwd(Frame f, const float* __restrict__ prm, float* __restrict__ E,
                                                 unsigned long long* __restrict__ mask1, float* __restrict__ X1) {
    __shared__ float sW[FE * W], sb[W];
    for (int t = threadIdx.x; t < FE * W; t += kT) sW[t] = prm[kWe1 + t];
    for (int t = threadIdx.x; t < W; t += kT) sb[t] = prm[kBe1 + t];
    __syncthreads();
    const long long gt = (long long)blockIdx.x * kT + threadIdx.x;
    const int i = (int)(gt / kGrp), g = (int)(gt % kGrp);
    if (i >= f.n) return;
    const float4 pi = f.pos[i], vi = f.vel[i];
    const int cnt = min(max(f.cnt[i], 0), K);
    float m[kGW];
#pragma unroll
    for (int o = 0; o < kGW; ++o) m[o] = 0.0f;
    unsigned short* mk = reinterpret_cast<unsigned short*>(mask1);
    for (int k = 0; k < K; ++k) {
        float e[FE];
        unsigned bits = 0u;
        const int j = k < cnt ? f.nb[i * K + k] : -1;
        if (j >= 0 && j < f.n) {
            edge_feat(pi, vi, f.pos[j], f.vel[j], f.fc, e);
#pragma unroll
            for (int u = 0; u < kGW; ++u) {
                const int o = g * kGW + u;
                float z = sb[o];
#pragma unroll
                for (int q = 0; q < FE; ++q) z = fmaf(e[q], sW[q * W + o], z);
                if (z > 0.0f) { m[u] += z; bits |= 1u << u; }
            }
        } else {
#pragma unroll
            for (int q = 0; q < FE; ++q) e[q] = 0.0f;
        }
        if (g == 0) {
#pragma unroll
            for (int q = 0; q < FE; ++q) E[((size_t)i * K + k) * FE + q] = e[q];
        }
        mk[((size_t)i * K + k) * kGrp + g] = (unsigned short)bits;  // bits 16 g .. 16 g + 15 of the u64
    }
    float* x = X1 + (size_t)i * (W + FN);
#pragma unroll
    for (int u = 0; u < kGW; ++u) x[g * kGW + u] = m[u] * (1.0f / K);
    if (g == 0) {
        float nf[FN];
        node_feat(vi, f.rhop[i].x, cnt, f.fc, nf);
#pragma unroll
        for (int q = 0; q < FN; ++q) x[W + q] = nf[q];
    }
}

// Round 2 edge layer: relu masks, X2 = [M2, H1].
__global__ void __launch_bounds__(kT) k_edge2_fwd(Frame f, const float* __restrict__ prm, const float* __restrict__ E,
                                                 const float* __restrict__ P, const float* __restrict__ H1,
                                                 unsigned long long* __restrict__ mask2, float* __restrict__ X2) {
    __shared__ float sW[FE * W], sb[W];
    for (int t = threadIdx.x; t < FE * W; t += kT) sW[t] = prm[kWe2 + t];
    for (int t = threadIdx.x; t < W; t += kT) sb[t] = prm[kBe2 + t];
    __syncthreads();
    const long long gt = (long long)blockIdx.x * kT + threadIdx.x;
    const int i = (int)(gt / kGrp), g = (int)(gt % kGrp);
    if (i >= f.n) return;
    const int cnt = min(max(f.cnt[i], 0), K);
    float m[kGW];
#pragma unroll
    for (int o = 0; o < kGW; ++o) m[o] = 0.0f;
    unsigned short* mk = reinterpret_cast<unsigned short*>(mask2);
    for (int k = 0; k < K; ++k) {
        unsigned bits = 0u;
        const int j = k < cnt ? f.nb[i * K + k] : -1;
        if (j >= 0 && j < f.n) {
            float e[FE];
#pragma unroll
            for (int q = 0; q < FE; ++q) e[q] = E[((size_t)i * K + k) * FE + q];
            const float* pj = P + (size_t)j * W + g * kGW;
#pragma unroll
            for (int u = 0; u < kGW; ++u) {
                const int o = g * kGW + u;
                float z = sb[o] + pj[u];
#pragma unroll
                for (int q = 0; q < FE; ++q) z = fmaf(e[q], sW[q * W + o], z);
                if (z > 0.0f) { m[u] += z; bits |= 1u << u; }
            }
        }
        mk[((size_t)i * K + k) * kGrp + g] = (unsigned short)bits;
    }
    float* x = X2 + (size_t)i * 2 * W;
#pragma unroll
    for (int u = 0; u < kGW; ++u) {
        x[g * kGW + u] = m[u] * (1.0f / K);
        x[W + g * kGW + u] = H1[(size_t)i * W + g * kGW + u];
    }
}

// Y[i, o] = act(sum_k X[i, k] W[k, o] + b[o]); one thread per (i, o).
__global__ void __launch_bounds__(kT) k_dense_fwd(const float* __restrict__ X, int ldx, int kin,
                                                 const float* __restrict__ Wt, const float* __restrict__ b, int nout,
                                                 float* __restrict__ Y, int ldy, int n, int relu) {
    const long long t = (long long)blockIdx.x * kT + threadIdx.x;
    if (t >= (long long)n * nout) return;
    const int i = (int)(t / nout), o = (int)(t % nout);
    const float* x = X + (size_t)i * ldx;
    float s = b ? b[o] : 0.0f;
    for (int k = 0; k < kin; ++k) s = fmaf(x[k], Wt[k * nout + o], s);
    Y[(size_t)i * ldy + o] = relu ? fmaxf(s, 0.0f) : s;
}

// dX[i, k] = (add[i, k] + sum_o dY[i, o] W[k, o]) * (H[i, k] > 0 if H).
__global__ void __launch_bounds__(kT) k_dense_bwd_data(const float* __restrict__ dY, int ldy, int nout,
                                                      const float* __restrict__ Wt, int kin,
                                                      const float* __restrict__ add, int lda,
                                                      const float* __restrict__ H, int ldh, float* __restrict__ dX,
                                                      int ldx, int n) {
    const long long t = (long long)blockIdx.x * kT + threadIdx.x;
    if (t >= (long long)n * kin) return;
    const int i = (int)(t / kin), k = (int)(t % kin);
    const float* dy = dY + (size_t)i * ldy;
    float s = add ? add[(size_t)i * lda + k] : 0.0f;
    for (int o = 0; o < nout; ++o) s = fmaf(dy[o], Wt[k * nout + o], s);
    if (H && !(H[(size_t)i * ldh + k] > 0.0f)) s = 0.0f;
    dX[(size_t)i * ldx + k] = s;
}

// Weight gradient partials: part[split][k][o] = sum_{i in split} X[i,k] dY[i,o]; row k == kin is
// the bias (X = 1). Rows of a split are summed in order: deterministic.
__global__ void __launch_bounds__(kT) k_wgrad_partial(const float* __restrict__ X, int ldx, int kin,
                                                     const float* __restrict__ dY, int ldy, int nout, int n,
                                                     int rows_per_split, float* __restrict__ part) {
    const int t = blockIdx.x * kT + threadIdx.x;
    const int total = (kin + 1) * nout;
    if (t >= total) return;
    const int k = t / nout, o = t % nout;
    const int a = blockIdx.y * rows_per_split, b = min(a + rows_per_split, n);
    float s = 0.0f;
    for (int i = a; i < b; ++i) s = fmaf(k < kin ? X[(size_t)i * ldx + k] : 1.0f, dY[(size_t)i * ldy + o], s);
    part[(size_t)blockIdx.y * total + t] = s;
}

// Edge-layer weight gradient partials over edges (kin = FE, bias row FE). Round 2 reads the
// materialised dZ; round 1 (dZ == null) forms dZ1 = dM1 / K masked by the relu bits.
__global__ void __launch_bounds__(kT) k_edge_wgrad_partial(const float* __restrict__ E, const float* __restrict__ dZ,
                                                          const float* __restrict__ dM, int ldm,
                                                          const unsigned long long* __restrict__ mask,
                                                          const int* __restrict__ cnt, int n, int rows_per_split,
                                                          float* __restrict__ part) {
    const int t = blockIdx.x * kT + threadIdx.x;
    const int total = (FE + 1) * W;
    if (t >= total) return;
    const int k = t / W, o = t % W;
    const long long a = (long long)blockIdx.y * rows_per_split;
    const long long b = min(a + rows_per_split, (long long)n * K);
    float s = 0.0f;
    for (long long r = a; r < b; ++r) {
        const int i = (int)(r / K), e = (int)(r % K);
        if (e >= cnt[i]) continue;
        float dz;
        if (dZ) dz = dZ[r * W + o];
        else dz = ((mask[r] >> o) & 1ull) ? dM[(size_t)i * ldm + o] * (1.0f / K) : 0.0f;
        s = fmaf(k < FE ? E[r * FE + k] : 1.0f, dz, s);
    }
    part[(size_t)blockIdx.y * total + t] = s;
}

__global__ void __launch_bounds__(kT) k_reduce_split(const float* __restrict__ part, int splits, int total,
                                                    float* __restrict__ gw, int nw, float* __restrict__ gb) {
    const int t = blockIdx.x * kT + threadIdx.x;
    if (t >= total) return;
    float s = 0.0f;
    for (int q = 0; q < splits; ++q) s += part[(size_t)q * total + t];
    if (t < nw) gw[t] = s;
    else if (gb) gb[t - nw] = s;
}

// Loss: mean over particles of |O - target|^2 (both heads); dO = 2 (O - target) / n.
__global__ void __launch_bounds__(kT) k_loss(const float* __restrict__ O, const float* __restrict__ target, int n,
                                            float* __restrict__ dO, double* __restrict__ part) {
    __shared__ double sh[kT];
    const int i = blockIdx.x * kT + threadIdx.x;
    double l = 0.0;
    if (i < n) {
        const float s = 2.0f / (float)n;
#pragma unroll
        for (int q = 0; q < kOS; ++q) {
            const float d = q < FO ? O[(size_t)i * kOS + q] - target[(size_t)i * kOS + q] : 0.0f;
            dO[(size_t)i * kOS + q] = s * d;
            l += (double)d * d;
        }
    }
    sh[threadIdx.x] = l;
    __syncthreads();
    for (int o = kT / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

// Per-edge round-2 gradient dZ2 = dM2 / K masked by the relu bits (zero on padded edges).
__global__ void __launch_bounds__(kT) k_edge2_bwd(const float* __restrict__ dX2, const unsigned long long* __restrict__ mask2,
                                                 const int* __restrict__ cnt, int n, float* __restrict__ dZ2) {
    const long long t = (long long)blockIdx.x * kT + threadIdx.x;
    if (t >= (long long)n * K * W) return;
    const long long r = t / W;
    const int o = (int)(t % W), i = (int)(r / K), e = (int)(r % K);
    float v = 0.0f;
    if (e < cnt[i] && ((mask2[r] >> o) & 1ull)) v = dX2[(size_t)i * 2 * W + o] * (1.0f / K);
    dZ2[t] = v;
}

__global__ void __launch_bounds__(kT) k_rev_count(const int* __restrict__ nb, const int* __restrict__ cnt, int n,
                                                 int* __restrict__ rc) {
    const long long r = (long long)blockIdx.x * kT + threadIdx.x;
    if (r >= (long long)n * K) return;
    const int i = (int)(r / K), e = (int)(r % K);
    const int j = e < cnt[i] ? nb[r] : -1;
    if (j >= 0 && j < n) atomicAdd(&rc[j], 1);
}

// Exclusive scan of rc[0, n) into off[0, n] by one CTA of 1024 threads (frames are small).
__global__ void __launch_bounds__(1024) k_scan_small(const int* __restrict__ rc, int n, int* __restrict__ off) {
    __shared__ int s[1024];
    const int per = (n + 1023) / 1024, a = threadIdx.x * per, b = min(a + per, n);
    int local = 0;
    for (int i = a; i < b; ++i) local += rc[i];
    s[threadIdx.x] = local;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {
        const int v = threadIdx.x >= o ? s[threadIdx.x - o] : 0;
        __syncthreads();
        s[threadIdx.x] += v;
        __syncthreads();
    }
    int run = s[threadIdx.x] - local;
    for (int i = a; i < b; ++i) { off[i] = run; run += rc[i]; }
    if (threadIdx.x == 1023) off[n] = s[1023];
}

__global__ void __launch_bounds__(kT) k_rev_fill(const int* __restrict__ nb, const int* __restrict__ cnt, int n,
                                                const int* __restrict__ off, int* __restrict__ cur,
                                                int* __restrict__ edges) {
    const long long r = (long long)blockIdx.x * kT + threadIdx.x;
    if (r >= (long long)n * K) return;
    const int i = (int)(r / K), e = (int)(r % K);
    const int j = e < cnt[i] ? nb[r] : -1;
    if (j < 0 || j >= n) return;
    edges[off[j] + atomicAdd(&cur[j], 1)] = (int)r;
}

// Each particle's reverse edges in ascending edge order (k_rev_fill places them in atomicAdd
// order): an insertion sort of the short list (~the neighbour count), one thread per particle,
// so that k_rev_gather sums dP in a fixed order and training is reproducible.
__global__ void __launch_bounds__(kT) k_rev_sort(const int* __restrict__ off, int n, int* __restrict__ edges) {
    const int j = blockIdx.x * kT + threadIdx.x;
    if (j >= n) return;
    const int a = off[j], b = off[j + 1];
    for (int q = a + 1; q < b; ++q) {
        const int x = edges[q];
        int u = q - 1;
        while (u >= a && edges[u] > x) {
            edges[u + 1] = edges[u];
            --u;
        }
        edges[u + 1] = x;
    }
}

// dP[j, o] = sum over the edges (i -> j) of dZ2[edge, o], in ascending edge order.
__global__ void __launch_bounds__(kT) k_rev_gather(const int* __restrict__ off, const int* __restrict__ edges,
                                                  const float* __restrict__ dZ2, int n, float* __restrict__ dP) {
    const long long t = (long long)blockIdx.x * kT + threadIdx.x;
    if (t >= (long long)n * W) return;
    const int j = (int)(t / W), o = (int)(t % W);
    float s = 0.0f;
    for (int q = off[j]; q < off[j + 1]; ++q) s += dZ2[(size_t)edges[q] * W + o];
    dP[t] = s;
}

// dP[j, o] = sum over the edges (i -> j), in ascending edge order, of dZ2[edge, o] formed on the
// fly: dX2[i, o] / K where relu bit o of the edge is set (the terms of k_rev_gather, without
// the materialised dZ2).
__global__ void __launch_bounds__(kT) k_rev_gather_masked(const int* __restrict__ off, const int* __restrict__ edges,
                                                         const float* __restrict__ dX2,
                                                         const unsigned long long* __restrict__ mask2, int n,
                                                         float* __restrict__ dP) {
    const long long t = (long long)blockIdx.x * kT + threadIdx.x;
    if (t >= (long long)n * W) return;
    const int j = (int)(t / W), o = (int)(t % W);
    float s = 0.0f;
    for (int q = off[j]; q < off[j + 1]; ++q) {
        const int e = edges[q];
        if ((mask2[e] >> o) & 1ull) s += dX2[(size_t)(e / K) * 2 * W + o] * (1.0f / K);
    }
    dP[t] = s;
}

__global__ void __launch_bounds__(kT) k_adam(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                                            float* __restrict__ v, int np, float lr, float b1, float b2, float eps,
                                            float c1, float c2) {
    const int t = blockIdx.x * kT + threadIdx.x;
    if (t >= np) return;
    const float gt = g[t];
    const float mt = b1 * m[t] + (1.0f - b1) * gt;
    const float vt = b2 * v[t] + (1.0f - b2) * gt * gt;
    m[t] = mt;
    v[t] = vt;
    p[t] -= lr * (mt * c1) / (sqrtf(vt * c2) + eps);
}

// ---- operands of the tensor-core path --------------------------------------------------
// BF16 copies of an FP32 activation or gradient matrix src [n][lds] (its first ncols columns):
// dst [n][ldd] row-major with column bias_col = 1 and the other columns >= ncols zero, and/or
// dstT [ldd][ldt] transposed (the K-major operand of a weight gradient, which contracts over
// particles), zero for particles n .. kpad - 1. 32 x 32 tiles through shared memory, so both
// the reads and the transposed writes are coalesced.
__global__ void __launch_bounds__(256) k_pack_bf16(const float* __restrict__ src, int lds, int ncols, int n, int kpad,
                                                  int bias_col, __nv_bfloat16* __restrict__ dst, int ldd,
                                                  __nv_bfloat16* __restrict__ dstT, int ldt) {
    __shared__ float tile[32][33];
    const int i0 = blockIdx.x * 32, c0 = blockIdx.y * 32;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
#pragma unroll
    for (int r = ty; r < 32; r += 8) {
        const int i = i0 + r, c = c0 + tx;
        float v = 0.0f;
        if (i < n && c < ldd) v = c < ncols ? src[(size_t)i * lds + c] : (c == bias_col ? 1.0f : 0.0f);
        tile[r][tx] = v;
        if (dst && i < n && c < ldd) dst[(size_t)i * ldd + c] = __float2bfloat16_rn(v);
    }
    if (!dstT) return;
    __syncthreads();
#pragma unroll
    for (int r = ty; r < 32; r += 8) {
        const int c = c0 + r, i = i0 + tx;
        if (c < ldd && i < kpad) dstT[(size_t)c * ldt + i] = __float2bfloat16_rn(tile[tx][r]);
    }
}

// Edge operands of the edge-layer weight gradients, transposed (K = edges, padded to rpad):
//   ET  [16][rpad]: rows 0..13 the edge features E, row 14 = 1 on real edges (the bias), 15 = 0;
//   dZT [64][rpad]: dZ[r][o] = dM[i][o] / K where relu bit o of edge r is set, 0 elsewhere
//                   (dM = columns 0..63 of dX, row stride ld).
// One thread per edge r, looping over the rows: the 32 lanes of a warp are the 32 edges of one
// particle, so each transposed write is 32 consecutive bf16 and the reads of dX broadcast.
__global__ void __launch_bounds__(kT) k_pack_et(const float* __restrict__ E, const int* __restrict__ cnt, int n, int rpad,
                                               __nv_bfloat16* __restrict__ ET) {
    const long long r = (long long)blockIdx.x * kT + threadIdx.x;
    if (r >= rpad) return;
    float v[16];
#pragma unroll
    for (int k = 0; k < 16; ++k) v[k] = 0.0f;
    if (r < (long long)n * K) {
        const int i = (int)(r / K), e = (int)(r % K);
#pragma unroll
        for (int k = 0; k < FE; ++k) v[k] = E[r * FE + k];
        v[FE] = e < cnt[i] ? 1.0f : 0.0f;
    }
#pragma unroll
    for (int k = 0; k < 16; ++k) ET[(size_t)k * rpad + r] = __float2bfloat16_rn(v[k]);
}

__global__ void __launch_bounds__(kT) k_pack_dzt(const float* __restrict__ dX, int ld,
                                                const unsigned long long* __restrict__ mask, const int* __restrict__ cnt,
                                                int n, int rpad, __nv_bfloat16* __restrict__ dZT) {
    const long long r = (long long)blockIdx.x * kT + threadIdx.x;
    if (r >= rpad) return;
    unsigned long long bits = 0ull;
    int i = 0;
    if (r < (long long)n * K) {
        i = (int)(r / K);
        if ((int)(r % K) < cnt[i]) bits = mask[r];
    }
    const float* dm = dX + (size_t)i * ld;
#pragma unroll 8
    for (int o = 0; o < W; ++o)
        dZT[(size_t)o * rpad + r] = __float2bfloat16_rn(((bits >> o) & 1ull) ? dm[o] * (1.0f / K) : 0.0f);
}

// Edge-layer weight gradient from the split-K partials part[split][64 (o)][16 (k)] of
// dZ^T E: rows k < FE of the gradient to gw[k][o], row FE (the bias) to gb[o].
__global__ void __launch_bounds__(kT) k_tc_reduce_edge(const float* __restrict__ part, int splits, float* __restrict__ gw,
                                                      float* __restrict__ gb) {
    const int t = blockIdx.x * kT + threadIdx.x;
    if (t >= (FE + 1) * W) return;
    const int k = t / W, o = t % W;
    float s = 0.0f;
    for (int q = 0; q < splits; ++q) s += part[((size_t)q * W + o) * 16 + k];
    if (k < FE) gw[k * W + o] = s;
    else gb[o] = s;
}

// Packed BF16 weights of the node layers, rebuilt whenever the parameters change:
//   forward  B operands [nout_pad][kin_pad] = W^T with the bias in column kin (the activations
//            carry a constant-1 column there);
//   backward B operands [kin_pad][nout_pad] = W (the data gradient dX = dY W^T).
constexpr int kTcK1 = 80, kTcK2 = 144, kTcKo = 80, kTcNo = 16;  // padded K of the node layers, N of the output
constexpr int kWfN1 = 0, kWfP = kWfN1 + W * kTcK1, kWfN2 = kWfP + W * W, kWfO = kWfN2 + W * kTcK2,
              kWfTotal = kWfO + kTcNo * kTcKo;
constexpr int kWbN1 = 0, kWbP = kWbN1 + kTcK1 * W, kWbN2 = kWbP + W * W, kWbO = kWbN2 + 2 * W * W,
              kWbTotal = kWbO + W * kTcNo;

__device__ __forceinline__ float wfwd(const float* prm, int woff, int boff, int kin, int nout, int o, int k) {
    if (o >= nout) return 0.0f;
    if (k < kin) return prm[woff + k * nout + o];
    return (k == kin && boff >= 0) ? prm[boff + o] : 0.0f;
}

__global__ void k_pack_weights(const float* __restrict__ prm, __nv_bfloat16* __restrict__ wf,
                               __nv_bfloat16* __restrict__ wb) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < kWfTotal) {
        float v;
        if (t < kWfP) { const int o = t / kTcK1, k = t % kTcK1; v = wfwd(prm, kWn1, kBn1, W + FN, W, o, k); }
        else if (t < kWfN2) { const int r = t - kWfP, o = r / W, k = r % W; v = wfwd(prm, kWp, -1, W, W, o, k); }
        else if (t < kWfO) { const int r = t - kWfN2, o = r / kTcK2, k = r % kTcK2; v = wfwd(prm, kWn2, kBn2, 2 * W, W, o, k); }
        else { const int r = t - kWfO, o = r / kTcKo, k = r % kTcKo; v = wfwd(prm, kWo, kBo, W, FO, o, k); }
        wf[t] = __float2bfloat16_rn(v);
    }
    if (t < kWbTotal) {
        float v;
        if (t < kWbP) { const int k = t / W, o = t % W; v = k < W + FN ? prm[kWn1 + k * W + o] : 0.0f; }
        else if (t < kWbN2) { const int r = t - kWbP; v = prm[kWp + r]; }
        else if (t < kWbO) { const int r = t - kWbN2; v = prm[kWn2 + r]; }
        else { const int r = t - kWbO, k = r / kTcNo, o = r % kTcNo; v = o < FO ? prm[kWo + k * FO + o] : 0.0f; }
        wb[t] = __float2bfloat16_rn(v);
    }
}

// Weight gradient from the split-K partials part[split][mpad][npad] of D = X^T dY: rows k < kin
// go to gw[k][nout], row kin (the constant-1 column) to gb, summed over the splits in order.
__global__ void __launch_bounds__(kT) k_tc_reduce(const float* __restrict__ part, int splits, int mpad, int npad,
                                                 int kin, int nout, float* __restrict__ gw, float* __restrict__ gb) {
    const int t = blockIdx.x * kT + threadIdx.x;
    const int rows = gb ? kin + 1 : kin;
    if (t >= rows * nout) return;
    const int k = t / nout, o = t % nout;
    float s = 0.0f;
    for (int q = 0; q < splits; ++q) s += part[((size_t)q * mpad + k) * npad + o];
    if (k < kin) gw[k * nout + o] = s;
    else gb[o] = s;
}

}  // namespace

// Workspace and passes of one training frame (up to n_max particles).
struct Trainer {
    int n_max = 0;
    float *prm = nullptr, *grad = nullptr, *adam_m = nullptr, *adam_v = nullptr;
    float *E = nullptr, *X1 = nullptr, *H1 = nullptr, *P = nullptr, *X2 = nullptr, *H2 = nullptr, *O = nullptr;
    float *dO = nullptr, *dY2 = nullptr, *dX2 = nullptr, *dZ2 = nullptr, *dP = nullptr, *dY1 = nullptr, *dX1 = nullptr;
    float* part = nullptr;
    double* loss_part = nullptr;
    unsigned long long *mask1 = nullptr, *mask2 = nullptr;
    int *rev_cnt = nullptr, *rev_off = nullptr, *rev_edges = nullptr;
    int splits = 64;
    // BF16 tensor-core path of the node layers (use_tc): row-major operands with the bias column,
    // transposed copies for the weight gradients (K = particles, padded to kpad), packed weights,
    // split-K partials and the GEMM's error word.
    bool use_tc = false;
    int kpad_max = 0;
    __nv_bfloat16 *X1b = nullptr, *H1b = nullptr, *X2b = nullptr, *H2b = nullptr;
    __nv_bfloat16 *dOb = nullptr, *dY2b = nullptr, *dPb = nullptr, *dY1b = nullptr;
    __nv_bfloat16 *X1bT = nullptr, *H1bT = nullptr, *X2bT = nullptr, *H2bT = nullptr;
    __nv_bfloat16 *dOT = nullptr, *dY2T = nullptr, *dPT = nullptr, *dY1T = nullptr;
    __nv_bfloat16 *Wf = nullptr, *Wb = nullptr;
    float* tpart = nullptr;
    uint32_t* tc_err = nullptr;
    static constexpr int kTcSplits = 128;
    // edge-layer weight gradients on the tensor cores: transposed edge operands, K = edges
    long long rpad_max = 0;
    __nv_bfloat16 *ET = nullptr, *dZT = nullptr;
    float* epart = nullptr;
    static constexpr int kEdgeSplits = 512;

    template <class T>
    static cudaError_t al(T** p, size_t n) { return cudaMalloc((void**)p, (n ? n : 1) * sizeof(T)); }

    // train = false allocates the forward pass only.
    cudaError_t init(int nmax, bool train) {
        n_max = nmax;
        const size_t n = (size_t)nmax, e = n * K;
        cudaError_t r = cudaSuccess;
        auto A = [&](cudaError_t x) { if (r == cudaSuccess) r = x; };
        A(al(&prm, kParams));
        A(al(&E, e * FE)); A(al(&X1, n * (W + FN))); A(al(&H1, n * W)); A(al(&P, n * W)); A(al(&X2, n * 2 * W));
        A(al(&H2, n * W)); A(al(&O, n * kOS)); A(al(&mask1, e)); A(al(&mask2, e));
        if (r == cudaSuccess) r = cudaMemset(O, 0, sizeof(float) * n * kOS);  // columns FO.. stay zero
        if (train) {
            A(al(&grad, kParams)); A(al(&adam_m, kParams)); A(al(&adam_v, kParams));
            A(al(&dO, n * kOS)); A(al(&dY2, n * W)); A(al(&dX2, n * 2 * W));
            A(al(&dZ2, e * W)); A(al(&dP, n * W)); A(al(&dY1, n * W)); A(al(&dX1, n * (W + FN)));
            A(al(&part, (size_t)splits * (2 * W + 1) * W)); A(al(&loss_part, (size_t)nblk(n) + 1));
            A(al(&rev_cnt, n)); A(al(&rev_off, n + 1)); A(al(&rev_edges, e));
            if (r == cudaSuccess) r = cudaMemset(adam_m, 0, sizeof(float) * kParams);
            if (r == cudaSuccess) r = cudaMemset(adam_v, 0, sizeof(float) * kParams);
        }
        // tensor-core path (forward operands always; transposed copies for training)
        kpad_max = (nmax + 63) / 64 * 64;
        const size_t kp = (size_t)kpad_max;
        A(al(&X1b, n * kTcK1)); A(al(&H1b, n * W)); A(al(&X2b, n * kTcK2)); A(al(&H2b, n * kTcKo));
        A(al(&Wf, (size_t)kWfTotal)); A(al(&Wb, (size_t)kWbTotal)); A(al(&tc_err, 1));
        if (r == cudaSuccess) r = cudaMemset(tc_err, 0, sizeof(uint32_t));
        if (train) {
            A(al(&dOb, n * kTcNo)); A(al(&dY2b, n * W)); A(al(&dPb, n * W)); A(al(&dY1b, n * W));
            A(al(&X1bT, kTcK1 * kp)); A(al(&H1bT, W * kp)); A(al(&X2bT, kTcK2 * kp)); A(al(&H2bT, kTcKo * kp));
            A(al(&dOT, kTcNo * kp)); A(al(&dY2T, W * kp)); A(al(&dPT, W * kp)); A(al(&dY1T, W * kp));
            A(al(&tpart, (size_t)kTcSplits * kTcK2 * W));
            rpad_max = ((long long)nmax * K + 63) / 64 * 64;
            A(al(&ET, (size_t)16 * rpad_max)); A(al(&dZT, (size_t)W * rpad_max));
            A(al(&epart, (size_t)kEdgeSplits * W * 16));
        }
        return r;
    }

    ~Trainer() {
        void* ptrs[] = {prm, grad, adam_m, adam_v, E, X1, H1, P, X2, H2, O, dO, dY2, dX2, dZ2, dP, dY1, dX1,
                        part, loss_part, mask1, mask2, rev_cnt, rev_off, rev_edges,
                        X1b, H1b, X2b, H2b, dOb, dY2b, dPb, dY1b, X1bT, H1bT, X2bT, H2bT, dOT, dY2T, dPT, dY1T,
                        Wf, Wb, tpart, tc_err, ET, dZT, epart};
        for (void* q : ptrs)
            if (q) cudaFree(q);
    }

    void dense(const float* X, int ldx, int kin, int woff, int boff, int nout, float* Y, int ldy, int n, int relu,
               cudaStream_t st) {
        k_dense_fwd<<<nblk((long long)n * nout), kT, 0, st>>>(X, ldx, kin, prm + woff, boff >= 0 ? prm + boff : nullptr,
                                                             nout, Y, ldy, n, relu);
    }

    void wgrad(const float* X, int ldx, int kin, const float* dY, int ldy, int nout, int n, int woff, int boff,
               cudaStream_t st) {
        const int rows = (n + splits - 1) / splits;
        const int total = (kin + 1) * nout;
        k_wgrad_partial<<<dim3(nblk(total), splits), kT, 0, st>>>(X, ldx, kin, dY, ldy, nout, n, rows, part);
        k_reduce_split<<<nblk(total), kT, 0, st>>>(part, splits, total, grad + woff, kin * nout,
                                                   boff >= 0 ? grad + boff : nullptr);
    }

    void edge_wgrad(const float* dZ, const float* dM, int ldm, const unsigned long long* mask, const int* cnt, int n,
                    int woff, int boff, cudaStream_t st) {
        const long long rows_total = (long long)n * K;
        const int rows = (int)((rows_total + splits - 1) / splits);
        const int total = (FE + 1) * W;
        k_edge_wgrad_partial<<<dim3(nblk(total), splits), kT, 0, st>>>(E, dZ, dM, ldm, mask, cnt, n, rows, part);
        k_reduce_split<<<nblk(total), kT, 0, st>>>(part, splits, total, grad + woff, FE * W, grad + boff);
    }

    // ---- tensor-core path ----------------------------------------------------------------
    static int kpad_of(int n) { return (n + 63) / 64 * 64; }

    // BF16 copies of src [n][lds] (ncols columns; bias_col = 1): row-major dst [n][ldd] and/or
    // the transposed dstT [ldd][kpad_max] (zero for particles n .. kpad - 1).
    void pack(const float* src, int lds, int ncols, int n, int bias_col, __nv_bfloat16* dst, int ldd,
              __nv_bfloat16* dstT, cudaStream_t st) {
        const int rows = dstT ? kpad_of(n) : n;
        const dim3 grid((unsigned)((rows + 31) / 32), (unsigned)((ldd + 31) / 32));
        k_pack_bf16<<<grid, 256, 0, st>>>(src, lds, ncols, n, kpad_of(n), bias_col, dst, ldd, dstT, kpad_max);
    }

    void tc_gemm(const __nv_bfloat16* A, int lda, const __nv_bfloat16* B, int ldb, int m, int nn, int k,
                 const tc::Epilogue& e, cudaStream_t st) {
        tc::gemm_bf16(A, lda, B, ldb, m, nn, k, e, 1, k, tc_err, st);
    }
    static tc::Epilogue epi(float* out, int ld, int ncols, int relu = 0) {
        tc::Epilogue e;
        e.out = out;
        e.ld_out = ld;
        e.ncols = ncols;
        e.relu = relu;
        return e;
    }

    // Weight gradient D = AT BT^T over the particles (AT [mpad][kpad_max], BT [npad][kpad_max],
    // K = kpad(n)), split over K and reduced in order into grad[woff] (rows < kin) and
    // grad[boff] (row kin).
    void tc_wgrad(const __nv_bfloat16* AT, int mpad, const __nv_bfloat16* BT, int npad, int n, int kin, int nout,
                  int woff, int boff, cudaStream_t st) {
        const int k = kpad_of(n);
        int kps = (k + kTcSplits - 1) / kTcSplits;
        kps = (kps + 63) / 64 * 64;
        const int sp = (k + kps - 1) / kps;
        tc::Epilogue e;
        e.out = tpart;
        e.ld_out = npad;
        e.ncols = npad;
        e.split_stride = (long long)mpad * npad;
        tc::gemm_bf16(AT, kpad_max, BT, kpad_max, mpad, npad, k, e, sp, kps, tc_err, st);
        const int rows = boff >= 0 ? kin + 1 : kin;
        k_tc_reduce<<<nblk((long long)rows * nout), kT, 0, st>>>(tpart, sp, mpad, npad, kin, nout, grad + woff,
                                                                boff >= 0 ? grad + boff : nullptr);
    }

    // Edge-layer weight gradient on the tensor cores: D^T = dZ^T E over the edges (M = 64
    // outputs, N = 16 features incl. the bias row, K = edges), split over K, reduced in order.
    // dX / ld: the data gradient whose first 64 columns are dM of this round; mask: its relu bits.
    void tc_edge_wgrad(const Frame& f, const float* dX, int ld, const unsigned long long* mask, int woff, int boff,
                       cudaStream_t st) {
        const long long r = (long long)f.n * K;
        const long long rpad = (r + 63) / 64 * 64;
        k_pack_dzt<<<(unsigned)((rpad + kT - 1) / kT), kT, 0, st>>>(dX, ld, mask, f.cnt, f.n, (int)rpad, dZT);
        long long kps = (rpad + kEdgeSplits - 1) / kEdgeSplits;
        kps = (kps + 63) / 64 * 64;
        const int sp = (int)((rpad + kps - 1) / kps);
        tc::Epilogue e;
        e.out = epart;
        e.ld_out = 16;
        e.ncols = 16;
        e.split_stride = (long long)W * 16;
        tc::gemm_bf16(dZT, (int)rpad, ET, (int)rpad, W, 16, (int)rpad, e, sp, (int)kps, tc_err, st);
        k_tc_reduce_edge<<<nblk((FE + 1) * W), kT, 0, st>>>(epart, sp, grad + woff, grad + boff);
    }

    void forward_tc(const Frame& f, bool train, cudaStream_t st) {
        const int n = f.n;
        k_pack_weights<<<nblk(kWfTotal), kT, 0, st>>>(prm, Wf, Wb);
        k_edge1_fwd<<<nblk((long long)n * kGrp), kT, 0, st>>>(f, prm, E, mask1, X1);
        if (train) {
            const long long rpad = ((long long)n * K + 63) / 64 * 64;
            k_pack_et<<<(unsigned)((rpad + kT - 1) / kT), kT, 0, st>>>(E, f.cnt, n, (int)rpad, ET);
        }
        pack(X1, W + FN, W + FN, n, W + FN, X1b, kTcK1, train ? X1bT : nullptr, st);
        tc_gemm(X1b, kTcK1, Wf + kWfN1, kTcK1, n, W, kTcK1, epi(H1, W, W, 1), st);
        pack(H1, W, W, n, -1, H1b, W, train ? H1bT : nullptr, st);
        tc_gemm(H1b, W, Wf + kWfP, W, n, W, W, epi(P, W, W), st);
        k_edge2_fwd<<<nblk((long long)n * kGrp), kT, 0, st>>>(f, prm, E, P, H1, mask2, X2);
        pack(X2, 2 * W, 2 * W, n, 2 * W, X2b, kTcK2, train ? X2bT : nullptr, st);
        tc_gemm(X2b, kTcK2, Wf + kWfN2, kTcK2, n, W, kTcK2, epi(H2, W, W, 1), st);
        pack(H2, W, W, n, W, H2b, kTcKo, train ? H2bT : nullptr, st);
        tc_gemm(H2b, kTcKo, Wf + kWfO, kTcKo, n, kTcNo, kTcKo, epi(O, kOS, FO), st);
    }

    void backward_tc(const Frame& f, cudaStream_t st) {
        const int n = f.n;
        k_loss<<<nblk(n), kT, 0, st>>>(O, f.target, n, dO, loss_part);
        pack(dO, kOS, FO, n, -1, dOb, kTcNo, dOT, st);
        tc_wgrad(H2bT, kTcKo, dOT, kTcNo, n, W, FO, kWo, kBo, st);
        {  // dY2 = (dO Wo^T) * (H2 > 0)
            tc::Epilogue e = epi(dY2, W, W);
            e.gate = H2;
            e.ld_gate = W;
            tc_gemm(dOb, kTcNo, Wb + kWbO, kTcNo, n, W, kTcNo, e, st);
        }
        pack(dY2, W, W, n, -1, dY2b, W, dY2T, st);
        tc_wgrad(X2bT, kTcK2, dY2T, W, n, 2 * W, W, kWn2, kBn2, st);
        tc_gemm(dY2b, W, Wb + kWbN2, W, n, 2 * W, W, epi(dX2, 2 * W, 2 * W), st);  // dX2 = dY2 Wn2^T
        tc_edge_wgrad(f, dX2, 2 * W, mask2, kWe2, kBe2, st);
        reverse_gather(f, st, true);
        pack(dP, W, W, n, -1, dPb, W, dPT, st);
        tc_wgrad(H1bT, W, dPT, W, n, W, W, kWp, -1, st);
        {  // dY1 = (dX2[:, W:] + dP Wp^T) * (H1 > 0)
            tc::Epilogue e = epi(dY1, W, W);
            e.add = dX2 + W;
            e.ld_add = 2 * W;
            e.gate = H1;
            e.ld_gate = W;
            tc_gemm(dPb, W, Wb + kWbP, W, n, W, W, e, st);
        }
        pack(dY1, W, W, n, -1, dY1b, W, dY1T, st);
        tc_wgrad(X1bT, kTcK1, dY1T, W, n, W + FN, W, kWn1, kBn1, st);
        tc_gemm(dY1b, W, Wb + kWbN1, W, n, kTcK1, W, epi(dX1, W + FN, W + FN), st);  // dX1 = dY1 Wn1^T
        tc_edge_wgrad(f, dX1, W + FN, mask1, kWe1, kBe1, st);
    }

    // dP from the reverse edges: from the materialised dZ2, or (masked) from dX2 and the relu bits.
    void reverse_gather(const Frame& f, cudaStream_t st, bool masked = false) {
        const int n = f.n;
        cudaMemsetAsync(rev_cnt, 0, sizeof(int) * n, st);
        k_rev_count<<<nblk((long long)n * K), kT, 0, st>>>(f.nb, f.cnt, n, rev_cnt);
        k_scan_small<<<1, 1024, 0, st>>>(rev_cnt, n, rev_off);
        cudaMemsetAsync(rev_cnt, 0, sizeof(int) * n, st);
        k_rev_fill<<<nblk((long long)n * K), kT, 0, st>>>(f.nb, f.cnt, n, rev_off, rev_cnt, rev_edges);
        k_rev_sort<<<nblk(n), kT, 0, st>>>(rev_off, n, rev_edges);
        if (masked)
            k_rev_gather_masked<<<nblk((long long)n * W), kT, 0, st>>>(rev_off, rev_edges, dX2, mask2, n, dP);
        else
            k_rev_gather<<<nblk((long long)n * W), kT, 0, st>>>(rev_off, rev_edges, dZ2, n, dP);
    }

    // Forward: O (n x kOS) from the frame.
    void forward(const Frame& f, cudaStream_t st) {
        if (use_tc) {
            forward_tc(f, grad != nullptr, st);
            return;
        }
        const int n = f.n;
        k_edge1_fwd<<<nblk((long long)n * kGrp), kT, 0, st>>>(f, prm, E, mask1, X1);
        dense(X1, W + FN, W + FN, kWn1, kBn1, W, H1, W, n, 1, st);
        dense(H1, W, W, kWp, -1, W, P, W, n, 0, st);
        k_edge2_fwd<<<nblk((long long)n * kGrp), kT, 0, st>>>(f, prm, E, P, H1, mask2, X2);
        dense(X2, 2 * W, 2 * W, kWn2, kBn2, W, H2, W, n, 1, st);
        dense(H2, W, W, kWo, kBo, FO, O, kOS, n, 0, st);
    }

    // Loss partials and the full parameter gradient (forward must have run).
    void backward(const Frame& f, cudaStream_t st) {
        if (use_tc) {
            backward_tc(f, st);
            return;
        }
        const int n = f.n;
        k_loss<<<nblk(n), kT, 0, st>>>(O, f.target, n, dO, loss_part);
        wgrad(H2, W, W, dO, kOS, FO, n, kWo, kBo, st);
        k_dense_bwd_data<<<nblk((long long)n * W), kT, 0, st>>>(dO, kOS, FO, prm + kWo, W, nullptr, 0, H2, W, dY2, W, n);
        wgrad(X2, 2 * W, 2 * W, dY2, W, W, n, kWn2, kBn2, st);
        k_dense_bwd_data<<<nblk((long long)n * 2 * W), kT, 0, st>>>(dY2, W, W, prm + kWn2, 2 * W, nullptr, 0, nullptr,
                                                                    0, dX2, 2 * W, n);
        k_edge2_bwd<<<nblk((long long)n * K * W), kT, 0, st>>>(dX2, mask2, f.cnt, n, dZ2);
        edge_wgrad(dZ2, nullptr, 0, nullptr, f.cnt, n, kWe2, kBe2, st);
        reverse_gather(f, st);
        wgrad(H1, W, W, dP, W, W, n, kWp, -1, st);
        // dY1 = (dX2[:, W:] + dP Wp^T) * (H1 > 0)
        k_dense_bwd_data<<<nblk((long long)n * W), kT, 0, st>>>(dP, W, W, prm + kWp, W, dX2 + W, 2 * W, H1, W, dY1, W,
                                                                n);
        wgrad(X1, W + FN, W + FN, dY1, W, W, n, kWn1, kBn1, st);
        k_dense_bwd_data<<<nblk((long long)n * (W + FN)), kT, 0, st>>>(dY1, W, W, prm + kWn1, W + FN, nullptr, 0,
                                                                        nullptr, 0, dX1, W + FN, n);
        edge_wgrad(nullptr, dX1, W + FN, mask1, f.cnt, n, kWe1, kBe1, st);
    }

    void adam(int t, float lr, cudaStream_t st) {
        const float b1 = 0.9f, b2 = 0.999f;
        const float c1 = (float)(1.0 / (1.0 - std::pow((double)b1, t)));
        const float c2 = (float)(1.0 / (1.0 - std::pow((double)b2, t)));
        k_adam<<<nblk(kParams), kT, 0, st>>>(prm, grad, adam_m, adam_v, kParams, lr, b1, b2, 1e-8f, c1, c2);
    }

    double loss(int n, cudaStream_t st) {
        std::vector<double> h(nblk(n));
        cudaMemcpyAsync(h.data(), loss_part, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, st);
        cudaStreamSynchronize(st);
        double s = 0.0;
        for (double x : h) s += x;
        return s / (double)n;
    }
};

Trainer* trainer_new(int n_max, bool train) {
    Trainer* t = new Trainer;
    if (t->init(n_max, train) != cudaSuccess) {
        delete t;
        return nullptr;
    }
    return t;
}
void trainer_delete(Trainer* t) { delete t; }
float* trainer_params(Trainer* t) { return t->prm; }
float* trainer_grad(Trainer* t) { return t->grad; }
float* trainer_out(Trainer* t) { return t->O; }
void trainer_reset_adam(Trainer* t) {
    if (t->adam_m) cudaMemset(t->adam_m, 0, sizeof(float) * kParams);
    if (t->adam_v) cudaMemset(t->adam_v, 0, sizeof(float) * kParams);
}
int trainer_capacity(Trainer* t) { return t->n_max; }
void trainer_set_tc(Trainer* t, bool on) { t->use_tc = on; }
bool trainer_tc(Trainer* t) { return t->use_tc; }
uint32_t trainer_tc_error(Trainer* t, cudaStream_t st) {
    uint32_t e = 0;
    cudaMemcpyAsync(&e, t->tc_err, sizeof(e), cudaMemcpyDeviceToHost, st);
    cudaStreamSynchronize(st);
    if (e) cudaMemsetAsync(t->tc_err, 0, sizeof(e), st);
    return e;
}
void trainer_forward(Trainer* t, const Frame& f, cudaStream_t st) { t->forward(f, st); }
double trainer_loss_grad(Trainer* t, const Frame& f, cudaStream_t st) {
    t->forward(f, st);
    t->backward(f, st);
    return t->loss(f.n, st);
}
void trainer_adam(Trainer* t, int step, float lr, cudaStream_t st) { t->adam(step, lr, st); }

}  // namespace mpnn
}  // namespace sphgb
