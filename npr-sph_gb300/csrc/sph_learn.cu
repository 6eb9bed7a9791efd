// sph_learn.cu -- the learned macro-step behind the C ABI (no counterpart in
// the reference): neighbour lists and density, frame recording from the SPH
// step itself, the training loop, the macro-step (4*dt per network pass) and
// the plain-SPH judge that takes over when the learned state drifts.
//
// Macro-step on a context (single scene):
//   sort -> neighbours+density -> network -> update
//   v' = v + 4 dt A O_v,  x' = x + 4 dt v + 10 dt^2 A O_x  (A = k/h; the exact
//   result of 4 symplectic sub-steps when O holds the sub-steps' mean
//   accelerations), then the wall clamp of integrate_comp.glsl:45-77 with the
//   damping, then the cell hash.
// Judge (every judge_every macro-steps): from the same state, one learned
// macro-step and 4 plain steps; the density deviation between the two results
// (of the mean density, or per particle: sph_learned_set_judge) and their
// momentum difference decide. Above the bounds the interval is rolled back and
// run by plain SPH.
#include <cmath>
#include <cstring>
#include <random>
#include <string>
#include <vector>

#include "sph_ctx.h"
#include "sph_device.cuh"
#include "sph_mpnn.h"
#include <cuda_bf16.h>

using namespace sphgb;
using sphgb::engine::fail;
namespace M = sphgb::mpnn;

struct sph_mpnn {
    int device = 0;
    std::string err;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    M::Trainer* tr = nullptr;   // training workspace (frames up to n_frame particles)
    M::Trainer* inf = nullptr;  // forward-only workspace for a context (grown on demand)
    struct Rec {
        void* arena = nullptr;
        M::Frame f{};
    };
    std::vector<Rec> frames;
    // context-sized scratch
    int cap = 0;
    int *nb = nullptr, *cnt = nullptr;
    float4 *snap_pos = nullptr, *snap_vel = nullptr, *l_pos = nullptr, *l_vel = nullptr, *acc = nullptr,
           *accx = nullptr, *ck_pos = nullptr, *ck_vel = nullptr;
    float2* ck_rhop = nullptr;
    float2 *snap_rhop = nullptr, *l_rhop = nullptr;
    float *rho_l = nullptr, *rho_p = nullptr;
    float* Obuf = nullptr;    // [n][kOS] network outputs of a macro-step
    double* osum = nullptr;   // [kSumBlocks][FO] partial sums of the outputs
    float* ocorr = nullptr;   // [FO] momentum projection added to every output
    float4 *vel_l = nullptr, *vel_p = nullptr;
    double* cmp = nullptr;
    // host-frame scratch (sph_mpnn_loss_grad)
    int hcap = 0;
    void* harena = nullptr;
    int adam_t = 0;  // Adam steps taken since the parameters were last set
    // BF16 tensor-core inference
    int precision = 3;               // inference: 3 BF16 tcgen05 round 1 (features on the TMEM lanes) +
                                     // mma.sync round 2 (default), 1 BF16 mma.sync, 2 BF16 tcgen05, 0 FP32
    int train_precision = 1;         // training node layers: 1 BF16 tcgen05 GEMMs (default), 0 FP32
    uint32_t* frags = nullptr;       // parameters in MMA fragment order (mma.sync kernels)
    __nv_bfloat16* tcw = nullptr;    // parameters as tcgen05 shared-memory images
    uint32_t* tc_err = nullptr;      // bit 0: a tensor-core wait of the inference timed out
    bool frags_dirty = true;
    __nv_bfloat16* H1b = nullptr;    // [n][64]
    uint16_t* Pperm = nullptr;       // [n][64], permuted
    int bcap = 0;
};

namespace {

constexpr int kT = 128;
inline int nblk(long long n, int t = kT) { return (int)((n + t - 1) / t); }

#define NCK(call)                                                                              \
    do {                                                                                       \
        cudaError_t e_ = (call);                                                               \
        if (e_ != cudaSuccess) {                                                               \
            net->err = std::string(#call) + ": " + cudaGetErrorString(e_);                     \
            return e_ == cudaErrorMemoryAllocation ? SPH_ERR_OUT_OF_MEMORY : SPH_ERR_CUDA;     \
        }                                                                                      \
    } while (0)

// ---- kernels ------------------------------------------------------------------------------

static_assert(M::K == kNbList, "the network reads the neighbour lists of launch_density_nb");

constexpr int kSumBlocks = 1024;

// Momentum projection, step 1: partial sums of the outputs, per thread in FP32 over its few rows
// (two 16-byte loads per 32-byte row), per block in FP64 (fixed order: deterministic).
__global__ void __launch_bounds__(kT) k_out_partial(const float* __restrict__ O, int n, double* __restrict__ part) {
    static_assert(M::kOS == 8 && M::FO <= 8, "an output row is two float4");
    __shared__ double sh[M::FO][kT];
    float a[M::FO] = {};
    for (int i = blockIdx.x * kT + threadIdx.x; i < n; i += gridDim.x * kT) {
        const float4* row = reinterpret_cast<const float4*>(O + (size_t)i * M::kOS);
        const float4 r0 = __ldg(row), r1 = __ldg(row + 1);
        const float v[8] = {r0.x, r0.y, r0.z, r0.w, r1.x, r1.y, r1.z, r1.w};
#pragma unroll
        for (int q = 0; q < M::FO; ++q) a[q] += v[q];
    }
#pragma unroll
    for (int q = 0; q < M::FO; ++q) sh[q][threadIdx.x] = (double)a[q];
    __syncthreads();
    for (int o = kT / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o)
#pragma unroll
            for (int q = 0; q < M::FO; ++q) sh[q][threadIdx.x] += sh[q][threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x < M::FO) part[blockIdx.x * M::FO + threadIdx.x] = sh[threadIdx.x][0];
}

// Step 2: the shift that makes the mean of each head G/A. Pressure and viscosity forces are
// pairwise antisymmetric (force_comp.glsl:59-60 with m_i = m_j), so over all particles the
// sum of m a over the 4 sub-steps is N m G exactly: both target heads average G/A. One block
// sums the partials in a fixed-order FP64 tree.
__global__ void __launch_bounds__(kT) k_out_corr(const double* __restrict__ part, int blocks, int n, SceneDev S,
                                                 float* __restrict__ corr) {
    __shared__ double sh[M::FO][kT];
    double a[M::FO] = {};
    for (int b = threadIdx.x; b < blocks; b += kT)
#pragma unroll
        for (int q = 0; q < M::FO; ++q) a[q] += part[b * M::FO + q];
#pragma unroll
    for (int q = 0; q < M::FO; ++q) sh[q][threadIdx.x] = a[q];
    __syncthreads();
    for (int o = kT / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o)
#pragma unroll
            for (int q = 0; q < M::FO; ++q) sh[q][threadIdx.x] += sh[q][threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x < M::FO) {
        const int q = threadIdx.x;
        const double ga = (double)S.g[q % 3] * (double)S.h / (double)S.gas_k;
        corr[q] = (float)(ga - sh[q][0] / (double)n);
    }
}

// Macro-step update from the network outputs O plus the projection corr, fused with the hash.
__global__ void __launch_bounds__(kT) k_macro_integrate(const float4* __restrict__ pos_s, const float4* __restrict__ vel_s,
                                                       const float* __restrict__ O, const float* __restrict__ corr,
                                                       SceneDev S, float4* __restrict__ pos_out,
                                                       float4* __restrict__ vel_out, int* __restrict__ key_out,
                                                       int* __restrict__ rank_out, int* __restrict__ count, int n) {
    const int t = blockIdx.x * kT + threadIdx.x;
    if (t >= n) return;
    float4 np, nv;
    const float* o = O + (size_t)t * M::kOS;
    M::macro_update(S, o[0] + corr[0], o[1] + corr[1], o[2] + corr[2], o[3] + corr[3], o[4] + corr[4],
                    o[5] + corr[5], pos_s[t], vel_s[t], np, nv);
    if (S.sdf) {  // the static obstacle's rule, after the wall clamp as in the plain step
        float x[3] = {np.x, np.y, np.z}, u[3] = {nv.x, nv.y, nv.z};
        obstacle_response(S, x, u);
        np = make_float4(x[0], x[1], x[2], np.w);
        nv = make_float4(u[0], u[1], u[2], nv.w);
    }
    pos_out[t] = np;
    vel_out[t] = nv;
    const int k = cell_key(S, np.x, np.y, np.z);
    key_out[t] = k;
    rank_out[t] = atomicAdd(&count[k], 1);
}

// After plain sub-step `sub` (0..3, slot order of that step): acc[id] += a and
// accx[id] += (4 - sub) a, with a = F / rho.
__global__ void __launch_bounds__(kT) k_accum_accel(const float4* __restrict__ vel, const float4* __restrict__ force_s,
                                                   const float2* __restrict__ rhop, int n, float wx,
                                                   float4* __restrict__ acc, float4* __restrict__ accx) {
    const int s = blockIdx.x * kT + threadIdx.x;
    if (s >= n) return;
    const int id = id_of(vel[s]);
    if (id < 0 || id >= n) return;
    const float4 f = force_s[s];
    const float ir = 1.0f / rhop[s].x;
    const float ax = f.x * ir, ay = f.y * ir, az = f.z * ir;
    float4 a = acc[id], b = accx[id];
    a.x += ax; a.y += ay; a.z += az;
    b.x += wx * ax; b.y += wx * ay; b.z += wx * az;
    acc[id] = a;
    accx[id] = b;
}

// Frame arrays of one scene from the sorted state: neighbour slots made frame-local.
__global__ void __launch_bounds__(kT) k_frame_copy(const float4* __restrict__ pos_s, const float4* __restrict__ vel_s,
                                                  const float2* __restrict__ rhop, const int* __restrict__ nb,
                                                  const int* __restrict__ cnt, int first, int m, float4* __restrict__ fpos,
                                                  float4* __restrict__ fvel, float2* __restrict__ frhop,
                                                  int* __restrict__ fnb, int* __restrict__ fcnt, int* __restrict__ fid) {
    const int k = blockIdx.x * kT + threadIdx.x;
    if (k >= m) return;
    const int s = first + k;
    fpos[k] = pos_s[s];
    fvel[k] = vel_s[s];
    frhop[k] = rhop[s];
    fid[k] = id_of(vel_s[s]);
    const int c = min(max(cnt[s], 0), M::K);
    int w = 0;  // neighbours are in the same scene; anything else is dropped, never passed on
    for (int q = 0; q < c; ++q) {
        const int j = nb[(size_t)s * M::K + q];
        if (j >= first && j < first + m) fnb[(size_t)k * M::K + w++] = j - first;
    }
    for (int q = w; q < M::K; ++q) fnb[(size_t)k * M::K + q] = -1;
    fcnt[k] = w;
}

// Targets of one frame: O_v = sum a / (4A), O_x = sum (4 - s) a / (10A) (inv_a = 1/A).
__global__ void __launch_bounds__(kT) k_frame_target(const int* __restrict__ fid, const float4* __restrict__ acc,
                                                    const float4* __restrict__ accx, int m, float inv_a,
                                                    float* __restrict__ target) {
    const int k = blockIdx.x * kT + threadIdx.x;
    if (k >= m) return;
    const float4 a = acc[fid[k]], b = accx[fid[k]];
    const float sv = 0.25f * inv_a, sx = 0.1f * inv_a;
    float4* row = reinterpret_cast<float4*>(target + (size_t)k * M::kOS);
    row[0] = make_float4(a.x * sv, a.y * sv, a.z * sv, b.x * sx);
    row[1] = make_float4(b.y * sx, b.z * sx, 0.0f, 0.0f);
}

// Density and velocity by particle id (slot order -> id order).
__global__ void __launch_bounds__(kT) k_by_id(const float4* __restrict__ vel, const float2* __restrict__ rhop, int n,
                                             float* __restrict__ rho_id, float4* __restrict__ vel_id) {
    const int s = blockIdx.x * kT + threadIdx.x;
    if (s >= n) return;
    const float4 v = vel[s];
    const int id = id_of(v);
    if (id < 0 || id >= n) return;
    rho_id[id] = rhop[s].x;
    vel_id[id] = v;
}

// Neighbour lists (sorted slots) to particle ids, by particle id, with the count and density.
__global__ void __launch_bounds__(kT) k_lists_by_id(const float4* __restrict__ vel_s, const int* __restrict__ nb,
                                                   const int* __restrict__ cnt, const float2* __restrict__ rhop, int n,
                                                   int* __restrict__ nb_id, int* __restrict__ cnt_id,
                                                   float* __restrict__ rho_id) {
    const int s = blockIdx.x * kT + threadIdx.x;
    if (s >= n) return;
    const int id = id_of(vel_s[s]);
    if (id < 0 || id >= n) return;
    const int c = min(max(cnt[s], 0), M::K);
    for (int q = 0; q < M::K; ++q) {
        const int j = q < c ? nb[(size_t)s * M::K + q] : -1;
        nb_id[(size_t)id * M::K + q] = (j >= 0 && j < n) ? id_of(vel_s[j]) : -1;
    }
    cnt_id[id] = c;
    rho_id[id] = rhop[s].x;
}

// FP64 partials of the judge: sum |rho_l - rho_p| / rho_p, sum (v_l - v_p) (3), sum |v_p|,
// sum rho_l, sum rho_p, max rho_l, max rho_p (fields 7 and 8 combine by max).
constexpr int kCmpFields = 9;
__global__ void __launch_bounds__(kT) k_compare(const float* __restrict__ rl, const float* __restrict__ rp,
                                               const float4* __restrict__ vl, const float4* __restrict__ vp, int n,
                                               double* __restrict__ out) {
    __shared__ double sh[kCmpFields][kT];
    double a[kCmpFields] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int i = blockIdx.x * kT + threadIdx.x; i < n; i += gridDim.x * kT) {
        a[0] += fabs((double)rl[i] - (double)rp[i]) / (double)rp[i];
        a[1] += (double)vl[i].x - (double)vp[i].x;
        a[2] += (double)vl[i].y - (double)vp[i].y;
        a[3] += (double)vl[i].z - (double)vp[i].z;
        a[4] += sqrt((double)vp[i].x * vp[i].x + (double)vp[i].y * vp[i].y + (double)vp[i].z * vp[i].z);
        a[5] += (double)rl[i];
        a[6] += (double)rp[i];
        a[7] = fmax(a[7], (double)rl[i]);
        a[8] = fmax(a[8], (double)rp[i]);
    }
    for (int f = 0; f < kCmpFields; ++f) sh[f][threadIdx.x] = a[f];
    __syncthreads();
    for (int o = kT / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o)
            for (int f = 0; f < kCmpFields; ++f)
                sh[f][threadIdx.x] = f >= 7 ? fmax(sh[f][threadIdx.x], sh[f][threadIdx.x + o])
                                            : sh[f][threadIdx.x] + sh[f][threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0)
        for (int f = 0; f < kCmpFields; ++f) out[blockIdx.x * kCmpFields + f] = sh[f][0];
}

constexpr int kCmpBlocks = 256;

M::FrameConst frame_const(const SceneDev& S, float visc) {
    M::FrameConst fc;
    const double PI = 3.141592741f, h = S.h;
    fc.h = S.h;
    fc.c = (float)std::sqrt((double)S.gas_k);
    fc.rho_self = (float)((double)S.mass * 315.0 / (64.0 * PI * h * h * h));
    fc.rho0 = S.rho0;
    fc.log_mu = (float)(std::log10((double)visc) / 4.0);
    fc.courant = (float)(std::sqrt((double)S.gas_k) * (double)S.dt / h);
    return fc;
}

// Neighbour lists and density of the sorted state of a context.
void launch_nb_density(sph_ctx* ctx, int* nb, int* cnt) {
    launch_density_nb(ctx->b, ctx->s0, ctx->batched, ctx->cfg, nb, cnt, ctx->stream);
}

template <class T>
cudaError_t dal(T** p, size_t n) {
    if (*p) cudaFree(*p);
    *p = nullptr;
    return cudaMalloc((void**)p, (n ? n : 1) * sizeof(T));
}

sph_status ensure_ctx_scratch(sph_mpnn* net, int n) {
    if (n <= net->cap) return SPH_OK;
    const size_t m = (size_t)n;
    NCK(dal(&net->nb, m * M::K)); NCK(dal(&net->cnt, m));
    NCK(dal(&net->snap_pos, m)); NCK(dal(&net->snap_vel, m)); NCK(dal(&net->snap_rhop, m));
    NCK(dal(&net->ck_pos, m)); NCK(dal(&net->ck_vel, m)); NCK(dal(&net->ck_rhop, m));
    NCK(dal(&net->l_pos, m)); NCK(dal(&net->l_vel, m)); NCK(dal(&net->l_rhop, m));
    NCK(dal(&net->acc, m)); NCK(dal(&net->accx, m)); NCK(dal(&net->rho_l, m)); NCK(dal(&net->rho_p, m));
    NCK(dal(&net->vel_l, m)); NCK(dal(&net->vel_p, m)); NCK(dal(&net->cmp, (size_t)kCmpBlocks * kCmpFields));
    NCK(dal(&net->Obuf, m * M::kOS)); NCK(dal(&net->osum, (size_t)kSumBlocks * M::FO)); NCK(dal(&net->ocorr, M::FO));
    net->cap = n;
    return SPH_OK;
}

// Density at the current positions; the sorted copy becomes the state (so rhop lines up with it).
sph_status refresh_density(sph_ctx* ctx) {
    engine::sort_state(ctx);
    launch_density(ctx->b, ctx->s0, ctx->batched, ctx->cfg, false, ctx->stream);
    const size_t n = (size_t)ctx->b.n;
    cudaMemcpyAsync(ctx->b.pos, ctx->b.pos_s, n * sizeof(float4), cudaMemcpyDeviceToDevice, ctx->stream);
    cudaMemcpyAsync(ctx->b.vel, ctx->b.vel_s, n * sizeof(float4), cudaMemcpyDeviceToDevice, ctx->stream);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(ctx, SPH_ERR_CUDA, std::string("density refresh: ") + cudaGetErrorString(e));
    return SPH_OK;
}

// Device staging of one host frame (sph_mpnn_loss_grad, sph_mpnn_forward): pos, vel, target /
// output rows, rhop, cnt, nb.
cudaError_t ensure_host_arena(sph_mpnn* net, uint32_t n) {
    if ((int)n <= net->hcap) return cudaSuccess;
    if (net->harena) cudaFree(net->harena);
    net->harena = nullptr;
    net->hcap = 0;
    const size_t bytes = (size_t)n * (16 + 16 + 4 * M::kOS + 8 + 4) + (size_t)n * M::K * 4;
    const cudaError_t e = cudaMalloc(&net->harena, bytes);
    if (e == cudaSuccess) net->hcap = (int)n;
    return e;
}

// Fragment-ordered parameters and the BF16 activations for n particles.
sph_status ensure_bf16(sph_mpnn* net, int n, cudaStream_t st) {
    if (!net->frags) {
        NCK(cudaMalloc(&net->frags, sizeof(uint32_t) * M::infer_frag_words()));
        NCK(cudaMalloc(&net->tcw, sizeof(__nv_bfloat16) * M::tc_infer_words()));
        NCK(cudaMalloc(&net->tc_err, sizeof(uint32_t)));
        NCK(cudaMemsetAsync(net->tc_err, 0, sizeof(uint32_t), st));
        net->frags_dirty = true;
    }
    if (n > net->bcap) {
        if (net->H1b) cudaFree(net->H1b);
        if (net->Pperm) cudaFree(net->Pperm);
        net->H1b = nullptr;
        net->Pperm = nullptr;
        NCK(cudaMalloc(&net->H1b, sizeof(__nv_bfloat16) * (size_t)n * M::W));
        NCK(cudaMalloc(&net->Pperm, sizeof(uint16_t) * (size_t)n * M::W));
        net->bcap = n;
    }
    if (net->frags_dirty) {
        M::infer_prep(M::trainer_params(net->tr), net->frags, st);
        M::tc_infer_prep(M::trainer_params(net->tr), net->tcw, st);
        net->frags_dirty = false;
    }
    return SPH_OK;
}

// One learned macro-step on ctx (4*dt).
sph_status learned_macro(sph_ctx* ctx, sph_mpnn* net) {
    const int n = ctx->b.n;
    engine::sort_state(ctx);
    launch_nb_density(ctx, net->nb, net->cnt);
    M::Frame f{ctx->b.pos_s, ctx->b.vel_s, ctx->b.rhop, net->nb, net->cnt, nullptr, n,
               frame_const(ctx->s0, ctx->params[0].visc)};
    const float* O = nullptr;
    if (net->precision == 2) {
        M::tc_infer_round1(f, net->tcw, net->H1b, reinterpret_cast<__half*>(net->Pperm), net->tc_err, ctx->stream);
        M::tc_infer_round2(f, net->tcw, net->H1b, reinterpret_cast<const __half*>(net->Pperm), net->Obuf, net->tc_err,
                           ctx->stream);
        O = net->Obuf;
    } else if (net->precision == 3) {
        M::tc_infer_round1_lanes(f, net->tcw, net->H1b, net->Pperm, net->tc_err, ctx->stream);
        M::infer_round2(f, net->frags, M::trainer_params(net->tr), net->H1b, net->Pperm, ctx->s0, nullptr, nullptr,
                        net->Obuf, nullptr, nullptr, nullptr, false, ctx->stream);
        O = net->Obuf;
    } else if (net->precision == 1) {
        M::infer_round1(f, net->frags, net->H1b, net->Pperm, ctx->stream);
        M::infer_round2(f, net->frags, M::trainer_params(net->tr), net->H1b, net->Pperm, ctx->s0, nullptr, nullptr,
                        net->Obuf, nullptr, nullptr, nullptr, false, ctx->stream);
        O = net->Obuf;
    } else {
        M::trainer_forward(net->inf, f, ctx->stream);
        O = M::trainer_out(net->inf);
    }
    // momentum projection, then the update
    k_out_partial<<<kSumBlocks, kT, 0, ctx->stream>>>(O, n, net->osum);
    k_out_corr<<<1, kT, 0, ctx->stream>>>(net->osum, kSumBlocks, n, ctx->s0, net->ocorr);
    k_macro_integrate<<<nblk(n), kT, 0, ctx->stream>>>(ctx->b.pos_s, ctx->b.vel_s, O, net->ocorr, ctx->s0, ctx->b.pos,
                                                       ctx->b.vel, ctx->b.key, ctx->b.rank, ctx->b.count, n);
    ctx->need_hash = false;  // the integrate hashed the new positions
    ctx->steps += 4;
    ctx->stepped = true;
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(ctx, SPH_ERR_CUDA, std::string("learned macro-step: ") + cudaGetErrorString(e));
    return SPH_OK;
}

void copy_state(sph_ctx* ctx, float4* dp, float4* dv, float2* dr, const float4* sp, const float4* sv, const float2* sr) {
    const size_t n = (size_t)ctx->b.n;
    cudaMemcpyAsync(dp, sp, n * sizeof(float4), cudaMemcpyDeviceToDevice, ctx->stream);
    cudaMemcpyAsync(dv, sv, n * sizeof(float4), cudaMemcpyDeviceToDevice, ctx->stream);
    cudaMemcpyAsync(dr, sr, n * sizeof(float2), cudaMemcpyDeviceToDevice, ctx->stream);
}

// A saved state of a context: the particles and the step count. Restoring it re-hashes at the
// next sort (the cell counts of whatever the integrate hashed last are cleared).
struct Saved {
    float4* pos;
    float4* vel;
    float2* rhop;
    uint64_t steps;
};

Saved save_state(sph_ctx* ctx, float4* p, float4* v, float2* r) {
    copy_state(ctx, p, v, r, ctx->b.pos, ctx->b.vel, ctx->b.rhop);
    return Saved{p, v, r, ctx->steps};
}

void restore_state(sph_ctx* ctx, const Saved& s) {
    copy_state(ctx, ctx->b.pos, ctx->b.vel, ctx->b.rhop, s.pos, s.vel, s.rhop);
    cudaMemsetAsync(ctx->b.count, 0, sizeof(int) * (size_t)ctx->b.ncell, ctx->stream);
    ctx->need_hash = true;
    ctx->steps = s.steps;
}

// One judged macro-step from the current state: a learned macro-step and 4 plain steps, both
// from that state, compared by particle id. Returns the mean relative density deviation and
// the momentum difference; the learned result is left in (l_pos, l_vel, l_rhop) and the plain
// one in the context.
sph_status judge_macro(sph_ctx* ctx, sph_mpnn* net, double& dev, double& mom, double& mdev, double& xdev) {
    const int n = ctx->b.n;
    const Saved s0 = save_state(ctx, net->snap_pos, net->snap_vel, net->snap_rhop);
    if (!ctx->need_hash) cudaMemsetAsync(ctx->b.count, 0, sizeof(int) * (size_t)ctx->b.ncell, ctx->stream);
    ctx->need_hash = true;
    sph_status st = learned_macro(ctx, net);
    if (!st) st = refresh_density(ctx);
    if (st) return st;
    k_by_id<<<nblk(n), kT, 0, ctx->stream>>>(ctx->b.vel, ctx->b.rhop, n, net->rho_l, net->vel_l);
    copy_state(ctx, net->l_pos, net->l_vel, net->l_rhop, ctx->b.pos, ctx->b.vel, ctx->b.rhop);
    restore_state(ctx, s0);
    st = engine::run_steps(ctx, 4);
    if (!st) st = refresh_density(ctx);
    if (st) return st;
    k_by_id<<<nblk(n), kT, 0, ctx->stream>>>(ctx->b.vel, ctx->b.rhop, n, net->rho_p, net->vel_p);
    k_compare<<<kCmpBlocks, kT, 0, ctx->stream>>>(net->rho_l, net->rho_p, net->vel_l, net->vel_p, n, net->cmp);
    std::vector<double> h((size_t)kCmpBlocks * kCmpFields);
    if (cudaMemcpyAsync(h.data(), net->cmp, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, ctx->stream) ||
        cudaStreamSynchronize(ctx->stream))
        return fail(ctx, SPH_ERR_CUDA, "judge readback");
    double sum[kCmpFields] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int b = 0; b < kCmpBlocks; ++b)
        for (int f = 0; f < kCmpFields; ++f) {
            const double x = h[(size_t)b * kCmpFields + f];
            sum[f] = f >= 7 ? std::max(sum[f], x) : sum[f] + x;
        }
    dev = sum[0] / n;
    mdev = sum[6] > 0.0 ? std::fabs(sum[5] - sum[6]) / sum[6] : INFINITY;
    xdev = sum[8] > 0.0 ? std::fabs(sum[7] - sum[8]) / sum[8] : INFINITY;
    const double g = std::sqrt((double)ctx->s0.g[0] * ctx->s0.g[0] + (double)ctx->s0.g[1] * ctx->s0.g[1] +
                               (double)ctx->s0.g[2] * ctx->s0.g[2]);
    mom = std::sqrt(sum[1] * sum[1] + sum[2] * sum[2] + sum[3] * sum[3]) / (sum[4] + n * g * 4.0 * ctx->s0.dt);
    return SPH_OK;
}

}  // namespace

extern "C" {

uint32_t sph_mpnn_num_params(void) { return (uint32_t)M::kParams; }

sph_status sph_mpnn_create(uint32_t n_frame, void* stream, sph_mpnn** out) {
    if (!out || n_frame == 0 || n_frame > (1u << 22)) return SPH_ERR_INVALID_ARG;
    *out = nullptr;
    sph_mpnn* net = new (std::nothrow) sph_mpnn;
    if (!net) return SPH_ERR_OUT_OF_MEMORY;
    if (cudaGetDevice(&net->device) != cudaSuccess) { delete net; return SPH_ERR_CUDA; }
    if (stream) net->stream = (cudaStream_t)stream;
    else if (cudaStreamCreateWithFlags(&net->stream, cudaStreamNonBlocking) == cudaSuccess) net->own_stream = true;
    else { delete net; return SPH_ERR_CUDA; }
    net->tr = M::trainer_new((int)n_frame, true);
    if (net->tr) M::trainer_set_tc(net->tr, net->train_precision == 1);
    if (!net->tr) { sph_mpnn_destroy(net); return SPH_ERR_OUT_OF_MEMORY; }
    *out = net;
    return SPH_OK;
}

sph_status sph_mpnn_destroy(sph_mpnn* net) {
    if (!net) return SPH_ERR_INVALID_ARG;
    cudaSetDevice(net->device);
    if (net->stream) cudaStreamSynchronize(net->stream);
    if (net->tr) M::trainer_delete(net->tr);
    if (net->inf) M::trainer_delete(net->inf);
    for (auto& r : net->frames) cudaFree(r.arena);
    void* ptrs[] = {net->nb, net->cnt, net->snap_pos, net->snap_vel, net->snap_rhop, net->ck_pos, net->ck_vel,
                    net->ck_rhop, net->l_pos, net->l_vel,
                    net->l_rhop, net->acc, net->accx, net->Obuf, net->osum, net->ocorr, net->rho_l, net->rho_p, net->vel_l, net->vel_p, net->cmp, net->harena,
                    net->frags, net->H1b, net->Pperm, net->tcw, net->tc_err};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    if (net->own_stream) cudaStreamDestroy(net->stream);
    delete net;
    return SPH_OK;
}

const char* sph_mpnn_last_error(const sph_mpnn* net) { return net ? net->err.c_str() : "null network"; }

sph_status sph_mpnn_set_params(sph_mpnn* net, const float* params, uint32_t n) {
    if (!net || !params || n != (uint32_t)M::kParams) return SPH_ERR_INVALID_ARG;
    NCK(cudaSetDevice(net->device));
    NCK(cudaMemcpyAsync(M::trainer_params(net->tr), params, sizeof(float) * n, cudaMemcpyHostToDevice, net->stream));
    if (net->inf)
        NCK(cudaMemcpyAsync(M::trainer_params(net->inf), params, sizeof(float) * n, cudaMemcpyHostToDevice,
                            net->stream));
    M::trainer_reset_adam(net->tr);
    net->adam_t = 0;
    net->frags_dirty = true;
    NCK(cudaStreamSynchronize(net->stream));
    return SPH_OK;
}

sph_status sph_mpnn_get_params(sph_mpnn* net, float* params, uint32_t n) {
    if (!net || !params || n != (uint32_t)M::kParams) return SPH_ERR_INVALID_ARG;
    NCK(cudaSetDevice(net->device));
    NCK(cudaMemcpyAsync(params, M::trainer_params(net->tr), sizeof(float) * n, cudaMemcpyDeviceToHost, net->stream));
    NCK(cudaStreamSynchronize(net->stream));
    return SPH_OK;
}

sph_status sph_mpnn_loss_grad(sph_mpnn* net, uint32_t n, const float* pos4, const float* vel4, const float* rhop2,
                              const int32_t* nb, const int32_t* cnt, const float* target8, const float fc[6],
                              double* loss, float* out8, float* grad) {
    if (!net || !pos4 || !vel4 || !rhop2 || !nb || !cnt || !target8 || !fc || n == 0) return SPH_ERR_INVALID_ARG;
    if ((int)n > M::trainer_capacity(net->tr)) { net->err = "frame larger than the training workspace"; return SPH_ERR_CAPACITY; }
    for (uint32_t i = 0; i < n; ++i) {
        if (cnt[i] < 0 || cnt[i] > M::K) { net->err = "neighbour count out of [0, 32]"; return SPH_ERR_INVALID_ARG; }
        for (int q = 0; q < cnt[i]; ++q)
            if (nb[(size_t)i * M::K + q] < 0 || nb[(size_t)i * M::K + q] >= (int)n) {
                net->err = "neighbour index out of range";
                return SPH_ERR_INVALID_ARG;
            }
    }
    NCK(cudaSetDevice(net->device));
    NCK(ensure_host_arena(net, n));
    char* a = (char*)net->harena;
    float4* dpos = (float4*)a; a += (size_t)n * 16;
    float4* dvel = (float4*)a; a += (size_t)n * 16;
    float* dtg = (float*)a; a += (size_t)n * 4 * M::kOS;
    float2* drh = (float2*)a; a += (size_t)n * 8;
    int* dcnt = (int*)a; a += (size_t)n * 4;
    int* dnb = (int*)a;
    cudaStream_t st = net->stream;
    NCK(cudaMemcpyAsync(dpos, pos4, (size_t)n * 16, cudaMemcpyHostToDevice, st));
    NCK(cudaMemcpyAsync(dvel, vel4, (size_t)n * 16, cudaMemcpyHostToDevice, st));
    NCK(cudaMemcpyAsync(dtg, target8, (size_t)n * 4 * M::kOS, cudaMemcpyHostToDevice, st));
    NCK(cudaMemcpyAsync(drh, rhop2, (size_t)n * 8, cudaMemcpyHostToDevice, st));
    NCK(cudaMemcpyAsync(dcnt, cnt, (size_t)n * 4, cudaMemcpyHostToDevice, st));
    NCK(cudaMemcpyAsync(dnb, nb, (size_t)n * M::K * 4, cudaMemcpyHostToDevice, st));
    M::Frame f{dpos, dvel, drh, dnb, dcnt, dtg, (int)n, {fc[0], fc[1], fc[2], fc[3], fc[4], fc[5]}};
    const double l = M::trainer_loss_grad(net->tr, f, st);
    if (M::trainer_tc_error(net->tr, st)) { net->err = "tensor-core GEMM wait timed out"; return SPH_ERR_DEVICE; }
    if (loss) *loss = l;
    if (out8)
        NCK(cudaMemcpyAsync(out8, M::trainer_out(net->tr), (size_t)n * 4 * M::kOS, cudaMemcpyDeviceToHost, st));
    if (grad) NCK(cudaMemcpyAsync(grad, M::trainer_grad(net->tr), sizeof(float) * M::kParams, cudaMemcpyDeviceToHost, st));
    NCK(cudaStreamSynchronize(st));
    NCK(cudaGetLastError());
    return SPH_OK;
}

sph_status sph_mpnn_set_precision(sph_mpnn* net, int32_t precision) {
    if (!net || precision < 0 || precision > 3) return SPH_ERR_INVALID_ARG;
    net->precision = precision;
    return SPH_OK;
}

sph_status sph_mpnn_set_train_precision(sph_mpnn* net, int32_t precision) {
    if (!net || (precision != 0 && precision != 1)) return SPH_ERR_INVALID_ARG;
    net->train_precision = precision;
    M::trainer_set_tc(net->tr, precision == 1);
    return SPH_OK;
}

sph_status sph_mpnn_forward(sph_mpnn* net, uint32_t n, const float* pos4, const float* vel4, const float* rhop2,
                            const int32_t* nb, const int32_t* cnt, const float fc[6], int32_t precision, float* out8) {
    if (!net || !pos4 || !vel4 || !rhop2 || !nb || !cnt || !fc || !out8 || n == 0) return SPH_ERR_INVALID_ARG;
    if (precision < 0 || precision > 4) return SPH_ERR_INVALID_ARG;
    if ((int)n > M::trainer_capacity(net->tr)) { net->err = "frame larger than the training workspace"; return SPH_ERR_CAPACITY; }
    for (uint32_t i = 0; i < n; ++i) {
        if (cnt[i] < 0 || cnt[i] > M::K) { net->err = "neighbour count out of [0, 32]"; return SPH_ERR_INVALID_ARG; }
        for (int q = 0; q < cnt[i]; ++q)
            if (nb[(size_t)i * M::K + q] < 0 || nb[(size_t)i * M::K + q] >= (int)n) {
                net->err = "neighbour index out of range";
                return SPH_ERR_INVALID_ARG;
            }
    }
    NCK(cudaSetDevice(net->device));
    NCK(ensure_host_arena(net, n));
    char* a = (char*)net->harena;
    float4* dpos = (float4*)a; a += (size_t)n * 16;
    float4* dvel = (float4*)a; a += (size_t)n * 16;
    float* dout = (float*)a; a += (size_t)n * 4 * M::kOS;
    float2* drh = (float2*)a; a += (size_t)n * 8;
    int* dcnt = (int*)a; a += (size_t)n * 4;
    int* dnb = (int*)a;
    cudaStream_t st = net->stream;
    NCK(cudaMemcpyAsync(dpos, pos4, (size_t)n * 16, cudaMemcpyHostToDevice, st));
    NCK(cudaMemcpyAsync(dvel, vel4, (size_t)n * 16, cudaMemcpyHostToDevice, st));
    NCK(cudaMemcpyAsync(drh, rhop2, (size_t)n * 8, cudaMemcpyHostToDevice, st));
    NCK(cudaMemcpyAsync(dcnt, cnt, (size_t)n * 4, cudaMemcpyHostToDevice, st));
    NCK(cudaMemcpyAsync(dnb, nb, (size_t)n * M::K * 4, cudaMemcpyHostToDevice, st));
    M::Frame f{dpos, dvel, drh, dnb, dcnt, nullptr, (int)n, {fc[0], fc[1], fc[2], fc[3], fc[4], fc[5]}};
    if (precision == 3) {  // the tcgen05 inference kernels
        sph_status s2 = ensure_bf16(net, (int)n, st);
        if (s2) return s2;
        M::tc_infer_round1(f, net->tcw, net->H1b, reinterpret_cast<__half*>(net->Pperm), net->tc_err, st);
        M::tc_infer_round2(f, net->tcw, net->H1b, reinterpret_cast<const __half*>(net->Pperm), dout, net->tc_err, st);
        NCK(cudaMemcpyAsync(out8, dout, (size_t)n * 4 * M::kOS, cudaMemcpyDeviceToHost, st));
        uint32_t e = 0;
        NCK(cudaMemcpyAsync(&e, net->tc_err, sizeof(e), cudaMemcpyDeviceToHost, st));
        NCK(cudaStreamSynchronize(st));
        if (e) {
            cudaMemsetAsync(net->tc_err, 0, sizeof(e), st);
            net->err = "tensor-core inference wait timed out";
            return SPH_ERR_DEVICE;
        }
    } else if (precision == 1 || precision == 4) {  // mma.sync (4: its round 1 on tcgen05, features on lanes)
        sph_status s2 = ensure_bf16(net, (int)n, st);
        if (s2) return s2;
        SceneDev S{};
        if (precision == 4) M::tc_infer_round1_lanes(f, net->tcw, net->H1b, net->Pperm, net->tc_err, st);
        else M::infer_round1(f, net->frags, net->H1b, net->Pperm, st);
        M::infer_round2(f, net->frags, M::trainer_params(net->tr), net->H1b, net->Pperm, S, nullptr, nullptr, dout,
                        nullptr, nullptr, nullptr, false, st);
        NCK(cudaMemcpyAsync(out8, dout, (size_t)n * 4 * M::kOS, cudaMemcpyDeviceToHost, st));
        if (precision == 4) {
            uint32_t e = 0;
            NCK(cudaMemcpyAsync(&e, net->tc_err, sizeof(e), cudaMemcpyDeviceToHost, st));
            NCK(cudaStreamSynchronize(st));
            if (e) {
                cudaMemsetAsync(net->tc_err, 0, sizeof(e), st);
                net->err = "tensor-core inference wait timed out";
                return SPH_ERR_DEVICE;
            }
        }
    } else {  // the training forward: 0 FP32, 2 BF16 tensor-core node layers
        const bool tc_was = M::trainer_tc(net->tr);
        M::trainer_set_tc(net->tr, precision == 2);
        M::trainer_forward(net->tr, f, st);
        M::trainer_set_tc(net->tr, tc_was);
        NCK(cudaMemcpyAsync(out8, M::trainer_out(net->tr), (size_t)n * 4 * M::kOS, cudaMemcpyDeviceToHost, st));
        if (M::trainer_tc_error(net->tr, st)) { net->err = "tensor-core GEMM wait timed out"; return SPH_ERR_DEVICE; }
    }
    NCK(cudaStreamSynchronize(st));
    NCK(cudaGetLastError());
    return SPH_OK;
}

sph_status sph_mpnn_record(sph_mpnn* net, sph_ctx* ctx, uint32_t n_frames, uint32_t* frames_total) {
    if (!net || !ctx) return SPH_ERR_INVALID_ARG;
    if (!ctx->have_state) { net->err = "context has no particles"; return SPH_ERR_NOT_READY; }
    if (!(ctx->params[0].flags & SPH_FLAG_KEEP_FORCE)) {
        net->err = "recording needs a context created with SPH_FLAG_KEEP_FORCE";
        return SPH_ERR_INVALID_ARG;
    }
    for (size_t s = 0; s < ctx->counts.size(); ++s)
        if ((int)ctx->counts[s] > M::trainer_capacity(net->tr)) {
            net->err = "a scene is larger than the training workspace";
            return SPH_ERR_CAPACITY;
        }
    NCK(cudaSetDevice(ctx->device));
    const int n = ctx->b.n;
    sph_status st = ensure_ctx_scratch(net, n);
    if (st) return st;
    for (uint32_t fr = 0; fr < n_frames; ++fr) {
        engine::sort_state(ctx);
        launch_nb_density(ctx, net->nb, net->cnt);
        std::vector<size_t> first_idx;
        for (size_t s = 0; s < ctx->sc_h.size(); ++s) {
            const SceneDev& S = ctx->sc_h[s];
            const int m = S.count;
            sph_mpnn::Rec r;
            const size_t bytes = (size_t)m * (16 + 16 + 4 * M::kOS + 8 + 4 + 4) + (size_t)m * M::K * 4;
            NCK(cudaMalloc(&r.arena, bytes));
            char* a = (char*)r.arena;
            float4* fpos = (float4*)a; a += (size_t)m * 16;
            float4* fvel = (float4*)a; a += (size_t)m * 16;
            float* ftg = (float*)a; a += (size_t)m * 4 * M::kOS;
            float2* frh = (float2*)a; a += (size_t)m * 8;
            int* fcnt = (int*)a; a += (size_t)m * 4;
            int* fid = (int*)a; a += (size_t)m * 4;
            int* fnb = (int*)a;
            k_frame_copy<<<nblk(m), kT, 0, ctx->stream>>>(ctx->b.pos_s, ctx->b.vel_s, ctx->b.rhop, net->nb, net->cnt,
                                                          S.first, m, fpos, fvel, frh, fnb, fcnt, fid);
            r.f = M::Frame{fpos, fvel, frh, fnb, fcnt, ftg, m, frame_const(S, ctx->params[s].visc)};
            net->frames.push_back(r);
            first_idx.push_back(net->frames.size() - 1);
        }
        // targets: the mean accelerations of the next 4 plain steps, from the forces alone (no wall clamp)
        NCK(cudaMemsetAsync(net->acc, 0, sizeof(float4) * n, ctx->stream));
        NCK(cudaMemsetAsync(net->accx, 0, sizeof(float4) * n, ctx->stream));
        for (int sub = 0; sub < 4; ++sub) {
            st = engine::run_steps(ctx, 1);
            if (st) { net->err = ctx->err; return st; }
            k_accum_accel<<<nblk(n), kT, 0, ctx->stream>>>(ctx->b.vel, ctx->b.force_s, ctx->b.rhop, n,
                                                           (float)(4 - sub), net->acc, net->accx);
        }
        for (size_t s = 0; s < ctx->sc_h.size(); ++s) {
            sph_mpnn::Rec& r = net->frames[first_idx[s]];
            const SceneDev& S = ctx->sc_h[s];
            const int* fid = (const int*)((const char*)r.arena + (size_t)S.count * (16 + 16 + 4 * M::kOS + 8 + 4));
            k_frame_target<<<nblk(S.count), kT, 0, ctx->stream>>>(fid, net->acc, net->accx, S.count, S.h / S.gas_k,
                                                                 const_cast<float*>(r.f.target));
        }
        NCK(cudaGetLastError());
    }
    NCK(cudaStreamSynchronize(ctx->stream));
    if (frames_total) *frames_total = (uint32_t)net->frames.size();
    return SPH_OK;
}

sph_status sph_mpnn_clear_frames(sph_mpnn* net) {
    if (!net) return SPH_ERR_INVALID_ARG;
    cudaSetDevice(net->device);
    for (auto& r : net->frames) cudaFree(r.arena);
    net->frames.clear();
    return SPH_OK;
}

sph_status sph_mpnn_train(sph_mpnn* net, uint32_t steps, float lr, uint64_t seed, float* loss_per_step) {
    if (!net || !(lr > 0.0f)) return SPH_ERR_INVALID_ARG;
    if (net->frames.empty()) { net->err = "no recorded frames"; return SPH_ERR_NOT_READY; }
    NCK(cudaSetDevice(net->device));
    std::mt19937_64 rng(seed);
    std::uniform_int_distribution<size_t> pick(0, net->frames.size() - 1);
    for (uint32_t s = 0; s < steps; ++s) {
        const M::Frame& f = net->frames[pick(rng)].f;
        const double l = M::trainer_loss_grad(net->tr, f, net->stream);
        M::trainer_adam(net->tr, ++net->adam_t, lr, net->stream);
        if (loss_per_step) loss_per_step[s] = (float)l;
    }
    net->frags_dirty = true;
    NCK(cudaStreamSynchronize(net->stream));
    NCK(cudaGetLastError());
    if (M::trainer_tc_error(net->tr, net->stream)) { net->err = "tensor-core GEMM wait timed out"; return SPH_ERR_DEVICE; }
    if (net->inf)
        NCK(cudaMemcpyAsync(M::trainer_params(net->inf), M::trainer_params(net->tr), sizeof(float) * M::kParams,
                            cudaMemcpyDeviceToDevice, net->stream));
    return SPH_OK;
}

sph_status sph_neighbor_lists(sph_ctx* ctx, int32_t* nb_ids, int32_t* counts, float* rho) {
    if (!ctx || !nb_ids || !counts || !rho) return SPH_ERR_INVALID_ARG;
    if (!ctx->have_state) return fail(ctx, SPH_ERR_NOT_READY, "no particles uploaded");
    cudaSetDevice(ctx->device);
    const int n = ctx->b.n;
    const size_t m = (size_t)n;
    char* buf = nullptr;
    const size_t bytes = m * M::K * 4 * 2 + m * 4 * 2 + m * 4;
    if (cudaMalloc(&buf, bytes) != cudaSuccess) return fail(ctx, SPH_ERR_OUT_OF_MEMORY, "neighbour-list scratch");
    int* nb = reinterpret_cast<int*>(buf);
    int* cnt = nb + m * M::K;
    int* nb_id = cnt + m;
    int* cnt_id = nb_id + m * M::K;
    float* rho_id = reinterpret_cast<float*>(cnt_id + m);
    engine::sort_state(ctx);
    launch_nb_density(ctx, nb, cnt);
    k_lists_by_id<<<nblk(n), kT, 0, ctx->stream>>>(ctx->b.vel_s, nb, cnt, ctx->b.rhop, n, nb_id, cnt_id, rho_id);
    // the sorted copy becomes the state, so rhop lines up with it (as after sph_refresh_density)
    cudaMemcpyAsync(ctx->b.pos, ctx->b.pos_s, m * sizeof(float4), cudaMemcpyDeviceToDevice, ctx->stream);
    cudaMemcpyAsync(ctx->b.vel, ctx->b.vel_s, m * sizeof(float4), cudaMemcpyDeviceToDevice, ctx->stream);
    cudaError_t e = cudaMemcpyAsync(nb_ids, nb_id, m * M::K * 4, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(counts, cnt_id, m * 4, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(rho, rho_id, m * 4, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    cudaFree(buf);
    if (e != cudaSuccess) return fail(ctx, SPH_ERR_CUDA, std::string("neighbour lists: ") + cudaGetErrorString(e));
    return engine::check_device_error(ctx);
}

sph_status sph_refresh_density(sph_ctx* ctx) {
    if (!ctx) return SPH_ERR_INVALID_ARG;
    if (!ctx->have_state) return fail(ctx, SPH_ERR_NOT_READY, "no particles uploaded");
    cudaSetDevice(ctx->device);
    sph_status st = refresh_density(ctx);
    if (st) return st;
    return engine::check_device_error(ctx);
}

sph_status sph_learned_set_judge(sph_ctx* ctx, int32_t metric) {
    if (!ctx) return SPH_ERR_INVALID_ARG;
    if (metric != SPH_JUDGE_MEAN_DENSITY && metric != SPH_JUDGE_PARTICLE_DENSITY)
        return fail(ctx, SPH_ERR_INVALID_ARG, "unknown judge metric");
    ctx->judge_metric = metric;
    return SPH_OK;
}

sph_status sph_learned_set_max_density_tol(sph_ctx* ctx, float tol) {
    if (!ctx) return SPH_ERR_INVALID_ARG;
    if (!(tol >= 0.0f)) return fail(ctx, SPH_ERR_INVALID_ARG, "max-density tolerance must be >= 0");
    ctx->judge_max_rho_tol = tol;
    return SPH_OK;
}

sph_status sph_learned_step(sph_ctx* ctx, sph_mpnn* net, int32_t n_macro, int32_t judge_every, float density_tol,
                            float momentum_tol, sph_learned_report* rep) {
    if (!ctx || !net) return SPH_ERR_INVALID_ARG;
    if (ctx->batched) return fail(ctx, SPH_ERR_UNSUPPORTED, "the learned macro-step runs on single-scene contexts");
    if (!ctx->have_state) return fail(ctx, SPH_ERR_NOT_READY, "no particles uploaded");
    if (n_macro < 0 || judge_every < 0) return fail(ctx, SPH_ERR_INVALID_ARG, "negative count");
    cudaSetDevice(ctx->device);
    const int n = ctx->b.n;
    if (net->precision == 0 && (!net->inf || M::trainer_capacity(net->inf) < n)) {
        if (net->inf) M::trainer_delete(net->inf);
        net->inf = M::trainer_new(n, false);
        if (!net->inf) return fail(ctx, SPH_ERR_OUT_OF_MEMORY, "network workspace");
        if (cudaMemcpy(M::trainer_params(net->inf), M::trainer_params(net->tr), sizeof(float) * M::kParams,
                       cudaMemcpyDeviceToDevice) != cudaSuccess)
            return fail(ctx, SPH_ERR_CUDA, "copy of the network parameters");
    }
    sph_status st = ensure_ctx_scratch(net, n);
    if (!st && net->precision >= 1) st = ensure_bf16(net, n, ctx->stream);
    if (st) return fail(ctx, st, net->err);
    sph_learned_report r{};
    int& backoff = ctx->judge_backoff;    // plain intervals still to run before the next learned attempt
    int& failures = ctx->judge_failures;  // consecutive failed judges
    for (int k = 0; k < n_macro;) {
        const int len = judge_every > 0 ? std::min(judge_every, n_macro - k) : n_macro - k;
        k += len;
        if (backoff > 0) {
            st = engine::run_steps(ctx, 4 * len);
            if (st) return st;
            r.plain_macro_steps += len;
            --backoff;
            continue;
        }
        if (judge_every == 0) {
            for (int q = 0; q < len; ++q) {
                st = learned_macro(ctx, net);
                if (st) return st;
            }
            r.learned_macro_steps += len;
            continue;
        }
        // a learned interval: checkpoint, len - 1 learned macro-steps, then the judged one
        const Saved ck = save_state(ctx, net->ck_pos, net->ck_vel, net->ck_rhop);
        for (int q = 0; q + 1 < len; ++q) {
            st = learned_macro(ctx, net);
            if (st) return st;
        }
        double dev = 0.0, mom = 0.0, mdev = 0.0, xdev = 0.0;
        st = judge_macro(ctx, net, dev, mom, mdev, xdev);
        if (st) return st;
        ++r.judged;
        r.last_density_dev = dev;
        r.last_momentum_dev = mom;
        r.max_density_dev = std::max(r.max_density_dev, dev);
        r.sum_density_dev += dev;
        r.last_mean_rho_dev = mdev;
        r.max_mean_rho_dev = std::max(r.max_mean_rho_dev, mdev);
        r.last_max_rho_dev = xdev;
        r.max_max_rho_dev = std::max(r.max_max_rho_dev, xdev);
        const double crit = ctx->judge_metric == SPH_JUDGE_PARTICLE_DENSITY ? dev : mdev;
        if (crit <= density_tol && mom <= momentum_tol && xdev <= ctx->judge_max_rho_tol) {
            copy_state(ctx, ctx->b.pos, ctx->b.vel, ctx->b.rhop, net->l_pos, net->l_vel, net->l_rhop);
            cudaMemsetAsync(ctx->b.count, 0, sizeof(int) * (size_t)ctx->b.ncell, ctx->stream);
            ctx->need_hash = true;
            r.learned_macro_steps += len;
            failures = 0;
        } else {
            // roll the interval back and run it with plain SPH; retry the network after
            // 0, 1, 3, 7, 7, ... further plain intervals
            restore_state(ctx, ck);
            st = engine::run_steps(ctx, 4 * len);
            if (st) return st;
            ++r.fallbacks;
            r.plain_macro_steps += len;
            r.discarded_macro_steps += len;
            ++failures;
            backoff = std::min((1 << std::min(failures - 1, 3)) - 1, 7);
        }
    }
    if (rep) *rep = r;
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(ctx, SPH_ERR_CUDA, std::string("learned step: ") + cudaGetErrorString(e));
    if (net->tc_err) {
        uint32_t te = 0;
        if (cudaMemcpyAsync(&te, net->tc_err, sizeof(te), cudaMemcpyDeviceToHost, ctx->stream) ||
            cudaStreamSynchronize(ctx->stream))
            return fail(ctx, SPH_ERR_CUDA, "learned step: error word readback");
        if (te) {
            cudaMemsetAsync(net->tc_err, 0, sizeof(te), ctx->stream);
            return fail(ctx, SPH_ERR_DEVICE, "learned step: a tensor-core wait of the inference timed out");
        }
    }
    return engine::check_device_error(ctx);
}

}  // extern "C"
