// sph_mpnn.h -- the learned macro-step: network shape, parameter layout, frame
// layout and the internal entry points shared by sph_mpnn.cu (training) and
// sph_mpnn_infer.cu (tensor-core inference).
//
// The network (no counterpart in the reference) predicts, for every particle,
// the mean accelerations over a macro-step of 4*dt from its <= 32 nearest
// neighbours:
//   e_ij = [d, u, r/h, q, q^2 d/(r/h), q u]    d = (x_j-x_i)/h, u = (v_j-v_i)/c, q = 1-r/h
//          (the last two are the shapes of the spiky gradient and of the viscosity
//          Laplacian, force_comp.glsl:59-60; the first at r = 0 is zero)        14 edge features
//   n_i  = [v_i/c, rho_i/rho_self-1, (rho_i-rho0)/rho_self, log10(mu)/4, cnt/K, 1, c dt/h]   9
//   round 1: M1 = sum_j relu(e_ij We1 + be1)/K;  H1 = relu([M1 n] Wn1 + bn1);  P = H1 Wp
//   round 2: M2 = sum_j relu(e_ij We2 + P_j + be2)/K;  H2 = relu([M2 H1] Wn2 + bn2)
//   output : O = H2 Wo + bo = (O_v, O_x), in units of A = k/h:
//            O_v = (a_0 + a_1 + a_2 + a_3) / (4A)            velocity head
//            O_x = (4a_0 + 3a_1 + 2a_2 + a_3) / (10A)        position head
// where a_s is the SPH acceleration F/rho of plain sub-step s. Four symplectic
// sub-steps give exactly
//   v(t+4dt) = v + 4 dt A O_v,   x(t+4dt) = x + 4 dt v + 10 dt^2 A O_x,
// which is the macro-step update (the wall clamp of integrate_comp.glsl:45-77
// is applied once, at its end). c = sqrt(k) is the sound speed of the linear
// EOS and rho_self = m*315/(64*pi*h^3) the density of an isolated particle.
#pragma once

#include <cstdint>
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "sph_internal.h"

namespace sphgb {
namespace mpnn {

constexpr int K = 32;   // neighbours per particle
constexpr int W = 64;   // hidden width
constexpr int FE = 14;  // edge features (the bias column FE of the 16-wide MMA k-tile is 1)
constexpr int FN = 9;   // node features
constexpr int FO = 6;   // outputs: O_v (3), O_x (3)
constexpr int kOS = 8;  // stride of an output / target row (floats)

// Flat FP32 parameter vector: We1, be1, Wn1, bn1, Wp, We2, be2, Wn2, bn2, Wo, bo (row-major [in][out]).
constexpr int kWe1 = 0;
constexpr int kBe1 = kWe1 + FE * W;
constexpr int kWn1 = kBe1 + W;
constexpr int kBn1 = kWn1 + (W + FN) * W;
constexpr int kWp = kBn1 + W;
constexpr int kWe2 = kWp + W * W;
constexpr int kBe2 = kWe2 + FE * W;
constexpr int kWn2 = kBe2 + W;
constexpr int kBn2 = kWn2 + 2 * W * W;
constexpr int kWo = kBn2 + W;
constexpr int kBo = kWo + W * FO;
constexpr int kParams = kBo + FO;

// Scene constants of a frame.
struct FrameConst {
    float h;         // smoothing length
    float c;         // sqrt(k)
    float rho_self;  // m*315/(64*pi*h^3)
    float rho0;
    float log_mu;    // log10(mu)/4
    float courant;   // c*dt/h
};

// One frame: n particles (any order), their <= K neighbours (slots into the
// same arrays, -1 padded), density, and the training target.
struct Frame {
    const float4* pos;
    const float4* vel;
    const float2* rhop;  // (rho, pres)
    const int* nb;       // [n][K]
    const int* cnt;      // [n]
    const float* target; // [n][kOS]: (O_v, O_x) targets, training only
    int n;
    FrameConst fc;
};

#ifdef __CUDACC__
// The macro-step update of one particle from its outputs O = (O_v, O_x): the velocity and
// position after 4 sub-steps, then the per-axis wall clamp of integrate_comp.glsl:45-77 once.
__device__ __forceinline__ void macro_update(const SceneDev& S, float ov0, float ov1, float ov2, float ox0, float ox1,
                                             float ox2, float4 p, float4 v, float4& p_out, float4& v_out) {
    const float A = S.gas_k / S.h;
    const float cv = 4.0f * S.dt * A, cx = 10.0f * S.dt * S.dt * A, c4 = 4.0f * S.dt;
    const float pp[3] = {p.x, p.y, p.z}, vv[3] = {v.x, v.y, v.z};
    const float ov[3] = {ov0, ov1, ov2}, ox[3] = {ox0, ox1, ox2};
    float np[3], nv[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        nv[a] = vv[a] + cv * ov[a];
        np[a] = pp[a] + c4 * vv[a] + cx * ox[a];
        if (np[a] < S.lo[a]) { np[a] = S.lo[a]; nv[a] *= -S.damp; }
        else if (np[a] > S.up[a]) { np[a] = S.up[a]; nv[a] *= -S.damp; }
    }
    p_out = make_float4(np[0], np[1], np[2], p.w);
    v_out = make_float4(nv[0], nv[1], nv[2], v.w);
}
#endif

// Workspace of the FP32 network passes (sph_mpnn.cu).
struct Trainer;
Trainer* trainer_new(int n_max, bool train);
void trainer_delete(Trainer* t);
int trainer_capacity(Trainer* t);
float* trainer_params(Trainer* t);  // device, kParams floats
float* trainer_grad(Trainer* t);    // device, kParams floats (train only)
float* trainer_out(Trainer* t);     // device, [n][kOS]: O of the last forward
void trainer_reset_adam(Trainer* t);
// Node layers (forward, data and weight gradients) on the BF16 tensor cores (tcgen05, FP32
// accumulation; FP32 master weights) instead of FP32 CUDA cores.
void trainer_set_tc(Trainer* t, bool on);
bool trainer_tc(Trainer* t);
// Nonzero if a tensor-core wait timed out since the last call (synchronous; clears the word).
uint32_t trainer_tc_error(Trainer* t, cudaStream_t st);
void trainer_forward(Trainer* t, const Frame& f, cudaStream_t st);
double trainer_loss_grad(Trainer* t, const Frame& f, cudaStream_t st);  // synchronous (reads the loss)
void trainer_adam(Trainer* t, int step, float lr, cudaStream_t st);

// BF16 tensor-core inference (sph_mpnn_infer.cu). `frags` (infer_frag_words() u32) holds the
// parameters in MMA fragment order, rebuilt by infer_prep whenever the parameters change.
int infer_frag_words();
void infer_prep(const float* prm, uint32_t* frags, cudaStream_t st);
// H1 and P (permuted) for all particles of f; bf16 [n][64] each.
void infer_round1(const Frame& f, const uint32_t* frags, __nv_bfloat16* H1, uint16_t* Pperm, cudaStream_t st);
// Round 2 and the output O (written to `out`, [n][kOS], if non-null); with `integrate` the
// macro-step update of f's state into (pos_out, vel_out) and the cell hash of the new positions.
void infer_round2(const Frame& f, const uint32_t* frags, const float* prm, const __nv_bfloat16* H1,
                  const uint16_t* Pperm, const SceneDev& S, float4* pos_out, float4* vel_out, float* out, int* key,
                  int* rank, int* count, bool integrate, cudaStream_t st);

// BF16 tcgen05 inference (sph_mpnn_tc.cu): the weights as bf16 images in the tensor cores'
// shared-memory layout (tc_infer_words() elements, rebuilt by tc_infer_prep when the parameters
// change); round 1 writes H1 (bf16 [n][64]) and P (f16 [n][64]), round 2 the outputs O
// ([n][kOS]). *err gets bit 0 if a tensor-core wait timed out.
int tc_infer_words();
void tc_infer_prep(const float* prm, __nv_bfloat16* img, cudaStream_t st);
void tc_infer_round1(const Frame& f, const __nv_bfloat16* img, __nv_bfloat16* H1, __half* P, uint32_t* err,
                     cudaStream_t st);
void tc_infer_round2(const Frame& f, const __nv_bfloat16* img, const __nv_bfloat16* H1, const __half* P, float* out,
                     uint32_t* err, cudaStream_t st);
// Round 1 with the features on the TMEM lanes (the edge sum inside each thread); writes H1 and P
// in the permuted BF16 layout of the mma.sync round 2 (infer_round2).
void tc_infer_round1_lanes(const Frame& f, const __nv_bfloat16* img, __nv_bfloat16* H1, uint16_t* Pperm, uint32_t* err,
                           cudaStream_t st);

}  // namespace mpnn
}  // namespace sphgb
