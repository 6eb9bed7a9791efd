// sph_mpnn.h -- the learned macro-step: network shape, parameter layout, frame
// layout and the internal entry points shared by sph_mpnn.cu (training) and
// sph_mpnn_infer.cu (tensor-core inference).
//
// The network (no counterpart in the reference) predicts the velocity change of
// every particle over a macro-step of 4*dt from its <= 32 nearest neighbours:
//   e_ij = [(x_j-x_i)/h, (v_j-v_i)/c, r/h, 1-r/h]                       8 edge features
//   n_i  = [v_i/c, rho_i/rho_self-1, (rho_i-rho0)/rho_self, log10(mu)/4, cnt/K, 1]   8
//   round 1: M1 = sum_j relu(e_ij We1 + be1)/K;  H1 = relu([M1 n] Wn1 + bn1);  P = H1 Wp
//   round 2: M2 = sum_j relu(e_ij We2 + P_j + be2)/K;  H2 = relu([M2 H1] Wn2 + bn2)
//   output : O = H2 Wo + bo = (v(t+4dt) - v(t)) / c
// with c = sqrt(k) (sound speed of the linear EOS) and rho_self = m*315/(64*pi*h^3).
#pragma once

#include <cstdint>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "sph_internal.h"

namespace sphgb {
namespace mpnn {

constexpr int K = 32;   // neighbours per particle
constexpr int W = 64;   // hidden width
constexpr int FE = 8;   // edge features
constexpr int FN = 8;   // node features
constexpr int FO = 3;   // outputs

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
};

// One frame: n particles (any order), their <= K neighbours (slots into the
// same arrays, -1 padded), density, and the training target.
struct Frame {
    const float4* pos;
    const float4* vel;
    const float2* rhop;  // (rho, pres)
    const int* nb;       // [n][K]
    const int* cnt;      // [n]
    const float4* target;// [n] velocity change / c (training only)
    int n;
    FrameConst fc;
};

// Workspace of the FP32 network passes (sph_mpnn.cu).
struct Trainer;
Trainer* trainer_new(int n_max, bool train);
void trainer_delete(Trainer* t);
int trainer_capacity(Trainer* t);
float* trainer_params(Trainer* t);  // device, kParams floats
float* trainer_grad(Trainer* t);    // device, kParams floats (train only)
float* trainer_out(Trainer* t);     // device, [n][4]: O of the last forward
void trainer_reset_adam(Trainer* t);
void trainer_forward(Trainer* t, const Frame& f, cudaStream_t st);
double trainer_loss_grad(Trainer* t, const Frame& f, cudaStream_t st);  // synchronous (reads the loss)
void trainer_adam(Trainer* t, int step, float lr, cudaStream_t st);

// BF16 tensor-core inference (sph_mpnn_infer.cu). `frags` (infer_frag_words() u32) holds the
// parameters in MMA fragment order, rebuilt by infer_prep whenever the parameters change.
int infer_frag_words();
void infer_prep(const float* prm, uint32_t* frags, cudaStream_t st);
// H1 and P (permuted) for all particles of f; bf16 [n][64] each.
void infer_round1(const Frame& f, const uint32_t* frags, __nv_bfloat16* H1, uint16_t* Pperm, cudaStream_t st);
// Round 2 and the output O (written to `out` if non-null); with `integrate` the macro-step
// update of f's state into (pos_out, vel_out) and the cell hash of the new positions.
void infer_round2(const Frame& f, const uint32_t* frags, const float* prm, const __nv_bfloat16* H1,
                  const uint16_t* Pperm, const SceneDev& S, float4* pos_out, float4* vel_out, float4* out, int* key,
                  int* rank, int* count, bool integrate, cudaStream_t st);

}  // namespace mpnn
}  // namespace sphgb
