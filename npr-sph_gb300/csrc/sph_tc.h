// sph_tc.h -- host interface of the BF16 tensor-core GEMM (sph_tc_gemm.cu), used by the
// training passes of the learned macro-step.
#pragma once

#include <cstdint>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

namespace sphgb {
namespace tc {

// What the GEMM does with each element v = D[i][j] (i < M, j < ncols) of its FP32 result:
//   v += add[i * ld_add + j]               (add non-null)
//   v = max(v, 0)                          (relu)
//   v = 0 where !(gate[i * ld_gate + j] > 0) (gate non-null: the derivative of a ReLU)
//   out[i * ld_out + j] = v, outb[i * ld_outb + j] = bf16(v)   (either may be null)
// With split-K (splits > 1) slice s of K writes its partial D, without add/relu/gate, to
// out + s * split_stride.
struct Epilogue {
    float* out = nullptr;
    int ld_out = 0;
    __nv_bfloat16* outb = nullptr;
    int ld_outb = 0;
    const float* add = nullptr;
    int ld_add = 0;
    const float* gate = nullptr;
    int ld_gate = 0;
    int relu = 0;
    int ncols = 0;
    long long split_stride = 0;
};

// D[M x N] = A[M x K] * B[N x K]^T with A, B bf16 row-major (K contiguous; lda, ldb multiples of
// 8 elements, 16-byte aligned bases), FP32 accumulation in TMEM. K a multiple of 16, N a
// multiple of 16 in [16, 256]. splits > 1 cuts K into `splits` slices of k_per_split elements
// (a multiple of 64), one CTA row each. err: device word, bit 0 set if a wait ran out.
cudaError_t gemm_bf16(const __nv_bfloat16* A, int lda, const __nv_bfloat16* B, int ldb, int M, int N, int K,
                      const Epilogue& epi, int splits, int k_per_split, uint32_t* err, cudaStream_t st);

}  // namespace tc
}  // namespace sphgb
