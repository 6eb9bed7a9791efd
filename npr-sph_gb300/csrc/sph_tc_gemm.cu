// sph_tc_gemm.cu -- BF16 GEMM on the sm_103a tensor cores (tcgen05, FP32 accumulation in
// TMEM) for the training passes of the learned macro-step: the node layers forward, their
// data gradients and the weight gradients (split over K, reduced in a fixed order).
//
// One CTA of 128 threads per 128-row tile of A (and per K slice with split-K):
//   - warp 0 allocates TMEM (a power of two >= N columns); thread 0 initialises two mbarriers;
//   - K runs in chunks of 64 through two shared-memory buffers: the threads copy the A and B
//     chunk (16-byte loads, rows beyond M / N and columns beyond K zero) into the canonical
//     K-major layout of sph_tc.cuh, fence it to the async proxy, and thread 0 issues the
//     chunk's MMAs (K = 16 each) and commits them to the buffer's mbarrier; a buffer is
//     refilled only after the MMAs that read it have completed;
//   - after the last commit every warp reads its 32 rows of D from TMEM, 16 columns at a time,
//     and applies the epilogue (sph_tc.h);
//   - warp 0 frees the TMEM.
// Every wait is bounded (sph_tc.cuh): on a timeout the CTA sets bit 0 of *err, skips its
// epilogue and still frees its TMEM.
#include <cuda_bf16.h>

#include "sph_internal.h"
#include "sph_tc.cuh"
#include "sph_tc.h"

namespace sphgb {
namespace tc {

namespace {

constexpr int kThreads = 128;
constexpr int kTileM = 128;
constexpr int kKC = 64;                 // K elements per staged chunk (4 MMAs)
constexpr int kChunkK8 = kKC / 8;       // 16-byte chunks per row of a staged chunk
constexpr uint32_t kLBO = 128;
constexpr uint32_t kSBO = kKC * 16;

// Copy rows row0 .. row0 + ROWS - 1, columns k0 .. k0 + kKC - 1 of G into the tile (zeros past
// nrow_valid and kend). Each thread issues all of its 16-byte loads before any store, so the
// loads of a chunk are in flight together.
template <int ROWS>
__device__ __forceinline__ void stage_rows(uint8_t* tile, const __nv_bfloat16* __restrict__ G, int ld, int row0,
                                           int nrow_valid, int k0, int kend) {
    constexpr int kTotal = ROWS * kChunkK8;
    constexpr int kPer = (kTotal + kThreads - 1) / kThreads;
    uint4 v[kPer];
#pragma unroll
    for (int i = 0; i < kPer; ++i) {
        const int c = threadIdx.x + i * kThreads;
        const int r = c / kChunkK8, k8 = c % kChunkK8;
        const int gr = row0 + r, gk = k0 + 8 * k8;
        v[i] = make_uint4(0u, 0u, 0u, 0u);
        if (c < kTotal && gr < nrow_valid && gk < kend) v[i] = __ldg(reinterpret_cast<const uint4*>(G + (size_t)gr * ld + gk));
    }
#pragma unroll
    for (int i = 0; i < kPer; ++i) {
        const int c = threadIdx.x + i * kThreads;
        if (c < kTotal) *reinterpret_cast<uint4*>(tile + tile_off(c / kChunkK8, c % kChunkK8, kKC)) = v[i];
    }
}

template <int N>
__global__ void __launch_bounds__(kThreads) k_gemm_bf16(const __nv_bfloat16* __restrict__ A, int lda,
                                                        const __nv_bfloat16* __restrict__ B, int ldb, int M, int K,
                                                        int k_per_split, Epilogue epi, uint32_t* __restrict__ err) {
    static_assert(N % 16 == 0 && N >= 16 && N <= 256, "tcgen05 M = 128 needs N in 16..256, a multiple of 16");
    constexpr uint32_t kCols = tmem_cols_for(N);
    constexpr int kTileBytesA = kTileM * kKC * 2, kTileBytesB = N * kKC * 2;
    extern __shared__ __align__(1024) uint8_t smem[];
    // buffer b: its A tile at smem + b * kBufBytes, its B tile right after
    constexpr int kBufBytes = kTileBytesA + kTileBytesB;
    __shared__ __align__(8) uint64_t mbar[2];
    __shared__ uint32_t tmem_slot;
    __shared__ int timed_out;

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int m0 = blockIdx.x * kTileM;
    const int split = blockIdx.y;
    const int kb = split * k_per_split, ke = min(K, kb + k_per_split);
    if (threadIdx.x == 0) {
        mbar_init(&mbar[0], 1);
        mbar_init(&mbar[1], 1);
        mbar_init_fence();
        timed_out = 0;
    }
    if (warp == 0) tmem_alloc(&tmem_slot, kCols);
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    const uint32_t tmem = tmem_slot;
    const uint32_t idesc = idesc_bf16_f32(kTileM, N);
    const int nchunks = ke > kb ? (ke - kb + kKC - 1) / kKC : 0;
    bool ok = true;
    for (int c = 0; c < nchunks; ++c) {
        const int b = c & 1;
        if (c >= 2 && !mbar_wait(&mbar[b], ((c - 2) >> 1) & 1)) ok = false;
        if (__syncthreads_or(!ok)) { ok = false; break; }
        const int k0 = kb + c * kKC;
        uint8_t* const tA = smem + b * kBufBytes;
        stage_rows<kTileM>(tA, A, lda, m0, M, k0, ke);
        stage_rows<N>(tA + kTileBytesA, B, ldb, 0, N, k0, ke);
        fence_smem_to_async();
        __syncthreads();
        if (threadIdx.x == 0) {
            fence_after_sync();
            const uint32_t a0 = smem_u32(smem + b * kBufBytes), b0 = a0 + (uint32_t)kTileBytesA;
            const int steps = min(kKC, ke - k0) / 16;
            for (int s = 0; s < steps; ++s)
                mma_bf16(tmem, smem_desc(a0 + 256u * s, kLBO, kSBO), smem_desc(b0 + 256u * s, kLBO, kSBO), idesc,
                         (c > 0 || s > 0) ? 1u : 0u);
            mma_commit(&mbar[b]);
        }
    }
    if (ok && nchunks > 0) ok = mbar_wait(&mbar[(nchunks - 1) & 1], ((nchunks - 1) >> 1) & 1);
    if (!ok) timed_out = 1;
    __syncthreads();
    fence_after_sync();
    if (!timed_out) {
        const int row = m0 + 32 * warp + lane;
        const bool split_k = gridDim.y > 1;
        float* out = epi.out ? epi.out + (split_k ? (long long)split * epi.split_stride : 0ll) : nullptr;
#pragma unroll 1
        for (int c0 = 0; c0 < N; c0 += 16) {
            float v[16];
            if (nchunks > 0) {
                tmem_ld16(tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)c0, v);
                tmem_wait_ld();
            } else {
#pragma unroll
                for (int j = 0; j < 16; ++j) v[j] = 0.0f;
            }
            if (row >= M) continue;
            const bool full = c0 + 16 <= epi.ncols;
            if (!split_k) {
                // 16-byte loads and stores where the chunk is whole and the rows are 16-byte aligned
                if (epi.add) {
                    const float* a = epi.add + (size_t)row * epi.ld_add + c0;
                    if (full && ((reinterpret_cast<uintptr_t>(a) & 15) == 0)) {
#pragma unroll
                        for (int j = 0; j < 16; j += 4) {
                            const float4 t = *reinterpret_cast<const float4*>(a + j);
                            v[j] += t.x; v[j + 1] += t.y; v[j + 2] += t.z; v[j + 3] += t.w;
                        }
                    } else {
                        for (int j = 0; j < 16 && c0 + j < epi.ncols; ++j) v[j] += a[j];
                    }
                }
                if (epi.relu) {
#pragma unroll
                    for (int j = 0; j < 16; ++j) v[j] = fmaxf(v[j], 0.0f);
                }
                if (epi.gate) {
                    const float* gt = epi.gate + (size_t)row * epi.ld_gate + c0;
                    if (full && ((reinterpret_cast<uintptr_t>(gt) & 15) == 0)) {
#pragma unroll
                        for (int j = 0; j < 16; j += 4) {
                            const float4 t = *reinterpret_cast<const float4*>(gt + j);
                            if (!(t.x > 0.0f)) v[j] = 0.0f;
                            if (!(t.y > 0.0f)) v[j + 1] = 0.0f;
                            if (!(t.z > 0.0f)) v[j + 2] = 0.0f;
                            if (!(t.w > 0.0f)) v[j + 3] = 0.0f;
                        }
                    } else {
                        for (int j = 0; j < 16 && c0 + j < epi.ncols; ++j)
                            if (!(gt[j] > 0.0f)) v[j] = 0.0f;
                    }
                }
                if (epi.outb)
                    for (int j = 0; j < 16 && c0 + j < epi.ncols; ++j)
                        epi.outb[(size_t)row * epi.ld_outb + c0 + j] = __float2bfloat16_rn(v[j]);
            }
            if (out) {
                float* o = out + (size_t)row * epi.ld_out + c0;
                if (full && ((reinterpret_cast<uintptr_t>(o) & 15) == 0)) {
#pragma unroll
                    for (int j = 0; j < 16; j += 4)
                        *reinterpret_cast<float4*>(o + j) = make_float4(v[j], v[j + 1], v[j + 2], v[j + 3]);
                } else {
                    for (int j = 0; j < 16 && c0 + j < epi.ncols; ++j) o[j] = v[j];
                }
            }
        }
    } else if (threadIdx.x == 0 && err) {
        atomicOr(err, 1u);
    }
    fence_before_sync();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tmem, kCols);
}

template <int N>
cudaError_t launch(const __nv_bfloat16* A, int lda, const __nv_bfloat16* B, int ldb, int M, int K, const Epilogue& epi,
                   int splits, int kps, uint32_t* err, cudaStream_t st) {
    constexpr size_t smem = 2 * (size_t)(kTileM + N) * kKC * 2;
    static bool attr = false;
    if (!attr) {
        const cudaError_t e = cudaFuncSetAttribute(k_gemm_bf16<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        attr = true;
    }
    const dim3 grid((unsigned)((M + kTileM - 1) / kTileM), (unsigned)splits);
    k_gemm_bf16<N><<<grid, kThreads, smem, st>>>(A, lda, B, ldb, M, K, kps, epi, err);
    return cudaGetLastError();
}

}  // namespace

cudaError_t gemm_bf16(const __nv_bfloat16* A, int lda, const __nv_bfloat16* B, int ldb, int M, int N, int K,
                      const Epilogue& epi, int splits, int k_per_split, uint32_t* err, cudaStream_t st) {
    if (M <= 0 || K <= 0 || K % 16 || lda % 8 || ldb % 8 || lda < K || ldb < K || splits < 1)
        return cudaErrorInvalidValue;
    if (splits == 1) k_per_split = K;
    else if (k_per_split % kKC || (long long)splits * k_per_split < K) return cudaErrorInvalidValue;
    if ((reinterpret_cast<uintptr_t>(A) | reinterpret_cast<uintptr_t>(B)) & 15) return cudaErrorInvalidValue;
    switch (N) {
        case 16: return launch<16>(A, lda, B, ldb, M, K, epi, splits, k_per_split, err, st);
        case 32: return launch<32>(A, lda, B, ldb, M, K, epi, splits, k_per_split, err, st);
        case 64: return launch<64>(A, lda, B, ldb, M, K, epi, splits, k_per_split, err, st);
        case 80: return launch<80>(A, lda, B, ldb, M, K, epi, splits, k_per_split, err, st);
        case 128: return launch<128>(A, lda, B, ldb, M, K, epi, splits, k_per_split, err, st);
        case 144: return launch<144>(A, lda, B, ldb, M, K, epi, splits, k_per_split, err, st);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace tc
}  // namespace sphgb

using namespace sphgb;

// Test entry point of the tensor-core GEMM: D = A B^T from host arrays (synchronous).
extern "C" sph_status sph_tc_gemm_bf16(const uint16_t* a, const uint16_t* b, int32_t m, int32_t n, int32_t k,
                                       int32_t splits, float* d) {
    if (!a || !b || !d || m <= 0 || n <= 0 || k <= 0 || splits < 1) return SPH_ERR_INVALID_ARG;
    if (k % 16 || n % 16) return SPH_ERR_INVALID_ARG;
    const int kps = splits > 1 ? ((k + splits - 1) / splits + 63) / 64 * 64 : k;
    if (splits > 1 && (long long)kps * (splits - 1) >= k) return SPH_ERR_INVALID_ARG;  // every slice non-empty
    __nv_bfloat16 *da = nullptr, *db = nullptr;
    float* dd = nullptr;
    uint32_t* derr = nullptr;
    const size_t na = (size_t)m * k, nb = (size_t)n * k, nd = (size_t)splits * m * n;
    sph_status st = SPH_OK;
    if (cudaMalloc(&da, na * 2) != cudaSuccess || cudaMalloc(&db, nb * 2) != cudaSuccess ||
        cudaMalloc(&dd, nd * 4) != cudaSuccess || cudaMalloc(&derr, 4) != cudaSuccess) {
        st = SPH_ERR_OUT_OF_MEMORY;
    } else {
        cudaMemcpy(da, a, na * 2, cudaMemcpyHostToDevice);
        cudaMemcpy(db, b, nb * 2, cudaMemcpyHostToDevice);
        cudaMemset(dd, 0, nd * 4);
        cudaMemset(derr, 0, 4);
        tc::Epilogue e;
        e.out = dd;
        e.ld_out = n;
        e.ncols = n;
        e.split_stride = (long long)m * n;
        if (tc::gemm_bf16(da, k, db, k, m, n, k, e, splits, kps, derr, nullptr) != cudaSuccess) st = SPH_ERR_INVALID_ARG;
        uint32_t herr = 0;
        if (cudaMemcpy(&herr, derr, 4, cudaMemcpyDeviceToHost) != cudaSuccess) st = SPH_ERR_CUDA;
        else if (herr) st = SPH_ERR_DEVICE;
        if (st == SPH_OK && cudaMemcpy(d, dd, nd * 4, cudaMemcpyDeviceToHost) != cudaSuccess) st = SPH_ERR_CUDA;
    }
    cudaFree(da);
    cudaFree(db);
    cudaFree(dd);
    cudaFree(derr);
    return st;
}
