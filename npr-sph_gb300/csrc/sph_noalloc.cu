// sph_noalloc.cu -- FP64 diagnostics of a caller's particle buffer without any
// allocation: sph_reduce_aos_noalloc.
//
// Some callers of this library cannot allocate device memory when they need
// the diagnostics: a renderer or game loop that reserves its GPU memory budget
// up front and must not allocate per frame, or a plugin host that owns every
// buffer and hands the library only pointers. They hold the particles in their own
// device buffer (the reference keeps them in an SSBO, Main.cpp:524-527) and
// pass that buffer and an output buffer in.
//
// The reduction needs scratch memory for its per-CTA partial sums. Here that
// scratch is a file-scope __device__ array of fixed size, so the call itself
// allocates nothing. Every GPU that loads this library holds the array
// (kNoAllocMaxBlocks * kDiagFields doubles = 96 KiB) until the process exits.
#include "sph_device.cuh"

namespace sphgb {
namespace {

constexpr int kNoAllocThreads = 256;
constexpr int kNoAllocPerBlock = 4096;   // particles reduced by one CTA
constexpr int kNoAllocMaxBlocks = 1024;  // CTAs, and rows of the scratch array
constexpr long long kNoAllocMaxParticles = (long long)kNoAllocMaxBlocks * kNoAllocPerBlock;  // 4,194,304

// The scratch: one row of kDiagFields partial sums per CTA. A call writes every
// row it later reads, so nothing has to be cleared between calls. All calls
// share it: calls whose kernels overlap on the GPU (on different streams
// without ordering between them) race on it.
static __device__ __align__(256) double g_noalloc_partials[kNoAllocMaxBlocks * kDiagFields];


__global__ void __launch_bounds__(kNoAllocThreads) k_noalloc_partial(const sph_particle* __restrict__ aos, int n,
                                                                     double mass, double rho0, double gx, double gy,
                                                                     double gz, double* __restrict__ partials) {
    double acc[kDiagFields];
#pragma unroll
    for (int f = 0; f < kDiagFields; ++f) acc[f] = 0.0;
    acc[6] = INFINITY;
    acc[7] = -INFINITY;
    const int a = blockIdx.x * kNoAllocPerBlock, b = min(a + kNoAllocPerBlock, n);
    for (int i = a + threadIdx.x; i < b; i += kNoAllocThreads) {
        const sph_particle& r = aos[i];
        const float px = r.pos[0], py = r.pos[1], pz = r.pos[2];
        const float vxf = r.vel[0], vyf = r.vel[1], vzf = r.vel[2];
        const float rho = r.extras[0];
        const bool fin = isfinite(px) && isfinite(py) && isfinite(pz) && isfinite(vxf) && isfinite(vyf) &&
                         isfinite(vzf) && isfinite(rho);
        if (!fin) { acc[9] += 1.0; continue; }
        const double vx = vxf, vy = vyf, vz = vzf;
        acc[0] += mass * vx; acc[1] += mass * vy; acc[2] += mass * vz;
        acc[3] += 0.5 * mass * (vx * vx + vy * vy + vz * vz);
        acc[4] -= mass * (gx * px + gy * py + gz * pz);
        acc[5] += rho;
        acc[6] = fmin(acc[6], (double)rho);
        acc[7] = fmax(acc[7], (double)rho);
        acc[8] += fabs((double)rho - rho0) / rho0;
        acc[10] += 1.0;
        acc[11] += (double)rho * rho;
    }
    __shared__ double sh[kNoAllocThreads];
    for (int f = 0; f < kDiagFields; ++f) {
        sh[threadIdx.x] = acc[f];
        __syncthreads();
        for (int o = kNoAllocThreads / 2; o > 0; o >>= 1) {
            if (threadIdx.x < o) {
                const double x = sh[threadIdx.x], y = sh[threadIdx.x + o];
                sh[threadIdx.x] = f == 6 ? fmin(x, y) : (f == 7 ? fmax(x, y) : x + y);
            }
            __syncthreads();
        }
        if (threadIdx.x == 0) partials[(size_t)blockIdx.x * kDiagFields + f] = sh[0];
        __syncthreads();
    }
}

__global__ void k_noalloc_final(const double* __restrict__ partials, int nblocks, double* __restrict__ out) {
    const int f = threadIdx.x;
    if (f >= kDiagFields) return;
    double r = f == 6 ? INFINITY : (f == 7 ? -INFINITY : 0.0);
    for (int c = 0; c < nblocks; ++c) {
        const double x = partials[(size_t)c * kDiagFields + f];
        r = f == 6 ? fmin(r, x) : (f == 7 ? fmax(r, x) : r + x);
    }
    out[f] = r;
}

// The device address of the scratch in the context current on the calling thread. In host
// code the array's name is only a host-side stand-in, not a device address. The address is
// looked up on every call, not kept: each context that loads the library has its own copy
// of the array (a caller's own driver context on a device differs from the device's primary
// context), and after cudaDeviceReset the old address is gone. The first lookup in a
// context loads the library's module there; later ones are a table lookup.
cudaError_t noalloc_scratch(double** out) {
    double* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress((void**)&p, g_noalloc_partials);
    if (e != cudaSuccess) return e;
    *out = p;
    return cudaSuccess;
}

}  // namespace
}  // namespace sphgb

using namespace sphgb;

extern "C" sph_status sph_reduce_aos_noalloc(const sph_particle* dev_particles, uint32_t n, const sph_params* p,
                                             double* dev_sums, void* stream) {
    if (!dev_particles || !p || !dev_sums) return SPH_ERR_INVALID_ARG;
    if ((long long)n > kNoAllocMaxParticles) return SPH_ERR_CAPACITY;
    if (!(p->resting_rho > 0.0f)) return SPH_ERR_INVALID_ARG;
    double* scratch = nullptr;
    if (noalloc_scratch(&scratch) != cudaSuccess) return SPH_ERR_CUDA;
    const cudaStream_t st = (cudaStream_t)stream;
    const int nblocks = n == 0 ? 0 : (int)((n + kNoAllocPerBlock - 1) / kNoAllocPerBlock);
    if (nblocks > 0)
        k_noalloc_partial<<<nblocks, kNoAllocThreads, 0, st>>>(dev_particles, (int)n, (double)p->mass,
                                                               (double)p->resting_rho, (double)p->gravity[0],
                                                               (double)p->gravity[1], (double)p->gravity[2], scratch);
    k_noalloc_final<<<1, 32, 0, st>>>(scratch, nblocks, dev_sums);
    return cudaGetLastError() == cudaSuccess ? SPH_OK : SPH_ERR_CUDA;
}
