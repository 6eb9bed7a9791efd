// sph_io.cu -- AoS <-> SoA adapter at the C ABI and the FP64 diagnostics.
//
// The reference keeps one 64-byte record per particle (struct Particle,
// Main.cpp:93-99). The device state here is SoA, cell-sorted:
//   pos  float4 (x, y, z, scene index as int bits)
//   vel  float4 (vx, vy, vz, particle id as int bits)
//   rhop float2 (rho, pres)
// plus the fields the step never touches (pos.w, vel.w, extras[2..3], force as
// uploaded) kept by particle id, so a download returns the caller's record
// with the simulated fields replaced.
#include "sph_device.cuh"

namespace sphgb {

namespace {

constexpr int kThreads = 256;
constexpr int kMaxChunks = 512;  // reduction partials per scene (at most)

__device__ __forceinline__ float4 ld4(const float* f) { return *reinterpret_cast<const float4*>(f); }
__device__ __forceinline__ void st4(float* f, float4 v) { *reinterpret_cast<float4*>(f) = v; }

// Scene of record i: scene_first is ascending (nscene+1 entries).
__device__ __forceinline__ int scene_lookup(const int* __restrict__ scene_first, int nscene, int i) {
    int lo = 0, hi = nscene - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (scene_first[mid] <= i) lo = mid; else hi = mid - 1;
    }
    return lo;
}

__global__ void __launch_bounds__(kThreads) k_aos_to_soa(const sph_particle* __restrict__ aos, int i0, int i1,
                                                         const int* __restrict__ scene_first, int nscene,
                                                         float4* __restrict__ pos, float4* __restrict__ vel,
                                                         float2* __restrict__ rhop, float4* __restrict__ force_up,
                                                         float4* __restrict__ aux) {
    for (int i = i0 + blockIdx.x * blockDim.x + threadIdx.x; i < i1; i += gridDim.x * blockDim.x) {
        const sph_particle& r = aos[i];
        float4 p = ld4(r.pos), v = ld4(r.vel), f = ld4(r.force), e = ld4(r.extras);
        int sc = nscene > 1 ? scene_lookup(scene_first, nscene, i) : 0;
        pos[i] = make_float4(p.x, p.y, p.z, __int_as_float(sc));
        vel[i] = make_float4(v.x, v.y, v.z, __int_as_float(i));
        rhop[i] = make_float2(e.x, e.y);
        force_up[i] = f;
        aux[i] = make_float4(p.w, v.w, e.z, e.w);
    }
}

// Slot s of the state -> record id (the upload index).
__global__ void __launch_bounds__(kThreads) k_soa_to_aos(const float4* __restrict__ pos, const float4* __restrict__ vel,
                                                         const float2* __restrict__ rhop,
                                                         const float4* __restrict__ force_s,
                                                         const float4* __restrict__ force_up,
                                                         const float4* __restrict__ aux, int n,
                                                         sph_particle* __restrict__ aos) {
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x) {
        float4 p = pos[s], v = vel[s];
        int id = id_of(v);
        if (id < 0 || id >= n) continue;
        float2 rp = rhop[s];
        float4 x = aux[id];
        float4 fu = force_up[id];
        float4 f = force_s ? make_float4(force_s[s].x, force_s[s].y, force_s[s].z, fu.w) : fu;
        sph_particle& r = aos[id];
        st4(r.pos, make_float4(p.x, p.y, p.z, x.x));
        st4(r.vel, make_float4(v.x, v.y, v.z, x.y));
        st4(r.force, f);
        st4(r.extras, make_float4(rp.x, rp.y, x.z, x.w));
    }
}

__global__ void __launch_bounds__(kThreads) k_slot_of_state_id(const float4* __restrict__ vel, int n,
                                                               int* __restrict__ slot_of_id) {
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x) {
        const int id = id_of(vel[s]);
        if (id >= 0 && id < n) slot_of_id[id] = s;
    }
}

// k_soa_to_aos by record: record i from the slot holding particle id i.
__global__ void __launch_bounds__(kThreads) k_soa_to_aos_ids(const float4* __restrict__ pos, const float4* __restrict__ vel,
                                                             const float2* __restrict__ rhop,
                                                             const float4* __restrict__ force_s,
                                                             const float4* __restrict__ force_up,
                                                             const float4* __restrict__ aux,
                                                             const int* __restrict__ slot_of_id, int n, int i0, int i1,
                                                             sph_particle* __restrict__ aos) {
    for (int id = i0 + blockIdx.x * blockDim.x + threadIdx.x; id < i1; id += gridDim.x * blockDim.x) {
        const int s = slot_of_id[id];
        if (s < 0 || s >= n) continue;
        const float4 p = pos[s], v = vel[s];
        const float2 rp = rhop[s];
        const float4 x = aux[id];
        const float4 fu = force_up[id];
        const float4 f = force_s ? make_float4(force_s[s].x, force_s[s].y, force_s[s].z, fu.w) : fu;
        sph_particle& r = aos[id];
        st4(r.pos, make_float4(p.x, p.y, p.z, x.x));
        st4(r.vel, make_float4(v.x, v.y, v.z, x.y));
        st4(r.force, f);
        st4(r.extras, make_float4(rp.x, rp.y, x.z, x.w));
    }
}

// FP64 per-scene sums. Grid (chunks, nscene); each CTA reduces a strided
// share of its scene's slots in a fixed order (deterministic).
__global__ void __launch_bounds__(kThreads) k_reduce_partial(const float4* __restrict__ pos, const float4* __restrict__ vel,
                                                             const float2* __restrict__ rhop,
                                                             const SceneDev* __restrict__ scenes,
                                                             double* __restrict__ partials) {
    const int sc = blockIdx.y;
    const SceneDev& S = scenes[sc];
    const double m = S.mass, rho0 = S.rho0;
    double acc[kDiagFields];
#pragma unroll
    for (int f = 0; f < kDiagFields; ++f) acc[f] = 0.0;
    acc[6] = INFINITY;
    acc[7] = -INFINITY;
    const int a = S.first, b = S.first + S.count;
    for (int s = a + blockIdx.x * blockDim.x + threadIdx.x; s < b; s += gridDim.x * blockDim.x) {
        float4 p = pos[s], v = vel[s];
        float rho = rhop[s].x;
        bool fin = isfinite(p.x) && isfinite(p.y) && isfinite(p.z) && isfinite(v.x) && isfinite(v.y) &&
                   isfinite(v.z) && isfinite(rho);
        if (!fin) { acc[9] += 1.0; continue; }
        double vx = v.x, vy = v.y, vz = v.z;
        acc[0] += m * vx; acc[1] += m * vy; acc[2] += m * vz;
        acc[3] += 0.5 * m * (vx * vx + vy * vy + vz * vz);
        acc[4] -= m * ((double)S.g[0] * p.x + (double)S.g[1] * p.y + (double)S.g[2] * p.z);
        acc[5] += rho;
        acc[6] = fmin(acc[6], (double)rho);
        acc[7] = fmax(acc[7], (double)rho);
        acc[8] += fabs((double)rho - rho0) / rho0;
        acc[10] += 1.0;
        acc[11] += (double)rho * rho;
    }
    __shared__ double sh[kThreads];
    for (int f = 0; f < kDiagFields; ++f) {
        sh[threadIdx.x] = acc[f];
        __syncthreads();
        for (int o = kThreads / 2; o > 0; o >>= 1) {
            if (threadIdx.x < o) {
                double x = sh[threadIdx.x], y = sh[threadIdx.x + o];
                sh[threadIdx.x] = f == 6 ? fmin(x, y) : (f == 7 ? fmax(x, y) : x + y);
            }
            __syncthreads();
        }
        if (threadIdx.x == 0) partials[((size_t)sc * gridDim.x + blockIdx.x) * kDiagFields + f] = sh[0];
        __syncthreads();
    }
}

// One CTA per scene: thread t combines chunks t, t + kThreads, ... of every field, then a
// fixed-order tree over the threads (deterministic, like the partial sums).
__global__ void __launch_bounds__(kThreads) k_reduce_final(const double* __restrict__ partials, int chunks,
                                                           double* __restrict__ out) {
    const int sc = blockIdx.x;
    __shared__ double sh[kThreads];
    for (int f = 0; f < kDiagFields; ++f) {
        double r = f == 6 ? INFINITY : (f == 7 ? -INFINITY : 0.0);
        for (int c = threadIdx.x; c < chunks; c += kThreads) {
            const double x = partials[((size_t)sc * chunks + c) * kDiagFields + f];
            r = f == 6 ? fmin(r, x) : (f == 7 ? fmax(r, x) : r + x);
        }
        sh[threadIdx.x] = r;
        __syncthreads();
        for (int o = kThreads / 2; o > 0; o >>= 1) {
            if (threadIdx.x < o) {
                const double x = sh[threadIdx.x], y = sh[threadIdx.x + o];
                sh[threadIdx.x] = f == 6 ? fmin(x, y) : (f == 7 ? fmax(x, y) : x + y);
            }
            __syncthreads();
        }
        if (threadIdx.x == 0) out[(size_t)sc * kDiagFields + f] = sh[0];
        __syncthreads();
    }
}

}  // namespace

void launch_aos_to_soa(const Buffers& b, const sph_particle* aos_dev, const int* scene_first, int i0, int i1,
                       cudaStream_t st) {
    if (i1 <= i0) return;
    int blocks = (i1 - i0 + kThreads - 1) / kThreads;
    k_aos_to_soa<<<blocks, kThreads, 0, st>>>(aos_dev, i0, i1, scene_first, b.nscene, b.pos, b.vel, b.rhop,
                                              b.force_up, b.aux);
}

void launch_slot_of_state_id(const Buffers& b, cudaStream_t st) {
    if (b.n <= 0) return;
    k_slot_of_state_id<<<(b.n + kThreads - 1) / kThreads, kThreads, 0, st>>>(b.vel, b.n, b.slot_of_id);
}

void launch_soa_to_aos_ids(const Buffers& b, bool force_from_step, sph_particle* aos_dev, int i0, int i1,
                           cudaStream_t st) {
    if (i1 <= i0) return;
    int blocks = (i1 - i0 + kThreads - 1) / kThreads;
    k_soa_to_aos_ids<<<blocks, kThreads, 0, st>>>(b.pos, b.vel, b.rhop, force_from_step ? b.force_s : nullptr,
                                                  b.force_up, b.aux, b.slot_of_id, b.n, i0, i1, aos_dev);
}

void launch_soa_to_aos(const Buffers& b, bool force_from_step, sph_particle* aos_dev, cudaStream_t st) {
    if (b.n <= 0) return;
    int blocks = (b.n + kThreads - 1) / kThreads;
    k_soa_to_aos<<<blocks, kThreads, 0, st>>>(b.pos, b.vel, b.rhop, force_from_step ? b.force_s : nullptr, b.force_up,
                                              b.aux, b.n, aos_dev);
}

static int reduce_chunks(int nscene) {
    int c = 4 * device_sm_count() / (nscene > 0 ? nscene : 1);
    return c < 1 ? 1 : (c > kMaxChunks ? kMaxChunks : c);
}

size_t reduce_partials_doubles(int nscene) { return (size_t)nscene * reduce_chunks(nscene) * kDiagFields; }

void launch_reduce(const Buffers& b, const SceneDev*, int nscene, double* out_dev, cudaStream_t st) {
    const int chunks = reduce_chunks(nscene);
    dim3 grid(chunks, nscene);
    k_reduce_partial<<<grid, kThreads, 0, st>>>(b.pos, b.vel, b.rhop, b.scenes, b.partials);
    k_reduce_final<<<nscene, kThreads, 0, st>>>(b.partials, chunks, out_dev);
}

}  // namespace sphgb
