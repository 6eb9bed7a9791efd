// sph_obstacle.cu -- signed distance field of a closed triangle mesh on a regular
// grid (sph_sdf_from_mesh), the input of sph_set_obstacle.
//
// The reference loads triangle meshes with assimp (LoadMesh.cpp:16-55) and lists
// "objects to collide with" as future work (README.md:59). Here a mesh becomes a
// static obstacle of the SPH step through its signed distance field:
//   |phi(p)| = min over triangles of the distance from p to the triangle, by the
//              closest-point construction of Ericson, Real-Time Collision Detection
//              (2005), section 5.1.5 (Voronoi regions of the vertices, edges and face);
//   sign     = negative where the generalised winding number w(p) = sum of the
//              triangles' solid angles / (4 pi) exceeds 1/2; the solid angle of a
//              triangle (a, b, c) seen from p is 2 atan2(det[a b c], |a||b||c| +
//              (a.b)|c| + (a.c)|b| + (b.c)|a|) with a, b, c relative to p (Van Oosterom
//              and Strackee, IEEE Trans. Biomed. Eng. 30 (1983) 125-126), positive for a
//              triangle counter-clockwise seen from outside and p inside.
// One thread per grid sample; the triangles pass through shared memory in tiles
// that every thread of the CTA reads.
#include <cmath>
#include <string>
#include <vector>

#include "sph_device.cuh"

namespace sphgb {
namespace {

constexpr int kSdfThreads = 256;
constexpr int kTriTile = 256;

struct V3 {
    float x, y, z;
};
__device__ __forceinline__ V3 sub(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ V3 cross(V3 a, V3 b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
__device__ __forceinline__ V3 axpy(float s, V3 d, V3 a) { return {a.x + s * d.x, a.y + s * d.y, a.z + s * d.z}; }

// Squared distance from p to triangle (a, b, c): the closest point by Voronoi region.
__device__ float tri_dist2(V3 p, V3 a, V3 b, V3 c) {
    const V3 ab = sub(b, a), ac = sub(c, a), ap = sub(p, a);
    const float d1 = dot(ab, ap), d2 = dot(ac, ap);
    V3 q;
    if (d1 <= 0.0f && d2 <= 0.0f) {
        q = a;  // vertex a
    } else {
        const V3 bp = sub(p, b);
        const float d3 = dot(ab, bp), d4 = dot(ac, bp);
        const V3 cp = sub(p, c);
        const float d5 = dot(ab, cp), d6 = dot(ac, cp);
        const float vc = d1 * d4 - d3 * d2, vb = d5 * d2 - d1 * d6, va = d3 * d6 - d5 * d4;
        if (d3 >= 0.0f && d4 <= d3) q = b;                                            // vertex b
        else if (vc <= 0.0f && d1 >= 0.0f && d3 <= 0.0f) q = axpy(d1 / (d1 - d3), ab, a);  // edge ab
        else if (d6 >= 0.0f && d5 <= d6) q = c;                                       // vertex c
        else if (vb <= 0.0f && d2 >= 0.0f && d6 <= 0.0f) q = axpy(d2 / (d2 - d6), ac, a);  // edge ac
        else if (va <= 0.0f && d4 - d3 >= 0.0f && d5 - d6 >= 0.0f)
            q = axpy((d4 - d3) / ((d4 - d3) + (d5 - d6)), sub(c, b), b);              // edge bc
        else {                                                                        // face
            const float den = 1.0f / (va + vb + vc);
            q = axpy(vc * den, ac, axpy(vb * den, ab, a));
        }
    }
    const V3 d = sub(p, q);
    return dot(d, d);
}

// Solid angle of triangle (a, b, c) seen from p.
__device__ float tri_solid_angle(V3 p, V3 a, V3 b, V3 c) {
    const V3 x = sub(a, p), y = sub(b, p), z = sub(c, p);
    const float lx = sqrtf(dot(x, x)), ly = sqrtf(dot(y, y)), lz = sqrtf(dot(z, z));
    const float num = dot(x, cross(y, z));
    const float den = lx * ly * lz + dot(x, y) * lz + dot(x, z) * ly + dot(y, z) * lx;
    return 2.0f * atan2f(num, den);
}

__global__ void __launch_bounds__(kSdfThreads) k_sdf_mesh(const float* __restrict__ verts,
                                                          const uint32_t* __restrict__ tris, int nt, int dx, int dy,
                                                          int dz, float ox, float oy, float oz, float spacing,
                                                          float* __restrict__ out) {
    __shared__ V3 ta[kTriTile], tb[kTriTile], tc[kTriTile];
    const long long total = (long long)dx * dy * dz;
    const long long g = (long long)blockIdx.x * kSdfThreads + threadIdx.x;
    const bool live = g < total;
    V3 p{0.f, 0.f, 0.f};
    if (live) {
        const int i = (int)(g % dx), j = (int)((g / dx) % dy), k = (int)(g / ((long long)dx * dy));
        p = {ox + spacing * (float)i, oy + spacing * (float)j, oz + spacing * (float)k};
    }
    float best = INFINITY, omega = 0.0f;
    for (int t0 = 0; t0 < nt; t0 += kTriTile) {
        const int m = min(kTriTile, nt - t0);
        for (int q = threadIdx.x; q < m; q += kSdfThreads) {
            const uint32_t* t = tris + 3ll * (t0 + q);
            const float* a = verts + 3ll * t[0];
            const float* b = verts + 3ll * t[1];
            const float* c = verts + 3ll * t[2];
            ta[q] = {a[0], a[1], a[2]};
            tb[q] = {b[0], b[1], b[2]};
            tc[q] = {c[0], c[1], c[2]};
        }
        __syncthreads();
        if (live)
            for (int q = 0; q < m; ++q) {
                best = fminf(best, tri_dist2(p, ta[q], tb[q], tc[q]));
                omega += tri_solid_angle(p, ta[q], tb[q], tc[q]);
            }
        __syncthreads();
    }
    if (live) {
        const float w = omega / (4.0f * 3.14159265358979f);
        const float d = sqrtf(best);
        out[g] = w > 0.5f ? -d : d;
    }
}

}  // namespace
}  // namespace sphgb

using namespace sphgb;

extern "C" sph_status sph_sdf_from_mesh(const float* verts, uint32_t nv, const uint32_t* tris, uint32_t nt,
                                        const int32_t dims[3], const float origin[3], float spacing, float* sdf_out) {
    if (!verts || !tris || !dims || !origin || !sdf_out || nv < 3 || nt < 1) return SPH_ERR_INVALID_ARG;
    long long total = 1;
    for (int a = 0; a < 3; ++a) {
        if (dims[a] < 1 || dims[a] > (1 << 20) || !std::isfinite(origin[a])) return SPH_ERR_INVALID_ARG;
        total *= dims[a];
    }
    if (total > (1ll << 28) || !(spacing > 0.0f) || !std::isfinite(spacing)) return SPH_ERR_INVALID_ARG;
    for (uint64_t q = 0; q < 3ull * nt; ++q)
        if (tris[q] >= nv) return SPH_ERR_INVALID_ARG;  // every index is checked before any launch
    float* dv = nullptr;
    uint32_t* dt = nullptr;
    float* dout = nullptr;
    sph_status st = SPH_OK;
    cudaError_t e = cudaMalloc(&dv, sizeof(float) * 3ull * nv);
    if (e == cudaSuccess) e = cudaMalloc(&dt, sizeof(uint32_t) * 3ull * nt);
    if (e == cudaSuccess) e = cudaMalloc(&dout, sizeof(float) * (size_t)total);
    if (e == cudaSuccess) e = cudaMemcpy(dv, verts, sizeof(float) * 3ull * nv, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(dt, tris, sizeof(uint32_t) * 3ull * nt, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        const long long blocks = (total + kSdfThreads - 1) / kSdfThreads;
        k_sdf_mesh<<<(unsigned)blocks, kSdfThreads>>>(dv, dt, (int)nt, dims[0], dims[1], dims[2], origin[0], origin[1],
                                                      origin[2], spacing, dout);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(sdf_out, dout, sizeof(float) * (size_t)total, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) st = e == cudaErrorMemoryAllocation ? SPH_ERR_OUT_OF_MEMORY : SPH_ERR_CUDA;
    if (dv) cudaFree(dv);
    if (dt) cudaFree(dt);
    if (dout) cudaFree(dout);
    return st;
}
