// sph_grid.cu -- the uniform-grid neighbour structure, rebuilt every step.
//
// The reference has no spatial structure: each invocation loops over all N
// particles (rho_pres_comp.glsl:46, force_comp.glsl:48). Here the particles
// are counting-sorted by cell each step:
//   hash     key = linearised cell of pos, rank = atomicAdd(count[key], 1)
//            (fused into the integrate epilogue of the previous step; this
//            kernel only runs after an upload or a neighbour query)
//   scan     start = exclusive prefix sum of count (tile sums, then each tile
//            adds the sums before it); zeroes count for the next step
//   scatter  perm[start[key] + rank] = s
//   gather   stable: within a cell, particles keep their previous slot order,
//            so the sort is deterministic; copies pos/vel into sorted order.
// All integer work: HBM-bound, coalesced, grid sized for the whole GPU.
#include <cstdio>

#include "sph_device.cuh"

namespace sphgb {

namespace {

constexpr int kThreads = 256;

inline int blocks_for(long long n, int threads) {
    long long b = (n + threads - 1) / threads;
    return (int)(b < 1 ? 1 : b);
}

template <bool BATCHED>
__global__ void __launch_bounds__(kThreads) k_hash(const float4* __restrict__ pos, int n, SceneDev s0,
                                                   const SceneDev* __restrict__ scenes, int nscene,
                                                   int* __restrict__ key, int* __restrict__ rank,
                                                   int* __restrict__ count) {
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x) {
        float4 p = pos[s];
        int sc = 0;
        if constexpr (BATCHED) sc = min(max(scene_of(p), 0), nscene - 1);
        const SceneDev& S = scene_params<BATCHED>(s0, scenes, sc);
        int c = cell_key(S, p.x, p.y, p.z);
        key[s] = c;
        rank[s] = atomicAdd(&count[c], 1);
    }
}

// Exclusive scan of count[0, ncell) into start[0, ncell], start[ncell] = total, count
// zeroed on the way, in two launches over tiles of kScanTile cells (tile = blockIdx.x):
//   k_scan_tiles  the sum of each tile's counts -> tile_sum[tile]
//   k_scan_apply  each tile adds up the sums of the tiles before it (at most a few thousand
//                 ints, read by the whole CTA), scans its own counts and writes start.
// No tile waits for another, so nothing can spin; the counts are read twice, the second
// time from L2 (4 bytes per cell).
__device__ __forceinline__ void load_tile_counts(const int* __restrict__ count, long long base, int ncell,
                                                 int (&v)[kScanItems]) {
    if (base + kScanItems <= ncell && ((base & 3) == 0)) {
        const int4* c4 = reinterpret_cast<const int4*>(count + base);
#pragma unroll
        for (int k = 0; k < kScanItems / 4; ++k) {
            const int4 q = c4[k];
            v[4 * k] = q.x; v[4 * k + 1] = q.y; v[4 * k + 2] = q.z; v[4 * k + 3] = q.w;
        }
    } else {
#pragma unroll
        for (int k = 0; k < kScanItems; ++k) v[k] = base + k < ncell ? count[base + k] : 0;
    }
}

// Block-wide sum of one int per thread (every thread gets the total).
__device__ __forceinline__ int block_sum(int x, int* s_warp) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    if (lane == 0) s_warp[warp] = x;
    __syncthreads();
    int t = 0;
#pragma unroll
    for (int w = 0; w < kScanThreads / 32; ++w) t += s_warp[w];
    __syncthreads();
    return t;
}

// Also the tile's same-cell pairs, the sum of count^2 over its cells (self included), into
// tile_sq[tile].
__global__ void __launch_bounds__(kScanThreads) k_scan_tiles(const int* __restrict__ count, int ncell,
                                                             int* __restrict__ tile_sum,
                                                             unsigned* __restrict__ tile_sq) {
    __shared__ int s_warp[kScanThreads / 32];
    __shared__ unsigned s_sq[kScanThreads / 32];
    const long long base = (long long)blockIdx.x * kScanTile + (long long)threadIdx.x * kScanItems;
    int v[kScanItems];
    load_tile_counts(count, base, ncell, v);
    int sum = 0;
    unsigned sq = 0;  // a cell counts at most 1024^2: a tile's 2048 cells stay below 2^31
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        sum += v[k];
        const unsigned c = (unsigned)min(max(v[k], 0), 1024);
        sq += c * c;
    }
    sq = __reduce_add_sync(0xffffffffu, sq);
    if ((threadIdx.x & 31) == 0) s_sq[threadIdx.x >> 5] = sq;
    const int total = block_sum(sum, s_warp);  // its barrier also publishes s_sq
    if (threadIdx.x == 0) {
        unsigned t = 0;
#pragma unroll
        for (int w = 0; w < kScanThreads / 32; ++w) t += s_sq[w];
        tile_sum[blockIdx.x] = total;
        tile_sq[blockIdx.x] = t;
    }
}

// The last tile's block also adds up the tiles' same-cell pairs and writes the sum to host-mapped
// memory (*cell_pairs_map: the host's choice of the neighbour-record form of the next steps).
__global__ void __launch_bounds__(kScanThreads) k_scan_apply(int* __restrict__ count, int* __restrict__ start, int ncell,
                                                             const int* __restrict__ tile_sum,
                                                             const unsigned* __restrict__ tile_sq,
                                                             unsigned long long* __restrict__ cell_pairs_map) {
    __shared__ int s_warp[kScanThreads / 32];
    __shared__ unsigned long long s_sq[kScanThreads / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int tile = blockIdx.x;
    int before = 0;
    for (int t = threadIdx.x; t < tile; t += kScanThreads) before += tile_sum[t];
    if (tile == (int)gridDim.x - 1) {  // uniform per block
        unsigned long long sq = 0;
        for (int t = threadIdx.x; t < (int)gridDim.x; t += kScanThreads) sq += tile_sq[t];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) sq += __shfl_xor_sync(0xffffffffu, sq, o);
        if (lane == 0) s_sq[warp] = sq;
        __syncthreads();
        if (threadIdx.x == 0) {
            unsigned long long t = 0;
#pragma unroll
            for (int w = 0; w < kScanThreads / 32; ++w) t += s_sq[w];
            *cell_pairs_map = t;
        }
    }
    const int prefix = block_sum(before, s_warp);
    const long long base = (long long)tile * kScanTile + (long long)threadIdx.x * kScanItems;
    int v[kScanItems];
    load_tile_counts(count, base, ncell, v);
    if (base + kScanItems <= ncell && ((base & 3) == 0)) {
        int4* z4 = reinterpret_cast<int4*>(count + base);
#pragma unroll
        for (int k = 0; k < kScanItems / 4; ++k) z4[k] = make_int4(0, 0, 0, 0);
    } else {
#pragma unroll
        for (int k = 0; k < kScanItems; ++k)
            if (base + k < ncell) count[base + k] = 0;
    }
    int sum = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) sum += v[k];
    // block-wide exclusive scan of the per-thread sums
    int incl = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
    }
    if (lane == 31) s_warp[warp] = incl;
    __syncthreads();
    int warp_excl = 0;
#pragma unroll
    for (int w = 0; w < kScanThreads / 32; ++w) warp_excl += w < warp ? s_warp[w] : 0;
    int run = prefix + warp_excl + incl - sum;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        const long long idx = base + k;
        if (idx < ncell) start[idx] = run;
        run += v[k];
        if (idx == ncell - 1) start[ncell] = run;
    }
}

__global__ void __launch_bounds__(kThreads) k_scatter(const int* __restrict__ key, const int* __restrict__ rank,
                                                      const int* __restrict__ start, int* __restrict__ perm,
                                                      int n, uint32_t* err) {
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x) {
        int t = start[key[s]] + rank[s];
        if (t >= 0 && t < n) perm[t] = s;
        else raise_err(err, ERR_BAD_SLOT);
    }
}

// Stable placement: the particle at sorted slot t (arrival order) moves to
// start[c] + #{u in cell c : perm[u] < perm[t]}, i.e. cells keep the previous
// slot order. Then pos/vel are copied into that slot.
__global__ void __launch_bounds__(kThreads) k_gather(const int* __restrict__ perm, const int* __restrict__ key,
                                                     const int* __restrict__ start, const float4* __restrict__ pos,
                                                     const float4* __restrict__ vel, float4* __restrict__ pos_s,
                                                     float4* __restrict__ vel_s, int n, uint32_t* err) {
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        int s = perm[t];
        if (s < 0 || s >= n) { raise_err(err, ERR_BAD_SLOT); continue; }
        int c = key[s];
        int a = max(start[c], 0), b = min(start[c + 1], n);
        int r = 0;
        for (int u = a; u < b; ++u) r += (perm[u] < s);
        int dst = a + r;
        if (dst >= n) { raise_err(err, ERR_BAD_SLOT); continue; }
        pos_s[dst] = pos[s];
        vel_s[dst] = vel[s];
    }
}

__global__ void __launch_bounds__(kThreads) k_slot_of_id(const float4* __restrict__ vel_s, int* __restrict__ slot_of_id,
                                                         int n) {
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        int id = id_of(vel_s[t]);
        if (id >= 0 && id < n) slot_of_id[id] = t;
    }
}

__global__ void __launch_bounds__(kThreads) k_query_gather(const int* __restrict__ slot_of_id,
                                                           const uint32_t* __restrict__ qids, int nq, int n,
                                                           const uint32_t* __restrict__ src_cnt,
                                                           const unsigned long long* __restrict__ src_sum,
                                                           uint32_t* __restrict__ cnt, unsigned long long* __restrict__ dig) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nq) return;
    const int qi = (int)qids[q];
    const int t = qi >= 0 && qi < n ? slot_of_id[qi] : -1;
    cnt[q] = t >= 0 && t < n ? src_cnt[t] : 0xffffffffu;
    dig[q] = t >= 0 && t < n ? src_sum[t] : 0ull;
}

// Neighbour count + digest over the grid (the same stencil walk as the step).
template <bool BATCHED>
__global__ void __launch_bounds__(kThreads) k_digest_grid(const float4* __restrict__ pos_s, const float4* __restrict__ vel_s,
                                                          const int* __restrict__ start, const int* __restrict__ slot_of_id,
                                                          SceneDev s0, const SceneDev* __restrict__ scenes, int nscene,
                                                          int R, const uint32_t* __restrict__ qids, int nq, int n,
                                                          uint32_t* __restrict__ cnt, unsigned long long* __restrict__ dig) {
    int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nq) return;
    int qi = (int)qids[q];
    if (qi < 0 || qi >= n) { cnt[q] = 0xffffffffu; dig[q] = 0; return; }
    int t = slot_of_id[qi];
    if (t < 0 || t >= n) { cnt[q] = 0xffffffffu; dig[q] = 0; return; }
    float4 p = pos_s[t];
    int sc = 0;
    if constexpr (BATCHED) sc = min(max(scene_of(p), 0), nscene - 1);
    const SceneDev& S = scene_params<BATCHED>(s0, scenes, sc);
    int cx = cell_coord(p.x, S.lo[0], S.inv_edge, S.dim[0]);
    int cy = cell_coord(p.y, S.lo[1], S.inv_edge, S.dim[1]);
    int cz = cell_coord(p.z, S.lo[2], S.inv_edge, S.dim[2]);
    uint32_t c = 0;
    unsigned long long d = 0;
    for (int z = max(cz - R, 0); z <= min(cz + R, S.dim[2] - 1); ++z)
        for (int y = max(cy - R, 0); y <= min(cy + R, S.dim[1] - 1); ++y) {
            int row = S.cell_base + S.dim[0] * (y + S.dim[1] * z);
            int a = max(start[row + max(cx - R, 0)], 0);
            int b = min(start[row + min(cx + R, S.dim[0] - 1) + 1], n);
            for (int j = a; j < b; ++j) {
                float4 o = pos_s[j];
                float dx, dy, dz;
                float d2 = canon_d2(p.x, p.y, p.z, o.x, o.y, o.z, dx, dy, dz);
                if (d2 < S.cut_d2) { ++c; d += mix64((unsigned long long)id_of(vel_s[j])); }
            }
        }
    cnt[q] = c;
    dig[q] = d;
}

// All-pairs check (the reference's j-loop): candidates of query q are every
// slot of q's scene, staged through shared memory in tiles shared by the CTA.
constexpr int kBruteTile = 1024;
template <bool BATCHED>
__global__ void __launch_bounds__(kThreads) k_digest_brute(const float4* __restrict__ pos_s, const float4* __restrict__ vel_s,
                                                           const int* __restrict__ start, const int* __restrict__ slot_of_id,
                                                           SceneDev s0, const SceneDev* __restrict__ scenes, int nscene,
                                                           const uint32_t* __restrict__ qids, int nq, int n,
                                                           uint32_t* __restrict__ cnt, unsigned long long* __restrict__ dig) {
    __shared__ float4 tile_p[kBruteTile];
    __shared__ int tile_id[kBruteTile];
    __shared__ int s_lo, s_hi;
    int q = blockIdx.x * blockDim.x + threadIdx.x;
    bool live = q < nq;
    int qi = live ? (int)qids[q] : 0;
    if (qi < 0 || qi >= n) live = false;
    float4 p = make_float4(0.f, 0.f, 0.f, 0.f);
    int a = 0, b = 0;
    float cut = s0.cut_d2;
    int slot = live ? slot_of_id[qi] : 0;
    if (slot < 0 || slot >= n) live = false;
    if (live) {
        p = pos_s[slot];
        int sc = 0;
        if constexpr (BATCHED) sc = min(max(scene_of(p), 0), nscene - 1);
        const SceneDev& S = scene_params<BATCHED>(s0, scenes, sc);
        cut = S.cut_d2;
        a = max(start[S.cell_base], 0);
        b = min(start[S.cell_base + S.dim[0] * S.dim[1] * S.dim[2]], n);
    }
    if (threadIdx.x == 0) { s_lo = n; s_hi = 0; }
    __syncthreads();
    if (live) { atomicMin(&s_lo, a); atomicMax(&s_hi, b); }
    __syncthreads();
    const int lo = s_lo, hi = s_hi;
    uint32_t c = 0;
    unsigned long long d = 0;
    for (int j0 = lo; j0 < hi; j0 += kBruteTile) {
        int m = min(kBruteTile, hi - j0);
        for (int k = threadIdx.x; k < m; k += blockDim.x) {
            tile_p[k] = pos_s[j0 + k];
            tile_id[k] = id_of(vel_s[j0 + k]);
        }
        __syncthreads();
        if (live) {
            for (int k = 0; k < m; ++k) {
                int j = j0 + k;
                float4 o = tile_p[k];
                float dx, dy, dz;
                float d2 = canon_d2(p.x, p.y, p.z, o.x, o.y, o.z, dx, dy, dz);
                if (d2 < cut && j >= a && j < b) { ++c; d += mix64((unsigned long long)tile_id[k]); }
            }
        }
        __syncthreads();
    }
    if (q < nq) {
        cnt[q] = live ? c : 0xffffffffu;
        dig[q] = live ? d : 0ull;
    }
}

// Work counters of the density pass at the current (sorted) positions: out[0] += the
// candidate tests (the particles of cells cx-R..cx+R of every stencil row, as the pass scans
// them), out[1] += the pairs with r < h (self included). Measurement only.
template <bool BATCHED>
__global__ void __launch_bounds__(kThreads) k_pair_counts(const float4* __restrict__ pos_s, const int* __restrict__ start,
                                                          SceneDev s0, const SceneDev* __restrict__ scenes, int nscene,
                                                          int R, int n, unsigned long long* __restrict__ out) {
    unsigned long long cand = 0, pairs = 0;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        const float4 p = pos_s[t];
        int sc = 0;
        if constexpr (BATCHED) sc = min(max(scene_of(p), 0), nscene - 1);
        const SceneDev& S = scene_params<BATCHED>(s0, scenes, sc);
        const int cx = cell_coord(p.x, S.lo[0], S.inv_edge, S.dim[0]);
        const int cy = cell_coord(p.y, S.lo[1], S.inv_edge, S.dim[1]);
        const int cz = cell_coord(p.z, S.lo[2], S.inv_edge, S.dim[2]);
        for (int z = max(cz - R, 0); z <= min(cz + R, S.dim[2] - 1); ++z)
            for (int y = max(cy - R, 0); y <= min(cy + R, S.dim[1] - 1); ++y) {
                const int row = S.cell_base + S.dim[0] * (y + S.dim[1] * z);
                const int a = max(start[row + max(cx - R, 0)], 0);
                const int b = min(start[row + min(cx + R, S.dim[0] - 1) + 1], n);
                cand += (unsigned long long)max(b - a, 0);
                for (int j = a; j < b; ++j) {
                    const float4 o = pos_s[j];
                    float dx, dy, dz;
                    pairs += canon_d2(p.x, p.y, p.z, o.x, o.y, o.z, dx, dy, dz) < S.cut_d2 ? 1ull : 0ull;
                }
            }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        cand += __shfl_xor_sync(0xffffffffu, cand, o);
        pairs += __shfl_xor_sync(0xffffffffu, pairs, o);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(out, cand);
        atomicAdd(out + 1, pairs);
    }
}

}  // namespace

int device_sm_count() {
    static int sms = 0;
    if (!sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (sms <= 0) sms = 1;
    }
    return sms;
}

static int grid_for(int n) {
    // Grid-stride kernels: at most 8 resident 256-thread CTAs per SM.
    int cap = device_sm_count() * 8;
    int b = blocks_for(n, kThreads);
    return b < cap ? b : cap;
}

void launch_hash(const Buffers& b, const SceneDev& s0, bool batched, cudaStream_t st) {
    if (b.n <= 0) return;
    if (batched)
        k_hash<true><<<grid_for(b.n), kThreads, 0, st>>>(b.pos, b.n, s0, b.scenes, b.nscene, b.key, b.rank, b.count);
    else
        k_hash<false><<<grid_for(b.n), kThreads, 0, st>>>(b.pos, b.n, s0, b.scenes, 1, b.key, b.rank, b.count);
}

void launch_scan(const Buffers& b, cudaStream_t st) {
    const int ntiles = (b.ncell + kScanTile - 1) / kScanTile;
    // ntiles 8-byte slots: the tiles' particle counts (int), then their same-cell pairs (unsigned)
    int* tile_sum = reinterpret_cast<int*>(b.scan_state);
    unsigned* tile_sq = reinterpret_cast<unsigned*>(b.scan_state) + ntiles;
    k_scan_tiles<<<ntiles, kScanThreads, 0, st>>>(b.count, b.ncell, tile_sum, tile_sq);
    k_scan_apply<<<ntiles, kScanThreads, 0, st>>>(b.count, b.start, b.ncell, tile_sum, tile_sq, b.cell_pairs_map);
}

void launch_scatter(const Buffers& b, cudaStream_t st) {
    if (b.n <= 0) return;
    k_scatter<<<grid_for(b.n), kThreads, 0, st>>>(b.key, b.rank, b.start, b.perm, b.n, b.err);
}

void launch_gather(const Buffers& b, cudaStream_t st) {
    if (b.n <= 0) return;
    k_gather<<<grid_for(b.n), kThreads, 0, st>>>(b.perm, b.key, b.start, b.pos, b.vel, b.pos_s, b.vel_s, b.n, b.err);
}

void launch_query_gather(const Buffers& b, const uint32_t* qids, int nq, const uint32_t* src_cnt,
                         const unsigned long long* src_sum, uint32_t* cnt, unsigned long long* dig, cudaStream_t st) {
    if (nq <= 0) return;
    k_query_gather<<<(nq + kThreads - 1) / kThreads, kThreads, 0, st>>>(b.slot_of_id, qids, nq, b.n, src_cnt, src_sum,
                                                                         cnt, dig);
}

void launch_slot_of_id(const Buffers& b, cudaStream_t st) {
    if (b.n <= 0) return;
    k_slot_of_id<<<grid_for(b.n), kThreads, 0, st>>>(b.vel_s, b.slot_of_id, b.n);
}

void launch_neighbor_digest(const Buffers& b, const SceneDev& s0, bool batched, int stencil, const uint32_t* qids,
                            int nq, int brute, uint32_t* cnt, unsigned long long* dig, cudaStream_t st) {
    if (nq <= 0) return;
    int blocks = blocks_for(nq, kThreads);
    if (brute) {
        if (batched)
            k_digest_brute<true><<<blocks, kThreads, 0, st>>>(b.pos_s, b.vel_s, b.start, b.slot_of_id, s0, b.scenes,
                                                              b.nscene, qids, nq, b.n, cnt, dig);
        else
            k_digest_brute<false><<<blocks, kThreads, 0, st>>>(b.pos_s, b.vel_s, b.start, b.slot_of_id, s0, b.scenes, 1,
                                                               qids, nq, b.n, cnt, dig);
    } else {
        if (batched)
            k_digest_grid<true><<<blocks, kThreads, 0, st>>>(b.pos_s, b.vel_s, b.start, b.slot_of_id, s0, b.scenes,
                                                             b.nscene, stencil, qids, nq, b.n, cnt, dig);
        else
            k_digest_grid<false><<<blocks, kThreads, 0, st>>>(b.pos_s, b.vel_s, b.start, b.slot_of_id, s0, b.scenes, 1,
                                                              stencil, qids, nq, b.n, cnt, dig);
    }
}

void launch_pair_counts(const Buffers& b, const SceneDev& s0, bool batched, int stencil, unsigned long long* out,
                        cudaStream_t st) {
    if (b.n <= 0) return;
    if (batched)
        k_pair_counts<true><<<grid_for(b.n), kThreads, 0, st>>>(b.pos_s, b.start, s0, b.scenes, b.nscene, stencil, b.n,
                                                                out);
    else
        k_pair_counts<false><<<grid_for(b.n), kThreads, 0, st>>>(b.pos_s, b.start, s0, b.scenes, 1, stencil, b.n, out);
}

}  // namespace sphgb
