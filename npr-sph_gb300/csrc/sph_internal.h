// sph_internal.h -- device-side parameter block, buffer set and kernel
// launchers shared by the translation units of libsph_gb300.so.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/sph_gb300.h"

namespace sphgb {

// Error bits of the device error word (ORed by kernels, read by the host).
enum : uint32_t {
    ERR_BAD_CELL = 1u << 1,    // a cell key fell outside its scene's cell range
    ERR_BAD_SLOT = 1u << 2,    // a slot/rank outside [0, n)
};

// Per-scene constants of one step, derived on the host from sph_params
// (all FP32; coefficients computed in FP64 then rounded).
struct SceneDev {
    float h;          // smoothing_coeff * particle_radius (rho_pres_comp.glsl:40), FP32 product
    float cut_d2;     // smallest float T with sqrtf(T) >= h: neighbour iff d2 < T
    float h2;         // h*h
    float inv_edge;   // 1 / cell edge
    float lo[3];      // lower wall (BoundaryUniform.lower), also the grid origin
    float up[3];      // upper wall
    int dim[3];       // cells per axis
    int cell_base;    // first cell key of this scene in the global cell table
    int first;        // first particle slot of this scene (sorted order)
    int count;        // particles of this scene
    float poly6c;     // mass*315/(64*PI*h^9)                  (rho_pres_comp.glsl:52)
    float gas_k;      // GAS_CONST                              (rho_pres_comp.glsl:33)
    float rho0;       // resting_rho
    float pres_c;     // mass*45/(PI*h^6)/2: f_p += pres_c*(p_i+p_j)/rho_j*(h-r)^2*d/r (force_comp.glsl:59)
    float visc_c;     // visc*mass*45/(PI*h^6): f_v += visc_c*(v_j-v_i)/rho_j*(h-r)   (force_comp.glsl:60,63)
    float g[3];       // G                                      (force_comp.glsl:33)
    float dt;         // integrate_comp.glsl:33
    float damp;       // DAMPING (integrate_comp.glsl:8)
    float mass;
    int keep_force;
    int row_base;     // first cell row (y, z) of this scene in the global row numbering
    int pad_;
    // Static obstacle (sph_set_obstacle): signed distance samples, null when there is none.
    const float* sdf; // [sdim z][sdim y][sdim x], device memory, negative inside
    int sdim[3];
    float sorg[3];    // position of sample (0, 0, 0)
    float sinv;       // 1 / sample spacing
};

// Device buffers of one engine (single scene or a batch of scenes).
// Sorted state lives in (pos_s, vel_s); the integrated state in (pos, vel).
// pos.w carries the scene index and vel.w the particle id, both as int bits.
struct Buffers {
    float4* pos = nullptr;     // state after the last step (slot order of the last sort)
    float4* vel = nullptr;
    float4* pos_s = nullptr;   // state sorted by cell (this step)
    float4* vel_s = nullptr;
    float2* rhop = nullptr;    // (rho, pres) in the sorted slot order of the last step
    float4* force_s = nullptr; // SPH_FLAG_KEEP_FORCE: force of the last step, sorted slot order
    float4* force_up = nullptr;// force as uploaded, id order (returned when not kept)
    float4* aux = nullptr;     // id order: uploaded (pos.w, vel.w, extras[2], extras[3])
    sph_particle* aos = nullptr;  // device AoS staging for host uploads/downloads
    int* key = nullptr;        // cell key of pos[s]
    int* rank = nullptr;       // arrival rank of s within its cell
    int* perm = nullptr;       // sorted slot -> state slot (before stabilising)
    int* count = nullptr;      // particles per cell (zero between steps)
    int* start = nullptr;      // first sorted slot of each cell; start[ncell] = n
    unsigned long long* scan_state = nullptr;  // per-tile sums of the scan (one 8-byte slot per tile)
    int* slot_of_id = nullptr; // id -> sorted slot (neighbour queries)
    uint32_t* err = nullptr;   // device error word
    double* partials = nullptr;// reduction partials
    SceneDev* scenes = nullptr;// scene table (batched mode)
    int n = 0;
    int ncell = 0;
    int nscene = 1;
    uint32_t* tile_stats = nullptr;  // [0] chunks staged, [1] chunks on the global-memory path
    uint32_t* pmask = nullptr; // [kPairMaskWords][n]: the density pass's neighbour predicates for the force pass
    float4* rec = nullptr;     // [n][2]: (x, y, z, p), (vx, vy, vz, 1/rho) per sorted slot, written by the
                               // density pass (stencil 1) for the force pass's neighbour reads
    unsigned long long* cell_pairs_map = nullptr;  // host-mapped: the last sort's sum over cells of count^2
};

// Stencil 1 (cells of edge h): the density pass stores, per particle and per neighbour-row
// segment, which candidates passed r < h as two 32-bit masks (even and odd candidates), and the
// force pass reads them instead of testing the candidates again.
constexpr int kPairMaskWords = 2 * 9;

// The neighbour records cost the density pass a fixed 48 bytes per particle (velocity read,
// record write) and save the force pass a part of every neighbour read: they pay in dense fluid.
// A step uses them when the last sort the host has seen found more than this many same-cell
// pairs per particle (sum over cells of count^2 over n, self included). On the 1M dam break
// pairs within h run at ~3.7 times that (8 on its starting 0.5h lattice, ~29 neighbours), and the
// records pay down to ~10 pairs within h. The choice changes only the speed: both forms compute
// the same interactions from the same values.
constexpr double kRecordCellPairs = 2.6;

// Launch shape chosen by the autotuner.
struct LaunchCfg {
    int block = 256;     // threads per CTA of the pair kernels (particles per shared-memory tile)
    int stencil = 1;     // cell edge = h/stencil, (2*stencil+1)^3 cells visited
};

constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;   // 2048 cells per tile: a 1M-cell grid is 512 tiles, 3 or 4 per SM
constexpr int kScanTile = kScanThreads * kScanItems;

// ---- launchers (sph_grid.cu) ----
void launch_hash(const Buffers& b, const SceneDev& s0, bool batched, cudaStream_t st);
void launch_scan(const Buffers& b, cudaStream_t st);
void launch_scatter(const Buffers& b, cudaStream_t st);
void launch_gather(const Buffers& b, cudaStream_t st);
void launch_slot_of_id(const Buffers& b, cudaStream_t st);
void launch_neighbor_digest(const Buffers& b, const SceneDev& s0, bool batched, int stencil,
                            const uint32_t* qids, int nq, int brute, uint32_t* cnt,
                            unsigned long long* dig, cudaStream_t st);
// Per query id: cnt[q] = src_cnt[slot_of_id[id]], dig[q] = src_sum[...] (0xffffffff / 0 for a
// bad id).
// Candidate tests and r < h pairs (self included) of the density pass at the sorted positions,
// added to out[0], out[1] (device; measurement only).
void launch_pair_counts(const Buffers& b, const SceneDev& s0, bool batched, int stencil, unsigned long long* out,
                        cudaStream_t st);
void launch_query_gather(const Buffers& b, const uint32_t* qids, int nq, const uint32_t* src_cnt,
                         const unsigned long long* src_sum, uint32_t* cnt, unsigned long long* dig, cudaStream_t st);
// ---- launchers (sph_step.cu) ----
// Kernel attributes (shared-memory opt-in); called once per process before any capture.
void init_step_kernels();
// rec (stencil 1): the density pass also writes the neighbour records and the force pass reads
// them; a step's two passes take the same rec.
void launch_density(const Buffers& b, const SceneDev& s0, bool batched, const LaunchCfg& c, bool rec,
                    cudaStream_t st);
// With dig_cnt/dig_sum (per sorted slot; stencil 1 only, without records), the force pass also
// reports the neighbour set it used: count (self included) and digest sum mix64(id).
void launch_force_integrate(const Buffers& b, const SceneDev& s0, bool batched, const LaunchCfg& c, bool rec,
                            cudaStream_t st, uint32_t* dig_cnt = nullptr, unsigned long long* dig_sum = nullptr);
// Density (bit-identical to launch_density) plus, per particle, the kNbList nearest neighbours
// j != i with r < h as sorted slots into nb[n][kNbList] (-1 padded) and their number in cnt
// (the learned macro-step's input), with the launch shape of launch_density.
constexpr int kNbList = 32;
void launch_density_nb(const Buffers& b, const SceneDev& s0, bool batched, const LaunchCfg& c, int* nb, int* cnt,
                       cudaStream_t st);
// ---- launchers (sph_io.cu) ----
// Per-scene FP64 sums into out[nscene * kDiagFields] (device), deterministic:
// 0-2 sum m v, 3 kinetic, 4 potential, 5 sum rho, 6 min rho, 7 max rho,
// 8 sum |rho-rho0|/rho0, 9 non-finite count, 10 finite count, 11 sum rho^2.
constexpr int kDiagFields = 12;
void launch_reduce(const Buffers& b, const SceneDev* host_scenes, int nscene, double* out_dev,
                   cudaStream_t st);
size_t reduce_partials_doubles(int nscene);
// Records [i0, i1) of aos_dev into the state (record i becomes slot i, particle id i).
void launch_aos_to_soa(const Buffers& b, const sph_particle* aos_dev, const int* scene_first, int i0, int i1,
                       cudaStream_t st);
void launch_soa_to_aos(const Buffers& b, bool force_from_step, sph_particle* aos_dev, cudaStream_t st);
// The same records by particle id: slot_of_id from the state's ids, then records [i0, i1).
void launch_slot_of_state_id(const Buffers& b, cudaStream_t st);
void launch_soa_to_aos_ids(const Buffers& b, bool force_from_step, sph_particle* aos_dev, int i0, int i1,
                           cudaStream_t st);
// Chunks of a host upload or download (copies overlap the conversion of the other chunks).
constexpr int kXferChunks = 4;

int device_sm_count();

}  // namespace sphgb
