// sph_ctx.h -- the context behind the C ABI (private to the library), and the
// engine helpers that the learned macro-step (sph_learn.cu) reuses.
#pragma once

#include <cmath>
#include <cstdint>
#include <string>
#include <vector>

#include "sph_internal.h"

struct sph_ctx {
    int device = 0;
    std::string err;
    std::vector<sph_params> params;   // per scene
    std::vector<uint32_t> counts;     // particles per scene
    bool batched = false;
    uint32_t n_max = 0;
    sphgb::Buffers b;
    std::vector<sphgb::SceneDev> sc_h;
    sphgb::SceneDev s0{};
    sphgb::LaunchCfg cfg;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    // the step's graph without [0] and with [1] the neighbour records (captured when first used)
    cudaGraph_t graph[2] = {nullptr, nullptr};
    cudaGraphExec_t gexec[2] = {nullptr, nullptr};
    unsigned long long* pair_host = nullptr;  // mapped host word: same-cell pairs of the last sort
    uint64_t record_steps[2] = {0, 0};        // steps run with [0] / without [1] neighbour records
    int record_mode = SPH_RECORDS_AUTO;       // sph_set_record_mode
    bool have_state = false, need_hash = true, stepped = false;
    uint64_t steps = 0;
    // judge state of the learned macro-step, kept across sph_learned_step calls (cleared by uploads)
    int judge_failures = 0;  // failed judges in a row
    int judge_backoff = 0;   // plain intervals still to run before the next learned attempt
    int judge_metric = SPH_JUDGE_PARTICLE_DENSITY;  // density deviation the judge decides on
    double judge_max_rho_tol = INFINITY;        // bound on the deviation of the maximum density
    long long cell_cap = 0;
    int tile_cap = 0;
    double* diag_dev = nullptr;
    int* scene_first_dev = nullptr;
    bool timing = false;
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
    // host uploads/downloads: record chunks copied on their own stream while the next (or the
    // previous) chunk is converted on `stream`
    cudaStream_t xfer = nullptr;
    cudaEvent_t xev[sphgb::kXferChunks + 1] = {};
    float pass_ms[3] = {0, 0, 0};
    uint32_t* q_ids = nullptr;
    uint32_t* q_cnt = nullptr;
    unsigned long long* q_dig = nullptr;
    int q_cap = 0;
    // sph_step_neighbor_digest: the force pass's neighbour counts and digests per sorted slot
    uint32_t* fd_cnt = nullptr;
    unsigned long long* fd_sum = nullptr;
    // sph_pair_counts: the density pass's candidate tests and r < h pairs (2 counters)
    unsigned long long* pc_dev = nullptr;
    // static obstacle (sph_set_obstacle): signed distance samples on the device, or null
    float* sdf_dev = nullptr;
    int sdf_dims[3] = {0, 0, 0};
    float sdf_org[3] = {0.f, 0.f, 0.f};
    float sdf_inv = 0.f;
    // render scratch (sph_render): depth/id keys, positions by id, a device image for host output
    void* render_buf = nullptr;
    size_t render_cap = 0;
};

namespace sphgb {
namespace engine {

sph_status fail(sph_ctx* c, sph_status code, const std::string& msg);
// Sort the current state into (pos_s, vel_s) with a valid cell table; hashes first if needed.
// Afterwards the cell counts are consumed (the next step re-hashes).
void sort_state(sph_ctx* ctx);
// n plain steps (graph replay, or eager with per-pass timing).
sph_status run_steps(sph_ctx* ctx, int n);
sph_status check_device_error(sph_ctx* ctx);
// The record index at each slot of the current state (the within-cell order that the next
// sort keeps), and its restore after an upload: resuming with it repeats a run bit for bit.
sph_status slot_order(sph_ctx* ctx, uint32_t* host_order);
sph_status apply_order(sph_ctx* ctx, const uint32_t* host_order);

}  // namespace engine
}  // namespace sphgb
