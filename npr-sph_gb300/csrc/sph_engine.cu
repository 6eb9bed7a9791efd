// sph_engine.cu -- the context behind the C ABI: device buffers, scene table,
// the captured per-step CUDA graph, uploads/downloads, reductions, neighbour
// queries and the launch-shape autotuner.
//
// One step = the reference's three dispatches (Main.cpp:291-304) re-planned:
//   scan -> scatter -> gather   (cell sort; the hash ran in the previous step's
//                                integrate epilogue, or eagerly after an upload)
//   density                     (rho_pres_comp.glsl)
//   force + integrate + hash    (force_comp.glsl + integrate_comp.glsl)
// captured once into a CUDA graph and replayed per step.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "sph_ctx.h"
#include "sph_host.h"
#include "sph_internal.h"

using namespace sphgb;

namespace sphgb {
namespace engine {

sph_status fail(sph_ctx* c, sph_status code, const std::string& msg) {
    if (c) c->err = msg;
    return code;
}

}  // namespace engine
}  // namespace sphgb

namespace {

// State in record order -> the given slot order (order[s] = record at slot s): positions,
// velocities and the uploaded (rho, pres), which live in slot order like the rest.
__global__ void __launch_bounds__(256) k_apply_order(const float4* __restrict__ pos, const float4* __restrict__ vel,
                                                     const float2* __restrict__ rhop, const uint32_t* __restrict__ order,
                                                     int n, float4* __restrict__ pos_out, float4* __restrict__ vel_out,
                                                     float2* __restrict__ rhop_out) {
    const int s = blockIdx.x * 256 + threadIdx.x;
    if (s >= n) return;
    const uint32_t id = order[s];
    if (id < (uint32_t)n) {
        pos_out[s] = pos[id];
        vel_out[s] = vel[id];
        rhop_out[s] = rhop[id];
    }
}

}  // namespace

namespace sphgb {
namespace engine {

sph_status slot_order(sph_ctx* ctx, uint32_t* host_order) {
    const size_t n = (size_t)ctx->b.n;
    std::vector<float4> v(n);
    cudaError_t e = cudaMemcpyAsync(v.data(), ctx->b.vel, n * sizeof(float4), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return fail(ctx, SPH_ERR_CUDA, std::string("slot order: ") + cudaGetErrorString(e));
    for (size_t s = 0; s < n; ++s) std::memcpy(&host_order[s], &v[s].w, 4);
    return SPH_OK;
}

sph_status apply_order(sph_ctx* ctx, const uint32_t* host_order) {
    const int n = ctx->b.n;
    std::vector<char> seen((size_t)n, 0);
    for (int s = 0; s < n; ++s) {
        if (host_order[s] >= (uint32_t)n || seen[host_order[s]])
            return fail(ctx, SPH_ERR_INVALID_ARG, "slot order is not a permutation");
        seen[host_order[s]] = 1;
    }
    uint32_t* d = nullptr;
    float2* rh = nullptr;
    cudaError_t e = cudaMalloc(&d, sizeof(uint32_t) * (size_t)n);
    if (e == cudaSuccess) e = cudaMalloc(&rh, sizeof(float2) * (size_t)n);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(d, host_order, sizeof(uint32_t) * (size_t)n, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) {
        k_apply_order<<<(n + 255) / 256, 256, 0, ctx->stream>>>(ctx->b.pos, ctx->b.vel, ctx->b.rhop, d, n, ctx->b.pos_s,
                                                                ctx->b.vel_s, rh);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(ctx->b.pos, ctx->b.pos_s, sizeof(float4) * (size_t)n, cudaMemcpyDeviceToDevice, ctx->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(ctx->b.vel, ctx->b.vel_s, sizeof(float4) * (size_t)n, cudaMemcpyDeviceToDevice, ctx->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(ctx->b.rhop, rh, sizeof(float2) * (size_t)n, cudaMemcpyDeviceToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (d) cudaFree(d);
    if (rh) cudaFree(rh);
    if (e != cudaSuccess) return fail(ctx, SPH_ERR_CUDA, std::string("slot order: ") + cudaGetErrorString(e));
    ctx->need_hash = true;
    return SPH_OK;
}

}  // namespace engine
}  // namespace sphgb

using sphgb::engine::fail;

namespace {

#define CK(call)                                                                          \
    do {                                                                                  \
        cudaError_t e_ = (call);                                                          \
        if (e_ != cudaSuccess)                                                            \
            return fail(ctx, e_ == cudaErrorMemoryAllocation ? SPH_ERR_OUT_OF_MEMORY : SPH_ERR_CUDA, \
                        std::string(#call) + ": " + cudaGetErrorString(e_));             \
    } while (0)

#define GUARD_BEGIN try {
#define GUARD_END                                                                         \
    }                                                                                     \
    catch (const std::bad_alloc&) { return fail(ctx, SPH_ERR_OUT_OF_MEMORY, "host allocation failed"); } \
    catch (...) { return fail(ctx, SPH_ERR_INVALID_ARG, "unexpected host exception"); }

template <class T>
cudaError_t dalloc(T** p, size_t count) {
    *p = nullptr;
    if (count == 0) count = 1;
    return cudaMalloc((void**)p, count * sizeof(T));
}

void free_graph(sph_ctx* ctx) {
    for (int m = 0; m < 2; ++m) {
        if (ctx->gexec[m]) cudaGraphExecDestroy(ctx->gexec[m]);
        if (ctx->graph[m]) cudaGraphDestroy(ctx->graph[m]);
        ctx->gexec[m] = nullptr;
        ctx->graph[m] = nullptr;
    }
}

// Recompute the scene table (cell ranges, particle ranges, constants) and grow
// the cell arrays when needed. Leaves count zeroed and asks for a fresh hash.
sph_status rebuild_geometry(sph_ctx* ctx) {
    std::vector<SceneDev> sc(ctx->params.size());
    long long cell = 0, first = 0, rows = 0;
    const bool keep = (ctx->params[0].flags & SPH_FLAG_KEEP_FORCE) != 0;
    for (size_t i = 0; i < sc.size(); ++i) {
        sc[i] = make_scene_dev(ctx->params[i], ctx->cfg.stencil, (int)cell, (int)first, (int)ctx->counts[i], keep);
        sc[i].row_base = (int)rows;
        sc[i].sdf = ctx->sdf_dev;
        for (int a = 0; a < 3; ++a) {
            sc[i].sdim[a] = ctx->sdf_dims[a];
            sc[i].sorg[a] = ctx->sdf_org[a];
        }
        sc[i].sinv = ctx->sdf_inv;
        cell += (long long)sc[i].dim[0] * sc[i].dim[1] * sc[i].dim[2];
        rows += (long long)sc[i].dim[1] * sc[i].dim[2];
        first += ctx->counts[i];
        if (cell >= (1ll << 31) - 1) return fail(ctx, SPH_ERR_INVALID_ARG, "too many grid cells");
    }
    if (cell > ctx->cell_cap) {
        cudaFree(ctx->b.count);
        cudaFree(ctx->b.start);
        cudaFree(ctx->b.scan_state);
        ctx->b.count = ctx->b.start = nullptr;
        ctx->b.scan_state = nullptr;
        long long cap = cell + cell / 8;
        int tiles = (int)((cap + kScanTile - 1) / kScanTile);
        CK(dalloc(&ctx->b.count, (size_t)cap));
        CK(dalloc(&ctx->b.start, (size_t)cap + 1));
        CK(dalloc(&ctx->b.scan_state, (size_t)tiles));
        CK(cudaMemsetAsync(ctx->b.scan_state, 0, sizeof(unsigned long long) * tiles, ctx->stream));
        ctx->cell_cap = cap;
        ctx->tile_cap = tiles;
    }
    CK(cudaMemsetAsync(ctx->b.count, 0, sizeof(int) * (size_t)cell, ctx->stream));
    CK(cudaMemcpyAsync(ctx->b.scenes, sc.data(), sizeof(SceneDev) * sc.size(), cudaMemcpyHostToDevice, ctx->stream));
    std::vector<int> sf(sc.size() + 1);
    for (size_t i = 0; i < sc.size(); ++i) sf[i] = sc[i].first;
    sf[sc.size()] = (int)first;
    CK(cudaMemcpyAsync(ctx->scene_first_dev, sf.data(), sizeof(int) * sf.size(), cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));  // host vectors die here
    ctx->sc_h = sc;
    ctx->s0 = sc[0];
    ctx->b.ncell = (int)cell;
    ctx->b.nscene = (int)sc.size();
    ctx->need_hash = true;
    free_graph(ctx);
    return SPH_OK;
}

void enqueue_sort(sph_ctx* ctx) {
    launch_scan(ctx->b, ctx->stream);
    launch_scatter(ctx->b, ctx->stream);
    launch_gather(ctx->b, ctx->stream);
}

// Whether the next step uses the neighbour records: from the same-cell pairs of the last sort
// that has written them to host-mapped memory (the host may be a few steps ahead of the device).
// Only the speed depends on the answer.
bool record_mode(const sph_ctx* ctx) {
    if (ctx->cfg.stencil != 1 || ctx->record_mode == SPH_RECORDS_NEVER) return false;
    if (ctx->record_mode == SPH_RECORDS_ALWAYS) return true;
    if (!ctx->pair_host || ctx->b.n <= 0) return false;
    const unsigned long long pairs = *reinterpret_cast<const volatile unsigned long long*>(ctx->pair_host);
    return (double)pairs > kRecordCellPairs * (double)ctx->b.n;
}

void enqueue_pairs(sph_ctx* ctx, bool rec) {
    launch_density(ctx->b, ctx->s0, ctx->batched, ctx->cfg, rec, ctx->stream);
    launch_force_integrate(ctx->b, ctx->s0, ctx->batched, ctx->cfg, rec, ctx->stream);
}

sph_status capture_graph(sph_ctx* ctx, int m) {
    if (ctx->gexec[m]) cudaGraphExecDestroy(ctx->gexec[m]);
    if (ctx->graph[m]) cudaGraphDestroy(ctx->graph[m]);
    ctx->gexec[m] = nullptr;
    ctx->graph[m] = nullptr;
    CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    enqueue_sort(ctx);
    enqueue_pairs(ctx, m != 0);
    cudaError_t e = cudaStreamEndCapture(ctx->stream, &ctx->graph[m]);
    cudaError_t launch_err = cudaGetLastError();  // also clears the thread's error state
    if (e == cudaSuccess) e = launch_err;
    if (e != cudaSuccess) {
        if (ctx->graph[m]) cudaGraphDestroy(ctx->graph[m]);
        ctx->graph[m] = nullptr;
        return fail(ctx, SPH_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
    }
    CK(cudaGraphInstantiate(&ctx->gexec[m], ctx->graph[m], 0));
    CK(cudaGraphUpload(ctx->gexec[m], ctx->stream));  // not on the first launch
    return SPH_OK;
}

sph_status check_device_error(sph_ctx* ctx) {
    uint32_t e = 0;
    CK(cudaMemcpyAsync(&e, ctx->b.err, sizeof(e), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    if (e) {
        CK(cudaMemsetAsync(ctx->b.err, 0, sizeof(uint32_t), ctx->stream));
        char buf[128];
        std::snprintf(buf, sizeof(buf), "device error word 0x%x (2: cell key out of range, 4: slot out of range)", e);
        return fail(ctx, SPH_ERR_DEVICE, buf);
    }
    return SPH_OK;
}

sph_status run_steps(sph_ctx* ctx, int n) {
    if (ctx->timing) {
        for (int s = 0; s < n; ++s) {
            CK(cudaEventRecord(ctx->ev[0], ctx->stream));
            if (ctx->need_hash) { launch_hash(ctx->b, ctx->s0, ctx->batched, ctx->stream); ctx->need_hash = false; }
            enqueue_sort(ctx);
            CK(cudaEventRecord(ctx->ev[1], ctx->stream));
            const bool rec = record_mode(ctx);
            ++ctx->record_steps[rec ? 0 : 1];
            launch_density(ctx->b, ctx->s0, ctx->batched, ctx->cfg, rec, ctx->stream);
            CK(cudaEventRecord(ctx->ev[2], ctx->stream));
            launch_force_integrate(ctx->b, ctx->s0, ctx->batched, ctx->cfg, rec, ctx->stream);
            CK(cudaEventRecord(ctx->ev[3], ctx->stream));
            CK(cudaEventSynchronize(ctx->ev[3]));
            for (int k = 0; k < 3; ++k) {
                float ms = 0;
                CK(cudaEventElapsedTime(&ms, ctx->ev[k], ctx->ev[k + 1]));
                ctx->pass_ms[k] += ms;
            }
        }
    } else {
        if (ctx->need_hash) {
            launch_hash(ctx->b, ctx->s0, ctx->batched, ctx->stream);
            ctx->need_hash = false;
        }
        for (int s = 0; s < n; ++s) {
            // A fresh context has no same-cell count yet: the first step publishes one before
            // the next is launched (one synchronisation per context).
            const bool first = s == 0 && ctx->cfg.stencil == 1 && ctx->pair_host &&
                               *reinterpret_cast<const volatile unsigned long long*>(ctx->pair_host) == 0;
            const int m = record_mode(ctx) ? 1 : 0;
            if (!ctx->gexec[m]) {  // both forms at once: a later switch costs no capture
                for (int k = 0; k < (ctx->cfg.stencil == 1 ? 2 : 1); ++k) {
                    if (ctx->gexec[k]) continue;
                    sph_status st = capture_graph(ctx, k);
                    if (st) return st;
                }
            }
            CK(cudaGraphLaunch(ctx->gexec[m], ctx->stream));
            ++ctx->record_steps[1 - m];
            if (first) CK(cudaStreamSynchronize(ctx->stream));
        }
    }
    CK(cudaGetLastError());
    ctx->steps += (uint64_t)n;
    ctx->stepped = true;
    return SPH_OK;
}

sph_status create_impl(const sph_params* params, const uint32_t* counts, uint32_t nscene, uint32_t n_max,
                       bool batched, void* stream, sph_ctx** out) {
    sph_ctx* ctx = nullptr;
    if (!params || !out || nscene == 0) return SPH_ERR_INVALID_ARG;
    *out = nullptr;
    for (uint32_t i = 0; i < nscene; ++i)
        if (sph_params_validate(&params[i]) != SPH_OK) return SPH_ERR_INVALID_ARG;
    // Every scene of a batch must agree on the KEEP_FORCE flag.
    for (uint32_t i = 1; i < nscene; ++i)
        if ((params[i].flags ^ params[0].flags) & SPH_FLAG_KEEP_FORCE) return SPH_ERR_INVALID_ARG;
    if (n_max == 0 || n_max > (1u << 30)) return SPH_ERR_INVALID_ARG;
    ctx = new (std::nothrow) sph_ctx;
    if (!ctx) return SPH_ERR_OUT_OF_MEMORY;
    GUARD_BEGIN
    ctx->params.assign(params, params + nscene);
    if (counts) ctx->counts.assign(counts, counts + nscene);
    else ctx->counts.assign(1, 0);
    ctx->batched = batched;
    ctx->n_max = n_max;
    sph_status st = SPH_OK;
    auto bail = [&](sph_status s) { sph_destroy(ctx); return s; };
    if (cudaGetDevice(&ctx->device) != cudaSuccess) return bail(SPH_ERR_CUDA);
    device_sm_count();  // cached before any stream capture
    init_step_kernels();
    if (stream) {
        ctx->stream = (cudaStream_t)stream;
    } else {
        if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) return bail(SPH_ERR_CUDA);
        ctx->own_stream = true;
    }
    Buffers& b = ctx->b;
    size_t n = n_max;
    if (dalloc(&b.pos, n) || dalloc(&b.vel, n) || dalloc(&b.pos_s, n) || dalloc(&b.vel_s, n) ||
        dalloc(&b.rhop, n) || dalloc(&b.force_s, n) || dalloc(&b.force_up, n) || dalloc(&b.aux, n) ||
        dalloc(&b.key, n) || dalloc(&b.rank, n) || dalloc(&b.perm, n) || dalloc(&b.slot_of_id, n) ||
        dalloc(&b.err, 1) || dalloc(&b.scenes, nscene) || dalloc(&b.tile_stats, 2) ||
        dalloc(&b.pmask, n * kPairMaskWords) || dalloc(&b.rec, 2 * n) ||
        dalloc(&b.partials, reduce_partials_doubles((int)nscene)) ||
        dalloc(&ctx->diag_dev, (size_t)nscene * kDiagFields) || dalloc(&ctx->scene_first_dev, nscene + 1))
        return bail(SPH_ERR_OUT_OF_MEMORY);
    if (cudaMemsetAsync(b.err, 0, sizeof(uint32_t), ctx->stream) ||
        cudaMemsetAsync(b.tile_stats, 0, sizeof(uint32_t) * 2, ctx->stream))
        return bail(SPH_ERR_CUDA);
    if (cudaHostAlloc(&ctx->pair_host, sizeof(unsigned long long), cudaHostAllocMapped) != cudaSuccess)
        return bail(SPH_ERR_OUT_OF_MEMORY);
    *ctx->pair_host = 0;
    if (cudaHostGetDevicePointer(&b.cell_pairs_map, ctx->pair_host, 0) != cudaSuccess) return bail(SPH_ERR_CUDA);
    for (auto& e : ctx->ev)
        if (cudaEventCreate(&e) != cudaSuccess) return bail(SPH_ERR_CUDA);
    if (cudaStreamCreateWithFlags(&ctx->xfer, cudaStreamNonBlocking) != cudaSuccess) return bail(SPH_ERR_CUDA);
    for (auto& e : ctx->xev)
        if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) return bail(SPH_ERR_CUDA);
    b.n = 0;
    st = rebuild_geometry(ctx);
    if (st) return bail(st);
    *out = ctx;
    return SPH_OK;
    GUARD_END
}

// Chunks of a host transfer of n records: a few for large transfers, so that the copy of one chunk
// overlaps the conversion of another.
static int xfer_chunks(uint32_t n) { return n >= (uint32_t)kXferChunks * 65536u ? kXferChunks : 1; }
static uint32_t chunk_begin(uint32_t n, int k, int chunks) { return (uint32_t)((uint64_t)n * k / chunks); }

sph_status upload_common(sph_ctx* ctx, const sph_particle* src, uint32_t n, bool host) {
    if (!ctx) return SPH_ERR_INVALID_ARG;
    if (!src) return fail(ctx, SPH_ERR_INVALID_ARG, "null particle pointer");
    if (n > ctx->n_max) return fail(ctx, SPH_ERR_CAPACITY, "more particles than n_max");
    if (ctx->batched) {
        uint64_t tot = 0;
        for (uint32_t c : ctx->counts) tot += c;
        if (tot != n) return fail(ctx, SPH_ERR_INVALID_ARG, "batch upload must hold the sum of the scene counts");
    }
    GUARD_BEGIN
    CK(cudaSetDevice(ctx->device));
    if (host && !ctx->b.aos) CK(dalloc(&ctx->b.aos, ctx->n_max));
    if (!ctx->batched && (int)n != ctx->b.n) {
        ctx->counts[0] = n;
        ctx->b.n = (int)n;
        sph_status st = rebuild_geometry(ctx);
        if (st) return st;
    }
    ctx->b.n = (int)n;
    const int chunks = xfer_chunks(n);
    if (host) {
        // The records are copied on the transfer stream, chunk by chunk; each chunk is converted
        // on the context's stream once its copy has landed, while the next one is copied.
        CK(cudaEventRecord(ctx->xev[kXferChunks], ctx->stream));  // earlier users of the staging buffer
        CK(cudaStreamWaitEvent(ctx->xfer, ctx->xev[kXferChunks], 0));
        for (int k = 0; k < chunks; ++k) {
            const uint32_t i0 = chunk_begin(n, k, chunks), i1 = chunk_begin(n, k + 1, chunks);
            CK(cudaMemcpyAsync(ctx->b.aos + i0, src + i0, sizeof(sph_particle) * (i1 - i0), cudaMemcpyHostToDevice,
                               ctx->xfer));
            CK(cudaEventRecord(ctx->xev[k], ctx->xfer));
            CK(cudaStreamWaitEvent(ctx->stream, ctx->xev[k], 0));
            launch_aos_to_soa(ctx->b, ctx->b.aos, ctx->scene_first_dev, (int)i0, (int)i1, ctx->stream);
        }
    } else {
        launch_aos_to_soa(ctx->b, src, ctx->scene_first_dev, 0, (int)n, ctx->stream);
    }
    CK(cudaMemsetAsync(ctx->b.count, 0, sizeof(int) * (size_t)ctx->b.ncell, ctx->stream));
    CK(cudaGetLastError());
    ctx->have_state = true;
    ctx->need_hash = true;
    ctx->stepped = false;
    ctx->steps = 0;
    ctx->judge_failures = 0;
    ctx->judge_backoff = 0;
    // The caller may reuse its buffer on return: wait for the copies (the conversion runs on).
    if (host) CK(cudaEventSynchronize(ctx->xev[chunks - 1]));
    return SPH_OK;
    GUARD_END
}

sph_status download_common(sph_ctx* ctx, sph_particle* dst, uint32_t n, bool host) {
    if (!ctx) return SPH_ERR_INVALID_ARG;
    if (!dst) return fail(ctx, SPH_ERR_INVALID_ARG, "null particle pointer");
    if (!ctx->have_state) return fail(ctx, SPH_ERR_NOT_READY, "no particles uploaded");
    if ((int)n != ctx->b.n) return fail(ctx, SPH_ERR_INVALID_ARG, "n must equal the uploaded particle count");
    GUARD_BEGIN
    CK(cudaSetDevice(ctx->device));
    const bool keep = (ctx->params[0].flags & SPH_FLAG_KEEP_FORCE) && ctx->stepped;
    if (host) {
        if (!ctx->b.aos) CK(dalloc(&ctx->b.aos, ctx->n_max));
        // Records are assembled by particle id, chunk by chunk, and each chunk is copied to the
        // host on the transfer stream while the next one is assembled.
        launch_slot_of_state_id(ctx->b, ctx->stream);
        const int chunks = xfer_chunks(n);
        for (int k = 0; k < chunks; ++k) {
            const uint32_t i0 = chunk_begin(n, k, chunks), i1 = chunk_begin(n, k + 1, chunks);
            launch_soa_to_aos_ids(ctx->b, keep, ctx->b.aos, (int)i0, (int)i1, ctx->stream);
            CK(cudaEventRecord(ctx->xev[k], ctx->stream));
            CK(cudaStreamWaitEvent(ctx->xfer, ctx->xev[k], 0));
            CK(cudaMemcpyAsync(dst + i0, ctx->b.aos + i0, sizeof(sph_particle) * (i1 - i0), cudaMemcpyDeviceToHost,
                               ctx->xfer));
        }
        CK(cudaEventRecord(ctx->xev[kXferChunks], ctx->xfer));
        CK(cudaStreamWaitEvent(ctx->stream, ctx->xev[kXferChunks], 0));  // later users of the staging buffer
    } else {
        launch_soa_to_aos(ctx->b, keep, dst, ctx->stream);
    }
    CK(cudaGetLastError());
    return check_device_error(ctx);  // synchronises the context's stream, which waits for the copies
    GUARD_END
}

void fill_diag(const double* d, uint64_t step, sph_diag* o) {
    for (int a = 0; a < 3; ++a) o->momentum[a] = d[a];
    o->kinetic_energy = d[3];
    o->potential_energy = d[4];
    double cnt = d[10];
    o->mean_rho = cnt > 0 ? d[5] / cnt : 0.0;
    o->min_rho = cnt > 0 ? d[6] : 0.0;
    o->max_rho = cnt > 0 ? d[7] : 0.0;
    o->mean_abs_rho_dev = cnt > 0 ? d[8] / cnt : 0.0;
    o->nonfinite = (uint64_t)d[9];
    o->n = (uint64_t)(d[9] + d[10]);
    o->step = step;
}

sph_status reduce_all(sph_ctx* ctx, std::vector<double>& h) {
    CK(cudaSetDevice(ctx->device));
    launch_reduce(ctx->b, nullptr, ctx->b.nscene, ctx->diag_dev, ctx->stream);
    CK(cudaGetLastError());
    h.assign((size_t)ctx->b.nscene * kDiagFields, 0.0);
    CK(cudaMemcpyAsync(h.data(), ctx->diag_dev, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, ctx->stream));
    return check_device_error(ctx);
}

}  // namespace

namespace sphgb {
namespace engine {

void sort_state(sph_ctx* ctx) {
    if (ctx->need_hash) launch_hash(ctx->b, ctx->s0, ctx->batched, ctx->stream);
    ::enqueue_sort(ctx);
    ctx->need_hash = true;  // the scan consumed the cell counts
}

sph_status run_steps(sph_ctx* ctx, int n) { return ::run_steps(ctx, n); }

sph_status check_device_error(sph_ctx* ctx) { return ::check_device_error(ctx); }

}  // namespace engine
}  // namespace sphgb

extern "C" {

sph_status sph_create(const sph_params* p, uint32_t n_max, void* stream, sph_ctx** out) {
    return create_impl(p, nullptr, 1, n_max, false, stream, out);
}

sph_status sph_create_batch(const sph_params* params, const uint32_t* counts, uint32_t n_scene, void* stream,
                            sph_ctx** out) {
    if (!counts || n_scene == 0) return SPH_ERR_INVALID_ARG;
    uint64_t tot = 0;
    for (uint32_t i = 0; i < n_scene; ++i) {
        if (counts[i] == 0) return SPH_ERR_INVALID_ARG;
        tot += counts[i];
    }
    if (tot > (1u << 30)) return SPH_ERR_INVALID_ARG;
    return create_impl(params, counts, n_scene, (uint32_t)tot, true, stream, out);
}

sph_status sph_destroy(sph_ctx* ctx) {
    if (!ctx) return SPH_ERR_INVALID_ARG;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    if (ctx->xfer) cudaStreamSynchronize(ctx->xfer);
    free_graph(ctx);
    Buffers& b = ctx->b;
    void* ptrs[] = {b.pos, b.vel, b.pos_s, b.vel_s, b.rhop, b.force_s, b.force_up, b.aux, b.aos, b.key, b.rank,
                    b.perm, b.count, b.start, b.scan_state, b.slot_of_id, b.err, b.partials,
                    b.scenes, b.tile_stats, b.pmask, b.rec, ctx->diag_dev, ctx->scene_first_dev, ctx->q_ids, ctx->q_cnt, ctx->q_dig,
                    ctx->fd_cnt, ctx->fd_sum, ctx->pc_dev,
                    ctx->render_buf, ctx->sdf_dev};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    if (ctx->pair_host) cudaFreeHost(ctx->pair_host);
    for (auto& e : ctx->ev)
        if (e) cudaEventDestroy(e);
    if (ctx->xfer) cudaStreamDestroy(ctx->xfer);
    for (auto& e : ctx->xev)
        if (e) cudaEventDestroy(e);
    if (ctx->own_stream && ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return SPH_OK;
}

const char* sph_last_error(const sph_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

sph_status sph_set_obstacle(sph_ctx* ctx, const float* sdf, const int32_t dims[3], const float origin[3],
                            float spacing) {
    if (!ctx) return SPH_ERR_INVALID_ARG;
    GUARD_BEGIN
    CK(cudaSetDevice(ctx->device));
    if (!sdf) {  // remove
        if (ctx->sdf_dev) {
            CK(cudaStreamSynchronize(ctx->stream));
            CK(cudaFree(ctx->sdf_dev));
        }
        ctx->sdf_dev = nullptr;
        ctx->sdf_dims[0] = ctx->sdf_dims[1] = ctx->sdf_dims[2] = 0;
        ctx->sdf_inv = 0.0f;
        return rebuild_geometry(ctx);
    }
    if (!dims || !origin) return fail(ctx, SPH_ERR_INVALID_ARG, "obstacle: null dims or origin");
    long long total = 1;
    for (int a = 0; a < 3; ++a) {
        if (dims[a] < 2 || dims[a] > (1 << 20)) return fail(ctx, SPH_ERR_INVALID_ARG, "obstacle: dims must be >= 2");
        if (!std::isfinite(origin[a])) return fail(ctx, SPH_ERR_INVALID_ARG, "obstacle: origin not finite");
        total *= dims[a];
    }
    if (total > (1ll << 28)) return fail(ctx, SPH_ERR_INVALID_ARG, "obstacle: more than 2^28 samples");
    if (!(spacing > 0.0f) || !std::isfinite(spacing)) return fail(ctx, SPH_ERR_INVALID_ARG, "obstacle: spacing");
    float* d = nullptr;
    CK(cudaStreamSynchronize(ctx->stream));
    CK(cudaMalloc(&d, sizeof(float) * (size_t)total));
    cudaError_t e = cudaMemcpy(d, sdf, sizeof(float) * (size_t)total, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        cudaFree(d);
        return fail(ctx, SPH_ERR_CUDA, std::string("obstacle upload: ") + cudaGetErrorString(e));
    }
    if (ctx->sdf_dev) cudaFree(ctx->sdf_dev);
    ctx->sdf_dev = d;
    for (int a = 0; a < 3; ++a) {
        ctx->sdf_dims[a] = dims[a];
        ctx->sdf_org[a] = origin[a];
    }
    ctx->sdf_inv = 1.0f / spacing;
    return rebuild_geometry(ctx);
    GUARD_END
}

sph_status sph_set_params(sph_ctx* ctx, const sph_params* p) {
    if (!ctx || !p) return SPH_ERR_INVALID_ARG;
    if (ctx->batched) return fail(ctx, SPH_ERR_UNSUPPORTED, "a batch takes its parameters at creation");
    if (sph_params_validate(p) != SPH_OK) return fail(ctx, SPH_ERR_INVALID_ARG, "invalid sph_params");
    // Callers upload the uniforms every frame (sendUniforms, Main.cpp:274-278): unchanged ones cost nothing.
    if (std::memcmp(&ctx->params[0], p, sizeof(sph_params)) == 0) return SPH_OK;
    GUARD_BEGIN
    CK(cudaSetDevice(ctx->device));
    ctx->params[0] = *p;
    sph_status st = rebuild_geometry(ctx);  // drops the fused hash of the last step
    return st;
    GUARD_END
}

sph_status sph_get_params(const sph_ctx* ctx, sph_params* p) {
    if (!ctx || !p) return SPH_ERR_INVALID_ARG;
    *p = ctx->params[0];
    return SPH_OK;
}

sph_status sph_upload_aos(sph_ctx* ctx, const sph_particle* host, uint32_t n) {
    return upload_common(ctx, host, n, true);
}
sph_status sph_upload_aos_device(sph_ctx* ctx, const sph_particle* dev, uint32_t n) {
    return upload_common(ctx, dev, n, false);
}
sph_status sph_download_aos(sph_ctx* ctx, sph_particle* host, uint32_t n) {
    return download_common(ctx, host, n, true);
}
sph_status sph_download_aos_device(sph_ctx* ctx, sph_particle* dev, uint32_t n) {
    return download_common(ctx, dev, n, false);
}

sph_status sph_step(sph_ctx* ctx, int32_t n_steps) {
    if (!ctx) return SPH_ERR_INVALID_ARG;
    if (n_steps < 0) return fail(ctx, SPH_ERR_INVALID_ARG, "n_steps < 0");
    if (!ctx->have_state) return fail(ctx, SPH_ERR_NOT_READY, "no particles uploaded");
    if (n_steps == 0 || ctx->b.n == 0) return SPH_OK;
    GUARD_BEGIN
    CK(cudaSetDevice(ctx->device));
    if (ctx->timing) for (float& t : ctx->pass_ms) t = 0.0f;
    return run_steps(ctx, n_steps);
    GUARD_END
}

sph_status sph_synchronize(sph_ctx* ctx) {
    if (!ctx) return SPH_ERR_INVALID_ARG;
    CK(cudaSetDevice(ctx->device));
    CK(cudaStreamSynchronize(ctx->stream));
    return check_device_error(ctx);
}

sph_status sph_reduce(sph_ctx* ctx, sph_diag* out) {
    if (!ctx || !out) return SPH_ERR_INVALID_ARG;
    if (!ctx->have_state) return fail(ctx, SPH_ERR_NOT_READY, "no particles uploaded");
    GUARD_BEGIN
    std::vector<double> h;
    sph_status st = reduce_all(ctx, h);
    if (st) return st;
    double tot[kDiagFields];
    for (int f = 0; f < kDiagFields; ++f) tot[f] = f == 6 ? INFINITY : (f == 7 ? -INFINITY : 0.0);
    for (int s = 0; s < ctx->b.nscene; ++s)
        for (int f = 0; f < kDiagFields; ++f) {
            double x = h[(size_t)s * kDiagFields + f];
            tot[f] = f == 6 ? std::min(tot[f], x) : (f == 7 ? std::max(tot[f], x) : tot[f] + x);
        }
    fill_diag(tot, ctx->steps, out);
    return SPH_OK;
    GUARD_END
}

sph_status sph_reduce_scenes(sph_ctx* ctx, sph_diag* out, uint32_t n_scene) {
    if (!ctx || !out) return SPH_ERR_INVALID_ARG;
    if (!ctx->have_state) return fail(ctx, SPH_ERR_NOT_READY, "no particles uploaded");
    if ((int)n_scene != ctx->b.nscene) return fail(ctx, SPH_ERR_INVALID_ARG, "n_scene mismatch");
    GUARD_BEGIN
    std::vector<double> h;
    sph_status st = reduce_all(ctx, h);
    if (st) return st;
    for (uint32_t s = 0; s < n_scene; ++s) fill_diag(&h[(size_t)s * kDiagFields], ctx->steps, &out[s]);
    return SPH_OK;
    GUARD_END
}

uint32_t sph_num_particles(const sph_ctx* ctx) { return ctx ? (uint32_t)ctx->b.n : 0u; }
uint64_t sph_step_count(const sph_ctx* ctx) { return ctx ? ctx->steps : 0ull; }
uint32_t sph_num_scenes(const sph_ctx* ctx) { return ctx ? (uint32_t)ctx->b.nscene : 0u; }

sph_status sph_enable_timing(sph_ctx* ctx, int32_t on) {
    if (!ctx) return SPH_ERR_INVALID_ARG;
    ctx->timing = on != 0;
    for (float& t : ctx->pass_ms) t = 0.0f;
    return SPH_OK;
}

sph_status sph_pass_times(sph_ctx* ctx, float out_ms[3]) {
    if (!ctx || !out_ms) return SPH_ERR_INVALID_ARG;
    if (!ctx->timing) return fail(ctx, SPH_ERR_NOT_READY, "timing not enabled");
    for (int k = 0; k < 3; ++k) out_ms[k] = ctx->pass_ms[k];
    return SPH_OK;
}

sph_status sph_neighbor_digest(sph_ctx* ctx, const uint32_t* query_ids, uint32_t n_query, int32_t brute_force,
                               uint32_t* count_out, uint64_t* digest_out) {
    if (!ctx) return SPH_ERR_INVALID_ARG;
    if (!query_ids || !count_out || !digest_out) return fail(ctx, SPH_ERR_INVALID_ARG, "null pointer");
    if (!ctx->have_state) return fail(ctx, SPH_ERR_NOT_READY, "no particles uploaded");
    if (n_query == 0) return SPH_OK;
    GUARD_BEGIN
    CK(cudaSetDevice(ctx->device));
    if ((int)n_query > ctx->q_cap) {
        cudaFree(ctx->q_ids); cudaFree(ctx->q_cnt); cudaFree(ctx->q_dig);
        ctx->q_ids = nullptr; ctx->q_cnt = nullptr; ctx->q_dig = nullptr;
        ctx->q_cap = 0;
        CK(dalloc(&ctx->q_ids, n_query));
        CK(dalloc(&ctx->q_cnt, n_query));
        CK(dalloc(&ctx->q_dig, n_query));
        ctx->q_cap = (int)n_query;
    }
    if (ctx->need_hash) launch_hash(ctx->b, ctx->s0, ctx->batched, ctx->stream);
    enqueue_sort(ctx);  // sorted copy of the current positions; the state itself is untouched
    launch_slot_of_id(ctx->b, ctx->stream);
    ctx->need_hash = true;  // the scan consumed the cell counts
    CK(cudaMemcpyAsync(ctx->q_ids, query_ids, sizeof(uint32_t) * n_query, cudaMemcpyHostToDevice, ctx->stream));
    launch_neighbor_digest(ctx->b, ctx->s0, ctx->batched, ctx->cfg.stencil, ctx->q_ids, (int)n_query,
                           brute_force ? 1 : 0, ctx->q_cnt, ctx->q_dig, ctx->stream);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(count_out, ctx->q_cnt, sizeof(uint32_t) * n_query, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaMemcpyAsync(digest_out, ctx->q_dig, sizeof(uint64_t) * n_query, cudaMemcpyDeviceToHost, ctx->stream));
    return check_device_error(ctx);
    GUARD_END
}

sph_status sph_step_neighbor_digest(sph_ctx* ctx, const uint32_t* query_ids, uint32_t n_query, uint32_t* count_out,
                                    uint64_t* digest_out) {
    if (!ctx) return SPH_ERR_INVALID_ARG;
    if (n_query && (!query_ids || !count_out || !digest_out)) return fail(ctx, SPH_ERR_INVALID_ARG, "null pointer");
    if (!ctx->have_state) return fail(ctx, SPH_ERR_NOT_READY, "no particles uploaded");
    if (ctx->cfg.stencil != 1)
        return fail(ctx, SPH_ERR_UNSUPPORTED, "the force pass reads neighbour masks with stencil 1 only");
    GUARD_BEGIN
    CK(cudaSetDevice(ctx->device));
    if ((int)n_query > ctx->q_cap) {
        cudaFree(ctx->q_ids); cudaFree(ctx->q_cnt); cudaFree(ctx->q_dig);
        ctx->q_ids = nullptr; ctx->q_cnt = nullptr; ctx->q_dig = nullptr;
        ctx->q_cap = 0;
        CK(dalloc(&ctx->q_ids, n_query));
        CK(dalloc(&ctx->q_cnt, n_query));
        CK(dalloc(&ctx->q_dig, n_query));
        ctx->q_cap = (int)n_query;
    }
    if (!ctx->fd_cnt) CK(dalloc(&ctx->fd_cnt, ctx->n_max));
    if (!ctx->fd_sum) CK(dalloc(&ctx->fd_sum, ctx->n_max));
    if (ctx->need_hash) {
        launch_hash(ctx->b, ctx->s0, ctx->batched, ctx->stream);
        ctx->need_hash = false;
    }
    enqueue_sort(ctx);
    launch_density(ctx->b, ctx->s0, ctx->batched, ctx->cfg, false, ctx->stream);
    launch_force_integrate(ctx->b, ctx->s0, ctx->batched, ctx->cfg, false, ctx->stream, ctx->fd_cnt, ctx->fd_sum);
    launch_slot_of_id(ctx->b, ctx->stream);  // id -> slot of the step's sorted state
    if (n_query) {
        CK(cudaMemcpyAsync(ctx->q_ids, query_ids, sizeof(uint32_t) * n_query, cudaMemcpyHostToDevice, ctx->stream));
        launch_query_gather(ctx->b, ctx->q_ids, (int)n_query, ctx->fd_cnt, ctx->fd_sum, ctx->q_cnt, ctx->q_dig,
                            ctx->stream);
    }
    CK(cudaGetLastError());
    ctx->steps += 1;
    ctx->stepped = true;
    if (n_query) {
        CK(cudaMemcpyAsync(count_out, ctx->q_cnt, sizeof(uint32_t) * n_query, cudaMemcpyDeviceToHost, ctx->stream));
        CK(cudaMemcpyAsync(digest_out, ctx->q_dig, sizeof(uint64_t) * n_query, cudaMemcpyDeviceToHost, ctx->stream));
    }
    return check_device_error(ctx);
    GUARD_END
}

sph_status sph_pair_counts(sph_ctx* ctx, uint64_t out[2]) {
    if (!ctx || !out) return SPH_ERR_INVALID_ARG;
    if (!ctx->have_state) return fail(ctx, SPH_ERR_NOT_READY, "no particles uploaded");
    GUARD_BEGIN
    CK(cudaSetDevice(ctx->device));
    if (!ctx->pc_dev) CK(dalloc(&ctx->pc_dev, 2));
    if (ctx->need_hash) launch_hash(ctx->b, ctx->s0, ctx->batched, ctx->stream);
    enqueue_sort(ctx);  // sorted copy of the current positions; the state itself is untouched
    ctx->need_hash = true;  // the scan consumed the cell counts
    CK(cudaMemsetAsync(ctx->pc_dev, 0, 2 * sizeof(unsigned long long), ctx->stream));
    launch_pair_counts(ctx->b, ctx->s0, ctx->batched, ctx->cfg.stencil, ctx->pc_dev, ctx->stream);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(out, ctx->pc_dev, 2 * sizeof(uint64_t), cudaMemcpyDeviceToHost, ctx->stream));
    return check_device_error(ctx);
    GUARD_END
}

sph_status sph_set_launch(sph_ctx* ctx, int32_t tpb, int32_t stencil) {
    if (!ctx) return SPH_ERR_INVALID_ARG;
    if ((tpb != 128 && tpb != 256) || (stencil != 1 && stencil != 2))
        return fail(ctx, SPH_ERR_INVALID_ARG, "threads_per_block 128 or 256, stencil 1 or 2");
    GUARD_BEGIN
    CK(cudaSetDevice(ctx->device));
    bool geo = stencil != ctx->cfg.stencil;
    ctx->cfg.block = tpb;
    ctx->cfg.stencil = stencil;
    if (geo) return rebuild_geometry(ctx);
    free_graph(ctx);
    return SPH_OK;
    GUARD_END
}

sph_status sph_tile_stats(sph_ctx* ctx, uint32_t out[2]) {
    if (!ctx || !out) return SPH_ERR_INVALID_ARG;
    CK(cudaSetDevice(ctx->device));
    CK(cudaMemcpyAsync(out, ctx->b.tile_stats, sizeof(uint32_t) * 2, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return SPH_OK;
}

sph_status sph_record_stats(const sph_ctx* ctx, uint64_t out[3]) {
    if (!ctx || !out) return SPH_ERR_INVALID_ARG;
    out[0] = ctx->record_steps[0];
    out[1] = ctx->record_steps[1];
    out[2] = ctx->pair_host ? *reinterpret_cast<const volatile unsigned long long*>(ctx->pair_host) : 0;
    return SPH_OK;
}

sph_status sph_set_record_mode(sph_ctx* ctx, int32_t mode) {
    if (!ctx) return SPH_ERR_INVALID_ARG;
    if (mode != SPH_RECORDS_AUTO && mode != SPH_RECORDS_ALWAYS && mode != SPH_RECORDS_NEVER)
        return fail(ctx, SPH_ERR_INVALID_ARG, "record mode: 0 auto, 1 always, 2 never");
    ctx->record_mode = mode;
    return SPH_OK;
}

sph_status sph_get_launch(const sph_ctx* ctx, int32_t* tpb, int32_t* stencil) {
    if (!ctx || !tpb || !stencil) return SPH_ERR_INVALID_ARG;
    *tpb = ctx->cfg.block;
    *stencil = ctx->cfg.stencil;
    return SPH_OK;
}

sph_status sph_autotune(sph_ctx* ctx, int32_t trial_steps, float* best_ms) {
    if (!ctx) return SPH_ERR_INVALID_ARG;
    if (!ctx->have_state) return fail(ctx, SPH_ERR_NOT_READY, "no particles uploaded");
    if (trial_steps < 1) return fail(ctx, SPH_ERR_INVALID_ARG, "trial_steps < 1");
    GUARD_BEGIN
    CK(cudaSetDevice(ctx->device));
    const size_t n = (size_t)ctx->b.n;
    float4 *bp = nullptr, *bv = nullptr;
    float2* br = nullptr;
    CK(dalloc(&bp, n));
    sph_status st = SPH_OK;
    auto cleanup = [&]() { cudaFree(bp); cudaFree(bv); cudaFree(br); };
    if (dalloc(&bv, n) || dalloc(&br, n)) { cleanup(); return fail(ctx, SPH_ERR_OUT_OF_MEMORY, "autotune backup"); }
    // Save the state; every trial restarts from it.
    cudaMemcpyAsync(bp, ctx->b.pos, n * sizeof(float4), cudaMemcpyDeviceToDevice, ctx->stream);
    cudaMemcpyAsync(bv, ctx->b.vel, n * sizeof(float4), cudaMemcpyDeviceToDevice, ctx->stream);
    cudaMemcpyAsync(br, ctx->b.rhop, n * sizeof(float2), cudaMemcpyDeviceToDevice, ctx->stream);
    const uint64_t steps0 = ctx->steps;
    const bool stepped0 = ctx->stepped, timing0 = ctx->timing;
    ctx->timing = false;
    // The current shape is timed first; another replaces it only when it is faster by more than
    // kSwitchMargin (trial steps of one state are noisy, and the state changes as the run goes on).
    constexpr float kSwitchMargin = 0.03f;
    const LaunchCfg cur = ctx->cfg;
    const int blocks[] = {cur.block, cur.block == 128 ? 256 : 128};
    const int stencils[] = {cur.stencil, cur.stencil == 1 ? 2 : 1};
    float best = 1e30f;
    LaunchCfg best_cfg = ctx->cfg;
    for (int sten : stencils) {
        for (int blk : blocks) {
            st = sph_set_launch(ctx, blk, sten);
            if (st) break;
            auto restore = [&]() {
                cudaMemcpyAsync(ctx->b.pos, bp, n * sizeof(float4), cudaMemcpyDeviceToDevice, ctx->stream);
                cudaMemcpyAsync(ctx->b.vel, bv, n * sizeof(float4), cudaMemcpyDeviceToDevice, ctx->stream);
                cudaMemcpyAsync(ctx->b.rhop, br, n * sizeof(float2), cudaMemcpyDeviceToDevice, ctx->stream);
                cudaMemsetAsync(ctx->b.count, 0, sizeof(int) * (size_t)ctx->b.ncell, ctx->stream);
                ctx->need_hash = true;
            };
            restore();
            st = run_steps(ctx, 1);  // warm-up (captures the graph)
            if (st) break;
            restore();
            if (ctx->need_hash) { launch_hash(ctx->b, ctx->s0, ctx->batched, ctx->stream); ctx->need_hash = false; }
            cudaEventRecord(ctx->ev[0], ctx->stream);
            st = run_steps(ctx, trial_steps);
            if (st) break;
            cudaEventRecord(ctx->ev[1], ctx->stream);
            cudaEventSynchronize(ctx->ev[1]);
            float ms = 0;
            cudaEventElapsedTime(&ms, ctx->ev[0], ctx->ev[1]);
            ms /= (float)trial_steps;
            const bool is_cur = ctx->cfg.block == cur.block && ctx->cfg.stencil == cur.stencil;
            if (is_cur ? ms < best : ms < best * (1.0f - kSwitchMargin)) { best = ms; best_cfg = ctx->cfg; }
            restore();
        }
        if (st) break;
    }
    ctx->timing = timing0;
    if (st == SPH_OK) st = sph_set_launch(ctx, best_cfg.block, best_cfg.stencil);
    // Final restore under the chosen geometry.
    cudaMemcpyAsync(ctx->b.pos, bp, n * sizeof(float4), cudaMemcpyDeviceToDevice, ctx->stream);
    cudaMemcpyAsync(ctx->b.vel, bv, n * sizeof(float4), cudaMemcpyDeviceToDevice, ctx->stream);
    cudaMemcpyAsync(ctx->b.rhop, br, n * sizeof(float2), cudaMemcpyDeviceToDevice, ctx->stream);
    cudaMemsetAsync(ctx->b.count, 0, sizeof(int) * (size_t)ctx->b.ncell, ctx->stream);
    ctx->need_hash = true;
    ctx->steps = steps0;
    ctx->stepped = stepped0;
    cudaStreamSynchronize(ctx->stream);
    cleanup();
    if (best_ms) *best_ms = best;
    if (st) return st;
    CK(cudaGetLastError());
    return check_device_error(ctx);
    GUARD_END
}

}  // extern "C"
