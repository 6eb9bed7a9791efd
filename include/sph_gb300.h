/*
 * sph_gb300.h -- C ABI of the GB300 SPH step.
 *
 * This library replaces the reference's per-frame SPH step, which is three
 * OpenGL compute dispatches over one particle SSBO:
 *
 *   glUseProgram(compute_programs[0]); glDispatchCompute(10,1,1); glMemoryBarrier(...);  // rho_pres_comp.glsl
 *   glUseProgram(compute_programs[1]); glDispatchCompute(10,1,1); glMemoryBarrier(...);  // force_comp.glsl
 *   glUseProgram(compute_programs[2]); glDispatchCompute(10,1,1); glMemoryBarrier(...);  // integrate_comp.glsl
 *
 * (NPR-SPH/Main.cpp:291-304), with one call:  sph_step(ctx, 1).
 *
 * Conventions
 *   - Every function returns sph_status (0 = OK, negative = error) except the
 *     small getters. No C++ exception crosses this boundary.
 *   - sph_last_error(ctx) returns a message for the last failed call on ctx.
 *   - Host arrays are owned by the caller and only touched during the call.
 *     Device buffers are owned by the context.
 *   - A context is used by one host thread at a time. Separate contexts are
 *     independent (they may share a device).
 *   - No torch or CUDA types appear in the signatures. A CUDA stream is passed
 *     as void* (a cudaStream_t); NULL selects a stream owned by the context.
 */
#ifndef SPH_GB300_H
#define SPH_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SPH_ABI_VERSION 1

typedef int32_t sph_status;
#define SPH_OK                  0
#define SPH_ERR_INVALID_ARG    (-1)  /* bad pointer, size or parameter value */
#define SPH_ERR_CUDA           (-2)  /* a CUDA runtime call failed */
#define SPH_ERR_OUT_OF_MEMORY  (-3)
#define SPH_ERR_CAPACITY       (-4)  /* more particles than the context was created for */
#define SPH_ERR_NOT_READY      (-5)  /* e.g. sph_step before any upload */
#define SPH_ERR_DEVICE         (-6)  /* a kernel raised its device error word */
#define SPH_ERR_UNSUPPORTED    (-7)

/*
 * One particle, 64 bytes: the reference's `struct Particle`
 * (NPR-SPH/Main.cpp:93-99; std430 copy in rho_pres_comp.glsl:12-18).
 *   pos.xyz position (w = 1 from make_grid, Main.cpp:499)
 *   vel.xyz velocity
 *   force.xyz force density of the last step (written only when
 *             SPH_FLAG_KEEP_FORCE is set; the fused step does not need it)
 *   extras[0] density rho, extras[1] pressure, extras[2] age (never written)
 */
typedef struct sph_particle {
    float pos[4];
    float vel[4];
    float force[4];
    float extras[4];
} sph_particle;

/* Flags of sph_params.flags */
#define SPH_FLAG_KEEP_FORCE  0x1u  /* also store force.xyz every step (for download) */

/*
 * Every uniform and compile-time constant of the three shaders, as runtime
 * fields. sph_params_default() gives the reference's literal values.
 */
typedef struct sph_params {
    /* ConstantsUniform, std140 binding 1 (Main.cpp:110-116; rho_pres_comp.glsl:25-31) */
    float mass;             /* 0.02 */
    float smoothing_coeff;  /* 4.0; h = smoothing_coeff * particle_radius (rho_pres_comp.glsl:40) */
    float visc;             /* 3000 (mu) */
    float resting_rho;      /* 1000 (rho0) */
    /* BoundaryUniform, std140 binding 2 (Main.cpp:118-122; integrate_comp.glsl:27-31) */
    float upper[4];         /* (0.5, 1.0, 0.5, 1) */
    float lower[4];         /* (-0.1, -0.35, -0.1, 1) */
    /* Shader compile-time constants */
    float particle_radius;  /* PARTICLE_RADIUS 0.005 (rho_pres_comp.glsl:5) */
    float gas_const;        /* GAS_CONST 2000 (rho_pres_comp.glsl:33), stiffness k */
    float gravity[3];       /* G = (0, -9806.65, 0) (force_comp.glsl:33) */
    float dt;               /* 1/NUM_PARTICLES = 1e-4 (integrate_comp.glsl:33) */
    float damping;          /* DAMPING 0.3 (integrate_comp.glsl:8) */
    /* New: neighbour grid. Cell edge = h * max(cell_scale, 1 + 2^-10). 0 => default. */
    float cell_scale;
    uint32_t flags;         /* SPH_FLAG_* */
    uint32_t reserved[3];   /* must be zero */
} sph_params;

/* FP64 diagnostics of the current state (drift judge). */
typedef struct sph_diag {
    double momentum[3];       /* sum m v */
    double kinetic_energy;    /* sum 1/2 m |v|^2 */
    double potential_energy;  /* sum -m G.x */
    double mean_rho;          /* sum rho / n (rho of the last density pass) */
    double min_rho;
    double max_rho;
    double mean_abs_rho_dev;  /* sum |rho - rho0| / rho0 / n */
    uint64_t nonfinite;       /* particles with a NaN/Inf in pos, vel or rho */
    uint64_t n;               /* particles */
    uint64_t step;            /* steps taken since the last upload */
} sph_diag;

typedef struct sph_ctx sph_ctx;

/* ---- library ----------------------------------------------------------- */

/* "sph_gb300 <version> sm_103a". */
const char* sph_version(void);

/* Fill *p with the reference's literal values (see sph_params). */
void sph_params_default(sph_params* p);

/* SPH_OK if p is usable (h > 0, mass > 0, rho0 > 0, dt > 0, lower < upper, ...). */
sph_status sph_params_validate(const sph_params* p);

/* Smallest float T with sqrtf(T) >= h: for the FP32 pair distance
 * d2 = (dx*dx + dy*dy) + dz*dz, `sqrtf(d2) < h` (the shaders' `length(delta) <
 * smoothing_length`, rho_pres_comp.glsl:49-50) holds exactly when d2 < T. */
float sph_cutoff_d2(float h);

/* Grid geometry for p: cell edge and cells per axis. */
sph_status sph_grid_dims(const sph_params* p, float* cell_edge, int32_t dims[3]);

/* ---- context: replaces the SSBO, the UBOs and the three dispatches ---- */

/* Allocate device state for up to n_max particles on the current device.
 * Mirrors the SSBO/UBO creation in init_particles / initOpenGL
 * (Main.cpp:510-527, :631-641). stream: cudaStream_t or NULL. */
sph_status sph_create(const sph_params* p, uint32_t n_max, void* stream, sph_ctx** out);
sph_status sph_destroy(sph_ctx* ctx);
const char* sph_last_error(const sph_ctx* ctx);

/* Replace the uniforms; takes effect at the next step.
 * Mirrors sendUniforms (Main.cpp:274-278). */
sph_status sph_set_params(sph_ctx* ctx, const sph_params* p);
sph_status sph_get_params(const sph_ctx* ctx, sph_params* p);

/* Load particles from host memory (pageable or pinned), in caller order.
 * Mirrors glBufferData of the SSBO (Main.cpp:524-527). Resets the step count. */
sph_status sph_upload_aos(sph_ctx* ctx, const sph_particle* host, uint32_t n);
/* Write the current state to host memory in the caller's original order:
 * pos, vel, extras = (rho, pres, age of the input), force if KEEP_FORCE. */
sph_status sph_download_aos(sph_ctx* ctx, sph_particle* host, uint32_t n);
/* Same two calls for an AoS buffer in device memory (the SSBO's place). */
sph_status sph_upload_aos_device(sph_ctx* ctx, const sph_particle* dev, uint32_t n);
sph_status sph_download_aos_device(sph_ctx* ctx, sph_particle* dev, uint32_t n);

/* Advance n_steps steps: density/pressure -> force -> integrate, each step
 * preceded by the grid rebuild. Replaces Main.cpp:291-304. Asynchronous on
 * the context's stream; errors of earlier asynchronous work surface here or
 * at sph_synchronize. */
sph_status sph_step(sph_ctx* ctx, int32_t n_steps);
sph_status sph_synchronize(sph_ctx* ctx);

/* FP64 reductions of the current state (synchronous). */
sph_status sph_reduce(sph_ctx* ctx, sph_diag* out);

uint32_t sph_num_particles(const sph_ctx* ctx);
uint64_t sph_step_count(const sph_ctx* ctx);

/* Per-pass device time of the last sph_step call in milliseconds, summed over
 * its steps, when the context was created with SPH_FLAG_* timing enabled by
 * sph_enable_timing(ctx, 1). passes: 0 grid, 1 density, 2 force+integrate. */
sph_status sph_enable_timing(sph_ctx* ctx, int32_t on);
sph_status sph_pass_times(sph_ctx* ctx, float out_ms[3]);

/* Neighbour sets of query particles (ids = indices in upload order) on the
 * current positions: count of j with `length(x_i - x_j) < h` (self
 * included) and an order-independent 64-bit digest sum_j mix64(j).
 * brute_force = 0: the uniform grid the step uses; 1: all-pairs scan.
 * New (no reference counterpart): the check that the grid loses no pair. */
sph_status sph_neighbor_digest(sph_ctx* ctx, const uint32_t* query_ids, uint32_t n_query,
                               int32_t brute_force, uint32_t* count_out, uint64_t* digest_out);
/* One plain step (as sph_step(ctx, 1), launched without the graph) that also reports, for the
 * query particles, the neighbour sets its force pass used -- with stencil 1 they are decoded
 * from the density pass's masks -- as count (self included) and digest, to compare with
 * sph_neighbor_digest on the positions before the step. Stencil 1 only (SPH_ERR_UNSUPPORTED
 * otherwise). New (no reference counterpart): the check that the force pass loses no pair. */
sph_status sph_step_neighbor_digest(sph_ctx* ctx, const uint32_t* query_ids, uint32_t n_query,
                                    uint32_t* count_out, uint64_t* digest_out);

/* ---- batched scenes (new; no reference counterpart) --------------------
 * n_scene independent boxes, each with its own sph_params and particle count,
 * advance together: one launch per pass covers every scene, and the passes of
 * a step are replayed from one captured CUDA graph. Uploads and downloads use
 * the scenes' records concatenated in scene order (sum of counts records).
 * sph_step, sph_synchronize, sph_download_*, sph_neighbor_digest, sph_reduce
 * (totals over all scenes) work on a batch context as on a single scene. */
sph_status sph_create_batch(const sph_params* params, const uint32_t* counts, uint32_t n_scene,
                            void* stream, sph_ctx** out);
uint32_t sph_num_scenes(const sph_ctx* ctx);
/* out[n_scene]: FP64 diagnostics of every scene. */
sph_status sph_reduce_scenes(sph_ctx* ctx, sph_diag* out, uint32_t n_scene);

/* ---- launch shape and autotuner (new) ----------------------------------
 * threads_per_block of the pair passes (128 or 256: the particles of one
 * shared-memory tile) and stencil (1: cell edge >= h, 27 cells; 2: cell edge
 * >= h/2, 125 smaller cells). A new context starts at (256, 1).
 * sph_autotune times `trial_steps` steps of every candidate shape on the
 * current state (restoring it afterwards) and keeps the fastest; the current
 * shape is kept unless another is more than 3% faster. */
sph_status sph_set_launch(sph_ctx* ctx, int32_t threads_per_block, int32_t stencil);
sph_status sph_get_launch(const sph_ctx* ctx, int32_t* threads_per_block, int32_t* stencil);
sph_status sph_autotune(sph_ctx* ctx, int32_t trial_steps, float* best_ms_per_step);
/* Work counters of the next step's pair passes at the current positions
 * (measurement; the state is not changed): out[0] = candidate tests of the
 * density pass (the particles of cells cx-R..cx+R of each of its (2R+1)^2
 * stencil rows, R the stencil), out[1] = pairs with r < h, self included
 * (rho_pres_comp.glsl:46-54); the force pass interacts with out[1] - n of
 * them (force_comp.glsl:48-62 skips j == i). Synchronous. */
sph_status sph_pair_counts(sph_ctx* ctx, uint64_t out[2]);
/* Chunks of the density (out[0]) and force (out[1]) passes, since creation,
 * that did not fit a shared-memory tile and read their neighbours from global
 * memory instead (heavy pile-ups). Synchronous. */
sph_status sph_tile_stats(sph_ctx* ctx, uint32_t out[2]);
/* Steps since creation whose force pass read each neighbour as one 32-byte
 * record written by the density pass (out[0]), steps that read position,
 * velocity and (rho, p) from the state arrays (out[1]), and the same-cell
 * pairs (sum over the grid's cells of count^2, self included) that the last
 * sort seen by the host found (out[2]). A step uses records when out[2] is
 * above 2.6 per particle (stencil 1 only; dense fluid); both forms compute
 * the same interactions from the same values, so the choice changes only the
 * speed. */
sph_status sph_record_stats(const sph_ctx* ctx, uint64_t out[3]);
/* The choice above: SPH_RECORDS_AUTO (default), SPH_RECORDS_ALWAYS or
 * SPH_RECORDS_NEVER (stencil 1; stencil 2 never uses records). */
enum { SPH_RECORDS_AUTO = 0, SPH_RECORDS_ALWAYS = 1, SPH_RECORDS_NEVER = 2 };
sph_status sph_set_record_mode(sph_ctx* ctx, int32_t mode);

/* ---- learned macro-step (new; no reference counterpart) -----------------
 * A message-passing network (2 rounds over the <= 32 nearest neighbours,
 * hidden width 64) predicts, per particle, the mean accelerations of the next
 * 4 plain steps: O_v = (a0+a1+a2+a3)/(4A) and O_x = (4a0+3a1+2a2+a3)/(10A),
 * A = k/h. One network pass replaces 4 plain steps:
 *   v' = v + 4 dt A O_v,  x' = x + 4 dt v + 10 dt^2 A O_x,  then the wall clamp.
 * The network is trained on the GPU, by this library's own forward/backward/Adam
 * kernels, on frames recorded from the plain step itself.
 * Judge: the macro-steps run in intervals of judge_every. Each learned interval
 * starts from a checkpoint; its last macro-step is judged: from the same state a
 * learned macro-step and 4 plain steps are compared with FP64 reductions. When the
 * density deviation exceeds density_tol, or the momentum difference (relative to
 * sum m|v| + M |G| 4 dt) exceeds momentum_tol, the interval is rolled back to its
 * checkpoint and run by plain SPH, and after the k-th failure in a row plain SPH
 * also runs the next 2^(k-1) - 1 intervals (at most 7). The density deviation is
 * (sph_learned_set_judge):
 *   SPH_JUDGE_PARTICLE_DENSITY (default): the mean over particles (by id) of
 *     |rho_learned - rho_plain| / rho_plain;
 *   SPH_JUDGE_MEAN_DENSITY: the deviation of the mean density,
 *     |sum rho_learned - sum rho_plain| / sum rho_plain, a much weaker bound
 *     (particles can be wrong one by one and still sum right).
 * Both are reported whichever decides. This judge state lives in the context
 * across sph_learned_step calls; an upload clears it (the metric setting stays). */
typedef struct sph_mpnn sph_mpnn;

typedef struct sph_learned_report {
    uint64_t learned_macro_steps;  /* macro-steps whose learned result was kept */
    uint64_t plain_macro_steps;    /* macro-steps (4 plain steps each) run by plain SPH */
    uint64_t judged;
    uint64_t fallbacks;            /* judged intervals that failed and were rolled back */
    double last_density_dev;       /* mean over particles of |rho_learned - rho_plain| / rho_plain at the last judge */
    double last_momentum_dev;
    double max_density_dev;
    double sum_density_dev;        /* over all judges */
    uint64_t discarded_macro_steps;/* learned macro-steps thrown away by roll-backs */
    double last_mean_rho_dev;      /* |sum rho_learned - sum rho_plain| / sum rho_plain at the last judge */
    double max_mean_rho_dev;
    double last_max_rho_dev;       /* |max rho_learned - max rho_plain| / max rho_plain at the last judge */
    double max_max_rho_dev;
} sph_learned_report;

#define SPH_JUDGE_MEAN_DENSITY      0
#define SPH_JUDGE_PARTICLE_DENSITY  1

uint32_t sph_mpnn_num_params(void);
/* Network with a training workspace for frames of up to n_frame particles. */
sph_status sph_mpnn_create(uint32_t n_frame, void* stream, sph_mpnn** out);
sph_status sph_mpnn_destroy(sph_mpnn* net);
const char* sph_mpnn_last_error(const sph_mpnn* net);
/* FP32 parameter vector in the layout We1, be1, Wn1, bn1, Wp, We2, be2, Wn2, bn2, Wo, bo. */
sph_status sph_mpnn_set_params(sph_mpnn* net, const float* params, uint32_t n);
sph_status sph_mpnn_get_params(sph_mpnn* net, float* params, uint32_t n);
/* Loss, outputs and gradient of one frame given in host memory (n particles; pos4/vel4
 * n x 4, rhop2 n x 2 (rho, pres), nb n x 32 (-1 padded), cnt n, target8 n x 8 = (O_v, O_x, 0, 0);
 * fc = {h, c = sqrt(k), rho_self, rho0, log10(mu)/4, c dt / h}). The loss is the mean over
 * particles of |O - target|^2. out8: n x 8 (O_v, O_x, 0, 0), grad: num_params. */
sph_status sph_mpnn_loss_grad(sph_mpnn* net, uint32_t n, const float* pos4, const float* vel4,
                              const float* rhop2, const int32_t* nb, const int32_t* cnt,
                              const float* target8, const float fc[6], double* loss, float* out8,
                              float* grad);
/* Network output (n x 8: O_v, O_x, 0, 0) of a host frame as above: precision 1 runs the
 * mma.sync inference kernels (BF16, FP32 accumulation), 4 the macro-step's default inference
 * (round 1 tcgen05 with the features on the tensor-memory lanes, round 2 mma.sync), 3 the
 * tcgen05 kernels of sph_mpnn_set_precision(net, 2), 0 the FP32 training forward, 2 the
 * training forward with the node layers on the BF16 tensor-core GEMMs. */
sph_status sph_mpnn_forward(sph_mpnn* net, uint32_t n, const float* pos4, const float* vel4,
                            const float* rhop2, const int32_t* nb, const int32_t* cnt, const float fc[6],
                            int32_t precision, float* out8);
/* Diagnostics of the BF16 tensor-core GEMM that the training passes use (tcgen05 MMA,
 * FP32 accumulation in tensor memory): D = A B^T for host arrays A (m x k) and B (n x k),
 * bf16 bit patterns, row-major; D (splits x m x n) FP32, one m x n partial per K slice
 * (splits = 1: the product). k and n multiples of 16, n <= 256 (16, 32, 64, 80, 128 or
 * 144). Synchronous; SPH_ERR_DEVICE if a tensor-core wait timed out. */
sph_status sph_tc_gemm_bf16(const uint16_t* a, const uint16_t* b, int32_t m, int32_t n, int32_t k, int32_t splits,
                            float* d);
/* Inference kernels of sph_learned_step, all BF16 on the tensor cores with FP32 accumulation
 * unless 0: 3 (default) round 1 as tcgen05 MMAs with the features on the tensor-memory lanes
 * and round 2 as mma.sync; 1 both rounds mma.sync; 2 both rounds tcgen05 with the edges on the
 * tensor-memory lanes (slower: the edge sum crosses lanes); 0 FP32 CUDA cores. */
sph_status sph_mpnn_set_precision(sph_mpnn* net, int32_t precision);
/* Precision of the training passes (sph_mpnn_loss_grad, sph_mpnn_train): 1 (default) runs
 * the node layers -- forward, data gradients and weight gradients -- as BF16 GEMMs on the
 * tensor cores (tcgen05, FP32 accumulation, FP32 master weights in Adam); 0 runs every layer
 * in FP32 on the CUDA cores. The per-edge layers run in FP32 either way. */
sph_status sph_mpnn_set_train_precision(sph_mpnn* net, int32_t precision);
/* Record n_frames frames of every scene of ctx (created with SPH_FLAG_KEEP_FORCE): the state,
 * its neighbour lists and density, and as targets (O_v, O_x) of the next 4 plain steps from
 * the forces alone (no wall clamp). Advances ctx by 4 * n_frames steps. */
sph_status sph_mpnn_record(sph_mpnn* net, sph_ctx* ctx, uint32_t n_frames, uint32_t* frames_total);
sph_status sph_mpnn_clear_frames(sph_mpnn* net);
/* `steps` Adam steps (lr), each on one recorded frame drawn from `seed`; loss_per_step may be NULL. */
sph_status sph_mpnn_train(sph_mpnn* net, uint32_t steps, float lr, uint64_t seed, float* loss_per_step);
/* n_macro learned macro-steps (4*dt each) on a single-scene context, judged as above
 * (judge_every = 0: never). */
sph_status sph_learned_step(sph_ctx* ctx, sph_mpnn* net, int32_t n_macro, int32_t judge_every,
                            float density_tol, float momentum_tol, sph_learned_report* report);
/* The density deviation the judge of sph_learned_step compares with density_tol:
 * SPH_JUDGE_PARTICLE_DENSITY (default) or SPH_JUDGE_MEAN_DENSITY. */
sph_status sph_learned_set_judge(sph_ctx* ctx, int32_t metric);
/* A further bound of the judge: the interval also fails when the maximum density deviates by
 * more than tol, |max rho_learned - max rho_plain| / max rho_plain (default: no bound). The
 * mean density can stay within 1% while a network packs particles into clusters; the
 * maximum density shows that. */
sph_status sph_learned_set_max_density_tol(sph_ctx* ctx, float tol);
/* Recompute rho and pres at the current positions (the state is re-sorted by cell). */
sph_status sph_refresh_density(sph_ctx* ctx);
/* The learned macro-step's input lists at the current positions, by particle id (record
 * order): the <= 32 nearest neighbours j != i with r < h (FP32 canonical distance; ids, -1
 * padded; nb_ids n x 32), their number, and rho (as the density pass computes it). The state
 * is re-sorted by cell as by sph_refresh_density. */
sph_status sph_neighbor_lists(sph_ctx* ctx, int32_t* nb_ids, int32_t* counts, float* rho);

/* ---- diagnostics without allocation -------------------------------------
 * No counterpart in the reference.
 *
 * sph_reduce_aos_noalloc: the FP64 sums behind sph_diag for n particle
 * records in the CALLER's device buffer, written to the caller's device
 * buffer dev_sums[12]:
 *   0-2 sum m v, 3 sum 1/2 m |v|^2, 4 sum -m G.x, 5 sum rho (extras[0]),
 *   6 min rho, 7 max rho, 8 sum |rho - rho0| / rho0, 9 non-finite records,
 *   10 finite records, 11 sum rho^2
 * (records with a NaN/Inf in pos, vel or rho are counted in 9 and left out of
 * every other field). Uses mass, resting_rho and gravity of *p.
 *
 * It exists for callers that cannot allocate device memory at the point they
 * need it: a render or game loop that reserves its GPU memory up front and
 * must not allocate per frame, or a plugin host that owns every buffer and
 * hands the library only pointers. It calls no cudaMalloc/cudaFree: its scratch is a fixed 96 KiB
 * array in device memory, which every GPU that loads this library holds until
 * the process exits.
 *   - n <= 4,194,304 records; larger n returns SPH_ERR_CAPACITY.
 *   - Asynchronous on `stream` (cudaStream_t, NULL = legacy default stream).
 *   - Every call looks up the scratch array's device address in the
 *     context current on the calling thread (the device's primary context,
 *     or a caller's own driver context), so a reset device or a second
 *     context never sees a stale address. The first call in a context also
 *     loads the library's device code there: make that first call before
 *     any stream capture.
 *   - All calls share the scratch: calls that overlap on the GPU (different
 *     streams without ordering between them) race and give wrong sums. */
sph_status sph_reduce_aos_noalloc(const sph_particle* dev_particles, uint32_t n, const sph_params* p,
                                  double* dev_sums, void* stream);

/* ---- static obstacles (new; the reference lists "objects to collide with" as
 * future work, README.md:59, and loads its meshes with LoadMesh, LoadMesh.cpp:16-55)
 * An obstacle is a signed distance field sampled on a regular grid: sample
 * (i, j, k) at origin + spacing * (i, j, k), stored x fastest, negative inside.
 * Every step, after the wall clamp of integrate_comp.glsl:45-77, a particle at
 * x with phi(x) < 0 (phi: trilinear interpolation of the samples; no obstacle
 * outside the sampled box) is moved out along n = g / |g|, g the trilinear
 * interpolation of the samples' central-difference gradients (one-sided on the
 * grid's faces), and its velocity's normal component gets the walls' rule,
 * v_n *= -damping:
 *   x -= phi(x) n;   if v.n < 0: v -= (1 + damping) (v.n) n;
 * then the position is clamped into the box again (velocity unchanged). The
 * learned macro-step applies the same rule after its update. One obstacle per
 * context; in a batch it applies to every scene, in each scene's coordinates. */

/* Set (sdf non-NULL) or remove (sdf NULL) the obstacle. dims >= 2 per axis, at most
 * 2^28 samples; spacing > 0. The samples are copied to the device. */
sph_status sph_set_obstacle(sph_ctx* ctx, const float* sdf, const int32_t dims[3], const float origin[3],
                            float spacing);

/* Signed distance field of a closed triangle mesh on the grid above, computed on the
 * current device: |phi| = the distance to the nearest triangle, negative where the
 * generalised winding number of the mesh exceeds 1/2 (the sum over triangles of their
 * solid angles, Van Oosterom and Strackee's formula, over 4 pi). verts: nv x 3 floats,
 * tris: nt x 3 vertex indices (counter-clockwise seen from outside), sdf_out: host array
 * of dims[0] * dims[1] * dims[2] floats. */
sph_status sph_sdf_from_mesh(const float* verts, uint32_t nv, const uint32_t* tris, uint32_t nt,
                             const int32_t dims[3], const float origin[3], float spacing, float* sdf_out);

/* Vertices and triangles of a Wavefront OBJ file (no GPU needed): `v x y z` and `f`
 * lines (vertex index forms a, a/b, a/b/c, a//c; negative indices count from the end;
 * polygons are split into a fan of triangles); other lines are ignored. In: *nv, *nt
 * the capacities of verts (nv x 3 floats) and tris (nt x 3); out: the file's counts.
 * With verts or tris NULL only the counts are returned. SPH_ERR_CAPACITY when the
 * arrays are too small, SPH_ERR_INVALID_ARG for a missing file or a bad index. */
sph_status sph_obj_read(const char* path, float* verts, uint32_t* nv, uint32_t* tris, uint32_t* nt);

/* ---- headless toon rendering of the particles ----------------------------
 * The reference draws the particles after the step (Main.cpp:311-337, SPH
 * mode): GL point sprites of sim_rad pixels through toon_vs.glsl /
 * toon_fs.glsl in two passes. Pass 0 writes a coverage texture (its green
 * channel is a flat depth 1.0, toon_vs.glsl:44); pass 1 shades each fragment
 * with the cel model (toon_fs.glsl:90-124) and draws a Sobel outline where the
 * 3x3 neighbourhood of the coverage texture has a gradient (:126-153). This
 * library renders the same image with CUDA kernels into an RGBA8 buffer, rows
 * bottom to top as GL stores them; there is no window, GL context or swapchain.
 * The restated pipeline, per particle i (record order = draw order):
 *   clip = (P V M)(x_i, 1); kept when w > 0 and |x|,|y|,|z| <= w;
 *   window x_w = (x/w + 1) W/2, y_w = (y/w + 1) H/2, depth d = (z/w + 1)/2,
 *     quantised to 24 bits;
 *   covered pixels: centres within [x_w - s/2, x_w + s/2) x [y_w - s/2, y_w + s/2)
 *     (s = point_size), with p = ((c_x - x_w), -(c_y - y_w)) / (s/2) and |p|^2 <= 1
 *     (toon_fs.glsl:97-99);
 *   depth test GL_LESS: per pixel the smallest (d, i) wins;
 *   normal n = normalize(p.x, p.y, sqrt(1 - |p|^2)), pw = M (x_i, 1),
 *   l = normalize(light - pw), v = normalize(eye - pw), r = normalize(reflect(-l, n));
 *   colour = dark if dot(n, l) < 0 else midtone; highlight if dot(r, v) > 0 and
 *     dot(r, v) > 0.95^(1/shininess) (the exact form of pow(dot(r,v), shininess) > 0.95);
 *   outline colour where the Sobel gradient of the coverage (outside the image:
 *     uncovered) is non-zero; clear colour where nothing is covered; alpha 1.
 * Every operation is FP32 with round-to-nearest, so the CPU restatement
 * matches the image byte for byte. */
typedef struct sph_view {
    float model[16];       /* M, column-major (glm): rotate(angle, y) * scale (Main.cpp:256) */
    float view[16];        /* V = lookAt(eye, center, up y) (Main.cpp:257) */
    float proj[16];        /* P = perspective(pi/4, aspect, 0.1, 100) (Main.cpp:258) */
    float eye_w[4];        /* SceneUniforms.eye_w (Main.cpp:105) */
    float light_w[4];      /* SceneUniforms.light_w (Main.cpp:106) */
    float dark[4];         /* MaterialUniforms (Main.cpp:126-133) */
    float midtone[4];
    float highlight[4];
    float outline[4];
    float clear_color[4];  /* clear_color (Main.cpp:80) */
    float shininess;       /* 0.3; >= 0 */
    float point_size;      /* sim_rad, pixels (Main.cpp:88): 10 */
    int32_t width, height;
} sph_view;

/* The reference's initial view (Main.cpp:80-89, :105-106, :126-133, :254-260): angle 0.75,
 * scale 2.5 (times model_scale, the loaded mesh's mScaleFactor in the reference), eye
 * (10, 2, 0) looking at the origin, light (0, 1, 1), aspect width/height. */
sph_status sph_view_default(sph_view* v, int32_t width, int32_t height, float model_scale);
/* M, V and P as sendUniforms builds them (Main.cpp:256-258) for the given camera. */
sph_status sph_view_camera(sph_view* v, float angle, float scale, const float eye[3], const float center[3]);
/* Render the context's particles (a single-scene context, or scene `scene` of a batch) into
 * rgba (width x height x 4 bytes, rows bottom to top), in device memory when rgba_on_device,
 * else in host memory. */
sph_status sph_render(sph_ctx* ctx, const sph_view* v, uint32_t scene, uint8_t* rgba, int32_t rgba_on_device);
/* Write an RGBA8 image (rows bottom to top) as a binary PPM (rows top to bottom, RGB). */
sph_status sph_image_write_ppm(const char* path, const uint8_t* rgba, int32_t width, int32_t height);

/* ---- snapshots and trajectories (new; no reference counterpart) --------
 * The reference keeps its state only in the GL buffer and re-creates it on 'r'
 * (Main.cpp:460-464). A snapshot file holds what resumes a run bit for bit:
 * the records in caller order, the uniforms and particle count of every scene
 * and the step count, with a checksum. The obstacle (sph_set_obstacle), the launch
 * shape and the learned judge's settings are not part of it: set them again after a
 * load. A trajectory file is the same header
 * followed by frames appended during a run. Format (little-endian):
 *   64-byte header: magic "NPRSPHS1" (snapshot) / "NPRSPHT1" (trajectory),
 *     u32 version 1, u32 header bytes 64, u64 particles, u32 scenes, u32 flags,
 *     u64 step count (trajectory: 0), u64 seed (a caller tag), u64 checksum
 *     (snapshot: of all bytes after the header; trajectory: of the scene
 *     table), u64 0;
 *   scene table: scenes x sph_params, scenes x u32 counts, zero padding to a
 *     multiple of 64 bytes;
 *   snapshot: particles x sph_particle; then, when flags bit 0 is set, particles x
 *     u32: the record index at each slot of the device state (the within-cell order
 *     the next neighbour sort keeps; restoring it makes a resumed run repeat the
 *     original bit for bit; sph_snapshot_save always writes it);
 *   trajectory frames: u64 step, u64 particles, u64 checksum of the records,
 *     u64 0, particles x sph_particle.
 * Checksum: FNV-1a 64 over the 64-bit little-endian words of the bytes (a final
 * partial word zero-padded), sph_checksum64. */
typedef struct sph_trajectory sph_trajectory;

sph_status sph_snapshot_save(sph_ctx* ctx, const char* path, uint64_t seed);
/* Header fields of a snapshot file (no GPU needed). */
sph_status sph_snapshot_info(const char* path, uint64_t* n, uint32_t* n_scene, uint64_t* steps, uint64_t* seed);
/* SPH_OK when the file is a complete snapshot whose checksum matches (no GPU needed). */
sph_status sph_snapshot_verify(const char* path);
/* A new context (single-scene or batch, as saved) holding the snapshot's particles and
 * uniforms, with the step count continued. A file that fails verification is refused. */
sph_status sph_snapshot_load(const char* path, void* stream, sph_ctx** out);
sph_status sph_trajectory_create(sph_ctx* ctx, const char* path, uint64_t seed, sph_trajectory** out);
/* Append the context's current records as one frame. */
sph_status sph_trajectory_append(sph_trajectory* t, sph_ctx* ctx);
uint64_t sph_trajectory_frames(const sph_trajectory* t);
sph_status sph_trajectory_close(sph_trajectory* t);
uint64_t sph_checksum64(const void* data, uint64_t bytes);

/* ---- scene generators (host only; no GPU needed) ----------------------- */

/* The reference's make_grid()+init_particles() (Main.cpp:488-539): 10x100x10
 * lattice at `spacing` (PARTICLE_RADIUS), i-j-k loop order, w = 1, all other
 * fields zero. n must be 10000. */
sph_status sph_scene_reference_grid(sph_particle* out, uint32_t n, float spacing);

/* n particles on a cubic lattice of `spacing` inside [lo, hi], first point at
 * lo + spacing/2, filled x fastest, then z, then y (bottom layer first); each
 * coordinate jittered by U(-jitter, +jitter) from `seed`. Zero velocity, w = 1.
 * SPH_ERR_CAPACITY if the region holds fewer than n points. */
sph_status sph_scene_fill(sph_particle* out, uint32_t n, const float lo[3], const float hi[3],
                          float spacing, float jitter, uint64_t seed);

/* The n lattice points (spacing, jittered as above) nearest to `center`:
 * a ball of fluid for a sphere-drop scene. */
sph_status sph_scene_ball(sph_particle* out, uint32_t n, const float center[3],
                          float spacing, float jitter, uint64_t seed);

/* Add vel.x += amplitude * sin(pi * (pos.x - x0) / length) (sloshing field). */
sph_status sph_scene_slosh(sph_particle* out, uint32_t n, float amplitude, float x0, float length);

#ifdef __cplusplus
} /* extern "C" */
#endif

#endif /* SPH_GB300_H */
