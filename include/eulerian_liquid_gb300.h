/*
 * eulerian_liquid_gb300.h -- C ABI of the GB300 (sm_103a) implementation of the
 * daichi-nama/eulerian-liquid per-step grid hot path: semi-Lagrangian (trilinear / WENO6,
 * RK2 / RK3) advection of the MAC velocity and the level set, and the ghost-fluid PCG
 * pressure projection, plus the step pieces on either side of them.
 *
 * Conventions
 *   - Every function returns an int status (EL_OK = 0); no exception crosses the ABI.
 *     el_ctx_last_error() gives a one-line message for the last failure on a context.
 *   - Arrays are i-fastest, flat index i + n0*(j + n1*k), exactly the reference's layout
 *     (include/nama/common/array.h:281-286), so a host Grid3f / StaggeredGrid3f component
 *     uploads with one contiguous copy.
 *       phi, pressure, cell solid phi, indices : ni x nj x nk
 *       u, weight_u, valid_u                    : (ni+1) x nj x nk
 *       v, weight_v, valid_v                    : ni x (nj+1) x nk
 *       w, weight_w, valid_w                    : ni x nj x (nk+1)
 *       nodal solid phi                         : (ni+1) x (nj+1) x (nk+1)
 *     Grid origins: cells at (0,0,0), faces shifted by -dx/2 along their normal, nodes by
 *     -dx/2 on every axis (include/nama/common/staggered_grid.h:100-112,
 *     src/project/3d/eulerian_liquid/simulator.cpp:52-70).
 *   - Field type is chosen per context: EL_F32 (the reference's Grid3f) or EL_F64.  The
 *     matrix diagonal, right-hand side and solution are always double, as in
 *     src/project/3d/fluid/projection.cpp:30-33.
 *   - One CUDA stream per context (its own, or one given with el_ctx_set_stream).  Calls
 *     on one context are not re-entrant, like the reference's Simulator.
 */
#ifndef EULERIAN_LIQUID_GB300_H
#define EULERIAN_LIQUID_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------------------- */
#define EL_OK 0
#define EL_ERR_INVALID_ARGUMENT 1
#define EL_ERR_NO_FLUID 2      /* projection.cpp:24-26 throws std::runtime_error("No fluid") */
#define EL_ERR_NOT_CONVERGED 3 /* simulator.cpp:107-109 never checks solver.info(); we report */
#define EL_ERR_NAN 4           /* a non-finite residual or field was detected */
#define EL_ERR_CUDA 5
#define EL_ERR_OUT_OF_MEMORY 6
#define EL_ERR_TIMEOUT 7 /* a bounded device wait gave up */

/* ---- field types and ids ------------------------------------------------------------ */
#define EL_F32 0
#define EL_F64 1

enum el_field {
    EL_FIELD_PHI = 0,         /* Simulator::m_level_set            (simulator.h:68)     */
    EL_FIELD_U = 1,           /* Simulator::m_velocity.u()         (simulator.h:64)     */
    EL_FIELD_V = 2,
    EL_FIELD_W = 3,
    EL_FIELD_SOLID_NODAL = 4, /* Simulator::m_nodal_solid_phi      (simulator.h:73)     */
    EL_FIELD_WEIGHT_U = 5,    /* Simulator::m_velocity_weight.u()  (simulator.h:66)     */
    EL_FIELD_WEIGHT_V = 6,
    EL_FIELD_WEIGHT_W = 7,
    EL_FIELD_PRESSURE = 8,    /* Simulator::m_pressure             (simulator.h:71)     */
    EL_FIELD_SOLID_CELL = 9,  /* m_cell_centered_solid_level_set   (simulator.h:74)     */
    EL_FIELD_VALID_U = 10,    /* m_velocity_valid.u(), uint8       (simulator.h:65)     */
    EL_FIELD_VALID_V = 11,
    EL_FIELD_VALID_W = 12,
    EL_FIELD_VALID_PHI = 13,  /* m_level_set_valid, uint8          (simulator.h:69)     */
    EL_FIELD_INDICES = 14,    /* m_indices, int32 (INT_MAX = not a fluid cell) (simulator.h:70) */
    EL_FIELD_COUNT = 15
};

/* ---- advection schemes -------------------------------------------------------------- */
#define EL_TRACE_RK2 0        /* math::trace_rk2, midpoint rule (include/nama/math/ode.h:30-35) */
#define EL_TRACE_RK3 1        /* Ralston RK3 (new; the reference has RK1/RK2 only)          */
#define EL_SAMPLE_TRILINEAR 0 /* math::lerp(x, grid) (include/nama/math/interpolation.h:35-72) */
#define EL_SAMPLE_WENO6 1     /* math::weno6_interp(x, grid) (interpolation.h:139-184)      */

/* ---- pressure solver ---------------------------------------------------------------- */
#define EL_SOLVER_JACOBI_FP64 0 /* plain FP64 PCG, Jacobi preconditioner                     */
#define EL_SOLVER_MG_FP64 1     /* FP64 PCG, multigrid V-cycle preconditioner                */
#define EL_SOLVER_MIXED 2       /* FP32 multigrid PCG inside FP64 iterative refinement       */

typedef struct el_solve_params {
    int solver;         /* EL_SOLVER_*                                                   */
    double tol;         /* relative residual |b - A p| / |b| to reach (reference: 1e-4)  */
    int max_iter;       /* PCG iteration cap, inner iterations summed for EL_SOLVER_MIXED */
    int check_every;    /* host convergence poll period in iterations (>= 1)             */
    int max_outer;      /* EL_SOLVER_MIXED: refinement sweeps cap                        */
    double inner_floor; /* EL_SOLVER_MIXED: smallest inner relative tolerance (FP32)     */
    int initial_guess;  /* 1: start from the EL_FIELD_PRESSURE grid as it stands (a warm
                           start, Eigen's solveWithGuess) instead of zero; the guess is first
                           scaled by the factor that minimises its energy-norm error,
                           (g.b)/(g.Ag), so it never starts worse than zero does        */
} el_solve_params;

typedef struct el_solve_stats {
    int status;          /* EL_OK, EL_ERR_NOT_CONVERGED, EL_ERR_NO_FLUID, EL_ERR_NAN        */
    int iterations;      /* PCG iterations (inner iterations summed for EL_SOLVER_MIXED)   */
    int outer_iterations;/* refinement sweeps (EL_SOLVER_MIXED), else 1                    */
    int fluid_cells;     /* matrix size: what assign_indices returns (projection.cpp:14-28)  */
    double relres;       /* final relative residual the solver stopped on                  */
} el_solve_stats;

typedef struct el_step_params {
    int trace_phi, sample_phi;   /* level-set advection scheme                              */
    int trace_vel, sample_vel;   /* velocity advection scheme                               */
    double gravity;              /* m/s^2 subtracted from v (reference: 9.80665)            */
    int extrapolation_layers;    /* reference: 10 (simulator.cpp:115-123)                   */
    el_solve_params solve;
} el_step_params;

typedef struct el_step_stats {
    double dt;
    el_solve_stats solve;
} el_step_stats;

typedef struct el_ctx el_ctx;

/* ---- context ------------------------------------------------------------------------ */
/* Simulator::create_grid (src/project/3d/eulerian_liquid/simulator.cpp:52-70): allocate a
 * device-resident scene of ni x nj x nk cells of size dx.  All fields start at zero except
 * the valid masks (1), as in create_grid.  device = CUDA ordinal. */
int el_ctx_create(int ni, int nj, int nk, double dx, int dtype, int device, el_ctx** out);
int el_ctx_destroy(el_ctx* ctx);
const char* el_ctx_last_error(const el_ctx* ctx);
const char* el_status_string(int status);
/* Use the caller's stream (a cudaStream_t) for all work on this context; NULL = own stream. */
int el_ctx_set_stream(el_ctx* ctx, void* cuda_stream);
void* el_ctx_get_stream(el_ctx* ctx);
int el_ctx_sync(el_ctx* ctx);
/* Number of kernels this library launched on the context since creation. */
int64_t el_ctx_kernel_launches(const el_ctx* ctx);

/* Launch shapes of the context's kernels (no counterpart in the reference).  Results do not
 * depend on them beyond the summation order of the device reductions.  A batch takes the
 * shapes its scenes have when it is created. */
typedef struct el_tuning {
    int seg_blocks_per_sm;       /* solver kernels over active row segments, 1..8 (default 8)   */
    int stencil_blocks_per_sm;   /* matrix build, masks, element-wise kernels, 1..16 (default 16)*/
    int extrapolate_blocks_per_sm; /* extrapolation tiles in flight per SM, 1..16 (default 12)  */
    int advect_rows;             /* per-sample advection: 32 x rows cells per block, 1, 2, 4 or 8 */
    int advect_tiled;            /* 1 (default): advection kernels that stage the velocity of a
                                    32x8x8 tile in shared memory, its boxes by TMA box copies
                                    where an array's row pitch is a multiple of 16 bytes; 2: the
                                    same kernels with every box staged by plain loads (identical
                                    results); 0: one thread per sample                          */
    int solver_tiles;            /* 1 (default): the mixed solver's finest level on the z-marching
                                    tile kernels with TMA-staged planes, where the grid allows
                                    (ni a multiple of 8, at least 64 x 16 x 16 cells); 0: the
                                    row-segment kernels everywhere                              */
    int coarse_fused;            /* 1: the mixed solver's multigrid levels below the finest, and
                                    the bottom pair, in one cooperative launch per V-cycle
                                    (identical results); 2: the same from the second level below
                                    the finest on; 0 (default): one launch per level pass      */
    int dependent_launch;        /* 1 (default): the mixed solver's chained kernels (finest-level
                                    tile kernels, coarse-level passes, the bottom) are launched as
                                    programmatic dependent launches, so that each is scheduled
                                    while the one before it drains (identical results); 0: not  */
} el_tuning;
int el_ctx_set_tuning(el_ctx* ctx, const el_tuning* t);
int el_ctx_get_tuning(const el_ctx* ctx, el_tuning* t);
/* *on = 1 when the mixed solver's finest level runs on the z-marching tile kernels on this
 * context (solver_tiles set and the grid meets their conditions), else 0 (no counterpart in the
 * reference).  Sets up the mixed solver's storage first if no mixed solve has run yet. */
int el_ctx_solver_tiles_active(el_ctx* ctx, int* on);

/* ---- per-kernel-class timing ---------------------------------------------------------
 * While profiling is on, every launch of a class in `class_mask` (bit = 1 << EL_KC_*) is
 * bracketed by CUDA events on the context's stream; el_ctx_profile_end synchronises and
 * returns, per class, the launches, their summed device time and their summed algorithmic
 * bytes (each array a kernel must read or write counted once per launch). */
enum el_kernel_class {
    EL_KC_ADVECT_PHI = 0,   /* level-set advection                                   */
    EL_KC_ADVECT_VEL = 1,   /* velocity advection (one launch per face component)    */
    EL_KC_EXTRAPOLATE = 2,  /* extrapolation layers                                  */
    EL_KC_MASKS = 3,        /* gravity + valid masks + zeroing                       */
    EL_KC_BUILD = 4,        /* cell flags + ghost-fluid coefficients                 */
    EL_KC_DIR_SPMV = 5,     /* PCG: p = z + beta p fused with A p and p.Ap           */
    EL_KC_UPDATE = 6,       /* PCG: x, r update fused with the residual norms        */
    EL_KC_SMOOTH = 7,       /* multigrid smoothing on the finest level               */
    EL_KC_RESTRICT = 8,     /* multigrid residual + restriction from the finest level */
    EL_KC_MG_COARSE = 9,    /* all multigrid work below the finest level             */
    EL_KC_RESIDUAL = 10,    /* FP64 refinement residual r = b - A x                  */
    EL_KC_OTHER = 11,
    EL_KC_COUNT = 12
};

typedef struct el_profile_entry {
    int64_t launches;
    double ms;
    double bytes;
} el_profile_entry;

int el_ctx_profile_begin(el_ctx* ctx, uint32_t class_mask);
/* out must hold EL_KC_COUNT entries */
int el_ctx_profile_end(el_ctx* ctx, el_profile_entry* out);

/* Debug build (libeulerian_liquid_gb300_checked.so, compiled with -DEL_CHECKED; no counterpart
 * in the reference): the kernels check each global store index (and their indirect loads)
 * against the array before the access, skip a failed access and record it.  *checked = 1 in
 * that build, 0 in the product build (where *word is always 0); *word = the first failed check
 * since the last call, (site << 40) | index, or 0.  Reading clears it.  Call it between steps,
 * with no work of the library in flight. */
int el_debug_check_take(uint64_t* word, int* checked);

/* Host <-> device copies of a whole field (bytes must equal the field's size). */
int el_upload(el_ctx* ctx, int field, const void* host, size_t bytes);
int el_download(el_ctx* ctx, int field, void* host, size_t bytes);
/* The same copies enqueued on `stream` (a cudaStream_t; NULL = the context's stream) without
 * waiting for them (no counterpart in the reference, whose grids live in host memory): the
 * caller orders them against the context's work (e.g. with events on el_ctx_get_stream), keeps
 * `host` alive until they complete, and gets overlapped transfers only from pinned memory.
 * Downloads and uploads of different fields on two streams run at the same time (the host link
 * is full duplex). */
int el_upload_async(el_ctx* ctx, int field, const void* host, size_t bytes, void* stream);
int el_download_async(el_ctx* ctx, int field, void* host, size_t bytes, void* stream);
/* Device pointer of a field, for zero-copy use by a caller that owns device memory. */
int el_field_device_ptr(el_ctx* ctx, int field, void** dptr, size_t* bytes);

/* ---- scene set-up (src/project/3d/fluid/levelset_emitter.cpp:10-79) -------------------
 * target 0 = liquid level set (cell centres), 1 = nodal solid level set.  Each emitter
 * writes min(field, f(x)); el_emit_clear fills with FLT_MAX like LevelSetEmitterList::apply. */
int el_emit_clear(el_ctx* ctx, int target);
int el_emit_sphere(el_ctx* ctx, int target, double cx, double cy, double cz, double r);
int el_emit_pool(el_ctx* ctx, int target, double height);
int el_emit_box(el_ctx* ctx, int target, const double lo[3], const double hi[3]);
int el_emit_room(el_ctx* ctx, int target);

/* ---- boundary (init time) ---------------------------------------------------------- */
int el_compute_weights(el_ctx* ctx);            /* fluid::compute_staggered_grid_weight, boundary.cpp:6-34 */
int el_calc_cell_centered_solid_phi(el_ctx* ctx);/* simulator.cpp:191-200 */
int el_find_valid_level_set(el_ctx* ctx);       /* simulator.cpp:160-167 */

/* ---- hot path: Simulator step methods (include/nama/project/3d/eulerian_liquid/simulator.h:32-53) */
int el_advect_level_set(el_ctx* ctx, double dt, int trace, int sample); /* simulator.cpp:84-87 */
int el_advect_velocity(el_ctx* ctx, double dt, int trace, int sample);  /* simulator.cpp:79-82 */
int el_add_gravity(el_ctx* ctx, double dt, double gravity);             /* simulator.cpp:90-93 */
int el_extrapolate_level_set(el_ctx* ctx, int layers);                  /* simulator.cpp:115-117 */
int el_extrapolate_velocity(el_ctx* ctx, int layers);                   /* simulator.cpp:119-123 */
int el_find_valid_velocity(el_ctx* ctx);                                /* simulator.cpp:125-158 */
int el_set_invalid_velocity_zero(el_ctx* ctx);                          /* simulator.cpp:169-178 */
int el_solve_pressure(el_ctx* ctx, double dt, const el_solve_params* params,
                      el_solve_stats* stats);                           /* simulator.cpp:96-112 */
/* fluid::calc_time_step (src/project/3d/fluid/time_stepping.cpp:5-7): cfl*dx/max(max|u|,1e-4) */
int el_calc_time_step(el_ctx* ctx, double cfl, double* dt_out);
/* update_second_order (apps/eulerian_liquid_3d.cpp:106-120) without reinitialize(), which
 * stays the reference's own CPU code: extrapolate velocity and level set, advect level set,
 * advect velocity, gravity, valid masks, zero invalid faces, solve pressure. */
int el_step(el_ctx* ctx, double dt, const el_step_params* params, el_step_stats* stats);

/* ---- projection pieces (include/nama/project/3d/fluid/projection.h:10-22) ------------- */
/* assign_indices (projection.cpp:14-28): k-j-i numbering into EL_FIELD_INDICES. */
int el_assign_indices(el_ctx* ctx, int* mat_size);
/* build_matrix (projection.cpp:30-83) into the context's grid-shaped coefficients. */
int el_build_matrix(el_ctx* ctx, double dt);
/* Copy the grid-shaped matrix out as doubles (ni*nj*nk each): diagonal, the couplings of
 * each cell with its +x / +y / +z neighbour, and the right-hand side.  Any may be NULL. */
int el_download_matrix(el_ctx* ctx, double* diag, double* offx, double* offy, double* offz,
                       double* rhs);
/* build_grid_from_vector + update_velocity_using_pressure (projection.cpp:85-134) using the
 * EL_FIELD_PRESSURE grid as it stands (after a solve, or after el_upload). */
int el_update_velocity_using_pressure(el_ctx* ctx, double dt);

/* ---- stateless operators on caller-owned device memory ------------------------------
 * The reference's free functions (include/nama/project/3d/fluid/advection.h:8-11,
 * boundary.h:8) over raw device pointers; no allocation, work enqueued on `stream`. */
typedef struct el_grid {
    int ni, nj, nk;
    double dx;
} el_grid;

/* advect_collocated_grid (advection.cpp:9-16): out = in(trace(x, -dt, vel)) at cell centres */
int el_advect_collocated_grid(const el_grid* g, int dtype, void* out, const void* in,
                              const void* vel_u, const void* vel_v, const void* vel_w,
                              double dt, int trace, int sample, void* stream);
/* advect_staggered_grid (advection.cpp:18-27): each face component of `in` through `vel` */
int el_advect_staggered_grid(const el_grid* g, int dtype, void* out_u, void* out_v, void* out_w,
                             const void* in_u, const void* in_v, const void* in_w,
                             const void* vel_u, const void* vel_v, const void* vel_w,
                             double dt, int trace, int sample, void* stream);
/* compute_staggered_grid_weight (boundary.cpp:6-34) */
int el_compute_staggered_grid_weight(const el_grid* g, int dtype, void* weight_u, void* weight_v,
                                     void* weight_w, const void* nodal_solid, void* stream);

/* ---- state dump / restore -----------------------------------------------------------
 * No counterpart in the reference (its only dumps are OBJ meshes and 2D text slices).  Writes
 * every field but EL_FIELD_INDICES (derived) to `path`, raw, behind a 64-byte header, so that a
 * run restarts exactly: header {char magic[8] = "ELGBSTAT"; uint32 version = 1; uint32 dtype;
 * int32 ni, nj, nk; uint32 nfields; double dx; double time; 16 zero bytes}, then per field
 * {uint32 field; uint32 element bytes; uint64 byte count; bytes in the layout of el_upload};
 * little-endian.  el_state_load checks magic, version, grid and field type against the context
 * and reads the whole file before changing anything; `time` is the caller's. */
int el_state_save(el_ctx* ctx, const char* path, double time);
int el_state_load(el_ctx* ctx, const char* path, double* time);

/* ---- batched scenes: many contexts advanced by one graph launch per step ----------------
 * No counterpart in the reference, which runs one Simulator per process.  A batch applies the
 * reference's Simulator::update(update_second_order, dt_frame, use_cfl=true) loop
 * (simulator.cpp:23-42, apps/eulerian_liquid_3d.cpp:106-120, reinitialize() excluded) to every
 * scene at once: each batch step is one sub-step of every scene, with the scene's own
 *   dt_sub = calc_time_step(cfl) (time_stepping.cpp:5-7), cut to end the frame exactly,
 * computed on the device, then el_step's work with EL_SOLVER_MIXED, whose refinement and PCG
 * loops run on the device (conditional graph nodes).  All scenes' steps form ONE CUDA graph
 * (a branch per scene, run concurrently), launched once per batch step.
 *   - scenes must be distinct contexts on one device, profiling off, solver EL_SOLVER_MIXED;
 *   - the graph holds the contexts' device buffers: destroy the batch before its contexts, and
 *     do not step a scene outside the batch between batch steps (el_batch_step checks);
 *   - uploads and downloads through the contexts are ordered with the batch's launches. */
typedef struct el_batch el_batch;

typedef struct el_batch_stats {
    int64_t steps;             /* sub-steps taken */
    int64_t frames;            /* frames completed (sub-steps summing to dt_frame) */
    int64_t iterations;        /* inner PCG iterations, summed */
    int64_t outer_iterations;  /* refinement sweeps, summed */
    int64_t kernels;           /* kernels the scene's branch ran */
    int64_t unconverged_steps; /* solves that stopped at max_iter / max_outer */
    int64_t no_fluid_steps;    /* projections with no fluid cell ("No fluid") */
    int64_t bad_steps;         /* non-finite residuals */
    double time;               /* simulated time */
    double last_dt;
    double max_relres;         /* largest final |r|/|b| over the steps */
    double frame_time;         /* time into the current frame */
} el_batch_stats;

int el_batch_create(el_ctx* const* scenes, int count, const el_step_params* params, double cfl,
                    double dt_frame, el_batch** out);
int el_batch_destroy(el_batch* batch);
const char* el_batch_last_error(const el_batch* batch);
/* Enqueue `steps` sub-steps (one graph launch each) on the batch's stream; returns without
 * waiting. */
int el_batch_step(el_batch* batch, int steps);
int el_batch_sync(el_batch* batch);
/* Waits for the batch, then copies `count` per-scene statistics (since creation or the last
 * reset) to `out`. */
int el_batch_stats_get(el_batch* batch, el_batch_stats* out);
int el_batch_stats_reset(el_batch* batch);
void* el_batch_get_stream(el_batch* batch);
/* Kernel nodes in the graph outside the solver loops, all scenes. */
int64_t el_batch_graph_kernels(const el_batch* batch);

/* ---- learned warm start --------------------------------------------------------------
 * No counterpart in the reference (its pressure solve always starts from zero).  A small 3D
 * convolutional encoder-decoder maps (level set, divergence, solid mask) to a pressure guess
 * that el_solve_pressure refines with initial_guess = 1.  Its kernels are below; the network,
 * the data recorder and the training loop that drive them are eulerian-liquid_gb300/warmstart.py.
 *
 * Scene side (contexts; grid sizes divisible by 8).  el_warmstart_features writes the network
 * input for the context's current system: 16 bf16 channels per cell, channels-last
 * ((k*nj + j)*ni + i)*16 + c: clamp(phi / 3dx, -1, 1), the right-hand side b / rms(b) on fluid
 * cells, the solid mask (cell-centred solid phi < 0), zeros.  With build = 1 it first builds the
 * system for time step dt (as el_build_matrix); with build = 0 it uses the one the last solve
 * built (recording after el_step).  target (nullable) receives the pressure in the same scaling,
 * p * a / rms(b) with a = mean(diagonal) / 6, couplings (nullable) the scaled operator A / a in
 * Laplacian form as 4 bf16 per cell: the diagonal's excess over the fluid faces (the
 * ghost-fluid terms) and the face weights -A(c, c+e) with the +x, +y, +z neighbours (zeros off
 * the fluid), and fluid (nullable) 1 on fluid cells: a training tuple.  el_warmstart_set_guess
 * writes pred * rms(b) / a into EL_FIELD_PRESSURE (0 off the fluid), the scaling of the last
 * el_warmstart_features call.  scales (nullable, synchronises) receives {rms(b), a, the energy
 * of the scaled solution target . (A / a) target}. */
int el_warmstart_features(el_ctx* ctx, int build, double dt, void* features, void* couplings,
                          float* target, uint8_t* fluid, double* scales);
int el_warmstart_set_guess(el_ctx* ctx, const float* pred);

/* Network side: stateless kernels on caller-owned device memory, work enqueued on `stream`.
 * Activations are bf16 channels-last (x fastest, then y, z; channels innermost), one sample.
 * A 3x3x3 convolution (zero padding, stride 1) reads the concatenation of in_a (ca channels,
 * optionally at half resolution and upsampled by nearest neighbour on the fly) and in_b (cb
 * channels); cin = ca + cb; channel counts multiples of 16 (ca, cb multiples of 8).  Supported
 * (cin, cout): (16,16) (16,32) (32,32) (32,64) (64,64) (128,64) (96,32) (48,16) and, for the
 * backward-data pass, (32,16) (64,32) (64,128) (32,96) (16,48).  BF16 tensor-core products with
 * FP32 accumulation. */
typedef struct el_nn_conv_args {
    int nx, ny, nz;          /* output grid = fine input grid                                    */
    int cin, cout;
    const void* in_a;        /* bf16 [.., ca]                                                    */
    int ca, upsample_a;      /* upsample_a: in_a is (nx/2, ny/2, nz/2)                            */
    const void* in_b;        /* bf16 [.., cb]; NULL reads cb channels of zeros                    */
    int cb;
    const void* mask;        /* NULL, or bf16 [.., cin]: input zeroed where mask <= 0 (ReLU')     */
    const void* weights;     /* packed by el_nn_pack_weights (forward or backward-data packing);
                                unused by el_nn_conv3_backward_weight                             */
    const float* bias;       /* [cout] or NULL                                                   */
    int relu;
    void* out_a;             /* bf16 [.., out_a_channels]: output channels [0, out_a_channels)    */
    int out_a_channels;
    void* out_b;             /* bf16 [.., cout - out_a_channels]: the rest (may be NULL if none)  */
    const void* weights_tc;  /* NULL, or the same weights packed by el_nn_pack_weights_tc: then
                                pairs with el_nn_tc_supported run on the tcgen05 kernel          */
} el_nn_conv_args;

/* y = act(conv(x, W) + bias).  The backward-data pass is the same call with the gradient of the
 * layer's output as in_a (ca = that layer's cout), mask = the layer's forward output (ReLU'),
 * the backward packing of W, no bias, no relu, and out_a / out_b the gradients of the layer's
 * two inputs (the upsampled part at fine resolution; see el_nn_gather8). */
int el_nn_conv3_forward(const el_nn_conv_args* args, void* stream);
/* dW[cout][27][cin] += sum_v gm[v][co] x[v + tap][ci] and db += sum_v gm, gm = grad_out * (y > 0)
 * with y = args->out_a (the layer's forward output); args describes the forward call.  FP32,
 * summed in a fixed order (deterministic). */
size_t el_nn_conv3_backward_weight_workspace(int nx, int ny, int nz, int cin, int cout);
int el_nn_conv3_backward_weight(const el_nn_conv_args* args, const void* grad_out, float* dw, float* db,
                                void* workspace, size_t workspace_bytes, void* stream);
/* FP32 master weights [cout][27][cin] -> bf16 forward packing (and, if packed_bwd is not NULL,
 * the backward-data packing of the transposed, tap-mirrored kernel); each 27*cin*cout*2 bytes. */
size_t el_nn_packed_weight_bytes(int cin, int cout);
int el_nn_pack_weights(int cin, int cout, const float* w, void* packed_fwd, void* packed_bwd, void* stream);
/* The same weights in the tcgen05 kernel's shared-memory operand layout (27*cin*cout*2 bytes
 * each), forward and (if packed_bwd is not NULL) backward data.  el_nn_tc_supported(cin, cout)
 * says whether a (cin, cout) call can use them: (16,16) (16,32) (32,32) (32,64) (48,16) (32,16)
 * (64,32) (16,48) (32,96), the pairs whose 27 taps fit in shared memory with the input brick.
 * el_nn_take_error returns (and clears) 1 if a tcgen05 kernel's bounded wait for its MMAs gave
 * up, 0 otherwise, -1 if it could not be read. */
int el_nn_pack_weights_tc(int cin, int cout, const float* w, void* packed_fwd, void* packed_bwd, void* stream);
int el_nn_tc_supported(int cin, int cout);
/* 1 where the tcgen05 kernel measured faster than the mma.sync one on GB300 (small cin) */
int el_nn_tc_preferred(int cin, int cout);
int el_nn_take_error(void);
/* 2x2x2 average pooling; its backward is el_nn_spread(scale 1/8, accumulate 1) */
int el_nn_pool(int nx, int ny, int nz, int c, const void* in, void* out, void* stream);
/* fine[v] = (accumulate ? fine[v] : 0) + scale * coarse[v / 2] ; (nx, ny, nz) = fine grid */
int el_nn_spread(int nx, int ny, int nz, int c, const void* coarse, void* fine, float scale, int accumulate,
                 void* stream);
/* coarse[V] = sum of its 8 fine children: the backward of nearest upsampling */
int el_nn_gather8(int nx, int ny, int nz, int c, const void* fine, void* coarse, void* stream);
/* head: pred[v] = w . d[v] + b over 16 channels (FP32 out) */
int el_nn_head_forward(int64_t n, const void* d, const float* w, const float* b, float* pred, void* stream);
/* masked MSE loss and the head's backward: on cells with mask != 0, e = pred - target;
 * loss[0] += sum e^2 inv_n, grad_d = 2 e inv_n w (bf16, 0 off the mask), dw[16] += dL/dw,
 * db[0] += dL/db.  The workspace (el_nn_head_workspace bytes) must be zeroed once. */
size_t el_nn_head_workspace(int64_t n);
int el_nn_head_loss_backward(int64_t n, const void* d, const float* pred, const float* target, const uint8_t* mask,
                             const float* w, double inv_n, void* grad_d, double* loss, float* dw, float* db,
                             void* workspace, size_t workspace_bytes, void* stream);
/* energy-norm loss (the norm conjugate gradients minimises) and the head's backward, on the
 * (nx, ny, nz) grid: e = pred - target on cells with fluid != 0, loss[0] += e . A^ e inv_n with
 * A^ the scaled operator from el_warmstart_features' couplings, grad_d = 2 (A^ e) inv_n w;
 * dw, db, workspace as el_nn_head_loss_backward. */
int el_nn_head_energy_loss_backward(int nx, int ny, int nz, const void* d, const float* pred, const float* target,
                                    const void* couplings, const uint8_t* fluid, const float* w, double inv_n,
                                    void* grad_d, double* loss, float* dw, float* db, void* workspace,
                                    size_t workspace_bytes, void* stream);
/* Adam (bias-corrected, step >= 1) on FP32 parameters; zeroes g afterwards. */
int el_nn_adam(int64_t n, float* w, float* g, float* m, float* v, float lr, float beta1, float beta2, float eps,
               int step, void* stream);

/* ---- pressure solve that allocates no device memory ------------------------------------
 * No counterpart in the reference.  Some callers of the pressure solve cannot call cudaMalloc:
 * applications whose device memory is reserved up front by another allocator (a renderer's
 * or framework's memory pool), where a further cudaMalloc fails or is not permitted, and
 * latency-critical loops that cannot afford an allocation, which may synchronise the whole
 * device.  el_solve_pressure_noalloc does what el_solve_pressure does with
 * EL_SOLVER_JACOBI_FP64 (plain FP64 PCG, Jacobi preconditioner), on caller-owned device arrays,
 * and allocates nothing: its scratch (cell flags, the grid-shaped matrix, the PCG vectors,
 * segment lists, reduction partials and scalars) is one fixed array of about 23 MB in the
 * library's device memory, which every GPU that loads the library holds until the process exits.
 *   - at most EL_NOALLOC_MAX_CELLS cells (64^3); larger grids return EL_ERR_TOO_LARGE before any
 *     device work;
 *   - FP32 fields in the layouts of el_upload: phi and the face weights are read, u, v, w are
 *     updated in place (update_velocity_using_pressure), pressure is written (0 outside the
 *     fluid); tol / max_iter as in el_solve_params;
 *   - the work goes on `stream` (a cudaStream_t, NULL = the default stream); the call returns
 *     after the solve, because it reads the convergence scalars back on the host;
 *   - the first call on a device looks up the scratch array's device address, once per device,
 *     with that device current, and keeps it for the life of the process; make that first call
 *     before any stream capture, and do not use this entry point after a cudaDeviceReset of
 *     that device (the reset unloads the library's device memory, so the kept address is stale);
 *   - all calls share the one array, which keeps the last call's contents: calls that overlap
 *     on the GPU (from several threads or streams) race, and the caller must serialise them. */
#define EL_ERR_TOO_LARGE 8
#define EL_NOALLOC_MAX_CELLS 262144
int el_solve_pressure_noalloc(const el_grid* g, const float* phi, float* u, float* v, float* w,
                              const float* weight_u, const float* weight_v, const float* weight_w,
                              float* pressure, double dt, double tol, int max_iter,
                              el_solve_stats* stats, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* EULERIAN_LIQUID_GB300_H */
