// el_capi.cu -- the C ABI (include/eulerian_liquid_gb300.h): contexts, field transfer and the
// entry points that stand in for the reference's Simulator step methods and fluid:: free
// functions.  No exception crosses this boundary; every call returns a status code.
#include <algorithm>
#include <cstring>
#include <mutex>
#include <new>

#include "el_internal.cuh"

namespace el {
// launchers defined in the kernel translation units
int advect_any(int dtype, int ni, int nj, int nk, double dx, int comp, void* out, const void* in, const void* vu,
               const void* vv, const void* vw, const Scalars* dts, double dtv, int trace, int sample,
               cudaStream_t s, int rows = 4);
int advect_phi_tiled(int dtype, int ni, int nj, int nk, double dx, void* out, const void* in, const void* vu,
                     const void* vv, const void* vw, const Scalars* dts, double dtv, int trace, int sample, bool copy,
                     cudaStream_t s);
int advect_velocity_tiled(int dtype, int ni, int nj, int nk, double dx, void* ou, void* ov, void* ow, const void* vu,
                          const void* vv, const void* vw, const Scalars* dts, double dtv, int trace, bool copy,
                          cudaStream_t s);
bool advect_fault_take();
int launch_weights(int dtype, int ni, int nj, int nk, const void* solid, void* wu, void* wv, void* ww,
                   cudaStream_t s);
int launch_cell_solid(el_ctx* ctx);
int launch_flags_build(el_ctx* ctx, bool inner32, bool build = true);
int launch_assign_indices(el_ctx* ctx, int* d_chunks, int* d_total);
int launch_scatter_pressure(el_ctx* ctx);
int launch_update_velocity(el_ctx* ctx, const Scalars* s, double dtv);
int launch_masks(el_ctx* ctx, bool gravity, double g, const Scalars* s, double dtv, bool zero);
int launch_gravity(el_ctx* ctx, double g, const Scalars* s, double dtv);
int launch_zero_invalid(el_ctx* ctx);
int launch_time_step(el_ctx* ctx, double cfl, unsigned long long* scratch_max);
int launch_set_dt(el_ctx* ctx, double dt);
int launch_emit(el_ctx* ctx, int target, int kind, const double* a, int na);
int solve_system(el_ctx* ctx, const el_solve_params& prm, el_solve_stats* st);
int setup_solver_storage(el_ctx* ctx, int solver);
int launch_substep(el_ctx* ctx, double cfl, double dt_frame, const BatchRecord* rec, unsigned long long* scratch_max);
int enqueue_solve_device(el_ctx* ctx, const el_solve_params& prm, int kernels[3]);
int enqueue_step_device(el_ctx* ctx, const el_step_params& p, double cfl, double dt_frame, const BatchRecord* rec,
                        int kernels[3], bool fork);
int prepare_device_step(el_ctx* ctx);
// debug-build check words of the kernel translation units (0 in the product build)
unsigned long long check_take_advect();
unsigned long long check_take_march();
unsigned long long check_take_extrap();
unsigned long long check_take_solve();
unsigned long long check_take_project();

int set_error(el_ctx* ctx, int code, const std::string& msg) {
    if (ctx) ctx->last_error = msg;
    return code;
}

cudaEvent_t prof_event(el_ctx* ctx) {
    if (ctx->ev_used == ctx->ev_pool.size()) {
        if (ctx->ev_pool.size() >= 200000) return nullptr;  // cap the record count
        cudaEvent_t e;
        if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
        ctx->ev_pool.push_back(e);
    }
    return ctx->ev_pool[ctx->ev_used++];
}

int check_launch(el_ctx* ctx, const char* what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return set_error(ctx, EL_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
    return EL_OK;
}

void* ctx_alloc(el_ctx* ctx, size_t bytes) {
    void* p = nullptr;
    if (cudaMalloc(&p, std::max<size_t>(bytes, 16)) != cudaSuccess) return nullptr;
    cudaMemsetAsync(p, 0, std::max<size_t>(bytes, 16), ctx->stream);
    ctx->allocations.push_back(p);
    return p;
}

static size_t field_count(const el_ctx* c, int f) {
    const size_t ni = c->ni, nj = c->nj, nk = c->nk;
    switch (f) {
        case EL_FIELD_U: case EL_FIELD_WEIGHT_U: case EL_FIELD_VALID_U: return (ni + 1) * nj * nk;
        case EL_FIELD_V: case EL_FIELD_WEIGHT_V: case EL_FIELD_VALID_V: return ni * (nj + 1) * nk;
        case EL_FIELD_W: case EL_FIELD_WEIGHT_W: case EL_FIELD_VALID_W: return ni * nj * (nk + 1);
        case EL_FIELD_SOLID_NODAL: return (ni + 1) * (nj + 1) * (nk + 1);
        default: return ni * nj * nk;
    }
}

static size_t field_elem(const el_ctx* c, int f) {
    if (f >= EL_FIELD_VALID_U && f <= EL_FIELD_VALID_PHI) return 1;
    if (f == EL_FIELD_INDICES) return 4;
    return c->esz;
}

int ensure_projection(el_ctx* ctx) {
    if (ctx->flags) return EL_OK;
    const size_t n = (size_t)ctx->ni * ctx->nj * ctx->nk;
    ctx->flags = (uint8_t*)ctx_alloc(ctx, n);
    ctx->built = (uint8_t*)ctx_alloc(ctx, n);  // zero: no row built yet (the outputs start zero)
    ctx->diag64 = (double*)ctx_alloc(ctx, n * 8);
    ctx->rhs64 = (double*)ctx_alloc(ctx, n * 8);
    for (int a = 0; a < 3; ++a) ctx->off[a] = ctx_alloc(ctx, n * ctx->esz);
    if (!ctx->flags || !ctx->built || !ctx->diag64 || !ctx->rhs64 || !ctx->off[0] || !ctx->off[1] || !ctx->off[2])
        return set_error(ctx, EL_ERR_OUT_OF_MEMORY, "projection buffers");
    return EL_OK;
}

int ensure_solver(el_ctx* ctx, int solver) {
    int st = ensure_projection(ctx);
    if (st != EL_OK) return st;
    return setup_solver_storage(ctx, solver);
}

}  // namespace el

using namespace el;

#define EL_API extern "C" __attribute__((visibility("default")))

// At the top of an entry point: the context is valid, and its device is current until the
// entry point returns (the caller's device is restored then).
#define CHECK_CTX(ctx)                                                                   \
    if (!(ctx)) return EL_ERR_INVALID_ARGUMENT;                                          \
    el::DeviceGuard _device_guard((ctx)->device);                                        \
    if (_device_guard.err != cudaSuccess)                                                \
    return set_error(ctx, EL_ERR_CUDA, cudaGetErrorString(_device_guard.err))

EL_API const char* el_status_string(int status) {
    switch (status) {
        case EL_OK: return "ok";
        case EL_ERR_INVALID_ARGUMENT: return "invalid argument";
        case EL_ERR_NO_FLUID: return "No fluid";
        case EL_ERR_NOT_CONVERGED: return "pressure solve did not converge";
        case EL_ERR_NAN: return "non-finite value";
        case EL_ERR_CUDA: return "CUDA error";
        case EL_ERR_OUT_OF_MEMORY: return "out of device memory";
        case EL_ERR_TIMEOUT: return "device wait timed out";
        case EL_ERR_TOO_LARGE: return "grid exceeds the no-allocation scratch limit (EL_NOALLOC_MAX_CELLS)";
        default: return "unknown status";
    }
}

EL_API int el_debug_check_take(uint64_t* word, int* checked) {
    if (!word || !checked) return EL_ERR_INVALID_ARGUMENT;
#ifdef EL_CHECKED
    *checked = 1;
#else
    *checked = 0;
#endif
    const unsigned long long w[5] = {check_take_advect(), check_take_march(), check_take_extrap(), check_take_solve(),
                                     check_take_project()};
    *word = 0;
    for (unsigned long long v : w)
        if (v && !*word) *word = v;
    return EL_OK;
}

EL_API const char* el_ctx_last_error(const el_ctx* ctx) { return ctx ? ctx->last_error.c_str() : "null context"; }

EL_API int el_ctx_create(int ni, int nj, int nk, double dx, int dtype, int device, el_ctx** out) {
    if (!out) return EL_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    if (ni < 1 || nj < 1 || nk < 1 || !(dx > 0) || (dtype != EL_F32 && dtype != EL_F64))
        return EL_ERR_INVALID_ARGUMENT;
    // the reference indexes with int and refuses sizes that overflow it (array.h:322-325)
    const long long biggest = (long long)(ni + 1) * (nj + 1) * (nk + 1);
    if (biggest >= 0x7fffffffLL) return EL_ERR_INVALID_ARGUMENT;
    el::DeviceGuard guard(device);
    if (guard.err != cudaSuccess) return EL_ERR_CUDA;
    el_ctx* ctx = new (std::nothrow) el_ctx();
    if (!ctx) return EL_ERR_OUT_OF_MEMORY;
    ctx->device = device;
    ctx->ni = ni;
    ctx->nj = nj;
    ctx->nk = nk;
    ctx->dx = dx;
    ctx->dtype = dtype;
    ctx->esz = dtype == EL_F64 ? 8 : 4;
    cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device);
    if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete ctx;
        return EL_ERR_CUDA;
    }
    ctx->own_stream = true;
    bool ok = true;
    for (int f = 0; f < EL_FIELD_COUNT; ++f) {
        ctx->field_bytes[f] = field_count(ctx, f) * field_elem(ctx, f);
        ctx->field[f] = ctx_alloc(ctx, ctx->field_bytes[f]);
        ok = ok && ctx->field[f];
    }
    for (int q = 0; q < 4; ++q) {
        ctx->tmp[q] = ctx_alloc(ctx, ctx->field_bytes[EL_FIELD_PHI + q]);
        ok = ok && ctx->tmp[q];
    }
    // extrapolation scratch sizes (allocated on first use): the padded bitmask of the largest
    // face grid, and one index per cell of it
    for (int f = EL_FIELD_U; f <= EL_FIELD_W; ++f) {
        int n0, n1, n2;
        field_dims(ctx, f, n0, n1, n2);
        ctx->ex_bits_bytes = std::max(ctx->ex_bits_bytes, extrapolation_bits_bytes(n0, n1, n2));
        ctx->ex_list_bytes = std::max(ctx->ex_list_bytes, (size_t)n0 * n1 * n2 * sizeof(int));
        ctx->ex_tile_count = std::max(ctx->ex_tile_count, extrapolation_tiles(n0, n1, n2));
    }
    ctx->dscal = (Scalars*)ctx_alloc(ctx, 4 * sizeof(Scalars));
    Geom g = stencil_geom(ni, nj, nk, ctx->num_sms);
    ctx->max_partials = std::max(g.blocks(), ctx->num_sms * 16) * 2 + 64;
    ctx->partials = (double*)ctx_alloc(ctx, ctx->max_partials * sizeof(double));
    ctx->counter = (unsigned*)ctx_alloc(ctx, 64);
    ok = ok && ctx->dscal && ctx->partials && ctx->counter;
    if (ok && cudaMallocHost(&ctx->hscal, 4 * sizeof(Scalars)) != cudaSuccess) ok = false;
    if (ok) {
        // create_grid (simulator.cpp:58-69): valid masks start at 1
        for (int f = EL_FIELD_VALID_U; f <= EL_FIELD_VALID_PHI; ++f)
            cudaMemsetAsync(ctx->field[f], 1, ctx->field_bytes[f], ctx->stream);
        ok = cudaStreamSynchronize(ctx->stream) == cudaSuccess;
    }
    if (!ok) {
        el_ctx_destroy(ctx);
        return EL_ERR_OUT_OF_MEMORY;
    }
    *out = ctx;
    return EL_OK;
}

EL_API int el_ctx_destroy(el_ctx* ctx) {
    if (!ctx) return EL_ERR_INVALID_ARGUMENT;
    el::DeviceGuard guard(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    for (void* p : ctx->allocations) cudaFree(p);
    for (cudaEvent_t e : ctx->ev_pool) cudaEventDestroy(e);
    for (auto& g : ctx->iter_graph)
        if (g) cudaGraphExecDestroy(g);
    for (auto& bs : ctx->body_stream)
        if (bs) cudaStreamDestroy(bs);
    for (auto& ss : ctx->side)
        if (ss) cudaStreamDestroy(ss);
    for (auto& e : ctx->side_join)
        if (e) cudaEventDestroy(e);
    if (ctx->side_fork) cudaEventDestroy(ctx->side_fork);
    if (ctx->hscal) cudaFreeHost(ctx->hscal);
    if (ctx->own_stream && ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return EL_OK;
}

EL_API int el_ctx_set_stream(el_ctx* ctx, void* stream) {
    CHECK_CTX(ctx);
    EL_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    if (ctx->own_stream) cudaStreamDestroy(ctx->stream);
    if (stream) {
        ctx->stream = (cudaStream_t)stream;
        ctx->own_stream = false;
    } else {
        EL_CUDA_TRY(ctx, cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
        ctx->own_stream = true;
    }
    return EL_OK;
}

EL_API void* el_ctx_get_stream(el_ctx* ctx) { return ctx ? (void*)ctx->stream : nullptr; }

EL_API int el_ctx_sync(el_ctx* ctx) {
    CHECK_CTX(ctx);
    EL_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    return EL_OK;
}

EL_API int64_t el_ctx_kernel_launches(const el_ctx* ctx) { return ctx ? ctx->launches : -1; }

EL_API int el_ctx_set_tuning(el_ctx* ctx, const el_tuning* t) {
    CHECK_CTX(ctx);
    if (!t || t->seg_blocks_per_sm < 1 || t->seg_blocks_per_sm > 8 || t->stencil_blocks_per_sm < 1 ||
        t->stencil_blocks_per_sm > 16 || t->extrapolate_blocks_per_sm < 1 || t->extrapolate_blocks_per_sm > 16 ||
        (t->advect_rows != 1 && t->advect_rows != 2 && t->advect_rows != 4 && t->advect_rows != 8) ||
        t->advect_tiled < 0 || t->advect_tiled > 2 || (t->solver_tiles != 0 && t->solver_tiles != 1) ||
        t->coarse_fused < 0 || t->coarse_fused > 2 || (t->dependent_launch != 0 && t->dependent_launch != 1))
        return set_error(ctx, EL_ERR_INVALID_ARGUMENT, "tuning out of range");
    // the reduction partials are sized for 16 stencil blocks per SM (el_ctx_create)
    ctx->seg_per_sm = t->seg_blocks_per_sm;
    ctx->stencil_per_sm = t->stencil_blocks_per_sm;
    ctx->extrap_per_sm = t->extrapolate_blocks_per_sm;
    ctx->advect_rows = t->advect_rows;
    ctx->advect_tiled = t->advect_tiled;
    ctx->solver_tiles = t->solver_tiles;
    ctx->coarse_fused = t->coarse_fused;
    ctx->dependent_launch = t->dependent_launch;
    // cached PCG iteration graphs hold the old launch shapes
    cudaStreamSynchronize(ctx->stream);
    for (auto& g : ctx->iter_graph)
        if (g) {
            cudaGraphExecDestroy(g);
            g = nullptr;
        }
    return EL_OK;
}

EL_API int el_ctx_get_tuning(const el_ctx* ctx, el_tuning* t) {
    if (!ctx || !t) return EL_ERR_INVALID_ARGUMENT;
    t->seg_blocks_per_sm = ctx->seg_per_sm;
    t->stencil_blocks_per_sm = ctx->stencil_per_sm;
    t->extrapolate_blocks_per_sm = ctx->extrap_per_sm;
    t->advect_rows = ctx->advect_rows;
    t->advect_tiled = ctx->advect_tiled;
    t->solver_tiles = ctx->solver_tiles;
    t->coarse_fused = ctx->coarse_fused;
    t->dependent_launch = ctx->dependent_launch;
    return EL_OK;
}

EL_API int el_ctx_solver_tiles_active(el_ctx* ctx, int* on) {
    CHECK_CTX(ctx);
    if (!on) return EL_ERR_INVALID_ARGUMENT;
    *on = 0;
    if (ctx->dtype != EL_F32) return EL_OK;  // the mixed solver's tile kernels are FP32-field only
    const int rc = ensure_solver(ctx, EL_SOLVER_MIXED);
    if (rc != EL_OK) return rc;
    *on = (ctx->march.on && ctx->solver_tiles) ? 1 : 0;
    return EL_OK;
}

EL_API int el_ctx_profile_begin(el_ctx* ctx, uint32_t class_mask) {
    CHECK_CTX(ctx);
    EL_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    ctx->prof.clear();
    ctx->ev_used = 0;
    ctx->prof_mask = class_mask;
    return EL_OK;
}

EL_API int el_ctx_profile_end(el_ctx* ctx, el_profile_entry* out) {
    CHECK_CTX(ctx);
    if (!out) return EL_ERR_INVALID_ARGUMENT;
    ctx->prof_mask = 0;
    EL_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    for (int c = 0; c < EL_KC_COUNT; ++c) out[c] = el_profile_entry{0, 0.0, 0.0};
    for (const auto& r : ctx->prof) {
        float ms = 0.f;
        EL_CUDA_TRY(ctx, cudaEventElapsedTime(&ms, r.a, r.b));
        out[r.cls].launches += 1;
        out[r.cls].ms += ms;
        out[r.cls].bytes += r.bytes;
    }
    ctx->prof.clear();
    ctx->ev_used = 0;
    return EL_OK;
}

EL_API int el_upload(el_ctx* ctx, int field, const void* host, size_t bytes) {
    CHECK_CTX(ctx);
    if (field < 0 || field >= EL_FIELD_COUNT || !host) return set_error(ctx, EL_ERR_INVALID_ARGUMENT, "bad field");
    if (bytes != ctx->field_bytes[field])
        return set_error(ctx, EL_ERR_INVALID_ARGUMENT,
                         "field size mismatch: expected " + std::to_string(ctx->field_bytes[field]) + " bytes");
    EL_CUDA_TRY(ctx, cudaMemcpyAsync(ctx->field[field], host, bytes, cudaMemcpyHostToDevice, ctx->stream));
    EL_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    return EL_OK;
}

EL_API int el_download(el_ctx* ctx, int field, void* host, size_t bytes) {
    CHECK_CTX(ctx);
    if (field < 0 || field >= EL_FIELD_COUNT || !host) return set_error(ctx, EL_ERR_INVALID_ARGUMENT, "bad field");
    if (bytes != ctx->field_bytes[field])
        return set_error(ctx, EL_ERR_INVALID_ARGUMENT,
                         "field size mismatch: expected " + std::to_string(ctx->field_bytes[field]) + " bytes");
    EL_CUDA_TRY(ctx, cudaMemcpyAsync(host, ctx->field[field], bytes, cudaMemcpyDeviceToHost, ctx->stream));
    EL_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    return EL_OK;
}

static int check_transfer(el_ctx* ctx, int field, const void* host, size_t bytes) {
    if (field < 0 || field >= EL_FIELD_COUNT || !host) return set_error(ctx, EL_ERR_INVALID_ARGUMENT, "bad field");
    if (bytes != ctx->field_bytes[field])
        return set_error(ctx, EL_ERR_INVALID_ARGUMENT,
                         "field size mismatch: expected " + std::to_string(ctx->field_bytes[field]) + " bytes");
    return EL_OK;
}

EL_API int el_upload_async(el_ctx* ctx, int field, const void* host, size_t bytes, void* stream) {
    CHECK_CTX(ctx);
    const int rc = check_transfer(ctx, field, host, bytes);
    if (rc != EL_OK) return rc;
    cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : ctx->stream;
    EL_CUDA_TRY(ctx, cudaMemcpyAsync(ctx->field[field], host, bytes, cudaMemcpyHostToDevice, s));
    return EL_OK;
}

EL_API int el_download_async(el_ctx* ctx, int field, void* host, size_t bytes, void* stream) {
    CHECK_CTX(ctx);
    const int rc = check_transfer(ctx, field, host, bytes);
    if (rc != EL_OK) return rc;
    cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : ctx->stream;
    EL_CUDA_TRY(ctx, cudaMemcpyAsync(host, ctx->field[field], bytes, cudaMemcpyDeviceToHost, s));
    return EL_OK;
}

EL_API int el_field_device_ptr(el_ctx* ctx, int field, void** dptr, size_t* bytes) {
    if (!ctx || field < 0 || field >= EL_FIELD_COUNT || !dptr) return EL_ERR_INVALID_ARGUMENT;
    *dptr = ctx->field[field];
    if (bytes) *bytes = ctx->field_bytes[field];
    return EL_OK;
}

static int finish(el_ctx* ctx, int launched, const char* what) {
    ctx->launches += launched;
    return check_launch(ctx, what);
}

// ---- scene set-up -----------------------------------------------------------------------

EL_API int el_emit_clear(el_ctx* ctx, int target) {
    CHECK_CTX(ctx);
    if (target != 0 && target != 1) return EL_ERR_INVALID_ARGUMENT;
    return finish(ctx, launch_emit(ctx, target, 0, nullptr, 0), "emit");
}

EL_API int el_emit_sphere(el_ctx* ctx, int target, double cx, double cy, double cz, double r) {
    CHECK_CTX(ctx);
    if (target != 0 && target != 1) return EL_ERR_INVALID_ARGUMENT;
    const double a[4] = {cx, cy, cz, r};
    return finish(ctx, launch_emit(ctx, target, 1, a, 4), "emit");
}

EL_API int el_emit_pool(el_ctx* ctx, int target, double height) {
    CHECK_CTX(ctx);
    if (target != 0 && target != 1) return EL_ERR_INVALID_ARGUMENT;
    return finish(ctx, launch_emit(ctx, target, 2, &height, 1), "emit");
}

EL_API int el_emit_box(el_ctx* ctx, int target, const double lo[3], const double hi[3]) {
    CHECK_CTX(ctx);
    if ((target != 0 && target != 1) || !lo || !hi) return EL_ERR_INVALID_ARGUMENT;
    const double a[6] = {lo[0], lo[1], lo[2], hi[0], hi[1], hi[2]};
    return finish(ctx, launch_emit(ctx, target, 3, a, 6), "emit");
}

EL_API int el_emit_room(el_ctx* ctx, int target) {
    CHECK_CTX(ctx);
    if (target != 0 && target != 1) return EL_ERR_INVALID_ARGUMENT;
    return finish(ctx, launch_emit(ctx, target, 4, nullptr, 0), "emit");
}

// ---- boundary ----------------------------------------------------------------------------

EL_API int el_compute_weights(el_ctx* ctx) {
    CHECK_CTX(ctx);
    int n = launch_weights(ctx->dtype, ctx->ni, ctx->nj, ctx->nk, ctx->field[EL_FIELD_SOLID_NODAL],
                           ctx->field[EL_FIELD_WEIGHT_U], ctx->field[EL_FIELD_WEIGHT_V], ctx->field[EL_FIELD_WEIGHT_W],
                           ctx->stream);
    return finish(ctx, n, "compute_weights");
}

EL_API int el_calc_cell_centered_solid_phi(el_ctx* ctx) {
    CHECK_CTX(ctx);
    // computes the cell-centred solid phi; the level-set valid mask is refreshed too (it is a
    // pure function of it, simulator.cpp:160-167)
    return finish(ctx, launch_cell_solid(ctx), "cell_centered_solid_phi");
}

EL_API int el_find_valid_level_set(el_ctx* ctx) {
    CHECK_CTX(ctx);
    return finish(ctx, launch_cell_solid(ctx), "find_valid_level_set");
}

// ---- hot path -----------------------------------------------------------------------------

static bool valid_scheme(int trace, int sample) {
    return (trace == EL_TRACE_RK2 || trace == EL_TRACE_RK3) &&
           (sample == EL_SAMPLE_TRILINEAR || sample == EL_SAMPLE_WENO6);
}

// phi <- phi(trace(x, -dt)) through the current velocity (simulator.cpp:84-87)
static double nbytes(el_ctx* ctx, int field) { return (double)ctx->field_bytes[field]; }

static int advect_level_set_impl(el_ctx* ctx, const Scalars* dts, double dt, int trace, int sample) {
    // reads phi, u, v, w; writes phi
    ProfScope prof(ctx, EL_KC_ADVECT_PHI, 2 * nbytes(ctx, EL_FIELD_PHI) + nbytes(ctx, EL_FIELD_U) +
                                              nbytes(ctx, EL_FIELD_V) + nbytes(ctx, EL_FIELD_W));
    // the tiled kernels (trilinear: the velocity staged in shared memory; WENO6: phi and the
    // x-pass smoothness indicators staged), unless launch-shape tuning asked for the
    // per-sample one
    int n = ctx->advect_tiled ? advect_phi_tiled(ctx->dtype, ctx->ni, ctx->nj, ctx->nk, ctx->dx, ctx->tmp[0],
                                                 ctx->field[EL_FIELD_PHI], ctx->field[EL_FIELD_U],
                                                 ctx->field[EL_FIELD_V], ctx->field[EL_FIELD_W], dts, dt, trace,
                                                 sample, ctx->advect_tiled == 1, ctx->stream)
                              : -1;
    if (n < 0)
        n = advect_any(ctx->dtype, ctx->ni, ctx->nj, ctx->nk, ctx->dx, 0, ctx->tmp[0], ctx->field[EL_FIELD_PHI],
                       ctx->field[EL_FIELD_U], ctx->field[EL_FIELD_V], ctx->field[EL_FIELD_W], dts, dt, trace,
                       sample, ctx->stream, ctx->advect_rows);
    std::swap(ctx->tmp[0], ctx->field[EL_FIELD_PHI]);
    return n;
}

// u, v, w <- each component advected through the old velocity (simulator.cpp:79-82)
static int advect_velocity_impl(el_ctx* ctx, const Scalars* dts, double dt, int trace, int sample) {
    int n = 0;
    const double vel_bytes = nbytes(ctx, EL_FIELD_U) + nbytes(ctx, EL_FIELD_V) + nbytes(ctx, EL_FIELD_W);
    if (ctx->advect_tiled && sample == EL_SAMPLE_TRILINEAR) {
        // one launch for the three components: reads u, v, w once; writes the three components
        ProfScope prof(ctx, EL_KC_ADVECT_VEL, 2 * vel_bytes);
        n = advect_velocity_tiled(ctx->dtype, ctx->ni, ctx->nj, ctx->nk, ctx->dx, ctx->tmp[1], ctx->tmp[2],
                                  ctx->tmp[3], ctx->field[EL_FIELD_U], ctx->field[EL_FIELD_V],
                                  ctx->field[EL_FIELD_W], dts, dt, trace, ctx->advect_tiled == 1, ctx->stream);
    }
    if (n <= 0) {  // one launch per component
        n = 0;
        for (int comp = 0; comp < 3; ++comp) {
            // reads u, v, w (the advected component among them); writes the component
            ProfScope prof(ctx, EL_KC_ADVECT_VEL, vel_bytes + nbytes(ctx, EL_FIELD_U + comp));
            n += advect_any(ctx->dtype, ctx->ni, ctx->nj, ctx->nk, ctx->dx, comp + 1, ctx->tmp[1 + comp],
                            ctx->field[EL_FIELD_U + comp], ctx->field[EL_FIELD_U], ctx->field[EL_FIELD_V],
                            ctx->field[EL_FIELD_W], dts, dt, trace, sample, ctx->stream, ctx->advect_rows);
        }
    }
    for (int comp = 0; comp < 3; ++comp) std::swap(ctx->tmp[1 + comp], ctx->field[EL_FIELD_U + comp]);
    return n;
}

EL_API int el_advect_level_set(el_ctx* ctx, double dt, int trace, int sample) {
    CHECK_CTX(ctx);
    if (!valid_scheme(trace, sample)) return set_error(ctx, EL_ERR_INVALID_ARGUMENT, "bad advection scheme");
    return finish(ctx, advect_level_set_impl(ctx, nullptr, dt, trace, sample), "advect_level_set");
}

EL_API int el_advect_velocity(el_ctx* ctx, double dt, int trace, int sample) {
    CHECK_CTX(ctx);
    if (!valid_scheme(trace, sample)) return set_error(ctx, EL_ERR_INVALID_ARGUMENT, "bad advection scheme");
    return finish(ctx, advect_velocity_impl(ctx, nullptr, dt, trace, sample), "advect_velocity");
}

EL_API int el_add_gravity(el_ctx* ctx, double dt, double gravity) {
    CHECK_CTX(ctx);
    return finish(ctx, launch_gravity(ctx, gravity, nullptr, dt), "add_gravity");
}

// the velocity components (write_back: extrapolate) and the level set (extrapolate_const)
static int extrapolate_fields(el_ctx* ctx, bool velocity, bool level_set, int layers) {
    int fields[4];
    uint8_t* valid[4];
    bool wb[4];
    int nf = 0;
    if (velocity)
        for (int c = 0; c < 3; ++c, ++nf) {
            fields[nf] = EL_FIELD_U + c;
            valid[nf] = (uint8_t*)ctx->field[EL_FIELD_VALID_U + c];
            wb[nf] = true;
        }
    if (level_set) {
        fields[nf] = EL_FIELD_PHI;
        valid[nf] = (uint8_t*)ctx->field[EL_FIELD_VALID_PHI];
        wb[nf] = false;
        ++nf;
    }
    // each field's mask and values read once
    double bytes = 0;
    for (int q = 0; q < nf; ++q) bytes += (double)ctx->field_bytes[fields[q]] / ctx->esz * (1 + ctx->esz);
    ProfScope prof(ctx, EL_KC_EXTRAPOLATE, bytes);
    return launch_extrapolate_fields(ctx, nf, fields, valid, wb, layers);
}

EL_API int el_extrapolate_level_set(el_ctx* ctx, int layers) {
    CHECK_CTX(ctx);
    if (layers < 0) return EL_ERR_INVALID_ARGUMENT;
    const int rc = ensure_extrapolation(ctx, 1);
    if (rc != EL_OK) return rc;
    return finish(ctx, extrapolate_fields(ctx, false, true, layers), "extrapolate_level_set");
}

EL_API int el_extrapolate_velocity(el_ctx* ctx, int layers) {
    CHECK_CTX(ctx);
    if (layers < 0) return EL_ERR_INVALID_ARGUMENT;
    const int rc = ensure_extrapolation(ctx, 3);
    if (rc != EL_OK) return rc;
    return finish(ctx, extrapolate_fields(ctx, true, false, layers), "extrapolate_velocity");
}

EL_API int el_find_valid_velocity(el_ctx* ctx) {
    CHECK_CTX(ctx);
    return finish(ctx, launch_masks(ctx, false, 0.0, nullptr, 0.0, false), "find_valid_velocity");
}

EL_API int el_set_invalid_velocity_zero(el_ctx* ctx) {
    CHECK_CTX(ctx);
    return finish(ctx, launch_zero_invalid(ctx), "set_invalid_velocity_zero");
}

static int masks_prof(el_ctx* ctx, bool gravity, double g, const Scalars* s, double dtv, bool zero) {
    // per face: the component read and written, its weight read, its mask written; phi read
    double b = nbytes(ctx, EL_FIELD_PHI);
    for (int c = 0; c < 3; ++c) b += 3 * nbytes(ctx, EL_FIELD_U + c) + nbytes(ctx, EL_FIELD_VALID_U + c);
    ProfScope prof(ctx, EL_KC_MASKS, b);
    return launch_masks(ctx, gravity, g, s, dtv, zero);
}

static int build_prof(el_ctx* ctx, bool inner32) {
    // flags: 3 weights + phi read, flags written; build: 3 velocities + 3 weights + phi + flags
    // read, diag (f64), 3 couplings, rhs (f64) written (+ the FP32 diagonal)
    const double N = (double)ctx->ni * ctx->nj * ctx->nk;
    double faces = 0;
    for (int c = 0; c < 3; ++c) faces += nbytes(ctx, EL_FIELD_U + c);
    double b = faces + nbytes(ctx, EL_FIELD_PHI) + N;
    b += 2 * faces + nbytes(ctx, EL_FIELD_PHI) + N + 16 * N + 3 * N * ctx->esz;
    if (inner32 && ctx->A32) b += 24 * N;  // the mixed solver's float4 and half4 records
    ProfScope prof(ctx, EL_KC_BUILD, b);
    return launch_flags_build(ctx, inner32);
}

static int solve_pressure_impl(el_ctx* ctx, const el_solve_params& prm, el_solve_stats* st) {
    int rc = ensure_solver(ctx, prm.solver);
    if (rc != EL_OK) return rc;
    const bool inner32 = prm.solver == EL_SOLVER_MIXED;
    ctx->launches += build_prof(ctx, inner32);
    rc = check_launch(ctx, "build_matrix");
    if (rc != EL_OK) return rc;
    EL_CUDA_TRY(ctx, cudaMemcpyAsync(ctx->hscal, ctx->dscal, sizeof(Scalars), cudaMemcpyDeviceToHost, ctx->stream));
    EL_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    st->fluid_cells = ctx->hscal->count;
    if (ctx->hscal->count == 0) {
        st->status = EL_ERR_NO_FLUID;
        return set_error(ctx, EL_ERR_NO_FLUID, "No fluid");
    }
    rc = solve_system(ctx, prm, st);
    if (rc != EL_OK) return rc;
    ctx->launches += launch_scatter_pressure(ctx);
    ctx->launches += launch_update_velocity(ctx, ctx->dscal, 0.0);
    return check_launch(ctx, "update_velocity_using_pressure");
}

static bool valid_params(const el_solve_params* p) {
    return p && (p->solver >= EL_SOLVER_JACOBI_FP64 && p->solver <= EL_SOLVER_MIXED) && p->tol > 0 &&
           p->max_iter > 0 && p->check_every > 0;
}

EL_API int el_solve_pressure(el_ctx* ctx, double dt, const el_solve_params* params, el_solve_stats* stats) {
    CHECK_CTX(ctx);
    if (!valid_params(params) || !(dt > 0)) return set_error(ctx, EL_ERR_INVALID_ARGUMENT, "bad solve parameters");
    el_solve_stats local{};
    el_solve_stats* st = stats ? stats : &local;
    *st = el_solve_stats{};
    ctx->launches += launch_set_dt(ctx, dt);
    int rc = solve_pressure_impl(ctx, *params, st);
    if (rc != EL_OK) return rc;
    return st->status == EL_OK ? EL_OK : set_error(ctx, st->status, "pressure solve did not converge");
}

EL_API int el_calc_time_step(el_ctx* ctx, double cfl, double* dt_out) {
    CHECK_CTX(ctx);
    if (!dt_out) return EL_ERR_INVALID_ARGUMENT;
    unsigned long long* scratch = (unsigned long long*)(ctx->dscal + 3);
    ctx->launches += launch_time_step(ctx, cfl, scratch);
    int rc = check_launch(ctx, "calc_time_step");
    if (rc != EL_OK) return rc;
    EL_CUDA_TRY(ctx, cudaMemcpyAsync(ctx->hscal, ctx->dscal, sizeof(Scalars), cudaMemcpyDeviceToHost, ctx->stream));
    EL_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    *dt_out = ctx->hscal->dt;
    return EL_OK;
}

EL_API int el_step(el_ctx* ctx, double dt, const el_step_params* p, el_step_stats* stats) {
    CHECK_CTX(ctx);
    if (!p || !valid_params(&p->solve) || !valid_scheme(p->trace_phi, p->sample_phi) ||
        !valid_scheme(p->trace_vel, p->sample_vel) || p->extrapolation_layers < 0 || !(dt > 0))
        return set_error(ctx, EL_ERR_INVALID_ARGUMENT, "bad step parameters");
    el_step_stats local{};
    el_step_stats* st = stats ? stats : &local;
    *st = el_step_stats{};
    st->dt = dt;
    int rc = ensure_solver(ctx, p->solve.solver);
    if (rc != EL_OK) return rc;
    int n = launch_set_dt(ctx, dt);
    const Scalars* dts = ctx->dscal;
    // update_second_order (apps/eulerian_liquid_3d.cpp:106-120), reinitialize() excluded
    rc = ensure_extrapolation(ctx, 4);
    if (rc != EL_OK) return rc;
    {
        NvtxRange r("el_step extrapolate");
        n += extrapolate_fields(ctx, true, true, p->extrapolation_layers);
    }
    {
        NvtxRange r("el_step advect");
        n += advect_level_set_impl(ctx, dts, dt, p->trace_phi, p->sample_phi);
        n += advect_velocity_impl(ctx, dts, dt, p->trace_vel, p->sample_vel);
    }
    {
        NvtxRange r("el_step gravity and masks");
        n += masks_prof(ctx, true, p->gravity, dts, dt, true);
    }
    ctx->launches += n;
    rc = check_launch(ctx, "step");
    if (rc != EL_OK) return rc;
    {
        NvtxRange r("el_step solve_pressure");
        rc = solve_pressure_impl(ctx, p->solve, &st->solve);
    }
    if (rc != EL_OK) {
        // a tile whose box copies never arrived wrote NaN, which the solve met
        if (rc == EL_ERR_NAN && advect_fault_take())
            return set_error(ctx, EL_ERR_TIMEOUT, "a wait for the advection's box copies gave up");
        return rc;
    }
    return st->solve.status == EL_OK ? EL_OK : set_error(ctx, st->solve.status, "pressure solve did not converge");
}

// One sub-step of a scene with nothing decided on the host, for capture into a batch graph:
// device dt (cut at the frame end), el_step's work, the solve with both loops on the device.
// kernels[0]: kernels outside the solver loops; [1] per refinement sweep; [2] per PCG pass.
// Streams and events of the captured step's side branches, and the extrapolation scratch (outside
// any capture: they allocate).
int el::prepare_device_step(el_ctx* ctx) {
    for (int q = 0; q < 3; ++q) {
        if (!ctx->side[q]) EL_CUDA_TRY(ctx, cudaStreamCreateWithFlags(&ctx->side[q], cudaStreamNonBlocking));
        if (!ctx->side_join[q]) EL_CUDA_TRY(ctx, cudaEventCreateWithFlags(&ctx->side_join[q], cudaEventDisableTiming));
    }
    const int rc = ensure_extrapolation(ctx, 4);
    if (rc != EL_OK) return rc;
    if (!ctx->side_fork) EL_CUDA_TRY(ctx, cudaEventCreateWithFlags(&ctx->side_fork, cudaEventDisableTiming));
    return EL_OK;
}

// Runs f(q) for q = 0..nwork-1 on nbranch streams (1 or nwork): with nbranch = nwork, f(q) runs
// with ctx->stream switched to branch q's stream (q = 0 is the context's own), forked from and
// joined back into the context's stream -- under capture these become parallel branches of the
// graph; with nbranch = 1 all of them run in order on the context's stream.
template <typename F>
static int branches(el_ctx* ctx, int nbranch, int nwork, F&& f) {
    int n = 0;
    if (nbranch <= 1) {
        for (int q = 0; q < nwork; ++q) n += f(q);
        return n;
    }
    cudaStream_t own = ctx->stream;
    EL_CUDA_TRY(ctx, cudaEventRecord(ctx->side_fork, own));
    for (int q = 1; q < nbranch; ++q) EL_CUDA_TRY(ctx, cudaStreamWaitEvent(ctx->side[q - 1], ctx->side_fork, 0));
    for (int q = 0; q < nbranch; ++q) {
        ctx->stream = q == 0 ? own : ctx->side[q - 1];
        n += f(q);
        if (q > 0) EL_CUDA_TRY(ctx, cudaEventRecord(ctx->side_join[q - 1], ctx->stream));
    }
    ctx->stream = own;
    for (int q = 1; q < nbranch; ++q) EL_CUDA_TRY(ctx, cudaStreamWaitEvent(own, ctx->side_join[q - 1], 0));
    return n;
}

int el::enqueue_step_device(el_ctx* ctx, const el_step_params& p, double cfl, double dt_frame,
                            const BatchRecord* rec, int kernels[3], bool fork) {
    int n = launch_substep(ctx, cfl, dt_frame, rec, (unsigned long long*)(ctx->dscal + 3));
    const Scalars* dts = ctx->dscal;
    // the four extrapolations go through each launch together
    n += extrapolate_fields(ctx, true, true, p.extrapolation_layers);
    // the level set and the velocity advect independently (both read the old velocity); the
    // level set is enqueued first because enqueueing the velocity's advection swaps the
    // context's velocity buffers on the host
    n += branches(ctx, fork ? 2 : 1, 2, [&](int q) {
        return q == 0 ? advect_level_set_impl(ctx, dts, 0.0, p.trace_phi, p.sample_phi)
                      : advect_velocity_impl(ctx, dts, 0.0, p.trace_vel, p.sample_vel);
    });
    n += launch_masks(ctx, true, p.gravity, dts, 0.0, true);
    n += launch_flags_build(ctx, true);
    int rc = check_launch(ctx, "captured step");
    if (rc != EL_OK) return rc;
    rc = enqueue_solve_device(ctx, p.solve, kernels);
    if (rc != EL_OK) return rc;
    n += launch_scatter_pressure(ctx);
    n += launch_update_velocity(ctx, ctx->dscal, 0.0);
    kernels[0] += n;
    return check_launch(ctx, "captured step");
}

// ---- projection pieces --------------------------------------------------------------------

EL_API int el_assign_indices(el_ctx* ctx, int* mat_size) {
    CHECK_CTX(ctx);
    int rc = ensure_projection(ctx);
    if (rc != EL_OK) return rc;
    ctx->launches += launch_flags_build(ctx, false, false);
    const long long n = (long long)ctx->ni * ctx->nj * ctx->nk;
    const int nchunks = (int)((n + 2047) / 2048);
    int* scratch = (int*)ctx_alloc(ctx, (size_t)(nchunks + 1) * sizeof(int));
    if (!scratch) return set_error(ctx, EL_ERR_OUT_OF_MEMORY, "assign_indices scratch");
    ctx->launches += launch_assign_indices(ctx, scratch, scratch + nchunks);
    rc = check_launch(ctx, "assign_indices");
    if (rc != EL_OK) return rc;
    int total = 0;
    EL_CUDA_TRY(ctx, cudaMemcpyAsync(&total, scratch + nchunks, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    EL_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    // the scratch is returned at once rather than kept for the context's lifetime
    ctx->allocations.pop_back();
    cudaFree(scratch);
    if (mat_size) *mat_size = total;
    if (total == 0) return set_error(ctx, EL_ERR_NO_FLUID, "No fluid");
    return EL_OK;
}

EL_API int el_build_matrix(el_ctx* ctx, double dt) {
    CHECK_CTX(ctx);
    if (!(dt > 0)) return EL_ERR_INVALID_ARGUMENT;
    int rc = ensure_projection(ctx);
    if (rc != EL_OK) return rc;
    ctx->launches += launch_set_dt(ctx, dt);
    ctx->launches += launch_flags_build(ctx, false);
    return check_launch(ctx, "build_matrix");
}

EL_API int el_download_matrix(el_ctx* ctx, double* diag, double* offx, double* offy, double* offz, double* rhs) {
    CHECK_CTX(ctx);
    if (!ctx->flags) return set_error(ctx, EL_ERR_INVALID_ARGUMENT, "no matrix built yet");
    const size_t n = (size_t)ctx->ni * ctx->nj * ctx->nk;
    if (diag) EL_CUDA_TRY(ctx, cudaMemcpyAsync(diag, ctx->diag64, n * 8, cudaMemcpyDeviceToHost, ctx->stream));
    if (rhs) EL_CUDA_TRY(ctx, cudaMemcpyAsync(rhs, ctx->rhs64, n * 8, cudaMemcpyDeviceToHost, ctx->stream));
    double* outs[3] = {offx, offy, offz};
    std::vector<float> tmp;
    for (int a = 0; a < 3; ++a) {
        if (!outs[a]) continue;
        if (ctx->dtype == EL_F64) {
            EL_CUDA_TRY(ctx, cudaMemcpyAsync(outs[a], ctx->off[a], n * 8, cudaMemcpyDeviceToHost, ctx->stream));
        } else {
            tmp.resize(n);
            EL_CUDA_TRY(ctx, cudaMemcpyAsync(tmp.data(), ctx->off[a], n * 4, cudaMemcpyDeviceToHost, ctx->stream));
            EL_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
            for (size_t q = 0; q < n; ++q) outs[a][q] = tmp[q];
        }
    }
    EL_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    return EL_OK;
}

EL_API int el_update_velocity_using_pressure(el_ctx* ctx, double dt) {
    CHECK_CTX(ctx);
    if (!(dt > 0)) return EL_ERR_INVALID_ARGUMENT;
    return finish(ctx, launch_update_velocity(ctx, nullptr, dt), "update_velocity_using_pressure");
}

// ---- stateless operators ----------------------------------------------------------------------

static bool valid_grid(const el_grid* g, int dtype) {
    return g && g->ni > 0 && g->nj > 0 && g->nk > 0 && g->dx > 0 && (dtype == EL_F32 || dtype == EL_F64) &&
           (long long)(g->ni + 1) * (g->nj + 1) * (g->nk + 1) < 0x7fffffffLL;
}

EL_API int el_advect_collocated_grid(const el_grid* g, int dtype, void* out, const void* in, const void* vu,
                                     const void* vv, const void* vw, double dt, int trace, int sample,
                                     void* stream) {
    if (!valid_grid(g, dtype) || !out || !in || !vu || !vv || !vw || out == in || !valid_scheme(trace, sample))
        return EL_ERR_INVALID_ARGUMENT;
    advect_any(dtype, g->ni, g->nj, g->nk, g->dx, 0, out, in, vu, vv, vw, nullptr, dt, trace, sample,
               (cudaStream_t)stream);
    return cudaGetLastError() == cudaSuccess ? EL_OK : EL_ERR_CUDA;
}

EL_API int el_advect_staggered_grid(const el_grid* g, int dtype, void* ou, void* ov, void* ow, const void* iu,
                                    const void* iv, const void* iw, const void* vu, const void* vv, const void* vw,
                                    double dt, int trace, int sample, void* stream) {
    if (!valid_grid(g, dtype) || !ou || !ov || !ow || !iu || !iv || !iw || !vu || !vv || !vw ||
        !valid_scheme(trace, sample))
        return EL_ERR_INVALID_ARGUMENT;
    const void* outs[3] = {ou, ov, ow};
    const void* ins[3] = {vu, vv, vw};
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b)
            if (outs[a] == ins[b] || outs[a] == (a == 0 ? iu : a == 1 ? iv : iw)) return EL_ERR_INVALID_ARGUMENT;
    const void* src[3] = {iu, iv, iw};
    void* dst[3] = {ou, ov, ow};
    for (int c = 0; c < 3; ++c)
        advect_any(dtype, g->ni, g->nj, g->nk, g->dx, c + 1, dst[c], src[c], vu, vv, vw, nullptr, dt, trace, sample,
                   (cudaStream_t)stream);
    return cudaGetLastError() == cudaSuccess ? EL_OK : EL_ERR_CUDA;
}

EL_API int el_compute_staggered_grid_weight(const el_grid* g, int dtype, void* wu, void* wv, void* ww,
                                            const void* solid, void* stream) {
    if (!valid_grid(g, dtype) || !wu || !wv || !ww || !solid) return EL_ERR_INVALID_ARGUMENT;
    launch_weights(dtype, g->ni, g->nj, g->nk, solid, wu, wv, ww, (cudaStream_t)stream);
    return cudaGetLastError() == cudaSuccess ? EL_OK : EL_ERR_CUDA;
}

// ---- pressure solve that allocates no device memory ----------------------------------------
//
// For callers that cannot call cudaMalloc (device memory reserved by another allocator, or
// loops that cannot afford an allocation's device synchronisation).  Everything the plain FP64
// Jacobi solve needs beyond the caller's fields is carved out of one file-scope device array
// sized for EL_NOALLOC_MAX_CELLS cells; a context that owns nothing points the existing kernels
// at the caller's arrays and at that scratch.

namespace {

constexpr long long kNoAllocCells = EL_NOALLOC_MAX_CELLS;
constexpr size_t round256(size_t b) { return (b + 255) & ~(size_t)255; }
constexpr long long kNoAllocPartials = 8192;  // doubles
constexpr size_t kNoAllocBytes =
    round256(kNoAllocCells)                                 // cell flags
    + round256(8 * kNoAllocCells)                           // diagonal (f64)
    + 3 * round256(4 * kNoAllocCells)                       // couplings (f32)
    + round256(8 * kNoAllocCells)                           // right-hand side (f64)
    + 5 * round256(8 * kNoAllocCells)                       // x, r, p, p', Ap (f64)
    + round256(16 * kNoAllocCells)                          // segment descriptors (<= one per cell)
    + round256(kNoAllocCells)                               // segment flags
    + round256(4 * (kNoAllocCells / 1024 + 2))              // scan chunks and the segment count
    + round256(8 * kNoAllocPartials)                        // reduction partials
    + round256(64)                                          // reduction ticket
    + round256(4 * sizeof(el::Scalars));                    // device scalars
constexpr int kNoAllocMaxDevices = 64;

std::mutex g_noalloc_mutex;
void* g_noalloc_address[kNoAllocMaxDevices] = {};

}  // namespace

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

EL_API int el_solve_pressure_noalloc(const el_grid* g, const float* phi, float* u, float* v, float* w,
                                     const float* weight_u, const float* weight_v, const float* weight_w,
                                     float* pressure, double dt, double tol, int max_iter, el_solve_stats* stats,
                                     void* stream) {
    if (!g || !phi || !u || !v || !w || !weight_u || !weight_v || !weight_w || !pressure || !(dt > 0) ||
        !(tol > 0) || max_iter < 1 || g->ni < 1 || g->nj < 1 || g->nk < 1 || !(g->dx > 0))
        return EL_ERR_INVALID_ARGUMENT;
    const long long n = (long long)g->ni * g->nj * g->nk;
    if (n > kNoAllocCells) return EL_ERR_TOO_LARGE;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kNoAllocMaxDevices) return EL_ERR_CUDA;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return EL_ERR_CUDA;
    const Geom geom = stencil_geom(g->ni, g->nj, g->nk, sms);
    const long long partials_needed = (long long)std::max(geom.blocks(), sms * 16) * 2 + 64;
    if (partials_needed > kNoAllocPartials) return EL_ERR_TOO_LARGE;

    // once per device, with that device current: the scratch array's device address
    unsigned char* base = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_noalloc_mutex);
        if (!g_noalloc_address[dev]) {
            void* addr = nullptr;
            if (cudaGetSymbolAddress(&addr, g_noalloc_scratch) != cudaSuccess || !addr) return EL_ERR_CUDA;
            g_noalloc_address[dev] = addr;
        }
        base = static_cast<unsigned char*>(g_noalloc_address[dev]);
    }

    el_ctx ctx;  // a view: the caller's fields and the scratch, nothing owned
    ctx.device = dev;
    ctx.ni = g->ni;
    ctx.nj = g->nj;
    ctx.nk = g->nk;
    ctx.dx = g->dx;
    ctx.dtype = EL_F32;
    ctx.esz = 4;
    ctx.num_sms = sms;
    ctx.stream = static_cast<cudaStream_t>(stream);
    ctx.own_stream = false;
    ctx.use_graphs = false;  // instantiating a graph would allocate
    ctx.build_skip_zero = false;  // the scratch keeps an earlier call's matrix: every row is written
    ctx.field[EL_FIELD_PHI] = const_cast<float*>(phi);
    ctx.field[EL_FIELD_U] = u;
    ctx.field[EL_FIELD_V] = v;
    ctx.field[EL_FIELD_W] = w;
    ctx.field[EL_FIELD_WEIGHT_U] = const_cast<float*>(weight_u);
    ctx.field[EL_FIELD_WEIGHT_V] = const_cast<float*>(weight_v);
    ctx.field[EL_FIELD_WEIGHT_W] = const_cast<float*>(weight_w);
    ctx.field[EL_FIELD_PRESSURE] = pressure;
    size_t off = 0;
    auto carve = [&](size_t bytes) {
        unsigned char* p = base + off;
        off += round256(bytes);
        return p;
    };
    ctx.flags = carve(kNoAllocCells);
    ctx.diag64 = (double*)carve(8 * kNoAllocCells);
    for (int a = 0; a < 3; ++a) ctx.off[a] = carve(4 * kNoAllocCells);
    ctx.rhs64 = (double*)carve(8 * kNoAllocCells);
    ctx.x64 = (double*)carve(8 * kNoAllocCells);
    ctx.r64 = (double*)carve(8 * kNoAllocCells);
    ctx.p64 = (double*)carve(8 * kNoAllocCells);
    ctx.p64b = (double*)carve(8 * kNoAllocCells);
    ctx.ap64 = (double*)carve(8 * kNoAllocCells);
    ctx.z64 = ctx.p64b;  // not read by the Jacobi solve
    SegList& seg = ctx.seg0;
    seg.nsr = (g->ni + 31) / 32;
    seg.total = (long long)seg.nsr * g->nj * g->nk;  // <= n
    seg.desc = (int4*)carve(16 * kNoAllocCells);
    seg.flags = (uint8_t*)carve(kNoAllocCells);
    seg.chunk = (int*)carve(4 * (kNoAllocCells / 1024 + 2));
    seg.count = seg.chunk + (seg.total + 1023) / 1024;
    ctx.partials = (double*)carve(8 * kNoAllocPartials);
    ctx.max_partials = (int)kNoAllocPartials;
    ctx.counter = (unsigned*)carve(64);
    ctx.dscal = (Scalars*)carve(4 * sizeof(Scalars));
    Scalars host_scalars[4] = {};
    ctx.hscal = host_scalars;  // pageable host copy of the device scalars

    // the array keeps the previous call's contents: the reduction ticket and the scalars start
    // at zero; everything else is written before it is read
    EL_CUDA_TRY(&ctx, cudaMemsetAsync(ctx.counter, 0, 64, ctx.stream));
    EL_CUDA_TRY(&ctx, cudaMemsetAsync(ctx.dscal, 0, 4 * sizeof(Scalars), ctx.stream));
    el_solve_stats local{};
    el_solve_stats* st = stats ? stats : &local;
    *st = el_solve_stats{};
    const el_solve_params prm{EL_SOLVER_JACOBI_FP64, tol, max_iter, 8, 1, 1e-4};
    ctx.launches += launch_set_dt(&ctx, dt);
    const int rc = solve_pressure_impl(&ctx, prm, st);
    if (rc != EL_OK) return rc;
    return st->status;
}
