// el_internal.cuh -- shared device helpers and the context layout of the GB300 hot path.
//
// Data layout in HBM: every field is a dense i-fastest array with the reference's index
// i + n0*(j + n1*k) (include/nama/common/array.h:281-286), so host grids move with one copy.
// The pressure system is grid-shaped: the solver's vectors have one entry per cell, the
// entries of non-fluid cells are zero and their matrix rows are empty (diag = 0).
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <cstdint>
#include <cstdio>
#include <string>
#include <unordered_map>
#include <utility>
#include <vector>

#include "../../include/eulerian_liquid_gb300.h"
#include "el_f2d.cuh"

namespace el {

constexpr int kMaxFields = EL_FIELD_COUNT;
constexpr int kIndexUnknown = 0x7fffffff;  // projection.cpp:6 UNKNOWN_INDEX = INT_MAX

// Cell flags written by the projection set-up kernel.
constexpr uint8_t kFlagPressureValid = 1;  // is_pressure_valid (projection.cpp:8-12)
constexpr uint8_t kFlagFluid = 2;          // pressure-valid and phi < 0

struct Status {
    int code = EL_OK;
    std::string msg;
};

// Device-resident scalars of one solve; kernels read and write them so that no host round
// trip is needed between iterations.
struct Scalars {
    double dt;       // step size the step kernels read
    double bb;       // |b|^2 of the current system
    double rz;       // r . z
    double alpha, beta;
    double rr;       // |r|^2 (recursively updated residual)
    double thresh;   // stop when rr < thresh (= tol^2 * bb)
    double norm;     // mixed solver: |r_outer| used to scale the inner system
    double maxabs;   // max |u| over the MAC grid (time step)
    double aux;
    int iter;        // iterations done
    int done;        // 1 once converged (later iteration kernels return at once)
    int bad;         // non-finite value met
    int count;       // fluid cells / changed cells, depending on the kernel
    int outer;       // mixed solver: refinement sweeps done
    int inner_total; // mixed solver: inner iterations summed over the sweeps
    int inner_passes;// device-driven mixed solver: passes of its PCG loop
    int fault;       // a bounded device wait gave up (the solve reports EL_ERR_TIMEOUT)
    int df_shift;    // mixed solver: the power of two 2^df_shift that brings |b| near 1 in the
                     // double-float residual (scale invariance for its float pairs)
};

// Per-scene running totals of a batch (el_batch_stats on the device).
struct BatchRecord {
    long long steps, frames, iterations, outer, passes, unconverged, no_fluid, bad;
    double time, last_dt, max_relres, frame_t;
};

// Active row segments of one grid level: a segment is 32 consecutive cells of one (j, k) row;
// `desc` lists, in increasing order, the segments that hold at least one active cell
// (diagonal > 0).  Solver kernels run one warp per listed segment.
struct SegList {
    int nsr = 0;            // segments per row = ceil(n0 / 32)
    long long total = 0;    // nsr * n1 * n2
    int4* desc = nullptr;   // active segments, ordered: {first cell index, i0, j, k}
    int* count = nullptr;   // number of active segments (device)
    uint8_t* flags = nullptr;
    int* chunk = nullptr;   // scan scratch
};

// Coefficient record of one cell: diagonal and the couplings with the +x, +y, +z neighbours.
struct Rec64 {
    double d, x, y, z;
};

// One level of the multigrid hierarchy.  `rec` points at records of the level's type: level 0
// half4 (mixed) or Rec64 (FP64 multigrid); coarse levels float4 or Rec64.
template <typename V>
struct MGLevel {
    int n0 = 0, n1 = 0, n2 = 0;
    void* rec = nullptr;
    V* b = nullptr;
    V* x = nullptr;
    V* t = nullptr;
    SegList seg;
};

// The smoother: two Jacobi sweeps with weights 1/t1 and 1/t2, t1,2 the roots of the degree-2
// Chebyshev polynomial on [1/3, 2] -- the high-frequency part of the spectrum of D^-1 A (a
// 7-point operator with D >= the sum of its couplings' magnitudes has its spectrum in [0, 2];
// modes with a wave number past pi/2 on any axis have lambda >= 1/3).  Two sweeps apply
// (1 - w1 D^-1 A)(1 - w2 D^-1 A), which reduces that band by at most 1/T2(7/5) = 0.34, against
// 0.51 for two sweeps at 6/7, for the same work; and, a polynomial in D^-1 A, the smoother is
// self-adjoint in the A inner product and contracts on (0, 2], so the V-cycle stays a
// symmetric positive definite preconditioner.  The first sweep of a pair takes w1, the second
// w2 (before and after the coarse correction alike).
constexpr double kChebMid = 7.0 / 6.0, kChebHalf = 5.0 / 6.0;
constexpr double kSweep1 = 1.0 / (kChebMid + kChebHalf * 0.70710678118654752);  // 0.5695
constexpr double kSweep2 = 1.0 / (kChebMid - kChebHalf * 0.70710678118654752);  // 1.7319

// The finest level of the FP32 multigrid as z-marching tile kernels (el_march.cu): work items
// of 32 x 16 cells x up to kMarchPlanes planes holding an active cell, and the TMA tensor maps
// of the arrays those kernels stage.  `on` when the grid meets the kernels' conditions (row
// pitch a multiple of 16 bytes on the finest and the next level, at least three levels).
constexpr int kMarchPlanes = 16;  // planes per work item (tiles are 32 x 16 cells)
struct MarchPlan {
    bool on = false;
    int nib = 0, njb = 0, nkc = 0;  // tiles along i, j and plane chunks along k
    int4* items = nullptr;          // {i0, j0, k0, k1}, ordered i-tile fastest, then j, then k
    int* count = nullptr;           // number of items (device)
    uint8_t* flags = nullptr;
    // tensor maps: 40 x 18 halo boxes of the vectors, 32 x 16 centre boxes, the records' halo
    // boxes and the coarse level's 24 x 10 box
    enum { Z, P, PB, AP, R, RB, T, NHALO };
    enum { CX, CP, CPB, CR, CRB, NCENTRE };
    CUtensorMap halo[NHALO];
    CUtensorMap centre[NCENTRE];
    CUtensorMap rec32, rec16, coarse_x;
    int per_sm[6] = {};  // resident CTAs per SM of each tile kernel
    int planes = kMarchPlanes;  // planes per work item
};

// Makes `device` current for the length of one entry point and gives the caller's current
// device back on return, so that no call leaves a caller that works on another GPU switched.
struct DeviceGuard {
    int prev = -1;
    cudaError_t err = cudaSuccess;
    explicit DeviceGuard(int device) {
        if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
        if (prev != device) err = cudaSetDevice(device);
    }
    ~DeviceGuard() {
        int now = -1;
        if (prev >= 0 && cudaGetDevice(&now) == cudaSuccess && now != prev) cudaSetDevice(prev);
    }
    DeviceGuard(const DeviceGuard&) = delete;
    DeviceGuard& operator=(const DeviceGuard&) = delete;
};

// Debug build (compiled with -DEL_CHECKED, the library libeulerian_liquid_gb300_checked.so):
// the main kernels check the index of each global store (and of the indirect loads) against
// its array before the access.  A failed check skips the access and records the first failure
// -- a site number and the index -- in its translation unit's check word; it never traps.
// el_checked_take() reads and clears every unit's word.  In the product build the checks are
// `true` and cost nothing.
#ifdef EL_CHECKED
static __device__ unsigned long long el_check_word;  // one per translation unit
__device__ __forceinline__ bool el_in_bounds(long long idx, long long n, unsigned site) {
    if (idx >= 0 && idx < n) return true;
    atomicCAS(&el_check_word, 0ull, ((unsigned long long)site << 40) | ((unsigned long long)idx & 0xffffffffffull));
    return false;
}
#define EL_IN(idx, n, site) el::el_in_bounds((long long)(idx), (long long)(n), (site))
#define EL_CHECK_EXPORT(unit)                                                  \
    unsigned long long check_take_##unit() {                                   \
        unsigned long long v = 0, z = 0;                                       \
        cudaMemcpyFromSymbol(&v, el_check_word, sizeof(v));                    \
        cudaMemcpyToSymbol(el_check_word, &z, sizeof(z));                      \
        return v;                                                              \
    }
#else
#define EL_IN(idx, n, site) true
#define EL_CHECK_EXPORT(unit) \
    unsigned long long check_take_##unit() { return 0ull; }
#endif

// Programmatic dependent launch: a kernel launched with launch_dependent() may be scheduled
// while the kernel before it on the stream is still running; its first act is pdl_wait(), which
// returns once that kernel has completed and its memory operations are visible (at once for a
// kernel launched the ordinary way).  pdl_trigger() lets the next such kernel be scheduled.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

// An NVTX range around one phase of a step on the host timeline (no cost unless a profiler
// that collects NVTX is attached).
struct NvtxRange {
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange&) = delete;
    NvtxRange& operator=(const NvtxRange&) = delete;
};

struct DeviceBuffer {
    void* ptr = nullptr;
    size_t bytes = 0;
};

}  // namespace el

struct el_ctx {
    int device = 0;
    int ni = 0, nj = 0, nk = 0;
    double dx = 0;
    int dtype = EL_F32;
    size_t esz = 4;
    int num_sms = 152;
    // launch-shape tuning (el_ctx_set_tuning): resident blocks per SM of the segment kernels,
    // of the grid-wide stencil / element-wise kernels and of the extrapolation, and the rows of
    // the advection tile (32 x rows cells per block)
    int seg_per_sm = 8, stencil_per_sm = 16, extrap_per_sm = 12, advect_rows = 4;
    int advect_tiled = 1;  // advection through the staged-tile kernels (2: boxes by plain loads only)
    int solver_tiles = 1;  // the mixed solver's finest level on the tile kernels (where supported)
    int coarse_fused = 0;  // the FP32 V-cycle's coarse levels in one cooperative launch (where supported)
    int dependent_launch = 1;  // the solver's chained kernels as programmatic dependent launches
    unsigned* coarse_bar = nullptr;  // its grid barrier words
    int coarse_per_sm = 0;           // its resident CTAs per SM (0: cannot run, per-level launches)
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    int64_t launches = 0;

    void* field[el::kMaxFields] = {};
    size_t field_bytes[el::kMaxFields] = {};

    // advection / extrapolation ping-pong buffers (same shapes as phi, u, v, w)
    void* tmp[4] = {};
    // extrapolation scratch per field slot (el_extrap.cu): two padded bitmasks of the valid
    // cells and the list of a layer's cells; cells per slot of the current and the next layer
    unsigned* ex_bits[4][2] = {};
    int* ex_list[4] = {};
    uint8_t* ex_tiles[4] = {};  // the dilation's tile states
    int* ex_counts = nullptr;
    size_t ex_bits_bytes = 0, ex_list_bytes = 0, ex_tile_count = 0;

    // projection
    uint8_t* flags = nullptr;
    double* diag64 = nullptr;  // A_ii (double, projection.cpp:80-107)
    void* off[3] = {};         // A(c, c+x/y/z) in the field type (exactly -weight)
    double* rhs64 = nullptr;
    // FP64 Krylov vectors
    double *x64 = nullptr, *r64 = nullptr, *z64 = nullptr, *p64 = nullptr, *ap64 = nullptr;
    double* p64b = nullptr;  // second direction buffer (the fused K1 writes p out of place)
    // FP32 inner system (mixed solver): the PCG operator as float4 records and the level-0
    // multigrid operator as half4 records
    float4* A32 = nullptr;
    ushort4* A16 = nullptr;
    bool records_fresh = false;  // the last matrix build also wrote A32 / A16 (no packing pass needed)
    // the build leaves the zero rows of cells that were not fluid in the previous build either
    // alone (`built`: 1 where the build's outputs at the cell may be nonzero); off where the
    // outputs' contents are not known (scratch reused)
    bool build_skip_zero = true;
    uint8_t* built = nullptr;
    float *x32 = nullptr, *r32 = nullptr, *z32 = nullptr, *p32 = nullptr, *ap32 = nullptr;
    float* p32b = nullptr;
    float* r32b = nullptr;  // second residual buffer (the fused update writes r out of place)
    float2* xs = nullptr;   // the mixed solver's FP64 iterate as float pairs (the double-float residual)
    el::MarchPlan march;    // finest-level tile kernels of the mixed solver
    el::Rec64* A64rec = nullptr;  // level-0 records of the FP64 multigrid
    el::SegList seg0;             // active segments of the finest level
    std::vector<el::MGLevel<float>> mg32;
    std::vector<el::MGLevel<double>> mg64;

    el::Scalars* dscal = nullptr;  // [0] outer / plain, [1] inner
    el::Scalars* hscal = nullptr;  // pinned mirror
    double* partials = nullptr;
    unsigned* counter = nullptr;
    int max_partials = 0;

    std::vector<void*> allocations;
    std::string last_error;

    // captured CUDA graphs of PCG iteration batches, one per solver (index EL_SOLVER_*)
    cudaGraphExec_t iter_graph[3] = {nullptr, nullptr, nullptr};
    cudaStream_t body_stream[2] = {nullptr, nullptr};  // capture of conditional-node bodies
    // branches of a captured step (the independent advections run side by side)
    cudaStream_t side[3] = {nullptr, nullptr, nullptr};
    cudaEvent_t side_fork = nullptr, side_join[3] = {nullptr, nullptr, nullptr};
    int iter_graph_len[3] = {0, 0, 0};
    int iter_graph_kernels[3] = {0, 0, 0};
    bool use_graphs = true;

    // per-kernel-class timing (el_ctx_profile_begin / _end)
    uint32_t prof_mask = 0;
    struct ProfRec {
        int cls;
        cudaEvent_t a, b;
        double bytes;
    };
    std::vector<cudaEvent_t> ev_pool;
    size_t ev_used = 0;
    std::vector<ProfRec> prof;
    // while profiling: cells covered by the active segments of each multigrid level of the
    // current solve (read back once per solve), for the byte counts of the segment kernels
    std::vector<double> prof_active;
    // resident CTAs per SM of the kernels launched through one_wave(), by kernel
    std::unordered_map<const void*, int> resident;
};

namespace el {
// launch `kernel` on the context's stream; with the context's `dependent_launch` set, as a
// programmatic dependent launch (the kernel must begin with pdl_wait())
template <typename... KArgs, typename... Args>
cudaError_t launch_dependent(const el_ctx* ctx, void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem,
                             Args&&... args) {
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = ctx->stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = ctx->dependent_launch ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

// A grid of `want` blocks of `threads` (no dynamic shared memory) capped at one wave of the
// kernel's resident CTAs, for grid-stride kernels whose work per warp does not depend on the
// grid: a second, partial wave only lengthens the tail.
template <typename... KArgs>
int one_wave(el_ctx* ctx, void (*kernel)(KArgs...), int threads, int want) {
    const void* key = reinterpret_cast<const void*>(kernel);
    auto it = ctx->resident.find(key);
    int per_sm = 0;
    if (it == ctx->resident.end()) {
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, 0) != cudaSuccess || per_sm < 1)
            per_sm = 1;
        ctx->resident.emplace(key, per_sm);
    } else {
        per_sm = it->second;
    }
    return std::max(1, std::min(want, ctx->num_sms * per_sm));
}
}  // namespace el

namespace el {

// ---------------------------------------------------------------------------------------
// error plumbing

#define EL_CUDA_TRY(ctx, expr)                                                                  \
    do {                                                                                        \
        cudaError_t _e = (expr);                                                                \
        if (_e != cudaSuccess) {                                                                \
            return ::el::set_error((ctx), _e == cudaErrorMemoryAllocation ? EL_ERR_OUT_OF_MEMORY \
                                                                          : EL_ERR_CUDA,        \
                                   std::string(#expr) + ": " + cudaGetErrorString(_e));         \
        }                                                                                       \
    } while (0)

int set_error(el_ctx* ctx, int code, const std::string& msg);
cudaEvent_t prof_event(el_ctx* ctx);

// Brackets the launches made during its lifetime with events when `cls` is being profiled.
struct ProfScope {
    el_ctx* ctx;
    int cls;
    double bytes;
    cudaEvent_t a = nullptr;
    ProfScope(el_ctx* c, int k, double b) : ctx(c), cls(k), bytes(b) {
        if (ctx && (ctx->prof_mask >> cls) & 1u) {
            a = prof_event(ctx);
            if (a) cudaEventRecord(a, ctx->stream);
        }
    }
    ~ProfScope() {
        if (!a) return;
        cudaEvent_t b = prof_event(ctx);
        if (!b) return;
        cudaEventRecord(b, ctx->stream);
        ctx->prof.push_back({cls, a, b, bytes});
    }
};
int check_launch(el_ctx* ctx, const char* what);
void* ctx_alloc(el_ctx* ctx, size_t bytes);  // zero-filled, owned by the context
int ensure_projection(el_ctx* ctx);
int ensure_solver(el_ctx* ctx, int solver);
void field_dims(const el_ctx* ctx, int field, int& n0, int& n1, int& n2);
size_t extrapolation_bits_bytes(int n0, int n1, int n2);
size_t extrapolation_tiles(int n0, int n1, int n2);
// extrapolation (el_extrap.cu): scratch for `nfields` slots (outside capture), and up to four
// fields extrapolated together; returns the kernels launched
int ensure_extrapolation(el_ctx* ctx, int nfields);
int launch_extrapolate_fields(el_ctx* ctx, int nf, const int* fields, uint8_t* const* valid, const bool* write_back,
                              int layers);

// finest-level tile kernels of the FP32 multigrid (el_march.cu); each returns its launches
bool march_supported(const el_ctx* ctx);
int march_setup(el_ctx* ctx);
int march_enqueue_items(el_ctx* ctx);
int march_dir_spmv(el_ctx* ctx, const float* z, const float* p_in, float* p_out, float* ap, Scalars* s, int first);
int march_update_smooth(el_ctx* ctx, float* x, const float* p, const float* r_in, float* r_out, const float* ap,
                        float* z, Scalars* s);
int march_zero2(el_ctx* ctx, const float* b, float* z, Scalars* s);
int march_restrict(el_ctx* ctx, const float* x, const float* b, float* coarse_b, Scalars* s);
int march_prolong(el_ctx* ctx, const float* x, const float* b, float* t, Scalars* s);
int march_last(el_ctx* ctx, const float* t, const float* b, float* x, Scalars* s, int dot);

// ---------------------------------------------------------------------------------------
// launch geometry: stencil kernels use blocks of 32 x 8 threads over (i, j) marching a chunk
// of planes along k, so the grid is (n0/32) x (n1/8) x (n2/kz) with no index division.

constexpr int kBX = 32, kBY = 8;

struct Geom {
    dim3 grid, block;
    int kz;  // planes per block
    int blocks() const { return grid.x * grid.y * grid.z; }
};

inline Geom stencil_geom(int n0, int n1, int n2, int num_sms, int per_sm = 8) {
    Geom g;
    g.block = dim3(kBX, kBY, 1);
    const int gx = (n0 + kBX - 1) / kBX, gy = (n1 + kBY - 1) / kBY;
    // aim for `per_sm` resident blocks of 256 threads per SM, at least one plane per block
    const long long want = (long long)num_sms * per_sm;
    int kz = (int)std::max<long long>(1, ((long long)gx * gy * n2 + want - 1) / want);
    kz = std::min(kz, n2);
    const int gz = (n2 + kz - 1) / kz;
    g.grid = dim3(gx, gy, gz);
    g.kz = kz;
    return g;
}

__host__ __device__ inline long long lin3(int i, int j, int k, int n0, int n1) {
    return i + (long long)n0 * (j + (long long)n1 * k);
}


// Round-to-nearest operations the compiler does not contract: an expression written with them
// has one evaluation in every kernel.  (a * b + c * d may be contracted to fma(a, b, c * d) or
// to fma(c, d, a * b), and different kernels may choose differently.)
__device__ __forceinline__ float rn_mul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double rn_mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float rn_fma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double rn_fma(double a, double b, double c) { return __fma_rn(a, b, c); }
__device__ __forceinline__ float rn_add(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double rn_add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float rn_sub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ double rn_sub(double a, double b) { return __dsub_rn(a, b); }

// The 7-point product d v0 + cxm vxm + cxp vxp + cym vym + cyp vyp + czm vzm + czp vzp in that
// order, one rounding per multiply-add: the solver's kernels (segment, tile and bottom) share it
template <typename V>
__device__ __forceinline__ V stencil7(V d, V v0, V cxm, V vxm, V cxp, V vxp, V cym, V vym, V cyp, V vyp, V czm,
                                      V vzm, V czp, V vzp) {
    V t = rn_mul(d, v0);
    t = rn_fma(cxm, vxm, t);
    t = rn_fma(cxp, vxp, t);
    t = rn_fma(cym, vym, t);
    t = rn_fma(cyp, vyp, t);
    t = rn_fma(czm, vzm, t);
    return rn_fma(czp, vzp, t);
}

template <typename T>
__device__ __forceinline__ T clampi(T v, T lo, T hi) {
    return v < lo ? lo : (v > hi ? hi : v);
}

// ---------------------------------------------------------------------------------------
// deterministic grid-wide reduction: warp shuffles, one partial per block, and the last
// block to finish (an atomic ticket, no waiting) sums the partials in block order.

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

template <int NV>
__device__ __forceinline__ void block_sum(double (&v)[NV], double (*sh)[32]) {
    const int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
    const int nthreads = blockDim.x * blockDim.y * blockDim.z;
    const int lane = tid & 31, warp = tid >> 5, nwarps = (nthreads + 31) >> 5;
#pragma unroll
    for (int q = 0; q < NV; ++q) {
        double s = warp_sum(v[q]);
        if (lane == 0) sh[q][warp] = s;
    }
    __syncthreads();
    if (warp == 0) {
#pragma unroll
        for (int q = 0; q < NV; ++q) {
            double s = lane < nwarps ? sh[q][lane] : 0.0;
            v[q] = warp_sum(s);
        }
    }
    __syncthreads();
}

// Returns true in thread 0 of the last block, with out[] holding the grid totals.
// `partials` must hold (number of blocks) * NV doubles.
template <int NV>
__device__ bool grid_sum(double (&v)[NV], double* partials, unsigned* counter, double (&out)[NV]) {
    __shared__ double sh[NV][32];
    __shared__ bool last;
    const int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
    const int nthreads = blockDim.x * blockDim.y * blockDim.z;
    const unsigned bid = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
    const unsigned nblocks = gridDim.x * gridDim.y * gridDim.z;
    block_sum<NV>(v, sh);
    if (tid == 0) {
#pragma unroll
        for (int q = 0; q < NV; ++q) partials[(size_t)bid * NV + q] = v[q];
        __threadfence();
        const unsigned ticket = atomicAdd(counter, 1u);
        last = (ticket == nblocks - 1);
    }
    __syncthreads();
    if (!last) return false;
    __threadfence();
    double acc[NV];
#pragma unroll
    for (int q = 0; q < NV; ++q) acc[q] = 0.0;
    for (unsigned b = tid; b < nblocks; b += nthreads) {
#pragma unroll
        for (int q = 0; q < NV; ++q) acc[q] += __ldcg(&partials[(size_t)b * NV + q]);
    }
    block_sum<NV>(acc, sh);
    if (tid == 0) {
#pragma unroll
        for (int q = 0; q < NV; ++q) out[q] = acc[q];
        *counter = 0u;
    }
    return tid == 0;
}

// ---------------------------------------------------------------------------------------
// interpolation (include/nama/math/interpolation.h)

template <typename T>
struct GridView {
    const T* __restrict__ d;
    int n0, n1, n2;
    T ox, oy, oz;
};

// calc_index_and_fraction (interpolation.h:10-15).  FP64 divides like the reference; FP32
// multiplies by 1/dx (differs from the division by at most an ulp of the cell coordinate).
template <typename T>
__device__ __forceinline__ void index_fraction(T pos, T origin, T dx, T inv_dx, int& idx, T& frac) {
    T t;
    if constexpr (sizeof(T) == 8)
        t = (pos - origin - T(0.5) * dx) / dx;
    else
        t = (pos - origin - T(0.5) * dx) * inv_dx;
    const T fl = floor(t);
    idx = (int)fl;
    frac = t - fl;
}

template <typename T>
__device__ __forceinline__ T lerp1(T a, T b, T f) {
    return (T(1) - f) * a + f * b;
}

// lerp(x, grid): clamped 8-point gather, x then y then z (interpolation.h:35-72, grid.h:369-377).
// Split in three so that every sampler (global or shared-memory data) rounds identically.
template <typename T>
struct TriIdx {
    int i0, i1, j0, j1, k0, k1;
    T fx, fy, fz;
};

template <typename T>
__device__ __forceinline__ TriIdx<T> tri_index(const GridView<T>& g, T x, T y, T z, T dx, T inv_dx) {
    int i, j, k;
    TriIdx<T> t;
    index_fraction(x, g.ox, dx, inv_dx, i, t.fx);
    index_fraction(y, g.oy, dx, inv_dx, j, t.fy);
    index_fraction(z, g.oz, dx, inv_dx, k, t.fz);
    t.i0 = clampi(i, 0, g.n0 - 1);
    t.i1 = clampi(i + 1, 0, g.n0 - 1);
    t.j0 = clampi(j, 0, g.n1 - 1);
    t.j1 = clampi(j + 1, 0, g.n1 - 1);
    t.k0 = clampi(k, 0, g.n2 - 1);
    t.k1 = clampi(k + 1, 0, g.n2 - 1);
    return t;
}

template <typename T>
__device__ __forceinline__ T tri_combine(const TriIdx<T>& t, T c000, T c100, T c010, T c110, T c001, T c101, T c011,
                                         T c111) {
    const T lo = lerp1(lerp1(c000, c100, t.fx), lerp1(c010, c110, t.fx), t.fy);
    const T hi = lerp1(lerp1(c001, c101, t.fx), lerp1(c011, c111, t.fx), t.fy);
    return lerp1(lo, hi, t.fz);
}

template <typename T>
__device__ __forceinline__ T tri_global(const GridView<T>& g, const TriIdx<T>& t) {
    const long long r00 = (long long)g.n0 * (t.j0 + (long long)g.n1 * t.k0);
    const long long r10 = (long long)g.n0 * (t.j1 + (long long)g.n1 * t.k0);
    const long long r01 = (long long)g.n0 * (t.j0 + (long long)g.n1 * t.k1);
    const long long r11 = (long long)g.n0 * (t.j1 + (long long)g.n1 * t.k1);
    const T c000 = __ldg(g.d + r00 + t.i0), c100 = __ldg(g.d + r00 + t.i1);
    const T c010 = __ldg(g.d + r10 + t.i0), c110 = __ldg(g.d + r10 + t.i1);
    const T c001 = __ldg(g.d + r01 + t.i0), c101 = __ldg(g.d + r01 + t.i1);
    const T c011 = __ldg(g.d + r11 + t.i0), c111 = __ldg(g.d + r11 + t.i1);
    return tri_combine(t, c000, c100, c010, c110, c001, c101, c011, c111);
}

template <typename T>
__device__ __forceinline__ T sample_trilinear(const GridView<T>& g, T x, T y, T z, T dx, T inv_dx) {
    return tri_global(g, tri_index(g, x, y, z, dx, inv_dx));
}

// Six-point WENO interpolation on nodes -2..3 at x = f in [0,1) (interpolation.h:74-111):
// three cubic candidates on nodes {-2..1}, {-1..2}, {0..3}; linear weights
// C = (2-x)(3-x)/20, (3-x)(x+2)/10, (x+2)(x+1)/20; smoothness indicators IS_s (the published
// quadratic forms / 180); alpha_s = C_s / (1e-6 + IS_s)^2; result sum(alpha p) / sum(alpha).
//
// Evaluation here: everything that depends only on x (the candidates' Lagrange weights and the
// linear weights) is formed once per axis and shared by all passes along that axis (36 along x,
// 6 along y, 1 along z per sample), and each IS is written as the equivalent quadratic form in
// the first differences d_m = v_m - v_{m-1} (the forms are translation invariant):
//   180 IS0 = 244 d1^2 - 1171 d1 d2 + 683 d1 d3 + 1561 d2^2 - 1951 d2 d3 + 814 d3^2
//   180 IS1 = 244 d2^2 -  781 d2 d3 + 293 d2 d4 +  961 d3^2 -  781 d3 d4 + 244 d4^2
//   180 IS2 = 814 d3^2 - 1951 d3 d4 + 683 d3 d5 + 1561 d4^2 - 1171 d4 d5 + 244 d5^2
// which avoids the cancellation of the value form (terms ~ v^2 cancelling to ~ d^2) in float.
template <typename T>
struct WenoAxis {
    T L[3][4];  // candidate s = sum_m L[s][m] v[s+m]
    T C[3];     // linear weights
};

template <typename T>
__device__ __forceinline__ WenoAxis<T> weno_axis(T x) {
    WenoAxis<T> w;
#pragma unroll
    for (int s = 0; s < 3; ++s) {
        // Newton form on nodes s-2, s-1, s, s+1: v_s + d e0 + d2 e0 e1 / 2 + d3 e0 e1 e2 / 6
        const T e0 = x + T(2 - s), e1 = x + T(1 - s), e2 = x - T(s);
        const T n1 = e0, n2 = e0 * e1 * T(0.5), n3 = e0 * e1 * e2 * T(1.0 / 6.0);
        w.L[s][0] = T(1) - n1 + n2 - n3;
        w.L[s][1] = n1 - T(2) * n2 + T(3) * n3;
        w.L[s][2] = n2 - T(3) * n3;
        w.L[s][3] = n3;
    }
    w.C[0] = (T(2) - x) * (T(3) - x) * T(1.0 / 20.0);
    w.C[1] = (T(3) - x) * (x + T(2)) * T(1.0 / 10.0);
    w.C[2] = (x + T(2)) * (x + T(1)) * T(1.0 / 20.0);
    return w;
}

// The data-only part of the nonlinear weights, independent of x: (eps + IS_s)^2 of the three
// candidates (FP64), or its reciprocal (FP32, fast reciprocal: the weights are then one
// multiplication each, alpha_s = C_s * q_s)
template <typename T>
__device__ __forceinline__ void weno6_sq(T v0, T v1, T v2, T v3, T v4, T v5, T& qa, T& qb, T& qc) {
    const T eps = T(1e-6);
    const T d1 = v1 - v0, d2 = v2 - v1, d3 = v3 - v2, d4 = v4 - v3, d5 = v5 - v4;
    const T k = T(1.0 / 180.0);
    const T ia = (d1 * (T(244) * d1 - T(1171) * d2 + T(683) * d3) + d2 * (T(1561) * d2 - T(1951) * d3) +
                  T(814) * d3 * d3) * k;
    const T ib = (d2 * (T(244) * d2 - T(781) * d3 + T(293) * d4) + d3 * (T(961) * d3 - T(781) * d4) +
                  T(244) * d4 * d4) * k;
    const T ic = (d3 * (T(814) * d3 - T(1951) * d4 + T(683) * d5) + d4 * (T(1561) * d4 - T(1171) * d5) +
                  T(244) * d5 * d5) * k;
    const T sa = eps + ia, sb = eps + ib, sc = eps + ic;
    if constexpr (sizeof(T) == 8) {
        qa = sa * sa;
        qb = sb * sb;
        qc = sc * sc;
    } else {
        qa = __fdividef(1.f, sa * sa);
        qb = __fdividef(1.f, sb * sb);
        qc = __fdividef(1.f, sc * sc);
    }
}

// the candidates at x and their nonlinear combination, given weno6_sq of the same values
template <typename T>
__device__ __forceinline__ T weno6_combine(const WenoAxis<T>& w, T v0, T v1, T v2, T v3, T v4, T v5, T qa, T qb,
                                           T qc) {
    const T pa = w.L[0][0] * v0 + w.L[0][1] * v1 + w.L[0][2] * v2 + w.L[0][3] * v3;
    const T pb = w.L[1][0] * v1 + w.L[1][1] * v2 + w.L[1][2] * v3 + w.L[1][3] * v4;
    const T pc = w.L[2][0] * v2 + w.L[2][1] * v3 + w.L[2][2] * v4 + w.L[2][3] * v5;
    if constexpr (sizeof(T) == 8) {
        const T aa = w.C[0] / qa, ab = w.C[1] / qb, ac = w.C[2] / qc;
        return (aa * pa + ab * pb + ac * pc) / (aa + ab + ac);
    } else {
        // FP32: qa, qb, qc hold the reciprocals; fast division for the normalisation (within 2 ulp)
        const T aa = w.C[0] * qa, ab = w.C[1] * qb, ac = w.C[2] * qc;
        return __fdividef(aa * pa + ab * pb + ac * pc, aa + ab + ac);
    }
}

// weno6_combine for two FP32 passes at once (lanes .x and .y) in packed float2 arithmetic:
// the candidates as FMA chains from the first product, the nonlinear combination
// (aa pa + ab pb + ac pc) / (aa + ab + ac), each lane rounded as its scalar operations
__device__ __forceinline__ float2 weno6_combine2(const WenoAxis<float>& w, const float2 (&v)[6], float2 qa, float2 qb,
                                                 float2 qc) {
    auto b2 = [](float x) { return make_float2(x, x); };
    float2 p[3];
#pragma unroll
    for (int s = 0; s < 3; ++s) {
        float2 t = __fmul2_rn(b2(w.L[s][0]), v[s]);
        t = __ffma2_rn(b2(w.L[s][1]), v[s + 1], t);
        t = __ffma2_rn(b2(w.L[s][2]), v[s + 2], t);
        p[s] = __ffma2_rn(b2(w.L[s][3]), v[s + 3], t);
    }
    const float2 aa = __fmul2_rn(b2(w.C[0]), qa), ab = __fmul2_rn(b2(w.C[1]), qb), ac = __fmul2_rn(b2(w.C[2]), qc);
    const float2 num = __ffma2_rn(ac, p[2], __ffma2_rn(ab, p[1], __fmul2_rn(aa, p[0])));
    const float2 den = __fadd2_rn(__fadd2_rn(aa, ab), ac);
    return make_float2(__fdividef(num.x, den.x), __fdividef(num.y, den.y));
}

// weno6_sq for two FP32 passes at once in packed float2 arithmetic (the reciprocals per lane)
__device__ __forceinline__ void weno6_sq2(const float2 (&v)[6], float2& qa, float2& qb, float2& qc) {
    auto b2 = [](float x) { return make_float2(x, x); };
    float2 d[6];
#pragma unroll
    for (int m = 1; m < 6; ++m) d[m] = __fadd2_rn(v[m], make_float2(-v[m - 1].x, -v[m - 1].y));  // exact negation
    const float2 k = b2(1.0f / 180.0f);
    auto form = [&](float2 a, float2 b, float2 c, float ca, float cb, float cc, float cbb, float cbc, float ccc) {
        // (a (ca a + cb b + cc c) + b (cbb b + cbc c) + ccc c c) k
        const float2 t1 = __ffma2_rn(b2(cc), c, __ffma2_rn(b2(cb), b, __fmul2_rn(b2(ca), a)));
        const float2 t2 = __ffma2_rn(b2(cbc), c, __fmul2_rn(b2(cbb), b));
        float2 t = __ffma2_rn(b, t2, __fmul2_rn(a, t1));
        t = __ffma2_rn(__fmul2_rn(b2(ccc), c), c, t);
        return __fmul2_rn(t, k);
    };
    const float2 ia = form(d[1], d[2], d[3], 244.f, -1171.f, 683.f, 1561.f, -1951.f, 814.f);
    const float2 ib = form(d[2], d[3], d[4], 244.f, -781.f, 293.f, 961.f, -781.f, 244.f);
    const float2 ic = form(d[3], d[4], d[5], 814.f, -1951.f, 683.f, 1561.f, -1171.f, 244.f);
    const float2 eps = b2(1e-6f);
    const float2 sa = __fadd2_rn(eps, ia), sb = __fadd2_rn(eps, ib), sc = __fadd2_rn(eps, ic);
    const float2 sa2 = __fmul2_rn(sa, sa), sb2 = __fmul2_rn(sb, sb), sc2 = __fmul2_rn(sc, sc);
    qa = make_float2(__fdividef(1.f, sa2.x), __fdividef(1.f, sa2.y));
    qb = make_float2(__fdividef(1.f, sb2.x), __fdividef(1.f, sb2.y));
    qc = make_float2(__fdividef(1.f, sc2.x), __fdividef(1.f, sc2.y));
}

__device__ __forceinline__ float2 weno6_eval2(const WenoAxis<float>& w, const float2 (&v)[6]) {
    float2 qa, qb, qc;
    weno6_sq2(v, qa, qb, qc);
    return weno6_combine2(w, v, qa, qb, qc);
}

template <typename T>
__device__ __forceinline__ T weno6_eval(const WenoAxis<T>& w, T v0, T v1, T v2, T v3, T v4, T v5) {
    T qa, qb, qc;
    weno6_sq(v0, v1, v2, v3, v4, v5, qa, qb, qc);
    return weno6_combine(w, v0, v1, v2, v3, v4, v5, qa, qb, qc);
}

// weno6_interp(x, grid) in 3-D: 6^3 clamped gather at offsets -2..3; x-passes, then y, then z
// (interpolation.h:124-137, 166-183).
template <typename T>
__device__ __forceinline__ T sample_weno6(const GridView<T>& g, T x, T y, T z, T dx, T inv_dx) {
    int i, j, k;
    T fx, fy, fz;
    index_fraction(x, g.ox, dx, inv_dx, i, fx);
    index_fraction(y, g.oy, dx, inv_dx, j, fy);
    index_fraction(z, g.oz, dx, inv_dx, k, fz);
    int ii[6], jr[6];
#pragma unroll
    for (int d = 0; d < 6; ++d) {
        ii[d] = clampi(i + d - 2, 0, g.n0 - 1);
        jr[d] = g.n0 * clampi(j + d - 2, 0, g.n1 - 1);
    }
    const long long plane = (long long)g.n0 * g.n1;
    const WenoAxis<T> wx = weno_axis(fx);
    T zl[6];
    // the z loop stays rolled: its body (six 6-point x-passes and a y-pass) already holds
    // plenty of independent loads, and unrolling it overflows the instruction cache
#pragma unroll 1
    for (int dk = 0; dk < 6; ++dk) {
        const T* base = g.d + plane * clampi(k + dk - 2, 0, g.n2 - 1);
        T yl[6];
#pragma unroll
        for (int dj = 0; dj < 6; ++dj) {
            const T* row = base + jr[dj];
            yl[dj] = weno6_eval(wx, __ldg(row + ii[0]), __ldg(row + ii[1]), __ldg(row + ii[2]), __ldg(row + ii[3]),
                                __ldg(row + ii[4]), __ldg(row + ii[5]));
        }
        const T zv = weno6_eval(weno_axis(fy), yl[0], yl[1], yl[2], yl[3], yl[4], yl[5]);
        // registers, not a dynamically indexed array
        zl[0] = dk == 0 ? zv : zl[0];
        zl[1] = dk == 1 ? zv : zl[1];
        zl[2] = dk == 2 ? zv : zl[2];
        zl[3] = dk == 3 ? zv : zl[3];
        zl[4] = dk == 4 ? zv : zl[4];
        zl[5] = dk == 5 ? zv : zl[5];
    }
    return weno6_eval(weno_axis(fz), zl[0], zl[1], zl[2], zl[3], zl[4], zl[5]);
}

// fraction_inside(phi_left, phi_right) (include/nama/math/level_set.h:68-80)
template <typename T>
__device__ __forceinline__ T fraction_inside(T a, T b) {
    if (a < T(0) && b < T(0)) return T(1);
    if (a < T(0) && b >= T(0)) return a / (a - b);
    if (a >= T(0) && b < T(0)) return b / (b - a);
    return T(0);
}

}  // namespace el
