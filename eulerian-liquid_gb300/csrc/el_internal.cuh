// el_internal.cuh -- shared device helpers and the context layout of the GB300 hot path.
//
// Data layout in HBM: every field is a dense i-fastest array with the reference's index
// i + n0*(j + n1*k) (include/nama/common/array.h:281-286), so host grids move with one copy.
// The pressure system is grid-shaped: the solver's vectors have one entry per cell, the
// entries of non-fluid cells are zero and their matrix rows are empty (diag = 0).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

#include "../../include/eulerian_liquid_gb300.h"

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
};

// One level of the multigrid hierarchy; level 0 aliases the fine inner matrix.
template <typename V>
struct MGLevel {
    int n0 = 0, n1 = 0, n2 = 0;
    V* diag = nullptr;
    V* off[3] = {nullptr, nullptr, nullptr};
    V* b = nullptr;
    V* x = nullptr;
    V* t = nullptr;
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
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    int64_t launches = 0;

    void* field[el::kMaxFields] = {};
    size_t field_bytes[el::kMaxFields] = {};

    // advection / extrapolation ping-pong buffers (same shapes as phi, u, v, w)
    void* tmp[4] = {};
    uint8_t* valid_tmp = nullptr;  // largest face mask

    // projection
    uint8_t* flags = nullptr;
    double* diag64 = nullptr;  // A_ii (double, projection.cpp:80-107)
    void* off[3] = {};         // A(c, c+x/y/z) in the field type (exactly -weight)
    double* rhs64 = nullptr;
    // FP64 Krylov vectors
    double *x64 = nullptr, *r64 = nullptr, *z64 = nullptr, *p64 = nullptr, *ap64 = nullptr;
    double* p64b = nullptr;  // second direction buffer (the fused K1 writes p out of place)
    // FP32 inner system (mixed solver)
    float* diag32 = nullptr;
    float* off32[3] = {};
    float *x32 = nullptr, *r32 = nullptr, *z32 = nullptr, *p32 = nullptr, *ap32 = nullptr;
    float* p32b = nullptr;
    std::vector<el::MGLevel<float>> mg32;
    std::vector<el::MGLevel<double>> mg64;

    el::Scalars* dscal = nullptr;  // [0] outer / plain, [1] inner
    el::Scalars* hscal = nullptr;  // pinned mirror
    double* partials = nullptr;
    unsigned* counter = nullptr;
    int max_partials = 0;

    std::vector<void*> allocations;
    std::string last_error;

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
};

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

// ---------------------------------------------------------------------------------------
// launch geometry: stencil kernels use blocks of 32 x 8 threads over (i, j) marching a chunk
// of planes along k, so the grid is (n0/32) x (n1/8) x (n2/kz) with no index division.

constexpr int kBX = 32, kBY = 8;

struct Geom {
    dim3 grid, block;
    int kz;  // planes per block
    int blocks() const { return grid.x * grid.y * grid.z; }
};

inline Geom stencil_geom(int n0, int n1, int n2, int num_sms) {
    Geom g;
    g.block = dim3(kBX, kBY, 1);
    const int gx = (n0 + kBX - 1) / kBX, gy = (n1 + kBY - 1) / kBY;
    // aim for ~8 resident blocks of 256 threads per SM, at least one plane per block
    const long long want = (long long)num_sms * 8;
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

// lerp(x, grid): clamped 8-point gather, x then y then z (interpolation.h:35-72, grid.h:369-377)
template <typename T>
__device__ __forceinline__ T sample_trilinear(const GridView<T>& g, T x, T y, T z, T dx, T inv_dx) {
    int i, j, k;
    T fx, fy, fz;
    index_fraction(x, g.ox, dx, inv_dx, i, fx);
    index_fraction(y, g.oy, dx, inv_dx, j, fy);
    index_fraction(z, g.oz, dx, inv_dx, k, fz);
    const int i0 = clampi(i, 0, g.n0 - 1), i1 = clampi(i + 1, 0, g.n0 - 1);
    const int j0 = clampi(j, 0, g.n1 - 1), j1 = clampi(j + 1, 0, g.n1 - 1);
    const int k0 = clampi(k, 0, g.n2 - 1), k1 = clampi(k + 1, 0, g.n2 - 1);
    const long long r00 = (long long)g.n0 * (j0 + (long long)g.n1 * k0);
    const long long r10 = (long long)g.n0 * (j1 + (long long)g.n1 * k0);
    const long long r01 = (long long)g.n0 * (j0 + (long long)g.n1 * k1);
    const long long r11 = (long long)g.n0 * (j1 + (long long)g.n1 * k1);
    const T c000 = __ldg(g.d + r00 + i0), c100 = __ldg(g.d + r00 + i1);
    const T c010 = __ldg(g.d + r10 + i0), c110 = __ldg(g.d + r10 + i1);
    const T c001 = __ldg(g.d + r01 + i0), c101 = __ldg(g.d + r01 + i1);
    const T c011 = __ldg(g.d + r11 + i0), c111 = __ldg(g.d + r11 + i1);
    const T lo = lerp1(lerp1(c000, c100, fx), lerp1(c010, c110, fx), fy);
    const T hi = lerp1(lerp1(c001, c101, fx), lerp1(c011, c111, fx), fy);
    return lerp1(lo, hi, fz);
}

// Six-point WENO interpolation on nodes -2..3 at x = f in [0,1) (interpolation.h:74-111):
// three cubic candidates in Newton form on nodes {-2..1}, {-1..2}, {0..3}; linear weights
// C = (2-x)(3-x)/20, (3-x)(x+2)/10, (x+2)(x+1)/20; the published smoothness indicators
// (quadratic forms / 180); alpha_s = C_s / (1e-6 + IS_s)^2; result sum(alpha p)/sum(alpha).
// Evaluated entirely in T (the reference's float instantiation forms a few products in
// double; the FP32 path differs from it at the 1e-7 relative level).
template <typename T>
__device__ __forceinline__ T weno6_1d(T v0, T v1, T v2, T v3, T v4, T v5, T x) {
    const T eps = T(1e-6);
    const T xm2 = x + T(2), xm1 = x + T(1), xp1 = x - T(1), xp2 = x - T(2), xp3 = x - T(3);
    // candidate on nodes -2,-1,0,1
    const T d1a = v1 - v0, d2a = v2 - T(2) * v1 + v0, d3a = v3 - T(3) * v2 + T(3) * v1 - v0;
    const T pa = v0 + d1a * xm2 + T(0.5) * d2a * xm2 * xm1 + d3a * T(1.0 / 6.0) * xm2 * xm1 * x;
    // candidate on nodes -1,0,1,2
    const T d1b = v2 - v1, d2b = v3 - T(2) * v2 + v1, d3b = v4 - T(3) * v3 + T(3) * v2 - v1;
    const T pb = v1 + d1b * xm1 + T(0.5) * d2b * xm1 * x + d3b * T(1.0 / 6.0) * xm1 * x * xp1;
    // candidate on nodes 0,1,2,3
    const T d1c = v3 - v2, d2c = v4 - T(2) * v3 + v2, d3c = v5 - T(3) * v4 + T(3) * v3 - v2;
    const T pc = v2 + d1c * x + T(0.5) * d2c * x * xp1 + d3c * T(1.0 / 6.0) * x * xp1 * xp2;
    const T ca = -xp2 * -xp3 * T(1.0 / 20.0);
    const T cb = -xp3 * xm2 * T(1.0 / 10.0);
    const T cc = xm2 * xm1 * T(1.0 / 20.0);
    const T ia = (T(814) * v3 * v3 + T(4326) * v2 * v2 + T(2976) * v1 * v1 + T(244) * v0 * v0
                  - T(3579) * v2 * v3 - T(6927) * v2 * v1 + T(1854) * v2 * v0 + T(2634) * v3 * v1
                  - T(683) * v3 * v0 - T(1659) * v1 * v0) * T(1.0 / 180.0);
    const T ib = (T(1986) * v3 * v3 + T(1986) * v2 * v2 + T(244) * v1 * v1 + T(244) * v4 * v4
                  + T(1074) * v2 * v4 - T(3777) * v2 * v3 - T(1269) * v2 * v1 + T(1074) * v3 * v1
                  - T(1269) * v4 * v3 - T(293) * v4 * v1) * T(1.0 / 180.0);
    const T ic = (T(814) * v2 * v2 + T(4326) * v3 * v3 + T(2976) * v4 * v4 + T(244) * v5 * v5
                  - T(683) * v2 * v5 + T(2634) * v2 * v4 - T(3579) * v2 * v3 - T(6927) * v3 * v4
                  + T(1854) * v3 * v5 - T(1659) * v4 * v5) * T(1.0 / 180.0);
    const T sa = eps + ia, sb = eps + ib, sc = eps + ic;
    const T aa = ca / (sa * sa), ab = cb / (sb * sb), ac = cc / (sc * sc);
    return (aa * pa + ab * pb + ac * pc) / (aa + ab + ac);
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
    int ii[6];
    long long jr[6], kr[6];
#pragma unroll
    for (int d = 0; d < 6; ++d) {
        ii[d] = clampi(i + d - 2, 0, g.n0 - 1);
        jr[d] = (long long)g.n0 * clampi(j + d - 2, 0, g.n1 - 1);
        kr[d] = (long long)g.n0 * g.n1 * clampi(k + d - 2, 0, g.n2 - 1);
    }
    T zl[6];
#pragma unroll 1
    for (int dk = 0; dk < 6; ++dk) {
        T yl[6];
#pragma unroll
        for (int dj = 0; dj < 6; ++dj) {
            const T* row = g.d + kr[dk] + jr[dj];
            yl[dj] = weno6_1d(__ldg(row + ii[0]), __ldg(row + ii[1]), __ldg(row + ii[2]),
                              __ldg(row + ii[3]), __ldg(row + ii[4]), __ldg(row + ii[5]), fx);
        }
        zl[dk] = weno6_1d(yl[0], yl[1], yl[2], yl[3], yl[4], yl[5], fy);
    }
    return weno6_1d(zl[0], zl[1], zl[2], zl[3], zl[4], zl[5], fz);
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
