// el_solve.cu -- conjugate-gradient pressure solves on the grid-shaped ghost-fluid matrix.
//
// Replaces the Eigen ConjugateGradient<..., Lower, IncompleteCholesky<double>> call of
// src/project/3d/eulerian_liquid/simulator.cpp:102-109 (x0 = 0, stop on |r|^2 < tol^2 |b|^2 of
// the recursively updated residual, iteration cap) with three GPU solvers:
//
//   EL_SOLVER_JACOBI_FP64  plain FP64 PCG, Jacobi preconditioner (the correctness baseline)
//   EL_SOLVER_MG_FP64      FP64 PCG with a multigrid V-cycle preconditioner
//   EL_SOLVER_MIXED        FP64 iterative refinement: r = b - A x in FP64, the correction
//                          solved by FP32 multigrid PCG on the FP32 operator, x += |r| e in FP64
//
// Work distribution: every level keeps an ordered list of its active row segments (32 cells
// of one (j, k) row holding at least one cell with a positive diagonal).  Kernels run one
// warp per listed segment with a fixed grid, so cells that are air or solid cost nothing,
// all loads of a cell are issued before any is used, and the partial sums of the dot
// products are formed in a fixed order (deterministic).  Vector entries outside the active
// segments are never written; they stay finite and always meet a zero coupling.
//
// Operators are stored as per-cell records {diagonal, coupling with +x, +y, +z}: float4 for
// the FP32 PCG operator, Rec64 for the FP64 multigrid, and half4 for the level-0 operator the
// FP32 multigrid smooths with (diagonal rounded up, couplings rounded towards zero, so the
// record operator stays diagonally dominant, hence SPD).
//
// Multigrid: coarse operators by aggregation of 2x2x2 blocks scaled by 1/2
// (A_c = 1/2 P^T A P, piecewise-constant P; it reproduces the rediscretised Laplacian for
// constant coefficients and carries the ghost-fluid Dirichlet terms down by summation),
// restriction R = P^T, two Jacobi sweeps before and two after with Chebyshev weights (see
// kSweep1 / kSweep2), and 30 damped-Jacobi sweeps on the coarsest level (at most 8 cells per
// axis) in one block's shared memory.  The same polynomial smoother on both legs and R = P^T
// make the V-cycle symmetric, as PCG needs.
//
// Per PCG iteration:  K1  p = z + beta p ; Ap = A p ; alpha = rz / p.Ap
//                     K2  x += alpha p ; r -= alpha Ap ; rr = r.r (; rz = r.D^-1 r for Jacobi)
//                     V   z = M^-1 r ; rz = r.z ; beta            (multigrid solvers)
// Scalars live in device memory; once converged the remaining launched kernels return at
// entry, so the host polls only every `check_every` iterations.
#include <cuda_fp16.h>

#include <type_traits>

#include "el_df.cuh"
#include "el_internal.cuh"

namespace el {

// Damped Jacobi on the coarsest level (a solve): the damping that balances the 3-D 7-point
// Laplacian's high-frequency error reduction.
constexpr double kOmega = 6.0 / 7.0;
// The smoother's sweep weights kSweep1 / kSweep2 are defined in el_internal.cuh.
constexpr int kCoarsestSweeps = 30;
constexpr int kCoarsestMaxDim = 8;
constexpr int kCoarsestMaxCells = 512;
constexpr int kSegThreads = 256;

__device__ __forceinline__ bool finite_d(double v) { return isfinite(v); }

// ---------------------------------------------------------------------------------------
// coefficient records

template <typename V>
struct Co {
    V d, x, y, z;
};

__device__ __forceinline__ Co<float> ldrec(const float4* r, long long c) {
    const float4 v = __ldg(r + c);
    return {v.x, v.y, v.z, v.w};
}
__device__ __forceinline__ Co<float> ldrec(const ushort4* r, long long c) {
    const ushort4 v = __ldg(r + c);
    return {__half2float(__ushort_as_half(v.x)), __half2float(__ushort_as_half(v.y)),
            __half2float(__ushort_as_half(v.z)), __half2float(__ushort_as_half(v.w))};
}
__device__ __forceinline__ Co<double> ldrec(const Rec64* r, long long c) {
    const double2* p = reinterpret_cast<const double2*>(r + c);
    const double2 a = __ldg(p), b = __ldg(p + 1);
    return {a.x, a.y, b.x, b.y};
}

// The FP64 operator of the context: diag64 plus three coupling arrays of the field type.
template <typename OT>
struct SplitOp {
    const double* __restrict__ d;
    const OT* __restrict__ x;
    const OT* __restrict__ y;
    const OT* __restrict__ z;
};

// ---------------------------------------------------------------------------------------
// segment geometry

struct LGeom {
    int n0, n1, n2, nsr;
    int s1, s2;  // strides of j and k (every grid holds fewer than 2^31 cells)
};

inline LGeom make_geom(int n0, int n1, int n2) {
    return LGeom{n0, n1, n2, (n0 + 31) / 32, n0, n0 * n1};
}

__device__ __forceinline__ void seg_cell(int id, const LGeom& g, int lane, int& i, int& j, int& k) {
    const int row = id / g.nsr;
    i = (id - row * g.nsr) * 32 + lane;
    j = row % g.n1;
    k = row / g.n1;
}

struct SegArg {
    const int4* __restrict__ desc;  // {first cell index, i0, j, k}
    const int* __restrict__ count;
};

// Walks the active segments, one warp per segment; defines lane, i, j, k, c (cell index, int:
// every grid holds fewer than 2^31 cells) and live (i < n0).  Lanes past the row end stay in
// the loop (live = false) so that warp shuffles see all 32 lanes.
#define SEG_LOOP_ALL_BEGIN(seg, g)                                                \
    const int lane = threadIdx.x & 31;                                            \
    const int warp_global = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;         \
    const int nwarps = (gridDim.x * blockDim.x) >> 5;                             \
    const int nseg = *(seg).count;                                                \
    for (int qs = warp_global; qs < nseg; qs += nwarps) {                         \
        const int4 sd = (seg).desc[qs];                                           \
        const int i = sd.y + lane, j = sd.z, k = sd.w;                            \
        const int c = sd.x + lane;                                                \
        const bool live = i < (g).n0;

// the same over an explicit warp numbering (warp wg of nw warps)
#define SEG_LOOP_ALL_W_BEGIN(seg, g, wg, nw)                                      \
    const int lane = threadIdx.x & 31;                                            \
    const int nseg = *(seg).count;                                                \
    for (int qs = (wg); qs < nseg; qs += (nw)) {                                  \
        const int4 sd = (seg).desc[qs];                                           \
        const int i = sd.y + lane, j = sd.z, k = sd.w;                            \
        const int c = sd.x + lane;                                                \
        const bool live = i < (g).n0;

// the same, with the next segment's descriptor loaded while the current one is processed (for
// the kernels whose registers leave room for it)
#define SEG_LOOP_ALL_PF_BEGIN(seg, g)                                             \
    const int lane = threadIdx.x & 31;                                            \
    const int warp_global = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;         \
    const int nwarps = (gridDim.x * blockDim.x) >> 5;                             \
    const int nseg = *(seg).count;                                                \
    int4 sd_next = warp_global < nseg ? (seg).desc[warp_global] : make_int4(0, 0, 0, 0); \
    for (int qs = warp_global; qs < nseg; qs += nwarps) {                         \
        const int4 sd = sd_next;                                                  \
        if (qs + nwarps < nseg) sd_next = (seg).desc[qs + nwarps];                \
        const int i = sd.y + lane, j = sd.z, k = sd.w;                            \
        const int c = sd.x + lane;                                                \
        const bool live = i < (g).n0;

#define SEG_LOOP_BEGIN(seg, g) \
    SEG_LOOP_ALL_PF_BEGIN(seg, g) \
    if (!live) continue;

#define SEG_LOOP_END }

constexpr unsigned kFull = 0xffffffffu;

// ---------------------------------------------------------------------------------------
// segment lists: per-segment activity flag, then an ordered compaction

constexpr int kSegChunk = 1024;

template <typename R>
__global__ void seg_flags_rec_kernel(LGeom g, const R* __restrict__ rec, long long total, uint8_t* __restrict__ flags) {
    const int lane = threadIdx.x & 31;
    const long long w0 = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
    const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
    for (long long id = w0; id < total; id += nw) {
        int i, j, k;
        seg_cell((int)id, g, lane, i, j, k);
        bool act = false;
        if (i < g.n0) act = ldrec(rec, i + g.s1 * j + g.s2 * k).d > 0;
        const unsigned m = __ballot_sync(0xffffffffu, act);
        if (lane == 0) flags[id] = m ? 1 : 0;
    }
}

__global__ void seg_flags_diag_kernel(LGeom g, const double* __restrict__ diag, long long total,
                                      uint8_t* __restrict__ flags) {
    // a warp per row (j, k): one index division a row, not one a segment, and up to eight of
    // the row's segments in flight together; segment id = row * nsr + segment of the row
    (void)total;
    const int lane = threadIdx.x & 31;
    const long long w0 = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
    const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
    const long long nrows = (long long)g.n1 * g.n2;
    constexpr int U = 8;
    for (long long row = w0; row < nrows; row += nw) {
        const int j = (int)(row % g.n1), k = (int)(row / g.n1);
        const double* drow = diag + (long long)g.s1 * j + (long long)g.s2 * k;
        for (int s0 = 0; s0 < g.nsr; s0 += U) {
            bool act[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const int i = (s0 + u) * 32 + lane;
                act[u] = s0 + u < g.nsr && i < g.n0 && d_positive(drow[i]);
            }
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const unsigned m = __ballot_sync(0xffffffffu, act[u]);
                if (lane == 0 && s0 + u < g.nsr) flags[row * g.nsr + s0 + u] = m ? 1 : 0;
            }
        }
    }
}

__global__ void seg_count_kernel(const uint8_t* __restrict__ flags, long long total, int* __restrict__ chunk) {
    __shared__ int sh[8];
    const long long base = (long long)blockIdx.x * kSegChunk;
    int cnt = 0;
    for (int q = threadIdx.x; q < kSegChunk; q += blockDim.x) {
        const long long id = base + q;
        if (id < total && flags[id]) ++cnt;
    }
    for (int o = 16; o > 0; o >>= 1) cnt += __shfl_down_sync(0xffffffffu, cnt, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = cnt;
    __syncthreads();
    if (threadIdx.x == 0) {
        int t = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += sh[w];
        chunk[blockIdx.x] = t;
    }
}

// Exclusive scan of the chunk counts in one block of 1024 threads: each thread sums a span of
// chunks, the span sums are scanned by warp shuffles (within a warp, then over the 32 warp
// totals), and each thread rewrites its span with running offsets.
__global__ void seg_scan_kernel(int* __restrict__ chunk, int nchunks, int* __restrict__ total_out) {
    __shared__ int wsum[32];
    const int per = (nchunks + blockDim.x - 1) / blockDim.x;
    const int lo = threadIdx.x * per, hi = min(nchunks, lo + per);
    int s = 0;
    for (int q = lo; q < hi; ++q) s += chunk[q];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    int x = s;  // inclusive scan within the warp
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(kFull, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) wsum[w] = x;
    __syncthreads();
    if (w == 0) {
        int v = lane < nw ? wsum[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(kFull, v, o);
            if (lane >= o) v += y;
        }
        wsum[lane] = v;  // inclusive over the warps
    }
    __syncthreads();
    int run = x - s + (w > 0 ? wsum[w - 1] : 0);
    if (threadIdx.x == blockDim.x - 1) *total_out = run + s;
    for (int q = lo; q < hi; ++q) {
        const int v = chunk[q];
        chunk[q] = run;
        run += v;
    }
}

// The descriptors of a chunk's active segments, in order: each warp of the block takes an equal
// run of the chunk's flags, counts its active ones, and writes them after the counts of the
// warps before it.
__global__ void seg_write_kernel(LGeom g, const uint8_t* __restrict__ flags, long long total,
                                 const int* __restrict__ chunk, int4* __restrict__ desc) {
    __shared__ int wcount[32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int span = kSegChunk / nw;
    const long long wb = (long long)blockIdx.x * kSegChunk + (long long)w * span;
    int cnt = 0;
    for (int q = 0; q < span; q += 32) {
        const long long id = wb + q + lane;
        cnt += __popc(__ballot_sync(kFull, id < total && flags[id]));
    }
    if (lane == 0) wcount[w] = cnt;
    __syncthreads();
    int run = chunk[blockIdx.x];
    for (int v = 0; v < w; ++v) run += wcount[v];
    for (int q = 0; q < span; q += 32) {
        const long long id = wb + q + lane;
        const bool f = id < total && flags[id];
        const unsigned m = __ballot_sync(kFull, f);
        if (f) {
            int i0, j, k;
            seg_cell((int)id, g, 0, i0, j, k);
            desc[run + __popc(m & ((1u << lane) - 1u))] = make_int4((int)(i0 + g.s1 * j + g.s2 * k), i0, j, k);
        }
        run += __popc(m);
    }
}

// ---------------------------------------------------------------------------------------
// operator packing (once per solve)

// float4 PCG records and half4 multigrid records of the FP32 inner system.
template <typename OT>
__global__ void pack32_kernel(long long n, const double* __restrict__ d, const OT* __restrict__ ox,
                              const OT* __restrict__ oy, const OT* __restrict__ oz, float4* __restrict__ a32,
                              ushort4* __restrict__ a16) {
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
        const float4 r = make_float4((float)d[c], (float)ox[c], (float)oy[c], (float)oz[c]);
        a32[c] = r;
        // diagonal rounded up, (non-positive) couplings rounded towards zero: the half record
        // operator keeps diag >= sum |couplings| row by row
        a16[c] = make_ushort4(__half_as_ushort(__float2half_ru(r.x)), __half_as_ushort(__float2half_rz(r.y)),
                              __half_as_ushort(__float2half_rz(r.z)), __half_as_ushort(__float2half_rz(r.w)));
    }
}

template <typename OT>
__global__ void pack64_kernel(long long n, const double* __restrict__ d, const OT* __restrict__ ox,
                              const OT* __restrict__ oy, const OT* __restrict__ oz, Rec64* __restrict__ a) {
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x)
        a[c] = Rec64{d[c], (double)ox[c], (double)oy[c], (double)oz[c]};
}

// Coarse records A_c = 1/2 P^T A P over 2x2x2 blocks.  The FP32 hierarchy (float4 coarse
// records, built from half4 or float4 records) sums in FP32 -- the eight children's values
// carry at most 24 significant bits, and FP64 arithmetic runs at a small fraction of the FP32
// rate on this GPU -- the FP64 hierarchy in FP64.
template <typename RF, typename RC>
__global__ void coarsen_kernel(LGeom F, const RF* __restrict__ fr, LGeom C, RC* __restrict__ cr) {
    using A = typename std::conditional<sizeof(RC) == sizeof(float4), float, double>::type;
    const int I = blockIdx.x * blockDim.x + threadIdx.x;
    const int J = blockIdx.y * blockDim.y + threadIdx.y;
    const int K = blockIdx.z;
    if (I >= C.n0 || J >= C.n1) return;
    A d = 0, sx = 0, sy = 0, sz = 0, inner = 0;
    for (int kk = 0; kk < 2; ++kk)
        for (int jj = 0; jj < 2; ++jj)
            for (int ii = 0; ii < 2; ++ii) {
                const int i = 2 * I + ii, j = 2 * J + jj, k = 2 * K + kk;
                if (i >= F.n0 || j >= F.n1 || k >= F.n2) continue;
                const auto r = ldrec(fr, i + F.s1 * j + F.s2 * k);
                d += r.d;
                if (ii == 0) inner += r.x; else sx += r.x;
                if (jj == 0) inner += r.y; else sy += r.y;
                if (kk == 0) inner += r.z; else sz += r.z;
            }
    A dc = A(0.5) * (d + A(2) * inner);
    // an aggregate coupled to nothing outside it (an enclosed Neumann pocket) has a zero row
    // sum; its diagonal is raised to half the children's, which keeps the operator SPD
    if (d > A(0) && !(dc > A(1e-6) * d)) dc = A(0.5) * d;
    const long long q = I + C.s1 * J + C.s2 * K;
    if constexpr (sizeof(RC) == sizeof(float4))
        cr[q] = make_float4(dc, A(0.5) * sx, A(0.5) * sy, A(0.5) * sz);
    else
        cr[q] = Rec64{dc, 0.5 * sx, 0.5 * sy, 0.5 * sz};
}

// ---------------------------------------------------------------------------------------
// The 7-point stencil around each lane's cell.  recf(q) loads a cell's record (diagonal and
// +x/+y/+z couplings), rawf(q, qi, qj, qk) loads the vector data of a cell and valf(raw, rec)
// turns it into the value the stencil applies to.  Every load of the stencil (including the
// cells just outside the segment, fetched by lanes 0 and 31) is issued before any value is
// formed, so a lane waits for memory once; the i-neighbours of the other lanes come by shuffle.
// ALL: every neighbour's record is needed (for its diagonal); else only those carrying a
// coupling (-x, -y, -z) are loaded.  Must be called by all 32 lanes.
// Per-thread partial sums of a dot product: FP32 for the FP32 solver (a thread sums a few
// dozen products; FP64 arithmetic runs at a small fraction of the FP32 rate on this GPU), FP64
// otherwise; the grid reduction is FP64 either way.
template <typename V>
using DotAcc = typename std::conditional<sizeof(V) == 4, float, double>::type;

template <typename V>
struct St7 {
    V v0, vxm, vxp, vym, vyp, vzm, vzp;  // values at the centre and the six neighbours
    V d, cxm, cxp, cym, cyp, czm, czp;   // diagonal and couplings
};

template <typename V, bool ALL, typename RF, typename LF, typename VF>
__device__ __forceinline__ St7<V> gather7(const LGeom& g, int c, int i, int j, int k, bool live, int lane, RF&& recf,
                                          LF&& rawf, VF&& valf) {
    const Co<V> z4{V(0), V(0), V(0), V(0)};
    const bool iym = live && j > 0, iyp = live && j < g.n1 - 1;
    const bool izm = live && k > 0, izp = live && k < g.n2 - 1;
    const bool ixm = lane == 0 && live && i > 0;
    const bool ixp = lane == 31 && live && i + 1 < g.n0;
    // loads
    const Co<V> r0 = live ? recf(c) : z4;
    const Co<V> rym = iym ? recf(c - g.s1) : z4;
    const Co<V> ryp = (ALL && iyp) ? recf(c + g.s1) : z4;
    const Co<V> rzm = izm ? recf(c - g.s2) : z4;
    const Co<V> rzp = (ALL && izp) ? recf(c + g.s2) : z4;
    const Co<V> rxm = ixm ? recf(c - 1) : z4;
    const Co<V> rxp = (ALL && ixp) ? recf(c + 1) : z4;
    using Raw = decltype(rawf(0, 0, 0, 0));
    const Raw a0 = live ? rawf(c, i, j, k) : Raw{};
    const Raw aym = iym ? rawf(c - g.s1, i, j - 1, k) : Raw{};
    const Raw ayp = iyp ? rawf(c + g.s1, i, j + 1, k) : Raw{};
    const Raw azm = izm ? rawf(c - g.s2, i, j, k - 1) : Raw{};
    const Raw azp = izp ? rawf(c + g.s2, i, j, k + 1) : Raw{};
    const Raw axm = ixm ? rawf(c - 1, i - 1, j, k) : Raw{};
    const Raw axp = ixp ? rawf(c + 1, i + 1, j, k) : Raw{};
    // values and couplings
    St7<V> st;
    st.d = r0.d;
    st.cxp = r0.x;
    st.cyp = r0.y;
    st.czp = r0.z;
    st.cym = rym.y;
    st.czm = rzm.z;
    st.v0 = live ? valf(a0, r0) : V(0);
    st.vym = iym ? valf(aym, rym) : V(0);
    st.vyp = iyp ? valf(ayp, ryp) : V(0);
    st.vzm = izm ? valf(azm, rzm) : V(0);
    st.vzp = izp ? valf(azp, rzp) : V(0);
    const V sxm = __shfl_up_sync(kFull, st.v0, 1);
    const V sxp = __shfl_down_sync(kFull, st.v0, 1);
    const V scm = __shfl_up_sync(kFull, r0.x, 1);
    st.vxm = lane == 0 ? (ixm ? valf(axm, rxm) : V(0)) : sxm;
    st.cxm = lane == 0 ? rxm.x : scm;
    st.vxp = (live && i + 1 < g.n0) ? (lane == 31 ? valf(axp, rxp) : sxp) : V(0);
    return st;
}

template <typename V>
__device__ __forceinline__ V apply7(const St7<V>& st) {
    return stencil7(st.d, st.v0, st.cxm, st.vxm, st.cxp, st.vxp, st.cym, st.vym, st.cyp, st.vyp, st.czm, st.vzm,
                    st.czp, st.vzp);
}

template <typename V, typename R>
struct RecLoad {
    const R* __restrict__ a;
    __device__ __forceinline__ Co<V> operator()(int q) const {
        const auto r = ldrec(a, q);
        return Co<V>{(V)r.d, (V)r.x, (V)r.y, (V)r.z};
    }
};

template <typename OT>
struct SplitLoad {
    SplitOp<OT> a;
    __device__ __forceinline__ Co<double> operator()(int q) const {
        return Co<double>{a.d[q], f2d(a.x[q]), f2d(a.y[q]), f2d(a.z[q])};
    }
};

// K1: new direction fused with A p and p.Ap over the active segments.
// Record operator (FP32 inner / FP64 multigrid).
template <typename V, typename R>
__global__ void __launch_bounds__(kSegThreads) dir_spmv_rec_kernel(LGeom g, SegArg seg, const R* __restrict__ A,
                                                                   const V* __restrict__ z, const V* __restrict__ p_in,
                                                                   V* __restrict__ p_out, V* __restrict__ ap,
                                                                   Scalars* s, int first, double* partials,
                                                                   unsigned* counter) {
    if (s->done) return;
    const V beta = first ? V(0) : (V)s->beta;
    DotAcc<V> part = 0;
    const RecLoad<V, R> recf{A};
    auto rawf = [&](int q, int, int, int) -> V { return first ? z[q] : z[q] + beta * p_in[q]; };
    auto valf = [](V raw, const Co<V>&) -> V { return raw; };
    SEG_LOOP_ALL_PF_BEGIN(seg, g)
    const St7<V> st = gather7<V, false>(g, c, i, j, k, live, lane, recf, rawf, valf);
    if (live) {
        V pc = V(0), apc = V(0);
        if (st.d > V(0)) {
            pc = st.v0;
            apc = apply7(st);
        }
        p_out[c] = pc;
        ap[c] = apc;
        part += (DotAcc<V>)pc * (DotAcc<V>)apc;
    }
    SEG_LOOP_END
    double acc[1] = {(double)part};
    double tot[1];
    if (grid_sum<1>(acc, partials, counter, tot)) {
        const double alpha = s->rz / tot[0];
        s->alpha = alpha;
        if (!finite_d(alpha)) {
            s->bad = 1;
            s->done = 1;
        }
    }
}

// Split FP64 operator with the Jacobi preconditioner applied on the fly (plain FP64 PCG).
template <typename OT>
__global__ void __launch_bounds__(kSegThreads) dir_spmv_jacobi_kernel(LGeom g, SegArg seg, SplitOp<OT> A,
                                                                      const double* __restrict__ r,
                                                                      const double* __restrict__ p_in,
                                                                      double* __restrict__ p_out,
                                                                      double* __restrict__ ap, Scalars* s, int first,
                                                                      double* partials, unsigned* counter) {
    if (s->done) return;
    const double beta = first ? 0.0 : s->beta;
    double acc[1] = {0.0};
    const SplitLoad<OT> recf{A};
    // raw = (r, p) packed as a pair of doubles
    auto rawf = [&](int q, int, int, int) -> double2 { return make_double2(r[q], first ? 0.0 : p_in[q]); };
    auto valf = [&](double2 raw, const Co<double>& rec) -> double {
        return rec.d > 0.0 ? raw.x / rec.d + beta * raw.y : 0.0;
    };
    SEG_LOOP_ALL_BEGIN(seg, g)
    const St7<double> st = gather7<double, true>(g, c, i, j, k, live, lane, recf, rawf, valf);
    if (live) {
        const double apc = st.d > 0.0 ? apply7(st) : 0.0;
        p_out[c] = st.v0;
        ap[c] = apc;
        acc[0] += st.v0 * apc;
    }
    SEG_LOOP_END
    double tot[1];
    if (grid_sum<1>(acc, partials, counter, tot)) {
        const double alpha = s->rz / tot[0];
        s->alpha = alpha;
        if (!finite_d(alpha)) {
            s->bad = 1;
            s->done = 1;
        }
    }
}

// K2: x += alpha p ; r -= alpha Ap ; |r|^2 (and r.D^-1 r for Jacobi, giving beta).
template <typename V, bool JAC>
__global__ void __launch_bounds__(kSegThreads) update_kernel(LGeom g, SegArg seg, const double* __restrict__ diag,
                                                             V* __restrict__ x, V* __restrict__ r,
                                                             const V* __restrict__ p, const V* __restrict__ ap,
                                                             Scalars* s, double* partials, unsigned* counter) {
    if (s->done) return;
    const V alpha = (V)s->alpha;
    double acc[2] = {0.0, 0.0};
    DotAcc<V> part = 0;
    // two segments per warp and iteration, all eight loads issued before any use: the kernel is
    // pure streaming and bound by the loads in flight
    const int lane = threadIdx.x & 31;
    const int warp_global = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    const int nseg = *seg.count;
    auto finish = [&](int c, V pc, V apc, V xc, V rc0) {
        const V rc = rc0 - alpha * apc;
        x[c] = xc + alpha * pc;
        r[c] = rc;
        part += (DotAcc<V>)rc * (DotAcc<V>)rc;
        if (JAC) {
            const double d = diag[c];
            if (d > 0.0) acc[1] += (double)rc * ((double)rc / d);
        }
    };
    for (int qs = warp_global; qs < nseg; qs += 2 * nwarps) {
        const int q2 = qs + nwarps;
        const int4 sa = seg.desc[qs];
        const int4 sb = q2 < nseg ? seg.desc[q2] : sa;
        const bool la = sa.y + lane < g.n0, lb = q2 < nseg && sb.y + lane < g.n0;
        const int ca = sa.x + lane, cb = sb.x + lane;
        V pa = V(0), apa = V(0), xa = V(0), ra = V(0), pb = V(0), apb = V(0), xb = V(0), rb = V(0);
        if (la) {
            pa = p[ca];
            apa = ap[ca];
            xa = x[ca];
            ra = r[ca];
        }
        if (lb) {
            pb = p[cb];
            apb = ap[cb];
            xb = x[cb];
            rb = r[cb];
        }
        if (la) finish(ca, pa, apa, xa, ra);
        if (lb) finish(cb, pb, apb, xb, rb);
    }
    acc[0] = (double)part;
    double tot[2];
    if (grid_sum<2>(acc, partials, counter, tot)) {
        s->rr = tot[0];
        s->iter += 1;
        if (!finite_d(tot[0])) {
            s->bad = 1;
            s->done = 1;
        } else if (tot[0] < s->thresh) {
            s->done = 1;
        }
        if (JAC) {
            s->beta = tot[1] / s->rz;
            s->rz = tot[1];
        }
    }
}

// Jacobi start: rz = r . D^-1 r
__global__ void jacobi_rz_kernel(LGeom g, SegArg seg, const double* __restrict__ diag, const double* __restrict__ r,
                                 Scalars* s, double* partials, unsigned* counter) {
    double acc[1] = {0.0};
    SEG_LOOP_BEGIN(seg, g)
    const double d = diag[c];
    if (d > 0.0) acc[0] += r[c] * (r[c] / d);
    SEG_LOOP_END
    double tot[1];
    if (grid_sum<1>(acc, partials, counter, tot)) s->rz = tot[0];
}

// The iterate as a float pair for the double-float residual (el_df.cuh), written with x by the
// kernels that change it (xs: null where no double-float residual reads it), shifted by the
// solve's power of two 2^df_shift (set from |b| by solve_init_kernel), which keeps the pairs
// of the whole system near 1 whatever its scale.  Beyond the pairs'
// range (|x| >= 2^128, an iterate no FP32 field can hold) the pair is infinite, so that the
// residual turns non-finite and the solve reports it.
__device__ __forceinline__ float2 x_pair(double x, int shift) {
    const double xs = d_shift(x, shift);
    bool ok = true;
    const F2 p = df_split(xs, ok);
    return ok ? make_float2(p.h, p.l) : make_float2(d2f(xs), 0.f);
}

// solve start (outer / plain): x = 0, r = b on the active segments, thresholds.
__global__ void solve_init_kernel(LGeom g, SegArg seg, const double* __restrict__ b, double* __restrict__ x,
                                  float2* __restrict__ xs, double* __restrict__ r, Scalars* s, double tol) {
    SEG_LOOP_BEGIN(seg, g)
    x[c] = 0.0;
    if (xs) xs[c] = make_float2(0.f, 0.f);
    r[c] = b[c];
    SEG_LOOP_END
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        const double bb = s->bb;
        // 2^df_shift |b| in [1, 2): the exponent of |b|^2 halved (0 for a zero or non-finite b)
        const unsigned long long bbits = (unsigned long long)__double_as_longlong(bb);
        const int eb = (int)((bbits >> 52) & 0x7ffu);
        s->df_shift = (eb == 0 || eb == 0x7ff) ? 0 : -((eb - 1023) >> 1);
        s->thresh = tol * tol * bb;
        s->rr = bb;
        s->iter = 0;
        s->bad = finite_d(bb) ? 0 : 1;
        s->done = (bb == 0.0 || bb < s->thresh || s->bad) ? 1 : 0;
        s->beta = 0.0;
        s->outer = 0;
        s->inner_total = 0;
        s->inner_passes = 0;
        s->fault = 0;
    }
}

// ---- warm start: x0 = alpha g with g the pressure grid as it stands --------------------
// x = g on fluid cells (0 elsewhere); the residual kernel then gives r0 = b - A g.
template <typename T>
__global__ void guess_load_kernel(LGeom g, SegArg seg, const T* __restrict__ guess, const double* __restrict__ diag,
                                  double* __restrict__ x) {
    SEG_LOOP_BEGIN(seg, g)
    x[c] = diag[c] > 0.0 ? (double)guess[c] : 0.0;
    SEG_LOOP_END
}

// alpha = (g.b) / (g.A g) with A g = b - r0: the scaling of g that minimises |x - x*|_A, so the
// scaled guess is never further from the solution in that norm than zero is.
__global__ void guess_alpha_kernel(LGeom g, SegArg seg, const double* __restrict__ x, const double* __restrict__ b,
                                   const double* __restrict__ r, Scalars* s, double* partials, unsigned* counter) {
    double acc[2] = {0.0, 0.0};
    SEG_LOOP_BEGIN(seg, g)
    const double xc = x[c];
    acc[0] += xc * b[c];
    acc[1] += xc * (b[c] - r[c]);
    SEG_LOOP_END
    double tot[2];
    if (grid_sum<2>(acc, partials, counter, tot)) {
        const double a = (tot[1] > 0.0 && finite_d(tot[0]) && finite_d(tot[1])) ? tot[0] / tot[1] : 0.0;
        s->aux = a;
    }
}

// x = alpha g, r = b - alpha A g = (1 - alpha) b + alpha r0, |r|^2 and the stopping test.
__global__ void guess_scale_kernel(LGeom g, SegArg seg, double* __restrict__ x, float2* __restrict__ xs,
                                   const double* __restrict__ b, double* __restrict__ r, Scalars* s,
                                   double* partials, unsigned* counter) {
    const double a = s->aux;
    double acc[1] = {0.0};
    SEG_LOOP_BEGIN(seg, g)
    // a == 0 (a useless or non-finite guess): exactly the zero start, whatever g held
    const double xc = a != 0.0 ? a * x[c] : 0.0;
    x[c] = xc;
    if (xs) xs[c] = x_pair(xc, s->df_shift);
    const double rc = a != 0.0 ? (1.0 - a) * b[c] + a * r[c] : b[c];
    r[c] = rc;
    acc[0] += rc * rc;
    SEG_LOOP_END
    double tot[1];
    if (grid_sum<1>(acc, partials, counter, tot)) {
        s->rr = tot[0];
        if (!finite_d(tot[0])) {
            s->bad = 1;
            s->done = 1;
        } else {
            s->done = (s->bb == 0.0 || tot[0] < s->thresh) ? 1 : 0;
        }
    }
}

// FP64 paths taken by few cells, kept out of line: the compiler would otherwise predicate them
// into the common path, where each FP64 instruction costs an issue slot of the FP64 pipe (the
// bound of these kernels) on every cell, switched off or not.
__device__ __noinline__ float scale_fp64(double r, double inv) { return (float)(r * inv); }

// |r| and 1 / |r| from |r|^2
__device__ __noinline__ double2 scale_from_norm(double rr) {
    const double norm = sqrt(rr);
    return make_double2(norm, norm > 0.0 ? 1.0 / norm : 0.0);
}

__device__ __noinline__ double residual_cell_fp64(double bc, double d, double x0, float cxm, double vxm, float cxp,
                                                  double vxp, float cym, double xym, float cyp, double xyp,
                                                  float czm, double xzm, float czp, double xzp) {
    return bc - stencil7(d, x0, f2d(cxm), vxm, f2d(cxp), vxp, f2d(cym), xym, f2d(cyp), xyp, f2d(czm), xzm, f2d(czp),
                         xzp);
}

// mixed solver: inner system r32 = r64 2^-k with 2^k the power of two at or below |r64| (the
// scaling is exact both ways, and |r32| lies in [1, 2)), x32 = 0, inner thresholds.  The scale
// comes from the exponent bits of |r|^2: square roots and divisions in FP64 by every thread cost
// more FP64 issue than the cells' own work.  A cell's value is shifted by the exponent field and
// rounded to float by integer arithmetic (d_shift, d2f): the inner system of a system scaled by
// a power of two is the same floats.  A zero, subnormal or non-finite |r|^2 takes the scale
// 1 / |r| in FP64.  The inner relative tolerance is what the outer one still needs,
// halved, kept within [floor, 1/2] (FP32 cannot go much below 1e-4 reliably):
// tau = clamp(0.5 tol |b| / |r|, floor, 0.5).
__global__ void inner_init_kernel(LGeom g, SegArg seg, const double* __restrict__ r64, float* __restrict__ r32,
                                  float* __restrict__ x32, const Scalars* so, Scalars* si, double tol,
                                  double tau_floor, double* partials, unsigned* counter) {
    const double rr = so->rr;
    const unsigned long long rb = (unsigned long long)__double_as_longlong(rr);
    const int erb = (int)((rb >> 52) & 0x7ffu);
    const int k = (erb - 1023) >> 1;
    // every positive normal |r|^2 gives a shift within the doubles' range (|k| <= 511)
    const bool pow2 = rb != 0ull && (rb >> 63) == 0ull && erb != 0 && erb != 0x7ff;
    double norm, inv;
    if (pow2) {
        norm = __longlong_as_double((long long)(1023 + k) << 52);
        inv = 0.0;
    } else {
        const double2 ni = scale_from_norm(rr);
        norm = ni.x;
        inv = ni.y;
    }
    float part = 0.f;
    // four segments a warp per pass, their loads in flight together (one load a cell)
    const int lane = threadIdx.x & 31;
    const int wg = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
    const int nseg = *seg.count;
    constexpr int U = 4;
    for (int q0 = wg; q0 < nseg; q0 += U * nw) {
        int cc[U];
        bool lv[U];
        double rc[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int qs = q0 + u * nw;
            const int4 sd = qs < nseg ? seg.desc[qs] : make_int4(0, g.n0, 0, 0);
            cc[u] = sd.x + lane;
            lv[u] = qs < nseg && sd.y + lane < g.n0;
        }
#pragma unroll
        for (int u = 0; u < U; ++u) rc[u] = lv[u] ? r64[cc[u]] : 0.0;
#pragma unroll
        for (int u = 0; u < U; ++u) {
            if (!lv[u]) continue;
            // r 2^-k by the exponent field, then rounded to float: exact scaling, integer pipe
            const float v = pow2 ? d2f(d_shift(rc[u], -k)) : scale_fp64(rc[u], inv);
            r32[cc[u]] = v;
            x32[cc[u]] = 0.0f;
            part += v * v;
        }
    }
    double acc[1] = {(double)part};
    double tot[1];
    if (grid_sum<1>(acc, partials, counter, tot)) {
        const double want = rr > 0.0 ? 0.5 * tol * sqrt(so->bb / rr) : 0.5;
        const double tau = fmin(0.5, fmax(tau_floor, want));
        si->bb = tot[0];
        si->rr = tot[0];
        si->thresh = tau * tau * tot[0];
        si->norm = norm;
        si->iter = 0;
        si->bad = 0;
        si->fault = 0;
        si->beta = 0.0;
        si->done = (tot[0] == 0.0 || tot[0] < si->thresh) ? 1 : 0;
    }
}

// mixed solver: x64 += |r| * x32 (and its float pair)
__global__ void accumulate_kernel(LGeom g, SegArg seg, double* __restrict__ x64, float2* __restrict__ xs,
                                  const float* __restrict__ x32, const Scalars* si, const Scalars* so) {
    const double norm = si->norm;
    const int shift = so->df_shift;
    SEG_LOOP_BEGIN(seg, g)
    const double xn = __fma_rn(norm, f2d(x32[c]), x64[c]);
    x64[c] = xn;
    if (xs) xs[c] = x_pair(xn, shift);
    SEG_LOOP_END
}

// |r|^2 of a refinement residual into the scalars and the stopping test
__device__ __forceinline__ void residual_done(Scalars* s, double rr) {
    s->rr = rr;
    if (!finite_d(rr)) {
        s->bad = 1;
        s->done = 1;
    } else if (rr < s->thresh) {
        s->done = 1;
    }
}

// FP64 residual r = b - A x and |r|^2 (outer refinement step).
template <typename OT>
__global__ void __launch_bounds__(kSegThreads) residual_kernel(LGeom g, SegArg seg, SplitOp<OT> A,
                                                               const double* __restrict__ b,
                                                               const double* __restrict__ x, double* __restrict__ r,
                                                               Scalars* s, double* partials, unsigned* counter) {
    double acc[1] = {0.0};
    const SplitLoad<OT> recf{A};
    auto rawf = [&](int q, int, int, int) -> double { return x[q]; };
    auto valf = [](double raw, const Co<double>&) -> double { return raw; };
    SEG_LOOP_ALL_BEGIN(seg, g)
    const St7<double> st = gather7<double, false>(g, c, i, j, k, live, lane, recf, rawf, valf);
    if (live) {
        const double rc = d_positive(st.d) ? b[c] - apply7(st) : 0.0;
        r[c] = rc;
        acc[0] += rc * rc;
    }
    SEG_LOOP_END
    double tot[1];
    if (grid_sum<1>(acc, partials, counter, tot)) residual_done(s, tot[0]);
}

// The mixed solver's refinement residual r = b - A x and |r|^2 for FP32 fields, whose couplings
// are exact floats: double-float arithmetic on the FP32 pipe (el_df.cuh) in place of the FP64
// operations, which bound the FP64 kernel above (nine a cell, its FP64 pipe 86 % busy).  The
// iterate comes as float pairs (xs, written with x); b and the diagonal are split into pairs by
// integer arithmetic, b and the iterate shifted by the solve's power of two 2^df_shift (|b| near
// 1: the pairs' exponent range then holds the system at any scale, and the shift is undone
// exactly on r and |r|^2); the pair of r is
// within 2^-41 of the sum of its row's term magnitudes, and is stored as a double.  A warp in
// which any operand lies outside the pairs' exponent range (el_df.cuh) takes the FP64
// arithmetic of the kernel above for all its lanes (the splits of b and the diagonal decide).  |r|^2 is summed in FP32 per thread (each
// takes a few dozen cells; SqAcc keeps every square in range) and in FP64 over the grid.
__global__ void __launch_bounds__(kSegThreads, 4) residual_df_kernel(LGeom g, SegArg seg, SplitOp<float> A,
                                                                  const double* __restrict__ b,
                                                                  const double* __restrict__ x,
                                                                  const float2* __restrict__ xs,
                                                                  double* __restrict__ r, Scalars* s,
                                                                  double* partials, unsigned* counter) {
    SqAcc acc2;
    // the pairs hold b and x times 2^k (x_pair); the residual pair is r 2^k, shifted back
    const int sk = s->df_shift;
    SEG_LOOP_ALL_BEGIN(seg, g)
    const bool iym = live && j > 0, iyp = live && j < g.n1 - 1;
    const bool izm = live && k > 0, izp = live && k < g.n2 - 1;
    const bool ixm = lane == 0 && live && i > 0;
    const bool ixp = lane == 31 && live && i + 1 < g.n0;
    // loads, all issued before any value is formed
    const double d = live ? A.d[c] : 0.0;
    const double bc = live ? b[c] : 0.0;
    const float cxp = live ? A.x[c] : 0.f, cyp = live ? A.y[c] : 0.f, czp = live ? A.z[c] : 0.f;
    const float cym = iym ? A.y[c - g.s1] : 0.f, czm = izm ? A.z[c - g.s2] : 0.f;
    const float cxm_e = ixm ? A.x[c - 1] : 0.f;
    const float2 z2 = make_float2(0.f, 0.f);
    const float2 q0 = live ? xs[c] : z2;
    const float2 qym = iym ? xs[c - g.s1] : z2, qyp = iyp ? xs[c + g.s1] : z2;
    const float2 qzm = izm ? xs[c - g.s2] : z2, qzp = izp ? xs[c + g.s2] : z2;
    const float2 qxm_e = ixm ? xs[c - 1] : z2, qxp_e = ixp ? xs[c + 1] : z2;
    const bool act = live && d_positive(d);
    const bool xp_in = live && i + 1 < g.n0;
    const float cxm_s = __shfl_up_sync(kFull, cxp, 1);
    const float cxm = lane == 0 ? cxm_e : cxm_s;
    const F2 p0{q0.x, q0.y}, pym{qym.x, qym.y}, pyp{qyp.x, qyp.y}, pzm{qzm.x, qzm.y}, pzp{qzp.x, qzp.y};
    const F2 pxm_e{qxm_e.x, qxm_e.y}, pxp_e{qxp_e.x, qxp_e.y};
    bool ok = true;
    const F2 pd = df_split(d, ok), pb = df_split(d_shift(bc, sk), ok);
    F2 pxm, pxp;
    pxm.h = __shfl_up_sync(kFull, p0.h, 1);
    pxm.l = __shfl_up_sync(kFull, p0.l, 1);
    pxp.h = __shfl_down_sync(kFull, p0.h, 1);
    pxp.l = __shfl_down_sync(kFull, p0.l, 1);
    if (lane == 0) pxm = pxm_e;
    if (lane == 31) pxp = pxp_e;
    if (!xp_in) pxp = F2{0.f, 0.f};
    if (__all_sync(kFull, ok)) {
        if (act) {
            const F2 q = df_residual7(pb, pd, p0, cxm, pxm, cxp, pxp, cym, pym, cyp, pyp, czm, pzm, czp, pzp);
            r[c] = d_shift(__dadd_rn(f2d(q.h), f2d(q.l)), -sk);
            acc2.add(q.h);
        } else if (live) {
            r[c] = 0.0;
        }
    } else {
        // the FP64 arithmetic of residual_kernel, for every lane of the warp, on the double iterate
        const double x0 = live ? x[c] : 0.0;
        const double xym = iym ? x[c - g.s1] : 0.0, xyp = iyp ? x[c + g.s1] : 0.0;
        const double xzm = izm ? x[c - g.s2] : 0.0, xzp = izp ? x[c + g.s2] : 0.0;
        const double xxm_e = ixm ? x[c - 1] : 0.0, xxp_e = ixp ? x[c + 1] : 0.0;
        const double sxm = __shfl_up_sync(kFull, x0, 1), sxp = __shfl_down_sync(kFull, x0, 1);
        if (live) {
            const double vxm = lane == 0 ? xxm_e : sxm;
            const double vxp = xp_in ? (lane == 31 ? xxp_e : sxp) : 0.0;
            const double rc = act ? residual_cell_fp64(bc, d, x0, cxm, vxm, cxp, vxp, cym, xym, cyp, xyp, czm, xzm,
                                                       czp, xzp)
                                  : 0.0;
            r[c] = rc;
            acc2.add(d2f(d_shift(rc, sk)));
        }
    }
    SEG_LOOP_END
    double acc[1] = {acc2.value()};
    double tot[1];
    if (grid_sum<1>(acc, partials, counter, tot)) residual_done(s, d_shift(tot[0], -2 * sk));
}


// ---------------------------------------------------------------------------------------
// multigrid smoothing over the active segments of one level
//
// MODE 0: two sweeps from x = 0 (the first, omega b / D, formed on the fly)
// MODE 1: one sweep from x_in + P e (e = coarse correction, formed on the fly)
// MODE 2: one sweep from x_in.   DOT (finest level, last sweep): rz = b . x_out and beta.
enum { SM_ZERO2 = 0, SM_PROLONG = 1, SM_PLAIN = 2 };

// a / b inside the multigrid preconditioner: FP32 takes the fast division (within 2 ulp; the
// preconditioner only has to be a fixed symmetric operator, not correctly rounded), FP64 the
// exact one
template <typename V>
__device__ __forceinline__ V mg_div(V a, V b) {
    if constexpr (sizeof(V) == 4)
        return __fdividef(a, b);
    else
        return a / b;
}
enum { DOT_NONE = 0, DOT_INIT = 1, DOT_BETA = 2 };

// A value of an iterate or right-hand side.  COH: through L2 only (ld.global.cg), for arrays
// that other CTAs of the same launch wrote (the fused coarse cycle); a read-only-cache load
// would not see those writes.
template <bool COH, typename V>
__device__ __forceinline__ V ldv(const V* p, int q) {
    if constexpr (COH)
        return __ldcg(p + q);
    else
        return p[q];
}

// One smoothing sweep over the active segments of a level, warp wg of nw warps taking segments
// wg, wg + nw, ...; returns the thread's share of b.x when DOT is set.
// ZERO2: first sweep (formed on the fly) w1, this sweep w2; PROLONG: w1; PLAIN: w2
template <typename V, typename R, int MODE, int DOT, bool COH = false>
__device__ __forceinline__ DotAcc<V> smooth_segments(const LGeom& g, const SegArg& seg, const R* __restrict__ A,
                                                     const V* __restrict__ b, const V* __restrict__ x_in,
                                                     const LGeom& gc, const V* __restrict__ e, V* __restrict__ x_out,
                                                     int wg, int nw) {
    const V w_first = V(kSweep1);
    const V omega = V(MODE == SM_PROLONG ? kSweep1 : kSweep2);
    DotAcc<V> part = 0;
    const RecLoad<V, R> recf{A};
    // value of the current iterate at a cell, zero on inactive cells
    auto rawf = [&](int q, int qi, int qj, int qk) -> V {
        if (MODE == SM_ZERO2) return ldv<COH>(b, q);
        V v = ldv<COH>(x_in, q);
        if (MODE == SM_PROLONG) v += ldv<COH>(e, (qi >> 1) + gc.s1 * (qj >> 1) + gc.s2 * (qk >> 1));
        return v;
    };
    auto valf = [&](V raw, const Co<V>& rec) -> V {
        if (!(rec.d > V(0))) return V(0);
        return MODE == SM_ZERO2 ? mg_div(rn_mul(w_first, raw), rec.d) : raw;
    };
    SEG_LOOP_ALL_W_BEGIN(seg, g, wg, nw)
    const St7<V> st = gather7<V, true>(g, c, i, j, k, live, lane, recf, rawf, valf);
    if (live) {
        const V bc = ldv<COH>(b, c);
        V xo = V(0);
        if (st.d > V(0)) xo = rn_add(st.v0, mg_div(rn_mul(omega, rn_sub(bc, apply7(st))), st.d));
        if (EL_IN(c, (long long)g.s2 * g.n2, 30)) x_out[c] = xo;
        if (DOT != DOT_NONE) part += (DotAcc<V>)bc * (DotAcc<V>)xo;
    }
    SEG_LOOP_END
    return part;
}

template <typename V, typename R, int MODE, int DOT>
__global__ void __launch_bounds__(kSegThreads) smooth_kernel(LGeom g, SegArg seg, const R* __restrict__ A,
                                                             const V* __restrict__ b, const V* __restrict__ x_in,
                                                             LGeom gc, const V* __restrict__ e,
                                                             V* __restrict__ x_out, Scalars* s, double* partials,
                                                             unsigned* counter) {
    pdl_wait();
    pdl_trigger();
    if (s->done) return;
    const DotAcc<V> part = smooth_segments<V, R, MODE, DOT>(g, seg, A, b, x_in, gc, e, x_out,
                                                            (blockIdx.x * blockDim.x + threadIdx.x) >> 5,
                                                            (gridDim.x * blockDim.x) >> 5);
    if (DOT != DOT_NONE) {
        double acc[1] = {(double)part};
        double tot[1];
        if (grid_sum<1>(acc, partials, counter, tot)) {
            if (DOT == DOT_BETA) s->beta = tot[0] / s->rz;
            s->rz = tot[0];
            if (!finite_d(tot[0])) {
                s->bad = 1;
                s->done = 1;
            }
        }
    }
}

// Residual of a level summed onto the coarse right-hand side (R = P^T), one warp per active
// coarse segment: the warp walks the 64 x 2 x 2 fine cells under it one fine row segment at a
// time (one fine cell per lane, coalesced), the i-pairs are summed by shuffle.  Used from the
// finest level, where the grid of warps is capped well below the number of coarse segments.
template <typename V, typename R>
__global__ void __launch_bounds__(kSegThreads, sizeof(V) == 4 ? 5 : 4) restrict_kernel(LGeom g, const R* __restrict__ A, const V* __restrict__ b,
                                                               const V* __restrict__ x, LGeom gc, SegArg cseg,
                                                               V* __restrict__ bc, const Scalars* s) {
    if (s->done) return;
    const RecLoad<V, R> recf{A};
    auto rawf = [&](int q, int, int, int) -> V { return x[q]; };
    auto valf = [](V raw, const Co<V>&) -> V { return raw; };
    const int lane = threadIdx.x & 31;
    const int warp_global = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    const int nseg = *cseg.count;
    for (int qs = warp_global; qs < nseg; qs += nwarps) {
        const int4 sd = cseg.desc[qs];
        const int I0 = sd.y, J = sd.z, K = sd.w;
        V sum[2] = {V(0), V(0)};  // fine i in [2*I0, 2*I0+32) and [2*I0+32, 2*I0+64)
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int i = 2 * I0 + 32 * h + lane;
#pragma unroll
            for (int kk = 0; kk < 2; ++kk)
#pragma unroll
                for (int jj = 0; jj < 2; ++jj) {
                    const int j = 2 * J + jj, k = 2 * K + kk;
                    // warp-uniform: the row exists for all lanes or for none
                    if (j >= g.n1 || k >= g.n2) continue;
                    const bool live = i < g.n0;
                    const int c = i + g.s1 * j + g.s2 * k;
                    const St7<V> st = gather7<V, false>(g, c, i, j, k, live, lane, recf, rawf, valf);
                    if (live && st.d > V(0)) sum[h] += rn_sub(b[c], apply7(st));
                }
        }
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const V pair = sum[h] + __shfl_down_sync(kFull, sum[h], 1);
            const int I = I0 + 16 * h + (lane >> 1);
            if ((lane & 1) == 0 && I < gc.n0 && EL_IN(I + gc.s1 * J + gc.s2 * K, (long long)gc.s2 * gc.n2, 31))
                bc[I + gc.s1 * J + gc.s2 * K] = pair;
        }
    }
}

// The same below the finest level, where the coarse segments are few: a quad of four
// warps takes one active coarse segment: warp (kk, jj) of the quad walks the fine row
// (2J + jj, 2K + kk) under it, 64 fine cells as two 32-cell halves (one fine cell per lane,
// coalesced), and sums the i-pairs by shuffle; the quad then adds its four rows in a fixed order
// through shared memory (deterministic).  Four rows in flight per coarse segment instead of
// eight gathers in sequence: the kernel is bound by the latency of the gathers.
constexpr int kQuadsPerBlock = kSegThreads / 128;

// The quads' walk: quad `quad` of `nquads`, the block's quad quad_b (named barrier 1 + quad_b),
// row `sub` of it; part = the block's [quads][4][2][16] sums in shared memory.
template <typename V, typename R, bool COH = false>
__device__ __forceinline__ void restrict_quad_segments(const LGeom& g, const R* __restrict__ A,
                                                       const V* __restrict__ b, const V* __restrict__ x,
                                                       const LGeom& gc, const SegArg& cseg, V* __restrict__ bc,
                                                       V (*part)[4][2][16], int quad, int nquads, int quad_b,
                                                       int sub) {
    const RecLoad<V, R> recf{A};
    auto rawf = [&](int q, int, int, int) -> V { return ldv<COH>(x, q); };
    auto valf = [](V raw, const Co<V>&) -> V { return raw; };
    const int lane = threadIdx.x & 31;
    const int kk = sub >> 1, jj = sub & 1;
    const int nseg = *cseg.count;
    for (int qs = quad; qs < nseg; qs += nquads) {
        const int4 sd = cseg.desc[qs];
        const int I0 = sd.y, J = sd.z, K = sd.w;
        const int j = 2 * J + jj, k = 2 * K + kk;
        V sum[2] = {V(0), V(0)};  // fine i in [2*I0, 2*I0+32) and [2*I0+32, 2*I0+64)
        // warp-uniform: the row exists for all lanes or for none
        if (j < g.n1 && k < g.n2) {
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int i = 2 * I0 + 32 * h + lane;
                const bool live = i < g.n0;
                const int c = i + g.s1 * j + g.s2 * k;
                const St7<V> st = gather7<V, false>(g, c, i, j, k, live, lane, recf, rawf, valf);
                if (live && st.d > V(0)) sum[h] = rn_sub(ldv<COH>(b, c), apply7(st));
            }
        }
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const V pair = sum[h] + __shfl_down_sync(kFull, sum[h], 1);
            if ((lane & 1) == 0) part[quad_b][sub][h][lane >> 1] = pair;
        }
        // the quad's four warps meet on their own named barrier (1 + quad in the block)
        asm volatile("bar.sync %0, %1;" ::"r"(1 + quad_b), "r"(128) : "memory");
        if (sub == 0) {
            const int h = lane >> 4, q = lane & 15;
            const V tot = ((part[quad_b][0][h][q] + part[quad_b][1][h][q]) + part[quad_b][2][h][q]) +
                          part[quad_b][3][h][q];
            const int I = I0 + 16 * h + q;
            if (I < gc.n0 && EL_IN(I + gc.s1 * J + gc.s2 * K, (long long)gc.s2 * gc.n2, 32))
                bc[I + gc.s1 * J + gc.s2 * K] = tot;
        }
        asm volatile("bar.sync %0, %1;" ::"r"(1 + quad_b), "r"(128) : "memory");
    }
}

template <typename V, typename R>
__global__ void __launch_bounds__(kSegThreads, 4) restrict_quad_kernel(LGeom g, const R* __restrict__ A,
                                                                    const V* __restrict__ b, const V* __restrict__ x,
                                                                    LGeom gc, SegArg cseg, V* __restrict__ bc,
                                                                    const Scalars* s) {
    pdl_wait();
    pdl_trigger();
    if (s->done) return;
    __shared__ V part[kQuadsPerBlock][4][2][16];
    const int wb = threadIdx.x >> 5;                  // warp in the block
    const int quad_b = wb >> 2, sub = wb & 3;         // quad in the block, row of the quad
    restrict_quad_segments<V, R>(g, A, b, x, gc, cseg, bc, part, blockIdx.x * kQuadsPerBlock + quad_b,
                                 gridDim.x * kQuadsPerBlock, quad_b, sub);
}


// Coarsest level: omega-Jacobi sweeps from zero in one block's shared memory.
template <typename V, typename R>
__global__ void __launch_bounds__(kCoarsestMaxCells) coarsest_kernel(LGeom g, const R* __restrict__ A,
                                                                     const V* __restrict__ b, V* __restrict__ x,
                                                                     int sweeps, const Scalars* s) {
    if (s->done) return;
    __shared__ V sd[kCoarsestMaxCells], sx[kCoarsestMaxCells], sy[kCoarsestMaxCells], sz[kCoarsestMaxCells];
    __shared__ V sb[kCoarsestMaxCells], xa[kCoarsestMaxCells], xb[kCoarsestMaxCells];
    const int n = g.n0 * g.n1 * g.n2;
    const int c = threadIdx.x;
    const V omega = V(kOmega);
    if (c < n) {
        const auto r = ldrec(A, c);
        sd[c] = (V)r.d;
        sx[c] = (V)r.x;
        sy[c] = (V)r.y;
        sz[c] = (V)r.z;
        sb[c] = b[c];
        xa[c] = sd[c] > V(0) ? mg_div(rn_mul(omega, sb[c]), sd[c]) : V(0);
    }
    __syncthreads();
    const int i = c % g.n0, j = (c / g.n0) % g.n1, k = c / (g.n0 * g.n1);
    const int s1 = g.n0, s2 = g.n0 * g.n1;
    V* cur = xa;
    V* nxt = xb;
    for (int it = 1; it < sweeps; ++it) {
        if (c < n) {
            V xo = V(0);
            const V d = sd[c];
            if (d > V(0)) {
                V a = rn_mul(d, cur[c]);
                if (i > 0) a = rn_fma(sx[c - 1], cur[c - 1], a);
                if (i < g.n0 - 1) a = rn_fma(sx[c], cur[c + 1], a);
                if (j > 0) a = rn_fma(sy[c - s1], cur[c - s1], a);
                if (j < g.n1 - 1) a = rn_fma(sy[c], cur[c + s1], a);
                if (k > 0) a = rn_fma(sz[c - s2], cur[c - s2], a);
                if (k < g.n2 - 1) a = rn_fma(sz[c], cur[c + s2], a);
                xo = rn_add(cur[c], mg_div(rn_mul(omega, rn_sub(sb[c], a)), d));
            }
            nxt[c] = xo;
        }
        __syncthreads();
        V* t = cur;
        cur = nxt;
        nxt = t;
    }
    if (c < n) x[c] = cur[c];
}

// ---------------------------------------------------------------------------------------
// The bottom of the FP32 V-cycle in one CTA.  Coarsening stops once the largest dimension is
// at most 8, so the level above the coarsest holds at most 16^3 = 4096 cells: that level and
// the coarsest fit in one CTA's shared memory (126 KB with float4 records).  One launch of 1024
// threads does what the segment kernels do in five: the two sweeps from zero, the restriction,
// the coarsest level's 30 sweeps, the prolongation sweep and the last sweep -- the same
// expressions in the same order, over the dense level (cells with no diagonal come out 0, as
// they contribute nothing to their neighbours), with barriers between the passes instead of
// kernel boundaries.  Only the level's final x goes back to global memory (the finer level's
// prolongation reads it).
constexpr int kBottomMaxCells = 4096;
constexpr int kBottomThreads = 1024;
// Each thread owns fixed cells: on the level, (i, j) = (t mod 16, t / 16 mod 16) and the planes
// k = t / 256 + 4 m, m = 0..3 (the level is at most 16 cells a side: its coarse level is at
// most 8); on the coarsest, thread t < 512 owns (t mod 8, t / 8 mod 8, t / 64).  No index is
// divided at run time, and the coarsest cell's record stays in registers across its sweeps.
constexpr int kBottomDim = 16, kBottomPlanes = kBottomThreads / (kBottomDim * kBottomDim);
constexpr int kBottomCells = kBottomDim / kBottomPlanes;  // cells per thread on the level

// neighbour bits of a cell: 1 -x, 2 +x, 4 -y, 8 +y, 16 -z, 32 +z inside the level
__device__ __forceinline__ unsigned inside_bits(int i, int j, int k, const LGeom& g) {
    return (i > 0 ? 1u : 0u) | (i < g.n0 - 1 ? 2u : 0u) | (j > 0 ? 4u : 0u) | (j < g.n1 - 1 ? 8u : 0u) |
           (k > 0 ? 16u : 0u) | (k < g.n2 - 1 ? 32u : 0u);
}

// the 7-point stencil of cell c of a dense level held in shared memory (float4 records); a
// neighbour outside the level gives coupling and value 0
__device__ __forceinline__ St7<float> dense_st7(const float4* rec, const float* v, int c, unsigned in,
                                                const LGeom& g) {
    St7<float> st;
    const float4 r0 = rec[c];
    st.d = r0.x;
    st.cxp = r0.y;
    st.cyp = r0.z;
    st.czp = r0.w;
    st.cxm = (in & 1u) ? rec[c - 1].y : 0.f;
    st.cym = (in & 4u) ? rec[c - g.s1].z : 0.f;
    st.czm = (in & 16u) ? rec[c - g.s2].w : 0.f;
    st.v0 = v[c];
    st.vxm = (in & 1u) ? v[c - 1] : 0.f;
    st.vxp = (in & 2u) ? v[c + 1] : 0.f;
    st.vym = (in & 4u) ? v[c - g.s1] : 0.f;
    st.vyp = (in & 8u) ? v[c + g.s1] : 0.f;
    st.vzm = (in & 16u) ? v[c - g.s2] : 0.f;
    st.vzp = (in & 32u) ? v[c + g.s2] : 0.f;
    return st;
}

constexpr int bottom_smem_bytes() {
    return kBottomMaxCells * (int)(sizeof(float4) + 3 * sizeof(float)) +
           kCoarsestMaxCells * (int)(sizeof(float4) + 3 * sizeof(float));
}

// the bottom's passes by one CTA of kBottomThreads threads, staged in bottom_smem
__device__ __forceinline__ void bottom_cycle(const LGeom& gf, const float4* __restrict__ recf,
                                             const float* __restrict__ bf, float* __restrict__ xf, const LGeom& gc,
                                             const float4* __restrict__ recc, int sweeps,
                                             unsigned char* bottom_smem) {
    float4* sr = reinterpret_cast<float4*>(bottom_smem);
    float* sb = reinterpret_cast<float*>(sr + kBottomMaxCells);
    float* s1 = sb + kBottomMaxCells;
    float* s2 = s1 + kBottomMaxCells;
    float4* cr = reinterpret_cast<float4*>(s2 + kBottomMaxCells);
    float* c1 = reinterpret_cast<float*>(cr + kCoarsestMaxCells);
    float* c2 = c1 + kCoarsestMaxCells;
    const float omega = (float)kOmega;  // the coarsest level's sweeps
    const float w1 = (float)kSweep1, w2 = (float)kSweep2;
    const int nf = gf.n0 * gf.n1 * gf.n2, nc = gc.n0 * gc.n1 * gc.n2;
    const int tid = threadIdx.x;
    // this thread's cells of the level: index (-1: none) and neighbour bits
    const int fi = tid & (kBottomDim - 1), fj = (tid / kBottomDim) & (kBottomDim - 1);
    const int fk0 = tid / (kBottomDim * kBottomDim);
    int fc[kBottomCells];
    unsigned fin[kBottomCells];
#pragma unroll
    for (int m = 0; m < kBottomCells; ++m) {
        const int k = fk0 + kBottomPlanes * m;
        const bool live = fi < gf.n0 && fj < gf.n1 && k < gf.n2;
        fc[m] = live ? fi + gf.s1 * fj + gf.s2 * k : -1;
        fin[m] = live ? inside_bits(fi, fj, k, gf) : 0u;
    }
    // this thread's cell of the coarsest level
    const int ci = tid & 7, cj = (tid >> 3) & 7, ck = tid >> 6;
    const bool clive = tid < kCoarsestMaxCells && ci < gc.n0 && cj < gc.n1 && ck < gc.n2;
    const int cq = clive ? ci + gc.s1 * cj + gc.s2 * ck : 0;
    for (int c = tid; c < nf; c += kBottomThreads) {
        sr[c] = recf[c];
        sb[c] = __ldcg(bf + c);  // written by other CTAs of the fused coarse cycle
    }
    for (int c = tid; c < nc; c += kBottomThreads) cr[c] = recc[c];
    __syncthreads();
    // two sweeps from zero: the first is pointwise
#pragma unroll
    for (int m = 0; m < kBottomCells; ++m) {
        const int c = fc[m];
        if (c < 0) continue;
        const float d = sr[c].x;
        s1[c] = d > 0.f ? mg_div(rn_mul(w1, sb[c]), d) : 0.f;
    }
    __syncthreads();
#pragma unroll
    for (int m = 0; m < kBottomCells; ++m) {
        const int c = fc[m];
        if (c < 0) continue;
        const St7<float> st = dense_st7(sr, s1, c, fin[m], gf);
        float xo = 0.f;
        if (st.d > 0.f) xo = rn_add(st.v0, mg_div(rn_mul(w2, rn_sub(sb[c], apply7(st))), st.d));
        s2[c] = xo;
    }
    __syncthreads();
    // residual, then its 2 x 2 x 2 sums onto the coarsest level (order of the segment kernels:
    // i-pairs of the rows (jj, kk) = (0,0), (1,0), (0,1), (1,1), summed in that order)
#pragma unroll
    for (int m = 0; m < kBottomCells; ++m) {
        const int c = fc[m];
        if (c < 0) continue;
        const St7<float> st = dense_st7(sr, s2, c, fin[m], gf);
        s1[c] = st.d > 0.f ? rn_sub(sb[c], apply7(st)) : 0.f;
    }
    __syncthreads();
    // the coarsest cell's record, rhs and neighbour bits in registers for all its sweeps
    float cbq = 0.f, cd = 0.f, cxm = 0.f, cxp = 0.f, cym = 0.f, cyp = 0.f, czm = 0.f, czp = 0.f;
    unsigned cin = 0u;
    if (clive) {
        auto res = [&](int i, int j, int k) -> float {
            return (i < gf.n0 && j < gf.n1 && k < gf.n2) ? s1[i + gf.s1 * j + gf.s2 * k] : 0.f;
        };
        float part[4];
#pragma unroll
        for (int sub = 0; sub < 4; ++sub) {
            const int jj = sub & 1, kk = sub >> 1;
            part[sub] = res(2 * ci, 2 * cj + jj, 2 * ck + kk) + res(2 * ci + 1, 2 * cj + jj, 2 * ck + kk);
        }
        cbq = ((part[0] + part[1]) + part[2]) + part[3];
        cin = inside_bits(ci, cj, ck, gc);
        const float4 r = cr[cq];
        cd = r.x;
        cxp = r.y;
        cyp = r.z;
        czp = r.w;
        if (cin & 1u) cxm = cr[cq - 1].y;
        if (cin & 4u) cym = cr[cq - gc.s1].z;
        if (cin & 16u) czm = cr[cq - gc.s2].w;
        // the coarsest level: damped Jacobi from zero, as coarsest_kernel
        c1[cq] = cd > 0.f ? mg_div(rn_mul(omega, cbq), cd) : 0.f;
    }
    __syncthreads();
    float* cur = c1;
    float* nxt = c2;
    for (int it = 1; it < sweeps; ++it) {
        if (clive) {
            float xo = 0.f;
            if (cd > 0.f) {
                const float x0 = cur[cq];
                float a = rn_mul(cd, x0);
                if (cin & 1u) a = rn_fma(cxm, cur[cq - 1], a);
                if (cin & 2u) a = rn_fma(cxp, cur[cq + 1], a);
                if (cin & 4u) a = rn_fma(cym, cur[cq - gc.s1], a);
                if (cin & 8u) a = rn_fma(cyp, cur[cq + gc.s1], a);
                if (cin & 16u) a = rn_fma(czm, cur[cq - gc.s2], a);
                if (cin & 32u) a = rn_fma(czp, cur[cq + gc.s2], a);
                xo = rn_add(x0, mg_div(rn_mul(omega, rn_sub(cbq, a)), cd));
            }
            nxt[cq] = xo;
        }
        __syncthreads();
        float* t = cur;
        cur = nxt;
        nxt = t;
    }
    // prolongation (x + P e) and a sweep, then the last sweep into global memory
#pragma unroll
    for (int m = 0; m < kBottomCells; ++m) {
        const int c = fc[m];
        if (c < 0) continue;
        const int k = fk0 + kBottomPlanes * m;
        s1[c] = s2[c] + cur[(fi >> 1) + gc.s1 * (fj >> 1) + gc.s2 * (k >> 1)];
    }
    __syncthreads();
#pragma unroll
    for (int m = 0; m < kBottomCells; ++m) {
        const int c = fc[m];
        if (c < 0) continue;
        const St7<float> st = dense_st7(sr, s1, c, fin[m], gf);
        float xo = 0.f;
        if (st.d > 0.f) xo = rn_add(st.v0, mg_div(rn_mul(w1, rn_sub(sb[c], apply7(st))), st.d));
        s2[c] = xo;
    }
    __syncthreads();
#pragma unroll
    for (int m = 0; m < kBottomCells; ++m) {
        const int c = fc[m];
        if (c < 0) continue;
        const St7<float> st = dense_st7(sr, s2, c, fin[m], gf);
        float xo = 0.f;
        if (st.d > 0.f) xo = rn_add(st.v0, mg_div(rn_mul(w2, rn_sub(sb[c], apply7(st))), st.d));
        xf[c] = xo;
    }
}

__global__ void __launch_bounds__(kBottomThreads) mg_bottom_kernel(LGeom gf, const float4* __restrict__ recf,
                                                                   const float* __restrict__ bf,
                                                                   float* __restrict__ xf, LGeom gc,
                                                                   const float4* __restrict__ recc, int sweeps,
                                                                   const Scalars* s) {
    pdl_wait();
    pdl_trigger();
    if (s->done) return;
    extern __shared__ __align__(16) unsigned char bottom_smem[];
    bottom_cycle(gf, recf, bf, xf, gc, recc, sweeps, bottom_smem);
}

// ---------------------------------------------------------------------------------------
// The coarse levels of one FP32 V-cycle in one cooperative launch.  Below the finest level the
// segment kernels are launches of a few microseconds each (about 13 per V-cycle at 256^3:
// two sweeps from zero and the restriction per level going down, the bottom, the prolongation
// sweep and the last sweep per level coming up), so the V-cycle's coarse part was bound by
// launch latency.  Here one launch of 1024-thread CTAs, all resident at once (a cooperative
// launch), runs the same passes -- the same device functions, so the same expressions in the
// same order and bit-identical results -- separated by grid barriers; the bottom pair (<= 16^3
// and the coarsest level) runs in CTA 0's shared memory while the others wait at the next
// barrier.  Arrays written by one pass and read by another are loaded through L2
// (ld.global.cg).  Every barrier wait is bounded: a CTA that gives up marks the solve as failed
// (fault, bad, done) and leaves; the other CTAs' waits then run out too.
constexpr int kCoarseMaxLevels = 16;
constexpr int kCoopQuads = kBottomThreads / 128;  // restriction quads per CTA
constexpr long long kBarrierPolls = 1ll << 21;    // past the first 4096, each poll sleeps ~100 ns: ~0.2 s

struct CoarseLevel {
    LGeom g;
    const float4* rec;
    float* b;
    float* x;
    float* t;
    SegArg seg;
};

struct CoarseCycle {
    CoarseLevel lv[kCoarseMaxLevels];  // by hierarchy level
    int from, pre_end;                 // levels [from, pre_end) go down and up; pre_end, pre_end + 1: bottom
    int sweeps;                        // coarsest-level sweeps
    unsigned* bar;                     // grid barrier: arrivals, generation (arrivals 0 before a launch)
};

__device__ __forceinline__ unsigned ld_acquire_gpu(const unsigned* p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// all CTAs of the launch meet; false when this CTA's wait ran out
__device__ __forceinline__ bool coarse_grid_barrier(unsigned* bar, unsigned nblocks) {
    __shared__ int ok_s;
    __syncthreads();
    if (threadIdx.x == 0) {
        int ok = 1;
        const unsigned gen = ld_acquire_gpu(bar + 1);  // cannot advance before this CTA arrives
        __threadfence();
        if (atomicAdd(bar, 1u) == nblocks - 1) {
            atomicExch(bar, 0u);
            __threadfence();
            atomicAdd(bar + 1, 1u);
        } else {
            long long n = 0;
            while (ld_acquire_gpu(bar + 1) == gen) {
                if (++n > kBarrierPolls) {
                    ok = 0;
                    break;
                }
                if (n > 4096) __nanosleep(100);  // a tight poll first: the others are usually close
            }
        }
        __threadfence();
        ok_s = ok;
    }
    __syncthreads();
    return ok_s != 0;
}

__global__ void __launch_bounds__(kBottomThreads, 1) mg_coarse_cycle_kernel(const __grid_constant__ CoarseCycle a,
                                                                            Scalars* s) {
    if (s->done) return;  // read by every CTA before any can change it: all leave, or none
    extern __shared__ __align__(16) unsigned char bottom_smem[];
    __shared__ float part[kCoopQuads][4][2][16];
    const unsigned nblk = gridDim.x;
    const int wg = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
    const int wb = threadIdx.x >> 5, quad_b = wb >> 2, sub = wb & 3;
    const int quad = blockIdx.x * kCoopQuads + quad_b, nquads = gridDim.x * kCoopQuads;
    auto fail = [&]() {
        if (threadIdx.x == 0) {
            s->fault = 1;
            s->bad = 1;
            s->done = 1;
        }
    };
    for (int l = a.from; l < a.pre_end; ++l) {
        const CoarseLevel& F = a.lv[l];
        const CoarseLevel& C = a.lv[l + 1];
        smooth_segments<float, float4, SM_ZERO2, DOT_NONE, true>(F.g, F.seg, F.rec, F.b, nullptr, F.g, nullptr, F.x,
                                                                 wg, nw);
        if (!coarse_grid_barrier(a.bar, nblk)) return fail();
        restrict_quad_segments<float, float4, true>(F.g, F.rec, F.b, F.x, C.g, C.seg, C.b, part, quad, nquads,
                                                    quad_b, sub);
        if (!coarse_grid_barrier(a.bar, nblk)) return fail();
    }
    if (blockIdx.x == 0) {
        const CoarseLevel& F = a.lv[a.pre_end];
        const CoarseLevel& C = a.lv[a.pre_end + 1];
        bottom_cycle(F.g, F.rec, F.b, F.x, C.g, C.rec, a.sweeps, bottom_smem);
    }
    for (int l = a.pre_end - 1; l >= a.from; --l) {
        const CoarseLevel& F = a.lv[l];
        const CoarseLevel& C = a.lv[l + 1];
        if (!coarse_grid_barrier(a.bar, nblk)) return fail();
        smooth_segments<float, float4, SM_PROLONG, DOT_NONE, true>(F.g, F.seg, F.rec, F.b, F.x, C.g, C.x, F.t, wg,
                                                                   nw);
        if (!coarse_grid_barrier(a.bar, nblk)) return fail();
        smooth_segments<float, float4, SM_PLAIN, DOT_NONE, true>(F.g, F.seg, F.rec, F.b, F.t, F.g, nullptr, F.x, wg,
                                                                 nw);
    }
}

// ---------------------------------------------------------------------------------------
// host side

static int seg_blocks(el_ctx* ctx, long long total_segments) {
    const long long warps = (long long)ctx->num_sms * ctx->seg_per_sm * (kSegThreads / 32);
    const long long need = std::max<long long>(1, std::min<long long>(total_segments, warps));
    return (int)((need * 32 + kSegThreads - 1) / kSegThreads);
}

static SegArg seg_arg(const SegList& l) { return SegArg{l.desc, l.count}; }

// The finest level's restriction is bound by the latency of its gathers: as many warps as can
// be resident (five CTAs of 256 threads per SM at its FP32 register budget), so that each walks a
// short chain of coarse segments.
static int restrict_blocks(el_ctx* ctx, long long total_segments) {
    const long long warps = (long long)ctx->num_sms * 5 * (kSegThreads / 32);
    const long long need = std::max<long long>(1, std::min<long long>(total_segments, warps));
    return (int)((need * 32 + kSegThreads - 1) / kSegThreads);
}

// Cells a segment kernel of multigrid level `level` visits (for the byte counts of profiled
// launches): the active segments' cells, as read back by record_active(), else `full`.
static double active_cells(const el_ctx* ctx, int level, double full) {
    if (level >= 0 && level < (int)ctx->prof_active.size() && ctx->prof_active[level] >= 0)
        return ctx->prof_active[level];
    return full;
}

// While profiling, reads back the active segment counts of the finest level (seg0) and of the
// coarse levels (one synchronisation per solve; not used outside profiling).
template <typename V>
static int record_active(el_ctx* ctx, const SegList& seg0, int n0, const std::vector<MGLevel<V>>* mg) {
    ctx->prof_active.clear();
    if (!ctx->prof_mask) return EL_OK;
    const size_t levels = mg ? mg->size() : 1;
    std::vector<int> counts(levels, 0);
    for (size_t l = 0; l < levels; ++l) {
        const int* c = l == 0 ? seg0.count : (*mg)[l].seg.count;
        EL_CUDA_TRY(ctx, cudaMemcpyAsync(&counts[l], c, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    }
    EL_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    for (size_t l = 0; l < levels; ++l) {
        const int w = l == 0 ? n0 : (*mg)[l].n0;
        ctx->prof_active.push_back((double)counts[l] * std::min(32, w));
    }
    return EL_OK;
}

static int alloc_seglist(el_ctx* ctx, SegList& l, int n0, int n1, int n2) {
    l.nsr = (n0 + 31) / 32;
    l.total = (long long)l.nsr * n1 * n2;
    const long long nchunks = (l.total + kSegChunk - 1) / kSegChunk;
    l.desc = (int4*)ctx_alloc(ctx, l.total * sizeof(int4));
    l.flags = (uint8_t*)ctx_alloc(ctx, l.total);
    l.chunk = (int*)ctx_alloc(ctx, (nchunks + 1) * sizeof(int));
    l.count = l.chunk + nchunks;
    return (l.desc && l.flags && l.chunk) ? EL_OK : set_error(ctx, EL_ERR_OUT_OF_MEMORY, "segment lists");
}

// compaction of the flags into the ordered id list
static int enqueue_compact(el_ctx* ctx, SegList& l, const LGeom& g) {
    const int nchunks = (int)((l.total + kSegChunk - 1) / kSegChunk);
    seg_count_kernel<<<nchunks, 256, 0, ctx->stream>>>(l.flags, l.total, l.chunk);
    seg_scan_kernel<<<1, 1024, 0, ctx->stream>>>(l.chunk, nchunks, l.count);
    seg_write_kernel<<<nchunks, 256, 0, ctx->stream>>>(g, l.flags, l.total, l.chunk, l.desc);
    return 3;
}

template <typename R>
static int enqueue_seglist_rec(el_ctx* ctx, SegList& l, const LGeom& g, const R* rec) {
    ProfScope prof(ctx, EL_KC_OTHER, (double)g.n0 * g.n1 * g.n2 * sizeof(R));
    seg_flags_rec_kernel<R><<<seg_blocks(ctx, l.total), kSegThreads, 0, ctx->stream>>>(g, rec, l.total, l.flags);
    return 1 + enqueue_compact(ctx, l, g);
}

static int grid1d(el_ctx* ctx, long long n) {
    return (int)std::max<long long>(1, std::min<long long>((n + 255) / 256, (long long)ctx->num_sms * ctx->stencil_per_sm));
}

// Hierarchy below the finest level (allocated once per context and solver precision).
template <typename V>
static int build_hierarchy(el_ctx* ctx, std::vector<MGLevel<V>>& mg, size_t coarse_rec_bytes) {
    mg.clear();
    MGLevel<V> L0;
    L0.n0 = ctx->ni;
    L0.n1 = ctx->nj;
    L0.n2 = ctx->nk;
    const long long n = (long long)ctx->ni * ctx->nj * ctx->nk;
    L0.t = (V*)ctx_alloc(ctx, n * sizeof(V));
    if (!L0.t) return set_error(ctx, EL_ERR_OUT_OF_MEMORY, "multigrid");
    mg.push_back(L0);
    while (std::max(mg.back().n0, std::max(mg.back().n1, mg.back().n2)) > kCoarsestMaxDim) {
        MGLevel<V> C;
        C.n0 = (mg.back().n0 + 1) / 2;
        C.n1 = (mg.back().n1 + 1) / 2;
        C.n2 = (mg.back().n2 + 1) / 2;
        const long long m = (long long)C.n0 * C.n1 * C.n2;
        C.rec = ctx_alloc(ctx, m * coarse_rec_bytes);
        C.b = (V*)ctx_alloc(ctx, m * sizeof(V));
        C.x = (V*)ctx_alloc(ctx, m * sizeof(V));
        C.t = (V*)ctx_alloc(ctx, m * sizeof(V));
        if (!C.rec || !C.b || !C.x || !C.t) return set_error(ctx, EL_ERR_OUT_OF_MEMORY, "multigrid");
        int rc = alloc_seglist(ctx, C.seg, C.n0, C.n1, C.n2);
        if (rc != EL_OK) return rc;
        mg.push_back(C);
    }
    return EL_OK;
}

// Coarse records and segment lists of every level below the finest.
template <typename V, typename R0, typename RC>
static int enqueue_coarsen(el_ctx* ctx, std::vector<MGLevel<V>>& mg) {
    int launched = 0;
    for (size_t l = 0; l + 1 < mg.size(); ++l) {
        const MGLevel<V>& F = mg[l];
        MGLevel<V>& C = mg[l + 1];
        const LGeom gf = make_geom(F.n0, F.n1, F.n2), gc = make_geom(C.n0, C.n1, C.n2);
        dim3 block(32, 4, 1);
        dim3 grid((C.n0 + 31) / 32, (C.n1 + 3) / 4, C.n2);
        {
            ProfScope prof(ctx, EL_KC_MG_COARSE, (double)F.n0 * F.n1 * F.n2 * (l == 0 ? sizeof(R0) : sizeof(RC)) +
                                                     (double)C.n0 * C.n1 * C.n2 * sizeof(RC));
            if (l == 0)
                coarsen_kernel<R0, RC><<<grid, block, 0, ctx->stream>>>(gf, (const R0*)F.rec, gc, (RC*)C.rec);
            else
                coarsen_kernel<RC, RC><<<grid, block, 0, ctx->stream>>>(gf, (const RC*)F.rec, gc, (RC*)C.rec);
        }
        launched += 1 + enqueue_seglist_rec<RC>(ctx, C.seg, gc, (const RC*)C.rec);
    }
    return launched;
}

template <typename V, typename R, int MODE, int DOT>
static void launch_smooth(el_ctx* ctx, const MGLevel<V>& F, const SegList& seg, const V* x_in, const MGLevel<V>* C,
                          V* x_out, Scalars* s) {
    const LGeom g = make_geom(F.n0, F.n1, F.n2);
    const LGeom gc = C ? make_geom(C->n0, C->n1, C->n2) : g;
    const int blocks = one_wave(ctx, smooth_kernel<V, R, MODE, DOT>, kSegThreads, seg_blocks(ctx, seg.total));
    launch_dependent(ctx, smooth_kernel<V, R, MODE, DOT>, dim3(blocks), dim3(kSegThreads), 0, g,
                     seg_arg(seg), (const R*)F.rec, (const V*)F.b, x_in, gc, C ? (const V*)C->x : (const V*)nullptr,
                     x_out, s, ctx->partials, ctx->counter);
}

// The coarse part of an FP32 V-cycle, levels [from, pre_end) and the bottom pair, as one
// cooperative launch of mg_coarse_cycle_kernel; the grid is one CTA per 32 rows of level
// `from` (a warp per row segment), at most every resident CTA.
static bool coarse_fused_usable(const el_ctx* ctx, int L) {
    return ctx->coarse_fused && ctx->coarse_per_sm > 0 && ctx->coarse_bar && L <= kCoarseMaxLevels;
}

static int coarse_cycle_grid(const el_ctx* ctx, const SegList& seg_from) {
    const long long cap = (long long)ctx->num_sms * ctx->coarse_per_sm;
    const long long want = (seg_from.total + kBottomThreads / 32 - 1) / (kBottomThreads / 32);
    return (int)std::max<long long>(1, std::min(cap, want));
}

static int launch_coarse_cycle(el_ctx* ctx, std::vector<MGLevel<float>>& mg, int from, int pre_end, Scalars* s) {
    CoarseCycle a{};
    for (int l = from; l <= pre_end + 1; ++l) {
        const MGLevel<float>& X = mg[l];
        a.lv[l] = CoarseLevel{make_geom(X.n0, X.n1, X.n2), (const float4*)X.rec, X.b, X.x, X.t, seg_arg(X.seg)};
    }
    a.from = from;
    a.pre_end = pre_end;
    a.sweeps = kCoarsestSweeps;
    a.bar = ctx->coarse_bar;
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(coarse_cycle_grid(ctx, mg[from].seg), 1, 1);
    cfg.blockDim = dim3(kBottomThreads, 1, 1);
    cfg.dynamicSmemBytes = bottom_smem_bytes();
    cfg.stream = ctx->stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, mg_coarse_cycle_kernel, a, s);
    return 1;
}

// z = M^-1 r with r = mg[0].b and z = mg[0].x; dot = DOT_INIT or DOT_BETA.  R0 / RC are the
// record types of the finest / coarse levels.  from > 0: the levels below `from` only (level
// from - 1 restricted onto mg[from].b before, and prolonged from mg[from].x after, by the caller).
template <typename V, typename R0, typename RC>
static int enqueue_vcycle(el_ctx* ctx, std::vector<MGLevel<V>>& mg, const SegList& seg0, Scalars* s, int dot,
                          int from = 0) {
    int launched = 0;
    const int L = (int)mg.size();
    auto segof = [&](int l) -> const SegList& { return l == 0 ? seg0 : mg[l].seg; };
    auto cells = [](const MGLevel<V>& X) { return (double)X.n0 * X.n1 * X.n2; };
    auto act = [&](int l, const MGLevel<V>& X) { return active_cells(ctx, l, cells(X)); };
    const double vs = sizeof(V);
    if (L == 1) {
        // too small to coarsen: the coarsest sweeps solve it, one more sweep gives the dot
        MGLevel<V>& C = mg[0];
        coarsest_kernel<V, R0><<<1, kCoarsestMaxCells, 0, ctx->stream>>>(make_geom(C.n0, C.n1, C.n2), (const R0*)C.rec,
                                                                         C.b, C.t, kCoarsestSweeps, s);
        if (dot == DOT_INIT)
            launch_smooth<V, R0, SM_PLAIN, DOT_INIT>(ctx, C, seg0, C.t, nullptr, C.x, s);
        else
            launch_smooth<V, R0, SM_PLAIN, DOT_BETA>(ctx, C, seg0, C.t, nullptr, C.x, s);
        return 2;
    }
    // the FP32 hierarchy's last two levels in one CTA (mg_bottom_kernel)
    constexpr bool kBottomType = std::is_same<V, float>::value && std::is_same<RC, float4>::value;
    const bool fused_bottom = kBottomType && L >= 3 && mg[L - 2].n0 <= kBottomDim && mg[L - 2].n1 <= kBottomDim &&
                              mg[L - 2].n2 <= kBottomDim && mg[L - 1].n0 <= 8 && mg[L - 1].n1 <= 8 &&
                              mg[L - 1].n2 <= 8;
    const int pre_end = fused_bottom ? L - 2 : L - 1;  // levels smoothed and restricted by the loops
    // levels [coop_from, pre_end) and the bottom in one cooperative launch (the FP32 hierarchy)
    int coop_from = -1;
    if constexpr (kBottomType)
        if (fused_bottom && coarse_fused_usable(ctx, L)) {
            // coarse_fused = 1: every level below the finest; 2: from the second one on (the
            // first, the largest, keeps its launches)
            const int c = std::max(from, ctx->coarse_fused);
            if (c < pre_end) coop_from = c;
        }
    const int down_end = coop_from >= 0 ? coop_from : pre_end;  // levels by per-level launches
    for (int l = from; l < down_end; ++l) {
        MGLevel<V>& F = mg[l];
        MGLevel<V>& C = mg[l + 1];
        const double rb = l == 0 ? sizeof(R0) : sizeof(RC);
        {
            // reads b and records; writes x
            ProfScope prof(ctx, l == 0 ? EL_KC_SMOOTH : EL_KC_MG_COARSE, act(l, F) * (2 * vs + rb));
            if (l == 0)
                launch_smooth<V, R0, SM_ZERO2, DOT_NONE>(ctx, F, segof(l), nullptr, nullptr, F.x, s);
            else
                launch_smooth<V, RC, SM_ZERO2, DOT_NONE>(ctx, F, segof(l), nullptr, nullptr, F.x, s);
        }
        {
            // reads b, x and records; writes the coarse b
            ProfScope prof(ctx, l == 0 ? EL_KC_RESTRICT : EL_KC_MG_COARSE, act(l, F) * (2 * vs + rb) + act(l + 1, C) * vs);
            const LGeom gf = make_geom(F.n0, F.n1, F.n2), gc = make_geom(C.n0, C.n1, C.n2);
            if (l == 0)
                restrict_kernel<V, R0><<<restrict_blocks(ctx, C.seg.total), kSegThreads, 0, ctx->stream>>>(
                    gf, (const R0*)F.rec, F.b, F.x, gc, seg_arg(C.seg), C.b, s);
            else
                launch_dependent(ctx, restrict_quad_kernel<V, RC>,
                                 dim3(one_wave(ctx, restrict_quad_kernel<V, RC>, kSegThreads,
                                               seg_blocks(ctx, 4 * C.seg.total))),
                                 dim3(kSegThreads), 0, gf, (const RC*)F.rec, (const V*)F.b, (const V*)F.x, gc,
                                 seg_arg(C.seg), C.b, (const Scalars*)s);
        }
        launched += 2;
    }
    if (coop_from >= 0) {
        if constexpr (kBottomType) {
            // reads and writes what the per-level launches and the bottom would
            double bytes = cells(mg[L - 2]) * (sizeof(RC) + 2 * vs) + cells(mg[L - 1]) * sizeof(RC);
            for (int l = coop_from; l < pre_end; ++l)
                bytes += act(l, mg[l]) * (2 * (2 * vs + sizeof(RC)) + 2 * (3 * vs + sizeof(RC))) +
                         act(l + 1, mg[l + 1]) * 2 * vs;
            ProfScope prof(ctx, EL_KC_MG_COARSE, bytes);
            launched += launch_coarse_cycle(ctx, mg, coop_from, pre_end, s);
        }
    } else if (fused_bottom) {
        if constexpr (kBottomType) {
            MGLevel<V>& F = mg[L - 2];
            MGLevel<V>& C = mg[L - 1];
            // reads the level's records and b and the coarsest records; writes the level's x
            ProfScope prof(ctx, EL_KC_MG_COARSE, cells(F) * (sizeof(RC) + 2 * vs) + cells(C) * sizeof(RC));
            launch_dependent(ctx, mg_bottom_kernel, dim3(1), dim3(kBottomThreads), bottom_smem_bytes(),
                             make_geom(F.n0, F.n1, F.n2), (const float4*)F.rec, (const float*)F.b, F.x,
                             make_geom(C.n0, C.n1, C.n2), (const float4*)C.rec, (int)kCoarsestSweeps,
                             (const Scalars*)s);
            ++launched;
        }
    } else {
        MGLevel<V>& C = mg[L - 1];
        ProfScope prof(ctx, EL_KC_MG_COARSE, cells(C) * (3 * vs + sizeof(RC)));
        coarsest_kernel<V, RC><<<1, kCoarsestMaxCells, 0, ctx->stream>>>(make_geom(C.n0, C.n1, C.n2), (const RC*)C.rec,
                                                                         C.b, C.x, kCoarsestSweeps, s);
        ++launched;
    }
    for (int l = down_end - 1; l >= from; --l) {
        MGLevel<V>& F = mg[l];
        MGLevel<V>& C = mg[l + 1];
        const double rb = l == 0 ? sizeof(R0) : sizeof(RC);
        const int cls = l == 0 ? EL_KC_SMOOTH : EL_KC_MG_COARSE;
        {
            // prolongation sweep: b, x, records, coarse x read, t written
            ProfScope prof(ctx, cls, act(l, F) * (3 * vs + rb) + act(l + 1, C) * vs);
            if (l == 0)
                launch_smooth<V, R0, SM_PROLONG, DOT_NONE>(ctx, F, segof(l), F.x, &C, F.t, s);
            else
                launch_smooth<V, RC, SM_PROLONG, DOT_NONE>(ctx, F, segof(l), F.x, &C, F.t, s);
        }
        {
            // last sweep: b, t, records read, x written
            ProfScope prof(ctx, cls, act(l, F) * (3 * vs + rb));
            if (l == 0 && dot == DOT_INIT)
                launch_smooth<V, R0, SM_PLAIN, DOT_INIT>(ctx, F, segof(l), F.t, nullptr, F.x, s);
            else if (l == 0)
                launch_smooth<V, R0, SM_PLAIN, DOT_BETA>(ctx, F, segof(l), F.t, nullptr, F.x, s);
            else
                launch_smooth<V, RC, SM_PLAIN, DOT_NONE>(ctx, F, segof(l), F.t, nullptr, F.x, s);
        }
        launched += 2;
    }
    return launched;
}

// The finest level of the FP32 V-cycle by the tile kernels (el_march.cu), from the pre-smoothed
// level on: restriction, the coarse levels (the segment kernels), prolongation sweep, last sweep
// with the dot product (dot = DOT_INIT or DOT_BETA).
static int enqueue_march_vcycle_rest(el_ctx* ctx, std::vector<MGLevel<float>>& mg, Scalars* s, int dot) {
    MGLevel<float>& F = mg[0];
    MGLevel<float>& C = mg[1];
    const double na = active_cells(ctx, 0, (double)F.n0 * F.n1 * F.n2);
    const double nc = active_cells(ctx, 1, (double)C.n0 * C.n1 * C.n2);
    int n = 0;
    {
        // reads x, b and half4 records; writes the coarse b
        ProfScope prof(ctx, EL_KC_RESTRICT, na * 16 + nc * 4);
        n += march_restrict(ctx, F.x, F.b, C.b, s);
    }
    n += enqueue_vcycle<float, ushort4, float4>(ctx, mg, ctx->seg0, s, DOT_NONE, 1);
    {
        // reads x, b, records and the coarse x; writes t
        ProfScope prof(ctx, EL_KC_SMOOTH, na * 20 + nc * 4);
        n += march_prolong(ctx, F.x, F.b, F.t, s);
    }
    {
        // reads t, b, records; writes x
        ProfScope prof(ctx, EL_KC_SMOOTH, na * 20);
        n += march_last(ctx, F.t, F.b, F.x, s, dot);
    }
    return n;
}

// z = M^-1 r by the tile kernels on the finest level (the V-cycle that opens a refinement sweep)
static int enqueue_march_vcycle(el_ctx* ctx, std::vector<MGLevel<float>>& mg, Scalars* s, int dot) {
    const double na = active_cells(ctx, 0, (double)mg[0].n0 * mg[0].n1 * mg[0].n2);
    int n = 0;
    {
        // reads b and records; writes x
        ProfScope prof(ctx, EL_KC_SMOOTH, na * 16);
        n += march_zero2(ctx, mg[0].b, mg[0].x, s);
    }
    return n + enqueue_march_vcycle_rest(ctx, mg, s, dot);
}

// One PCG iteration of the mixed solver's inner system with the finest level on the tile
// kernels: K1 (direction, A p, alpha), then the update fused with the pre-smoother (x, r out of
// place, |r|^2, z's first two sweeps), then the rest of the V-cycle.  The direction and the
// residual each alternate between two buffers; mg[0].b follows r.
static int enqueue_march_iteration(el_ctx* ctx, float*& p, float*& p_alt, float*& r, float*& r_alt, Scalars* s,
                                   int first, std::vector<MGLevel<float>>& mg) {
    const double na = active_cells(ctx, 0, (double)ctx->ni * ctx->nj * ctx->nk);
    int n = 0;
    {
        // reads z, p (not on the first iteration), float4 records; writes p, Ap
        ProfScope prof(ctx, EL_KC_DIR_SPMV, na * (4.0 * (first ? 3 : 4) + 16));
        n += march_dir_spmv(ctx, ctx->z32, p, p_alt, ctx->ap32, s, first);
    }
    std::swap(p, p_alt);
    {
        // reads r, Ap, x, p, half4 records; writes x, r, z
        ProfScope prof(ctx, EL_KC_UPDATE, na * 36);
        n += march_update_smooth(ctx, ctx->x32, p, r, r_alt, ctx->ap32, ctx->z32, s);
    }
    std::swap(r, r_alt);
    mg[0].b = r;
    return n + enqueue_march_vcycle_rest(ctx, mg, s, DOT_BETA);
}

static int poll(el_ctx* ctx, Scalars* host_copy, int which) {
    EL_CUDA_TRY(ctx, cudaMemcpyAsync(host_copy, ctx->dscal + which, sizeof(Scalars), cudaMemcpyDeviceToHost,
                                     ctx->stream));
    EL_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    return EL_OK;
}

// One PCG iteration of a multigrid-preconditioned solve (record operator A).
template <typename V, typename RA, typename R0, typename RC>
static int enqueue_mg_iteration(el_ctx* ctx, const RA* A, V* x, V* r, V* z, V*& p, V*& p_alt, V* ap, Scalars* s,
                                int first, std::vector<MGLevel<V>>& mg) {
    const LGeom g = make_geom(ctx->ni, ctx->nj, ctx->nk);
    const SegList& seg = ctx->seg0;
    const double N = active_cells(ctx, 0, (double)ctx->ni * ctx->nj * ctx->nk), vs = sizeof(V);
    {
        // reads z, p (not on the first iteration), records; writes p, Ap
        ProfScope prof(ctx, EL_KC_DIR_SPMV, N * (vs * (first ? 3 : 4) + sizeof(RA)));
        dir_spmv_rec_kernel<V, RA><<<seg_blocks(ctx, seg.total), kSegThreads, 0, ctx->stream>>>(
            g, seg_arg(seg), A, z, p, p_alt, ap, s, first, ctx->partials, ctx->counter);
    }
    std::swap(p, p_alt);
    {
        // reads x, r, p, Ap; writes x, r
        ProfScope prof(ctx, EL_KC_UPDATE, N * vs * 6);
        update_kernel<V, false><<<seg_blocks(ctx, seg.total), kSegThreads, 0, ctx->stream>>>(
            g, seg_arg(seg), nullptr, x, r, p, ap, s, ctx->partials, ctx->counter);
    }
    return 2 + enqueue_vcycle<V, R0, RC>(ctx, mg, seg, s, DOT_BETA);
}

template <typename OT>
static int enqueue_jacobi_iteration(el_ctx* ctx, const SplitOp<OT>& A, double*& p, double*& p_alt, Scalars* s,
                                    int first) {
    const LGeom g = make_geom(ctx->ni, ctx->nj, ctx->nk);
    const SegList& seg = ctx->seg0;
    const double N = active_cells(ctx, 0, (double)ctx->ni * ctx->nj * ctx->nk);
    {
        // reads r, p (not on the first iteration), diag, 3 couplings; writes p, Ap
        ProfScope prof(ctx, EL_KC_DIR_SPMV, N * (8.0 * (first ? 4 : 5) + 3 * sizeof(OT)));
        dir_spmv_jacobi_kernel<OT><<<seg_blocks(ctx, seg.total), kSegThreads, 0, ctx->stream>>>(
            g, seg_arg(seg), A, ctx->r64, p, p_alt, ctx->ap64, s, first, ctx->partials, ctx->counter);
    }
    std::swap(p, p_alt);
    {
        // reads x, r, p, Ap, diag; writes x, r
        ProfScope prof(ctx, EL_KC_UPDATE, N * 8.0 * 7);
        update_kernel<double, true><<<seg_blocks(ctx, seg.total), kSegThreads, 0, ctx->stream>>>(
            g, seg_arg(seg), A.d, ctx->x64, ctx->r64, p, ctx->ap64, s, ctx->partials, ctx->counter);
    }
    return 2;
}

// Launch PCG iterations (check_every per poll) until converged or `budget` are launched.
//
// The first iteration is launched directly; the following ones in batches of `check_every`
// (rounded up to even, so the two direction buffers are back in place after a batch).  A batch
// is captured once per context and solver as a CUDA graph and replayed afterwards: all its
// pointers and launch shapes are fixed per context, and the kernels read everything that
// changes (scalars, segment lists) from device memory.  While kernel classes are being
// profiled the batches are launched directly instead.
template <typename F>
static int run_iterations(el_ctx* ctx, int solver, int which, int budget, int check_every, Scalars* out,
                          F&& enqueue) {
    int launched_iters = 0;
    int st = poll(ctx, out, which);
    if (st != EL_OK) return st;
    if (out->done || budget <= 0) return EL_OK;
    ctx->launches += enqueue(1);
    launched_iters = 1;
    const int batch = std::max(2, (check_every + 1) / 2 * 2);
    const bool graphs = ctx->use_graphs && ctx->prof_mask == 0;
    if (graphs && ctx->iter_graph[solver] && ctx->iter_graph_len[solver] != batch) {
        cudaGraphExecDestroy(ctx->iter_graph[solver]);
        ctx->iter_graph[solver] = nullptr;
    }
    st = poll(ctx, out, which);
    if (st != EL_OK) return st;
    while (!out->done && launched_iters < budget) {
        // a full batch may run past the budget by up to batch - 1 iterations only when the
        // budget is not a multiple of it; the iteration count reported is the device's
        if (graphs && budget - launched_iters >= batch) {
            if (!ctx->iter_graph[solver]) {
                cudaGraph_t graph = nullptr;
                EL_CUDA_TRY(ctx, cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
                int n = 0;
                for (int q = 0; q < batch; ++q) n += enqueue(0);
                EL_CUDA_TRY(ctx, cudaStreamEndCapture(ctx->stream, &graph));
                const cudaError_t e = cudaGraphInstantiate(&ctx->iter_graph[solver], graph, 0);
                cudaGraphDestroy(graph);
                if (e != cudaSuccess) return set_error(ctx, EL_ERR_CUDA, std::string("graph: ") + cudaGetErrorString(e));
                ctx->iter_graph_len[solver] = batch;
                ctx->iter_graph_kernels[solver] = n;
            }
            EL_CUDA_TRY(ctx, cudaGraphLaunch(ctx->iter_graph[solver], ctx->stream));
            ctx->launches += ctx->iter_graph_kernels[solver];
            launched_iters += batch;
        } else {
            const int b = std::min(batch, budget - launched_iters);
            for (int q = 0; q < b; ++q) ctx->launches += enqueue(0);
            launched_iters += b;
        }
        st = check_launch(ctx, "pcg iteration");
        if (st != EL_OK) return st;
        st = poll(ctx, out, which);
        if (st != EL_OK) return st;
    }
    return EL_OK;
}

template <typename T>
static SplitOp<T> split_op(el_ctx* ctx) {
    return SplitOp<T>{ctx->diag64, (const T*)ctx->off[0], (const T*)ctx->off[1], (const T*)ctx->off[2]};
}

static void reset_vectors(el_ctx* ctx) {
    const size_t n = (size_t)ctx->ni * ctx->nj * ctx->nk;
    for (double* v : {ctx->x64, ctx->r64, ctx->z64, ctx->p64, ctx->p64b, ctx->ap64})
        if (v) cudaMemsetAsync(v, 0, n * 8, ctx->stream);
    for (float* v : {ctx->x32, ctx->r32, ctx->r32b, ctx->z32, ctx->p32, ctx->p32b, ctx->ap32})
        if (v) cudaMemsetAsync(v, 0, n * 4, ctx->stream);
    if (ctx->xs) cudaMemsetAsync(ctx->xs, 0, n * 8, ctx->stream);
    for (auto& L : ctx->mg32) {
        const size_t m = (size_t)L.n0 * L.n1 * L.n2 * 4;
        for (float* v : {L.t, L.rec ? L.b : nullptr, L.rec ? L.x : nullptr})
            if (v) cudaMemsetAsync(v, 0, m, ctx->stream);
    }
    for (auto& L : ctx->mg64) {
        const size_t m = (size_t)L.n0 * L.n1 * L.n2 * 8;
        for (double* v : {L.t, L.rec ? L.b : nullptr, L.rec ? L.x : nullptr})
            if (v) cudaMemsetAsync(v, 0, m, ctx->stream);
    }
}

// mg[0].b follows the residual buffer during a solve; between solves it is r32 again
static void mg_restore_pointers(el_ctx* ctx) {
    if (!ctx->mg32.empty()) ctx->mg32[0].b = ctx->r32;
}

// The float pair of the iterate, kept where the refinement residual is double-float: the mixed
// solver on FP32 fields (exact float couplings); null otherwise.
template <typename T>
static float2* iterate_pairs(el_ctx* ctx, int solver) {
    return (solver == EL_SOLVER_MIXED && std::is_same<T, float>::value) ? ctx->xs : nullptr;
}

// The mixed solver's refinement residual: double-float arithmetic for FP32 fields (exact float
// couplings), FP64 for FP64 fields.
template <typename T>
static void enqueue_refine_residual(el_ctx* ctx, const LGeom& g, const SplitOp<T>& A64, Scalars* s0) {
    const int nb = seg_blocks(ctx, ctx->seg0.total);
    if constexpr (std::is_same<T, float>::value)
        // the resident four CTAs per SM (its launch bounds) in one wave: 102 -> 94 us at 256^3
        residual_df_kernel<<<std::min(nb, ctx->num_sms * 4), kSegThreads, 0, ctx->stream>>>(
            g, seg_arg(ctx->seg0), A64, ctx->rhs64, ctx->x64, ctx->xs, ctx->r64, s0, ctx->partials, ctx->counter);
    else
        residual_kernel<T><<<nb, kSegThreads, 0, ctx->stream>>>(g, seg_arg(ctx->seg0), A64, ctx->rhs64, ctx->x64,
                                                                ctx->r64, s0, ctx->partials, ctx->counter);
}

// Solve A x64 = rhs64 (matrix already built, s0.bb set).  Fills stats.
template <typename T>
static int solve_t(el_ctx* ctx, const el_solve_params& prm, el_solve_stats* st) {
    const long long n = (long long)ctx->ni * ctx->nj * ctx->nk;
    const LGeom g = make_geom(ctx->ni, ctx->nj, ctx->nk);
    const int check = std::max(1, prm.check_every);
    Scalars* s0 = ctx->dscal;
    Scalars* h = ctx->hscal;
    const SplitOp<T> A64 = split_op<T>(ctx);
    // active segments of the finest level
    {
        ProfScope prof(ctx, EL_KC_OTHER, (double)n * 8);
        seg_flags_diag_kernel<<<seg_blocks(ctx, ctx->seg0.total), kSegThreads, 0, ctx->stream>>>(
            g, ctx->diag64, ctx->seg0.total, ctx->seg0.flags);
    }
    ctx->launches += 1 + enqueue_compact(ctx, ctx->seg0, g);
    int rc = record_active<double>(ctx, ctx->seg0, ctx->ni, nullptr);
    if (rc != EL_OK) return rc;
    const double na = active_cells(ctx, 0, (double)n);
    {
        ProfScope prof(ctx, EL_KC_OTHER, na * 24);
        solve_init_kernel<<<seg_blocks(ctx, ctx->seg0.total), kSegThreads, 0, ctx->stream>>>(
            g, seg_arg(ctx->seg0), ctx->rhs64, ctx->x64, iterate_pairs<T>(ctx, prm.solver), ctx->r64, s0, prm.tol);
    }
    ctx->launches += 1;
    if (prm.initial_guess) {
        ProfScope prof(ctx, EL_KC_OTHER, na * 56);
        const int nb = seg_blocks(ctx, ctx->seg0.total);
        guess_load_kernel<T><<<nb, kSegThreads, 0, ctx->stream>>>(g, seg_arg(ctx->seg0),
                                                                  (const T*)ctx->field[EL_FIELD_PRESSURE], ctx->diag64,
                                                                  ctx->x64);
        residual_kernel<T><<<nb, kSegThreads, 0, ctx->stream>>>(g, seg_arg(ctx->seg0), A64, ctx->rhs64, ctx->x64,
                                                                ctx->r64, s0, ctx->partials, ctx->counter);
        guess_alpha_kernel<<<nb, kSegThreads, 0, ctx->stream>>>(g, seg_arg(ctx->seg0), ctx->x64, ctx->rhs64, ctx->r64,
                                                                s0, ctx->partials, ctx->counter);
        guess_scale_kernel<<<nb, kSegThreads, 0, ctx->stream>>>(g, seg_arg(ctx->seg0), ctx->x64,
                                                                iterate_pairs<T>(ctx, prm.solver), ctx->rhs64,
                                                                ctx->r64, s0, ctx->partials, ctx->counter);
        ctx->launches += 4;
    }
    st->outer_iterations = 1;
    if (prm.solver == EL_SOLVER_JACOBI_FP64) {
        jacobi_rz_kernel<<<seg_blocks(ctx, ctx->seg0.total), kSegThreads, 0, ctx->stream>>>(
            g, seg_arg(ctx->seg0), ctx->diag64, ctx->r64, s0, ctx->partials, ctx->counter);
        ctx->launches += 1;
        double* p = ctx->p64;
        double* p_alt = ctx->p64b;
        rc = run_iterations(ctx, EL_SOLVER_JACOBI_FP64, 0, prm.max_iter, check, h,
                            [&](int first) { return enqueue_jacobi_iteration<T>(ctx, A64, p, p_alt, s0, first); });
        st->iterations = h->iter;
        st->relres = h->bb > 0 ? sqrt(h->rr / h->bb) : 0.0;
    } else if (prm.solver == EL_SOLVER_MG_FP64) {
        auto& mg = ctx->mg64;
        mg[0].rec = ctx->A64rec;
        mg[0].b = ctx->r64;
        mg[0].x = ctx->z64;
        pack64_kernel<T><<<grid1d(ctx, n), 256, 0, ctx->stream>>>(n, ctx->diag64, A64.x, A64.y, A64.z, ctx->A64rec);
        ctx->launches += 1 + enqueue_coarsen<double, Rec64, Rec64>(ctx, mg);
        rc = record_active(ctx, ctx->seg0, ctx->ni, &mg);
        if (rc != EL_OK) return rc;
        ctx->launches += enqueue_vcycle<double, Rec64, Rec64>(ctx, mg, ctx->seg0, s0, DOT_INIT);
        double* p = ctx->p64;
        double* p_alt = ctx->p64b;
        rc = run_iterations(ctx, EL_SOLVER_MG_FP64, 0, prm.max_iter, check, h, [&](int first) {
            return enqueue_mg_iteration<double, Rec64, Rec64, Rec64>(ctx, ctx->A64rec, ctx->x64, ctx->r64, ctx->z64, p,
                                                                    p_alt, ctx->ap64, s0, first, mg);
        });
        st->iterations = h->iter;
        st->relres = h->bb > 0 ? sqrt(h->rr / h->bb) : 0.0;
    } else {
        // mixed: FP64 refinement around FP32 multigrid PCG
        auto& mg = ctx->mg32;
        mg[0].rec = ctx->A16;
        mg[0].b = ctx->r32;
        mg[0].x = ctx->z32;
        if (!ctx->records_fresh) {
            ProfScope prof(ctx, EL_KC_OTHER, (double)n * (8 + 3 * sizeof(T) + 24));
            pack32_kernel<T><<<grid1d(ctx, n), 256, 0, ctx->stream>>>(n, ctx->diag64, A64.x, A64.y, A64.z, ctx->A32,
                                                                      ctx->A16);
            ctx->launches += 1;
        }
        ctx->launches += enqueue_coarsen<float, ushort4, float4>(ctx, mg);
        const bool march = ctx->march.on && ctx->solver_tiles;
        if (march) {
            ProfScope prof(ctx, EL_KC_OTHER, (double)n * 8);
            ctx->launches += march_enqueue_items(ctx);
        }
        // the fused coarse cycle's barrier starts clear (a failed solve may have left arrivals)
        if (ctx->coarse_bar) EL_CUDA_TRY(ctx, cudaMemsetAsync(ctx->coarse_bar, 0, 8, ctx->stream));
        rc = record_active(ctx, ctx->seg0, ctx->ni, &mg);
        if (rc != EL_OK) return rc;
        Scalars* s1 = ctx->dscal + 1;
        Scalars hi;
        rc = poll(ctx, h, 0);
        int inner_total = 0, outer = 0;
        float *p = ctx->p32, *p_alt = ctx->p32b, *r = ctx->r32, *r_alt = ctx->r32b;
        while (rc == EL_OK && !h->done && outer < std::max(1, prm.max_outer) && inner_total < prm.max_iter) {
            // every sweep starts from the same buffer assignment, so that the captured iteration
            // batches (run_iterations) see the pointers they were captured with
            p = ctx->p32;
            p_alt = ctx->p32b;
            r = ctx->r32;
            r_alt = ctx->r32b;
            mg[0].b = ctx->r32;
            {
                ProfScope prof(ctx, EL_KC_OTHER, na * 16);
                inner_init_kernel<<<seg_blocks(ctx, ctx->seg0.total), kSegThreads, 0, ctx->stream>>>(
                    g, seg_arg(ctx->seg0), ctx->r64, ctx->r32, ctx->x32, s0, s1, prm.tol, prm.inner_floor,
                    ctx->partials, ctx->counter);
            }
            ctx->launches += 1;
            if (march)
                ctx->launches += enqueue_march_vcycle(ctx, mg, s1, DOT_INIT);
            else
                ctx->launches += enqueue_vcycle<float, ushort4, float4>(ctx, mg, ctx->seg0, s1, DOT_INIT);
            rc = run_iterations(ctx, EL_SOLVER_MIXED, 1, prm.max_iter - inner_total, check, &hi, [&](int first) {
                if (march) return enqueue_march_iteration(ctx, p, p_alt, r, r_alt, s1, first, mg);
                return enqueue_mg_iteration<float, float4, ushort4, float4>(ctx, ctx->A32, ctx->x32, ctx->r32, ctx->z32,
                                                                            p, p_alt, ctx->ap32, s1, first, mg);
            });
            if (rc != EL_OK) break;
            inner_total += hi.iter;
            if (hi.fault) h->fault = 1;
            if (hi.bad) {
                h->bad = 1;
                break;
            }
            {
                ProfScope prof(ctx, EL_KC_OTHER, na * 20);
                accumulate_kernel<<<seg_blocks(ctx, ctx->seg0.total), kSegThreads, 0, ctx->stream>>>(
                    g, seg_arg(ctx->seg0), ctx->x64, iterate_pairs<T>(ctx, prm.solver), ctx->x32, s1, s0);
            }
            {
                // reads x, b, diag (f64), 3 couplings; writes r (f64)
                ProfScope prof(ctx, EL_KC_RESIDUAL, na * (32 + 3 * sizeof(T)));
                enqueue_refine_residual(ctx, g, A64, s0);
            }
            ctx->launches += 2;
            ++outer;
            rc = poll(ctx, h, 0);
        }
        st->iterations = inner_total;
        st->outer_iterations = outer;
        st->relres = h->bb > 0 ? sqrt(h->rr / h->bb) : 0.0;
    }
    mg_restore_pointers(ctx);
    if (rc != EL_OK) return rc;
    if (h->bad) {
        // entries outside the active segments are never rewritten and must stay finite (they
        // meet zero couplings), so a failed solve leaves every solver vector cleared
        reset_vectors(ctx);
        if (h->fault) return set_error(ctx, EL_ERR_TIMEOUT, "a bounded wait of the pressure solve gave up");
        return set_error(ctx, EL_ERR_NAN, "non-finite value in the pressure solve");
    }
    st->status = h->done ? EL_OK : EL_ERR_NOT_CONVERGED;
    return EL_OK;
}

// ---------------------------------------------------------------------------------------
// Capture-safe mixed solve: the same kernels, with the refinement sweeps and the PCG iterations
// driven on the device by conditional WHILE nodes of a CUDA graph (no host polling), for
// steps that are captured whole.  Must be enqueued on a stream that is being captured.

// Condition of the PCG loop: not converged and the inner iteration budget not spent.
__global__ void inner_cond_kernel(cudaGraphConditionalHandle h, Scalars* so, const Scalars* si, int max_iter,
                                  int count_pass) {
    if (count_pass) so->inner_passes += 1;
    cudaGraphSetConditional(h, (!si->done && si->iter + so->inner_total < max_iter) ? 1u : 0u);
}

// Condition of the refinement loop.  count_sweep: called after a sweep (adds its iterations);
// otherwise it sets the condition for the first sweep.
__global__ void outer_cond_kernel(cudaGraphConditionalHandle h, Scalars* so, const Scalars* si, int max_outer,
                                  int max_iter, int count_sweep) {
    if (count_sweep) {
        so->outer += 1;
        so->inner_total += si->iter;
        if (si->bad) so->bad = 1;
        if (si->fault) so->fault = 1;
    }
    const bool go = !so->done && !so->bad && so->outer < max_outer && so->inner_total < max_iter;
    cudaGraphSetConditional(h, go ? 1u : 0u);
}

// A conditional handle on the graph being captured on ctx->stream.
static int new_handle(el_ctx* ctx, cudaGraphConditionalHandle* handle) {
    cudaStreamCaptureStatus cs;
    cudaGraph_t graph = nullptr;
    EL_CUDA_TRY(ctx, cudaStreamGetCaptureInfo(ctx->stream, &cs, nullptr, &graph, nullptr, nullptr, nullptr));
    if (cs != cudaStreamCaptureStatusActive) return set_error(ctx, EL_ERR_INVALID_ARGUMENT, "stream is not capturing");
    EL_CUDA_TRY(ctx, cudaGraphConditionalHandleCreate(handle, graph, 0, cudaGraphCondAssignDefault));
    return EL_OK;
}

// Adds a WHILE node on `handle` after the work captured so far on ctx->stream and redirects
// ctx->stream to the capture of its body (ended by end_while).  The condition must have been
// set by a kernel captured before this call.
static int begin_while(el_ctx* ctx, int depth, cudaGraphConditionalHandle handle, cudaStream_t* parent) {
    cudaStreamCaptureStatus cs;
    cudaGraph_t graph = nullptr;
    const cudaGraphNode_t* deps = nullptr;
    const cudaGraphEdgeData* edges = nullptr;
    size_t ndeps = 0;
    EL_CUDA_TRY(ctx, cudaStreamGetCaptureInfo(ctx->stream, &cs, nullptr, &graph, &deps, &edges, &ndeps));
    if (cs != cudaStreamCaptureStatusActive) return set_error(ctx, EL_ERR_INVALID_ARGUMENT, "stream is not capturing");
    cudaGraphNodeParams prm = {};
    prm.type = cudaGraphNodeTypeConditional;
    prm.conditional.handle = handle;
    prm.conditional.type = cudaGraphCondTypeWhile;
    prm.conditional.size = 1;
    cudaGraphNode_t node;
    EL_CUDA_TRY(ctx, cudaGraphAddNode(&node, graph, deps, edges, ndeps, &prm));
    EL_CUDA_TRY(ctx, cudaStreamUpdateCaptureDependencies(ctx->stream, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
    if (!ctx->body_stream[depth]) return set_error(ctx, EL_ERR_INVALID_ARGUMENT, "loop streams not prepared");
    EL_CUDA_TRY(ctx, cudaStreamBeginCaptureToGraph(ctx->body_stream[depth], prm.conditional.phGraph_out[0], nullptr,
                                                   nullptr, 0, cudaStreamCaptureModeThreadLocal));
    *parent = ctx->stream;
    ctx->stream = ctx->body_stream[depth];
    return EL_OK;
}

static int end_while(el_ctx* ctx, cudaStream_t parent) {
    cudaGraph_t body = nullptr;
    const cudaError_t e = cudaStreamEndCapture(ctx->stream, &body);
    ctx->stream = parent;
    if (e != cudaSuccess) return set_error(ctx, EL_ERR_CUDA, std::string("loop body: ") + cudaGetErrorString(e));
    return EL_OK;
}

// The mixed solve with both loops on the device: no host polling, so it can sit inside a
// captured step.  The PCG loop runs iterations in pairs (the two direction buffers are back in
// place after each pass), so it may run one iteration past the budget.
template <typename T>
static int enqueue_solve_device_t(el_ctx* ctx, const el_solve_params& prm, int kernels[3]) {
    const long long n = (long long)ctx->ni * ctx->nj * ctx->nk;
    const LGeom g = make_geom(ctx->ni, ctx->nj, ctx->nk);
    Scalars* s0 = ctx->dscal;
    Scalars* s1 = ctx->dscal + 1;
    const SplitOp<T> A64 = split_op<T>(ctx);
    const int max_outer = std::max(1, prm.max_outer);
    auto& mg = ctx->mg32;
    mg[0].rec = ctx->A16;
    mg[0].b = ctx->r32;
    mg[0].x = ctx->z32;
    int nk = 0;
    seg_flags_diag_kernel<<<seg_blocks(ctx, ctx->seg0.total), kSegThreads, 0, ctx->stream>>>(
        g, ctx->diag64, ctx->seg0.total, ctx->seg0.flags);
    nk += 1 + enqueue_compact(ctx, ctx->seg0, g);
    solve_init_kernel<<<seg_blocks(ctx, ctx->seg0.total), kSegThreads, 0, ctx->stream>>>(
        g, seg_arg(ctx->seg0), ctx->rhs64, ctx->x64, iterate_pairs<T>(ctx, EL_SOLVER_MIXED), ctx->r64, s0, prm.tol);
    if (!ctx->records_fresh) {
        pack32_kernel<T><<<grid1d(ctx, n), 256, 0, ctx->stream>>>(n, ctx->diag64, A64.x, A64.y, A64.z, ctx->A32,
                                                                  ctx->A16);
        ++nk;
    }
    nk += 1 + enqueue_coarsen<float, ushort4, float4>(ctx, mg);
    const bool march = ctx->march.on && ctx->solver_tiles;
    if (march) nk += march_enqueue_items(ctx);
    if (ctx->coarse_bar) EL_CUDA_TRY(ctx, cudaMemsetAsync(ctx->coarse_bar, 0, 8, ctx->stream));
    float *p = ctx->p32, *p_alt = ctx->p32b, *r = ctx->r32, *r_alt = ctx->r32b;
    mg[0].b = ctx->r32;
    cudaGraphConditionalHandle h_outer, h_inner;
    cudaStream_t parent_outer, parent_inner;
    int rc = new_handle(ctx, &h_outer);
    if (rc != EL_OK) return rc;
    outer_cond_kernel<<<1, 1, 0, ctx->stream>>>(h_outer, s0, s1, max_outer, prm.max_iter, 0);
    rc = begin_while(ctx, 0, h_outer, &parent_outer);
    if (rc != EL_OK) return rc;
    // one refinement sweep: inner system, its PCG loop, correction and FP64 residual
    inner_init_kernel<<<seg_blocks(ctx, ctx->seg0.total), kSegThreads, 0, ctx->stream>>>(
        g, seg_arg(ctx->seg0), ctx->r64, ctx->r32, ctx->x32, s0, s1, prm.tol, prm.inner_floor, ctx->partials,
        ctx->counter);
    auto iteration = [&](int first) {
        if (march) return enqueue_march_iteration(ctx, p, p_alt, r, r_alt, s1, first, mg);
        return enqueue_mg_iteration<float, float4, ushort4, float4>(ctx, ctx->A32, ctx->x32, ctx->r32, ctx->z32, p,
                                                                   p_alt, ctx->ap32, s1, first, mg);
    };
    int body = 1 + (march ? enqueue_march_vcycle(ctx, mg, s1, DOT_INIT)
                          : enqueue_vcycle<float, ushort4, float4>(ctx, mg, ctx->seg0, s1, DOT_INIT));
    body += iteration(1);
    rc = new_handle(ctx, &h_inner);
    if (rc == EL_OK) {
        inner_cond_kernel<<<1, 1, 0, ctx->stream>>>(h_inner, s0, s1, prm.max_iter, 0);
        rc = begin_while(ctx, 1, h_inner, &parent_inner);
    }
    if (rc != EL_OK) {
        end_while(ctx, parent_outer);
        return rc;
    }
    int inner = 0;
    for (int q = 0; q < 2; ++q) inner += iteration(0);
    inner_cond_kernel<<<1, 1, 0, ctx->stream>>>(h_inner, s0, s1, prm.max_iter, 1);
    rc = end_while(ctx, parent_inner);
    accumulate_kernel<<<seg_blocks(ctx, ctx->seg0.total), kSegThreads, 0, ctx->stream>>>(
        g, seg_arg(ctx->seg0), ctx->x64, iterate_pairs<T>(ctx, EL_SOLVER_MIXED), ctx->x32, s1, s0);
    enqueue_refine_residual(ctx, g, A64, s0);
    outer_cond_kernel<<<1, 1, 0, ctx->stream>>>(h_outer, s0, s1, max_outer, prm.max_iter, 1);
    const int rc2 = end_while(ctx, parent_outer);
    mg_restore_pointers(ctx);
    if (rc != EL_OK) return rc;
    if (rc2 != EL_OK) return rc2;
    // kernels outside the loops, per refinement sweep, per pass of the PCG loop
    kernels[0] = nk + 1;
    kernels[1] = body + 1 + 2 + 1;
    kernels[2] = inner + 1;
    return check_launch(ctx, "captured solve");
}

// Streams on which the loop bodies are captured (created outside any capture).
int prepare_device_solve(el_ctx* ctx) {
    for (auto& bs : ctx->body_stream)
        if (!bs) EL_CUDA_TRY(ctx, cudaStreamCreateWithFlags(&bs, cudaStreamNonBlocking));
    return EL_OK;
}

// Enqueues (for stream capture) the mixed solve of the built system; results land in the
// device scalars (s0: converged flag, |r|^2, |b|^2, sweeps, inner iterations).
int enqueue_solve_device(el_ctx* ctx, const el_solve_params& prm, int kernels[3]) {
    if (prm.solver != EL_SOLVER_MIXED) return set_error(ctx, EL_ERR_INVALID_ARGUMENT, "captured steps use the mixed solver");
    return ctx->dtype == EL_F64 ? enqueue_solve_device_t<double>(ctx, prm, kernels)
                                : enqueue_solve_device_t<float>(ctx, prm, kernels);
}

int solve_system(el_ctx* ctx, const el_solve_params& prm, el_solve_stats* st) {
    return ctx->dtype == EL_F64 ? solve_t<double>(ctx, prm, st) : solve_t<float>(ctx, prm, st);
}

int setup_solver_storage(el_ctx* ctx, int solver) {
    const long long n = (long long)ctx->ni * ctx->nj * ctx->nk;
    if (!ctx->x64) {
        ctx->x64 = (double*)ctx_alloc(ctx, n * 8);
        ctx->r64 = (double*)ctx_alloc(ctx, n * 8);
        ctx->z64 = (double*)ctx_alloc(ctx, n * 8);
        ctx->p64 = (double*)ctx_alloc(ctx, n * 8);
        ctx->p64b = (double*)ctx_alloc(ctx, n * 8);
        ctx->ap64 = (double*)ctx_alloc(ctx, n * 8);
        if (!ctx->x64 || !ctx->r64 || !ctx->z64 || !ctx->p64 || !ctx->p64b || !ctx->ap64)
            return set_error(ctx, EL_ERR_OUT_OF_MEMORY, "solver vectors");
        int rc = alloc_seglist(ctx, ctx->seg0, ctx->ni, ctx->nj, ctx->nk);
        if (rc != EL_OK) return rc;
    }
    if (solver == EL_SOLVER_MG_FP64 && ctx->mg64.empty()) {
        ctx->A64rec = (Rec64*)ctx_alloc(ctx, n * sizeof(Rec64));
        if (!ctx->A64rec) return set_error(ctx, EL_ERR_OUT_OF_MEMORY, "multigrid records");
        int rc = build_hierarchy<double>(ctx, ctx->mg64, sizeof(Rec64));
        if (rc != EL_OK) return rc;
    }
    if (solver == EL_SOLVER_MIXED && !ctx->x32) {
        EL_CUDA_TRY(ctx, cudaFuncSetAttribute(mg_bottom_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                              bottom_smem_bytes()));
        // the fused coarse cycle: 1024-thread CTAs, all resident, where cooperative launches
        // exist; otherwise the per-level launches stay in use
        int coop = 0;
        cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, ctx->device);
        ctx->coarse_per_sm = 0;
        if (coop) {
            EL_CUDA_TRY(ctx, cudaFuncSetAttribute(mg_coarse_cycle_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                  bottom_smem_bytes()));
            int per_sm = 0;
            EL_CUDA_TRY(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, mg_coarse_cycle_kernel,
                                                                          kBottomThreads, bottom_smem_bytes()));
            ctx->coarse_bar = (unsigned*)ctx_alloc(ctx, 64);
            if (!ctx->coarse_bar) return set_error(ctx, EL_ERR_OUT_OF_MEMORY, "coarse cycle barrier");
            ctx->coarse_per_sm = per_sm;
        }
        ctx->x32 = (float*)ctx_alloc(ctx, n * 4);
        ctx->r32 = (float*)ctx_alloc(ctx, n * 4);
        ctx->z32 = (float*)ctx_alloc(ctx, n * 4);
        ctx->p32 = (float*)ctx_alloc(ctx, n * 4);
        ctx->p32b = (float*)ctx_alloc(ctx, n * 4);
        ctx->ap32 = (float*)ctx_alloc(ctx, n * 4);
        ctx->r32b = (float*)ctx_alloc(ctx, n * 4);
        ctx->xs = (float2*)ctx_alloc(ctx, n * sizeof(float2));
        ctx->A32 = (float4*)ctx_alloc(ctx, n * sizeof(float4));
        ctx->A16 = (ushort4*)ctx_alloc(ctx, n * sizeof(ushort4));
        if (!ctx->x32 || !ctx->r32 || !ctx->r32b || !ctx->z32 || !ctx->p32 || !ctx->p32b || !ctx->ap32 || !ctx->A32 ||
            !ctx->A16 || !ctx->xs)
            return set_error(ctx, EL_ERR_OUT_OF_MEMORY, "mixed solver vectors");
        int rc = build_hierarchy<float>(ctx, ctx->mg32, sizeof(float4));
        if (rc != EL_OK) return rc;
        ctx->mg32[0].rec = ctx->A16;
        ctx->mg32[0].b = ctx->r32;
        ctx->mg32[0].x = ctx->z32;
        rc = march_setup(ctx);
        if (rc != EL_OK) return rc;
    }
    return EL_OK;
}

EL_CHECK_EXPORT(solve)

}  // namespace el
