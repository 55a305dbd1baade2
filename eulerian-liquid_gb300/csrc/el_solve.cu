// el_solve.cu -- conjugate-gradient pressure solves on the grid-shaped ghost-fluid matrix.
//
// Replaces the Eigen ConjugateGradient<..., Lower, IncompleteCholesky<double>> call of
// src/project/3d/eulerian_liquid/simulator.cpp:102-109 (x0 = 0, stop on |r|^2 < tol^2 |b|^2 of
// the recursively updated residual, iteration cap) with three GPU solvers:
//
//   EL_SOLVER_JACOBI_FP64  plain FP64 PCG, Jacobi preconditioner (the correctness baseline)
//   EL_SOLVER_MG_FP64      FP64 PCG with a multigrid V-cycle preconditioner
//   EL_SOLVER_MIXED        FP64 iterative refinement: r = b - A x in FP64, the correction
//                          solved by FP32 multigrid PCG on the FP32 copy of the matrix,
//                          x += |r| * e accumulated in FP64
//
// Multigrid: coarse operators by aggregation of 2x2x2 blocks scaled by 1/2
// (A_c = 1/2 P^T A P with piecewise-constant P, which reproduces the rediscretised Laplacian
// for constant coefficients and carries the ghost-fluid Dirichlet terms down by summation),
// restriction R = P^T, damped Jacobi (omega = 0.8) with two sweeps before and two after, and
// 30 Jacobi sweeps on the coarsest level (at most 8 cells per axis) in one block's shared
// memory.  Same smoother before and after and R = P^T make the V-cycle a symmetric
// operator, as PCG needs.
//
// Per PCG iteration:  K1  p = z + beta p ; Ap = A p ; alpha = rz / p.Ap
//                     K2  x += alpha p ; r -= alpha Ap ; rr = r.r (; rz = r.D^-1 r for Jacobi)
//                     V   z = M^-1 r ; rz = r.z ; beta            (multigrid solvers)
// Scalars live in device memory; once converged the remaining launched kernels return at
// entry, so the host polls only every `check_every` iterations.
#include "el_internal.cuh"

namespace el {

constexpr double kOmega = 0.8;
constexpr int kCoarsestSweeps = 30;
constexpr int kCoarsestMaxDim = 8;
constexpr int kCoarsestMaxCells = 512;

template <typename DT, typename OT>
struct Stencil {
    int n0, n1, n2;
    const DT* __restrict__ diag;
    const OT* __restrict__ ox;
    const OT* __restrict__ oy;
    const OT* __restrict__ oz;
};

// (A y)(c) for y given by a functor of the neighbour's linear index and coordinates;
// neighbours outside the grid are skipped (their couplings are zero anyway).
template <typename V, typename DT, typename OT, typename F>
__device__ __forceinline__ V apply_row(const Stencil<DT, OT>& A, int i, int j, int k, long long c, V yc,
                                       F&& y) {
    const long long s1 = A.n0, s2 = (long long)A.n0 * A.n1;
    V s = (V)A.diag[c] * yc;
    if (i > 0) s += (V)A.ox[c - 1] * y(c - 1, i - 1, j, k);
    if (i < A.n0 - 1) s += (V)A.ox[c] * y(c + 1, i + 1, j, k);
    if (j > 0) s += (V)A.oy[c - s1] * y(c - s1, i, j - 1, k);
    if (j < A.n1 - 1) s += (V)A.oy[c] * y(c + s1, i, j + 1, k);
    if (k > 0) s += (V)A.oz[c - s2] * y(c - s2, i, j, k - 1);
    if (k < A.n2 - 1) s += (V)A.oz[c] * y(c + s2, i, j, k + 1);
    return s;
}

__device__ __forceinline__ bool finite_d(double v) { return isfinite(v); }

// ---------------------------------------------------------------------------------------
// K1: new search direction fused with the SpMV and p.Ap.  JAC: z = r / diag on the fly.
template <typename V, typename DT, typename OT, bool JAC>
__global__ void __launch_bounds__(256) dir_spmv_kernel(Stencil<DT, OT> A, const V* __restrict__ zr,
                                                       const V* __restrict__ p_in, V* __restrict__ p_out,
                                                       V* __restrict__ ap, Scalars* s, int first,
                                                       double* partials, unsigned* counter) {
    if (s->done) return;
    const V beta = first ? V(0) : (V)s->beta;
    auto pn = [&](long long q, int, int, int) -> V {
        const DT d = A.diag[q];
        if (d == DT(0)) return V(0);
        const V z = JAC ? zr[q] / (V)d : zr[q];
        return first ? z : z + beta * p_in[q];
    };
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    double acc[1] = {0.0};
    if (i < A.n0 && j < A.n1) {
        for (int k = blockIdx.z; k < A.n2; k += gridDim.z) {
            const long long c = lin3(i, j, k, A.n0, A.n1);
            V pc = V(0), apc = V(0);
            if (A.diag[c] != DT(0)) {
                pc = pn(c, i, j, k);
                apc = apply_row<V>(A, i, j, k, c, pc, pn);
            }
            p_out[c] = pc;
            ap[c] = apc;
            acc[0] += (double)pc * (double)apc;
        }
    }
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
template <typename V, typename DT, bool JAC>
__global__ void __launch_bounds__(256) update_kernel(long long n, const DT* __restrict__ diag,
                                                     V* __restrict__ x, V* __restrict__ r,
                                                     const V* __restrict__ p, const V* __restrict__ ap,
                                                     Scalars* s, double* partials, unsigned* counter) {
    if (s->done) return;
    const V alpha = (V)s->alpha;
    double acc[2] = {0.0, 0.0};
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n;
         c += (long long)gridDim.x * blockDim.x) {
        const V rc = r[c] - alpha * ap[c];
        x[c] = x[c] + alpha * p[c];
        r[c] = rc;
        acc[0] += (double)rc * (double)rc;
        if (JAC) {
            const DT d = diag[c];
            if (d != DT(0)) acc[1] += (double)rc * (double)(rc / (V)d);
        }
    }
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
template <typename V, typename DT>
__global__ void jacobi_rz_kernel(long long n, const DT* __restrict__ diag, const V* __restrict__ r, Scalars* s,
                                 double* partials, unsigned* counter) {
    double acc[1] = {0.0};
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n;
         c += (long long)gridDim.x * blockDim.x) {
        const DT d = diag[c];
        if (d != DT(0)) acc[0] += (double)r[c] * (double)(r[c] / (V)d);
    }
    double tot[1];
    if (grid_sum<1>(acc, partials, counter, tot)) s->rz = tot[0];
}

// solve start (outer / plain): x = 0, r = b, thresholds.
__global__ void solve_init_kernel(long long n, const double* __restrict__ b, double* __restrict__ x,
                                  double* __restrict__ r, Scalars* s, double tol) {
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n;
         c += (long long)gridDim.x * blockDim.x) {
        x[c] = 0.0;
        r[c] = b[c];
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        const double bb = s->bb;
        s->thresh = tol * tol * bb;
        s->rr = bb;
        s->iter = 0;
        s->bad = finite_d(bb) ? 0 : 1;
        s->done = (bb == 0.0 || bb < s->thresh || s->bad) ? 1 : 0;
        s->beta = 0.0;
    }
}

// mixed solver: inner system r32 = r64 / |r64|, x32 = 0, inner thresholds.
__global__ void inner_init_kernel(long long n, const double* __restrict__ r64, float* __restrict__ r32,
                                  float* __restrict__ x32, const Scalars* so, Scalars* si, double tau,
                                  double* partials, unsigned* counter) {
    const double norm = sqrt(so->rr);
    const double inv = norm > 0.0 ? 1.0 / norm : 0.0;
    double acc[1] = {0.0};
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n;
         c += (long long)gridDim.x * blockDim.x) {
        const float v = (float)(r64[c] * inv);
        r32[c] = v;
        x32[c] = 0.0f;
        acc[0] += (double)v * (double)v;
    }
    double tot[1];
    if (grid_sum<1>(acc, partials, counter, tot)) {
        si->bb = tot[0];
        si->rr = tot[0];
        si->thresh = tau * tau * tot[0];
        si->norm = norm;
        si->iter = 0;
        si->bad = 0;
        si->beta = 0.0;
        si->done = (tot[0] == 0.0 || tot[0] < si->thresh) ? 1 : 0;
    }
}

// mixed solver: x64 += |r| * x32
__global__ void accumulate_kernel(long long n, double* __restrict__ x64, const float* __restrict__ x32,
                                  const Scalars* si) {
    const double norm = si->norm;
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n;
         c += (long long)gridDim.x * blockDim.x)
        x64[c] += norm * (double)x32[c];
}

// FP64 residual r = b - A x and |r|^2 (outer refinement step).
template <typename OT>
__global__ void __launch_bounds__(256) residual_kernel(Stencil<double, OT> A, const double* __restrict__ b,
                                                       const double* __restrict__ x, double* __restrict__ r,
                                                       Scalars* s, double* partials, unsigned* counter) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    double acc[1] = {0.0};
    auto xv = [&](long long q, int, int, int) -> double { return x[q]; };
    if (i < A.n0 && j < A.n1) {
        for (int k = blockIdx.z; k < A.n2; k += gridDim.z) {
            const long long c = lin3(i, j, k, A.n0, A.n1);
            double rc = 0.0;
            if (A.diag[c] != 0.0) rc = b[c] - apply_row<double>(A, i, j, k, c, x[c], xv);
            r[c] = rc;
            acc[0] += rc * rc;
        }
    }
    double tot[1];
    if (grid_sum<1>(acc, partials, counter, tot)) {
        s->rr = tot[0];
        if (!finite_d(tot[0])) {
            s->bad = 1;
            s->done = 1;
        } else if (tot[0] < s->thresh) {
            s->done = 1;
        }
    }
}

template <typename S, typename D>
__global__ void convert_kernel(long long n, const S* __restrict__ a, D* __restrict__ b) {
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n;
         c += (long long)gridDim.x * blockDim.x)
        b[c] = (D)a[c];
}

// ---------------------------------------------------------------------------------------
// multigrid kernels

template <typename V>
struct Level {
    int n0, n1, n2;
    const V* __restrict__ diag;
    const V* __restrict__ ox;
    const V* __restrict__ oy;
    const V* __restrict__ oz;
};

template <typename V>
__device__ __forceinline__ Stencil<V, V> as_stencil(const Level<V>& L) {
    return Stencil<V, V>{L.n0, L.n1, L.n2, L.diag, L.ox, L.oy, L.oz};
}

// Coarse operator A_c = 1/2 P^T A P over 2x2x2 blocks.
template <typename V>
__global__ void coarsen_kernel(Level<V> F, int m0, int m1, int m2, V* __restrict__ cd, V* __restrict__ cx,
                               V* __restrict__ cy, V* __restrict__ cz) {
    const int I = blockIdx.x * blockDim.x + threadIdx.x;
    const int J = blockIdx.y * blockDim.y + threadIdx.y;
    const int K = blockIdx.z;
    if (I >= m0 || J >= m1) return;
    V d = 0, sx = 0, sy = 0, sz = 0, inner = 0;
    for (int kk = 0; kk < 2; ++kk)
        for (int jj = 0; jj < 2; ++jj)
            for (int ii = 0; ii < 2; ++ii) {
                const int i = 2 * I + ii, j = 2 * J + jj, k = 2 * K + kk;
                if (i >= F.n0 || j >= F.n1 || k >= F.n2) continue;
                const long long c = lin3(i, j, k, F.n0, F.n1);
                d += F.diag[c];
                if (ii == 0) inner += F.ox[c]; else sx += F.ox[c];
                if (jj == 0) inner += F.oy[c]; else sy += F.oy[c];
                if (kk == 0) inner += F.oz[c]; else sz += F.oz[c];
            }
    V dc = V(0.5) * (d + V(2) * inner);
    const long long q = lin3(I, J, K, m0, m1);
    // an aggregate with no coupling to anything outside it (an enclosed Neumann pocket) has
    // a zero row sum; it is left out of the coarse problem
    const bool active = dc > V(1e-30) * (d > V(0) ? d : V(1));
    cd[q] = active ? dc : V(0);
    cx[q] = active ? V(0.5) * sx : V(0);
    cy[q] = active ? V(0.5) * sy : V(0);
    cz[q] = active ? V(0.5) * sz : V(0);
}

// Smoothing sweeps.  MODE 0: two sweeps from x = 0 (the first, omega b / D, formed on the
// fly).  MODE 1: one sweep from x_in + P e (e = coarse correction, formed on the fly).
// MODE 2: one sweep from x_in.  DOT (level 0, last sweep): rz = b . x_out and beta.
enum { SM_ZERO2 = 0, SM_PROLONG = 1, SM_PLAIN = 2 };
enum { DOT_NONE = 0, DOT_INIT = 1, DOT_BETA = 2 };

template <typename V, int MODE, int DOT>
__global__ void __launch_bounds__(256) smooth_kernel(Level<V> L, const V* __restrict__ b, const V* __restrict__ x_in,
                                                     const V* __restrict__ e, int m0, int m1,
                                                     V* __restrict__ x_out, Scalars* s, double* partials,
                                                     unsigned* counter) {
    if (s->done) return;
    const V omega = V(kOmega);
    const Stencil<V, V> A = as_stencil(L);
    auto xv = [&](long long q, int qi, int qj, int qk) -> V {
        const V d = L.diag[q];
        if (d == V(0)) return V(0);
        if (MODE == SM_ZERO2) return omega * b[q] / d;
        if (MODE == SM_PROLONG) return x_in[q] + e[lin3(qi >> 1, qj >> 1, qk >> 1, m0, m1)];
        return x_in[q];
    };
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    double acc[1] = {0.0};
    if (i < L.n0 && j < L.n1) {
        for (int k = blockIdx.z; k < L.n2; k += gridDim.z) {
            const long long c = lin3(i, j, k, L.n0, L.n1);
            const V d = L.diag[c];
            V xo = V(0);
            if (d != V(0)) {
                const V xc = xv(c, i, j, k);
                const V ax = apply_row<V>(A, i, j, k, c, xc, xv);
                xo = xc + omega * (b[c] - ax) / d;
            }
            x_out[c] = xo;
            if (DOT != DOT_NONE) acc[0] += (double)b[c] * (double)xo;
        }
    }
    if (DOT != DOT_NONE) {
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

// Residual of the fine level summed onto the coarse right-hand side (R = P^T).  Blocks are
// 32 x 8 fine cells in (i, j) and march over coarse planes K (fine planes 2K, 2K+1).
template <typename V>
__global__ void __launch_bounds__(256) restrict_kernel(Level<V> L, const V* __restrict__ b, const V* __restrict__ x,
                                                       int m0, int m1, int m2, V* __restrict__ bc, const Scalars* s) {
    if (s->done) return;
    __shared__ V sh[kBY][kBX];
    const Stencil<V, V> A = as_stencil(L);
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int i = blockIdx.x * kBX + tx;
    const int j = blockIdx.y * kBY + ty;
    auto xv = [&](long long q, int, int, int) -> V { return x[q]; };
    for (int K = blockIdx.z; K < m2; K += gridDim.z) {
        V rsum = V(0);
        if (i < L.n0 && j < L.n1) {
            for (int kk = 0; kk < 2; ++kk) {
                const int k = 2 * K + kk;
                if (k >= L.n2) break;
                const long long c = lin3(i, j, k, L.n0, L.n1);
                if (L.diag[c] != V(0)) rsum += b[c] - apply_row<V>(A, i, j, k, c, x[c], xv);
            }
        }
        rsum += __shfl_down_sync(0xffffffffu, rsum, 1);
        sh[ty][tx] = rsum;
        __syncthreads();
        if ((tx & 1) == 0 && (ty & 1) == 0) {
            const int I = i >> 1, J = j >> 1;
            if (I < m0 && J < m1) bc[lin3(I, J, K, m0, m1)] = sh[ty][tx] + sh[ty + 1][tx];
        }
        __syncthreads();
    }
}

// Coarsest level: omega-Jacobi sweeps from zero in one block's shared memory.
template <typename V>
__global__ void __launch_bounds__(kCoarsestMaxCells) coarsest_kernel(Level<V> L, const V* __restrict__ b,
                                                                     V* __restrict__ x, int sweeps, const Scalars* s) {
    if (s->done) return;
    __shared__ V sd[kCoarsestMaxCells], sx[kCoarsestMaxCells], sy[kCoarsestMaxCells], sz[kCoarsestMaxCells];
    __shared__ V sb[kCoarsestMaxCells], xa[kCoarsestMaxCells], xb[kCoarsestMaxCells];
    const int n = L.n0 * L.n1 * L.n2;
    const int c = threadIdx.x;
    const V omega = V(kOmega);
    if (c < n) {
        sd[c] = L.diag[c];
        sx[c] = L.ox[c];
        sy[c] = L.oy[c];
        sz[c] = L.oz[c];
        sb[c] = b[c];
        xa[c] = sd[c] != V(0) ? omega * sb[c] / sd[c] : V(0);
    }
    __syncthreads();
    const int i = c % L.n0, j = (c / L.n0) % L.n1, k = c / (L.n0 * L.n1);
    const int s1 = L.n0, s2 = L.n0 * L.n1;
    V* cur = xa;
    V* nxt = xb;
    for (int it = 1; it < sweeps; ++it) {
        if (c < n) {
            V xo = V(0);
            const V d = sd[c];
            if (d != V(0)) {
                V a = d * cur[c];
                if (i > 0) a += sx[c - 1] * cur[c - 1];
                if (i < L.n0 - 1) a += sx[c] * cur[c + 1];
                if (j > 0) a += sy[c - s1] * cur[c - s1];
                if (j < L.n1 - 1) a += sy[c] * cur[c + s1];
                if (k > 0) a += sz[c - s2] * cur[c - s2];
                if (k < L.n2 - 1) a += sz[c] * cur[c + s2];
                xo = cur[c] + omega * (sb[c] - a) / d;
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
// host side

static int grid1d(el_ctx* ctx, long long n) {
    return (int)std::max<long long>(1, std::min<long long>((n + 255) / 256, (long long)ctx->num_sms * 8));
}

template <typename V>
static Level<V> level_view(const MGLevel<V>& L) {
    return Level<V>{L.n0, L.n1, L.n2, L.diag, L.off[0], L.off[1], L.off[2]};
}

// Allocate the hierarchy below the given level-0 dimensions (level 0 arrays set by caller).
template <typename V>
static void build_hierarchy(el_ctx* ctx, std::vector<MGLevel<V>>& mg) {
    mg.clear();
    MGLevel<V> L0;
    L0.n0 = ctx->ni;
    L0.n1 = ctx->nj;
    L0.n2 = ctx->nk;
    const long long n = (long long)ctx->ni * ctx->nj * ctx->nk;
    L0.t = (V*)ctx_alloc(ctx, n * sizeof(V));
    mg.push_back(L0);
    while (std::max(mg.back().n0, std::max(mg.back().n1, mg.back().n2)) > kCoarsestMaxDim) {
        MGLevel<V> C;
        C.n0 = (mg.back().n0 + 1) / 2;
        C.n1 = (mg.back().n1 + 1) / 2;
        C.n2 = (mg.back().n2 + 1) / 2;
        const long long m = (long long)C.n0 * C.n1 * C.n2;
        C.diag = (V*)ctx_alloc(ctx, m * sizeof(V));
        for (int a = 0; a < 3; ++a) C.off[a] = (V*)ctx_alloc(ctx, m * sizeof(V));
        C.b = (V*)ctx_alloc(ctx, m * sizeof(V));
        C.x = (V*)ctx_alloc(ctx, m * sizeof(V));
        C.t = (V*)ctx_alloc(ctx, m * sizeof(V));
        mg.push_back(C);
    }
}

template <typename V>
static int enqueue_coarsen(el_ctx* ctx, std::vector<MGLevel<V>>& mg) {
    int launched = 0;
    for (size_t l = 0; l + 1 < mg.size(); ++l) {
        const MGLevel<V>& F = mg[l];
        MGLevel<V>& C = mg[l + 1];
        ProfScope prof(ctx, EL_KC_MG_COARSE,
                       (double)F.n0 * F.n1 * F.n2 * 4 * sizeof(V) + (double)C.n0 * C.n1 * C.n2 * 4 * sizeof(V));
        dim3 block(32, 4, 1);
        dim3 grid((C.n0 + 31) / 32, (C.n1 + 3) / 4, C.n2);
        coarsen_kernel<V><<<grid, block, 0, ctx->stream>>>(level_view(F), C.n0, C.n1, C.n2, C.diag, C.off[0],
                                                           C.off[1], C.off[2]);
        ++launched;
    }
    return launched;
}

// z = M^-1 r with r = mg[0].b and z = mg[0].x; dot = DOT_INIT or DOT_BETA
template <typename V>
static int enqueue_vcycle(el_ctx* ctx, std::vector<MGLevel<V>>& mg, Scalars* s, int dot) {
    int launched = 0;
    const int L = (int)mg.size();
    if (L == 1) {
        // grid too small to coarsen: the whole problem is solved by the coarsest sweeps, then
        // one plain sweep computes the dot product
        MGLevel<V>& C = mg[0];
        coarsest_kernel<V><<<1, kCoarsestMaxCells, 0, ctx->stream>>>(level_view(C), C.b, C.t, kCoarsestSweeps, s);
        Geom g = stencil_geom(C.n0, C.n1, C.n2, ctx->num_sms);
        if (dot == DOT_INIT)
            smooth_kernel<V, SM_PLAIN, DOT_INIT><<<g.grid, g.block, 0, ctx->stream>>>(
                level_view(C), C.b, C.t, nullptr, 0, 0, C.x, s, ctx->partials, ctx->counter);
        else
            smooth_kernel<V, SM_PLAIN, DOT_BETA><<<g.grid, g.block, 0, ctx->stream>>>(
                level_view(C), C.b, C.t, nullptr, 0, 0, C.x, s, ctx->partials, ctx->counter);
        return 2;
    }
    auto cells = [](const MGLevel<V>& X) { return (double)X.n0 * X.n1 * X.n2; };
    const double vs = sizeof(V);
    for (int l = 0; l < L - 1; ++l) {
        MGLevel<V>& F = mg[l];
        MGLevel<V>& C = mg[l + 1];
        Geom g = stencil_geom(F.n0, F.n1, F.n2, ctx->num_sms);
        {
            // reads b, diag, 3 couplings; writes x
            ProfScope prof(ctx, l == 0 ? EL_KC_SMOOTH : EL_KC_MG_COARSE, cells(F) * vs * 6);
            smooth_kernel<V, SM_ZERO2, DOT_NONE><<<g.grid, g.block, 0, ctx->stream>>>(
                level_view(F), F.b, nullptr, nullptr, 0, 0, F.x, s, ctx->partials, ctx->counter);
        }
        Geom gr = stencil_geom(F.n0, F.n1, C.n2, ctx->num_sms);
        {
            // reads b, x, diag, 3 couplings; writes the coarse b
            ProfScope prof(ctx, l == 0 ? EL_KC_RESTRICT : EL_KC_MG_COARSE, cells(F) * vs * 6 + cells(C) * vs);
            restrict_kernel<V><<<gr.grid, gr.block, 0, ctx->stream>>>(level_view(F), F.b, F.x, C.n0, C.n1, C.n2,
                                                                      C.b, s);
        }
        launched += 2;
    }
    {
        MGLevel<V>& C = mg[L - 1];
        ProfScope prof(ctx, EL_KC_MG_COARSE, cells(C) * vs * 6);
        coarsest_kernel<V><<<1, kCoarsestMaxCells, 0, ctx->stream>>>(level_view(C), C.b, C.x, kCoarsestSweeps, s);
        ++launched;
    }
    for (int l = L - 2; l >= 0; --l) {
        MGLevel<V>& F = mg[l];
        MGLevel<V>& C = mg[l + 1];
        Geom g = stencil_geom(F.n0, F.n1, F.n2, ctx->num_sms);
        // prolongation sweep reads b, x, diag, 3 couplings and the coarse x, writes t; the last
        // sweep reads b, t, diag, 3 couplings and writes x
        ProfScope prof(ctx, l == 0 ? EL_KC_SMOOTH : EL_KC_MG_COARSE, cells(F) * vs * 14 + cells(C) * vs);
        smooth_kernel<V, SM_PROLONG, DOT_NONE><<<g.grid, g.block, 0, ctx->stream>>>(
            level_view(F), F.b, F.x, C.x, C.n0, C.n1, F.t, s, ctx->partials, ctx->counter);
        if (l > 0)
            smooth_kernel<V, SM_PLAIN, DOT_NONE><<<g.grid, g.block, 0, ctx->stream>>>(
                level_view(F), F.b, F.t, nullptr, 0, 0, F.x, s, ctx->partials, ctx->counter);
        else if (dot == DOT_INIT)
            smooth_kernel<V, SM_PLAIN, DOT_INIT><<<g.grid, g.block, 0, ctx->stream>>>(
                level_view(F), F.b, F.t, nullptr, 0, 0, F.x, s, ctx->partials, ctx->counter);
        else
            smooth_kernel<V, SM_PLAIN, DOT_BETA><<<g.grid, g.block, 0, ctx->stream>>>(
                level_view(F), F.b, F.t, nullptr, 0, 0, F.x, s, ctx->partials, ctx->counter);
        launched += 2;
    }
    return launched;
}

// One PCG iteration: K1, K2 and, for the multigrid solvers, the V-cycle.
template <typename V, typename DT, typename OT, bool JAC>
static int enqueue_iteration(el_ctx* ctx, const Stencil<DT, OT>& A, V* x, V* r, V* z, V*& p, V*& p_alt, V* ap,
                             Scalars* s, int first, std::vector<MGLevel<V>>* mg) {
    Geom g = stencil_geom(A.n0, A.n1, A.n2, ctx->num_sms);
    const long long n = (long long)A.n0 * A.n1 * A.n2;
    const double nv = (double)n * sizeof(V);
    {
        // reads z (or r), p (not on the first iteration), diag, 3 couplings; writes p, Ap
        ProfScope prof(ctx, EL_KC_DIR_SPMV,
                       nv * (first ? 3 : 4) + (double)n * (sizeof(DT) + 3 * sizeof(OT)));
        dir_spmv_kernel<V, DT, OT, JAC><<<g.grid, g.block, 0, ctx->stream>>>(A, JAC ? r : z, p, p_alt, ap, s, first,
                                                                            ctx->partials, ctx->counter);
    }
    std::swap(p, p_alt);
    {
        // reads x, r, p, Ap (and diag for Jacobi); writes x, r
        ProfScope prof(ctx, EL_KC_UPDATE, nv * 6 + (JAC ? (double)n * sizeof(DT) : 0.0));
        update_kernel<V, DT, JAC><<<grid1d(ctx, n), 256, 0, ctx->stream>>>(n, A.diag, x, r, p, ap, s, ctx->partials,
                                                                          ctx->counter);
    }
    int launched = 2;
    if (!JAC) launched += enqueue_vcycle<V>(ctx, *mg, s, DOT_BETA);
    return launched;
}

static int poll(el_ctx* ctx, Scalars* host_copy, int which) {
    EL_CUDA_TRY(ctx, cudaMemcpyAsync(host_copy, ctx->dscal + which, sizeof(Scalars), cudaMemcpyDeviceToHost,
                                     ctx->stream));
    EL_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    return EL_OK;
}

// Run PCG iterations until converged or `budget` iterations were launched; returns status.
template <typename V, typename DT, typename OT, bool JAC>
static int run_pcg(el_ctx* ctx, const Stencil<DT, OT>& A, V* x, V* r, V* z, V* p, V* p_alt, V* ap, int which,
                   std::vector<MGLevel<V>>* mg, int budget, int check_every, Scalars* out) {
    Scalars* s = ctx->dscal + which;
    int launched_iters = 0;
    bool first = true;
    int st = poll(ctx, out, which);
    if (st != EL_OK) return st;
    while (!out->done && launched_iters < budget) {
        const int batch = std::min(check_every, budget - launched_iters);
        for (int q = 0; q < batch; ++q) {
            ctx->launches += enqueue_iteration<V, DT, OT, JAC>(ctx, A, x, r, z, p, p_alt, ap, s, first ? 1 : 0, mg);
            first = false;
        }
        launched_iters += batch;
        st = check_launch(ctx, "pcg iteration");
        if (st != EL_OK) return st;
        st = poll(ctx, out, which);
        if (st != EL_OK) return st;
    }
    return EL_OK;
}

template <typename T>
static Stencil<double, T> fine_stencil64(el_ctx* ctx) {
    return Stencil<double, T>{ctx->ni, ctx->nj, ctx->nk, ctx->diag64, (const T*)ctx->off[0], (const T*)ctx->off[1],
                              (const T*)ctx->off[2]};
}

// Solve A x64 = rhs64 (matrix already built, s0.bb set).  Fills stats.
template <typename T>
static int solve_t(el_ctx* ctx, const el_solve_params& prm, el_solve_stats* st) {
    const long long n = (long long)ctx->ni * ctx->nj * ctx->nk;
    const int check = std::max(1, prm.check_every);
    Scalars* s0 = ctx->dscal;
    Scalars* h = ctx->hscal;
    solve_init_kernel<<<grid1d(ctx, n), 256, 0, ctx->stream>>>(n, ctx->rhs64, ctx->x64, ctx->r64, s0, prm.tol);
    ctx->launches += 1;
    int rc = EL_OK;
    const Stencil<double, T> A64 = fine_stencil64<T>(ctx);
    st->outer_iterations = 1;
    if (prm.solver == EL_SOLVER_JACOBI_FP64) {
        jacobi_rz_kernel<double, double><<<grid1d(ctx, n), 256, 0, ctx->stream>>>(n, ctx->diag64, ctx->r64, s0,
                                                                                 ctx->partials, ctx->counter);
        ctx->launches += 1;
        rc = run_pcg<double, double, T, true>(ctx, A64, ctx->x64, ctx->r64, nullptr, ctx->p64, ctx->z64, ctx->ap64, 0,
                                              nullptr, prm.max_iter, check, h);
        st->iterations = h->iter;
        st->relres = h->bb > 0 ? sqrt(h->rr / h->bb) : 0.0;
    } else if (prm.solver == EL_SOLVER_MG_FP64) {
        auto& mg = ctx->mg64;
        // level 0 views: coefficients in double (copies when the field type is float)
        mg[0].diag = ctx->diag64;
        mg[0].b = ctx->r64;
        mg[0].x = ctx->z64;
        if (sizeof(T) == 4) {
            for (int a = 0; a < 3; ++a) {
                convert_kernel<float, double><<<grid1d(ctx, n), 256, 0, ctx->stream>>>(n, (const float*)ctx->off[a],
                                                                                       mg[0].off[a]);
            }
            ctx->launches += 3;
        } else {
            for (int a = 0; a < 3; ++a) mg[0].off[a] = (double*)ctx->off[a];
        }
        ctx->launches += enqueue_coarsen<double>(ctx, mg);
        ctx->launches += enqueue_vcycle<double>(ctx, mg, s0, DOT_INIT);
        rc = run_pcg<double, double, T, false>(ctx, A64, ctx->x64, ctx->r64, ctx->z64, ctx->p64, ctx->p64b,
                                               ctx->ap64, 0, &mg, prm.max_iter, check, h);
        st->iterations = h->iter;
        st->relres = h->bb > 0 ? sqrt(h->rr / h->bb) : 0.0;
    } else {
        // mixed: FP64 refinement around FP32 multigrid PCG
        auto& mg = ctx->mg32;
        mg[0].diag = ctx->diag32;
        for (int a = 0; a < 3; ++a) mg[0].off[a] = ctx->off32[a];
        mg[0].b = ctx->r32;
        mg[0].x = ctx->z32;
        ctx->launches += enqueue_coarsen<float>(ctx, mg);
        const Stencil<float, float> A32{ctx->ni, ctx->nj, ctx->nk, ctx->diag32, ctx->off32[0], ctx->off32[1],
                                        ctx->off32[2]};
        Scalars* s1 = ctx->dscal + 1;
        Scalars hi;
        rc = poll(ctx, h, 0);
        int inner_total = 0, outer = 0;
        Geom g = stencil_geom(ctx->ni, ctx->nj, ctx->nk, ctx->num_sms);
        while (rc == EL_OK && !h->done && outer < std::max(1, prm.max_outer) && inner_total < prm.max_iter) {
            const double want = prm.tol * sqrt(h->bb / h->rr);
            const double tau = std::min(0.5, std::max(prm.inner_floor, 0.5 * want));
            inner_init_kernel<<<grid1d(ctx, n), 256, 0, ctx->stream>>>(n, ctx->r64, ctx->r32, ctx->x32, s0, s1, tau,
                                                                       ctx->partials, ctx->counter);
            ctx->launches += 1;
            ctx->launches += enqueue_vcycle<float>(ctx, mg, s1, DOT_INIT);
            rc = run_pcg<float, float, float, false>(ctx, A32, ctx->x32, ctx->r32, ctx->z32, ctx->p32, ctx->p32b,
                                                     ctx->ap32, 1, &mg, prm.max_iter - inner_total, check, &hi);
            if (rc != EL_OK) break;
            inner_total += hi.iter;
            if (hi.bad) {
                h->bad = 1;
                break;
            }
            {
                ProfScope prof(ctx, EL_KC_OTHER, (double)n * 20);
                accumulate_kernel<<<grid1d(ctx, n), 256, 0, ctx->stream>>>(n, ctx->x64, ctx->x32, s1);
            }
            {
                // reads x, b, diag (f64), 3 couplings; writes r (f64)
                ProfScope prof(ctx, EL_KC_RESIDUAL, (double)n * (32 + 3 * sizeof(T)));
                residual_kernel<T><<<g.grid, g.block, 0, ctx->stream>>>(A64, ctx->rhs64, ctx->x64, ctx->r64, s0,
                                                                        ctx->partials, ctx->counter);
            }
            ctx->launches += 2;
            ++outer;
            rc = poll(ctx, h, 0);
        }
        st->iterations = inner_total;
        st->outer_iterations = outer;
        st->relres = h->bb > 0 ? sqrt(h->rr / h->bb) : 0.0;
    }
    if (rc != EL_OK) return rc;
    if (h->bad) return set_error(ctx, EL_ERR_NAN, "non-finite value in the pressure solve");
    st->status = h->done ? EL_OK : EL_ERR_NOT_CONVERGED;
    return EL_OK;
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
        ctx->ap64 = (double*)ctx_alloc(ctx, n * 8);
        if (!ctx->x64 || !ctx->r64 || !ctx->z64 || !ctx->p64 || !ctx->ap64)
            return set_error(ctx, EL_ERR_OUT_OF_MEMORY, "solver vectors");
    }
    if (solver == EL_SOLVER_MG_FP64 && ctx->mg64.empty()) {
        build_hierarchy<double>(ctx, ctx->mg64);
        if (ctx->dtype == EL_F32)
            for (int a = 0; a < 3; ++a) ctx->mg64[0].off[a] = (double*)ctx_alloc(ctx, n * 8);
        ctx->p64b = (double*)ctx_alloc(ctx, n * 8);
    }
    if (solver == EL_SOLVER_MIXED && !ctx->x32) {
        ctx->x32 = (float*)ctx_alloc(ctx, n * 4);
        ctx->r32 = (float*)ctx_alloc(ctx, n * 4);
        ctx->z32 = (float*)ctx_alloc(ctx, n * 4);
        ctx->p32 = (float*)ctx_alloc(ctx, n * 4);
        ctx->ap32 = (float*)ctx_alloc(ctx, n * 4);
        ctx->p32b = (float*)ctx_alloc(ctx, n * 4);
        ctx->diag32 = (float*)ctx_alloc(ctx, n * 4);
        for (int a = 0; a < 3; ++a)
            ctx->off32[a] = ctx->dtype == EL_F32 ? (float*)ctx->off[a] : (float*)ctx_alloc(ctx, n * 4);
        build_hierarchy<float>(ctx, ctx->mg32);
        if (!ctx->x32 || !ctx->diag32) return set_error(ctx, EL_ERR_OUT_OF_MEMORY, "mixed solver vectors");
    }
    return EL_OK;
}

}  // namespace el
