// el_project.cu -- ghost-fluid pressure projection set-up and velocity update.
//
// Reference: src/project/3d/fluid/projection.cpp (is_pressure_valid, assign_indices,
// build_matrix, build_grid_from_vector, update_velocity_using_pressure),
// src/project/3d/fluid/boundary.cpp (compute_staggered_grid_weight),
// include/nama/math/level_set.h:68-163 (fraction_inside).
//
// The matrix is kept grid-shaped: diag64[c] = A(c,c) (double, summed in the reference's
// neighbour order -x,+x,-y,+y,-z,+z), off[a][c] = A(c, c+e_a) = -weight (field type, exact),
// rhs64[c] = b(c) (double).  Products are rounded with __*_rn intrinsics where the reference
// rounds them, so the coefficients match the CPU restatement bit for bit.
#include <cuda_fp16.h>

#include "el_df.cuh"
#include "el_internal.cuh"

namespace el {

// ---------------------------------------------------------------------------------------
// rounding-explicit arithmetic (no FMA contraction), for bit-exact coefficients

__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }

// fraction_inside(bl, br, tl, tr) (level_set.h:82-163): corners walked bl, br, tr, tl; the
// reference forms its 0.5 / 0.25 products in double and rounds to T on return.
template <typename T>
__device__ T fraction_inside4(T bl, T br, T tl, T tr) {
    const int inside = (bl < T(0)) + (tl < T(0)) + (br < T(0)) + (tr < T(0));
    T c[4] = {bl, br, tr, tl};
    auto rotate = [&c]() {
        T t = c[0];
        c[0] = c[1];
        c[1] = c[2];
        c[2] = c[3];
        c[3] = t;
    };
    if (inside == 4) return T(1);
    if (inside == 3) {
        for (int r = 0; r < 4 && c[0] < T(0); ++r) rotate();
        T s0 = T(1) - fraction_inside(c[0], c[3]);
        T s1 = T(1) - fraction_inside(c[0], c[1]);
        return (T)dsub(1.0, dmul(dmul(0.5, (double)s0), (double)s1));
    }
    if (inside == 2) {
        for (int r = 0; r < 4 && (c[0] >= T(0) || !(c[1] < T(0) || c[2] < T(0))); ++r) rotate();
        if (c[1] < T(0)) {
            T left = fraction_inside(c[0], c[3]);
            T right = fraction_inside(c[1], c[2]);
            return (T)dmul(0.5, (double)(left + right));
        }
        T centre = (T)dmul(0.25, (double)(c[0] + c[1] + c[2] + c[3]));
        if (centre < T(0)) {
            T area = 0;
            T s1 = T(1) - fraction_inside(c[0], c[3]);
            T s3 = T(1) - fraction_inside(c[2], c[3]);
            area = (T)dadd((double)area, dmul(dmul(0.5, (double)s1), (double)s3));
            T s2 = T(1) - fraction_inside(c[2], c[1]);
            T s0 = T(1) - fraction_inside(c[0], c[1]);
            area = (T)dadd((double)area, dmul(dmul(0.5, (double)s0), (double)s2));
            return T(1) - area;
        }
        T area = 0;
        T s0 = fraction_inside(c[0], c[1]);
        T s1 = fraction_inside(c[0], c[3]);
        area = (T)dadd((double)area, dmul(dmul(0.5, (double)s0), (double)s1));
        T s2 = fraction_inside(c[2], c[1]);
        T s3 = fraction_inside(c[2], c[3]);
        area = (T)dadd((double)area, dmul(dmul(0.5, (double)s2), (double)s3));
        return area;
    }
    if (inside == 1) {
        for (int r = 0; r < 4 && c[0] >= T(0); ++r) rotate();
        T s0 = fraction_inside(c[0], c[3]);
        T s1 = fraction_inside(c[0], c[1]);
        return (T)dmul(dmul(0.5, (double)s0), (double)s1);
    }
    return T(0);
}

// compute_staggered_grid_weight (boundary.cpp:6-34): comp 0/1/2 = u/v/w faces.
template <typename T>
__global__ void weights_kernel(int ni, int nj, int nk, const T* __restrict__ solid, T* __restrict__ wt,
                               int comp) {
    const int n0 = ni + (comp == 0), n1 = nj + (comp == 1), n2 = nk + (comp == 2);
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    if (i >= n0 || j >= n1 || k >= n2) return;
    const int s0 = ni + 1, s1 = nj + 1;
    auto S = [&](int a, int b, int c) { return solid[lin3(a, b, c, s0, s1)]; };
    T f;
    if (comp == 0)
        f = fraction_inside4(S(i, j, k), S(i, j + 1, k), S(i, j, k + 1), S(i, j + 1, k + 1));
    else if (comp == 1)
        f = fraction_inside4(S(i, j, k), S(i, j, k + 1), S(i + 1, j, k), S(i + 1, j, k + 1));
    else
        f = fraction_inside4(S(i, j, k), S(i, j + 1, k), S(i + 1, j, k), S(i + 1, j + 1, k));
    T wv = T(1) - f;
    wv = wv < T(0) ? T(0) : (wv > T(1) ? T(1) : wv);
    wt[lin3(i, j, k, n0, n1)] = wv;
}

// calc_cell_centered_solid_phi (simulator.cpp:191-200) and find_valid_level_set (:160-167)
template <typename T>
__global__ void cell_solid_kernel(int ni, int nj, int nk, const T* __restrict__ solid, T* __restrict__ out,
                                  uint8_t* __restrict__ valid_phi) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    if (i >= ni || j >= nj) return;
    const int s0 = ni + 1, s1 = nj + 1;
    auto S = [&](int a, int b, int c) { return solid[lin3(a, b, c, s0, s1)]; };
    T sum = S(i, j, k) + S(i + 1, j, k);
    sum = sum + S(i, j + 1, k);
    sum = sum + S(i + 1, j + 1, k);
    sum = sum + S(i, j, k + 1);
    sum = sum + S(i + 1, j, k + 1);
    sum = sum + S(i, j + 1, k + 1);
    sum = sum + S(i + 1, j + 1, k + 1);
    const T v = (T)dmul((double)sum, 0.125);
    const long long c = lin3(i, j, k, ni, nj);
    out[c] = v;
    if (valid_phi) valid_phi[c] = v < T(0) ? 0 : 1;
}

template <typename T>
struct FaceView {
    const T* __restrict__ u;
    const T* __restrict__ v;
    const T* __restrict__ w;
    int ni, nj, nk;
    // read-only for the kernels that take a view: non-coherent loads, which the compiler may
    // issue ahead of the kernel's byte stores (a byte pointer may alias anything)
    __device__ __forceinline__ T U(int i, int j, int k) const { return __ldg(u + lin3(i, j, k, ni + 1, nj)); }
    __device__ __forceinline__ T V(int i, int j, int k) const { return __ldg(v + lin3(i, j, k, ni, nj + 1)); }
    __device__ __forceinline__ T W(int i, int j, int k) const { return __ldg(w + lin3(i, j, k, ni, nj)); }
};

// Cell flags (is_pressure_valid, projection.cpp:8-12; fluid = valid and phi < 0) and the
// fluid-cell count.
template <typename T>
__global__ void flags_kernel(FaceView<T> wt, const T* __restrict__ phi, uint8_t* __restrict__ flags,
                             Scalars* s, double* partials, unsigned* counter, int kz) {
    const int ni = wt.ni, nj = wt.nj, nk = wt.nk;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    int count = 0;  // an integer: one FP64 addition a cell was most of this kernel's FP64 pipe time
    if (i < ni && j < nj) {
        // a contiguous chunk of planes per block: the neighbour planes come from L1
        const int k_end = min(nk, (int)(blockIdx.z + 1) * kz);
#pragma unroll 4
        for (int k = blockIdx.z * kz; k < k_end; ++k) {
            const T w0 = wt.U(i, j, k), w1 = wt.U(i + 1, j, k), w2 = wt.V(i, j, k), w3 = wt.V(i, j + 1, k),
                    w4 = wt.W(i, j, k), w5 = wt.W(i, j, k + 1);
            const long long c = lin3(i, j, k, ni, nj);
            const T pc = __ldg(phi + c);
            const bool pv = w0 > T(0) || w1 > T(0) || w2 > T(0) || w3 > T(0) || w4 > T(0) || w5 > T(0);
            const bool fl = pv && pc < T(0);
            flags[c] = (pv ? kFlagPressureValid : 0) | (fl ? kFlagFluid : 0);
            count += fl ? 1 : 0;
        }
    }
    double cnt[1] = {(double)count};
    double tot[1];
    if (grid_sum<1>(cnt, partials, counter, tot)) s->count = (int)tot[0];
}

template <typename T>
struct CoeffOut {
    double* diag64;
    T* off[3];
    double* rhs64;
    // when set, also the mixed solver's FP32 records of the same row: {d, cx, cy, cz} as float4,
    // and as half4 with the diagonal rounded up and the couplings rounded toward zero
    float4* a32;
    ushort4* a16;
};

// build_matrix (projection.cpp:30-83), grid-shaped, plus |b|^2.
// The diagonal: its terms added in the neighbours' order in double from zero (an absent
// neighbour adds zero, which leaves the sum as it is).  FP32 fields: the exact integer sum where
// no addition rounds (exact_sum6, nearly every row: the terms are weights of at most a few
// powers of two apart), else the FP64 additions, out of line so that their instructions are not
// issued, predicated off, for every row.
__device__ __noinline__ double diag_sum_fp64(float t0, float t1, float t2, float t3, float t4, float t5) {
    double d = dadd(0.0, f2d(t0));
    d = dadd(d, f2d(t1));
    d = dadd(d, f2d(t2));
    d = dadd(d, f2d(t3));
    d = dadd(d, f2d(t4));
    return dadd(d, f2d(t5));
}

template <typename T>
__device__ __forceinline__ double diag_sum(const T (&t)[6]) {
    if constexpr (sizeof(T) == 4) {
        double d;
        if (exact_sum6(t[0], t[1], t[2], t[3], t[4], t[5], d)) return d;
        return diag_sum_fp64(t[0], t[1], t[2], t[3], t[4], t[5]);
    } else {
        double d = 0.0;
#pragma unroll
        for (int f = 0; f < 6; ++f) d = dadd(d, t[f]);
        return d;
    }
}

// four blocks of 256 per SM for FP32 fields (64 registers, no spills)
template <typename T>
__global__ void __launch_bounds__(256, sizeof(T) == 4 ? 4 : 2) build_kernel(FaceView<T> vel, FaceView<T> wt, const T* __restrict__ phi,
                             const uint8_t* __restrict__ flags, uint8_t* __restrict__ built, CoeffOut<T> o, T dx,
                             Scalars* s, double* partials, unsigned* counter, int kz) {
    const int ni = wt.ni, nj = wt.nj, nk = wt.nk;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const T dt = (T)s->dt;
    const T scale = dx / dt;
    // |b|^2: squares of the float-rounded b summed in FP32 per thread (a thread takes one column
    // of kz cells; SqAcc keeps every square in range) and in FP64 over the grid -- FP64
    // arithmetic per cell is what bounds this kernel
    SqAcc bbs;
    if (i < ni && j < nj) {
        // a contiguous chunk of planes per block: the neighbour planes come from L1; every load
        // is a read-only one (the flags are not written here)
        const int k_end = min(nk, (int)(blockIdx.z + 1) * kz);
        for (int k = blockIdx.z * kz; k < k_end; ++k) {
            const long long c = lin3(i, j, k, ni, nj);
            const uint8_t fc = __ldg(flags + c);
            const bool fluid = (fc & kFlagFluid) != 0;
            // a row that is zero now and was zero after the previous build is left as it is
            // (built: the marker of rows the build may have left nonzero, null where the outputs'
            // contents are not known and every row is written)
            const uint8_t bc = built ? built[c] : (uint8_t)1;
            if (!fluid && !bc) continue;
            double d = 0.0, b = 0.0;
            T offv[3] = {T(0), T(0), T(0)};  // exactly -weight: no rounding, so in the field type
            if (fluid) {
                // every load of the row first (a neighbour outside the grid reads the cell itself
                // and is masked), so that a thread waits for memory once per row
                const long long s1 = ni, s2 = (long long)ni * nj;
                const bool inb[6] = {i > 0, i + 1 < ni, j > 0, j + 1 < nj, k > 0, k + 1 < nk};
                const long long off[6] = {-1, 1, -s1, s1, -s2, s2};
                uint8_t nf[6];
                T np[6];
#pragma unroll
                for (int f = 0; f < 6; ++f) {
                    const long long q = inb[f] ? c + off[f] : c;
                    nf[f] = __ldg(flags + q);
                    np[f] = __ldg(phi + q);
                }
                const T pc = __ldg(phi + c);
                const T fv[6] = {vel.U(i, j, k), vel.U(i + 1, j, k), vel.V(i, j, k),
                                 vel.V(i, j + 1, k), vel.W(i, j, k), vel.W(i, j, k + 1)};
                const T fw[6] = {wt.U(i, j, k), wt.U(i + 1, j, k), wt.V(i, j, k),
                                 wt.V(i, j + 1, k), wt.W(i, j, k), wt.W(i, j, k + 1)};
                // the diagonal's terms (zero for a neighbour that adds none), summed below
                T dterm[6] = {T(0), T(0), T(0), T(0), T(0), T(0)};
#pragma unroll
                for (int f = 0; f < 6; ++f) {
                    const T weight = fw[f];
                    if (inb[f] && (nf[f] & kFlagPressureValid)) {
                        const T pn = np[f];
                        if (pn < T(0)) {
                            dterm[f] = weight;
                            if (f & 1) offv[f >> 1] = -weight;
                        } else {
                            T theta = fraction_inside(pc, pn);
                            theta = theta < T(0.01) ? T(0.01) : theta;
                            dterm[f] = weight / theta;
                        }
                    }
                    // b: + for the lower face, - for the upper one, in the neighbours' order
                    const double prod = f2d(mul_rn(weight, fv[f]));
                    b = (f & 1) ? dsub(b, prod) : dadd(b, prod);
                }
                b = dmul(b, f2d(scale));
                d = diag_sum(dterm);
            }
            if (!EL_IN(c, (long long)ni * nj * nk, 40)) continue;
            o.diag64[c] = d;
            o.rhs64[c] = b;
#pragma unroll
            for (int a = 0; a < 3; ++a) o.off[a][c] = offv[a];
            if (o.a32) {
                const float4 r = make_float4(d2f(d), (float)offv[0], (float)offv[1], (float)offv[2]);
                o.a32[c] = r;
                o.a16[c] = make_ushort4(__half_as_ushort(__float2half_ru(r.x)), __half_as_ushort(__float2half_rz(r.y)),
                                        __half_as_ushort(__float2half_rz(r.z)), __half_as_ushort(__float2half_rz(r.w)));
            }
            if (built && (fluid ? 1 : 0) != bc) built[c] = fluid ? 1 : 0;
            bbs.add(d2f(b));
        }
    }
    double bb[1] = {bbs.value()};
    double tot[1];
    if (grid_sum<1>(bb, partials, counter, tot)) s->bb = tot[0];
}

// assign_indices (projection.cpp:14-28): exclusive scan of the fluid flag in linear (k-j-i)
// order.  Three passes over chunks of kScanChunk cells.
constexpr int kScanChunk = 2048;
constexpr int kScanThreads = 256;

__global__ void scan_count_kernel(const uint8_t* __restrict__ flags, long long n, int* __restrict__ chunk_counts) {
    __shared__ int sh[kScanThreads / 32];
    const long long base = (long long)blockIdx.x * kScanChunk;
    int cnt = 0;
    for (int q = threadIdx.x; q < kScanChunk; q += blockDim.x) {
        const long long c = base + q;
        if (c < n && (flags[c] & kFlagFluid)) ++cnt;
    }
    for (int o = 16; o > 0; o >>= 1) cnt += __shfl_down_sync(0xffffffffu, cnt, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = cnt;
    __syncthreads();
    if (threadIdx.x == 0) {
        int t = 0;
        for (int w = 0; w < kScanThreads / 32; ++w) t += sh[w];
        chunk_counts[blockIdx.x] = t;
    }
}

__global__ void scan_chunks_kernel(int* __restrict__ chunk_counts, int nchunks, int* __restrict__ total) {
    // single block: sequential-per-thread spans, then a block scan of span sums
    __shared__ int span[1024];
    const int per = (nchunks + blockDim.x - 1) / blockDim.x;
    const int lo = threadIdx.x * per, hi = min(nchunks, lo + per);
    int s = 0;
    for (int q = lo; q < hi; ++q) s += chunk_counts[q];
    span[threadIdx.x] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        int run = 0;
        for (int t = 0; t < (int)blockDim.x; ++t) {
            const int v = span[t];
            span[t] = run;
            run += v;
        }
        *total = run;
    }
    __syncthreads();
    int run = span[threadIdx.x];
    for (int q = lo; q < hi; ++q) {
        const int v = chunk_counts[q];
        chunk_counts[q] = run;
        run += v;
    }
}

__global__ void scan_write_kernel(const uint8_t* __restrict__ flags, long long n,
                                  const int* __restrict__ chunk_offsets, int* __restrict__ indices) {
    // one warp walks the chunk in 32-cell steps keeping a running offset
    const long long base = (long long)blockIdx.x * kScanChunk;
    const int lane = threadIdx.x;
    int run = chunk_offsets[blockIdx.x];
    for (int q = 0; q < kScanChunk; q += 32) {
        const long long c = base + q + lane;
        const bool fl = c < n && (flags[c] & kFlagFluid);
        const unsigned m = __ballot_sync(0xffffffffu, fl);
        if (c < n) indices[c] = fl ? run + __popc(m & ((1u << lane) - 1u)) : kIndexUnknown;
        run += __popc(m);
    }
}

// a double into the field type (the float conversion on the integer pipe)
template <typename T>
__device__ __forceinline__ T to_field(double v) {
    if constexpr (sizeof(T) == 4)
        return d2f(v);
    else
        return v;
}

// build_grid_from_vector (projection.cpp:85-91): pressure = p on fluid cells, 0 elsewhere.
template <typename T>
__global__ void scatter_pressure_kernel(long long n, const double* __restrict__ x,
                                        const uint8_t* __restrict__ flags, T* __restrict__ p) {
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n;
         c += (long long)gridDim.x * blockDim.x)
        p[c] = (flags[c] & kFlagFluid) ? to_field<T>(x[c]) : T(0);
}

// update_velocity_using_pressure (projection.cpp:93-134): faces with index in [1, n) along
// their normal and [1, n-1) along the two tangential axes, as the reference's loops.
// one face given the level set and pressure of its two cells (a: below, b: above)
template <typename T>
__device__ __forceinline__ void update_face(T pa, T pb, T qa, T qb, long long fi, T* __restrict__ f, T dt, T dx) {
    if (pb < T(0) || pa < T(0)) {
        T theta = T(1);
        if (pb >= T(0) || pa >= T(0)) theta = fraction_inside(pa, pb);
        theta = theta < T(0.01) ? T(0.01) : theta;
        const T num = mul_rn(dt, qb - qa);
        const T den = mul_rn(dx, theta);
        f[fi] = f[fi] - num / den;
    }
}

// The three components in one launch: a thread takes the faces u, v and w at (i, j, k) down a
// column, each within its component's range, so that the pressure and the level set are read
// once for all three (their neighbouring cells' values come from L1); the loads of a cell's
// faces are issued together.
template <typename T>
__global__ void update_velocity3_kernel(int ni, int nj, int nk, T* __restrict__ u, T* __restrict__ v,
                                        T* __restrict__ w, const T* __restrict__ p, const T* __restrict__ phi, T dx,
                                        const Scalars* s, double dt_value, int kz) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
    if (i >= ni || j >= nj) return;
    const T dt = (T)(s ? s->dt : dt_value);
    const long long plane = (long long)ni * nj;
#pragma unroll
    for (int kk = 0; kk < kz; ++kk) {
        const int k = blockIdx.z * kz + kk + 1;
        if (k >= nk) break;
        // u: i in [1, ni), j in [1, nj - 1), k in [1, nk - 1); v and w likewise
        const bool hu = j < nj - 1 && k < nk - 1, hv = i < ni - 1 && k < nk - 1, hw = i < ni - 1 && j < nj - 1;
        const long long b = lin3(i, j, k, ni, nj);
        const T pc = __ldg(phi + b), qc = __ldg(p + b);
        const T pxm = hu ? __ldg(phi + b - 1) : T(0), qxm = hu ? __ldg(p + b - 1) : T(0);
        const T pym = hv ? __ldg(phi + b - ni) : T(0), qym = hv ? __ldg(p + b - ni) : T(0);
        const T pzm = hw ? __ldg(phi + b - plane) : T(0), qzm = hw ? __ldg(p + b - plane) : T(0);
        if (hu) update_face(pxm, pc, qxm, qc, lin3(i, j, k, ni + 1, nj), u, dt, dx);
        if (hv) update_face(pym, pc, qym, qc, lin3(i, j, k, ni, nj + 1), v, dt, dx);
        if (hw) update_face(pzm, pc, qzm, qc, lin3(i, j, k, ni, nj), w, dt, dx);
    }
}

// ---------------------------------------------------------------------------------------
// launchers

static dim3 plane_grid(int n0, int n1, int n2, dim3 block) {
    return dim3((n0 + block.x - 1) / block.x, (n1 + block.y - 1) / block.y, n2);
}

template <typename T>
void launch_weights_t(int ni, int nj, int nk, const void* solid, void* wu, void* wv, void* ww, cudaStream_t s) {
    dim3 block(32, 4, 1);
    weights_kernel<T><<<plane_grid(ni + 1, nj, nk, block), block, 0, s>>>(ni, nj, nk, (const T*)solid, (T*)wu, 0);
    weights_kernel<T><<<plane_grid(ni, nj + 1, nk, block), block, 0, s>>>(ni, nj, nk, (const T*)solid, (T*)wv, 1);
    weights_kernel<T><<<plane_grid(ni, nj, nk + 1, block), block, 0, s>>>(ni, nj, nk, (const T*)solid, (T*)ww, 2);
}

int launch_weights(int dtype, int ni, int nj, int nk, const void* solid, void* wu, void* wv, void* ww,
                   cudaStream_t s) {
    if (dtype == EL_F64)
        launch_weights_t<double>(ni, nj, nk, solid, wu, wv, ww, s);
    else
        launch_weights_t<float>(ni, nj, nk, solid, wu, wv, ww, s);
    return 3;
}

int launch_cell_solid(el_ctx* ctx) {
    dim3 block(32, 4, 1);
    dim3 grid = plane_grid(ctx->ni, ctx->nj, ctx->nk, block);
    uint8_t* vphi = (uint8_t*)ctx->field[EL_FIELD_VALID_PHI];
    if (ctx->dtype == EL_F64)
        cell_solid_kernel<double><<<grid, block, 0, ctx->stream>>>(
            ctx->ni, ctx->nj, ctx->nk, (const double*)ctx->field[EL_FIELD_SOLID_NODAL],
            (double*)ctx->field[EL_FIELD_SOLID_CELL], vphi);
    else
        cell_solid_kernel<float><<<grid, block, 0, ctx->stream>>>(
            ctx->ni, ctx->nj, ctx->nk, (const float*)ctx->field[EL_FIELD_SOLID_NODAL],
            (float*)ctx->field[EL_FIELD_SOLID_CELL], vphi);
    return 1;
}

static Geom plane_geom(el_ctx* ctx) {
    Geom g = stencil_geom(ctx->ni, ctx->nj, ctx->nk, ctx->num_sms, ctx->stencil_per_sm);
    return g;
}

template <typename T>
static int launch_flags_build_t(el_ctx* ctx, bool inner32, bool build) {
    Geom g = plane_geom(ctx);
    FaceView<T> wt{(const T*)ctx->field[EL_FIELD_WEIGHT_U], (const T*)ctx->field[EL_FIELD_WEIGHT_V],
                   (const T*)ctx->field[EL_FIELD_WEIGHT_W], ctx->ni, ctx->nj, ctx->nk};
    FaceView<T> vel{(const T*)ctx->field[EL_FIELD_U], (const T*)ctx->field[EL_FIELD_V],
                    (const T*)ctx->field[EL_FIELD_W], ctx->ni, ctx->nj, ctx->nk};
    const T* phi = (const T*)ctx->field[EL_FIELD_PHI];
    flags_kernel<T><<<g.grid, g.block, 0, ctx->stream>>>(wt, phi, ctx->flags, ctx->dscal, ctx->partials,
                                                         ctx->counter, g.kz);
    if (!build) return 1;
    CoeffOut<T> o;
    o.diag64 = ctx->diag64;
    o.rhs64 = ctx->rhs64;
    for (int a = 0; a < 3; ++a) o.off[a] = (T*)ctx->off[a];
    // the mixed solver's records written by the build itself (no separate packing pass)
    const bool records = inner32 && ctx->A32 && ctx->A16;
    o.a32 = records ? ctx->A32 : nullptr;
    o.a16 = records ? ctx->A16 : nullptr;
    ctx->records_fresh = records;
    build_kernel<T><<<g.grid, g.block, 0, ctx->stream>>>(vel, wt, phi, ctx->flags, ctx->build_skip_zero ? ctx->built : nullptr,
                                                         o, (T)ctx->dx, ctx->dscal, ctx->partials, ctx->counter, g.kz);
    return 2;
}

int launch_flags_build(el_ctx* ctx, bool inner32, bool build) {
    return ctx->dtype == EL_F64 ? launch_flags_build_t<double>(ctx, inner32, build)
                                : launch_flags_build_t<float>(ctx, inner32, build);
}

int launch_assign_indices(el_ctx* ctx, int* d_chunks, int* d_total) {
    const long long n = (long long)ctx->ni * ctx->nj * ctx->nk;
    const int nchunks = (int)((n + kScanChunk - 1) / kScanChunk);
    scan_count_kernel<<<nchunks, kScanThreads, 0, ctx->stream>>>(ctx->flags, n, d_chunks);
    scan_chunks_kernel<<<1, 1024, 0, ctx->stream>>>(d_chunks, nchunks, d_total);
    scan_write_kernel<<<nchunks, 32, 0, ctx->stream>>>(ctx->flags, n, d_chunks, (int*)ctx->field[EL_FIELD_INDICES]);
    return 3;
}

int launch_scatter_pressure(el_ctx* ctx) {
    const long long n = (long long)ctx->ni * ctx->nj * ctx->nk;
    const int blocks = (int)std::min<long long>((n + 255) / 256, (long long)ctx->num_sms * 16);
    if (ctx->dtype == EL_F64)
        scatter_pressure_kernel<double><<<blocks, 256, 0, ctx->stream>>>(n, ctx->x64, ctx->flags,
                                                                         (double*)ctx->field[EL_FIELD_PRESSURE]);
    else
        scatter_pressure_kernel<float><<<blocks, 256, 0, ctx->stream>>>(n, ctx->x64, ctx->flags,
                                                                        (float*)ctx->field[EL_FIELD_PRESSURE]);
    return 1;
}

template <typename T>
static int launch_update_velocity_t(el_ctx* ctx, const Scalars* s, double dtv) {
    const int ni = ctx->ni, nj = ctx->nj, nk = ctx->nk;
    if (ni <= 1 || nj <= 1 || nk <= 1) return 0;
    dim3 block(32, 8, 1);
    constexpr int kz = 8;
    dim3 grid = plane_grid(ni - 1, nj - 1, (nk - 1 + kz - 1) / kz, block);
    update_velocity3_kernel<T><<<grid, block, 0, ctx->stream>>>(
        ni, nj, nk, (T*)ctx->field[EL_FIELD_U], (T*)ctx->field[EL_FIELD_V], (T*)ctx->field[EL_FIELD_W],
        (const T*)ctx->field[EL_FIELD_PRESSURE], (const T*)ctx->field[EL_FIELD_PHI], (T)ctx->dx, s, dtv, kz);
    return 1;
}

int launch_update_velocity(el_ctx* ctx, const Scalars* s, double dtv) {
    return ctx->dtype == EL_F64 ? launch_update_velocity_t<double>(ctx, s, dtv)
                                : launch_update_velocity_t<float>(ctx, s, dtv);
}

EL_CHECK_EXPORT(project)

}  // namespace el
