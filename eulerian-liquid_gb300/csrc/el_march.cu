// el_march.cu -- the finest level of the FP32 multigrid PCG (the mixed-precision solver's inner
// iterations) as z-marching tile kernels with TMA-staged halo planes.
//
// The segment kernels of el_solve.cu give every warp one 32-cell row and fetch its +-y and +-z
// rows again from L2; those rows are shared with four other warps, so each stencil value is
// read about five times and the kernels wait on L2 latency.  Here a CTA owns a tile of 32 (i) x
// 16 (j) cells and marches it along k: every plane of every staged array arrives once, by one
// cp.async.bulk.tensor copy of a 40 x 18 box (the tile, one row above and below, four cells left
// and right so that the box starts on a 16-byte boundary; a record box one or two cells, its
// nearest boundary) into a ring of shared-memory plane buffers, and the 7-point stencil reads its -z / centre / +z planes and its +-y rows from
// shared memory.  Copies of the next planes are in flight while a plane is computed (one
// mbarrier per ring slot, transaction-counted); the box's parts outside the grid arrive as
// zeros, which is the zero value and zero coupling the segment kernels use there.
//
// A CTA is eight compute warps (one per tile row) and a producer warp whose one thread issues
// the copies: full / empty mbarrier pairs per ring slot, no CTA-wide barrier per plane.  CTAs
// take the work items round robin, so the CTAs running at any moment hold neighbouring tiles of
// the same planes and read each other's halo rows from L2 rather than from DRAM; a CTA's planes
// stream in one sequence across its items.  (Splitting the items of the last, partly filled
// round into equal plane runs over all CTAs measured 3.5 % slower: each run stages two more
// planes, and the kernels are bound by the planes they move, not by the CTAs left in the tail.)
//
// Kernels (one launch each, over the work items of el::MarchPlan):
//   DIRSPMV   p' = z + beta p ; Ap' ; p'.Ap'                            (K1 of a PCG iteration)
//   UPDZ      x += alpha p ; r' = r - alpha Ap ; |r'|^2 ; and the first two smoothing sweeps of
//             the V-cycle on r', from zero (update fused with the pre-smoother: r' is formed
//             from r and Ap in shared memory wherever the stencil needs it)
//   ZERO2     the two sweeps from zero alone (the V-cycle that starts a refinement sweep)
//   RESTRICT  residual of the pre-smoothed level summed over 2x2x2 blocks onto the coarse rhs
//   PROLONG   one sweep from x + P e (e = the coarse correction)
//   LAST      the last sweep, and r.z for beta
// The expressions and their order are those of el_solve.cu's dir_spmv_rec_kernel,
// update_kernel, smooth_kernel and restrict_kernel; only the dot products' summation order
// differs (per CTA instead of per segment warp).
//
// Conditions (el::march_supported): the finest level's rows are a multiple of 16 bytes (ni a
// multiple of 8, so that the next level's rows are too) -- a tensor map's strides must be.
// Other grids keep the segment kernels.

#include <cuda.h>
#include <cuda_fp16.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cstring>

#include "el_internal.cuh"
#include "el_tma.cuh"

namespace el {

namespace {

constexpr int kTI = 32;          // tile cells along i (one warp's lanes)
constexpr int kTJ = 16;          // tile rows along j (two per compute warp)
constexpr int kHX = 40;          // staged row: i0 - 4 .. i0 + 35
constexpr int kHY = kTJ + 2;     // staged rows: j0 - 1 .. j0 + 16
constexpr int kCX = 24;          // staged coarse row: i0/2 - 4 .. i0/2 + 19
constexpr int kCY = kTJ / 2 + 2; // staged coarse rows: j0/2 - 1 .. j0/2 + 8
constexpr int kComputeWarps = kTJ / 2;             // rows 2w and 2w + 1 each
constexpr int kThreads = 32 * (kComputeWarps + 1);  // and one producer warp
constexpr int kMaxStages = 6;    // plane buffers in the ring: three in use, the rest in flight
constexpr int kMVW = kTI + 2;    // masked-value plane: columns i0 - 1 .. i0 + 32 of the staged rows
constexpr unsigned kFull = 0xffffffffu;

enum Mode { DIRSPMV = 0, UPDZ = 1, ZERO2 = 2, RESTRICT = 3, PROLONG = 4, LAST = 5 };

// staged arrays of a mode: halo f32 arrays (40 x 18), the record halo (float4 or half4 records,
// 34 / 36 x 18), centre f32 arrays (32 x 16), the coarse box (24 x 10)
template <int M>
struct Layout {
    static constexpr int nhalo = M == DIRSPMV ? 2 : (M == UPDZ ? 2 : 1);
    static constexpr int ncentre = M == UPDZ ? 2 : (M == ZERO2 || M == DIRSPMV ? 0 : 1);
    static constexpr bool coarse = M == PROLONG;
    static constexpr bool f4 = M == DIRSPMV;  // float4 records (the PCG operator), else half4
    static constexpr int rec_bytes = f4 ? 16 : 8;
    // the record box starts one (float4) or two (half4) cells left of the tile, the nearest
    // 16-byte boundary, and ends as far right of it
    static constexpr int rec_x0 = f4 ? 1 : 2;
    static constexpr int rec_w = kTI + 2 * rec_x0;                // 34 / 36
    static constexpr int halo_bytes = kHX * kHY * 4;             // 2880
    static constexpr int rec_box_bytes = rec_w * kHY * rec_bytes; // 9792 / 5184
    static constexpr int centre_bytes = kTI * kTJ * 4;           // 2048
    static constexpr int coarse_bytes = kCX * kCY * 4;           // 960
    // ZERO2 and UPDZ read the first sweep's values x1 = w1 b / D (0 where D is not positive) at
    // all seven stencil points: those of a plane are formed once, when it lands.  The other modes
    // read stored vectors, which are finite everywhere, and a coupling with a cell outside the
    // system is zero, so their neighbour values need no mask (as in DIRSPMV)
    static constexpr bool mv = M == UPDZ || M == ZERO2;
    static constexpr int mv_bytes = kMVW * kHY * 4;              // 2448
    static constexpr int al(int b) { return (b + 127) / 128 * 128; }
    static constexpr int off_rec = 0;
    static constexpr int off_halo = al(rec_box_bytes);
    static constexpr int off_centre = off_halo + nhalo * al(halo_bytes);
    static constexpr int off_coarse = off_centre + ncentre * al(centre_bytes);
    static constexpr int off_mv = off_coarse + (coarse ? al(coarse_bytes) : 0);
    static constexpr int stage = al(off_mv + (mv ? mv_bytes : 0));
    // six slots; five for ZERO2 (four of its CTAs fit an SM); four for UPDZ (three CTAs per SM
    // instead of two: 0.67 -> 0.70 of HBM; the same for DIRSPMV, RESTRICT or LAST measured slower)
    static constexpr int stages = M == ZERO2 ? 5 : (M == UPDZ ? 4 : 6);
    static constexpr int smem = 128 + stages * stage + 128;  // barriers first; alignment slack
    // the CTAs an SM holds by shared memory, which the register budget must not lower
    static constexpr int min_blocks = M == ZERO2 ? 4 : (M == DIRSPMV ? 2 : 3);
    static_assert(stages <= kMaxStages && 2 * kMaxStages * 8 <= 128, "barriers fit in front of the ring");
};

struct Maps {
    CUtensorMap halo[2];
    CUtensorMap rec;
    CUtensorMap centre[2];
    CUtensorMap coarse;
};

struct Args {
    int n0, n1, n2;             // the level
    int c0, c1, c2;             // the next coarser level (RESTRICT, PROLONG)
    const int4* items;
    const int* count;
    float* out0;
    float* out1;
    float* out2;
    Scalars* s;
    double* partials;
    unsigned* counter;
    int first;                  // DIRSPMV: first iteration (p' = z)
    int dot;                    // LAST: DOT_INIT (1) or DOT_BETA (2)
};

__device__ __forceinline__ float mg_divf(float a, float b) { return __fdividef(a, b); }

// named barrier 1 over the compute warps (the producer warp does not take part), returning the
// OR of `pred` over them: the same value in every compute warp
__device__ __forceinline__ bool compute_barrier_or(int pred) {
    unsigned r;
    asm volatile(
        "{\n\t.reg .pred p, q;\n\t"
        "setp.ne.u32 p, %1, 0;\n\t"
        "barrier.cta.red.or.pred q, 1, %2, p;\n\t"
        "selp.u32 %0, 1, 0, q;\n\t}"
        : "=r"(r)
        : "r"(pred), "r"(32 * kComputeWarps)
        : "memory");
    return r != 0;
}

// records of a staged plane: {diagonal, +x, +y, +z couplings}
struct Rc {
    float d, x, y, z;
};
__device__ __forceinline__ Rc ld_rec(const unsigned char* base, int idx, int bytes) {
    if (bytes == 16) {
        const float4 v = reinterpret_cast<const float4*>(base)[idx];
        return {v.x, v.y, v.z, v.w};
    }
    const ushort4 v = reinterpret_cast<const ushort4*>(base)[idx];
    return {__half2float(__ushort_as_half(v.x)), __half2float(__ushort_as_half(v.y)),
            __half2float(__ushort_as_half(v.z)), __half2float(__ushort_as_half(v.w))};
}

// the 7 values and couplings of one cell's stencil; value(plane, y, x) is a staged value with
// plane 0 = k-1, 1 = k, 2 = k+1 and (y, x) staged-box coordinates
struct S7 {
    float v0, vxm, vxp, vym, vyp, vzm, vzp;
    float d, cxm, cxp, cym, cyp, czm, czp;
};
__device__ __forceinline__ float apply7(const S7& st) {
    return stencil7(st.d, st.v0, st.cxm, st.vxm, st.cxp, st.vxp, st.cym, st.vym, st.cyp, st.vyp, st.czm, st.vzm,
                    st.czp, st.vzp);
}

template <int M>
__device__ __forceinline__ unsigned char* stage_ptr(unsigned char* smem, int slot) {
    return smem + 128 + slot * Layout<M>::stage;
}

}  // namespace

// ---------------------------------------------------------------------------------------

// a half record's diagonal is positive: sign bit clear and not zero
__device__ __forceinline__ bool dpos(const unsigned char* rec, int idx, int bytes) {
    if (bytes == 16) return reinterpret_cast<const float4*>(rec)[idx].x > 0.f;
    return static_cast<short>(reinterpret_cast<const ushort4*>(rec)[idx].x) > 0;
}

template <int M>
__global__ void __launch_bounds__(kThreads, Layout<M>::min_blocks) march_kernel(const __grid_constant__ Maps maps,
                                                                             const Args a) {
    using L = Layout<M>;
    Scalars* s = a.s;
    pdl_wait();
    pdl_trigger();
    if (s->done) return;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    unsigned char* smem = align128(smem_raw);
    uint64_t* full = reinterpret_cast<uint64_t*>(smem);   // a plane landed (transaction count)
    constexpr int kStages = L::stages;
    uint64_t* empty = full + kMaxStages;                  // every compute warp is done with it
    __shared__ volatile int abort_flag;
    const int tid = threadIdx.x;
    const int lane = tid & 31, w = tid >> 5;
    const int n = *a.count;
    const int G = gridDim.x, b = blockIdx.x;
    if (tid == 0) {
        abort_flag = 0;
        for (int q = 0; q < kStages; ++q) {
            mbar_init(&full[q], 1);
            mbar_init(&empty[q], kComputeWarps);
        }
        mbar_init_fence();
    }
    __syncthreads();
    float part = 0.f;  // this thread's share of the mode's dot product

    if (w == kComputeWarps) {
        // ---- producer warp: one thread streams the planes of this CTA's items ------------
        if (lane == 0) {
            const int nhalo = (M == DIRSPMV && a.first) ? 1 : L::nhalo;
            const unsigned tx = (unsigned)(L::rec_box_bytes + nhalo * L::halo_bytes + L::ncentre * L::centre_bytes +
                                           (L::coarse ? L::coarse_bytes : 0));
            int slot = 0, round = 0, issued = 0;
            for (int it = b; it < n && !abort_flag; it += G) {
                const int4 d = a.items[it];
                const int i0 = d.x, j0 = d.y;
                for (int k = d.z - 1; k <= d.w; ++k) {
                    // the slot's previous plane must have been released by every compute warp
                    if (round > 0 && !mbar_wait(&empty[slot], (unsigned)((round - 1) & 1))) {
                        abort_flag = 1;
                        break;
                    }
                    unsigned char* st = stage_ptr<M>(smem, slot);
                    uint64_t* bar = &full[slot];
                    mbar_expect_tx(bar, tx);
                    tma_load_3d(st + L::off_rec, &maps.rec, bar, 4 * (i0 - L::rec_x0), j0 - 1, k);
                    for (int h = 0; h < nhalo; ++h)
                        tma_load_3d(st + L::off_halo + h * L::al(L::halo_bytes), &maps.halo[h], bar, i0 - 4, j0 - 1, k);
                    for (int c = 0; c < L::ncentre; ++c)
                        tma_load_3d(st + L::off_centre + c * L::al(L::centre_bytes), &maps.centre[c], bar, i0, j0, k);
                    if (L::coarse) tma_load_3d(st + L::off_coarse, &maps.coarse, bar, i0 / 2 - 4, j0 / 2 - 1, k >> 1);
                    ++issued;
                    if (++slot == kStages) {
                        slot = 0;
                        ++round;
                    }
                }
            }
            if (abort_flag) {
                // a fault: no copy may still be in flight when the CTA's shared memory goes
                for (int q = (issued > kStages ? issued - kStages : 0); q < issued; ++q)
                    mbar_wait(&full[q % kStages], (unsigned)((q / kStages) & 1));
            }
        }
    } else {
        // ---- compute warps: warp w owns rows j0 + 2w and j0 + 2w + 1, lane l cell i0 + l ---
        const float alpha = (M == UPDZ) ? (float)s->alpha : 0.f;
        const float beta = (M == DIRSPMV && !a.first) ? (float)s->beta : 0.f;
        const float w1 = (float)kSweep1, w2 = (float)kSweep2;
        bool ok = true;
        int wslot = 0;        // the next plane to wait for: its slot and phase parity
        unsigned wpar = 0;
        int rslot = 0;        // the next plane to release
        auto wait_next = [&]() -> int {
            const int sl = wslot;
            if (ok && !mbar_wait(&full[sl], wpar)) {
                ok = false;
                abort_flag = 1;
            }
            if (++wslot == kStages) {
                wslot = 0;
                wpar ^= 1u;
            }
            return sl;
        };
        auto release_next = [&]() {
            __syncwarp();
            if (lane == 0) mbar_arrive(&empty[rslot]);
            if (++rslot == kStages) rslot = 0;
        };
        // the masked values of a landed plane, by all compute warps, then a barrier of the
        // compute warps.  A wait that ran out does not skip the barrier: every compute warp meets
        // it, and the barrier ORs the warps' abort state, so that all of them stop together.
        bool stop = false;
        auto prepass = [&](int sl) {
            if constexpr (L::mv) {
                unsigned char* Pp = stage_ptr<M>(smem, sl);
                const float* h0 = reinterpret_cast<const float*>(Pp + L::off_halo);
                const float* h1 = reinterpret_cast<const float*>(Pp + L::off_halo + L::al(L::halo_bytes));
                float* mvp = reinterpret_cast<float*>(Pp + L::off_mv);
                for (int e = w * 32 + lane; e < kMVW * kHY; e += 32 * kComputeWarps) {
                    const int hy = e / kMVW, hx = e - hy * kMVW + 3;    // in the staged value box
                    const int ridx = hy * L::rec_w + (hx - 4) + L::rec_x0;  // the same cell's record
                    float out = 0.f;
                    if (dpos(Pp + L::off_rec, ridx, L::rec_bytes)) {
                        float raw = h0[hy * kHX + hx];
                        if (M == UPDZ) raw = raw - alpha * h1[hy * kHX + hx];
                        out = mg_divf(rn_mul(w1, raw), ld_rec(Pp + L::off_rec, ridx, L::rec_bytes).d);
                    }
                    mvp[e] = out;
                }
                stop = compute_barrier_or(!ok || abort_flag != 0);
            }
        };
        auto aborted = [&]() -> bool { return L::mv ? stop : !ok; };
        for (int it = b; it < n && !aborted(); it += G) {
            const int4 d = a.items[it];
            const int i0 = d.x, j0 = d.y, k0 = d.z, k1 = d.w;
            const int i = i0 + lane;
            int sa = wait_next();  // plane k0 - 1
            prepass(sa);
            int sb = wait_next();  // plane k0
            prepass(sb);
            float racc0 = 0.f;                     // RESTRICT: this lane's 2x2 (j, k) sum
            for (int k = k0; k < k1; ++k) {
                const int sc = wait_next();        // plane k + 1
                prepass(sc);
                if (aborted()) break;
                const unsigned char* P[3] = {stage_ptr<M>(smem, sa), stage_ptr<M>(smem, sb), stage_ptr<M>(smem, sc)};
                auto MV = [&](int pl, int idx) -> float {
                    return reinterpret_cast<const float*>(P[pl] + L::off_mv)[idx];
                };
                auto H = [&](int pl, int h, int idx) -> float {
                    return reinterpret_cast<const float*>(P[pl] + L::off_halo + h * L::al(L::halo_bytes))[idx];
                };
                auto Cn = [&](int c, int row) -> float {
                    return reinterpret_cast<const float*>(P[1] + L::off_centre + c * L::al(L::centre_bytes))[row * kTI + lane];
                };
                auto R = [&](int pl, int idx) -> Rc { return ld_rec(P[pl] + L::off_rec, idx, L::rec_bytes); };
                float res[2];  // RESTRICT: the two rows' residuals
                // the stencils of the thread's two rows first, then their arithmetic in packed
                // float2 operations (lane r = row 2w + r; each lane rounded as the scalar
                // operations of stencil7 and the sweeps, so the results are those of the scalar
                // expressions)
                S7 sts[2];
                float bcs[2];
#pragma unroll
                for (int r = 0; r < 2; ++r) {
                    const int row = 2 * w + r;
                    const int hc = (row + 1) * kHX + lane + 4;               // in a staged value box
                    const int rc = (row + 1) * L::rec_w + lane + L::rec_x0;  // in the staged record box
                    // records of the stencil: the cell's own ({d, +x, +y, +z}), and the -x, -y,
                    // -z neighbours' (their +x/+y/+z couplings are the cell's -x/-y/-z ones)
                    const Rc r0 = R(1, rc);
                    S7& st = sts[r];
                    st.d = r0.d;
                    st.cxp = r0.x;
                    st.cyp = r0.y;
                    st.czp = r0.z;
                    st.cxm = R(1, rc - 1).x;
                    st.cym = R(1, rc - L::rec_w).y;
                    st.czm = R(0, rc).z;
                    // stencil points: centre, -x, +x, -y, +y (plane k), -z (k - 1), +z (k + 1)
                    const int vo[7] = {0, -1, 1, -kHX, kHX, 0, 0};
                    const int pq[7] = {1, 1, 1, 1, 1, 0, 2};
                    float v[7];
                    if (M == DIRSPMV) {
                        // p' = z + beta p at every stencil point
#pragma unroll
                        for (int q = 0; q < 7; ++q) {
                            const float zq = H(pq[q], 0, hc + vo[q]);
                            v[q] = a.first ? zq : zq + beta * H(pq[q], 1, hc + vo[q]);
                        }
                        bcs[r] = 0.f;
                    } else if constexpr (L::mv) {
                        // ZERO2 / UPDZ read the stencil's first-sweep values x1 = w1 b / D from
                        // the planes' masked values, with b = r' = r - alpha Ap (UPDZ) or b (ZERO2)
                        const int e0 = (row + 1) * kMVW + lane + 1;
                        const int mo[7] = {0, -1, 1, -kMVW, kMVW, 0, 0};
#pragma unroll
                        for (int q = 0; q < 7; ++q) v[q] = MV(pq[q], e0 + mo[q]);
                        bcs[r] = M == UPDZ ? H(1, 0, hc) - alpha * H(1, 1, hc) : H(1, 0, hc);
                    } else {
                        // RESTRICT / PROLONG / LAST read the level's stored values as they are: a
                        // neighbour outside the system holds a finite value (zero where the kernels
                        // wrote it) and meets a zero coupling
#pragma unroll
                        for (int q = 0; q < 7; ++q) {
                            float raw = H(pq[q], 0, hc + vo[q]);
                            if (M == PROLONG) {
                                // + the coarse parent's correction; each ring slot holds the
                                // coarse plane of its fine plane
                                const int fi = lane + (q == 1 ? -1 : (q == 2 ? 1 : 0));
                                const int fj = row + (q == 3 ? -1 : (q == 4 ? 1 : 0));
                                const int cx = (fi >> 1) + 4, cy = (fj >> 1) + 1;
                                raw += reinterpret_cast<const float*>(P[pq[q]] + L::off_coarse)[cy * kCX + cx];
                            }
                            v[q] = raw;
                        }
                        bcs[r] = Cn(0, row);
                    }
                    st.v0 = v[0];
                    st.vxm = v[1];
                    st.vxp = v[2];
                    st.vym = v[3];
                    st.vyp = v[4];
                    st.vzm = v[5];
                    st.vzp = v[6];
                }
                auto f2 = [](float x, float y) { return make_float2(x, y); };
                // the 7-point product d v0 + cxm vxm + ... in stencil7's order
                float2 a7 = __fmul2_rn(f2(sts[0].d, sts[1].d), f2(sts[0].v0, sts[1].v0));
                a7 = __ffma2_rn(f2(sts[0].cxm, sts[1].cxm), f2(sts[0].vxm, sts[1].vxm), a7);
                a7 = __ffma2_rn(f2(sts[0].cxp, sts[1].cxp), f2(sts[0].vxp, sts[1].vxp), a7);
                a7 = __ffma2_rn(f2(sts[0].cym, sts[1].cym), f2(sts[0].vym, sts[1].vym), a7);
                a7 = __ffma2_rn(f2(sts[0].cyp, sts[1].cyp), f2(sts[0].vyp, sts[1].vyp), a7);
                a7 = __ffma2_rn(f2(sts[0].czm, sts[1].czm), f2(sts[0].vzm, sts[1].vzm), a7);
                a7 = __ffma2_rn(f2(sts[0].czp, sts[1].czp), f2(sts[0].vzp, sts[1].vzp), a7);
                // a sweep x = v0 + omega (b - A v) / D in the scalar sweeps' operations, per lane
                auto sweep2 = [&](float omega) {
                    const float2 dr = __fmul2_rn(f2(omega, omega), __fadd2_rn(f2(bcs[0], bcs[1]), f2(-a7.x, -a7.y)));
                    return __fadd2_rn(f2(sts[0].v0, sts[1].v0), f2(mg_divf(dr.x, sts[0].d), mg_divf(dr.y, sts[1].d)));
                };
                float2 sw = f2(0.f, 0.f);
                if (M == UPDZ || M == ZERO2) sw = sweep2(w2);
                if (M == PROLONG) sw = sweep2(w1);
                if (M == LAST) sw = sweep2(w2);
#pragma unroll
                for (int r = 0; r < 2; ++r) {
                    const int row = 2 * w + r;
                    const int j = j0 + row;
                    const bool live = i < a.n0 && j < a.n1;
                    const int hc = (row + 1) * kHX + lane + 4;
                    const int c = i + a.n0 * (j + a.n1 * k);
                    const S7& st = sts[r];
                    const bool dp0 = st.d > 0.f;
                    const float a7r = r == 0 ? a7.x : a7.y;
                    const float swr = r == 0 ? sw.x : sw.y;
                    const float bc = bcs[r];
                    if (M == DIRSPMV) {
                        // Ap' and p'.Ap' at the cell
                        const float pc = dp0 ? st.v0 : 0.f, apc = dp0 ? a7r : 0.f;
                        if (live && EL_IN(c, (long long)a.n0 * a.n1 * a.n2, 10)) {
                            a.out0[c] = pc;
                            a.out1[c] = apc;
                            part += pc * apc;
                        }
                    } else if (M == UPDZ || M == ZERO2) {
                        const float x2 = dp0 ? swr : 0.f;
                        if (live && EL_IN(c, (long long)a.n0 * a.n1 * a.n2, 11)) {
                            if (M == UPDZ) {
                                // x += alpha p; r' out of place.  A tile also covers cells
                                // outside the system (diagonal 0), whose r may still hold an
                                // earlier solve's values: their r' is 0 and they stay out of
                                // |r'|^2, as in the segment kernels (where r is 0 on every
                                // such cell of an active segment).
                                const float rn = dp0 ? bc : 0.f;
                                a.out0[c] = Cn(0, row) + alpha * Cn(1, row);
                                a.out1[c] = rn;
                                part += rn * rn;
                                a.out2[c] = x2;
                            } else {
                                a.out0[c] = x2;
                            }
                        }
                    } else if (M == RESTRICT) {
                        res[r] = dp0 ? rn_sub(bc, a7r) : 0.f;
                    } else {
                        const float xo = dp0 ? swr : 0.f;
                        if (live && EL_IN(c, (long long)a.n0 * a.n1 * a.n2, 12)) {
                            a.out0[c] = xo;
                            if (M == LAST) part += bc * xo;
                        }
                    }
                    (void)hc;
                }
                if (M == RESTRICT) {
                    // the residuals summed over 2x2x2 blocks onto the coarse rhs in the segment
                    // kernels' order: the i pairs first (by shuffle), then the block's four rows
                    // (j, k) = (0, 0), (1, 0), (0, 1), (1, 1) -- the thread's two rows are a j pair,
                    // the k pairs add in registers
                    const float p0 = res[0] + __shfl_down_sync(kFull, res[0], 1);
                    const float p1 = res[1] + __shfl_down_sync(kFull, res[1], 1);
                    racc0 = (k & 1) ? (racc0 + p0) + p1 : p0 + p1;
                    if ((k & 1) || k + 1 == a.n2) {
                        const int I = i0 / 2 + (lane >> 1), J = j0 / 2 + w, K = k >> 1;
                        if (!(lane & 1) && I < a.c0 && J < a.c1 &&
                            EL_IN(I + a.c0 * (J + a.c1 * K), (long long)a.c0 * a.c1 * a.c2, 13))
                            a.out0[I + a.c0 * (J + a.c1 * K)] = racc0;
                        racc0 = 0.f;
                    }
                }
                release_next();  // plane k - 1 is not read again
                sa = sb;
                sb = sc;
            }
            if (aborted()) break;
            // the item's last two planes are not needed any more
            release_next();
            release_next();
        }
    }
    __syncthreads();
    if (abort_flag && tid == 0) {
        s->fault = 1;
        s->bad = 1;
        s->done = 1;
    }
    if (M == DIRSPMV || M == UPDZ || M == LAST) {
        double acc[1] = {(double)part};
        double tot[1];
        if (grid_sum<1>(acc, a.partials, a.counter, tot)) {
            if (M == DIRSPMV) {
                const double al = s->rz / tot[0];
                s->alpha = al;
                if (!isfinite(al)) {
                    s->bad = 1;
                    s->done = 1;
                }
            } else if (M == UPDZ) {
                s->rr = tot[0];
                s->iter += 1;
                if (!isfinite(tot[0])) {
                    s->bad = 1;
                    s->done = 1;
                } else if (tot[0] < s->thresh) {
                    s->done = 1;
                }
            } else {
                if (a.dot == 2) s->beta = tot[0] / s->rz;
                s->rz = tot[0];
                if (!isfinite(tot[0])) {
                    s->bad = 1;
                    s->done = 1;
                }
            }
        }
    }
}

// ---------------------------------------------------------------------------------------
// work items: tiles of 32 x 16 cells x `planes` planes holding a cell with a positive diagonal,
// in the order i-tile fastest, then j-tile, then plane chunk

__device__ __forceinline__ bool rec_active(const ushort4& r) { return __half2float(__ushort_as_half(r.x)) > 0.f; }
__device__ __forceinline__ bool rec_active(const float4& r) { return r.x > 0.f; }

template <typename R>
__global__ void march_flags_kernel(int n0, int n1, int n2, int nib, int njb, int planes, const R* __restrict__ rec,
                                   uint8_t* __restrict__ flags) {
    const int item = blockIdx.x;
    const int ib = item % nib, jb = (item / nib) % njb, kc = item / (nib * njb);
    const int i = ib * kTI + (threadIdx.x & 31), j = jb * kTJ + (threadIdx.x >> 5);
    const int k0 = kc * planes, k1 = min(n2, k0 + planes);
    int act = 0;
    if (i < n0 && j < n1)
        for (int k = k0; k < k1 && !act; ++k) act = rec_active(rec[i + n0 * (j + n1 * k)]);
    act = __syncthreads_or(act);
    if (threadIdx.x == 0) flags[item] = act ? 1 : 0;
}

// ordered compaction of the flags (one block)
__global__ void march_compact_kernel(int total, int nib, int njb, int n2, int planes, const uint8_t* __restrict__ flags,
                                     int4* __restrict__ items, int* __restrict__ count) {
    __shared__ int scan[1024];
    const int t = threadIdx.x;
    const int per = (total + blockDim.x - 1) / blockDim.x;
    const int lo = min(total, t * per), hi = min(total, lo + per);
    int c = 0;
    for (int q = lo; q < hi; ++q) c += flags[q];
    scan[t] = c;
    __syncthreads();
    for (int o = 1; o < (int)blockDim.x; o <<= 1) {
        const int v = t >= o ? scan[t - o] : 0;
        __syncthreads();
        scan[t] += v;
        __syncthreads();
    }
    int run = scan[t] - c;
    for (int q = lo; q < hi; ++q)
        if (flags[q]) {
            const int ib = q % nib, jb = (q / nib) % njb, kc = q / (nib * njb);
            const int k0 = kc * planes;
            items[run++] = make_int4(ib * kTI, jb * kTJ, k0, min(n2, k0 + planes));
        }
    if (t == blockDim.x - 1) *count = scan[t];
}

// ---------------------------------------------------------------------------------------
// host side

namespace {

template <int M>
int smem_bytes() {
    return Layout<M>::smem;
}

// dynamic shared memory, and the CTAs of the mode one SM holds (the grid is that many per SM,
// or the number of tiles when smaller)
template <int M>
int set_smem(el_ctx* ctx, MarchPlan& mp) {
    EL_CUDA_TRY(ctx, cudaFuncSetAttribute(march_kernel<M>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          smem_bytes<M>()));
    int per_sm = 0;
    EL_CUDA_TRY(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, march_kernel<M>, kThreads, smem_bytes<M>()));
    mp.per_sm[M] = std::max(1, per_sm);
    return EL_OK;
}

template <int M>
int march_grid(el_ctx* ctx, const MarchPlan& mp) {
    const long long total = (long long)mp.nib * mp.njb * mp.nkc;
    return (int)std::max<long long>(1, std::min<long long>(total, (long long)ctx->num_sms * mp.per_sm[M]));
}

template <int M>
void launch(el_ctx* ctx, const Maps& maps, const Args& a) {
    const MarchPlan& mp = ctx->march;
    launch_dependent(ctx, march_kernel<M>, dim3(march_grid<M>(ctx, mp)), dim3(kThreads), (size_t)smem_bytes<M>(), maps,
                     a);
}

Args base_args(el_ctx* ctx, Scalars* s) {
    Args a{};
    a.n0 = ctx->ni;
    a.n1 = ctx->nj;
    a.n2 = ctx->nk;
    const auto& mg = ctx->mg32;
    if (mg.size() > 1) {
        a.c0 = mg[1].n0;
        a.c1 = mg[1].n1;
        a.c2 = mg[1].n2;
    }
    a.items = ctx->march.items;
    a.count = ctx->march.count;
    a.s = s;
    a.partials = ctx->partials;
    a.counter = ctx->counter;
    return a;
}

int halo_index(el_ctx* ctx, const float* v) {
    if (v == ctx->z32) return MarchPlan::Z;
    if (v == ctx->p32) return MarchPlan::P;
    if (v == ctx->p32b) return MarchPlan::PB;
    if (v == ctx->ap32) return MarchPlan::AP;
    if (v == ctx->r32) return MarchPlan::R;
    if (v == ctx->r32b) return MarchPlan::RB;
    if (!ctx->mg32.empty() && v == ctx->mg32[0].t) return MarchPlan::T;
    return -1;
}

int centre_index(el_ctx* ctx, const float* v) {
    if (v == ctx->x32) return MarchPlan::CX;
    if (v == ctx->p32) return MarchPlan::CP;
    if (v == ctx->p32b) return MarchPlan::CPB;
    if (v == ctx->r32) return MarchPlan::CR;
    if (v == ctx->r32b) return MarchPlan::CRB;
    return -1;
}

}  // namespace

bool march_supported(const el_ctx* ctx) {
    return ctx->dtype == EL_F32 && ctx->ni % 8 == 0 && ctx->ni >= 64 && ctx->nj >= 16 && ctx->nk >= 16 &&
           ctx->mg32.size() >= 3 && tma_encode_fn() != nullptr;
}

// Tensor maps and the work-item storage, once per context (the arrays never move).
int march_setup(el_ctx* ctx) {
    MarchPlan& mp = ctx->march;
    mp.on = false;
    if (!march_supported(ctx)) return EL_OK;
    const int ni = ctx->ni, nj = ctx->nj, nk = ctx->nk;
    mp.nib = (ni + kTI - 1) / kTI;
    mp.njb = (nj + kTJ - 1) / kTJ;
    mp.nkc = (nk + kMarchPlanes - 1) / kMarchPlanes;
    const long long total = (long long)mp.nib * mp.njb * mp.nkc;
    mp.items = (int4*)ctx_alloc(ctx, total * sizeof(int4));
    mp.count = (int*)ctx_alloc(ctx, sizeof(int));
    mp.flags = (uint8_t*)ctx_alloc(ctx, total);
    if (!mp.items || !mp.count || !mp.flags) return set_error(ctx, EL_ERR_OUT_OF_MEMORY, "march items");
    const float* halo_src[MarchPlan::NHALO] = {ctx->z32,   ctx->p32, ctx->p32b, ctx->ap32,
                                               ctx->r32,   ctx->r32b, ctx->mg32[0].t};
    bool ok = true;
    for (int h = 0; h < MarchPlan::NHALO; ++h)
        ok = ok && tma_encode_3d(&mp.halo[h], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, halo_src[h], ni, nj, nk, ni, kHX, kHY);
    const float* centre_src[MarchPlan::NCENTRE] = {ctx->x32, ctx->p32, ctx->p32b, ctx->r32, ctx->r32b};
    for (int c = 0; c < MarchPlan::NCENTRE; ++c)
        ok = ok && tma_encode_3d(&mp.centre[c], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, centre_src[c], ni, nj, nk, ni, kTI, kTJ);
    // records: four components per cell as the innermost dimension
    ok = ok && tma_encode_3d(&mp.rec32, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, ctx->A32, 4ll * ni, nj, nk, 4ll * ni,
                      4 * Layout<DIRSPMV>::rec_w, kHY);
    ok = ok && tma_encode_3d(&mp.rec16, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2, ctx->A16, 4ll * ni, nj, nk, 4ll * ni,
                      4 * Layout<LAST>::rec_w, kHY);
    const auto& C = ctx->mg32[1];
    ok = ok && tma_encode_3d(&mp.coarse_x, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, C.x, C.n0, C.n1, C.n2, C.n0, kCX, kCY);
    if (!ok) return EL_OK;  // the segment kernels stay in use
    int rc;
    if ((rc = set_smem<DIRSPMV>(ctx, mp)) != EL_OK || (rc = set_smem<UPDZ>(ctx, mp)) != EL_OK ||
        (rc = set_smem<ZERO2>(ctx, mp)) != EL_OK || (rc = set_smem<RESTRICT>(ctx, mp)) != EL_OK ||
        (rc = set_smem<PROLONG>(ctx, mp)) != EL_OK || (rc = set_smem<LAST>(ctx, mp)) != EL_OK)
        return rc;
    mp.on = true;
    return EL_OK;
}

// Work items of the system just packed (A16 written): 2 launches.
int march_enqueue_items(el_ctx* ctx) {
    const MarchPlan& mp = ctx->march;
    const int total = mp.nib * mp.njb * mp.nkc;
    march_flags_kernel<<<total, kTI * kTJ, 0, ctx->stream>>>(ctx->ni, ctx->nj, ctx->nk, mp.nib, mp.njb, mp.planes,
                                                            ctx->A16, mp.flags);
    march_compact_kernel<<<1, 1024, 0, ctx->stream>>>(total, mp.nib, mp.njb, ctx->nk, mp.planes, mp.flags, mp.items,
                                                      mp.count);
    return 2;
}

// K1: p_out = z + beta p_in, ap = A p_out, alpha
int march_dir_spmv(el_ctx* ctx, const float* z, const float* p_in, float* p_out, float* ap, Scalars* s, int first) {
    const MarchPlan& mp = ctx->march;
    Maps maps;
    std::memset(&maps, 0, sizeof(maps));
    maps.halo[0] = mp.halo[halo_index(ctx, z)];
    maps.halo[1] = mp.halo[halo_index(ctx, p_in)];
    maps.rec = mp.rec32;
    Args a = base_args(ctx, s);
    a.out0 = p_out;
    a.out1 = ap;
    a.first = first;
    launch<DIRSPMV>(ctx, maps, a);
    return 1;
}

// K2 fused with the pre-smoother: x += alpha p; r_out = r_in - alpha ap; |r_out|^2; z = two
// sweeps from zero on r_out
int march_update_smooth(el_ctx* ctx, float* x, const float* p, const float* r_in, float* r_out, const float* ap,
                        float* z, Scalars* s) {
    const MarchPlan& mp = ctx->march;
    Maps maps;
    std::memset(&maps, 0, sizeof(maps));
    maps.halo[0] = mp.halo[halo_index(ctx, r_in)];
    maps.halo[1] = mp.halo[halo_index(ctx, ap)];
    maps.rec = mp.rec16;
    maps.centre[0] = mp.centre[centre_index(ctx, x)];
    maps.centre[1] = mp.centre[centre_index(ctx, p)];
    Args a = base_args(ctx, s);
    a.out0 = x;
    a.out1 = r_out;
    a.out2 = z;
    launch<UPDZ>(ctx, maps, a);
    return 1;
}

// two sweeps from zero: z = S(b)
int march_zero2(el_ctx* ctx, const float* b, float* z, Scalars* s) {
    const MarchPlan& mp = ctx->march;
    Maps maps;
    std::memset(&maps, 0, sizeof(maps));
    maps.halo[0] = mp.halo[halo_index(ctx, b)];
    maps.rec = mp.rec16;
    Args a = base_args(ctx, s);
    a.out0 = z;
    launch<ZERO2>(ctx, maps, a);
    return 1;
}

// coarse rhs = P^T (b - A x)
int march_restrict(el_ctx* ctx, const float* x, const float* b, float* coarse_b, Scalars* s) {
    const MarchPlan& mp = ctx->march;
    Maps maps;
    std::memset(&maps, 0, sizeof(maps));
    maps.halo[0] = mp.halo[halo_index(ctx, x)];
    maps.rec = mp.rec16;
    maps.centre[0] = mp.centre[centre_index(ctx, b)];
    Args a = base_args(ctx, s);
    a.out0 = coarse_b;
    launch<RESTRICT>(ctx, maps, a);
    return 1;
}

// t = one sweep from x + P e (e = the next level's x)
int march_prolong(el_ctx* ctx, const float* x, const float* b, float* t, Scalars* s) {
    const MarchPlan& mp = ctx->march;
    Maps maps;
    std::memset(&maps, 0, sizeof(maps));
    maps.halo[0] = mp.halo[halo_index(ctx, x)];
    maps.rec = mp.rec16;
    maps.centre[0] = mp.centre[centre_index(ctx, b)];
    maps.coarse = mp.coarse_x;
    Args a = base_args(ctx, s);
    a.out0 = t;
    launch<PROLONG>(ctx, maps, a);
    return 1;
}

// x = the last sweep from t, and b.x (dot = 1: rz; 2: beta and rz)
int march_last(el_ctx* ctx, const float* t, const float* b, float* x, Scalars* s, int dot) {
    const MarchPlan& mp = ctx->march;
    Maps maps;
    std::memset(&maps, 0, sizeof(maps));
    maps.halo[0] = mp.halo[halo_index(ctx, t)];
    maps.rec = mp.rec16;
    maps.centre[0] = mp.centre[centre_index(ctx, b)];
    Args a = base_args(ctx, s);
    a.out0 = x;
    a.dot = dot;
    launch<LAST>(ctx, maps, a);
    return 1;
}

EL_CHECK_EXPORT(march)

}  // namespace el
