// el_nn.cu -- the learned warm start's network kernels: BF16 implicit-GEMM 3x3x3 convolutions
// on the tensor cores (mma.sync m16n8k16, FP32 accumulation), forward and both backward passes,
// and the small kernels around them (pooling, upsampling, the 1x1x1 head with its loss, Adam,
// weight packing).  No counterpart in the reference, which has no learned component.
//
// Layout: activations are channels-last bf16, element (x, y, z, c) at ((z*Y + y)*X + x)*C + c,
// one sample per call.  A convolution's input may be the concatenation of two tensors (the
// decoder's [upsampled coarse, skip]) with the upsampling (nearest, factor 2) folded into the
// load: nothing concatenated or upsampled is ever written out.
//
// Forward = implicit GEMM with M = output voxels, N = output channels, K = 27 taps x input
// channels.  A CTA owns a 16 (x) x 8 (y) x 1 (z) brick of output voxels, one warp per y row:
// the input brick with its one-voxel halo (18 x 10 x 3 voxels, all input channels) is staged
// once in shared memory and the 27 taps read it through ldmatrix at shifted rows.  Weights are
// pre-packed in the mma B-fragment order, so each lane fetches its fragments with one 16-byte
// load per pair of n-blocks (they stay in L1: every warp of the CTA reads the same ones).
//
// Backward data is the same kernel: grad_in = conv(grad_out masked by ReLU', W') with W' the
// weights transposed in channels and mirrored in taps (packed separately); its output splits
// back into the two concatenated inputs.  Backward weight is a second implicit GEMM,
// M = output channels, N = input channels, K = voxels, per tap; each CTA keeps a group of taps'
// accumulators in registers over a range of bricks and writes one partial, summed in a fixed
// order by a reduction kernel (deterministic).
#include <cuda_bf16.h>

#include <cstdint>

#include "el_internal.cuh"

namespace el {
namespace nn {

constexpr int kTX = 16, kTY = 8;                     // output brick (x, y); z = 1
constexpr int kHX = kTX + 2, kHY = kTY + 2, kHZ = 3;  // with halo
constexpr int kHV = kHX * kHY * kHZ;                 // 540 halo voxels
constexpr int kThreads = 256;

struct ConvIn {
    const __nv_bfloat16* a;  // channels [0, ca)
    const __nv_bfloat16* b;  // channels [ca, ca + cb), fine resolution; NULL: cb channels of zeros
    const __nv_bfloat16* mask;  // optional, fine resolution, ca + cb channels: zero where <= 0
    int ca, cb, up_a;           // up_a: `a` is at half resolution (nearest upsampling)
    int ax, ay, az;             // dims of `a`
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void ldsm_x4(uint32_t addr, uint32_t (&r)[4]) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(addr));
}

__device__ __forceinline__ void ldsm_x4_t(uint32_t addr, uint32_t (&r)[4]) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(addr));
}

__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// zero the bf16 lanes of v whose mask lane is not > 0 (bf16 sign/magnitude test)
__device__ __forceinline__ uint4 apply_relu_mask(uint4 v, uint4 m) {
    uint32_t* pv = reinterpret_cast<uint32_t*>(&v);
    const uint32_t* pm = reinterpret_cast<const uint32_t*>(&m);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        uint32_t keep = 0;
        const uint32_t lo = pm[q] & 0xffffu, hi = pm[q] >> 16;
        // > 0: sign bit clear and not +0
        if (!(lo & 0x8000u) && lo != 0u) keep |= 0x0000ffffu;
        if (!(hi & 0x8000u) && hi != 0u) keep |= 0xffff0000u;
        pv[q] &= keep;
    }
    return v;
}

// Stage the input brick (with halo) of output brick (x0, y0, z0) into smem rows of `srow`
// bf16 (channel-contiguous, 16 bytes of padding per row against bank conflicts).
template <int CIN>
__device__ __forceinline__ void stage_halo(__nv_bfloat16* halo, const ConvIn& in, int X, int Y, int Z, int x0, int y0,
                                           int z0) {
    constexpr int CV = CIN / 8;
    constexpr int SROW = CIN + 8;
    for (int idx = threadIdx.x; idx < kHV * CV; idx += kThreads) {
        const int hv = idx / CV, cv = idx - hv * CV;
        const int hx = hv % kHX, t = hv / kHX, hy = t % kHY, hz = t / kHY;
        const int x = x0 + hx - 1, y = y0 + hy - 1, z = z0 + hz - 1;
        uint4 val = make_uint4(0u, 0u, 0u, 0u);
        if (x >= 0 && x < X && y >= 0 && y < Y && z >= 0 && z < Z) {
            const int c = cv * 8;
            const long long fine = ((long long)z * Y + y) * X + x;
            if (c < in.ca) {
                const long long va = in.up_a ? ((long long)(z >> 1) * in.ay + (y >> 1)) * in.ax + (x >> 1) : fine;
                val = __ldg(reinterpret_cast<const uint4*>(in.a + va * in.ca + c));
            } else if (in.b) {
                val = __ldg(reinterpret_cast<const uint4*>(in.b + fine * in.cb + (c - in.ca)));
            }
            if (in.mask) val = apply_relu_mask(val, __ldg(reinterpret_cast<const uint4*>(in.mask + fine * CIN + c)));
        }
        *reinterpret_cast<uint4*>(halo + hv * SROW + cv * 8) = val;
    }
}

// ---------------------------------------------------------------------------------------
// forward / backward-data convolution
template <int CIN, int COUT>
__global__ void __launch_bounds__(kThreads) conv3_kernel(int X, int Y, int Z, ConvIn in, const uint4* __restrict__ wf,
                                                         const float* __restrict__ bias, int relu,
                                                         __nv_bfloat16* __restrict__ out_a, int oca,
                                                         __nv_bfloat16* __restrict__ out_b) {
    constexpr int KS = CIN / 16, NB = COUT / 8, SROW = CIN + 8;
    static_assert(CIN % 16 == 0 && COUT % 16 == 0, "channels must be multiples of 16");
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __nv_bfloat16* halo = reinterpret_cast<__nv_bfloat16*>(smem_raw);
    const int x0 = blockIdx.x * kTX, y0 = blockIdx.y * kTY, z0 = blockIdx.z;
    stage_halo<CIN>(halo, in, X, Y, Z, x0, y0, z0);
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float acc[NB][4];
#pragma unroll
    for (int nb = 0; nb < NB; ++nb) acc[nb][0] = acc[nb][1] = acc[nb][2] = acc[nb][3] = 0.f;
    // ldmatrix row of this lane: voxel x = r, channel offset kofs within the 16-channel step
    const int r = (lane & 7) + ((lane >> 3) & 1) * 8, kofs = (lane >> 4) * 8;
#pragma unroll 1
    for (int tap = 0; tap < 27; ++tap) {
        const int dz = tap / 9 - 1, dy = (tap / 3) % 3 - 1, dx = tap % 3 - 1;
        const int hv = ((1 + dz) * kHY + (warp + 1 + dy)) * kHX + (1 + dx) + r;
        const uint32_t abase = smem_u32(halo + hv * SROW + kofs);
        const uint4* wp = wf + (size_t)tap * KS * (NB / 2) * 32 + lane;
#pragma unroll
        for (int ks = 0; ks < KS; ++ks) {
            uint32_t a[4];
            ldsm_x4(abase + ks * 32, a);
#pragma unroll
            for (int p = 0; p < NB / 2; ++p) {
                const uint4 b = __ldg(wp + (ks * (NB / 2) + p) * 32);
                mma_bf16(acc[2 * p], a, b.x, b.y);
                mma_bf16(acc[2 * p + 1], a, b.z, b.w);
            }
        }
    }
    const int y = y0 + warp;
    if (y >= Y) return;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const int x = x0 + (lane >> 2) + 8 * h;
        if (x >= X) continue;
        const long long v = ((long long)z0 * Y + y) * X + x;
#pragma unroll
        for (int nb = 0; nb < NB; ++nb) {
            const int co = nb * 8 + (lane & 3) * 2;
            float v0 = acc[nb][2 * h], v1 = acc[nb][2 * h + 1];
            if (bias) {
                v0 += bias[co];
                v1 += bias[co + 1];
            }
            if (relu) {
                v0 = fmaxf(v0, 0.f);
                v1 = fmaxf(v1, 0.f);
            }
            const __nv_bfloat162 pr = __floats2bfloat162_rn(v0, v1);
            if (co < oca)
                *reinterpret_cast<__nv_bfloat162*>(out_a + v * oca + co) = pr;
            else
                *reinterpret_cast<__nv_bfloat162*>(out_b + v * (COUT - oca) + (co - oca)) = pr;
        }
    }
}

// ---------------------------------------------------------------------------------------
// The same convolution on the 5th-generation tensor cores (tcgen05), for layers whose 27 taps
// of weights fit in shared memory next to the input brick.  A CTA of 4 warps owns an
// 8 (x) x 16 (y) x 1 (z) brick: M = 128 voxels, one TMEM lane each; N = output channels in TMEM
// columns (FP32).  Both operands sit in shared memory in the no-swizzle K-major layout, whose
// unit is an 8-row x 16-byte core matrix:
//   A: the input brick with its halo (10 x 18 x 3 voxels), channel-chunk major: chunk c
//      (channels 8c..8c+7) of voxel v at (c * 540 + v) * 16 bytes.  Eight x-consecutive voxels
//      are one core matrix, the next 8 rows (the next y) are 10 voxels further (SBO = 160 B),
//      the next chunk along K is 540 voxels further (LBO = 8640 B); tap (dx, dy, dz) only moves
//      the start address, so the 27 shifted operands need no copies.
//   B: per tap, [channel chunk][output channel] x 16 bytes: SBO = 128 B, LBO = cout * 16 B.
// One thread issues the 27 * cin / 16 MMAs (K = 16 each) into one accumulator and commits them to
// an mbarrier; the 4 warps wait (bounded), read their 32 TMEM lanes (tcgen05.ld) and store.
// The CTA is persistent over bricks: the weights are staged once.
namespace tc {

__device__ int g_error;  // set when a bounded wait gave up; read and cleared by el_nn_take_error

constexpr int TX = 8, TY = 16, HX = TX + 2, HY = TY + 2, HZ = 3, HV = HX * HY * HZ;  // 540 halo voxels
constexpr int kThreads = 128;

template <int CIN, int COUT>
struct Shape {
    static constexpr int KC = CIN / 8;                 // 16-byte channel chunks
    static constexpr int WB = 27 * KC * COUT * 16;     // weight bytes
    static constexpr int HB = KC * HV * 16;            // input brick bytes
    static constexpr int SMEM = WB + HB + 16;          // + mbarrier and TMEM address
    static constexpr uint32_t NCOL = COUT <= 32 ? 32u : (COUT <= 64 ? 64u : 128u);
    // BF16 x BF16 -> FP32, both K-major, M = 128, N = COUT
    static constexpr uint32_t IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(COUT >> 3) << 17) |
                                      ((uint32_t)(128 >> 4) << 24);
};

__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = (uint64_t)((addr & 0x3FFFFu) >> 4);
    d |= (uint64_t)((lbo & 0x3FFFFu) >> 4) << 16;
    d |= (uint64_t)((sbo & 0x3FFFFu) >> 4) << 32;
    d |= (uint64_t)1 << 46;  // descriptor version of the 5th-generation tensor cores; no swizzle
    return d;
}

__device__ __forceinline__ bool mbar_wait(uint32_t addr, uint32_t phase) {
    // polls without suspending; gives up (and reports) after about two seconds of SM clock
    const long long start = clock64();
    while (true) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}\n"
            : "=r"(done)
            : "r"(addr), "r"(phase)
            : "memory");
        if (done) return true;
        if (clock64() - start > (1LL << 32)) return false;
    }
}

template <int CIN>
__device__ __forceinline__ void stage_brick(unsigned char* hsm, const ConvIn& in, int X, int Y, int Z, int x0, int y0,
                                            int z0) {
    constexpr int KC = CIN / 8;
    for (int idx = threadIdx.x; idx < HV * KC; idx += kThreads) {
        const int hv = idx / KC, cv = idx - hv * KC;
        const int hx = hv % HX, t = hv / HX, hy = t % HY, hz = t / HY;
        const int x = x0 + hx - 1, y = y0 + hy - 1, z = z0 + hz - 1;
        uint4 val = make_uint4(0u, 0u, 0u, 0u);
        if (x >= 0 && x < X && y >= 0 && y < Y && z >= 0 && z < Z) {
            const int c = cv * 8;
            const long long fine = ((long long)z * Y + y) * X + x;
            if (c < in.ca) {
                const long long va = in.up_a ? ((long long)(z >> 1) * in.ay + (y >> 1)) * in.ax + (x >> 1) : fine;
                val = __ldg(reinterpret_cast<const uint4*>(in.a + va * in.ca + c));
            } else if (in.b) {
                val = __ldg(reinterpret_cast<const uint4*>(in.b + fine * in.cb + (c - in.ca)));
            }
            if (in.mask) val = apply_relu_mask(val, __ldg(reinterpret_cast<const uint4*>(in.mask + fine * CIN + c)));
        }
        *reinterpret_cast<uint4*>(hsm + ((size_t)cv * HV + hv) * 16) = val;
    }
}

template <int CIN, int COUT>
__global__ void __launch_bounds__(kThreads) conv3_tc_kernel(int X, int Y, int Z, ConvIn in,
                                                            const uint4* __restrict__ wtc,
                                                            const float* __restrict__ bias, int relu,
                                                            __nv_bfloat16* __restrict__ out_a, int oca,
                                                            __nv_bfloat16* __restrict__ out_b) {
    using S = Shape<CIN, COUT>;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    unsigned char* wsm = smem_raw;
    unsigned char* hsm = smem_raw + S::WB;
    uint64_t* mbar = reinterpret_cast<uint64_t*>(smem_raw + S::WB + S::HB);
    uint32_t* tslot = reinterpret_cast<uint32_t*>(smem_raw + S::WB + S::HB + 8);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    for (int q = tid; q < S::WB / 16; q += kThreads) reinterpret_cast<uint4*>(wsm)[q] = __ldg(wtc + q);
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(tslot)),
                     "r"(S::NCOL)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(mbar)), "r"(1) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    const uint32_t tmem = *tslot;
    const uint32_t wbase = smem_u32(wsm), hbase = smem_u32(hsm), mbar_a = smem_u32(mbar);
    const int bx = (X + TX - 1) / TX, by = (Y + TY - 1) / TY;
    const long long nbricks = (long long)bx * by * Z;
    uint32_t phase = 0;
    for (long long br = blockIdx.x; br < nbricks; br += gridDim.x) {
        const int x0 = (int)(br % bx) * TX;
        const long long rest = br / bx;
        const int y0 = (int)(rest % by) * TY, z0 = (int)(rest / by);
        stage_brick<CIN>(hsm, in, X, Y, Z, x0, y0, z0);
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");  // visible to the tensor cores
        __syncthreads();
        if (tid == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
#pragma unroll 1
            for (int tap = 0; tap < 27; ++tap) {
                const int dz = tap / 9, dy = (tap / 3) % 3, dx = tap % 3;
                const uint32_t a0 = hbase + (uint32_t)(((dz * HY + dy) * HX + dx) * 16);
                const uint32_t b0 = wbase + (uint32_t)(tap * S::KC * COUT * 16);
#pragma unroll
                for (int s = 0; s < S::KC / 2; ++s) {
                    const uint64_t da = smem_desc(a0 + (uint32_t)(2 * s * HV * 16), HV * 16, HX * 16);
                    const uint64_t db = smem_desc(b0 + (uint32_t)(2 * s * COUT * 16), COUT * 16, 128);
                    const uint32_t acc = (tap | s) ? 1u : 0u;
                    asm volatile(
                        "{\n\t.reg .pred p;\n\t"
                        "setp.ne.b32 p, %4, 0;\n\t"
                        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem),
                        "l"(da), "l"(db), "r"(S::IDESC), "r"(acc)
                        : "memory");
                }
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                             mbar_a)
                         : "memory");
        }
        const bool ok = mbar_wait(mbar_a, phase);
        phase ^= 1u;
        if (!__syncthreads_and(ok)) {
            if (tid == 0) atomicExch(&g_error, 1);
            break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
        // row r = 32 warp + lane of the accumulator is voxel (x0 + r % 8, y0 + r / 8, z0)
        const int r = warp * 32 + lane;
        const int x = x0 + (r & 7), y = y0 + (r >> 3);
        const bool live = x < X && y < Y;
        const long long v = ((long long)z0 * Y + y) * X + x;
#pragma unroll
        for (int c0 = 0; c0 < COUT; c0 += 16) {
            uint32_t q[16];
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, "
                "[%16];\n"
                : "=r"(q[0]), "=r"(q[1]), "=r"(q[2]), "=r"(q[3]), "=r"(q[4]), "=r"(q[5]), "=r"(q[6]), "=r"(q[7]),
                  "=r"(q[8]), "=r"(q[9]), "=r"(q[10]), "=r"(q[11]), "=r"(q[12]), "=r"(q[13]), "=r"(q[14]),
                  "=r"(q[15])
                : "r"(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0));
            asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
            if (live) {
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    uint4 o;
                    __nv_bfloat162* op = reinterpret_cast<__nv_bfloat162*>(&o);
#pragma unroll
                    for (int e = 0; e < 4; ++e) {
                        const int co = c0 + h * 8 + 2 * e;
                        float f0 = __uint_as_float(q[h * 8 + 2 * e]), f1 = __uint_as_float(q[h * 8 + 2 * e + 1]);
                        if (bias) {
                            f0 += bias[co];
                            f1 += bias[co + 1];
                        }
                        if (relu) {
                            f0 = fmaxf(f0, 0.f);
                            f1 = fmaxf(f1, 0.f);
                        }
                        op[e] = __floats2bfloat162_rn(f0, f1);
                    }
                    const int cb = c0 + h * 8;
                    if (cb < oca)
                        *reinterpret_cast<uint4*>(out_a + v * oca + cb) = o;
                    else
                        *reinterpret_cast<uint4*>(out_b + v * (COUT - oca) + (cb - oca)) = o;
                }
            }
        }
        asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
        __syncthreads();  // accumulator read and brick consumed before the next brick
    }
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(S::NCOL) : "memory");
}

// Pipelined variant, for the layers where two input bricks fit next to the weights: the copy of
// brick i+1 (cp.async, 16 bytes per thread and chunk, zero-filled outside the grid) and the
// epilogue of brick i-1 run while the tensor cores work on brick i, with two input buffers and
// two accumulators (2 * cout TMEM columns) used in turn.  A ReLU mask (backward data) is applied
// while staging, so that case stages with ordinary loads at the same point.
template <int CIN, int COUT>
struct PipeShape {
    static constexpr int KC = CIN / 8;
    static constexpr int WB = 27 * KC * COUT * 16;
    static constexpr int HB = KC * HV * 16;
    static constexpr int SMEM = WB + 2 * HB + 32;
    static constexpr uint32_t NCOL = 2 * COUT <= 32 ? 32u : (2 * COUT <= 64 ? 64u : (2 * COUT <= 128 ? 128u : 256u));
    static constexpr bool FITS = SMEM <= 220 * 1024;
};

__device__ __forceinline__ void cp_async16(uint32_t dst, const void* src, bool valid) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(dst), "l"(src), "r"(valid ? 16 : 0)
                 : "memory");
}

template <int CIN>
__device__ __forceinline__ void stage_brick_async(unsigned char* hsm, const ConvIn& in, int X, int Y, int Z, int x0,
                                                  int y0, int z0) {
    if (in.mask) {  // needs the mask applied on the way: ordinary loads
        stage_brick<CIN>(hsm, in, X, Y, Z, x0, y0, z0);
        return;
    }
    constexpr int KC = CIN / 8;
    const uint32_t base = smem_u32(hsm);
    for (int idx = threadIdx.x; idx < HV * KC; idx += kThreads) {
        const int hv = idx / KC, cv = idx - hv * KC;
        const int hx = hv % HX, t = hv / HX, hy = t % HY, hz = t / HY;
        const int x = x0 + hx - 1, y = y0 + hy - 1, z = z0 + hz - 1;
        const bool inside = x >= 0 && x < X && y >= 0 && y < Y && z >= 0 && z < Z;
        const int c = cv * 8;
        const __nv_bfloat16* src = in.a;  // a valid address even when nothing is read
        bool valid = false;
        if (inside) {
            const long long fine = ((long long)z * Y + y) * X + x;
            if (c < in.ca) {
                const long long va = in.up_a ? ((long long)(z >> 1) * in.ay + (y >> 1)) * in.ax + (x >> 1) : fine;
                src = in.a + va * in.ca + c;
                valid = true;
            } else if (in.b) {
                src = in.b + fine * in.cb + (c - in.ca);
                valid = true;
            }
        }
        cp_async16(base + (uint32_t)(((size_t)cv * HV + hv) * 16), src, valid);
    }
    asm volatile("cp.async.commit_group;\n" ::: "memory");
}

__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// accumulator columns [col, col + COUT) of this warp's 32 lanes -> bias, ReLU, bf16, store
template <int COUT>
__device__ __forceinline__ void tc_epilogue(uint32_t tmem, uint32_t col, int X, int Y, int x0, int y0, int z0,
                                            const float* __restrict__ bias, int relu, __nv_bfloat16* out_a, int oca,
                                            __nv_bfloat16* out_b) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int r = warp * 32 + lane;
    const int x = x0 + (r & 7), y = y0 + (r >> 3);
    const bool live = x < X && y < Y;
    const long long v = ((long long)z0 * Y + y) * X + x;
#pragma unroll
    for (int c0 = 0; c0 < COUT; c0 += 16) {
        uint32_t q[16];
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, "
            "[%16];\n"
            : "=r"(q[0]), "=r"(q[1]), "=r"(q[2]), "=r"(q[3]), "=r"(q[4]), "=r"(q[5]), "=r"(q[6]), "=r"(q[7]),
              "=r"(q[8]), "=r"(q[9]), "=r"(q[10]), "=r"(q[11]), "=r"(q[12]), "=r"(q[13]), "=r"(q[14]), "=r"(q[15])
            : "r"(tmem + ((uint32_t)(warp * 32) << 16) + col + (uint32_t)c0));
        asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
        if (!live) continue;
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            uint4 o;
            __nv_bfloat162* op = reinterpret_cast<__nv_bfloat162*>(&o);
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                const int co = c0 + h * 8 + 2 * e;
                float f0 = __uint_as_float(q[h * 8 + 2 * e]), f1 = __uint_as_float(q[h * 8 + 2 * e + 1]);
                if (bias) {
                    f0 += bias[co];
                    f1 += bias[co + 1];
                }
                if (relu) {
                    f0 = fmaxf(f0, 0.f);
                    f1 = fmaxf(f1, 0.f);
                }
                op[e] = __floats2bfloat162_rn(f0, f1);
            }
            const int cb = c0 + h * 8;
            if (cb < oca)
                *reinterpret_cast<uint4*>(out_a + v * oca + cb) = o;
            else
                *reinterpret_cast<uint4*>(out_b + v * (COUT - oca) + (cb - oca)) = o;
        }
    }
}

template <int CIN, int COUT>
__device__ __forceinline__ void tc_issue(uint32_t tmem_acc, uint32_t hbase, uint32_t wbase, uint32_t mbar) {
    using S = PipeShape<CIN, COUT>;
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
#pragma unroll 1
    for (int tap = 0; tap < 27; ++tap) {
        const int dz = tap / 9, dy = (tap / 3) % 3, dx = tap % 3;
        const uint32_t a0 = hbase + (uint32_t)(((dz * HY + dy) * HX + dx) * 16);
        const uint32_t b0 = wbase + (uint32_t)(tap * S::KC * COUT * 16);
#pragma unroll
        for (int s = 0; s < S::KC / 2; ++s) {
            const uint64_t da = smem_desc(a0 + (uint32_t)(2 * s * HV * 16), HV * 16, HX * 16);
            const uint64_t db = smem_desc(b0 + (uint32_t)(2 * s * COUT * 16), COUT * 16, 128);
            const uint32_t acc = (tap | s) ? 1u : 0u;
            asm volatile(
                "{\n\t.reg .pred p;\n\t"
                "setp.ne.b32 p, %4, 0;\n\t"
                "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem_acc),
                "l"(da), "l"(db), "r"(Shape<CIN, COUT>::IDESC), "r"(acc)
                : "memory");
        }
    }
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(mbar)
                 : "memory");
}

template <int CIN, int COUT>
__global__ void __launch_bounds__(kThreads) conv3_tc_pipe_kernel(int X, int Y, int Z, ConvIn in,
                                                                 const uint4* __restrict__ wtc,
                                                                 const float* __restrict__ bias, int relu,
                                                                 __nv_bfloat16* __restrict__ out_a, int oca,
                                                                 __nv_bfloat16* __restrict__ out_b) {
    using S = PipeShape<CIN, COUT>;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    unsigned char* wsm = smem_raw;
    unsigned char* hsm[2] = {smem_raw + S::WB, smem_raw + S::WB + S::HB};
    uint64_t* mbar = reinterpret_cast<uint64_t*>(smem_raw + S::WB + 2 * S::HB);  // two
    uint32_t* tslot = reinterpret_cast<uint32_t*>(smem_raw + S::WB + 2 * S::HB + 16);
    const int tid = threadIdx.x, warp = tid >> 5;
    for (int q = tid; q < S::WB / 16; q += kThreads) reinterpret_cast<uint4*>(wsm)[q] = __ldg(wtc + q);
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(tslot)),
                     "r"(S::NCOL)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(mbar)), "r"(1) : "memory");
        asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(mbar + 1)), "r"(1) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    const uint32_t tmem = *tslot;
    const uint32_t wbase = smem_u32(wsm), hb[2] = {smem_u32(hsm[0]), smem_u32(hsm[1])};
    const uint32_t mb[2] = {smem_u32(mbar), smem_u32(mbar + 1)};
    const int bx = (X + TX - 1) / TX, by = (Y + TY - 1) / TY;
    const long long nbricks = (long long)bx * by * Z;
    const long long mine = nbricks > blockIdx.x ? (nbricks - 1 - blockIdx.x) / gridDim.x + 1 : 0;
    auto origin = [&](long long i, int& x0, int& y0, int& z0) {
        const long long br = blockIdx.x + i * gridDim.x;
        x0 = (int)(br % bx) * TX;
        const long long rest = br / bx;
        y0 = (int)(rest % by) * TY;
        z0 = (int)(rest / by);
    };
    uint32_t phase[2] = {0u, 0u};
    bool ok = true;
    int x0, y0, z0;
    if (mine > 0) {
        origin(0, x0, y0, z0);
        stage_brick_async<CIN>(hsm[0], in, X, Y, Z, x0, y0, z0);
    }
    for (long long i = 0; i < mine && ok; ++i) {
        const int b = (int)(i & 1);
        cp_async_wait_all();
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");  // brick i visible to the tensor cores
        __syncthreads();
        if (tid == 0) tc_issue<CIN, COUT>(tmem + (uint32_t)(b * COUT), hb[b], wbase, mb[b]);
        if (i > 0) {
            // brick i-1: its MMAs are done, so its buffer takes brick i+1 while its result is stored
            const bool mine_ok = mbar_wait(mb[b ^ 1], phase[b ^ 1]);
            phase[b ^ 1] ^= 1u;
            ok = __syncthreads_and(mine_ok) != 0;  // uniform across the block
            if (!ok) break;
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
        }
        if (i + 1 < mine) {
            int x1, y1, z1;
            origin(i + 1, x1, y1, z1);
            stage_brick_async<CIN>(hsm[b ^ 1], in, X, Y, Z, x1, y1, z1);
        }
        if (i > 0) {
            int xp, yp, zp;
            origin(i - 1, xp, yp, zp);
            tc_epilogue<COUT>(tmem, (uint32_t)((b ^ 1) * COUT), X, Y, xp, yp, zp, bias, relu, out_a, oca, out_b);
        }
        asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
        __syncthreads();  // the accumulator just read is free for brick i+1
    }
    if (ok && mine > 0) {  // ok is uniform here
        const long long i = mine - 1;
        const int b = (int)(i & 1);
        ok = __syncthreads_and(mbar_wait(mb[b], phase[b])) != 0;
        if (ok) {
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
            origin(i, x0, y0, z0);
            tc_epilogue<COUT>(tmem, (uint32_t)(b * COUT), X, Y, x0, y0, z0, bias, relu, out_a, oca, out_b);
        }
    }
    if (!ok && tid == 0) atomicExch(&g_error, 1);
    cp_async_wait_all();
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(S::NCOL) : "memory");
}

// FP32 master [co][27][ci] -> the B layout above: [tap][ci / 8][co][ci % 8]
__global__ void pack_weights_tc_kernel(int cin, int cout, const float* __restrict__ w, __nv_bfloat16* __restrict__ tf,
                                       __nv_bfloat16* __restrict__ tb) {
    const long long n = 27LL * cin * cout;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        const int ci = (int)(e % cin);
        const long long t2 = e / cin;
        const int tap = (int)(t2 % 27), co = (int)(t2 / 27);
        const __nv_bfloat16 v = __float2bfloat16_rn(w[e]);
        tf[(((size_t)tap * (cin / 8) + ci / 8) * cout + co) * 8 + (ci % 8)] = v;
        // backward data: the transposed, tap-mirrored kernel (cin' = cout, cout' = cin)
        if (tb) tb[(((size_t)(26 - tap) * (cout / 8) + co / 8) * cin + ci) * 8 + (co % 8)] = v;
    }
}

}  // namespace tc

// ---------------------------------------------------------------------------------------
// backward weight: dW[co][tap][ci] = sum_v gm[v][co] x[v + off(tap)][ci], gm = g * (y > 0),
// one 16 (co) x 16 (ci) tile of one tap per warp task; the CTA covers taps
// [tap0, tap0 + ntaps) for all channels over bricks split, split + nsplit, ...
template <int CIN, int COUT>
struct WGrad {
    static constexpr int MB = COUT / 16, NP = CIN / 16;
    static constexpr int TILES_PER_TAP = MB * NP;
    static constexpr int TAPS = (64 / TILES_PER_TAP) < 1 ? 1 : ((64 / TILES_PER_TAP) > 27 ? 27 : 64 / TILES_PER_TAP);
    static constexpr int GROUPS = (27 + TAPS - 1) / TAPS;
    static constexpr int MAXT = (TAPS * TILES_PER_TAP + 7) / 8;  // tasks per warp
};

template <int CIN, int COUT>
__global__ void __launch_bounds__(kThreads) conv3_wgrad_kernel(int X, int Y, int Z, ConvIn in,
                                                               const __nv_bfloat16* __restrict__ g,
                                                               const __nv_bfloat16* __restrict__ y_out, int nsplit,
                                                               float* __restrict__ part_w, float* __restrict__ part_b) {
    using W = WGrad<CIN, COUT>;
    constexpr int SROW = CIN + 8, GROW = COUT + 8;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __nv_bfloat16* halo = reinterpret_cast<__nv_bfloat16*>(smem_raw);
    __nv_bfloat16* gt = halo + kHV * SROW;  // [128 voxels][COUT]
    const int group = blockIdx.x, split = blockIdx.y;
    const int tap0 = group * W::TAPS;
    const int ntaps = min(W::TAPS, 27 - tap0);
    const int ntasks = ntaps * W::TILES_PER_TAP;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int bx = (X + kTX - 1) / kTX, by = (Y + kTY - 1) / kTY;
    const long long nbricks = (long long)bx * by * Z;
    float acc[W::MAXT][2][4];
#pragma unroll
    for (int t = 0; t < W::MAXT; ++t)
#pragma unroll
        for (int h = 0; h < 2; ++h) acc[t][h][0] = acc[t][h][1] = acc[t][h][2] = acc[t][h][3] = 0.f;
    float bsum = 0.f;  // bias gradient: channel threadIdx.x % COUT (group 0 only)
    const int r = (lane & 7), m = lane >> 3;
#pragma unroll 1
    for (long long br = split; br < nbricks; br += nsplit) {
        const int bxi = (int)(br % bx);
        const long long rest = br / bx;
        const int byi = (int)(rest % by), z0 = (int)(rest / by);
        const int x0 = bxi * kTX, y0 = byi * kTY;
        __syncthreads();  // previous brick's reads done
        stage_halo<CIN>(halo, in, X, Y, Z, x0, y0, z0);
        // output gradient tile, masked by ReLU'; zero outside the grid
        for (int idx = threadIdx.x; idx < 128 * (COUT / 8); idx += kThreads) {
            const int vv = idx / (COUT / 8), cv = idx - vv * (COUT / 8);
            const int x = x0 + (vv & 15), y = y0 + (vv >> 4);
            uint4 val = make_uint4(0u, 0u, 0u, 0u);
            if (x < X && y < Y) {
                const long long v = ((long long)z0 * Y + y) * X + x;
                val = apply_relu_mask(__ldg(reinterpret_cast<const uint4*>(g + v * COUT + cv * 8)),
                                      __ldg(reinterpret_cast<const uint4*>(y_out + v * COUT + cv * 8)));
            }
            *reinterpret_cast<uint4*>(gt + vv * GROW + cv * 8) = val;
        }
        __syncthreads();
        if (group == 0 && threadIdx.x < 2 * COUT) {
            const int co = threadIdx.x % COUT, half = threadIdx.x / COUT;
            for (int vv = half * 64; vv < half * 64 + 64; ++vv) bsum += __bfloat162float(gt[vv * GROW + co]);
        }
#pragma unroll 1
        for (int row = 0; row < kTY; ++row) {  // k-step: the 16 voxels of brick row `row`
#pragma unroll
            for (int t = 0; t < W::MAXT; ++t) {
                const int task = warp + 8 * t;
                if (task >= ntasks) break;
                const int tl = task / W::TILES_PER_TAP, rem = task - tl * W::TILES_PER_TAP;
                const int mb = rem / W::NP, np = rem - mb * W::NP;
                const int tap = tap0 + tl;
                const int dz = tap / 9 - 1, dy = (tap / 3) % 3 - 1, dx = tap % 3 - 1;
                // A = gm^T (co x v): matrices (v 0-7|co 0-7), (v 0-7|co 8-15), (v 8-15|co 0-7), (v 8-15|co 8-15)
                uint32_t a[4];
                ldsm_x4_t(smem_u32(gt + (row * 16 + r + (m >> 1) * 8) * GROW + mb * 16 + (m & 1) * 8), a);
                // B = x shifted (v x ci): matrices (v 0-7|ci 0-7), (v 8-15|ci 0-7), (v 0-7|ci 8-15), (v 8-15|ci 8-15)
                const int hv = ((1 + dz) * kHY + (row + 1 + dy)) * kHX + (1 + dx) + r + (m & 1) * 8;
                uint32_t b[4];
                ldsm_x4_t(smem_u32(halo + hv * SROW + np * 16 + (m >> 1) * 8), b);
                mma_bf16(acc[t][0], a, b[0], b[1]);
                mma_bf16(acc[t][1], a, b[2], b[3]);
            }
        }
    }
    // partial [split][tap][co][ci]
#pragma unroll
    for (int t = 0; t < W::MAXT; ++t) {
        const int task = warp + 8 * t;
        if (task >= ntasks) break;
        const int tl = task / W::TILES_PER_TAP, rem = task - tl * W::TILES_PER_TAP;
        const int mb = rem / W::NP, np = rem - mb * W::NP;
        float* dst = part_w + ((size_t)split * 27 + tap0 + tl) * COUT * CIN;
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int ci = np * 16 + h * 8 + (lane & 3) * 2;
            const int co = mb * 16 + (lane >> 2);
            dst[(size_t)co * CIN + ci] = acc[t][h][0];
            dst[(size_t)co * CIN + ci + 1] = acc[t][h][1];
            dst[(size_t)(co + 8) * CIN + ci] = acc[t][h][2];
            dst[(size_t)(co + 8) * CIN + ci + 1] = acc[t][h][3];
        }
    }
    if (group == 0) {
        __shared__ float bs[2 * 128];
        if (threadIdx.x < 2 * COUT) bs[threadIdx.x] = bsum;
        __syncthreads();
        if (threadIdx.x < COUT) part_b[(size_t)split * COUT + threadIdx.x] = bs[threadIdx.x] + bs[threadIdx.x + COUT];
    }
}

// dW[co][tap][ci] += sum over splits (fixed order); db[co] += likewise
__global__ void wgrad_reduce_kernel(int cin, int cout, int nsplit, const float* __restrict__ part_w,
                                    const float* __restrict__ part_b, float* __restrict__ dw, float* __restrict__ db) {
    const long long per = 27LL * cout * cin;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < per + cout;
         e += (long long)gridDim.x * blockDim.x) {
        if (e < per) {
            // e indexes the partial layout [tap][co][ci]; dW is [co][tap][ci]
            const int ci = (int)(e % cin);
            const long long t2 = e / cin;
            const int co = (int)(t2 % cout), tap = (int)(t2 / cout);
            float s = 0.f;
            for (int q = 0; q < nsplit; ++q) s += part_w[(size_t)q * per + e];
            dw[((size_t)co * 27 + tap) * cin + ci] += s;
        } else if (db) {
            const int co = (int)(e - per);
            float s = 0.f;
            for (int q = 0; q < nsplit; ++q) s += part_b[(size_t)q * cout + co];
            db[co] += s;
        }
    }
}

// ---------------------------------------------------------------------------------------
// weights: FP32 master [co][27][ci] -> bf16 B fragments for the forward (K = ci) and for the
// backward data pass (the transposed, tap-mirrored kernel, K = co)
__device__ __forceinline__ size_t frag_index(int tap, int n, int k, int kdim, int ndim) {
    const int ks = k >> 4, kk = k & 15, nb = n >> 3, nn = n & 7;
    const int ln = nn * 4 + ((kk & 7) >> 1);
    const int comp = (nb & 1) * 2 + (kk >> 3);
    const size_t u4 = (((size_t)tap * (kdim / 16) + ks) * (ndim / 16) + (nb >> 1)) * 32 + ln;
    return (u4 * 4 + comp) * 2 + (kk & 1);
}

__global__ void pack_weights_kernel(int cin, int cout, const float* __restrict__ w, __nv_bfloat16* __restrict__ wf,
                                    __nv_bfloat16* __restrict__ wb) {
    const long long n = 27LL * cin * cout;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        const int ci = (int)(e % cin);
        const long long t2 = e / cin;
        const int tap = (int)(t2 % 27), co = (int)(t2 / 27);
        const __nv_bfloat16 v = __float2bfloat16_rn(w[e]);
        wf[frag_index(tap, co, ci, cin, cout)] = v;
        if (wb) wb[frag_index(26 - tap, ci, co, cout, cin)] = v;
    }
}

// ---------------------------------------------------------------------------------------
// 2x2x2 average pooling, its backward (accumulated into the fine gradient) and the backward
// of nearest upsampling (sum of the 8 children); 8 channels per thread
__global__ void pool_fwd_kernel(int X, int Y, int Z, int C, const __nv_bfloat16* __restrict__ in,
                                __nv_bfloat16* __restrict__ out) {
    const int Xc = X / 2, Yc = Y / 2, Zc = Z / 2, CV = C / 8;
    const long long n = (long long)Xc * Yc * Zc * CV;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        const int cv = (int)(e % CV);
        const long long V = e / CV;
        const int xc = (int)(V % Xc), yc = (int)((V / Xc) % Yc), zc = (int)(V / ((long long)Xc * Yc));
        float s[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        for (int q = 0; q < 8; ++q) {
            const long long v = ((long long)(2 * zc + (q >> 2)) * Y + 2 * yc + ((q >> 1) & 1)) * X + 2 * xc + (q & 1);
            const uint4 u = __ldg(reinterpret_cast<const uint4*>(in + v * C + cv * 8));
            const __nv_bfloat162* h = reinterpret_cast<const __nv_bfloat162*>(&u);
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const float2 f = __bfloat1622float2(h[j]);
                s[2 * j] += f.x;
                s[2 * j + 1] += f.y;
            }
        }
        uint4 o;
        __nv_bfloat162* h = reinterpret_cast<__nv_bfloat162*>(&o);
#pragma unroll
        for (int j = 0; j < 4; ++j) h[j] = __floats2bfloat162_rn(s[2 * j] * 0.125f, s[2 * j + 1] * 0.125f);
        *reinterpret_cast<uint4*>(out + V * C + cv * 8) = o;
    }
}

// fine[v] (+)= scale * coarse[v / 2]: pooling backward (scale 1/8, accumulate)
__global__ void spread_kernel(int X, int Y, int Z, int C, const __nv_bfloat16* __restrict__ coarse,
                              __nv_bfloat16* __restrict__ fine, float scale, int accumulate) {
    const int CV = C / 8, Xc = X / 2, Yc = Y / 2;
    const long long n = (long long)X * Y * Z * CV;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        const int cv = (int)(e % CV);
        const long long v = e / CV;
        const int x = (int)(v % X), y = (int)((v / X) % Y), z = (int)(v / ((long long)X * Y));
        const long long V = ((long long)(z >> 1) * Yc + (y >> 1)) * Xc + (x >> 1);
        const uint4 cu = __ldg(reinterpret_cast<const uint4*>(coarse + V * C + cv * 8));
        const __nv_bfloat162* ch = reinterpret_cast<const __nv_bfloat162*>(&cu);
        uint4* fp = reinterpret_cast<uint4*>(fine + v * C + cv * 8);
        uint4 fu = accumulate ? *fp : make_uint4(0u, 0u, 0u, 0u);
        __nv_bfloat162* fh = reinterpret_cast<__nv_bfloat162*>(&fu);
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const float2 c2 = __bfloat1622float2(ch[j]);
            const float2 f2 = accumulate ? __bfloat1622float2(fh[j]) : make_float2(0.f, 0.f);
            fh[j] = __floats2bfloat162_rn(f2.x + scale * c2.x, f2.y + scale * c2.y);
        }
        *fp = fu;
    }
}

// coarse[V] = sum of the 8 fine children: backward of nearest upsampling
__global__ void gather8_kernel(int X, int Y, int Z, int C, const __nv_bfloat16* __restrict__ fine,
                               __nv_bfloat16* __restrict__ coarse) {
    const int Xc = X / 2, Yc = Y / 2, Zc = Z / 2, CV = C / 8;
    const long long n = (long long)Xc * Yc * Zc * CV;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        const int cv = (int)(e % CV);
        const long long V = e / CV;
        const int xc = (int)(V % Xc), yc = (int)((V / Xc) % Yc), zc = (int)(V / ((long long)Xc * Yc));
        float s[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        for (int q = 0; q < 8; ++q) {
            const long long v = ((long long)(2 * zc + (q >> 2)) * Y + 2 * yc + ((q >> 1) & 1)) * X + 2 * xc + (q & 1);
            const uint4 u = __ldg(reinterpret_cast<const uint4*>(fine + v * C + cv * 8));
            const __nv_bfloat162* h = reinterpret_cast<const __nv_bfloat162*>(&u);
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const float2 f = __bfloat1622float2(h[j]);
                s[2 * j] += f.x;
                s[2 * j + 1] += f.y;
            }
        }
        uint4 o;
        __nv_bfloat162* h = reinterpret_cast<__nv_bfloat162*>(&o);
#pragma unroll
        for (int j = 0; j < 4; ++j) h[j] = __floats2bfloat162_rn(s[2 * j], s[2 * j + 1]);
        *reinterpret_cast<uint4*>(coarse + V * C + cv * 8) = o;
    }
}

// ---------------------------------------------------------------------------------------
// head: pred = w . d + b (16 channels -> 1, FP32)
constexpr int kHeadC = 16;

__global__ void head_fwd_kernel(long long n, const __nv_bfloat16* __restrict__ d, const float* __restrict__ w,
                                const float* __restrict__ b, float* __restrict__ pred) {
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < n; v += (long long)gridDim.x * blockDim.x) {
        const uint4* p = reinterpret_cast<const uint4*>(d + v * kHeadC);
        float s = b[0];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const uint4 u = __ldg(p + h);
            const __nv_bfloat162* q = reinterpret_cast<const __nv_bfloat162*>(&u);
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const float2 f = __bfloat1622float2(q[j]);
                s += w[h * 8 + 2 * j] * f.x + w[h * 8 + 2 * j + 1] * f.y;
            }
        }
        pred[v] = s;
    }
}

// Masked mean-square loss and the head's backward: e = pred - target on cells with mask != 0,
// loss += e^2 * inv_n, g = 2 e inv_n, grad_d = g w (bf16), dw += g d, db += g.  Totals by a
// deterministic grid reduction, added to loss (FP64) and to the head's FP32 gradients.
__global__ void head_loss_bwd_kernel(long long n, const __nv_bfloat16* __restrict__ d, const float* __restrict__ pred,
                                     const float* __restrict__ target, const uint8_t* __restrict__ mask,
                                     const float* __restrict__ w, double inv_n, __nv_bfloat16* __restrict__ grad_d,
                                     double* __restrict__ loss, float* __restrict__ dw, float* __restrict__ db,
                                     double* partials, unsigned* counter) {
    double acc[18];
#pragma unroll
    for (int q = 0; q < 18; ++q) acc[q] = 0.0;
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < n; v += (long long)gridDim.x * blockDim.x) {
        float gv = 0.f;
        if (mask[v]) {
            const float e = pred[v] - target[v];
            acc[0] += (double)e * e * inv_n;
            gv = (float)(2.0 * inv_n) * e;
        }
        const uint4* p = reinterpret_cast<const uint4*>(d + v * kHeadC);
        uint4* o = reinterpret_cast<uint4*>(grad_d + v * kHeadC);
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const uint4 u = __ldg(p + h);
            const __nv_bfloat162* q = reinterpret_cast<const __nv_bfloat162*>(&u);
            uint4 go;
            __nv_bfloat162* gq = reinterpret_cast<__nv_bfloat162*>(&go);
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const float2 f = __bfloat1622float2(q[j]);
                const int c = h * 8 + 2 * j;
                acc[1 + c] += (double)gv * f.x;
                acc[2 + c] += (double)gv * f.y;
                gq[j] = __floats2bfloat162_rn(gv * w[c], gv * w[c + 1]);
            }
            o[h] = go;
        }
        acc[17] += gv;
    }
    double tot[18];
    if (grid_sum<18>(acc, partials, counter, tot)) {
        loss[0] += tot[0];
#pragma unroll
        for (int q = 0; q < kHeadC; ++q) dw[q] += (float)tot[1 + q];
        db[0] += (float)tot[17];
    }
}

// Energy-norm loss and the head's backward.  With e = pred - target on fluid cells and A^ the
// scaled operator in Laplacian form (per cell: the diagonal excess delta and the face weights w
// with +x, +y, +z, all >= 0), the loss is e . A^ e * inv_n = (sum_faces w (e_c - e_n)^2 +
// sum delta e^2) * inv_n -- the error in the norm that conjugate gradients minimises, positive
// whatever the rounding of the weights -- and its gradient 2 (A^ e) inv_n with
// (A^ e)_c = delta e_c + sum_n w (e_c - e_n).  The rest as head_loss_bwd_kernel.
__device__ __forceinline__ float4 load_coup(const __nv_bfloat16* coup, long long v) {
    const uint2 q = __ldg(reinterpret_cast<const uint2*>(coup + v * 4));
    const __nv_bfloat162* h = reinterpret_cast<const __nv_bfloat162*>(&q);
    const float2 a = __bfloat1622float2(h[0]), b = __bfloat1622float2(h[1]);
    return make_float4(a.x, a.y, b.x, b.y);
}

__global__ void head_energy_bwd_kernel(int X, int Y, int Z, const __nv_bfloat16* __restrict__ d,
                                       const float* __restrict__ pred, const float* __restrict__ target,
                                       const __nv_bfloat16* __restrict__ coup, const uint8_t* __restrict__ fluid,
                                       const float* __restrict__ w,
                                       double inv_n, __nv_bfloat16* __restrict__ grad_d, double* __restrict__ loss,
                                       float* __restrict__ dw, float* __restrict__ db, double* partials,
                                       unsigned* counter) {
    const long long n = (long long)X * Y * Z;
    const long long sy = X, sz = (long long)X * Y;
    double acc[18];
#pragma unroll
    for (int q = 0; q < 18; ++q) acc[q] = 0.0;
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < n; v += (long long)gridDim.x * blockDim.x) {
        const int x = (int)(v % X), y = (int)((v / X) % Y), z = (int)(v / sz);
        const float4 cv = load_coup(coup, v);
        float gv = 0.f;
        if (fluid[v]) {
            const float e = pred[v] - target[v];
            float r = cv.x * e;                     // delta e
            double en = (double)cv.x * e * e;       // this cell's share of the energy: delta e^2
            auto face = [&](float w, long long q) { // a face to a fluid neighbour (w > 0 only then)
                if (w != 0.f) {
                    const float de = e - (pred[q] - target[q]);
                    r += w * de;
                    en += 0.5 * (double)w * de * de;  // each face is seen from both cells
                }
            };
            if (x + 1 < X) face(cv.y, v + 1);
            if (y + 1 < Y) face(cv.z, v + sy);
            if (z + 1 < Z) face(cv.w, v + sz);
            if (x > 0) face(load_coup(coup, v - 1).y, v - 1);
            if (y > 0) face(load_coup(coup, v - sy).z, v - sy);
            if (z > 0) face(load_coup(coup, v - sz).w, v - sz);
            acc[0] += en * inv_n;
            gv = (float)(2.0 * inv_n) * r;
        }
        const uint4* p = reinterpret_cast<const uint4*>(d + v * kHeadC);
        uint4* o = reinterpret_cast<uint4*>(grad_d + v * kHeadC);
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const uint4 u = __ldg(p + h);
            const __nv_bfloat162* q = reinterpret_cast<const __nv_bfloat162*>(&u);
            uint4 go;
            __nv_bfloat162* gq = reinterpret_cast<__nv_bfloat162*>(&go);
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const float2 f = __bfloat1622float2(q[j]);
                const int c = h * 8 + 2 * j;
                acc[1 + c] += (double)gv * f.x;
                acc[2 + c] += (double)gv * f.y;
                gq[j] = __floats2bfloat162_rn(gv * w[c], gv * w[c + 1]);
            }
            o[h] = go;
        }
        acc[17] += gv;
    }
    double tot[18];
    if (grid_sum<18>(acc, partials, counter, tot)) {
        loss[0] += tot[0];
#pragma unroll
        for (int q = 0; q < kHeadC; ++q) dw[q] += (float)tot[1 + q];
        db[0] += (float)tot[17];
    }
}

// Adam on FP32 parameters; the gradient is zeroed for the next accumulation.
__global__ void adam_kernel(long long n, float* __restrict__ w, float* __restrict__ g, float* __restrict__ m,
                            float* __restrict__ v, float lr, float b1, float b2, float eps, float c1, float c2) {
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        const float ge = g[e];
        const float me = b1 * m[e] + (1.f - b1) * ge;
        const float ve = b2 * v[e] + (1.f - b2) * ge * ge;
        m[e] = me;
        v[e] = ve;
        w[e] -= lr * (me * c1) / (sqrtf(ve * c2) + eps);
        g[e] = 0.f;
    }
}

}  // namespace nn
}  // namespace el

// =========================================================================================
// host side: launchers and the C ABI (include/eulerian_liquid_gb300.h, "learned warm start")
#include <algorithm>

using namespace el;
using namespace el::nn;

namespace {

int num_sms_current() {
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return sms;
}

// resident CTAs per SM for a kernel of `threads` threads and `smem` dynamic shared bytes, from the
// device's shared memory per SM (the occupancy query alone reported one CTA per SM for these)
int resident_per_sm(int threads, int smem) {
    int dev = 0, per_sm_smem = 0, reserved = 0, max_threads = 2048;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&per_sm_smem, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
    cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, dev);
    cudaDeviceGetAttribute(&max_threads, cudaDevAttrMaxThreadsPerMultiProcessor, dev);
    const int by_smem = per_sm_smem / (smem + reserved);
    return std::max(1, std::min(by_smem, max_threads / threads));
}

int grid_elems(long long n) { return (int)std::max<long long>(1, std::min<long long>((n + 255) / 256, 152LL * 16)); }

ConvIn conv_in(const el_nn_conv_args* a) {
    ConvIn in;
    in.a = static_cast<const __nv_bfloat16*>(a->in_a);
    in.b = static_cast<const __nv_bfloat16*>(a->in_b);
    in.mask = static_cast<const __nv_bfloat16*>(a->mask);
    in.ca = a->ca;
    in.cb = a->cb;
    in.up_a = a->upsample_a;
    in.ax = a->upsample_a ? a->nx / 2 : a->nx;
    in.ay = a->upsample_a ? a->ny / 2 : a->ny;
    in.az = a->upsample_a ? a->nz / 2 : a->nz;
    return in;
}

template <int CIN, int COUT>
int launch_conv(const el_nn_conv_args* a, cudaStream_t s) {
    const size_t smem = (size_t)kHV * (CIN + 8) * sizeof(__nv_bfloat16);
    if (cudaFuncSetAttribute(conv3_kernel<CIN, COUT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
        cudaSuccess)
        return EL_ERR_CUDA;
    const dim3 grid((a->nx + kTX - 1) / kTX, (a->ny + kTY - 1) / kTY, a->nz);
    conv3_kernel<CIN, COUT><<<grid, kThreads, smem, s>>>(
        a->nx, a->ny, a->nz, conv_in(a), static_cast<const uint4*>(a->weights), a->bias, a->relu,
        static_cast<__nv_bfloat16*>(a->out_a), a->out_a_channels, static_cast<__nv_bfloat16*>(a->out_b));
    return cudaGetLastError() == cudaSuccess ? EL_OK : EL_ERR_CUDA;
}

template <int CIN, int COUT>
int launch_conv_tc_pipe(const el_nn_conv_args* a, cudaStream_t s) {
    using S = tc::PipeShape<CIN, COUT>;
    // the largest shared-memory carve-out, so that the occupancy below (and the launch) get it
    if (cudaFuncSetAttribute(tc::conv3_tc_pipe_kernel<CIN, COUT>, cudaFuncAttributePreferredSharedMemoryCarveout,
                             (int)cudaSharedmemCarveoutMaxShared) != cudaSuccess)
        return EL_ERR_CUDA;
    if (cudaFuncSetAttribute(tc::conv3_tc_pipe_kernel<CIN, COUT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             S::SMEM) != cudaSuccess)
        return EL_ERR_CUDA;
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, tc::conv3_tc_pipe_kernel<CIN, COUT>, tc::kThreads,
                                                      S::SMEM) != cudaSuccess)
        return EL_ERR_CUDA;
    per_sm = std::max(per_sm, resident_per_sm(tc::kThreads, S::SMEM));
    const long long bricks =
        (long long)((a->nx + tc::TX - 1) / tc::TX) * ((a->ny + tc::TY - 1) / tc::TY) * a->nz;
    const int grid = (int)std::max<long long>(1, std::min<long long>(bricks, (long long)num_sms_current() * per_sm));
    tc::conv3_tc_pipe_kernel<CIN, COUT><<<grid, tc::kThreads, S::SMEM, s>>>(
        a->nx, a->ny, a->nz, conv_in(a), static_cast<const uint4*>(a->weights_tc), a->bias, a->relu,
        static_cast<__nv_bfloat16*>(a->out_a), a->out_a_channels, static_cast<__nv_bfloat16*>(a->out_b));
    return cudaGetLastError() == cudaSuccess ? EL_OK : EL_ERR_CUDA;
}

template <int CIN, int COUT>
int launch_conv_tc(const el_nn_conv_args* a, cudaStream_t s) {
    if constexpr (tc::PipeShape<CIN, COUT>::FITS) return launch_conv_tc_pipe<CIN, COUT>(a, s);
    using S = tc::Shape<CIN, COUT>;
    // the largest shared-memory carve-out, so that the occupancy below (and the launch) get it
    if (cudaFuncSetAttribute(tc::conv3_tc_kernel<CIN, COUT>, cudaFuncAttributePreferredSharedMemoryCarveout,
                             (int)cudaSharedmemCarveoutMaxShared) != cudaSuccess)
        return EL_ERR_CUDA;
    if (cudaFuncSetAttribute(tc::conv3_tc_kernel<CIN, COUT>, cudaFuncAttributeMaxDynamicSharedMemorySize, S::SMEM) !=
        cudaSuccess)
        return EL_ERR_CUDA;
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, tc::conv3_tc_kernel<CIN, COUT>, tc::kThreads,
                                                      S::SMEM) != cudaSuccess)
        return EL_ERR_CUDA;
    per_sm = std::max(per_sm, resident_per_sm(tc::kThreads, S::SMEM));
    const long long bricks =
        (long long)((a->nx + tc::TX - 1) / tc::TX) * ((a->ny + tc::TY - 1) / tc::TY) * a->nz;
    const int grid = (int)std::max<long long>(1, std::min<long long>(bricks, (long long)num_sms_current() * per_sm));
    tc::conv3_tc_kernel<CIN, COUT><<<grid, tc::kThreads, S::SMEM, s>>>(
        a->nx, a->ny, a->nz, conv_in(a), static_cast<const uint4*>(a->weights_tc), a->bias, a->relu,
        static_cast<__nv_bfloat16*>(a->out_a), a->out_a_channels, static_cast<__nv_bfloat16*>(a->out_b));
    return cudaGetLastError() == cudaSuccess ? EL_OK : EL_ERR_CUDA;
}

template <int CIN, int COUT>
int wgrad_splits(int nx, int ny, int nz) {
    const long long bricks = (long long)((nx + kTX - 1) / kTX) * ((ny + kTY - 1) / kTY) * nz;
    const int want = (2 * num_sms_current() + WGrad<CIN, COUT>::GROUPS - 1) / WGrad<CIN, COUT>::GROUPS;
    return (int)std::max<long long>(1, std::min<long long>(want, bricks));
}

template <int CIN, int COUT>
size_t wgrad_ws(int nx, int ny, int nz) {
    const int ns = wgrad_splits<CIN, COUT>(nx, ny, nz);
    return ((size_t)ns * 27 * CIN * COUT + (size_t)ns * COUT) * sizeof(float);
}

template <int CIN, int COUT>
int launch_wgrad(const el_nn_conv_args* a, const void* grad_out, float* dw, float* db, void* ws, size_t ws_bytes,
                 cudaStream_t s) {
    using W = WGrad<CIN, COUT>;
    const int ns = wgrad_splits<CIN, COUT>(a->nx, a->ny, a->nz);
    if (ws_bytes < wgrad_ws<CIN, COUT>(a->nx, a->ny, a->nz)) return EL_ERR_INVALID_ARGUMENT;
    float* part_w = static_cast<float*>(ws);
    float* part_b = part_w + (size_t)ns * 27 * CIN * COUT;
    const size_t smem = ((size_t)kHV * (CIN + 8) + 128 * (COUT + 8)) * sizeof(__nv_bfloat16);
    if (cudaFuncSetAttribute(conv3_wgrad_kernel<CIN, COUT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
        cudaSuccess)
        return EL_ERR_CUDA;
    conv3_wgrad_kernel<CIN, COUT><<<dim3(W::GROUPS, ns), kThreads, smem, s>>>(
        a->nx, a->ny, a->nz, conv_in(a), static_cast<const __nv_bfloat16*>(grad_out),
        static_cast<const __nv_bfloat16*>(a->out_a), ns, part_w, part_b);
    const long long n = 27LL * CIN * COUT + COUT;
    wgrad_reduce_kernel<<<grid_elems(n), 256, 0, s>>>(CIN, COUT, ns, part_w, part_b, dw, db);
    return cudaGetLastError() == cudaSuccess ? EL_OK : EL_ERR_CUDA;
}

// (cin, cout) pairs of the network, forward and backward-data
#define EL_NN_CONV_PAIRS(X)                                                                                      \
    X(16, 16) X(16, 32) X(32, 32) X(32, 64) X(64, 64) X(128, 64) X(96, 32) X(48, 16) X(32, 16) X(64, 32) X(64, 128) \
        X(32, 96) X(16, 48)
// pairs whose 27 taps of weights fit in shared memory with the input brick: the tcgen05 kernel
#define EL_NN_TC_PAIRS(X) \
    X(16, 16) X(16, 32) X(32, 32) X(32, 64) X(48, 16) X(32, 16) X(64, 32) X(16, 48) X(32, 96)
// forward pairs (backward weight)
#define EL_NN_FWD_PAIRS(X) X(16, 16) X(16, 32) X(32, 32) X(32, 64) X(64, 64) X(128, 64) X(96, 32) X(48, 16)

bool valid_conv(const el_nn_conv_args* a) {
    if (!a || a->nx < 1 || a->ny < 1 || a->nz < 1 || a->ca < 0 || a->cb < 0 || a->ca % 8 || a->cb % 8 ||
        a->ca + a->cb != a->cin || !a->in_a)
        return false;
    if (a->upsample_a && (a->nx % 2 || a->ny % 2 || a->nz % 2)) return false;
    return true;
}

}  // namespace

#define EL_API extern "C" __attribute__((visibility("default")))

EL_API int el_nn_tc_supported(int cin, int cout) {
#define EL_NN_CASE(CI, CO) \
    if (cin == CI && cout == CO) return 1;
    EL_NN_TC_PAIRS(EL_NN_CASE)
#undef EL_NN_CASE
    return 0;
}

// pairs where the tcgen05 kernel measured faster than the mma.sync one on GB300 (128^3 network
// grids): the small-cin layers; with cin >= 32 and cout <= 64 the persistent tcgen05 CTAs are
// limited to one or two per SM by the staged weights and lose to the register-tiled kernel
EL_API int el_nn_tc_preferred(int cin, int cout) {
    return (cin == 16 && (cout == 16 || cout == 32 || cout == 48)) || (cin == 32 && cout == 96);
}

EL_API int el_nn_take_error(void) {
    int e = 0;
    const int zero = 0;
    if (cudaMemcpyFromSymbol(&e, tc::g_error, sizeof(int)) != cudaSuccess) return -1;
    if (e && cudaMemcpyToSymbol(tc::g_error, &zero, sizeof(int)) != cudaSuccess) return -1;
    return e;
}

EL_API int el_nn_conv3_forward(const el_nn_conv_args* a, void* stream) {
    if (a && a->weights_tc && el_nn_tc_supported(a->cin, a->cout) && valid_conv(a) && a->out_a &&
        a->out_a_channels > 0 && a->out_a_channels <= a->cout && a->out_a_channels % 8 == 0 &&
        (a->out_a_channels == a->cout || a->out_b)) {
        cudaStream_t s = static_cast<cudaStream_t>(stream);
#define EL_NN_CASE(CI, CO) \
        if (a->cin == CI && a->cout == CO) return launch_conv_tc<CI, CO>(a, s);
        EL_NN_TC_PAIRS(EL_NN_CASE)
#undef EL_NN_CASE
    }
    if (!valid_conv(a) || !a->weights || !a->out_a || a->out_a_channels <= 0 || a->out_a_channels > a->cout ||
        a->out_a_channels % 8 || (a->out_a_channels < a->cout && !a->out_b))
        return EL_ERR_INVALID_ARGUMENT;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
#define EL_NN_CASE(CI, CO) \
    if (a->cin == CI && a->cout == CO) return launch_conv<CI, CO>(a, s);
    EL_NN_CONV_PAIRS(EL_NN_CASE)
#undef EL_NN_CASE
    return EL_ERR_INVALID_ARGUMENT;
}

EL_API size_t el_nn_conv3_backward_weight_workspace(int nx, int ny, int nz, int cin, int cout) {
#define EL_NN_CASE(CI, CO) \
    if (cin == CI && cout == CO) return wgrad_ws<CI, CO>(nx, ny, nz);
    EL_NN_FWD_PAIRS(EL_NN_CASE)
#undef EL_NN_CASE
    return 0;
}

EL_API int el_nn_conv3_backward_weight(const el_nn_conv_args* a, const void* grad_out, float* dw, float* db,
                                       void* workspace, size_t workspace_bytes, void* stream) {
    if (!valid_conv(a) || !a->out_a || !grad_out || !dw || !workspace) return EL_ERR_INVALID_ARGUMENT;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
#define EL_NN_CASE(CI, CO) \
    if (a->cin == CI && a->cout == CO) return launch_wgrad<CI, CO>(a, grad_out, dw, db, workspace, workspace_bytes, s);
    EL_NN_FWD_PAIRS(EL_NN_CASE)
#undef EL_NN_CASE
    return EL_ERR_INVALID_ARGUMENT;
}

EL_API size_t el_nn_packed_weight_bytes(int cin, int cout) { return (size_t)27 * cin * cout * sizeof(__nv_bfloat16); }

EL_API int el_nn_pack_weights(int cin, int cout, const float* w, void* packed_fwd, void* packed_bwd, void* stream) {
    if (cin % 16 || cout % 16 || cin <= 0 || cout <= 0 || !w || !packed_fwd) return EL_ERR_INVALID_ARGUMENT;
    const long long n = 27LL * cin * cout;
    pack_weights_kernel<<<grid_elems(n), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        cin, cout, w, static_cast<__nv_bfloat16*>(packed_fwd), static_cast<__nv_bfloat16*>(packed_bwd));
    return cudaGetLastError() == cudaSuccess ? EL_OK : EL_ERR_CUDA;
}

EL_API int el_nn_pack_weights_tc(int cin, int cout, const float* w, void* packed_fwd, void* packed_bwd,
                                  void* stream) {
    if (cin % 16 || cout % 16 || cin <= 0 || cout <= 0 || !w || !packed_fwd) return EL_ERR_INVALID_ARGUMENT;
    const long long n = 27LL * cin * cout;
    tc::pack_weights_tc_kernel<<<grid_elems(n), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        cin, cout, w, static_cast<__nv_bfloat16*>(packed_fwd), static_cast<__nv_bfloat16*>(packed_bwd));
    return cudaGetLastError() == cudaSuccess ? EL_OK : EL_ERR_CUDA;
}

EL_API int el_nn_pool(int nx, int ny, int nz, int c, const void* in, void* out, void* stream) {
    if (nx % 2 || ny % 2 || nz % 2 || c % 8 || !in || !out) return EL_ERR_INVALID_ARGUMENT;
    const long long n = (long long)(nx / 2) * (ny / 2) * (nz / 2) * (c / 8);
    pool_fwd_kernel<<<grid_elems(n), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        nx, ny, nz, c, static_cast<const __nv_bfloat16*>(in), static_cast<__nv_bfloat16*>(out));
    return cudaGetLastError() == cudaSuccess ? EL_OK : EL_ERR_CUDA;
}

EL_API int el_nn_spread(int nx, int ny, int nz, int c, const void* coarse, void* fine, float scale, int accumulate,
                        void* stream) {
    if (nx % 2 || ny % 2 || nz % 2 || c % 8 || !coarse || !fine) return EL_ERR_INVALID_ARGUMENT;
    const long long n = (long long)nx * ny * nz * (c / 8);
    spread_kernel<<<grid_elems(n), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        nx, ny, nz, c, static_cast<const __nv_bfloat16*>(coarse), static_cast<__nv_bfloat16*>(fine), scale, accumulate);
    return cudaGetLastError() == cudaSuccess ? EL_OK : EL_ERR_CUDA;
}

EL_API int el_nn_gather8(int nx, int ny, int nz, int c, const void* fine, void* coarse, void* stream) {
    if (nx % 2 || ny % 2 || nz % 2 || c % 8 || !coarse || !fine) return EL_ERR_INVALID_ARGUMENT;
    const long long n = (long long)(nx / 2) * (ny / 2) * (nz / 2) * (c / 8);
    gather8_kernel<<<grid_elems(n), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        nx, ny, nz, c, static_cast<const __nv_bfloat16*>(fine), static_cast<__nv_bfloat16*>(coarse));
    return cudaGetLastError() == cudaSuccess ? EL_OK : EL_ERR_CUDA;
}

EL_API int el_nn_head_forward(int64_t n, const void* d, const float* w, const float* b, float* pred, void* stream) {
    if (n < 0 || !d || !w || !b || !pred) return EL_ERR_INVALID_ARGUMENT;
    head_fwd_kernel<<<grid_elems(n), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        n, static_cast<const __nv_bfloat16*>(d), w, b, pred);
    return cudaGetLastError() == cudaSuccess ? EL_OK : EL_ERR_CUDA;
}

EL_API size_t el_nn_head_workspace(int64_t n) { return (size_t)grid_elems(n) * 18 * sizeof(double) + 64; }

EL_API int el_nn_head_loss_backward(int64_t n, const void* d, const float* pred, const float* target,
                                    const uint8_t* mask, const float* w, double inv_n, void* grad_d, double* loss,
                                    float* dw, float* db, void* workspace, size_t workspace_bytes, void* stream) {
    if (n < 0 || !d || !pred || !target || !mask || !w || !grad_d || !loss || !dw || !db || !workspace ||
        workspace_bytes < el_nn_head_workspace(n))
        return EL_ERR_INVALID_ARGUMENT;
    const int blocks = grid_elems(n);
    double* partials = static_cast<double*>(workspace);
    unsigned* counter = reinterpret_cast<unsigned*>(static_cast<char*>(workspace) + (size_t)blocks * 18 * sizeof(double));
    head_loss_bwd_kernel<<<blocks, 256, 0, static_cast<cudaStream_t>(stream)>>>(
        n, static_cast<const __nv_bfloat16*>(d), pred, target, mask, w, inv_n, static_cast<__nv_bfloat16*>(grad_d),
        loss, dw, db, partials, counter);
    return cudaGetLastError() == cudaSuccess ? EL_OK : EL_ERR_CUDA;
}

EL_API int el_nn_head_energy_loss_backward(int nx, int ny, int nz, const void* d, const float* pred,
                                           const float* target, const void* couplings, const uint8_t* fluid,
                                           const float* w, double inv_n, void* grad_d, double* loss, float* dw,
                                           float* db, void* workspace, size_t workspace_bytes, void* stream) {
    const int64_t n = (int64_t)nx * ny * nz;
    if (nx < 1 || ny < 1 || nz < 1 || !d || !pred || !target || !couplings || !fluid || !w || !grad_d || !loss ||
        !dw || !db ||
        !workspace || workspace_bytes < el_nn_head_workspace(n))
        return EL_ERR_INVALID_ARGUMENT;
    const int blocks = grid_elems(n);
    double* partials = static_cast<double*>(workspace);
    unsigned* counter = reinterpret_cast<unsigned*>(static_cast<char*>(workspace) + (size_t)blocks * 18 * sizeof(double));
    head_energy_bwd_kernel<<<blocks, 256, 0, static_cast<cudaStream_t>(stream)>>>(
        nx, ny, nz, static_cast<const __nv_bfloat16*>(d), pred, target, static_cast<const __nv_bfloat16*>(couplings),
        fluid, w, inv_n, static_cast<__nv_bfloat16*>(grad_d), loss, dw, db, partials, counter);
    return cudaGetLastError() == cudaSuccess ? EL_OK : EL_ERR_CUDA;
}

EL_API int el_nn_adam(int64_t n, float* w, float* g, float* m, float* v, float lr, float beta1, float beta2,
                      float eps, int step, void* stream) {
    if (n < 0 || !w || !g || !m || !v || step < 1) return EL_ERR_INVALID_ARGUMENT;
    const float c1 = 1.f / (1.f - powf(beta1, (float)step));
    const float c2 = 1.f / (1.f - powf(beta2, (float)step));
    adam_kernel<<<grid_elems(n), 256, 0, static_cast<cudaStream_t>(stream)>>>(n, w, g, m, v, lr, beta1, beta2, eps, c1,
                                                                              c2);
    return cudaGetLastError() == cudaSuccess ? EL_OK : EL_ERR_CUDA;
}
