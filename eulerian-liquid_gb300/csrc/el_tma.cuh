// el_tma.cuh -- tensor-memory-accelerator copies of 3-D boxes into shared memory, with the
// mbarriers that count their bytes (the solver's tile kernels and the advection tiles).
//
// A box copy (cp.async.bulk.tensor) lands a [z][y][x] box of an i-fastest array in shared
// memory and completes a transaction count on an mbarrier; the box's parts outside the array
// arrive as zeros.  A copy's innermost coordinate times the element size must be a multiple of
// 16 bytes, and so must the array's row pitch and plane pitch (the tensor map checks the
// pitches and the base address, not the coordinate): callers start every box on a multiple of
// 4 floats (2 doubles).
#pragma once

#include <cuda.h>
#include <cudaTypedefs.h>

#include <cstdint>

namespace el {

__device__ __forceinline__ unsigned smem_u32(const void* p) {
    return static_cast<unsigned>(__cvta_generic_to_shared(p));
}

// dynamic shared memory rounded up to a 128-byte boundary (the launch reserves 128 bytes of
// slack); box copies land at 128-byte aligned addresses
__device__ __forceinline__ unsigned char* align128(unsigned char* raw) {
    const unsigned a = smem_u32(raw);
    return raw + ((128u - (a & 127u)) & 127u);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// makes initialised mbarriers visible to the copy engine
__device__ __forceinline__ void mbar_init_fence() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// a bounded wait: this many polls (each try_wait may itself suspend for a while) before the
// caller gives up, records the fault and stops
constexpr long long kWaitPolls = 1ll << 24;

// bounded wait for the completion of the phase with the given parity
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, unsigned parity) {
    for (long long n = 0; n < kWaitPolls; ++n)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, uint64_t* bar, int x, int y, int z) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
        "[%5];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
        : "memory");
}

// ---- host side -------------------------------------------------------------------------

// the driver's tensor-map encoder, found once through the runtime (null if unavailable)
inline PFN_cuTensorMapEncodeTiled_v12000 tma_encode_fn() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static bool tried = false;
    if (!tried) {
        tried = true;
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }
    return fn;
}

// A 3-D tensor map over an i-fastest array of d0 x n1 x n2 elements of `type` (row pitch
// row_elems) copying boxes of bx x by x bz; false when the encoder refuses it (a base address
// or pitch not a multiple of 16 bytes, a box over 256 elements a side) or is unavailable.
inline bool tma_encode_3d(CUtensorMap* map, CUtensorMapDataType type, int esize, const void* base, long long d0,
                          int n1, int n2, long long row_elems, unsigned bx, unsigned by, unsigned bz = 1) {
    auto fn = tma_encode_fn();
    if (!fn) return false;
    if ((reinterpret_cast<uintptr_t>(base) & 15) != 0 || ((row_elems * esize) & 15) != 0) return false;
    const cuuint64_t dims[3] = {(cuuint64_t)d0, (cuuint64_t)n1, (cuuint64_t)n2};
    const cuuint64_t strides[2] = {(cuuint64_t)(row_elems * esize), (cuuint64_t)(row_elems * esize * n1)};
    const cuuint32_t box[3] = {bx, by, bz};
    const cuuint32_t estr[3] = {1, 1, 1};
    return fn(map, type, 3, const_cast<void*>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
              CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace el
