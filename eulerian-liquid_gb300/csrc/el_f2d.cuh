// el_f2d.cuh -- float -> double conversion on the integer pipe.
//
// This GPU's FP64 pipe runs at a small fraction of its integer rate, and the float -> double
// conversion instruction occupies it: in the kernels bound by that pipe (the matrix build's
// double sums, the FP64 refinement residual) the conversions of the float weights, couplings
// and products were a third of its instructions.  The conversion is exact bit arithmetic: the
// exponent rebased (bias 127 -> 1023) and the 23-bit mantissa shifted into the 52-bit one; zero
// keeps its sign; subnormal, infinite and NaN inputs, which a rebase does not cover, take the
// conversion itself.  The same value as the conversion for every input (a host test checks all
// 2^32 bit patterns); host and device compile the same code.
#pragma once

#include <cstdint>
#include <cstring>

#if defined(__CUDACC__)
#define EL_F2D_HD __host__ __device__ __forceinline__
#else
#define EL_F2D_HD inline
#endif

namespace el {

EL_F2D_HD double f2d(float f) {
    uint32_t u;
    std::memcpy(&u, &f, sizeof(u));
    const uint32_t mag = u & 0x7fffffffu;
    const uint32_t e = mag >> 23;
    uint64_t bits;
    if (mag == 0u) {
        bits = (uint64_t)(u & 0x80000000u) << 32;
    } else if (e == 0u || e == 0xffu) {
        return (double)f;
    } else {
        const uint32_t hi = (u & 0x80000000u) | ((e + 896u) << 20) | ((mag >> 3) & 0xfffffu);
        bits = ((uint64_t)hi << 32) | (uint64_t)(u << 29);
    }
    double d;
    std::memcpy(&d, &bits, sizeof(d));
    return d;
}

EL_F2D_HD double f2d(double d) { return d; }

}  // namespace el
