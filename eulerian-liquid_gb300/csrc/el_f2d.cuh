// el_f2d.cuh -- float <-> double conversions on the integer pipe.
//
// This GPU's FP64 pipe runs at a small fraction of its integer rate, and the conversion
// instructions between float and double occupy it: in the kernels bound by that pipe (the
// matrix build's double sums, the FP64 refinement residual) the conversions of the float
// weights, couplings and products were a third of its instructions.  Both conversions here are
// exact bit arithmetic throughout, rare inputs (subnormal, infinite, NaN) included: a branch to
// the conversion instruction for those would still cost an FP64 issue slot on every call where
// the compiler predicates it.  The same value as the conversion for every input (host tests);
// host and device compile the same code.
#pragma once

#include <cstdint>
#include <cstring>

#if defined(__CUDACC__)
#define EL_F2D_HD __host__ __device__ __forceinline__
#else
#define EL_F2D_HD inline
#endif

namespace el {

EL_F2D_HD int clz32(uint32_t x) {
#if defined(__CUDA_ARCH__)
    return __clz((int)x);
#else
    return x ? __builtin_clz(x) : 32;
#endif
}

EL_F2D_HD double f2d(float f) {
    uint32_t u;
    std::memcpy(&u, &f, sizeof(u));
    const uint32_t sign = u & 0x80000000u, mag = u & 0x7fffffffu;
    const uint32_t e = mag >> 23, m = mag & 0x7fffffu;
    uint32_t hi, lo;
    if (e - 1u < 254u) {
        hi = sign | ((e + 896u) << 20) | (m >> 3);
        lo = m << 29;
    } else if (e == 0u) {
        if (m == 0u) {
            hi = sign;
            lo = 0u;
        } else {
            // subnormal: m 2^-149 with m's top bit at p, normal as a double
            const int p = 31 - clz32(m);
            const uint64_t mm = ((uint64_t)m << (52 - p)) & 0xfffffffffffffull;
            hi = sign | ((uint32_t)(p + 874) << 20) | (uint32_t)(mm >> 32);
            lo = (uint32_t)mm;
        }
    } else {
        // infinity; NaN quietened, its payload kept
        hi = sign | 0x7ff00000u | (m >> 3) | (m ? 0x80000u : 0u);
        lo = m << 29;
    }
    const uint64_t bits = ((uint64_t)hi << 32) | (uint64_t)lo;
    double d;
    std::memcpy(&d, &bits, sizeof(d));
    return d;
}

EL_F2D_HD double f2d(double d) { return d; }

// double -> float, round to nearest even, on the integer pipe: for a normal float result the 23
// mantissa bits are kept and the 29 below them decide the rounding (a carry out of the mantissa
// moves into the exponent, up to infinity); a subnormal result is the 53-bit significand shifted
// to units of 2^-149 and rounded the same way; beyond the float range infinity; zero keeps its
// sign, NaN stays NaN.  The same value as the conversion for every non-NaN input (a host test
// checks every exponent at the rounding boundaries and random patterns).
EL_F2D_HD float d2f(double d) {
    uint64_t bits;
    std::memcpy(&bits, &d, sizeof(bits));
    const uint32_t hi = (uint32_t)(bits >> 32), lo = (uint32_t)bits;
    const uint32_t sign = hi & 0x80000000u, em = hi & 0x7fffffffu;
    const uint32_t e = em >> 20;
    uint32_t fb;
    if (e >= 897u && e <= 1150u) {
        const uint32_t m = ((em & 0xfffffu) << 3) | (lo >> 29);
        const uint32_t rem = lo & 0x1fffffffu;
        const uint32_t up = (rem > 0x10000000u || (rem == 0x10000000u && (m & 1u))) ? 1u : 0u;
        fb = sign | (((e - 896u) << 23) + m + up);
    } else if (e > 1150u) {
        const bool nan = e == 2047u && ((em & 0xfffffu) | lo) != 0u;
        fb = sign | (nan ? (0x7fc00000u | ((em & 0xfffffu) << 3) | (lo >> 29)) : 0x7f800000u);
    } else if (e < 872u) {
        fb = sign;  // below half the smallest subnormal (and zero)
    } else {
        const uint64_t sig = ((uint64_t)((em & 0xfffffu) | 0x100000u) << 32) | (uint64_t)lo;
        const uint32_t sh = 926u - e;  // 30 .. 54
        const uint64_t q = sig >> sh, rem = sig & ((1ull << sh) - 1ull), half = 1ull << (sh - 1u);
        const uint64_t up = (rem > half || (rem == half && (q & 1ull))) ? 1ull : 0ull;
        fb = sign | (uint32_t)(q + up);
    }
    float f;
    std::memcpy(&f, &fb, sizeof(f));
    return f;
}

}  // namespace el
