// el_df.cuh -- double-float arithmetic on the FP32 pipe for the mixed solver's refinement
// residual.
//
// This GPU issues FP64 operations at about one per clock per SM, against 128 FP32 operations:
// the FP64 refinement residual r = b - A x (nine FP64 operations a cell) kept its FP64 pipe 86 %
// busy and took several times its memory time.  A value here is a pair of floats h + l (a
// "double-float"): a double is split into its top 24 significant bits and the next 23 by integer
// arithmetic, products of a float coupling with a pair are exact by FMA (two-product), and the
// seven products are summed by the error-free transformation TwoSum with the rounding errors
// collected in a second float (the cascaded summation of Ogita, Rump and Oishi, "Accurate sum and
// dot product", SIAM J. Sci. Comput. 26, 2005).  The pair's value differs from the exact residual
// of the stored operands by less than 2^-41 of the sum of the terms' magnitudes (the summation's
// bound with the splits' truncation; below 2^-44 in the host test's rows), against 2^-50 or so
// for FP64 arithmetic, plus 2^-126 for each operand below 2^-103; the refinement stops at a
// relative residual of 1e-6 or above.  A host test compares the routines with exact
// rational arithmetic; host and device compile the same code.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>

#include "el_f2d.cuh"

namespace el {

struct F2 {
    float h, l;  // the value h + l
};

#if defined(__CUDA_ARCH__)
EL_F2D_HD float df_add(float a, float b) { return __fadd_rn(a, b); }
EL_F2D_HD float df_sub(float a, float b) { return __fsub_rn(a, b); }
EL_F2D_HD float df_mul(float a, float b) { return __fmul_rn(a, b); }
EL_F2D_HD float df_fma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
#else
EL_F2D_HD float df_add(float a, float b) { return a + b; }
EL_F2D_HD float df_sub(float a, float b) { return a - b; }
EL_F2D_HD float df_mul(float a, float b) { return a * b; }
EL_F2D_HD float df_fma(float a, float b, float c) { return std::fmaf(a, b, c); }
#endif

// d = h + l: h holds the top 24 significant bits of d and l the next 23, both truncated, so
// |d - (h + l)| < 2^-46 |d|; h and l carry d's sign.  Integer arithmetic and one float
// subtraction.  Below 2^-103 (where l would leave the normal float range) the pair is the
// float nearest d and zero: an absolute error below 2^-126 (2^-24 relative at most); the
// residual kernel shifts its system by a power of two that brings |b| near 1, so only values
// some 2^100 below the system's scale come this close.  Zero gives
// (0, 0).  ok is cleared for |d| at or above 2^128 (infinities and NaN among them), which the
// float pair cannot hold: the caller then takes FP64 arithmetic.
EL_F2D_HD F2 df_split(double d, bool& ok) {
    uint64_t bits;
    std::memcpy(&bits, &d, sizeof(bits));
    const uint32_t hi = (uint32_t)(bits >> 32), lo = (uint32_t)bits;
    const uint32_t sign = hi & 0x80000000u, em = hi & 0x7fffffffu;
    const uint32_t e = em >> 20;
    ok = ok && e <= 1150u;
    F2 r;
    if (e >= 920u) {
        // h: the exponent rebased (bias 1023 -> 127) above the 20 + 3 leading mantissa bits
        const uint32_t hb = sign | ((em - (896u << 20)) << 3) | (lo >> 29);
        // l: mantissa bits 28..6 under the exponent of 2^(E - 1046), less that power of two
        // (exact: both floats share the exponent)
        const uint32_t eb = sign | ((e - 919u) << 23);
        const uint32_t ab = eb | ((lo >> 6) & 0x7fffffu);
        float a, b;
        std::memcpy(&r.h, &hb, sizeof(float));
        std::memcpy(&a, &ab, sizeof(a));
        std::memcpy(&b, &eb, sizeof(b));
        r.l = df_sub(a, b);
    } else {
        r.h = d2f(d);
        r.l = 0.f;
    }
    return r;
}

// d 2^k for a power-of-two shift k by integer arithmetic on the exponent field: exact while the
// result is a normal double; zero stays zero; a result below the normal range flushes to zero
// (the shifts here bring values near 1, so only values 2^-1000 or so below the largest reach
// that), one above it, or an infinite or NaN input, is NaN.
EL_F2D_HD double d_shift(double d, int k) {
    uint64_t bits;
    std::memcpy(&bits, &d, sizeof(bits));
    const int e = (int)((bits >> 52) & 0x7ffu);
    const int ne = e + k;
    uint64_t out;
    if (e == 0) {
        out = bits & 0x8000000000000000ull;  // zero (or subnormal: flushed), sign kept
    } else if (e == 0x7ff || ne >= 0x7ff) {
        out = 0x7ff8000000000000ull;
    } else if (ne <= 0) {
        out = bits & 0x8000000000000000ull;
    } else {
        out = (bits & ~(0x7ffull << 52)) | ((uint64_t)ne << 52);
    }
    double r;
    std::memcpy(&r, &out, sizeof(r));
    return r;
}

// d > 0 for a double, by integer comparison of its bits (the same answer for every input,
// NaN included, without an FP64 instruction)
EL_F2D_HD bool d_positive(double d) {
    int64_t bits;
    std::memcpy(&bits, &d, sizeof(bits));
    return bits > 0 && bits <= (int64_t)0x7ff0000000000000ll;
}

// s + e = a + b exactly (TwoSum, six operations, no condition on the magnitudes)
EL_F2D_HD void df_two_sum(float a, float b, float& s, float& e) {
    const float t = df_add(a, b);
    const float bb = df_sub(t, a);
    e = df_add(df_sub(a, df_sub(t, bb)), df_sub(b, bb));
    s = t;
}

// (S, E) -= c x for a float c and a pair x: c x.h is split exactly into p + pe by FMA; S - p is
// formed by TwoSum, its error and -(pe + c x.l) go to E.
EL_F2D_HD void df_sub_prod(float& S, float& E, float c, F2 x) {
    const float p = df_mul(c, x.h);
    const float pe = df_fma(c, x.h, -p);
    float s, t;
    df_two_sum(S, -p, s, t);
    S = s;
    E = df_sub(df_add(E, t), df_fma(c, x.l, pe));
}

// r = b - (d x0 + cxm xxm + cxp xxp + cym xym + cyp xyp + czm xzm + czp xzp) for pairs b, d and
// x, float couplings c; the result as a pair (h, l) with |l| <= ulp(h) / 2.  d x0 is split as
// d.h x0.h (exact) + d.h x0.l + d.l x0.h; d.l x0.l (below 2^-46 of the product) is left out.
EL_F2D_HD F2 df_residual7(F2 b, F2 d, F2 x0, float cxm, F2 xxm, float cxp, F2 xxp, float cym, F2 xym, float cyp,
                          F2 xyp, float czm, F2 xzm, float czp, F2 xzp) {
    float S = b.h, E = b.l;
    {
        const float p = df_mul(d.h, x0.h);
        const float pe = df_fma(d.h, x0.h, -p);
        float s, t;
        df_two_sum(S, -p, s, t);
        S = s;
        E = df_sub(df_add(E, t), df_fma(d.l, x0.h, df_fma(d.h, x0.l, pe)));
    }
    df_sub_prod(S, E, cxm, xxm);
    df_sub_prod(S, E, cxp, xxp);
    df_sub_prod(S, E, cym, xym);
    df_sub_prod(S, E, cyp, xyp);
    df_sub_prod(S, E, czm, xzm);
    df_sub_prod(S, E, czp, xzp);
    F2 r;
    df_two_sum(S, E, r.h, r.l);
    return r;
}

// The double sum of six floats added in order from zero, as fl(fl(fl(0 + t0) + t1) ...), when
// no partial sum needs more than 53 significant bits: every nonzero term within 2^26 of the
// largest in exponent (six terms below 2^(e_max + 1) sum below 2^(e_max + 4), in units of the
// smallest term's last bit 2^(e_min - 23): 27 + e_max - e_min bits).  Each addition is then
// exact, so the result is the exact sum, formed here in a 64-bit integer and packed as a
// double; zero is +0, as the additions give.  Returns false otherwise (and for non-finite
// terms), when the caller adds in FP64.  Integer arithmetic only.
EL_F2D_HD bool exact_sum6(float t0, float t1, float t2, float t3, float t4, float t5, double& out) {
    const float t[6] = {t0, t1, t2, t3, t4, t5};
    uint32_t u[6];
    uint32_t emax = 0u, emin = 255u, fin = 1u;
#pragma unroll
    for (int q = 0; q < 6; ++q) {
        std::memcpy(&u[q], &t[q], sizeof(uint32_t));
        const uint32_t mag = u[q] & 0x7fffffffu;
        uint32_t e = mag >> 23;
        fin &= e != 255u ? 1u : 0u;
        e = e ? e : 1u;  // a subnormal counts at exponent 1, without the leading one
        if (mag) {
            emax = e > emax ? e : emax;
            emin = e < emin ? e : emin;
        }
    }
    uint64_t bits = 0ull;
    if (emax) {
        if (!fin || emax - emin > 26u) return false;
        int64_t S = 0;
#pragma unroll
        for (int q = 0; q < 6; ++q) {
            const uint32_t mag = u[q] & 0x7fffffffu;
            const uint32_t e = mag >> 23;
            const uint32_t m = (mag & 0x7fffffu) | (e ? 0x800000u : 0u);
            const int64_t v = (int64_t)((uint64_t)m << ((e ? e : 1u) - emin));
            S += (u[q] >> 31) ? -v : v;
        }
        if (S != 0) {
            const uint64_t sg = S < 0 ? 1ull : 0ull;
            const uint64_t A = sg ? (uint64_t)(-S) : (uint64_t)S;  // below 2^53
            const uint32_t ah = (uint32_t)(A >> 32);
            const int p = ah ? 63 - clz32(ah) : 31 - clz32((uint32_t)A);
            const uint64_t mant = (A << (52 - p)) & 0xfffffffffffffull;
            bits = (sg << 63) | ((uint64_t)(p + (int)emin + 873) << 52) | mant;
        }
    }
    std::memcpy(&out, &bits, sizeof(out));
    return true;
}

// A sum of squares of floats in three FP32 accumulators by magnitude (below 2^-60, up to
// 2^60, beyond), so that no square leaves the normal float range; the total in FP64.  For the
// per-thread partial norms of kernels bound by FP64 issue.
struct SqAcc {
    float lo = 0.f, mid = 0.f, hi = 0.f;
    EL_F2D_HD void add(float v) {
        const float a = v < 0.f ? -v : v;
        if (a < 0x1p-60f) {
            const float t = df_mul(v, 0x1p64f);
            lo = df_fma(t, t, lo);
        } else if (a < 0x1p60f) {
            mid = df_fma(v, v, mid);
        } else {
            const float t = df_mul(v, 0x1p-64f);
            hi = df_fma(t, t, hi);
        }
    }
    EL_F2D_HD double value() const { return f2d(mid) + f2d(lo) * 0x1p-128 + f2d(hi) * 0x1p128; }
};

}  // namespace el
