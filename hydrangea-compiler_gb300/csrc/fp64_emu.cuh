// fp64_emu.cuh -- binary64 addition on the integer pipe.
//
// GB300 issues FP64 at 1.9 operations per clock per SM, so an FP64 stencil is
// bound by that pipe long before HBM.  The integer pipe is idle there; moving
// some of the stencil's additions onto it raises throughput while the results
// stay bit-identical to IEEE-754 round-to-nearest-even.
//
// dadd_pos() takes the textbook route for two non-negative normal operands
// whose exponents differ by at most 10 (the usual case of a stencil's sums):
//   1. order the operands by magnitude (for non-negative doubles the bit
//      patterns order like the values);
//   2. widen both significands (hidden bit set) by 10 guard bits; the smaller
//      one is aligned by shifting it left by 10 - gap, which is exact;
//   3. add, and renormalise by one place if the sum carried out, keeping the
//      bit shifted out as a sticky bit;
//   4. round to nearest, ties to even, on the 10 discarded bits, and
//      renormalise once more if rounding carried into bit 53.
// Any other case -- an operand that is zero, subnormal, negative, infinite or
// NaN, a larger exponent gap, or a result that overflows the exponent range --
// takes __dadd_rn on the FP64 unit, so the function is exact for every input.
#pragma once

#include <stdint.h>

namespace hyd {

// The fallback lives behind a call so that the compiler cannot if-convert it
// into an unconditional FP64 add on every lane: warps whose operands are all
// on the fast path branch over it and issue nothing on the FP64 pipe.
static __device__ __noinline__ double dadd_fallback(double x, double y) { return __dadd_rn(x, y); }

__device__ __forceinline__ double dadd_pos(double x, double y) {
    const unsigned long long X = (unsigned long long)__double_as_longlong(x);
    const unsigned long long Y = (unsigned long long)__double_as_longlong(y);
    const unsigned long long hi = X > Y ? X : Y, lo = X > Y ? Y : X;
    const unsigned eh = (unsigned)(hi >> 52), el = (unsigned)(lo >> 52);
    const unsigned d = eh - el;
    // fast path: both exponent fields in [1, 2046] with the sign bit clear (a
    // set sign bit makes the field >= 2048; hi >= lo, so testing el >= 1 and
    // eh <= 2046 covers both operands) and an exponent gap of at most 10, so
    // that aligning the smaller significand below 10 guard bits drops no bit
    bool ok = el >= 1u && eh <= 2046u && d <= 10u;
    constexpr unsigned long long kM52 = (1ULL << 52) - 1ULL, kH = 1ULL << 52;
    const unsigned long long mh = ((hi & kM52) | kH) << 10;                 // in [2^62, 2^63)
    const unsigned long long al = ((lo & kM52) | kH) << ((10u - d) & 15u);  // exact
    unsigned long long s = mh + al;                                          // < 2^64
    unsigned e = eh;
    if (s >> 63) {  // carry out: one place right, keeping the lost bit as sticky
        s = (s >> 1) | (s & 1ULL);
        e += 1u;
    }
    unsigned long long mant = s >> 10;  // in [2^52, 2^53)
    const unsigned rem = (unsigned)s & 0x3FFu;
    mant += (unsigned long long)((rem > 0x200u) | ((rem == 0x200u) & ((unsigned)mant & 1u)));
    if (mant >> 53) {  // rounded up to 2^53: exactly 2^52 one exponent higher
        mant >>= 1;
        e += 1u;
    }
    ok &= e <= 2046u;
    if (!ok) return dadd_fallback(x, y);
    return __longlong_as_double((long long)(((unsigned long long)e << 52) + (mant - kH)));
}

// ddiv_small_rn<D>(x) = x / D rounded to nearest even, for D = 3 or 5, in one
// multiply and two FMAs instead of a full IEEE division (the published
// correction scheme for division by a constant: Markstein, IBM J. R&D 1990;
// Brisebarre, Muller, Raina, IEEE Trans. Computers 53(8), 2004):
//   q0 = RN(x * z)            z = RN(1/D)
//   r  = x - D * q0           exact (one FMA): |r| <= D/2 ulp(q0) plus a hair,
//                             a multiple of ulp(q0) well inside 53 bits
//   q  = RN(q0 + r * z)       one FMA
// Why q is RN(x / D) for every finite x: q0 + r/D equals x/D exactly, and
// replacing 1/D by z moves the FMA's exact argument by |r| * |z - 1/D|, under
// 2^-54 ulp(q0).  x/D is either exact (then r = 0) or, since D is odd, lies k/D
// of an ulp past a representable value (0 < k < D), at least 1/(2D) ulp away
// from any rounding midpoint -- with subnormal results too, whose ulp is fixed.
// A tiny shift cannot cross such a midpoint, so the single rounding of the FMA
// gives the correctly rounded quotient.  A zero remainder (x/D exact, x = +-0
// keeping its sign) and a non-finite q0 (x infinite or NaN) return q0 itself.
template <int D>
__device__ __forceinline__ double ddiv_small_rn(double x) {
    static_assert(D == 3 || D == 5, "the correction is proved here for odd D = 3, 5");
    constexpr double z = 1.0 / D;  // RN(1/D)
    const double q0 = __dmul_rn(x, z);
    const double r = __fma_rn(-(double)D, q0, x);
    const unsigned long long qb = (unsigned long long)__double_as_longlong(q0);
    const unsigned long long rb = (unsigned long long)__double_as_longlong(r);
    if (((qb >> 52) & 0x7FFULL) == 0x7FFULL || (rb << 1) == 0ULL) return q0;
    return __fma_rn(r, z, q0);
}

}  // namespace hyd
