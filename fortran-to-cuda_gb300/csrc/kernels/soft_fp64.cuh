// Binary64 addition and multiplication on the integer pipes, rounded to
// nearest-even exactly as IEEE 754-2019 (clauses 4.3.1 and 5.4.1) defines them.
//
// GB300 issues FP64 at about two lane operations per clock per SM while its
// integer pipes (logic, shifts and compares on the ALU pipe, wide multiplies
// and adds on the FMA pipe) take 64 or more; the advection kernels are bound
// by the FP64 pipe with the integer pipes nearly idle. Computing part of the
// additions and multiplications here moves that work to the idle pipes. The
// results are the correctly rounded ones, so they equal the hardware's DADD and
// DMUL bit for bit: substituting one for the other changes no value.
//
// The method is the textbook one (align, add or subtract the significands with
// a sticky bit jammed into the lowest position, normalise, round to nearest with
// ties to even; the product's significand as a 106-bit integer), written for the
// common case only: both operands normal, the result normal. Every other case
// (zeros, subnormals, infinities, NaN, results that overflow or underflow; all
// rare in the stencils' fields) is handed to the hardware instruction.
//
// The kernels use the product (mul_rn_int). The two additions are kept beside
// it, checked by the same tests, as the measured alternatives: in the advection
// kernels, whose integer pipes already carry the products, moving additions
// off the FP64 pipe made every kernel slower (add_rn_int by about as much time
// as the DADD it replaces; add_rn_near, about half the integer work, still
// 4-21 % slower for 6-17 additions per point of the fast-fp kernel).
#pragma once
#include <cuda_runtime.h>

namespace f2c {

constexpr unsigned long long kSignBit = 0x8000000000000000ull;
constexpr unsigned long long kFracMask = 0x000FFFFFFFFFFFFFull;
constexpr unsigned long long kHiddenBit = 0x0010000000000000ull;

// The cases the integer paths leave out, kept out of line: a call stays a
// branch that only lanes needing it take, where an inline hardware operation
// would be if-converted into an FP64 instruction that every lane issues.
static __device__ __noinline__ double add_rn_hw(double a, double b) { return __dadd_rn(a, b); }
static __device__ __noinline__ double mul_rn_hw(double a, double b) { return __dmul_rn(a, b); }

// Round a significand with its leading one at bit 63 (bits below bit 0 jammed
// into bit 0) to 53 bits, nearest-even; the result keeps the hidden bit, or is
// 2^53 after a carry out of the significand.
__device__ __forceinline__ unsigned long long round_top53(unsigned long long s) {
    const unsigned long long m = s >> 11;
    const unsigned rem = (unsigned)s & 0x7FFu;
    return m + ((rem > 0x400u || (rem == 0x400u && (m & 1ull))) ? 1ull : 0ull);
}

// a + b, rounded to nearest-even.
__device__ __forceinline__ double add_rn_int(double a, double b) {
    const unsigned long long ia = (unsigned long long)__double_as_longlong(a);
    const unsigned long long ib = (unsigned long long)__double_as_longlong(b);
    const unsigned long long ma = ia & ~kSignBit, mb = ib & ~kSignBit;
    const bool swap = ma < mb;
    const unsigned long long x = swap ? ib : ia;  // the operand of larger magnitude: the result's sign
    const unsigned long long mx = swap ? mb : ma, my = swap ? ma : mb;
    const int ex = (int)(mx >> 52), ey = (int)(my >> 52);
    if (ey == 0 || ex > 0x7FC) return add_rn_hw(a, b);
    // significands with the hidden bit at bit 62 (ten spare low bits)
    const unsigned long long fx = ((mx & kFracMask) | kHiddenBit) << 10;
    unsigned long long fy = ((my & kFracMask) | kHiddenBit) << 10;
    const unsigned d = (unsigned)min(ex - ey, 63);
    const unsigned long long kept = fy >> d;
    fy = kept | (unsigned long long)((kept << d) != fy);  // jam the bits shifted out into bit 0
    const bool sub = (long long)(ia ^ ib) < 0;
    unsigned long long s = sub ? fx - fy : fx + fy;
    if (s == 0) return 0.0;  // x + (-x) is +0 when rounding to nearest
    const int lz = __clzll((long long)s);
    s <<= lz;                 // leading one at bit 63
    const int e = ex + 1 - lz;  // biased exponent of the result
    if (e < 1) return add_rn_hw(a, b);
    const unsigned long long m = round_top53(s);
    // m carries the hidden bit (or 2^53 after a rounding carry), so adding it to (e - 1) << 52 also
    // carries into the exponent when rounding overflowed the significand
    return __longlong_as_double((long long)((x & kSignBit) | (((unsigned long long)(e - 1) << 52) + m)));
}

// a + b, rounded to nearest-even, for operands whose exponents differ by at
// most 9 (the sum of neighbouring values of a smooth field): aligned to the
// smaller exponent the significands add exactly in 64 bits, so the only
// rounding is the final one, which needs no sticky bit. About half the
// integer work of add_rn_int; other operands go to the hardware addition.
__device__ __forceinline__ double add_rn_near(double a, double b) {
    const long long ia = __double_as_longlong(a), ib = __double_as_longlong(b);
    const int ea = (int)((unsigned long long)ia >> 52) & 0x7FF, eb = (int)((unsigned long long)ib >> 52) & 0x7FF;
    const int d = ea - eb;
    if ((unsigned)(ea - 1) >= 0x7FCu || (unsigned)(eb - 1) >= 0x7FCu || (unsigned)(d + 9) > 18u) return add_rn_hw(a, b);
    long long ma = (ia & (long long)kFracMask) | (long long)kHiddenBit;
    long long mb = (ib & (long long)kFracMask) | (long long)kHiddenBit;
    ma <<= (d > 0 ? d : 0);  // below 2^62
    mb <<= (d < 0 ? -d : 0);
    const int e0 = d > 0 ? eb : ea;
    const long long s = (ia < 0 ? -ma : ma) + (ib < 0 ? -mb : mb);  // exact, |s| < 2^63
    const unsigned long long mag = (unsigned long long)(s < 0 ? -s : s);
    if (mag == 0) return 0.0;  // x + (-x) is +0 when rounding to nearest
    const int sh = 11 - __clzll((long long)mag);  // bits below the 53 the result keeps
    unsigned long long m;
    if (sh > 0) {
        const unsigned long long half = 1ull << (sh - 1), rest = mag & ((half << 1) - 1);
        m = (mag + half) >> sh;
        if (rest == half) m &= ~1ull;  // a tie goes to the even significand
    } else {
        m = mag << (-sh);
    }
    const int e = e0 + sh;  // biased exponent of the result
    if (e < 1) return add_rn_hw(a, b);
    return __longlong_as_double((long long)((s < 0 ? kSignBit : 0ull) | (((unsigned long long)(e - 1) << 52) + m)));
}

// a * b, rounded to nearest-even.
__device__ __forceinline__ double mul_rn_int(double a, double b) {
    const unsigned long long ia = (unsigned long long)__double_as_longlong(a);
    const unsigned long long ib = (unsigned long long)__double_as_longlong(b);
    const int ea = (int)((ia >> 52) & 0x7FF), eb = (int)((ib >> 52) & 0x7FF);
    int e = ea + eb - 1023;  // biased exponent when the significand product is below 2
    if (ea == 0 || eb == 0 || ea == 0x7FF || eb == 0x7FF || e < 1 || e > 0x7FC) return mul_rn_hw(a, b);
    const unsigned long long fa = (ia & kFracMask) | kHiddenBit, fb = (ib & kFracMask) | kHiddenBit;
    // the 106-bit product hi * 2^64 + lo from 32-bit pieces (the high pieces are below 2^21)
    const unsigned al = (unsigned)fa, ah = (unsigned)(fa >> 32), bl = (unsigned)fb, bh = (unsigned)(fb >> 32);
    const unsigned long long ll = (unsigned long long)al * bl;
    const unsigned long long mid = (unsigned long long)al * bh + (unsigned long long)ah * bl;  // below 2^54
    const unsigned long long lo = ll + (mid << 32);
    const unsigned long long hi = (unsigned long long)ah * bh + (mid >> 32) + (lo < ll ? 1ull : 0ull);
    // top 64 bits of the product (it lies in [2^104, 2^106)), the 42 bits below jammed into bit 0
    unsigned long long t = (hi << 22) | (lo >> 42) | ((lo & ((1ull << 42) - 1)) != 0 ? 1ull : 0ull);
    const int lz = (int)(~t >> 63);  // 0 when the product reached 2^105
    t <<= lz;
    e += 1 - lz;
    const unsigned long long m = round_top53(t);
    return __longlong_as_double(
        (long long)(((ia ^ ib) & kSignBit) | (((unsigned long long)(e - 1) << 52) + m)));
}

} // namespace f2c
