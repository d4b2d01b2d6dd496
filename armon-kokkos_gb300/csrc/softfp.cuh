// softfp.cuh -- exact IEEE-754 binary64 operations on the integer and FP32 pipes.
//
// GB300 executes FP64 arithmetic at 1/64 of its FP32 rate (2 DFMA per SM per clock), and an IEEE
// double division costs about 9 DFMA slots there, while the integer and FP32 pipes of the fused
// pass are almost idle.  The helpers below compute bit-identical results to the FP64 instructions
// they replace, for the operands the fast paths accept, using integer arithmetic:
//
//   lt(x, y)      x < y  (false when either is NaN; -0 == +0)
//   gt0(x)        x > 0
//   lt_pos(x, c)  x < c for a positive constant c
//   neg_if(x, c)  c ? -x : x  (a sign flip: what multiplying by -1 gives for non-NaN x)
//   scale(x, k)   x * 2^k, exact (half(x) = x * 0.5, twice(x) = x * 2)
//   absval(x)     |x|
//   div(a, b)     the correctly rounded quotient (round to nearest, ties to even)
//   sqrt(x)       the correctly rounded square root
//   mul(a, b)     the correctly rounded product
//   add(a, b)     the correctly rounded sum (add_bits: the same on bit patterns, host or device)
//
// Division (my own construction from the arithmetic, not a library's sequence).  With
// significands ma, mb in [2^52, 2^53) and ma doubled when ma < mb, the result significand is
// Q = floor(ma * 2^52 / mb) rounded with the remainder R = ma * 2^52 - Q * mb.  Q is estimated
// with a reciprocal of d = mb * 2^11: an FP32 seed (rcp.approx of the top 24 bits), biased below
// the true value, then two Newton steps y <- y + y (1 - d y) in 64-bit fixed point, each of which
// keeps the estimate below 2^128 / d; then Q_est = floor(U * V / 2^128) for U = ma * 2^63.  The
// remainder is computed exactly in 64 bits and Q_est is raised once if R >= mb.  If R still is not
// in [0, mb) -- which the error bounds exclude -- the hardware division is used, so a fast-path
// result always satisfies ma * 2^52 = Q * mb + R with 0 <= R < mb, i.e. Q is exact.  Zero
// dividends are handled; subnormal, infinite and NaN operands and quotients outside the normal
// range go to the hardware division.
#pragma once

#include <cstdint>

namespace armon {
namespace sfp {

// The bit pattern is taken in inline PTX so that the compiler cannot see the integer tests that
// follow as floating-point class tests (zero, NaN, normal), which it would otherwise fold back into
// FP64 compares on the FP64 pipe.
__device__ __forceinline__ uint64_t bits(double x)
{
    uint64_t u;
    asm("mov.b64 %0, %1;" : "=l"(u) : "d"(x));
    return u;
}
__device__ __forceinline__ double from_bits(uint64_t u) { return __longlong_as_double((long long)u); }

constexpr uint64_t kAbs = 0x7FFFFFFFFFFFFFFFull;
constexpr uint64_t kInf = 0x7FF0000000000000ull;
constexpr uint64_t kMant = 0x000FFFFFFFFFFFFFull;
constexpr uint64_t kHidden = 0x0010000000000000ull;

// Monotone key of a non-NaN double: -x and +x map to -k and +k, and -0, +0 both to 0.
__device__ __forceinline__ int64_t key(uint64_t u)
{
    const int64_t a = (int64_t)(u & kAbs);
    return (int64_t)u < 0 ? -a : a;
}

__device__ __forceinline__ bool lt(double x, double y)
{
    const uint64_t ux = bits(x), uy = bits(y);
    const bool nan = ((ux & kAbs) > kInf) | ((uy & kAbs) > kInf);
    return !nan && key(ux) < key(uy);
}

__device__ __forceinline__ bool gt0(double x)
{
    const int64_t u = (int64_t)bits(x);
    return u > 0 && (uint64_t)u <= kInf;
}

// x < c for a constant c > 0 given by its bit pattern: the signed order of the patterns is the
// IEEE order against a positive value, except for NaNs with the sign bit set.
__device__ __forceinline__ bool lt_pos(double x, uint64_t c)
{
    const uint64_t u = bits(x);
    return (int64_t)u < (int64_t)c && (u & kAbs) <= kInf;
}

// The sign-bit operations are written on the high word in inline PTX: a plain xor / and of the
// bit pattern is recognised as an FP negation / absolute value, which can be materialised on the
// FP64 pipe.
__device__ __forceinline__ double neg_if(double x, bool c)
{
    const uint32_t m = (uint32_t)c << 31;
    uint32_t hi;
    asm("xor.b32 %0, %1, %2;" : "=r"(hi) : "r"((uint32_t)__double2hiint(x)), "r"(m));
    return __hiloint2double((int)hi, __double2loint(x));
}

__device__ __forceinline__ double absval(double x)
{
    uint32_t hi;
    asm("and.b32 %0, %1, 0x7FFFFFFF;" : "=r"(hi) : "r"((uint32_t)__double2hiint(x)));
    return __hiloint2double((int)hi, __double2loint(x));
}

// x * 2^k for |k| < 2046: exact whenever x and the result are normal, so the exponent field moves
// by k; zeros are returned as they are; everything else (subnormal operand or result, overflow,
// infinities, NaN) takes the FP64 multiply by the power of two `p2` (== 2^k).
__device__ __forceinline__ double scale(double x, int k, double p2)
{
    const uint64_t u = bits(x);
    const int e = (int)((u >> 52) & 0x7FFu);
    if ((unsigned)(e - 1) < 2046u && (unsigned)(e + k - 1) < 2046u)
        return from_bits(u + ((uint64_t)(int64_t)k << 52));
    if ((u << 1) == 0) return x;
    return x * p2;
}
__device__ __forceinline__ double half(double x) { return scale(x, -1, 0.5); }
__device__ __forceinline__ double twice(double x) { return scale(x, 1, 2.0); }

// The reciprocal of a divisor significand mb in (2^52, 2^53): V = 2^64 + v ~ 2^128 / d for
// d = mb 2^11, from below.
__device__ __forceinline__ uint64_t recip_v(uint64_t mb)
{
    const uint64_t d = mb << 11;                                   // [2^63, 2^64)
    const uint32_t top = (uint32_t)(d >> 40);                      // [2^23, 2^24)
    const float fd = __uint_as_float(0x4B000000u | (top & 0x7FFFFFu));   // == top
    float rf;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(rf) : "f"(fd));
    const uint32_t urf = __float_as_uint(rf);
    // rf in (2^-24, 2^-23]; rf * 2^88 = 2^64 (1 + m 2^-23) when rf < 2^-23.  The seed is lowered
    // by 2^44 (2^-21 relative) so that it is below 2^128 / d.
    uint64_t v;
    if ((urf >> 23) >= 104u) {
        v = 0xFFFFF00000000000ull;
    } else {
        const uint64_t m = (uint64_t)(urf & 0x7FFFFFu) << 41;
        v = m > (1ull << 44) ? m - (1ull << 44) : 0;
    }
#pragma unroll
    for (int it = 0; it < 2; it++) {
        // e = 2^128 - d (2^64 + v) >= 0; its high word, then V += V e / 2^128 (from below)
        const uint64_t ph = __umul64hi(d, v);
        const uint64_t pl = d * v;
        const uint64_t eh = 0ull - d - ph - (pl != 0 ? 1ull : 0ull);
        v = v + eh + __umul64hi(v, eh);
    }
    return v;
}

// The quotient estimate of significands ma in [2^52, 2^54) and mb (reciprocal V = 2^64 + v):
// floor(x (2^64 + v) / 2^74) for x = ma 2^9 (< 2^63).  V lies within 2^-62 below 2^128 / d, so the
// estimate is floor(ma 2^52 / mb) or one less.
__device__ __forceinline__ uint64_t quot_estimate(uint64_t ma, uint64_t v)
{
    const uint64_t x = ma << 9;
    return (x + __umul64hi(x, v)) >> 10;
}

// a / b; the reciprocal comes from get_v(mb), called only on the integer path.
template <class GetV>
__device__ __forceinline__ double div_core(double a, double b, uint64_t ub, GetV get_v)
{
    const uint64_t ua = bits(a);
    const uint32_t ea = (uint32_t)(ua >> 52) & 0x7FFu;
    const uint32_t eb = (uint32_t)(ub >> 52) & 0x7FFu;
    const uint64_t sign = (ua ^ ub) & ~kAbs;
    const int e0 = (int)ea - (int)eb;
    const bool b_normal = (eb - 1u) < 2046u;
    if (b_normal && (ua << 1) == 0) return from_bits(sign);   // +-0 / normal
    if (!(b_normal && (ea - 1u) < 2046u && e0 >= -1021 && e0 <= 1022)) return a / b;

    uint64_t ma = (ua & kMant) | kHidden;
    const uint64_t mb = (ub & kMant) | kHidden;
    int e = e0;
    if (ma < mb) {
        ma <<= 1;
        e -= 1;
    }
    uint64_t q;
    uint64_t r;
    if (mb == kHidden) {
        // a power-of-two divisor: the quotient is the dividend's significand, exactly
        q = ma;
        r = 0;
    } else {
        // Q_est is Q or Q - 1, and one correction step makes it Q
        q = quot_estimate(ma, get_v(mb));
        r = (ma << 52) - q * mb;          // exact: the true remainder lies in [0, 2 mb)
        const bool up1 = r >= mb;
        r = up1 ? r - mb : r;
        q = up1 ? q + 1 : q;
        if (r >= mb) return a / b;        // outside the error bounds: the hardware decides
    }
    // round to nearest, ties to even, on the exact remainder
    const uint64_t r2 = r << 1;
    const bool up = r2 > mb || (r2 == mb && (q & 1));
    q += up ? 1ull : 0ull;
    return from_bits(sign + ((uint64_t)(e + 1022) << 52) + q);
}

__device__ __forceinline__ double div(double a, double b)
{
    return div_core(a, b, bits(b), [](uint64_t mb) { return recip_v(mb); });
}

// A divisor's reciprocal computed once for several quotients (when it is not a power of two and
// the divisor is normal; div(a, R, b) is exact whatever R holds for other divisors).
struct Recip {
    uint64_t ub, v;
};

__device__ __forceinline__ Recip recip(double b)
{
    Recip R;
    R.ub = bits(b);
    const uint64_t mb = (R.ub & kMant) | kHidden;
    const uint32_t eb = (uint32_t)(R.ub >> 52) & 0x7FFu;
    R.v = (mb != kHidden && (eb - 1u) < 2046u) ? recip_v(mb) : 0;
    return R;
}

__device__ __forceinline__ double div(double a, const Recip& R, double b)
{
    return div_core(a, b, R.ub, [&](uint64_t) { return R.v; });
}

// Multiplication (my own construction).  For normal operands with significands ma, mb in
// [2^52, 2^53) the exact product ma mb lies in [2^104, 2^106); with both significands shifted to
// bit 63, the high word of their 128-bit product holds its top 64 bits and the low word the rest.
// The top 53 bits are the result significand, the next bit the rounding bit and everything below
// it the sticky part; round to nearest, ties to even.  Zero operands give signed zeros; subnormal,
// infinite and NaN operands and results outside the normal range take the FP64 multiply.
__device__ __forceinline__ double mul(double a, double b)
{
    const uint64_t ua = bits(a), ub = bits(b);
    const uint32_t ea = (uint32_t)(ua >> 52) & 0x7FFu;
    const uint32_t eb = (uint32_t)(ub >> 52) & 0x7FFu;
    const uint64_t sign = (ua ^ ub) & ~kAbs;
    if ((ea - 1u) < 2046u && (eb - 1u) < 2046u) {
        const uint64_t xa = ((ua & kMant) | kHidden) << 11;      // [2^63, 2^64)
        const uint64_t xb = ((ub & kMant) | kHidden) << 11;
        const uint64_t hi = __umul64hi(xa, xb);                  // [2^62, 2^64)
        const bool lo_nz = xa * xb != 0;
        const uint32_t top = (uint32_t)(hi >> 63);               // product >= 2^105
        const uint32_t sh = 10 + top;
        const uint64_t m = hi >> sh;                             // [2^52, 2^53)
        const uint64_t rem = hi & ((1ull << sh) - 1);
        const uint64_t halfw = 1ull << (sh - 1);
        const bool up = rem > halfw || (rem == halfw && (lo_nz || (m & 1)));
        const int e = (int)ea + (int)eb - 1023 + (int)top;      // biased exponent of the result
        if ((unsigned)(e - 1) < 2046u) return from_bits(sign + ((uint64_t)(e - 1) << 52) + m + (up ? 1u : 0u));
        return a * b;
    }
    if (((ua << 1) == 0 && (eb - 1u) < 2046u) || ((ub << 1) == 0 && (ea - 1u) < 2046u) ||
        ((ua << 1) == 0 && (ub << 1) == 0))
        return from_bits(sign);                                  // +-0 * normal or zero
    return a * b;
}

// Addition (my own construction).  For normal operands, x the one of larger magnitude and y the
// other, the significands are placed at bits 62..10 of 64-bit words (ten guard bits) and y's is
// shifted right by the exponent difference d, what falls off kept as a sticky bit.  Same signs:
// the sum, renormalised by one place when it carries into bit 63.  Opposite signs: the
// difference, minus one more unit when the sticky bit is set (the true value then lies strictly
// between that integer and the next), renormalised to bit 62; a sticky bit only arises for
// d >= 11, where at most one place of renormalisation is needed and the guard bits still decide
// the rounding.  Round to nearest, ties to even, on the ten guard bits and the sticky bit.  x - x
// gives +0; a zero operand gives the other operand (-0 only for -0 + -0); subnormal, infinite and
// NaN operands, subnormal results and overflow take the FP64 addition (ok = false).
__host__ __device__ __forceinline__ int clz64(uint64_t x)
{
#ifdef __CUDA_ARCH__
    return __clzll((long long)x);
#else
    return __builtin_clzll(x);
#endif
}

__host__ __device__ __forceinline__ uint64_t add_bits(uint64_t ua, uint64_t ub, bool& ok)
{
    const uint32_t ea = (uint32_t)(ua >> 52) & 0x7FFu, eb = (uint32_t)(ub >> 52) & 0x7FFu;
    ok = false;
    if (!((ea - 1u) < 2046u && (eb - 1u) < 2046u)) {
        const bool za = (ua << 1) == 0, zb = (ub << 1) == 0;
        if (za && zb) { ok = true; return ua & ub; }
        if (zb && (ea - 1u) < 2046u) { ok = true; return ua; }
        if (za && (eb - 1u) < 2046u) { ok = true; return ub; }
        return 0;
    }
    const bool swap = (ub & kAbs) > (ua & kAbs);
    const uint64_t ux = swap ? ub : ua, uy = swap ? ua : ub;
    const uint32_t d = swap ? eb - ea : ea - eb;
    int e = (int)(swap ? eb : ea);
    const uint64_t mx = ((ux & kMant) | kHidden) << 10;     // [2^62, 2^63)
    const uint64_t my = ((uy & kMant) | kHidden) << 10;
    uint64_t ys;
    bool sticky;
    if (d >= 64) {
        ys = 0;
        sticky = true;
    } else {
        ys = my >> d;
        sticky = d != 0 && (my << (64 - d)) != 0;
    }
    uint64_t sum;
    if (((ux ^ uy) >> 63) == 0) {
        sum = mx + ys;                                       // < 2^64
        if (sum >> 63) {
            sticky = sticky || (sum & 1) != 0;
            sum >>= 1;
            e += 1;
        }
    } else {
        sum = mx - ys - (sticky ? 1u : 0u);
        if (sum == 0) { ok = true; return 0; }               // x - x = +0
        const int sh = clz64(sum) - 1;
        sum <<= sh;
        e -= sh;
        if (e < 1) return 0;                                 // subnormal result
    }
    if (e > 2046) return 0;                                  // overflow
    const uint64_t m = sum >> 10, rem = sum & 0x3FFu;
    const bool up = rem > 0x200u || (rem == 0x200u && (sticky || (m & 1)));
    ok = true;
    return (ux & ~kAbs) + ((uint64_t)(e - 1) << 52) + m + (up ? 1u : 0u);
}

__device__ __forceinline__ double add(double a, double b)
{
    bool ok;
    const uint64_t r = add_bits(bits(a), bits(b), ok);
    return ok ? from_bits(r) : a + b;
}

// Square root (my own construction, in the manner of the division above).  A positive normal
// x = m 2^(e-1075), m in [2^52, 2^53), has its significand doubled when e - 1075 is odd, giving
// M = m 2^odd in [2^52, 2^54) over an even exponent.  The result significand is
// Q = floor(sqrt(M 2^52)) in [2^52, 2^53), rounded up when the remainder R = M 2^52 - Q^2 exceeds
// Q (a square root is never exactly halfway between two doubles, so there are no ties).  Q is
// estimated from y ~ 1/sqrt(a), a = M / 2^52 in [1, 4): an FP32 seed (rsqrt.approx of the top
// 24 bits of a), two Newton steps y <- y + y (1 - a y^2) / 2 in 64-bit fixed point, then
// g = a y.  The estimate, lowered by one, is corrected on the exact remainder (computed modulo
// 2^64, exact because |R| < 2^58 for an estimate within a few units); if R is still outside
// [0, 2Q] the hardware square root is used.  Zeros are returned as they are; negative, subnormal,
// infinite and NaN operands take the hardware square root.
__device__ __forceinline__ double sqrt(double x)
{
    const uint64_t u = bits(x);
    const uint32_t e = (uint32_t)(u >> 52);                  // sign and exponent
    if (e - 1u >= 2046u) return (u << 1) == 0 ? x : ::sqrt(x);
    const uint32_t odd = (e & 1u) ^ 1u;                      // e - 1075 is odd
    const uint64_t M = ((u & kMant) | kHidden) << odd;       // [2^52, 2^54)
    const uint64_t A = M << 10;                              // a in Q62
    const uint32_t fa = ((127u + odd) << 23) | ((uint32_t)(M >> (29 + odd)) & 0x7FFFFFu);   // a, truncated
    float rf;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(rf) : "f"(__uint_as_float(fa)));
    const uint32_t ur = __float_as_uint(rf);
    const uint32_t er = ur >> 23;
    int64_t Y;                                               // y in Q62, in [2^61, 2^62]
    if (er >= 127u) Y = 1ll << 62;
    else if (er < 126u) Y = 1ll << 61;
    else Y = (int64_t)((ur & 0x7FFFFFu) | 0x800000u) << 38;
#pragma unroll
    for (int it = 0; it < 2; it++) {
        const uint64_t y2 = __umul64hi((uint64_t)Y, (uint64_t)Y);   // y^2 in Q60
        const uint64_t ay2 = __umul64hi(A, y2);                     // a y^2 in Q58
        const int64_t err = (int64_t)((1ull << 58) - ay2);          // 1 - a y^2 in Q58
        Y += __mul64hi(Y, err) << 5;                                // + y (1 - a y^2) / 2
    }
    uint64_t Q = (__umul64hi(A, (uint64_t)Y) >> 8) - 1;             // g = a y in Q60, to Q52
    int64_t R = (int64_t)((M << 52) - Q * Q);
    if (R < 0) {
        Q -= 1;
        R += (int64_t)(2 * Q + 1);
    }
#pragma unroll
    for (int it = 0; it < 3; it++) {
        const bool up = R > (int64_t)(2 * Q);
        R -= up ? (int64_t)(2 * Q + 1) : 0;
        Q += up ? 1u : 0u;
    }
    if (R < 0 || R > (int64_t)(2 * Q)) return ::sqrt(x);   // outside the error bounds
    Q += R > (int64_t)Q ? 1u : 0u;
    const int be = ((int)e - 1075 - (int)odd) / 2 + 1049;          // biased exponent of the result
    return from_bits(((uint64_t)(be - 1) << 52) + Q);
}

}  // namespace sfp
}  // namespace armon
