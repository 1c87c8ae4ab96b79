// dev_fpint.cuh — IEEE double division and square root, rounded to nearest
// even, on the integer pipes.
//
// GB300 executes FP64 at 1/64 of its FP32 rate; the compiler's correctly
// rounded double division and square root each take about ten FP64
// operations, and the SPH pair kernels (which must round exactly as the
// reference's C does) are bound by them. Both operations are correctly
// rounded by definition, so any exact method returns the same bits: here the
// quotient and the root are formed with 64-bit integer multiplies from an
// FP32 seed, made exact by a remainder test, and rounded by the IEEE rule.
// Operands or results outside the normal range (zero divisors, subnormals,
// infinities, NaNs, results near overflow or underflow) take the compiler's
// operator instead.
//
// Method (a restatement of the standard reciprocal-and-correct scheme for
// multiword division, e.g. Moller & Granlund, "Improved division by
// invariant integers", IEEE Trans. Computers 60(2), 2011, and of the
// Newton iteration for the inverse square root):
//   a / b: D = Mb 2^11 (Mb the 53-bit significand of b) lies in [2^63, 2^64);
//     v ~ 2^128 / D - 2^64 from an FP32 reciprocal seed and two Newton steps
//     in 64-bit fixed point (saturating at 2^64 - 1); the quotient estimate
//     Q = u + hi(u v), u = 2 Ma, of floor(Ma 2^54 / Mb) is off by at most one
//     and is corrected with the remainder Ma 2^54 - Q Mb, which is small, so
//     its low 64 bits hold it exactly. Q has 54 or 55 bits: the bits below
//     the 53 kept and the remainder give round-to-nearest-even.
//   sqrt(x): t = Mx 2^(odd-52) in [1, 4) (odd: the parity of the unbiased
//     exponent); y ~ t^-1/2 from an FP32 rsqrt seed and two Newton steps in
//     fixed point; S ~ t y 2^54 = floor(sqrt(Mx 2^(56+odd))), corrected with
//     the remainder Mx 2^(56+odd) - S^2, then rounded as above.
// Checked bit for bit against the compiler's operators on the GPU
// (csg_check_div_sqrt) and against exact arithmetic on the CPU.
#pragma once

#include <cuda_runtime.h>

namespace fpint {

constexpr unsigned long long MANT = 0xfffffffffffffull;
constexpr unsigned long long HID = 1ull << 52;

__device__ __forceinline__ float rcp_approx(float x)
{
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

__device__ __forceinline__ float rsqrt_approx(float x)
{
    float r;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// v ~ 2^128 / (Mb 2^11) - 2^64 for a 53-bit significand Mb (within a few
// units; saturates at 2^64 - 1 when Mb = 2^52).
__device__ __forceinline__ unsigned long long recip_word(unsigned long long Mb)
{
    const unsigned long long D = Mb << 11;
    const unsigned m24 = (unsigned)(Mb >> 29); // [2^23, 2^24): exactly a float
    const unsigned rb = __float_as_uint(rcp_approx(__uint_as_float((150u << 23) | (m24 & 0x7fffffu))));
    const int e = (int)(rb >> 23) - 103; // exponent of r 2^24 (in (1, 2])
    unsigned long long v = e >= 1 ? ~0ull : (e < 0 ? 0ull : (unsigned long long)(rb & 0x7fffffu) << 41);
#pragma unroll
    for (int k = 0; k < 2; k++) {
        // e 2^64 = (1 - d x) 2^64, d = D 2^-64, x = 1 + v 2^-64 (small, signed)
        const long long E = (long long)((0ull - D) - __umul64hi(D, v));
        const unsigned long long aE = E < 0 ? 0ull - (unsigned long long)E : (unsigned long long)E;
        const unsigned long long d = aE + __umul64hi(v, aE); // x |e| 2^64
        if (E >= 0)
            v = v + d < v ? ~0ull : v + d;
        else
            v = v >= d ? v - d : 0ull;
    }
    return v;
}

} // namespace fpint

// a / b, rounded to nearest even (bit-identical to the compiler's operator).
__device__ __forceinline__ double div_rn(double a, double b)
{
    using namespace fpint;
    const unsigned long long ab = (unsigned long long)__double_as_longlong(a);
    const unsigned long long bb = (unsigned long long)__double_as_longlong(b);
    const int ea = (int)(ab >> 52) & 0x7ff, eb = (int)(bb >> 52) & 0x7ff;
    const int E = ea - eb + 1023; // biased exponent when Ma >= Mb
    const unsigned long long sign = (ab ^ bb) & (1ull << 63);
    const bool bnorm = (unsigned)(eb - 1) < 2046u;
    const bool azero = (ab << 1) == 0ull;
    if (!(bnorm && (azero || ((unsigned)(ea - 1) < 2046u && (unsigned)(E - 2) < 2044u))))
        return a / b;
    if (azero)
        return __longlong_as_double((long long)sign);
    const unsigned long long Ma = (ab & MANT) | HID, Mb = (bb & MANT) | HID;
    const unsigned long long u = Ma << 1;
    unsigned long long Q = u + __umul64hi(u, recip_word(Mb));
    long long rem = (long long)((Ma << 54) - Q * Mb);
#pragma unroll
    for (int k = 0; k < 2; k++)
        if (rem < 0) {
            Q--;
            rem += (long long)Mb;
        }
#pragma unroll
    for (int k = 0; k < 2; k++)
        if (rem >= (long long)Mb) {
            Q++;
            rem -= (long long)Mb;
        }
    const int hi = (int)(Q >> 54); // 1: Q in [2^54, 2^55), two bits below the 53 kept
    const unsigned long long M0 = Q >> (1 + hi);
    const unsigned g = (unsigned)(Q >> hi) & 1u;
    const unsigned st = (hi ? (unsigned)Q & 1u : 0u) | (rem != 0 ? 1u : 0u);
    const unsigned long long M = M0 + (g & (st | ((unsigned)M0 & 1u)));
    return __longlong_as_double((long long)(sign | (((unsigned long long)(E - 2 + hi) << 52) + M)));
}

// sqrt(x), rounded to nearest even (bit-identical to the compiler's sqrt).
__device__ __forceinline__ double sqrt_rn(double x)
{
    using namespace fpint;
    const unsigned long long xb = (unsigned long long)__double_as_longlong(x);
    const int ex = (int)(xb >> 52); // sign included: negative x fails the range test
    if ((unsigned)(ex - 1) >= 2046u)
        return sqrt(x);
    const unsigned long long Mx = (xb & MANT) | HID;
    const int odd = (ex - 1075) & 1;
    const unsigned yb = __float_as_uint(
        rsqrt_approx(__uint_as_float(((127u + (unsigned)odd) << 23) | ((unsigned)(Mx >> 29) & 0x7fffffu))));
    const int ey = (int)(yb >> 23) - 127; // y in (0.5, 1]: -1, or 0 when y = 1
    unsigned long long Y = ey >= 0 ? (1ull << 63)
                                   : (ey == -1 ? (unsigned long long)((yb & 0x7fffffu) | 0x800000u) << 39
                                               : (1ull << 62)); // y 2^63
    const unsigned long long T = Mx << (10 + odd);              // t 2^62
#pragma unroll
    for (int k = 0; k < 2; k++) {
        const unsigned long long Y2 = __umul64hi(Y, Y);                          // y^2 2^62
        const long long Ee = (long long)((1ull << 60) - __umul64hi(T, Y2));      // (1 - t y^2) 2^60
        const unsigned long long aE = Ee < 0 ? 0ull - (unsigned long long)Ee : (unsigned long long)Ee;
        const unsigned long long c = __umul64hi(Y, aE) << 3; // y |e| / 2, in units of 2^-63
        Y = Ee >= 0 ? Y + c : Y - c;
    }
    unsigned long long S = __umul64hi(T, Y) >> 7; // t y 2^54
    long long rem = (long long)((Mx << (56 + odd)) - S * S);
#pragma unroll
    for (int k = 0; k < 2; k++)
        if (rem < 0) {
            rem += (long long)(2 * S - 1);
            S--;
        }
#pragma unroll
    for (int k = 0; k < 2; k++)
        if (rem > (long long)(2 * S)) {
            S++;
            rem -= (long long)(2 * S - 1);
        }
    const unsigned long long M0 = S >> 2;
    const unsigned g = (unsigned)(S >> 1) & 1u;
    const unsigned st = ((unsigned)S & 1u) | (rem != 0 ? 1u : 0u);
    const unsigned long long M = M0 + (g & (st | ((unsigned)M0 & 1u)));
    const int E = ((ex - 1075 - 56 - odd) >> 1) + 1077;
    return __longlong_as_double((long long)(((unsigned long long)(E - 1) << 52) + M));
}
