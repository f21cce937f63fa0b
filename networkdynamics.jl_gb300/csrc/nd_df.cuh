// Double-float arithmetic on the FP32 pipe: a value is the unevaluated sum hi + lo of two
// floats (|lo| <= ulp(hi) / 2), about 48 significant bits.  GB300 retires FP32 at 64 times
// its FP64 rate, so a double-float sine (a few hundred FP32 operations) costs a fraction of
// an FP64 one while keeping errors near 1e-14 relative.
//
// The building blocks are the published error-free transformations: Knuth's two-sum and
// Dekker's fast two-sum (TAOCP vol. 2, 4.2.2; Dekker 1971) and the product error of one
// fused multiply-add.  Every operation is written with explicitly rounded intrinsics so that
// no contraction or reassociation changes them.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace nd {
namespace df {

struct Df {
    float hi, lo;
};

__device__ __forceinline__ Df two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return {s, e};
}
// |a| >= |b| (or a == 0)
__device__ __forceinline__ Df fast_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ Df two_prod(float a, float b) {
    const float p = __fmul_rn(a, b);
    return {p, __fmaf_rn(a, b, -p)};
}

__device__ __forceinline__ Df add(Df x, Df y) {
    Df s = two_sum(x.hi, y.hi);
    const Df t = two_sum(x.lo, y.lo);
    s.lo = __fadd_rn(s.lo, t.hi);
    s = fast_two_sum(s.hi, s.lo);
    s.lo = __fadd_rn(s.lo, t.lo);
    return fast_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ Df neg(Df x) { return {-x.hi, -x.lo}; }
__device__ __forceinline__ Df sub(Df x, Df y) { return add(x, neg(y)); }
__device__ __forceinline__ Df mul(Df x, Df y) {
    Df p = two_prod(x.hi, y.hi);
    p.lo = __fmaf_rn(x.hi, y.lo, p.lo);
    p.lo = __fmaf_rn(x.lo, y.hi, p.lo);
    return fast_two_sum(p.hi, p.lo);
}
__device__ __forceinline__ Df mul_f(Df x, float f) {
    Df p = two_prod(x.hi, f);
    p.lo = __fmaf_rn(x.lo, f, p.lo);
    return fast_two_sum(p.hi, p.lo);
}
// x / y by one float quotient and two correction steps of the remainder
__device__ __forceinline__ Df div(Df x, Df y) {
    const float q1 = __fdiv_rn(x.hi, y.hi);
    const Df r = sub(x, mul_f(y, q1));
    const float q2 = __fdiv_rn(r.hi, y.hi);
    const Df r2 = sub(r, mul_f(y, q2));
    const float q3 = __fdiv_rn(r2.hi, y.hi);
    const Df q = fast_two_sum(q1, q2);
    return add(q, Df{q3, 0.f});
}

// A double as hi + lo by bit operations (no FP64 instruction): hi keeps the sign, the
// exponent and the leading 24 significant bits; lo is the remaining 29 bits rounded to a
// float.  Magnitudes below 2^-100 become 0 (far below the 48-bit resolution of any value
// these kernels combine them with); magnitudes from 2^128 up, infinities and NaN go
// through the hardware conversion and stay infinite or NaN.
__device__ __forceinline__ Df from_double(double d) {
    const uint64_t b = (uint64_t)__double_as_longlong(d);
    const uint32_t sign = (uint32_t)(b >> 63);
    const int e = (int)((b >> 52) & 0x7ff) - 1023;
    if (e < -100) return {sign ? -0.f : 0.f, 0.f};
    if (e > 127) return {__double2float_rn(d), 0.f};
    const uint64_t mant = b & 0xFFFFFFFFFFFFFull;
    const float hi = __int_as_float((int)((sign << 31) | ((uint32_t)(e + 127) << 23) | (uint32_t)(mant >> 29)));
    // the remaining bits are low * 2^(e - 52), low < 2^29: the conversion rounds them to 24
    // bits and the exact power-of-two scaling may give a subnormal, lost at 48 bits
    const uint32_t low = (uint32_t)(mant & 0x1FFFFFFFu);
    float lo = ldexpf(__uint2float_rn(low), e - 52);
    if (sign) lo = -lo;
    return {hi, lo};
}

// A double exactly as hi + mid + lo: the leading 24, the next 24 and the last 5 significant
// bits.  Used where the argument's absolute accuracy matters (phases reduced modulo π/2).
struct Df3 {
    Df hm;  // hi + mid, a normalised double-float
    float lo;
};
__device__ __forceinline__ Df3 from_double3(double d) {
    const uint64_t b = (uint64_t)__double_as_longlong(d);
    const uint32_t sign = (uint32_t)(b >> 63);
    const int e = (int)((b >> 52) & 0x7ff) - 1023;
    if (e < -100) return {{sign ? -0.f : 0.f, 0.f}, 0.f};
    if (e > 127) return {{__double2float_rn(d), 0.f}, 0.f};
    const uint64_t mant = b & 0xFFFFFFFFFFFFFull;
    const float hi = __int_as_float((int)((sign << 31) | ((uint32_t)(e + 127) << 23) | (uint32_t)(mant >> 29)));
    // bits 28..5 and 4..0 of the stored significand, scaled exactly (integers below 2^24)
    float mid = ldexpf(__uint2float_rn((uint32_t)((mant >> 5) & 0xFFFFFFu)), e - 47);
    float lo = ldexpf(__uint2float_rn((uint32_t)(mant & 0x1Fu)), e - 52);
    if (sign) {
        mid = -mid;
        lo = -lo;
    }
    return {fast_two_sum(hi, mid), lo};
}

// hi + lo rounded to a double (one FP64 add of two exactly converted floats)
__device__ __forceinline__ double to_double(Df x) { return __dadd_rn((double)x.hi, (double)x.lo); }

// π/2 as the sum of three floats and 2/π rounded to a float (from π to 80 digits by
// Machin's formula).
constexpr float kPio2Hi = 1.5707963705062866f;
constexpr float kPio2Mid = -4.371138828673793e-08f;
constexpr float kPio2Lo = -1.7151245100058819e-15f;
constexpr float kTwoOverPi = 0.6366197466850281f;

// Taylor coefficients (-1)^k / (2k+1)! (sine) and (-1)^k / (2k)! (cosine), each the
// nearest float plus the nearest float to the remainder, for k = 0..8.  On |r| <= π/4 the
// first omitted terms are below 1e-18.
template <bool Sine>
struct Taylor;
template <>
struct Taylor<true> {
    static __device__ __forceinline__ float hi(int k) {
        switch (k) {
            case 0: return 1.0f;
            case 1: return -0.1666666716337204f;
            case 2: return 0.008333333767950535f;
            case 3: return -0.00019841270113829523f;
            case 4: return 2.7557318844628753e-06f;
            case 5: return -2.5052107943679403e-08f;
            case 6: return 1.6059044372074283e-10f;
            case 7: return -7.647163609812713e-13f;
            default: return 2.8114573589663704e-15f;
        }
    }
    static __device__ __forceinline__ float lo(int k) {
        switch (k) {
            case 0: return 0.0f;
            case 1: return 4.967053879312289e-09f;
            case 2: return -4.34617203337595e-10f;
            case 3: return 2.725596874933456e-12f;
            case 4: return 3.793571224297229e-14f;
            default: return -4.4176230446483665e-16f;
        }
    }
};
template <>
struct Taylor<false> {
    static __device__ __forceinline__ float hi(int k) {
        switch (k) {
            case 0: return 1.0f;
            case 1: return -0.5f;
            case 2: return 0.0416666679084301f;
            case 3: return -0.0013888889225199819f;
            case 4: return 2.4801587642286904e-05f;
            case 5: return -2.755731998149713e-07f;
            case 6: return 2.0876755879584152e-09f;
            case 7: return -1.147074536050896e-11f;
            default: return 4.7794772561329454e-14f;
        }
    }
    static __device__ __forceinline__ float lo(int k) {
        switch (k) {
            case 0: return 0.0f;
            case 1: return 0.0f;
            case 2: return -1.2417634698280722e-09f;
            case 3: return 3.3631094437103215e-11f;
            case 4: return -3.40699609366682e-13f;
            default: return 7.575112209051195e-15f;
        }
    }
};

// Σ_k c_k s^k by Horner: the terms k >= 6 (below 1e-11 of the sum on |r| <= π/4) in float,
// the rest in double-float.
template <bool Sine>
__device__ __forceinline__ Df series(Df s) {
    using C = Taylor<Sine>;
    const float t = __fmaf_rn(__fmaf_rn(C::hi(8), s.hi, C::hi(7)), s.hi, C::hi(6));
    Df acc = add(Df{C::hi(5), C::lo(5)}, two_prod(t, s.hi));
#pragma unroll
    for (int k = 4; k >= 0; --k) acc = add(Df{C::hi(k), C::lo(k)}, mul(acc, s));
    return acc;
}

// sin(x) of a double given exactly as three floats, |x| below ~2^20 (phase differences of
// wound-up phases): x = q π/2 + r with r in [-π/4, π/4] (π/2 in three floats, the
// products q·π/2 exact, the reduction carried out on all 53 bits of x), then
// sin r = r Σ (-1)^k r^2k / (2k+1)! or cos r = Σ (-1)^k r^2k / (2k)! by the quadrant.
__device__ __forceinline__ Df sin(Df3 x) {
    const float q = rintf(__fmul_rn(x.hm.hi, kTwoOverPi));
    Df r = sub(x.hm, two_prod(q, kPio2Hi));
    r = sub(r, two_prod(q, kPio2Mid));
    r = sub(r, Df{__fmul_rn(q, kPio2Lo), 0.f});
    r = add(r, Df{x.lo, 0.f});
    const Df s = mul(r, r);
    const int quad = (int)q & 3;
    const Df v = (quad & 1) ? series<false>(s) : mul(r, series<true>(s));
    return (quad & 2) ? neg(v) : v;
}

}  // namespace df
}  // namespace nd
