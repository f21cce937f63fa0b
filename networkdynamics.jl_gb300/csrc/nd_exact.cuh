// Exact IEEE-754 binary64 addition (round to nearest, ties to even) in integer
// arithmetic.
//
// On GB300 the FP64 pipe retires about two lanes per clock per SM (1/64 of FP32), and a
// DADD holds its sub-partition's FP64 pipe for the whole warp even with one lane active.
// The per-vertex sums of the RHS are long chains of dependent additions that must round
// exactly like the reference's sequential `aggbuf[i] += o[k]`.  Running those chains on
// the integer pipes keeps the FP64 pipe for the edge functions.
//
// Method (textbook binary floating-point addition): order the operands by magnitude,
// align the smaller significand with 8 guard bits and a sticky bit, add or subtract,
// normalise (left shifts are exact because no bit was shifted out when the exponents
// differ by at most one), round to nearest even on the guard bits, repack.  Zeros,
// subnormals and the signs of exact-zero results follow IEEE-754 round-to-nearest.
// NaN / infinity operands are handed to the hardware adder.
//
// The header compiles as CUDA (device) and as plain C++ (host, for the CPU self-test).
#pragma once

#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#define ND_HD __host__ __device__ __forceinline__
#else
#define ND_HD inline
#endif

namespace nd {
namespace exact {

constexpr uint64_t kSign = 0x8000000000000000ull;
constexpr uint64_t kFrac = 0x000FFFFFFFFFFFFFull;
constexpr uint64_t kHidden = 0x0010000000000000ull;
constexpr int kGuard = 8;

ND_HD uint64_t to_bits(double x) {
#if defined(__CUDA_ARCH__)
    return (uint64_t)__double_as_longlong(x);
#else
    uint64_t u;
    memcpy(&u, &x, sizeof u);
    return u;
#endif
}

ND_HD double from_bits(uint64_t u) {
#if defined(__CUDA_ARCH__)
    return __longlong_as_double((long long)u);
#else
    double x;
    memcpy(&x, &u, sizeof x);
    return x;
#endif
}

ND_HD int clz64(uint64_t x) {
#if defined(__CUDA_ARCH__)
    return __clzll((long long)x);
#else
    return x ? __builtin_clzll(x) : 64;
#endif
}

// Hardware addition for the rare inputs the integer path hands off (inf, nan, overflow).
// On the device it is a volatile asm statement: a plain __dadd_rn behind the branch gets
// if-converted and issued on every call (measured: two DADDs per call), which costs a
// full FP64 warp slot each time.
ND_HD double hw_add(double a, double b) {
#if defined(__CUDA_ARCH__)
    double s;
    asm volatile("add.rn.f64 %0, %1, %2;" : "=d"(s) : "d"(a), "d"(b));
    return s;
#else
    volatile double s = a + b;
    return s;
#endif
}

// a + b rounded to nearest even, computed with integer operations.  Written with selects
// instead of branches so that the lanes of a warp stay converged; only non-finite inputs
// and overflow leave the straight-line path.
ND_HD double add_rn(double a, double b) {
    const uint64_t ia0 = to_bits(a), ib0 = to_bits(b);
    const uint64_t ma0 = ia0 & ~kSign, mb0 = ib0 & ~kSign;
    if (ma0 >= 0x7FF0000000000000ull || mb0 >= 0x7FF0000000000000ull) return hw_add(a, b);  // inf / nan
    const bool sw = ma0 < mb0;  // order so that |a| >= |b|
    const uint64_t ia = sw ? ib0 : ia0, ib = sw ? ia0 : ib0;
    const uint64_t ma = sw ? mb0 : ma0, mb = sw ? ma0 : mb0;
    int ea = (int)(ma >> 52), eb = (int)(mb >> 52);
    uint64_t fa = ((ma & kFrac) | (ea ? kHidden : 0)) << kGuard;  // < 2^61
    uint64_t fb = ((mb & kFrac) | (eb ? kHidden : 0)) << kGuard;
    ea += (ea == 0);  // subnormals share exponent 1 with the smallest normals
    eb += (eb == 0);
    // align b: shift by d with a sticky bit; d >= 63 leaves only the sticky bit (fb < 2^61)
    const int d = ea - eb < 63 ? ea - eb : 63;
    const uint64_t sticky = d ? (uint64_t)((fb << (64 - d)) != 0) : 0;
    const uint64_t fbs = (fb >> d) | sticky;
    const bool sub = ((ia ^ ib) & kSign) != 0;
    uint64_t r = sub ? fa - fbs : fa + fbs;
    int e = ea;
    const int carry = (int)(r >> (52 + kGuard + 1));  // 0 or 1
    r = (r >> carry) | (r & (uint64_t)carry);
    e += carry;
    // normalise left (exact: nothing was shifted out when a left shift is needed by more
    // than one bit); stop at the subnormal range
    int s = clz64(r) - (63 - 52 - kGuard);
    s = s < 0 ? 0 : s;
    s = s > e - 1 ? e - 1 : s;
    r <<= s;
    e -= s;
    const uint64_t half = 1ull << (kGuard - 1);
    const uint64_t g = r & ((1ull << kGuard) - 1);
    r >>= kGuard;
    r += (uint64_t)((g > half) | ((g == half) & (r & 1)));
    const int ov = (int)(r >> 53);  // rounding carried into a new binade
    r >>= ov;
    e += ov;
    if (e >= 0x7FF) return hw_add(a, b);  // overflow to infinity
    const uint64_t efield = (r >= kHidden) ? (uint64_t)e : 0;  // subnormal result keeps field 0
    uint64_t out = (ia & kSign) | (efield << 52) | (r & kFrac);
    out = (r == 0) ? 0ull : out;        // exact cancellation: +0 in round-to-nearest
    out = (ma == 0) ? (ia & ib) : out;  // both zero: -0 only for (-0) + (-0)
    return from_bits(out);
}

}  // namespace exact
}  // namespace nd
