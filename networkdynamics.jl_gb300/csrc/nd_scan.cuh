// Device building blocks shared by the RHS kernels: cache-policy loads and the exact
// (bitwise sequential) summation of FP64 terms on the integer pipes.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "nd_components.cuh"
#include "nd_exact.cuh"
#include "nd_internal.h"

namespace nd {
namespace dev {

constexpr int kBlock = 256;
constexpr int kWarpsPerBlock = kBlock / 32;
constexpr unsigned kFull = 0xffffffffu;
constexpr int kTile = 2048;  // heavy rows: terms per shared-memory tile

// ---- loads with an L2 eviction policy -------------------------------------------------
__device__ __forceinline__ uint64_t policy_evict_first() {
    uint64_t p;
    asm("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
    return p;
}
__device__ __forceinline__ uint64_t policy_evict_last() {
    uint64_t p;
    asm("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
    return p;
}
__device__ __forceinline__ int2 ld_hint(const int2* ptr, uint64_t pol) {
    int2 r;
    asm("ld.global.nc.L2::cache_hint.v2.s32 {%0, %1}, [%2], %3;" : "=r"(r.x), "=r"(r.y) : "l"(ptr), "l"(pol));
    return r;
}
__device__ __forceinline__ double ld_hint(const double* ptr, uint64_t pol) {
    double r;
    asm("ld.global.nc.L2::cache_hint.f64 %0, [%1], %2;" : "=d"(r) : "l"(ptr), "l"(pol));
    return r;
}
__device__ __forceinline__ int32_t ld_hint(const int32_t* ptr, uint64_t pol) {
    int32_t r;
    asm("ld.global.nc.L2::cache_hint.s32 %0, [%1], %2;" : "=r"(r) : "l"(ptr), "l"(pol));
    return r;
}
__device__ __forceinline__ uint32_t ld_hint(const uint32_t* ptr, uint64_t pol) {
    uint32_t r;
    asm("ld.global.nc.L2::cache_hint.u32 %0, [%1], %2;" : "=r"(r) : "l"(ptr), "l"(pol));
    return r;
}
__device__ __forceinline__ int4 ld_hint(const int4* ptr, uint64_t pol) {
    int4 r;
    asm("ld.global.nc.L2::cache_hint.v4.s32 {%0, %1, %2, %3}, [%4], %5;"
        : "=r"(r.x), "=r"(r.y), "=r"(r.z), "=r"(r.w)
        : "l"(ptr), "l"(pol));
    return r;
}
__device__ __forceinline__ double2 ld_hint(const double2* ptr, uint64_t pol) {
    double2 r;
    asm("ld.global.nc.L2::cache_hint.v2.f64 {%0, %1}, [%2], %3;" : "=d"(r.x), "=d"(r.y) : "l"(ptr), "l"(pol));
    return r;
}
__device__ __forceinline__ float2 ld_hint(const float2* ptr, uint64_t pol) {
    float2 r;
    asm("ld.global.nc.L2::cache_hint.v2.f32 {%0, %1}, [%2], %3;" : "=f"(r.x), "=f"(r.y) : "l"(ptr), "l"(pol));
    return r;
}
__device__ __forceinline__ float ld_hint(const float* ptr, uint64_t pol) {
    float r;
    asm("ld.global.nc.L2::cache_hint.f32 %0, [%1], %2;" : "=f"(r) : "l"(ptr), "l"(pol));
    return r;
}
// Stores with an L2 eviction-priority hint (streamed outputs: evict_first).
__device__ __forceinline__ void st_hint(double* ptr, double v, uint64_t pol) {
    asm volatile("st.global.L2::cache_hint.f64 [%0], %1, %2;" ::"l"(ptr), "d"(v), "l"(pol) : "memory");
}
__device__ __forceinline__ void st_hint(float* ptr, float v, uint64_t pol) {
    asm volatile("st.global.L2::cache_hint.f32 [%0], %1, %2;" ::"l"(ptr), "f"(v), "l"(pol) : "memory");
}
__device__ __forceinline__ void st_hint(double2* ptr, double2 v, uint64_t pol) {
    asm volatile("st.global.L2::cache_hint.v2.f64 [%0], {%1, %2}, %3;" ::"l"(ptr), "d"(v.x), "d"(v.y), "l"(pol)
                 : "memory");
}
__device__ __forceinline__ void st_hint(float2* ptr, float2 v, uint64_t pol) {
    asm volatile("st.global.L2::cache_hint.v2.f32 [%0], {%1, %2}, %3;" ::"l"(ptr), "f"(v.x), "f"(v.y), "l"(pol)
                 : "memory");
}

// Edge parameter of edge e (0 for the parameter-free unit diffusion edge).
template <typename T, int EK>
__device__ __forceinline__ T edge_param(const T* __restrict__ pe, int32_t e, uint64_t pol) {
    if constexpr (EK == ND_E_DIFFUSION_UNIT) {
        return T(0);
    } else {
        return ld_hint(pe + e, pol);
    }
}

// ---- exact sequential sums on the integer pipes ----------------------------------------

// Scaled term R = RN(t / 2^(eS-1075)) for a running sum whose exponent field is eS.
// ok = false when the step cannot be taken by the scan (too large, inf/nan).  For a
// tie (t / ulp exactly halfway between two integers) the truncated magnitude is returned
// with tie = true; the scan then rounds it to even against the running sum's parity.
__device__ __forceinline__ int64_t scaled_term(double t, int eS, bool& ok, bool& tie) {
    const uint64_t tb = exact::to_bits(t);
    uint64_t ft = tb & exact::kFrac;
    int et = (int)((tb >> 52) & 0x7ff);
    if ((tb & ~exact::kSign) == 0) return 0;
    if (et == 0x7ff) {
        ok = false;
        return 0;
    }
    if (et) ft |= exact::kHidden;
    else et = 1;
    const int sh = eS - et;  // t / ulp(S) = ft · 2^-sh
    uint64_t mag;
    if (sh <= 0) {
        if (sh < -9) {
            ok = false;
            return 0;
        }
        mag = ft << (-sh);
    } else if (sh >= 64) {
        mag = 0;  // |t| < 2^-11 ulp: rounds to zero, never a tie
    } else {
        mag = ft >> sh;
        const uint64_t rem = ft & ((1ull << sh) - 1);
        const uint64_t half = 1ull << (sh - 1);
        if (rem > half) mag += 1;
        else if (rem == half) tie = true;
    }
    if (mag >= (1ull << 52)) ok = false;
    return (tb & exact::kSign) ? -(int64_t)mag : (int64_t)mag;
}

// Add the terms held by lanes [0, n) of the warp to S, in lane order, exactly as the
// sequential loop S = S + t_0; S = S + t_1; ... would.  S is warp-uniform.
__device__ __forceinline__ double exact_scan_add(double S, double t, int n, int lane) {
    int j0 = 0;
    while (j0 < n) {
        const uint64_t sb = exact::to_bits(S);
        const int eS = (int)((sb >> 52) & 0x7ff);
        if (eS == 0 || eS == 0x7ff) {  // zero / subnormal / non-finite sum: one exact step
            S = exact::add_rn(S, __shfl_sync(kFull, t, j0));
            ++j0;
            continue;
        }
        const bool active = lane >= j0 && lane < n;
        bool ok = true, tie = false;
        int64_t x = active ? scaled_term(t, eS, ok, tie) : 0;
        // Ties round to even against the running sum.  Its parity evolves as p -> p ^ (R & 1)
        // for ordinary steps and p -> 0 after a tie step; the composition of such maps
        // (p -> (p & ka) ^ kb) is scanned to give each lane the parity before its step.
        unsigned ka = tie ? 0u : 1u, kb = tie ? 0u : (unsigned)(x & 1);
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const unsigned pa = __shfl_up_sync(kFull, ka, off), pb = __shfl_up_sync(kFull, kb, off);
            if (lane >= off) {
                kb = (pb & ka) ^ kb;
                ka = pa & ka;
            }
        }
        if (__any_sync(kFull, tie)) {
            unsigned xa = __shfl_up_sync(kFull, ka, 1), xb = __shfl_up_sync(kFull, kb, 1);
            if (lane == 0) {
                xa = 1u;
                xb = 0u;
            }
            const unsigned p_prev = ((unsigned)(sb & 1) & xa) ^ xb;
            if (tie) {
                const uint64_t mag = (uint64_t)(x < 0 ? -x : x);
                const uint64_t c = (p_prev ^ (unsigned)(mag & 1)) & 1u;  // 1: round away from zero
                x = (exact::to_bits(t) & exact::kSign) ? -(int64_t)(mag + c) : (int64_t)(mag + c);
            }
        }
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const int64_t y = __shfl_up_sync(kFull, x, off);
            if (lane >= off) x += y;
        }
        const int64_t mS = (int64_t)((sb & exact::kFrac) | exact::kHidden);
        const int64_t m = (sb & exact::kSign) ? x - mS : x + mS;
        const uint64_t am = (uint64_t)(m < 0 ? -m : m);
        const bool valid = ok && am >= (1ull << 52) + 1 && am <= (1ull << 53) - 2;
        const unsigned bad = __ballot_sync(kFull, active && !valid);
        const int L = bad ? __ffs(bad) - 1 : n;
        if (L > j0) {
            const int64_t mL = __shfl_sync(kFull, m, L - 1);
            const uint64_t aL = (uint64_t)(mL < 0 ? -mL : mL);
            S = exact::from_bits((mL < 0 ? exact::kSign : 0) | ((uint64_t)eS << 52) | (aL & exact::kFrac));
        }
        if (L < n) S = exact::add_rn(S, __shfl_sync(kFull, t, L));
        j0 = L + 1;
    }
    return S;
}

// Sequential exact sum of n terms in shared memory by one warp, 32 at a time.
__device__ __forceinline__ double exact_scan_smem(double S, const double* __restrict__ tile, int n, int lane) {
    for (int c = 0; c < n; c += 32) {
        const int k = c + lane;
        const double t = k < n ? tile[k] : 0.0;
        S = exact_scan_add(S, t, min(32, n - c), lane);
    }
    return S;
}

// The same sum with a sliding window of 8 terms per lane (256 per step): each lane scales
// its 8 terms (resolving ties against the running sum's parity) and prefix-sums them
// locally, one warp scan adds the lanes before it, and every position checks that its
// running sum stays strictly inside S's binade.  The window then slides to just past the
// first position that failed (a binade change), which is added with the hardware adder.
// Long hub rows change binade every ~100 terms, so a step advances far at the cost of a
// single warp scan.
constexpr int kScanPer = 8;
constexpr int kScanFallback = 16;
constexpr int kScanFallbackMax = 1024;
static __device__ __forceinline__ double exact_scan_wide(double S, const double* __restrict__ tile, int n, int lane) {
    int pos = 0;
    int fallback = kScanFallback;  // length of the next run of hardware adds after a stall
    while (pos < n) {
        const uint64_t sb = exact::to_bits(S);
        const int eS = (int)((sb >> 52) & 0x7ff);
        if (eS == 0 || eS == 0x7ff) {  // zero / subnormal / non-finite sum: one exact step
            S = exact::add_rn(S, tile[pos]);
            ++pos;
            continue;
        }
        const int end = min(n, pos + 32 * kScanPer);
        const int base = pos + lane * kScanPer;
        int64_t pre[kScanPer];
        unsigned okmask = 0, tiemask = 0;
#pragma unroll
        for (int i = 0; i < kScanPer; ++i) {
            bool ok = true, tie = false;
            const int q = base + i;
            pre[i] = q < end ? scaled_term(tile[q], eS, ok, tie) : 0;
            okmask |= (unsigned)ok << i;
            tiemask |= (unsigned)tie << i;
        }
        if (__any_sync(kFull, tiemask != 0)) {
            // Ties round to even against the running sum, whose parity evolves as
            // p -> p ^ (R & 1) for an ordinary step and p -> 0 after a tie.  Each lane
            // composes its steps into p -> (p & ka) ^ kb, a warp scan composes the lanes,
            // and each lane replays its steps from the parity before its first one.
            unsigned ka = 1u, kb = 0u;
#pragma unroll
            for (int i = 0; i < kScanPer; ++i) {
                if ((tiemask >> i) & 1u) ka = kb = 0u;
                else kb ^= (unsigned)(pre[i] & 1);
            }
#pragma unroll
            for (int off = 1; off < 32; off <<= 1) {
                const unsigned pa = __shfl_up_sync(kFull, ka, off), pb = __shfl_up_sync(kFull, kb, off);
                if (lane >= off) {
                    kb = (pb & ka) ^ kb;
                    ka = pa & ka;
                }
            }
            unsigned xa = __shfl_up_sync(kFull, ka, 1), xb = __shfl_up_sync(kFull, kb, 1);
            if (lane == 0) {
                xa = 1u;
                xb = 0u;
            }
            unsigned par = ((unsigned)(sb & 1) & xa) ^ xb;
#pragma unroll
            for (int i = 0; i < kScanPer; ++i) {
                if ((tiemask >> i) & 1u) {
                    const uint64_t mag = (uint64_t)(pre[i] < 0 ? -pre[i] : pre[i]);
                    const uint64_t c = (par ^ (unsigned)(mag & 1)) & 1u;  // 1: away from zero
                    pre[i] = (exact::to_bits(tile[base + i]) & exact::kSign) ? -(int64_t)(mag + c)
                                                                              : (int64_t)(mag + c);
                    par = 0u;
                } else {
                    par ^= (unsigned)(pre[i] & 1);
                }
            }
        }
        int64_t run = 0;
#pragma unroll
        for (int i = 0; i < kScanPer; ++i) {
            run += pre[i];
            pre[i] = run;
        }
        int64_t x = run;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const int64_t y = __shfl_up_sync(kFull, x, off);
            if (lane >= off) x += y;
        }
        const int64_t mS0 = (int64_t)((sb & exact::kFrac) | exact::kHidden);
        const int64_t mS = (sb & exact::kSign) ? -mS0 : mS0;
        const int64_t before = mS + x - run;  // running sum before this lane's first term
        int firstbad = 0x7fffffff;
#pragma unroll
        for (int i = kScanPer - 1; i >= 0; --i) {
            const int64_t m = before + pre[i];
            const uint64_t am = (uint64_t)(m < 0 ? -m : m);
            const bool valid = ((okmask >> i) & 1u) && am >= (1ull << 52) + 1 && am <= (1ull << 53) - 2;
            if (base + i < end && !valid) firstbad = base + i;
        }
        const int P = (int)__reduce_min_sync(kFull, (unsigned)firstbad);
        const int acc_end = P < end ? P : end;  // positions [pos, acc_end) are exact
        if (acc_end > pos) {
            const int q = acc_end - 1 - pos, owner = q / kScanPer, idx = q % kScanPer;
            int64_t mine = 0;
#pragma unroll
            for (int i = 0; i < kScanPer; ++i)
                if (i == idx) mine = before + pre[i];
            const int64_t mL = __shfl_sync(kFull, mine, owner);
            const uint64_t aL = (uint64_t)(mL < 0 ? -mL : mL);
            S = exact::from_bits((mL < 0 ? exact::kSign : 0) | ((uint64_t)eS << 52) | (aL & exact::kFrac));
        }
        if (P < end) {
            S = __dadd_rn(S, tile[P]);
            const int advanced = P + 1 - pos;
            pos = P + 1;
            // A sum hovering at a binade boundary changes binade every few terms and the
            // scan stalls; then a run of hardware adds on lane 0 is cheaper per term.  The
            // run doubles while the stalls persist (up to kScanFallbackMax terms) and drops
            // back once a step advances far, so a row never costs much more than a plain
            // chain of adds.
            if (advanced < kScanPer && pos < n) {
                const int stop = min(n, pos + fallback);
                if (lane == 0)
                    for (int i = pos; i < stop; ++i) S = __dadd_rn(S, tile[i]);
                S = __shfl_sync(kFull, S, 0);
                pos = stop;
                fallback = min(2 * fallback, kScanFallbackMax);
            } else if (advanced >= 64) {
                fallback = kScanFallback;
            }
        } else {
            pos = end;
            fallback = kScanFallback;
        }
    }
    return S;
}


}  // namespace dev
}  // namespace nd
