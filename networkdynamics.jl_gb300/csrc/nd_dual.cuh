// Forward-mode dual numbers: a value with N partial derivatives, carried through the
// component functions of nd_components.cuh (which are templates on their arithmetic type),
// so that the Jacobian of a component with respect to its inputs comes out of the same code
// that computes its output -- what ForwardDiff does for the reference's colored Jacobians.
// Rules: sums and products by the usual derivative rules, the quotient as
// (a' - (a / b) b') / b, sin' = cos and cos' = -sin of the value.
#pragma once

#include "nd_components.cuh"

namespace nd {

template <typename T, int N>
struct Dual {
    T v;
    T d[N];
    __device__ __forceinline__ Dual() : v(T(0)) {
#pragma unroll
        for (int k = 0; k < N; ++k) d[k] = T(0);
    }
    __device__ __forceinline__ explicit Dual(T x) : v(x) {
#pragma unroll
        for (int k = 0; k < N; ++k) d[k] = T(0);
    }
    // the k-th independent variable with value x
    static __device__ __forceinline__ Dual seed(T x, int k) {
        Dual r(x);
        r.d[k] = T(1);
        return r;
    }
};

template <typename T, int N>
__device__ __forceinline__ Dual<T, N> operator-(const Dual<T, N>& a) {
    Dual<T, N> r;
    r.v = -a.v;
#pragma unroll
    for (int k = 0; k < N; ++k) r.d[k] = -a.d[k];
    return r;
}
template <typename T, int N>
__device__ __forceinline__ bool operator!=(const Dual<T, N>& a, const Dual<T, N>& b) {
    return a.v != b.v;
}
// |x| as the branch tests of the robust complex division read it: on the value
template <typename T, int N>
__device__ __forceinline__ T fabs(const Dual<T, N>& a) {
    return a.v < T(0) ? -a.v : a.v;
}
template <typename T, int N>
__device__ __forceinline__ Dual<T, N> ldv(const Dual<T, N>* p) {
    return *p;
}

template <typename T, int N>
struct Arith<Dual<T, N>> {
    using D = Dual<T, N>;
    using A = Arith<T>;
    static __device__ __forceinline__ D add(const D& a, const D& b) {
        D r;
        r.v = A::add(a.v, b.v);
#pragma unroll
        for (int k = 0; k < N; ++k) r.d[k] = A::add(a.d[k], b.d[k]);
        return r;
    }
    static __device__ __forceinline__ D sub(const D& a, const D& b) {
        D r;
        r.v = A::sub(a.v, b.v);
#pragma unroll
        for (int k = 0; k < N; ++k) r.d[k] = A::sub(a.d[k], b.d[k]);
        return r;
    }
    static __device__ __forceinline__ D mul(const D& a, const D& b) {
        D r;
        r.v = A::mul(a.v, b.v);
#pragma unroll
        for (int k = 0; k < N; ++k) r.d[k] = A::add(A::mul(a.d[k], b.v), A::mul(a.v, b.d[k]));
        return r;
    }
    static __device__ __forceinline__ D div(const D& a, const D& b) {
        D r;
        r.v = A::div(a.v, b.v);
#pragma unroll
        for (int k = 0; k < N; ++k) r.d[k] = A::div(A::sub(a.d[k], A::mul(r.v, b.d[k])), b.v);
        return r;
    }
    static __device__ __forceinline__ D sin_phase(const D& a) {
        D r;
        r.v = A::sin_phase(a.v);
        const T c = A::cos_phase(a.v);
#pragma unroll
        for (int k = 0; k < N; ++k) r.d[k] = A::mul(c, a.d[k]);
        return r;
    }
    static __device__ __forceinline__ D cos_phase(const D& a) {
        D r;
        r.v = A::cos_phase(a.v);
        const T s = -A::sin_phase(a.v);
#pragma unroll
        for (int k = 0; k < N; ++k) r.d[k] = A::mul(s, a.d[k]);
        return r;
    }
};

}  // namespace nd
