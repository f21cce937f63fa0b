// Host build of the integer-exact binary64 adder, for the CPU self-test (tests/test_exact_add.py).
#include <stdint.h>

#include "nd_exact.cuh"

extern "C" void nd_exact_add_host(const double* a, const double* b, double* out, int64_t n) {
    for (int64_t i = 0; i < n; ++i) out[i] = nd::exact::add_rn(a[i], b[i]);
}
