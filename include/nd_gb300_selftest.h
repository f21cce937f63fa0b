/*
 * nd_gb300_selftest.h — diagnostic entry points of libnd_b200.so.
 *
 * These have no counterpart in the reference: they run the device building blocks of
 * the FP64 RHS on caller data so that tests can compare them with the CPU's IEEE-754
 * arithmetic.  Device pointers, stream-ordered.
 */
#ifndef ND_GB300_SELFTEST_H
#define ND_GB300_SELFTEST_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* out[i] = a[i] + b[i] with the integer-exact binary64 adder of the RHS sums. */
int nd_selftest_exact_add(const double* a, const double* b, double* out, int64_t n, void* stream);

/* out[w] = (((s0[w] + terms[seg[w]]) + terms[seg[w]+1]) + ...) over the segment
 * [seg[w], seg[w+1]), computed with the warp exact scan used for hub rows. */
int nd_selftest_exact_scan(const double* terms, const int64_t* seg, const double* s0, double* out, int64_t nseg,
                           void* stream);

#ifdef __cplusplus
}
#endif
#endif /* ND_GB300_SELFTEST_H */
