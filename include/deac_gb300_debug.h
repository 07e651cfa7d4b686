/*
 * deac_gb300_debug.h -- test aids of the GB300 DEAC engine, in their own
 * library (lib/libdeac_gb300_debug.so).  Not part of the
 * drop-in boundary (include/deac_gb300.h) and with no counterpart in the
 * reference: they expose single device routines so that tests can check
 * them on inputs the full engine would rarely produce.
 */
#ifndef DEAC_GB300_DEBUG_H
#define DEAC_GB300_DEBUG_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* For each of `count` chains c: acc = start[c]; acc = fma(x[c*n+k],
 * w[c*n+k], acc) for k = 0..n-1, evaluated on device 0 twice -- by the
 * warp-parallel exact chain of the row-sum kernels (fast_out[c]) and one
 * step at a time (plain_out[c]).  Host arrays; allocates device memory;
 * synchronous.  Returns 0 or a DEAC_E_* code. */
int deac_debug_fma_chains(const double* x, const double* w, uint64_t n, const double* start, uint32_t count,
                          double* fast_out, double* plain_out);

/* Message for the last failing call of this library on this thread. */
const char* deac_debug_last_error(void);

#ifdef __cplusplus
}
#endif

#endif /* DEAC_GB300_DEBUG_H */
