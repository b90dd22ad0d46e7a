/*
 * fasttools2d_debug.h -- diagnostic entry of the GB300 spectral Ewald library.
 * No counterpart in the reference: it exposes the device evaluation of the
 * special functions used by the real-space kernels so that tests can compare
 * them with CUDA's exp/division and with a reference E1, the coordinate wrap
 * for a bitwise comparison with the drivers' formula, and a host-side
 * allocation fault injection for tests of the error path.
 */
#ifndef FASTTOOLS2D_DEBUG_H
#define FASTTOOLS2D_DEBUG_H
#ifdef __cplusplus
extern "C" {
#endif

/* Evaluate on the current device, for device arrays x[n] -> out[n]:
 * which = 0: E1(x); 1: exp(-x); 2: 0.5 E1(x) - exp(-x); 3: 1/x; 4, 5: the
 * drivers' coordinate wrap mod(x + L/2, L) - L/2 for L = 1 and L = 2.75.
 * Synchronises the device. */
int fte_debug_special(int which, const double* x_dev, double* out_dev, int n);

/* Host-side fault injection: with after = k > 0, the k-th device allocation
 * the library makes from now on (context workspaces, plan memory) fails as if
 * the device were out of memory, and the entry that needed it returns
 * FTE_ERR_ALLOC; after = 0 cancels a pending failure.  One-shot: later
 * allocations succeed again.  Process-wide; for tests of the error path. */
int fte_debug_fail_alloc(int after);

#ifdef __cplusplus
}
#endif
#endif
