/* dg_test.h -- checks of the library's own arithmetic (dgcuda_gb300).
 *
 * Not part of the drop-in interface of include/dg.h: these entry points run
 * the device helpers the kernels use -- the flux reciprocal, the sound
 * speed's square root and the single-precision positivity filter -- beside
 * the IEEE operations they stand in for, so that tests can check them on the
 * GPU.  No reference counterpart.  The oracle's and the tests' own use only.
 */
#ifndef DG_GB300_TEST_H
#define DG_GB300_TEST_H
#include "dg.h"

#ifdef __cplusplus
extern "C" {
#endif

/* the reciprocal the flux kernels use (Newton-Raphson from the hardware's
 * approximate reciprocal) and IEEE division, on the device, for n host
 * values: r[i] = rcp(x[i]), q[i] = 1 / x[i] (a check of the former) */
dg_status dg_probe_reciprocal(int device, int n, const double *x, double *r, double *q);
/* the sound speed's square root and IEEE sqrt on the device: r[i] =
 * sqrt_pos(x[i]), q[i] = sqrt(x[i]) (checks) */
dg_status dg_probe_sqrt(int device, int n, const double *x, double *r, double *q);
/* the Euler positivity test (rho >= 0, p >= 0) on the device for n states
 * U[4i..4i+3] = (rho, m_x, m_y, E): fast[i] = 1 where its single-precision
 * filter settles the state as physical, exact[i] = 1 where the FP64 test
 * finds it physical (fast implies exact; checks of the filter) */
dg_status dg_probe_physical(int device, int n, const double *U, int *fast, int *exact);

#ifdef __cplusplus
}
#endif
#endif
