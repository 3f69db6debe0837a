// Device-side forms of the complex dots, the sums of magnitudes, the norms,
// complex AXPY and the plane rotations (l1x.cu). Arrays are device pointers.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "l1.h"

namespace mw {

// mode 0 dotu, 1 dotc (complex x, y; result re, im), 2 asum (real x),
// 3 |Re|+|Im| sum (complex x), 4 nrm2 (real x), 5 nrm2 (complex x); the
// result (one or two double-doubles) is copied to result_host and the call
// synchronises.
bool launch_reduce(int mode, int64_t n, const void *x, int64_t incx, const void *y, int64_t incy,
                   double2 *result_host, const char *routine);

// y += alpha * x (complex).
void launch_waxpy(int64_t n, cdd_host alpha, const void *x, int64_t incx, void *y, int64_t incy);

// (x, y) := (h11*x + h12*y, h21*x + h22*y), h = {h11, h12, h21, h22} real,
// each of e2 components (1 real, 2 complex).
void launch_rot(int64_t n, void *x, int64_t incx, void *y, int64_t incy, int e2, const dd_host h[4]);

}  // namespace mw
