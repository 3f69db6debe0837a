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

// Scalar generators, run as one device thread so every result comes from the
// same double-double arithmetic as the vector routines.
//   GEN_CABS1  in: z (re, im)          out: 0 |Re z| + |Im z|
//   GEN_ROTG   in: a, b                out: 0 a (= r), 1 b (= z), 2 c, 3 s
//   GEN_ROTMG  in: d1, d2, x1, y1      out: 0 d1, 1 d2, 2 x1, 3..7 dparam(1..5)
//   GEN_WROTG  in: a (re, im), b (re, im)   out: 0/1 a, 2 c, 3/4 s
// Bit i of mask is set when result i is to be written back.
enum { GEN_CABS1 = 0, GEN_ROTG = 1, GEN_ROTMG = 2, GEN_WROTG = 3 };
struct GenInput {
    double2 v[4];
};
struct GenResult {
    double2 v[8];
    unsigned mask;
};
bool launch_generator(int op, const GenInput &in, GenResult *result_host, const char *routine);

}  // namespace mw
