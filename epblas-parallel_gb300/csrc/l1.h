// Internal launch interface of the level-1 kernels (device pointers only).
#pragma once
#include <stdint.h>

namespace mw {

struct dd_host { double hi, lo; };
struct cdd_host { dd_host re, im; };

// unit: the CALLER's increments are all 1, which selects the reference's
// unit-stride kernel (fast multiply on the body of each slice) even when the
// staged device copy has been compacted. team: reference OpenMP team size used
// to reproduce the per-slice body/tail split of that kernel.
void launch_mscal(int64_t n, dd_host alpha, void *x, int64_t inc, bool unit, int64_t team);
void launch_wscal(int64_t n, cdd_host alpha, void *x, int64_t inc, bool unit, int64_t team);
void launch_wmscal(int64_t n, dd_host alpha, void *x, int64_t inc, bool unit, int64_t team);
void launch_maxpy(int64_t n, dd_host alpha, const void *x, int64_t incx, void *y, int64_t incy, bool unit,
                  int64_t team);
// elem2: 16-byte words per element (1 real, 2 complex)
void launch_copy(int64_t n, const void *x, int64_t incx, void *y, int64_t incy, int elem2);
void launch_swap(int64_t n, void *x, int64_t incx, void *y, int64_t incy, int elem2);
// 0-based index of the maximum (or -1 for an empty range).
bool launch_iamax(int64_t n, const void *x, int64_t inc, bool cplx, int64_t *result_host, const char *routine);
bool launch_mdot(int64_t n, const void *x, int64_t incx, const void *y, int64_t incy, dd_host *result_host,
                 const char *routine);

}  // namespace mw
