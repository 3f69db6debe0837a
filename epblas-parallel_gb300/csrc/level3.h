// Internal interface of the routines built on the GEMM engines and of the
// level-2 kernels (device pointers only).
#pragma once
#include <stdint.h>

#include "../../include/mwblas_gb300.h"
#include "gemm.h"

namespace mw {

// Engine dispatch shared by mgemm_/wgemm_ and the level-3 routines.
// force_engine < 0 follows the library setting.
bool run_gemm(GemmArgs &g, bool cplx, int force_engine, const char *routine);

// True when the integer-exact tensor-core engine can run on this device.
bool ozaki_available();

// SYRK (cplx=false) / HERK (cplx=herm=true) on device arrays. `scal` carries
// alpha/beta (real or complex with zero imaginary part) and beta_kind.
// uplo: 1 upper, 2 lower. trans=false: C = alpha*A*op(A) with A n x k.
bool syrk_device(bool cplx, bool herm, int uplo, bool trans, int64_t n, int64_t k, const void *A, int64_t lda,
                 const GemmArgs &scal, void *C, int64_t ldc, const char *routine);

// Blocked triangular solve on device arrays (flags already upper-case and
// validated; real 'C' folded to 'T').
bool trsm_device(char side, char uplo, char transa, char diag, int64_t m, int64_t n, dd_host alpha, const void *A,
                 int64_t lda, void *B, int64_t ldb, const char *routine);
void launch_zero_matrix(int64_t m, int64_t n, void *B, int64_t ldb);

// Grouped GEMM on device arrays for internal use (arguments valid, no sync,
// launched directly); instances with m, n >= tensor_min (> 0) and k >= 64 run
// on the tensor cores.
bool grouped_gemm_device(int64_t count, const char *ta, const char *tb, const int64_t *m, const int64_t *n,
                         const int64_t *k, const mwblas_real64x2 *alpha, const mwblas_real64x2 *const *a,
                         const int64_t *lda, const mwblas_real64x2 *const *b, const int64_t *ldb,
                         const mwblas_real64x2 *beta, mwblas_real64x2 *const *c, const int64_t *ldc,
                         int tensor_min, const char *routine);

// y := alpha*op(A)*x + beta*y on device arrays (increments may be negative).
bool gemv_device(bool trans, int64_t m, int64_t n, dd_host alpha, const void *A, int64_t lda, const void *x,
                 int64_t incx, dd_host beta, int beta_kind, void *y, int64_t incy, const char *routine);

}  // namespace mw
