/*
 * mwblas_gb300.h — C ABI of libmwblas_gb300.so, a double-double ("mw") BLAS
 * for one NVIDIA GB300 (sm_103a).
 *
 * Drop-in boundary. Every routine below exports the same Fortran-style
 * by-reference symbols as the reference library epblas-parallel::mwblas:
 * an LP64 `name_` taking `int *` sizes and an ILP64 `name_64_` taking
 * `int64_t *` sizes, generated in the reference by EPBLAS_FACADE_PAIR
 * (src/epblas-parallel/common/epblas_facade.h:63-65). As in the reference:
 *   - hidden Fortran string-length arguments are NOT declared
 *     (epblas_facade.h:24-35);
 *   - flag characters are case-insensitive; real routines fold 'C' to 'T'
 *     (common/blas_char.h:33-39);
 *   - arrays are column-major with leading dimensions, owned by the caller;
 *   - every call returns with its outputs complete (synchronous BLAS).
 * Arrays may be host memory (staged through device memory by the library) or
 * device/managed memory (used in place, no copies).
 *
 * Differences from the reference, which has no argument checking at all
 * (invalid arguments are undefined behaviour there): invalid leading
 * dimensions, flags or unreachable memory are reported through
 * mwblas_last_error() and the optional error hook, and the outputs are left
 * untouched. Sizes <= 0 are quick returns exactly as in the reference.
 *
 * The element types are layout-compatible with the reference's
 * multifloats::float64x2 / complex64x2 (mgemm_parallel.cpp:20-22).
 */
#ifndef MWBLAS_GB300_H
#define MWBLAS_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* double-double: value = limbs[0] + limbs[1], |limbs[1]| <= ulp(limbs[0])/2 */
typedef struct { double limbs[2]; } mwblas_real64x2;
/* complex double-double */
typedef struct { mwblas_real64x2 re, im; } mwblas_complex64x2;

#define MWBLAS_R mwblas_real64x2
#define MWBLAS_C mwblas_complex64x2

/* ======================= Level 3 ======================================= */

/* C := alpha*op(A)*op(B) + beta*C.  Replaces mgemm_/mgemm_64_
 * (multifloats/mgemm_parallel.cpp:44-191, facade epblas_facade.h:234-240). */
void mgemm_(const char *transa, const char *transb, const int *m, const int *n,
            const int *k, const MWBLAS_R *alpha, const MWBLAS_R *a, const int *lda,
            const MWBLAS_R *b, const int *ldb, const MWBLAS_R *beta, MWBLAS_R *c,
            const int *ldc);
void mgemm_64_(const char *transa, const char *transb, const int64_t *m,
               const int64_t *n, const int64_t *k, const MWBLAS_R *alpha,
               const MWBLAS_R *a, const int64_t *lda, const MWBLAS_R *b,
               const int64_t *ldb, const MWBLAS_R *beta, MWBLAS_R *c,
               const int64_t *ldc);

/* Complex C := alpha*op(A)*op(B) + beta*C, op in {N,T,C}.  Replaces
 * wgemm_/wgemm_64_ (multifloats/wgemm_parallel.cpp:44-200). */
void wgemm_(const char *transa, const char *transb, const int *m, const int *n,
            const int *k, const MWBLAS_C *alpha, const MWBLAS_C *a, const int *lda,
            const MWBLAS_C *b, const int *ldb, const MWBLAS_C *beta, MWBLAS_C *c,
            const int *ldc);
void wgemm_64_(const char *transa, const char *transb, const int64_t *m,
               const int64_t *n, const int64_t *k, const MWBLAS_C *alpha,
               const MWBLAS_C *a, const int64_t *lda, const MWBLAS_C *b,
               const int64_t *ldb, const MWBLAS_C *beta, MWBLAS_C *c,
               const int64_t *ldc);

/* C := alpha*A*A**T + beta*C (trans='N') or alpha*A**T*A + beta*C, on the
 * uplo triangle only.  Replaces msyrk_/msyrk_64_
 * (multifloats/msyrk_parallel.cpp:36-90, facade epblas_facade.h:259-265). */
void msyrk_(const char *uplo, const char *trans, const int *n, const int *k,
            const MWBLAS_R *alpha, const MWBLAS_R *a, const int *lda,
            const MWBLAS_R *beta, MWBLAS_R *c, const int *ldc);
void msyrk_64_(const char *uplo, const char *trans, const int64_t *n,
               const int64_t *k, const MWBLAS_R *alpha, const MWBLAS_R *a,
               const int64_t *lda, const MWBLAS_R *beta, MWBLAS_R *c,
               const int64_t *ldc);

/* Hermitian rank-k update with real alpha/beta; the imaginary part of the
 * diagonal is set to zero.  Replaces wherk_/wherk_64_
 * (multifloats/wherk_parallel.cpp:40-88, wherk_serial.cpp:369-405). */
void wherk_(const char *uplo, const char *trans, const int *n, const int *k,
            const MWBLAS_R *alpha, const MWBLAS_C *a, const int *lda,
            const MWBLAS_R *beta, MWBLAS_C *c, const int *ldc);
void wherk_64_(const char *uplo, const char *trans, const int64_t *n,
               const int64_t *k, const MWBLAS_R *alpha, const MWBLAS_C *a,
               const int64_t *lda, const MWBLAS_R *beta, MWBLAS_C *c,
               const int64_t *ldc);

/* C := alpha*op(A)*op(B) + beta*C on the uplo triangle of the n x n C.
 * Replaces mgemmtr_/mgemmtr_64_ and wgemmtr_/wgemmtr_64_
 * (multifloats/mgemmtr_parallel.cpp:35-82, wgemmtr_parallel.cpp:40-85,
 * facade epblas_facade.h:242-247). */
void mgemmtr_(const char *uplo, const char *transa, const char *transb, const int *n, const int *k,
              const MWBLAS_R *alpha, const MWBLAS_R *a, const int *lda, const MWBLAS_R *b, const int *ldb,
              const MWBLAS_R *beta, MWBLAS_R *c, const int *ldc);
void mgemmtr_64_(const char *uplo, const char *transa, const char *transb, const int64_t *n, const int64_t *k,
                 const MWBLAS_R *alpha, const MWBLAS_R *a, const int64_t *lda, const MWBLAS_R *b,
                 const int64_t *ldb, const MWBLAS_R *beta, MWBLAS_R *c, const int64_t *ldc);
void wgemmtr_(const char *uplo, const char *transa, const char *transb, const int *n, const int *k,
              const MWBLAS_C *alpha, const MWBLAS_C *a, const int *lda, const MWBLAS_C *b, const int *ldb,
              const MWBLAS_C *beta, MWBLAS_C *c, const int *ldc);
void wgemmtr_64_(const char *uplo, const char *transa, const char *transb, const int64_t *n, const int64_t *k,
                 const MWBLAS_C *alpha, const MWBLAS_C *a, const int64_t *lda, const MWBLAS_C *b,
                 const int64_t *ldb, const MWBLAS_C *beta, MWBLAS_C *c, const int64_t *ldc);

/* C := alpha*A*B + beta*C (side='L') or alpha*B*A + beta*C (side='R'), A
 * symmetric (msymm_, wsymm_) or Hermitian with a real diagonal (whemm_),
 * read from its uplo triangle.  Replaces msymm_/wsymm_/whemm_ and the _64_
 * twins (multifloats/msymm_parallel.cpp:37-104, wsymm_parallel.cpp:40-105,
 * whemm_parallel.cpp:40-104, whemm_serial.cpp:11-12, facade
 * epblas_facade.h:250-255). */
void msymm_(const char *side, const char *uplo, const int *m, const int *n, const MWBLAS_R *alpha,
            const MWBLAS_R *a, const int *lda, const MWBLAS_R *b, const int *ldb, const MWBLAS_R *beta,
            MWBLAS_R *c, const int *ldc);
void msymm_64_(const char *side, const char *uplo, const int64_t *m, const int64_t *n, const MWBLAS_R *alpha,
               const MWBLAS_R *a, const int64_t *lda, const MWBLAS_R *b, const int64_t *ldb,
               const MWBLAS_R *beta, MWBLAS_R *c, const int64_t *ldc);
void wsymm_(const char *side, const char *uplo, const int *m, const int *n, const MWBLAS_C *alpha,
            const MWBLAS_C *a, const int *lda, const MWBLAS_C *b, const int *ldb, const MWBLAS_C *beta,
            MWBLAS_C *c, const int *ldc);
void wsymm_64_(const char *side, const char *uplo, const int64_t *m, const int64_t *n, const MWBLAS_C *alpha,
               const MWBLAS_C *a, const int64_t *lda, const MWBLAS_C *b, const int64_t *ldb,
               const MWBLAS_C *beta, MWBLAS_C *c, const int64_t *ldc);
void whemm_(const char *side, const char *uplo, const int *m, const int *n, const MWBLAS_C *alpha,
            const MWBLAS_C *a, const int *lda, const MWBLAS_C *b, const int *ldb, const MWBLAS_C *beta,
            MWBLAS_C *c, const int *ldc);
void whemm_64_(const char *side, const char *uplo, const int64_t *m, const int64_t *n, const MWBLAS_C *alpha,
               const MWBLAS_C *a, const int64_t *lda, const MWBLAS_C *b, const int64_t *ldb,
               const MWBLAS_C *beta, MWBLAS_C *c, const int64_t *ldc);

/* Rank-2k updates on the uplo triangle: C := alpha*A*B**T + alpha*B*A**T +
 * beta*C (trans='N') or alpha*A**T*B + alpha*B**T*A + beta*C (msyr2k_,
 * wsyr2k_); wher2k_ uses A**H, conj(alpha) on the second product, a real beta
 * and keeps the diagonal real.  Replaces msyr2k_/wsyr2k_/wher2k_ and the
 * _64_ twins (multifloats/msyr2k_parallel.cpp:38-85,
 * wsyr2k_parallel.cpp:40-86, wher2k_parallel.cpp:40-91, facade
 * epblas_facade.h:268-273). */
void msyr2k_(const char *uplo, const char *trans, const int *n, const int *k, const MWBLAS_R *alpha,
             const MWBLAS_R *a, const int *lda, const MWBLAS_R *b, const int *ldb, const MWBLAS_R *beta,
             MWBLAS_R *c, const int *ldc);
void msyr2k_64_(const char *uplo, const char *trans, const int64_t *n, const int64_t *k, const MWBLAS_R *alpha,
                const MWBLAS_R *a, const int64_t *lda, const MWBLAS_R *b, const int64_t *ldb,
                const MWBLAS_R *beta, MWBLAS_R *c, const int64_t *ldc);
void wsyr2k_(const char *uplo, const char *trans, const int *n, const int *k, const MWBLAS_C *alpha,
             const MWBLAS_C *a, const int *lda, const MWBLAS_C *b, const int *ldb, const MWBLAS_C *beta,
             MWBLAS_C *c, const int *ldc);
void wsyr2k_64_(const char *uplo, const char *trans, const int64_t *n, const int64_t *k, const MWBLAS_C *alpha,
                const MWBLAS_C *a, const int64_t *lda, const MWBLAS_C *b, const int64_t *ldb,
                const MWBLAS_C *beta, MWBLAS_C *c, const int64_t *ldc);
void wher2k_(const char *uplo, const char *trans, const int *n, const int *k, const MWBLAS_C *alpha,
             const MWBLAS_C *a, const int *lda, const MWBLAS_C *b, const int *ldb, const MWBLAS_R *beta,
             MWBLAS_C *c, const int *ldc);
void wher2k_64_(const char *uplo, const char *trans, const int64_t *n, const int64_t *k, const MWBLAS_C *alpha,
                const MWBLAS_C *a, const int64_t *lda, const MWBLAS_C *b, const int64_t *ldb,
                const MWBLAS_R *beta, MWBLAS_C *c, const int64_t *ldc);

/* Complex symmetric (not Hermitian) rank-k update with complex alpha/beta:
 * C := alpha*A*A**T + beta*C (trans='N') or alpha*A**T*A + beta*C, uplo
 * triangle.  Replaces wsyrk_/wsyrk_64_ (multifloats/wsyrk_parallel.cpp:40-86,
 * facade epblas_facade.h:259-265). */
void wsyrk_(const char *uplo, const char *trans, const int *n, const int *k, const MWBLAS_C *alpha,
            const MWBLAS_C *a, const int *lda, const MWBLAS_C *beta, MWBLAS_C *c, const int *ldc);
void wsyrk_64_(const char *uplo, const char *trans, const int64_t *n, const int64_t *k, const MWBLAS_C *alpha,
               const MWBLAS_C *a, const int64_t *lda, const MWBLAS_C *beta, MWBLAS_C *c, const int64_t *ldc);

/* Triangular multiply B := alpha*op(A)*B (side='L') or alpha*B*op(A)
 * (side='R'), B overwritten.  Replaces mtrmm_/wtrmm_ and the _64_ twins
 * (multifloats/mtrmm_parallel.cpp:37-108, wtrmm_parallel.cpp:40-110, facade
 * epblas_facade.h:276-282). */
void mtrmm_(const char *side, const char *uplo, const char *transa, const char *diag, const int *m, const int *n,
            const MWBLAS_R *alpha, const MWBLAS_R *a, const int *lda, MWBLAS_R *b, const int *ldb);
void mtrmm_64_(const char *side, const char *uplo, const char *transa, const char *diag, const int64_t *m,
               const int64_t *n, const MWBLAS_R *alpha, const MWBLAS_R *a, const int64_t *lda, MWBLAS_R *b,
               const int64_t *ldb);
void wtrmm_(const char *side, const char *uplo, const char *transa, const char *diag, const int *m, const int *n,
            const MWBLAS_C *alpha, const MWBLAS_C *a, const int *lda, MWBLAS_C *b, const int *ldb);
void wtrmm_64_(const char *side, const char *uplo, const char *transa, const char *diag, const int64_t *m,
               const int64_t *n, const MWBLAS_C *alpha, const MWBLAS_C *a, const int64_t *lda, MWBLAS_C *b,
               const int64_t *ldb);

/* Complex triangular solve op(A)*X = alpha*B (side='L') or X*op(A) = alpha*B
 * (side='R'), op in {N, T, C}; B is overwritten by X.  Replaces
 * wtrsm_/wtrsm_64_ (multifloats/wtrsm_parallel.cpp:39-105, facade
 * epblas_facade.h:276-282). */
void wtrsm_(const char *side, const char *uplo, const char *transa, const char *diag, const int *m, const int *n,
            const MWBLAS_C *alpha, const MWBLAS_C *a, const int *lda, MWBLAS_C *b, const int *ldb);
void wtrsm_64_(const char *side, const char *uplo, const char *transa, const char *diag, const int64_t *m,
               const int64_t *n, const MWBLAS_C *alpha, const MWBLAS_C *a, const int64_t *lda, MWBLAS_C *b,
               const int64_t *ldb);

/* Triangular solve op(A)*X = alpha*B (side='L') or X*op(A) = alpha*B
 * (side='R'); B is overwritten by X.  Replaces mtrsm_/mtrsm_64_
 * (multifloats/mtrsm_parallel.cpp:36-105, facade epblas_facade.h:276-282). */
void mtrsm_(const char *side, const char *uplo, const char *transa, const char *diag,
            const int *m, const int *n, const MWBLAS_R *alpha, const MWBLAS_R *a,
            const int *lda, MWBLAS_R *b, const int *ldb);
void mtrsm_64_(const char *side, const char *uplo, const char *transa,
               const char *diag, const int64_t *m, const int64_t *n,
               const MWBLAS_R *alpha, const MWBLAS_R *a, const int64_t *lda,
               MWBLAS_R *b, const int64_t *ldb);

/* ======================= Level 2 ======================================= */

/* y := alpha*op(A)*x + beta*y.  Replaces mgemv_/mgemv_64_
 * (multifloats/mgemv.cpp:237-280, facade epblas_facade.h:132-138). */
void mgemv_(const char *trans, const int *m, const int *n, const MWBLAS_R *alpha,
            const MWBLAS_R *a, const int *lda, const MWBLAS_R *x, const int *incx,
            const MWBLAS_R *beta, MWBLAS_R *y, const int *incy);
void mgemv_64_(const char *trans, const int64_t *m, const int64_t *n,
               const MWBLAS_R *alpha, const MWBLAS_R *a, const int64_t *lda,
               const MWBLAS_R *x, const int64_t *incx, const MWBLAS_R *beta,
               MWBLAS_R *y, const int64_t *incy);

/* ======================= Level 2 (beyond mgemv_) ========================
 * Matrix-vector products, solves and rank updates with dense, band (LAPACK
 * band layout) or packed operands, real and complex; vectors take any
 * non-zero increment.  Replace the reference's routines of the same names and
 * their _64_ twins (facade epblas_facade.h:132-223). */

/* y := alpha*op(A)*x + beta*y, complex A (multifloats/wgemv.cpp), banded A
 * (mgbmv.cpp, wgbmv.cpp). */
void wgemv_(const char *trans, const int *m, const int *n, const MWBLAS_C *alpha, const MWBLAS_C *a, const int *lda, const MWBLAS_C *x, const int *incx, const MWBLAS_C *beta, MWBLAS_C *y, const int *incy);
void wgemv_64_(const char *trans, const int64_t *m, const int64_t *n, const MWBLAS_C *alpha, const MWBLAS_C *a, const int64_t *lda, const MWBLAS_C *x, const int64_t *incx, const MWBLAS_C *beta, MWBLAS_C *y, const int64_t *incy);
void mgbmv_(const char *trans, const int *m, const int *n, const int *kl, const int *ku, const MWBLAS_R *alpha, const MWBLAS_R *a, const int *lda, const MWBLAS_R *x, const int *incx, const MWBLAS_R *beta, MWBLAS_R *y, const int *incy);
void mgbmv_64_(const char *trans, const int64_t *m, const int64_t *n, const int64_t *kl, const int64_t *ku, const MWBLAS_R *alpha, const MWBLAS_R *a, const int64_t *lda, const MWBLAS_R *x, const int64_t *incx, const MWBLAS_R *beta, MWBLAS_R *y, const int64_t *incy);
void wgbmv_(const char *trans, const int *m, const int *n, const int *kl, const int *ku, const MWBLAS_C *alpha, const MWBLAS_C *a, const int *lda, const MWBLAS_C *x, const int *incx, const MWBLAS_C *beta, MWBLAS_C *y, const int *incy);
void wgbmv_64_(const char *trans, const int64_t *m, const int64_t *n, const int64_t *kl, const int64_t *ku, const MWBLAS_C *alpha, const MWBLAS_C *a, const int64_t *lda, const MWBLAS_C *x, const int64_t *incx, const MWBLAS_C *beta, MWBLAS_C *y, const int64_t *incy);

/* y := alpha*A*x + beta*y with A symmetric / Hermitian: dense (msymv.cpp,
 * whemv.cpp), band (msbmv.cpp, whbmv.cpp), packed (mspmv.cpp, whpmv.cpp). */
void msymv_(const char *uplo, const int *n, const MWBLAS_R *alpha, const MWBLAS_R *a, const int *lda, const MWBLAS_R *x, const int *incx, const MWBLAS_R *beta, MWBLAS_R *y, const int *incy);
void msymv_64_(const char *uplo, const int64_t *n, const MWBLAS_R *alpha, const MWBLAS_R *a, const int64_t *lda, const MWBLAS_R *x, const int64_t *incx, const MWBLAS_R *beta, MWBLAS_R *y, const int64_t *incy);
void whemv_(const char *uplo, const int *n, const MWBLAS_C *alpha, const MWBLAS_C *a, const int *lda, const MWBLAS_C *x, const int *incx, const MWBLAS_C *beta, MWBLAS_C *y, const int *incy);
void whemv_64_(const char *uplo, const int64_t *n, const MWBLAS_C *alpha, const MWBLAS_C *a, const int64_t *lda, const MWBLAS_C *x, const int64_t *incx, const MWBLAS_C *beta, MWBLAS_C *y, const int64_t *incy);
void msbmv_(const char *uplo, const int *n, const int *k, const MWBLAS_R *alpha, const MWBLAS_R *a, const int *lda, const MWBLAS_R *x, const int *incx, const MWBLAS_R *beta, MWBLAS_R *y, const int *incy);
void msbmv_64_(const char *uplo, const int64_t *n, const int64_t *k, const MWBLAS_R *alpha, const MWBLAS_R *a, const int64_t *lda, const MWBLAS_R *x, const int64_t *incx, const MWBLAS_R *beta, MWBLAS_R *y, const int64_t *incy);
void whbmv_(const char *uplo, const int *n, const int *k, const MWBLAS_C *alpha, const MWBLAS_C *a, const int *lda, const MWBLAS_C *x, const int *incx, const MWBLAS_C *beta, MWBLAS_C *y, const int *incy);
void whbmv_64_(const char *uplo, const int64_t *n, const int64_t *k, const MWBLAS_C *alpha, const MWBLAS_C *a, const int64_t *lda, const MWBLAS_C *x, const int64_t *incx, const MWBLAS_C *beta, MWBLAS_C *y, const int64_t *incy);
void mspmv_(const char *uplo, const int *n, const MWBLAS_R *alpha, const MWBLAS_R *ap, const MWBLAS_R *x, const int *incx, const MWBLAS_R *beta, MWBLAS_R *y, const int *incy);
void mspmv_64_(const char *uplo, const int64_t *n, const MWBLAS_R *alpha, const MWBLAS_R *ap, const MWBLAS_R *x, const int64_t *incx, const MWBLAS_R *beta, MWBLAS_R *y, const int64_t *incy);
void whpmv_(const char *uplo, const int *n, const MWBLAS_C *alpha, const MWBLAS_C *ap, const MWBLAS_C *x, const int *incx, const MWBLAS_C *beta, MWBLAS_C *y, const int *incy);
void whpmv_64_(const char *uplo, const int64_t *n, const MWBLAS_C *alpha, const MWBLAS_C *ap, const MWBLAS_C *x, const int64_t *incx, const MWBLAS_C *beta, MWBLAS_C *y, const int64_t *incy);

/* x := op(A)*x and x := op(A)^-1*x with A triangular: dense (mtrmv.cpp,
 * mtrsv.cpp, wtrmv.cpp, wtrsv.cpp), band (mtbmv.cpp, mtbsv.cpp, ...), packed
 * (mtpmv.cpp, mtpsv.cpp, ...). */
void mtrmv_(const char *uplo, const char *trans, const char *diag, const int *n, const MWBLAS_R *a, const int *lda, MWBLAS_R *x, const int *incx);
void mtrmv_64_(const char *uplo, const char *trans, const char *diag, const int64_t *n, const MWBLAS_R *a, const int64_t *lda, MWBLAS_R *x, const int64_t *incx);
void wtrmv_(const char *uplo, const char *trans, const char *diag, const int *n, const MWBLAS_C *a, const int *lda, MWBLAS_C *x, const int *incx);
void wtrmv_64_(const char *uplo, const char *trans, const char *diag, const int64_t *n, const MWBLAS_C *a, const int64_t *lda, MWBLAS_C *x, const int64_t *incx);
void mtrsv_(const char *uplo, const char *trans, const char *diag, const int *n, const MWBLAS_R *a, const int *lda, MWBLAS_R *x, const int *incx);
void mtrsv_64_(const char *uplo, const char *trans, const char *diag, const int64_t *n, const MWBLAS_R *a, const int64_t *lda, MWBLAS_R *x, const int64_t *incx);
void wtrsv_(const char *uplo, const char *trans, const char *diag, const int *n, const MWBLAS_C *a, const int *lda, MWBLAS_C *x, const int *incx);
void wtrsv_64_(const char *uplo, const char *trans, const char *diag, const int64_t *n, const MWBLAS_C *a, const int64_t *lda, MWBLAS_C *x, const int64_t *incx);
void mtbmv_(const char *uplo, const char *trans, const char *diag, const int *n, const int *k, const MWBLAS_R *a, const int *lda, MWBLAS_R *x, const int *incx);
void mtbmv_64_(const char *uplo, const char *trans, const char *diag, const int64_t *n, const int64_t *k, const MWBLAS_R *a, const int64_t *lda, MWBLAS_R *x, const int64_t *incx);
void wtbmv_(const char *uplo, const char *trans, const char *diag, const int *n, const int *k, const MWBLAS_C *a, const int *lda, MWBLAS_C *x, const int *incx);
void wtbmv_64_(const char *uplo, const char *trans, const char *diag, const int64_t *n, const int64_t *k, const MWBLAS_C *a, const int64_t *lda, MWBLAS_C *x, const int64_t *incx);
void mtbsv_(const char *uplo, const char *trans, const char *diag, const int *n, const int *k, const MWBLAS_R *a, const int *lda, MWBLAS_R *x, const int *incx);
void mtbsv_64_(const char *uplo, const char *trans, const char *diag, const int64_t *n, const int64_t *k, const MWBLAS_R *a, const int64_t *lda, MWBLAS_R *x, const int64_t *incx);
void wtbsv_(const char *uplo, const char *trans, const char *diag, const int *n, const int *k, const MWBLAS_C *a, const int *lda, MWBLAS_C *x, const int *incx);
void wtbsv_64_(const char *uplo, const char *trans, const char *diag, const int64_t *n, const int64_t *k, const MWBLAS_C *a, const int64_t *lda, MWBLAS_C *x, const int64_t *incx);
void mtpmv_(const char *uplo, const char *trans, const char *diag, const int *n, const MWBLAS_R *ap, MWBLAS_R *x, const int *incx);
void mtpmv_64_(const char *uplo, const char *trans, const char *diag, const int64_t *n, const MWBLAS_R *ap, MWBLAS_R *x, const int64_t *incx);
void wtpmv_(const char *uplo, const char *trans, const char *diag, const int *n, const MWBLAS_C *ap, MWBLAS_C *x, const int *incx);
void wtpmv_64_(const char *uplo, const char *trans, const char *diag, const int64_t *n, const MWBLAS_C *ap, MWBLAS_C *x, const int64_t *incx);
void mtpsv_(const char *uplo, const char *trans, const char *diag, const int *n, const MWBLAS_R *ap, MWBLAS_R *x, const int *incx);
void mtpsv_64_(const char *uplo, const char *trans, const char *diag, const int64_t *n, const MWBLAS_R *ap, MWBLAS_R *x, const int64_t *incx);
void wtpsv_(const char *uplo, const char *trans, const char *diag, const int *n, const MWBLAS_C *ap, MWBLAS_C *x, const int *incx);
void wtpsv_64_(const char *uplo, const char *trans, const char *diag, const int64_t *n, const MWBLAS_C *ap, MWBLAS_C *x, const int64_t *incx);

/* Rank-1/2 updates: A := alpha*x*y**T (+A) (mger.cpp; wgeru.cpp, wgerc.cpp
 * with y**H), A := alpha*x*x**T(**H) + A on a triangle (msyr.cpp, wher.cpp
 * with real alpha; packed mspr.cpp, whpr.cpp), A := alpha*x*y**T +
 * alpha*y*x**T + A (msyr2.cpp; wher2.cpp with conj(alpha); packed mspr2.cpp,
 * whpr2.cpp). */
void mger_(const int *m, const int *n, const MWBLAS_R *alpha, const MWBLAS_R *x, const int *incx, const MWBLAS_R *y, const int *incy, MWBLAS_R *a, const int *lda);
void mger_64_(const int64_t *m, const int64_t *n, const MWBLAS_R *alpha, const MWBLAS_R *x, const int64_t *incx, const MWBLAS_R *y, const int64_t *incy, MWBLAS_R *a, const int64_t *lda);
void wgeru_(const int *m, const int *n, const MWBLAS_C *alpha, const MWBLAS_C *x, const int *incx, const MWBLAS_C *y, const int *incy, MWBLAS_C *a, const int *lda);
void wgeru_64_(const int64_t *m, const int64_t *n, const MWBLAS_C *alpha, const MWBLAS_C *x, const int64_t *incx, const MWBLAS_C *y, const int64_t *incy, MWBLAS_C *a, const int64_t *lda);
void wgerc_(const int *m, const int *n, const MWBLAS_C *alpha, const MWBLAS_C *x, const int *incx, const MWBLAS_C *y, const int *incy, MWBLAS_C *a, const int *lda);
void wgerc_64_(const int64_t *m, const int64_t *n, const MWBLAS_C *alpha, const MWBLAS_C *x, const int64_t *incx, const MWBLAS_C *y, const int64_t *incy, MWBLAS_C *a, const int64_t *lda);
void msyr_(const char *uplo, const int *n, const MWBLAS_R *alpha, const MWBLAS_R *x, const int *incx, MWBLAS_R *a, const int *lda);
void msyr_64_(const char *uplo, const int64_t *n, const MWBLAS_R *alpha, const MWBLAS_R *x, const int64_t *incx, MWBLAS_R *a, const int64_t *lda);
void wher_(const char *uplo, const int *n, const MWBLAS_R *alpha, const MWBLAS_C *x, const int *incx, MWBLAS_C *a, const int *lda);
void wher_64_(const char *uplo, const int64_t *n, const MWBLAS_R *alpha, const MWBLAS_C *x, const int64_t *incx, MWBLAS_C *a, const int64_t *lda);
void mspr_(const char *uplo, const int *n, const MWBLAS_R *alpha, const MWBLAS_R *x, const int *incx, MWBLAS_R *ap);
void mspr_64_(const char *uplo, const int64_t *n, const MWBLAS_R *alpha, const MWBLAS_R *x, const int64_t *incx, MWBLAS_R *ap);
void whpr_(const char *uplo, const int *n, const MWBLAS_R *alpha, const MWBLAS_C *x, const int *incx, MWBLAS_C *ap);
void whpr_64_(const char *uplo, const int64_t *n, const MWBLAS_R *alpha, const MWBLAS_C *x, const int64_t *incx, MWBLAS_C *ap);
void msyr2_(const char *uplo, const int *n, const MWBLAS_R *alpha, const MWBLAS_R *x, const int *incx, const MWBLAS_R *y, const int *incy, MWBLAS_R *a, const int *lda);
void msyr2_64_(const char *uplo, const int64_t *n, const MWBLAS_R *alpha, const MWBLAS_R *x, const int64_t *incx, const MWBLAS_R *y, const int64_t *incy, MWBLAS_R *a, const int64_t *lda);
void wher2_(const char *uplo, const int *n, const MWBLAS_C *alpha, const MWBLAS_C *x, const int *incx, const MWBLAS_C *y, const int *incy, MWBLAS_C *a, const int *lda);
void wher2_64_(const char *uplo, const int64_t *n, const MWBLAS_C *alpha, const MWBLAS_C *x, const int64_t *incx, const MWBLAS_C *y, const int64_t *incy, MWBLAS_C *a, const int64_t *lda);
void mspr2_(const char *uplo, const int *n, const MWBLAS_R *alpha, const MWBLAS_R *x, const int *incx, const MWBLAS_R *y, const int *incy, MWBLAS_R *ap);
void mspr2_64_(const char *uplo, const int64_t *n, const MWBLAS_R *alpha, const MWBLAS_R *x, const int64_t *incx, const MWBLAS_R *y, const int64_t *incy, MWBLAS_R *ap);
void whpr2_(const char *uplo, const int *n, const MWBLAS_C *alpha, const MWBLAS_C *x, const int *incx, const MWBLAS_C *y, const int *incy, MWBLAS_C *ap);
void whpr2_64_(const char *uplo, const int64_t *n, const MWBLAS_C *alpha, const MWBLAS_C *x, const int64_t *incx, const MWBLAS_C *y, const int64_t *incy, MWBLAS_C *ap);

/* ======================= Level 1 ======================================= */

/* Complex dots sum x(i)*y(i) (wdotu_) and sum conj(x(i))*y(i) (wdotc_), the
 * complex result returned by value.  Replaces wdotu_/wdotc_ and the _64_
 * twins (multifloats/wdotu.cpp:121-140, wdotc.cpp:121-140, facade
 * epblas_facade.h:102-107). */
MWBLAS_C wdotu_(const int *n, const MWBLAS_C *x, const int *incx, const MWBLAS_C *y, const int *incy);
MWBLAS_C wdotu_64_(const int64_t *n, const MWBLAS_C *x, const int64_t *incx, const MWBLAS_C *y,
                   const int64_t *incy);
MWBLAS_C wdotc_(const int *n, const MWBLAS_C *x, const int *incx, const MWBLAS_C *y, const int *incy);
MWBLAS_C wdotc_64_(const int64_t *n, const MWBLAS_C *x, const int64_t *incx, const MWBLAS_C *y,
                   const int64_t *incy);

/* sum |x(i)| (masum_), sum |Re x(i)| + |Im x(i)| (mwasum_), and the Euclidean
 * norms (mnrm2_, mwnrm2_); 0 for n < 1 or incx < 1.  Replaces masum_,
 * mwasum_, mnrm2_, mwnrm2_ and the _64_ twins (multifloats/masum.cpp:115-127,
 * mwasum.cpp:116-128, mnrm2.cpp:178-195, mwnrm2.cpp:176-192, facade
 * epblas_facade.h:76-79). */
MWBLAS_R masum_(const int *n, const MWBLAS_R *x, const int *incx);
MWBLAS_R masum_64_(const int64_t *n, const MWBLAS_R *x, const int64_t *incx);
MWBLAS_R mwasum_(const int *n, const MWBLAS_C *x, const int *incx);
MWBLAS_R mwasum_64_(const int64_t *n, const MWBLAS_C *x, const int64_t *incx);
MWBLAS_R mnrm2_(const int *n, const MWBLAS_R *x, const int *incx);
MWBLAS_R mnrm2_64_(const int64_t *n, const MWBLAS_R *x, const int64_t *incx);
MWBLAS_R mwnrm2_(const int *n, const MWBLAS_C *x, const int *incx);
MWBLAS_R mwnrm2_64_(const int64_t *n, const MWBLAS_C *x, const int64_t *incx);

/* y := alpha*x + y, complex.  Replaces waxpy_/waxpy_64_
 * (multifloats/waxpy.cpp:97-110, facade epblas_facade.h:81-86). */
void waxpy_(const int *n, const MWBLAS_C *alpha, const MWBLAS_C *x, const int *incx, MWBLAS_C *y, const int *incy);
void waxpy_64_(const int64_t *n, const MWBLAS_C *alpha, const MWBLAS_C *x, const int64_t *incx, MWBLAS_C *y,
               const int64_t *incy);

/* Plane rotation (x, y) := (c*x + s*y, c*y - s*x) with real c, s, for real
 * (mrot_) and complex (wmrot_) vectors; mrotm_ applies the modified-Givens
 * matrix of dparam (flag, h11, h21, h12, h22).  Replaces mrot_, wmrot_,
 * mrotm_ and the _64_ twins (multifloats/mrot.cpp:102-115,
 * wmrot.cpp:119-132, mrotm.cpp:196-215, facade epblas_facade.h:109-121). */
void mrot_(const int *n, MWBLAS_R *x, const int *incx, MWBLAS_R *y, const int *incy, const MWBLAS_R *c,
           const MWBLAS_R *s);
void mrot_64_(const int64_t *n, MWBLAS_R *x, const int64_t *incx, MWBLAS_R *y, const int64_t *incy,
              const MWBLAS_R *c, const MWBLAS_R *s);
void wmrot_(const int *n, MWBLAS_C *x, const int *incx, MWBLAS_C *y, const int *incy, const MWBLAS_R *c,
            const MWBLAS_R *s);
void wmrot_64_(const int64_t *n, MWBLAS_C *x, const int64_t *incx, MWBLAS_C *y, const int64_t *incy,
               const MWBLAS_R *c, const MWBLAS_R *s);
void mrotm_(const int *n, MWBLAS_R *x, const int *incx, MWBLAS_R *y, const int *incy, const MWBLAS_R *dparam);
void mrotm_64_(const int64_t *n, MWBLAS_R *x, const int64_t *incx, MWBLAS_R *y, const int64_t *incy,
               const MWBLAS_R *dparam);

/* Scalar generators, computed by one device thread in double-double.
 * mcabs1_: |Re z| + |Im z| (multifloats/mcabs1.cpp:20-25).
 * mrotg_: Givens rotation of (a, b); on return a = r, b = z
 *   (multifloats/mrotg.cpp:21-35).
 * mrotmg_: modified Givens (DROTMG); updates d1, d2, x1 and the dparam
 *   entries the flag uses (multifloats/mrotmg.cpp:25-110).
 * wrotg_: complex Givens; a := r, real c, complex s (multifloats/wrotg.cpp:27-52).
 * The arguments are host variables.  No integer arguments, so each _64_ twin
 * has the same signature. */
MWBLAS_R mcabs1_(const MWBLAS_C *z);
MWBLAS_R mcabs1_64_(const MWBLAS_C *z);
void mrotg_(MWBLAS_R *a, MWBLAS_R *b, MWBLAS_R *c, MWBLAS_R *s);
void mrotg_64_(MWBLAS_R *a, MWBLAS_R *b, MWBLAS_R *c, MWBLAS_R *s);
void mrotmg_(MWBLAS_R *d1, MWBLAS_R *d2, MWBLAS_R *x1, const MWBLAS_R *y1, MWBLAS_R *dparam);
void mrotmg_64_(MWBLAS_R *d1, MWBLAS_R *d2, MWBLAS_R *x1, const MWBLAS_R *y1, MWBLAS_R *dparam);
void wrotg_(MWBLAS_C *a, const MWBLAS_C *b, MWBLAS_R *c, MWBLAS_C *s);
void wrotg_64_(MWBLAS_C *a, const MWBLAS_C *b, MWBLAS_R *c, MWBLAS_C *s);

/* sum x(i)*y(i).  Replaces mdot_/mdot_64_ (multifloats/mdot.cpp:127-148). */
MWBLAS_R mdot_(const int *n, const MWBLAS_R *x, const int *incx, const MWBLAS_R *y,
               const int *incy);
MWBLAS_R mdot_64_(const int64_t *n, const MWBLAS_R *x, const int64_t *incx,
                  const MWBLAS_R *y, const int64_t *incy);

/* y := alpha*x + y, bit-exact to the reference (multifloats/maxpy.cpp:42-113). */
void maxpy_(const int *n, const MWBLAS_R *alpha, const MWBLAS_R *x, const int *incx,
            MWBLAS_R *y, const int *incy);
void maxpy_64_(const int64_t *n, const MWBLAS_R *alpha, const MWBLAS_R *x,
               const int64_t *incx, MWBLAS_R *y, const int64_t *incy);

/* x := alpha*x, bit-exact to the reference (multifloats/mscal.cpp:42-104). */
void mscal_(const int *n, const MWBLAS_R *alpha, MWBLAS_R *x, const int *incx);
void mscal_64_(const int64_t *n, const MWBLAS_R *alpha, MWBLAS_R *x,
               const int64_t *incx);

/* y := x (multifloats/mcopy.cpp:30-58). */
void mcopy_(const int *n, const MWBLAS_R *x, const int *incx, MWBLAS_R *y,
            const int *incy);
void mcopy_64_(const int64_t *n, const MWBLAS_R *x, const int64_t *incx, MWBLAS_R *y,
               const int64_t *incy);

/* x <-> y (multifloats/mswap.cpp:40-70). */
void mswap_(const int *n, MWBLAS_R *x, const int *incx, MWBLAS_R *y, const int *incy);
void mswap_64_(const int64_t *n, MWBLAS_R *x, const int64_t *incx, MWBLAS_R *y,
               const int64_t *incy);

/* 1-based index of the first element of maximal |x|, lexicographic
 * double-double compare (multifloats/imamax.cpp:178-203). */
int imamax_(const int *n, const MWBLAS_R *x, const int *incx);
int64_t imamax_64_(const int64_t *n, const MWBLAS_R *x, const int64_t *incx);

/* complex x := alpha*x, bit-exact (multifloats/wscal.cpp). */
void wscal_(const int *n, const MWBLAS_C *alpha, MWBLAS_C *x, const int *incx);
void wscal_64_(const int64_t *n, const MWBLAS_C *alpha, MWBLAS_C *x,
               const int64_t *incx);

/* complex x := alpha*x with real alpha, bit-exact (multifloats/wmscal.cpp). */
void wmscal_(const int *n, const MWBLAS_R *alpha, MWBLAS_C *x, const int *incx);
void wmscal_64_(const int64_t *n, const MWBLAS_R *alpha, MWBLAS_C *x,
                const int64_t *incx);

/* complex y := x (multifloats/wcopy.cpp). */
void wcopy_(const int *n, const MWBLAS_C *x, const int *incx, MWBLAS_C *y,
            const int *incy);
void wcopy_64_(const int64_t *n, const MWBLAS_C *x, const int64_t *incx, MWBLAS_C *y,
               const int64_t *incy);

/* complex x <-> y (multifloats/wswap.cpp). */
void wswap_(const int *n, MWBLAS_C *x, const int *incx, MWBLAS_C *y, const int *incy);
void wswap_64_(const int64_t *n, MWBLAS_C *x, const int64_t *incx, MWBLAS_C *y,
               const int64_t *incy);

/* 1-based argmax of |re|+|im| (multifloats/iwamax.cpp:174-200). */
int iwamax_(const int *n, const MWBLAS_C *x, const int *incx);
int64_t iwamax_64_(const int64_t *n, const MWBLAS_C *x, const int64_t *incx);

/* ======================= Extensions (no reference counterpart) ========== */

/* GEMM engine selection for mgemm_/wgemm_ and the level-3 routines built on
 * them.  MWBLAS_GEMM_AUTO picks by size; PLAIN is the FP64 error-free-
 * transform kernel; OZAKI is the integer-exact tensor-core scheme; FIXED is
 * the fixed-point kernel on the integer pipes (real routines; complex ones
 * fall back to PLAIN).  The MWBLAS_GEMM environment variable ("auto",
 * "plain", "ozaki", "fixed") sets the initial value. */
enum { MWBLAS_GEMM_AUTO = 0, MWBLAS_GEMM_PLAIN = 1, MWBLAS_GEMM_OZAKI = 2, MWBLAS_GEMM_FIXED = 3 };
int mwblas_set_gemm_engine(int engine);   /* returns the previous value */
int mwblas_get_gemm_engine(void);

/* Triangular band solves (mtbsv_/wtbsv_): MWBLAS_BAND_SOLVE_AUTO solves in
 * place from the band (O(n k) memory; bandwidth k <= 31: the rows cut into
 * chunks solved in parallel and joined by a k x k carry, wider bands: one
 * warp) when k <= 31 or a dense copy of the triangle would exceed 256 MB, and
 * through a dense copy and the blocked TRSM otherwise; the other two values
 * force one way. */
enum { MWBLAS_BAND_SOLVE_AUTO = 0, MWBLAS_BAND_SOLVE_IN_PLACE = 1, MWBLAS_BAND_SOLVE_DENSE = 2 };
int mwblas_set_band_solve(int mode);   /* returns the previous value */

/* Same arguments as mgemm_64_, forcing one engine. */
void mgemm_plain_64_(const char *transa, const char *transb, const int64_t *m,
                     const int64_t *n, const int64_t *k, const MWBLAS_R *alpha,
                     const MWBLAS_R *a, const int64_t *lda, const MWBLAS_R *b,
                     const int64_t *ldb, const MWBLAS_R *beta, MWBLAS_R *c,
                     const int64_t *ldc);
void mgemm_fixed_64_(const char *transa, const char *transb, const int64_t *m,
                     const int64_t *n, const int64_t *k, const MWBLAS_R *alpha,
                     const MWBLAS_R *a, const int64_t *lda, const MWBLAS_R *b,
                     const int64_t *ldb, const MWBLAS_R *beta, MWBLAS_R *c,
                     const int64_t *ldc);
void mgemm_ozaki_64_(const char *transa, const char *transb, const int64_t *m,
                     const int64_t *n, const int64_t *k, const MWBLAS_R *alpha,
                     const MWBLAS_R *a, const int64_t *lda, const MWBLAS_R *b,
                     const int64_t *ldb, const MWBLAS_R *beta, MWBLAS_R *c,
                     const int64_t *ldc);

/* Batched uneven double-double GEMM (no reference counterpart): for
 * i < count, C[i] := alpha[i]*op(A[i])*op(B[i]) + beta[i]*C[i], with per-instance
 * flags transa[i]/transb[i], sizes and leading dimensions. The matrix pointers
 * must be 16-byte aligned device (or managed) memory; the per-instance arrays
 * are host arrays.
 * One persistent kernel runs every instance, launched from a CUDA graph that is
 * reused while the batch layout is unchanged. Returns 0 or an error code. */
int mgemm_grouped(int64_t count, const char *transa, const char *transb, const int64_t *m, const int64_t *n,
                  const int64_t *k, const MWBLAS_R *alpha, const MWBLAS_R *const *a, const int64_t *lda,
                  const MWBLAS_R *const *b, const int64_t *ldb, const MWBLAS_R *beta, MWBLAS_R *const *c,
                  const int64_t *ldc);
/* Autotuner for mgemm_grouped: times the output tile edge (16, 32, 64) and
 * then the split-K policies on this batch (results go to scratch copies; C is
 * not modified) and keeps the fastest for batches of the same shape class.
 * *chosen = minimum K per split (0 = none); the tile edge is returned by
 * mwblas_grouped_tuned_tile(). */
int mgemm_grouped_tune(int64_t count, const char *transa, const char *transb, const int64_t *m,
                       const int64_t *n, const int64_t *k, const MWBLAS_R *alpha, const MWBLAS_R *const *a,
                       const int64_t *lda, const MWBLAS_R *const *b, const int64_t *ldb, const MWBLAS_R *beta,
                       MWBLAS_R *const *c, const int64_t *ldc, int *chosen);
/* Tile edge (16, 32 or 64) chosen by this thread's most recent
 * mgemm_grouped_tune call (0 before any). No counterpart in the reference. */
int mwblas_grouped_tuned_tile(void);
/* Forces mgemm_grouped's tile edge (16, 32 or 64; anything else = 0 = the
 * tuned or default choice). All give results within the same bound. Returns
 * the previous setting. */
int mwblas_set_grouped_tile(int tile);
/* mgemm_grouped runs instances with m, n >= size and 64 <= k <= 16384 on the
 * tensor cores (Ozaki scheme, full 106-bit width, padded to classes of
 * 256-row/column and 64..512-deep tiles, one residue GEMM per class) and the
 * rest on the integer pipes; 0 = none, -1 = the tuned or default choice
 * (default 128). Returns the previous setting. mwblas_grouped_tuned_tensor_min
 * returns the size this thread's most recent mgemm_grouped_tune chose (0 =
 * integer pipes only). No counterpart in the reference. */
int mwblas_set_grouped_tensor_min(int size);
int mwblas_grouped_tuned_tensor_min(void);
/* mgemm_grouped packs the remaining instances with k >= kmin several to a
 * 256 x 256 tensor-core slot (block-diagonal: each instance owns its rows and
 * output columns; the blocks mixing two instances are computed and never
 * read), an instance with m or n above 256 as pieces of at most 256 x 256;
 * 0 = none, -1 = the tuned or default choice. Returns the
 * previous setting; mwblas_grouped_tuned_tensor_pack returns the depth this
 * thread's most recent mgemm_grouped_tune chose (0 = none). No counterpart in
 * the reference. */
int mwblas_set_grouped_tensor_pack(int kmin);
int mwblas_grouped_tuned_tensor_pack(void);
/* Batched triangular solves with shared flags and per-instance sizes: for
 * i < count, op(A[i]) X = alpha[i] B[i] (side 'L') or X op(A[i]) = alpha[i] B[i]
 * ('R'); B[i] is overwritten. Device (or managed) matrix pointers. */
int mtrsm_grouped(int64_t count, char side, char uplo, char transa, char diag, const int64_t *m,
                  const int64_t *n, const MWBLAS_R *alpha, const MWBLAS_R *const *a, const int64_t *lda,
                  MWBLAS_R *const *b, const int64_t *ldb);

/* Ozaki scheme controls.  bits = significant bits kept per scaled operand
 * row/column, 40..120.  0 (the default) = automatic: 106 bits (a
 * double-double's), reduced per operand to its significant width when every
 * entry of op(A) (or op(B)) is an exact integer at fewer bits after its
 * row's (column's) power-of-two scaling -- FP64 values with lo = 0 over a
 * limited exponent range, for instance; the result is then unchanged in
 * accuracy and computed with fewer moduli.  The width is measured for the
 * products of GEMM, the rank-k family (SYRK/HERK/SYR2K/HER2K), GEMMTR and
 * SYMM/HEMM with m*n*k >= 1024^3, and costs one stream synchronisation
 * after the exponent scan; it is skipped while the library's stream is being
 * captured, for host arrays that are uploaded block by block, and inside the
 * blocked solvers.  The number of moduli (integer GEMMs) follows from the two
 * widths and k.  Returns the previous value. */
int mwblas_set_ozaki_bits(int bits);
/* Moduli count used by the most recent Ozaki GEMM (process-wide). */
int mwblas_last_ozaki_moduli(void);
/* Bits the most recent Ozaki GEMM scaled op(A) (operand 0) or op(B)
 * (operand 1) to. */
int mwblas_last_ozaki_bits(int operand);
/* Residue-GEMM unit of the Ozaki engine: 0 = tcgen05 tensor cores, one CTA
 * per (modulus, tile), 1 = CUDA cores (an independent exact path used to
 * cross-check the tensor cores), 2 = tcgen05 in a persistent kernel (one CTA
 * per SM walking the (modulus, tile) units two at a time, so that one unit's
 * final reduction overlaps the other's MMAs), 3 = as 2 with pairs of CTAs on
 * two SMs computing 256 x 256 tiles with cta_group::2 MMAs (the default). The
 * MWBLAS_OZAKI_MMA environment variable ("pertile", "simt", "persistent",
 * "pair") selects them too. All produce bit-identical results. Returns the
 * previous value. */
int mwblas_set_ozaki_mma(int kind);

/* Operand staging of the FP64 error-free-transform engine: 1 (default) =
 * TMA tensor copies into a ring of shared-memory stages, 0 = plain loads.
 * Both give identical results. Returns the previous value. */
int mwblas_set_plain_tma(int on);

/* Residue conversion of real operands in the Ozaki engine: 1 (default) = the
 * limb dot products as tcgen05 MMAs, 0 = FP32 FMAs on the CUDA cores. Both
 * write identical residues. Returns the previous value. */
int mwblas_set_residue_tc(int on);

/* Real symmetric band (msbmv, bandwidth k <= 32) and packed (mspmv)
 * products: 1 (default) = band: a block of rows per shared-memory tile of the
 * band, copied with coalesced loads; packed: the row halves of the rows in
 * column chunks (a thread per row) and the column halves a warp per row, both
 * read with coalesced loads. 0 = the stored triangle read in place, a thread
 * or a warp per row. Both keep each row's sum exact to about 2^-130 of its
 * largest term and round once; the last bit of the low word may differ.
 * Returns the previous value. */
int mwblas_set_band_tile(int on);

/* Per-phase device timing of the Ozaki engine (CUDA events on the library
 * stream; off by default). Phases: 0 exponent scan, 1 residue conversion,
 * 2 residue GEMMs (tensor cores), 3 CRT reconstruction. mwblas_last_phase_ms
 * returns the durations of the calling thread's most recent Ozaki GEMM. */
int mwblas_set_kernel_timing(int on);
float mwblas_last_phase_ms(int phase);

/* Team size used to reproduce the reference's per-thread body/tail split in
 * the bit-exact level-1 routines (mscal/maxpy/wscal/wmscal).  0 = follow the
 * calling process's OpenMP settings exactly as the reference does
 * (omp_get_max_threads() and omp_in_parallel() when an OpenMP runtime is
 * loaded, else OMP_NUM_THREADS, else the CPU count).  Returns the previous
 * value. */
int64_t mwblas_set_l1_partition(int64_t team);

/* Stream control.  By default every call runs on the calling host thread's
 * per-thread default stream and synchronises before returning.  With a
 * user stream and sync disabled, calls on device pointers return as soon as
 * their work is enqueued (host-pointer calls always synchronise). */
int mwblas_set_stream(void *cuda_stream);       /* cudaStream_t; NULL = default */
int mwblas_set_sync(int sync);                  /* returns previous */
/* 1 when the current device reads pageable host memory in place (through the
 * system page tables, as on the GB300's coherent host link): the pipelined
 * GEMM then uploads ordinary (pageable) host arrays with device reads that
 * overlap its kernels. 0 otherwise. No counterpart in the reference. */
int mwblas_pageable_direct(void);

/* Errors. */
enum {
    MWBLAS_OK = 0,
    MWBLAS_ERR_CUDA = -1,       /* CUDA runtime error */
    MWBLAS_ERR_ALLOC = -2,      /* device allocation failed */
    MWBLAS_ERR_DEVICE = -3,     /* no usable sm_103 device */
    MWBLAS_ERR_TIMEOUT = -4,    /* a bounded device wait gave up */
    MWBLAS_ERR_UNSUPPORTED = -5 /* argument combination not implemented */
};
typedef void (*mwblas_error_hook)(const char *routine, int info, const char *message);
/* Installs a hook called on every recorded error; returns the previous one. */
mwblas_error_hook mwblas_set_error_hook(mwblas_error_hook hook);
/* Last error recorded on this thread (0 if none since mwblas_clear_error). */
int mwblas_last_error(void);
const char *mwblas_last_error_message(void);
const char *mwblas_last_error_routine(void);
void mwblas_clear_error(void);

/* Test hook: the next `count` device allocations succeed, the one after
 * fails (negative = never fail).  Used to test error propagation without a
 * GPU fault. */
void mwblas_debug_fail_alloc_after(int64_t count);

/* Limit of the bounded device waits of the tensor-core kernels, in
 * nanoseconds, on the current device (0 restores the default of 2 s; values
 * below 1 ms are raised to 1 ms). A wait that runs out makes the kernel drain
 * its own copies and MMAs, free its tensor memory and return; the routine then
 * reports MWBLAS_ERR_TIMEOUT and the contents of its output are unspecified.
 * Returns the previous limit. No counterpart in the reference. */
uint64_t mwblas_set_wait_limit_ns(uint64_t ns);

/* Test hook: the next `count` launches of the CTA-pair residue GEMM issue no
 * operand loads, so their first wait for a landed operand stage runs out (with
 * nothing in flight) and the call reports MWBLAS_ERR_TIMEOUT. Exercises the
 * timeout path without a GPU fault. */
void mwblas_debug_lose_operand_loads(int count);

/* Number of kernels this library has launched in the process. */
int64_t mwblas_launch_count(void);

/* y := alpha*A*x + beta*y (no transpose) without allocating any device memory,
 * for callers that must not allocate on the call path (a framework whose own
 * allocator owns the device memory under a fixed budget, or code that cannot
 * afford the driver allocator's locks or cudaFree's device-wide sync). No
 * counterpart in the reference. A, x and y must already be device or managed
 * memory; nothing is staged. The kernel's partial sums live in a fixed 1 MiB
 * device array (65536 double-double values) that the library holds on every
 * GPU until exit, so m may not exceed 65536 (larger m is rejected with info 1).
 * All calls share that array: calls whose kernels overlap on the GPU race. The
 * first call on a device looks up the array's device address (do it before
 * any stream capture). Work is enqueued on `cuda_stream` (NULL: the library's
 * stream) and the call returns without synchronising. Returns 0, a positive
 * argument position, or a negative MWBLAS_ERR_* code. */
int mgemv_n_noalloc(int64_t m, int64_t n, const mwblas_real64x2 *alpha, const mwblas_real64x2 *a, int64_t lda,
                    const mwblas_real64x2 *x, int64_t incx, const mwblas_real64x2 *beta, mwblas_real64x2 *y,
                    int64_t incy, void *cuda_stream);

/* Library version string. */
const char *mwblas_version(void);

#undef MWBLAS_R
#undef MWBLAS_C

#ifdef __cplusplus
}
#endif

#endif /* MWBLAS_GB300_H */
