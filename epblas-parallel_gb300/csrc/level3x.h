// Device-side forms of GEMMTR, SYMM/HEMM, SYR2K/HER2K, TRMM and complex TRSM
// (level3x.cu). Arrays are device pointers; flags are upper-case and valid.
#pragma once
#include <stdint.h>

#include "gemm.h"

namespace mw {

// C (n x n, triangle uplo: 1 upper, 2 lower) := alpha*op(A)*op(B) + beta*C.
bool gemmtr_device(bool cplx, int uplo, bool ta, bool ca, bool tb, bool cb, int64_t n, int64_t k,
                   const GemmArgs &scal, const void *A, int64_t lda, const void *B, int64_t ldb, void *C, int64_t ldc,
                   const char *routine);

// SYMM (herm=false) / HEMM (herm=true): A symmetric/Hermitian from its `uplo`
// triangle; side 'L': C = alpha*A*B + beta*C, 'R': C = alpha*B*A + beta*C.
bool symm_device(bool cplx, bool herm, char side, char uplo, int64_t m, int64_t n, const GemmArgs &scal,
                 const void *A, int64_t lda, const void *B, int64_t ldb, void *C, int64_t ldc, const char *routine);

// SYR2K / HER2K (herm: conj(alpha) on the second product, real diagonal).
// trans=false: C = alpha*A*B^T + alpha'*B*A^T + beta*C, A and B n x k.
bool syr2k_device(bool cplx, bool herm, int uplo, bool trans, int64_t n, int64_t k, const GemmArgs &scal,
                  const void *A, int64_t lda, const void *B, int64_t ldb, void *C, int64_t ldc, const char *routine);

// TRMM: B := alpha*op(A)*B (side 'L') or alpha*B*op(A) (side 'R').
bool trmm_device(bool cplx, char side, char uplo, char transa, char diag, int64_t m, int64_t n, const GemmArgs &scal,
                 const void *A, int64_t lda, void *B, int64_t ldb, const char *routine);

// Complex TRSM: op(A)*X = alpha*B (side 'L') or X*op(A) = alpha*B, X over B.
bool ctrsm_device(char side, char uplo, char transa, char diag, int64_t m, int64_t n, cdd_host alpha, const void *A,
                  int64_t lda, void *B, int64_t ldb, const char *routine);

}  // namespace mw
