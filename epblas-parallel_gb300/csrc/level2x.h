// Device-side forms of the level-2 family beyond real GEMV (level2x.cu).
// Arrays are device pointers; vectors may have any non-zero increment.
#pragma once
#include <stdint.h>

#include "gemm.h"

namespace mw {

enum MvShape { MV_GENERAL = 0, MV_SYMMETRIC = 1, MV_HERMITIAN = 2 };

// y := alpha*op(A)*x + beta*y (GENERAL, op from trans) or alpha*A*x + beta*y
// with A symmetric/Hermitian from its uplo triangle; A dense.
struct MvArgs {
    bool cplx = false;
    int shape = MV_GENERAL;
    char trans = 'N', uplo = 'U';
    int64_t lenx = 0, leny = 0;
    const void *A = nullptr;
    int64_t lda = 0;
    const void *x = nullptr;
    int64_t incx = 1;
    void *y = nullptr;
    int64_t incy = 1;
    dd_host alpha{1.0, 0.0}, beta{0.0, 0.0};
    cdd_host calpha{{1.0, 0.0}, {0.0, 0.0}}, cbeta{{0.0, 0.0}, {0.0, 0.0}};
    int beta_kind = 0;
    bool alpha_zero = false;   // y := beta*y only (x and A unused)
};
bool mv_device(const MvArgs &a, const char *routine);

// x := op(A)*x (solve=false) or x := op(A)^-1 * x, A dense triangular.
bool trv_device(bool cplx, bool solve, char uplo, char trans, char diag, int64_t n, const void *A, int64_t lda,
                void *x, int64_t incx, const char *routine);

// Dense general (fmt 0, kind 0, leading dimension ldab), band (fmt 1, LAPACK
// layout, leading dimension ldab) or packed (fmt 2) operand, read in place:
// y := alpha*op(A)*x + beta*y with op(A) rows x cols.
// kind 0 general band (kl, ku); 1 symmetric, 2 Hermitian, 3 triangular
// (unit diagonal when `unit`), the stored triangle given by `upper` with,
// for a band, kl = 0, ku = k (upper) or kl = k, ku = 0 (lower); n is the
// order of a packed matrix. x and y have any increment; they may be the same
// vector when beta_kind == 0 (x is gathered before y is written).
struct SmvArgs {
    bool cplx = false;
    int fmt = 1, kind = 0;
    char trans = 'N';
    bool upper = true, unit = false;
    int64_t rows = 0, cols = 0, n = 0, kl = 0, ku = 0, ldab = 1;
    const void *A = nullptr;
    const void *x = nullptr;
    int64_t incx = 1;
    void *y = nullptr;
    int64_t incy = 1;
    dd_host alpha{1.0, 0.0}, beta{0.0, 0.0};
    cdd_host calpha{{1.0, 0.0}, {0.0, 0.0}}, cbeta{{0.0, 0.0}, {0.0, 0.0}};
    int beta_kind = 0;
};
bool smv_device(const SmvArgs &a, const char *routine);

// op(A) x = b with A a band triangle (LAPACK band storage, bandwidth k,
// leading dimension ldab) read in place: one warp, 32-row tiles,
// double-double row sums. x has any increment.
bool tbsv_device(bool cplx, char uplo, char trans, char diag, int64_t n, int64_t k, const void *AB, int64_t ldab,
                 void *x, int64_t incx, const char *routine);

// Rank updates: uplo 0: GER (A m x n += alpha x op(y), conj for GERC);
// uplo 1/2 (upper/lower triangle of the n = m square A): SYR/HER (y null),
// SYR2/HER2; conj selects the Hermitian forms.
struct RankArgs {
    bool cplx = false, conj = false;
    int uplo = 0;
    int64_t m = 0, n = 0;
    const void *x = nullptr;
    int64_t incx = 1;
    const void *y = nullptr;
    int64_t incy = 1;
    void *A = nullptr;
    int64_t lda = 0;   // < 0 (SYR/HER forms only): A is the packed triangle
    dd_host alpha{1.0, 0.0};
    cdd_host calpha{{1.0, 0.0}, {0.0, 0.0}};
};
bool rank_update_device(const RankArgs &r, const char *routine);

// Band storage to dense: kind 0 general (kl, ku), 1 symmetric, 2 Hermitian
// (full matrix), 3 triangular (stored triangle, unit diagonal when `unit`);
// for kinds 1-3 the band width is ku (upper) or kl (lower).
bool band_expand(int64_t rows, int64_t cols, int64_t kl, int64_t ku, const void *AB, int64_t ldab, int e2, int kind,
                 bool upper, bool unit, void *out);

// Packed triangle <-> dense n x n triangle (unpack: AP -> dense).
void pack_move(int64_t n, void *AP, int e2, bool upper, void *dense, bool unpack);

}  // namespace mw
