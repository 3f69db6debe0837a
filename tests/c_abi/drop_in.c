/*
 * A plain C caller of the drop-in library, linked the way a C or Fortran
 * program that used the reference's `mwblas` archive would be: against
 * libmwblas_gb300.so or the static libmwblas_gb300.a, with host arrays and
 * the Fortran-style symbols of include/mwblas_gb300.h.
 *
 * Inputs are small integers, so every expected result is exact and checked
 * here with integer arithmetic: GEMM (real and complex, LP64 and ILP64),
 * GEMV, DOT, I*AMAX, SYRK, TRSM and ROTG. Prints "drop_in ok" and exits 0 when
 * every check passes.
 */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>

#include "mwblas_gb300.h"

static int failures = 0;

#define CHECK(cond, ...)                      \
    do {                                      \
        if (!(cond)) {                        \
            if (failures < 10) {              \
                fprintf(stderr, "FAIL: " __VA_ARGS__); \
                fputc('\n', stderr);          \
            }                                 \
            ++failures;                       \
        }                                     \
    } while (0)

static uint64_t state = 88172645463325252ull;
static int small_int(void)
{
    state ^= state << 13;
    state ^= state >> 7;
    state ^= state << 17;
    return (int)(state % 17) - 8;
}

static mwblas_real64x2 dd(double v)
{
    mwblas_real64x2 r;
    r.limbs[0] = v;
    r.limbs[1] = 0.0;
    return r;
}

static void check_error(const char *what)
{
    CHECK(mwblas_last_error() == 0, "%s reported error %d (%s)", what, mwblas_last_error(),
          mwblas_last_error_message());
}

static void test_gemm(void)
{
    enum { M = 37, N = 29, K = 53 };
    static mwblas_real64x2 a[K * M], b[K * N], c[M * N];
    static long ia[K * M], ib[K * N];
    for (int i = 0; i < K * M; ++i) { ia[i] = small_int(); a[i] = dd((double)ia[i]); }
    for (int i = 0; i < K * N; ++i) { ib[i] = small_int(); b[i] = dd((double)ib[i]); }
    const mwblas_real64x2 one = dd(1.0), zero = dd(0.0);
    /* C = A^T * B with A stored K x M */
    const int m = M, n = N, k = K, lda = K, ldb = K, ldc = M;
    mgemm_("T", "N", &m, &n, &k, &one, a, &lda, b, &ldb, &zero, c, &ldc);
    check_error("mgemm_");
    for (int j = 0; j < N; ++j)
        for (int i = 0; i < M; ++i) {
            long s = 0;
            for (int p = 0; p < K; ++p) s += ia[p + i * K] * ib[p + j * K];
            CHECK(c[i + j * M].limbs[0] == (double)s && c[i + j * M].limbs[1] == 0.0, "mgemm_ (%d,%d)", i, j);
        }
    /* the same product through the ILP64 entry, beta = 1 doubles it */
    const int64_t m8 = M, n8 = N, k8 = K, lda8 = K, ldb8 = K, ldc8 = M;
    mgemm_64_("T", "N", &m8, &n8, &k8, &one, a, &lda8, b, &ldb8, &one, c, &ldc8);
    check_error("mgemm_64_");
    for (int j = 0; j < N; ++j)
        for (int i = 0; i < M; ++i) {
            long s = 0;
            for (int p = 0; p < K; ++p) s += ia[p + i * K] * ib[p + j * K];
            CHECK(c[i + j * M].limbs[0] == (double)(2 * s), "mgemm_64_ (%d,%d)", i, j);
        }
}

static void test_wgemm(void)
{
    enum { M = 9, N = 7, K = 11 };
    static mwblas_complex64x2 a[M * K], b[K * N], c[M * N];
    static long ar[M * K], ai[M * K], br[K * N], bi[K * N];
    for (int i = 0; i < M * K; ++i) {
        ar[i] = small_int(); ai[i] = small_int();
        a[i].re = dd((double)ar[i]); a[i].im = dd((double)ai[i]);
    }
    for (int i = 0; i < K * N; ++i) {
        br[i] = small_int(); bi[i] = small_int();
        b[i].re = dd((double)br[i]); b[i].im = dd((double)bi[i]);
    }
    mwblas_complex64x2 one, zero;
    one.re = dd(1.0); one.im = dd(0.0);
    zero.re = dd(0.0); zero.im = dd(0.0);
    const int m = M, n = N, k = K, lda = M, ldb = K, ldc = M;
    wgemm_("N", "N", &m, &n, &k, &one, a, &lda, b, &ldb, &zero, c, &ldc);
    check_error("wgemm_");
    for (int j = 0; j < N; ++j)
        for (int i = 0; i < M; ++i) {
            long sr = 0, si = 0;
            for (int p = 0; p < K; ++p) {
                sr += ar[i + p * M] * br[p + j * K] - ai[i + p * M] * bi[p + j * K];
                si += ar[i + p * M] * bi[p + j * K] + ai[i + p * M] * br[p + j * K];
            }
            CHECK(c[i + j * M].re.limbs[0] == (double)sr && c[i + j * M].im.limbs[0] == (double)si,
                  "wgemm_ (%d,%d)", i, j);
        }
}

static void test_level12(void)
{
    enum { N = 1000 };
    static mwblas_real64x2 x[N], y[N], a[N * 3], yv[3];
    static long ix[N], iy[N], iav[N * 3];
    for (int i = 0; i < N; ++i) {
        ix[i] = small_int(); iy[i] = small_int();
        x[i] = dd((double)ix[i]); y[i] = dd((double)iy[i]);
    }
    const int n = N, one_i = 1;
    mwblas_real64x2 d = mdot_(&n, x, &one_i, y, &one_i);
    check_error("mdot_");
    long s = 0;
    for (int i = 0; i < N; ++i) s += ix[i] * iy[i];
    CHECK(d.limbs[0] == (double)s && d.limbs[1] == 0.0, "mdot_ %g vs %ld", d.limbs[0], s);

    x[611] = dd(-1.0e6);
    const int imax = imamax_(&n, x, &one_i);
    CHECK(imax == 612, "imamax_ returned %d", imax);
    x[611] = dd((double)ix[611]);

    /* y(3) := A^T x, A is N x 3 */
    for (int i = 0; i < N * 3; ++i) { iav[i] = small_int(); a[i] = dd((double)iav[i]); }
    const mwblas_real64x2 one = dd(1.0), zero = dd(0.0);
    const int three = 3;
    mgemv_("T", &n, &three, &one, a, &n, x, &one_i, &zero, yv, &one_i);
    check_error("mgemv_");
    for (int j = 0; j < 3; ++j) {
        long t = 0;
        for (int i = 0; i < N; ++i) t += iav[i + j * N] * ix[i];
        CHECK(yv[j].limbs[0] == (double)t, "mgemv_ row %d", j);
    }
}

static void test_syrk_trsm(void)
{
    enum { N = 24, K = 40 };
    static mwblas_real64x2 a[N * K], c[N * N], t[N * N], b[N * 5];
    static long ia[N * K], it[N * N], ix[N * 5];
    for (int i = 0; i < N * K; ++i) { ia[i] = small_int(); a[i] = dd((double)ia[i]); }
    for (int i = 0; i < N * N; ++i) c[i] = dd(12345.0);
    const mwblas_real64x2 one = dd(1.0), zero = dd(0.0);
    const int n = N, k = K;
    msyrk_("L", "N", &n, &k, &one, a, &n, &zero, c, &n);
    check_error("msyrk_");
    for (int j = 0; j < N; ++j)
        for (int i = 0; i < N; ++i) {
            long s = 0;
            for (int p = 0; p < K; ++p) s += ia[i + p * N] * ia[j + p * N];
            const double want = i >= j ? (double)s : 12345.0;   /* upper triangle untouched */
            CHECK(c[i + j * N].limbs[0] == want, "msyrk_ (%d,%d)", i, j);
        }
    /* unit lower-triangular T with integer entries: B = T X has the exact solution X */
    for (int j = 0; j < N; ++j)
        for (int i = 0; i < N; ++i) {
            it[i + j * N] = i > j ? small_int() % 3 : (i == j ? 1 : 0);
            t[i + j * N] = dd((double)it[i + j * N]);
        }
    for (int i = 0; i < N * 5; ++i) ix[i] = small_int();
    for (int j = 0; j < 5; ++j)
        for (int i = 0; i < N; ++i) {
            long s = 0;
            for (int p = 0; p <= i; ++p) s += it[i + p * N] * ix[p + j * N];
            b[i + j * N] = dd((double)s);
        }
    const int five = 5;
    mtrsm_("L", "L", "N", "U", &n, &five, &one, t, &n, b, &n);
    check_error("mtrsm_");
    for (int i = 0; i < N * 5; ++i)
        CHECK(fabs(b[i].limbs[0] - (double)ix[i]) <= 1e-20 * (1.0 + fabs((double)ix[i])), "mtrsm_ entry %d", i);
}

static void test_rotg(void)
{
    mwblas_real64x2 a = dd(3.0), b = dd(4.0), c, s;
    mrotg_(&a, &b, &c, &s);
    check_error("mrotg_");
    CHECK(a.limbs[0] == 5.0 && a.limbs[1] == 0.0, "mrotg_ r = %g", a.limbs[0]);
    CHECK(fabs(c.limbs[0] * 5.0 - 3.0) < 1e-15 && fabs(s.limbs[0] * 5.0 - 4.0) < 1e-15, "mrotg_ c, s");
}

int main(void)
{
    test_gemm();
    test_wgemm();
    test_level12();
    test_syrk_trsm();
    test_rotg();
    if (failures) {
        fprintf(stderr, "drop_in: %d failure(s)\n", failures);
        return 1;
    }
    printf("drop_in ok\n");
    return 0;
}
