/*
 * Dual-link timing harness: several implementations of the double-double
 * BLAS in ONE process, timed back to back on the same host buffers.
 *
 * This follows the reference's dual-link protocol (benchmark/dual/
 * BENCH_PROTOCOL.md:24-74): each implementation's static archive has its
 * exported symbols renamed to a per-leg prefix (objcopy --redefine-syms, done
 * by run_dual.py), so the legs coexist in one binary without symbol clashes;
 * every repetition runs the legs one after another on the same inputs (the
 * output reset happens outside the timed region), and each leg reports the
 * minimum wall time over the repetitions (CLOCK_MONOTONIC). Ratios are
 * reported as wall-time ratios, smaller = faster.
 *
 * Legs:
 *   gb300      this library (libmwblas_gb300.a, symbols gb_*), called on host
 *              arrays exactly as a caller of the reference would, so its time
 *              includes the host<->device copies;
 *   port       the C restatement of the reference's algorithms in oracle/
 *              (or_port_mgemm, or_port_mdot, or_maxpy, or_mscal), pinned bit for
 *              bit to the reference's own builds by tests/test_oracle_pin.py;
 *   reference  the reference's own double-double sources built from a checkout
 *              (symbols ref_*), only where run_dual.py found them (-DHAVE_REF).
 *
 * Output: one JSON object per (routine, size) on stdout.
 * Usage (through run_dual.py): dual_driver <reps> <gemm n> <vector n>
 */
#include <math.h>
#include <omp.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

typedef struct { double hi, lo; } dd;

/* this library, renamed */
void gb_mgemm_64_(const char *, const char *, const int64_t *, const int64_t *, const int64_t *, const dd *,
                  const dd *, const int64_t *, const dd *, const int64_t *, const dd *, dd *, const int64_t *);
dd gb_mdot_64_(const int64_t *, const dd *, const int64_t *, const dd *, const int64_t *);
void gb_maxpy_64_(const int64_t *, const dd *, const dd *, const int64_t *, dd *, const int64_t *);
void gb_mscal_64_(const int64_t *, const dd *, dd *, const int64_t *);
int64_t gb_mwblas_set_l1_partition(int64_t team);
int gb_mwblas_last_error(void);
const char *gb_mwblas_last_error_message(void);

/* the port of the reference's algorithms (oracle/ddoracle.c) */
void or_port_mgemm(char ta, char tb, int64_t m, int64_t n, int64_t k, const dd *alpha, const dd *A, int64_t lda,
                   const dd *B, int64_t ldb, const dd *beta, dd *C, int64_t ldc, int simd_order);
void or_port_mdot(int64_t n, const dd *x, const dd *y, int64_t team, dd *out);
void or_maxpy(int64_t n, const dd *alpha, const dd *x, int64_t incx, dd *y, int64_t incy, int64_t team);
void or_mscal(int64_t n, const dd *alpha, dd *x, int64_t incx, int64_t team);

#ifdef HAVE_REF
void ref_mgemm_64_(const char *, const char *, const int64_t *, const int64_t *, const int64_t *, const dd *,
                   const dd *, const int64_t *, const dd *, const int64_t *, const dd *, dd *, const int64_t *);
dd ref_mdot_64_(const int64_t *, const dd *, const int64_t *, const dd *, const int64_t *);
void ref_maxpy_64_(const int64_t *, const dd *, const dd *, const int64_t *, dd *, const int64_t *);
void ref_mscal_64_(const int64_t *, const dd *, dd *, const int64_t *);
#endif

enum { GB = 0, PORT = 1, REF = 2, NLEG = 3 };
static const char *leg_name[NLEG] = {"gb300", "port", "reference"};

static double now(void)
{
    struct timespec t;
    clock_gettime(CLOCK_MONOTONIC, &t);
    return (double)t.tv_sec + 1e-9 * (double)t.tv_nsec;
}

/* hi ~ U[-1,1), lo = hi * 2^-53 * U[-1,1), renormalised (seeded LCG) */
static uint64_t g_seed = 0x9e3779b97f4a7c15ull;
static double urand(void)
{
    g_seed = g_seed * 6364136223846793005ull + 1442695040888963407ull;
    return (double)(g_seed >> 11) * (1.0 / 9007199254740992.0);
}
static void fill(dd *v, int64_t n)
{
    for (int64_t i = 0; i < n; ++i) {
        const double hi = 2.0 * urand() - 1.0, lo = hi * ldexp(2.0 * urand() - 1.0, -53);
        const double s = hi + lo;
        v[i].hi = s;
        v[i].lo = lo - (s - hi);
    }
}

static double max_rel_diff(const dd *a, const dd *b, int64_t n)
{
    double num = 0.0, den = 0.0;
    for (int64_t i = 0; i < n; ++i) {
        const double d = fabs((a[i].hi - b[i].hi) + (a[i].lo - b[i].lo));
        if (d > num) num = d;
        if (fabs(b[i].hi) > den) den = fabs(b[i].hi);
    }
    return den > 0.0 ? num / den : num;
}

static void report(const char *routine, int64_t n, int reps, const double *best, int have, double diff_port,
                   double diff_ref)
{
    printf("{\"routine\": \"%s\", \"n\": %lld, \"reps\": %d, \"host_threads\": %d, \"ns_per_call\": {", routine,
           (long long)n, reps, omp_get_max_threads());
    int first = 1;
    for (int l = 0; l < NLEG; ++l)
        if (have & (1 << l)) {
            printf("%s\"%s\": %.0f", first ? "" : ", ", leg_name[l], best[l] * 1e9);
            first = 0;
        }
    printf("}, \"ratio_gb300_over_port\": %.4g", best[GB] / best[PORT]);
    if (have & (1 << REF)) printf(", \"ratio_gb300_over_reference\": %.4g", best[GB] / best[REF]);
    printf(", \"max_rel_diff_vs_port\": %.3g", diff_port);
    if (have & (1 << REF)) printf(", \"max_rel_diff_vs_reference\": %.3g", diff_ref);
    printf("}\n");
    fflush(stdout);
}

static int check_gb(const char *what)
{
    if (gb_mwblas_last_error() != 0) {
        fprintf(stderr, "%s: gb300 leg failed: %s\n", what, gb_mwblas_last_error_message());
        return 0;
    }
    return 1;
}

static int run_gemm(int64_t n, int reps)
{
    const int64_t nn = n * n;
    dd *A = malloc(sizeof(dd) * nn), *B = malloc(sizeof(dd) * nn), *C0 = malloc(sizeof(dd) * nn);
    dd *C[NLEG];
    for (int l = 0; l < NLEG; ++l) C[l] = malloc(sizeof(dd) * nn);
    fill(A, nn);
    fill(B, nn);
    fill(C0, nn);
    const dd al = {1.1, 0.0}, be = {0.9, 0.0};
#if defined(__x86_64__)
    const int simd = 1;   /* the reference's AVX2 kernel order */
#else
    const int simd = 0;   /* its scalar kernel (what it compiles to without AVX2) */
#endif
    int have = (1 << GB) | (1 << PORT);
#ifdef HAVE_REF
    have |= 1 << REF;
#endif
    double best[NLEG] = {1e30, 1e30, 1e30};
    for (int r = 0; r < reps; ++r) {
        for (int l = 0; l < NLEG; ++l) {
            if (!(have & (1 << l))) continue;
            memcpy(C[l], C0, sizeof(dd) * nn);
            const double t0 = now();
            if (l == GB) gb_mgemm_64_("N", "N", &n, &n, &n, &al, A, &n, B, &n, &be, C[l], &n);
            else if (l == PORT) or_port_mgemm('N', 'N', n, n, n, &al, A, n, B, n, &be, C[l], n, simd);
#ifdef HAVE_REF
            else ref_mgemm_64_("N", "N", &n, &n, &n, &al, A, &n, B, &n, &be, C[l], &n);
#endif
            const double dt = now() - t0;
            if (dt < best[l]) best[l] = dt;
            if (l == GB && !check_gb("mgemm")) return 0;
        }
    }
    report("mgemm", n, reps, best, have, max_rel_diff(C[GB], C[PORT], nn),
           (have & (1 << REF)) ? max_rel_diff(C[GB], C[REF], nn) : 0.0);
    free(A); free(B); free(C0);
    for (int l = 0; l < NLEG; ++l) free(C[l]);
    return 1;
}

/* vector routines: DOT, AXPY, SCAL at n */
static int run_vectors(int64_t n, int reps)
{
    dd *x = malloc(sizeof(dd) * n), *y0 = malloc(sizeof(dd) * n), *y[NLEG];
    for (int l = 0; l < NLEG; ++l) y[l] = malloc(sizeof(dd) * n);
    fill(x, n);
    fill(y0, n);
    const int64_t one = 1, team = omp_get_max_threads();
    /* the bit-exact routines follow the same OpenMP team split in both legs */
    gb_mwblas_set_l1_partition(team);
    int have = (1 << GB) | (1 << PORT);
#ifdef HAVE_REF
    have |= 1 << REF;
#endif
    const dd a = {0.75, 0.75 * 0x1p-55};
    /* DOT */
    {
        double best[NLEG] = {1e30, 1e30, 1e30};
        dd res[NLEG];
        for (int r = 0; r < reps; ++r)
            for (int l = 0; l < NLEG; ++l) {
                if (!(have & (1 << l))) continue;
                const double t0 = now();
                if (l == GB) res[l] = gb_mdot_64_(&n, x, &one, y0, &one);
                else if (l == PORT) or_port_mdot(n, x, y0, team, &res[l]);
#ifdef HAVE_REF
                else res[l] = ref_mdot_64_(&n, x, &one, y0, &one);
#endif
                const double dt = now() - t0;
                if (dt < best[l]) best[l] = dt;
                if (l == GB && !check_gb("mdot")) return 0;
            }
        double scale = 0.0;   /* n max|x| max|y|: the normwise denominator */
        for (int64_t i = 0; i < n; ++i) scale = fmax(scale, fabs(x[i].hi));
        double sy = 0.0;
        for (int64_t i = 0; i < n; ++i) sy = fmax(sy, fabs(y0[i].hi));
        scale *= sy * (double)n;
        const double dp = fabs((res[GB].hi - res[PORT].hi) + (res[GB].lo - res[PORT].lo)) / scale;
        double dr = 0.0;
#ifdef HAVE_REF
        dr = fabs((res[GB].hi - res[REF].hi) + (res[GB].lo - res[REF].lo)) / scale;
#endif
        report("mdot", n, reps, best, have, dp, dr);
    }
    /* AXPY and SCAL (bit-exact: the differences must be 0) */
    for (int which = 0; which < 2; ++which) {
        double best[NLEG] = {1e30, 1e30, 1e30};
        for (int r = 0; r < reps; ++r)
            for (int l = 0; l < NLEG; ++l) {
                if (!(have & (1 << l))) continue;
                memcpy(y[l], y0, sizeof(dd) * n);
                const double t0 = now();
                if (which == 0) {
                    if (l == GB) gb_maxpy_64_(&n, &a, x, &one, y[l], &one);
                    else if (l == PORT) or_maxpy(n, &a, x, 1, y[l], 1, team);
#ifdef HAVE_REF
                    else ref_maxpy_64_(&n, &a, x, &one, y[l], &one);
#endif
                } else {
                    if (l == GB) gb_mscal_64_(&n, &a, y[l], &one);
                    else if (l == PORT) or_mscal(n, &a, y[l], 1, team);
#ifdef HAVE_REF
                    else ref_mscal_64_(&n, &a, y[l], &one);
#endif
                }
                const double dt = now() - t0;
                if (dt < best[l]) best[l] = dt;
                if (l == GB && !check_gb(which ? "mscal" : "maxpy")) return 0;
            }
        report(which ? "mscal" : "maxpy", n, reps, best, have, max_rel_diff(y[GB], y[PORT], n),
               (have & (1 << REF)) ? max_rel_diff(y[GB], y[REF], n) : 0.0);
    }
    free(x); free(y0);
    for (int l = 0; l < NLEG; ++l) free(y[l]);
    return 1;
}

int main(int argc, char **argv)
{
    const int reps = argc > 1 ? atoi(argv[1]) : 10;
    const int64_t gn = argc > 2 ? atoll(argv[2]) : 1024;
    const int64_t vn = argc > 3 ? atoll(argv[3]) : (1 << 22);
    if (reps < 1 || gn < 1 || vn < 1) return 2;
    if (!run_gemm(gn, reps)) return 1;
    if (!run_vectors(vn, reps)) return 1;
    return 0;
}
