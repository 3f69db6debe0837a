// The remaining level-3 routines of the multifloats overlay, built on the GEMM
// engines the way the reference builds them on mgemm_serial/wgemm_serial:
//
//   GEMMTR  C := alpha*op(A)*op(B) + beta*C, one triangle of C
//           (mgemmtr_parallel.cpp:35-80, wgemmtr_parallel.cpp)
//   SYMM/HEMM  C := alpha*A*B + beta*C or alpha*B*A + beta*C, A symmetric
//           (Hermitian) from one stored triangle (msymm_parallel.cpp:37-102,
//           wsymm_parallel.cpp, whemm_parallel.cpp; whemm_serial.cpp:11-12:
//           the diagonal of a Hermitian A is taken as real)
//   SYR2K/HER2K  C := alpha*op(A)*op(B)^T + alpha*op(B)*op(A)^T + beta*C
//           (conj(alpha) and ^H for HER2K, real beta, real diagonal)
//           (msyr2k_parallel.cpp:38-83, wsyr2k_parallel.cpp, wher2k_parallel.cpp)
//   TRMM    B := alpha*op(A)*B or alpha*B*op(A), A triangular
//           (mtrmm_parallel.cpp:37-106, wtrmm_parallel.cpp)
//   complex TRSM  op(A)*X = alpha*B or X*op(A) = alpha*B (wtrsm_parallel.cpp)
//
// GPU form: the symmetric / triangular operand is expanded once into a dense
// scratch matrix by a bandwidth-bound kernel and the product runs through
// the engine dispatch (tensor cores for large sizes), in place of the
// reference's diagonal-block kernels plus GEMM wings. SYR2K/HER2K are two
// triangular GEMMs into C. The complex TRSM scales each row of op(A) by its
// inverse diagonal and solves the resulting unit triangle, written as a real
// triangle of twice the order over interleaved (re, im) unknowns, with the
// real blocked TRSM in place in B.
#include <cstring>

#include "dd.cuh"
#include "level3.h"
#include "level3x.h"
#include "runtime.h"

namespace mw {

namespace {

constexpr int kThreads = 256;

unsigned blocks_for(int64_t n)
{
    int64_t b = (n + kThreads - 1) / kThreads;
    int64_t cap = (int64_t)device_sm_count() * 16;
    if (b > cap) b = cap;
    return (unsigned)(b < 1 ? 1 : b);
}

// Dense na x na copy of a symmetric (sym) / Hermitian (herm) / triangular
// (neither) matrix given by its `upper` or lower stored triangle. Elements
// are `e2` double2 wide (1 real, 2 complex). Triangular: zeros outside the
// triangle and ones on the diagonal when `unit`. Hermitian: the mirrored
// half is conjugated and the diagonal's imaginary part is zero.
__global__ void k_expand(int64_t na, const double2 *__restrict__ A, int64_t lda, int e2, bool upper, int kind,
                         bool unit, double2 *__restrict__ out)
{
    // kind: 0 triangular, 1 symmetric, 2 Hermitian
    const int64_t total = na * na;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = t % na, j = t / na;
        const bool stored = upper ? (i <= j) : (i >= j);
        double2 *o = out + e2 * (i + j * na);
        double2 v0 = make_double2(0.0, 0.0), v1 = make_double2(0.0, 0.0);
        if (kind == 0) {
            if (i == j && unit) {
                v0 = make_double2(1.0, 0.0);
            } else if (stored) {
                const double2 *a = A + e2 * (i + j * lda);
                v0 = a[0];
                if (e2 == 2) v1 = a[1];
            }
        } else {
            const double2 *a = A + e2 * (stored ? (i + j * lda) : (j + i * lda));
            v0 = a[0];
            if (e2 == 2) {
                v1 = a[1];
                if (kind == 2) {
                    if (i == j) v1 = make_double2(0.0, 0.0);
                    else if (!stored) v1 = make_double2(-v1.x, -v1.y);
                }
            }
        }
        o[0] = v0;
        if (e2 == 2) o[1] = v1;
    }
}

// out (n x m, ld n) = X^T for X (m x n, ld ldx); e2 double2 per element.
__global__ void k_transpose(int64_t m, int64_t n, const double2 *__restrict__ X, int64_t ldx, int e2,
                            double2 *__restrict__ out, int64_t ldo)
{
    __shared__ double2 tile[32][33][2];
    const int64_t i0 = (int64_t)blockIdx.x * 32, j0 = (int64_t)blockIdx.y * 32;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    for (int r = ty; r < 32; r += 8) {
        const int64_t i = i0 + tx, j = j0 + r;
        if (i < m && j < n) {
            const double2 *x = X + e2 * (i + j * ldx);
            tile[r][tx][0] = x[0];
            if (e2 == 2) tile[r][tx][1] = x[1];
        }
    }
    __syncthreads();
    for (int r = ty; r < 32; r += 8) {
        const int64_t j = j0 + tx, i = i0 + r;   // out(j, i) = X(i, j)
        if (i < m && j < n) {
            double2 *o = out + e2 * (j + i * ldo);
            o[0] = tile[tx][r][0];
            if (e2 == 2) o[1] = tile[tx][r][1];
        }
    }
}

// Dense copy of an m x n matrix (e2 double2 per element).
__global__ void k_copy_matrix(int64_t m, int64_t n, const double2 *__restrict__ X, int64_t ldx, int e2,
                              double2 *__restrict__ Y, int64_t ldy)
{
    const int64_t total = m * n * e2;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t w = t % e2, q = t / e2, i = q % m, j = q / m;
        Y[e2 * (i + j * ldy) + w] = X[e2 * (i + j * ldx) + w];
    }
}

// op(A)(i, j) of a stored complex A: trans reads A(j, i), conj conjugates.
__device__ __forceinline__ dd::cplx opAc(const double2 *A, int64_t lda, bool trans, bool conj, int64_t i, int64_t j)
{
    dd::cplx v = dd::cload(A + 2 * (trans ? (j + i * lda) : (i + j * lda)));
    if (conj) v.im = dd::neg(v.im);
    return v;
}

// ---- complex triangular solve through the real one --------------------------------------
// Row i of op(A) X = B scaled by s_i = 1/op(A)(i, i) gives a unit-diagonal
// complex triangle A'. Written as 2 x 2 real blocks [[re, -im], [im, re]]
// over interleaved (re, im) unknowns, A' is a unit-diagonal REAL triangle of
// order 2m, and a column-major complex B (ldb) read as real IS the interleaved
// right-hand side (2m rows, leading dimension 2 ldb). So the complex solve is
// the real blocked TRSM on that 2m x 2m matrix, in place in B.

// inv[i] = 1 / op(A)(i, i) and s[i] = alpha * inv[i] (inv = 1 on a unit diagonal).
__global__ void k_cdiag_inv(int64_t n, const double2 *__restrict__ A, int64_t lda, bool trans, bool conj, bool unit,
                            dd::cplx alpha, double2 *__restrict__ inv, double2 *__restrict__ s)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        dd::cplx r;
        r.re = dd::make(1.0, 0.0);
        r.im = dd::make(0.0, 0.0);
        if (!unit) {
            const dd::cplx d = opAc(A, lda, trans, conj, i, i);
            const dd::real m2 = dd::add_exact(dd::mul_exact(d.re, d.re), dd::mul_exact(d.im, d.im));
            const dd::real q = dd::div(dd::make(1.0, 0.0), m2);
            r.re = dd::mul_exact(d.re, q);
            r.im = dd::neg(dd::mul_exact(d.im, q));
        }
        dd::cstore(inv + 2 * i, r);
        dd::cstore(s + 2 * i, dd::cmul_exact(alpha, r));
    }
}

// L (2n x 2n real, ld 2n): the 2 x 2 block (i, j) is [[v.re, -v.im], [v.im,
// v.re]] with v = inv[i] * op(A)(i, j) inside the triangle, the identity on
// the diagonal and zero outside.
__global__ void k_ctri_to_real(int64_t n, const double2 *__restrict__ A, int64_t lda, bool trans, bool conj,
                               bool lower, bool unit, const double2 *__restrict__ inv, double2 *__restrict__ L)
{
    const int64_t ld = 2 * n;
    const double2 zero = make_double2(0.0, 0.0);
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n * n; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = t % n, j = t / n;
        double2 v00 = zero, v10 = zero, v01 = zero, v11 = zero;
        if (i == j) {
            v00 = v11 = make_double2(1.0, 0.0);
        } else if (lower ? i > j : i < j) {
            dd::cplx v = opAc(A, lda, trans, conj, i, j);
            if (!unit) v = dd::cmul_exact(dd::cload(inv + 2 * i), v);
            v00 = v11 = make_double2(v.re.hi, v.re.lo);
            v10 = make_double2(v.im.hi, v.im.lo);
            v01 = make_double2(-v.im.hi, -v.im.lo);
        }
        double2 *c0 = L + 2 * j * ld + 2 * i;   // column 2j, rows 2i and 2i + 1
        c0[0] = v00;
        c0[1] = v10;
        c0[ld] = v01;
        c0[ld + 1] = v11;
    }
}

// B(i, :) := s[i] * B(i, :)
__global__ void k_crow_scale(int64_t n, int64_t nrhs, const double2 *__restrict__ s, double2 *B, int64_t ldb)
{
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n * nrhs;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = t % n, j = t / n;
        double2 *p = B + 2 * (i + j * ldb);
        dd::cstore(p, dd::cmul_exact(dd::cload(s + 2 * i), dd::cload(p)));
    }
}

unsigned grid_cap(int64_t work)
{
    int64_t b = (work + kThreads - 1) / kThreads;
    const int64_t cap = (int64_t)device_sm_count() * 16;
    if (b > cap) b = cap;
    return (unsigned)(b < 1 ? 1 : b);
}

// Scratch allocation released on scope exit.
struct Scratch {
    void *p = nullptr;
    explicit Scratch(size_t bytes, const char *routine) { p = dev_alloc(bytes, routine); }
    ~Scratch() { dev_free(p); }
};

// op(A) X = alpha B for all nrhs columns of B (stored A with trans/conj
// flags; `lower`: op(A) is lower triangular), through the real solve above.
bool ctrsm_left_real(int64_t n, int64_t nrhs, const double2 *A, int64_t lda, bool trans, bool conj, bool lower,
                     bool unit, cdd_host alpha, double2 *B, int64_t ldb, const char *routine)
{
    Scratch sc((size_t)n * 64 + (size_t)4 * n * n * 16, routine);
    if (!sc.p) return false;
    double2 *inv = (double2 *)sc.p, *sv = inv + 2 * n, *L = sv + 2 * n;
    dd::cplx al;
    al.re = dd::make(alpha.re.hi, alpha.re.lo);
    al.im = dd::make(alpha.im.hi, alpha.im.lo);
    k_cdiag_inv<<<grid_cap(n), kThreads, 0, stream()>>>(n, A, lda, trans, conj, unit, al, inv, sv);
    k_ctri_to_real<<<grid_cap(n * n), kThreads, 0, stream()>>>(n, A, lda, trans, conj, lower, unit, inv, L);
    k_crow_scale<<<grid_cap(n * nrhs), kThreads, 0, stream()>>>(n, nrhs, sv, B, ldb);
    count_launch(3);
    return trsm_device('L', lower ? 'L' : 'U', 'N', 'U', 2 * n, nrhs, dd_host{1.0, 0.0}, L, 2 * n, B, 2 * ldb,
                       routine);
}

}  // namespace

bool gemmtr_device(bool cplx, int uplo, bool ta, bool ca, bool tb, bool cb, int64_t n, int64_t k,
                   const GemmArgs &scal, const void *A, int64_t lda, const void *B, int64_t ldb, void *C, int64_t ldc,
                   const char *routine)
{
    GemmArgs g = scal;
    g.m = n;
    g.n = n;
    g.k = k;
    g.ta = ta;
    g.ca = ca;
    g.tb = tb;
    g.cb = cb;
    g.uplo = uplo;
    g.A = A;
    g.lda = lda;
    g.B = B;
    g.ldb = ldb;
    g.C = C;
    g.ldc = ldc;
    return run_gemm(g, cplx, -1, routine);
}

bool symm_device(bool cplx, bool herm, char side, char uplo, int64_t m, int64_t n, const GemmArgs &scal,
                 const void *A, int64_t lda, const void *B, int64_t ldb, void *C, int64_t ldc, const char *routine)
{
    const int64_t na = side == 'L' ? m : n;
    const int e2 = cplx ? 2 : 1;
    Scratch full((size_t)na * na * 16 * e2, routine);
    if (!full.p) return false;
    k_expand<<<blocks_for(na * na), kThreads, 0, stream()>>>(na, (const double2 *)A, lda, e2, uplo == 'U',
                                                            herm ? 2 : 1, false, (double2 *)full.p);
    count_launch();
    GemmArgs g = scal;
    g.m = m;
    g.n = n;
    g.k = na;
    g.C = C;
    g.ldc = ldc;
    if (side == 'L') {
        g.A = full.p;
        g.lda = na;
        g.B = B;
        g.ldb = ldb;
    } else {
        g.A = B;
        g.lda = ldb;
        g.B = full.p;
        g.ldb = na;
    }
    return run_gemm(g, cplx, -1, routine);
}

bool syr2k_device(bool cplx, bool herm, int uplo, bool trans, int64_t n, int64_t k, const GemmArgs &scal,
                  const void *A, int64_t lda, const void *B, int64_t ldb, void *C, int64_t ldc, const char *routine)
{
    // C = beta*C + alpha*op(A)*op(B)^T (^H), then C += alpha'*op(B)*op(A)^T (^H)
    // with alpha' = alpha (SYR2K) or conj(alpha) (HER2K); HER2K keeps the
    // diagonal real.
    GemmArgs g = scal;
    g.m = n;
    g.n = n;
    g.k = k;
    g.uplo = uplo;
    g.herm = herm;
    g.C = C;
    g.ldc = ldc;
    g.ta = trans;
    g.ca = herm && trans;
    g.tb = !trans;
    g.cb = herm && !trans;
    g.A = A;
    g.lda = lda;
    g.B = B;
    g.ldb = ldb;
    if (!run_gemm(g, cplx, -1, routine)) return false;
    GemmArgs h = g;
    h.A = B;
    h.lda = ldb;
    h.B = A;
    h.ldb = lda;
    h.beta = dd_host{1.0, 0.0};
    h.cbeta = cdd_host{{1.0, 0.0}, {0.0, 0.0}};
    h.beta_kind = 1;
    if (herm) h.calpha.im = dd_host{-scal.calpha.im.hi, -scal.calpha.im.lo};
    return run_gemm(h, cplx, -1, routine);
}

bool trmm_device(bool cplx, char side, char uplo, char transa, char diag, int64_t m, int64_t n, const GemmArgs &scal,
                 const void *A, int64_t lda, void *B, int64_t ldb, const char *routine)
{
    const int64_t na = side == 'L' ? m : n;
    const int e2 = cplx ? 2 : 1;
    Scratch full((size_t)na * na * 16 * e2, routine);
    Scratch prod((size_t)m * n * 16 * e2, routine);
    if (!full.p || !prod.p) return false;
    k_expand<<<blocks_for(na * na), kThreads, 0, stream()>>>(na, (const double2 *)A, lda, e2, uplo == 'U', 0,
                                                            diag == 'U', (double2 *)full.p);
    count_launch();
    GemmArgs g = scal;
    g.beta_kind = 0;
    g.m = m;
    g.n = n;
    g.k = na;
    g.C = prod.p;
    g.ldc = m;
    const bool t = transa != 'N', c = cplx && transa == 'C';
    if (side == 'L') {
        g.A = full.p;
        g.lda = na;
        g.ta = t;
        g.ca = c;
        g.B = B;
        g.ldb = ldb;
    } else {
        g.A = B;
        g.lda = ldb;
        g.B = full.p;
        g.ldb = na;
        g.tb = t;
        g.cb = c;
    }
    if (!run_gemm(g, cplx, -1, routine)) return false;
    k_copy_matrix<<<blocks_for(m * n * e2), kThreads, 0, stream()>>>(m, n, (const double2 *)prod.p, m, e2,
                                                                     (double2 *)B, ldb);
    count_launch();
    return true;
}

bool ctrsm_device(char side, char uplo, char transa, char diag, int64_t m, int64_t n, cdd_host alpha, const void *A,
                  int64_t lda, void *B, int64_t ldb, const char *routine)
{
    const bool unit = diag == 'U';
    bool t = transa != 'N', c = transa == 'C';
    if (side == 'L') {
        const bool lower = (uplo == 'L') != t;
        return ctrsm_left_real(m, n, (const double2 *)A, lda, t, c, lower, unit, alpha, (double2 *)B, ldb, routine);
    }
    // X * op(A) = B  <=>  op(A)^T * X^T = B^T, with op(A)^T = A (N -> T),
    // A (T -> N) or conj(A) (C -> conjugate, no transpose)
    Scratch bt((size_t)m * n * 32, routine);
    if (!bt.p) return false;
    dim3 gt((unsigned)((m + 31) / 32), (unsigned)((n + 31) / 32));
    k_transpose<<<gt, kThreads, 0, stream()>>>(m, n, (const double2 *)B, ldb, 2, (double2 *)bt.p, n);
    count_launch();
    const bool t2 = !t;
    const bool lower = (uplo == 'L') != t2;
    if (!ctrsm_left_real(n, m, (const double2 *)A, lda, t2, c, lower, unit, alpha, (double2 *)bt.p, n, routine))
        return false;
    dim3 gb((unsigned)((n + 31) / 32), (unsigned)((m + 31) / 32));
    k_transpose<<<gb, kThreads, 0, stream()>>>(n, m, (const double2 *)bt.p, n, 2, (double2 *)B, ldb);
    count_launch();
    return true;
}

}  // namespace mw
