// The level-2 family beyond GEMV, built on the level-3 machinery:
//
//   GEMV (complex), GBMV       y := alpha*op(A)*x + beta*y        (mgbmv.cpp, wgemv.cpp, wgbmv.cpp)
//   SYMV/HEMV, SBMV/HBMV, SPMV/HPMV   A symmetric / Hermitian     (msymv.cpp, whemv.cpp, msbmv.cpp, ...)
//   TRMV/TBMV/TPMV, TRSV/TBSV/TPSV    A triangular               (mtrmv.cpp, mtrsv.cpp, mtbmv.cpp, ...)
//   GER/GERU/GERC, SYR/HER, SYR2/HER2, SPR/HPR, SPR2/HPR2  rank-1/2 updates (mger.cpp, msyr.cpp, ...)
//
// Band and packed operands are first expanded into a dense scratch matrix by
// one bandwidth-bound kernel (packed outputs are packed back); vectors with
// any increment are gathered into contiguous scratch in BLAS order (a
// negative increment walks backwards) and written back the same way. The
// products then run as GEMM/SYMM/TRMM/TRSM/SYRK/SYR2K on the engines with
// one right-hand side or a rank of one, so the arithmetic is the engines'
// (exact fixed point or tensor-core residues) and the error bounds are the
// level-3 ones.
#include "dd.cuh"
#include "level2x.h"
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

__device__ __forceinline__ int64_t vpos(int64_t i, int64_t n, int64_t inc)
{
    return inc >= 0 ? i * inc : (n - 1 - i) * (-inc);
}

// dst[i] = src[vpos(i)] (gather=true) or src[vpos(i)] = dst[i] (scatter)
__global__ void k_vgather(int64_t n, double2 *strided, int64_t inc, int e2, double2 *dense, bool gather)
{
    const int64_t total = n * e2;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = t / e2, w = t % e2;
        double2 *s = strided + e2 * vpos(i, n, inc) + w;
        double2 *d = dense + e2 * i + w;
        if (gather) *d = *s;
        else *s = *d;
    }
}

// Band storage (LAPACK layout) to a dense rows x cols matrix (ld rows):
//   general (kind 0): A(i, j) = AB(ku + i - j, j) for j - ku <= i <= j + kl;
//   symmetric/Hermitian (kind 1/2): the stored triangle (k super- or
//     sub-diagonals) mirrored, conjugated for Hermitian, real diagonal;
//   triangular (kind 3): the stored triangle, zeros elsewhere, ones on the
//     diagonal when unit.
__global__ void k_band_expand(int64_t rows, int64_t cols, int64_t kl, int64_t ku, const double2 *__restrict__ AB,
                              int64_t ldab, int e2, int kind, bool upper, bool unit, double2 *__restrict__ out)
{
    const int64_t total = rows * cols;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = t % rows, j = t / rows;
        double2 v0 = make_double2(0.0, 0.0), v1 = make_double2(0.0, 0.0);
        int64_t si = i, sj = j;
        bool conj = false, have = false;
        if (kind == 0) {
            have = (i >= j - ku) && (i <= j + kl);
        } else {
            const int64_t k = upper ? ku : kl;
            const bool in_tri = upper ? (i <= j && i >= j - k) : (i >= j && i <= j + k);
            const bool in_mir = upper ? (j <= i && j >= i - k) : (j >= i && j <= i + k);
            if (kind == 3) {
                have = in_tri;
            } else if (in_tri) {
                have = true;
            } else if (in_mir) {
                have = true;
                si = j;
                sj = i;
                conj = kind == 2;
            }
        }
        if (have) {
            // band row of stored (si, sj): general / upper: ku + si - sj; lower: si - sj
            const int64_t br = (kind == 0 || upper) ? (ku + si - sj) : (si - sj);
            const double2 *a = AB + e2 * (br + sj * ldab);
            v0 = a[0];
            if (e2 == 2) {
                v1 = a[1];
                if (conj) v1 = make_double2(-v1.x, -v1.y);
                if (kind == 2 && si == sj) v1 = make_double2(0.0, 0.0);
            }
        }
        if (kind == 3 && unit && i == j) {
            v0 = make_double2(1.0, 0.0);
            v1 = make_double2(0.0, 0.0);
        }
        double2 *o = out + e2 * (i + j * rows);
        o[0] = v0;
        if (e2 == 2) o[1] = v1;
    }
}

// Packed triangle <-> the same triangle of a dense n x n matrix (ld n):
// upper AP[i + j(j+1)/2] (i <= j), lower AP[i + j(2n-j-1)/2] (i >= j). The
// other triangle of the dense matrix is left as it is (unpack) / ignored.
__global__ void k_pack(int64_t n, double2 *AP, int e2, bool upper, double2 *dense, bool unpack)
{
    const int64_t total = n * n;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = t % n, j = t / n;
        if (upper ? (i > j) : (i < j)) continue;
        const int64_t p = upper ? (i + j * (j + 1) / 2) : (i + j * (2 * n - j - 1) / 2);
        for (int w = 0; w < e2; ++w) {
            if (unpack) dense[e2 * (i + j * n) + w] = AP[e2 * p + w];
            else AP[e2 * p + w] = dense[e2 * (i + j * n) + w];
        }
    }
}

struct Buf {
    void *p = nullptr;
    Buf(size_t bytes, const char *routine) { p = dev_alloc(bytes, routine); }
    ~Buf() { dev_free(p); }
};

void vgather(int64_t n, const void *x, int64_t inc, int e2, void *dense, bool gather)
{
    k_vgather<<<blocks_for(n * e2), kThreads, 0, stream()>>>(n, (double2 *)x, inc, e2, (double2 *)dense, gather);
    count_launch();
}

}  // namespace

bool band_expand(int64_t rows, int64_t cols, int64_t kl, int64_t ku, const void *AB, int64_t ldab, int e2, int kind,
                 bool upper, bool unit, void *out)
{
    k_band_expand<<<blocks_for(rows * cols), kThreads, 0, stream()>>>(rows, cols, kl, ku, (const double2 *)AB, ldab,
                                                                      e2, kind, upper, unit, (double2 *)out);
    count_launch();
    return true;
}

void pack_move(int64_t n, void *AP, int e2, bool upper, void *dense, bool unpack)
{
    k_pack<<<blocks_for(n * n), kThreads, 0, stream()>>>(n, (double2 *)AP, e2, upper, (double2 *)dense, unpack);
    count_launch();
}

bool mv_device(const MvArgs &a, const char *routine)
{
    const int e2 = a.cplx ? 2 : 1;
    const size_t es = 16 * (size_t)e2;
    // contiguous copies of the vectors
    const int64_t lx = a.lenx, ly = a.leny;
    Buf xb((size_t)(lx > 0 ? lx : 1) * es, routine), yb((size_t)(ly > 0 ? ly : 1) * es, routine);
    if (!xb.p || !yb.p) return false;
    if (a.beta_kind != 0 && ly > 0) vgather(ly, a.y, a.incy, e2, yb.p, true);
    if (a.alpha_zero) {
        // y := beta * y (beta == 0 writes zeros without reading y)
        if (a.cplx) launch_scale_matrix_c(ly, 1, a.cbeta, a.beta_kind, yb.p, ly);
        else launch_scale_matrix(ly, 1, a.beta, a.beta_kind, yb.p, ly);
        vgather(ly, a.y, a.incy, e2, yb.p, false);
        return true;
    }
    vgather(lx, a.x, a.incx, e2, xb.p, true);
    GemmArgs g;
    g.alpha = a.alpha;
    g.beta = a.beta;
    g.calpha = a.calpha;
    g.cbeta = a.cbeta;
    g.beta_kind = a.beta_kind;
    bool ok;
    switch (a.shape) {
    case MV_GENERAL: {
        // y = alpha*op(A)*x + beta*y: op(A) (leny x lenx) times x (lenx x 1)
        g.m = ly;
        g.n = 1;
        g.k = lx;
        g.ta = a.trans != 'N';
        g.ca = a.cplx && a.trans == 'C';
        g.A = a.A;
        g.lda = a.lda;
        g.B = xb.p;
        g.ldb = lx;
        g.C = yb.p;
        g.ldc = ly;
        ok = run_gemm(g, a.cplx, -1, routine);
        break;
    }
    case MV_SYMMETRIC:
    case MV_HERMITIAN:
        ok = symm_device(a.cplx, a.shape == MV_HERMITIAN, 'L', a.uplo, ly, 1, g, a.A, a.lda, xb.p, lx, yb.p, ly,
                         routine);
        break;
    default:
        ok = false;
    }
    if (!ok) return false;
    vgather(ly, a.y, a.incy, e2, yb.p, false);
    return true;
}

bool trv_device(bool cplx, bool solve, char uplo, char trans, char diag, int64_t n, const void *A, int64_t lda,
                void *x, int64_t incx, const char *routine)
{
    const int e2 = cplx ? 2 : 1;
    Buf xb((size_t)n * 16 * e2, routine);
    if (!xb.p) return false;
    vgather(n, x, incx, e2, xb.p, true);
    bool ok;
    if (solve) {
        ok = cplx ? ctrsm_device('L', uplo, trans, diag, n, 1, cdd_host{{1.0, 0.0}, {0.0, 0.0}}, A, lda, xb.p, n,
                                 routine)
                  : trsm_device('L', uplo, trans == 'C' ? 'T' : trans, diag, n, 1, dd_host{1.0, 0.0}, A, lda, xb.p,
                                n, routine);
    } else {
        GemmArgs g;
        g.alpha = dd_host{1.0, 0.0};
        g.calpha = cdd_host{{1.0, 0.0}, {0.0, 0.0}};
        ok = trmm_device(cplx, 'L', uplo, trans, diag, n, 1, g, A, lda, xb.p, n, routine);
    }
    if (!ok) return false;
    vgather(n, x, incx, e2, xb.p, false);
    return true;
}

bool rank_update_device(const RankArgs &r, const char *routine)
{
    const int e2 = r.cplx ? 2 : 1;
    Buf xb((size_t)r.m * 16 * e2, routine), yb((size_t)(r.y ? r.n : 1) * 16 * e2, routine);
    if (!xb.p || !yb.p) return false;
    vgather(r.m, r.x, r.incx, e2, xb.p, true);
    if (r.y) vgather(r.n, r.y, r.incy, e2, yb.p, true);
    GemmArgs g;
    g.alpha = r.alpha;
    g.calpha = r.calpha;
    g.beta = dd_host{1.0, 0.0};
    g.cbeta = cdd_host{{1.0, 0.0}, {0.0, 0.0}};
    g.beta_kind = 1;
    if (r.uplo == 0) {
        // GER: A += alpha * x * op(y) with op = transpose (conjugated for GERC)
        g.m = r.m;
        g.n = r.n;
        g.k = 1;
        g.A = xb.p;
        g.lda = r.m;
        g.B = yb.p;
        g.ldb = r.n;
        g.tb = true;
        g.cb = r.conj;
        g.C = r.A;
        g.ldc = r.lda;
        return run_gemm(g, r.cplx, -1, routine);
    }
    if (!r.y)   // SYR / HER: A += alpha * x * x^T (x^H), triangle
        return syrk_device(r.cplx, r.conj, r.uplo, false, r.m, 1, xb.p, r.m, g, r.A, r.lda, routine);
    // SYR2 / HER2
    return syr2k_device(r.cplx, r.conj, r.uplo, false, r.m, 1, g, xb.p, r.m, yb.p, r.m, r.A, r.lda, routine);
}

}  // namespace mw
