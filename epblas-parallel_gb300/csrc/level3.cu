// SYRK, HERK and TRSM on top of the GEMM engines.
//
// SYRK/HERK (msyrk_parallel.cpp:36-83, wherk_parallel.cpp:40-83): one GEMM
// launch restricted to the stored triangle; tiles wholly outside it are not
// launched, and HERK forces a real diagonal. The reference's nb=64 column
// blocks with a diagonal kernel plus a serial GEMM trailing update are a CPU
// cache strategy; on the GPU the triangle is a single grid.
//
// TRSM (mtrsm_parallel.cpp:36-101, mtrsm_serial.cpp:738-822): blocked
// substitution. B is prescaled by alpha, then for each diagonal block of nb
// rows (side 'L') or columns (side 'R'), in the order the triangle dictates:
//   1. a diagonal-block kernel solves the block in double-double, one thread
//      per right-hand side, multiplying by the double-double reciprocal of
//      the diagonal (the reference's `inv = one_dd / A(k,k)`,
//      mtrsm_serial.cpp:144) with the fast multiply;
//   2. the rest of B is updated with one GEMM (alpha = -1, beta = 1) through
//      the engine dispatch, so large solves run their O(m^2 n) work on the
//      same GEMM engines as mgemm_.
#include "dd.cuh"
#include "level3.h"
#include "runtime.h"

namespace mw {

namespace {

// Double-double division a / b (Hida, Li, Bailey 2001, "accurate" DD
// division): three quotient digits from the hi limbs, the remainder
// recomputed in double-double after each.
__device__ __forceinline__ dd::real dd_div(dd::real a, dd::real b)
{
    double q1 = __ddiv_rn(a.hi, b.hi);
    dd::real r = dd::sub_exact(a, dd::mul_exact(dd::make(q1, 0.0), b));
    double q2 = __ddiv_rn(r.hi, b.hi);
    r = dd::sub_exact(r, dd::mul_exact(dd::make(q2, 0.0), b));
    double q3 = __ddiv_rn(r.hi, b.hi);
    dd::real q;
    dd::fast_two_sum(q1, q2, q.hi, q.lo);
    return dd::add_exact(q, dd::make(q3, 0.0));
}

// op(A)(i, j) for a column-major A with optional transpose.
__device__ __forceinline__ dd::real opA(const double2 *A, int64_t lda, bool trans, int64_t i, int64_t j)
{
    return dd::load(trans ? A + j + i * lda : A + i + j * lda);
}

// Side 'L': solve op(A)[blk,blk] * X = B[blk, :] in place for a block of nb
// rows starting at r0. lower: op(A) is lower triangular (forward order).
// Thread per right-hand-side column.
__global__ void k_trsm_diag_left(int64_t r0, int nb, int64_t ncols, const double2 *A, int64_t lda, bool trans,
                                 bool lower, bool unit, double2 *B, int64_t ldb)
{
    int64_t col = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (col >= ncols) return;
    double2 *b = B + col * ldb;
    for (int s = 0; s < nb; ++s) {
        int r = lower ? s : nb - 1 - s;
        int64_t gr = r0 + r;
        dd::real acc = dd::load(b + gr);
        if (lower) {
            for (int p = 0; p < r; ++p)
                acc = dd::add_fast(acc, dd::neg(dd::mul_fast(opA(A, lda, trans, gr, r0 + p), dd::load(b + r0 + p))));
        } else {
            for (int p = r + 1; p < nb; ++p)
                acc = dd::add_fast(acc, dd::neg(dd::mul_fast(opA(A, lda, trans, gr, r0 + p), dd::load(b + r0 + p))));
        }
        if (!unit) acc = dd::mul_fast(acc, dd_div(dd::make(1.0, 0.0), opA(A, lda, trans, gr, gr)));
        dd::store(b + gr, acc);
    }
}

// Side 'R': solve X * op(A)[blk,blk] = B[:, blk] for a block of nb columns
// starting at c0. upper: op(A) is upper triangular (columns in forward order).
// Thread per row of B.
__global__ void k_trsm_diag_right(int64_t c0, int nb, int64_t nrows, const double2 *A, int64_t lda, bool trans,
                                  bool upper, bool unit, double2 *B, int64_t ldb)
{
    int64_t row = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (row >= nrows) return;
    for (int s = 0; s < nb; ++s) {
        int c = upper ? s : nb - 1 - s;
        int64_t gc = c0 + c;
        dd::real acc = dd::load(B + row + gc * ldb);
        if (upper) {
            for (int p = 0; p < c; ++p)
                acc = dd::add_fast(acc,
                                   dd::neg(dd::mul_fast(dd::load(B + row + (c0 + p) * ldb), opA(A, lda, trans, c0 + p, gc))));
        } else {
            for (int p = c + 1; p < nb; ++p)
                acc = dd::add_fast(acc,
                                   dd::neg(dd::mul_fast(dd::load(B + row + (c0 + p) * ldb), opA(A, lda, trans, c0 + p, gc))));
        }
        if (!unit) acc = dd::mul_fast(acc, dd_div(dd::make(1.0, 0.0), opA(A, lda, trans, gc, gc)));
        dd::store(B + row + gc * ldb, acc);
    }
}

// B := alpha * B with the fast multiply (mtrsm_serial.cpp:111-132).
__global__ void k_scale_fast(int64_t m, int64_t n, dd::real alpha, double2 *B, int64_t ldb)
{
    int64_t total = m * n;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        int64_t i = t % m, j = t / m;
        double2 *p = B + i + j * ldb;
        dd::store(p, dd::mul_fast(dd::load(p), alpha));
    }
}

unsigned blocks_for(int64_t total, int threads)
{
    int64_t b = (total + threads - 1) / threads;
    int64_t cap = (int64_t)device_sm_count() * 8;
    if (b > cap) b = cap;
    return (unsigned)(b < 1 ? 1 : b);
}

// Sub-block of op(A): rows [r0, r0+rows) and columns [c0, c0+cols) of op(A)
// as a (pointer, transpose flag) pair usable as a GEMM operand.
const void *op_block(const void *A, int64_t lda, bool trans, int64_t r0, int64_t c0)
{
    const double2 *a = (const double2 *)A;
    return trans ? (const void *)(a + c0 + r0 * lda) : (const void *)(a + r0 + c0 * lda);
}

}  // namespace

bool syrk_device(bool cplx, bool herm, int uplo, bool trans, int64_t n, int64_t k, const void *A, int64_t lda,
                 const GemmArgs &scal, void *C, int64_t ldc, const char *routine)
{
    GemmArgs g = scal;
    g.m = n;
    g.n = n;
    g.k = k;
    g.uplo = uplo;
    g.herm = herm;
    g.A = A;
    g.lda = lda;
    g.B = A;
    g.ldb = lda;
    g.C = C;
    g.ldc = ldc;
    if (!trans) {
        // C = alpha * A * A^T (A^H): op(A) = A, op(B) = A^T (A^H)
        g.ta = false;
        g.tb = true;
        g.ca = false;
        g.cb = herm;
    } else {
        // C = alpha * A^T * A (A^H * A)
        g.ta = true;
        g.tb = false;
        g.ca = herm;
        g.cb = false;
    }
    return run_gemm(g, cplx, -1, routine);
}

bool trsm_device(char side, char uplo, char transa, char diag, int64_t m, int64_t n, dd_host alpha, const void *A,
                 int64_t lda, void *B, int64_t ldb, const char *routine)
{
    bool trans = (transa != 'N');
    bool unit = (diag == 'U');
    // op(A) is lower triangular iff (uplo == 'L') xor transposed.
    bool lower = ((uplo == 'L') != trans);
    double2 *b = (double2 *)B;
    if (!(alpha.hi == 1.0 && alpha.lo == 0.0)) {
        k_scale_fast<<<blocks_for(m * n, 256), 256, 0, stream()>>>(m, n, dd::make(alpha.hi, alpha.lo), b, ldb);
        count_launch();
    }
    const int64_t nb = 64;
    GemmArgs g;
    g.alpha = dd_host{-1.0, 0.0};
    g.beta = dd_host{1.0, 0.0};
    g.beta_kind = 1;
    if (side == 'L') {
        int64_t nblk = (m + nb - 1) / nb;
        for (int64_t s = 0; s < nblk; ++s) {
            int64_t blk = lower ? s : nblk - 1 - s;
            int64_t r0 = blk * nb, rb = (m - r0 < nb) ? m - r0 : nb;
            k_trsm_diag_left<<<blocks_for(n, 128), 128, 0, stream()>>>(r0, (int)rb, n, (const double2 *)A, lda, trans,
                                                                     lower, unit, b, ldb);
            count_launch();
            // trailing rows: lower -> rows below the block, upper -> rows above
            int64_t t0 = lower ? r0 + rb : 0;
            int64_t tr = lower ? m - (r0 + rb) : r0;
            if (tr <= 0) continue;
            g.m = tr;
            g.n = n;
            g.k = rb;
            g.A = op_block(A, lda, trans, t0, r0);
            g.lda = lda;
            g.ta = trans;
            g.B = b + r0;
            g.ldb = ldb;
            g.tb = false;
            g.C = b + t0;
            g.ldc = ldb;
            if (!run_gemm(g, false, -1, routine)) return false;
        }
    } else {
        // X * op(A) = B: op(A) upper -> columns solved left to right.
        bool upper = !lower;
        int64_t nblk = (n + nb - 1) / nb;
        for (int64_t s = 0; s < nblk; ++s) {
            int64_t blk = upper ? s : nblk - 1 - s;
            int64_t c0 = blk * nb, cb = (n - c0 < nb) ? n - c0 : nb;
            k_trsm_diag_right<<<blocks_for(m, 128), 128, 0, stream()>>>(c0, (int)cb, m, (const double2 *)A, lda, trans,
                                                                      upper, unit, b, ldb);
            count_launch();
            // remaining columns: upper -> right of the block, lower -> left
            int64_t t0 = upper ? c0 + cb : 0;
            int64_t tc = upper ? n - (c0 + cb) : c0;
            if (tc <= 0) continue;
            // B[:, T] -= X[:, blk] * op(A)[blk, T]
            g.m = m;
            g.n = tc;
            g.k = cb;
            g.A = b + c0 * ldb;
            g.lda = ldb;
            g.ta = false;
            g.B = op_block(A, lda, trans, c0, t0);
            g.ldb = lda;
            g.tb = trans;
            g.C = b + t0 * ldb;
            g.ldc = ldb;
            if (!run_gemm(g, false, -1, routine)) return false;
        }
    }
    return true;
}

void launch_zero_matrix(int64_t m, int64_t n, void *B, int64_t ldb)
{
    launch_scale_matrix(m, n, dd_host{0.0, 0.0}, 0, B, ldb, 0);
}

}  // namespace mw
