// SYRK, HERK and TRSM on top of the GEMM engines.
//
// SYRK/HERK (msyrk_parallel.cpp:36-83, wherk_parallel.cpp:40-83): one GEMM
// launch restricted to the stored triangle; tiles wholly outside it are not
// launched, and HERK forces a real diagonal. The reference's nb=64 column
// blocks with a diagonal kernel plus a serial GEMM trailing update are a CPU
// cache strategy; on the GPU the triangle is a single grid.
//
// TRSM (mtrsm_parallel.cpp:36-101, mtrsm_serial.cpp:738-822): B is prescaled
// by alpha, then the triangle is split in halves recursively: solve one half,
// update the other half of B with one GEMM (alpha = -1, beta = 1) through the
// engine dispatch, solve the other half. The O(m^2 n) update work thus lands
// in a few large GEMMs (half the triangle at the top level), which is the
// shape the tensor-core engine needs. Blocks of at most 64 rows/columns:
//  * with many right-hand sides, all 64 x 64 diagonal blocks are inverted in
//    one launch (substitution with the double-double reciprocal of the
//    diagonal, the reference's `inv = one_dd / A(k,k)`, mtrsm_serial.cpp:144)
//    and each block of B is solved as one GEMM with its inverse, as GPU BLAS
//    libraries do for their TRSM;
//  * with few, each block is solved by substitution in double-double, one
//    thread per right-hand side.
#include <algorithm>
#include <vector>

#include "dd.cuh"
#include "fixacc.cuh"
#include "level3.h"
#include "runtime.h"

namespace mw {

namespace {

__device__ __forceinline__ dd::real dd_div(dd::real a, dd::real b) { return dd::div(a, b); }

// op(A)(i, j) for a column-major A with optional transpose.
__device__ __forceinline__ dd::real opA(const double2 *A, int64_t lda, bool trans, int64_t i, int64_t j)
{
    return dd::load(trans ? A + j + i * lda : A + i + j * lda);
}

// Side 'L': solve op(A)[blk,blk] * X = B[blk, :] in place for a block of nb
// rows starting at r0. lower: op(A) is lower triangular (forward order).
// Thread per right-hand-side column; four partial sums break the dependency
// chain of the dot product.
__global__ void k_trsm_diag_left(int64_t r0, int nb, int64_t ncols, const double2 *A, int64_t lda, bool trans,
                                 bool lower, bool unit, double2 *B, int64_t ldb)
{
    int64_t col = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (col >= ncols) return;
    double2 *b = B + col * ldb;
    for (int s = 0; s < nb; ++s) {
        int r = lower ? s : nb - 1 - s;
        int64_t gr = r0 + r;
        int p0 = lower ? 0 : r + 1, p1 = lower ? r : nb;
        dd::real acc[4] = {dd::load(b + gr), dd::make(0.0, 0.0), dd::make(0.0, 0.0), dd::make(0.0, 0.0)};
        int p = p0;
        for (; p + 4 <= p1; p += 4) {
#pragma unroll
            for (int u = 0; u < 4; ++u)
                acc[u] = dd::add_fast(acc[u], dd::neg(dd::mul_fast(opA(A, lda, trans, gr, r0 + p + u), dd::load(b + r0 + p + u))));
        }
        for (; p < p1; ++p) acc[0] = dd::add_fast(acc[0], dd::neg(dd::mul_fast(opA(A, lda, trans, gr, r0 + p), dd::load(b + r0 + p))));
        dd::real v = dd::add_fast(dd::add_fast(acc[0], acc[1]), dd::add_fast(acc[2], acc[3]));
        if (!unit) v = dd::mul_fast(v, dd_div(dd::make(1.0, 0.0), opA(A, lda, trans, gr, gr)));
        dd::store(b + gr, v);
    }
}

// Side 'R': solve X * op(A)[blk,blk] = B[:, blk] for a block of nb columns
// starting at c0. upper: op(A) is upper triangular (columns in forward order).
// Thread per row of B, four partial sums per dot product.
__global__ void k_trsm_diag_right(int64_t c0, int nb, int64_t nrows, const double2 *A, int64_t lda, bool trans,
                                  bool upper, bool unit, double2 *B, int64_t ldb)
{
    int64_t row = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (row >= nrows) return;
    for (int s = 0; s < nb; ++s) {
        int c = upper ? s : nb - 1 - s;
        int64_t gc = c0 + c;
        int p0 = upper ? 0 : c + 1, p1 = upper ? c : nb;
        dd::real acc[4] = {dd::load(B + row + gc * ldb), dd::make(0.0, 0.0), dd::make(0.0, 0.0), dd::make(0.0, 0.0)};
        int p = p0;
        for (; p + 4 <= p1; p += 4) {
#pragma unroll
            for (int u = 0; u < 4; ++u)
                acc[u] = dd::add_fast(acc[u], dd::neg(dd::mul_fast(dd::load(B + row + (c0 + p + u) * ldb),
                                                                     opA(A, lda, trans, c0 + p + u, gc))));
        }
        for (; p < p1; ++p)
            acc[0] = dd::add_fast(acc[0], dd::neg(dd::mul_fast(dd::load(B + row + (c0 + p) * ldb), opA(A, lda, trans, c0 + p, gc))));
        dd::real v = dd::add_fast(dd::add_fast(acc[0], acc[1]), dd::add_fast(acc[2], acc[3]));
        if (!unit) v = dd::mul_fast(v, dd_div(dd::make(1.0, 0.0), opA(A, lda, trans, gc, gc)));
        dd::store(B + row + gc * ldb, v);
    }
}

// Inverses of the 32 x 32 diagonal blocks of op(A) (the last block may be
// shorter), one CTA per block, four threads per column c of the inverse:
// solve op(A)_blk x = e_c by substitution over all rows (x is zero above c
// for a lower triangle, so every thread walks the same rows and the block
// entries are shared-memory broadcasts). The four threads of a column split
// each sum sum_p L(r,p) x(p) by p mod 4, accumulate their shares in integer
// fixed point (fixacc.cuh) and add the four results as extended floats in a
// fixed order (lanes 0 + 2, 1 + 3, then the two), rounded once; each row is
// then multiplied by the double-double reciprocal of the diagonal, as the
// reference's substitution does (mtrsm_serial.cpp:144).
// Inv: block b at Inv + b*32*32, column-major with leading dimension 32.
constexpr int kInvNB = 32;   // order of the directly inverted blocks (merged up to the leaf order)
constexpr int kInvSplit = 4;  // threads per column

__global__ void __launch_bounds__(kInvNB * kInvSplit) k_trsm_diag_inv(int64_t na, const double2 *__restrict__ A,
                                                                      int64_t lda, bool trans, bool lower, bool unit,
                                                                      double2 *Inv)
{
    extern __shared__ fx::OpPod smem_inv[];
    fx::OpPod *sA = smem_inv;                    // [p][r]: sA[p * 32 + r] = -op(A)(o + r, o + p)
    fx::OpPod *sX = smem_inv + kInvNB * kInvNB;  // [r][c]: x_c(r)
    __shared__ double2 sInvDiag[kInvNB];
    const int64_t o = (int64_t)blockIdx.x * kInvNB;
    const int nb = (int)min((int64_t)kInvNB, na - o);
    for (int idx = threadIdx.x; idx < nb * nb; idx += blockDim.x) {
        const int r = idx % nb, c = idx / nb;
        const dd::real v = opA(A, lda, trans, o + r, o + c);
        fx::Op d = fx::decode(make_double2(v.hi, v.lo));
        d.flags ^= fx::kNeg;   // the substitution subtracts
        sA[c * kInvNB + r] = fx::to_pod(d);
    }
    for (int r = threadIdx.x; r < nb; r += blockDim.x) {
        const dd::real d = opA(A, lda, trans, o + r, o + r);
        const dd::real iv = unit ? dd::make(1.0, 0.0) : dd_div(dd::make(1.0, 0.0), d);
        sInvDiag[r] = make_double2(iv.hi, iv.lo);
    }
    __syncthreads();
    const int c = threadIdx.x / kInvSplit, part = threadIdx.x % kInvSplit;
    const bool active = c < nb;   // every lane stays for the shuffles
    const fx::Op one = fx::decode(make_double2(1.0, 0.0));
    double2 *out = Inv + (int64_t)blockIdx.x * kInvNB * kInvNB + (int64_t)c * kInvNB;
    for (int s = 0; s < nb; ++s) {
        const int r = lower ? s : nb - 1 - s;
        fx::Acc acc;
        acc.reset();
        if (active) {
            if (r == c && part == 0) acc.add_prod(one, one);
            const int p0 = lower ? 0 : r + 1, p1 = lower ? r : nb;
            for (int p = p0 + part; p < p1; p += kInvSplit)
                acc.add_prod(fx::from_pod(sA[p * kInvNB + r]), fx::from_pod(sX[p * kInvNB + c]));
        }
        xfp::XF v = acc.finish();
        v = xfp::xf_add(v, fx::xf_shfl_down(v, 2));   // parts 0 + 2, 1 + 3
        v = xfp::xf_add(v, fx::xf_shfl_down(v, 1));   // (0 + 2) + (1 + 3)
        if (active && part == 0) {
            double h, l;
            xfp::xf_to_dd(v, h, l);
            const dd::real x = dd::mul_fast(dd::make(h, l), dd::load(&sInvDiag[r]));
            sX[r * kInvNB + c] = fx::to_pod(fx::decode(make_double2(x.hi, x.lo)));
            out[r] = make_double2(x.hi, x.lo);
        }
        __syncwarp();   // x_c(r) is read by the column's other three threads (same warp) from the next row on
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

namespace {

constexpr int64_t kTrsmLeaf = 64;

// B[:, :] -= op(A)-block * X (side L) or X * op(A)-block (side R) through the
// engine dispatch.
bool trsm_update(bool left, int64_t m, int64_t n, int64_t k, const void *Ablk, int64_t lda, bool ta,
                 const void *X, int64_t ldx, void *C, int64_t ldc, const char *routine)
{
    GemmArgs g;
    g.alpha = dd_host{-1.0, 0.0};
    g.beta = dd_host{1.0, 0.0};
    g.beta_kind = 1;
    g.m = m;
    g.n = n;
    g.k = k;
    g.C = C;
    g.ldc = ldc;
    if (left) {
        g.A = Ablk; g.lda = lda; g.ta = ta;
        g.B = X; g.ldb = ldx; g.tb = false;
    } else {
        g.A = X; g.lda = ldx; g.ta = false;
        g.B = Ablk; g.ldb = lda; g.tb = ta;
    }
    return run_gemm(g, false, -1, routine);
}

// Recursive substitution on the na x na triangle of op(A) starting at (o, o).
// Side L: B is na x nrhs (rows o..o+na of the caller's B). Side R: B is
// nrhs x na (columns o..o+na). lower refers to op(A).
// Leaf by explicit block inverse: X_blk = Inv_blk * B_blk (side L) or
// B_blk * Inv_blk (side R) as one GEMM into T, copied back into B.
struct TrsmInv {
    const double2 *inv = nullptr;   // inverses of the leaf diagonal blocks, block b at inv + b*nb*nb (ld nb)
    int64_t nb = kTrsmLeaf;         // leaf (and inverse block) order
    double2 *T = nullptr;           // nb x nrhs (or nrhs x nb) scratch
};

bool trsm_leaf_inv(bool left, int64_t o, int64_t na, int64_t nrhs, const TrsmInv &w, double2 *B, int64_t ldb,
                   const char *routine)
{
    GemmArgs g;
    g.alpha = dd_host{1.0, 0.0};
    g.beta = dd_host{0.0, 0.0};
    g.beta_kind = 0;
    const double2 *blk = w.inv + (o / w.nb) * w.nb * w.nb;
    if (left) {
        g.m = na; g.n = nrhs; g.k = na;
        g.A = blk; g.lda = w.nb; g.ta = false;
        g.B = B + o; g.ldb = ldb; g.tb = false;
        g.C = w.T; g.ldc = na;
    } else {
        g.m = nrhs; g.n = na; g.k = na;
        g.A = B + o * ldb; g.lda = ldb; g.ta = false;
        g.B = blk; g.ldb = w.nb; g.tb = false;
        g.C = w.T; g.ldc = nrhs;
    }
    if (!run_gemm(g, false, -1, routine)) return false;
    cudaError_t st = left ? cudaMemcpy2DAsync(B + o, ldb * sizeof(double2), w.T, na * sizeof(double2),
                                              na * sizeof(double2), nrhs, cudaMemcpyDeviceToDevice, stream())
                          : cudaMemcpy2DAsync(B + o * ldb, ldb * sizeof(double2), w.T, nrhs * sizeof(double2),
                                              nrhs * sizeof(double2), na, cudaMemcpyDeviceToDevice, stream());
    return cuda_ok(st, routine, "trsm leaf copy");
}

bool trsm_rec(bool left, bool lower, bool trans, bool unit, int64_t o, int64_t na, int64_t nrhs, const void *A,
              int64_t lda, double2 *B, int64_t ldb, const TrsmInv &w, const char *routine)
{
    const int64_t leaf = w.inv ? w.nb : kTrsmLeaf;
    if (na <= leaf && w.inv) return trsm_leaf_inv(left, o, na, nrhs, w, B, ldb, routine);
    if (na <= leaf) {
        if (left)
            k_trsm_diag_left<<<blocks_for(nrhs, 64), 64, 0, stream()>>>(o, (int)na, nrhs, (const double2 *)A, lda,
                                                                      trans, lower, unit, B, ldb);
        else
            k_trsm_diag_right<<<blocks_for(nrhs, 64), 64, 0, stream()>>>(o, (int)na, nrhs, (const double2 *)A, lda,
                                                                       trans, !lower, unit, B, ldb);
        count_launch();
        return true;
    }
    int64_t h = (na / 2 + leaf - 1) / leaf * leaf;
    if (h >= na) h = na - leaf;
    const int64_t o1 = o, n1 = h, o2 = o + h, n2 = na - h;
    if (left) {
        // rows of B: first block B1 = rows o1.., second B2 = rows o2..
        if (lower) {
            if (!trsm_rec(true, lower, trans, unit, o1, n1, nrhs, A, lda, B, ldb, w, routine)) return false;
            // B2 -= op(A)[o2:, o1:o1+n1] * X1
            if (!trsm_update(true, n2, nrhs, n1, op_block(A, lda, trans, o2, o1), lda, trans, B + o1, ldb, B + o2,
                             ldb, routine))
                return false;
            return trsm_rec(true, lower, trans, unit, o2, n2, nrhs, A, lda, B, ldb, w, routine);
        }
        if (!trsm_rec(true, lower, trans, unit, o2, n2, nrhs, A, lda, B, ldb, w, routine)) return false;
        // B1 -= op(A)[o1:o1+n1, o2:] * X2
        if (!trsm_update(true, n1, nrhs, n2, op_block(A, lda, trans, o1, o2), lda, trans, B + o2, ldb, B + o1, ldb,
                         routine))
            return false;
        return trsm_rec(true, lower, trans, unit, o1, n1, nrhs, A, lda, B, ldb, w, routine);
    }
    // side R: columns of B; op(A) upper -> left block first
    const bool upper = !lower;
    if (upper) {
        if (!trsm_rec(false, lower, trans, unit, o1, n1, nrhs, A, lda, B, ldb, w, routine)) return false;
        // B2 -= X1 * op(A)[o1:o1+n1, o2:]
        if (!trsm_update(false, nrhs, n2, n1, op_block(A, lda, trans, o1, o2), lda, trans, B + o1 * ldb, ldb,
                         B + o2 * ldb, ldb, routine))
            return false;
        return trsm_rec(false, lower, trans, unit, o2, n2, nrhs, A, lda, B, ldb, w, routine);
    }
    if (!trsm_rec(false, lower, trans, unit, o2, n2, nrhs, A, lda, B, ldb, w, routine)) return false;
    // B1 -= X2 * op(A)[o2:, o1:o1+n1]
    if (!trsm_update(false, nrhs, n1, n2, op_block(A, lda, trans, o2, o1), lda, trans, B + o2 * ldb, ldb,
                     B + o1 * ldb, ldb, routine))
        return false;
    return trsm_rec(false, lower, trans, unit, o1, n1, nrhs, A, lda, B, ldb, w, routine);
}

// Copies the two half-block inverses into the diagonal of each merged block
// and zeroes its off-diagonal triangle (upper right for lower, lower left for
// upper). CTAs (merged block, 32-column group).
__global__ void k_inv_merge_copy(int64_t na, int64_t S, const double2 *__restrict__ src, double2 *__restrict__ dst,
                                 bool lower)
{
    const int64_t h = S / 2;
    const int64_t o = (int64_t)blockIdx.x * S;
    const int64_t n1 = min(h, na - o), n2 = max((int64_t)0, min(h, na - o - h));
    const double2 *i1 = src + (2 * blockIdx.x) * h * h;
    const double2 *i2 = src + (2 * blockIdx.x + 1) * h * h;
    double2 *d = dst + (int64_t)blockIdx.x * S * S;
    const int nt = (int)(n1 + n2), n1i = (int)n1, hi = (int)h, Si = (int)S;
    // column per warp-strided loop, rows across the threads of a warp (coalesced)
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int cend = min(nt, (int)(blockIdx.y + 1) * 32);
    for (int c = (int)blockIdx.y * 32 + wid; c < cend; c += nw) {
        for (int r = lane; r < nt; r += 32) {
            double2 v = make_double2(0.0, 0.0);
            if (r < n1i && c < n1i) v = i1[r + c * hi];
            else if (r >= n1i && c >= n1i) v = i2[(r - n1i) + (c - n1i) * hi];
            d[r + c * Si] = v;   // the off-diagonal block is then written by the GEMMs
        }
    }
    (void)lower;
}

// Doubles the order of the diagonal-block inverses from h to 2h:
//   lower: inv [L11 0; L21 L22] = [I1 0; -I2 L21 I1  I2]
//   upper: inv [U11 U12; 0 U22] = [I1 -I1 U12 I2; 0  I2]
// with two grouped GEMMs over all merged blocks.
bool trsm_merge_inverses(int64_t na, int64_t h, const void *A, int64_t lda, bool trans, bool lower,
                         const double2 *src, double2 *dst, double2 *tmp, const char *routine)
{
    const int64_t S = 2 * h;
    const int64_t nblk = (na + S - 1) / S;
    k_inv_merge_copy<<<dim3((unsigned)nblk, (unsigned)((S + 31) / 32)), 256, 0, stream()>>>(na, S, src, dst, lower);
    count_launch();
    std::vector<int64_t> m1, n1, k1, lda1, ldb1, ldc1, m2, n2, k2, lda2, ldb2, ldc2;
    std::vector<const mwblas_real64x2 *> a1, b1, a2, b2;
    std::vector<mwblas_real64x2 *> c1, c2;
    std::vector<char> t1a, t1b, t2a, t2b;
    for (int64_t b = 0; b < nblk; ++b) {
        const int64_t o = b * S;
        const int64_t p1 = std::min(h, na - o), p2 = std::max((int64_t)0, std::min(h, na - o - h));
        if (p2 == 0) continue;
        const double2 *I1 = src + (2 * b) * h * h, *I2 = src + (2 * b + 1) * h * h;
        double2 *T = tmp + b * h * h;
        double2 *D = dst + b * S * S;
        if (lower) {
            // T = L21 * I1 (p2 x p1), off = -(I2 * T) into D[p1:, 0:p1]
            t1a.push_back(trans ? 'T' : 'N'); t1b.push_back('N');
            m1.push_back(p2); n1.push_back(p1); k1.push_back(p1);
            a1.push_back((const mwblas_real64x2 *)op_block(A, lda, trans, o + p1, o)); lda1.push_back(lda);
            b1.push_back((const mwblas_real64x2 *)I1); ldb1.push_back(h);
            c1.push_back((mwblas_real64x2 *)T); ldc1.push_back(h);
            t2a.push_back('N'); t2b.push_back('N');
            m2.push_back(p2); n2.push_back(p1); k2.push_back(p2);
            a2.push_back((const mwblas_real64x2 *)I2); lda2.push_back(h);
            b2.push_back((const mwblas_real64x2 *)T); ldb2.push_back(h);
            c2.push_back((mwblas_real64x2 *)(D + p1)); ldc2.push_back(S);
        } else {
            // T = U12 * I2 (p1 x p2), off = -(I1 * T) into D[0:p1, p1:]
            t1a.push_back(trans ? 'T' : 'N'); t1b.push_back('N');
            m1.push_back(p1); n1.push_back(p2); k1.push_back(p2);
            a1.push_back((const mwblas_real64x2 *)op_block(A, lda, trans, o, o + p1)); lda1.push_back(lda);
            b1.push_back((const mwblas_real64x2 *)I2); ldb1.push_back(h);
            c1.push_back((mwblas_real64x2 *)T); ldc1.push_back(h);
            t2a.push_back('N'); t2b.push_back('N');
            m2.push_back(p1); n2.push_back(p2); k2.push_back(p1);
            a2.push_back((const mwblas_real64x2 *)I1); lda2.push_back(h);
            b2.push_back((const mwblas_real64x2 *)T); ldb2.push_back(h);
            c2.push_back((mwblas_real64x2 *)(D + p1 * S)); ldc2.push_back(S);
        }
    }
    const int64_t cnt = (int64_t)m1.size();
    if (cnt == 0) return true;
    std::vector<mwblas_real64x2> one((size_t)cnt, mwblas_real64x2{{1.0, 0.0}}),
        mone((size_t)cnt, mwblas_real64x2{{-1.0, 0.0}}), zero((size_t)cnt, mwblas_real64x2{{0.0, 0.0}});
    // merges of 128 x 128 blocks and larger run on the tensor cores
    const int tensor_min = h >= 128 && ozaki_available() ? 128 : 0;
    if (!grouped_gemm_device(cnt, t1a.data(), t1b.data(), m1.data(), n1.data(), k1.data(), one.data(), a1.data(),
                             lda1.data(), b1.data(), ldb1.data(), zero.data(), c1.data(), ldc1.data(), tensor_min,
                             routine))
        return false;
    return grouped_gemm_device(cnt, t2a.data(), t2b.data(), m2.data(), n2.data(), k2.data(), mone.data(), a2.data(),
                               lda2.data(), b2.data(), ldb2.data(), zero.data(), c2.data(), ldc2.data(), tensor_min,
                               routine);
}

}  // namespace

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
    const bool left = (side == 'L');
    const int64_t na = left ? m : n, nrhs = left ? n : m;
    // Many right-hand sides, or a large triangle: invert the diagonal blocks
    // once (one launch) and apply them as GEMMs; otherwise substitute
    // directly (a substitution leaf runs a thread per right-hand side, so
    // with few of them it is latency-bound: TRSV at n = 1024 took 27 ms).
    TrsmInv w;
    void *scratch = nullptr;
    bool ok = true;
    if (nrhs >= 2 * kTrsmLeaf || na >= 128) {
        // leaf order 64, or 256 when the right-hand sides make the leaf GEMMs
        // worth it or there are only a few of them; the 32 x 32 inverses are
        // doubled up to it by merging with grouped GEMMs
        // (512 for large triangles with many right-hand sides: half the GEMMs
        // of 256 leaves, the two extra merge levels on the tensor cores;
        // 1024 from na = 4096: 7 instead of 15 GEMMs for one more merge level)
        const bool big = nrhs >= 512 && ozaki_available();
        const int64_t nb = (na >= 4096 && big)                                       ? 1024
                           : (na >= 2048 && big)                                     ? 512
                           : (na >= 1024 && (nrhs >= 256 || nrhs < 2 * kTrsmLeaf)) ? 256
                                                                                    : kTrsmLeaf;
        const int64_t nblk64 = (na + kInvNB - 1) / kInvNB;
        const int64_t nblk = (na + nb - 1) / nb;
        const size_t inv64_bytes = (size_t)nblk64 * kInvNB * kInvNB * sizeof(double2);
        const size_t inv_bytes = (size_t)nblk * nb * nb * sizeof(double2);
        const size_t t_bytes = (size_t)nb * nrhs * sizeof(double2);
        // the merges' products: ceil(na / 2h) blocks of h x h at each level h
        size_t m_elems = 0;
        for (int64_t h = kInvNB; h < nb; h *= 2)
            m_elems = std::max(m_elems, (size_t)((na + 2 * h - 1) / (2 * h)) * h * h);
        const size_t m_bytes = (m_elems * sizeof(double2) + 255) / 256 * 256;
        // [inverse buffer A][inverse buffer B][merge products][T]: merges ping-pong between A and B
        const size_t buf_bytes = (std::max(inv64_bytes, inv_bytes) + 255) / 256 * 256;
        scratch = dev_alloc(2 * buf_bytes + m_bytes + t_bytes, routine);
        if (!scratch) return false;
        double2 *bufA = (double2 *)scratch, *bufB = (double2 *)((char *)scratch + buf_bytes);
        double2 *mtmp = (double2 *)((char *)scratch + 2 * buf_bytes);
        w.T = (double2 *)((char *)scratch + 2 * buf_bytes + m_bytes);
        const size_t smem = 2 * (size_t)kInvNB * kInvNB * sizeof(fx::OpPod);
        cudaFuncSetAttribute(k_trsm_diag_inv, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        k_trsm_diag_inv<<<(unsigned)nblk64, kInvNB * kInvSplit, smem, stream()>>>(na, (const double2 *)A, lda, trans, lower,
                                                                     unit, bufA);
        count_launch();
        double2 *cur = bufA, *nxt = bufB;
        for (int64_t h = kInvNB; h < nb && ok; h *= 2) {
                ok = trsm_merge_inverses(na, h, A, lda, trans, lower, cur, nxt, mtmp, routine);
            std::swap(cur, nxt);
        }
        w.inv = cur;
        w.nb = nb;
    }
    if (ok) ok = trsm_rec(left, lower, trans, unit, 0, na, nrhs, A, lda, b, ldb, w, routine);
    if (scratch) dev_free(scratch);
    return ok;
}

void launch_zero_matrix(int64_t m, int64_t n, void *B, int64_t ldb)
{
    launch_scale_matrix(m, n, dd_host{0.0, 0.0}, 0, B, ldb, 0);
}

}  // namespace mw
