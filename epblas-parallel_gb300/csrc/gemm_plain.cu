// Plain double-double GEMM on the FP64 pipe ("FP64-EFT" engine).
//
// Computes C := alpha*op(A)*op(B) + beta*C for the reference's mgemm_
// (multifloats/mgemm_parallel.cpp:44-187) and, in the complex kernel below,
// wgemm_ (wgemm_parallel.cpp:44-194).
//
// Arithmetic. The reference accumulates every product with a full fast DD
// multiply and a full fast DD add, 18 FP64 instructions per multiply-add
// (mgemm_serial.cpp:249-269 over mf_simd_fast.h:79-102). On GB300 the FP64
// pipe is the scarce resource, so this kernel accumulates with the
// error-free "extraction" transformation of Rump, Ogita and Oishi (SIAM J.
// Sci. Comput. 31(1), 2008, ExtractScalar): with sigma = 1.5 * 2^E chosen so
// that every partial sum of a K-block stays below 2^(E-1) in magnitude, the
// running value X = sigma + S lives in one binade, so
//     t = fl(X + a.hi*b.hi)          (one FMA)
//     q = X - t                      (exact, Sterbenz)
//     r = fl(a.hi*b.hi + q)          (one FMA; the part of the product below ulp(sigma))
// moves the high part of every product into X exactly and leaves a residual r
// of at most ulp(sigma)/2. The residual and the two cross products
// a.hi*b.lo + a.lo*b.hi go to a plain double L. Every KB products, X - sigma
// (exact) and L are folded into a double-double accumulator. That is 6 FP64
// instructions per multiply-add plus 12 per fold.
//
// sigma is per output element: 2^E >= 16*KB*2^(ea_i + eb_j), where ea_i and eb_j
// bound the binary exponents of row i of op(A) and column j of op(B)
// (computed by the exponent pre-pass below). The result is normwise accurate:
// |C - C_exact| <= ~(3*KB^2 + 4) * 2^-104 * |alpha| * k * max|A| * max|B|
// in the worst case, independent of k, and ~2^-106 relative in typical use;
// the reference's own fuzz tolerance is max(10, 4k) * 2^-104 of the same norm
// (fuzz_mgemm.fypp tolerance line).
#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <atomic>
#include <string>

#include "dd.cuh"
#include "gemm.h"
#include "runtime.h"
#include "sm100.cuh"

namespace mw {

namespace {

constexpr int kNoExp = -30000;   // row/column with no nonzero entry

__device__ __forceinline__ int exp_bound(double x)
{
    // |x| < 2^(e+1) with e = biased exponent - 1023 (subnormals use -1023).
    uint64_t b = (uint64_t)__double_as_longlong(x) & 0x7fffffffffffffffull;
    if (b == 0) return kNoExp;
    return (int)(b >> 52) - 1023;
}

// Binary exponent of the lowest set bit of the double-double value hi + lo
// (kLowNone for zero). With |lo| <= ulp(hi)/2, lo's lowest bit lies below
// hi's, so it is lo's when lo != 0. Non-finite values give kLowNone too (their
// rows are NaN in the output whatever the width).
constexpr int kLowNone = 0x3f3f3f3f;   // also the byte-wise memset value below
// A row holding one entry that alone spans >= 104 bits (hi's top bit to lo's
// lowest) needs the full width whatever the rest holds: its low bound is set
// to this, and its remaining entries are not examined.
constexpr int kLowFull = -(1 << 28);
__device__ __forceinline__ int low_bit(double2 v)
{
    // 32-bit words only (64-bit shifts and bit scans issue at the FP64 rate here)
    uint32_t w1 = (uint32_t)__double2hiint(v.y) & 0x7fffffffu, w0 = (uint32_t)__double2loint(v.y);
    if ((w1 | w0) == 0) {
        w1 = (uint32_t)__double2hiint(v.x) & 0x7fffffffu;
        w0 = (uint32_t)__double2loint(v.x);
    }
    const uint32_t bx = w1 >> 20;
    if ((w1 | w0) == 0 || bx == 0x7ffu) return kLowNone;
    const uint32_t mh = (w1 & 0xfffffu) | (bx ? 0x100000u : 0u);
    const int tz = w0 ? __ffs((int)w0) - 1 : 32 + __ffs((int)mh) - 1;
    return (bx ? (int)bx : 1) - 1075 + tz;
}

// Row exponent bound of a column-major matrix M (rows x cols, ld): out[i] =
// max over j of exp_bound(M[i + j*ld].hi); with `low`, also low[i] = min over
// j of low_bit(M[i + j*ld]). Thread per row, grid.y splits the columns;
// combined with atomicMax / atomicMin.
__global__ void k_exp_rows(int64_t rows, int64_t cols, const double2 *M, int64_t ld, int elem2, int *out,
                           int64_t cols_per_y, int *low)
{
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= rows) return;
    int64_t j0 = blockIdx.y * cols_per_y;
    int64_t j1 = min(cols, j0 + cols_per_y);
    int e = kNoExp, lb = kLowNone;
    if (low) {
#pragma unroll 4
        for (int64_t j = j0; j < j1; ++j) {
            const double2 *p = M + elem2 * (i + j * ld);
            for (int w = 0; w < elem2; ++w) {
                const double2 v = p[w];
                const int ev = exp_bound(v.x);
                e = max(e, ev);
                if (lb != kLowFull) {
                    const int lv = low_bit(v);
                    lb = (lv != kLowNone && ev - lv >= 104) ? kLowFull : min(lb, lv);
                }
            }
        }
        atomicMin(low + i, lb);
    } else {
#pragma unroll 8
        for (int64_t j = j0; j < j1; ++j) {
            const double2 *p = M + elem2 * (i + j * ld);
            for (int w = 0; w < elem2; ++w) e = max(e, exp_bound(p[w].x));
        }
    }
    atomicMax(out + i, e);
}

// Column exponent bound: out[j] = max over i of exp_bound(M[i + j*ld].hi)
// (and low[j] = min of low_bit). Warp per column (or per rows_per-long piece
// of a column along grid.y, combined with atomics), lanes stride down the
// contiguous column.
__global__ void k_exp_cols(int64_t rows, int64_t cols, const double2 *M, int64_t ld, int elem2, int *out, int *low,
                           int64_t rows_per)
{
    int64_t j = blockIdx.x * (int64_t)(blockDim.x / 32) + threadIdx.x / 32;
    int lane = threadIdx.x & 31;
    if (j >= cols) return;
    int e = kNoExp, lb = kLowNone;
    const int64_t i1 = min(rows, (int64_t)(blockIdx.y + 1) * rows_per);
    for (int64_t i = (int64_t)blockIdx.y * rows_per + lane; i < i1; i += 32) {
        const double2 *p = M + elem2 * (i + j * ld);
        for (int w = 0; w < elem2; ++w) {
            const double2 v = p[w];
            const int ev = exp_bound(v.x);
            e = max(e, ev);
            if (low && lb != kLowFull) {
                const int lv = low_bit(v);
                lb = (lv != kLowNone && ev - lv >= 104) ? kLowFull : min(lb, lv);
            }
        }
    }
    for (int off = 16; off > 0; off >>= 1) {
        e = max(e, __shfl_down_sync(0xffffffffu, e, off));
        lb = min(lb, __shfl_down_sync(0xffffffffu, lb, off));
    }
    if (lane == 0) {
        if (gridDim.y == 1) {
            out[j] = e;
            if (low) low[j] = lb;
        } else {
            atomicMax(out + j, e);
            if (low) atomicMin(low + j, lb);
        }
    }
}

// Exponent offset of sigma above ea + eb: a fold block holds at most
// terms = min(KB, k) * per_step products, each below 2^(ea+eb+2), so with
// 2^lg >= terms and sigma = 1.5 * 2^(ea+eb+lg+3) every partial sum stays below
// 2^(E-1) and X stays inside (2^E, 2^(E+1)): the fold's X - sigma is exact
// (Sterbenz) and every extracted remainder is at most ulp(X)/2.
int sigma_shift(int KB, int64_t k, int per_step)
{
    int64_t terms = (k < KB ? k : KB) * per_step;
    int lg = 0;
    while (((int64_t)1 << lg) < terms) ++lg;
    return lg + 3;
}

// Products with k at most this use the second extraction level (X2 below):
// at small k the reference's tolerance, max(10, 4k) * 2^-104 normwise, is
// tighter than the ~2^(shift-106) * |max product| rounding of the one-level
// remainder accumulator.
constexpr int64_t kCompMaxK = 64;

__device__ __forceinline__ double make_sigma(int ea, int eb, int shift)
{
    int e;
    if (ea <= kNoExp / 2 || eb <= kNoExp / 2)
        e = -1000;
    else
        e = ea + eb + shift;
    e = max(-1000, min(1000, e));
    uint64_t bits = ((uint64_t)(e + 1023) << 52) | (1ull << 51);   // 1.5 * 2^e
    return __longlong_as_double((long long)bits);
}

// Second-level sigma for the extracted remainders r (|r| <= 2^(E-53), at most
// 2^lg = 2^(shift-3) of them per fold): 1.5 * 2^(E - 51 + lg) keeps their
// running sum inside the binade, so each X2 + r is split exactly (Fast2Sum)
// and only remainders below ulp(X2)/2 reach L.
__device__ __forceinline__ double make_sigma2(int ea, int eb, int shift)
{
    return make_sigma(ea, eb, 2 * shift - 54);
}

template <int BM, int BN, int TM, int TN, bool TA, bool TB, int KB>
__global__ void __launch_bounds__((BM / TM) * (BN / TN))
    k_gemm_plain(int64_t m, int64_t n, int64_t k, dd::real alpha, const double2 *__restrict__ A, int64_t lda,
                 const double2 *__restrict__ B, int64_t ldb, dd::real beta, int beta_kind, double2 *C, int64_t ldc,
                 const int *__restrict__ ea, const int *__restrict__ eb, int uplo, int SHIFT, int COMP)
{
    constexpr int NTX = BM / TM;   // threads along rows
    constexpr int NTY = BN / TN;   // threads along columns
    constexpr int NT = NTX * NTY;
    constexpr int BK = 8;
    static_assert(KB % BK == 0, "fold interval must be a multiple of the k-slab");

    __shared__ double2 sA[BK][BM];
    __shared__ double2 sB[BK][BN];

    const int tid = threadIdx.x;
    const int tx = tid % NTX, ty = tid / NTX;
    const int64_t i0 = (int64_t)blockIdx.x * BM, j0 = (int64_t)blockIdx.y * BN;
    // Triangular output (SYRK): skip tiles wholly outside the stored triangle.
    if ((uplo == 1 && i0 > j0 + BN - 1) || (uplo == 2 && i0 + BM - 1 < j0)) return;

    int eai[TM], ebj[TN];
#pragma unroll
    for (int a = 0; a < TM; ++a) {
        int64_t i = i0 + tx + a * NTX;
        eai[a] = (i < m) ? ea[i] : kNoExp;
    }
#pragma unroll
    for (int b = 0; b < TN; ++b) {
        int64_t j = j0 + ty + b * NTY;
        ebj[b] = (j < n) ? eb[j] : kNoExp;
    }

    double X[TM][TN], X2[TM][TN], L[TM][TN], Ah[TM][TN], Al[TM][TN];
#pragma unroll
    for (int a = 0; a < TM; ++a)
#pragma unroll
        for (int b = 0; b < TN; ++b) {
            X[a][b] = make_sigma(eai[a], ebj[b], SHIFT);
            X2[a][b] = make_sigma2(eai[a], ebj[b], SHIFT);
            L[a][b] = 0.0;
            Ah[a][b] = 0.0;
            Al[a][b] = 0.0;
        }

    int since_fold = 0;
    for (int64_t kk = 0; kk < k; kk += BK) {
        // ---- stage op(A)[i0:i0+BM, kk:kk+BK] and op(B)[kk:kk+BK, j0:j0+BN]
        for (int idx = tid; idx < BM * BK; idx += NT) {
            int r, p;
            if (!TA) { r = idx % BM; p = idx / BM; }      // A col-major: rows contiguous
            else     { p = idx % BK; r = idx / BK; }      // A^T: k contiguous
            int64_t gi = i0 + r, gp = kk + p;
            double2 v = make_double2(0.0, 0.0);
            if (gi < m && gp < k) v = TA ? A[gp + gi * lda] : A[gi + gp * lda];
            sA[p][r] = v;
        }
        for (int idx = tid; idx < BN * BK; idx += NT) {
            int c, p;
            if (!TB) { p = idx % BK; c = idx / BK; }      // B col-major: k contiguous
            else     { c = idx % BN; p = idx / BN; }      // B^T: columns contiguous
            int64_t gj = j0 + c, gp = kk + p;
            double2 v = make_double2(0.0, 0.0);
            if (gj < n && gp < k) v = TB ? B[gj + gp * ldb] : B[gp + gj * ldb];
            sB[p][c] = v;
        }
        __syncthreads();

#pragma unroll
        for (int p = 0; p < BK; ++p) {
            double2 av[TM], bv[TN];
#pragma unroll
            for (int a = 0; a < TM; ++a) av[a] = sA[p][tx + a * NTX];
#pragma unroll
            for (int b = 0; b < TN; ++b) bv[b] = sB[p][ty + b * NTY];
#pragma unroll
            for (int a = 0; a < TM; ++a)
#pragma unroll
                for (int b = 0; b < TN; ++b) {
                    double t = __fma_rn(av[a].x, bv[b].x, X[a][b]);
                    double q = __dsub_rn(X[a][b], t);
                    double r = __fma_rn(av[a].x, bv[b].x, q);
                    X[a][b] = t;
                    if (COMP) {
                        double t2 = __dadd_rn(X2[a][b], r);
                        double q2 = __dsub_rn(X2[a][b], t2);
                        r = __dadd_rn(q2, r);
                        X2[a][b] = t2;
                    }
                    double l = __dadd_rn(L[a][b], r);
                    l = __fma_rn(av[a].x, bv[b].y, l);
                    L[a][b] = __fma_rn(av[a].y, bv[b].x, l);
                }
        }
        __syncthreads();

        since_fold += BK;
        if (since_fold == KB || kk + BK >= k) {
            since_fold = 0;
#pragma unroll
            for (int a = 0; a < TM; ++a)
#pragma unroll
                for (int b = 0; b < TN; ++b) {
                    double sg = make_sigma(eai[a], ebj[b], SHIFT);
                    double s = __dsub_rn(X[a][b], sg);   // exact
                    double lsum = L[a][b];
                    if (COMP) {
                        double sg2 = make_sigma2(eai[a], ebj[b], SHIFT);
                        lsum = __dadd_rn(lsum, __dsub_rn(X2[a][b], sg2));
                        X2[a][b] = sg2;
                    }
                    double h, e;
                    dd::two_sum(Ah[a][b], s, h, e);
                    double lo = __dadd_rn(Al[a][b], __dadd_rn(e, lsum));
                    dd::fast_two_sum(h, lo, Ah[a][b], Al[a][b]);
                    X[a][b] = sg;
                    L[a][b] = 0.0;
                }
        }
    }

    // ---- epilogue: C = alpha*acc (+ beta*C) with the reference's operator
    // choices: fast multiply by alpha (mgemm_serial.cpp:173-191), scalar add
    // into C, scalar multiply for the beta pre-scale (mgemm_parallel.cpp:68-77).
#pragma unroll
    for (int b = 0; b < TN; ++b) {
        int64_t j = j0 + ty + b * NTY;
        if (j >= n) continue;
#pragma unroll
        for (int a = 0; a < TM; ++a) {
            int64_t i = i0 + tx + a * NTX;
            if (i >= m) continue;
            if ((uplo == 1 && i > j) || (uplo == 2 && i < j)) continue;
            dd::real acc = dd::make(Ah[a][b], Al[a][b]);
            dd::real r = dd::mul_fast(alpha, acc);
            double2 *pc = C + i + j * ldc;
            if (beta_kind == 0) {
                dd::store(pc, r);
            } else {
                dd::real c0 = dd::load(pc);
                if (beta_kind == 2) c0 = dd::mul_exact(c0, beta);
                dd::store(pc, dd::add_exact(c0, r));
            }
        }
    }
}

// ---- the same kernel with TMA-staged operand tiles ---------------------------------------
//
// One thread issues 2-D tensor copies (cp.async.bulk.tensor) of the next
// k-slabs of op(A) and op(B) into a ring of NS shared-memory stages while all
// threads run the extraction MACs on the current one; completion is counted
// on one mbarrier per stage. The tensor maps describe A and B as 2-D arrays of
// doubles (a double-double is two consecutive doubles) bounded by the operand
// sizes, so slabs past m, n or k are filled with zeros by the copy engine
// instead of by per-element bounds checks. A tile arrives in the storage order
// of its operand: op(A) = A and op(B) = B^T stage as [k][row] (rows
// contiguous), op(A) = A^T and op(B) = B as [row][k]. The arithmetic, its
// order and hence the results are those of k_gemm_plain, bit for bit.
//
// Every wait is bounded (sm100::mbar_wait); when one gives up, the whole
// block leaves the k loop together (__syncthreads_or), the issuing thread
// waits for the copies it still has in flight, and the routine reports
// MWBLAS_ERR_TIMEOUT at its synchronisation.
template <int BM, int BN, int TM, int TN, bool TA, bool TB, int KB, int NS, bool COMP>
__global__ void __launch_bounds__((BM / TM) * (BN / TN))
    k_gemm_plain_tma(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapB, int64_t m,
                     int64_t n, int64_t k, dd::real alpha, dd::real beta, int beta_kind, double2 *C, int64_t ldc,
                     const int *__restrict__ ea, const int *__restrict__ eb, int uplo, int SHIFT, int *status)
{
    constexpr int NTX = BM / TM;
    constexpr int NTY = BN / TN;
    constexpr int BK = 8;
    constexpr uint32_t A_BYTES = BM * BK * 16, B_BYTES = BN * BK * 16;
    static_assert(KB % BK == 0, "fold interval must be a multiple of the k-slab");

    extern __shared__ __align__(128) unsigned char plain_smem_raw[];
    // stages on a 128-byte boundary (the launch reserves 128 bytes for this)
    unsigned char *plain_smem = (unsigned char *)(((uintptr_t)plain_smem_raw + 127) & ~(uintptr_t)127);
    double2 *sA = reinterpret_cast<double2 *>(plain_smem);                   // [NS][BM * BK]
    double2 *sB = reinterpret_cast<double2 *>(plain_smem + NS * A_BYTES);    // [NS][BN * BK]
    uint64_t *full = reinterpret_cast<uint64_t *>(plain_smem + NS * (A_BYTES + B_BYTES));

    const int tid = threadIdx.x;
    const int tx = tid % NTX, ty = tid / NTX;
    const int64_t i0 = (int64_t)blockIdx.x * BM, j0 = (int64_t)blockIdx.y * BN;
    if ((uplo == 1 && i0 > j0 + BN - 1) || (uplo == 2 && i0 + BM - 1 < j0)) return;

    const int nslabs = (int)((k + BK - 1) / BK);
    if (tid == 0) {
        sm100::tma_prefetch_desc(&mapA);
        sm100::tma_prefetch_desc(&mapB);
        for (int st = 0; st < NS; ++st) sm100::mbar_init(&full[st], 1);
        sm100::fence_mbar_init();
    }
    __syncthreads();
    // slab t into stage t % NS: A at (x, y) = (2 i0, k0) or (2 k0, i0), B likewise
    auto issue = [&](int t) {
        const int st = t % NS;
        const int32_t k0 = t * BK;
        sm100::mbar_arrive_expect_tx(&full[st], A_BYTES + B_BYTES);
        if (!TA) sm100::tma_load_2d(sA + st * (BM * BK), &mapA, &full[st], (int32_t)(2 * i0), k0);
        else sm100::tma_load_2d(sA + st * (BM * BK), &mapA, &full[st], 2 * k0, (int32_t)i0);
        if (TB) sm100::tma_load_2d(sB + st * (BN * BK), &mapB, &full[st], (int32_t)(2 * j0), k0);
        else sm100::tma_load_2d(sB + st * (BN * BK), &mapB, &full[st], 2 * k0, (int32_t)j0);
    };
    if (tid == 0)
        for (int t = 0; t < NS - 1 && t < nslabs; ++t) issue(t);

    int eai[TM], ebj[TN];
#pragma unroll
    for (int a = 0; a < TM; ++a) {
        int64_t i = i0 + tx + a * NTX;
        eai[a] = (i < m) ? ea[i] : kNoExp;
    }
#pragma unroll
    for (int b = 0; b < TN; ++b) {
        int64_t j = j0 + ty + b * NTY;
        ebj[b] = (j < n) ? eb[j] : kNoExp;
    }

    // X2 (the second extraction level) only exists in the short-k kernel
    double X[TM][TN], X2[COMP ? TM : 1][COMP ? TN : 1], L[TM][TN], Ah[TM][TN], Al[TM][TN];
#pragma unroll
    for (int a = 0; a < TM; ++a)
#pragma unroll
        for (int b = 0; b < TN; ++b) {
            X[a][b] = make_sigma(eai[a], ebj[b], SHIFT);
            if (COMP) X2[COMP ? a : 0][COMP ? b : 0] = make_sigma2(eai[a], ebj[b], SHIFT);
            L[a][b] = 0.0;
            Ah[a][b] = 0.0;
            Al[a][b] = 0.0;
        }

    int since_fold = 0, issued = min(NS - 1, nslabs), t = 0;
    bool failed = false;
    for (; t < nslabs; ++t) {
        // the stage of slab t - 1 was released by the barrier that ended the
        // previous iteration: refill it with slab t + NS - 1
        if (tid == 0 && t + NS - 1 < nslabs) {
            issue(t + NS - 1);
            issued = t + NS;
        }
        const int st = t % NS;
        const bool ok = sm100::mbar_wait(&full[st], (uint32_t)(t / NS) & 1u, status, 5);
        if (__syncthreads_or(!ok)) {
            failed = true;
            break;
        }
        const double2 *tA = sA + st * (BM * BK);
        const double2 *tB = sB + st * (BN * BK);
#pragma unroll
        for (int p = 0; p < BK; ++p) {
            double2 av[TM], bv[TN];
#pragma unroll
            for (int a = 0; a < TM; ++a) av[a] = TA ? tA[(tx + a * NTX) * BK + p] : tA[p * BM + tx + a * NTX];
#pragma unroll
            for (int b = 0; b < TN; ++b) bv[b] = TB ? tB[p * BN + ty + b * NTY] : tB[(ty + b * NTY) * BK + p];
#pragma unroll
            for (int a = 0; a < TM; ++a)
#pragma unroll
                for (int b = 0; b < TN; ++b) {
                    double tt = __fma_rn(av[a].x, bv[b].x, X[a][b]);
                    double q = __dsub_rn(X[a][b], tt);
                    double r = __fma_rn(av[a].x, bv[b].x, q);
                    X[a][b] = tt;
                    if (COMP) {
                        double &x2 = X2[COMP ? a : 0][COMP ? b : 0];
                        double t2 = __dadd_rn(x2, r);
                        double q2 = __dsub_rn(x2, t2);
                        r = __dadd_rn(q2, r);
                        x2 = t2;
                    }
                    double l = __dadd_rn(L[a][b], r);
                    l = __fma_rn(av[a].x, bv[b].y, l);
                    L[a][b] = __fma_rn(av[a].y, bv[b].x, l);
                }
        }
        __syncthreads();   // stage st is free for the refill at the top of iteration t + 1

        since_fold += BK;
        if (since_fold == KB || t + 1 == nslabs) {
            since_fold = 0;
#pragma unroll
            for (int a = 0; a < TM; ++a)
#pragma unroll
                for (int b = 0; b < TN; ++b) {
                    double sg = make_sigma(eai[a], ebj[b], SHIFT);
                    double s = __dsub_rn(X[a][b], sg);   // exact
                    double lsum = L[a][b];
                    if (COMP) {
                        double &x2 = X2[COMP ? a : 0][COMP ? b : 0];
                        double sg2 = make_sigma2(eai[a], ebj[b], SHIFT);
                        lsum = __dadd_rn(lsum, __dsub_rn(x2, sg2));
                        x2 = sg2;
                    }
                    double h, e;
                    dd::two_sum(Ah[a][b], s, h, e);
                    double lo = __dadd_rn(Al[a][b], __dadd_rn(e, lsum));
                    dd::fast_two_sum(h, lo, Ah[a][b], Al[a][b]);
                    X[a][b] = sg;
                    L[a][b] = 0.0;
                }
        }
    }
    if (failed) {
        // never leave with copies in flight: the slabs issued but not consumed
        if (tid == 0)
            for (int u = t; u < issued; ++u) sm100::mbar_wait(&full[u % NS], (uint32_t)(u / NS) & 1u, nullptr, 0);
        return;
    }

#pragma unroll
    for (int b = 0; b < TN; ++b) {
        int64_t j = j0 + ty + b * NTY;
        if (j >= n) continue;
#pragma unroll
        for (int a = 0; a < TM; ++a) {
            int64_t i = i0 + tx + a * NTX;
            if (i >= m) continue;
            if ((uplo == 1 && i > j) || (uplo == 2 && i < j)) continue;
            dd::real acc = dd::make(Ah[a][b], Al[a][b]);
            dd::real r = dd::mul_fast(alpha, acc);
            double2 *pc = C + i + j * ldc;
            if (beta_kind == 0) {
                dd::store(pc, r);
            } else {
                dd::real c0 = dd::load(pc);
                if (beta_kind == 2) c0 = dd::mul_exact(c0, beta);
                dd::store(pc, dd::add_exact(c0, r));
            }
        }
    }
}

// C := beta*C over an m x n block (beta == 0 writes zeros without reading).
__global__ void k_scale_matrix(int64_t m, int64_t n, dd::real beta, int beta_kind, double2 *C, int64_t ldc,
                               int uplo)
{
    int64_t total = m * n;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        int64_t i = t % m, j = t / m;
        if ((uplo == 1 && i > j) || (uplo == 2 && i < j)) continue;
        double2 *p = C + i + j * ldc;
        if (beta_kind == 0)
            *p = make_double2(0.0, 0.0);
        else
            dd::store(p, dd::mul_exact(dd::load(p), beta));
    }
}

// A 2-D tensor map over a column-major double-double matrix (rows x cols,
// leading dimension ld), in doubles: dimension 0 = 2 * rows, dimension 1 =
// cols; box = (2 * box_rows, box_cols).
bool dd_map(CUtensorMap *map, const void *base, int64_t rows, int64_t cols, int64_t ld, uint32_t box_rows,
            uint32_t box_cols, const char *routine)
{
    auto enc = (PFN_cuTensorMapEncodeTiled_v12000)tensor_map_encoder();
    if (!enc) return false;
    cuuint64_t dims[2] = {(cuuint64_t)(2 * rows), (cuuint64_t)cols};
    cuuint64_t strides[1] = {(cuuint64_t)ld * 16};
    cuuint32_t box[2] = {2 * box_rows, box_cols};
    cuuint32_t es[2] = {1, 1};
    CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 2, const_cast<void *>(base), dims, strides, box, es,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        set_error(routine, MWBLAS_ERR_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
        return false;
    }
    return true;
}

// TMA staging of the FP64 engine's tiles (default on; 0 = plain loads).
std::atomic<int> g_plain_tma{1};

template <int BM, int BN, int TM, int TN, int KB>
bool dispatch_plain_tma(const GemmArgs &g, const int *ea, const int *eb, const char *routine)
{
    constexpr int NS = 4, BK = 8;
    constexpr size_t SMEM = NS * (size_t)(BM + BN) * BK * 16 + NS * sizeof(uint64_t) + 128;
    // op(A) tiles: A (m x k) boxes of BM rows x BK columns, or A^T's storage (k x m) boxes of BK x BM
    CUtensorMap ma, mb;
    const bool ok = (g.ta ? dd_map(&ma, g.A, g.k, g.m, g.lda, BK, BM, routine)
                          : dd_map(&ma, g.A, g.m, g.k, g.lda, BM, BK, routine)) &&
                    (g.tb ? dd_map(&mb, g.B, g.n, g.k, g.ldb, BN, BK, routine)
                          : dd_map(&mb, g.B, g.k, g.n, g.ldb, BK, BN, routine));
    if (!ok) return false;
    dim3 grid((unsigned)((g.m + BM - 1) / BM), (unsigned)((g.n + BN - 1) / BN));
    dim3 block((BM / TM) * (BN / TN));
    dd::real al = dd::make(g.alpha.hi, g.alpha.lo), be = dd::make(g.beta.hi, g.beta.lo);
    double2 *C = (double2 *)g.C;
#define MW_LAUNCH(TA, TB)                                                                                          \
    {                                                                                                              \
        auto kern = g.k <= kCompMaxK ? k_gemm_plain_tma<BM, BN, TM, TN, TA, TB, KB, NS, true>                      \
                                     : k_gemm_plain_tma<BM, BN, TM, TN, TA, TB, KB, NS, false>;                    \
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM);                        \
        kern<<<grid, block, SMEM, stream()>>>(ma, mb, g.m, g.n, g.k, al, be, g.beta_kind, C, g.ldc, ea, eb, g.uplo, \
                                              sigma_shift(KB, g.k, 1), device_status_word());                      \
    }
    if (!g.ta && !g.tb) MW_LAUNCH(false, false)
    else if (!g.ta && g.tb) MW_LAUNCH(false, true)
    else if (g.ta && !g.tb) MW_LAUNCH(true, false)
    else MW_LAUNCH(true, true)
#undef MW_LAUNCH
    count_launch();
    return true;
}

template <int BM, int BN, int TM, int TN, int KB>
void dispatch_plain(const GemmArgs &g, const int *ea, const int *eb)
{
    dim3 grid((unsigned)((g.m + BM - 1) / BM), (unsigned)((g.n + BN - 1) / BN));
    dim3 block((BM / TM) * (BN / TN));
    dd::real al = dd::make(g.alpha.hi, g.alpha.lo), be = dd::make(g.beta.hi, g.beta.lo);
    const double2 *A = (const double2 *)g.A;
    const double2 *B = (const double2 *)g.B;
    double2 *C = (double2 *)g.C;
#define MW_LAUNCH(TA, TB)                                                                                     \
    k_gemm_plain<BM, BN, TM, TN, TA, TB, KB><<<grid, block, 0, stream()>>>(g.m, g.n, g.k, al, A, g.lda, B, g.ldb, \
                                                                          be, g.beta_kind, C, g.ldc, ea, eb, g.uplo, \
                                                                          sigma_shift(KB, g.k, 1), g.k <= kCompMaxK)
    if (!g.ta && !g.tb) MW_LAUNCH(false, false);
    else if (!g.ta && g.tb) MW_LAUNCH(false, true);
    else if (g.ta && !g.tb) MW_LAUNCH(true, false);
    else MW_LAUNCH(true, true);
#undef MW_LAUNCH
    count_launch();
}


// ---- complex ------------------------------------------------------------------
// Same extraction scheme, one (X, L, DD) accumulator per real and imaginary
// part; each complex multiply-add feeds two products into each part
// (re += ar*br - ai*bi, im += ar*bi + ai*br), 24 FP64 instructions against
// the reference's ~72 (wgemm_serial.cpp:274-302). Conjugation of op(A)/op(B)
// negates the imaginary limbs at load, as the reference does at pack time
// (wgemm_serial.cpp:52-75, :143-157).

__device__ __forceinline__ void xacc(double ah, double al, double bh, double bl, double &X, double &X2, double &L,
                                     int comp)
{
    double t = __fma_rn(ah, bh, X);
    double q = __dsub_rn(X, t);
    double r = __fma_rn(ah, bh, q);
    X = t;
    if (comp) {
        double t2 = __dadd_rn(X2, r);
        double q2 = __dsub_rn(X2, t2);
        r = __dadd_rn(q2, r);
        X2 = t2;
    }
    double l = __dadd_rn(L, r);
    l = __fma_rn(ah, bl, l);
    L = __fma_rn(al, bh, l);
}

__device__ __forceinline__ void xfold(double sg, double sg2, double &X, double &X2, double &L, double &Ah, double &Al,
                                      int comp)
{
    double s = __dsub_rn(X, sg);
    double lsum = L;
    if (comp) {
        lsum = __dadd_rn(lsum, __dsub_rn(X2, sg2));
        X2 = sg2;
    }
    double h, e;
    dd::two_sum(Ah, s, h, e);
    double lo = __dadd_rn(Al, __dadd_rn(e, lsum));
    dd::fast_two_sum(h, lo, Ah, Al);
    X = sg;
    L = 0.0;
}

template <int BM, int BN, int TM, int TN, bool TA, bool TB, bool CA, bool CB, int KB>
__global__ void __launch_bounds__((BM / TM) * (BN / TN))
    k_gemm_plain_c(int64_t m, int64_t n, int64_t k, dd::cplx alpha, const double2 *__restrict__ A, int64_t lda,
                   const double2 *__restrict__ B, int64_t ldb, dd::cplx beta, int beta_kind, double2 *C,
                   int64_t ldc, const int *__restrict__ ea, const int *__restrict__ eb, int uplo, int herm,
                   int SHIFT, int COMP)
{
    constexpr int NTX = BM / TM;
    constexpr int NTY = BN / TN;
    constexpr int NT = NTX * NTY;
    constexpr int BK = 8;

    __shared__ double2 sA[BK][BM][2];
    __shared__ double2 sB[BK][BN][2];

    const int tid = threadIdx.x;
    const int tx = tid % NTX, ty = tid / NTX;
    const int64_t i0 = (int64_t)blockIdx.x * BM, j0 = (int64_t)blockIdx.y * BN;
    if ((uplo == 1 && i0 > j0 + BN - 1) || (uplo == 2 && i0 + BM - 1 < j0)) return;

    int eai[TM], ebj[TN];
#pragma unroll
    for (int a = 0; a < TM; ++a) {
        int64_t i = i0 + tx + a * NTX;
        eai[a] = (i < m) ? ea[i] : kNoExp;
    }
#pragma unroll
    for (int b = 0; b < TN; ++b) {
        int64_t j = j0 + ty + b * NTY;
        ebj[b] = (j < n) ? eb[j] : kNoExp;
    }

    double Xr[TM][TN], Lr[TM][TN], Rh[TM][TN], Rl[TM][TN], Xr2[TM][TN];
    double Xi[TM][TN], Li[TM][TN], Ih[TM][TN], Il[TM][TN], Xi2[TM][TN];
#pragma unroll
    for (int a = 0; a < TM; ++a)
#pragma unroll
        for (int b = 0; b < TN; ++b) {
            double sg = make_sigma(eai[a], ebj[b], SHIFT);
            Xr[a][b] = sg; Lr[a][b] = 0.0; Rh[a][b] = 0.0; Rl[a][b] = 0.0;
            Xi[a][b] = sg; Li[a][b] = 0.0; Ih[a][b] = 0.0; Il[a][b] = 0.0;
            Xr2[a][b] = Xi2[a][b] = make_sigma2(eai[a], ebj[b], SHIFT);
        }

    int since_fold = 0;
    for (int64_t kk = 0; kk < k; kk += BK) {
        for (int idx = tid; idx < BM * BK; idx += NT) {
            int r, p;
            if (!TA) { r = idx % BM; p = idx / BM; }
            else     { p = idx % BK; r = idx / BK; }
            int64_t gi = i0 + r, gp = kk + p;
            double2 vr = make_double2(0.0, 0.0), vi = vr;
            if (gi < m && gp < k) {
                const double2 *src = TA ? A + 2 * (gp + gi * lda) : A + 2 * (gi + gp * lda);
                vr = src[0];
                vi = src[1];
                if (CA) { vi.x = -vi.x; vi.y = -vi.y; }
            }
            sA[p][r][0] = vr;
            sA[p][r][1] = vi;
        }
        for (int idx = tid; idx < BN * BK; idx += NT) {
            int c, p;
            if (!TB) { p = idx % BK; c = idx / BK; }
            else     { c = idx % BN; p = idx / BN; }
            int64_t gj = j0 + c, gp = kk + p;
            double2 vr = make_double2(0.0, 0.0), vi = vr;
            if (gj < n && gp < k) {
                const double2 *src = TB ? B + 2 * (gj + gp * ldb) : B + 2 * (gp + gj * ldb);
                vr = src[0];
                vi = src[1];
                if (CB) { vi.x = -vi.x; vi.y = -vi.y; }
            }
            sB[p][c][0] = vr;
            sB[p][c][1] = vi;
        }
        __syncthreads();

#pragma unroll
        for (int p = 0; p < BK; ++p) {
            double2 ar[TM], ai[TM], br[TN], bi[TN];
#pragma unroll
            for (int a = 0; a < TM; ++a) { ar[a] = sA[p][tx + a * NTX][0]; ai[a] = sA[p][tx + a * NTX][1]; }
#pragma unroll
            for (int b = 0; b < TN; ++b) { br[b] = sB[p][ty + b * NTY][0]; bi[b] = sB[p][ty + b * NTY][1]; }
#pragma unroll
            for (int a = 0; a < TM; ++a)
#pragma unroll
                for (int b = 0; b < TN; ++b) {
                    xacc(ar[a].x, ar[a].y, br[b].x, br[b].y, Xr[a][b], Xr2[a][b], Lr[a][b], COMP);
                    xacc(-ai[a].x, -ai[a].y, bi[b].x, bi[b].y, Xr[a][b], Xr2[a][b], Lr[a][b], COMP);
                    xacc(ar[a].x, ar[a].y, bi[b].x, bi[b].y, Xi[a][b], Xi2[a][b], Li[a][b], COMP);
                    xacc(ai[a].x, ai[a].y, br[b].x, br[b].y, Xi[a][b], Xi2[a][b], Li[a][b], COMP);
                }
        }
        __syncthreads();

        since_fold += BK;
        if (since_fold == KB || kk + BK >= k) {
            since_fold = 0;
#pragma unroll
            for (int a = 0; a < TM; ++a)
#pragma unroll
                for (int b = 0; b < TN; ++b) {
                    double sg = make_sigma(eai[a], ebj[b], SHIFT);
                    double sg2 = make_sigma2(eai[a], ebj[b], SHIFT);
                    xfold(sg, sg2, Xr[a][b], Xr2[a][b], Lr[a][b], Rh[a][b], Rl[a][b], COMP);
                    xfold(sg, sg2, Xi[a][b], Xi2[a][b], Li[a][b], Ih[a][b], Il[a][b], COMP);
                }
        }
    }

#pragma unroll
    for (int b = 0; b < TN; ++b) {
        int64_t j = j0 + ty + b * NTY;
        if (j >= n) continue;
#pragma unroll
        for (int a = 0; a < TM; ++a) {
            int64_t i = i0 + tx + a * NTX;
            if (i >= m) continue;
            if ((uplo == 1 && i > j) || (uplo == 2 && i < j)) continue;
            dd::cplx acc;
            acc.re = dd::make(Rh[a][b], Rl[a][b]);
            acc.im = dd::make(Ih[a][b], Il[a][b]);
            dd::cplx r = dd::cmul_fast(alpha, acc);
            double2 *pc = C + 2 * (i + j * ldc);
            dd::cplx out = r;
            if (beta_kind != 0) {
                dd::cplx c0 = dd::cload(pc);
                if (beta_kind == 2) c0 = dd::cmul_exact(c0, beta);
                out = dd::cadd_exact(c0, r);
            }
            // HERK: the diagonal of a Hermitian result is real
            // (wherk_serial.cpp:369-405).
            if (herm && i == j) out.im = dd::make(0.0, 0.0);
            dd::cstore(pc, out);
        }
    }
}

__global__ void k_scale_matrix_c(int64_t m, int64_t n, dd::cplx beta, int beta_kind, double2 *C, int64_t ldc,
                                 int uplo, int herm)
{
    int64_t total = m * n;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        int64_t i = t % m, j = t / m;
        if ((uplo == 1 && i > j) || (uplo == 2 && i < j)) continue;
        double2 *p = C + 2 * (i + j * ldc);
        if (beta_kind == 0) {
            p[0] = make_double2(0.0, 0.0);
            p[1] = make_double2(0.0, 0.0);
        } else if (herm) {
            // wherk_serial.cpp:373-384: real beta scales both parts; the
            // diagonal keeps beta*re and a zero imaginary part.
            dd::cplx v = dd::cload(p);
            v.re = dd::mul_exact(beta.re, v.re);
            v.im = (i == j) ? dd::make(0.0, 0.0) : dd::mul_exact(beta.re, v.im);
            dd::cstore(p, v);
        } else {
            dd::cstore(p, dd::cmul_exact(dd::cload(p), beta));
        }
    }
}

template <bool TA, bool TB, bool CA, bool CB>
void launch_plain_c(const GemmArgs &g, const int *ea, const int *eb)
{
    constexpr int BM = 32, BN = 32, TM = 2, TN = 2, KB = 8;
    dim3 grid((unsigned)((g.m + BM - 1) / BM), (unsigned)((g.n + BN - 1) / BN));
    dim3 block((BM / TM) * (BN / TN));
    dd::cplx al, be;
    al.re = dd::make(g.calpha.re.hi, g.calpha.re.lo);
    al.im = dd::make(g.calpha.im.hi, g.calpha.im.lo);
    be.re = dd::make(g.cbeta.re.hi, g.cbeta.re.lo);
    be.im = dd::make(g.cbeta.im.hi, g.cbeta.im.lo);
    k_gemm_plain_c<BM, BN, TM, TN, TA, TB, CA, CB, KB><<<grid, block, 0, stream()>>>(
        g.m, g.n, g.k, al, (const double2 *)g.A, g.lda, (const double2 *)g.B, g.ldb, be, g.beta_kind,
        (double2 *)g.C, g.ldc, ea, eb, g.uplo, g.herm ? 1 : 0, sigma_shift(KB, g.k, 2), g.k <= kCompMaxK);
    count_launch();
}

template <bool TA, bool TB>
void launch_plain_c_conj(const GemmArgs &g, const int *ea, const int *eb)
{
    if (g.ca) {
        if (g.cb) launch_plain_c<TA, TB, true, true>(g, ea, eb);
        else launch_plain_c<TA, TB, true, false>(g, ea, eb);
    } else {
        if (g.cb) launch_plain_c<TA, TB, false, true>(g, ea, eb);
        else launch_plain_c<TA, TB, false, false>(g, ea, eb);
    }
}

}  // namespace

// Row exponents of op(X) where X is stored column-major (rows_x x cols_x) and
// op(X) = X (trans=false) or X^T (trans=true). Produces one int per row of
// op(X), and with `low` the exponent of the lowest set bit in that row.
void launch_exp_rows_of_op(const void *X, int64_t rows_x, int64_t cols_x, int64_t ld, bool trans, int elem2,
                           int *out, int *low)
{
    if (!trans) {
        // rows of X: thread per row, column range split over grid.y
        // enough (rows, column-range) blocks to cover the GPU a few times
        const int64_t rb = (rows_x + 255) / 256;
        int64_t want_y = (4 * (int64_t)device_sm_count() + rb - 1) / rb;
        int64_t per_y = (cols_x + want_y - 1) / want_y;
        if (per_y < 16) per_y = 16;
        if ((cols_x + per_y - 1) / per_y > 65535) per_y = (cols_x + 65534) / 65535;
        dim3 grid((unsigned)rb, (unsigned)((cols_x + per_y - 1) / per_y));
        cudaMemsetAsync(out, 0x80, sizeof(int) * rows_x, stream());
        if (low) cudaMemsetAsync(low, 0x3f, sizeof(int) * rows_x, stream());   // kLowNone
        k_exp_rows<<<grid, 256, 0, stream()>>>(rows_x, cols_x, (const double2 *)X, ld, elem2, out, per_y, low);
    } else {
        // rows of X^T = columns of X: a warp per column, long columns cut into
        // pieces of at least 256 rows when there are too few columns to cover
        // the GPU a few times
        const int64_t want = 32 * (int64_t)device_sm_count();
        int64_t ys = (want + cols_x - 1) / cols_x;
        ys = std::min<int64_t>(ys, (rows_x + 255) / 256);
        ys = std::max<int64_t>(1, std::min<int64_t>(ys, 65535));
        const int64_t rows_per = (rows_x + ys - 1) / ys;
        if (ys > 1) {
            cudaMemsetAsync(out, 0x80, sizeof(int) * cols_x, stream());
            if (low) cudaMemsetAsync(low, 0x3f, sizeof(int) * cols_x, stream());   // kLowNone
        }
        dim3 grid((unsigned)((cols_x + 7) / 8), (unsigned)ys);
        k_exp_cols<<<grid, 256, 0, stream()>>>(rows_x, cols_x, (const double2 *)X, ld, elem2, out, low, rows_per);
    }
    count_launch();
}

// Column exponents of op(X): columns of X^T are rows of X and vice versa.
void launch_exp_cols_of_op(const void *X, int64_t rows_x, int64_t cols_x, int64_t ld, bool trans, int elem2,
                           int *out, int *low)
{
    launch_exp_rows_of_op(X, rows_x, cols_x, ld, !trans, elem2, out, low);
}

void launch_scale_matrix(int64_t m, int64_t n, dd_host beta, int beta_kind, void *C, int64_t ldc, int uplo)
{
    if (m <= 0 || n <= 0 || beta_kind == 1) return;
    int64_t total = m * n;
    int64_t blocks = (total + 255) / 256;
    int64_t cap = (int64_t)device_sm_count() * 8;
    if (blocks > cap) blocks = cap;
    k_scale_matrix<<<(unsigned)blocks, 256, 0, stream()>>>(m, n, dd::make(beta.hi, beta.lo), beta_kind, (double2 *)C,
                                                           ldc, uplo);
    count_launch();
}

bool gemm_plain_real(const GemmArgs &g, const char *routine)
{
    int *ex = (int *)dev_alloc(sizeof(int) * (size_t)(g.m + g.n), routine);
    if (!ex) return false;
    int *ea = ex, *eb = ex + g.m;
    // op(A) is m x k: A stored (ta ? k x m : m x k)
    launch_exp_rows_of_op(g.A, g.ta ? g.k : g.m, g.ta ? g.m : g.k, g.lda, g.ta, 1, ea);
    // op(B) is k x n: B stored (tb ? n x k : k x n)
    launch_exp_cols_of_op(g.B, g.tb ? g.n : g.k, g.tb ? g.k : g.n, g.ldb, g.tb, 1, eb);
    int64_t tiles64 = ((g.m + 63) / 64) * ((g.n + 63) / 64);
    const bool big = tiles64 >= 2 * (int64_t)device_sm_count();
    // TMA staging wants 16-byte aligned operands (always true of device
    // double-double arrays) and dimensions a tensor map can describe
    const bool tma = g_plain_tma.load() != 0 && ((uintptr_t)g.A & 15) == 0 && ((uintptr_t)g.B & 15) == 0 &&
                     g.m < ((int64_t)1 << 31) && g.n < ((int64_t)1 << 31) && g.k < ((int64_t)1 << 31) &&
                     tensor_map_encoder() != nullptr;
    bool done = false;
    if (tma) {
        done = big ? dispatch_plain_tma<64, 64, 4, 4, 8>(g, ea, eb, routine)
                   : dispatch_plain_tma<32, 32, 2, 2, 8>(g, ea, eb, routine);
        if (!done) {
            dev_free(ex);
            return false;
        }
    }
    if (!done) {
        if (big) dispatch_plain<64, 64, 4, 4, 8>(g, ea, eb);
        else dispatch_plain<32, 32, 2, 2, 8>(g, ea, eb);
    }
    dev_free(ex);
    return true;
}

void set_plain_wait_limit(uint64_t ns)
{
    cudaMemcpyToSymbol(sm100::g_wait_limit_ns, &ns, sizeof(ns));
}

void launch_scale_matrix_c(int64_t m, int64_t n, cdd_host beta, int beta_kind, void *C, int64_t ldc, int uplo,
                           bool herm)
{
    if (m <= 0 || n <= 0 || (beta_kind == 1 && !herm)) return;
    int64_t total = m * n;
    int64_t blocks = (total + 255) / 256;
    int64_t cap = (int64_t)device_sm_count() * 8;
    if (blocks > cap) blocks = cap;
    dd::cplx be;
    be.re = dd::make(beta.re.hi, beta.re.lo);
    be.im = dd::make(beta.im.hi, beta.im.lo);
    k_scale_matrix_c<<<(unsigned)blocks, 256, 0, stream()>>>(m, n, be, beta_kind, (double2 *)C, ldc, uplo,
                                                             herm ? 1 : 0);
    count_launch();
}

bool gemm_plain_cplx(const GemmArgs &g, const char *routine)
{
    int *ex = (int *)dev_alloc(sizeof(int) * (size_t)(g.m + g.n), routine);
    if (!ex) return false;
    int *ea = ex, *eb = ex + g.m;
    launch_exp_rows_of_op(g.A, g.ta ? g.k : g.m, g.ta ? g.m : g.k, g.lda, g.ta, 2, ea);
    launch_exp_cols_of_op(g.B, g.tb ? g.n : g.k, g.tb ? g.k : g.n, g.ldb, g.tb, 2, eb);
    if (!g.ta && !g.tb) launch_plain_c_conj<false, false>(g, ea, eb);
    else if (!g.ta && g.tb) launch_plain_c_conj<false, true>(g, ea, eb);
    else if (g.ta && !g.tb) launch_plain_c_conj<true, false>(g, ea, eb);
    else launch_plain_c_conj<true, true>(g, ea, eb);
    dev_free(ex);
    return true;
}

}  // namespace mw

extern "C" int mwblas_set_plain_tma(int on)
{
    return mw::g_plain_tma.exchange(on ? 1 : 0);
}
