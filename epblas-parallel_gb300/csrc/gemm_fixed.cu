// Fixed-point double-double GEMM on the integer pipes ("fixed" engine).
//
// The FP64 pipe of this part issues ~1.6 lane-operations per clock per SM,
// the integer multiply-add pipe ~40x more. This engine therefore forms the
// double-double products in integers:
//
//  * op(A)'s rows and op(B)'s columns are scaled by powers of two from their
//    exponent bounds (as the tensor-core engine does): a(i,p) * 2^(S - ea_i)
//    is rounded to an integer below 2^116 (S = 115), the exact image of the
//    106-bit hi + lo; likewise b(p,j) * 2^(S - eb_j).
//  * Each integer is held as five signed ("balanced") 24-bit digits,
//    d_0 + d_1 2^24 + ... + d_4 2^96 with |d_t| <= 2^23, converted on the fly
//    when the tile is staged in shared memory.
//  * A multiply-add is 15 IMAD.WIDE: the digit products d_s e_t with
//    s + t >= 4, accumulated exactly in five signed 64-bit column sums (one per
//    weight 2^(24w), w = 4..8). The 10 dropped products with s + t <= 3 are
//    below 2^-110 of |a|max |b|max per term.
//  * The epilogue assembles the column sums into one 256-bit integer, scales
//    it back by 2^(ea_i + eb_j - 2S + 96) and computes alpha*X + beta*C in
//    128-bit extended floats with a single rounding to double-double.
//
// Column sums stay below 2^63 for up to 16384 multiply-adds (5 products of
// at most 2^46 per step), so longer K runs in chunks of 16384 with beta = 1
// for all but the first. Rows or columns with a non-finite entry give NaN
// outputs, as the reference's double-double products of an infinity do (the
// TwoProduct error term is inf - inf). Accuracy is normwise, like the tensor-
// core engine's: entries far below their row/column maximum keep fewer bits.
#include <cmath>

#include "dd.cuh"
#include "fixacc.cuh"
#include "fixgemm.cuh"
#include "gemm.h"
#include "runtime.h"
#include "xfloat.cuh"

namespace mw {

namespace {

using xfp::XF;
using namespace fxg;

constexpr int FX_BM = 64, FX_BN = 64, FX_BK = 8;
constexpr int FX_THREADS = 256;      // 16 x 16 threads, 4 x 4 outputs each
constexpr int64_t FX_MAX_K = 16384;  // per launch (column-sum headroom)
constexpr int kNoExpFx = -30000;

template <bool TA, bool TB>
__global__ void __launch_bounds__(FX_THREADS, 1)
    k_gemm_fixed(int64_t m, int64_t n, int64_t k, const double2 *__restrict__ A, int64_t lda,
                 const double2 *__restrict__ B, int64_t ldb, const int *__restrict__ ea, const int *__restrict__ eb,
                 dd::real alpha, int alpha_one, dd::real beta, int beta_kind, double2 *C, int64_t ldc, int uplo)
{
    __shared__ __align__(16) int sA[FX_BK][5][FX_BM];   // digit planes, rows contiguous
    __shared__ __align__(16) int sB[FX_BK][5][FX_BN];
    __shared__ int s_sa[FX_BM], s_sb[FX_BN];

    const int tid = threadIdx.x;
    const int tx = tid & 15, ty = tid >> 4;   // rows 4tx..4tx+3, columns 4ty..4ty+3
    const int64_t i0 = (int64_t)blockIdx.x * FX_BM, j0 = (int64_t)blockIdx.y * FX_BN;
    if ((uplo == 1 && i0 > j0 + FX_BN - 1) || (uplo == 2 && i0 + FX_BM - 1 < j0)) return;

    if (tid < FX_BM) {
        const int64_t i = i0 + tid;
        const int e = (i < m) ? ea[i] : kNoExpFx;
        s_sa[tid] = (e <= kNoExpFx / 2) ? -100000 : FX_S - e;
    } else if (tid < FX_BM + FX_BN) {
        const int64_t j = j0 + (tid - FX_BM);
        const int e = (j < n) ? eb[j] : kNoExpFx;
        s_sb[tid - FX_BM] = (e <= kNoExpFx / 2) ? -100000 : FX_S - e;
    }
    __syncthreads();

    long long acc[4][4][5];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b)
#pragma unroll
            for (int w = 0; w < 5; ++w) acc[a][b][w] = 0;

    // each thread stages 2 elements of the A tile and 2 of the B tile per slab
    double2 ra[2], rb[2];
    auto load = [&](int64_t kk) {
#pragma unroll
        for (int u = 0; u < 2; ++u) {
            const int idx = tid + u * FX_THREADS;
            int r, p;
            if (!TA) { r = idx % FX_BM; p = idx / FX_BM; }
            else     { p = idx % FX_BK; r = idx / FX_BK; }
            const int64_t gi = i0 + r, gp = kk + p;
            ra[u] = (gi < m && gp < k) ? (TA ? A[gp + gi * lda] : A[gi + gp * lda]) : make_double2(0.0, 0.0);
            int c;
            if (!TB) { p = idx % FX_BK; c = idx / FX_BK; }
            else     { c = idx % FX_BN; p = idx / FX_BN; }
            const int64_t gj = j0 + c, gq = kk + p;
            rb[u] = (gj < n && gq < k) ? (TB ? B[gj + gq * ldb] : B[gq + gj * ldb]) : make_double2(0.0, 0.0);
        }
    };
    auto stage = [&]() {
#pragma unroll
        for (int u = 0; u < 2; ++u) {
            const int idx = tid + u * FX_THREADS;
            int r, p, d[5];
            if (!TA) { r = idx % FX_BM; p = idx / FX_BM; }
            else     { p = idx % FX_BK; r = idx / FX_BK; }
            dd_digits(ra[u], s_sa[r], d);
#pragma unroll
            for (int t = 0; t < 5; ++t) sA[p][t][r] = d[t];
            int c;
            if (!TB) { p = idx % FX_BK; c = idx / FX_BK; }
            else     { c = idx % FX_BN; p = idx / FX_BN; }
            dd_digits(rb[u], s_sb[c], d);
#pragma unroll
            for (int t = 0; t < 5; ++t) sB[p][t][c] = d[t];
        }
    };

    load(0);
    for (int64_t kk = 0; kk < k; kk += FX_BK) {
        stage();
        __syncthreads();
        if (kk + FX_BK < k) load(kk + FX_BK);   // next slab in flight during the products
#pragma unroll 2
        for (int p = 0; p < FX_BK; ++p) {
            int da[5][4], db[5][4];
#pragma unroll
            for (int t = 0; t < 5; ++t) {
                const int4 va = *reinterpret_cast<const int4 *>(&sA[p][t][4 * tx]);
                const int4 vb = *reinterpret_cast<const int4 *>(&sB[p][t][4 * ty]);
                da[t][0] = va.x; da[t][1] = va.y; da[t][2] = va.z; da[t][3] = va.w;
                db[t][0] = vb.x; db[t][1] = vb.y; db[t][2] = vb.z; db[t][3] = vb.w;
            }
#pragma unroll
            for (int a = 0; a < 4; ++a)
#pragma unroll
                for (int b = 0; b < 4; ++b) {
                    long long *c = acc[a][b];
                    c[0] += (long long)da[0][a] * db[4][b] + (long long)da[1][a] * db[3][b] +
                            (long long)da[2][a] * db[2][b] + (long long)da[3][a] * db[1][b] +
                            (long long)da[4][a] * db[0][b];
                    c[1] += (long long)da[1][a] * db[4][b] + (long long)da[2][a] * db[3][b] +
                            (long long)da[3][a] * db[2][b] + (long long)da[4][a] * db[1][b];
                    c[2] += (long long)da[2][a] * db[4][b] + (long long)da[3][a] * db[3][b] +
                            (long long)da[4][a] * db[2][b];
                    c[3] += (long long)da[3][a] * db[4][b] + (long long)da[4][a] * db[3][b];
                    c[4] += (long long)da[4][a] * db[4][b];
                }
        }
        __syncthreads();
    }

    const XF xa = xfp::xf_from_dd(alpha.hi, alpha.lo), xb = xfp::xf_from_dd(beta.hi, beta.lo);
#pragma unroll
    for (int b = 0; b < 4; ++b) {
        const int64_t j = j0 + 4 * ty + b;
        if (j >= n) continue;
#pragma unroll
        for (int a = 0; a < 4; ++a) {
            const int64_t i = i0 + 4 * tx + a;
            if (i >= m) continue;
            if ((uplo == 1 && i > j) || (uplo == 2 && i < j)) continue;
            const int ei = ea[i], ej = eb[j];
            double2 *pc = C + i + j * ldc;
            if (ei >= 1024 || ej >= 1024) {   // a non-finite entry in row i of op(A) or column j of op(B)
                const double qnan = __longlong_as_double(0x7ff8000000000000ll);
                *pc = make_double2(qnan, qnan);
                continue;
            }
            XF v;
            if (ei <= kNoExpFx / 2 || ej <= kNoExpFx / 2) {
                v.zero = true; v.neg = false; v.m = 0; v.e = 0;
            } else {
                v = sums_to_xf(acc[a][b], ei, ej);
            }
            store_axpby(pc, v, xa, alpha_one != 0, xb, beta, beta_kind);
        }
    }
}

}  // namespace

bool gemm_fixed_real(const GemmArgs &g0, const char *routine)
{
    GemmArgs g = g0;
    if (!std::isfinite(g.alpha.hi) || !std::isfinite(g.beta.hi)) return gemm_plain_real(g, routine);
    if (g.k == 0) {
        launch_scale_matrix(g.m, g.n, g.beta, g.beta_kind, g.C, g.ldc, g.uplo);
        return true;
    }
    int *ex = (int *)dev_alloc(sizeof(int) * (size_t)(g.m + g.n), routine);
    if (!ex) return false;
    int *ea = ex, *eb = ex + g.m;
    dim3 grid((unsigned)((g.m + FX_BM - 1) / FX_BM), (unsigned)((g.n + FX_BN - 1) / FX_BN));
    const dd::real al = dd::make(g.alpha.hi, g.alpha.lo);
    const int alpha_one = (g.alpha.hi == 1.0 && g.alpha.lo == 0.0);
    for (int64_t k0 = 0; k0 < g.k; k0 += FX_MAX_K) {
        const int64_t kc = (g.k - k0 < FX_MAX_K) ? g.k - k0 : FX_MAX_K;
        const double2 *A = (const double2 *)g.A + (g.ta ? k0 : k0 * g.lda);
        const double2 *B = (const double2 *)g.B + (g.tb ? k0 * g.ldb : k0);
        // exponent bounds of this chunk's rows of op(A) and columns of op(B)
        launch_exp_rows_of_op(A, g.ta ? kc : g.m, g.ta ? g.m : kc, g.lda, g.ta, 1, ea);
        launch_exp_cols_of_op(B, g.tb ? g.n : kc, g.tb ? kc : g.n, g.ldb, g.tb, 1, eb);
        const dd::real be = (k0 == 0) ? dd::make(g.beta.hi, g.beta.lo) : dd::make(1.0, 0.0);
        const int bk = (k0 == 0) ? g.beta_kind : 1;
#define MW_FX(TA, TB)                                                                                         \
    k_gemm_fixed<TA, TB><<<grid, FX_THREADS, 0, stream()>>>(g.m, g.n, kc, A, g.lda, B, g.ldb, ea, eb, al,    \
                                                            alpha_one, be, bk, (double2 *)g.C, g.ldc, g.uplo)
        if (!g.ta && !g.tb) MW_FX(false, false);
        else if (!g.ta && g.tb) MW_FX(false, true);
        else if (g.ta && !g.tb) MW_FX(true, false);
        else MW_FX(true, true);
#undef MW_FX
        count_launch();
    }
    dev_free(ex);
    return true;
}

}  // namespace mw
