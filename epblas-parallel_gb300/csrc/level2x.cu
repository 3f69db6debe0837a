// The level-2 family beyond GEMV, built on the level-3 machinery:
//
//   GEMV (complex), GBMV       y := alpha*op(A)*x + beta*y        (mgbmv.cpp, wgemv.cpp, wgbmv.cpp)
//   SYMV/HEMV, SBMV/HBMV, SPMV/HPMV   A symmetric / Hermitian     (msymv.cpp, whemv.cpp, msbmv.cpp, ...)
//   TRMV/TBMV/TPMV, TRSV/TBSV/TPSV    A triangular               (mtrmv.cpp, mtrsv.cpp, mtbmv.cpp, ...)
//   GER/GERU/GERC, SYR/HER, SYR2/HER2, SPR/HPR, SPR2/HPR2  rank-1/2 updates (mger.cpp, msyr.cpp, ...)
//
// Band and packed matrix-vector products read the operand in place from its
// storage, in the fixed point of fixacc.cuh (k_smv; real symmetric bands of
// small bandwidth from shared-memory tiles, k_sbmv_tile; real symmetric
// packed matrices in two coalesced halves, k_spmv_*). Band solves of small
// bandwidth run in place (k_tbsv, k_spike_*). Otherwise band and packed
// operands are expanded into a dense scratch matrix by one bandwidth-bound
// kernel (packed outputs are packed back); vectors with any increment are
// gathered into contiguous scratch in BLAS order (a negative increment walks
// backwards) and written back the same way. Those products then run as
// GEMM/SYMM/TRMM/TRSM/SYRK/SYR2K on the engines with one right-hand side or a
// rank of one, so the arithmetic is the engines' (exact fixed point or
// tensor-core residues) and the error bounds are the level-3 ones.
#include <atomic>
#include <climits>

#include "dd.cuh"
#include "fixacc.cuh"
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

// ---- band and packed matrix-vector products, read in place ---------------------------
// Row r of op(A) has its stored entries in the columns [r - lo, r + hi]; each
// is decoded into the fixed point of fixacc.cuh and multiplied with x exactly
// (as DOT and GEMV), one thread (T = 1) or one warp (T = 32, lanes over the
// columns, partial sums combined in a fixed order) per output element, then
// y := beta*y + alpha*s with one rounding. Traffic is the stored entries and
// the vectors, O(n k) for a band, instead of the O(n^2) of a dense copy.

// Kernel parameters of smv_device (vectors contiguous).
struct SmvParams {
    int64_t rows, cols, n, kl, ku, ldab;
    const double2 *A;
    int fmt, kind, op;   // op 0 'N', 1 'T', 2 'C'
    bool upper, unit;
    const fx::Dig *xd;   // x decoded and split into digits once (complex: re, im)
    double2 *y;
    dd::real ar, ai, br, bi;
    int beta_kind;
};

// x (any increment, BLAS order) decoded and split for the products.
__global__ void k_vdig(int64_t n, const double2 *x, int64_t inc, int e2, fx::Dig *out)
{
    const int64_t total = n * e2;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = t / e2, w = t % e2;
        out[t] = fx::to_dig(fx::decode(x[e2 * vpos(i, n, inc) + w]));
    }
}

__device__ __forceinline__ void smv_range(const SmvParams &p, int64_t r, int64_t &c0, int64_t &c1)
{
    if (p.fmt == 0) {   // dense general: every column
        c0 = 0;
        c1 = p.cols - 1;
        return;
    }
    int64_t lo, hi;
    if (p.kind == 0) {
        lo = p.op == 0 ? p.kl : p.ku;
        hi = p.op == 0 ? p.ku : p.kl;
    } else {
        const int64_t k = p.fmt == 2 ? p.n - 1 : (p.upper ? p.ku : p.kl);
        if (p.kind != 3) {
            lo = hi = k;
        } else {
            const bool right = p.upper == (p.op == 0);   // stored entries right of the diagonal
            lo = right ? 0 : k;
            hi = right ? k : 0;
        }
    }
    c0 = r - lo < 0 ? 0 : r - lo;
    c1 = r + hi > p.cols - 1 ? p.cols - 1 : r + hi;
}

// Position of stored entry (i, j): packed upper i + j(j+1)/2, packed lower
// i + j(2n-j-1)/2, band AB(ku + i - j, j) (ku = 0 for a lower triangle).
__device__ __forceinline__ int64_t smv_addr(const SmvParams &p, int64_t i, int64_t j)
{
    if (p.fmt == 0) return i + j * p.ldab;
    if (p.fmt == 2) return p.upper ? i + j * (j + 1) / 2 : i + j * (2 * p.n - j - 1) / 2;
    return (p.ku + i - j) + j * p.ldab;
}

template <bool CX>
__device__ __forceinline__ void smv_elem(const SmvParams &p, int64_t r, int64_t c, fx::Op &er, fx::Op &ei)
{
    int64_t i, j;
    bool cj, realdiag = false;
    if (p.kind == 1 || p.kind == 2) {
        const bool stored = p.upper ? r <= c : r >= c;
        i = stored ? r : c;
        j = stored ? c : r;
        cj = !stored && p.kind == 2;
        realdiag = p.kind == 2 && r == c;
    } else {
        i = p.op == 0 ? r : c;
        j = p.op == 0 ? c : r;
        cj = p.op == 2;
        if (p.kind == 3 && p.unit && i == j) {
            er = fx::decode(make_double2(1.0, 0.0));
            ei = fx::decode(make_double2(0.0, 0.0));
            return;
        }
    }
    const double2 *a = p.A + (CX ? 2 : 1) * smv_addr(p, i, j);
    er = fx::decode(a[0]);
    if (CX) {
        ei = fx::decode(realdiag ? make_double2(0.0, 0.0) : a[1]);
        if (cj) ei.flags ^= fx::kNeg;
    }
}

__device__ __forceinline__ xfp::XF xneg(xfp::XF v)
{
    if (!v.zero) v.neg = !v.neg;
    return v;
}

__device__ __forceinline__ xfp::XF xzero()
{
    xfp::XF z;
    z.zero = true;
    z.neg = false;
    z.m = 0;
    z.e = 0;
    return z;
}

// y := b + t, one rounding (b = beta*y as a double-double; non-finite b is
// added in double-double as the reference's operator+ would).
__device__ __forceinline__ double2 smv_round(dd::real b, bool have_b, xfp::XF t)
{
    double h, l;
    if (have_b && !fx::finite_dd(make_double2(b.hi, b.lo))) {
        xfp::xf_to_dd(t, h, l);
        const dd::real s = dd::add_exact(b, dd::make(h, l));
        return make_double2(s.hi, s.lo);
    }
    if (have_b) t = xfp::xf_add(xfp::xf_from_dd(b.hi, b.lo), t);
    xfp::xf_to_dd(t, h, l);
    return make_double2(h, l);
}

// y := beta*y + alpha*s for a real row sum s (alpha as an extended float).
__device__ __forceinline__ void smv_store_real(double2 *py, const xfp::XF &xar, dd::real br, int beta_kind,
                                               const xfp::XF &s)
{
    dd::real b = dd::make(0.0, 0.0);
    if (beta_kind == 1) b = dd::load(py);
    else if (beta_kind == 2) b = dd::mul_exact(br, dd::load(py));
    py[0] = smv_round(b, beta_kind != 0, xfp::xf_mul(xar, s));
}

template <bool CX, int T>
__global__ void __launch_bounds__(256) k_smv(SmvParams p)
{
    const double nan = __longlong_as_double(0x7ff8000000000000ll);
    const int lane = T == 1 ? 0 : (threadIdx.x & 31);
    const int64_t teams = (int64_t)gridDim.x * blockDim.x / T;
    for (int64_t r = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) / T; r < p.rows; r += teams) {
        int64_t c0, c1;
        smv_range(p, r, c0, c1);
        fx::Acc acc[CX ? 2 : 1];
        xfp::XF tot[CX ? 2 : 1];
        bool bad = false;
        for (int w = 0; w < (CX ? 2 : 1); ++w) {
            acc[w].reset();
            tot[w] = xzero();
        }
        int cnt = 0;
        for (int64_t c = c0 + lane; c <= c1; c += T) {
            fx::Op er, ei;
            smv_elem<CX>(p, r, c, er, ei);
            if (CX) {
                const fx::Dig xr = p.xd[2 * c], xi = p.xd[2 * c + 1];
                fx::Op nei = ei;
                nei.flags ^= fx::kNeg;
                acc[0].add_dig(er, xr);
                acc[0].add_dig(nei, xi);
                acc[1].add_dig(er, xi);
                acc[1].add_dig(ei, xr);
                cnt += 2;
            } else {
                acc[0].add_dig(er, p.xd[c]);
                ++cnt;
            }
            if (cnt >= fx::kMaxAdds - 2) {
                for (int w = 0; w < (CX ? 2 : 1); ++w) {
                    bad |= acc[w].bad;
                    tot[w] = xfp::xf_add(tot[w], acc[w].finish());
                    acc[w].reset();
                }
                cnt = 0;
            }
        }
        for (int w = 0; w < (CX ? 2 : 1); ++w) {
            bad |= acc[w].bad;
            tot[w] = xfp::xf_add(tot[w], acc[w].finish());
            if (T == 32) tot[w] = fx::xf_warp_sum(tot[w]);
        }
        if (T == 32) bad = __any_sync(0xffffffffu, bad);
        if (lane != 0) continue;
        double2 *py = p.y + (CX ? 2 : 1) * r;
        if (bad) {
            py[0] = make_double2(nan, nan);
            if (CX) py[1] = make_double2(nan, nan);
            continue;
        }
        const xfp::XF xar = xfp::xf_from_dd(p.ar.hi, p.ar.lo);
        if (!CX) {
            smv_store_real(py, xar, p.br, p.beta_kind, tot[0]);
        } else {
            const xfp::XF xai = xfp::xf_from_dd(p.ai.hi, p.ai.lo);
            const xfp::XF tr = xfp::xf_add(xfp::xf_mul(xar, tot[0]), xneg(xfp::xf_mul(xai, tot[1])));
            const xfp::XF ti = xfp::xf_add(xfp::xf_mul(xar, tot[1]), xfp::xf_mul(xai, tot[0]));
            dd::cplx b;
            b.re = b.im = dd::make(0.0, 0.0);
            if (p.beta_kind == 1) {
                b = dd::cload(py);
            } else if (p.beta_kind == 2) {
                dd::cplx be;
                be.re = p.br;
                be.im = p.bi;
                b = dd::cmul_exact(be, dd::cload(py));
            }
            const double2 yr = smv_round(b.re, p.beta_kind != 0, tr);
            const double2 yi = smv_round(b.im, p.beta_kind != 0, ti);
            py[0] = yr;
            py[1] = yi;
        }
    }
}

// ---- real symmetric band product from a shared-memory tile ---------------------------
// For bandwidth k <= kSbMaxK. A thread per row reading its band row straight
// from band storage walks the array at a stride of ldab entries (every warp
// load touches 32 lines), which bounds k_smv on the L1. Here a block of
// kSbRows threads owns kSbRows consecutive rows and first copies, with
// coalesced loads, every stored column those rows touch (upper storage:
// columns [r0, r0 + R + k); lower: [r0 - k, r0 + R)) into shared memory, and
// decodes x_c for columns [r0 - k, r0 + R + k) into digit sets there (x read
// in place, any increment). Each thread then forms its row's 2k + 1 products
// from shared memory. A first pass over the row's exponents fixes the
// accumulator's block exponent, so no product has to move it (with rows this
// short, moving it as larger terms arrive, the way the long sums of DOT and
// GEMV do, would cost more than the products).
constexpr int kSbRows = 128;
constexpr int kSbMaxK = 32;
std::atomic<int> g_band_tile{1};   // mwblas_set_band_tile

struct SbParams {
    int64_t n, ldab;
    int k;
    bool upper;
    const double2 *AB;
    const double2 *x;
    int64_t incx;
    double2 *y;   // y itself (any increment) or a contiguous copy (incy 1)
    int64_t incy;
    dd::real ar, br;
    int beta_kind;
};

// Shared bytes of a tile for bandwidth k: the band columns at an odd stride
// (16-byte reads of consecutive rows then fall in distinct banks) and the
// digit sets of x as two arrays of 16-byte halves.
constexpr size_t sb_smem_bytes(int k)
{
    return (size_t)(kSbRows + k) * ((k + 1) | 1) * sizeof(double2) + (size_t)(kSbRows + 2 * k) * 2 * sizeof(int4);
}

__global__ void __launch_bounds__(kSbRows) k_sbmv_tile(SbParams p)
{
    extern __shared__ int4 sb_smem[];
    const int k = p.k, kp = k + 1, sp = kp | 1, t = threadIdx.x;
    const int64_t r0 = (int64_t)blockIdx.x * kSbRows;
    const int64_t cb = p.upper ? r0 : (r0 > k ? r0 - k : 0);
    const int64_t cend = p.upper ? r0 + kSbRows + k : r0 + kSbRows;
    const int64_t ce = cend < p.n ? cend : p.n;
    const int64_t xb = r0 > k ? r0 - k : 0;
    const int64_t xe = r0 + kSbRows + k < p.n ? r0 + kSbRows + k : p.n;
    double2 *S = reinterpret_cast<double2 *>(sb_smem);
    int4 *X0 = sb_smem + (size_t)(kSbRows + k) * sp;   // digits 0..3 of x_c
    int4 *X1 = X0 + (kSbRows + 2 * k);                 // digit 4, exponent, flags
    // band columns [cb, ce): entry b of column c goes to S[(c - cb) * sp + b];
    // idx / kp by a multiply-shift, exact while idx * (m * kp - 2^20) < 2^20
    // (idx < (R + k) kp <= 160 * 33 and m * kp - 2^20 < kp; idx * m < 2^28)
    const int total = (int)(ce - cb) * kp;
    const uint32_t m = ((1u << 20) + kp - 1) / kp;
    const double2 *src = p.AB + cb * p.ldab;
    for (int idx = t; idx < total; idx += kSbRows) {
        const int col = (int)(((uint32_t)idx * m) >> 20), b = idx - col * kp;
        S[col * sp + b] = src[(int64_t)col * p.ldab + b];
    }
    for (int c = t; c < (int)(xe - xb); c += kSbRows) {
        const fx::Dig g = fx::to_dig(fx::decode(p.x[vpos(xb + c, p.n, p.incx)]));
        X0[c] = make_int4(g.d[0], g.d[1], g.d[2], g.d[3]);
        X1[c] = make_int4(g.d[4], g.e, (int)g.flags, 0);
    }
    __syncthreads();
    const int64_t r = r0 + t;
    if (r >= p.n) return;
    const int lo = (int)(r < k ? r : k), hi = (int)(p.n - 1 - r < k ? p.n - 1 - r : k);
    const int cofs = (int)(r0 - cb), xofs = (int)(r0 - xb) + t;
    // stored entry (min(r, c), max(r, c)) (upper) or (max, min) (lower) of
    // c = r + d: column max (upper) / min (lower), band row k - |d| / |d|
    auto at = [&](int d) {
        const int ad = d < 0 ? -d : d;
        const int lj = t + cofs + (p.upper ? (d > 0 ? d : 0) : (d < 0 ? d : 0));
        return lj * sp + (p.upper ? k - ad : ad);
    };
    // block exponent: the largest exponent of a product with a finite,
    // nonzero factor pair (hi's exponent field as decode takes it)
    int emax = INT_MIN;
    for (int d = -lo; d <= hi; ++d) {
        const uint32_t hh = (uint32_t)__double2hiint(S[at(d)].x);
        const int eh = (int)((hh >> 20) & 0x7FFu);
        const int4 g1 = X1[xofs + d];
        if (eh == 0x7FF || (g1.z & (int)(fx::kZero | fx::kBad))) continue;
        const int ep = (eh ? eh : 1) - 1139 + g1.y;
        emax = ep > emax ? ep : emax;
    }
    fx::Acc acc;
    acc.reset();
    if (emax != INT_MIN) acc.preset(emax);
#pragma unroll 2
    for (int d = -lo; d <= hi; ++d) {
        const int4 g0 = X0[xofs + d], g1 = X1[xofs + d];
        fx::Dig g;
        g.d[0] = g0.x;
        g.d[1] = g0.y;
        g.d[2] = g0.z;
        g.d[3] = g0.w;
        g.d[4] = g1.x;
        g.e = g1.y;
        g.flags = (uint32_t)g1.z;
        g.pad = 0;
        acc.add_at(fx::decode(S[at(d)]), g);
    }
    double2 *py = p.y + vpos(r, p.n, p.incy);
    if (acc.bad) {
        const double nan = __longlong_as_double(0x7ff8000000000000ll);
        py[0] = make_double2(nan, nan);
        return;
    }
    const xfp::XF tot = xfp::xf_add(xzero(), acc.finish());
    smv_store_real(py, xfp::xf_from_dd(p.ar.hi, p.ar.lo), p.br, p.beta_kind, tot);
}

// ---- real symmetric packed product in two coalesced halves ----------------------------
// Row r of a symmetric packed matrix takes half of its entries from row r of
// the stored triangle and half from column r. k_smv's warp per row reads the
// column half contiguously but the row half at a stride of about r entries
// (32 lines per warp load). Here the row half goes GEMV-style, a thread per
// row over a chunk of kSpChunk columns, where for a fixed column consecutive
// rows are consecutive entries (k_spmv_rows, one partial sum per row and
// chunk), and the column half a warp per row, lanes over the contiguous
// column (k_spmv_cols). k_spmv_final adds each row's partial sums in a fixed
// order and forms y := beta*y + alpha*s with one rounding.
//   upper: AP[i + j(j+1)/2], i <= j: row half c >= r, column half c < r;
//   lower: AP[i + j(2n-j-1)/2], i >= j: row half c <= r, column half c > r.
constexpr int kSpChunk = 512;   // columns per row-half partial (<= 2048: no carry propagation needed)

template <bool UPPER>
__global__ void __launch_bounds__(256, 3) k_spmv_rows(int64_t n, const double2 *__restrict__ AP,
                                                      const fx::Dig *__restrict__ xd, fx::XFPod *__restrict__ part)
{
    const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t c0 = (int64_t)blockIdx.y * kSpChunk, c1 = min(n, c0 + kSpChunk);
    if (r >= n) return;
    // the row's columns in this chunk: upper [max(c0, r), c1), lower [c0, min(c1, r + 1))
    const int64_t cb = UPPER ? max(c0, r) : c0, ce = UPPER ? c1 : min(c1, r + 1);
    if (cb >= ce) return;   // no entries here (the final sum skips this chunk for row r)
    // entry (r, c): upper c(c+1)/2 + r, stepping by c + 1; lower r + c(2n-c-1)/2, stepping by n - c - 1
    int64_t at = UPPER ? cb * (cb + 1) / 2 + r : r + cb * (2 * n - cb - 1) / 2;
    auto step = [&](int64_t c) { return UPPER ? c + 1 : n - c - 1; };
    fx::Acc acc;
    acc.reset();
    int64_t c = cb;
    for (; c + 4 <= ce; c += 4) {
        const int64_t at1 = at + step(c), at2 = at1 + step(c + 1), at3 = at2 + step(c + 2);
        const double2 a0 = __ldcs(AP + at), a1 = __ldcs(AP + at1), a2 = __ldcs(AP + at2), a3 = __ldcs(AP + at3);
        at = at3 + step(c + 3);
        const fx::Dig x0 = xd[c], x1 = xd[c + 1], x2 = xd[c + 2], x3 = xd[c + 3];
        if (fx::decode_is_fast(a0) && fx::decode_is_fast(a1) && fx::decode_is_fast(a2) && fx::decode_is_fast(a3) &&
            ((x0.flags | x1.flags | x2.flags | x3.flags) & (fx::kZero | fx::kBad)) == 0) {
            const fx::Op o0 = fx::decode_fast(a0), o1 = fx::decode_fast(a1);
            const fx::Op o2 = fx::decode_fast(a2), o3 = fx::decode_fast(a3);
            const int e0 = o0.e + x0.e, e1 = o1.e + x1.e, e2 = o2.e + x2.e, e3 = o3.e + x3.e;
            acc.admit(max(max(e0, e1), max(e2, e3)));
            acc.mul_fast(o0, x0, acc.B - e0);
            acc.mul_fast(o1, x1, acc.B - e1);
            acc.mul_fast(o2, x2, acc.B - e2);
            acc.mul_fast(o3, x3, acc.B - e3);
        } else {
            acc.add_core(fx::decode(a0), x0);
            acc.add_core(fx::decode(a1), x1);
            acc.add_core(fx::decode(a2), x2);
            acc.add_core(fx::decode(a3), x3);
        }
    }
    for (; c < ce; ++c) {
        acc.add_core(fx::decode(__ldcs(AP + at)), xd[c]);
        at += step(c);
    }
    part[blockIdx.y * n + r] = fx::to_pod(acc.finish(), acc.bad);
}

template <bool UPPER>
__global__ void __launch_bounds__(256, 3) k_spmv_cols(int64_t n, const double2 *__restrict__ AP,
                                                   const fx::Dig *__restrict__ xd, fx::XFPod *__restrict__ partc)
{
    const int lane = threadIdx.x & 31;
    const int64_t warps = (int64_t)gridDim.x * blockDim.x / 32;
    for (int64_t w = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) / 32; w < n; w += warps) {
        // longest columns first (upper: row r's column has r entries, lower
        // n - 1 - r), so that the blocks the scheduler hands out last are the
        // short ones
        const int64_t r = UPPER ? n - 1 - w : w;
        // column r of the stored triangle: upper rows [0, r) at r(r+1)/2,
        // lower rows (r, n) at r + 1 + r(2n-r-1)/2, both contiguous
        const int64_t cb = UPPER ? 0 : r + 1, ce = UPPER ? r : n;
        const double2 *col = AP + (UPPER ? r * (r + 1) / 2 : r * (2 * n - r - 1) / 2 + r + 1) - cb;
        // fewer than fx::kMaxAdds products per lane (the host keeps n within
        // 65535 chunks, below 2^25); four loads in flight per lane, carries
        // propagated after each run of 2048 products
        fx::Acc acc;
        acc.reset();
        int64_t c = cb + lane;
        while (c + 96 < ce) {
            const int64_t cend = c + 128 * 512;
            for (; c + 96 < ce && c < cend; c += 128) {
                const double2 a0 = __ldcs(col + c), a1 = __ldcs(col + c + 32);
                const double2 a2 = __ldcs(col + c + 64), a3 = __ldcs(col + c + 96);
                const fx::Dig x0 = xd[c], x1 = xd[c + 32], x2 = xd[c + 64], x3 = xd[c + 96];
                if (fx::decode_is_fast(a0) && fx::decode_is_fast(a1) && fx::decode_is_fast(a2) &&
                    fx::decode_is_fast(a3) && ((x0.flags | x1.flags | x2.flags | x3.flags) & (fx::kZero | fx::kBad)) == 0) {
                    const fx::Op o0 = fx::decode_fast(a0), o1 = fx::decode_fast(a1);
                    const fx::Op o2 = fx::decode_fast(a2), o3 = fx::decode_fast(a3);
                    const int e0 = o0.e + x0.e, e1 = o1.e + x1.e, e2 = o2.e + x2.e, e3 = o3.e + x3.e;
                    acc.admit(max(max(e0, e1), max(e2, e3)));
                    acc.mul_fast(o0, x0, acc.B - e0);
                    acc.mul_fast(o1, x1, acc.B - e1);
                    acc.mul_fast(o2, x2, acc.B - e2);
                    acc.mul_fast(o3, x3, acc.B - e3);
                } else {
                    acc.add_core(fx::decode(a0), x0);
                    acc.add_core(fx::decode(a1), x1);
                    acc.add_core(fx::decode(a2), x2);
                    acc.add_core(fx::decode(a3), x3);
                }
            }
            acc.normalize();
        }
        for (; c < ce; c += 32) acc.add_core(fx::decode(__ldcs(col + c)), xd[c]);
        const xfp::XF tot = fx::xf_warp_sum(xfp::xf_add(xzero(), acc.finish()));
        const bool bad = __any_sync(0xffffffffu, acc.bad);
        if (lane == 0) partc[r] = fx::to_pod(tot, bad);
    }
}

// y(r) := beta*y(r) + alpha*(column half + row-half chunks in ascending order)
__global__ void k_spmv_final(int64_t n, bool upper, const fx::XFPod *__restrict__ part,
                             const fx::XFPod *__restrict__ partc, dd::real ar, dd::real br, int beta_kind, double2 *y,
                             int64_t incy)
{
    const xfp::XF xar = xfp::xf_from_dd(ar.hi, ar.lo);
    const int64_t nch = (n + kSpChunk - 1) / kSpChunk;
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
        const fx::XFPod pc = partc[r];
        bool bad = (pc.flags & 4) != 0;
        xfp::XF s = fx::from_pod(pc);
        const int64_t q0 = upper ? r / kSpChunk : 0, q1 = upper ? nch : r / kSpChunk + 1;
        for (int64_t q = q0; q < q1; ++q) {
            const fx::XFPod p = part[q * n + r];
            bad |= (p.flags & 4) != 0;
            s = xfp::xf_add(s, fx::from_pod(p));
        }
        double2 *py = y + vpos(r, n, incy);
        if (bad) {
            const double nan = __longlong_as_double(0x7ff8000000000000ll);
            *py = make_double2(nan, nan);
            continue;
        }
        smv_store_real(py, xar, br, beta_kind, s);
    }
}

// ---- triangular band solve, read in place ----------------------------------------------
// op(A) x = b for a band triangle of bandwidth k, by one warp: rows are taken
// 32 at a time in solve order (lane l owns the l-th row of the tile). Each
// lane first sums its row's band entries against the solutions of earlier
// tiles (independent across lanes); then 32 steps finish one row each: the
// owner forms x_r = (b_r - s_r) * (1 / a_rr), broadcasts it, and the later
// rows of the tile add their entry times x_r. The sums are double-double
// (scalar operators): with a single warp, finishing a fixed-point sum per row
// (a 256-bit conversion on one lane) costs more than the products. Work
// O(n k), memory the band itself.
struct TbsvParams {
    int64_t n, k, ldab;
    const double2 *AB;
    int op;             // 0 'N', 1 'T', 2 'C'
    bool upper, unit;   // stored triangle, unit diagonal
    double2 *x;         // contiguous, b on entry
};

template <bool CX>
__device__ __forceinline__ dd::cplx tbsv_entry(const TbsvParams &p, int64_t r, int64_t c)
{
    const int64_t i = p.op == 0 ? r : c, j = p.op == 0 ? c : r;
    const double2 *a = p.AB + (CX ? 2 : 1) * ((p.upper ? p.k : 0) + i - j + j * p.ldab);
    dd::cplx v;
    v.re = dd::load(a);
    v.im = CX ? dd::load(a + 1) : dd::make(0.0, 0.0);
    if (CX && p.op == 2) v.im = dd::neg(v.im);
    return v;
}

// s += a * x in double-double (scalar operators; complex: re = ar xr - ai xi,
// im = ar xi + ai xr)
template <bool CX>
__device__ __forceinline__ void tbsv_add(dd::cplx &s, const dd::cplx &a, const dd::cplx &x)
{
    if (CX) {
        s = dd::cadd_exact(s, dd::cmul_exact(a, x));
    } else {
        s.re = dd::add_exact(s.re, dd::mul_exact(a.re, x.re));
    }
}

template <bool CX>
__global__ void __launch_bounds__(32) k_tbsv(TbsvParams p)
{
    const int lane = threadIdx.x & 31;
    const bool forward = p.upper == (p.op != 0);   // op(A) lower: rows in increasing order
    auto row_of = [&](int64_t s) { return forward ? s : p.n - 1 - s; };
    const dd::real zero = dd::make(0.0, 0.0);
    for (int64_t t0 = 0; t0 < p.n; t0 += 32) {
        const int64_t s = t0 + lane;
        const bool live = s < p.n;
        const int64_t r = live ? row_of(s) : row_of(p.n - 1);
        dd::cplx acc{zero, zero};
        dd::cplx b;
        if (CX) {
            b = dd::cload(p.x + 2 * r);
        } else {
            b.re = dd::load(p.x + r);
            b.im = zero;
        }
        // 1/a_rr (complex: conj(d) / |d|^2)
        dd::cplx inv{dd::make(1.0, 0.0), zero};
        if (!p.unit) {
            const dd::cplx d = tbsv_entry<CX>(p, r, r);
            if (CX) {
                const dd::real m2 = dd::add_exact(dd::mul_exact(d.re, d.re), dd::mul_exact(d.im, d.im));
                const dd::real q = dd::div(dd::make(1.0, 0.0), m2);
                inv.re = dd::mul_exact(d.re, q);
                inv.im = dd::neg(dd::mul_exact(d.im, q));
            } else {
                inv.re = dd::div(dd::make(1.0, 0.0), d.re);
            }
        }
        // solutions of earlier tiles within the band
        if (live) {
            for (int64_t s2 = (s - p.k > 0 ? s - p.k : 0); s2 < t0; ++s2) {
                const int64_t c = row_of(s2);
                dd::cplx xc;
                xc.re = dd::load(p.x + (CX ? 2 * c : c));
                xc.im = CX ? dd::load(p.x + 2 * c + 1) : zero;
                tbsv_add<CX>(acc, tbsv_entry<CX>(p, r, c), xc);
            }
        }
        // the tile, one row per step
        const int steps = (p.n - t0 < 32) ? (int)(p.n - t0) : 32;
        for (int u = 0; u < steps; ++u) {
            dd::cplx v{zero, zero};
            if (lane == u) {
                v.re = dd::sub_exact(b.re, acc.re);
                v.im = CX ? dd::sub_exact(b.im, acc.im) : zero;
                if (!p.unit) {
                    if (CX) v = dd::cmul_exact(v, inv);
                    else v.re = dd::mul_exact(v.re, inv.re);
                }
                if (CX) dd::cstore(p.x + 2 * r, v);
                else dd::store(p.x + r, v.re);
            }
            v.re.hi = __shfl_sync(0xffffffffu, v.re.hi, u);
            v.re.lo = __shfl_sync(0xffffffffu, v.re.lo, u);
            if (CX) {
                v.im.hi = __shfl_sync(0xffffffffu, v.im.hi, u);
                v.im.lo = __shfl_sync(0xffffffffu, v.im.lo, u);
            }
            if (live && lane > u && lane - u <= p.k) tbsv_add<CX>(acc, tbsv_entry<CX>(p, r, row_of(t0 + u)), v);
        }
        __syncwarp();
    }
}

// ---- partitioned band solve (k <= 31) ----------------------------------------------
// The rows, in solve order, are cut into P chunks of L >= 2k. With the
// incoming solutions of the previous chunk's last k rows t_{c-1}, chunk c
// satisfies T_c x_c = b_c - E_c t_{c-1} (E_c: the band entries reaching back
// into chunk c-1). So x_c = y_c - V_c t_{c-1} with T_c y_c = b_c and
// T_c V_c = E_c, all chunks solved independently (lane 0: y, lane 1 + j:
// column j of V); then one warp carries t_c = tail(y_c) - tail(V_c) t_{c-1}
// across the chunks, and every row is corrected in parallel. Work (k + 1)
// times the serial solve's, in parallel over P chunks; memory O(n k).
struct SpikeParams {
    TbsvParams t;
    int64_t L, P;
    double2 *invd;   // n entries: 1 / op(A)(r, r) by solve position (complex: 2 per entry)
    double2 *Y;      // n: local solutions for b
    double2 *V;      // n * k: local solutions for the coupling columns, [s][j]
    double2 *T;      // P * k: t_c
};

template <bool CX>
__device__ __forceinline__ dd::cplx sp_load(const double2 *p, int64_t i)
{
    dd::cplx v;
    if (CX) {
        v = dd::cload(p + 2 * i);
    } else {
        v.re = dd::load(p + i);
        v.im = dd::make(0.0, 0.0);
    }
    return v;
}

template <bool CX>
__device__ __forceinline__ void sp_store(double2 *p, int64_t i, const dd::cplx &v)
{
    if (CX) dd::cstore(p + 2 * i, v);
    else dd::store(p + i, v.re);
}

__device__ __forceinline__ int64_t sp_row(const TbsvParams &p, bool forward, int64_t s)
{
    return forward ? s : p.n - 1 - s;
}

template <bool CX>
__global__ void k_spike_invdiag(SpikeParams q)
{
    const TbsvParams &p = q.t;
    const bool forward = p.upper == (p.op != 0);
    for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < p.n; s += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = sp_row(p, forward, s);
        dd::cplx inv{dd::make(1.0, 0.0), dd::make(0.0, 0.0)};
        if (!p.unit) {
            const dd::cplx d = tbsv_entry<CX>(p, r, r);
            if (CX) {
                const dd::real m2 = dd::add_exact(dd::mul_exact(d.re, d.re), dd::mul_exact(d.im, d.im));
                const dd::real qq = dd::div(dd::make(1.0, 0.0), m2);
                inv.re = dd::mul_exact(d.re, qq);
                inv.im = dd::neg(dd::mul_exact(d.im, qq));
            } else {
                inv.re = dd::div(dd::make(1.0, 0.0), d.re);
            }
        }
        sp_store<CX>(q.invd, s, inv);
    }
}

// one warp per chunk: lane 0 solves for b, lane 1 + j for coupling column j
template <bool CX>
__global__ void __launch_bounds__(128) k_spike_local(SpikeParams q)
{
    const TbsvParams &p = q.t;
    const bool forward = p.upper == (p.op != 0);
    const int lane = threadIdx.x & 31;
    const int64_t c = blockIdx.x * (int64_t)(blockDim.x / 32) + (threadIdx.x >> 5);
    if (c >= q.P) return;
    const int k = (int)p.k;
    if (lane > k || (c == 0 && lane > 0)) return;   // chunk 0 has no incoming coupling
    const int64_t s0 = c * q.L, s1 = (s0 + q.L < p.n) ? s0 + q.L : p.n;
    const int j = lane - 1;
    const int64_t sj = s0 - k + j;   // the previous chunk's row that coupling column j stands for
    const dd::real zero = dd::make(0.0, 0.0);
    for (int64_t s = s0; s < s1; ++s) {
        const int64_t r = sp_row(p, forward, s);
        dd::cplx rhs{zero, zero};
        if (lane == 0) rhs = sp_load<CX>(p.x, r);
        else if (s - sj <= k) rhs = tbsv_entry<CX>(p, r, sp_row(p, forward, sj));
        dd::cplx acc{zero, zero};
        for (int64_t s2 = (s - k > s0 ? s - k : s0); s2 < s; ++s2) {
            const dd::cplx xv = lane == 0 ? sp_load<CX>(q.Y, s2) : sp_load<CX>(q.V, s2 * k + j);
            tbsv_add<CX>(acc, tbsv_entry<CX>(p, r, sp_row(p, forward, s2)), xv);
        }
        dd::cplx v;
        v.re = dd::sub_exact(rhs.re, acc.re);
        v.im = CX ? dd::sub_exact(rhs.im, acc.im) : zero;
        if (!p.unit) {
            const dd::cplx inv = sp_load<CX>(q.invd, s);
            if (CX) v = dd::cmul_exact(v, inv);
            else v.re = dd::mul_exact(v.re, inv.re);
        }
        if (lane == 0) sp_store<CX>(q.Y, s, v);
        else sp_store<CX>(q.V, s * k + j, v);
    }
}

// one warp, chunk after chunk: t_c[i] = Y[s_i] - sum_j V[s_i][j] t_{c-1}[j]
// for the last k rows s_i of chunk c (t_0 = the tail of Y in chunk 0)
template <bool CX>
__global__ void __launch_bounds__(32) k_spike_carry(SpikeParams q)
{
    const TbsvParams &p = q.t;
    const int lane = threadIdx.x & 31;
    const int k = (int)p.k;
    const dd::real zero = dd::make(0.0, 0.0);
    const unsigned mk = (1u << k) - 1u;   // lanes 0 .. k-1 (1 <= k <= 31)
    dd::cplx t{zero, zero};   // lane i < k: t_{c-1}[i]
    for (int64_t c = 0; c + 1 < q.P; ++c) {
        const int64_t si = (c + 1) * q.L - k + lane;
        dd::cplx v{zero, zero};
        if (lane < k) {
            v = sp_load<CX>(q.Y, si);
            if (c > 0) {
                dd::cplx acc{zero, zero};
                for (int jj = 0; jj < k; ++jj) {
                    dd::cplx tj;
                    tj.re.hi = __shfl_sync(mk, t.re.hi, jj);
                    tj.re.lo = __shfl_sync(mk, t.re.lo, jj);
                    tj.im = zero;
                    if (CX) {
                        tj.im.hi = __shfl_sync(mk, t.im.hi, jj);
                        tj.im.lo = __shfl_sync(mk, t.im.lo, jj);
                    }
                    tbsv_add<CX>(acc, sp_load<CX>(q.V, si * k + jj), tj);
                }
                v.re = dd::sub_exact(v.re, acc.re);
                if (CX) v.im = dd::sub_exact(v.im, acc.im);
            }
            sp_store<CX>(q.T, c * k + lane, v);
        }
        t = v;
        __syncwarp();
    }
}

// x(row of s) = Y[s] - sum_j V[s][j] t_{c-1}[j] for s in chunk c >= 1; Y[s] in chunk 0
template <bool CX>
__global__ void k_spike_correct(SpikeParams q)
{
    const TbsvParams &p = q.t;
    const bool forward = p.upper == (p.op != 0);
    const int k = (int)p.k;
    for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < p.n; s += (int64_t)gridDim.x * blockDim.x) {
        const int64_t c = s / q.L;
        dd::cplx v = sp_load<CX>(q.Y, s);
        if (c > 0) {
            dd::cplx acc{dd::make(0.0, 0.0), dd::make(0.0, 0.0)};
            for (int jj = 0; jj < k; ++jj)
                tbsv_add<CX>(acc, sp_load<CX>(q.V, s * k + jj), sp_load<CX>(q.T, (c - 1) * k + jj));
            v.re = dd::sub_exact(v.re, acc.re);
            if (CX) v.im = dd::sub_exact(v.im, acc.im);
        }
        sp_store<CX>(p.x, sp_row(p, forward, s), v);
    }
}

// ---- rank-1 / rank-2 updates, elementwise -------------------------------------------
// A(i, j) += u_i v_j (+ u2_i v2_j) over the whole matrix (uplo 0) or one
// triangle (1 upper, 2 lower), with u = x, v_j = alpha op(y_j) and, for the
// rank-2 forms, u2 = y, v2_j = alpha x_j (symmetric) or conj(alpha x_j)
// (Hermitian): the reference BLAS association (temp = alpha * y(j);
// a(i, j) += x(i) * temp). Hermitian updates leave the diagonal real.

// v[j] = a * op(w[j]) with op = conj when `conj`; conj_after: v = conj(a w)
template <bool CX>
__global__ void k_rank_prep(int64_t n, const double2 *w, dd::cplx a, bool conj, bool conj_after, double2 *v)
{
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x) {
        if (CX) {
            dd::cplx wj = dd::cload(w + 2 * j);
            if (conj) wj.im = dd::neg(wj.im);
            dd::cplx r = dd::cmul_exact(a, wj);
            if (conj_after) r.im = dd::neg(r.im);
            dd::cstore(v + 2 * j, r);
        } else {
            dd::store(v + j, dd::mul_exact(a.re, dd::load(w + j)));
        }
    }
}

// lda < 0: A is the packed triangle (upper: i + j(j+1)/2, lower: i + j(2m-j-1)/2)
template <bool CX, bool TWO>
__global__ void k_rank_update(int64_t m, int64_t n, const double2 *__restrict__ u, const double2 *__restrict__ v,
                              const double2 *__restrict__ u2, const double2 *__restrict__ v2, int uplo, bool herm,
                              double2 *A, int64_t lda)
{
    const int64_t total = m * n;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = t % m, j = t / m;
        if ((uplo == 1 && i > j) || (uplo == 2 && i < j)) continue;
        const int64_t pos = lda >= 0 ? i + j * lda : (uplo == 1 ? i + j * (j + 1) / 2 : i + j * (2 * m - j - 1) / 2);
        double2 *pa = A + (CX ? 2 : 1) * pos;
        if (CX) {
            dd::cplx acc = dd::cadd_exact(dd::cload(pa), dd::cmul_exact(dd::cload(u + 2 * i), dd::cload(v + 2 * j)));
            if (TWO) acc = dd::cadd_exact(acc, dd::cmul_exact(dd::cload(u2 + 2 * i), dd::cload(v2 + 2 * j)));
            if (herm && i == j) acc.im = dd::make(0.0, 0.0);
            dd::cstore(pa, acc);
        } else {
            dd::real acc = dd::add_exact(dd::load(pa), dd::mul_exact(dd::load(u + i), dd::load(v + j)));
            if (TWO) acc = dd::add_exact(acc, dd::mul_exact(dd::load(u2 + i), dd::load(v2 + j)));
            dd::store(pa, acc);
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

// Real symmetric band of bandwidth <= kSbMaxK on the shared-memory tile
// kernel, x read in place; y too unless it overlaps x (then through a
// contiguous copy).
bool sbmv_tile(const SmvArgs &a, const char *routine)
{
    SbParams q;
    q.n = a.n;
    q.ldab = a.ldab;
    q.k = (int)(a.upper ? a.ku : a.kl);
    q.upper = a.upper;
    q.AB = (const double2 *)a.A;
    q.x = (const double2 *)a.x;
    q.incx = a.incx;
    q.ar = dd::make(a.alpha.hi, a.alpha.lo);
    q.br = dd::make(a.beta.hi, a.beta.lo);
    q.beta_kind = a.beta_kind;
    // byte ranges of the two vectors
    auto span = [&](const void *v, int64_t inc, uintptr_t &lo, uintptr_t &hi) {
        const int64_t ext = (a.n - 1) * (inc < 0 ? -inc : inc);
        lo = (uintptr_t)v;
        hi = lo + (uintptr_t)(ext + 1) * sizeof(double2);
    };
    uintptr_t xl, xh, yl, yh;
    span(a.x, a.incx, xl, xh);
    span(a.y, a.incy, yl, yh);
    const bool direct = xh <= yl || yh <= xl;
    void *yb = nullptr;
    if (direct) {
        q.y = (double2 *)a.y;
        q.incy = a.incy;
    } else {
        yb = dev_alloc((size_t)a.n * sizeof(double2), routine);
        if (!yb) return false;
        if (a.beta_kind != 0) vgather(a.n, a.y, a.incy, 1, yb, true);
        q.y = (double2 *)yb;
        q.incy = 1;
    }
    static int attr_set[64];
    int dev = 0;
    cudaGetDevice(&dev);
    if (!attr_set[dev & 63]) {
        cudaFuncSetAttribute(k_sbmv_tile, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sb_smem_bytes(kSbMaxK));
        attr_set[dev & 63] = 1;
    }
    k_sbmv_tile<<<(unsigned)((a.n + kSbRows - 1) / kSbRows), kSbRows, sb_smem_bytes(q.k), stream()>>>(q);
    count_launch();
    if (!direct) {
        vgather(a.n, a.y, a.incy, 1, yb, false);
        dev_free(yb);
    }
    return true;
}

// Real symmetric packed matrix: the row halves in column chunks, the column
// halves a warp per row, then the per-row sums (x as digit sets; y in place
// unless it overlaps x).
bool spmv_split(const SmvArgs &a, const char *routine)
{
    const int64_t n = a.n, nch = (n + kSpChunk - 1) / kSpChunk;
    const size_t xd_bytes = ((size_t)n * sizeof(fx::Dig) + 255) / 256 * 256;
    const size_t part_bytes = ((size_t)(nch * n) * sizeof(fx::XFPod) + 255) / 256 * 256;
    char *buf = (char *)dev_alloc(xd_bytes + part_bytes + (size_t)n * sizeof(fx::XFPod), routine);
    if (!buf) return false;
    fx::Dig *xd = (fx::Dig *)buf;
    fx::XFPod *part = (fx::XFPod *)(buf + xd_bytes), *partc = (fx::XFPod *)(buf + xd_bytes + part_bytes);
    k_vdig<<<blocks_for(n), kThreads, 0, stream()>>>(n, (const double2 *)a.x, a.incx, 1, xd);
    const double2 *AP = (const double2 *)a.A;
    const dim3 grid((unsigned)((n + 255) / 256), (unsigned)nch);
    // a warp per row, every row in the grid: the block scheduler balances
    // the uneven column lengths
    const int64_t wblocks = (n * 32 + 255) / 256;
    if (a.upper) {
        k_spmv_rows<true><<<grid, 256, 0, stream()>>>(n, AP, xd, part);
        k_spmv_cols<true><<<(unsigned)wblocks, 256, 0, stream()>>>(n, AP, xd, partc);
    } else {
        k_spmv_rows<false><<<grid, 256, 0, stream()>>>(n, AP, xd, part);
        k_spmv_cols<false><<<(unsigned)wblocks, 256, 0, stream()>>>(n, AP, xd, partc);
    }
    // y in place unless it overlaps x
    const uintptr_t xl = (uintptr_t)a.x, xh = xl + (uintptr_t)((n - 1) * (a.incx < 0 ? -a.incx : a.incx) + 1) * 16;
    const uintptr_t yl = (uintptr_t)a.y, yh = yl + (uintptr_t)((n - 1) * (a.incy < 0 ? -a.incy : a.incy) + 1) * 16;
    const bool direct = xh <= yl || yh <= xl;
    void *yb = nullptr;
    if (!direct) {
        yb = dev_alloc((size_t)n * sizeof(double2), routine);
        if (!yb) {
            dev_free(buf);
            return false;
        }
        if (a.beta_kind != 0) vgather(n, a.y, a.incy, 1, yb, true);
    }
    k_spmv_final<<<blocks_for(n), kThreads, 0, stream()>>>(
        n, a.upper, part, partc, dd::make(a.alpha.hi, a.alpha.lo), dd::make(a.beta.hi, a.beta.lo), a.beta_kind,
        direct ? (double2 *)a.y : (double2 *)yb, direct ? a.incy : 1);
    count_launch(4);
    if (!direct) {
        vgather(n, a.y, a.incy, 1, yb, false);
        dev_free(yb);
    }
    dev_free(buf);
    return true;
}

bool smv_device(const SmvArgs &a, const char *routine)
{
    if (!a.cplx && a.kind == 1 && a.fmt == 1 && a.n > 0 && (a.upper ? a.ku : a.kl) <= kSbMaxK &&
        g_band_tile.load() != 0)
        return sbmv_tile(a, routine);
    if (!a.cplx && a.kind == 1 && a.fmt == 2 && a.n > 0 && a.n <= (int64_t)65535 * kSpChunk && g_band_tile.load() != 0)
        return spmv_split(a, routine);
    const int e2 = a.cplx ? 2 : 1;
    const size_t es = 16 * (size_t)e2;
    Buf xb((size_t)(a.cols > 0 ? a.cols : 1) * e2 * sizeof(fx::Dig), routine),
        yb((size_t)(a.rows > 0 ? a.rows : 1) * es, routine);
    if (!xb.p || !yb.p) return false;
    k_vdig<<<blocks_for(a.cols * e2), kThreads, 0, stream()>>>(a.cols, (const double2 *)a.x, a.incx, e2,
                                                              (fx::Dig *)xb.p);
    count_launch();
    if (a.beta_kind != 0) vgather(a.rows, a.y, a.incy, e2, yb.p, true);
    SmvParams p;
    p.rows = a.rows;
    p.cols = a.cols;
    p.n = a.n;
    p.kl = a.kl;
    p.ku = a.ku;
    p.ldab = a.ldab;
    p.A = (const double2 *)a.A;
    p.fmt = a.fmt;
    p.kind = a.kind;
    p.op = a.trans == 'N' ? 0 : (a.trans == 'T' ? 1 : 2);
    p.upper = a.upper;
    p.unit = a.unit;
    p.xd = (const fx::Dig *)xb.p;
    p.y = (double2 *)yb.p;
    if (a.cplx) {
        p.ar = dd::make(a.calpha.re.hi, a.calpha.re.lo);
        p.ai = dd::make(a.calpha.im.hi, a.calpha.im.lo);
        p.br = dd::make(a.cbeta.re.hi, a.cbeta.re.lo);
        p.bi = dd::make(a.cbeta.im.hi, a.cbeta.im.lo);
    } else {
        p.ar = dd::make(a.alpha.hi, a.alpha.lo);
        p.ai = dd::make(0.0, 0.0);
        p.br = dd::make(a.beta.hi, a.beta.lo);
        p.bi = dd::make(0.0, 0.0);
    }
    p.beta_kind = a.beta_kind;
    // average stored entries per row: a warp per row once rows are long
    int64_t len;
    if (a.fmt == 0) len = a.cols;
    else if (a.fmt == 2) len = a.kind == 3 ? (a.n + 1) / 2 : a.n;
    else if (a.kind == 0) len = a.kl + a.ku + 1;
    else len = (a.kind == 3 ? 1 : 2) * (a.kl > a.ku ? a.kl : a.ku) + 1;
    const bool warp = len >= 48;
    const int64_t threads = a.rows * (warp ? 32 : 1);
    int64_t blocks = (threads + 255) / 256;
    const int64_t cap = (int64_t)device_sm_count() * 8;
    if (blocks > cap) blocks = cap;
    if (blocks < 1) blocks = 1;
    if (a.cplx) {
        if (warp) k_smv<true, 32><<<(unsigned)blocks, 256, 0, stream()>>>(p);
        else k_smv<true, 1><<<(unsigned)blocks, 256, 0, stream()>>>(p);
    } else {
        if (warp) k_smv<false, 32><<<(unsigned)blocks, 256, 0, stream()>>>(p);
        else k_smv<false, 1><<<(unsigned)blocks, 256, 0, stream()>>>(p);
    }
    count_launch();
    vgather(a.rows, a.y, a.incy, e2, yb.p, false);
    return true;
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

bool tbsv_device(bool cplx, char uplo, char trans, char diag, int64_t n, int64_t k, const void *AB, int64_t ldab,
                 void *x, int64_t incx, const char *routine)
{
    const int e2 = cplx ? 2 : 1;
    Buf xb((size_t)n * 16 * e2, routine);
    if (!xb.p) return false;
    vgather(n, x, incx, e2, xb.p, true);
    TbsvParams p;
    p.n = n;
    p.k = k;
    p.ldab = ldab;
    p.AB = (const double2 *)AB;
    p.op = trans == 'N' ? 0 : (trans == 'T' ? 1 : 2);
    p.upper = uplo == 'U';
    p.unit = diag == 'U';
    p.x = (double2 *)xb.p;
    // chunks of L >= 2k rows, about a thousand of them
    int64_t L = (n + 1023) / 1024;
    if (L < 2 * k) L = 2 * k;
    if (L < 64) L = 64;
    const int64_t P = (n + L - 1) / L;
    if (k >= 1 && k <= 31 && P >= 2) {
        SpikeParams q;
        q.t = p;
        q.L = L;
        q.P = P;
        const size_t es = (size_t)16 * e2;
        Buf sb(es * ((size_t)n * (2 + (size_t)k) + (size_t)P * k), routine);
        if (!sb.p) return false;
        q.invd = (double2 *)sb.p;
        q.Y = q.invd + (size_t)n * e2;
        q.V = q.Y + (size_t)n * e2;
        q.T = q.V + (size_t)n * k * e2;
        const unsigned gl = (unsigned)((P + 3) / 4);
        if (cplx) {
            k_spike_invdiag<true><<<blocks_for(n), kThreads, 0, stream()>>>(q);
            k_spike_local<true><<<gl, 128, 0, stream()>>>(q);
            k_spike_carry<true><<<1, 32, 0, stream()>>>(q);
            k_spike_correct<true><<<blocks_for(n), kThreads, 0, stream()>>>(q);
        } else {
            k_spike_invdiag<false><<<blocks_for(n), kThreads, 0, stream()>>>(q);
            k_spike_local<false><<<gl, 128, 0, stream()>>>(q);
            k_spike_carry<false><<<1, 32, 0, stream()>>>(q);
            k_spike_correct<false><<<blocks_for(n), kThreads, 0, stream()>>>(q);
        }
        count_launch(4);
    } else {
        if (cplx) k_tbsv<true><<<1, 32, 0, stream()>>>(p);
        else k_tbsv<false><<<1, 32, 0, stream()>>>(p);
        count_launch();
    }
    vgather(n, x, incx, e2, xb.p, false);
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
    if (r.lda < 0 && r.uplo == 0) {
        // lda < 0 marks a packed triangle, which only SPR/HPR/SPR2/HPR2 (uplo
        // set) hand over; a general rank update never has one
        set_error(routine, MWBLAS_ERR_UNSUPPORTED, "packed storage without a triangle");
        return false;
    }
    const int e2 = r.cplx ? 2 : 1;
    const bool two = r.y && r.uplo != 0;           // SYR2 / HER2
    const bool herm = r.cplx && r.conj && r.uplo != 0;
    const int64_t ny = r.uplo == 0 ? r.n : r.m;    // length of y (GER) or of x (SYR/HER)
    // u = x, v = alpha op(y) (GER) or alpha op(x) (SYR/HER); for rank 2: u2 = y, v2 = alpha x or conj(alpha x)
    Buf xb((size_t)r.m * 16 * e2, routine), yb((size_t)ny * 16 * e2, routine), vb((size_t)ny * 16 * e2, routine),
        v2b((size_t)(two ? r.m : 1) * 16 * e2, routine);
    if (!xb.p || !yb.p || !vb.p || !v2b.p) return false;
    vgather(r.m, r.x, r.incx, e2, xb.p, true);
    if (r.y) vgather(ny, r.y, r.incy, e2, yb.p, true);
    dd::cplx a;
    if (r.cplx) {
        a.re = dd::make(r.calpha.re.hi, r.calpha.re.lo);
        a.im = dd::make(r.calpha.im.hi, r.calpha.im.lo);
    } else {
        a.re = dd::make(r.alpha.hi, r.alpha.lo);
        a.im = dd::make(0.0, 0.0);
    }
    if (herm && !two) a.im = dd::make(0.0, 0.0);   // HER: alpha real
    const double2 *ysrc = (const double2 *)(r.y ? yb.p : xb.p);
    const double2 *u = (const double2 *)xb.p, *v = (const double2 *)vb.p;
    const double2 *u2 = two ? (const double2 *)yb.p : nullptr, *v2 = two ? (const double2 *)v2b.p : nullptr;
    if (r.cplx) {
        k_rank_prep<true><<<blocks_for(ny), kThreads, 0, stream()>>>(ny, ysrc, a, r.conj, false, (double2 *)vb.p);
        if (two)
            k_rank_prep<true><<<blocks_for(r.m), kThreads, 0, stream()>>>(r.m, (const double2 *)xb.p, a, false, herm,
                                                                        (double2 *)v2b.p);
    } else {
        k_rank_prep<false><<<blocks_for(ny), kThreads, 0, stream()>>>(ny, ysrc, a, false, false, (double2 *)vb.p);
        if (two)
            k_rank_prep<false><<<blocks_for(r.m), kThreads, 0, stream()>>>(r.m, (const double2 *)xb.p, a, false, false,
                                                                         (double2 *)v2b.p);
    }
    const int64_t cols = r.uplo == 0 ? r.n : r.m;
    const unsigned g = blocks_for(r.m * cols);
    double2 *A = (double2 *)r.A;
    if (r.cplx) {
        if (two) k_rank_update<true, true><<<g, kThreads, 0, stream()>>>(r.m, cols, u, v, u2, v2, r.uplo, herm, A, r.lda);
        else k_rank_update<true, false><<<g, kThreads, 0, stream()>>>(r.m, cols, u, v, u2, v2, r.uplo, herm, A, r.lda);
    } else {
        if (two) k_rank_update<false, true><<<g, kThreads, 0, stream()>>>(r.m, cols, u, v, u2, v2, r.uplo, false, A, r.lda);
        else k_rank_update<false, false><<<g, kThreads, 0, stream()>>>(r.m, cols, u, v, u2, v2, r.uplo, false, A, r.lda);
    }
    count_launch(two ? 3 : 2);
    return true;
}

}  // namespace mw

extern "C" int mwblas_set_band_tile(int on) { return mw::g_band_tile.exchange(on ? 1 : 0); }
