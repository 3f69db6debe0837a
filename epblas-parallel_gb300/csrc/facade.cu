// The drop-in boundary: extern "C" Fortran-ABI entry points.
//
// Each routine is written once as a template over the integer type and
// instantiated twice, as `name_` (int, LP64) and `name_64_` (int64_t, ILP64),
// mirroring EPBLAS_FACADE_PAIR (src/epblas-parallel/common/epblas_facade.h:
// 63-65). Scalars arrive by pointer and are read on the host; arrays may be
// host or device memory (see runtime.h). Quick returns and special scalar
// values follow the reference's *_core functions line for line; the checks
// the reference does not have (leading dimensions, flag letters, null
// pointers) record an error and leave the outputs untouched.
#include <atomic>
#include <cctype>
#include <cstring>

#include "gemm.h"
#include "l1.h"
#include "l1x.h"
#include "level3.h"
#include "level3x.h"
#include "level2x.h"
#include "runtime.h"

namespace mw {

namespace {

inline char up(const char *c) { return (char)std::toupper((unsigned char)*c); }
// blas_trans_real (common/blas_char.h:36): 'C' folds to 'T'.
inline char trans_real(const char *c)
{
    char t = up(c);
    return t == 'C' ? 'T' : t;
}

inline dd_host rd(const mwblas_real64x2 *p) { return dd_host{p->limbs[0], p->limbs[1]}; }
inline cdd_host cd(const mwblas_complex64x2 *p)
{
    return cdd_host{{p->re.limbs[0], p->re.limbs[1]}, {p->im.limbs[0], p->im.limbs[1]}};
}
// mf_pred.h:28-32
inline bool eq0(dd_host a) { return a.hi == 0.0 && a.lo == 0.0; }
inline bool eq1(dd_host a) { return a.hi == 1.0 && a.lo == 0.0; }
inline bool ceq0(cdd_host a) { return eq0(a.re) && eq0(a.im); }
inline bool ceq1(cdd_host a) { return eq1(a.re) && eq0(a.im); }
inline int beta_kind(dd_host b) { return eq0(b) ? 0 : (eq1(b) ? 1 : 2); }
inline int beta_kind(cdd_host b) { return ceq0(b) ? 0 : (ceq1(b) ? 1 : 2); }

int g_engine_init = -1;
int g_engine = MWBLAS_GEMM_AUTO;
int g_ozaki_bits = 0;

int engine()
{
    if (g_engine_init < 0) {
        g_engine_init = 1;
        const char *e = getenv("MWBLAS_GEMM");
        if (e) {
            if (!strcmp(e, "plain")) g_engine = MWBLAS_GEMM_PLAIN;
            else if (!strcmp(e, "ozaki")) g_engine = MWBLAS_GEMM_OZAKI;
            else if (!strcmp(e, "fixed")) g_engine = MWBLAS_GEMM_FIXED;
        }
    }
    return g_engine;
}

// A scope that owns staged arrays and releases them on every exit path.
struct Scope {
    const char *routine;
    std::vector<Staged *> items;
    explicit Scope(const char *r) : routine(r) { clear_error(); }
    Staged &add(Staged &s)
    {
        items.push_back(&s);
        return s;
    }
    ~Scope()
    {
        for (Staged *s : items) release(*s);
    }
};

}  // namespace

// ---- GEMM dispatch shared by mgemm_/wgemm_ and the level-3 routines ---------------

// The engine a product of this shape runs on.
int pick_engine(const GemmArgs &g, bool cplx, int force_engine)
{
    int eng = force_engine >= 0 ? force_engine : engine();
    if (eng == MWBLAS_GEMM_AUTO) {
        // The tensor-core scheme wins once the k-dimension and the output tile
        // count amortise its operand conversion; below that, real products run
        // on the integer pipes and complex ones on the FP64 pipe.
        double work = (double)g.m * (double)g.n * (double)g.k;
        eng = (work >= 64.0 * 64.0 * 64.0 * 8.0 && g.k >= 32) ? MWBLAS_GEMM_OZAKI : MWBLAS_GEMM_FIXED;
        if (eng == MWBLAS_GEMM_OZAKI && !ozaki_available()) eng = MWBLAS_GEMM_FIXED;
        if (eng == MWBLAS_GEMM_FIXED && cplx) eng = MWBLAS_GEMM_PLAIN;
    }
    return eng;
}

bool run_gemm(GemmArgs &g, bool cplx, int force_engine, const char *routine)
{
    if (!cplx && g.n == 1 && g.uplo == 0 && !g.hs && force_engine < 0 && engine() == MWBLAS_GEMM_AUTO) {
        // a real matrix-vector product (the updates and leaf solves of TRSV,
        // for instance): the fixed-point GEMV kernels, three launches
        return gemv_device(g.ta, g.ta ? g.k : g.m, g.ta ? g.m : g.k, g.alpha, g.A, g.lda, g.B, g.tb ? g.ldb : 1,
                           g.beta, g.beta_kind, g.C, 1, routine);
    }
    if (cplx && g.n == 1 && !g.tb && !g.cb && !(g.ca && !g.ta) && g.uplo == 0 && !g.herm && !g.hs &&
        force_engine < 0 && engine() == MWBLAS_GEMM_AUTO) {
        // a complex matrix-vector product: the fixed-point matrix-vector
        // kernel reading the dense operand in place (a conjugate without a
        // transpose, which the kernel cannot express, takes the general engine)
        SmvArgs v;
        v.cplx = true;
        v.fmt = 0;
        v.kind = 0;
        v.trans = g.ta ? (g.ca ? 'C' : 'T') : 'N';
        v.rows = g.m;
        v.cols = g.k;
        v.ldab = g.lda;
        v.A = g.A;
        v.x = g.B;
        v.incx = 1;
        v.y = g.C;
        v.incy = 1;
        v.calpha = g.calpha;
        v.cbeta = g.cbeta;
        v.beta_kind = g.beta_kind;
        return smv_device(v, routine);
    }
    const int eng = pick_engine(g, cplx, force_engine);
    if (g.hs && eng != MWBLAS_GEMM_OZAKI && !g.hs->wait_all(routine)) return false;
    if (eng == MWBLAS_GEMM_FIXED && !cplx) return gemm_fixed_real(g, routine);
    if (eng == MWBLAS_GEMM_OZAKI) {
        if (!ozaki_available()) {
            set_error(routine, MWBLAS_ERR_UNSUPPORTED, "tensor-core engine unavailable on this device");
            return false;
        }
        return cplx ? gemm_ozaki_cplx(g, g_ozaki_bits, routine) : gemm_ozaki_real(g, g_ozaki_bits, routine);
    }
    return cplx ? gemm_plain_cplx(g, routine) : gemm_plain_real(g, routine);
}

std::atomic<int> g_band_solve{MWBLAS_BAND_SOLVE_AUTO};

namespace {

// ---- mgemm / wgemm ------------------------------------------------------------------

template <typename INT>
void gemm_entry(const char *routine, bool cplx, int force_engine, const char *transa, const char *transb,
                const INT *m, const INT *n, const INT *k, const void *alpha, const void *a, const INT *lda,
                const void *b, const INT *ldb, const void *beta, void *c, const INT *ldc)
{
    Scope sc(routine);
    if (!transa || !transb || !m || !n || !k || !alpha || !beta || !lda || !ldb || !ldc) {
        set_error(routine, 1, "null argument pointer");
        return;
    }
    char TA = cplx ? up(transa) : trans_real(transa);
    char TB = cplx ? up(transb) : trans_real(transb);
    int64_t M = *m, N = *n, K = *k;
    if (!(TA == 'N' || TA == 'T' || TA == 'C')) { set_error(routine, 1, "invalid transa"); return; }
    if (!(TB == 'N' || TB == 'T' || TB == 'C')) { set_error(routine, 2, "invalid transb"); return; }
    // mgemm_parallel.cpp:66: m <= 0 || n <= 0 returns before touching C.
    if (M <= 0 || N <= 0) return;
    if (K < 0) K = 0;
    int64_t nrowa = (TA == 'N') ? M : K, nrowb = (TB == 'N') ? K : N;
    if (*lda < (nrowa > 1 ? nrowa : 1)) { set_error(routine, 8, "lda too small"); return; }
    if (*ldb < (nrowb > 1 ? nrowb : 1)) { set_error(routine, 10, "ldb too small"); return; }
    if (*ldc < (M > 1 ? M : 1)) { set_error(routine, 13, "ldc too small"); return; }
    if (!c) { set_error(routine, 12, "null C"); return; }

    GemmArgs g;
    g.width = true;
    g.m = M; g.n = N; g.k = K;
    g.ta = TA != 'N'; g.tb = TB != 'N';
    g.ca = TA == 'C'; g.cb = TB == 'C';
    bool alpha0;
    if (cplx) {
        g.calpha = cd((const mwblas_complex64x2 *)alpha);
        g.cbeta = cd((const mwblas_complex64x2 *)beta);
        g.beta_kind = beta_kind(g.cbeta);
        alpha0 = ceq0(g.calpha);
    } else {
        g.alpha = rd((const mwblas_real64x2 *)alpha);
        g.beta = rd((const mwblas_real64x2 *)beta);
        g.beta_kind = beta_kind(g.beta);
        alpha0 = eq0(g.alpha);
    }
    bool compute = !(alpha0 || K == 0);
    if (compute && (!a || !b)) { set_error(routine, a ? 9 : 7, "null A or B"); return; }
    if (!ensure_device(routine)) return;
    size_t es = cplx ? 32 : 16;

    Staged SA, SB, SC;
    sc.add(SA); sc.add(SB); sc.add(SC);
    // Large products on host arrays for the tensor-core engine: the three
    // uploads run on the copy stream in the order the engine needs them and
    // C comes back in chunks behind the reconstruction.
    const double host_bytes = (double)es * ((double)nrowa * (TA == 'N' ? K : M) + (double)nrowb * (TB == 'N' ? N : K) +
                                            (double)M * N);
    if (compute && K <= 65536 && M <= INT32_MAX && N <= INT32_MAX && host_bytes >= 64.0 * 1048576.0 &&
        pick_engine(g, cplx, force_engine) == MWBLAS_GEMM_OZAKI && ozaki_available() && !is_dd_device_pointer(a) &&
        !is_dd_device_pointer(b) && !is_dd_device_pointer(c)) {
        HostStage hs;
        // on every exit: stream(), which frees the buffers, waits for the copies
        struct JoinCopies {
            const char *r;
            ~JoinCopies() { join_copy_stream(r); }
        } join_guard{routine};
        // op(B) and C in about eight blocks of whole 256-column tiles; with
        // them, op(A) in about four blocks of whole 256-row tiles. Queued in
        // the order the engine uses them: A0, B0, B1, A1.., C0, C1, B2, C2, ...
        // (two column blocks are multiplied while A arrives: about the work
        // that keeps pace with the copies)
        int64_t w = ((N + 7) / 8 + 255) / 256 * 256;
        if (w < 512) w = 512;
        int64_t h = ((M + 3) / 4 + 255) / 256 * 256;
        if (h < 512) h = 512;
        const bool colblocks = w < N, rowblocks = colblocks && h < M;
        auto upload_a = [&](int64_t i0) -> bool {
            const int64_t i1 = (M - i0 < h) ? M : i0 + h;
            cudaEvent_t e = nullptr;
            const bool ok = TA == 'N' ? upload_block_async(SA, i0, i1, 0, K, e, routine)
                                      : upload_block_async(SA, 0, K, i0, i1, e, routine);
            hs.a_block.push_back(e);
            return ok;
        };
        if (rowblocks) {
            hs.a_rows = h;
            if (!stage_matrix(SA, a, nrowa, TA == 'N' ? K : M, *lda, es, false, routine)) return;
            if (!upload_a(0)) return;
        } else if (!stage_matrix_async(SA, a, nrowa, TA == 'N' ? K : M, *lda, es, true, hs.a_ready, routine)) {
            return;
        }
        if (colblocks) {
            hs.block_cols = w;
            const int64_t nblocks = (N + w - 1) / w;
            const int64_t early = rowblocks ? (nblocks < 2 ? nblocks : 2) : 0;
            hs.early_blocks = early;
            if (!stage_matrix(SB, b, nrowb, TB == 'N' ? N : K, *ldb, es, false, routine)) return;
            if (!stage_matrix(SC, c, M, N, *ldc, es, false, routine)) return;
            hs.b_block.assign((size_t)nblocks, nullptr);
            hs.c_block.assign((size_t)nblocks, nullptr);
            auto upload_b = [&](int64_t jb) -> bool {
                const int64_t j0 = jb * w, j1 = (N - j0 < w) ? N : j0 + w;
                return TB == 'N' ? upload_block_async(SB, 0, K, j0, j1, hs.b_block[jb], routine)
                                 : upload_block_async(SB, j0, j1, 0, K, hs.b_block[jb], routine);
            };
            auto upload_c = [&](int64_t jb) -> bool {
                const int64_t j0 = jb * w, j1 = (N - j0 < w) ? N : j0 + w;
                return g.beta_kind == 0 || upload_block_async(SC, 0, M, j0, j1, hs.c_block[jb], routine);
            };
            for (int64_t jb = 0; jb < early; ++jb)
                if (!upload_b(jb)) return;
            if (rowblocks)
                for (int64_t i0 = h; i0 < M; i0 += h)
                    if (!upload_a(i0)) return;
            for (int64_t jb = 0; jb < early; ++jb)
                if (!upload_c(jb)) return;
            for (int64_t jb = early; jb < nblocks; ++jb)
                if (!upload_b(jb) || !upload_c(jb)) return;
        } else {
            if (!stage_matrix_async(SB, b, nrowb, TB == 'N' ? N : K, *ldb, es, true, hs.b_ready, routine)) return;
            if (!stage_matrix_async(SC, c, M, N, *ldc, es, g.beta_kind != 0, hs.c_ready, routine)) return;
        }
        hs.c = &SC;
        g.A = SA.dev; g.lda = *lda;
        g.B = SB.dev; g.ldb = *ldb;
        g.C = SC.dev; g.ldc = *ldc;
        g.hs = &hs;
        const bool ok = run_gemm(g, cplx, force_engine, routine);
        // whatever happened, nothing may be freed before the copies are done
        // (copies back still noted after a failure are queued all the same)
        const bool flushed = flush_columns_back(SC, routine);
        const bool joined = hs.wait_all(routine) && join_copy_stream(routine) && flushed;
        if (!ok || !joined) return;
        if (!hs.c_written && !unstage_matrix(SC, routine)) return;
        finish(routine);
        return;
    }
    // C is read unless beta == 0.
    if (!stage_matrix(SC, c, M, N, *ldc, es, g.beta_kind != 0, routine)) return;
    g.C = SC.dev; g.ldc = *ldc;
    if (!compute) {
        // beta pre-pass only (mgemm_parallel.cpp:68-78)
        if (cplx) launch_scale_matrix_c(M, N, g.cbeta, g.beta_kind, g.C, g.ldc);
        else launch_scale_matrix(M, N, g.beta, g.beta_kind, g.C, g.ldc);
    } else {
        if (!stage_matrix(SA, a, nrowa, TA == 'N' ? K : M, *lda, es, true, routine)) return;
        if (!stage_matrix(SB, b, nrowb, TB == 'N' ? N : K, *ldb, es, true, routine)) return;
        g.A = SA.dev; g.lda = *lda;
        g.B = SB.dev; g.ldb = *ldb;
        if (!run_gemm(g, cplx, force_engine, routine)) return;
    }
    if (!unstage_matrix(SC, routine)) return;
    finish(routine);
}

// ---- msyrk / wherk ------------------------------------------------------------------

template <typename INT>
void syrk_entry(const char *routine, bool herm, const char *uplo, const char *trans, const INT *n, const INT *k,
                const mwblas_real64x2 *alpha, const void *a, const INT *lda, const mwblas_real64x2 *beta, void *c,
                const INT *ldc)
{
    Scope sc(routine);
    if (!uplo || !trans || !n || !k || !alpha || !beta || !lda || !ldc) {
        set_error(routine, 1, "null argument pointer");
        return;
    }
    char U = up(uplo);
    char T = up(trans);
    if (!herm && T == 'C') T = 'T';          // msyrk_parallel.cpp:53-54
    if (herm && T == 'T') T = 'C';           // wherk_serial.cpp:412-433 treats non-'N' as 'C'
    if (U != 'U' && U != 'L') { set_error(routine, 1, "invalid uplo"); return; }
    if (T != 'N' && T != (herm ? 'C' : 'T')) { set_error(routine, 2, "invalid trans"); return; }
    int64_t N = *n, K = *k;
    if (N < 0) { set_error(routine, 3, "n < 0"); return; }
    if (K < 0) { set_error(routine, 4, "k < 0"); return; }
    if (N == 0) return;
    int64_t nrowa = (T == 'N') ? N : K;
    if (*lda < (nrowa > 1 ? nrowa : 1)) { set_error(routine, 7, "lda too small"); return; }
    if (*ldc < (N > 1 ? N : 1)) { set_error(routine, 10, "ldc too small"); return; }
    if (!c) { set_error(routine, 9, "null C"); return; }
    dd_host al = rd(alpha), be = rd(beta);
    int bk = beta_kind(be);
    bool compute = !(eq0(al) || K == 0);
    // msyrk_parallel.cpp:57-65 / wherk_parallel.cpp:57-70
    if (!compute && bk == 1 && !herm) return;
    if (compute && !a) { set_error(routine, 6, "null A"); return; }
    if (!ensure_device(routine)) return;
    size_t es = herm ? 32 : 16;
    int ul = (U == 'U') ? 1 : 2;
    Staged SA, SC;
    sc.add(SA); sc.add(SC);
    if (!stage_matrix(SC, c, N, N, *ldc, es, true, routine)) return;
    if (!compute) {
        if (herm) launch_scale_matrix_c(N, N, cdd_host{be, {0.0, 0.0}}, bk, SC.dev, *ldc, ul, true);
        else launch_scale_matrix(N, N, be, bk, SC.dev, *ldc, ul);
    } else {
        if (!stage_matrix(SA, a, nrowa, T == 'N' ? K : N, *lda, es, true, routine)) return;
        GemmArgs g;
        g.width = true;
        g.alpha = al;
        g.beta = be;
        g.calpha = cdd_host{al, {0.0, 0.0}};
        g.cbeta = cdd_host{be, {0.0, 0.0}};
        g.beta_kind = bk;
        if (!syrk_device(herm, herm, ul, T != 'N', N, K, SA.dev, *lda, g, SC.dev, *ldc, routine)) return;
    }
    if (!unstage_matrix(SC, routine)) return;
    finish(routine);
}

// ---- mtrsm --------------------------------------------------------------------------------

template <typename INT>
void trsm_entry(const char *routine, const char *side, const char *uplo, const char *transa, const char *diag,
                const INT *m, const INT *n, const mwblas_real64x2 *alpha, const void *a, const INT *lda, void *b,
                const INT *ldb)
{
    Scope sc(routine);
    if (!side || !uplo || !transa || !diag || !m || !n || !alpha || !lda || !ldb) {
        set_error(routine, 1, "null argument pointer");
        return;
    }
    char S = up(side), U = up(uplo), T = trans_real(transa), D = up(diag);
    if (S != 'L' && S != 'R') { set_error(routine, 1, "invalid side"); return; }
    if (U != 'U' && U != 'L') { set_error(routine, 2, "invalid uplo"); return; }
    if (T != 'N' && T != 'T') { set_error(routine, 3, "invalid transa"); return; }
    if (D != 'U' && D != 'N') { set_error(routine, 4, "invalid diag"); return; }
    int64_t M = *m, N = *n;
    if (M < 0) { set_error(routine, 5, "m < 0"); return; }
    if (N < 0) { set_error(routine, 6, "n < 0"); return; }
    if (M == 0 || N == 0) return;   // mtrsm_parallel.cpp:57
    int64_t na = (S == 'L') ? M : N;
    if (*lda < (na > 1 ? na : 1)) { set_error(routine, 9, "lda too small"); return; }
    if (*ldb < (M > 1 ? M : 1)) { set_error(routine, 11, "ldb too small"); return; }
    if (!b) { set_error(routine, 10, "null B"); return; }
    dd_host al = rd(alpha);
    if (!eq0(al) && !a) { set_error(routine, 8, "null A"); return; }
    if (!ensure_device(routine)) return;
    Staged SA, SB;
    sc.add(SA); sc.add(SB);
    bool zero = eq0(al);   // mtrsm_parallel.cpp:59: alpha == 0 zeroes B
    if (!stage_matrix(SB, b, M, N, *ldb, 16, !zero, routine)) return;
    if (zero) {
        launch_zero_matrix(M, N, SB.dev, *ldb);
    } else {
        if (!stage_matrix(SA, a, na, na, *lda, 16, true, routine)) return;
        if (!trsm_device(S, U, T, D, M, N, al, SA.dev, *lda, SB.dev, *ldb, routine)) return;
    }
    if (!unstage_matrix(SB, routine)) return;
    finish(routine);
}

// ---- mgemv --------------------------------------------------------------------------------

template <typename INT>
void gemv_entry(const char *routine, const char *trans, const INT *m, const INT *n, const mwblas_real64x2 *alpha,
                const void *a, const INT *lda, const void *x, const INT *incx, const mwblas_real64x2 *beta, void *y,
                const INT *incy)
{
    Scope sc(routine);
    if (!trans || !m || !n || !alpha || !lda || !incx || !beta || !incy) {
        set_error(routine, 1, "null argument pointer");
        return;
    }
    char T = trans_real(trans);
    if (T != 'N' && T != 'T') { set_error(routine, 1, "invalid trans"); return; }
    int64_t M = *m, N = *n;
    if (M < 0) { set_error(routine, 2, "m < 0"); return; }
    if (N < 0) { set_error(routine, 3, "n < 0"); return; }
    if (*lda < (M > 1 ? M : 1)) { set_error(routine, 6, "lda too small"); return; }
    if (*incx == 0) { set_error(routine, 8, "incx == 0"); return; }
    if (*incy == 0) { set_error(routine, 11, "incy == 0"); return; }
    if (M == 0 || N == 0) return;   // mgemv.cpp:252
    if (!y) { set_error(routine, 10, "null y"); return; }
    dd_host al = rd(alpha), be = rd(beta);
    int bk = beta_kind(be);
    if (eq0(al) && bk == 1) return;
    if (!eq0(al) && (!a || !x)) { set_error(routine, a ? 7 : 5, "null A or x"); return; }
    if (!ensure_device(routine)) return;
    int64_t lenx = (T == 'N') ? N : M, leny = (T == 'N') ? M : N;
    Staged SA, SX, SY;
    sc.add(SA); sc.add(SX); sc.add(SY);
    int64_t dix = *incx, diy;
    if (!stage_vector(SY, y, leny, *incy, 16, bk != 0, diy, routine)) return;
    if (!eq0(al)) {
        if (!stage_matrix(SA, a, M, N, *lda, 16, true, routine)) return;
        if (!stage_vector(SX, x, lenx, *incx, 16, true, dix, routine)) return;
    }
    if (!gemv_device(T != 'N', M, N, al, SA.dev, *lda, SX.dev, dix, be, bk, SY.dev, diy, routine)) return;
    if (!unstage_vector(SY, routine)) return;
    finish(routine);
}

// ---- level 1 --------------------------------------------------------------------------

// Thresholds of the reference's threaded unit-stride paths.
constexpr int64_t kScalOmpMin = 2048;   // MSCAL_OMP_MIN, WSCAL_OMP_MIN, WMSCAL_OMP_MIN
constexpr int64_t kAxpyOmpMin = 2048;   // MAXPY_OMP_MIN

template <typename INT>
void scal_entry(const char *routine, int kind, const INT *n, const void *alpha, void *x, const INT *incx)
{
    // kind: 0 mscal (real), 1 wscal (complex alpha), 2 wmscal (real alpha, complex x)
    Scope sc(routine);
    if (!n || !alpha || !incx) { set_error(routine, 1, "null argument pointer"); return; }
    int64_t N = *n, inc = *incx;
    if (N <= 0) return;
    if (kind == 1) {
        if (ceq1(cd((const mwblas_complex64x2 *)alpha))) return;
    } else {
        if (eq1(rd((const mwblas_real64x2 *)alpha))) return;
    }
    if (!x) { set_error(routine, 3, "null x"); return; }
    if (!ensure_device(routine)) return;
    size_t es = kind == 0 ? 16 : 32;
    Staged SX;
    sc.add(SX);
    int64_t dinc;
    if (!stage_vector(SX, x, N, inc, es, true, dinc, routine)) return;
    int64_t team = (inc == 1) ? l1_team(N, kScalOmpMin) : 1;
    bool unit = (inc == 1);
    if (kind == 0) launch_mscal(N, rd((const mwblas_real64x2 *)alpha), SX.dev, dinc, unit, team);
    else if (kind == 1) launch_wscal(N, cd((const mwblas_complex64x2 *)alpha), SX.dev, dinc, unit, team);
    else launch_wmscal(N, rd((const mwblas_real64x2 *)alpha), SX.dev, dinc, unit, team);
    if (!unstage_vector(SX, routine)) return;
    finish(routine);
}

template <typename INT>
void axpy_entry(const char *routine, const INT *n, const mwblas_real64x2 *alpha, const void *x, const INT *incx,
                void *y, const INT *incy)
{
    Scope sc(routine);
    if (!n || !alpha || !incx || !incy) { set_error(routine, 1, "null argument pointer"); return; }
    int64_t N = *n;
    dd_host a = rd(alpha);
    // maxpy.cpp:99
    if (N <= 0 || eq0(a)) return;
    if (!x || !y) { set_error(routine, x ? 5 : 3, "null vector"); return; }
    if (!ensure_device(routine)) return;
    Staged SX, SY;
    sc.add(SX); sc.add(SY);
    int64_t dix, diy;
    if (!stage_vector(SX, x, N, *incx, 16, true, dix, routine)) return;
    if (!stage_vector(SY, y, N, *incy, 16, true, diy, routine)) return;
    bool unit = (*incx == 1 && *incy == 1);
    int64_t team = unit ? l1_team(N, kAxpyOmpMin) : 1;
    launch_maxpy(N, a, SX.dev, dix, SY.dev, diy, unit, team);
    if (!unstage_vector(SY, routine)) return;
    finish(routine);
}

template <typename INT>
void copy_entry(const char *routine, bool cplx, const INT *n, const void *x, const INT *incx, void *y,
                const INT *incy)
{
    Scope sc(routine);
    if (!n || !incx || !incy) { set_error(routine, 1, "null argument pointer"); return; }
    int64_t N = *n;
    if (N <= 0) return;
    if (!x || !y) { set_error(routine, x ? 4 : 2, "null vector"); return; }
    if (!ensure_device(routine)) return;
    size_t es = cplx ? 32 : 16;
    Staged SX, SY;
    sc.add(SX); sc.add(SY);
    int64_t dix, diy;
    if (!stage_vector(SX, x, N, *incx, es, true, dix, routine)) return;
    // y is write-only, except that a zero increment writes one element.
    if (!stage_vector(SY, y, N, *incy, es, false, diy, routine)) return;
    launch_copy(N, SX.dev, dix, SY.dev, diy, cplx ? 2 : 1);
    if (!unstage_vector(SY, routine)) return;
    finish(routine);
}

template <typename INT>
void swap_entry(const char *routine, bool cplx, const INT *n, void *x, const INT *incx, void *y, const INT *incy)
{
    Scope sc(routine);
    if (!n || !incx || !incy) { set_error(routine, 1, "null argument pointer"); return; }
    int64_t N = *n;
    if (N <= 0) return;
    if (!x || !y) { set_error(routine, x ? 4 : 2, "null vector"); return; }
    if (!ensure_device(routine)) return;
    size_t es = cplx ? 32 : 16;
    Staged SX, SY;
    sc.add(SX); sc.add(SY);
    int64_t dix, diy;
    if (!stage_vector(SX, x, N, *incx, es, true, dix, routine)) return;
    if (!stage_vector(SY, y, N, *incy, es, true, diy, routine)) return;
    launch_swap(N, SX.dev, dix, SY.dev, diy, cplx ? 2 : 1);
    if (!unstage_vector(SX, routine)) return;
    if (!unstage_vector(SY, routine)) return;
    finish(routine);
}

template <typename INT>
int64_t iamax_entry(const char *routine, bool cplx, const INT *n, const void *x, const INT *incx)
{
    Scope sc(routine);
    if (!n || !incx) { set_error(routine, 1, "null argument pointer"); return 0; }
    int64_t N = *n, inc = *incx;
    // imamax.cpp:180-181
    if (N < 1 || inc <= 0) return 0;
    if (N == 1) return 1;
    if (!x) { set_error(routine, 2, "null x"); return 0; }
    if (!ensure_device(routine)) return 0;
    Staged SX;
    sc.add(SX);
    int64_t dinc;
    if (!stage_vector(SX, x, N, inc, cplx ? 32 : 16, true, dinc, routine)) return 0;
    int64_t idx = -1;
    if (!launch_iamax(N, SX.dev, dinc, cplx, &idx, routine)) return 0;
    return idx + 1;
}

template <typename INT>
mwblas_real64x2 dot_entry(const char *routine, const INT *n, const void *x, const INT *incx, const void *y,
                          const INT *incy)
{
    Scope sc(routine);
    mwblas_real64x2 r{{0.0, 0.0}};
    if (!n || !incx || !incy) { set_error(routine, 1, "null argument pointer"); return r; }
    int64_t N = *n;
    if (N <= 0) return r;
    if (!x || !y) { set_error(routine, x ? 4 : 2, "null vector"); return r; }
    if (!ensure_device(routine)) return r;
    Staged SX, SY;
    sc.add(SX); sc.add(SY);
    int64_t dix, diy;
    if (!stage_vector(SX, x, N, *incx, 16, true, dix, routine)) return r;
    if (!stage_vector(SY, y, N, *incy, 16, true, diy, routine)) return r;
    dd_host out{0.0, 0.0};
    if (!launch_mdot(N, SX.dev, dix, SY.dev, diy, &out, routine)) return r;
    r.limbs[0] = out.hi;
    r.limbs[1] = out.lo;
    return r;
}

// ---- mgemmtr / wgemmtr (mgemmtr_parallel.cpp:35-80) -------------------------------------

GemmArgs scalars(bool cplx, const void *alpha, const void *beta)
{
    GemmArgs g;
    if (cplx) {
        g.calpha = cd((const mwblas_complex64x2 *)alpha);
        g.cbeta = cd((const mwblas_complex64x2 *)beta);
        g.beta_kind = beta_kind(g.cbeta);
    } else {
        g.alpha = rd((const mwblas_real64x2 *)alpha);
        g.beta = rd((const mwblas_real64x2 *)beta);
        g.beta_kind = beta_kind(g.beta);
    }
    return g;
}

bool is_zero(bool cplx, const void *v)
{
    return cplx ? ceq0(cd((const mwblas_complex64x2 *)v)) : eq0(rd((const mwblas_real64x2 *)v));
}
bool is_one(bool cplx, const void *v)
{
    return cplx ? ceq1(cd((const mwblas_complex64x2 *)v)) : eq1(rd((const mwblas_real64x2 *)v));
}

template <typename INT>
void gemmtr_entry(const char *routine, bool cplx, const char *uplo, const char *transa, const char *transb,
                  const INT *n, const INT *k, const void *alpha, const void *a, const INT *lda, const void *b,
                  const INT *ldb, const void *beta, void *c, const INT *ldc)
{
    Scope sc(routine);
    if (!uplo || !transa || !transb || !n || !k || !alpha || !beta || !lda || !ldb || !ldc) {
        set_error(routine, 1, "null argument pointer");
        return;
    }
    char U = up(uplo);
    char TA = cplx ? up(transa) : trans_real(transa);
    char TB = cplx ? up(transb) : trans_real(transb);
    if (U != 'U' && U != 'L') { set_error(routine, 1, "invalid uplo"); return; }
    if (!(TA == 'N' || TA == 'T' || TA == 'C')) { set_error(routine, 2, "invalid transa"); return; }
    if (!(TB == 'N' || TB == 'T' || TB == 'C')) { set_error(routine, 3, "invalid transb"); return; }
    int64_t N = *n, K = *k;
    if (N <= 0) return;   // mgemmtr_parallel.cpp:56
    if (K < 0) K = 0;
    int64_t nrowa = (TA == 'N') ? N : K, nrowb = (TB == 'N') ? K : N;
    if (*lda < (nrowa > 1 ? nrowa : 1)) { set_error(routine, 8, "lda too small"); return; }
    if (*ldb < (nrowb > 1 ? nrowb : 1)) { set_error(routine, 10, "ldb too small"); return; }
    if (*ldc < (N > 1 ? N : 1)) { set_error(routine, 13, "ldc too small"); return; }
    if (!c) { set_error(routine, 12, "null C"); return; }
    const bool compute = !(is_zero(cplx, alpha) || K == 0);
    if (!compute && is_one(cplx, beta)) return;   // mgemmtr_parallel.cpp:58-59
    if (compute && (!a || !b)) { set_error(routine, a ? 9 : 7, "null A or B"); return; }
    if (!ensure_device(routine)) return;
    const size_t es = cplx ? 32 : 16;
    const int ul = U == 'U' ? 1 : 2;
    Staged SA, SB, SC;
    sc.add(SA); sc.add(SB); sc.add(SC);
    if (!stage_matrix(SC, c, N, N, *ldc, es, true, routine)) return;   // the other triangle is written back as read
    GemmArgs g = scalars(cplx, alpha, beta);
    g.width = true;
    if (!compute) {
        if (cplx) launch_scale_matrix_c(N, N, g.cbeta, g.beta_kind, SC.dev, *ldc, ul);
        else launch_scale_matrix(N, N, g.beta, g.beta_kind, SC.dev, *ldc, ul);
    } else {
        if (!stage_matrix(SA, a, nrowa, TA == 'N' ? K : N, *lda, es, true, routine)) return;
        if (!stage_matrix(SB, b, nrowb, TB == 'N' ? N : K, *ldb, es, true, routine)) return;
        if (!gemmtr_device(cplx, ul, TA != 'N', TA == 'C', TB != 'N', TB == 'C', N, K, g, SA.dev, *lda, SB.dev,
                           *ldb, SC.dev, *ldc, routine))
            return;
    }
    if (!unstage_matrix(SC, routine)) return;
    finish(routine);
}

// ---- msymm / wsymm / whemm (msymm_parallel.cpp:37-102) -------------------------------------

template <typename INT>
void symm_entry(const char *routine, bool cplx, bool herm, const char *side, const char *uplo, const INT *m,
                const INT *n, const void *alpha, const void *a, const INT *lda, const void *b, const INT *ldb,
                const void *beta, void *c, const INT *ldc)
{
    Scope sc(routine);
    if (!side || !uplo || !m || !n || !alpha || !beta || !lda || !ldb || !ldc) {
        set_error(routine, 1, "null argument pointer");
        return;
    }
    char S = up(side), U = up(uplo);
    if (S != 'L' && S != 'R') { set_error(routine, 1, "invalid side"); return; }
    if (U != 'U' && U != 'L') { set_error(routine, 2, "invalid uplo"); return; }
    int64_t M = *m, N = *n;
    if (M < 0) { set_error(routine, 3, "m < 0"); return; }
    if (N < 0) { set_error(routine, 4, "n < 0"); return; }
    if (M == 0 || N == 0) return;   // msymm_parallel.cpp:58
    int64_t na = S == 'L' ? M : N;
    if (*lda < (na > 1 ? na : 1)) { set_error(routine, 7, "lda too small"); return; }
    if (*ldb < (M > 1 ? M : 1)) { set_error(routine, 9, "ldb too small"); return; }
    if (*ldc < (M > 1 ? M : 1)) { set_error(routine, 12, "ldc too small"); return; }
    if (!c) { set_error(routine, 11, "null C"); return; }
    const bool alpha0 = is_zero(cplx, alpha);
    if (alpha0 && is_one(cplx, beta)) return;   // msymm_parallel.cpp:60-61
    if (!alpha0 && (!a || !b)) { set_error(routine, a ? 8 : 6, "null A or B"); return; }
    if (!ensure_device(routine)) return;
    const size_t es = cplx ? 32 : 16;
    GemmArgs g = scalars(cplx, alpha, beta);
    g.width = true;
    Staged SA, SB, SC;
    sc.add(SA); sc.add(SB); sc.add(SC);
    if (!stage_matrix(SC, c, M, N, *ldc, es, g.beta_kind != 0, routine)) return;
    if (alpha0) {
        if (cplx) launch_scale_matrix_c(M, N, g.cbeta, g.beta_kind, SC.dev, *ldc);
        else launch_scale_matrix(M, N, g.beta, g.beta_kind, SC.dev, *ldc);
    } else {
        if (!stage_matrix(SA, a, na, na, *lda, es, true, routine)) return;
        if (!stage_matrix(SB, b, M, N, *ldb, es, true, routine)) return;
        if (!symm_device(cplx, herm, S, U, M, N, g, SA.dev, *lda, SB.dev, *ldb, SC.dev, *ldc, routine)) return;
    }
    if (!unstage_matrix(SC, routine)) return;
    finish(routine);
}

// ---- msyr2k / wsyr2k / wher2k (msyr2k_parallel.cpp:38-83, wher2k_parallel.cpp) ------------
// beta is real for HER2K (beta_cplx=false), alpha always of the matrix type.

template <typename INT>
void syr2k_entry(const char *routine, bool cplx, bool herm, const char *uplo, const char *trans, const INT *n,
                 const INT *k, const void *alpha, const void *a, const INT *lda, const void *b, const INT *ldb,
                 const void *beta, void *c, const INT *ldc)
{
    Scope sc(routine);
    if (!uplo || !trans || !n || !k || !alpha || !beta || !lda || !ldb || !ldc) {
        set_error(routine, 1, "null argument pointer");
        return;
    }
    char U = up(uplo), T = up(trans);
    if (!herm && T == 'C') T = 'T';   // msyr2k / wsyr2k_parallel.cpp:58
    if (herm && T == 'T') T = 'C';
    if (U != 'U' && U != 'L') { set_error(routine, 1, "invalid uplo"); return; }
    if (T != 'N' && T != (herm ? 'C' : 'T')) { set_error(routine, 2, "invalid trans"); return; }
    int64_t N = *n, K = *k;
    if (N < 0) { set_error(routine, 3, "n < 0"); return; }
    if (K < 0) { set_error(routine, 4, "k < 0"); return; }
    if (N == 0) return;
    int64_t nrow = (T == 'N') ? N : K;
    if (*lda < (nrow > 1 ? nrow : 1)) { set_error(routine, 7, "lda too small"); return; }
    if (*ldb < (nrow > 1 ? nrow : 1)) { set_error(routine, 9, "ldb too small"); return; }
    if (*ldc < (N > 1 ? N : 1)) { set_error(routine, 12, "ldc too small"); return; }
    if (!c) { set_error(routine, 11, "null C"); return; }
    // scalars: HER2K has a complex alpha and a real beta
    GemmArgs g;
    g.width = true;
    if (cplx) {
        g.calpha = cd((const mwblas_complex64x2 *)alpha);
        g.cbeta = herm ? cdd_host{rd((const mwblas_real64x2 *)beta), {0.0, 0.0}} : cd((const mwblas_complex64x2 *)beta);
        g.beta_kind = beta_kind(g.cbeta);
    } else {
        g.alpha = rd((const mwblas_real64x2 *)alpha);
        g.beta = rd((const mwblas_real64x2 *)beta);
        g.beta_kind = beta_kind(g.beta);
    }
    const bool compute = !(is_zero(cplx, alpha) || K == 0);
    if (!compute && g.beta_kind == 1 && !herm) return;   // msyr2k_parallel.cpp:62-63
    if (compute && (!a || !b)) { set_error(routine, a ? 8 : 6, "null A or B"); return; }
    if (!ensure_device(routine)) return;
    const size_t es = cplx ? 32 : 16;
    const int ul = U == 'U' ? 1 : 2;
    Staged SA, SB, SC;
    sc.add(SA); sc.add(SB); sc.add(SC);
    if (!stage_matrix(SC, c, N, N, *ldc, es, true, routine)) return;
    if (!compute) {
        // wher2k_parallel.cpp:65-75: beta == 1 still zeroes Im(diag)
        if (cplx) launch_scale_matrix_c(N, N, g.cbeta, g.beta_kind, SC.dev, *ldc, ul, herm);
        else launch_scale_matrix(N, N, g.beta, g.beta_kind, SC.dev, *ldc, ul);
    } else {
        if (!stage_matrix(SA, a, nrow, T == 'N' ? K : N, *lda, es, true, routine)) return;
        if (!stage_matrix(SB, b, nrow, T == 'N' ? K : N, *ldb, es, true, routine)) return;
        if (!syr2k_device(cplx, herm, ul, T != 'N', N, K, g, SA.dev, *lda, SB.dev, *ldb, SC.dev, *ldc, routine))
            return;
    }
    if (!unstage_matrix(SC, routine)) return;
    finish(routine);
}

// ---- wsyrk (wsyrk_parallel.cpp): complex symmetric rank-k, complex alpha/beta -----------

template <typename INT>
void csyrk_entry(const char *routine, const char *uplo, const char *trans, const INT *n, const INT *k,
                 const mwblas_complex64x2 *alpha, const void *a, const INT *lda, const mwblas_complex64x2 *beta,
                 void *c, const INT *ldc)
{
    Scope sc(routine);
    if (!uplo || !trans || !n || !k || !alpha || !beta || !lda || !ldc) {
        set_error(routine, 1, "null argument pointer");
        return;
    }
    char U = up(uplo), T = up(trans);
    if (T == 'C') T = 'T';
    if (U != 'U' && U != 'L') { set_error(routine, 1, "invalid uplo"); return; }
    if (T != 'N' && T != 'T') { set_error(routine, 2, "invalid trans"); return; }
    int64_t N = *n, K = *k;
    if (N < 0) { set_error(routine, 3, "n < 0"); return; }
    if (K < 0) { set_error(routine, 4, "k < 0"); return; }
    if (N == 0) return;   // wsyrk_parallel.cpp:55
    int64_t nrowa = (T == 'N') ? N : K;
    if (*lda < (nrowa > 1 ? nrowa : 1)) { set_error(routine, 7, "lda too small"); return; }
    if (*ldc < (N > 1 ? N : 1)) { set_error(routine, 10, "ldc too small"); return; }
    if (!c) { set_error(routine, 9, "null C"); return; }
    GemmArgs g = scalars(true, alpha, beta);
    g.width = true;
    const bool compute = !(ceq0(g.calpha) || K == 0);
    if (!compute && g.beta_kind == 1) return;   // wsyrk_parallel.cpp:57-58
    if (compute && !a) { set_error(routine, 6, "null A"); return; }
    if (!ensure_device(routine)) return;
    const int ul = U == 'U' ? 1 : 2;
    Staged SA, SC;
    sc.add(SA); sc.add(SC);
    if (!stage_matrix(SC, c, N, N, *ldc, 32, true, routine)) return;
    if (!compute) {
        launch_scale_matrix_c(N, N, g.cbeta, g.beta_kind, SC.dev, *ldc, ul);
    } else {
        if (!stage_matrix(SA, a, nrowa, T == 'N' ? K : N, *lda, 32, true, routine)) return;
        if (!syrk_device(true, false, ul, T != 'N', N, K, SA.dev, *lda, g, SC.dev, *ldc, routine)) return;
    }
    if (!unstage_matrix(SC, routine)) return;
    finish(routine);
}

// ---- mtrmm / wtrmm (mtrmm_parallel.cpp:37-106) and wtrsm (wtrsm_parallel.cpp) ------------

template <typename INT>
void trxm_entry(const char *routine, bool cplx, bool solve, const char *side, const char *uplo, const char *transa,
                const char *diag, const INT *m, const INT *n, const void *alpha, const void *a, const INT *lda,
                void *b, const INT *ldb)
{
    Scope sc(routine);
    if (!side || !uplo || !transa || !diag || !m || !n || !alpha || !lda || !ldb) {
        set_error(routine, 1, "null argument pointer");
        return;
    }
    char S = up(side), U = up(uplo), T = cplx ? up(transa) : trans_real(transa), D = up(diag);
    if (S != 'L' && S != 'R') { set_error(routine, 1, "invalid side"); return; }
    if (U != 'U' && U != 'L') { set_error(routine, 2, "invalid uplo"); return; }
    if (T != 'N' && T != 'T' && T != 'C') { set_error(routine, 3, "invalid transa"); return; }
    if (D != 'U' && D != 'N') { set_error(routine, 4, "invalid diag"); return; }
    int64_t M = *m, N = *n;
    if (M < 0) { set_error(routine, 5, "m < 0"); return; }
    if (N < 0) { set_error(routine, 6, "n < 0"); return; }
    if (M == 0 || N == 0) return;   // mtrmm_parallel.cpp:58, wtrsm_parallel.cpp:58
    int64_t na = (S == 'L') ? M : N;
    if (*lda < (na > 1 ? na : 1)) { set_error(routine, 9, "lda too small"); return; }
    if (*ldb < (M > 1 ? M : 1)) { set_error(routine, 11, "ldb too small"); return; }
    if (!b) { set_error(routine, 10, "null B"); return; }
    const bool zero = is_zero(cplx, alpha);   // mtrmm_parallel.cpp:60: alpha == 0 zeroes B
    if (!zero && !a) { set_error(routine, 8, "null A"); return; }
    if (!ensure_device(routine)) return;
    const size_t es = cplx ? 32 : 16;
    Staged SA, SB;
    sc.add(SA); sc.add(SB);
    if (!stage_matrix(SB, b, M, N, *ldb, es, !zero, routine)) return;
    if (zero) {
        if (cplx) launch_scale_matrix_c(M, N, cdd_host{{0.0, 0.0}, {0.0, 0.0}}, 0, SB.dev, *ldb);
        else launch_zero_matrix(M, N, SB.dev, *ldb);
    } else {
        if (!stage_matrix(SA, a, na, na, *lda, es, true, routine)) return;
        GemmArgs g = scalars(cplx, alpha, alpha);
        bool ok = solve ? ctrsm_device(S, U, T, D, M, N, g.calpha, SA.dev, *lda, SB.dev, *ldb, routine)
                        : trmm_device(cplx, S, U, T, D, M, N, g, SA.dev, *lda, SB.dev, *ldb, routine);
        if (!ok) return;
    }
    if (!unstage_matrix(SB, routine)) return;
    finish(routine);
}

// ---- wdotu / wdotc / masum / mwasum / mnrm2 / mwnrm2 -------------------------------------

// mode as launch_reduce; returns (re, im) (im zero for the real results).
template <typename INT>
void reduce_entry(const char *routine, int mode, const INT *n, const void *x, const INT *incx, const void *y,
                  const INT *incy, double2 out[2])
{
    Scope sc(routine);
    out[0] = make_double2(0.0, 0.0);
    out[1] = make_double2(0.0, 0.0);
    const bool dot = mode <= 1;
    if (!n || !incx || (dot && !incy)) { set_error(routine, 1, "null argument pointer"); return; }
    int64_t N = *n, ix = *incx, iy = dot ? *incy : 0;
    if (N <= 0) return;                 // wdotc.cpp:127, masum.cpp:119
    if (!dot && ix < 1) return;         // masum.cpp:119, mnrm2.cpp:182
    if (!x || (dot && !y)) { set_error(routine, 2, "null vector"); return; }
    const size_t es = (mode == 2 || mode == 4) ? 16 : 32;
    if (mode == 4 && N == 1) {
        // mnrm2.cpp:183: |x(1)| exactly
        const mwblas_real64x2 *p = (const mwblas_real64x2 *)x;
        mwblas_real64x2 v;
        if (!ensure_device(routine)) return;
        if (is_device_pointer(x)) {
            if (!cuda_ok(cudaMemcpy(&v, p, 16, cudaMemcpyDefault), routine, "read x(1)")) return;
        } else {
            v = *p;
        }
        const bool neg = v.limbs[0] < 0.0 || (v.limbs[0] == 0.0 && v.limbs[1] < 0.0);
        out[0] = neg ? make_double2(-v.limbs[0], -v.limbs[1]) : make_double2(v.limbs[0], v.limbs[1]);
        return;
    }
    if (!ensure_device(routine)) return;
    Staged SX, SY;
    sc.add(SX); sc.add(SY);
    int64_t dix, diy = 0;
    if (!stage_vector(SX, x, N, ix, es, true, dix, routine)) return;
    if (dot && !stage_vector(SY, y, N, iy, es, true, diy, routine)) return;
    if (!launch_reduce(mode, N, SX.dev, dix, dot ? SY.dev : nullptr, diy, out, routine)) return;
}

// ---- waxpy (waxpy.cpp:101) --------------------------------------------------------------

template <typename INT>
void waxpy_entry(const INT *n, const mwblas_complex64x2 *alpha, const void *x, const INT *incx, void *y,
                 const INT *incy)
{
    const char *routine = "waxpy";
    Scope sc(routine);
    if (!n || !alpha || !incx || !incy) { set_error(routine, 1, "null argument pointer"); return; }
    int64_t N = *n;
    const cdd_host a = cd(alpha);
    if (N <= 0 || ceq0(a)) return;
    if (!x || !y) { set_error(routine, 3, "null vector"); return; }
    if (!ensure_device(routine)) return;
    Staged SX, SY;
    sc.add(SX); sc.add(SY);
    int64_t dix, diy;
    if (!stage_vector(SX, x, N, *incx, 32, true, dix, routine)) return;
    if (!stage_vector(SY, y, N, *incy, 32, true, diy, routine)) return;
    launch_waxpy(N, a, SX.dev, dix, SY.dev, diy);
    if (!unstage_vector(SY, routine)) return;
    finish(routine);
}

// ---- mrot / wmrot / mrotm (mrot.cpp:106, mrotm.cpp:200) ---------------------------------

template <typename INT>
void rot_entry(const char *routine, int e2, const INT *n, void *x, const INT *incx, void *y, const INT *incy,
               const dd_host h[4])
{
    Scope sc(routine);
    int64_t N = *n;
    if (N <= 0) return;
    if (!x || !y) { set_error(routine, 2, "null vector"); return; }
    if (!ensure_device(routine)) return;
    Staged SX, SY;
    sc.add(SX); sc.add(SY);
    int64_t dix, diy;
    if (!stage_vector(SX, x, N, *incx, 16 * e2, true, dix, routine)) return;
    if (!stage_vector(SY, y, N, *incy, 16 * e2, true, diy, routine)) return;
    launch_rot(N, SX.dev, dix, SY.dev, diy, e2, h);
    if (!unstage_vector(SX, routine)) return;
    if (!unstage_vector(SY, routine)) return;
    finish(routine);
}

template <typename INT>
void rotcs_entry(const char *routine, int e2, const INT *n, void *x, const INT *incx, void *y, const INT *incy,
                 const mwblas_real64x2 *c, const mwblas_real64x2 *s)
{
    if (!n || !incx || !incy || !c || !s) { set_error(routine, 1, "null argument pointer"); return; }
    const dd_host cc = rd(c), ss = rd(s);
    const dd_host h[4] = {cc, ss, {-ss.hi, -ss.lo}, cc};
    rot_entry(routine, e2, n, x, incx, y, incy, h);
}

template <typename INT>
void rotm_entry(const INT *n, void *x, const INT *incx, void *y, const INT *incy, const mwblas_real64x2 *param)
{
    const char *routine = "mrotm";
    if (!n || !incx || !incy || !param) { set_error(routine, 1, "null argument pointer"); return; }
    const dd_host flag = rd(param);
    // mrotm.cpp:200: flag == -2 is the identity; otherwise H from dparam(2:5)
    // = (h11, h21, h12, h22) with the implied entries of flags 0 and 1
    if (flag.hi == -2.0 && flag.lo == 0.0) return;
    const dd_host one{1.0, 0.0}, mone{-1.0, 0.0};
    dd_host h11 = rd(param + 1), h21 = rd(param + 2), h12 = rd(param + 3), h22 = rd(param + 4);
    if (flag.hi == 0.0 && flag.lo == 0.0) {
        h11 = one;
        h22 = one;
    } else if (flag.hi == 1.0 && flag.lo == 0.0) {
        h12 = one;
        h21 = mone;
    }
    const dd_host h[4] = {h11, h12, h21, h22};
    rot_entry(routine, 1, n, x, incx, y, incy, h);
}

// ---- mcabs1 / mrotg / mrotmg / wrotg (mcabs1.cpp:20, mrotg.cpp:21, mrotmg.cpp:25, wrotg.cpp:27) ----
// Scalar arguments are host variables, as in the reference's signatures.

bool gen_run(const char *routine, int op, const double2 *in, int nin, GenResult &r)
{
    Scope sc(routine);
    if (!ensure_device(routine)) return false;
    GenInput gi;
    for (int i = 0; i < 4; ++i) gi.v[i] = i < nin ? in[i] : make_double2(0.0, 0.0);
    if (!launch_generator(op, gi, &r, routine)) return false;
    return true;
}

inline double2 d2(const mwblas_real64x2 *p) { return make_double2(p->limbs[0], p->limbs[1]); }
inline void put(mwblas_real64x2 *p, const GenResult &r, int i)
{
    if (r.mask & (1u << i)) {
        p->limbs[0] = r.v[i].x;
        p->limbs[1] = r.v[i].y;
    }
}

mwblas_real64x2 cabs1_entry(const mwblas_complex64x2 *z)
{
    mwblas_real64x2 out{{0.0, 0.0}};
    if (!z) { set_error("mcabs1", 1, "null argument pointer"); return out; }
    const double2 in[2] = {d2(&z->re), d2(&z->im)};
    GenResult r;
    if (gen_run("mcabs1", GEN_CABS1, in, 2, r)) put(&out, r, 0);
    return out;
}

void rotg_entry(mwblas_real64x2 *a, mwblas_real64x2 *b, mwblas_real64x2 *c, mwblas_real64x2 *s)
{
    if (!a || !b || !c || !s) { set_error("mrotg", 1, "null argument pointer"); return; }
    const double2 in[2] = {d2(a), d2(b)};
    GenResult r;
    if (!gen_run("mrotg", GEN_ROTG, in, 2, r)) return;
    put(a, r, 0);
    put(b, r, 1);
    put(c, r, 2);
    put(s, r, 3);
}

void rotmg_entry(mwblas_real64x2 *d1, mwblas_real64x2 *d2_, mwblas_real64x2 *x1, const mwblas_real64x2 *y1,
                 mwblas_real64x2 *param)
{
    if (!d1 || !d2_ || !x1 || !y1 || !param) { set_error("mrotmg", 1, "null argument pointer"); return; }
    const double2 in[4] = {d2(d1), d2(d2_), d2(x1), d2(y1)};
    GenResult r;
    if (!gen_run("mrotmg", GEN_ROTMG, in, 4, r)) return;
    put(d1, r, 0);
    put(d2_, r, 1);
    put(x1, r, 2);
    for (int i = 0; i < 5; ++i) put(param + i, r, 3 + i);
}

void wrotg_entry(mwblas_complex64x2 *a, const mwblas_complex64x2 *b, mwblas_real64x2 *c, mwblas_complex64x2 *s)
{
    if (!a || !b || !c || !s) { set_error("wrotg", 1, "null argument pointer"); return; }
    const double2 in[4] = {d2(&a->re), d2(&a->im), d2(&b->re), d2(&b->im)};
    GenResult r;
    if (!gen_run("wrotg", GEN_WROTG, in, 4, r)) return;
    put(&a->re, r, 0);
    put(&a->im, r, 1);
    put(c, r, 2);
    put(&s->re, r, 3);
    put(&s->im, r, 4);
}

// ---- level 2 beyond real GEMV (gbmv, symv/hemv/sbmv/hbmv/spmv/hpmv, trmv/tbmv/tpmv,
//      trsv/tbsv/tpsv, ger/geru/gerc, syr/her/spr/hpr, syr2/her2/spr2/hpr2) ------------
// Matrix formats: 0 dense (lda), 1 band (ldab, k or kl/ku), 2 packed (n(n+1)/2).

void set_scalars(bool cplx, const void *alpha, const void *beta, dd_host &a, dd_host &b, cdd_host &ca, cdd_host &cb,
                 int &bk)
{
    if (cplx) {
        ca = cd((const mwblas_complex64x2 *)alpha);
        cb = beta ? cd((const mwblas_complex64x2 *)beta) : cdd_host{{0.0, 0.0}, {0.0, 0.0}};
        bk = beta_kind(cb);
    } else {
        a = rd((const mwblas_real64x2 *)alpha);
        b = beta ? rd((const mwblas_real64x2 *)beta) : dd_host{0.0, 0.0};
        bk = beta_kind(b);
    }
}

// GEMV (complex) and GBMV: y := alpha*op(A)*x + beta*y (mgbmv.cpp, wgemv.cpp)
template <typename INT>
void gemv2_entry(const char *routine, bool cplx, bool band, const char *trans, const INT *m, const INT *n,
                 const INT *kl, const INT *ku, const void *alpha, const void *a, const INT *lda, const void *x,
                 const INT *incx, const void *beta, void *y, const INT *incy)
{
    Scope sc(routine);
    if (!trans || !m || !n || !alpha || !lda || !incx || !beta || !incy || (band && (!kl || !ku))) {
        set_error(routine, 1, "null argument pointer");
        return;
    }
    char T = cplx ? up(trans) : trans_real(trans);
    if (T != 'N' && T != 'T' && T != 'C') { set_error(routine, 1, "invalid trans"); return; }
    int64_t M = *m, N = *n, KL = band ? *kl : 0, KU = band ? *ku : 0;
    if (M < 0 || N < 0 || KL < 0 || KU < 0) { set_error(routine, 2, "negative size"); return; }
    const int64_t ldmin = band ? KL + KU + 1 : (M > 1 ? M : 1);
    if (*lda < ldmin) { set_error(routine, band ? 8 : 6, "lda too small"); return; }
    if (*incx == 0 || *incy == 0) { set_error(routine, *incx == 0 ? 10 : 13, "zero increment"); return; }
    if (M == 0 || N == 0) return;
    MvArgs v;
    v.cplx = cplx;
    v.trans = T;
    set_scalars(cplx, alpha, beta, v.alpha, v.beta, v.calpha, v.cbeta, v.beta_kind);
    const bool alpha0 = is_zero(cplx, alpha);
    if (alpha0 && v.beta_kind == 1) return;
    if (!y || (!alpha0 && (!a || !x))) { set_error(routine, 3, "null array"); return; }
    if (!ensure_device(routine)) return;
    const int e2 = cplx ? 2 : 1;
    const size_t es = 16 * (size_t)e2;
    v.lenx = (T == 'N') ? N : M;
    v.leny = (T == 'N') ? M : N;
    Staged SA, SX, SY;
    sc.add(SA); sc.add(SX); sc.add(SY);
    int64_t dix = 1, diy;
    if (!stage_vector(SY, y, v.leny, *incy, es, v.beta_kind != 0, diy, routine)) return;
    v.alpha_zero = alpha0;
    if (!alpha0) {
        if (!stage_vector(SX, x, v.lenx, *incx, es, true, dix, routine)) return;
        if (!stage_matrix(SA, a, band ? (KL + KU + 1) : M, N, *lda, es, true, routine)) return;
    }
    bool ok;
    if (band && !alpha0) {
        SmvArgs b;
        b.cplx = cplx;
        b.fmt = 1;
        b.kind = 0;
        b.trans = T;
        b.rows = v.leny;
        b.cols = v.lenx;
        b.kl = KL;
        b.ku = KU;
        b.ldab = *lda;
        b.A = SA.dev;
        b.x = SX.dev;
        b.incx = dix;
        b.y = SY.dev;
        b.incy = diy;
        b.alpha = v.alpha;
        b.beta = v.beta;
        b.calpha = v.calpha;
        b.cbeta = v.cbeta;
        b.beta_kind = v.beta_kind;
        ok = smv_device(b, routine);
    } else {
        v.A = SA.dev;
        v.lda = *lda;
        v.x = SX.dev;
        v.incx = dix;
        v.y = SY.dev;
        v.incy = diy;
        ok = mv_device(v, routine);
    }
    if (!ok) return;
    if (!unstage_vector(SY, routine)) return;
    finish(routine);
}

// SYMV/HEMV (dense), SBMV/HBMV (band, k), SPMV/HPMV (packed)
template <typename INT>
void symv_entry(const char *routine, bool cplx, bool herm, int fmt, const char *uplo, const INT *n, const INT *k,
                const void *alpha, const void *a, const INT *lda, const void *x, const INT *incx, const void *beta,
                void *y, const INT *incy)
{
    Scope sc(routine);
    if (!uplo || !n || !alpha || !incx || !beta || !incy || (fmt != 2 && !lda) || (fmt == 1 && !k)) {
        set_error(routine, 1, "null argument pointer");
        return;
    }
    char U = up(uplo);
    if (U != 'U' && U != 'L') { set_error(routine, 1, "invalid uplo"); return; }
    int64_t N = *n, K = fmt == 1 ? *k : 0;
    if (N < 0 || K < 0) { set_error(routine, 2, "negative size"); return; }
    if (fmt == 0 && *lda < (N > 1 ? N : 1)) { set_error(routine, 5, "lda too small"); return; }
    if (fmt == 1 && *lda < K + 1) { set_error(routine, 6, "lda too small"); return; }
    if (*incx == 0 || *incy == 0) { set_error(routine, 7, "zero increment"); return; }
    if (N == 0) return;
    MvArgs v;
    v.cplx = cplx;
    set_scalars(cplx, alpha, beta, v.alpha, v.beta, v.calpha, v.cbeta, v.beta_kind);
    const bool alpha0 = is_zero(cplx, alpha);
    if (alpha0 && v.beta_kind == 1) return;
    if (!y || (!alpha0 && (!a || !x))) { set_error(routine, 3, "null array"); return; }
    if (!ensure_device(routine)) return;
    const int e2 = cplx ? 2 : 1;
    const size_t es = 16 * (size_t)e2;
    Staged SA, SX, SY;
    sc.add(SA); sc.add(SX); sc.add(SY);
    int64_t dix = 1, diy;
    if (!stage_vector(SY, y, N, *incy, es, v.beta_kind != 0, diy, routine)) return;
    if (alpha0) {
        v.alpha_zero = true;
        v.lenx = N;
        v.leny = N;
        v.y = SY.dev;
        v.incy = diy;
        if (!mv_device(v, routine)) return;
    } else {
        if (!stage_vector(SX, x, N, *incx, es, true, dix, routine)) return;
        bool ok;
        if (fmt == 0) {
            if (!stage_matrix(SA, a, N, N, *lda, es, true, routine)) return;
            v.shape = herm ? MV_HERMITIAN : MV_SYMMETRIC;
            v.trans = 'N';
            v.uplo = U;
            v.lenx = N;
            v.leny = N;
            v.A = SA.dev;
            v.lda = *lda;
            v.x = SX.dev;
            v.incx = dix;
            v.y = SY.dev;
            v.incy = diy;
            ok = mv_device(v, routine);
        } else {
            const int64_t len = N * (N + 1) / 2;
            if (fmt == 1) {
                if (!stage_matrix(SA, a, K + 1, N, *lda, es, true, routine)) return;
            } else {
                if (!stage_matrix(SA, a, len, 1, len, es, true, routine)) return;
            }
            SmvArgs b;
            b.cplx = cplx;
            b.fmt = fmt;
            b.kind = herm ? 2 : 1;
            b.upper = U == 'U';
            b.rows = b.cols = b.n = N;
            b.kl = U == 'L' ? K : 0;
            b.ku = U == 'U' ? K : 0;
            b.ldab = fmt == 1 ? *lda : 1;
            b.A = SA.dev;
            b.x = SX.dev;
            b.incx = dix;
            b.y = SY.dev;
            b.incy = diy;
            b.alpha = v.alpha;
            b.beta = v.beta;
            b.calpha = v.calpha;
            b.cbeta = v.cbeta;
            b.beta_kind = v.beta_kind;
            ok = smv_device(b, routine);
        }
        if (!ok) return;
    }
    if (!unstage_vector(SY, routine)) return;
    finish(routine);
}

// TRMV/TBMV/TPMV (solve=false), TRSV/TBSV/TPSV (solve=true)
template <typename INT>
void trv_entry(const char *routine, bool cplx, bool solve, int fmt, const char *uplo, const char *trans,
               const char *diag, const INT *n, const INT *k, const void *a, const INT *lda, void *x, const INT *incx)
{
    Scope sc(routine);
    if (!uplo || !trans || !diag || !n || !incx || (fmt != 2 && !lda) || (fmt == 1 && !k)) {
        set_error(routine, 1, "null argument pointer");
        return;
    }
    char U = up(uplo), T = cplx ? up(trans) : trans_real(trans), D = up(diag);
    if (U != 'U' && U != 'L') { set_error(routine, 1, "invalid uplo"); return; }
    if (T != 'N' && T != 'T' && T != 'C') { set_error(routine, 2, "invalid trans"); return; }
    if (D != 'U' && D != 'N') { set_error(routine, 3, "invalid diag"); return; }
    int64_t N = *n, K = fmt == 1 ? *k : 0;
    if (N < 0 || K < 0) { set_error(routine, 4, "negative size"); return; }
    if (fmt == 0 && *lda < (N > 1 ? N : 1)) { set_error(routine, 6, "lda too small"); return; }
    if (fmt == 1 && *lda < K + 1) { set_error(routine, 7, "lda too small"); return; }
    if (*incx == 0) { set_error(routine, 8, "zero increment"); return; }
    if (N == 0) return;
    if (!a || !x) { set_error(routine, 5, "null array"); return; }
    if (!ensure_device(routine)) return;
    const int e2 = cplx ? 2 : 1;
    const size_t es = 16 * (size_t)e2;
    Staged SA, SX;
    sc.add(SA); sc.add(SX);
    int64_t dix;
    if (!stage_vector(SX, x, N, *incx, es, true, dix, routine)) return;
    void *dense = nullptr;
    char Dd = D;
    const int band_mode = g_band_solve.load();
    if (fmt == 1 && solve &&
        (band_mode == MWBLAS_BAND_SOLVE_IN_PLACE ||
         (band_mode == MWBLAS_BAND_SOLVE_AUTO && (K <= 31 || (double)N * (double)N * (double)es > 268435456.0)))) {
        // solved in place from the band: a narrow band (partitioned solve), a
        // dense copy too large, or asked for
        if (!stage_matrix(SA, a, K + 1, N, *lda, es, true, routine)) return;
        if (!tbsv_device(cplx, U, T, D, N, K, SA.dev, *lda, SX.dev, dix, routine)) return;
        if (!unstage_vector(SX, routine)) return;
        finish(routine);
        return;
    }
    if (fmt != 0 && !solve) {
        // x := op(A) x with A read in place from its band or packed storage
        const int64_t len = N * (N + 1) / 2;
        if (fmt == 1) {
            if (!stage_matrix(SA, a, K + 1, N, *lda, es, true, routine)) return;
        } else {
            if (!stage_matrix(SA, a, len, 1, len, es, true, routine)) return;
        }
        SmvArgs b;
        b.cplx = cplx;
        b.fmt = fmt;
        b.kind = 3;
        b.trans = T;
        b.upper = U == 'U';
        b.unit = D == 'U';
        b.rows = b.cols = b.n = N;
        b.kl = U == 'L' ? K : 0;
        b.ku = U == 'U' ? K : 0;
        b.ldab = fmt == 1 ? *lda : 1;
        b.A = SA.dev;
        b.x = SX.dev;
        b.incx = dix;
        b.y = SX.dev;   // x is gathered before y is written
        b.incy = dix;
        if (!smv_device(b, routine)) return;
        if (!unstage_vector(SX, routine)) return;
        finish(routine);
        return;
    }
    if (fmt == 0) {
        if (!stage_matrix(SA, a, N, N, *lda, es, true, routine)) return;
    } else {
        const int64_t len = N * (N + 1) / 2;
        if (fmt == 1) {
            if (!stage_matrix(SA, a, K + 1, N, *lda, es, true, routine)) return;
        } else {
            if (!stage_matrix(SA, a, len, 1, len, es, true, routine)) return;
        }
        dense = dev_alloc((size_t)N * N * es, routine);
        if (!dense) return;
        if (fmt == 1) {
            band_expand(N, N, U == 'L' ? K : 0, U == 'U' ? K : 0, SA.dev, *lda, e2, 3, U == 'U', D == 'U', dense);
            Dd = 'N';   // the unit diagonal is in the dense copy
        } else {
            pack_move(N, SA.dev, e2, U == 'U', dense, true);
        }
    }
    const bool ok = trv_device(cplx, solve, U, T, Dd, N, fmt == 0 ? SA.dev : dense, fmt == 0 ? *lda : N, SX.dev, dix,
                               routine);
    if (dense) dev_free(dense);
    if (!ok) return;
    if (!unstage_vector(SX, routine)) return;
    finish(routine);
}

// GER / GERU / GERC: A := alpha*x*y^T (y^H for GERC) + A
template <typename INT>
void ger_entry(const char *routine, bool cplx, bool conj, const INT *m, const INT *n, const void *alpha, const void *x,
               const INT *incx, const void *y, const INT *incy, void *a, const INT *lda)
{
    Scope sc(routine);
    if (!m || !n || !alpha || !incx || !incy || !lda) { set_error(routine, 1, "null argument pointer"); return; }
    int64_t M = *m, N = *n;
    if (M < 0 || N < 0) { set_error(routine, 1, "negative size"); return; }
    if (*incx == 0 || *incy == 0) { set_error(routine, 5, "zero increment"); return; }
    if (*lda < (M > 1 ? M : 1)) { set_error(routine, 9, "lda too small"); return; }
    if (M == 0 || N == 0 || is_zero(cplx, alpha)) return;
    if (!a || !x || !y) { set_error(routine, 4, "null array"); return; }
    if (!ensure_device(routine)) return;
    const size_t es = cplx ? 32 : 16;
    Staged SA, SX, SY;
    sc.add(SA); sc.add(SX); sc.add(SY);
    int64_t dix, diy;
    if (!stage_vector(SX, x, M, *incx, es, true, dix, routine)) return;
    if (!stage_vector(SY, y, N, *incy, es, true, diy, routine)) return;
    if (!stage_matrix(SA, a, M, N, *lda, es, true, routine)) return;
    RankArgs r;
    r.cplx = cplx;
    r.conj = conj;
    r.uplo = 0;
    r.m = M;
    r.n = N;
    r.x = SX.dev;
    r.incx = dix;
    r.y = SY.dev;
    r.incy = diy;
    r.A = SA.dev;
    r.lda = *lda;
    dd_host b;
    cdd_host cb;
    int bk;
    set_scalars(cplx, alpha, nullptr, r.alpha, b, r.calpha, cb, bk);
    if (!rank_update_device(r, routine)) return;
    if (!unstage_matrix(SA, routine)) return;
    finish(routine);
}

// SYR/HER (two=false) and SYR2/HER2 (two=true), dense or packed; HER/HPR take
// a real alpha (the Hermitian forms keep the diagonal real).
template <typename INT>
void syr_entry(const char *routine, bool cplx, bool herm, bool packed, bool two, const char *uplo, const INT *n,
               const void *alpha, const void *x, const INT *incx, const void *y, const INT *incy, void *a,
               const INT *lda)
{
    Scope sc(routine);
    if (!uplo || !n || !alpha || !incx || (two && !incy) || (!packed && !lda)) {
        set_error(routine, 1, "null argument pointer");
        return;
    }
    char U = up(uplo);
    if (U != 'U' && U != 'L') { set_error(routine, 1, "invalid uplo"); return; }
    int64_t N = *n;
    if (N < 0) { set_error(routine, 2, "n < 0"); return; }
    if (*incx == 0 || (two && *incy == 0)) { set_error(routine, 5, "zero increment"); return; }
    if (!packed && *lda < (N > 1 ? N : 1)) { set_error(routine, two ? 9 : 7, "lda too small"); return; }
    // real alpha for HER / HPR; complex for HER2 / HPR2
    const bool alpha_real = !cplx || (herm && !two);
    if (N == 0 || is_zero(!alpha_real, alpha)) return;
    if (!a || !x || (two && !y)) { set_error(routine, 4, "null array"); return; }
    if (!ensure_device(routine)) return;
    const int e2 = cplx ? 2 : 1;
    const size_t es = 16 * (size_t)e2;
    Staged SA, SX, SY;
    sc.add(SA); sc.add(SX); sc.add(SY);
    int64_t dix, diy = 1;
    if (!stage_vector(SX, x, N, *incx, es, true, dix, routine)) return;
    if (two && !stage_vector(SY, y, N, *incy, es, true, diy, routine)) return;
    const int64_t len = N * (N + 1) / 2;
    if (packed) {
        // updated in place in the packed triangle
        if (!stage_matrix(SA, a, len, 1, len, es, true, routine)) return;
    } else {
        if (!stage_matrix(SA, a, N, N, *lda, es, true, routine)) return;
    }
    RankArgs r;
    r.cplx = cplx;
    r.conj = herm;
    r.uplo = U == 'U' ? 1 : 2;
    r.m = N;
    r.n = N;
    r.x = SX.dev;
    r.incx = dix;
    r.y = two ? SY.dev : nullptr;
    r.incy = diy;
    r.A = SA.dev;
    r.lda = packed ? -1 : *lda;
    if (alpha_real) {
        r.alpha = rd((const mwblas_real64x2 *)alpha);
        r.calpha = cdd_host{r.alpha, {0.0, 0.0}};
    } else {
        r.calpha = cd((const mwblas_complex64x2 *)alpha);
    }
    if (!rank_update_device(r, routine)) return;
    if (!unstage_matrix(SA, routine)) return;
    finish(routine);
}

}  // namespace
}  // namespace mw

using mw::dd_host;
typedef mwblas_real64x2 TR;
typedef mwblas_complex64x2 TC;

extern "C" {

// ---- level 3 -----------------------------------------------------------------------------

#define MW_GEMM_PAIR(NAME, T, CPLX, ENG)                                                                          \
    void NAME##_(const char *ta, const char *tb, const int *m, const int *n, const int *k, const T *alpha,      \
                 const T *a, const int *lda, const T *b, const int *ldb, const T *beta, T *c, const int *ldc)   \
    {                                                                                                           \
        mw::gemm_entry<int>(#NAME, CPLX, ENG, ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc);            \
    }                                                                                                           \
    void NAME##_64_(const char *ta, const char *tb, const int64_t *m, const int64_t *n, const int64_t *k,      \
                    const T *alpha, const T *a, const int64_t *lda, const T *b, const int64_t *ldb,             \
                    const T *beta, T *c, const int64_t *ldc)                                                    \
    {                                                                                                           \
        mw::gemm_entry<int64_t>(#NAME, CPLX, ENG, ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc);        \
    }

MW_GEMM_PAIR(mgemm, TR, false, -1)
MW_GEMM_PAIR(wgemm, TC, true, -1)
#undef MW_GEMM_PAIR

#define MW_SYRK_PAIR(NAME, VT, HERM)                                                                              \
    void NAME##_(const char *uplo, const char *trans, const int *n, const int *k, const TR *alpha, const VT *a,  \
                 const int *lda, const TR *beta, VT *c, const int *ldc)                                         \
    {                                                                                                           \
        mw::syrk_entry<int>(#NAME, HERM, uplo, trans, n, k, alpha, a, lda, beta, c, ldc);                        \
    }                                                                                                           \
    void NAME##_64_(const char *uplo, const char *trans, const int64_t *n, const int64_t *k, const TR *alpha,   \
                    const VT *a, const int64_t *lda, const TR *beta, VT *c, const int64_t *ldc)                 \
    {                                                                                                           \
        mw::syrk_entry<int64_t>(#NAME, HERM, uplo, trans, n, k, alpha, a, lda, beta, c, ldc);                    \
    }
MW_SYRK_PAIR(msyrk, TR, false)
MW_SYRK_PAIR(wherk, TC, true)
#undef MW_SYRK_PAIR

void mtrsm_(const char *side, const char *uplo, const char *transa, const char *diag, const int *m, const int *n,
            const TR *alpha, const TR *a, const int *lda, TR *b, const int *ldb)
{
    mw::trsm_entry<int>("mtrsm", side, uplo, transa, diag, m, n, alpha, a, lda, b, ldb);
}
void mtrsm_64_(const char *side, const char *uplo, const char *transa, const char *diag, const int64_t *m,
               const int64_t *n, const TR *alpha, const TR *a, const int64_t *lda, TR *b, const int64_t *ldb)
{
    mw::trsm_entry<int64_t>("mtrsm", side, uplo, transa, diag, m, n, alpha, a, lda, b, ldb);
}

#define MW_GEMMTR_PAIR(NAME, T, CPLX)                                                                             \
    void NAME##_(const char *uplo, const char *ta, const char *tb, const int *n, const int *k, const T *alpha,  \
                 const T *a, const int *lda, const T *b, const int *ldb, const T *beta, T *c, const int *ldc)   \
    {                                                                                                           \
        mw::gemmtr_entry<int>(#NAME, CPLX, uplo, ta, tb, n, k, alpha, a, lda, b, ldb, beta, c, ldc);            \
    }                                                                                                           \
    void NAME##_64_(const char *uplo, const char *ta, const char *tb, const int64_t *n, const int64_t *k,      \
                    const T *alpha, const T *a, const int64_t *lda, const T *b, const int64_t *ldb,             \
                    const T *beta, T *c, const int64_t *ldc)                                                    \
    {                                                                                                           \
        mw::gemmtr_entry<int64_t>(#NAME, CPLX, uplo, ta, tb, n, k, alpha, a, lda, b, ldb, beta, c, ldc);        \
    }
MW_GEMMTR_PAIR(mgemmtr, TR, false)
MW_GEMMTR_PAIR(wgemmtr, TC, true)
#undef MW_GEMMTR_PAIR

#define MW_SYMM_PAIR(NAME, T, CPLX, HERM)                                                                         \
    void NAME##_(const char *side, const char *uplo, const int *m, const int *n, const T *alpha, const T *a,    \
                 const int *lda, const T *b, const int *ldb, const T *beta, T *c, const int *ldc)               \
    {                                                                                                           \
        mw::symm_entry<int>(#NAME, CPLX, HERM, side, uplo, m, n, alpha, a, lda, b, ldb, beta, c, ldc);          \
    }                                                                                                           \
    void NAME##_64_(const char *side, const char *uplo, const int64_t *m, const int64_t *n, const T *alpha,     \
                    const T *a, const int64_t *lda, const T *b, const int64_t *ldb, const T *beta, T *c,        \
                    const int64_t *ldc)                                                                         \
    {                                                                                                           \
        mw::symm_entry<int64_t>(#NAME, CPLX, HERM, side, uplo, m, n, alpha, a, lda, b, ldb, beta, c, ldc);      \
    }
MW_SYMM_PAIR(msymm, TR, false, false)
MW_SYMM_PAIR(wsymm, TC, true, false)
MW_SYMM_PAIR(whemm, TC, true, true)
#undef MW_SYMM_PAIR

#define MW_SYR2K_PAIR(NAME, SA, SB, VT, CPLX, HERM)                                                                \
    void NAME##_(const char *uplo, const char *trans, const int *n, const int *k, const SA *alpha, const VT *a,  \
                 const int *lda, const VT *b, const int *ldb, const SB *beta, VT *c, const int *ldc)             \
    {                                                                                                            \
        mw::syr2k_entry<int>(#NAME, CPLX, HERM, uplo, trans, n, k, alpha, a, lda, b, ldb, beta, c, ldc);         \
    }                                                                                                            \
    void NAME##_64_(const char *uplo, const char *trans, const int64_t *n, const int64_t *k, const SA *alpha,   \
                    const VT *a, const int64_t *lda, const VT *b, const int64_t *ldb, const SB *beta, VT *c,     \
                    const int64_t *ldc)                                                                          \
    {                                                                                                            \
        mw::syr2k_entry<int64_t>(#NAME, CPLX, HERM, uplo, trans, n, k, alpha, a, lda, b, ldb, beta, c, ldc);     \
    }
MW_SYR2K_PAIR(msyr2k, TR, TR, TR, false, false)
MW_SYR2K_PAIR(wsyr2k, TC, TC, TC, true, false)
MW_SYR2K_PAIR(wher2k, TC, TR, TC, true, true)
#undef MW_SYR2K_PAIR

void wsyrk_(const char *uplo, const char *trans, const int *n, const int *k, const TC *alpha, const TC *a,
            const int *lda, const TC *beta, TC *c, const int *ldc)
{
    mw::csyrk_entry<int>("wsyrk", uplo, trans, n, k, alpha, a, lda, beta, c, ldc);
}
void wsyrk_64_(const char *uplo, const char *trans, const int64_t *n, const int64_t *k, const TC *alpha, const TC *a,
               const int64_t *lda, const TC *beta, TC *c, const int64_t *ldc)
{
    mw::csyrk_entry<int64_t>("wsyrk", uplo, trans, n, k, alpha, a, lda, beta, c, ldc);
}

#define MW_TRXM_PAIR(NAME, T, CPLX, SOLVE)                                                                          \
    void NAME##_(const char *side, const char *uplo, const char *transa, const char *diag, const int *m,          \
                 const int *n, const T *alpha, const T *a, const int *lda, T *b, const int *ldb)                  \
    {                                                                                                             \
        mw::trxm_entry<int>(#NAME, CPLX, SOLVE, side, uplo, transa, diag, m, n, alpha, a, lda, b, ldb);           \
    }                                                                                                             \
    void NAME##_64_(const char *side, const char *uplo, const char *transa, const char *diag, const int64_t *m,   \
                    const int64_t *n, const T *alpha, const T *a, const int64_t *lda, T *b, const int64_t *ldb)   \
    {                                                                                                             \
        mw::trxm_entry<int64_t>(#NAME, CPLX, SOLVE, side, uplo, transa, diag, m, n, alpha, a, lda, b, ldb);       \
    }
MW_TRXM_PAIR(mtrmm, TR, false, false)
MW_TRXM_PAIR(wtrmm, TC, true, false)
MW_TRXM_PAIR(wtrsm, TC, true, true)
#undef MW_TRXM_PAIR

// ---- further level 1 -----------------------------------------------------------------------

#define MW_CDOT_PAIR(NAME, MODE)                                                                                \
    TC NAME##_(const int *n, const TC *x, const int *incx, const TC *y, const int *incy)                       \
    {                                                                                                          \
        double2 o[2];                                                                                          \
        mw::reduce_entry<int>(#NAME, MODE, n, x, incx, y, incy, o);                                            \
        return TC{{{o[0].x, o[0].y}}, {{o[1].x, o[1].y}}};                                                     \
    }                                                                                                          \
    TC NAME##_64_(const int64_t *n, const TC *x, const int64_t *incx, const TC *y, const int64_t *incy)        \
    {                                                                                                          \
        double2 o[2];                                                                                          \
        mw::reduce_entry<int64_t>(#NAME, MODE, n, x, incx, y, incy, o);                                        \
        return TC{{{o[0].x, o[0].y}}, {{o[1].x, o[1].y}}};                                                     \
    }
MW_CDOT_PAIR(wdotu, 0)
MW_CDOT_PAIR(wdotc, 1)
#undef MW_CDOT_PAIR

#define MW_ASUM_PAIR(NAME, VT, MODE)                                                                           \
    TR NAME##_(const int *n, const VT *x, const int *incx)                                                    \
    {                                                                                                          \
        double2 o[2];                                                                                          \
        mw::reduce_entry<int>(#NAME, MODE, n, x, incx, (const VT *)nullptr, (const int *)nullptr, o);          \
        return TR{{o[0].x, o[0].y}};                                                                           \
    }                                                                                                          \
    TR NAME##_64_(const int64_t *n, const VT *x, const int64_t *incx)                                         \
    {                                                                                                          \
        double2 o[2];                                                                                          \
        mw::reduce_entry<int64_t>(#NAME, MODE, n, x, incx, (const VT *)nullptr, (const int64_t *)nullptr, o);  \
        return TR{{o[0].x, o[0].y}};                                                                           \
    }
MW_ASUM_PAIR(masum, TR, 2)
MW_ASUM_PAIR(mwasum, TC, 3)
MW_ASUM_PAIR(mnrm2, TR, 4)
MW_ASUM_PAIR(mwnrm2, TC, 5)
#undef MW_ASUM_PAIR

void waxpy_(const int *n, const TC *alpha, const TC *x, const int *incx, TC *y, const int *incy)
{
    mw::waxpy_entry<int>(n, alpha, x, incx, y, incy);
}
void waxpy_64_(const int64_t *n, const TC *alpha, const TC *x, const int64_t *incx, TC *y, const int64_t *incy)
{
    mw::waxpy_entry<int64_t>(n, alpha, x, incx, y, incy);
}

#define MW_ROT_PAIR(NAME, VT, E2)                                                                               \
    void NAME##_(const int *n, VT *x, const int *incx, VT *y, const int *incy, const TR *c, const TR *s)        \
    {                                                                                                          \
        mw::rotcs_entry<int>(#NAME, E2, n, x, incx, y, incy, c, s);                                            \
    }                                                                                                          \
    void NAME##_64_(const int64_t *n, VT *x, const int64_t *incx, VT *y, const int64_t *incy, const TR *c,     \
                    const TR *s)                                                                               \
    {                                                                                                          \
        mw::rotcs_entry<int64_t>(#NAME, E2, n, x, incx, y, incy, c, s);                                        \
    }
MW_ROT_PAIR(mrot, TR, 1)
MW_ROT_PAIR(wmrot, TC, 2)
#undef MW_ROT_PAIR

void mrotm_(const int *n, TR *x, const int *incx, TR *y, const int *incy, const TR *dparam)
{
    mw::rotm_entry<int>(n, x, incx, y, incy, dparam);
}
void mrotm_64_(const int64_t *n, TR *x, const int64_t *incx, TR *y, const int64_t *incy, const TR *dparam)
{
    mw::rotm_entry<int64_t>(n, x, incx, y, incy, dparam);
}

TR mcabs1_(const TC *z) { return mw::cabs1_entry(z); }
TR mcabs1_64_(const TC *z) { return mw::cabs1_entry(z); }
void mrotg_(TR *a, TR *b, TR *c, TR *s) { mw::rotg_entry(a, b, c, s); }
void mrotg_64_(TR *a, TR *b, TR *c, TR *s) { mw::rotg_entry(a, b, c, s); }
void mrotmg_(TR *d1, TR *d2, TR *x1, const TR *y1, TR *dparam) { mw::rotmg_entry(d1, d2, x1, y1, dparam); }
void mrotmg_64_(TR *d1, TR *d2, TR *x1, const TR *y1, TR *dparam) { mw::rotmg_entry(d1, d2, x1, y1, dparam); }
void wrotg_(TC *a, const TC *b, TR *c, TC *s) { mw::wrotg_entry(a, b, c, s); }
void wrotg_64_(TC *a, const TC *b, TR *c, TC *s) { mw::wrotg_entry(a, b, c, s); }

// ---- level 2 beyond real GEMV -------------------------------------------------------------

void wgemv_(const char *trans, const int *m, const int *n, const TC *alpha, const TC *a, const int *lda, const TC *x,
            const int *incx, const TC *beta, TC *y, const int *incy)
{
    mw::gemv2_entry<int>("wgemv", true, false, trans, m, n, (const int *)nullptr, (const int *)nullptr, alpha, a, lda,
                         x, incx, beta, y, incy);
}
void wgemv_64_(const char *trans, const int64_t *m, const int64_t *n, const TC *alpha, const TC *a, const int64_t *lda,
               const TC *x, const int64_t *incx, const TC *beta, TC *y, const int64_t *incy)
{
    mw::gemv2_entry<int64_t>("wgemv", true, false, trans, m, n, (const int64_t *)nullptr, (const int64_t *)nullptr,
                             alpha, a, lda, x, incx, beta, y, incy);
}

#define MW_GBMV_PAIR(NAME, T, CPLX)                                                                              \
    void NAME##_(const char *trans, const int *m, const int *n, const int *kl, const int *ku, const T *alpha,   \
                 const T *a, const int *lda, const T *x, const int *incx, const T *beta, T *y, const int *incy) \
    {                                                                                                          \
        mw::gemv2_entry<int>(#NAME, CPLX, true, trans, m, n, kl, ku, alpha, a, lda, x, incx, beta, y, incy);   \
    }                                                                                                          \
    void NAME##_64_(const char *trans, const int64_t *m, const int64_t *n, const int64_t *kl, const int64_t *ku, \
                    const T *alpha, const T *a, const int64_t *lda, const T *x, const int64_t *incx,            \
                    const T *beta, T *y, const int64_t *incy)                                                   \
    {                                                                                                          \
        mw::gemv2_entry<int64_t>(#NAME, CPLX, true, trans, m, n, kl, ku, alpha, a, lda, x, incx, beta, y,      \
                                 incy);                                                                         \
    }
MW_GBMV_PAIR(mgbmv, TR, false)
MW_GBMV_PAIR(wgbmv, TC, true)
#undef MW_GBMV_PAIR

#define MW_SYMV_PAIR(NAME, T, CPLX, HERM)                                                                          \
    void NAME##_(const char *uplo, const int *n, const T *alpha, const T *a, const int *lda, const T *x,          \
                 const int *incx, const T *beta, T *y, const int *incy)                                           \
    {                                                                                                            \
        mw::symv_entry<int>(#NAME, CPLX, HERM, 0, uplo, n, (const int *)nullptr, alpha, a, lda, x, incx, beta, y, \
                            incy);                                                                                \
    }                                                                                                            \
    void NAME##_64_(const char *uplo, const int64_t *n, const T *alpha, const T *a, const int64_t *lda,           \
                    const T *x, const int64_t *incx, const T *beta, T *y, const int64_t *incy)                    \
    {                                                                                                            \
        mw::symv_entry<int64_t>(#NAME, CPLX, HERM, 0, uplo, n, (const int64_t *)nullptr, alpha, a, lda, x, incx,  \
                                beta, y, incy);                                                                   \
    }
MW_SYMV_PAIR(msymv, TR, false, false)
MW_SYMV_PAIR(whemv, TC, true, true)
#undef MW_SYMV_PAIR

#define MW_SBMV_PAIR(NAME, T, CPLX, HERM)                                                                          \
    void NAME##_(const char *uplo, const int *n, const int *k, const T *alpha, const T *a, const int *lda,        \
                 const T *x, const int *incx, const T *beta, T *y, const int *incy)                               \
    {                                                                                                            \
        mw::symv_entry<int>(#NAME, CPLX, HERM, 1, uplo, n, k, alpha, a, lda, x, incx, beta, y, incy);            \
    }                                                                                                            \
    void NAME##_64_(const char *uplo, const int64_t *n, const int64_t *k, const T *alpha, const T *a,             \
                    const int64_t *lda, const T *x, const int64_t *incx, const T *beta, T *y, const int64_t *incy) \
    {                                                                                                            \
        mw::symv_entry<int64_t>(#NAME, CPLX, HERM, 1, uplo, n, k, alpha, a, lda, x, incx, beta, y, incy);        \
    }
MW_SBMV_PAIR(msbmv, TR, false, false)
MW_SBMV_PAIR(whbmv, TC, true, true)
#undef MW_SBMV_PAIR

#define MW_SPMV_PAIR(NAME, T, CPLX, HERM)                                                                          \
    void NAME##_(const char *uplo, const int *n, const T *alpha, const T *ap, const T *x, const int *incx,        \
                 const T *beta, T *y, const int *incy)                                                            \
    {                                                                                                            \
        mw::symv_entry<int>(#NAME, CPLX, HERM, 2, uplo, n, (const int *)nullptr, alpha, ap, (const int *)nullptr, \
                            x, incx, beta, y, incy);                                                              \
    }                                                                                                            \
    void NAME##_64_(const char *uplo, const int64_t *n, const T *alpha, const T *ap, const T *x,                  \
                    const int64_t *incx, const T *beta, T *y, const int64_t *incy)                                \
    {                                                                                                            \
        mw::symv_entry<int64_t>(#NAME, CPLX, HERM, 2, uplo, n, (const int64_t *)nullptr, alpha, ap,               \
                                (const int64_t *)nullptr, x, incx, beta, y, incy);                                \
    }
MW_SPMV_PAIR(mspmv, TR, false, false)
MW_SPMV_PAIR(whpmv, TC, true, true)
#undef MW_SPMV_PAIR

#define MW_TRV_PAIR(NAME, T, CPLX, SOLVE)                                                                          \
    void NAME##_(const char *uplo, const char *trans, const char *diag, const int *n, const T *a, const int *lda, \
                 T *x, const int *incx)                                                                           \
    {                                                                                                            \
        mw::trv_entry<int>(#NAME, CPLX, SOLVE, 0, uplo, trans, diag, n, (const int *)nullptr, a, lda, x, incx);  \
    }                                                                                                            \
    void NAME##_64_(const char *uplo, const char *trans, const char *diag, const int64_t *n, const T *a,          \
                    const int64_t *lda, T *x, const int64_t *incx)                                                \
    {                                                                                                            \
        mw::trv_entry<int64_t>(#NAME, CPLX, SOLVE, 0, uplo, trans, diag, n, (const int64_t *)nullptr, a, lda, x, \
                               incx);                                                                             \
    }
MW_TRV_PAIR(mtrmv, TR, false, false)
MW_TRV_PAIR(wtrmv, TC, true, false)
MW_TRV_PAIR(mtrsv, TR, false, true)
MW_TRV_PAIR(wtrsv, TC, true, true)
#undef MW_TRV_PAIR

#define MW_TBV_PAIR(NAME, T, CPLX, SOLVE)                                                                          \
    void NAME##_(const char *uplo, const char *trans, const char *diag, const int *n, const int *k, const T *a,  \
                 const int *lda, T *x, const int *incx)                                                           \
    {                                                                                                            \
        mw::trv_entry<int>(#NAME, CPLX, SOLVE, 1, uplo, trans, diag, n, k, a, lda, x, incx);                      \
    }                                                                                                            \
    void NAME##_64_(const char *uplo, const char *trans, const char *diag, const int64_t *n, const int64_t *k,    \
                    const T *a, const int64_t *lda, T *x, const int64_t *incx)                                    \
    {                                                                                                            \
        mw::trv_entry<int64_t>(#NAME, CPLX, SOLVE, 1, uplo, trans, diag, n, k, a, lda, x, incx);                  \
    }
MW_TBV_PAIR(mtbmv, TR, false, false)
MW_TBV_PAIR(wtbmv, TC, true, false)
MW_TBV_PAIR(mtbsv, TR, false, true)
MW_TBV_PAIR(wtbsv, TC, true, true)
#undef MW_TBV_PAIR

#define MW_TPV_PAIR(NAME, T, CPLX, SOLVE)                                                                          \
    void NAME##_(const char *uplo, const char *trans, const char *diag, const int *n, const T *ap, T *x,          \
                 const int *incx)                                                                                 \
    {                                                                                                            \
        mw::trv_entry<int>(#NAME, CPLX, SOLVE, 2, uplo, trans, diag, n, (const int *)nullptr, ap,                 \
                           (const int *)nullptr, x, incx);                                                        \
    }                                                                                                            \
    void NAME##_64_(const char *uplo, const char *trans, const char *diag, const int64_t *n, const T *ap, T *x,   \
                    const int64_t *incx)                                                                          \
    {                                                                                                            \
        mw::trv_entry<int64_t>(#NAME, CPLX, SOLVE, 2, uplo, trans, diag, n, (const int64_t *)nullptr, ap,         \
                               (const int64_t *)nullptr, x, incx);                                                \
    }
MW_TPV_PAIR(mtpmv, TR, false, false)
MW_TPV_PAIR(wtpmv, TC, true, false)
MW_TPV_PAIR(mtpsv, TR, false, true)
MW_TPV_PAIR(wtpsv, TC, true, true)
#undef MW_TPV_PAIR

#define MW_GER_PAIR(NAME, T, CPLX, CONJ)                                                                           \
    void NAME##_(const int *m, const int *n, const T *alpha, const T *x, const int *incx, const T *y,            \
                 const int *incy, T *a, const int *lda)                                                           \
    {                                                                                                            \
        mw::ger_entry<int>(#NAME, CPLX, CONJ, m, n, alpha, x, incx, y, incy, a, lda);                            \
    }                                                                                                            \
    void NAME##_64_(const int64_t *m, const int64_t *n, const T *alpha, const T *x, const int64_t *incx,          \
                    const T *y, const int64_t *incy, T *a, const int64_t *lda)                                    \
    {                                                                                                            \
        mw::ger_entry<int64_t>(#NAME, CPLX, CONJ, m, n, alpha, x, incx, y, incy, a, lda);                        \
    }
MW_GER_PAIR(mger, TR, false, false)
MW_GER_PAIR(wgeru, TC, true, false)
MW_GER_PAIR(wgerc, TC, true, true)
#undef MW_GER_PAIR

#define MW_SYR_PAIR(NAME, ST, VT, CPLX, HERM)                                                                      \
    void NAME##_(const char *uplo, const int *n, const ST *alpha, const VT *x, const int *incx, VT *a,           \
                 const int *lda)                                                                                  \
    {                                                                                                            \
        mw::syr_entry<int>(#NAME, CPLX, HERM, false, false, uplo, n, alpha, x, incx, (const VT *)nullptr,         \
                           (const int *)nullptr, a, lda);                                                         \
    }                                                                                                            \
    void NAME##_64_(const char *uplo, const int64_t *n, const ST *alpha, const VT *x, const int64_t *incx, VT *a, \
                    const int64_t *lda)                                                                           \
    {                                                                                                            \
        mw::syr_entry<int64_t>(#NAME, CPLX, HERM, false, false, uplo, n, alpha, x, incx, (const VT *)nullptr,     \
                               (const int64_t *)nullptr, a, lda);                                                 \
    }
MW_SYR_PAIR(msyr, TR, TR, false, false)
MW_SYR_PAIR(wher, TR, TC, true, true)
#undef MW_SYR_PAIR

#define MW_SPR_PAIR(NAME, ST, VT, CPLX, HERM)                                                                      \
    void NAME##_(const char *uplo, const int *n, const ST *alpha, const VT *x, const int *incx, VT *ap)          \
    {                                                                                                            \
        mw::syr_entry<int>(#NAME, CPLX, HERM, true, false, uplo, n, alpha, x, incx, (const VT *)nullptr,          \
                           (const int *)nullptr, ap, (const int *)nullptr);                                       \
    }                                                                                                            \
    void NAME##_64_(const char *uplo, const int64_t *n, const ST *alpha, const VT *x, const int64_t *incx,        \
                    VT *ap)                                                                                       \
    {                                                                                                            \
        mw::syr_entry<int64_t>(#NAME, CPLX, HERM, true, false, uplo, n, alpha, x, incx, (const VT *)nullptr,      \
                               (const int64_t *)nullptr, ap, (const int64_t *)nullptr);                           \
    }
MW_SPR_PAIR(mspr, TR, TR, false, false)
MW_SPR_PAIR(whpr, TR, TC, true, true)
#undef MW_SPR_PAIR

#define MW_SYR2_PAIR(NAME, T, CPLX, HERM, PACKED)                                                                 \
    void NAME##_(const char *uplo, const int *n, const T *alpha, const T *x, const int *incx, const T *y,       \
                 const int *incy, T *a, const int *lda)                                                          \
    {                                                                                                           \
        mw::syr_entry<int>(#NAME, CPLX, HERM, PACKED, true, uplo, n, alpha, x, incx, y, incy, a, lda);          \
    }                                                                                                           \
    void NAME##_64_(const char *uplo, const int64_t *n, const T *alpha, const T *x, const int64_t *incx,         \
                    const T *y, const int64_t *incy, T *a, const int64_t *lda)                                   \
    {                                                                                                           \
        mw::syr_entry<int64_t>(#NAME, CPLX, HERM, PACKED, true, uplo, n, alpha, x, incx, y, incy, a, lda);      \
    }
MW_SYR2_PAIR(msyr2, TR, false, false, false)
MW_SYR2_PAIR(wher2, TC, true, true, false)
#undef MW_SYR2_PAIR

#define MW_SPR2_PAIR(NAME, T, CPLX, HERM)                                                                          \
    void NAME##_(const char *uplo, const int *n, const T *alpha, const T *x, const int *incx, const T *y,        \
                 const int *incy, T *ap)                                                                          \
    {                                                                                                            \
        mw::syr_entry<int>(#NAME, CPLX, HERM, true, true, uplo, n, alpha, x, incx, y, incy, ap,                  \
                           (const int *)nullptr);                                                                 \
    }                                                                                                            \
    void NAME##_64_(const char *uplo, const int64_t *n, const T *alpha, const T *x, const int64_t *incx,          \
                    const T *y, const int64_t *incy, T *ap)                                                       \
    {                                                                                                            \
        mw::syr_entry<int64_t>(#NAME, CPLX, HERM, true, true, uplo, n, alpha, x, incx, y, incy, ap,              \
                               (const int64_t *)nullptr);                                                         \
    }
MW_SPR2_PAIR(mspr2, TR, false, false)
MW_SPR2_PAIR(whpr2, TC, true, true)
#undef MW_SPR2_PAIR

// ---- level 2 -----------------------------------------------------------------------------

void mgemv_(const char *trans, const int *m, const int *n, const TR *alpha, const TR *a, const int *lda, const TR *x,
            const int *incx, const TR *beta, TR *y, const int *incy)
{
    mw::gemv_entry<int>("mgemv", trans, m, n, alpha, a, lda, x, incx, beta, y, incy);
}
void mgemv_64_(const char *trans, const int64_t *m, const int64_t *n, const TR *alpha, const TR *a,
               const int64_t *lda, const TR *x, const int64_t *incx, const TR *beta, TR *y, const int64_t *incy)
{
    mw::gemv_entry<int64_t>("mgemv", trans, m, n, alpha, a, lda, x, incx, beta, y, incy);
}

void mgemm_plain_64_(const char *ta, const char *tb, const int64_t *m, const int64_t *n, const int64_t *k,
                     const TR *alpha, const TR *a, const int64_t *lda, const TR *b, const int64_t *ldb,
                     const TR *beta, TR *c, const int64_t *ldc)
{
    mw::gemm_entry<int64_t>("mgemm_plain", false, MWBLAS_GEMM_PLAIN, ta, tb, m, n, k, alpha, a, lda, b, ldb, beta,
                            c, ldc);
}

void mgemm_fixed_64_(const char *ta, const char *tb, const int64_t *m, const int64_t *n, const int64_t *k,
                     const TR *alpha, const TR *a, const int64_t *lda, const TR *b, const int64_t *ldb,
                     const TR *beta, TR *c, const int64_t *ldc)
{
    mw::gemm_entry<int64_t>("mgemm_fixed", false, MWBLAS_GEMM_FIXED, ta, tb, m, n, k, alpha, a, lda, b, ldb, beta,
                            c, ldc);
}

void mgemm_ozaki_64_(const char *ta, const char *tb, const int64_t *m, const int64_t *n, const int64_t *k,
                     const TR *alpha, const TR *a, const int64_t *lda, const TR *b, const int64_t *ldb,
                     const TR *beta, TR *c, const int64_t *ldc)
{
    mw::gemm_entry<int64_t>("mgemm_ozaki", false, MWBLAS_GEMM_OZAKI, ta, tb, m, n, k, alpha, a, lda, b, ldb, beta,
                            c, ldc);
}

int mwblas_set_gemm_engine(int engine)
{
    int prev = mw::engine();
    if (engine >= MWBLAS_GEMM_AUTO && engine <= MWBLAS_GEMM_FIXED) mw::g_engine = engine;
    return prev;
}
int mwblas_get_gemm_engine(void) { return mw::engine(); }
int mwblas_set_band_solve(int mode)
{
    int prev = mw::g_band_solve.load();
    if (mode >= MWBLAS_BAND_SOLVE_AUTO && mode <= MWBLAS_BAND_SOLVE_DENSE) mw::g_band_solve = mode;
    return prev;
}
int mwblas_set_ozaki_bits(int bits)
{
    int prev = mw::g_ozaki_bits;
    mw::g_ozaki_bits = bits < 0 ? 0 : bits;
    return prev;
}
int mwblas_last_ozaki_moduli(void) { return mw::ozaki_last_moduli(); }
int mwblas_last_ozaki_bits(int operand) { return mw::ozaki_last_bits(operand); }

// ---- level 1 -----------------------------------------------------------------------------

void mscal_(const int *n, const TR *alpha, TR *x, const int *incx) { mw::scal_entry<int>("mscal", 0, n, alpha, x, incx); }
void mscal_64_(const int64_t *n, const TR *alpha, TR *x, const int64_t *incx)
{
    mw::scal_entry<int64_t>("mscal", 0, n, alpha, x, incx);
}
void wscal_(const int *n, const TC *alpha, TC *x, const int *incx) { mw::scal_entry<int>("wscal", 1, n, alpha, x, incx); }
void wscal_64_(const int64_t *n, const TC *alpha, TC *x, const int64_t *incx)
{
    mw::scal_entry<int64_t>("wscal", 1, n, alpha, x, incx);
}
void wmscal_(const int *n, const TR *alpha, TC *x, const int *incx) { mw::scal_entry<int>("wmscal", 2, n, alpha, x, incx); }
void wmscal_64_(const int64_t *n, const TR *alpha, TC *x, const int64_t *incx)
{
    mw::scal_entry<int64_t>("wmscal", 2, n, alpha, x, incx);
}

void maxpy_(const int *n, const TR *alpha, const TR *x, const int *incx, TR *y, const int *incy)
{
    mw::axpy_entry<int>("maxpy", n, alpha, x, incx, y, incy);
}
void maxpy_64_(const int64_t *n, const TR *alpha, const TR *x, const int64_t *incx, TR *y, const int64_t *incy)
{
    mw::axpy_entry<int64_t>("maxpy", n, alpha, x, incx, y, incy);
}

void mcopy_(const int *n, const TR *x, const int *incx, TR *y, const int *incy)
{
    mw::copy_entry<int>("mcopy", false, n, x, incx, y, incy);
}
void mcopy_64_(const int64_t *n, const TR *x, const int64_t *incx, TR *y, const int64_t *incy)
{
    mw::copy_entry<int64_t>("mcopy", false, n, x, incx, y, incy);
}
void wcopy_(const int *n, const TC *x, const int *incx, TC *y, const int *incy)
{
    mw::copy_entry<int>("wcopy", true, n, x, incx, y, incy);
}
void wcopy_64_(const int64_t *n, const TC *x, const int64_t *incx, TC *y, const int64_t *incy)
{
    mw::copy_entry<int64_t>("wcopy", true, n, x, incx, y, incy);
}

void mswap_(const int *n, TR *x, const int *incx, TR *y, const int *incy)
{
    mw::swap_entry<int>("mswap", false, n, x, incx, y, incy);
}
void mswap_64_(const int64_t *n, TR *x, const int64_t *incx, TR *y, const int64_t *incy)
{
    mw::swap_entry<int64_t>("mswap", false, n, x, incx, y, incy);
}
void wswap_(const int *n, TC *x, const int *incx, TC *y, const int *incy)
{
    mw::swap_entry<int>("wswap", true, n, x, incx, y, incy);
}
void wswap_64_(const int64_t *n, TC *x, const int64_t *incx, TC *y, const int64_t *incy)
{
    mw::swap_entry<int64_t>("wswap", true, n, x, incx, y, incy);
}

int imamax_(const int *n, const TR *x, const int *incx) { return (int)mw::iamax_entry<int>("imamax", false, n, x, incx); }
int64_t imamax_64_(const int64_t *n, const TR *x, const int64_t *incx)
{
    return mw::iamax_entry<int64_t>("imamax", false, n, x, incx);
}
int iwamax_(const int *n, const TC *x, const int *incx) { return (int)mw::iamax_entry<int>("iwamax", true, n, x, incx); }
int64_t iwamax_64_(const int64_t *n, const TC *x, const int64_t *incx)
{
    return mw::iamax_entry<int64_t>("iwamax", true, n, x, incx);
}

TR mdot_(const int *n, const TR *x, const int *incx, const TR *y, const int *incy)
{
    return mw::dot_entry<int>("mdot", n, x, incx, y, incy);
}
TR mdot_64_(const int64_t *n, const TR *x, const int64_t *incx, const TR *y, const int64_t *incy)
{
    return mw::dot_entry<int64_t>("mdot", n, x, incx, y, incy);
}

}  // extern "C"
