/*
 * ddoracle.c — CPU oracle for the double-double BLAS path.
 *
 * TEST INFRASTRUCTURE ONLY. Only tests/, __graft_entry__.smoke() and the CPU
 * baseline legs of bench.py may load this library, and only as the checker
 * or the timed CPU baseline; the GPU library never calls it.
 *
 * Two kinds of function live here:
 *   1. Restatements of the reference's double-double algorithms, op for op,
 *      each citing the reference file:line it follows (paths relative to the
 *      reference project root). These give the bit-exact expectations for
 *      SCAL/AXPY/COPY/SWAP/I*AMAX and the "port" CPU baseline for the
 *      level-2/3 routines.
 *   2. Binary128 references (the reference's kind16 __float128 precision,
 *      src/epblas-parallel/kind16/) used to measure the normwise error of the
 *      floating-point routines: every DD input converts exactly to binary128
 *      (hi + lo), the operation runs in binary128, the result rounds back to DD.
 *
 * Parity pinning: the bit-exact restatements are checked against outputs of
 * the reference's own sources built here with a clean-room multifloats shim,
 * and the binary128 functions against the reference's kind16 routines (golden
 * fixtures in tests/golden/, made by tests/golden/make_golden.py). The shim's
 * scalar operators follow the reference's own description of them
 * (mf_simd_exact.h:60-99); the upstream multifloats v0.8.1 source is absent,
 * so its non-finite/-0 short-circuits and its operator/ bits are unpinned.
 *
 * Build with -ffp-contract=off: every a*b+c below that is not an explicit
 * fma() must round twice.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#if defined(__x86_64__) || defined(__i386__)
typedef __float128 qreal;
#elif defined(__aarch64__)
typedef long double qreal; /* IEEE binary128 on AArch64 Linux */
#else
#error "binary128 type unknown for this target"
#endif

typedef struct { double hi, lo; } dd;
typedef struct { dd re, im; } cdd;

/* ====================== error-free transforms ============================ */
/* mf_simd_fast.h:49-75 */
static inline void two_prod(double a, double b, double *p, double *e)
{
    *p = a * b;
    *e = fma(a, b, -*p);
}
static inline void two_sum(double a, double b, double *s, double *e)
{
    double ss = a + b;
    double bb = ss - a;
    double aa = ss - bb;
    double da = a - aa;
    double db = b - bb;
    *s = ss;
    *e = da + db;
}
static inline void fast_two_sum(double a, double b, double *s, double *e)
{
    double ss = a + b;
    double t = ss - a;
    *s = ss;
    *e = b - t;
}

/* mf_simd_fast.h:79-89 (fast mul: cross terms fused, a first) */
static inline dd mul_fast(dd a, dd b)
{
    double ph, pe;
    two_prod(a.hi, b.hi, &ph, &pe);
    pe = fma(a.hi, b.lo, pe);
    pe = fma(a.lo, b.hi, pe);
    dd r;
    fast_two_sum(ph, pe, &r.hi, &r.lo);
    return r;
}
/* mf_simd_fast.h:93-102 (fast "sloppy" add) */
static inline dd add_fast(dd a, dd b)
{
    double sh, se;
    two_sum(a.hi, b.hi, &sh, &se);
    double t = a.lo + b.lo;
    se = se + t;
    dd r;
    fast_two_sum(sh, se, &r.hi, &r.lo);
    return r;
}
/* mf_simd_exact.h:62-73 (scalar operator*) */
static inline dd mul_exact(dd a, dd b)
{
    double p00, e00;
    two_prod(a.hi, b.hi, &p00, &e00);
    double p01 = a.hi * b.lo;
    double p10 = a.lo * b.hi;
    p01 = p01 + p10;
    e00 = e00 + p01;
    dd r;
    fast_two_sum(p00, e00, &r.hi, &r.lo);
    return r;
}
/* mf_simd_exact.h:77-88 (scalar operator+) */
static inline dd add_exact(dd x, dd y)
{
    double a, b, c, d;
    two_sum(x.hi, y.hi, &a, &b);
    two_sum(x.lo, y.lo, &c, &d);
    fast_two_sum(a, c, &a, &c);
    b = b + d;
    b = b + c;
    dd r;
    fast_two_sum(a, b, &r.hi, &r.lo);
    return r;
}
static inline dd dneg(dd a) { dd r = {-a.hi, -a.lo}; return r; }
/* mf_simd_exact.h:90-99 */
static inline dd sub_exact(dd x, dd y) { return add_exact(x, dneg(y)); }

/* mf_simd_fast.h:119-134 */
static inline cdd cmul_fast(cdd a, cdd b)
{
    cdd r;
    dd p = mul_fast(a.re, b.re), q = mul_fast(a.im, b.im);
    r.re = add_fast(p, dneg(q));
    p = mul_fast(a.re, b.im);
    q = mul_fast(a.im, b.re);
    r.im = add_fast(p, q);
    return r;
}
/* mf_kernels.h:43-45 */
static inline cdd cmul_exact(cdd a, cdd b)
{
    cdd r;
    r.re = sub_exact(mul_exact(a.re, b.re), mul_exact(a.im, b.im));
    r.im = add_exact(mul_exact(a.re, b.im), mul_exact(a.im, b.re));
    return r;
}

static inline int eq0(dd a) { return a.hi == 0.0 && a.lo == 0.0; }
static inline int eq1(dd a) { return a.hi == 1.0 && a.lo == 0.0; }

/* Exported EFT probes (used to pin the device vocabulary bit for bit). */
void or_dd_mul_fast(const dd *a, const dd *b, dd *r, int64_t n)
{
    for (int64_t i = 0; i < n; ++i) r[i] = mul_fast(a[i], b[i]);
}
void or_dd_add_fast(const dd *a, const dd *b, dd *r, int64_t n)
{
    for (int64_t i = 0; i < n; ++i) r[i] = add_fast(a[i], b[i]);
}
void or_dd_mul_exact(const dd *a, const dd *b, dd *r, int64_t n)
{
    for (int64_t i = 0; i < n; ++i) r[i] = mul_exact(a[i], b[i]);
}
void or_dd_add_exact(const dd *a, const dd *b, dd *r, int64_t n)
{
    for (int64_t i = 0; i < n; ++i) r[i] = add_exact(a[i], b[i]);
}

/* ====================== partition (common/blas_omp.h:79-84) ============== */
static inline int64_t part_bound(int64_t total, int64_t idx, int64_t nparts)
{
    int64_t base = total / nparts, rem = total % nparts;
    return idx * base + (idx < rem ? idx : rem);
}

/* ====================== bit-exact level 1 ================================ */

/* mscal.cpp:42-58 (unit kernel), :88-102 (core); team = reference OpenMP
 * team size for the unit-stride path (1 = serial). */
void or_mscal(int64_t n, const dd *alpha, dd *x, int64_t incx, int64_t team)
{
    dd a = *alpha;
    if (n <= 0 || eq1(a)) return;
    if (incx == 1) {
        if (team < 1) team = 1;
        for (int64_t t = 0; t < team; ++t) {
            int64_t lo = part_bound(n, t, team), hi = part_bound(n, t + 1, team);
            int64_t len = hi - lo, n4 = len & ~(int64_t)3;
            for (int64_t i = 0; i < n4; ++i) x[lo + i] = mul_fast(x[lo + i], a);
            for (int64_t i = n4; i < len; ++i) x[lo + i] = mul_exact(x[lo + i], a);
        }
    } else {
        int64_t ix = (incx < 0) ? (-n + 1) * incx : 0;
        for (int64_t i = 0; i < n; ++i) { x[ix] = mul_exact(x[ix], a); ix += incx; }
    }
}

/* wscal.cpp (unit kernel: simd_fast::cmul(x, alpha) body, mf_kernels::cmul
 * tail; strided: cmul) */
void or_wscal(int64_t n, const cdd *alpha, cdd *x, int64_t incx, int64_t team)
{
    cdd a = *alpha;
    if (n <= 0 || (eq1(a.re) && eq0(a.im))) return;
    if (incx == 1) {
        if (team < 1) team = 1;
        for (int64_t t = 0; t < team; ++t) {
            int64_t lo = part_bound(n, t, team), hi = part_bound(n, t + 1, team);
            int64_t len = hi - lo, n4 = len & ~(int64_t)3;
            for (int64_t i = 0; i < n4; ++i) x[lo + i] = cmul_fast(x[lo + i], a);
            for (int64_t i = n4; i < len; ++i) x[lo + i] = cmul_exact(x[lo + i], a);
        }
    } else {
        int64_t ix = (incx < 0) ? (-n + 1) * incx : 0;
        for (int64_t i = 0; i < n; ++i) { x[ix] = cmul_exact(x[ix], a); ix += incx; }
    }
}

/* wmscal.cpp (real alpha scales both parts; body fast mul(x, alpha)) */
void or_wmscal(int64_t n, const dd *alpha, cdd *x, int64_t incx, int64_t team)
{
    dd a = *alpha;
    if (n <= 0 || eq1(a)) return;
    if (incx == 1) {
        if (team < 1) team = 1;
        for (int64_t t = 0; t < team; ++t) {
            int64_t lo = part_bound(n, t, team), hi = part_bound(n, t + 1, team);
            int64_t len = hi - lo, n4 = len & ~(int64_t)3;
            for (int64_t i = 0; i < n4; ++i) {
                x[lo + i].re = mul_fast(x[lo + i].re, a);
                x[lo + i].im = mul_fast(x[lo + i].im, a);
            }
            for (int64_t i = n4; i < len; ++i) {
                x[lo + i].re = mul_exact(x[lo + i].re, a);
                x[lo + i].im = mul_exact(x[lo + i].im, a);
            }
        }
    } else {
        int64_t ix = (incx < 0) ? (-n + 1) * incx : 0;
        for (int64_t i = 0; i < n; ++i) {
            x[ix].re = mul_exact(x[ix].re, a);
            x[ix].im = mul_exact(x[ix].im, a);
            ix += incx;
        }
    }
}

/* maxpy.cpp:42-58 (body: fast mul(alpha, x) then fast add(y, p); tail:
 * y + alpha*x with the scalar operators), :94-111 (core) */
void or_maxpy(int64_t n, const dd *alpha, const dd *x, int64_t incx, dd *y, int64_t incy, int64_t team)
{
    dd a = *alpha;
    if (n <= 0 || eq0(a)) return;
    if (incx == 1 && incy == 1) {
        if (team < 1) team = 1;
        for (int64_t t = 0; t < team; ++t) {
            int64_t lo = part_bound(n, t, team), hi = part_bound(n, t + 1, team);
            int64_t len = hi - lo, n4 = len & ~(int64_t)3;
            for (int64_t i = 0; i < n4; ++i) y[lo + i] = add_fast(y[lo + i], mul_fast(a, x[lo + i]));
            for (int64_t i = n4; i < len; ++i) y[lo + i] = add_exact(y[lo + i], mul_exact(a, x[lo + i]));
        }
    } else {
        int64_t ix = (incx < 0) ? (-n + 1) * incx : 0;
        int64_t iy = (incy < 0) ? (-n + 1) * incy : 0;
        for (int64_t i = 0; i < n; ++i) {
            y[iy] = add_exact(y[iy], mul_exact(a, x[ix]));
            ix += incx;
            iy += incy;
        }
    }
}

/* mcopy.cpp:30-56; elem = 1 (real) or 2 (complex) DD words */
void or_copy(int64_t n, const dd *x, int64_t incx, dd *y, int64_t incy, int elem)
{
    if (n <= 0) return;
    int64_t ix = (incx < 0) ? (-n + 1) * incx : 0;
    int64_t iy = (incy < 0) ? (-n + 1) * incy : 0;
    for (int64_t i = 0; i < n; ++i) {
        for (int w = 0; w < elem; ++w) y[iy * elem + w] = x[ix * elem + w];
        ix += incx;
        iy += incy;
    }
}

/* mswap.cpp:40-68 (negative increments start at the far end) */
void or_swap(int64_t n, dd *x, int64_t incx, dd *y, int64_t incy, int elem)
{
    if (n <= 0) return;
    int64_t ix = (incx < 0) ? (-n + 1) * incx : 0;
    int64_t iy = (incy < 0) ? (-n + 1) * incy : 0;
    for (int64_t i = 0; i < n; ++i) {
        for (int w = 0; w < elem; ++w) {
            dd t = x[ix * elem + w];
            x[ix * elem + w] = y[iy * elem + w];
            y[iy * elem + w] = t;
        }
        ix += incx;
        iy += incy;
    }
}

/* imamax.cpp:60-72 magnitude (|hi|, sign-adjusted lo) and mf_pred.h:60-63 */
static inline dd vmag(dd a)
{
    uint64_t hb, lb;
    memcpy(&hb, &a.hi, 8);
    memcpy(&lb, &a.lo, 8);
    uint64_t s = hb & 0x8000000000000000ull;
    hb &= 0x7fffffffffffffffull;
    lb ^= s;
    dd r;
    memcpy(&r.hi, &hb, 8);
    memcpy(&r.lo, &lb, 8);
    return r;
}
static inline int dgt(dd a, dd b) { return a.hi > b.hi || (a.hi == b.hi && a.lo > b.lo); }

/* imamax.cpp:178-201: 1-based, lowest index on ties, incx<=0 -> 0 */
int64_t or_imamax(int64_t n, const dd *x, int64_t incx)
{
    if (n < 1 || incx <= 0) return 0;
    if (n == 1) return 1;
    int64_t best = 1;
    dd bv = vmag(x[0]);
    for (int64_t i = 1; i < n; ++i) {
        dd v = vmag(x[i * incx]);
        if (dgt(v, bv)) { bv = v; best = i + 1; }
    }
    return best;
}

/* iwamax.cpp:27, :65-76: cabs1 = |re| + |im| with the scalar operator+ */
int64_t or_iwamax(int64_t n, const cdd *x, int64_t incx)
{
    if (n < 1 || incx <= 0) return 0;
    if (n == 1) return 1;
    int64_t best = 1;
    dd bv = add_exact(vmag(x[0].re), vmag(x[0].im));
    for (int64_t i = 1; i < n; ++i) {
        dd v = add_exact(vmag(x[i * incx].re), vmag(x[i * incx].im));
        if (dgt(v, bv)) { bv = v; best = i + 1; }
    }
    return best;
}

/* ====================== scalar generators ================================== */
/* Double-double division and square root, step for step as the shim's
 * operator/ and sqrtdd (Hida, Li and Bailey 2001 accurate division; Karp and
 * Markstein 1997 square root); the reference does not describe either. */
static inline dd dd_div(dd a, dd b)
{
    double q1 = a.hi / b.hi;
    dd t = {q1, 0.0};
    dd r = sub_exact(a, mul_exact(t, b));
    double q2 = r.hi / b.hi;
    t.hi = q2;
    r = sub_exact(r, mul_exact(t, b));
    double q3 = r.hi / b.hi;
    dd q;
    fast_two_sum(q1, q2, &q.hi, &q.lo);
    dd q3d = {q3, 0.0};
    return add_exact(q, q3d);
}

static inline dd dd_sqrt(dd v)
{
    dd out = {0.0, 0.0};
    if (v.hi <= 0.0) { out.hi = v.hi == 0.0 ? 0.0 : NAN; return out; }
    double s = sqrt(v.hi), p, e;
    two_prod(s, s, &p, &e);
    dd pe = {p, e};
    dd r = sub_exact(v, pe);
    double t = r.hi / (2.0 * s);
    fast_two_sum(s, t, &out.hi, &out.lo);
    return out;
}

/* mf_pred.h:54-70 */
static inline int dlt0(dd x) { return x.hi < 0.0 || (x.hi == 0.0 && x.lo < 0.0); }
static inline int dgt0(dd x) { return x.hi > 0.0 || (x.hi == 0.0 && x.lo > 0.0); }
static inline dd dmag(dd a) { return dlt0(a) ? dneg(a) : a; }
static inline dd dmk(double h) { dd r = {h, 0.0}; return r; }

/* mcabs1.cpp:20-24 */
dd or_mcabs1(const cdd *z) { return add_exact(dmag(z->re), dmag(z->im)); }

/* mrotg.cpp:21-34 (fabsdd is the limb-negating magnitude) */
void or_mrotg(dd *a, dd *b, dd *c, dd *s)
{
    dd an = a->hi < 0.0 ? dneg(*a) : *a, bn = b->hi < 0.0 ? dneg(*b) : *b;
    if (eq0(bn)) { *c = dmk(1.0); *s = dmk(0.0); *b = dmk(0.0); return; }
    if (eq0(an)) { *c = dmk(0.0); *s = dmk(1.0); *a = *b; *b = dmk(1.0); return; }
    dd r = dd_sqrt(add_exact(mul_exact(an, an), mul_exact(bn, bn)));
    if (dgt(dmk(0.0), *a)) r = dneg(r);
    *c = dd_div(*a, r);
    *s = dd_div(*b, r);
    dd z = dgt(an, bn) ? *s : dd_div(dmk(1.0), *c);
    *a = r;
    *b = z;
}

/* mrotmg.cpp:25-106 (DROTMG) */
void or_mrotmg(dd *d1p, dd *d2p, dd *x1p, const dd *y1p, dd *dparam)
{
    const dd zero = dmk(0.0), one = dmk(1.0), mone = dmk(-1.0);
    const dd gam = dmk(4096.0), gamsq = dmk(16777216.0), rgamsq = dmk(5.9604645e-8);
    dd d1 = *d1p, d2 = *d2p, x1 = *x1p, y1 = *y1p;
    dd flag, h11 = zero, h12 = zero, h21 = zero, h22 = zero;
    if (dlt0(d1)) {
        flag = mone;
        d1 = d2 = x1 = zero;
    } else {
        dd p2 = mul_exact(d2, y1);
        if (eq0(p2)) { dparam[0] = dmk(-2.0); return; }
        dd p1 = mul_exact(d1, x1), q2 = mul_exact(p2, y1), q1 = mul_exact(p1, x1);
        if (dgt(dmag(q1), dmag(q2))) {
            h21 = dd_div(dneg(y1), x1);
            h12 = dd_div(p2, p1);
            dd u = sub_exact(one, mul_exact(h12, h21));
            if (dgt0(u)) {
                flag = zero;
                d1 = dd_div(d1, u); d2 = dd_div(d2, u); x1 = mul_exact(x1, u);
            } else {
                flag = mone;
                h11 = h12 = h21 = h22 = zero;
                d1 = d2 = x1 = zero;
            }
        } else if (dlt0(q2)) {
            flag = mone;
            h11 = h12 = h21 = h22 = zero;
            d1 = d2 = x1 = zero;
        } else {
            flag = one;
            h11 = dd_div(p1, p2);
            h22 = dd_div(x1, y1);
            dd u = add_exact(one, mul_exact(h11, h22));
            dd t = dd_div(d2, u);
            d2 = dd_div(d1, u);
            d1 = t;
            x1 = mul_exact(y1, u);
        }
        if (!eq0(d1)) {
            while (!dgt(d1, rgamsq) || !dgt(gamsq, d1)) {
                if (eq0(flag)) { h11 = one; h22 = one; } else { h21 = mone; h12 = one; }
                flag = mone;
                if (!dgt(d1, rgamsq)) {
                    d1 = mul_exact(mul_exact(d1, gam), gam);
                    x1 = dd_div(x1, gam); h11 = dd_div(h11, gam); h12 = dd_div(h12, gam);
                } else {
                    d1 = dd_div(d1, mul_exact(gam, gam));
                    x1 = mul_exact(x1, gam); h11 = mul_exact(h11, gam); h12 = mul_exact(h12, gam);
                }
            }
        }
        if (!eq0(d2)) {
            dd ad2 = dmag(d2);
            while (!dgt(ad2, rgamsq) || !dgt(gamsq, ad2)) {
                if (eq0(flag)) { h11 = one; h22 = one; } else { h21 = mone; h12 = one; }
                flag = mone;
                if (!dgt(ad2, rgamsq)) {
                    d2 = mul_exact(mul_exact(d2, gam), gam);
                    h21 = dd_div(h21, gam); h22 = dd_div(h22, gam);
                } else {
                    d2 = dd_div(d2, mul_exact(gam, gam));
                    h21 = mul_exact(h21, gam); h22 = mul_exact(h22, gam);
                }
                ad2 = dmag(d2);
            }
        }
    }
    dparam[0] = flag;
    if (dlt0(flag)) { dparam[1] = h11; dparam[2] = h21; dparam[3] = h12; dparam[4] = h22; }
    else if (eq0(flag)) { dparam[3] = h12; dparam[2] = h21; }
    else { dparam[1] = h11; dparam[4] = h22; }
    *d1p = d1; *d2p = d2; *x1p = x1;
}

/* wrotg.cpp:27-48 */
void or_wrotg(cdd *a, const cdd *b, dd *c, cdd *s)
{
    dd g2 = add_exact(mul_exact(b->re, b->re), mul_exact(b->im, b->im));
    if (eq0(g2)) { *c = dmk(1.0); s->re = s->im = dmk(0.0); return; }
    dd f2 = add_exact(mul_exact(a->re, a->re), mul_exact(a->im, a->im));
    if (eq0(f2)) {
        *c = dmk(0.0);
        dd d = dd_sqrt(g2);
        s->re = dd_div(b->re, d);
        s->im = dd_div(dneg(b->im), d);
        a->re = d;
        a->im = dmk(0.0);
        return;
    }
    dd h2 = add_exact(f2, g2);
    *c = dd_sqrt(dd_div(f2, h2));
    cdd av = *a;
    a->re = dd_div(av.re, *c);
    a->im = dd_div(av.im, *c);
    dd d = dd_sqrt(mul_exact(f2, h2));
    cdd bc = {b->re, dneg(b->im)};
    cdd p = cmul_exact(bc, av);
    s->re = dd_div(p.re, d);
    s->im = dd_div(p.im, d);
}

/* ====================== binary128 helpers ================================= */
static inline qreal q_of(dd a) { return (qreal)a.hi + (qreal)a.lo; }
static inline dd dd_of(qreal q)
{
    dd r;
    r.hi = (double)q;
    r.lo = (double)(q - (qreal)r.hi);
    return r;
}
typedef struct { qreal re, im; } cq;
static inline cq cq_of(cdd a) { cq r = {q_of(a.re), q_of(a.im)}; return r; }
static inline cdd cdd_of(cq a) { cdd r = {dd_of(a.re), dd_of(a.im)}; return r; }
static inline cq cqmul(cq a, cq b) { cq r = {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; return r; }

/* op(X)(i,j) for column-major X with flag 'N','T','C' */
static inline qreal opq(const dd *X, int64_t ld, char t, int64_t i, int64_t j)
{
    return (t == 'N') ? q_of(X[i + j * ld]) : q_of(X[j + i * ld]);
}
static inline cq opcq(const cdd *X, int64_t ld, char t, int64_t i, int64_t j)
{
    cq v = (t == 'N') ? cq_of(X[i + j * ld]) : cq_of(X[j + i * ld]);
    if (t == 'C') v.im = -v.im;
    return v;
}

/* C := alpha*op(A)*op(B) + beta*C in binary128 (kind16 qgemm_ semantics,
 * src/epblas-parallel/kind16/qgemm_parallel.c). beta == 0 does not read C.
 * If nsample > 0, only the (rows[s], cols[s]) entries are computed and
 * written to out[s]; C is read for them but not modified. */
void or_qgemm(char ta, char tb, int64_t m, int64_t n, int64_t k, const dd *alpha, const dd *A, int64_t lda,
              const dd *B, int64_t ldb, const dd *beta, dd *C, int64_t ldc, int64_t nsample, const int64_t *rows,
              const int64_t *cols, dd *out)
{
    qreal al = q_of(*alpha), be = q_of(*beta);
    int beta0 = eq0(*beta);
    if (ta == 'C') ta = 'T';
    if (tb == 'C') tb = 'T';
    if (nsample > 0) {
#pragma omp parallel for schedule(dynamic, 4)
        for (int64_t s = 0; s < nsample; ++s) {
            int64_t i = rows[s], j = cols[s];
            qreal acc = 0;
            for (int64_t p = 0; p < k; ++p) acc += opq(A, lda, ta, i, p) * opq(B, ldb, tb, p, j);
            qreal c0 = beta0 ? 0 : be * q_of(C[i + j * ldc]);
            out[s] = dd_of(al * acc + c0);
        }
        return;
    }
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t j = 0; j < n; ++j) {
        qreal *acc = (qreal *)calloc((size_t)(m > 0 ? m : 1), sizeof(qreal));
        for (int64_t p = 0; p < k; ++p) {
            qreal b = opq(B, ldb, tb, p, j);
            if (ta == 'N') {
                const dd *ap = A + p * lda;
                for (int64_t i = 0; i < m; ++i) acc[i] += q_of(ap[i]) * b;
            } else {
                for (int64_t i = 0; i < m; ++i) acc[i] += q_of(A[p + i * lda]) * b;
            }
        }
        for (int64_t i = 0; i < m; ++i) {
            qreal c0 = beta0 ? 0 : be * q_of(C[i + j * ldc]);
            C[i + j * ldc] = dd_of(al * acc[i] + c0);
        }
        free(acc);
    }
}

/* complex GEMM in binary128 (kind16 xgemm_ semantics) */
void or_qwgemm(char ta, char tb, int64_t m, int64_t n, int64_t k, const cdd *alpha, const cdd *A, int64_t lda,
               const cdd *B, int64_t ldb, const cdd *beta, cdd *C, int64_t ldc, int64_t nsample,
               const int64_t *rows, const int64_t *cols, cdd *out)
{
    cq al = cq_of(*alpha), be = cq_of(*beta);
    int beta0 = eq0(beta->re) && eq0(beta->im);
    int64_t total = nsample > 0 ? nsample : m * n;
#pragma omp parallel for schedule(dynamic, 16)
    for (int64_t s = 0; s < total; ++s) {
        int64_t i = nsample > 0 ? rows[s] : s % m;
        int64_t j = nsample > 0 ? cols[s] : s / m;
        cq acc = {0, 0};
        for (int64_t p = 0; p < k; ++p) {
            cq t = cqmul(opcq(A, lda, ta, i, p), opcq(B, ldb, tb, p, j));
            acc.re += t.re;
            acc.im += t.im;
        }
        cq r = cqmul(al, acc);
        if (!beta0) {
            cq c0 = cqmul(be, cq_of(C[i + j * ldc]));
            r.re += c0.re;
            r.im += c0.im;
        }
        if (nsample > 0) out[s] = cdd_of(r);
        else C[i + j * ldc] = cdd_of(r);
    }
}

/* SYRK in binary128 on the uplo triangle (kind16 qsyrk_ semantics):
 * trans 'N': C = alpha*A*A^T + beta*C (A n x k), 'T'/'C': alpha*A^T*A. */
void or_qsyrk(char uplo, char trans, int64_t n, int64_t k, const dd *alpha, const dd *A, int64_t lda,
              const dd *beta, dd *C, int64_t ldc)
{
    qreal al = q_of(*alpha), be = q_of(*beta);
    int beta0 = eq0(*beta);
    char t = (trans == 'N') ? 'N' : 'T';
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t j = 0; j < n; ++j) {
        int64_t i0 = (uplo == 'U') ? 0 : j, i1 = (uplo == 'U') ? j + 1 : n;
        for (int64_t i = i0; i < i1; ++i) {
            qreal acc = 0;
            for (int64_t p = 0; p < k; ++p) {
                qreal a = (t == 'N') ? q_of(A[i + p * lda]) : q_of(A[p + i * lda]);
                qreal b = (t == 'N') ? q_of(A[j + p * lda]) : q_of(A[p + j * lda]);
                acc += a * b;
            }
            qreal c0 = beta0 ? 0 : be * q_of(C[i + j * ldc]);
            C[i + j * ldc] = dd_of(al * acc + c0);
        }
    }
}

/* HERK in binary128 with real alpha/beta; Im(diag) = 0 (kind16 xherk_):
 * trans 'N': C = alpha*A*A^H + beta*C, 'C': alpha*A^H*A + beta*C. */
void or_qherk(char uplo, char trans, int64_t n, int64_t k, const dd *alpha, const cdd *A, int64_t lda,
              const dd *beta, cdd *C, int64_t ldc)
{
    qreal al = q_of(*alpha), be = q_of(*beta);
    int beta0 = eq0(*beta);
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t j = 0; j < n; ++j) {
        int64_t i0 = (uplo == 'U') ? 0 : j, i1 = (uplo == 'U') ? j + 1 : n;
        for (int64_t i = i0; i < i1; ++i) {
            cq acc = {0, 0};
            for (int64_t p = 0; p < k; ++p) {
                cq a, b;
                if (trans == 'N') {
                    a = cq_of(A[i + p * lda]);
                    b = cq_of(A[j + p * lda]);
                    b.im = -b.im;
                } else {
                    a = cq_of(A[p + i * lda]);
                    a.im = -a.im;
                    b = cq_of(A[p + j * lda]);
                }
                cq t = cqmul(a, b);
                acc.re += t.re;
                acc.im += t.im;
            }
            cq r = {al * acc.re, al * acc.im};
            if (!beta0) {
                cq c0 = cq_of(C[i + j * ldc]);
                r.re += be * c0.re;
                r.im += be * c0.im;
            }
            if (i == j) r.im = 0;
            C[i + j * ldc] = cdd_of(r);
        }
    }
}

/* TRSM in binary128 (kind16 qtrsm_ semantics): side 'L': op(A) X = alpha B,
 * side 'R': X op(A) = alpha B; B (m x n) overwritten. */
void or_qtrsm(char side, char uplo, char transa, char diag, int64_t m, int64_t n, const dd *alpha, const dd *A,
              int64_t lda, dd *B, int64_t ldb)
{
    qreal al = q_of(*alpha);
    int unit = (diag == 'U');
    char t = (transa == 'N') ? 'N' : 'T';
    int64_t na = (side == 'L') ? m : n;
    /* op(A) element */
#define OPA(i, j) ((t == 'N') ? q_of(A[(i) + (j) * lda]) : q_of(A[(j) + (i) * lda]))
    /* effective lower-ness of op(A) */
    int lower = ((uplo == 'L') != (t == 'T'));
    if (side == 'L') {
#pragma omp parallel for schedule(dynamic, 1)
        for (int64_t j = 0; j < n; ++j) {
            qreal *x = (qreal *)malloc(sizeof(qreal) * (size_t)(m > 0 ? m : 1));
            for (int64_t i = 0; i < m; ++i) x[i] = al * q_of(B[i + j * ldb]);
            if (lower) {
                for (int64_t i = 0; i < m; ++i) {
                    qreal s = x[i];
                    for (int64_t p = 0; p < i; ++p) s -= OPA(i, p) * x[p];
                    x[i] = unit ? s : s / OPA(i, i);
                }
            } else {
                for (int64_t i = m - 1; i >= 0; --i) {
                    qreal s = x[i];
                    for (int64_t p = i + 1; p < m; ++p) s -= OPA(i, p) * x[p];
                    x[i] = unit ? s : s / OPA(i, i);
                }
            }
            for (int64_t i = 0; i < m; ++i) B[i + j * ldb] = dd_of(x[i]);
            free(x);
        }
    } else {
        /* X op(A) = alpha B  <=>  op(A)^T X^T = alpha B^T : row i of X */
#pragma omp parallel for schedule(dynamic, 1)
        for (int64_t i = 0; i < m; ++i) {
            qreal *x = (qreal *)malloc(sizeof(qreal) * (size_t)(n > 0 ? n : 1));
            for (int64_t j = 0; j < n; ++j) x[j] = al * q_of(B[i + j * ldb]);
            /* solve x * op(A) = b: x_j * a_jj + sum_{p != j} x_p a_pj = b_j */
            if (lower) {
                /* op(A) lower: a_pj nonzero for p >= j -> solve j from n-1 down */
                for (int64_t j = n - 1; j >= 0; --j) {
                    qreal s = x[j];
                    for (int64_t p = j + 1; p < n; ++p) s -= x[p] * OPA(p, j);
                    x[j] = unit ? s : s / OPA(j, j);
                }
            } else {
                for (int64_t j = 0; j < n; ++j) {
                    qreal s = x[j];
                    for (int64_t p = 0; p < j; ++p) s -= x[p] * OPA(p, j);
                    x[j] = unit ? s : s / OPA(j, j);
                }
            }
            for (int64_t j = 0; j < n; ++j) B[i + j * ldb] = dd_of(x[j]);
            free(x);
        }
    }
    (void)na;
#undef OPA
}

/* GEMV in binary128 (kind16 qgemv_): y := alpha*op(A)*x + beta*y */
void or_qgemv(char trans, int64_t m, int64_t n, const dd *alpha, const dd *A, int64_t lda, const dd *x,
              int64_t incx, const dd *beta, dd *y, int64_t incy)
{
    if (m <= 0 || n <= 0) return;
    qreal al = q_of(*alpha), be = q_of(*beta);
    int beta0 = eq0(*beta);
    char t = (trans == 'N') ? 'N' : 'T';
    int64_t lenx = (t == 'N') ? n : m, leny = (t == 'N') ? m : n;
    int64_t kx = incx < 0 ? -(lenx - 1) * incx : 0;
    int64_t ky = incy < 0 ? -(leny - 1) * incy : 0;
#pragma omp parallel for schedule(static)
    for (int64_t r = 0; r < leny; ++r) {
        qreal acc = 0;
        for (int64_t c = 0; c < lenx; ++c) {
            qreal a = (t == 'N') ? q_of(A[r + c * lda]) : q_of(A[c + r * lda]);
            acc += a * q_of(x[kx + c * incx]);
        }
        dd *py = &y[ky + r * incy];
        qreal y0 = beta0 ? 0 : be * q_of(*py);
        *py = dd_of(al * acc + y0);
    }
}

/* DOT in binary128. Long vectors are summed in 64 contiguous slices in
 * parallel, the slice sums added in slice order (deterministic); the binary128
 * rounding of either order is far below the double-double tolerance. */
void or_qdot(int64_t n, const dd *x, int64_t incx, const dd *y, int64_t incy, dd *out)
{
    const int64_t ix0 = (incx < 0) ? (-n + 1) * incx : 0;
    const int64_t iy0 = (incy < 0) ? (-n + 1) * incy : 0;
    enum { SLICES = 64 };
    qreal part[SLICES];
    const int64_t ns = n >= (1 << 20) ? SLICES : 1;
#pragma omp parallel for schedule(dynamic, 1) if (ns > 1)
    for (int64_t s = 0; s < ns; ++s) {
        const int64_t i0 = n * s / ns, i1 = n * (s + 1) / ns;
        qreal acc = 0;
        int64_t ix = ix0 + i0 * incx, iy = iy0 + i0 * incy;
        for (int64_t i = i0; i < i1; ++i) {
            acc += q_of(x[ix]) * q_of(y[iy]);
            ix += incx;
            iy += incy;
        }
        part[s] = acc;
    }
    qreal acc = 0;
    for (int64_t s = 0; s < ns; ++s) acc += part[s];
    *out = dd_of(acc);
}

/* AXPY in binary128 (reference value for tolerance checks) */
void or_qaxpy(int64_t n, const dd *alpha, const dd *x, dd *y)
{
    qreal a = q_of(*alpha);
    for (int64_t i = 0; i < n; ++i) y[i] = dd_of(q_of(y[i]) + a * q_of(x[i]));
}

/* ====================== CPU-baseline ports ================================= */

/* mgemm_parallel.cpp:44-187 with the scalar micro-kernel of
 * mgemm_serial.cpp:85-99 (what the reference compiles to where its AVX2 path
 * is unavailable): beta pre-pass with the scalar operator*, then blocks
 * MC=64 / KC=128 / NC=256 (mgemm_serial.cpp:35-37), OpenMP over the jc loop,
 * and per block c(i,j) += (alpha*b(p,j)) * a(i,p) with the scalar operators.
 * When simd_order != 0 the accumulation instead follows the AVX2 path
 * (mgemm_serial.cpp:220-309): a fast-mul/fast-add DD accumulator per KC block,
 * alpha applied at writeback with the fast mul and merged with operator+. */
void or_port_mgemm(char ta, char tb, int64_t m, int64_t n, int64_t k, const dd *alpha, const dd *A, int64_t lda,
                   const dd *B, int64_t ldb, const dd *beta, dd *C, int64_t ldc, int simd_order)
{
    const int64_t MC = 64, KC = 128, NC = 256;
    dd al = *alpha, be = *beta;
    if (ta == 'C') ta = 'T';
    if (tb == 'C') tb = 'T';
    if (m <= 0 || n <= 0) return;
    for (int64_t j = 0; j < n; ++j) {
        dd *cj = C + j * ldc;
        if (eq0(be)) {
            for (int64_t i = 0; i < m; ++i) { cj[i].hi = 0.0; cj[i].lo = 0.0; }
        } else if (!eq1(be)) {
            for (int64_t i = 0; i < m; ++i) cj[i] = mul_exact(cj[i], be);
        }
    }
    if (eq0(al) || k == 0) return;
#pragma omp parallel
    {
        dd *Ap = (dd *)malloc(sizeof(dd) * (size_t)(MC * KC));
        dd *Bp = (dd *)malloc(sizeof(dd) * (size_t)(KC * NC));
#pragma omp for schedule(static)
        for (int64_t jc = 0; jc < n; jc += NC) {
            int64_t jb = (n - jc < NC) ? n - jc : NC;
            for (int64_t pc = 0; pc < k; pc += KC) {
                int64_t pb = (k - pc < KC) ? k - pc : KC;
                for (int64_t j = 0; j < jb; ++j)
                    for (int64_t p = 0; p < pb; ++p)
                        Bp[j * pb + p] = (tb == 'N') ? B[(pc + p) + (jc + j) * ldb] : B[(jc + j) + (pc + p) * ldb];
                for (int64_t ic = 0; ic < m; ic += MC) {
                    int64_t ib = (m - ic < MC) ? m - ic : MC;
                    for (int64_t p = 0; p < pb; ++p)
                        for (int64_t i = 0; i < ib; ++i)
                            Ap[p * ib + i] = (ta == 'N') ? A[(ic + i) + (pc + p) * lda] : A[(pc + p) + (ic + i) * lda];
                    for (int64_t j = 0; j < jb; ++j) {
                        dd *cj = C + (jc + j) * ldc + ic;
                        const dd *bj = Bp + j * pb;
                        if (!simd_order) {
                            for (int64_t p = 0; p < pb; ++p) {
                                dd t = mul_exact(al, bj[p]);
                                const dd *ap = Ap + p * ib;
                                for (int64_t i = 0; i < ib; ++i) cj[i] = add_exact(cj[i], mul_exact(t, ap[i]));
                            }
                        } else {
                            for (int64_t i = 0; i < ib; ++i) {
                                dd acc = {0.0, 0.0};
                                for (int64_t p = 0; p < pb; ++p) acc = add_fast(acc, mul_fast(Ap[p * ib + i], bj[p]));
                                cj[i] = add_exact(cj[i], mul_fast(al, acc));
                            }
                        }
                    }
                }
            }
        }
        free(Ap);
        free(Bp);
    }
}

/* mdot.cpp:48-87 (per-slice Bailey 3-limb accumulator, renormalised every 64
 * four-lane steps, xl*yl dropped) merged over slices in thread order
 * (mf_omp.h:186-202) -- the reference's unit-stride DOT, run with `team`
 * threads. */
static dd mdot_slice(int64_t n, const dd *x, const dd *y)
{
    double a0[4] = {0, 0, 0, 0}, a1[4] = {0, 0, 0, 0}, a2[4] = {0, 0, 0, 0};
    int64_t n4 = n & ~(int64_t)3;
    int counter = 64;
    for (int64_t i = 0; i < n4; i += 4) {
        for (int l = 0; l < 4; ++l) {
            double ph, pl;
            two_prod(x[i + l].hi, y[i + l].hi, &ph, &pl);
            pl = pl + (x[i + l].hi * y[i + l].lo + x[i + l].lo * y[i + l].hi);
            double e0, e1, e2;
            two_sum(a0[l], ph, &a0[l], &e0);
            two_sum(a1[l], pl, &a1[l], &e1);
            two_sum(a1[l], e0, &a1[l], &e2);
            a2[l] = a2[l] + (e1 + e2);
        }
        if (--counter == 0) {
            for (int l = 0; l < 4; ++l) {
                double t, e;
                fast_two_sum(a1[l], a2[l], &t, &e);
                a1[l] = t;
                a2[l] = e;
                fast_two_sum(a0[l], a1[l], &a0[l], &a1[l]);
                a1[l] = a1[l] + a2[l];
                fast_two_sum(a0[l], a1[l], &a0[l], &a1[l]);
                a2[l] = 0.0;
            }
            counter = 64;
        }
    }
    dd s = {a0[0], a1[0] + a2[0]};
    for (int l = 1; l < 4; ++l) {
        dd v = {a0[l], a1[l] + a2[l]};
        s = add_exact(s, v);
    }
    for (int64_t i = n4; i < n; ++i) s = add_exact(s, mul_exact(x[i], y[i]));
    return s;
}

void or_port_mdot(int64_t n, const dd *x, const dd *y, int64_t team, dd *out)
{
    if (team < 1) team = 1;
    if (team > 64) team = 64;
    dd part[64];
    for (int64_t t = 0; t < team; ++t) part[t].hi = part[t].lo = 0.0;
#pragma omp parallel for num_threads((int)team) schedule(static, 1)
    for (int64_t t = 0; t < team; ++t) {
        int64_t lo = part_bound(n, t, team), hi = part_bound(n, t + 1, team);
        if (lo < hi) part[t] = mdot_slice(hi - lo, x + lo, y + lo);
    }
    dd s = {0.0, 0.0};
    for (int64_t t = 0; t < team; ++t) s = add_exact(s, part[t]);
    *out = s;
}

int or_max_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* DD <-> binary128 conversion (for driving the reference's kind16 routines,
 * whose arrays are __float128). */
void or_dd_to_q(const dd *x, qreal *q, int64_t n)
{
    for (int64_t i = 0; i < n; ++i) q[i] = q_of(x[i]);
}
void or_q_to_dd(const qreal *q, dd *x, int64_t n)
{
    for (int64_t i = 0; i < n; ++i) x[i] = dd_of(q[i]);
}
