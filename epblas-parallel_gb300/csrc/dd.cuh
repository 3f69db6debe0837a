// Double-double arithmetic on the FP64 pipe of sm_103a.
//
// A double-double ("DD") value is an unevaluated sum hi + lo of two IEEE
// doubles with |lo| <= ulp(hi)/2. In memory it is 16 bytes {hi, lo}, which is
// layout-compatible with the reference's multifloats::float64x2 (two packed
// doubles, src/epblas-parallel/multifloats/mgemm_parallel.cpp:20-22) and with
// CUDA's double2 (x = hi, y = lo).
//
// Every primitive is written with the explicit round-to-nearest intrinsics
// __dadd_rn / __dsub_rn / __dmul_rn / __fma_rn, which nvcc never contracts or
// reassociates, so each line is exactly one IEEE operation. That is what makes
// the "bit-exact" routines (SCAL, AXPY) reproduce the reference's bits.
//
// Two operator families, mirroring the reference's split:
//   * fast   : the FMA-fused 1-ulp set of src/epblas-parallel/multifloats/
//              mf_simd_fast.h:49-102 (twoprod, twosum, fast2sum, mul, add).
//   * exact  : the set that mirrors the scalar float64x2 operators op for op,
//              mf_simd_exact.h:60-99 (cross products added, not fused).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace dd {

struct real { double hi, lo; };
struct cplx { real re, im; };

__host__ __device__ __forceinline__ real make(double h, double l) { real r; r.hi = h; r.lo = l; return r; }

__device__ __forceinline__ real load(const double2 *p)
{
    double2 v = *p;
    return make(v.x, v.y);
}
__device__ __forceinline__ void store(double2 *p, real v) { *p = make_double2(v.hi, v.lo); }

// ---- error-free transforms (mf_simd_fast.h:49-75) -------------------------

__device__ __forceinline__ void two_prod(double a, double b, double &p, double &e)
{
    p = __dmul_rn(a, b);
    e = __fma_rn(a, b, -p);
}

__device__ __forceinline__ void two_sum(double a, double b, double &s, double &e)
{
    s = __dadd_rn(a, b);
    double bb = __dsub_rn(s, a);
    double aa = __dsub_rn(s, bb);
    double da = __dsub_rn(a, aa);
    double db = __dsub_rn(b, bb);
    e = __dadd_rn(da, db);
}

// |a| >= |b| assumed.
__device__ __forceinline__ void fast_two_sum(double a, double b, double &s, double &e)
{
    s = __dadd_rn(a, b);
    double t = __dsub_rn(s, a);
    e = __dsub_rn(b, t);
}

// ---- fast set (mf_simd_fast.h:79-102) ------------------------------------
// Operand order matters for mul_fast: the cross terms are fused as
// fma(a.hi, b.lo, .) first, then fma(a.lo, b.hi, .), exactly as the reference.

__device__ __forceinline__ real mul_fast(real a, real b)
{
    double ph, pe;
    two_prod(a.hi, b.hi, ph, pe);
    pe = __fma_rn(a.hi, b.lo, pe);
    pe = __fma_rn(a.lo, b.hi, pe);
    real r;
    fast_two_sum(ph, pe, r.hi, r.lo);
    return r;
}

__device__ __forceinline__ real add_fast(real a, real b)
{
    double sh, se;
    two_sum(a.hi, b.hi, sh, se);
    double t = __dadd_rn(a.lo, b.lo);
    se = __dadd_rn(se, t);
    real r;
    fast_two_sum(sh, se, r.hi, r.lo);
    return r;
}

// ---- exact set: mirrors the scalar operators (mf_simd_exact.h:60-99) ------

__device__ __forceinline__ real mul_exact(real a, real b)
{
    double p00, e00;
    two_prod(a.hi, b.hi, p00, e00);
    double p01 = __dmul_rn(a.hi, b.lo);
    double p10 = __dmul_rn(a.lo, b.hi);
    p01 = __dadd_rn(p01, p10);
    e00 = __dadd_rn(e00, p01);
    real r;
    fast_two_sum(p00, e00, r.hi, r.lo);
    return r;
}

__device__ __forceinline__ real add_exact(real x, real y)
{
    double a, b, c, d;
    two_sum(x.hi, y.hi, a, b);
    two_sum(x.lo, y.lo, c, d);
    fast_two_sum(a, c, a, c);
    b = __dadd_rn(b, d);
    b = __dadd_rn(b, c);
    real r;
    fast_two_sum(a, b, r.hi, r.lo);
    return r;
}

__device__ __forceinline__ real neg(real a) { return make(-a.hi, -a.lo); }

__device__ __forceinline__ real sub_exact(real x, real y) { return add_exact(x, neg(y)); }
__device__ __forceinline__ real sub_fast(real x, real y) { return add_fast(x, neg(y)); }

// Double-double division a / b (Hida, Li, Bailey 2001, "accurate" DD
// division): three quotient digits from the hi limbs, the remainder
// recomputed in double-double after each.
__device__ __forceinline__ real div(real a, real b)
{
    double q1 = __ddiv_rn(a.hi, b.hi);
    real r = sub_exact(a, mul_exact(make(q1, 0.0), b));
    double q2 = __ddiv_rn(r.hi, b.hi);
    r = sub_exact(r, mul_exact(make(q2, 0.0), b));
    double q3 = __ddiv_rn(r.hi, b.hi);
    real q;
    fast_two_sum(q1, q2, q.hi, q.lo);
    return add_exact(q, make(q3, 0.0));
}

// Double-double square root (Karp and Markstein 1997: one correction of the
// FP64 root s by the exact residual, s + (v - s^2) / (2s)). v <= 0 gives 0
// (v == 0) or NaN.
__device__ __forceinline__ real sqrt(real v)
{
    if (v.hi <= 0.0) return make(v.hi == 0.0 ? 0.0 : __longlong_as_double(0x7ff8000000000000ll), 0.0);
    const double s = __dsqrt_rn(v.hi);
    double p, e;
    two_prod(s, s, p, e);
    const real r = sub_exact(v, make(p, e));
    const double t = __ddiv_rn(r.hi, __dmul_rn(2.0, s));
    real out;
    fast_two_sum(s, t, out.hi, out.lo);
    return out;
}

// ---- complex (mf_simd_fast.h:119-144 and mf_kernels.h:43-53) -------------

// fast complex multiply: re = a.re*b.re - a.im*b.im ; im = a.re*b.im + a.im*b.re
__device__ __forceinline__ cplx cmul_fast(cplx a, cplx b)
{
    cplx r;
    real p = mul_fast(a.re, b.re);
    real q = mul_fast(a.im, b.im);
    r.re = add_fast(p, neg(q));
    p = mul_fast(a.re, b.im);
    q = mul_fast(a.im, b.re);
    r.im = add_fast(p, q);
    return r;
}

// scalar-operator complex multiply (mf_kernels.h:43-45):
//   re = (a.re*b.re) - (a.im*b.im) ; im = (a.re*b.im) + (a.im*b.re)
__device__ __forceinline__ cplx cmul_exact(cplx a, cplx b)
{
    cplx r;
    r.re = sub_exact(mul_exact(a.re, b.re), mul_exact(a.im, b.im));
    r.im = add_exact(mul_exact(a.re, b.im), mul_exact(a.im, b.re));
    return r;
}

__device__ __forceinline__ cplx cadd_fast(cplx a, cplx b)
{
    cplx r;
    r.re = add_fast(a.re, b.re);
    r.im = add_fast(a.im, b.im);
    return r;
}

__device__ __forceinline__ cplx cadd_exact(cplx a, cplx b)
{
    cplx r;
    r.re = add_exact(a.re, b.re);
    r.im = add_exact(a.im, b.im);
    return r;
}

__device__ __forceinline__ cplx cload(const double2 *p)
{
    cplx r;
    r.re = load(p);
    r.im = load(p + 1);
    return r;
}
__device__ __forceinline__ void cstore(double2 *p, cplx v)
{
    store(p, v.re);
    store(p + 1, v.im);
}

// ---- predicates (mf_pred.h:28-63) -----------------------------------------

__device__ __forceinline__ bool gt(real a, real b)
{
    return a.hi > b.hi || (a.hi == b.hi && a.lo > b.lo);
}
__device__ __forceinline__ bool lt(real a, real b) { return gt(b, a); }
__device__ __forceinline__ bool eq0(real a) { return a.hi == 0.0 && a.lo == 0.0; }
__device__ __forceinline__ bool lt0(real a) { return a.hi < 0.0 || (a.hi == 0.0 && a.lo < 0.0); }
__device__ __forceinline__ bool gt0(real a) { return a.hi > 0.0 || (a.hi == 0.0 && a.lo > 0.0); }

// a < 0 ? -a : a with the limb-lexicographic sign (mf_pred.h:70).
__device__ __forceinline__ real absv(real a) { return lt0(a) ? neg(a) : a; }

// Branch-free magnitude used by the reference's vector argmax
// (imamax.cpp:60-72): (|hi|, lo with its sign flipped when hi is negative).
__device__ __forceinline__ real mag(real a)
{
    uint64_t hb = (uint64_t)__double_as_longlong(a.hi);
    uint64_t sign = hb & 0x8000000000000000ull;
    double h = __longlong_as_double((long long)(hb & 0x7fffffffffffffffull));
    double l = __longlong_as_double((long long)((uint64_t)__double_as_longlong(a.lo) ^ sign));
    return make(h, l);
}

}  // namespace dd
