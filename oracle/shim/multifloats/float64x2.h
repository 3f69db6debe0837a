/*
 * Clean-room stand-in for the third-party `multifloats` v0.8.1 scalar types.
 *
 * TEST INFRASTRUCTURE ONLY. This header exists so that the reference's own
 * double-double BLAS sources (src/epblas-parallel/multifloats/ *.cpp) can be
 * compiled unmodified on a machine without the upstream header, giving a
 * runnable copy of the reference for parity pinning and CPU timing. It is
 * never linked into the GPU library.
 *
 * What is pinned and what is not:
 *   - operator* and operator+ follow, op for op, the sequences the reference
 *     states are faithful to the upstream scalar operators:
 *       mul: src/epblas-parallel/multifloats/mf_simd_exact.h:60-73
 *            (two_prod of the hi limbs, the two cross products added without
 *             FMA fusion, then fast_two_sum)
 *       add: mf_simd_exact.h:75-88 (two_sum on both limbs, fast_two_sum,
 *            two adds, fast_two_sum)
 *       sub: mf_simd_exact.h:90-99 (add of the limb-negated operand)
 *   - The upstream operators short-circuit non-finite inputs and the
 *     both-hi-zero signed-zero case (mf_simd_exact.h:29-31). Those branches
 *     are not reproduced; results on such inputs are unpinned.
 *   - operator/ is not described anywhere in the reference. It is written here
 *     from the published "accurate" double-double division of Hida, Li and
 *     Bailey (2001, "Algorithms for quad-double precision floating point
 *     arithmetic"): three quotient digits, each from the hi limbs, with the
 *     remainder recomputed in double-double. Its last bits are therefore
 *     unpinned against upstream.
 *   - Comparisons are limb-lexicographic (hi first, lo on a hi tie), which is
 *     what the reference's own predicates assume (mf_pred.h:51-63).
 */
#pragma once

#include <cmath>

namespace multifloats {

struct float64x2 {
    double limbs[2];
};

struct complex64x2 {
    float64x2 re, im;
};

namespace shim_detail {

/* Keep these out of the compiler's contraction reach: the reference builds
 * with -ffp-contract=on, under which a*b+c may fuse. Each step below is one
 * rounding, written through volatile-free helpers with explicit fma where
 * the reference uses one. */
static inline void two_sum(double a, double b, double &s, double &e)
{
    s = a + b;
    double bb = s - a;
    double aa = s - bb;
    double da = a - aa;
    double db = b - bb;
    e = da + db;
}

static inline void fast_two_sum(double a, double b, double &s, double &e)
{
    s = a + b;
    double t = s - a;
    e = b - t;
}

static inline void two_prod(double a, double b, double &p, double &e)
{
    p = a * b;
    e = std::fma(a, b, -p);
}

}  // namespace shim_detail

static inline float64x2 operator-(const float64x2 &a)
{
    return float64x2{{-a.limbs[0], -a.limbs[1]}};
}

static inline float64x2 operator*(const float64x2 &a, const float64x2 &b)
{
    using namespace shim_detail;
    double p00, e00;
    two_prod(a.limbs[0], b.limbs[0], p00, e00);
    double p01 = a.limbs[0] * b.limbs[1];
    double p10 = a.limbs[1] * b.limbs[0];
    p01 = p01 + p10;
    e00 = e00 + p01;
    float64x2 r;
    fast_two_sum(p00, e00, r.limbs[0], r.limbs[1]);
    return r;
}

static inline float64x2 operator+(const float64x2 &x, const float64x2 &y)
{
    using namespace shim_detail;
    double a, b, c, d;
    two_sum(x.limbs[0], y.limbs[0], a, b);
    two_sum(x.limbs[1], y.limbs[1], c, d);
    fast_two_sum(a, c, a, c);
    b = b + d;
    b = b + c;
    float64x2 r;
    fast_two_sum(a, b, r.limbs[0], r.limbs[1]);
    return r;
}

static inline float64x2 operator-(const float64x2 &x, const float64x2 &y)
{
    return x + (-y);
}

static inline float64x2 operator/(const float64x2 &a, const float64x2 &b)
{
    using namespace shim_detail;
    /* q1: leading quotient digit; r = a - q1*b in double-double. */
    double q1 = a.limbs[0] / b.limbs[0];
    float64x2 r = a - float64x2{{q1, 0.0}} * b;
    double q2 = r.limbs[0] / b.limbs[0];
    r = r - float64x2{{q2, 0.0}} * b;
    double q3 = r.limbs[0] / b.limbs[0];
    float64x2 q;
    fast_two_sum(q1, q2, q.limbs[0], q.limbs[1]);
    return q + float64x2{{q3, 0.0}};
}

static inline float64x2 &operator+=(float64x2 &a, const float64x2 &b) { a = a + b; return a; }
static inline float64x2 &operator-=(float64x2 &a, const float64x2 &b) { a = a - b; return a; }
static inline float64x2 &operator*=(float64x2 &a, const float64x2 &b) { a = a * b; return a; }
static inline float64x2 &operator/=(float64x2 &a, const float64x2 &b) { a = a / b; return a; }

static inline bool operator==(const float64x2 &a, const float64x2 &b)
{
    return a.limbs[0] == b.limbs[0] && a.limbs[1] == b.limbs[1];
}
static inline bool operator!=(const float64x2 &a, const float64x2 &b) { return !(a == b); }
static inline bool operator<(const float64x2 &a, const float64x2 &b)
{
    return a.limbs[0] < b.limbs[0] || (a.limbs[0] == b.limbs[0] && a.limbs[1] < b.limbs[1]);
}
static inline bool operator>(const float64x2 &a, const float64x2 &b) { return b < a; }
static inline bool operator<=(const float64x2 &a, const float64x2 &b) { return !(b < a); }
static inline bool operator>=(const float64x2 &a, const float64x2 &b) { return !(a < b); }

/* Mixed comparisons against a plain number (the reference writes `a < 0`). */
static inline bool operator<(const float64x2 &a, double b) { return a < float64x2{{b, 0.0}}; }
static inline bool operator>(const float64x2 &a, double b) { return a > float64x2{{b, 0.0}}; }
static inline bool operator==(const float64x2 &a, double b) { return a == float64x2{{b, 0.0}}; }
static inline bool operator!=(const float64x2 &a, double b) { return a != float64x2{{b, 0.0}}; }

static inline float64x2 abs(const float64x2 &a) { return (a.limbs[0] < 0.0) ? -a : a; }

/* fabsdd / sqrtdd (used by the Givens generators mrotg.cpp, wrotg.cpp).
 * Neither is described in the reference. fabsdd is the limb-negating
 * magnitude above. sqrtdd is written from Karp and Markstein (1997, "High
 * precision division and square root"): the FP64 root s of the hi limb,
 * corrected once by the exactly formed residual, s + (v - s*s) / (2s).
 * Its last bits are therefore unpinned against upstream. */
static inline float64x2 fabsdd(const float64x2 &a) { return abs(a); }

static inline float64x2 sqrtdd(const float64x2 &v)
{
    using namespace shim_detail;
    if (v.limbs[0] <= 0.0) return float64x2{{v.limbs[0] == 0.0 ? 0.0 : std::nan(""), 0.0}};
    double s = std::sqrt(v.limbs[0]);
    double p, e;
    two_prod(s, s, p, e);
    float64x2 r = v - float64x2{{p, e}};
    double t = r.limbs[0] / (2.0 * s);
    float64x2 out;
    fast_two_sum(s, t, out.limbs[0], out.limbs[1]);
    return out;
}

}  // namespace multifloats
