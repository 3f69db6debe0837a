// The remaining level-1 vector routines of the multifloats overlay:
//
//   wdotu / wdotc   sum x_i*y_i, sum conj(x_i)*y_i (complex)   (wdotu.cpp, wdotc.cpp)
//   masum / mwasum  sum |x_i|, sum |Re x_i| + |Im x_i|          (masum.cpp, mwasum.cpp)
//   mnrm2 / mwnrm2  sqrt(sum |x_i|^2)                           (mnrm2.cpp, mwnrm2.cpp)
//   waxpy           y += alpha*x (complex)                      (waxpy.cpp)
//   mrot / wmrot    (x, y) := (c*x + s*y, c*y - s*x), real c, s (mrot.cpp, wmrot.cpp)
//   mrotm           (x, y) := H (x, y) for the modified-Givens H of dparam (mrotm.cpp)
//
// The reductions accumulate in the integer fixed point of fixacc.cuh (exact
// products to 2^-126, thread sums combined as extended floats in a fixed
// order, one final rounding), like DOT: deterministic and at least as
// accurate as the reference's double-double accumulators. The norms take
// the square root of the exact sum of squares after moving an even power of
// two out of it, so no intermediate overflows or underflows. The updates are
// elementwise double-double arithmetic.
#include "dd.cuh"
#include "fixacc.cuh"
#include "l1x.h"
#include "runtime.h"

namespace mw {

namespace {

constexpr int kThreads = 256;

__device__ __forceinline__ int64_t vix(int64_t i, int64_t n, int64_t inc)
{
    return inc >= 0 ? i * inc : (n - 1 - i) * (-inc);
}

int grid_for(int64_t n)
{
    int64_t blocks = (n + kThreads - 1) / kThreads;
    int64_t cap = (int64_t)device_sm_count() * 8;
    if (blocks > cap) blocks = cap;
    if (blocks < 1) blocks = 1;
    return (int)blocks;
}

__device__ fx::XF block_sum(fx::XF v)
{
    __shared__ fx::XFPod sh[kThreads / 32];
    v = fx::xf_warp_sum(v);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) sh[wid] = fx::to_pod(v, false);
    __syncthreads();
    if (wid == 0) {
        if (lane < (int)(blockDim.x >> 5)) {
            v = fx::from_pod(sh[lane]);
        } else {
            v.zero = true; v.neg = false; v.m = 0; v.e = 0;
        }
        v = fx::xf_warp_sum(v);
    }
    return v;
}

__device__ __forceinline__ fx::Op negate(fx::Op o)
{
    o.flags ^= fx::kNeg;
    return o;
}

__device__ __forceinline__ fx::Op absval(fx::Op o)
{
    o.flags &= ~fx::kNeg;
    return o;
}

// One (or two, for the complex products) fixed-point sums per thread over
// the elements, folded into extended floats every kMaxAdds terms.
//   mode 0: dotu  (re: xr*yr - xi*yi, im: xr*yi + xi*yr)
//   mode 1: dotc  (re: xr*yr + xi*yi, im: xr*yi - xi*yr)
//   mode 2: asum of a real x       3: |xr| + |xi| of a complex x
//   mode 4: sum x^2 of a real x    5: xr^2 + xi^2 of a complex x
template <int MODE>
__global__ void __launch_bounds__(kThreads) k_reduce(int64_t n, const double2 *__restrict__ x, int64_t incx,
                                                    const double2 *__restrict__ y, int64_t incy, fx::XFPod *part)
{
    constexpr bool CX = MODE != 2 && MODE != 4;   // complex elements
    constexpr bool TWO = MODE <= 1;                // two sums (re, im)
    fx::Acc acc[TWO ? 2 : 1];
    fx::XF total[TWO ? 2 : 1];
    for (int r = 0; r < (TWO ? 2 : 1); ++r) {
        acc[r].reset();
        total[r].zero = true; total[r].neg = false; total[r].m = 0; total[r].e = 0;
    }
    bool bad = false;
    int cnt = 0;
    const fx::Op one = fx::decode(make_double2(1.0, 0.0));
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += stride) {
        const double2 *px = x + (CX ? 2 : 1) * vix(i, n, incx);
        const fx::Op xr = fx::decode(__ldcs(px));
        if (MODE <= 1) {
            const fx::Op xi = fx::decode(__ldcs(px + 1));
            const double2 *py = y + 2 * vix(i, n, incy);
            const fx::Op yr = fx::decode(__ldcs(py)), yi = fx::decode(__ldcs(py + 1));
            acc[0].add_prod(xr, yr);
            acc[0].add_prod(MODE == 0 ? negate(xi) : xi, yi);
            acc[1].add_prod(xr, yi);
            acc[1].add_prod(MODE == 0 ? xi : negate(xi), yr);
        } else if (MODE == 2) {
            acc[0].add_prod(absval(xr), one);
        } else if (MODE == 3) {
            acc[0].add_prod(absval(xr), one);
            acc[0].add_prod(absval(fx::decode(__ldcs(px + 1))), one);
        } else if (MODE == 4) {
            acc[0].add_prod(xr, xr);
        } else {
            const fx::Op xi = fx::decode(__ldcs(px + 1));
            acc[0].add_prod(xr, xr);
            acc[0].add_prod(xi, xi);
        }
        if ((cnt += (CX ? 2 : 1)) >= fx::kMaxAdds - 2) {
            for (int r = 0; r < (TWO ? 2 : 1); ++r) {
                bad |= acc[r].bad;
                total[r] = xfp::xf_add(total[r], acc[r].finish());
                acc[r].reset();
            }
            cnt = 0;
        }
    }
    for (int r = 0; r < (TWO ? 2 : 1); ++r) {
        bad |= acc[r].bad;
        total[r] = xfp::xf_add(total[r], acc[r].finish());
    }
    bad = __syncthreads_or(bad ? 1 : 0) != 0;
    for (int r = 0; r < (TWO ? 2 : 1); ++r) {
        const fx::XF v = block_sum(total[r]);
        if (threadIdx.x == 0) part[r * gridDim.x + blockIdx.x] = fx::to_pod(v, bad);
    }
}

// Double-double square root of v * 2^(2k): sqrt(hi) refined by one Newton
// step in double-double, then scaled by 2^k.
__device__ dd::real dd_sqrt_scaled(dd::real v, int k)
{
    const dd::real out = dd::sqrt(v);
    const double f = ldexp(1.0, k);
    return dd::make(out.hi * f, out.lo * f);
}

// Sum of the block partials; out[0..1] = the result (mode 0/1: re, im; 2, 3:
// the sum; 4, 5: its square root).
template <int MODE>
__global__ void __launch_bounds__(kThreads) k_reduce_final(int nparts, const fx::XFPod *part, double2 *out)
{
    constexpr int NR = MODE <= 1 ? 2 : 1;
    for (int r = 0; r < NR; ++r) {
        fx::XF acc;
        acc.zero = true; acc.neg = false; acc.m = 0; acc.e = 0;
        bool bad = false;
        for (int i = threadIdx.x; i < nparts; i += blockDim.x) {
            const fx::XFPod p = part[r * nparts + i];
            bad |= (p.flags & 4) != 0;
            acc = xfp::xf_add(acc, fx::from_pod(p));
        }
        bad = __syncthreads_or(bad ? 1 : 0) != 0;
        acc = block_sum(acc);
        if (threadIdx.x == 0) {
            double h, l;
            if (MODE >= 4 && !acc.zero) {
                // acc = m * 2^e: take 2^(2k) out so the double-double lies near 1
                const int k = (acc.e + 127) >> 1;
                acc.e -= 2 * k;
                xfp::xf_to_dd(acc, h, l);
                const dd::real s = dd_sqrt_scaled(dd::make(h, l), k);
                h = s.hi;
                l = s.lo;
            } else {
                xfp::xf_to_dd(acc, h, l);
            }
            if (bad) h = l = __longlong_as_double(0x7ff8000000000000ll);
            out[r] = make_double2(h, l);
        }
        __syncthreads();
    }
}

// y += alpha * x, complex, elementwise (scalar-operator multiply and add).
__global__ void k_waxpy(int64_t n, dd::cplx alpha, const double2 *__restrict__ x, int64_t incx, double2 *y,
                        int64_t incy)
{
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += stride) {
        double2 *py = y + 2 * vix(i, n, incy);
        const dd::cplx xv = dd::cload(x + 2 * vix(i, n, incx));
        dd::cstore(py, dd::cadd_exact(dd::cload(py), dd::cmul_exact(alpha, xv)));
    }
}

// (x, y) := (h11*x + h12*y, h21*x + h22*y) with real h, elementwise on each
// of `e2` components (1 real, 2 complex). Rotation: h = (c, s, -s, c).
__global__ void k_rot(int64_t n, double2 *x, int64_t incx, double2 *y, int64_t incy, int e2, dd::real h11,
                      dd::real h12, dd::real h21, dd::real h22)
{
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += stride) {
        double2 *px = x + e2 * vix(i, n, incx), *py = y + e2 * vix(i, n, incy);
        for (int w = 0; w < e2; ++w) {
            const dd::real a = dd::load(px + w), b = dd::load(py + w);
            const dd::real u = dd::add_exact(dd::mul_exact(h11, a), dd::mul_exact(h12, b));
            const dd::real v = dd::add_exact(dd::mul_exact(h21, a), dd::mul_exact(h22, b));
            dd::store(px + w, u);
            dd::store(py + w, v);
        }
    }
}

// ---- scalar generators: one thread, scalar-operator double-double arithmetic ----------
// out->v holds the results in the order documented at launch_generator; bit i
// of out->mask says whether result i is written back (the reference leaves
// the others untouched).

__device__ __forceinline__ void gput(GenResult *out, int i, dd::real v)
{
    out->v[i] = make_double2(v.hi, v.lo);
    out->mask |= 1u << i;
}

// mcabs1.cpp:20-24: |Re z| + |Im z|.
__device__ void gen_cabs1(const double2 *in, GenResult *out)
{
    gput(out, 0, dd::add_exact(dd::absv(dd::load(in)), dd::absv(dd::load(in + 1))));
}

// mrotg.cpp:21-34: (a, b) -> (r, z), c, s with [c s; -s c](a; b) = (r; 0),
// r = sign(a) sqrt(a^2 + b^2), z = s when |a| > |b| else 1/c.
// Results: 0 a, 1 b, 2 c, 3 s.
__device__ void gen_rotg(const double2 *in, GenResult *out)
{
    const dd::real zero = dd::make(0.0, 0.0), one = dd::make(1.0, 0.0);
    const dd::real a = dd::load(in), b = dd::load(in + 1);
    const dd::real an = dd::absv(a), bn = dd::absv(b);
    if (dd::eq0(bn)) {
        gput(out, 2, one);
        gput(out, 3, zero);
        gput(out, 1, zero);
        return;
    }
    if (dd::eq0(an)) {
        gput(out, 2, zero);
        gput(out, 3, one);
        gput(out, 0, b);
        gput(out, 1, one);
        return;
    }
    dd::real r = dd::sqrt(dd::add_exact(dd::mul_exact(an, an), dd::mul_exact(bn, bn)));
    if (dd::lt(a, zero)) r = dd::neg(r);
    const dd::real c = dd::div(a, r), s = dd::div(b, r);
    gput(out, 2, c);
    gput(out, 3, s);
    gput(out, 0, r);
    gput(out, 1, dd::gt(an, bn) ? s : dd::div(one, c));
}

// mrotmg.cpp:25-106 (the DROTMG algorithm): modified Givens for
// (sqrt(d1) x1, sqrt(d2) y1). Inputs d1, d2, x1, y1. Results: 0 d1, 1 d2,
// 2 x1, 3..7 dparam(1..5).
__device__ void gen_rotmg(const double2 *in, GenResult *out)
{
    const dd::real zero = dd::make(0.0, 0.0), one = dd::make(1.0, 0.0), mone = dd::make(-1.0, 0.0);
    const dd::real gam = dd::make(4096.0, 0.0), gamsq = dd::make(16777216.0, 0.0);
    const dd::real rgamsq = dd::make(5.9604645e-8, 0.0);   // the reference's literal, not 2^-24
    dd::real d1 = dd::load(in), d2 = dd::load(in + 1), x1 = dd::load(in + 2);
    const dd::real y1 = dd::load(in + 3);
    dd::real flag, h11 = zero, h12 = zero, h21 = zero, h22 = zero;
    if (dd::lt0(d1)) {
        flag = mone;
        d1 = d2 = x1 = zero;
    } else {
        const dd::real p2 = dd::mul_exact(d2, y1);
        if (dd::eq0(p2)) {
            gput(out, 3, dd::make(-2.0, 0.0));
            return;
        }
        const dd::real p1 = dd::mul_exact(d1, x1);
        const dd::real q2 = dd::mul_exact(p2, y1);
        const dd::real q1 = dd::mul_exact(p1, x1);
        if (dd::gt(dd::absv(q1), dd::absv(q2))) {
            h21 = dd::div(dd::neg(y1), x1);
            h12 = dd::div(p2, p1);
            const dd::real u = dd::sub_exact(one, dd::mul_exact(h12, h21));
            if (dd::gt0(u)) {
                flag = zero;
                d1 = dd::div(d1, u);
                d2 = dd::div(d2, u);
                x1 = dd::mul_exact(x1, u);
            } else {
                flag = mone;
                h11 = h12 = h21 = h22 = zero;
                d1 = d2 = x1 = zero;
            }
        } else if (dd::lt0(q2)) {
            flag = mone;
            h11 = h12 = h21 = h22 = zero;
            d1 = d2 = x1 = zero;
        } else {
            flag = one;
            h11 = dd::div(p1, p2);
            h22 = dd::div(x1, y1);
            const dd::real u = dd::add_exact(one, dd::mul_exact(h11, h22));
            const dd::real t = dd::div(d2, u);
            d2 = dd::div(d1, u);
            d1 = t;
            x1 = dd::mul_exact(y1, u);
        }
        // Rescale by gam = 2^12 until rgamsq < d < gamsq. Each pass moves the
        // exponent by 24, so a finite d leaves the loop within 90 passes; the
        // cap only guards non-finite values.
        if (!dd::eq0(d1)) {
            for (int it = 0; it < 200 && (!dd::gt(d1, rgamsq) || !dd::lt(d1, gamsq)); ++it) {
                if (dd::eq0(flag)) {
                    h11 = one;
                    h22 = one;
                } else {
                    h21 = mone;
                    h12 = one;
                }
                flag = mone;
                if (!dd::gt(d1, rgamsq)) {
                    d1 = dd::mul_exact(dd::mul_exact(d1, gam), gam);
                    x1 = dd::div(x1, gam);
                    h11 = dd::div(h11, gam);
                    h12 = dd::div(h12, gam);
                } else {
                    d1 = dd::div(d1, dd::mul_exact(gam, gam));
                    x1 = dd::mul_exact(x1, gam);
                    h11 = dd::mul_exact(h11, gam);
                    h12 = dd::mul_exact(h12, gam);
                }
            }
        }
        if (!dd::eq0(d2)) {
            dd::real ad2 = dd::absv(d2);
            for (int it = 0; it < 200 && (!dd::gt(ad2, rgamsq) || !dd::lt(ad2, gamsq)); ++it) {
                if (dd::eq0(flag)) {
                    h11 = one;
                    h22 = one;
                } else {
                    h21 = mone;
                    h12 = one;
                }
                flag = mone;
                if (!dd::gt(ad2, rgamsq)) {
                    d2 = dd::mul_exact(dd::mul_exact(d2, gam), gam);
                    h21 = dd::div(h21, gam);
                    h22 = dd::div(h22, gam);
                } else {
                    d2 = dd::div(d2, dd::mul_exact(gam, gam));
                    h21 = dd::mul_exact(h21, gam);
                    h22 = dd::mul_exact(h22, gam);
                }
                ad2 = dd::absv(d2);
            }
        }
    }
    gput(out, 3, flag);
    if (dd::lt0(flag)) {
        gput(out, 4, h11);
        gput(out, 5, h21);
        gput(out, 6, h12);
        gput(out, 7, h22);
    } else if (dd::eq0(flag)) {
        gput(out, 6, h12);
        gput(out, 5, h21);
    } else {
        gput(out, 4, h11);
        gput(out, 7, h22);
    }
    gput(out, 0, d1);
    gput(out, 1, d2);
    gput(out, 2, x1);
}

// wrotg.cpp:27-48 (ZROTG analogue): c = |a|/sqrt(|a|^2+|b|^2),
// s = conj(b) a / sqrt(|a|^2 (|a|^2+|b|^2)), a := a/c. Inputs a, b (complex).
// Results: 0/1 a (re, im), 2 c, 3/4 s (re, im).
__device__ void gen_wrotg(const double2 *in, GenResult *out)
{
    const dd::real zero = dd::make(0.0, 0.0);
    const dd::cplx a = dd::cload(in), b = dd::cload(in + 2);
    const dd::real g2 = dd::add_exact(dd::mul_exact(b.re, b.re), dd::mul_exact(b.im, b.im));
    if (dd::eq0(g2)) {
        gput(out, 2, dd::make(1.0, 0.0));
        gput(out, 3, zero);
        gput(out, 4, zero);
        return;
    }
    const dd::real f2 = dd::add_exact(dd::mul_exact(a.re, a.re), dd::mul_exact(a.im, a.im));
    if (dd::eq0(f2)) {
        gput(out, 2, zero);
        const dd::real d = dd::sqrt(g2);
        gput(out, 3, dd::div(b.re, d));
        gput(out, 4, dd::div(dd::neg(b.im), d));
        gput(out, 0, d);
        gput(out, 1, zero);
        return;
    }
    const dd::real h2 = dd::add_exact(f2, g2);
    const dd::real c = dd::sqrt(dd::div(f2, h2));
    gput(out, 2, c);
    gput(out, 0, dd::div(a.re, c));
    gput(out, 1, dd::div(a.im, c));
    const dd::real d = dd::sqrt(dd::mul_exact(f2, h2));
    dd::cplx bc;
    bc.re = b.re;
    bc.im = dd::neg(b.im);
    const dd::cplx p = dd::cmul_exact(bc, a);
    gput(out, 3, dd::div(p.re, d));
    gput(out, 4, dd::div(p.im, d));
}

__global__ void k_generator(int op, GenInput in, GenResult *out)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    out->mask = 0;
    switch (op) {
    case GEN_CABS1: gen_cabs1(in.v, out); break;
    case GEN_ROTG: gen_rotg(in.v, out); break;
    case GEN_ROTMG: gen_rotmg(in.v, out); break;
    default: gen_wrotg(in.v, out); break;
    }
}

}  // namespace

bool launch_generator(int op, const GenInput &in, GenResult *result_host, const char *routine)
{
    GenResult *d = (GenResult *)dev_alloc(sizeof(GenResult), routine);
    if (!d) return false;
    k_generator<<<1, 32, 0, stream()>>>(op, in, d);
    count_launch();
    bool ok = cuda_ok(cudaMemcpyAsync(result_host, d, sizeof(GenResult), cudaMemcpyDeviceToHost, stream()), routine,
                      "generator result readback");
    ok = ok && cuda_ok(cudaStreamSynchronize(stream()), routine, "generator sync");
    dev_free(d);
    return ok;
}

bool launch_reduce(int mode, int64_t n, const void *x, int64_t incx, const void *y, int64_t incy,
                   double2 *result_host, const char *routine)
{
    const int g = grid_for(n);
    const int nr = mode <= 1 ? 2 : 1;
    const size_t pbytes = (size_t)nr * g * sizeof(fx::XFPod);
    char *buf = (char *)dev_alloc(pbytes + 256, routine);
    if (!buf) return false;
    fx::XFPod *part = (fx::XFPod *)buf;
    double2 *res = (double2 *)(buf + (pbytes + 15) / 16 * 16);
    const double2 *xd = (const double2 *)x, *yd = (const double2 *)y;
    switch (mode) {
    case 0: k_reduce<0><<<g, kThreads, 0, stream()>>>(n, xd, incx, yd, incy, part);
            k_reduce_final<0><<<1, kThreads, 0, stream()>>>(g, part, res); break;
    case 1: k_reduce<1><<<g, kThreads, 0, stream()>>>(n, xd, incx, yd, incy, part);
            k_reduce_final<1><<<1, kThreads, 0, stream()>>>(g, part, res); break;
    case 2: k_reduce<2><<<g, kThreads, 0, stream()>>>(n, xd, incx, yd, incy, part);
            k_reduce_final<2><<<1, kThreads, 0, stream()>>>(g, part, res); break;
    case 3: k_reduce<3><<<g, kThreads, 0, stream()>>>(n, xd, incx, yd, incy, part);
            k_reduce_final<3><<<1, kThreads, 0, stream()>>>(g, part, res); break;
    case 4: k_reduce<4><<<g, kThreads, 0, stream()>>>(n, xd, incx, yd, incy, part);
            k_reduce_final<4><<<1, kThreads, 0, stream()>>>(g, part, res); break;
    default: k_reduce<5><<<g, kThreads, 0, stream()>>>(n, xd, incx, yd, incy, part);
             k_reduce_final<5><<<1, kThreads, 0, stream()>>>(g, part, res); break;
    }
    count_launch(2);
    bool ok = cuda_ok(cudaMemcpyAsync(result_host, res, nr * sizeof(double2), cudaMemcpyDeviceToHost, stream()),
                      routine, "reduction result readback");
    dev_free(buf);
    if (!ok) return false;
    return cuda_ok(cudaStreamSynchronize(stream()), routine, "reduction sync");
}

void launch_waxpy(int64_t n, cdd_host alpha, const void *x, int64_t incx, void *y, int64_t incy)
{
    dd::cplx a;
    a.re = dd::make(alpha.re.hi, alpha.re.lo);
    a.im = dd::make(alpha.im.hi, alpha.im.lo);
    const bool seq = incy == 0;   // every update hits the same element: keep the order
    k_waxpy<<<seq ? 1 : grid_for(n), seq ? 1 : kThreads, 0, stream()>>>(n, a, (const double2 *)x, incx, (double2 *)y,
                                                                     incy);
    count_launch();
}

void launch_rot(int64_t n, void *x, int64_t incx, void *y, int64_t incy, int e2, const dd_host h[4])
{
    const bool seq = incx == 0 || incy == 0;
    k_rot<<<seq ? 1 : grid_for(n), seq ? 1 : kThreads, 0, stream()>>>(
        n, (double2 *)x, incx, (double2 *)y, incy, e2, dd::make(h[0].hi, h[0].lo), dd::make(h[1].hi, h[1].lo),
        dd::make(h[2].hi, h[2].lo), dd::make(h[3].hi, h[3].lo));
    count_launch();
}

}  // namespace mw
