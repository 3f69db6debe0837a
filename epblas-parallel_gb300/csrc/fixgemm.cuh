// Device helpers shared by the fixed-point GEMM kernels (gemm_fixed.cu and
// the grouped kernel in batched.cu): conversion of double-double entries to
// balanced 24-bit digits at a row/column scale, the digit multiply-add, and
// the epilogue from exact column sums to alpha*X + beta*C with one rounding.
#pragma once
#include "dd.cuh"
#include "fixacc.cuh"
#include "xfloat.cuh"

namespace mw {
namespace fxg {

using xfp::XF;
using fx::add_shifted;
using fx::w256_to_xf;

// Scaled operands are integers below 2^(FX_S + 1).
constexpr int FX_S = 115;

// v * 2^sh rounded to an integer (|v * 2^sh| < 2^116), as five balanced
// 24-bit digits; bit operations only (fixacc.cuh's decode).
__device__ __forceinline__ void dd_digits(double2 v, int sh, int d[5])
{
#pragma unroll
    for (int t = 0; t < 5; ++t) d[t] = 0;
    const fx::Op o = fx::decode(v);
    if (o.flags & (fx::kZero | fx::kBad)) return;   // non-finite rows are handled by the epilogue
    const int r = -(o.e + sh);   // N = W * 2^-r; r >= 2 for in-range values
    if (r >= 118 || r < 1) return;
    uint32_t y[4], h[4];
    fx::shr128(o.w, r, y);
    fx::shr128(o.w, r - 1, h);   // rounding bit
    const uint32_t rb = h[0] & 1u;
    asm("add.cc.u32 %0, %0, %4;\n\t"
        "addc.cc.u32 %1, %1, 0;\n\t"
        "addc.cc.u32 %2, %2, 0;\n\t"
        "addc.u32 %3, %3, 0;"
        : "+r"(y[0]), "+r"(y[1]), "+r"(y[2]), "+r"(y[3])
        : "r"(rb));
    int u[5];
    fx::digits24(y, u);
    // balanced digits: |d| <= 2^23
#pragma unroll
    for (int t = 0; t < 4; ++t) {
        if (u[t] >= 0x800000) {
            u[t] -= 0x1000000;
            u[t + 1] += 1;
        }
        d[t] = u[t];
    }
    d[4] = u[4];
    if (o.flags & fx::kNeg) {
#pragma unroll
        for (int t = 0; t < 5; ++t) d[t] = -d[t];
    }
}

__device__ __forceinline__ dd::real xf_to_real(const XF &x)
{
    dd::real r;
    xfp::xf_to_dd(x, r.hi, r.lo);
    return r;
}

// C := alpha*X + beta*C with one rounding (non-finite C through the DD operators).
__device__ __forceinline__ void store_axpby(double2 *pc, XF v, const XF &xa, bool alpha_one, const XF &xb,
                                            dd::real beta, int beta_kind)
{
    if (!alpha_one) v = xfp::xf_mul(xa, v);
    if (beta_kind != 0) {
        const double2 c0 = *pc;
        if (!isfinite(c0.x)) {
            dd::real cv = dd::make(c0.x, c0.y);
            if (beta_kind == 2) cv = dd::mul_exact(cv, beta);
            dd::store(pc, dd::add_exact(cv, xf_to_real(v)));
            return;
        }
        XF xc = xfp::xf_from_dd(c0.x, c0.y);
        if (beta_kind == 2) xc = xfp::xf_mul(xb, xc);
        v = xfp::xf_add(v, xc);
    }
    dd::store(pc, xf_to_real(v));
}

// Column sums of one output: acc[w] += sum of digit products of weight 2^(24(w+4)).
__device__ __forceinline__ void mac_digits(long long acc[5], const int a[5], const int b[5])
{
    acc[0] += (long long)a[0] * b[4] + (long long)a[1] * b[3] + (long long)a[2] * b[2] + (long long)a[3] * b[1] +
              (long long)a[4] * b[0];
    acc[1] += (long long)a[1] * b[4] + (long long)a[2] * b[3] + (long long)a[3] * b[2] + (long long)a[4] * b[1];
    acc[2] += (long long)a[2] * b[4] + (long long)a[3] * b[3] + (long long)a[4] * b[2];
    acc[3] += (long long)a[3] * b[4] + (long long)a[4] * b[3];
    acc[4] += (long long)a[4] * b[4];
}

// The column sums as an extended float: X = sum_w acc[w] 2^(24(w+4)) * 2^(ea + eb - 2 FX_S).
__device__ __forceinline__ XF sums_to_xf(const long long acc[5], int ea, int eb)
{
    uint64_t W[4] = {0, 0, 0, 0};
#pragma unroll
    for (int w = 0; w < 5; ++w) add_shifted(W, acc[w], 24 * w);
    return w256_to_xf(W, 96 + ea + eb - 2 * FX_S);
}

}  // namespace fxg
}  // namespace mw
