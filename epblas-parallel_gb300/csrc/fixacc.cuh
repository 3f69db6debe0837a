// Integer fixed-point accumulation of double-double products, for the
// bandwidth-bound reductions (DOT, GEMV).
//
// On this part an FP64 instruction issues at ~1/40 of the integer rate, so a
// double-double multiply-add on the FP64 pipe (12 instructions) cannot keep
// up with HBM. Here each product is formed exactly enough in integers: both
// operands become 128-bit mantissas (the exact image of hi + lo), their
// product keeps its top 128 bits (relative truncation < 2^-126), and it is
// added, shifted to a per-thread block exponent, into a 192-bit two's
// complement accumulator. The accumulator keeps 2^-160 of its leading product
// below the binary point; when a product arrives that would not fit under the
// 32-bit headroom, the accumulator moves to a higher exponent (a right shift,
// rare after the first few terms). Sums of these accumulators (warp, block,
// grid) use the 128-bit extended-float addition, in a fixed order.
//
// Non-finite inputs make the double-double operators of the reference return
// NaN (the TwoProduct error term of an infinity is inf - inf); the
// accumulator records them and the result is NaN.
#pragma once
#include "xfloat.cuh"

namespace fx {

using xfp::XF;

constexpr int kHead = 32;    // headroom bits above the largest product so far
constexpr int kSlack = 12;   // extra room left when the exponent moves up

struct Acc {
    uint64_t w0, w1, w2;   // value = W * 2^lsb, W two's complement
    int lsb;
    bool init;
    bool bad;

    __device__ __forceinline__ void reset()
    {
        w0 = w1 = w2 = 0;
        lsb = 0;
        init = false;
        bad = false;
    }

    __device__ __forceinline__ void shift_right(int d)
    {
        // arithmetic shift of the 192-bit W by d >= 1
        const uint64_t sgn = (uint64_t)((int64_t)w2 >> 63);
        if (d >= 192) {
            w0 = w1 = w2 = 0;   // all previous terms are below the new resolution
            return;
        }
        while (d >= 64) {
            w0 = w1;
            w1 = w2;
            w2 = sgn;
            d -= 64;
        }
        if (d) {
            w0 = (w0 >> d) | (w1 << (64 - d));
            w1 = (w1 >> d) | (w2 << (64 - d));
            w2 = (uint64_t)((int64_t)w2 >> d);
        }
    }

    // W += (neg ? -1 : 1) * m * 2^e
    __device__ __forceinline__ void add(const XF &p)
    {
        if (p.zero) return;
        const int need = p.e + 128 + kHead - 191;   // smallest lsb that keeps the headroom
        if (!init) {
            lsb = need + kSlack;
            init = true;
        } else if (need > lsb) {
            const int nl = need + kSlack;
            shift_right(nl - lsb);
            lsb = nl;
        }
        const int sh = p.e - lsb;   // position of m's bit 0; <= 63 - kHead
        const uint64_t m1 = (uint64_t)(p.m >> 64), m0 = (uint64_t)p.m;
        uint64_t v0, v1, v2;
        if (sh >= 0) {
            v0 = m0 << sh;
            v1 = sh ? ((m1 << sh) | (m0 >> (64 - sh))) : m1;
            v2 = sh ? (m1 >> (64 - sh)) : 0;
        } else {
            const int r = -sh;
            if (r >= 128) return;
            if (r >= 64) {
                v0 = m1 >> (r - 64);
                v1 = 0;
            } else {
                v0 = r ? ((m0 >> r) | (m1 << (64 - r))) : m0;
                v1 = m1 >> r;
            }
            v2 = 0;
        }
        if (p.neg) {
            asm("sub.cc.u64 %0, %0, %3;\n\t"
                "subc.cc.u64 %1, %1, %4;\n\t"
                "subc.u64 %2, %2, %5;"
                : "+l"(w0), "+l"(w1), "+l"(w2)
                : "l"(v0), "l"(v1), "l"(v2));
        } else {
            asm("add.cc.u64 %0, %0, %3;\n\t"
                "addc.cc.u64 %1, %1, %4;\n\t"
                "addc.u64 %2, %2, %5;"
                : "+l"(w0), "+l"(w1), "+l"(w2)
                : "l"(v0), "l"(v1), "l"(v2));
        }
    }

    // double-double product a * b, both finite, added exactly to 2^-126
    __device__ __forceinline__ void add_dd_product(double ah, double al, double bh, double bl)
    {
        if (ah == 0.0 || bh == 0.0) return;
        add(xfp::xf_mul(xfp::xf_from_dd(ah, al), xfp::xf_from_dd(bh, bl)));
    }

    __device__ __forceinline__ XF finish() const
    {
        XF r;
        r.neg = false;
        r.zero = true;
        r.m = 0;
        r.e = 0;
        if (!init) return r;
        uint64_t a0 = w0, a1 = w1, a2 = w2;
        const bool neg = (int64_t)a2 < 0;
        if (neg) {
            asm("sub.cc.u64 %0, 0, %0;\n\t"
                "subc.cc.u64 %1, 0, %1;\n\t"
                "subc.u64 %2, 0, %2;"
                : "+l"(a0), "+l"(a1), "+l"(a2));
        }
        // top 128 bits of the 192-bit magnitude
        unsigned __int128 m;
        int e;
        if (a2) {
            const int z = xfp::clz64(a2);
            m = ((unsigned __int128)a2 << 64) | a1;
            if (z) m = (m << z) | (a0 >> (64 - z));
            e = lsb + 64 - z;
        } else if (a1) {
            m = ((unsigned __int128)a1 << 64) | a0;
            e = lsb;
        } else if (a0) {
            m = a0;
            e = lsb;
        } else {
            return r;
        }
        return xfp::xf_norm(neg, m, e);
    }
};

// Extended-float warp reduction (lane 0 holds the sum; fixed order).
__device__ __forceinline__ XF xf_shfl_down(const XF &v, int off)
{
    XF r;
    const uint64_t hi = __shfl_down_sync(0xffffffffu, (unsigned long long)(v.m >> 64), off);
    const uint64_t lo = __shfl_down_sync(0xffffffffu, (unsigned long long)v.m, off);
    r.m = ((unsigned __int128)hi << 64) | lo;
    r.e = __shfl_down_sync(0xffffffffu, v.e, off);
    const int fl = __shfl_down_sync(0xffffffffu, (v.neg ? 1 : 0) | (v.zero ? 2 : 0), off);
    r.neg = fl & 1;
    r.zero = (fl & 2) != 0;
    return r;
}

__device__ __forceinline__ XF xf_warp_sum(XF v)
{
    for (int off = 16; off > 0; off >>= 1) v = xfp::xf_add(v, xf_shfl_down(v, off));
    return v;
}

// Extended float in a plain-old-data form for global memory.
struct XFPod {
    unsigned long long hi, lo;
    int e;
    int flags;   // 1 neg, 2 zero, 4 non-finite input seen
};

__device__ __forceinline__ XFPod to_pod(const XF &v, bool bad)
{
    XFPod p;
    p.hi = (unsigned long long)(v.m >> 64);
    p.lo = (unsigned long long)v.m;
    p.e = v.e;
    p.flags = (v.neg ? 1 : 0) | (v.zero ? 2 : 0) | (bad ? 4 : 0);
    return p;
}

__device__ __forceinline__ XF from_pod(const XFPod &p)
{
    XF v;
    v.m = ((unsigned __int128)p.hi << 64) | p.lo;
    v.e = p.e;
    v.neg = p.flags & 1;
    v.zero = (p.flags & 2) != 0;
    return v;
}

__device__ __forceinline__ bool finite_dd(double2 v)
{
    // exponent field of hi below 0x7FF (lo is finite whenever hi is, for
    // any value a double-double operator produces)
    return (((uint64_t)__double_as_longlong(v.x) >> 52) & 0x7FF) != 0x7FF &&
           (((uint64_t)__double_as_longlong(v.y) >> 52) & 0x7FF) != 0x7FF;
}

}  // namespace fx
