// Integer fixed-point accumulation of double-double products, for the
// bandwidth-bound reductions (DOT, GEMV) and the TRSM block inverses.
//
// On this part an FP64 instruction issues at ~1/40 of the integer rate, so a
// double-double multiply-add on the FP64 pipe (12 instructions) cannot keep
// up with HBM. Here everything is integer work on the bit patterns:
//
//  * decode: a double-double (hi, lo) becomes |hi + lo| = (x1:x0) * 2^e with
//    x1 < 2^54 holding hi's mantissa and x0 the 64 bits below it (lo's
//    mantissa shifted into place, added or subtracted): the exact value to
//    2^-117, from shifts and adds only;
//  * product: Q = floor(|a| |b| / 2^64), three 64 x 64 -> 128-bit products
//    (the dropped x0*y0 term is below 2^-106 of the product's top), Q < 2^172;
//  * accumulate: Q is shifted to the accumulator's block exponent and added
//    into a 192-bit two's complement integer; when a product would reach above
//    the 12-bit headroom the block exponent moves up (a right shift, rare after
//    the first terms). At most 4096 products per accumulator (callers size
//    their grids for it).
//
// Sums of accumulators (warp, block, grid) use the 128-bit extended-float
// addition of xfloat.cuh in a fixed order, so results are deterministic.
// Non-finite inputs make the double-double operators of the reference return
// NaN (the TwoProduct error term of an infinity is inf - inf): they are
// flagged and the result is NaN.
#pragma once
#include "xfloat.cuh"

namespace fx {

using xfp::XF;

constexpr int kMaxAdds = 4096;   // products per accumulator (12-bit headroom)

enum : uint32_t { kNeg = 1, kZero = 2, kBad = 4 };

// |v| = (x1:x0) * 2^e, sign and zero / non-finite flags.
struct Op {
    uint64_t x1, x0;
    int e;
    uint32_t flags;
};

__device__ __forceinline__ Op decode(double2 v)
{
    Op o;
    const uint64_t bh = (uint64_t)__double_as_longlong(v.x), bl = (uint64_t)__double_as_longlong(v.y);
    int eh = (int)((bh >> 52) & 0x7FF), el = (int)((bl >> 52) & 0x7FF);
    o.flags = (uint32_t)(bh >> 63);
    if (eh == 0x7FF || el == 0x7FF) {
        o.flags |= kBad;
        o.x1 = o.x0 = 0;
        o.e = 0;
        return o;
    }
    if ((bh << 1) == 0) {   // hi == +-0: a normalised double-double is zero
        o.flags |= kZero;
        o.x1 = o.x0 = 0;
        o.e = 0;
        return o;
    }
    const uint64_t mh = (bh & 0xFFFFFFFFFFFFFull) | (eh ? (1ull << 52) : 0);
    eh = eh ? eh : 1;
    o.e = eh - 1075 - 64;
    o.x1 = mh;
    o.x0 = 0;
    if ((bl << 1) != 0) {
        const uint64_t ml = (bl & 0xFFFFFFFFFFFFFull) | (el ? (1ull << 52) : 0);
        el = el ? el : 1;
        const int s = 64 - (eh - el);   // lo's mantissa sits s bits above x0's bit 0
        uint64_t t1 = 0, t0;
        if (s >= 64) {
            // |lo| >= |hi| / 2: not a normalised double-double; keep hi's frame
            // and fold lo in at 2^64 granularity (the value stays within
            // 2^-52 of hi + lo relative to lo)
            const int s1 = s - 64;
            t1 = s1 < 11 ? (ml << s1) : (ml << 10);
            t0 = 0;
        } else if (s >= 0) {
            t0 = ml << s;
            t1 = s ? (ml >> (64 - s)) : 0;
        } else {
            t0 = (-s < 64) ? (ml >> -s) : 0;
        }
        if ((bh ^ bl) >> 63) {   // lo has the opposite sign
            const uint64_t borrow = t0 != 0;
            o.x0 = 0 - t0;
            o.x1 = mh - t1 - borrow;
        } else {
            o.x0 = t0;
            o.x1 = mh + t1;
        }
    }
    return o;
}

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
            w0 = w1 = w2 = 0;   // all earlier terms lie below the new resolution
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

    // W += +-(q2:q1:q0) * 2^(eq - lsb), q < 2^172
    __device__ __forceinline__ void add_q(uint64_t q0, uint64_t q1, uint64_t q2, int eq, bool neg)
    {
        if (!init) {
            lsb = eq - 4;
            init = true;
        }
        int s = eq - lsb;
        if (s > 8) {   // keep Q's top (bit 171 + s) at or below bit 179
            shift_right(s - 4);
            lsb += s - 4;
            s = 4;
        }
        uint64_t v0, v1, v2;
        if (s >= 0) {
            v0 = q0 << s;
            v1 = s ? ((q1 << s) | (q0 >> (64 - s))) : q1;
            v2 = s ? ((q2 << s) | (q1 >> (64 - s))) : q2;
        } else {
            const int r = -s;
            if (r >= 172) return;   // below the accumulator's resolution
            const int ws = r >> 6, b = r & 63;
            const uint64_t a0 = ws == 0 ? q0 : (ws == 1 ? q1 : q2);
            const uint64_t a1 = ws == 0 ? q1 : (ws == 1 ? q2 : 0);
            const uint64_t a2 = ws == 0 ? q2 : 0;
            v0 = b ? ((a0 >> b) | (a1 << (64 - b))) : a0;
            v1 = b ? ((a1 >> b) | (a2 << (64 - b))) : a1;
            v2 = a2 >> b;
        }
        if (neg) {
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

    // += a * b (decoded operands)
    __device__ __forceinline__ void add_prod(const Op &a, const Op &b)
    {
        const uint32_t f = a.flags | b.flags;
        if (f & kBad) {
            bad = true;
            return;
        }
        if (f & kZero) return;
        // Q = (a1 b1) 2^64 + a1 b0 + a0 b1 + hi(a0 b0 dropped)
        const uint64_t p11l = a.x1 * b.x1, p11h = __umul64hi(a.x1, b.x1);
        const uint64_t p10l = a.x1 * b.x0, p10h = __umul64hi(a.x1, b.x0);
        const uint64_t p01l = a.x0 * b.x1, p01h = __umul64hi(a.x0, b.x1);
        uint64_t q0, q1, q2;
        asm("add.cc.u64 %0, %3, %4;\n\t"
            "addc.cc.u64 %1, %5, %6;\n\t"
            "addc.u64 %2, %7, 0;\n\t"
            "add.cc.u64 %1, %1, %8;\n\t"
            "addc.u64 %2, %2, 0;"
            : "=l"(q0), "=l"(q1), "=l"(q2)
            : "l"(p10l), "l"(p01l), "l"(p11l), "l"(p10h), "l"(p11h), "l"(p01h));
        add_q(q0, q1, q2, a.e + b.e + 64, ((a.flags ^ b.flags) & kNeg) != 0);
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

// An extended float as a decoded operand (for values produced by the CRT or
// by a previous reduction): |v| = m * 2^e -> (x1:x0) with x1 < 2^54.
__device__ __forceinline__ Op op_from_xf(const XF &v)
{
    Op o;
    o.flags = (v.neg ? kNeg : 0) | (v.zero ? kZero : 0);
    o.x1 = (uint64_t)(v.m >> 74);
    o.x0 = (uint64_t)(v.m >> 10);
    o.e = v.e + 10;
    return o;
}

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

// A decoded operand in the same 24-byte form.
struct OpPod {
    unsigned long long x1, x0;
    int e;
    unsigned int flags;
};

__device__ __forceinline__ OpPod to_pod(const Op &o)
{
    OpPod p;
    p.x1 = o.x1;
    p.x0 = o.x0;
    p.e = o.e;
    p.flags = o.flags;
    return p;
}

__device__ __forceinline__ Op from_pod(const OpPod &p)
{
    Op o;
    o.x1 = p.x1;
    o.x0 = p.x0;
    o.e = p.e;
    o.flags = p.flags;
    return o;
}

__device__ __forceinline__ bool finite_dd(double2 v)
{
    return (((uint64_t)__double_as_longlong(v.x) >> 52) & 0x7FF) != 0x7FF &&
           (((uint64_t)__double_as_longlong(v.y) >> 52) & 0x7FF) != 0x7FF;
}

}  // namespace fx
