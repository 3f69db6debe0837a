// Extended floats in 32-bit words: sign, 128-bit mantissa held as four 32-bit
// words, binary exponent. The same operations as xfloat.cuh (exact
// double-double import, truncated products, sums, rounding to double-double)
// written so that the device code uses only 32-bit integer instructions,
// funnel shifts and 32 x 32 -> 64-bit multiplies. On this part 64-bit shifts,
// compares and multiply-highs issue at the FP64 rate, so the __int128 forms
// of xfloat.cuh spend most of an element's time in the per-element epilogues
// (CRT reconstruction). __host__ __device__: the host build is unit-tested.
#pragma once
#include <stdint.h>
#include <string.h>

#ifdef __CUDACC__
#define XW_HD __host__ __device__ __forceinline__
#else
#define XW_HD static inline
#endif

namespace xw {

// value = (neg ? -1 : 1) * W * 2^e, W = w[3]:w[2]:w[1]:w[0]; normalised
// values have bit 31 of w[3] set; zero has w[3] == 0.
struct XW {
    uint32_t w[4];
    int e;
    uint32_t neg;
};

XW_HD uint32_t fshr(uint32_t lo, uint32_t hi, int r)   // low word of (hi:lo) >> r, 0 <= r < 32
{
#ifdef __CUDA_ARCH__
    return __funnelshift_r(lo, hi, r);
#else
    return r ? (lo >> r) | (hi << (32 - r)) : lo;
#endif
}

XW_HD uint32_t fshl(uint32_t lo, uint32_t hi, int r)   // high word of (hi:lo) << r, 0 <= r < 32
{
#ifdef __CUDA_ARCH__
    return __funnelshift_l(lo, hi, r);
#else
    return r ? (hi << r) | (lo >> (32 - r)) : hi;
#endif
}

XW_HD int clz32(uint32_t v)
{
#ifdef __CUDA_ARCH__
    return __clz((int)v);
#else
    return v ? __builtin_clz(v) : 32;
#endif
}

XW_HD uint32_t lo32(uint64_t v) { return (uint32_t)v; }
XW_HD uint32_t hi32(uint64_t v) { return (uint32_t)(v >> 32); }

// a += b over four words; returns the carry out.
XW_HD uint32_t add4(uint32_t a[4], const uint32_t b[4])
{
#ifdef __CUDA_ARCH__
    uint32_t c;
    asm("add.cc.u32 %0, %0, %5;\n\t"
        "addc.cc.u32 %1, %1, %6;\n\t"
        "addc.cc.u32 %2, %2, %7;\n\t"
        "addc.cc.u32 %3, %3, %8;\n\t"
        "addc.u32 %4, 0, 0;"
        : "+r"(a[0]), "+r"(a[1]), "+r"(a[2]), "+r"(a[3]), "=r"(c)
        : "r"(b[0]), "r"(b[1]), "r"(b[2]), "r"(b[3]));
    return c;
#else
    uint64_t c = 0;
    for (int t = 0; t < 4; ++t) {
        c += (uint64_t)a[t] + b[t];
        a[t] = (uint32_t)c;
        c >>= 32;
    }
    return (uint32_t)c;
#endif
}

// a -= b over four words (a >= b).
XW_HD void sub4(uint32_t a[4], const uint32_t b[4])
{
#ifdef __CUDA_ARCH__
    asm("sub.cc.u32 %0, %0, %4;\n\t"
        "subc.cc.u32 %1, %1, %5;\n\t"
        "subc.cc.u32 %2, %2, %6;\n\t"
        "subc.u32 %3, %3, %7;"
        : "+r"(a[0]), "+r"(a[1]), "+r"(a[2]), "+r"(a[3])
        : "r"(b[0]), "r"(b[1]), "r"(b[2]), "r"(b[3]));
#else
    uint64_t br = 0;
    for (int t = 0; t < 4; ++t) {
        const uint64_t d = (uint64_t)a[t] - b[t] - br;
        a[t] = (uint32_t)d;
        br = (d >> 63) & 1u;
    }
#endif
}

// W >> sh for 0 <= sh < 128.
XW_HD void shr4(const uint32_t w[4], int sh, uint32_t y[4])
{
    const int q = sh >> 5, r = sh & 31;
    const uint32_t a0 = q == 0 ? w[0] : (q == 1 ? w[1] : (q == 2 ? w[2] : w[3]));
    const uint32_t a1 = q == 0 ? w[1] : (q == 1 ? w[2] : (q == 2 ? w[3] : 0u));
    const uint32_t a2 = q == 0 ? w[2] : (q == 1 ? w[3] : 0u);
    const uint32_t a3 = q == 0 ? w[3] : 0u;
    y[0] = fshr(a0, a1, r);
    y[1] = fshr(a1, a2, r);
    y[2] = fshr(a2, a3, r);
    y[3] = r ? (a3 >> r) : a3;
}

// Shift W left until bit 127 is set (W != 0), lowering e by the shift.
XW_HD void norm4(uint32_t w[4], int &e)
{
    for (int k = 0; k < 3 && w[3] == 0u; ++k) {
        w[3] = w[2];
        w[2] = w[1];
        w[1] = w[0];
        w[0] = 0u;
        e -= 32;
    }
    const int z = clz32(w[3]);
    if (z > 0 && z < 32) {
        w[3] = fshl(w[2], w[3], z);
        w[2] = fshl(w[1], w[2], z);
        w[1] = fshl(w[0], w[1], z);
        w[0] <<= z;
        e -= z;
    }
}

XW_HD XW zero()
{
    XW r;
    r.w[0] = r.w[1] = r.w[2] = r.w[3] = 0u;
    r.e = 0;
    r.neg = 0u;
    return r;
}

XW_HD uint32_t dbl_lo(double d)
{
#ifdef __CUDA_ARCH__
    return (uint32_t)__double2loint(d);
#else
    uint64_t u;
    memcpy(&u, &d, 8);
    return (uint32_t)u;
#endif
}

XW_HD uint32_t dbl_hi(double d)
{
#ifdef __CUDA_ARCH__
    return (uint32_t)__double2hiint(d);
#else
    uint64_t u;
    memcpy(&u, &d, 8);
    return (uint32_t)(u >> 32);
#endif
}

XW_HD double dbl_make(uint32_t hi, uint32_t lo)
{
#ifdef __CUDA_ARCH__
    return __hiloint2double((int)hi, (int)lo);
#else
    const uint64_t u = ((uint64_t)hi << 32) | lo;
    double d;
    memcpy(&d, &u, 8);
    return d;
#endif
}

// 53-bit mantissa (mh:ml, mh < 2^21) shifted left by s (0 <= s < 96) into
// four words.
XW_HD void place53(uint32_t mh, uint32_t ml, int s, uint32_t t[4])
{
    const int q = s >> 5, r = s & 31;
    const uint32_t a0 = ml << r;
    const uint32_t a1 = fshl(ml, mh, r);
    const uint32_t a2 = r ? (mh >> (32 - r)) : 0u;
    t[0] = q == 0 ? a0 : 0u;
    t[1] = q == 0 ? a1 : (q == 1 ? a0 : 0u);
    t[2] = q == 0 ? a2 : (q == 1 ? a1 : a0);
    t[3] = q == 0 ? 0u : (q == 1 ? a2 : a1);
}

// Image of a finite double-double hi + lo (normalised: |lo| <= ulp(hi)/2),
// exact unless lo lies more than 74 bits below hi (then lo is truncated at
// 2^-128 of hi). Non-finite input is the caller's to screen.
XW_HD XW from_dd(double hi, double lo)
{
    const uint32_t hh = dbl_hi(hi), hl = dbl_lo(hi), lh = dbl_hi(lo), ll = dbl_lo(lo);
    if (((hh << 1) | hl) == 0u) return zero();
    int eh = (int)((hh >> 20) & 0x7FFu), el = (int)((lh >> 20) & 0x7FFu);
    const uint32_t mhh = (hh & 0xFFFFFu) | (eh ? 0x100000u : 0u);
    eh = eh ? eh : 1;
    XW r;
    // hi's mantissa at bits 74..126
    place53(mhh, hl, 74, r.w);
    r.e = eh - 1075 - 74;
    r.neg = hh >> 31;
    if (((lh << 1) | ll) != 0u) {
        const uint32_t mlh = (lh & 0xFFFFFu) | (el ? 0x100000u : 0u);
        el = el ? el : 1;
        const int s = 74 - (eh - el);   // lo's mantissa sits s bits above bit 0
        uint32_t t[4] = {0u, 0u, 0u, 0u};
        if (s >= 0) {
            place53(mlh, ll, s < 95 ? s : 95, t);
        } else if (s > -53) {
            const int rr = -s;
            t[0] = rr >= 32 ? (mlh >> (rr - 32)) : fshr(ll, mlh, rr);
            t[1] = rr >= 32 ? 0u : (mlh >> rr);
        }
        if ((hh ^ lh) >> 31) sub4(r.w, t);
        else {
            const uint32_t c = add4(r.w, t);
            (void)c;   // no carry: |lo| <= ulp(hi)/2 keeps W below 2^128
        }
    }
    norm4(r.w, r.e);
    return r;
}

// Top 128 bits of the product of two normalised mantissas (the partial
// products of columns 0..2 of the 256-bit product are dropped: relative error
// < 2^-122). The host and device forms sum the same partial products.
XW_HD XW mul(const XW &a, const XW &b)
{
    if (a.w[3] == 0u || b.w[3] == 0u) return zero();
    const uint32_t a0 = a.w[0], a1 = a.w[1], a2 = a.w[2], a3 = a.w[3];
    const uint32_t b0 = b.w[0], b1 = b.w[1], b2 = b.w[2], b3 = b.w[3];
#ifdef __CUDA_ARCH__
    // Row by row (b3, b2, b1, b0) with 32-bit multiply-add carry chains into
    // the columns 3..7 of the 256-bit product.
    uint32_t c3, c4, c5, c6, c7;
    asm("mul.lo.u32 %0, %5, %9;\n\t"
        "mul.lo.u32 %1, %6, %9;\n\t"
        "mul.lo.u32 %2, %7, %9;\n\t"
        "mul.lo.u32 %3, %8, %9;\n\t"
        "mad.hi.cc.u32 %1, %5, %9, %1;\n\t"
        "madc.hi.cc.u32 %2, %6, %9, %2;\n\t"
        "madc.hi.cc.u32 %3, %7, %9, %3;\n\t"
        "madc.hi.u32 %4, %8, %9, 0;\n\t"
        // b2: a1, a2, a3 at columns 3, 4, 5
        "mad.lo.cc.u32 %0, %6, %10, %0;\n\t"
        "madc.lo.cc.u32 %1, %7, %10, %1;\n\t"
        "madc.lo.cc.u32 %2, %8, %10, %2;\n\t"
        "addc.cc.u32 %3, %3, 0;\n\t"
        "addc.u32 %4, %4, 0;\n\t"
        "mad.hi.cc.u32 %1, %6, %10, %1;\n\t"
        "madc.hi.cc.u32 %2, %7, %10, %2;\n\t"
        "madc.hi.cc.u32 %3, %8, %10, %3;\n\t"
        "addc.u32 %4, %4, 0;\n\t"
        // b1: a2, a3 at columns 3, 4
        "mad.lo.cc.u32 %0, %7, %11, %0;\n\t"
        "madc.lo.cc.u32 %1, %8, %11, %1;\n\t"
        "addc.cc.u32 %2, %2, 0;\n\t"
        "addc.cc.u32 %3, %3, 0;\n\t"
        "addc.u32 %4, %4, 0;\n\t"
        "mad.hi.cc.u32 %1, %7, %11, %1;\n\t"
        "madc.hi.cc.u32 %2, %8, %11, %2;\n\t"
        "addc.cc.u32 %3, %3, 0;\n\t"
        "addc.u32 %4, %4, 0;\n\t"
        // b0: a3 at column 3
        "mad.lo.cc.u32 %0, %8, %12, %0;\n\t"
        "addc.cc.u32 %1, %1, 0;\n\t"
        "addc.cc.u32 %2, %2, 0;\n\t"
        "addc.cc.u32 %3, %3, 0;\n\t"
        "addc.u32 %4, %4, 0;\n\t"
        "mad.hi.cc.u32 %1, %8, %12, %1;\n\t"
        "addc.cc.u32 %2, %2, 0;\n\t"
        "addc.cc.u32 %3, %3, 0;\n\t"
        "addc.u32 %4, %4, 0;"
        : "=&r"(c3), "=&r"(c4), "=&r"(c5), "=&r"(c6), "=&r"(c7)
        : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b3), "r"(b2), "r"(b1), "r"(b0));
    XW r;
    r.neg = a.neg ^ b.neg;
    r.e = a.e + b.e + 128;
    r.w[3] = c7;
    r.w[2] = c6;
    r.w[1] = c5;
    r.w[0] = c4;
    if (!(c7 >> 31)) {   // product below 2^255: one more bit from column 3
        r.w[3] = fshl(c6, c7, 1);
        r.w[2] = fshl(c5, c6, 1);
        r.w[1] = fshl(c4, c5, 1);
        r.w[0] = fshl(c3, c4, 1);
        r.e -= 1;
    }
    return r;
#else
    const uint64_t p03 = (uint64_t)a0 * b3, p12 = (uint64_t)a1 * b2, p21 = (uint64_t)a2 * b1, p30 = (uint64_t)a3 * b0;
    const uint64_t p13 = (uint64_t)a1 * b3, p22 = (uint64_t)a2 * b2, p31 = (uint64_t)a3 * b1;
    const uint64_t p23 = (uint64_t)a2 * b3, p32 = (uint64_t)a3 * b2;
    const uint64_t p33 = (uint64_t)a3 * b3;
    const uint64_t s3 = (uint64_t)lo32(p03) + lo32(p12) + lo32(p21) + lo32(p30);
    const uint64_t s4 = (s3 >> 32) + hi32(p03) + hi32(p12) + hi32(p21) + hi32(p30) + lo32(p13) + lo32(p22) +
                        lo32(p31);
    const uint64_t s5 = (s4 >> 32) + hi32(p13) + hi32(p22) + hi32(p31) + lo32(p23) + lo32(p32);
    const uint64_t s6 = (s5 >> 32) + hi32(p23) + hi32(p32) + lo32(p33);
    const uint32_t r7 = (uint32_t)((s6 >> 32) + hi32(p33));
    XW r;
    r.neg = a.neg ^ b.neg;
    r.e = a.e + b.e + 128;
    r.w[3] = r7;
    r.w[2] = lo32(s6);
    r.w[1] = lo32(s5);
    r.w[0] = lo32(s4);
    if (!(r7 >> 31)) {   // product below 2^255: one more bit from column 3
        r.w[3] = fshl(r.w[2], r.w[3], 1);
        r.w[2] = fshl(r.w[1], r.w[2], 1);
        r.w[1] = fshl(r.w[0], r.w[1], 1);
        r.w[0] = fshl(lo32(s3), r.w[0], 1);
        r.e -= 1;
    }
    return r;
#endif
}

// a + b, truncating the smaller operand's bits below 2^-128 of the larger.
XW_HD XW add(XW a, XW b)
{
    if (a.w[3] == 0u) return b;
    if (b.w[3] == 0u) return a;
    bool swap = b.e > a.e;
    if (b.e == a.e) {
        // equal exponents: compare the mantissas word by word from the top
        const uint32_t d3 = b.w[3] != a.w[3], d2 = b.w[2] != a.w[2], d1 = b.w[1] != a.w[1];
        swap = d3 ? b.w[3] > a.w[3] : (d2 ? b.w[2] > a.w[2] : (d1 ? b.w[1] > a.w[1] : b.w[0] > a.w[0]));
    }
    if (swap) {
        const XW t = a;
        a = b;
        b = t;
    }
    const int d = a.e - b.e;
    if (d >= 128) return a;
    uint32_t bs[4];
    shr4(b.w, d, bs);
    if (a.neg == b.neg) {
        if (add4(a.w, bs)) {   // carry out of bit 127
            a.w[0] = fshr(a.w[0], a.w[1], 1);
            a.w[1] = fshr(a.w[1], a.w[2], 1);
            a.w[2] = fshr(a.w[2], a.w[3], 1);
            a.w[3] = (a.w[3] >> 1) | 0x80000000u;
            a.e += 1;
        }
        return a;
    }
    sub4(a.w, bs);
    if ((a.w[0] | a.w[1] | a.w[2] | a.w[3]) == 0u) return zero();
    norm4(a.w, a.e);
    return a;
}

// m * 2^e as a double for an integer mantissa m = mh:ml with 2^52 <= m < 2^53
// (2^53 allowed: a rounding carry), correctly rounded below the normal range.
XW_HD double scaled53(uint32_t mh, uint32_t ml, int e)
{
    if (mh >> 21) {   // 2^53: halve
        ml = fshr(ml, mh, 1);
        mh >>= 1;
        e += 1;
    }
    const int ex = e + 52;   // unbiased exponent of the value
    if (ex >= -1022 && ex <= 1023)
        return dbl_make(((uint32_t)(ex + 1023) << 20) | (mh & 0xFFFFFu), ml);
    // outside the normal range: scale in steps (rare)
    double d = (double)(((uint64_t)mh << 32) | ml);
    int e2 = e;
    while (e2 > 1000) { d *= 0x1p1000; e2 -= 1000; }
    while (e2 < -1000) { d *= 0x1p-1000; e2 += 1000; }
    return d * dbl_make((uint32_t)(e2 + 1023) << 20, 0u);
}

// Round to double-double: hi = the top 53 bits rounded (half up), lo = the
// rest rounded to 53 bits; |lo| <= ulp(hi)/2.
XW_HD void to_dd(const XW &x, double &out_hi, double &out_lo)
{
    if (x.w[3] == 0u) {
        out_hi = 0.0;
        out_lo = 0.0;
        return;
    }
    // hi mantissa: bits 127..75 = w3 (32 bits) and bits 31..11 of w2
    uint32_t mh = x.w[3] >> 11, ml = fshl(x.w[2], x.w[3], 21);
    // the rest, bits 74..0: (w2 & 0x7FF) : w1 : w0
    uint32_t r2 = x.w[2] & 0x7FFu, r1 = x.w[1], r0 = x.w[0];
    const bool up = (r2 >> 10) & 1u;
    uint32_t lneg = 0u;
    if (up) {
        // hi + 1 ulp; the rest becomes rem - 2^75, of magnitude 2^75 - rem
        ml += 1u;
        mh += (ml == 0u);
        const uint32_t n0 = ~r0 + 1u;
        const uint32_t c0 = (r0 == 0u);
        const uint32_t n1 = ~r1 + c0;
        const uint32_t c1 = c0 & (r1 == 0u);
        r2 = ((~r2) + c1) & 0x7FFu;
        r1 = n1;
        r0 = n0;
        lneg = 1u;
    }
    const double hi = scaled53(mh, ml, x.e + 75);
    double lo = 0.0;
    const bool has_lo = (r2 | r1 | r0) != 0u;
    if (has_lo) {
        // normalise the 75-bit rest into (u2:u1:u0) with bit 74 ... and round to 53 bits
        uint32_t u[4] = {r0, r1, r2, 0u};
        int e = x.e;
        norm4(u, e);   // bit 127 set; value = U * 2^e
        uint32_t lh = u[3] >> 11, llw = fshl(u[2], u[3], 21);
        if ((u[2] >> 10) & 1u) {
            llw += 1u;
            lh += (llw == 0u);
        }
        lo = scaled53(lh, llw, e + 75);
    }
    const uint32_t sh = x.neg << 31, sl = (x.neg ^ lneg) << 31;
    out_hi = dbl_make(dbl_hi(hi) ^ sh, dbl_lo(hi));
    out_lo = has_lo ? dbl_make(dbl_hi(lo) ^ sl, dbl_lo(lo)) : 0.0;
}

}  // namespace xw
