// Extended-float helpers shared by the CRT reconstruction: exact conversion
// between double-double values and a (sign, 128-bit mantissa, exponent)
// representation, products and sums on that representation, and rounding back
// to double-double, all in integer arithmetic. Written __host__ __device__ so
// the same code is unit-tested on the CPU.
#pragma once
#include <stdint.h>
#include <string.h>

#ifdef __CUDACC__
#define XF_HD __host__ __device__ __forceinline__
#else
#define XF_HD static inline
#endif

namespace xfp {

XF_HD int clz64(uint64_t v)
{
#ifdef __CUDA_ARCH__
    return __clzll((long long)v);
#else
    return v ? __builtin_clzll(v) : 64;
#endif
}
// Full 64 x 64 -> 128-bit product. On the device it is built from four
// 32 x 32 -> 64-bit multiply-adds: the 64-bit multiply-high instruction
// issues at the FP64 rate on this part.
XF_HD void mul64x64(uint64_t a, uint64_t b, uint64_t &hi, uint64_t &lo)
{
#ifdef __CUDA_ARCH__
    const uint32_t al = (uint32_t)a, ah = (uint32_t)(a >> 32), bl = (uint32_t)b, bh = (uint32_t)(b >> 32);
    const uint64_t ll = (uint64_t)al * bl, lh = (uint64_t)al * bh, hl = (uint64_t)ah * bl, hh = (uint64_t)ah * bh;
    const uint64_t mid = (ll >> 32) + (uint32_t)lh + (uint32_t)hl;
    lo = (mid << 32) | (uint32_t)ll;
    hi = hh + (lh >> 32) + (hl >> 32) + (mid >> 32);
#else
    const unsigned __int128 p = (unsigned __int128)a * b;
    hi = (uint64_t)(p >> 64);
    lo = (uint64_t)p;
#endif
}
XF_HD uint64_t mulhi64(uint64_t a, uint64_t b)
{
    uint64_t hi, lo;
    mul64x64(a, b, hi, lo);
    return hi;
}
XF_HD uint64_t dbits(double d)
{
#ifdef __CUDA_ARCH__
    return (uint64_t)__double_as_longlong(d);
#else
    uint64_t u;
    memcpy(&u, &d, 8);
    return u;
#endif
}
XF_HD double bitsd(uint64_t u)
{
#ifdef __CUDA_ARCH__
    return __longlong_as_double((long long)u);
#else
    double d;
    memcpy(&d, &u, 8);
    return d;
#endif
}

// v * 2^e for an integer 0 <= v < 2^54, as an exact (or correctly rounded on
// underflow) double.
XF_HD double scaled_u54(uint64_t v, int e)
{
    if (v == 0) return 0.0;
    int lz = clz64(v) - 11;   // leading zeros within 53 bits (may be -1 for 2^53)
    int64_t mant;
    int ex;
    if (lz >= 0) {
        mant = (int64_t)(v << lz);
        ex = e - lz + 52;
    } else {   // v == 2^53 exactly (after rounding)
        mant = (int64_t)(v >> 1);
        ex = e + 53;
    }
    if (ex >= -1022 && ex <= 1023) {
        uint64_t b = ((uint64_t)(ex + 1023) << 52) | ((uint64_t)mant & ((1ull << 52) - 1));
        return bitsd(b);
    }
    // outside the normal range: let the FP unit round (rare)
    double d = (double)mant;
    int e2 = ex - 52;
    while (e2 > 1000) { d *= 0x1p1000; e2 -= 1000; }
    while (e2 < -1000) { d *= 0x1p-1000; e2 += 1000; }
    uint64_t pb = (uint64_t)(e2 + 1023) << 52;
    return d * bitsd(pb);
}

// ---- extended floats: sign, 128-bit mantissa (bit 127 set), binary exponent ----
// value = (neg ? -1 : 1) * m * 2^e. Used to apply alpha and beta*C in integer
// arithmetic: on this part an FP64 instruction costs the issue time of ~39
// integer multiply-adds, and the double-double alpha/beta update would take
// ~25 of them per element.
struct XF {
    unsigned __int128 m;
    int e;
    bool neg;
    bool zero;
};

XF_HD int clz128(unsigned __int128 v)
{
    uint64_t hi = (uint64_t)(v >> 64), lo = (uint64_t)v;
    return hi ? clz64(hi) : 64 + clz64(lo);
}

XF_HD XF xf_norm(bool neg, unsigned __int128 m, int e)
{
    XF r;
    r.neg = neg;
    r.zero = (m == 0);
    if (r.zero) {
        r.m = 0;
        r.e = 0;
        return r;
    }
    int z = clz128(m);
    r.m = m << z;
    r.e = e - z;
    return r;
}

// Exact image of a finite double-double (hi, lo).
XF_HD XF xf_from_dd(double hi, double lo)
{
    uint64_t bh = dbits(hi), bl = dbits(lo);
    int eh = (int)((bh >> 52) & 0x7FF), el = (int)((bl >> 52) & 0x7FF);
    uint64_t mh = bh & 0xFFFFFFFFFFFFFull, ml = bl & 0xFFFFFFFFFFFFFull;
    if (eh) mh |= 1ull << 52; else eh = 1;
    if (el) ml |= 1ull << 52; else el = 1;
    if (hi == 0.0) {   // normalised DD: lo is 0 too
        XF z;
        z.zero = true; z.neg = false; z.m = 0; z.e = 0;
        return z;
    }
    // hi's mantissa occupies bits 74..126 of a signed 128-bit integer
    __int128 v = (__int128)(mh) << 74;
    if (bh >> 63) v = -v;
    int d = eh - el;   // lo sits d bits below hi
    if (ml && d < 74 + 53) {
        __int128 w;
        int sh = 74 - d;
        if (sh >= 0) w = (__int128)ml << sh;
        else w = (__int128)((ml + (1ull << (-sh - 1))) >> (-sh));
        v += (bl >> 63) ? -w : w;
    }
    bool neg = v < 0;
    return xf_norm(neg, (unsigned __int128)(neg ? -v : v), eh - 1075 - 74);
}

// Top 128 bits of the product of two mantissas.
XF_HD XF xf_mul(const XF &a, const XF &b)
{
    if (a.zero || b.zero) {
        XF z;
        z.zero = true; z.neg = false; z.m = 0; z.e = 0;
        return z;
    }
    uint64_t a1 = (uint64_t)(a.m >> 64), a0 = (uint64_t)a.m, b1 = (uint64_t)(b.m >> 64), b0 = (uint64_t)b.m;
    uint64_t h, l;
    mul64x64(a1, b1, h, l);
    unsigned __int128 p11 = ((unsigned __int128)h << 64) | l;
    mul64x64(a1, b0, h, l);
    unsigned __int128 p10 = ((unsigned __int128)h << 64) | l;
    mul64x64(a0, b1, h, l);
    unsigned __int128 p01 = ((unsigned __int128)h << 64) | l;
    uint64_t p00h = mulhi64(a0, b0);
    unsigned __int128 mid = (p10 & 0xFFFFFFFFFFFFFFFFull) + (p01 & 0xFFFFFFFFFFFFFFFFull) + p00h;
    unsigned __int128 hi = p11 + (p10 >> 64) + (p01 >> 64) + (mid >> 64);
    // product = hi * 2^128 + (mid mod 2^64) * 2^64 + ...; hi >= 2^126
    XF r;
    r.neg = a.neg != b.neg;
    r.zero = false;
    if (!(hi >> 127)) {
        hi = (hi << 1) | (((uint64_t)mid >> 63) & 1);
        r.e = a.e + b.e + 127;
    } else {
        r.e = a.e + b.e + 128;
    }
    r.m = hi;
    return r;
}

XF_HD XF xf_add(XF a, XF b)
{
    if (a.zero) return b;
    if (b.zero) return a;
    if (b.e > a.e || (b.e == a.e && b.m > a.m)) {
        XF t = a; a = b; b = t;
    }
    int d = a.e - b.e;
    unsigned __int128 bm = (d >= 128) ? 0 : (b.m >> d);
    if (a.neg == b.neg) {
        unsigned __int128 s = a.m + bm;
        if (s < a.m) {   // carry out of bit 127
            XF r;
            r.neg = a.neg; r.zero = false;
            r.m = (s >> 1) | ((unsigned __int128)1 << 127);
            r.e = a.e + 1;
            return r;
        }
        XF r;
        r.neg = a.neg; r.zero = false; r.m = s; r.e = a.e;
        return r;
    }
    return xf_norm(a.neg, a.m - bm, a.e);
}

XF_HD void xf_to_dd(const XF &x, double &out_hi, double &out_lo)
{
    if (x.zero) {
        out_hi = 0.0;
        out_lo = 0.0;
        return;
    }
    uint64_t a = (uint64_t)(x.m >> 75);                       // 53 bits
    uint64_t rem = (uint64_t)((x.m & (((unsigned __int128)1 << 75) - 1)) >> 11);   // top 64 of the 75-bit rest
    // round hi to nearest on bit 74 of the mantissa (bit 63 of rem)
    bool up = (rem >> 63) != 0;
    int64_t lo_int;   // remaining value in units of 2^(e+11)
    if (up) ++a;
    // rounding hi up leaves rem - 2^64, which is rem's two's-complement value
    lo_int = (int64_t)rem;
    double hi = scaled_u54(a, x.e + 75);
    double lo;
    if (lo_int >= 0) {
        uint64_t u = (uint64_t)lo_int;
        int lz = u ? clz64(u) : 64;
        int sh = 11 - lz;   // bring to <= 53 bits
        uint64_t mnt = sh > 0 ? ((u + (1ull << (sh - 1))) >> sh) : (u << -sh);
        lo = u ? scaled_u54(mnt, x.e + 11 + sh) : 0.0;
    } else {
        uint64_t u = (uint64_t)(-lo_int);
        int lz = clz64(u);
        int sh = 11 - lz;
        uint64_t mnt = sh > 0 ? ((u + (1ull << (sh - 1))) >> sh) : (u << -sh);
        lo = -scaled_u54(mnt, x.e + 11 + sh);
    }
    out_hi = x.neg ? -hi : hi;
    out_lo = x.neg ? -lo : lo;
}

}  // namespace xfp
