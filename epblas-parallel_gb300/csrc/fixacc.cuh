// Integer fixed-point accumulation of double-double products, for the
// bandwidth-bound reductions (DOT, GEMV) and the TRSM block inverses.
//
// On this part an FP64 instruction issues at ~1/40 of the integer rate, so a
// double-double multiply-add on the FP64 pipe (12 instructions) cannot keep
// up with HBM. The 64-bit multiply-high (IMAD.HI) also issues at the FP64
// rate here, so only 32 x 32 -> 64-bit multiply-adds (IMAD.WIDE) are used:
//
//  * decode: a double-double (hi, lo) becomes |hi + lo| = W * 2^e, W a
//    118-bit integer in four 32-bit words holding hi's mantissa above 64 bits
//    of lo's mantissa shifted into place (added or subtracted): the exact
//    value to 2^-117, from 32-bit shifts and adds only (64-bit shifts issue
//    at the FP64 rate on this part);
//  * accumulate: each thread keeps a block exponent B. For a product x*y the
//    integer X is shifted right to the block (X' = X >> (B - ex - ey)) so that
//    X' * Y lands at 2^B; X' and Y are split into five 24-bit digits and the
//    19 digit products of weight >= 2^72 are added with IMAD.WIDE into six
//    64-bit column sums that persist across products (no per-product
//    alignment of the result). The dropped products are below 2^-130 of the
//    block. Every 2048 products the column carries are propagated; a product
//    above the block's headroom moves B up (a right shift of the whole sum,
//    rare after the first terms).
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

constexpr int kMaxAdds = 1 << 20;   // products per accumulator before it is folded into an extended float

enum : uint32_t { kNeg = 1, kZero = 2, kBad = 4 };

// |v| = W * 2^e with W = w[3]:w[2]:w[1]:w[0] (32-bit words, W < 2^118),
// sign and zero / non-finite flags. Everything here is 32-bit integer work:
// on this part the 64-bit shifts and multiplies run at the FP64 rate.
struct Op {
    uint32_t w[4];
    int e;
    uint32_t flags;
};

// 64-bit mantissa (hi:lo words, < 2^53) shifted left by s (0 <= s < 64) into
// four words.
__device__ __forceinline__ void shl53(uint32_t hi, uint32_t lo, int s, uint32_t t[4])
{
    const int q = s >> 5, r = s & 31;
    const uint32_t a0 = lo << r;
    const uint32_t a1 = __funnelshift_l(lo, hi, r);
    const uint32_t a2 = r ? (hi >> (32 - r)) : 0u;
    t[0] = q ? 0u : a0;
    t[1] = q ? a0 : a1;
    t[2] = q ? a1 : a2;
    t[3] = q ? a2 : 0u;
}

// Every case: zeros, non-finite limbs, subnormals, lo far below or (not
// normalised) above hi. Kept out of line: decode() calls it only off its fast
// path, so the common case does not pay for these branches.
static __device__ __noinline__ Op decode_general(double2 v)
{
    Op o;
    const uint32_t hl = (uint32_t)__double2loint(v.x), hh = (uint32_t)__double2hiint(v.x);
    const uint32_t ll = (uint32_t)__double2loint(v.y), lh = (uint32_t)__double2hiint(v.y);
    int eh = (int)((hh >> 20) & 0x7FF), el = (int)((lh >> 20) & 0x7FF);
    o.flags = hh >> 31;
    o.w[0] = o.w[1] = o.w[2] = o.w[3] = 0;
    o.e = 0;
    if (eh == 0x7FF || el == 0x7FF) {
        o.flags |= kBad;
        return o;
    }
    if (((hh << 1) | hl) == 0) {   // hi == +-0: a normalised double-double is zero
        o.flags |= kZero;
        return o;
    }
    const uint32_t mhh = (hh & 0xFFFFFu) | (eh ? 0x100000u : 0u);
    eh = eh ? eh : 1;
    o.e = eh - 1075 - 64;
    o.w[3] = mhh;
    o.w[2] = hl;
    if (((lh << 1) | ll) != 0) {
        const uint32_t mlh = (lh & 0xFFFFFu) | (el ? 0x100000u : 0u);
        el = el ? el : 1;
        int s = 64 - (eh - el);   // lo's mantissa sits s bits above bit 0 of W
        uint32_t t[4];
        if (s >= 64) {
            // |lo| >= |hi| / 2: not a normalised double-double; fold lo in at
            // 2^64 granularity (within 2^-52 of hi + lo relative to lo)
            const int s1 = s - 64 < 10 ? s - 64 : 10;
            uint32_t u[4];
            shl53(mlh, ll, s1, u);
            t[0] = 0; t[1] = 0; t[2] = u[0]; t[3] = u[1];
        } else if (s >= 0) {
            shl53(mlh, ll, s, t);
        } else {
            const int r = -s;   // right shift of the 53-bit mantissa
            t[2] = t[3] = 0;
            t[0] = r >= 64 ? 0u : (r >= 32 ? (mlh >> (r - 32)) : __funnelshift_r(ll, mlh, r));
            t[1] = r >= 32 ? 0u : (mlh >> r);
        }
        if ((hh ^ lh) >> 31) {   // lo has the opposite sign
            asm("sub.cc.u32 %0, %0, %4;\n\t"
                "subc.cc.u32 %1, %1, %5;\n\t"
                "subc.cc.u32 %2, %2, %6;\n\t"
                "subc.u32 %3, %3, %7;"
                : "+r"(o.w[0]), "+r"(o.w[1]), "+r"(o.w[2]), "+r"(o.w[3])
                : "r"(t[0]), "r"(t[1]), "r"(t[2]), "r"(t[3]));
        } else {
            asm("add.cc.u32 %0, %0, %4;\n\t"
                "addc.cc.u32 %1, %1, %5;\n\t"
                "addc.cc.u32 %2, %2, %6;\n\t"
                "addc.u32 %3, %3, %7;"
                : "+r"(o.w[0]), "+r"(o.w[1]), "+r"(o.w[2]), "+r"(o.w[3])
                : "r"(t[0]), "r"(t[1]), "r"(t[2]), "r"(t[3]));
        }
    }
    return o;
}

// The operands decode takes on its straight-line path: hi normal and finite,
// and lo zero, or normal with its exponent 33 to 64 below hi's (lo's mantissa
// then lands in the low three words with a left shift s = 64 - gap below 32;
// a normalised double-double has gap >= 53).
__device__ __forceinline__ bool decode_is_fast(double2 v)
{
    const uint32_t hh = (uint32_t)__double2hiint(v.x);
    const uint32_t ll = (uint32_t)__double2loint(v.y), lh = (uint32_t)__double2hiint(v.y);
    const uint32_t eh = (hh >> 20) & 0x7FFu, el = (lh >> 20) & 0x7FFu;
    const bool lo_zero = ((lh << 1) | ll) == 0u;
    const uint32_t gap = eh - el;   // unsigned: wraps when lo's exponent is above hi's
    return (eh - 1u) < 0x7FEu && (lo_zero || ((el - 1u) < 0x7FEu && gap - 33u <= 31u));
}

// decode for an operand that passes decode_is_fast (so finite and nonzero:
// the flags hold only the sign). The sum W = hi's mantissa * 2^64 +- lo's
// shifted mantissa is formed as W + (t ^ mask) + (mask & 1), mask = all ones
// when the signs differ; W < 2^118.
__device__ __forceinline__ Op decode_fast(double2 v)
{
    const uint32_t hl = (uint32_t)__double2loint(v.x), hh = (uint32_t)__double2hiint(v.x);
    const uint32_t ll = (uint32_t)__double2loint(v.y), lh = (uint32_t)__double2hiint(v.y);
    const uint32_t eh = (hh >> 20) & 0x7FFu, el = (lh >> 20) & 0x7FFu;
    const bool lo_zero = ((lh << 1) | ll) == 0u;
    const uint32_t gap = eh - el;
    Op o;
    o.flags = hh >> 31;
    o.e = (int)eh - 1075 - 64;
    const uint32_t mlh = lo_zero ? 0u : ((lh & 0xFFFFFu) | 0x100000u);
    const uint32_t lw = lo_zero ? 0u : ll;
    const int s = (int)(64u - gap) & 31;
    const uint32_t t0 = lw << s, t1 = __funnelshift_l(lw, mlh, s), t2 = __funnelshift_l(mlh, 0u, s);
    const uint32_t mask = 0u - ((hh ^ lh) >> 31);
    uint32_t w0, w1, w2, w3;
    asm("add.cc.u32 %0, %4, %8;\n\t"
        "addc.cc.u32 %1, %5, 0;\n\t"
        "addc.cc.u32 %2, %6, %9;\n\t"
        "addc.u32 %3, %7, %10;"
        : "=r"(w0), "=r"(w1), "=r"(w2), "=r"(w3)
        : "r"(t0 ^ mask), "r"(t1 ^ mask), "r"(t2 ^ mask), "r"((hh & 0xFFFFFu) | 0x100000u), "r"(mask & 1u),
          "r"(hl), "r"(mask));
    o.w[0] = w0;
    o.w[1] = w1;
    o.w[2] = w2;
    o.w[3] = w3;
    return o;
}

// The same result as decode_general, with decode_fast's straight-line path
// inline for the operands that pass decode_is_fast.
__device__ __forceinline__ Op decode(double2 v)
{
    const uint32_t hl = (uint32_t)__double2loint(v.x), hh = (uint32_t)__double2hiint(v.x);
    const uint32_t ll = (uint32_t)__double2loint(v.y), lh = (uint32_t)__double2hiint(v.y);
    const uint32_t eh = (hh >> 20) & 0x7FFu, el = (lh >> 20) & 0x7FFu;
    const bool lo_zero = ((lh << 1) | ll) == 0u;
    const uint32_t gap = eh - el;   // unsigned: wraps when lo's exponent is above hi's
    const bool fast = (eh - 1u) < 0x7FEu && (lo_zero || ((el - 1u) < 0x7FEu && gap - 33u <= 31u));
    if (!fast) {
        if (((hh << 1) | hl) == 0u && el != 0x7FFu) {   // hi == +-0 (lo finite): zero
            Op z;
            z.w[0] = z.w[1] = z.w[2] = z.w[3] = 0u;
            z.e = 0;
            z.flags = (hh >> 31) | kZero;
            return z;
        }
        return decode_general(v);
    }
    Op o;
    o.flags = hh >> 31;
    o.e = (int)eh - 1075 - 64;
    const uint32_t mlh = lo_zero ? 0u : ((lh & 0xFFFFFu) | 0x100000u);
    const uint32_t lw = lo_zero ? 0u : ll;
    const int s = (int)(64u - gap) & 31;
    const uint32_t t0 = lw << s, t1 = __funnelshift_l(lw, mlh, s), t2 = __funnelshift_l(mlh, 0u, s);
    const uint32_t mask = 0u - ((hh ^ lh) >> 31);
    uint32_t w0, w1, w2, w3;
    asm("add.cc.u32 %0, %4, %8;\n\t"
        "addc.cc.u32 %1, %5, 0;\n\t"
        "addc.cc.u32 %2, %6, %9;\n\t"
        "addc.u32 %3, %7, %10;"
        : "=r"(w0), "=r"(w1), "=r"(w2), "=r"(w3)
        : "r"(t0 ^ mask), "r"(t1 ^ mask), "r"(t2 ^ mask), "r"((hh & 0xFFFFFu) | 0x100000u), "r"(mask & 1u),
          "r"(hl), "r"(mask));
    o.w[0] = w0;
    o.w[1] = w1;
    o.w[2] = w2;
    o.w[3] = w3;
    return o;
}

// W >> sh (0 <= sh < 128) in four words.
__device__ __forceinline__ void shr128(const uint32_t w[4], int sh, uint32_t y[4])
{
    const int q = sh >> 5, r = sh & 31;
    // word shift by q
    const uint32_t a0 = q == 0 ? w[0] : (q == 1 ? w[1] : (q == 2 ? w[2] : w[3]));
    const uint32_t a1 = q == 0 ? w[1] : (q == 1 ? w[2] : (q == 2 ? w[3] : 0u));
    const uint32_t a2 = q == 0 ? w[2] : (q == 1 ? w[3] : 0u);
    const uint32_t a3 = q == 0 ? w[3] : 0u;
    y[0] = __funnelshift_r(a0, a1, r);
    y[1] = __funnelshift_r(a1, a2, r);
    y[2] = __funnelshift_r(a2, a3, r);
    y[3] = a3 >> r;
}

// 256-bit two's complement accumulation of x * 2^s (x signed, s < 128).
__device__ __forceinline__ void add_shifted(uint64_t W[4], int64_t x, int s)
{
    const uint64_t ext = x < 0 ? ~0ull : 0ull;
    const int b = s & 63;
    uint64_t v[4];
    const uint64_t lo = (uint64_t)x << b;
    const uint64_t hi = b ? (((uint64_t)x >> (64 - b)) | (ext << b)) : ext;
    if (s < 64) {
        v[0] = lo; v[1] = hi; v[2] = ext; v[3] = ext;
    } else {
        v[0] = 0; v[1] = lo; v[2] = hi; v[3] = ext;
    }
    asm("add.cc.u64 %0, %0, %4;\n\t"
        "addc.cc.u64 %1, %1, %5;\n\t"
        "addc.cc.u64 %2, %2, %6;\n\t"
        "addc.u64 %3, %3, %7;"
        : "+l"(W[0]), "+l"(W[1]), "+l"(W[2]), "+l"(W[3])
        : "l"(v[0]), "l"(v[1]), "l"(v[2]), "l"(v[3]));
}

// W * 2^e as an extended float (W two's complement, 256 bits).
__device__ __forceinline__ XF w256_to_xf(uint64_t W[4], int e)
{
    XF r;
    r.neg = (int64_t)W[3] < 0;
    if (r.neg) {
        asm("sub.cc.u64 %0, 0, %0;\n\t"
            "subc.cc.u64 %1, 0, %1;\n\t"
            "subc.cc.u64 %2, 0, %2;\n\t"
            "subc.u64 %3, 0, %3;"
            : "+l"(W[0]), "+l"(W[1]), "+l"(W[2]), "+l"(W[3]));
    }
    int top = 3;
    while (top > 0 && W[top] == 0) --top;
    if (W[top] == 0) {
        r.zero = true; r.neg = false; r.m = 0; r.e = 0;
        return r;
    }
    const int z = xfp::clz64(W[top]);
    const uint64_t w1 = W[top], w0 = top >= 1 ? W[top - 1] : 0, wm = top >= 2 ? W[top - 2] : 0;
    unsigned __int128 m = ((unsigned __int128)w1 << 64) | w0;
    if (z) m = (m << z) | (wm >> (64 - z));
    r.m = m;
    r.e = e + 64 * (top - 1) - z;
    r.zero = false;
    return r;
}

// Five unsigned 24-bit digits of a 120-bit integer in four words, least significant first.
__device__ __forceinline__ void digits24(const uint32_t w[4], int d[5])
{
    d[0] = (int)(w[0] & 0xFFFFFFu);
    d[1] = (int)(__funnelshift_r(w[0], w[1], 24) & 0xFFFFFFu);
    d[2] = (int)(__funnelshift_r(w[1], w[2], 16) & 0xFFFFFFu);
    d[3] = (int)(w[2] >> 8);
    d[4] = (int)(w[3] & 0xFFFFFFu);
}

// y pre-split for repeated use (GEMV's x vector): Y's digits, exponent, flags.
struct Dig {
    int d[5];
    int e;
    uint32_t flags;
    int pad;
};

__device__ __forceinline__ Dig to_dig(const Op &o)
{
    Dig g;
    digits24(o.w, g.d);
    g.e = o.e;
    g.flags = o.flags;
    g.pad = 0;
    return g;
}

struct Acc {
    long long c[6];   // column q has weight 2^(24(q+3) + B)
    int B;
    int cnt;
    bool init;
    bool bad;

    __device__ __forceinline__ void reset()
    {
#pragma unroll
        for (int q = 0; q < 6; ++q) c[q] = 0;
        B = 0;
        cnt = 0;
        init = false;
        bad = false;
    }

    // carries up: columns 0..4 end in [0, 2^24)
    __device__ __forceinline__ void normalize()
    {
#pragma unroll
        for (int q = 0; q < 5; ++q) {
            const long long carry = c[q] >> 24;
            c[q] -= carry << 24;
            c[q + 1] += carry;
        }
        cnt = 0;
    }

    // the sum as a 256-bit integer W with value W * 2^(B + 72)
    __device__ __forceinline__ void to_w256(uint64_t W[4]) const
    {
        W[0] = W[1] = W[2] = W[3] = 0;
#pragma unroll
        for (int q = 0; q < 6; ++q) add_shifted(W, c[q], 24 * q);
    }

    // move the block exponent up by d >= 1 bits (rare)
    __device__ __forceinline__ void raise(int d)
    {
        uint64_t W[4];
        to_w256(W);
        const uint64_t sgn = (uint64_t)((int64_t)W[3] >> 63);
        if (d >= 256) {
            W[0] = W[1] = W[2] = W[3] = 0;
        } else {
            while (d >= 64) {
                W[0] = W[1]; W[1] = W[2]; W[2] = W[3]; W[3] = sgn;
                d -= 64;
            }
            if (d) {
                W[0] = (W[0] >> d) | (W[1] << (64 - d));
                W[1] = (W[1] >> d) | (W[2] << (64 - d));
                W[2] = (W[2] >> d) | (W[3] << (64 - d));
                W[3] = (uint64_t)((int64_t)W[3] >> d);
            }
        }
        // back to columns: 24-bit chunks, the rest (signed) in the top column
        c[0] = (long long)(W[0] & 0xFFFFFFu);
        c[1] = (long long)((W[0] >> 24) & 0xFFFFFFu);
        c[2] = (long long)(((W[0] >> 48) | (W[1] << 16)) & 0xFFFFFFu);
        c[3] = (long long)((W[1] >> 8) & 0xFFFFFFu);
        c[4] = (long long)((W[1] >> 32) & 0xFFFFFFu);
        c[5] = (long long)((W[1] >> 56) | (W[2] << 8));   // bits 120..183 (the sum stays far below 2^183)
        cnt = 0;
    }

    // += x * y, y given as digits
    __device__ __forceinline__ void add_dig(const Op &x, const Dig &y)
    {
        add_core(x, y);
        if (++cnt >= 2048) normalize();
    }

    // add_dig without the carry bookkeeping: the caller runs normalize()
    // after at most 2048 of these (the column sums stay below 2^63).
    __device__ __forceinline__ void add_core(const Op &x, const Dig &y)
    {
        const uint32_t f = x.flags | y.flags;
        if (f & kBad) {
            bad = true;
            return;
        }
        if (f & kZero) return;
        const int ep = x.e + y.e;   // x*y = X*Y*2^ep, X < 2^118, Y < 2^118
        if (!init) {
            B = ep + 4;
            init = true;
        } else if (ep > B - 2) {
            const int nb = ep + 4;
            if (cnt) normalize();
            raise(nb - B);
            B = nb;
        }
        mul_at(x, y, B - ep);   // B - ep >= 2: X' = X >> sh < 2^116
    }

    // The block exponent set beforehand: B = ep_max + 4 for a bound ep_max on
    // the exponents x.e + y.e of every product that follows (then add_at
    // never has to move it).
    __device__ __forceinline__ void preset(int ep_max)
    {
        B = ep_max + 4;
        init = true;
    }

    // add_core after preset(): no first-term or raise branches
    __device__ __forceinline__ void add_at(const Op &x, const Dig &y)
    {
        const uint32_t f = x.flags | y.flags;
        if (f & kBad) {
            bad = true;
            return;
        }
        if (f & kZero) return;
        mul_at(x, y, B - (x.e + y.e));
    }

    // += X' * Y at the block, X' = X >> sh (sh >= 2)
    __device__ __forceinline__ void mul_at(const Op &x, const Dig &y, int sh)
    {
        if (sh >= 118) return;
        uint32_t xs[4];
        shr128(x.w, sh, xs);
        int a[5];
        digits24(xs, a);
        if ((x.flags ^ y.flags) & kNeg) {
#pragma unroll
            for (int t = 0; t < 5; ++t) a[t] = -a[t];
        }
        mads(a, y.d);
    }

    // Room for a group of products of exponents up to ep_max (the first
    // group fixes the block, later ones move it up when needed); the group
    // then goes in with mul_fast(x, y, B - ep), one test per group. (Where a
    // group moves the block, its smaller products are aligned to the new
    // block rather than shifted with the sum: the dropped bits, below 2^-130
    // of the block, can differ from add_core's one product at a time.)
    __device__ __forceinline__ void admit(int ep_max)
    {
        if (!init) {
            B = ep_max + 4;
            init = true;
        } else if (ep_max > B - 2) {
            const int nb = ep_max + 4;
            if (cnt) normalize();
            raise(nb - B);
            B = nb;
        }
    }

    // += X' * Y at the block, X' = X >> sh, for an operand from decode_fast
    // and the digit set of a finite nonzero value: no flag tests, the sign as
    // a factor of the digits, and the shift clamped instead of tested
    // (X < 2^118, so X >> sh is zero for every sh >= 118). At the same block,
    // the same sum as add_core.
    __device__ __forceinline__ void mul_fast(const Op &x, const Dig &y, int sh)
    {
        uint32_t xs[4];
        shr128(x.w, sh < 127 ? sh : 127, xs);
        int a[5];
        digits24(xs, a);
        const int sg = 1 - 2 * (int)((x.flags ^ y.flags) & kNeg);
#pragma unroll
        for (int t = 0; t < 5; ++t) a[t] *= sg;
        mads(a, y.d);
    }

    // the 19 digit products of weight >= 2^72, one 32 x 32 -> 64-bit
    // multiply-add each
    __device__ __forceinline__ void mads(const int a[5], const int *b)
    {
        madw(c[0], a[0], b[3]); madw(c[0], a[1], b[2]); madw(c[0], a[2], b[1]); madw(c[0], a[3], b[0]);
        madw(c[1], a[0], b[4]); madw(c[1], a[1], b[3]); madw(c[1], a[2], b[2]); madw(c[1], a[3], b[1]);
        madw(c[1], a[4], b[0]);
        madw(c[2], a[1], b[4]); madw(c[2], a[2], b[3]); madw(c[2], a[3], b[2]); madw(c[2], a[4], b[1]);
        madw(c[3], a[2], b[4]); madw(c[3], a[3], b[3]); madw(c[3], a[4], b[2]);
        madw(c[4], a[3], b[4]); madw(c[4], a[4], b[3]);
        madw(c[5], a[4], b[4]);
    }

    __device__ __forceinline__ static void madw(long long &acc, int x, int y)
    {
        asm("mad.wide.s32 %0, %1, %2, %0;" : "+l"(acc) : "r"(x), "r"(y));
    }

    // += a * b (decoded operands)
    __device__ __forceinline__ void add_prod(const Op &a, const Op &b) { add_dig(a, to_dig(b)); }

    __device__ __forceinline__ XF finish() const
    {
        XF r;
        r.neg = false;
        r.zero = true;
        r.m = 0;
        r.e = 0;
        if (!init) return r;
        uint64_t W[4];
        to_w256(W);
        return w256_to_xf(W, B + 72);
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

// A decoded operand in a 24-byte form.
struct OpPod {
    uint32_t w[4];
    int e;
    uint32_t flags;
};

__device__ __forceinline__ OpPod to_pod(const Op &o)
{
    OpPod p;
#pragma unroll
    for (int t = 0; t < 4; ++t) p.w[t] = o.w[t];
    p.e = o.e;
    p.flags = o.flags;
    return p;
}

__device__ __forceinline__ Op from_pod(const OpPod &p)
{
    Op o;
#pragma unroll
    for (int t = 0; t < 4; ++t) o.w[t] = p.w[t];
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
