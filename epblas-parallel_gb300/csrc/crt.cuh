// Chinese-remainder reconstruction of the Ozaki residue products in
// fractional fixed point.
//
// For pairwise-coprime moduli p_l with product M and residues c_l of an
// integer X with |X| < M/2:
//     X / M = frac( sum_l c_l * u_l / p_l ),  u_l = (M/p_l)^-1 mod p_l,
// taking the representative of the fraction in [-1/2, 1/2). The constants
// F_l = round(2^160 * u_l / p_l) are 160-bit fixed-point fractions; the sum
// sum_l c_l F_l is accumulated modulo 2^160 (the integer part of the sum is
// the multiple of M to drop, so the carries out of the top limb are simply
// discarded). The error of the sum is at most nmod * max(c) / 2 * 2^-160 of a
// unit, so X comes out with an absolute error below M * 2^-145, far below
// the product's own scale. Only the final |T| * M (T the signed fraction) is
// formed as an extended float.
//
// Against a plain integer CRT (sum_l c_l W_l with W_l = u_l M/p_l, a
// correction q*M and a sign fix, all on ~300-bit integers) this needs 5
// instead of 9 limb products per residue and no quotient estimate.
//
// __host__ __device__ so the same code is unit-tested on the CPU.
#pragma once
#include "xfloat.cuh"
#include "xword.cuh"

#ifdef __CUDACC__
#define CRT_HD __host__ __device__ __forceinline__
#else
#define CRT_HD inline
#endif

namespace crt {

// The 128-bit extended float of xfloat.cuh in 32-bit words.
CRT_HD xw::XW to_xw(const xfp::XF &x)
{
    if (x.zero) return xw::zero();
    xw::XW r;
    r.w[3] = (uint32_t)(x.m >> 96);
    r.w[2] = (uint32_t)(x.m >> 64);
    r.w[1] = (uint32_t)(x.m >> 32);
    r.w[0] = (uint32_t)x.m;
    r.e = x.e;
    r.neg = x.neg ? 1u : 0u;
    return r;
}

constexpr int kFL = 5;       // 32-bit limbs of the 160-bit fractions
constexpr int kFLPad = 8;    // row stride (two 16-byte vectors)

struct Frac {
    uint64_t S[kFL];

    CRT_HD void reset()
    {
        for (int t = 0; t < kFL; ++t) S[t] = 0;
    }
    // F: the 160-bit constant of this modulus (little-endian limbs).
    CRT_HD void add(const uint32_t *F, uint32_t c)
    {
        for (int t = 0; t < kFL; ++t) S[t] += (uint64_t)c * F[t];
    }
    // X * 2^-S2 as an extended float; Mx = M as an extended float.
    CRT_HD xfp::XF finish(const xfp::XF &Mx, int S2) const
    {
        uint32_t x[kFL];
        uint64_t carry = 0;
        for (int t = 0; t < kFL; ++t) {
            uint64_t v = S[t] + carry;
            x[t] = (uint32_t)v;
            carry = v >> 32;
        }
        const bool neg = (x[kFL - 1] >> 31) != 0;
        if (neg) {
            uint64_t cy = 1;
            for (int t = 0; t < kFL; ++t) {
                uint64_t v = (uint64_t)(uint32_t)~x[t] + cy;
                x[t] = (uint32_t)v;
                cy = v >> 32;
            }
        }
        // 160-bit |T| as (hi 128 bits, lo 32 bits)
        unsigned __int128 hi = ((unsigned __int128)(((uint64_t)x[4] << 32) | x[3]) << 64) |
                               (((uint64_t)x[2] << 32) | x[1]);
        uint32_t lo = x[0];
        xfp::XF t;
        if (hi == 0 && lo == 0) {
            t.zero = true; t.neg = false; t.m = 0; t.e = 0;
            return t;
        }
        // top 128 bits of the 160-bit value, value = m * 2^e
        int e;
        unsigned __int128 m;
        if (hi != 0) {
            const int z = xfp::clz128(hi);
            const unsigned __int128 L = (unsigned __int128)lo;
            m = (hi << z) | (z <= 32 ? (L >> (32 - z)) : (L << (z - 32)));
            e = 32 - z - 160;
        } else {
            m = (unsigned __int128)lo;
            e = -160;
        }
        t = xfp::xf_norm(neg, m, e);
        xfp::XF r = xfp::xf_mul(t, Mx);
        r.e -= S2;
        return r;
    }
    // The same value in 32-bit words: X * 2^-S2 = T * M * 2^-S2 with T the
    // signed 160-bit fraction; Mx = M (times any folded scale factor).
    CRT_HD xw::XW finish_xw(const xw::XW &Mx, int S2) const
    {
        uint32_t x[kFL];
        uint32_t carry = 0;
        for (int t = 0; t < kFL; ++t) {
            const uint64_t v = S[t] + carry;
            x[t] = (uint32_t)v;
            carry = (uint32_t)(v >> 32);
        }
        const uint32_t neg = x[kFL - 1] >> 31;
        if (neg) {
            uint32_t c = 1;
            for (int t = 0; t < kFL; ++t) {
                const uint32_t v = ~x[t] + c;
                c = c & (x[t] == 0u);
                x[t] = v;
            }
        }
        // normalise |T| (bit 159 set), keep the top 128 bits
        int sh = 0;
        for (int k = 0; k < kFL - 1 && x[kFL - 1] == 0u; ++k) {
            for (int t = kFL - 1; t > 0; --t) x[t] = x[t - 1];
            x[0] = 0u;
            sh += 32;
        }
        if (x[kFL - 1] == 0u) return xw::zero();
        const int z = xw::clz32(x[kFL - 1]);
        xw::XW r;
        if (z) {
            for (int t = kFL - 1; t > 0; --t) x[t] = xw::fshl(x[t - 1], x[t], z);
            sh += z;
        }
        r.w[3] = x[4];
        r.w[2] = x[3];
        r.w[1] = x[2];
        r.w[0] = x[1];
        r.e = -128 - sh;
        r.neg = neg;
        r = xw::mul(r, Mx);
        r.e -= S2;
        return r;
    }
};

// ---- host: constants ------------------------------------------------------------

inline int64_t inv_mod(int64_t a, int64_t m)
{
    int64_t g = m, x = 0, x1 = 1, a1 = a % m;
    while (a1) {
        int64_t q = g / a1;
        int64_t t = g - q * a1; g = a1; a1 = t;
        t = x - q * x1; x = x1; x1 = t;
    }
    return ((x % m) + m) % m;
}

// F[l] = round(2^160 * u_l / p_l) and M = prod p_l as an extended float
// (truncated to 128 bits). At most 40 moduli below 2^9.
inline void constants(const int *p, int n, uint32_t (*F)[kFLPad], xfp::XF &Mx)
{
    constexpr int NL = 12;
    uint32_t M[NL] = {1};
    for (int l = 0; l < n; ++l) {
        uint64_t carry = 0;
        for (int t = 0; t < NL; ++t) {
            uint64_t v = (uint64_t)M[t] * (uint32_t)p[l] + carry;
            M[t] = (uint32_t)v;
            carry = v >> 32;
        }
    }
    for (int l = 0; l < n; ++l) {
        int64_t r = 1;
        for (int j = 0; j < n; ++j)
            if (j != l) r = r * (p[j] % p[l]) % p[l];
        const uint32_t u = (uint32_t)inv_mod(r, p[l]);
        // (u * 2^160 + floor(p/2)) / p, six limbs, long division by a small divisor
        uint32_t N[6] = {(uint32_t)(p[l] / 2), 0, 0, 0, 0, u};
        uint64_t rem = 0;
        for (int t = 5; t >= 0; --t) {
            uint64_t cur = (rem << 32) | N[t];
            N[t] = (uint32_t)(cur / (uint32_t)p[l]);
            rem = cur % (uint32_t)p[l];
        }
        for (int t = 0; t < kFLPad; ++t) F[l][t] = t < kFL ? N[t] : 0u;
    }
    int top = NL - 1;
    while (top > 0 && M[top] == 0) --top;
    auto limb = [&](int t) -> uint32_t { return t >= 0 ? M[t] : 0u; };
    unsigned __int128 m = ((unsigned __int128)(((uint64_t)limb(top) << 32) | limb(top - 1)) << 64) |
                          (((uint64_t)limb(top - 2) << 32) | limb(top - 3));
    int e = 32 * (top - 3);
    const int z = xfp::clz128(m);   // < 32: the top limb is nonzero
    if (z) m = (m << z) | (unsigned __int128)(limb(top - 4) >> (32 - z));
    Mx.m = m;
    Mx.e = e - z;
    Mx.neg = false;
    Mx.zero = false;
}

}  // namespace crt
