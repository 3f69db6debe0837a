// Integer-exact tensor-core double-double GEMM ("Ozaki" engine).
//
// Scheme (Ozaki scheme II: Ozaki, Uchino, Imamura, "Ozaki Scheme II: A
// GEMM-oriented emulation of floating-point matrix multiplication using an
// integer modular technique", 2025), adapted to what sm_103a offers:
//
//  1. Scaling. Row i of op(A) and column j of op(B) are scaled by powers of
//     two so that every entry becomes an integer of at most `bits` bits:
//     A'_ip = round(a_ip * 2^(bits-2-ea_i)), B'_pj likewise (ea_i, eb_j bound
//     the binary exponents of the row / column). The error of this step is
//     <= 2^(3-bits) of max|row| * max|column| per product, i.e. normwise.
//  2. Residues. A'B' is an integer matrix with |entries| <= k * 2^(2 bits - 2).
//     It is computed exactly modulo L pairwise-coprime moduli p_l <= 361 whose
//     product M exceeds 2^4 * k * 2^(2 bits - 1). Each residue matrix (entries
//     in [-(p-1)/2, (p-1)/2], |r| <= 180) is exact in fp16.
//  3. Residue GEMMs on the tensor cores. sm_103a's tcgen05 has no integer
//     kind (kind::i8 is rejected by ptxas for sm_103a), so the residue GEMMs
//     use kind::f16 with fp32 accumulation in tensor memory. Products of
//     residues are exact; an fp32 sum stays exact while it is an integer
//     below 2^24. K is therefore processed in chunks of 512
//     (512 * 180^2 + 361 < 2^24) and after each chunk the accumulator is
//     reduced modulo p in place; two accumulators alternate so the MMA pipe
//     keeps running while the epilogue reduces the other one.
//  4. CRT reconstruction (integer only): X = sum_l c_l * W_l - q * M with
//     W_l = (M/p_l) * ((M/p_l)^-1 mod p_l) and q = round(sum_l c_l u_l / p_l)
//     estimated in fp32 (exact because |X| << M by construction), then the
//     top 106 bits of X become the double-double (hi, lo) with exponents
//     built directly, scaled back by 2^-(sA_i + sB_j); the alpha/beta update
//     runs in double-double on the FP64 pipe, which the scheme otherwise
//     does not touch.
//
// A modulus count L of ~27 (8192^3, bits = 106) replaces the 18 FP64
// instructions per multiply-add of the reference's kernel by 27 fp16
// tensor-core multiply-adds.
#include <cuda.h>
#include <cuda_fp16.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <map>
#include <tuple>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <vector>

#include "dd.cuh"
#include "level3.h"
#include "runtime.h"
#include "sm100.cuh"
#include "crt.cuh"
#include "fixacc.cuh"
#include "xfloat.cuh"

namespace mw {

namespace {

constexpr int kMaxMod = 40;
constexpr int kResLimbs = 11;   // 11-bit limbs of |A'| (bits <= 120)
constexpr int kNoExp = -30000;
constexpr int kMaxP = 361;      // largest modulus: residues |r| <= 180 are exact in fp16
constexpr int kChunk = 512;     // K per exact fp32 chunk: 512 * 180^2 + 361 < 2^24

// ---- host-side moduli / CRT constants --------------------------------------------------

struct Moduli {
    int n = 0;
    int p[kMaxMod];
};

struct OzResParams {
    int nmod;
    float p[kMaxMod], invp[kMaxMod];
    float t[kMaxMod][kResLimbs];   // 2^(11k) mod p, symmetric representative
};

// Per residue-GEMM batch entry z (component * nmod + modulus).
struct OzModParams {
    float p[3 * kMaxMod], invp[3 * kMaxMod];
};

struct OzCrtParams {
    int nmod;
    uint32_t F[kMaxMod][crt::kFLPad];   // 160-bit fractions u_l / p_l
    float pm[kMaxMod];
    uint64_t Mhi, Mlo;                  // M = (Mhi:Mlo) * 2^Me, truncated
    int Me;
};

int gcd(int a, int b) { return b ? gcd(b, a % b) : a; }

// The largest pairwise-coprime moduli <= kMaxP (greedy from the top), enough
// of them for `need_bits` bits of product.
Moduli choose_moduli(double need_bits)
{
    Moduli md;
    double have = 0.0;
    for (int c = kMaxP; c >= 3 && have < need_bits && md.n < kMaxMod; --c) {
        bool ok = true;
        for (int i = 0; i < md.n && ok; ++i) ok = gcd(md.p[i], c) == 1;
        if (!ok) continue;
        md.p[md.n++] = c;
        have += std::log2((double)c);
    }
    return md;
}

int g_last_moduli = 0;
int g_last_bits[2] = {0, 0};   // bits of op(A), op(B) in the most recent call
int g_mma_kind = -1;   // 0 tcgen05 per tile, 1 SIMT cross-check, 2 tcgen05 persistent, 3 CTA pairs (default)

// Failure injection for the bounded-wait path: the next g_lose_loads launches
// of the CTA-pair residue GEMM issue no operand loads (see k_oz_gemm_tc_2sm).
std::atomic<int> g_lose_loads{0};
int take_lost_load_injection()
{
    int v = g_lose_loads.load();
    while (v > 0 && !g_lose_loads.compare_exchange_weak(v, v - 1)) {
    }
    return v > 0 ? 1 : 0;
}

// Optional per-phase timing with CUDA events on the library stream.
enum { PH_EXP = 0, PH_RES, PH_GEMM, PH_REC, PH_N };
bool g_timing = false;
thread_local cudaEvent_t t_ev[PH_N + 1] = {};
thread_local float t_phase_ms[PH_N] = {};

// Residue GEMM launches of a blocked product, timed one by one (their sum is
// the GEMM phase; the rest of the block loop is reported as reconstruction).
constexpr int kTimedGemms = 64;
thread_local cudaEvent_t t_gev[2 * kTimedGemms] = {};
thread_local int t_gemm_n = 0;

void phase_mark(int i)
{
    if (!g_timing) return;
    if (i == PH_EXP) t_gemm_n = 0;
    if (!t_ev[i]) cudaEventCreate(&t_ev[i]);
    cudaEventRecord(t_ev[i], stream());
}

void gemm_mark(bool begin)
{
    if (!g_timing) return;
    const int i = 2 * t_gemm_n + (begin ? 0 : 1);
    if (i >= 2 * kTimedGemms) return;
    if (!t_gev[i]) cudaEventCreate(&t_gev[i]);
    cudaEventRecord(t_gev[i], stream());
    if (!begin) ++t_gemm_n;
}

void phase_collect()
{
    if (!g_timing) return;
    cudaEventSynchronize(t_ev[PH_N]);
    for (int i = 0; i < PH_N; ++i) {
        float ms = 0.0f;
        if (t_ev[i] && t_ev[i + 1]) cudaEventElapsedTime(&ms, t_ev[i], t_ev[i + 1]);
        t_phase_ms[i] = ms;
    }
    if (t_gemm_n > 0) {
        float sum = 0.0f;
        for (int i = 0; i < t_gemm_n && i < kTimedGemms; ++i) {
            float ms = 0.0f;
            cudaEventElapsedTime(&ms, t_gev[2 * i], t_gev[2 * i + 1]);
            sum += ms;
        }
        const float span = t_phase_ms[PH_GEMM] + t_phase_ms[PH_REC];
        t_phase_ms[PH_GEMM] = sum;
        t_phase_ms[PH_REC] = span > sum ? span - sum : 0.0f;
    }
}

int mma_kind()
{
    if (g_mma_kind < 0) {
        const char *e = getenv("MWBLAS_OZAKI_MMA");
        g_mma_kind = (e && !strcmp(e, "simt"))         ? 1
                     : (e && !strcmp(e, "pertile"))    ? 0
                     : (e && !strcmp(e, "persistent")) ? 2
                                                       : 3;
    }
    return g_mma_kind;
}

// ---- device: residues -----------------------------------------------------------------------

// rint(y) for |y| < 2^22 with two FP32 adds (round-to-nearest-even on the
// 1.5 * 2^23 grid), keeping the rounding off the conversion unit.
__device__ __forceinline__ float rint_small(float y)
{
    return __fsub_rn(__fadd_rn(y, 12582912.0f), 12582912.0f);
}

// The low 16 bits of a float holding an integer 0 <= v < 2^16, without a
// float-to-int conversion (v + 2^23 puts the integer in the mantissa).
__device__ __forceinline__ uint32_t small_uint(float v)
{
    return __float_as_uint(__fadd_rn(v, 8388608.0f)) & 0xFFFFu;
}


__device__ __forceinline__ float u11_to_float(uint32_t c)
{
    return __int_as_float(0x4B000000 | c) - 8388608.0f;   // exact for c < 2^23
}

// op(X) is rows x kdim; element (r, c) lives at X[r + c*ld] (ROWC) or
// X[c + r*ld]. Writes out[l][r][c] (fp16, row stride kpad) for the padded
// ranges r < rows_pad, c < kpad (zeros outside op(X)).
// Integer image F = round(v * 2^sc) of a double-double, as sign and 11-bit
// limbs of |F| (bits <= 120 keeps |F| below 2^121).
__device__ __forceinline__ void to_limbs(double2 v, int sc, float (&fl)[kResLimbs], bool &neg)
{
    // |v| = W * 2^e exactly (fixacc.cuh's decode, 32-bit words); F = round(|v| * 2^sc) = round(W * 2^-r)
    const fx::Op o = fx::decode(v);
    neg = (o.flags & fx::kNeg) != 0;
    uint32_t y[4] = {0u, 0u, 0u, 0u};
    const int r = -(o.e + sc);
    if (!(o.flags & (fx::kZero | fx::kBad)) && r >= 1 && r < 128) {
        fx::shr128(o.w, r, y);
        // rounding bit: bit r - 1 of W
        const int rb = r - 1, wq = rb >> 5;
        const uint32_t word = wq == 0 ? o.w[0] : (wq == 1 ? o.w[1] : (wq == 2 ? o.w[2] : o.w[3]));
        asm("add.cc.u32 %0, %0, %4;\n\t"
            "addc.cc.u32 %1, %1, 0;\n\t"
            "addc.cc.u32 %2, %2, 0;\n\t"
            "addc.u32 %3, %3, 0;"
            : "+r"(y[0]), "+r"(y[1]), "+r"(y[2]), "+r"(y[3])
            : "r"((word >> (rb & 31)) & 1u));
    }
    // 11-bit limbs: bits [11q, 11q + 11) of the 128-bit F
#pragma unroll
    for (int q = 0; q < kResLimbs; ++q) {
        const int b = 11 * q, w = b >> 5, sh = b & 31;
        const uint32_t lo = y[w], hi = (w + 1 < 4) ? y[w + 1] : 0u;
        fl[q] = u11_to_float(__funnelshift_r(lo, hi, sh) & 0x7FFu);
    }
}

// Symmetric residues modulo p of two integers F given as signed 11-bit limbs
// (|limb| <= 2047), with packed FP32 arithmetic (two lanes per instruction).
// With symmetric constants |t_q| <= p/2 the limb dot product x is an exact
// fp32 integer, |x| <= 11 * 2047 * p/2 < 2^22. The quotient estimate
// y = fl(x * fl(1/p)) is within 11258 * 2^-24 + 2^-11 < 0.0012 of x/p; for odd
// p, x/p is at least 1/(2p) >= 0.0013 away from a half-integer, so rint(y) is
// the nearest integer to x/p and x - p * rint(y) (exact) lies in [-p/2, p/2].
// For even p the same holds except at exact half-integers, where either
// neighbour gives a residue of +-p/2. No correction step is needed.
__device__ __forceinline__ float2 sym_residue2(const float2 (&fl)[kResLimbs], const float2 (&t)[12], float2 negp,
                                               float2 invp)
{
    float2 x = __fmul2_rn(fl[0], t[0]);
#pragma unroll
    for (int q = 1; q < kResLimbs; ++q) x = __ffma2_rn(fl[q], t[q], x);
    float2 y = __fmul2_rn(x, invp);
    y = __fadd2_rn(y, make_float2(12582912.0f, 12582912.0f));    // rint for |y| < 2^22
    y = __fadd2_rn(y, make_float2(-12582912.0f, -12582912.0f));
    return __ffma2_rn(y, negp, x);
}

// (a + b) wrapped back into [-p/2, p/2] for |a|, |b| <= p/2: the quotient is
// -1, 0 or 1 and the estimate of (a + b)/p is exact to 2^-22.
__device__ __forceinline__ float2 sym_wrap2(float2 a, float2 b, float2 negp, float2 invp)
{
    const float2 x = __fadd2_rn(a, b);
    float2 y = __fmul2_rn(x, invp);
    y = __fadd2_rn(y, make_float2(12582912.0f, 12582912.0f));
    y = __fadd2_rn(y, make_float2(-12582912.0f, -12582912.0f));
    return __ffma2_rn(y, negp, x);
}

__device__ __forceinline__ void store4h(__half *dst, float2 a, float2 b)
{
    const __half2 ha = __floats2half2_rn(a.x, a.y), hb = __floats2half2_rn(b.x, b.y);
    uint2 u;
    u.x = *reinterpret_cast<const uint32_t *>(&ha);
    u.y = *reinterpret_cast<const uint32_t *>(&hb);
    *reinterpret_cast<uint2 *>(dst) = u;
}

// op(X) is rows x kdim; element (r, c) lives at X[r + c*ld] (ROWC) or
// X[c + r*ld] (complex elements are two double2). Writes the residues for
// every modulus as fp16, out[comp][l][r][c] (row stride kpad, component stride
// nmod*rows_pad*kpad), over the padded ranges r < rows_pad, c < kpad (zeros
// outside op(X)). Real: one component. Complex: the real part, the imaginary
// part (negated when `conj`) and their sum, for the 3-product (Karatsuba)
// complex multiply. A block converts a 32 x 32 tile; each thread converts four
// consecutive elements of one row, so every modulus constant read from shared
// memory serves four elements and the four residues leave as one 8-byte store.
__device__ __forceinline__ void cp_async16(void *smem, const void *gmem, int src_bytes)
{
    const uint32_t sa = (uint32_t)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(sa), "l"(gmem), "r"(src_bytes) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait1() { asm volatile("cp.async.wait_group 1;\n" ::: "memory"); }

template <bool CPLX>
constexpr size_t residue_smem_bytes()
{
    return 2 * 32 * 33 * (CPLX ? 2 : 1) * sizeof(double2);
}

// Signed 11-bit limbs of the four elements cg .. cg + 3 of one staged tile row
// (E double2 per element: E = 2 complex, the imaginary part negated when
// conj), scaled by 2^(bits - 2 - e); rows without a live exponent give zeros.
// Elements (cg, cg+1) and (cg+2, cg+3) share the two lanes of fr[0] / fr[1].
template <bool CPLX>
__device__ __forceinline__ void tile_limbs(const double2 (*row)[CPLX ? 2 : 1], int cg, int e, int bits, int conj,
                                           float2 (&fr)[2][kResLimbs], float2 (&fi)[CPLX ? 2 : 1][kResLimbs])
{
    constexpr int E = CPLX ? 2 : 1;
    const bool live = e > kNoExp / 2;
    const int sc = bits - 2 - e;
#pragma unroll
    for (int v = 0; v < 4; ++v) {
        float f[kResLimbs];
        bool ng = false;
        if (live) {
            to_limbs(row[cg + v][0], sc, f, ng);
        } else {
#pragma unroll
            for (int q = 0; q < kResLimbs; ++q) f[q] = 0.0f;
        }
#pragma unroll
        for (int q = 0; q < kResLimbs; ++q) {
            const float sv = ng ? -f[q] : f[q];
            if (v & 1) fr[v >> 1][q].y = sv;
            else fr[v >> 1][q].x = sv;
        }
        if (CPLX) {
            bool ngi = false;
            if (live) {
                to_limbs(row[cg + v][E - 1], sc, f, ngi);
                if (conj) ngi = !ngi;
            }
#pragma unroll
            for (int q = 0; q < kResLimbs; ++q) {
                const float sv = ngi ? -f[q] : f[q];
                if (v & 1) fi[CPLX ? v >> 1 : 0][q].y = sv;
                else fi[CPLX ? v >> 1 : 0][q].x = sv;
            }
        }
    }
}

// The residues of those four elements for every modulus (constants in shared
// memory), four fp16 per 8-byte store at o + l * plane; complex also writes
// the imaginary part and the sum (Karatsuba) at o + cstride and o + 2 cstride.
template <bool CPLX>
__device__ __forceinline__ void store_residues(const float2 (&fr)[2][kResLimbs],
                                               const float2 (&fi)[CPLX ? 2 : 1][kResLimbs], int nmod,
                                               const float2 (*s_t)[12], const float4 *s_pp, __half *o, int64_t plane,
                                               int64_t cstride)
{
    for (int l = 0; l < nmod; ++l) {
        float2 t[12];
#pragma unroll
        for (int q = 0; q < 12; q += 2) {
            const float4 u = *reinterpret_cast<const float4 *>(&s_t[l][q]);
            t[q] = make_float2(u.x, u.y);
            t[q + 1] = make_float2(u.z, u.w);
        }
        const float4 pp = s_pp[l];
        const float2 negp = make_float2(pp.x, pp.y), invp = make_float2(pp.z, pp.w);
        const float2 ra = sym_residue2(fr[0], t, negp, invp), rb = sym_residue2(fr[1], t, negp, invp);
        store4h(o, ra, rb);
        if (CPLX) {
            const float2 ia = sym_residue2(fi[0], t, negp, invp), ib = sym_residue2(fi[CPLX ? 1 : 0], t, negp, invp);
            store4h(o + cstride, ia, ib);
            store4h(o + 2 * cstride, sym_wrap2(ra, ia, negp, invp), sym_wrap2(rb, ib, negp, invp));
        }
        o += plane;
    }
}

template <bool ROWC, bool CPLX>
__global__ void __launch_bounds__(256) k_oz_residues(int64_t rows, int64_t kdim, const double2 *__restrict__ X,
                                                     int64_t ld, const int *__restrict__ rexp, int bits,
                                                     OzResParams P, __half *__restrict__ out, int64_t rows_pad,
                                                     int64_t kpad, int conj, int64_t plane_rows)
{
    constexpr int E = CPLX ? 2 : 1;
    extern __shared__ __align__(16) unsigned char res_smem[];
    typedef double2 Tile[32][33][E];
    Tile *tiles = reinterpret_cast<Tile *>(res_smem);   // two buffers
    __shared__ __align__(16) float2 s_t[kMaxMod][12];   // {t, t}
    __shared__ __align__(16) float4 s_pp[kMaxMod];      // {-p, -p, 1/p, 1/p}
    const int nmod = P.nmod;
    for (int i = threadIdx.x; i < nmod * 12; i += blockDim.x) {
        int l = i / 12, q = i % 12;
        const float t = (q < kResLimbs) ? P.t[l][q] : 0.0f;
        s_t[l][q] = make_float2(t, t);
    }
    for (int i = threadIdx.x; i < nmod; i += blockDim.x)
        s_pp[i] = make_float4(-P.p[i], -P.p[i], P.invp[i], P.invp[i]);
    const int ntc = (int)(kpad / 32);
    const int ntiles = ntc * (int)(rows_pad / 32);
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    // Tile loads go through cp.async into the other buffer while this tile is
    // converted (zero fill outside op(X)).
    auto issue = [&](int tile, int buf) {
        const int64_t r0 = (int64_t)(tile / ntc) * 32, c0 = (int64_t)(tile % ntc) * 32;
        for (int s = ty; s < 32; s += 8) {
            const int64_t r = ROWC ? r0 + tx : r0 + s;
            const int64_t c = ROWC ? c0 + s : c0 + tx;
            const bool ok = r < rows && c < kdim;
            const double2 *src = ok ? X + E * (ROWC ? r + c * ld : c + r * ld) : X;
#pragma unroll
            for (int w = 0; w < E; ++w)
                cp_async16(ROWC ? &tiles[buf][tx][s][w] : &tiles[buf][s][tx][w], src + (ok ? w : 0), ok ? 16 : 0);
        }
    };
    int tile = blockIdx.x, buf = 0;
    if (tile < ntiles) issue(tile, 0);
    cp_async_commit();
    const int s = threadIdx.x >> 3, cg = (threadIdx.x & 7) * 4;
    for (; tile < ntiles; tile += gridDim.x, buf ^= 1) {
        const int next = tile + gridDim.x;
        if (next < ntiles) issue(next, buf ^ 1);
        cp_async_commit();
        cp_async_wait1();   // this tile's group has landed
        __syncthreads();
        const int64_t r = (int64_t)(tile / ntc) * 32 + s, cb = (int64_t)(tile % ntc) * 32 + cg;
        const int e = (r < rows) ? rexp[r] : kNoExp;
        // signed limbs of elements (cg, cg+1) and (cg+2, cg+3) in the two lanes
        float2 fr[2][kResLimbs], fi[CPLX ? 2 : 1][kResLimbs];
        tile_limbs<CPLX>(tiles[buf][s], cg, e, bits, conj, fr, fi);
        __syncthreads();   // the buffer is refilled two iterations on; the limbs are in registers
        store_residues<CPLX>(fr, fi, nmod, s_t, s_pp, out + (r * kpad + cb), plane_rows * kpad,
                             (int64_t)nmod * plane_rows * kpad);
    }
}

// One block per SM slot (as many as fit), each walking tiles with the next
// tile's load in flight.
template <bool ROWC, bool CPLX>
void launch_residues(int64_t rows, int64_t kdim, const double2 *X, int64_t ld, const int *rexp, int bits,
                     const OzResParams &rp, __half *out, int64_t rows_pad, int64_t kpad, int conj,
                     int64_t plane_rows = -1)
{
    if (plane_rows < 0) plane_rows = rows_pad;
    static int per_sm[64];   // resident blocks per SM, per device (0 = not queried yet)
    const size_t smem = residue_smem_bytes<CPLX>();
    int dev = 0;
    cudaGetDevice(&dev);
    cudaFuncSetAttribute(k_oz_residues<ROWC, CPLX>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    int &b = per_sm[dev & 63];
    if (b <= 0) {
        int q = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&q, k_oz_residues<ROWC, CPLX>, 256, smem);
        b = q > 0 ? q : 1;
    }
    const int64_t ntiles = (kpad / 32) * (rows_pad / 32);
    int64_t grid = (int64_t)b * device_sm_count();
    if (grid > ntiles) grid = ntiles;
    if (grid < 1) grid = 1;
    k_oz_residues<ROWC, CPLX><<<(unsigned)grid, 256, smem, stream()>>>(rows, kdim, X, ld, rexp, bits, rp, out, rows_pad,
                                                                        kpad, conj, plane_rows);
    count_launch();
}

// ---- device: residues on the tensor cores -------------------------------------------------
//
// The limb dot products x_l = sum_q c_q * t_lq (c_q the 10-bit limbs of the
// scaled integer, t_lq = 2^(10q) mod p_l, symmetric) are a small matrix
// product, so they run as tcgen05 MMAs instead of FMAs per element and
// modulus. Row i of the A operand (K = 64 fp16, 128-byte swizzled rows,
// written by thread i) holds four consecutive elements of op(X), 16 halves
// each: the limbs as s * (1024 + c_q) for q < 13 (fp16 0x6400 | c_q with the
// element's sign bit: no conversion instruction), then -s * 1024 twice, then
// a zero. B is block-diagonal: row v * 32 + l holds, at halves 16 v .. 16 v +
// 15, t_l0 .. t_l12, then T1, T2 with T1 + T2 = sum_q t_lq (|T1|, |T2| <=
// 1170, exact in fp16), then 0, so the offsets cancel exactly:
//     x = s * sum_q (1024 + c_q) t_lq - s * 1024 (T1 + T2) = s * sum_q c_q t_lq.
// Every partial sum is an integer below 13 * 2047 * 180 + 2 * 1024 * 1170 <
// 2^23 (exact in fp32) and |x| <= 13 * 1023 * 180 < 2^22, so the symmetric
// reduction of the FMA path (quotient estimate, no correction step) applies
// and both paths store the same residues.
//
// Four MMAs of M = 128, N = 32, K = 16 (one per element slot v) leave x for
// element v, modulus l in TMEM column v * 32 + l of lane i. A tile is 16 rows
// x 32 k of op(X) (thread i: row i / 8, k 4 (i % 8) .. + 3; a warp stores 4
// rows x 64 bytes per modulus). Up to four CTAs share an SM (128 TMEM columns
// each); in each CTA the limbs of tile t + 1 are written while the MMA of
// tile t runs (two A tiles), and the epilogue of tile t runs before the MMA
// of tile t + 1 reuses the TMEM columns.
constexpr int RT_ROWS = 16, RT_COLS = 32, RT_THREADS = 128;
constexpr int RT_TILE_BYTES = 128 * 128;   // 128 rows x 64 fp16
// Two A tiles and B, barriers; sized so that at most four CTAs (4 x 128 TMEM
// columns) share an SM.
constexpr int RT_SMEM = 56 * 1024;
constexpr int RT_MAX_MOD = 32;
constexpr int RT_LIMBS = 13;   // 10-bit limbs of |F| < 2^121 (bits <= 120)

// Chunk j (halves 8j .. 8j + 7) of a 128-byte operand row, 128-byte swizzle.
__device__ __forceinline__ void st_row_chunk(uint8_t *tile, int row, int j, uint4 v)
{
    *reinterpret_cast<uint4 *>(tile + row * 128 + ((j ^ (row & 7)) << 4)) = v;
}

__device__ __forceinline__ uint32_t h2_bits(float a, float b)
{
    const __half2 h = __floats2half2_rn(a, b);
    return *reinterpret_cast<const uint32_t *>(&h);
}

// F = round(|v| * 2^sc) as four words (0 for zero and non-finite entries;
// the caller's exponent bound keeps F below 2^121), and the sign of v.
__device__ __forceinline__ void scaled_int(double2 v, int sc, uint32_t (&y)[4], bool &neg)
{
    const fx::Op o = fx::decode(v);
    neg = (o.flags & fx::kNeg) != 0;
    y[0] = y[1] = y[2] = y[3] = 0u;
    const int r = -(o.e + sc);
    if (!(o.flags & (fx::kZero | fx::kBad)) && r >= 1 && r < 128) {
        fx::shr128(o.w, r, y);
        const int rb = r - 1, wq = rb >> 5;
        const uint32_t word = wq == 0 ? o.w[0] : (wq == 1 ? o.w[1] : (wq == 2 ? o.w[2] : o.w[3]));
        asm("add.cc.u32 %0, %0, %4;\n\t"
            "addc.cc.u32 %1, %1, 0;\n\t"
            "addc.cc.u32 %2, %2, 0;\n\t"
            "addc.u32 %3, %3, 0;"
            : "+r"(y[0]), "+r"(y[1]), "+r"(y[2]), "+r"(y[3])
            : "r"((word >> (rb & 31)) & 1u));
    }
}

// Halves 2w, 2w + 1 of an element's A row: limbs 2w, 2w + 1 as 0x6400 | c
// with the sign bit s; past limb 12 the two offset corrections and a zero.
template <int W>
__device__ __forceinline__ uint32_t limb_word(const uint32_t (&y)[4], uint32_t s)
{
    constexpr int b = 20 * W, wd = b >> 5, sh = b & 31;
    const uint32_t corr = 0xE400u ^ (s & 0xFFFFu);   // -s * 1024
    if (W < 6) {
        const uint32_t g = __funnelshift_r(y[wd], wd + 1 < 4 ? y[wd + 1] : 0u, sh);   // bits b .. b + 31
        return ((g & 0x3FFu) | ((g & 0xFFC00u) << 6) | 0x64006400u) ^ s;
    } else if (W == 6) {
        const uint32_t c12 = (__funnelshift_r(y[3], 0u, 120 - 96) & 0x3FFu);   // bits 120 .. 129
        return ((c12 | 0x6400u) ^ (s & 0xFFFFu)) | (corr << 16);
    } else {
        return corr;
    }
}

// B of the tensor-core residue conversion, row tid = v * 32 + l (block-diagonal).
__device__ __forceinline__ void rt_constants(uint8_t *sB, const OzResParams &P, int tid)
{
    const int v = tid >> 5, l = tid & 31;
    float t[16];
#pragma unroll
    for (int q = 0; q < 16; ++q) t[q] = 0.0f;
    if (l < P.nmod) {
        const int p = (int)P.p[l];
        int pw = 1, sum = 0;
#pragma unroll
        for (int q = 0; q < RT_LIMBS; ++q) {
            const int ts = pw > p / 2 ? pw - p : pw;
            t[q] = (float)ts;
            sum += ts;
            pw = (pw * 1024) % p;
        }
        t[RT_LIMBS] = (float)(sum / 2);
        t[RT_LIMBS + 1] = (float)(sum - sum / 2);
    }
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        uint4 w = make_uint4(0u, 0u, 0u, 0u);
        if ((j >> 1) == v) {
            const int q0 = (j & 1) * 8;
            w = make_uint4(h2_bits(t[q0], t[q0 + 1]), h2_bits(t[q0 + 2], t[q0 + 3]), h2_bits(t[q0 + 4], t[q0 + 5]),
                           h2_bits(t[q0 + 6], t[q0 + 7]));
        }
        st_row_chunk(sB, tid, j, w);
    }
}

// A row tid: the limbs of four elements scaled by 2^(bits - 2 - e) (zeros
// when the row has no live exponent).
__device__ __forceinline__ void rt_limbs(uint8_t *a, int tid, const double2 (&cur)[4], int e, int bits)
{
    const bool live = e > kNoExp / 2;
    const int sc = bits - 2 - e;
#pragma unroll
    for (int u = 0; u < 4; ++u) {
        uint32_t y[4] = {0u, 0u, 0u, 0u};
        bool ng = false;
        if (live) scaled_int(cur[u], sc, y, ng);
        const uint32_t s = ng ? 0x80008000u : 0u;
        st_row_chunk(a, tid, 2 * u,
                     make_uint4(limb_word<0>(y, s), limb_word<1>(y, s), limb_word<2>(y, s), limb_word<3>(y, s)));
        st_row_chunk(a, tid, 2 * u + 1,
                     make_uint4(limb_word<4>(y, s), limb_word<5>(y, s), limb_word<6>(y, s), limb_word<7>(y, s)));
    }
}

// The tile's four MMAs (one thread), completion on `done`.
__device__ __forceinline__ void rt_mma(uint32_t tmem, const uint8_t *a, const uint8_t *sB, uint64_t *done)
{
    const uint32_t idesc = sm100::idesc_f16_f32(128, 32);
    const uint64_t ad = sm100::smem_desc_sw128(sm100::smem_u32(a));
#pragma unroll
    for (int v = 0; v < 4; ++v) {
        const uint64_t bd = sm100::smem_desc_sw128(sm100::smem_u32(sB + v * 32 * 128));
        sm100::mma_f16(tmem + v * 32, ad + 2 * v, bd + 2 * v, idesc, 0u);
    }
    sm100::mma_commit(done);
}

// Residues of this thread's four elements for every modulus from the sums in
// TMEM, 16 moduli at a time, four fp16 per 8-byte store at o + l * plane
// (nothing stored when !ok; the TMEM loads are warp-wide either way).
__device__ __forceinline__ void rt_store(uint32_t lane_base, const OzResParams &P, __half *o, int64_t plane, bool ok)
{
    const int nmod = P.nmod;
#pragma unroll
    for (int l0 = 0; l0 < RT_MAX_MOD; l0 += 16) {
        if (l0 >= nmod) break;   // uniform
        uint32_t x[4][16];
#pragma unroll
        for (int v = 0; v < 4; ++v) sm100::tmem_ld16(lane_base + v * 32 + l0, x[v]);
        sm100::tmem_wait_ld();
#pragma unroll
        for (int i = 0; i < 16; ++i) {
            const int l = l0 + i;
            if (l < nmod && ok) {
                const float2 negp = make_float2(-P.p[l], -P.p[l]), invp = make_float2(P.invp[l], P.invp[l]);
                float2 s[2];
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    const float2 xv = make_float2(__uint_as_float(x[2 * h][i]), __uint_as_float(x[2 * h + 1][i]));
                    float2 y = __fmul2_rn(xv, invp);
                    y = __fadd2_rn(y, make_float2(12582912.0f, 12582912.0f));
                    y = __fadd2_rn(y, make_float2(-12582912.0f, -12582912.0f));
                    s[h] = __ffma2_rn(y, negp, xv);
                }
                store4h(o, s[0], s[1]);
            }
            o += plane;
        }
    }
}

// Shared-memory layout, barriers and TMEM of the tensor-core residue kernels.
struct RtCta {
    uint8_t *sA, *sB;
    uint64_t *done, *drain;
    uint32_t tmem, lane_base;
};

__device__ __forceinline__ RtCta rt_setup(uint8_t *raw, const OzResParams &P)
{
    RtCta c;
    uint8_t *smem = (uint8_t *)(((uintptr_t)raw + 1023) & ~(uintptr_t)1023);
    c.sA = smem;                          // [2] limb tiles
    c.sB = smem + 2 * RT_TILE_BYTES;      // constants
    c.done = (uint64_t *)(c.sB + RT_TILE_BYTES);   // the MMA of the latest tile retired
    c.drain = c.done + 1;
    uint32_t *tslot = (uint32_t *)(c.drain + 1);
    const int tid = threadIdx.x, warp = tid >> 5;
    rt_constants(c.sB, P, tid);
    if (tid == 0) {
        sm100::mbar_init(c.done, 1);
        sm100::mbar_init(c.drain, 1);
        sm100::fence_mbar_init();
    }
    if (warp == 0) {
        sm100::tmem_alloc(tslot, 128);
        sm100::tmem_relinquish();
    }
    sm100::fence_proxy_async_smem();
    sm100::tc_fence_before();
    __syncthreads();
    sm100::tc_fence_after();
    c.tmem = *tslot;
    c.lane_base = c.tmem + ((uint32_t)(warp * 32) << 16);
    return c;
}

// No MMA may still be writing TMEM when it is freed.
__device__ __forceinline__ void rt_teardown(const RtCta &c)
{
    if (threadIdx.x == 0) {
        sm100::mma_commit(c.drain);
        sm100::mbar_wait(c.drain, 0, nullptr, 0);
    }
    sm100::tc_fence_before();
    __syncthreads();
    if ((threadIdx.x >> 5) == 0) {
        sm100::tc_fence_after();
        sm100::tmem_dealloc(c.tmem, 128);
    }
}

// One step of the tile pipeline: the limbs of the current tile are in A[b];
// waits for the previous tile's MMA and stores its residues, then issues the
// current tile's MMA. Returns false (on every thread) once a wait gave up.
__device__ __forceinline__ bool rt_step(const RtCta &c, const OzResParams &P, int b, int it, bool have_prev,
                                        __half *po, int64_t pplane, bool pok, int *status, int &failed)
{
    if (have_prev) {
        if (__all_sync(0xffffffffu, sm100::mbar_wait(c.done, (it - 1) & 1, status, 21))) {
            sm100::tc_fence_after();
            rt_store(c.lane_base, P, po, pplane, pok);
        } else {
            failed = 1;
        }
    }
    sm100::fence_proxy_async_smem();
    sm100::tc_fence_before();
    if (__syncthreads_or(failed)) return false;
    sm100::tc_fence_after();
    if (threadIdx.x == 0) rt_mma(c.tmem, c.sA + b * RT_TILE_BYTES, c.sB, c.done);
    __syncwarp();
    return true;
}

// The last tile's residues (after its MMA).
__device__ __forceinline__ void rt_finish(const RtCta &c, const OzResParams &P, int it, bool have_prev, __half *po,
                                          int64_t pplane, bool pok, int *status, int failed)
{
    if (failed || !have_prev) return;
    if (__all_sync(0xffffffffu, sm100::mbar_wait(c.done, (it - 1) & 1, status, 21))) {
        sm100::tc_fence_after();
        rt_store(c.lane_base, P, po, pplane, pok);
    }
}

template <bool ROWC>
__global__ void __launch_bounds__(RT_THREADS, 4)
    k_oz_residues_tc(int64_t rows, int64_t kdim, const double2 *__restrict__ X, int64_t ld,
                     const int *__restrict__ rexp, int bits, OzResParams P, __half *__restrict__ out, int64_t rows_pad,
                     int64_t kpad, int64_t plane_rows, int *status)
{
    extern __shared__ uint8_t rt_raw[];
    const RtCta cta = rt_setup(rt_raw, P);
    const int tid = threadIdx.x;
    // tiles t = blockIdx.x + i * gridDim.x as (row, column) tile pairs, stepped
    // without divisions (32-bit: fewer than 2^31 tiles)
    const int nct = (int)(kpad / RT_COLS);
    const int ntr = (int)((rows_pad + RT_ROWS - 1) / RT_ROWS);
    const int rl = tid >> 3, cq = (tid & 7) * 4;
    const int64_t plane = plane_rows * kpad;
    const int step_r = (int)(gridDim.x / (unsigned)nct), step_c = (int)(gridDim.x % (unsigned)nct);

    auto fetch = [&](int tr, int tc, double2 (&v)[4]) {
        const int r = tr * RT_ROWS + rl, c = tc * RT_COLS + cq;
        const bool rok = r < rows;
        const double2 *x = ROWC ? X + r + (int64_t)c * ld : X + c + (int64_t)r * ld;
#pragma unroll
        for (int u = 0; u < 4; ++u)
            v[u] = (rok && c + u < kdim) ? x[ROWC ? u * ld : u] : make_double2(0.0, 0.0);
    };

    double2 cur[4];
    int tr = (int)(blockIdx.x / (unsigned)nct), tc = (int)(blockIdx.x % (unsigned)nct);
    if (tr < ntr) fetch(tr, tc, cur);
    __half *po = nullptr;   // the previous tile (its sums in TMEM): this thread's output
    bool pok = false, have_prev = false;
    int it = 0, failed = 0;
    for (; tr < ntr; ++it) {
        const int b = it & 1;
        const int r = tr * RT_ROWS + rl;
        rt_limbs(cta.sA + b * RT_TILE_BYTES, tid, cur, r < rows ? rexp[r] : kNoExp, bits);
        __half *o = out + (int64_t)r * kpad + tc * RT_COLS + cq;
        const bool ok = r < rows_pad;
        int tr2 = tr + step_r, tc2 = tc + step_c;
        if (tc2 >= nct) {
            tc2 -= nct;
            tr2 += 1;
        }
        if (tr2 < ntr) fetch(tr2, tc2, cur);   // in flight during the epilogue and the MMA below
        if (!rt_step(cta, P, b, it, have_prev, po, plane, pok, status, failed)) break;
        po = o;
        pok = ok;
        have_prev = true;
        tr = tr2;
        tc = tc2;
    }
    rt_finish(cta, P, it, have_prev, po, plane, pok, status, failed);
    rt_teardown(cta);
}

std::atomic<int> g_res_tc{1};   // mwblas_set_residue_tc

// Real operands on the tensor-core path when the layout allows it (k padded
// to the tile width, at most 32 moduli); false: the caller uses the FMA path.
template <bool ROWC>
bool launch_residues_tc(int64_t rows, int64_t kdim, const double2 *X, int64_t ld, const int *rexp, int bits,
                        const OzResParams &rp, __half *out, int64_t rows_pad, int64_t kpad, int64_t plane_rows)
{
    if (g_res_tc.load() == 0 || rp.nmod > RT_MAX_MOD || kpad % RT_COLS != 0 || rows_pad <= 0 || !ozaki_available())
        return false;
    static int attr_set[64];
    int dev = 0;
    cudaGetDevice(&dev);
    if (!attr_set[dev & 63]) {
        cudaFuncSetAttribute(k_oz_residues_tc<ROWC>, cudaFuncAttributeMaxDynamicSharedMemorySize, RT_SMEM);
        attr_set[dev & 63] = 1;
    }
    const int64_t ntiles = ((rows_pad + RT_ROWS - 1) / RT_ROWS) * (kpad / RT_COLS);
    if (ntiles >= ((int64_t)1 << 31) || rows_pad >= ((int64_t)1 << 31)) return false;
    int64_t grid = 4 * (int64_t)device_sm_count();
    if (grid > ntiles) grid = ntiles;
    k_oz_residues_tc<ROWC><<<(unsigned)grid, RT_THREADS, RT_SMEM, stream()>>>(
        rows, kdim, X, ld, rexp, bits, rp, out, rows_pad, kpad, plane_rows, device_status_word());
    count_launch();
    return true;
}

// ---- device: residue GEMM, tensor cores ---------------------------------------------------

constexpr int TC_BM = 128, TC_BN = 256, TC_BK = 64, TC_STAGES = 4;
constexpr int TC_A_BYTES = TC_BM * TC_BK * 2;   // 16 KB
constexpr int TC_B_BYTES = TC_BN * TC_BK * 2;   // 32 KB
constexpr int TC_SMEM = TC_STAGES * (TC_A_BYTES + TC_B_BYTES) + 1024 /*align*/ + 256 /*barriers*/;

__device__ __forceinline__ float mod_sym(float x, float p, float invp)
{
    float q = rint_small(__fmul_rn(x, invp));
    return __fmaf_rn(-q, p, x);   // in (-p, p), exact
}

// One CTA: a 128 x 256 tile of the residue product for modulus blockIdx.z.
// Warp 0: TMA producer. Warp 1: TMEM owner and MMA issuer. Warps 2-5:
// epilogue (TMEM lane quadrant = warp % 4).
__global__ void __launch_bounds__(192, 1)
    k_oz_gemm_tc(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, int64_t Mp,
                 int64_t Np, int64_t Kp, int64_t M, int64_t N, OzModParams P, uint16_t *__restrict__ R, int *status,
                 int uplo)
{
    // Triangular output (SYRK/HERK): tiles wholly outside the triangle do no work.
    {
        const int64_t i0 = (int64_t)blockIdx.y * TC_BM, j0 = (int64_t)blockIdx.x * TC_BN;
        if ((uplo == 1 && i0 > j0 + TC_BN - 1) || (uplo == 2 && i0 + TC_BM - 1 < j0)) return;
    }
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint8_t *sA = smem;
    uint8_t *sB = smem + TC_STAGES * TC_A_BYTES;
    uint64_t *bars = (uint64_t *)(smem + TC_STAGES * (TC_A_BYTES + TC_B_BYTES));
    uint64_t *full = bars;                 // [TC_STAGES]
    uint64_t *empty = bars + TC_STAGES;    // [TC_STAGES]
    uint64_t *accf = bars + 2 * TC_STAGES; // [2]
    uint64_t *acce = accf + 2;             // [2]
    uint64_t *drain = acce + 2;            // [1] all MMAs of this CTA retired
    uint32_t *tmem_slot = (uint32_t *)(drain + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int tile_n = blockIdx.x, tile_m = blockIdx.y, l = blockIdx.z;
    const int nsteps = (int)(Kp / TC_BK);
    const int kcs = kChunk / TC_BK;
    const int nch = (nsteps + kcs - 1) / kcs;

    if (warp == 0 && lane == 0) {
        for (int s = 0; s < TC_STAGES; ++s) {
            sm100::mbar_init(&full[s], 1);
            sm100::mbar_init(&empty[s], 1);
        }
        for (int b = 0; b < 2; ++b) {
            sm100::mbar_init(&accf[b], 1);
            sm100::mbar_init(&acce[b], 128);
        }
        sm100::mbar_init(drain, 1);
        sm100::fence_mbar_init();
    }
    if (warp == 1) {
        sm100::tmem_alloc(tmem_slot, 512);
        sm100::tmem_relinquish();
    }
    sm100::tc_fence_before();
    __syncthreads();
    sm100::tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    if (warp == 0) {
        if (lane == 0) {
            sm100::tma_prefetch_desc(&tmA);
            sm100::tma_prefetch_desc(&tmB);
            const int32_t ya = (int32_t)(l * Mp + (int64_t)tile_m * TC_BM);
            const int32_t yb = (int32_t)(l * Np + (int64_t)tile_n * TC_BN);
            int issued = 0;
            for (int step = 0; step < nsteps; ++step) {
                int s = step % TC_STAGES, u = step / TC_STAGES;
                if (u > 0 && !sm100::mbar_wait(&empty[s], (u - 1) & 1, status, 1)) break;
                sm100::mbar_arrive_expect_tx(&full[s], TC_A_BYTES + TC_B_BYTES);
                sm100::tma_load_2d(sA + s * TC_A_BYTES, &tmA, &full[s], step * TC_BK, ya);
                sm100::tma_load_2d(sB + s * TC_B_BYTES, &tmB, &full[s], step * TC_BK, yb);
                issued = step + 1;
            }
            // Never leave with copies in flight: wait (bounded) for the last
            // use of every stage this thread issued.
            for (int step = (issued > TC_STAGES ? issued - TC_STAGES : 0); step < issued; ++step)
                sm100::mbar_wait(&full[step % TC_STAGES], (step / TC_STAGES) & 1, nullptr, 0);
        }
    } else if (warp == 1) {
        if (lane == 0) {
            const uint32_t idesc = sm100::idesc_f16_f32(TC_BM, TC_BN);
            bool ok = true;
            for (int c = 0; c < nch && ok; ++c) {
                const int b = c & 1;
                if (c >= 2) {
                    if (!sm100::mbar_wait(&acce[b], ((c - 2) >> 1) & 1, status, 2)) { ok = false; break; }
                    sm100::tc_fence_after();
                }
                const int s0 = c * kcs, s1 = min(nsteps, s0 + kcs);
                for (int step = s0; step < s1; ++step) {
                    const int s = step % TC_STAGES;
                    if (!sm100::mbar_wait(&full[s], (step / TC_STAGES) & 1, status, 3)) { ok = false; break; }
                    sm100::tc_fence_after();
                    const uint64_t ad = sm100::smem_desc_sw128(sm100::smem_u32(sA + s * TC_A_BYTES));
                    const uint64_t bd = sm100::smem_desc_sw128(sm100::smem_u32(sB + s * TC_B_BYTES));
#pragma unroll
                    for (int kk = 0; kk < TC_BK / 16; ++kk) {
                        uint32_t acc = (c >= 2 || step > s0 || kk > 0) ? 1u : 0u;
                        sm100::mma_f16(tmem + b * TC_BN, ad + 2 * kk, bd + 2 * kk, idesc, acc);
                    }
                    sm100::mma_commit(&empty[s]);
                }
                if (ok) sm100::mma_commit(&accf[b]);
            }
            // Drain: no MMA may still be writing TMEM when it is freed.
            sm100::mma_commit(drain);
            sm100::mbar_wait(drain, 0, nullptr, 0);
        }
    } else {
        // ---- epilogue: 128 threads, one TMEM lane (tile row) each
        const int q = warp & 3;
        const int row = q * 32 + lane;
        const uint32_t lane_base = tmem + ((uint32_t)(q * 32) << 16);
        const float p = P.p[l], invp = P.invp[l];
        bool ok = true;
        for (int c = 0; c < nch && ok; ++c) {
            const int b = c & 1;
            // warp-uniform outcome before the .sync.aligned TMEM accesses
            if (!__all_sync(0xffffffffu, sm100::mbar_wait(&accf[b], (c >> 1) & 1, status, 4))) { ok = false; break; }
            sm100::tc_fence_after();
            if (c >= nch - 2) continue;   // the last chunk of each buffer is reduced in the combine
#pragma unroll 1
            for (int sl = 0; sl < TC_BN / 32; ++sl) {
                uint32_t r[32];
                const uint32_t ta = lane_base + b * TC_BN + sl * 32;
                sm100::tmem_ld32(ta, r);
                sm100::tmem_wait_ld();
#pragma unroll
                for (int i = 0; i < 32; ++i) r[i] = __float_as_uint(mod_sym(__uint_as_float(r[i]), p, invp));
                sm100::tmem_st32(ta, r);
            }
            sm100::tmem_wait_st();
            sm100::tc_fence_before();
            sm100::mbar_arrive(&acce[b]);
        }
        if (ok) {
            // Both accumulators hold their last chunk's sums (below 2^24,
            // exact); reduce each, combine and store c = (P + Q) mod p in
            // [0, p) as R[l][j][i] (32-bit index arithmetic inside the tile:
            // 64-bit compares and multiplies issue at the FP64 rate on this
            // part).
            const int64_t i = (int64_t)tile_m * TC_BM + row;
            const int64_t j0 = (int64_t)tile_n * TC_BN;
            const bool row_ok = i < M;
            const int jn = (int)min((int64_t)TC_BN, N - j0);
            uint16_t *q = R + ((int64_t)l * Np + j0) * Mp + i;   // advanced by Mp per column
#pragma unroll 1
            for (int sl = 0; sl < TC_BN / 32; ++sl) {
                uint32_t r0[32], r1[32];
                sm100::tmem_ld32(lane_base + sl * 32, r0);
                if (nch > 1) sm100::tmem_ld32(lane_base + TC_BN + sl * 32, r1);
                sm100::tmem_wait_ld();
#pragma unroll
                for (int t = 0; t < 32; ++t) {
                    float v = mod_sym(__uint_as_float(r0[t]), p, invp);
                    if (nch > 1) v = __fadd_rn(v, mod_sym(__uint_as_float(r1[t]), p, invp));
                    float fq = rint_small(__fmul_rn(v, invp));
                    float rr = __fmaf_rn(-fq, p, v);   // in (-p, p)
                    if (rr < 0.0f) rr = __fadd_rn(rr, p);
                    if (row_ok && sl * 32 + t < jn) *q = (uint16_t)small_uint(rr);
                    q += Mp;
                }
            }
        }
    }

    sm100::tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        __syncwarp();
        sm100::tc_fence_after();
        sm100::tmem_dealloc(tmem, 512);
    }
}

// Persistent form of k_oz_gemm_tc: one CTA per SM walks the (modulus, tile)
// units u = blockIdx.x, blockIdx.x + gridDim.x, ... (tiles along N fastest,
// then M, then the modulus, the order of the per-tile grid), two units at a
// time. Unit A of a pair accumulates in TMEM buffer 0 and unit B in buffer 1,
// and the MMA warp interleaves their K chunks (A.c0, B.c0, A.c1, B.c1, ...):
// while it fills one buffer, the epilogue reduces the other in place (chunk
// c + 1 accumulates onto the reduced chunk c, 512 * 180^2 + 361 < 2^24, so
// every fp32 sum stays exact) or, after a unit's last chunk, reduces it and
// stores the residues. The final store of one unit therefore overlaps the
// other unit's MMAs instead of stalling the tensor pipe. Eight epilogue warps,
// two per TMEM lane quadrant, each take half of the 256 columns.
constexpr int TCP_EPI_WARPS = 8;
constexpr int TCP_THREADS = 64 + 32 * TCP_EPI_WARPS;

__global__ void __launch_bounds__(TCP_THREADS, 1)
    k_oz_gemm_tc_p(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, int64_t Mp,
                   int64_t Np, int64_t Kp, int64_t M, int64_t N, OzModParams P, uint16_t *__restrict__ R, int *status,
                   int uplo, int tiles_m, int tiles_n, int nz)
{
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint8_t *sA = smem;
    uint8_t *sB = smem + TC_STAGES * TC_A_BYTES;
    uint64_t *bars = (uint64_t *)(smem + TC_STAGES * (TC_A_BYTES + TC_B_BYTES));
    uint64_t *full = bars;                 // [TC_STAGES]
    uint64_t *empty = bars + TC_STAGES;    // [TC_STAGES]
    uint64_t *accf = bars + 2 * TC_STAGES; // [2] chunk committed into buffer b
    uint64_t *acce = accf + 2;             // [2] buffer b released by the epilogue
    uint64_t *drain = acce + 2;            // [1] all MMAs of this CTA retired
    uint32_t *tmem_slot = (uint32_t *)(drain + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nsteps = (int)(Kp / TC_BK);
    const int kcs = kChunk / TC_BK;
    const int nch = (nsteps + kcs - 1) / kcs;
    const int64_t units = (int64_t)nz * tiles_m * tiles_n;
    // unit -> (tile_n, tile_m, modulus); false for tiles outside the stored triangle
    auto unit_at = [&](int64_t u, int &tn, int &tm, int &l) -> bool {
        tn = (int)(u % tiles_n);
        tm = (int)((u / tiles_n) % tiles_m);
        l = (int)(u / ((int64_t)tiles_n * tiles_m));
        const int64_t i0 = (int64_t)tm * TC_BM, j0 = (int64_t)tn * TC_BN;
        return !((uplo == 1 && i0 > j0 + TC_BN - 1) || (uplo == 2 && i0 + TC_BM - 1 < j0));
    };
    // the next unit of this CTA at or after u that has work (units if none)
    auto next_unit = [&](int64_t u) -> int64_t {
        int tn, tm, l;
        while (u < units && !unit_at(u, tn, tm, l)) u += gridDim.x;
        return u < units ? u : units;
    };

    if (warp == 0 && lane == 0) {
        for (int s = 0; s < TC_STAGES; ++s) {
            sm100::mbar_init(&full[s], 1);
            sm100::mbar_init(&empty[s], 1);
        }
        for (int b = 0; b < 2; ++b) {
            sm100::mbar_init(&accf[b], 1);
            sm100::mbar_init(&acce[b], 32 * TCP_EPI_WARPS);
        }
        sm100::mbar_init(drain, 1);
        sm100::fence_mbar_init();
    }
    if (warp == 1) {
        sm100::tmem_alloc(tmem_slot, 512);
        sm100::tmem_relinquish();
    }
    sm100::tc_fence_before();
    __syncthreads();
    sm100::tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    if (warp == 0) {
        if (lane == 0) {
            sm100::tma_prefetch_desc(&tmA);
            sm100::tma_prefetch_desc(&tmB);
            uint32_t gs = 0;   // k-steps issued by this CTA
            bool ok = true;
            for (int64_t ua = next_unit(blockIdx.x); ua < units && ok;) {
                const int64_t ub = next_unit(ua + gridDim.x);
                const int nu = ub < units ? 2 : 1;
                int32_t ya[2], yb[2];
                for (int v = 0; v < nu; ++v) {
                    int tn, tm, l;
                    unit_at(v ? ub : ua, tn, tm, l);
                    ya[v] = (int32_t)(l * Mp + (int64_t)tm * TC_BM);
                    yb[v] = (int32_t)(l * Np + (int64_t)tn * TC_BN);
                }
                for (int c = 0; c < nch && ok; ++c) {
                    const int s0 = c * kcs, s1 = min(nsteps, s0 + kcs);
                    for (int v = 0; v < nu && ok; ++v) {
                        for (int step = s0; step < s1; ++step) {
                            const int s = gs % TC_STAGES;
                            const uint32_t ph = gs / TC_STAGES;
                            if (ph > 0 && !sm100::mbar_wait(&empty[s], (ph - 1) & 1, status, 1)) { ok = false; break; }
                            sm100::mbar_arrive_expect_tx(&full[s], TC_A_BYTES + TC_B_BYTES);
                            sm100::tma_load_2d(sA + s * TC_A_BYTES, &tmA, &full[s], step * TC_BK, ya[v]);
                            sm100::tma_load_2d(sB + s * TC_B_BYTES, &tmB, &full[s], step * TC_BK, yb[v]);
                            ++gs;
                        }
                    }
                }
                ua = nu == 2 ? next_unit(ub + gridDim.x) : units;
            }
            // never leave with copies in flight: wait (bounded) for the last use of every stage
            for (uint32_t t = (gs > TC_STAGES ? gs - TC_STAGES : 0); t < gs; ++t)
                sm100::mbar_wait(&full[t % TC_STAGES], (t / TC_STAGES) & 1, nullptr, 0);
        }
    } else if (warp == 1) {
        if (lane == 0) {
            const uint32_t idesc = sm100::idesc_f16_f32(TC_BM, TC_BN);
            uint32_t gs = 0;
            uint32_t uses[2] = {0, 0};   // chunks written into each buffer so far
            bool ok = true;
            for (int64_t ua = next_unit(blockIdx.x); ua < units && ok;) {
                const int64_t ub = next_unit(ua + gridDim.x);
                const int nu = ub < units ? 2 : 1;
                for (int c = 0; c < nch && ok; ++c) {
                    const int s0 = c * kcs, s1 = min(nsteps, s0 + kcs);
                    for (int b = 0; b < nu && ok; ++b) {
                        if (uses[b] > 0) {   // the previous chunk in this buffer has been released
                            if (!sm100::mbar_wait(&acce[b], (uses[b] - 1) & 1, status, 2)) { ok = false; break; }
                            sm100::tc_fence_after();
                        }
                        for (int step = s0; step < s1; ++step) {
                            const int s = gs % TC_STAGES;
                            if (!sm100::mbar_wait(&full[s], (gs / TC_STAGES) & 1, status, 3)) { ok = false; break; }
                            sm100::tc_fence_after();
                            const uint64_t ad = sm100::smem_desc_sw128(sm100::smem_u32(sA + s * TC_A_BYTES));
                            const uint64_t bd = sm100::smem_desc_sw128(sm100::smem_u32(sB + s * TC_B_BYTES));
#pragma unroll
                            for (int kk = 0; kk < TC_BK / 16; ++kk) {
                                const uint32_t acc = (c > 0 || step > s0 || kk > 0) ? 1u : 0u;
                                sm100::mma_f16(tmem + b * TC_BN, ad + 2 * kk, bd + 2 * kk, idesc, acc);
                            }
                            sm100::mma_commit(&empty[s]);
                            ++gs;
                        }
                        if (!ok) break;
                        sm100::mma_commit(&accf[b]);
                        ++uses[b];
                    }
                }
                ua = nu == 2 ? next_unit(ub + gridDim.x) : units;
            }
            // no MMA may still be writing TMEM when it is freed
            sm100::mma_commit(drain);
            sm100::mbar_wait(drain, 0, nullptr, 0);
        }
    } else {
        // ---- epilogue: warps 2..9, TMEM lane quadrant warp % 4, column half (warp - 2) / 4
        const int q = warp & 3;
        const int half = (warp - 2) >> 2;
        const int row = q * 32 + lane;
        const uint32_t lane_base = tmem + ((uint32_t)(q * 32) << 16) + half * (TC_BN / 2);
        uint32_t fcnt[2] = {0, 0};   // chunk completions consumed per buffer
        bool ok = true;
        for (int64_t ua = next_unit(blockIdx.x); ua < units && ok;) {
            const int64_t ub = next_unit(ua + gridDim.x);
            const int nu = ub < units ? 2 : 1;
            for (int c = 0; c < nch && ok; ++c) {
                for (int b = 0; b < nu; ++b) {
                    int tn, tm, l;
                    unit_at(b ? ub : ua, tn, tm, l);
                    const float p = P.p[l], invp = P.invp[l];
                    // warp-uniform outcome before the .sync.aligned TMEM accesses
                    if (!__all_sync(0xffffffffu, sm100::mbar_wait(&accf[b], fcnt[b] & 1, status, 4))) {
                        ok = false;
                        break;
                    }
                    ++fcnt[b];
                    sm100::tc_fence_after();
                    const uint32_t tb = lane_base + b * TC_BN;
                    // this warp's 128 columns, 64 at a time (two loads in flight per wait)
                    const float2 negp2 = make_float2(-p, -p), invp2 = make_float2(invp, invp);
                    const int64_t i = (int64_t)tm * TC_BM + row;
                    const int64_t j0 = (int64_t)tn * TC_BN + half * (TC_BN / 2);
                    const bool row_ok = i < M;
                    const int jn = (int)max((int64_t)0, min((int64_t)(TC_BN / 2), N - j0));
                    uint16_t *o = R + ((int64_t)l * Np + j0) * Mp + i;   // advanced by Mp per column
#pragma unroll 1
                    for (int hh = 0; hh < 2; ++hh) {
                        uint32_t r[2][32];
                        sm100::tmem_ld32(tb + hh * 64, r[0]);
                        sm100::tmem_ld32(tb + hh * 64 + 32, r[1]);
                        sm100::tmem_wait_ld();
                        // x - p * rint(x / p), two columns per packed instruction (in (-p, p), exact)
#pragma unroll
                        for (int sl = 0; sl < 2; ++sl) {
#pragma unroll
                            for (int t = 0; t < 32; t += 2) {
                                float2 x = make_float2(__uint_as_float(r[sl][t]), __uint_as_float(r[sl][t + 1]));
                                float2 y = __fmul2_rn(x, invp2);
                                y = __fadd2_rn(y, make_float2(12582912.0f, 12582912.0f));
                                y = __fadd2_rn(y, make_float2(-12582912.0f, -12582912.0f));
                                x = __ffma2_rn(y, negp2, x);
                                r[sl][t] = __float_as_uint(x.x);
                                r[sl][t + 1] = __float_as_uint(x.y);
                            }
                        }
                        if (c < nch - 1) {
                            // reduce in place; the next chunk accumulates onto it
                            sm100::tmem_st32(tb + hh * 64, r[0]);
                            sm100::tmem_st32(tb + hh * 64 + 32, r[1]);
                        } else {
                            // last chunk: c = sum mod p in [0, p) as R[l][j][i]
#pragma unroll
                            for (int sl = 0; sl < 2; ++sl) {
#pragma unroll
                                for (int t = 0; t < 32; ++t) {
                                    float rr = __uint_as_float(r[sl][t]);
                                    if (rr < 0.0f) rr = __fadd_rn(rr, p);
                                    if (row_ok && hh * 64 + sl * 32 + t < jn) *o = (uint16_t)small_uint(rr);
                                    o += Mp;
                                }
                            }
                        }
                    }
                    if (c < nch - 1) sm100::tmem_wait_st();
                    sm100::tc_fence_before();
                    sm100::mbar_arrive(&acce[b]);
                }
            }
            ua = nu == 2 ? next_unit(ub + gridDim.x) : units;
        }
    }

    sm100::tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        __syncwarp();
        sm100::tc_fence_after();
        sm100::tmem_dealloc(tmem, 512);
    }
}

// Pair form of k_oz_gemm_tc_p: clusters of two CTAs on two SMs compute 256 x 256
// tiles with tcgen05.mma.cta_group::2 (M = 256 across the pair, N = 256). Each
// CTA stages its 128 rows of A and 128 of the 256 rows of B per K-step, so a
// K-step moves 32 KB into each SM instead of 48 KB and six stages fit in shared
// memory; each CTA's TMEM holds its 128 rows of the tile. Units are
// (modulus, 256-row tile, 256-column tile), walked two at a time per cluster
// with interleaved K chunks as in k_oz_gemm_tc_p. The MMAs are issued by the
// even CTA; stage and accumulator barriers of both CTAs are released by its
// multicast commits; both CTAs' loads complete on the even CTA's stage barrier
// and both CTAs' epilogue warps release accumulators on the even CTA's barrier.
constexpr int T2_STAGES = 6;
constexpr int T2_A_BYTES = 128 * TC_BK * 2;   // 16 KB
constexpr int T2_B_BYTES = 128 * TC_BK * 2;   // 16 KB (half of the 256-row B tile)
constexpr int T2_SMEM = T2_STAGES * (T2_A_BYTES + T2_B_BYTES) + 1024 + 256;

__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(TCP_THREADS, 1)
    k_oz_gemm_tc_2sm(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, int64_t Mp,
                     int64_t Np, int64_t Kp, int64_t M, int64_t N, OzModParams P, uint16_t *__restrict__ R,
                     int *status, int uplo, int tiles_m2, int tiles_n, int nz, int tn0, int tm0, int lose_loads,
                     int zmod)
{
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint8_t *sA = smem;
    uint8_t *sB = smem + T2_STAGES * T2_A_BYTES;
    uint64_t *bars = (uint64_t *)(smem + T2_STAGES * (T2_A_BYTES + T2_B_BYTES));
    uint64_t *full = bars;                  // [T2_STAGES] even CTA: both CTAs' loads landed
    uint64_t *empty = bars + T2_STAGES;     // [T2_STAGES] each CTA: stage free again
    uint64_t *accf = bars + 2 * T2_STAGES;  // [2] each CTA: chunk committed into buffer b
    uint64_t *acce = accf + 2;              // [2] even CTA: buffer b released by both epilogues
    uint64_t *drain = acce + 2;             // [1] even CTA: all MMAs retired
    uint32_t *tmem_slot = (uint32_t *)(drain + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t rank = sm100::cluster_ctarank();
    const bool lead = rank == 0;
    const int cid = (int)(blockIdx.x >> 1), ncl = (int)(gridDim.x >> 1);
    const int nsteps = (int)(Kp / TC_BK);
    const int kcs = kChunk / TC_BK;
    const int nch = (nsteps + kcs - 1) / kcs;
    const int64_t units = (int64_t)nz * tiles_m2 * tiles_n;
    auto unit_at = [&](int64_t u, int &tn, int &tm2, int &l) -> bool {
        tn = tn0 + (int)(u % tiles_n);             // column tiles [tn0, tn0 + tiles_n)
        tm2 = tm0 + (int)((u / tiles_n) % tiles_m2);   // row tile pairs [tm0, tm0 + tiles_m2)
        l = (int)(u / ((int64_t)tiles_n * tiles_m2));
        const int64_t i0 = (int64_t)tm2 * 256, j0 = (int64_t)tn * TC_BN;
        return !((uplo == 1 && i0 > j0 + TC_BN - 1) || (uplo == 2 && i0 + 255 < j0));
    };
    auto next_unit = [&](int64_t u) -> int64_t {
        int tn, tm2, l;
        while (u < units && !unit_at(u, tn, tm2, l)) u += ncl;
        return u < units ? u : units;
    };

    if (warp == 0 && lane == 0) {
        for (int st = 0; st < T2_STAGES; ++st) {
            sm100::mbar_init(&full[st], 1);
            sm100::mbar_init(&empty[st], 1);
        }
        for (int b = 0; b < 2; ++b) {
            sm100::mbar_init(&accf[b], 1);
            sm100::mbar_init(&acce[b], 2 * TCP_EPI_WARPS);
        }
        sm100::mbar_init(drain, 1);
        sm100::fence_mbar_init();
    }
    if (warp == 1) {
        sm100::tmem_alloc_pair(tmem_slot, 512);
        sm100::tmem_relinquish_pair();
    }
    sm100::tc_fence_before();
    __syncthreads();
    sm100::cluster_sync();   // both CTAs' barriers initialised, TMEM allocated
    sm100::tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    if (warp == 0) {
        if (lane == 0) {
            sm100::tma_prefetch_desc(&tmA);
            sm100::tma_prefetch_desc(&tmB);
            uint32_t gs = 0;
            bool ok = true;
            // lose_loads (a failure-injection hook): issue no operand load at
            // all, so that the MMA issuer's first wait for a landed stage runs
            // out with nothing in flight anywhere in the pair
            for (int64_t ua = lose_loads ? units : next_unit(cid); ua < units && ok;) {
                const int64_t ub = next_unit(ua + ncl);
                const int nu = ub < units ? 2 : 1;
                int32_t ya[2], yb[2];
                for (int v = 0; v < nu; ++v) {
                    int tn, tm2, l;
                    unit_at(v ? ub : ua, tn, tm2, l);
                    ya[v] = (int32_t)(l * Mp + (int64_t)tm2 * 256 + rank * 128);
                    yb[v] = (int32_t)(l * Np + (int64_t)tn * TC_BN + rank * 128);
                }
                for (int c = 0; c < nch && ok; ++c) {
                    const int s0 = c * kcs, s1 = min(nsteps, s0 + kcs);
                    for (int v = 0; v < nu && ok; ++v) {
                        for (int step = s0; step < s1; ++step) {
                            const int st = gs % T2_STAGES;
                            const uint32_t ph = gs / T2_STAGES;
                            if (ph > 0 && !sm100::mbar_wait(&empty[st], (ph - 1) & 1, status, 1)) { ok = false; break; }
                            if (lead) sm100::mbar_arrive_expect_tx(&full[st], 2 * (T2_A_BYTES + T2_B_BYTES));
                            const uint32_t fb = sm100::mapa(&full[st], 0);
                            sm100::tma_load_2d_pair(sA + st * T2_A_BYTES, &tmA, fb, step * TC_BK, ya[v]);
                            sm100::tma_load_2d_pair(sB + st * T2_B_BYTES, &tmB, fb, step * TC_BK, yb[v]);
                            ++gs;
                        }
                    }
                }
                ua = nu == 2 ? next_unit(ub + ncl) : units;
            }
            // Never leave with copies in flight. A stage is released (empty, in
            // both CTAs) only after the MMAs that read it retired, i.e. after
            // both CTAs' loads into it landed; after a failure, give loads
            // still in flight time to land.
            if (ok) {
                for (uint32_t t = (gs > T2_STAGES ? gs - T2_STAGES : 0); t < gs; ++t)
                    if (!sm100::mbar_wait(&empty[t % T2_STAGES], (t / T2_STAGES) & 1, status, 1)) { ok = false; break; }
            }
            if (!ok) {
                const uint64_t t0 = sm100::globaltimer_ns();
                while (sm100::globaltimer_ns() - t0 < 2000000ull) __nanosleep(1000);
            }
        }
    } else if (warp == 1) {
        if (lead && lane == 0) {
            const uint32_t idesc = sm100::idesc_f16_f32(256, TC_BN);
            uint32_t gs = 0;
            uint32_t uses[2] = {0, 0};
            bool ok = true;
            for (int64_t ua = next_unit(cid); ua < units && ok;) {
                const int64_t ub = next_unit(ua + ncl);
                const int nu = ub < units ? 2 : 1;
                for (int c = 0; c < nch && ok; ++c) {
                    const int s0 = c * kcs, s1 = min(nsteps, s0 + kcs);
                    for (int b = 0; b < nu && ok; ++b) {
                        if (uses[b] > 0) {   // both CTAs' epilogues released the previous chunk in this buffer
                            if (!sm100::mbar_wait_cluster(&acce[b], (uses[b] - 1) & 1, status, 2)) { ok = false; break; }
                            sm100::tc_fence_after();
                        }
                        for (int step = s0; step < s1; ++step) {
                            const int st = gs % T2_STAGES;
                            if (!sm100::mbar_wait_cluster(&full[st], (gs / T2_STAGES) & 1, status, 3)) { ok = false; break; }
                            sm100::tc_fence_after();
                            const uint64_t ad = sm100::smem_desc_sw128(sm100::smem_u32(sA + st * T2_A_BYTES));
                            const uint64_t bd = sm100::smem_desc_sw128(sm100::smem_u32(sB + st * T2_B_BYTES));
#pragma unroll
                            for (int kk = 0; kk < TC_BK / 16; ++kk) {
                                const uint32_t acc = (c > 0 || step > s0 || kk > 0) ? 1u : 0u;
                                sm100::mma_f16_pair(tmem + b * TC_BN, ad + 2 * kk, bd + 2 * kk, idesc, acc);
                            }
                            sm100::mma_commit_pair(&empty[st], 3);
                            ++gs;
                        }
                        if (!ok) break;
                        sm100::mma_commit_pair(&accf[b], 3);
                        ++uses[b];
                    }
                }
                ua = nu == 2 ? next_unit(ub + ncl) : units;
            }
            sm100::mma_commit_pair(drain, 1);
            sm100::mbar_wait(drain, 0, nullptr, 0);
        }
    } else {
        // ---- epilogue: warps 2..9 of each CTA on its 128 rows (TMEM lane quadrant
        // warp % 4, column half (warp - 2) / 4)
        const int q = warp & 3;
        const int half = (warp - 2) >> 2;
        const int row = q * 32 + lane;
        const uint32_t lane_base = tmem + ((uint32_t)(q * 32) << 16) + half * (TC_BN / 2);
        const uint32_t acce_lead[2] = {sm100::mapa(&acce[0], 0), sm100::mapa(&acce[1], 0)};
        uint32_t fcnt[2] = {0, 0};
        bool ok = true;
        for (int64_t ua = next_unit(cid); ua < units && ok;) {
            const int64_t ub = next_unit(ua + ncl);
            const int nu = ub < units ? 2 : 1;
            for (int c = 0; c < nch && ok; ++c) {
                for (int b = 0; b < nu; ++b) {
                    int tn, tm2, l;
                    unit_at(b ? ub : ua, tn, tm2, l);
                    const float p = P.p[l % zmod], invp = P.invp[l % zmod];   // plane l holds modulus l % zmod
                    if (!__all_sync(0xffffffffu, sm100::mbar_wait(&accf[b], fcnt[b] & 1, status, 4))) {
                        ok = false;
                        break;
                    }
                    ++fcnt[b];
                    sm100::tc_fence_after();
                    const uint32_t tb = lane_base + b * TC_BN;
                    const float2 negp2 = make_float2(-p, -p), invp2 = make_float2(invp, invp);
                    const int64_t i = (int64_t)tm2 * 256 + rank * 128 + row;
                    const int64_t j0 = (int64_t)tn * TC_BN + half * (TC_BN / 2);
                    const bool row_ok = i < M;
                    const int jn = (int)max((int64_t)0, min((int64_t)(TC_BN / 2), N - j0));
                    uint16_t *o = R + ((int64_t)l * Np + j0) * Mp + i;   // advanced by Mp per column
#pragma unroll 1
                    for (int hh = 0; hh < 2; ++hh) {
                        uint32_t r[2][32];
                        sm100::tmem_ld32(tb + hh * 64, r[0]);
                        sm100::tmem_ld32(tb + hh * 64 + 32, r[1]);
                        sm100::tmem_wait_ld();
#pragma unroll
                        for (int sl = 0; sl < 2; ++sl) {
#pragma unroll
                            for (int t = 0; t < 32; t += 2) {
                                float2 x = make_float2(__uint_as_float(r[sl][t]), __uint_as_float(r[sl][t + 1]));
                                float2 y = __fmul2_rn(x, invp2);
                                y = __fadd2_rn(y, make_float2(12582912.0f, 12582912.0f));
                                y = __fadd2_rn(y, make_float2(-12582912.0f, -12582912.0f));
                                x = __ffma2_rn(y, negp2, x);
                                r[sl][t] = __float_as_uint(x.x);
                                r[sl][t + 1] = __float_as_uint(x.y);
                            }
                        }
                        if (c < nch - 1) {
                            sm100::tmem_st32(tb + hh * 64, r[0]);
                            sm100::tmem_st32(tb + hh * 64 + 32, r[1]);
                        } else {
#pragma unroll
                            for (int sl = 0; sl < 2; ++sl) {
#pragma unroll
                                for (int t = 0; t < 32; ++t) {
                                    float rr = __uint_as_float(r[sl][t]);
                                    if (rr < 0.0f) rr = __fadd_rn(rr, p);
                                    if (row_ok && hh * 64 + sl * 32 + t < jn) *o = (uint16_t)small_uint(rr);
                                    o += Mp;
                                }
                            }
                        }
                    }
                    if (c < nch - 1) sm100::tmem_wait_st();
                    sm100::tc_fence_before();
                    __syncwarp();
                    if (lane == 0) sm100::mbar_arrive_cluster(acce_lead[b]);
                }
            }
            ua = nu == 2 ? next_unit(ub + ncl) : units;
        }
    }

    // Both CTAs stay resident until every role of both is done: the even CTA's
    // MMAs write the odd CTA's TMEM and read its shared memory, and the odd
    // CTA's epilogue arrives on the even CTA's barriers.
    sm100::tc_fence_before();
    __syncthreads();
    sm100::cluster_sync();
    if (warp == 1) {
        sm100::tc_fence_after();
        sm100::tmem_dealloc_pair(tmem, 512);
    }
}

// ---- device: residue GEMM, CUDA cores (cross-check engine) ---------------------------------

__global__ void __launch_bounds__(256) k_oz_gemm_simt(const __half *__restrict__ A, const __half *__restrict__ B,
                                                      int64_t Mp, int64_t Np, int64_t Kp, int64_t M, int64_t N,
                                                      OzModParams P, uint16_t *__restrict__ R)
{
    __shared__ float sa[16][65], sb[16][65];
    const int l = blockIdx.z;
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    const int64_t i = (int64_t)blockIdx.y * 16 + ty, j = (int64_t)blockIdx.x * 16 + tx;
    const __half *Al = A + (int64_t)l * Mp * Kp;
    const __half *Bl = B + (int64_t)l * Np * Kp;
    long long acc = 0;   // |sum| <= Kp * 180^2
    for (int64_t k0 = 0; k0 < Kp; k0 += 64) {
        for (int t = threadIdx.x; t < 16 * 64; t += 256) {
            int rr = t / 64, cc = t % 64;
            int64_t gi = (int64_t)blockIdx.y * 16 + rr, gj = (int64_t)blockIdx.x * 16 + rr;
            sa[rr][cc] = __half2float(Al[gi * Kp + k0 + cc]);
            sb[rr][cc] = __half2float(Bl[gj * Kp + k0 + cc]);
        }
        __syncthreads();
        for (int cc = 0; cc < 64; ++cc) acc += (long long)((int)sa[ty][cc] * (int)sb[tx][cc]);
        __syncthreads();
    }
    if (i < M && j < N) {
        int p = (int)P.p[l];
        int r = (int)(acc % p);
        if (r < 0) r += p;
        R[((int64_t)l * Np + j) * Mp + i] = (uint16_t)r;
    }
}

// ---- device: CRT reconstruction ----------------------------------------------------------

using xfp::XF;
using xfp::xf_add;
using xfp::xf_from_dd;
using xfp::xf_mul;

// Shared-memory copy of the CRT constants (broadcast reads; each row of F is
// 32 bytes so a modulus' constants are two 16-byte loads).
struct CrtSmem {
    alignas(16) uint32_t F[kMaxMod][crt::kFLPad];
    float pm[kMaxMod];
};

__device__ __forceinline__ void crt_smem_fill(CrtSmem &sm, const OzCrtParams &K)
{
    for (int i = threadIdx.x; i < K.nmod * crt::kFLPad; i += blockDim.x)
        sm.F[i / crt::kFLPad][i % crt::kFLPad] = K.F[i / crt::kFLPad][i % crt::kFLPad];
    for (int i = threadIdx.x; i < K.nmod; i += blockDim.x) sm.pm[i] = K.pm[i];
}

__device__ __forceinline__ dd::real xw_dd(const xw::XW &x)
{
    dd::real r;
    xw::to_dd(x, r.hi, r.lo);
    return r;
}

__device__ __forceinline__ bool finite_hi(double x)
{
    return ((__double2hiint(x) >> 20) & 0x7FF) != 0x7FF;   // exponent field test, no FP64 compare
}

// Triangular outputs (uplo 1: i <= j, 2: i >= j) are walked as a list of
// (row slab x, column j) tasks holding stored entries: slab x (rows
// [S x, S x + S)) needs columns [S x, n) of an upper triangle and
// [0, min(n, S x + S)) of a lower one. The blocks of a grid stride over that
// list, so every block gets about the same share of the triangle (a slab per
// block and all columns would leave the top slabs of an upper triangle with
// 16 times the work of the bottom ones at n = 8192).
__device__ __forceinline__ int64_t tri_prefix(int uplo, int64_t x, int64_t n, int64_t S)
{
    if (uplo == 1) {   // sum over x' < x of n - min(n, S x')
        const int64_t q = min(x, (n + S - 1) / S);
        return q * n - S * q * (q - 1) / 2;
    }
    const int64_t qf = n / S;   // sum over x' < x of min(n, S (x' + 1)); the first qf terms are S (x' + 1)
    const int64_t q = min(x, qf);
    return S * q * (q + 1) / 2 + max((int64_t)0, x - qf) * n;
}

__device__ __forceinline__ void tri_task(int uplo, int64_t t, int64_t slabs, int64_t n, int64_t S, int64_t &x,
                                         int64_t &j)
{
    int64_t lo = 0, hi = slabs - 1;   // the first slab whose tasks extend past t
    while (lo < hi) {
        const int64_t mid = (lo + hi) >> 1;
        if (tri_prefix(uplo, mid + 1, n, S) > t) hi = mid;
        else lo = mid + 1;
    }
    x = lo;
    j = t - tri_prefix(uplo, x, n, S) + (uplo == 1 ? min(n, S * x) : 0);
}

// Output rows i0 and i0 + 1 (when `two`) of column j: the CRT sums of their
// residues over the nmod planes (rcol points at row i0, column j of plane 0;
// planes `plane` entries apart), then alpha M (folded into Mx), the power-of-
// two scaling and beta C (beta as the extended float xb), one rounding to
// double-double. pc points at C(i0, j).
__device__ __forceinline__ void reconstruct_pair(const CrtSmem &sm, int nmod, const uint16_t *rcol, int64_t plane,
                                                 int i0, bool two, int ea0, int ea1, int j, int ebj, int bsum,
                                                 const xw::XW &Mx, const xw::XW &xb, dd::real beta, int beta_kind,
                                                 double2 *pc, int uplo)
{
    // both rows outside the stored triangle: nothing to compute
    if ((uplo == 1 && i0 > j) || (uplo == 2 && i0 + 1 < j)) return;
    crt::Frac acc0, acc1;
    acc0.reset();
    acc1.reset();
    const bool live0 = ea0 > kNoExp / 2 && ea0 < 1024 && ebj > kNoExp / 2 && ebj < 1024;
    const bool live1 = two && ea1 > kNoExp / 2 && ea1 < 1024 && ebj > kNoExp / 2 && ebj < 1024;
    if (live0 || live1) {
        // residues of all moduli for both rows: the loads of 8 planes are
        // issued together so that their latencies overlap
        const uint32_t *q = reinterpret_cast<const uint32_t *>(rcol);
        const int64_t qstep = plane / 2;
        int l = 0;
        for (; l + 8 <= nmod; l += 8) {
            uint32_t c[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                c[u] = __ldcs(q);
                q += qstep;
            }
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                acc0.add(sm.F[l + u], c[u] & 0xFFFFu);
                acc1.add(sm.F[l + u], c[u] >> 16);
            }
        }
        for (; l < nmod; ++l, q += qstep) {
            const uint32_t c = __ldcs(q);
            acc0.add(sm.F[l], c & 0xFFFFu);
            acc1.add(sm.F[l], c >> 16);
        }
    }
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const int i = i0 + h;
        if (h == 1 && !two) break;
        if ((uplo == 1 && i > j) || (uplo == 2 && i < j)) continue;
        const int eai = h ? ea1 : ea0;
        double2 *pe = pc + h;
        if (eai >= 1024 || ebj >= 1024) {   // a non-finite entry in row i of op(A) or column j of op(B)
            const double qnan = __longlong_as_double(0x7ff8000000000000ll);
            *pe = make_double2(qnan, qnan);
            continue;
        }
        xw::XW v = xw::zero();
        if (h ? live1 : live0) v = (h ? acc1 : acc0).finish_xw(Mx, bsum - 4 - eai - ebj);
        if (beta_kind != 0) {
            const double2 c0 = *pe;
            if (!finite_hi(c0.x)) {
                // non-finite C: the double-double operators propagate it
                dd::real cv = dd::make(c0.x, c0.y);
                if (beta_kind == 2) cv = dd::mul_exact(cv, beta);
                dd::store(pe, dd::add_exact(cv, xw_dd(v)));
                continue;
            }
            xw::XW xc = xw::from_dd(c0.x, c0.y);
            if (beta_kind == 2) xc = xw::mul(xb, xc);
            v = xw::add(v, xc);
        }
        dd::store(pe, xw_dd(v));
    }
}

// C(i, j) := alpha * X(i, j) * 2^-S2 + beta * C(i, j), real. Thread per pair
// of rows, columns j = blockIdx.y, blockIdx.y + gridDim.y, ...; m and n below 2^31
// (the host routes larger sizes elsewhere), so the per-element index work is
// 32-bit or pointer increments.
__global__ void __launch_bounds__(256) k_oz_reconstruct(int m, int n, const uint16_t *__restrict__ R,
                                                        int64_t Mp, int64_t Np, const int *__restrict__ ea,
                                                        const int *__restrict__ eb, int bsum, OzCrtParams K,
                                                        xw::XW Mx, xw::XW xb, dd::real beta, int beta_kind,
                                                        double2 *C, int64_t ldc, int uplo)
{
    // Mx = alpha * M and xb = beta as extended floats (formed on the host).
    // A thread takes rows i0, i0 + 1 (one 32-bit load per modulus serves both).
    __shared__ CrtSmem sm;
    crt_smem_fill(sm, K);
    __syncthreads();
    const int nmod = K.nmod;
    const int64_t plane = Np * Mp;
    if (uplo != 0) {
        // a triangle: (512-row slab, column) tasks shared evenly by all blocks
        const int64_t S = 2 * (int64_t)blockDim.x, slabs = (m + S - 1) / S, total = tri_prefix(uplo, slabs, n, S);
        for (int64_t t = (int64_t)blockIdx.y * gridDim.x + blockIdx.x; t < total;
             t += (int64_t)gridDim.x * gridDim.y) {
            int64_t x, j;
            tri_task(uplo, t, slabs, n, S, x, j);
            const int i0 = (int)(x * S) + 2 * threadIdx.x;
            if (i0 >= m) continue;
            const bool two = i0 + 1 < m;
            reconstruct_pair(sm, nmod, R + j * Mp + i0, plane, i0, two, ea[i0], two ? ea[i0 + 1] : kNoExp, (int)j,
                             eb[j], bsum, Mx, xb, beta, beta_kind, C + i0 + j * ldc, uplo);
        }
        return;
    }
    const int i0 = 2 * (blockIdx.x * blockDim.x + threadIdx.x);
    if (i0 >= m) return;
    const bool two = i0 + 1 < m;
    const int ea0 = ea[i0], ea1 = two ? ea[i0 + 1] : kNoExp;
    const int jstep = gridDim.y;
    const uint16_t *rcol = R + (int64_t)blockIdx.y * Mp + i0;
    double2 *pc = C + i0 + (int64_t)blockIdx.y * ldc;
    const int64_t rstep = (int64_t)jstep * Mp, cstep = (int64_t)jstep * ldc;
    for (int j = blockIdx.y; j < n; j += jstep, rcol += rstep, pc += cstep)
        reconstruct_pair(sm, nmod, rcol, plane, i0, two, ea0, ea1, j, eb[j], bsum, Mx, xb, beta, beta_kind, pc, uplo);
}

// Complex: R holds the residues of P1 = Ar*Br, P2 = Ai*Bi and
// P3 = (Ar+Ai)*(Br+Bi) as components 0..2; Re = P1 - P2, Im = P3 - P1 - P2.
__global__ void __launch_bounds__(256) k_oz_reconstruct_c(int m, int n, const uint16_t *__restrict__ R,
                                                          int64_t Mp, int64_t Np, const int *__restrict__ ea,
                                                          const int *__restrict__ eb, int bsum, OzCrtParams K,
                                                          xw::XW Mx, xw::XW ar, xw::XW ai, int alpha_one,
                                                          dd::cplx beta, xw::XW br, xw::XW bi, int beta_kind,
                                                          double2 *C, int64_t ldc, int uplo, int herm, int real_beta)
{
    // Mx = M, (ar, ai) = alpha and (br, bi) = beta as extended floats (formed on the host)
    __shared__ CrtSmem sm;
    crt_smem_fill(sm, K);
    __syncthreads();
    const int nmod = K.nmod;
    const int64_t cstride = (int64_t)nmod * Np * Mp;
    // output (i, j)
    auto one = [&](const int i, const int j) {
        if ((uplo == 1 && i > j) || (uplo == 2 && i < j)) return;
        if (ea[i] >= 1024 || eb[j] >= 1024) {
            const double qnan = __longlong_as_double(0x7ff8000000000000ll);
            double2 *pc = C + 2 * (i + (int64_t)j * ldc);
            pc[0] = make_double2(qnan, qnan);
            pc[1] = make_double2(qnan, qnan);
            return;
        }
        xw::XW vr, vi;
        vr = vi = xw::zero();
        if (ea[i] > kNoExp / 2 && eb[j] > kNoExp / 2) {
            crt::Frac accr, acci;
            accr.reset();
            acci.reset();
            auto add_l = [&](int l, int p1, int p2, int p3) {
                const int p = (int)sm.pm[l];
                int re = p1 - p2;
                if (re < 0) re += p;
                int im = p3 - p1 - p2;
                if (im < 0) im += p;
                if (im < 0) im += p;
                accr.add(sm.F[l], (uint32_t)re);
                acci.add(sm.F[l], (uint32_t)im);
            };
            const uint16_t *rp = R + (int64_t)j * Mp + i;
            const int64_t plane = Np * Mp;
            int l = 0;
            for (; l + 4 <= nmod; l += 4) {
                int c[4][3];
#pragma unroll
                for (int u = 0; u < 4; ++u)
#pragma unroll
                    for (int z = 0; z < 3; ++z) c[u][z] = __ldcs(rp + z * cstride + (int64_t)(l + u) * plane);
#pragma unroll
                for (int u = 0; u < 4; ++u) add_l(l + u, c[u][0], c[u][1], c[u][2]);
            }
            for (; l < nmod; ++l) {
                const uint16_t *q = rp + (int64_t)l * plane;
                add_l(l, __ldcs(q), __ldcs(q + cstride), __ldcs(q + 2 * cstride));
            }
            const int S2 = bsum - 4 - ea[i] - eb[j];
            vr = accr.finish_xw(Mx, S2);
            vi = acci.finish_xw(Mx, S2);
        }
        xw::XW rr = vr, ri = vi;
        if (!alpha_one) {
            xw::XW t = xw::mul(ai, vi);
            t.neg ^= 1u;
            rr = xw::add(xw::mul(ar, vr), t);
            ri = xw::add(xw::mul(ar, vi), xw::mul(ai, vr));
        }
        double2 *pc = C + 2 * (i + (int64_t)j * ldc);
        if (beta_kind != 0) {
            double2 c0r = pc[0], c0i = pc[1];
            if (!finite_hi(c0r.x) || !finite_hi(c0i.x)) {
                dd::cplx c0;
                c0.re = dd::make(c0r.x, c0r.y);
                c0.im = dd::make(c0i.x, c0i.y);
                if (beta_kind == 2) {
                    if (real_beta) {
                        c0.re = dd::mul_exact(beta.re, c0.re);
                        c0.im = dd::mul_exact(beta.re, c0.im);
                    } else {
                        c0 = dd::cmul_exact(c0, beta);
                    }
                }
                dd::cplx out;
                out.re = dd::add_exact(c0.re, xw_dd(rr));
                out.im = dd::add_exact(c0.im, xw_dd(ri));
                if (herm && i == j) out.im = dd::make(0.0, 0.0);
                dd::cstore(pc, out);
                return;
            }
            xw::XW cr = xw::from_dd(c0r.x, c0r.y), ci = xw::from_dd(c0i.x, c0i.y);
            if (beta_kind == 2) {
                if (real_beta) {
                    cr = xw::mul(br, cr);
                    ci = xw::mul(br, ci);
                } else {
                    xw::XW t = xw::mul(bi, ci);
                    t.neg ^= 1u;
                    xw::XW nr = xw::add(xw::mul(br, cr), t);
                    xw::XW ni = xw::add(xw::mul(br, ci), xw::mul(bi, cr));
                    cr = nr;
                    ci = ni;
                }
            }
            rr = xw::add(rr, cr);
            ri = xw::add(ri, ci);
        }
        dd::cplx out;
        out.re = xw_dd(rr);
        out.im = (herm && i == j) ? dd::make(0.0, 0.0) : xw_dd(ri);
        dd::cstore(pc, out);
    };
    if (uplo != 0) {
        // a triangle: (256-row slab, column) tasks shared evenly by all blocks
        const int64_t S = blockDim.x, slabs = (m + S - 1) / S, total = tri_prefix(uplo, slabs, n, S);
        for (int64_t t = (int64_t)blockIdx.y * gridDim.x + blockIdx.x; t < total;
             t += (int64_t)gridDim.x * gridDim.y) {
            int64_t x, j;
            tri_task(uplo, t, slabs, n, S, x, j);
            const int i = (int)(x * S) + threadIdx.x;
            if (i < m) one(i, (int)j);
        }
        return;
    }
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    for (int j = blockIdx.y; j < n; j += gridDim.y) one(i, j);
}

// ---- host ---------------------------------------------------------------------------------

PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;

bool get_encode()
{
    if (!g_encode) g_encode = (PFN_cuTensorMapEncodeTiled_v12000)tensor_map_encoder();
    return g_encode != nullptr;
}

bool make_map(CUtensorMap *map, const void *base, uint64_t kpad, uint64_t rows, uint32_t box_rows, const char *routine)
{
    cuuint64_t dims[2] = {kpad, rows};
    cuuint64_t strides[1] = {kpad * 2};
    cuuint32_t box[2] = {64, box_rows};
    cuuint32_t es[2] = {1, 1};
    CUresult r = g_encode(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2, const_cast<void *>(base), dims, strides, box, es,
                          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                          CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        set_error(routine, MWBLAS_ERR_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
        return false;
    }
    return true;
}

void fill_res_params(const Moduli &md, OzResParams &rp, OzModParams &mp)
{
    rp.nmod = md.n;
    for (int l = 0; l < md.n; ++l) {
        int p = md.p[l];
        rp.p[l] = (float)p;
        rp.invp[l] = 1.0f / (float)p;
        for (int comp = 0; comp < 3; ++comp) {
            mp.p[comp * md.n + l] = (float)p;
            mp.invp[comp * md.n + l] = 1.0f / (float)p;
        }
        int64_t t = 1;
        for (int q = 0; q < kResLimbs; ++q) {
            rp.t[l][q] = (float)(t > p / 2 ? t - p : t);   // symmetric: |t| <= p/2
            t = (t * 2048) % p;
        }
    }
}

void fill_crt_params(const Moduli &md, OzCrtParams &cp)
{
    cp.nmod = md.n;
    xfp::XF Mx;
    crt::constants(md.p, md.n, cp.F, Mx);
    for (int l = 0; l < md.n; ++l) cp.pm[l] = (float)md.p[l];
    cp.Mhi = (uint64_t)(Mx.m >> 64);
    cp.Mlo = (uint64_t)Mx.m;
    cp.Me = Mx.e;
}

unsigned blocks_cap(int64_t want)
{
    int64_t cap = 65535;
    if (want > cap) want = cap;
    return (unsigned)(want < 1 ? 1 : want);
}

}  // namespace

bool ozaki_available()
{
    const char *e = getenv("MWBLAS_OZAKI");
    if (e && !strcmp(e, "0")) return false;
    int dev = 0, major = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return false;
    cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev);
    if (major != 10) return false;
    return get_encode();
}

int ozaki_last_moduli() { return g_last_moduli; }
int ozaki_last_bits(int operand) { return (operand == 0 || operand == 1) ? g_last_bits[operand] : 0; }

namespace {

// Significant width of op(X)'s rows (or op(B)'s columns): the largest
// e_i - low_i + 2 over rows that hold a nonzero finite entry, where e_i bounds
// the row's binary exponents and low_i is the exponent of its lowest set bit.
// Scaled to that many bits (A'_ip = a_ip * 2^(bits - 2 - e_i)), every entry of
// such a row is an exact integer below 2^(bits - 1).
constexpr int kLowNone = 0x3f3f3f3f;   // no nonzero finite entry (the scan's fill value)
__global__ void k_width(int64_t rows, const int *__restrict__ e, const int *__restrict__ low, int *out)
{
    int w = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < rows; i += (int64_t)gridDim.x * blockDim.x) {
        const int ei = e[i], li = low[i];
        if (ei > kNoExp / 2 && ei < 1024 && li != kLowNone) w = max(w, ei - li + 2);
    }
    for (int off = 16; off > 0; off >>= 1) w = max(w, __shfl_down_sync(0xffffffffu, w, off));
    if ((threadIdx.x & 31) == 0) atomicMax(out, w);
}


// Products at least this large (m n k) on device-resident operands size their
// moduli from the operands' significant width; the readback of the two widths
// costs one stream synchronisation (the GPU idles ~10-20 us meanwhile, about
// 1 % of a 1024^3 product).
constexpr double kWidthMinWork = 1024.0 * 1024.0 * 1024.0;

// The significant widths of op(A)'s rows and op(B)'s columns, read back to the
// host; false when they could not be (the caller then keeps the full width).
bool read_widths(int64_t m, int64_t n, const int *ea, const int *eb, const int *la, const int *lb, int *w,
                 int &wa, int &wb)
{
    thread_local int *host = nullptr;
    if (!host && cudaHostAlloc((void **)&host, 2 * sizeof(int), cudaHostAllocDefault) != cudaSuccess) {
        cudaGetLastError();
        host = nullptr;
        return false;
    }
    cudaMemsetAsync(w, 0, 2 * sizeof(int), stream());
    const int ga = (int)std::min<int64_t>((m + 255) / 256, 4 * (int64_t)device_sm_count());
    const int gb = (int)std::min<int64_t>((n + 255) / 256, 4 * (int64_t)device_sm_count());
    k_width<<<ga, 256, 0, stream()>>>(m, ea, la, w);
    k_width<<<gb, 256, 0, stream()>>>(n, eb, lb, w + 1);
    count_launch(2);
    if (cudaMemcpyAsync(host, w, 2 * sizeof(int), cudaMemcpyDeviceToHost, stream()) != cudaSuccess ||
        cudaStreamSynchronize(stream()) != cudaSuccess) {
        return false;   // the routine's own synchronisation reports the error
    }
    wa = host[0];
    wb = host[1];
    return true;
}

bool gemm_ozaki(const GemmArgs &g0, bool cplx, int bits_req, const char *routine)
{
    // Split K so that the residue sums and the CRT bound stay in range.
    const int64_t kmax = 65536;
    const int E = cplx ? 2 : 1;
    if (g0.k > kmax) {
        GemmArgs g = g0;
        for (int64_t k0 = 0; k0 < g0.k; k0 += kmax) {
            g.k = (g0.k - k0 < kmax) ? g0.k - k0 : kmax;
            g.A = (const double2 *)g0.A + E * (g0.ta ? k0 : k0 * g0.lda);
            g.B = (const double2 *)g0.B + E * (g0.tb ? k0 * g0.ldb : k0);
            if (k0 > 0) {
                g.beta = dd_host{1.0, 0.0};
                g.cbeta = cdd_host{{1.0, 0.0}, {0.0, 0.0}};
                g.beta_kind = 1;
            }
            if (!gemm_ozaki(g, cplx, bits_req, routine)) return false;
        }
        return true;
    }
    const GemmArgs &g = g0;
    const int64_t m = g.m, n = g.n, k = g.k;
    if (m > INT32_MAX || n > INT32_MAX) {   // the reconstruction indexes rows and columns in 32 bits
        if (g.hs && !g.hs->wait_all(routine)) return false;
        return cplx ? gemm_plain_cplx(g, routine) : gemm_fixed_real(g, routine);
    }
    const int nc = cplx ? 3 : 1;
    // Real SYRK (op(B) = op(A)^T on the same array): op(B)'s residue rows are
    // op(A)'s, so one conversion serves both operands; both then use the same
    // per-modulus row padding.
    const bool shared_ops = !cplx && g.uplo != 0 && g.A == g.B && g.lda == g.ldb && g.ta != g.tb && m == n;
    const int64_t Np = (n + TC_BN - 1) / TC_BN * TC_BN;
    const int64_t Mp = shared_ops ? Np : (m + 255) / 256 * 256;   // the pair kernel's 256-row tiles
    const int64_t Kp = (k + TC_BK - 1) / TC_BK * TC_BK;

    // 1. exponent bounds of the rows of op(A) / columns of op(B)
    const bool scal_nonfinite =
        cplx ? !(std::isfinite(g.calpha.re.hi) && std::isfinite(g.calpha.im.hi) && std::isfinite(g.cbeta.re.hi) &&
                 std::isfinite(g.cbeta.im.hi))
             : !(std::isfinite(g.alpha.hi) && std::isfinite(g.beta.hi));
    if (scal_nonfinite) {
        // Inf/NaN alpha or beta: the FP64 engine propagates them as the
        // reference's operators do.
        if (g.hs && !g.hs->wait_all(routine)) return false;
        return cplx ? gemm_plain_cplx(g, routine) : gemm_plain_real(g, routine);
    }
    // Inf/NaN entries of A or B need no host round trip: their rows/columns
    // carry exponent bound 1024, the residues there are don't-care values,
    // and the reconstruction writes NaN to every output they reach (the
    // reference's double-double product of an infinity is NaN).
    // The moduli count follows from the operands' significant width where the
    // operands are on the device and the call may wait for the exponent scan
    // (not while a stream is being captured); otherwise from the full width.
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(stream(), &cap) != cudaSuccess) {
        cudaGetLastError();
        cap = cudaStreamCaptureStatusActive;
    }
    const bool detect = bits_req <= 0 && g.width && !g.hs && cap == cudaStreamCaptureStatusNone &&
                        (double)m * (double)n * (double)k >= kWidthMinWork;
    int *ex = (int *)dev_alloc(sizeof(int) * (size_t)(detect ? 2 * (m + n) + 4 : m + n + 2), routine);
    if (!ex) return false;
    int *ea = ex, *eb = ex + m;
    int *la = detect ? ex + m + n : nullptr, *lb = detect ? la + m : nullptr, *wbuf = detect ? lb + n : nullptr;
    // Operands still arriving from the host: A's exponents and residues are
    // computed while B is copied, and C is waited for only by the
    // reconstruction, so its copy runs under the residue GEMMs.
    HostStage *hs = g.hs;
    phase_mark(PH_EXP);
    const bool a_blocks = hs && hs->a_rows > 0;   // op(A) scanned and converted block by block below
    if (hs && !wait_event(hs->a_ready, routine)) {
        dev_free(ex);
        return false;
    }
    if (!a_blocks) launch_exp_rows_of_op(g.A, g.ta ? k : m, g.ta ? m : k, g.lda, g.ta, E, ea, la);
    if (!hs) launch_exp_cols_of_op(g.B, g.tb ? n : k, g.tb ? k : n, g.ldb, g.tb, E, eb, lb);

    // 2. precision and moduli. Rows of op(A) are scaled to bits_a bits and
    // columns of op(B) to bits_b: by default the 106 bits of a double-double,
    // fewer where every entry is an exact integer at fewer bits (double values
    // with lo = 0 over a limited exponent range, say), which loses nothing.
    // |A'B'| <= k 2^(bits_a + bits_b - 2) (complex: |Re|, |Im| twice that).
    int bits = bits_req > 0 ? bits_req : 106;
    if (bits < 40) bits = 40;
    if (bits > 120) bits = 120;
    int bits_a = bits, bits_b = bits;
    if (detect) {
        int wa = 0, wb = 0;
        if (read_widths(m, n, ea, eb, la, lb, wbuf, wa, wb)) {
            bits_a = std::max(8, std::min(bits, wa));
            bits_b = std::max(8, std::min(bits, wb));
        }
    }
    if (shared_ops) bits_a = bits_b = std::max(bits_a, bits_b);   // one conversion serves both operands
    const double need = (bits_a - 1) + (bits_b - 1) + std::log2((double)(k > 1 ? k : 1)) + 1.0 + 4.0 + (cplx ? 1.0 : 0.0);
    Moduli md = choose_moduli(need);
    g_last_moduli = md.n;
    g_last_bits[0] = bits_a;
    g_last_bits[1] = bits_b;
    OzResParams rp;
    OzModParams mp;
    OzCrtParams cp;
    fill_res_params(md, rp, mp);
    fill_crt_params(md, cp);

    // 3. residue operands: [comp][modulus][row][k] fp16
    const size_t a_bytes = (size_t)nc * md.n * Mp * Kp * 2;
    const size_t b_bytes = shared_ops ? 0 : (size_t)nc * md.n * Np * Kp * 2;
    const size_t r_bytes = (size_t)nc * md.n * Np * Mp * sizeof(uint16_t);
    uint8_t *work = (uint8_t *)dev_alloc(a_bytes + b_bytes + r_bytes + 256, routine);
    if (!work) {
        dev_free(ex);
        return false;
    }
    __half *Ares = (__half *)work;
    __half *Bres = shared_ops ? Ares : (__half *)(work + a_bytes);
    uint16_t *R = (uint16_t *)(work + a_bytes + b_bytes);
    phase_mark(PH_RES);
    // op(B) and C arriving in column blocks (pair kernel, full output): the
    // columns of block j are converted, multiplied, reconstructed and copied
    // back while later blocks are still being uploaded.
    // (Device operands are not blocked: a reconstruction running beside the
    // residue GEMM slows it by about as much as it hides, 8192^3: 17.2 ->
    // 19.3 ms for 2.1 ms of reconstruction.)
    const int64_t block_w = hs ? hs->block_cols : 0;
    const bool blocked = block_w > 0 && block_w < n + TC_BN && mma_kind() == 3 && !shared_ops && g.uplo == 0 &&
                         !g.herm;
    const bool ok_pre = !(hs && hs->block_cols > 0 && !blocked) || hs->wait_all(routine);
    // op(A) = A: A[i + p*lda] is contiguous along rows; op(A) = A^T along k.
    // Rows [i0, i0 + ni) of op(A), with their exponent bounds, go to residue
    // rows [i0, i0 + rpad) of every plane (zeros past m).
    auto a_rows_at = [&](int64_t i0) { return (const double2 *)g.A + (int64_t)E * (g.ta ? i0 * g.lda : i0); };
    auto convert_A = [&](int64_t i0, int64_t ni, int64_t rpad) {
        const double2 *Ai = a_rows_at(i0);
        __half *Ao = Ares + i0 * Kp;
        if (cplx) {
            if (!g.ta) launch_residues<true, true>(ni, k, Ai, g.lda, ea + i0, bits_a, rp, Ao, rpad, Kp, g.ca, Mp);
            else launch_residues<false, true>(ni, k, Ai, g.lda, ea + i0, bits_a, rp, Ao, rpad, Kp, g.ca, Mp);
        } else {
            const bool tc = !g.ta ? launch_residues_tc<true>(ni, k, Ai, g.lda, ea + i0, bits_a, rp, Ao, rpad, Kp, Mp)
                                  : launch_residues_tc<false>(ni, k, Ai, g.lda, ea + i0, bits_a, rp, Ao, rpad, Kp, Mp);
            if (tc) return;
            if (!g.ta) launch_residues<true, false>(ni, k, Ai, g.lda, ea + i0, bits_a, rp, Ao, rpad, Kp, 0, Mp);
            else launch_residues<false, false>(ni, k, Ai, g.lda, ea + i0, bits_a, rp, Ao, rpad, Kp, 0, Mp);
        }
    };
    // row block ib of op(A): wait for it, scan its exponents, convert it
    auto a_block = [&](int64_t ib) {
        const int64_t h = hs->a_rows, i0 = ib * h, ni = (m - i0 < h) ? m - i0 : h;
        wait_event(ib < (int64_t)hs->a_block.size() ? hs->a_block[ib] : nullptr, routine);
        launch_exp_rows_of_op(a_rows_at(i0), g.ta ? k : ni, g.ta ? ni : k, g.lda, g.ta, E, ea + i0);
        convert_A(i0, ni, i0 + h >= m ? Mp - i0 : ni);
    };
    const int64_t n_ablocks = a_blocks ? (m + hs->a_rows - 1) / hs->a_rows : 0;
    if (!a_blocks) {
        convert_A(0, m, Mp);
    } else if (!blocked) {
        for (int64_t ib = 0; ib < n_ablocks; ++ib) a_block(ib);
    }
    // op(B)(p, j) = B[p + j*ldb] is contiguous along k; op(B) = B^T along the
    // columns j. Columns [j0, j0 + nn) of op(B), and their exponent bounds,
    // go to residue rows [j0, j0 + rpad) of every plane (zeros past n).
    auto b_cols = [&](int64_t j0) { return (const double2 *)g.B + (int64_t)E * (g.tb ? j0 : j0 * g.ldb); };
    auto exp_B = [&](int64_t j0, int64_t nn) {
        launch_exp_cols_of_op(b_cols(j0), g.tb ? nn : k, g.tb ? k : nn, g.ldb, g.tb, E, eb + j0);
    };
    auto convert_B = [&](int64_t j0, int64_t nn, int64_t rpad) {
        const double2 *Bj = b_cols(j0);
        __half *Bo = Bres + j0 * Kp;
        if (cplx) {
            if (!g.tb) launch_residues<false, true>(nn, k, Bj, g.ldb, eb + j0, bits_b, rp, Bo, rpad, Kp, g.cb, Np);
            else launch_residues<true, true>(nn, k, Bj, g.ldb, eb + j0, bits_b, rp, Bo, rpad, Kp, g.cb, Np);
        } else {
            const bool tc = !g.tb ? launch_residues_tc<false>(nn, k, Bj, g.ldb, eb + j0, bits_b, rp, Bo, rpad, Kp, Np)
                                  : launch_residues_tc<true>(nn, k, Bj, g.ldb, eb + j0, bits_b, rp, Bo, rpad, Kp, Np);
            if (tc) return;
            if (!g.tb) launch_residues<false, false>(nn, k, Bj, g.ldb, eb + j0, bits_b, rp, Bo, rpad, Kp, 0, Np);
            else launch_residues<true, false>(nn, k, Bj, g.ldb, eb + j0, bits_b, rp, Bo, rpad, Kp, 0, Np);
        }
    };
    if (!blocked) {
        if (hs) {
            wait_event(hs->b_ready, routine);
            exp_B(0, n);
        }
        if (!shared_ops) convert_B(0, n, Np);
    }

    // 4. residue GEMMs, one batch entry per (component, modulus)
    phase_mark(PH_GEMM);
    bool ok = ok_pre;
    const int nz = nc * md.n;
    CUtensorMap ma, mb;
    // CTA-pair kernel over the column tiles [tn0, tn0 + ntn) and the 256-row
    // tile pairs [tm0, tm0 + ntm) of the product (ntm = 0: all of them)
    auto pair_gemm = [&](int tn0, int ntn, int tm0 = 0, int ntm = 0) {
        cudaFuncSetAttribute(k_oz_gemm_tc_2sm, cudaFuncAttributeMaxDynamicSharedMemorySize, T2_SMEM);
        const int tiles_m2 = ntm > 0 ? ntm : (int)(Mp / 256);
        const int64_t units = (int64_t)nz * tiles_m2 * ntn;
        const int64_t pairs = device_sm_count() / 2;
        const unsigned grid = 2u * (unsigned)(units < pairs ? units : pairs);
        k_oz_gemm_tc_2sm<<<grid, TCP_THREADS, T2_SMEM, stream()>>>(ma, mb, Mp, Np, Kp, m, n, mp, R,
                                                                   device_status_word(), g.uplo, tiles_m2, ntn, nz,
                                                                   tn0, tm0, take_lost_load_injection(), nz);
    };
    if (blocked) {
        // launched block by block with the reconstruction below
        ok = ok && make_map(&ma, Ares, (uint64_t)Kp, (uint64_t)(nz * Mp), TC_BM, routine) &&
             make_map(&mb, Bres, (uint64_t)Kp, (uint64_t)(nz * Np), 128, routine);
    } else if (mma_kind() == 0 || mma_kind() == 2 || mma_kind() == 3) {
        ok = ok && make_map(&ma, Ares, (uint64_t)Kp, (uint64_t)(nz * Mp), TC_BM, routine) &&
             make_map(&mb, Bres, (uint64_t)Kp, (uint64_t)(nz * Np), mma_kind() == 3 ? 128 : TC_BN, routine);
        if (ok) {
            if (mma_kind() == 3) {
                pair_gemm(0, (int)(Np / TC_BN));
            } else if (mma_kind() == 2) {
                cudaFuncSetAttribute(k_oz_gemm_tc_p, cudaFuncAttributeMaxDynamicSharedMemorySize, TC_SMEM);
                const int tiles_m = (int)(Mp / TC_BM), tiles_n = (int)(Np / TC_BN);
                const int64_t units = (int64_t)nz * tiles_m * tiles_n;
                const int64_t sms = device_sm_count();
                const unsigned grid = (unsigned)(units < sms ? units : sms);
                k_oz_gemm_tc_p<<<grid, TCP_THREADS, TC_SMEM, stream()>>>(ma, mb, Mp, Np, Kp, m, n, mp, R,
                                                                         device_status_word(), g.uplo, tiles_m,
                                                                         tiles_n, nz);
            } else {
                cudaFuncSetAttribute(k_oz_gemm_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, TC_SMEM);
                dim3 grid((unsigned)(Np / TC_BN), (unsigned)(Mp / TC_BM), (unsigned)nz);
                k_oz_gemm_tc<<<grid, 192, TC_SMEM, stream()>>>(ma, mb, Mp, Np, Kp, m, n, mp, R, device_status_word(),
                                                               g.uplo);
            }
            count_launch();
        }
    } else {
        dim3 grid((unsigned)(Np / 16), (unsigned)(Mp / 16), (unsigned)nz);
        k_oz_gemm_simt<<<grid, 256, 0, stream()>>>(Ares, Bres, Mp, Np, Kp, m, n, mp, R);
        count_launch();
    }


    // 5. reconstruction + alpha/beta
    phase_mark(PH_REC);
    // a thread per row and several columns: about 16 blocks per SM in all
    const unsigned gx = (unsigned)((m + (cplx ? 255 : 511)) / (cplx ? 256 : 512));
    const int64_t want_y = ((int64_t)device_sm_count() * 16 + gx - 1) / gx;
    xw::XW Mx;
    Mx.w[3] = (uint32_t)(cp.Mhi >> 32);
    Mx.w[2] = (uint32_t)cp.Mhi;
    Mx.w[1] = (uint32_t)(cp.Mlo >> 32);
    Mx.w[0] = (uint32_t)cp.Mlo;
    Mx.e = cp.Me;
    Mx.neg = 0u;
    // columns [j0, j0 + nn) of C
    auto reconstruct_cols = [&](int64_t j0, int64_t nn) {
        dim3 grid(gx, blocks_cap(want_y < nn ? want_y : nn));
        const uint16_t *Rj = R + j0 * Mp;     // column j0 of every residue plane
        double2 *Cj = (double2 *)g.C + (int64_t)E * j0 * g.ldc;
        if (!cplx) {
            bool alpha_one = (g.alpha.hi == 1.0 && g.alpha.lo == 0.0);
            // alpha folded into M: alpha * X = T * (alpha M)
            const xw::XW aM = alpha_one ? Mx : xw::mul(xw::from_dd(g.alpha.hi, g.alpha.lo), Mx);
            k_oz_reconstruct<<<grid, 256, 0, stream()>>>((int)m, (int)nn, Rj, Mp, Np, ea, eb + j0, bits_a + bits_b, cp, aM,
                                                        xw::from_dd(g.beta.hi, g.beta.lo),
                                                        dd::make(g.beta.hi, g.beta.lo), g.beta_kind, Cj, g.ldc,
                                                        g.uplo);
        } else {
            dd::cplx al, be;
            al.re = dd::make(g.calpha.re.hi, g.calpha.re.lo);
            al.im = dd::make(g.calpha.im.hi, g.calpha.im.lo);
            be.re = dd::make(g.cbeta.re.hi, g.cbeta.re.lo);
            be.im = dd::make(g.cbeta.im.hi, g.cbeta.im.lo);
            bool alpha_one = (g.calpha.re.hi == 1.0 && g.calpha.re.lo == 0.0 && g.calpha.im.hi == 0.0 &&
                              g.calpha.im.lo == 0.0);
            k_oz_reconstruct_c<<<grid, 256, 0, stream()>>>(
                (int)m, (int)nn, Rj, Mp, Np, ea, eb + j0, bits_a + bits_b, cp, Mx, xw::from_dd(al.re.hi, al.re.lo),
                xw::from_dd(al.im.hi, al.im.lo), alpha_one ? 1 : 0, be, xw::from_dd(be.re.hi, be.re.lo),
                xw::from_dd(be.im.hi, be.im.lo), g.beta_kind, Cj, g.ldc, g.uplo, g.herm ? 1 : 0, g.herm ? 1 : 0);
        }
        count_launch();
    };
    if (ok && blocked) {
        // block j: its columns of op(B) converted and multiplied on this stream;
        // its reconstruction (and, for host arrays, write-back) on the side
        // stream, where it runs beside the next blocks' residue GEMMs (the
        // pair kernel leaves registers and shared memory for it on every SM)
        const int64_t w = block_w;
        static const std::vector<cudaEvent_t> none;
        const std::vector<cudaEvent_t> &bev = hs ? hs->b_block : none, &cev = hs ? hs->c_block : none;
        auto ev = [&](const std::vector<cudaEvent_t> &v, int64_t i) -> cudaEvent_t {
            return i < (int64_t)v.size() ? v[i] : nullptr;
        };
        const cudaStream_t main_s = stream(), side = side_stream();
        auto finish_block = [&](int64_t jb, int64_t j0, int64_t nn) -> bool {
            if (!order_streams(main_s, side, routine)) return false;
            StreamOverride so(side);
            if (!wait_event(ev(cev, jb), routine)) return false;
            reconstruct_cols(j0, nn);
            return !hs || unstage_columns_async(*hs->c, j0, j0 + nn, routine);
        };
        int64_t first = 0;   // column blocks done in the row-blocked phase
        if (a_blocks && hs->early_blocks > 0) {
            // the first early_blocks column blocks row block by row block, as A arrives
            first = hs->early_blocks;
            const int64_t jend = (first * w < n) ? first * w : n;
            const int ntn = (int)(((jend >= n) ? Np : jend) / TC_BN);
            for (int64_t ib = 0; ok && ib < n_ablocks; ++ib) {
                a_block(ib);
                for (int64_t jb = 0; ok && ib == 0 && jb < first; ++jb) {
                    const int64_t j0 = jb * w, nn = (n - j0 < w) ? n - j0 : w;
                    ok = wait_event(ev(bev, jb), routine);
                    if (!ok) break;
                    exp_B(j0, nn);
                    convert_B(j0, nn, (j0 + w >= n) ? Np - j0 : nn);
                }
                if (!ok) break;
                const int64_t i0 = ib * hs->a_rows;
                const int64_t rows = (i0 + hs->a_rows >= m) ? Mp - i0 : hs->a_rows;
                gemm_mark(true);
                pair_gemm(0, ntn, (int)(i0 / 256), (int)(rows / 256));
                gemm_mark(false);
                count_launch();
            }
            for (int64_t jb = 0; ok && jb < first; ++jb) {
                const int64_t j0 = jb * w, nn = (n - j0 < w) ? n - j0 : w;
                ok = finish_block(jb, j0, nn);
            }
        }
        for (int64_t j0 = first * w, jb = first; ok && j0 < n; j0 += w, ++jb) {
            const int64_t nn = (n - j0 < w) ? n - j0 : w;
            const bool last = j0 + w >= n;
            const int ntn = (int)((last ? Np - j0 : nn) / TC_BN);
            ok = wait_event(ev(bev, jb), routine);
            if (!ok) break;
            exp_B(j0, nn);
            convert_B(j0, nn, last ? Np - j0 : nn);
            gemm_mark(true);
            pair_gemm((int)(j0 / TC_BN), ntn);
            gemm_mark(false);
            count_launch();
            ok = finish_block(jb, j0, nn);
        }
        // the buffers are freed on this stream: order that after the side
        // stream's kernels and the copies back
        if (hs && !flush_columns_back(*hs->c, routine)) ok = false;
        if (!order_streams(side, main_s, routine)) ok = false;
        if (ok && hs) {
            ok = join_copy_stream(routine);
            hs->c_written = ok;
        }
    } else if (ok) {
        if (hs) ok = wait_event(hs->c_ready, routine);
        // C going back to the host: the reconstruction runs in column chunks,
        // each copied back while the next one is computed
        const bool chunked = hs && hs->c && g.uplo == 0 && !g.herm;
        const int64_t cw = chunked ? (n + 7) / 8 : n;
        for (int64_t j0 = 0; ok && j0 < n; j0 += cw) {
            const int64_t nn = (n - j0 < cw) ? n - j0 : cw;
            reconstruct_cols(j0, nn);
            if (chunked) ok = unstage_columns_async(*hs->c, j0, j0 + nn, routine);
        }
        if (chunked && !flush_columns_back(*hs->c, routine)) ok = false;
        if (ok && chunked) {
            ok = join_copy_stream(routine);
            hs->c_written = ok;
        }
    }
    phase_mark(PH_N);
    dev_free(work);
    dev_free(ex);
    if (!ok) return false;
    // a bounded wait that gave up is reported when the calling routine
    // synchronises (finish() reads the device status word)
    phase_collect();
    return true;
}

// ---- grouped products on the tensor cores (large instances of mgemm_grouped) ----------
//
// Instances are padded to classes (Mp, Np multiples of 256, Kp of 64) and every
// class runs as one CTA-pair residue GEMM over count x L planes: plane
// slot * L + l holds modulus l of the slot's product. Exponents, residues and
// the reconstruction run as one batched launch each over all instances.
// Everything is enqueued without host round trips (full 106-bit width), so
// the whole sequence can be captured in a CUDA graph.
//
// Small instances share slots: in a 256 x 256 slot, instance t takes rows
// [r_t, r_t + m_t) of op(A)'s plane and of the product, columns
// [c_t, c_t + n_t) (rows of op(B)'s plane), disjoint from the other
// instances', and K columns [0, k_t). The slot product is then
// block-diagonal where it is read: its (r_t, c_t) block sums only over
// instance t's own K range (its rows are zero beyond k_t), and the blocks
// mixing two instances are never read. Only an instance's own rows are
// written; the rest of every plane was zeroed when the plan was prepared.

struct OzGrpDesc {
    const double2 *A, *B;
    double2 *C;
    int64_t lda, ldb, ldc;
    int m, n, k, ta, tb;
    int cls, slot;
    int64_t ea_off, eb_off;   // row exponents of op(A), column exponents of op(B)
    int64_t line_begin;       // first exponent work item: ceil(m/32) row groups of op(A), then ceil(n/32) column groups of op(B)
    int64_t tile_begin;       // first conversion tile: op(A)'s ceil(m/R) ceil(k/32), then op(B)'s ceil(n/R) ceil(k/32) (R = 16 on the tensor cores, else 32)
    int64_t rec_begin;        // first reconstruction item: ceil(m/64) row slabs x ceil(n/8) column groups
    xw::XW aM, xb;            // alpha * M and beta as extended floats
    double2 beta;
    int beta_kind;
    int r_off, c_off;         // first row of op(A) / of op(B)^T (= output column) in the slot
};

struct OzGrpClass {
    int64_t Mp, Np, Kp;
    __half *Ares, *Bres;      // [slot][l][row][k]
    uint16_t *R;              // [slot][l][col][row]
};

__device__ __forceinline__ int grp_find(const OzGrpDesc *__restrict__ d, int count, int64_t w, int which)
{
    int lo = 0, hi = count - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        const int64_t b = which == 0 ? d[mid].line_begin : (which == 1 ? d[mid].tile_begin : d[mid].rec_begin);
        if (b <= w) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

__device__ __forceinline__ int grp_exp_bound(double x)
{
    const uint64_t b = (uint64_t)__double_as_longlong(x) & 0x7fffffffffffffffull;
    return b == 0 ? kNoExp : (int)(b >> 52) - 1023;
}

// Exponent bound of every row of op(A) and column of op(B). A work item is a
// group of 32 consecutive lines of one operand (line_begin counts groups:
// ceil(m/32) of op(A), then ceil(n/32) of op(B)), taken by a block of eight
// warps: lines contiguous along k are split among the warps, each walked with
// the lanes over k; lines strided along k (rows of A, columns of B^T) take a
// lane each and the warps split k, so every load reads 32 neighbouring lines
// of one k (coalesced either way), and the eight partial maxima meet in
// shared memory.
__global__ void __launch_bounds__(256) k_grp_exp(const OzGrpDesc *__restrict__ descs, int count, int64_t lines,
                                                 int *__restrict__ ex)
{
    __shared__ int part[8][33];
    const int lane = threadIdx.x & 31, wq = threadIdx.x >> 5;
    for (int64_t w = blockIdx.x; w < lines; w += gridDim.x) {
        const OzGrpDesc &d = descs[grp_find(descs, count, w, 0)];
        const int ga = (d.m + 31) / 32;
        int g = (int)(w - d.line_begin);
        const bool isA = g < ga;
        if (!isA) g -= ga;
        const int nl = isA ? d.m : d.n, l0 = 32 * g, l1 = min(nl, l0 + 32);
        const double2 *X = isA ? d.A : d.B;
        const int64_t ld = isA ? d.lda : d.ldb;
        // line t of op(A) is A's column t (A^T) or row t; line j of op(B) is B's column j or row j (B^T)
        const bool along_k = isA ? d.ta : !d.tb;
        int *out = ex + (isA ? d.ea_off : d.eb_off);
        if (along_k) {
            for (int t = l0 + wq; t < l1; t += 8) {
                const double2 *p = X + (int64_t)t * ld;
                int e = kNoExp;
                for (int q = lane; q < d.k; q += 32) e = max(e, grp_exp_bound(p[q].x));
                for (int off = 16; off > 0; off >>= 1) e = max(e, __shfl_down_sync(0xffffffffu, e, off));
                if (lane == 0) out[t] = e;
            }
        } else {
            const int t = l0 + lane;
            int e = kNoExp;
            if (t < l1) {
                const double2 *p = X + t;
                for (int q = wq; q < d.k; q += 8) e = max(e, grp_exp_bound(p[(int64_t)q * ld].x));
            }
            part[wq][lane] = e;
            __syncthreads();
            if (wq == 0 && t < l1) {
#pragma unroll
                for (int u = 1; u < 8; ++u) e = max(e, part[u][lane]);
                out[t] = e;
            }
            __syncthreads();   // part is reused by the next item
        }
    }
}

// Residues of op(A) and op(B) of every instance into its class planes, one
// 32 x 32 tile per block and step. Tiles cover each operand's own rows and k
// (rounded up to 32, the excess filled with zeros); the rest of the class
// padding is zeroed once when the plan is prepared and never written.
__global__ void __launch_bounds__(256) k_grp_residues(const OzGrpDesc *__restrict__ descs, int count, int64_t tiles,
                                                      const OzGrpClass *__restrict__ classes, const int *__restrict__ ex,
                                                      int bits, OzResParams P)
{
    __shared__ __align__(16) double2 tile[32][33][1];
    __shared__ __align__(16) float2 s_t[kMaxMod][12];
    __shared__ __align__(16) float4 s_pp[kMaxMod];
    const int nmod = P.nmod;
    for (int i = threadIdx.x; i < nmod * 12; i += blockDim.x) {
        const int l = i / 12, q = i % 12;
        const float t = (q < kResLimbs) ? P.t[l][q] : 0.0f;
        s_t[l][q] = make_float2(t, t);
    }
    for (int i = threadIdx.x; i < nmod; i += blockDim.x) s_pp[i] = make_float4(-P.p[i], -P.p[i], P.invp[i], P.invp[i]);
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const int s = threadIdx.x >> 3, cg = (threadIdx.x & 7) * 4;
    for (int64_t w = blockIdx.x; w < tiles; w += gridDim.x) {
        const OzGrpDesc &d = descs[grp_find(descs, count, w, 1)];
        const OzGrpClass &c = classes[d.cls];
        // tiles cover op(X)'s own rows and k (the class padding was zeroed once)
        const int64_t ntc = (d.k + 31) / 32, ta_tiles = ((d.m + 31) / 32) * ntc;
        int64_t t = w - d.tile_begin;
        const bool isA = t < ta_tiles;
        if (!isA) t -= ta_tiles;
        const int64_t r0 = (t / ntc) * 32, c0 = (t % ntc) * 32;
        // op(X) element (r, c): op(A) = A or A^T; op(B)^T rows are B's columns (B) or rows (B^T)
        const double2 *X = isA ? d.A : d.B;
        const int64_t ld = isA ? d.lda : d.ldb;
        const int rows = isA ? d.m : d.n;
        const bool rowc = isA ? !d.ta : d.tb;   // rows contiguous in memory
        __syncthreads();   // the previous tile's limbs are taken
        for (int u = ty; u < 32; u += 8) {
            const int64_t r = rowc ? r0 + tx : r0 + u, col = rowc ? c0 + u : c0 + tx;
            double2 v = make_double2(0.0, 0.0);
            if (r < rows && col < d.k) v = rowc ? X[r + col * ld] : X[col + r * ld];
            if (rowc) tile[tx][u][0] = v;
            else tile[u][tx][0] = v;
        }
        __syncthreads();
        const int64_t r = r0 + s;
        const int e = r < rows ? ex[(isA ? d.ea_off : d.eb_off) + r] : kNoExp;
        float2 fr[2][kResLimbs], fi[1][kResLimbs];
        tile_limbs<false>(tile[s], cg, e, bits, 0, fr, fi);
        if (r < rows) {   // rows past the instance belong to the next one in a shared slot (or stay zero)
            const int64_t prow = isA ? c.Mp : c.Np;
            __half *base = isA ? c.Ares : c.Bres;
            __half *o = base + ((int64_t)d.slot * nmod * prow + (isA ? d.r_off : d.c_off) + r) * c.Kp + c0 + cg;
            store_residues<false>(fr, fi, nmod, s_t, s_pp, o, prow * c.Kp, 0);
        }
    }
}

// The same conversion on the tensor cores (the tile pipeline of
// k_oz_residues_tc): tiles of 16 rows x 32 k of one operand of one instance,
// listed per instance as op(A)'s ceil(m/16) ceil(k/32), then op(B)'s; rows
// past the instance are not stored (they belong to the next instance of a
// shared slot, or stay zero).
__global__ void __launch_bounds__(RT_THREADS, 4)
    k_grp_residues_tc(const OzGrpDesc *__restrict__ descs, int count, int64_t tiles,
                      const OzGrpClass *__restrict__ classes, const int *__restrict__ ex, int bits, OzResParams P,
                      int *status)
{
    extern __shared__ uint8_t rt_raw[];
    const RtCta cta = rt_setup(rt_raw, P);
    const int tid = threadIdx.x;
    const int rl = tid >> 3, cq = (tid & 7) * 4;
    const int nmod = P.nmod;
    struct Tile {
        __half *o;
        int64_t plane;
        int e;
        bool ok;
    };
    // loads this thread's four elements of tile w and locates their residues
    auto fetch = [&](int64_t w, double2 (&v)[4]) {
        const OzGrpDesc &d = descs[grp_find(descs, count, w, 1)];
        const OzGrpClass &c = classes[d.cls];
        const int ntc = (d.k + RT_COLS - 1) / RT_COLS, ta_tiles = ((d.m + RT_ROWS - 1) / RT_ROWS) * ntc;
        int t = (int)(w - d.tile_begin);
        const bool isA = t < ta_tiles;
        if (!isA) t -= ta_tiles;
        const int r = (t / ntc) * RT_ROWS + rl, col = (t % ntc) * RT_COLS + cq;
        const int rows = isA ? d.m : d.n;
        const bool rowc = isA ? !d.ta : d.tb;   // rows contiguous in memory
        const int64_t ld = isA ? d.lda : d.ldb;
        const bool ok = r < rows;
        const double2 *x = (isA ? d.A : d.B) + (rowc ? r + (int64_t)col * ld : col + (int64_t)r * ld);
        const int64_t step = rowc ? ld : 1;
#pragma unroll
        for (int u = 0; u < 4; ++u) v[u] = (ok && col + u < d.k) ? x[u * step] : make_double2(0.0, 0.0);
        const int64_t prow = isA ? c.Mp : c.Np;
        Tile T;
        T.plane = prow * c.Kp;
        T.o = (isA ? c.Ares : c.Bres) + ((int64_t)d.slot * nmod * prow + (isA ? d.r_off : d.c_off) + r) * c.Kp + col;
        T.e = ok ? ex[(isA ? d.ea_off : d.eb_off) + r] : kNoExp;
        T.ok = ok;
        return T;
    };
    double2 cur[4];
    int64_t w = blockIdx.x;
    Tile T{}, Tp{};
    if (w < tiles) T = fetch(w, cur);
    bool have_prev = false;
    int it = 0, failed = 0;
    for (; w < tiles; ++it) {
        const int b = it & 1;
        rt_limbs(cta.sA + b * RT_TILE_BYTES, tid, cur, T.e, bits);
        const int64_t w2 = w + gridDim.x;
        Tile T2{};
        if (w2 < tiles) T2 = fetch(w2, cur);   // in flight during the epilogue and the MMA below
        if (!rt_step(cta, P, b, it, have_prev, Tp.o, Tp.plane, Tp.ok, status, failed)) break;
        Tp = T;
        have_prev = true;
        T = T2;
        w = w2;
    }
    rt_finish(cta, P, it, have_prev, Tp.o, Tp.plane, Tp.ok, status, failed);
    rt_teardown(cta);
}

// alpha * X * 2^-S2 + beta C for every instance. A work item is 64 rows x 8
// columns of one instance; thread t takes the row pair t % 32 of column t / 32
// (the 32 threads of a column read consecutive residue words).
__global__ void __launch_bounds__(256) k_grp_reconstruct(const OzGrpDesc *__restrict__ descs, int count,
                                                         int64_t items, const OzGrpClass *__restrict__ classes,
                                                         const int *__restrict__ ex, int bsum, OzCrtParams K)
{
    __shared__ CrtSmem sm;
    crt_smem_fill(sm, K);
    __syncthreads();
    const int nmod = K.nmod;
    for (int64_t w = blockIdx.x; w < items; w += gridDim.x) {
        const OzGrpDesc &d = descs[grp_find(descs, count, w, 2)];
        const OzGrpClass &c = classes[d.cls];
        const int64_t t = w - d.rec_begin, ncg = (d.n + 7) / 8;
        const int slab = (int)(t / ncg), j = (int)(t % ncg) * 8 + (threadIdx.x >> 5);
        const int i0 = slab * 64 + 2 * (threadIdx.x & 31);
        if (i0 >= d.m || j >= d.n) continue;
        const bool two = i0 + 1 < d.m;
        const int ea0 = ex[d.ea_off + i0], ea1 = two ? ex[d.ea_off + i0 + 1] : kNoExp;
        const int64_t plane = c.Np * c.Mp;
        const uint16_t *R0 = c.R + (int64_t)d.slot * nmod * plane + d.r_off + i0;
        const dd::real beta = dd::make(d.beta.x, d.beta.y);
        reconstruct_pair(sm, nmod, R0 + (int64_t)(d.c_off + j) * c.Mp, plane, i0, two, ea0, ea1, j,
                         ex[d.eb_off + j], bsum, d.aM, d.xb, beta, d.beta_kind, d.C + i0 + (int64_t)j * d.ldc, 0);
    }
}

}  // namespace

struct OzGroupPlan {
    std::vector<OzGrpDesc> descs;
    std::vector<OzGrpClass> classes;
    std::vector<int64_t> class_count;
    int64_t lines = 0, tiles = 0, items = 0;
    bool res_tc = false;   // residues on the tensor cores (16-row conversion tiles)
    Moduli md;
    OzResParams rp;
    OzModParams mp;
    OzCrtParams cp;
    std::vector<CUtensorMap> maps;   // two per class
    void *dev = nullptr;
    size_t dev_bytes = 0;
    OzGrpDesc *d_descs = nullptr;
    OzGrpClass *d_classes = nullptr;
    int *d_ex = nullptr;
};

OzGroupPlan *ozgroup_create() { return new OzGroupPlan(); }

void ozgroup_destroy(OzGroupPlan *p)
{
    if (!p) return;
    if (p->dev) cudaFree(p->dev);
    delete p;
}

int64_t ozgroup_count(const OzGroupPlan *p) { return p ? (int64_t)p->descs.size() : 0; }

namespace {

constexpr int kGroupBits = 106;

int64_t round_up(int64_t v, int64_t q) { return (v + q - 1) / q * q; }

// Kp of a class: 64, 128, 256, 512, then multiples of 512 (fewer classes)
int64_t class_kp(int64_t k)
{
    int64_t kp = 64;
    while (kp < k && kp < 512) kp *= 2;
    return kp >= k ? kp : round_up(k, 512);
}

}  // namespace

bool ozgroup_prepare(OzGroupPlan *pl, const std::vector<OzGroupItem> &items, const char *routine)
{
    pl->descs.clear();
    pl->classes.clear();
    pl->class_count.clear();
    pl->lines = pl->tiles = pl->items = 0;
    if (items.empty()) return true;
    if (!ozaki_available() || !get_encode()) {
        set_error(routine, MWBLAS_ERR_UNSUPPORTED, "tensor-core engine unavailable on this device");
        return false;
    }
    // moduli for the longest k (full width: no readback inside the graph)
    int64_t kmax = 1;
    for (const OzGroupItem &it : items) kmax = std::max<int64_t>(kmax, it.k);
    pl->md = choose_moduli(2.0 * (kGroupBits - 1) + std::log2((double)kmax) + 1.0 + 4.0);
    pl->res_tc = g_res_tc.load() != 0 && pl->md.n <= RT_MAX_MOD;
    const int trows = pl->res_tc ? RT_ROWS : 32;   // conversion tile rows
    fill_res_params(pl->md, pl->rp, pl->mp);
    fill_crt_params(pl->md, pl->cp);
    const int L = pl->md.n;
    xw::XW Mx;
    Mx.w[3] = (uint32_t)(pl->cp.Mhi >> 32);
    Mx.w[2] = (uint32_t)pl->cp.Mhi;
    Mx.w[1] = (uint32_t)(pl->cp.Mlo >> 32);
    Mx.w[0] = (uint32_t)pl->cp.Mlo;
    Mx.e = pl->cp.Me;
    Mx.neg = 0u;
    // classes and slots; shared slots are filled next-fit (rows and columns
    // in steps of 8) per class of Kp, deepest instances first
    std::map<std::tuple<int64_t, int64_t, int64_t, int>, int> cls_of;
    std::vector<int> pack_rows, pack_cols;   // per class: rows / columns used in its open shared slot
    std::vector<size_t> order(items.size());
    for (size_t t = 0; t < items.size(); ++t) order[t] = t;
    std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) {
        return items[a].pack != items[b].pack ? items[a].pack < items[b].pack : items[a].k > items[b].k;
    });
    int64_t exn = 0;
    for (const size_t t : order) {
        const OzGroupItem &it = items[t];
        const bool shared = it.pack && it.m <= 256 && it.n <= 256;
        const auto key = shared ? std::make_tuple((int64_t)256, (int64_t)256, class_kp(it.k), 1)
                                : std::make_tuple(round_up(it.m, 256), round_up(it.n, 256), class_kp(it.k), 0);
        auto f = cls_of.find(key);
        int ci;
        if (f == cls_of.end()) {
            ci = (int)pl->classes.size();
            cls_of[key] = ci;
            OzGrpClass c{};
            c.Mp = std::get<0>(key);
            c.Np = std::get<1>(key);
            c.Kp = std::get<2>(key);
            pl->classes.push_back(c);
            pl->class_count.push_back(0);
            pack_rows.push_back(256);   // no open slot yet
            pack_cols.push_back(256);
        } else {
            ci = f->second;
        }
        int slot, r_off = 0, c_off = 0;
        if (shared) {
            const int fm = (int)round_up(it.m, 8), fn = (int)round_up(it.n, 8);
            if (pack_rows[ci] + fm > 256 || pack_cols[ci] + fn > 256) {   // open the next slot
                pl->class_count[ci]++;
                pack_rows[ci] = pack_cols[ci] = 0;
            }
            slot = (int)pl->class_count[ci] - 1;
            r_off = pack_rows[ci];
            c_off = pack_cols[ci];
            pack_rows[ci] += fm;
            pack_cols[ci] += fn;
        } else {
            slot = (int)pl->class_count[ci]++;
        }
        OzGrpDesc d{};
        d.A = (const double2 *)it.A;
        d.B = (const double2 *)it.B;
        d.C = (double2 *)it.C;
        d.lda = it.lda;
        d.ldb = it.ldb;
        d.ldc = it.ldc;
        d.m = (int)it.m;
        d.n = (int)it.n;
        d.k = (int)it.k;
        d.ta = it.ta ? 1 : 0;
        d.tb = it.tb ? 1 : 0;
        d.cls = ci;
        d.slot = slot;
        d.r_off = r_off;
        d.c_off = c_off;
        d.ea_off = exn;
        d.eb_off = exn + it.m;
        exn += it.m + it.n;
        const OzGrpClass &c = pl->classes[ci];
        d.line_begin = pl->lines;
        pl->lines += (it.m + 31) / 32 + (it.n + 31) / 32;
        d.tile_begin = pl->tiles;
        pl->tiles += ((it.m + trows - 1) / trows + (it.n + trows - 1) / trows) * ((it.k + 31) / 32);
        d.rec_begin = pl->items;
        pl->items += ((it.m + 63) / 64) * ((it.n + 7) / 8);
        (void)c;
        const bool alpha_one = it.alpha.hi == 1.0 && it.alpha.lo == 0.0;
        d.aM = alpha_one ? Mx : xw::mul(xw::from_dd(it.alpha.hi, it.alpha.lo), Mx);
        d.xb = xw::from_dd(it.beta.hi, it.beta.lo);
        d.beta = make_double2(it.beta.hi, it.beta.lo);
        d.beta_kind = it.beta_kind;
        pl->descs.push_back(d);
    }
    // one buffer: [descriptors][classes][exponents][per class: A residues, B residues, products]
    const size_t d_bytes = round_up((int64_t)(pl->descs.size() * sizeof(OzGrpDesc)), 256);
    const size_t c_bytes = round_up((int64_t)(pl->classes.size() * sizeof(OzGrpClass)), 256);
    const size_t e_bytes = round_up(exn * (int64_t)sizeof(int), 256);
    size_t need = d_bytes + c_bytes + e_bytes;
    std::vector<size_t> off(pl->classes.size());
    for (size_t ci = 0; ci < pl->classes.size(); ++ci) {
        const OzGrpClass &c = pl->classes[ci];
        const int64_t planes = pl->class_count[ci] * L;
        off[ci] = need;
        need += round_up(planes * c.Mp * c.Kp * 2, 256) + round_up(planes * c.Np * c.Kp * 2, 256) +
                round_up(planes * c.Np * c.Mp * 2, 256);
    }
    if (pl->dev_bytes < need) {
        if (pl->dev) cudaFree(pl->dev);
        pl->dev = nullptr;
        pl->dev_bytes = 0;
        if (!cuda_ok(cudaMalloc(&pl->dev, need), routine, "grouped tensor-core plan buffer")) return false;
        pl->dev_bytes = need;
    }
    char *base = (char *)pl->dev;
    pl->d_descs = (OzGrpDesc *)base;
    pl->d_classes = (OzGrpClass *)(base + d_bytes);
    pl->d_ex = (int *)(base + d_bytes + c_bytes);
    pl->maps.assign(2 * pl->classes.size(), CUtensorMap{});
    for (size_t ci = 0; ci < pl->classes.size(); ++ci) {
        OzGrpClass &c = pl->classes[ci];
        const int64_t planes = pl->class_count[ci] * L;
        char *p = base + off[ci];
        c.Ares = (__half *)p;
        p += round_up(planes * c.Mp * c.Kp * 2, 256);
        c.Bres = (__half *)p;
        p += round_up(planes * c.Np * c.Kp * 2, 256);
        c.R = (uint16_t *)p;
        if (!make_map(&pl->maps[2 * ci], c.Ares, (uint64_t)c.Kp, (uint64_t)(planes * c.Mp), TC_BM, routine) ||
            !make_map(&pl->maps[2 * ci + 1], c.Bres, (uint64_t)c.Kp, (uint64_t)(planes * c.Np), 128, routine))
            return false;
        // the padding of the residue planes (rows past m or n, k past the 32-rounded k) is never
        // converted: zero it once
        if (!cuda_ok(cudaMemsetAsync(c.Ares, 0, (char *)c.R - (char *)c.Ares, stream()), routine,
                     "grouped residue clear"))
            return false;
    }
    cudaFuncSetAttribute(k_oz_gemm_tc_2sm, cudaFuncAttributeMaxDynamicSharedMemorySize, T2_SMEM);
    if (pl->res_tc) cudaFuncSetAttribute(k_grp_residues_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, RT_SMEM);
    cudaStream_t st = stream();
    return cuda_ok(cudaMemcpyAsync(pl->d_descs, pl->descs.data(), pl->descs.size() * sizeof(OzGrpDesc),
                                   cudaMemcpyHostToDevice, st),
                   routine, "grouped descriptor upload") &&
           cuda_ok(cudaMemcpyAsync(pl->d_classes, pl->classes.data(), pl->classes.size() * sizeof(OzGrpClass),
                                   cudaMemcpyHostToDevice, st),
                   routine, "grouped class upload");
}

void ozgroup_launch(OzGroupPlan *pl, cudaStream_t s)
{
    if (pl->descs.empty()) return;
    const int count = (int)pl->descs.size();
    const int sms = device_sm_count();
    const int L = pl->md.n;
    k_grp_exp<<<(unsigned)std::min<int64_t>(pl->lines, (int64_t)sms * 8), 256, 0, s>>>(
        pl->d_descs, count, pl->lines, pl->d_ex);
    if (pl->res_tc)
        k_grp_residues_tc<<<(unsigned)std::min<int64_t>(pl->tiles, (int64_t)sms * 4), RT_THREADS, RT_SMEM, s>>>(
            pl->d_descs, count, pl->tiles, pl->d_classes, pl->d_ex, kGroupBits, pl->rp, device_status_word());
    else
        k_grp_residues<<<(unsigned)std::min<int64_t>(pl->tiles, (int64_t)sms * 8), 256, 0, s>>>(
            pl->d_descs, count, pl->tiles, pl->d_classes, pl->d_ex, kGroupBits, pl->rp);
    for (size_t ci = 0; ci < pl->classes.size(); ++ci) {
        const OzGrpClass &c = pl->classes[ci];
        const int nz = (int)(pl->class_count[ci] * L);
        const int tiles_m2 = (int)(c.Mp / 256), tiles_n = (int)(c.Np / TC_BN);
        const int64_t units = (int64_t)nz * tiles_m2 * tiles_n;
        const int64_t pairs = sms / 2;
        const unsigned grid = 2u * (unsigned)(units < pairs ? units : pairs);
        k_oz_gemm_tc_2sm<<<grid, TCP_THREADS, T2_SMEM, s>>>(pl->maps[2 * ci], pl->maps[2 * ci + 1], c.Mp, c.Np, c.Kp,
                                                             c.Mp, c.Np, pl->mp, c.R, device_status_word(), 0,
                                                             tiles_m2, tiles_n, nz, 0, 0, take_lost_load_injection(), L);
    }
    k_grp_reconstruct<<<(unsigned)std::min<int64_t>(pl->items, (int64_t)sms * 8), 256, 0, s>>>(
        pl->d_descs, count, pl->items, pl->d_classes, pl->d_ex, 2 * kGroupBits, pl->cp);
    count_launch(3 + (int64_t)pl->classes.size());
}

namespace {

}  // namespace

bool gemm_ozaki_real(const GemmArgs &g, int bits, const char *routine) { return gemm_ozaki(g, false, bits, routine); }
bool gemm_ozaki_cplx(const GemmArgs &g, int bits, const char *routine) { return gemm_ozaki(g, true, bits, routine); }

}  // namespace mw

extern "C" int mwblas_set_kernel_timing(int on)
{
    int prev = mw::g_timing ? 1 : 0;
    mw::g_timing = on != 0;
    return prev;
}

extern "C" float mwblas_last_phase_ms(int phase)
{
    return (phase >= 0 && phase < mw::PH_N) ? mw::t_phase_ms[phase] : -1.0f;
}

extern "C" uint64_t mwblas_set_wait_limit_ns(uint64_t ns)
{
    static std::atomic<uint64_t> current{sm100::kWaitLimitNs};
    const uint64_t v = ns == 0 ? sm100::kWaitLimitNs : (ns < 1000000ull ? 1000000ull : ns);
    mw::clear_error();
    const cudaError_t st = cudaMemcpyToSymbol(sm100::g_wait_limit_ns, &v, sizeof(v));
    if (st == cudaSuccess) mw::set_plain_wait_limit(v);
    if (st != cudaSuccess) {
        mw::cuda_ok(st, "mwblas_set_wait_limit_ns", "cudaMemcpyToSymbol");
        return current.load();
    }
    return current.exchange(v);
}

extern "C" int mwblas_set_residue_tc(int on) { return mw::g_res_tc.exchange(on ? 1 : 0); }

extern "C" void mwblas_debug_lose_operand_loads(int count) { mw::g_lose_loads.store(count > 0 ? count : 0); }

extern "C" int mwblas_set_ozaki_mma(int kind)
{
    int prev = mw::mma_kind();
    mw::g_mma_kind = (kind >= 0 && kind <= 3) ? kind : 3;
    return prev;
}
