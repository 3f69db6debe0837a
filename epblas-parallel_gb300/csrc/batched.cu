// Batched uneven-size double-double GEMM and TRSM (no reference counterpart:
// the reference's CPU baseline for this workload is an OpenMP loop over
// instances calling mgemm_/mtrsm_, whose nested calls run serially,
// mgemm_parallel.cpp:53-60).
//
// mgemm_grouped: one persistent kernel over all instances. The work list is
// every (instance, 32x32 output tile, K split); CTAs of 256 threads pull items
// from an atomic counter, so thousands of uneven instances keep all SMs busy.
// Each item runs the fixed-point arithmetic of the integer-pipe engine
// (gemm_fixed.cu, fixgemm.cuh): its A rows / B columns are scaled from an
// exponent scan over the item's own K range (no pre-pass, no extra scratch),
// converted to balanced 24-bit digits while staged, and multiplied with
// exact 64-bit column sums. Items of a split instance write partial tiles as
// extended floats; the CTA that completes a tile's last split sums the
// partials in split order (deterministic) and applies alpha/beta with one
// rounding. The per-call state (descriptors, work counter, split counters,
// partial tiles) is uploaded and the kernel launched from a CUDA graph that is
// captured once per batch layout and replayed.
//
// The split-K policy (how many K elements a split must keep, and below how
// many tiles an instance is split) is chosen by mgemm_grouped_tune, which
// times the candidates on the caller's batch (writing to scratch copies of C)
// and caches the winner for batches of the same shape class.
//
// mtrsm_grouped: one persistent kernel; a work item is (instance, 32 right-hand
// sides), pulled by a warp from an atomic counter (longest triangles first);
// the warp solves them by substitution, one lane per right-hand side, each
// row's sum exact in fixed point, using the double-double reciprocal of the
// diagonal as the reference does (mtrsm_serial.cpp:144). Descriptors and
// scratch are kept per batch layout and the launch is replayed from a CUDA
// graph, as for the grouped GEMM.
#include <algorithm>
#include <atomic>
#include <cstring>
#include <map>
#include <mutex>
#include <vector>

#include "dd.cuh"
#include "fixgemm.cuh"
#include "level3.h"
#include "runtime.h"

namespace mw {

namespace {

constexpr int kNoExp = -30000;
constexpr int GTHREADS = 256;  // 16 x 16 threads
constexpr int GBK = 8;         // k-slab

struct GemmDesc {
    const double2 *A, *B;
    double2 *C;
    int64_t lda, ldb, ldc;
    int m, n, k;
    int ta, tb;
    double2 alpha, beta;
    int beta_kind;
    int tiles_m, tiles_n, splitk, klen;
    int64_t work_begin;   // first work item of this instance
    int64_t tile_begin;   // first tile counter (split instances only)
    int64_t part_begin;   // first partial-tile slot: earlier split instances
                          // hold tiles * splitk slots each
};

__device__ __forceinline__ int exp_bound(double x)
{
    uint64_t b = (uint64_t)__double_as_longlong(x) & 0x7fffffffffffffffull;
    if (b == 0) return kNoExp;
    return (int)(b >> 52) - 1023;
}

__device__ __forceinline__ double2 opA_at(const GemmDesc &d, int64_t i, int64_t p)
{
    return d.ta ? d.A[p + i * d.lda] : d.A[i + p * d.lda];
}
__device__ __forceinline__ double2 opB_at(const GemmDesc &d, int64_t p, int64_t j)
{
    return d.tb ? d.B[j + p * d.ldb] : d.B[p + j * d.ldb];
}

// R consecutive digits of a staged row (R = 1, 2 or 4 ints, one vector load).
template <int R>
__device__ __forceinline__ void load_digits(const int *src, int (&dst)[R])
{
    if constexpr (R == 4) {
        const int4 v = *reinterpret_cast<const int4 *>(src);
        dst[0] = v.x; dst[1] = v.y; dst[2] = v.z; dst[3] = v.w;
    } else if constexpr (R == 2) {
        const int2 v = *reinterpret_cast<const int2 *>(src);
        dst[0] = v.x; dst[1] = v.y;
    } else {
        dst[0] = *src;
    }
}

// GT x GT output tiles (GT = 16, 32 or 64; chosen per batch by the tuner),
// 256 threads as 16 x 16, each with R x R outputs (R = GT / 16): rows R tx ..,
// columns R ty ...
template <int GT>
__global__ void __launch_bounds__(GTHREADS) k_gemm_grouped(const GemmDesc *__restrict__ descs, int count,
                                                          int64_t total, unsigned long long *work_counter,
                                                          int *tile_counters, fx::XFPod *partials)
{
    constexpr int R = GT / 16;
    __shared__ __align__(16) int sA[GBK][5][GT], sB[GBK][5][GT];
    __shared__ int s_ea[GT], s_eb[GT];
    __shared__ long long s_item;
    __shared__ int s_last;
    const int tid = threadIdx.x;
    const int tx = tid & 15, ty = tid >> 4;
    for (;;) {
        if (tid == 0) s_item = (long long)atomicAdd(work_counter, 1ull);
        __syncthreads();
        const long long w = s_item;
        __syncthreads();
        if (w >= total) return;
        // locate the instance (descs sorted by work_begin)
        int lo = 0, hi = count - 1;
        while (lo < hi) {
            int mid = (lo + hi + 1) >> 1;
            if (descs[mid].work_begin <= w) lo = mid;
            else hi = mid - 1;
        }
        const GemmDesc d = descs[lo];
        const int64_t local = w - d.work_begin;
        const int split = (int)(local % d.splitk);
        const int64_t tile = local / d.splitk;
        const int tm = (int)(tile % d.tiles_m), tn = (int)(tile / d.tiles_m);
        const int64_t i0 = (int64_t)tm * GT, j0 = (int64_t)tn * GT;
        const int64_t k0 = (int64_t)split * d.klen, k1 = min((int64_t)d.k, k0 + d.klen);

        // exponent bounds of the tile's rows / columns over [k0, k1)
        if (tid < GT) {
            int e = kNoExp;
            const int64_t i = i0 + tid;
            if (i < d.m)
                for (int64_t p = k0; p < k1; ++p) e = max(e, exp_bound(opA_at(d, i, p).x));
            s_ea[tid] = e;
        } else if (tid < 2 * GT) {
            int e = kNoExp;
            const int64_t j = j0 + (tid - GT);
            if (j < d.n)
                for (int64_t p = k0; p < k1; ++p) e = max(e, exp_bound(opB_at(d, p, j).x));
            s_eb[tid - GT] = e;
        }
        __syncthreads();

        long long acc[R][R][5];
#pragma unroll
        for (int a = 0; a < R; ++a)
#pragma unroll
            for (int b = 0; b < R; ++b)
#pragma unroll
                for (int q = 0; q < 5; ++q) acc[a][b][q] = 0;

        for (int64_t kk = k0; kk < k1; kk += GBK) {
            // stage the A and B tiles (GT x GBK elements each) as digits
            for (int idx = tid; idx < GT * GBK; idx += GTHREADS) {
                int dg[5];
                {
                    int r, p;
                    if (!d.ta) { r = idx % GT; p = idx / GT; }
                    else       { p = idx % GBK; r = idx / GBK; }
                    const int64_t gi = i0 + r, gp = kk + p;
                    const double2 v = (gp < k1 && gi < d.m) ? opA_at(d, gi, gp) : make_double2(0.0, 0.0);
                    const int e = s_ea[r];
                    fxg::dd_digits(v, (e <= kNoExp / 2 || e >= 1024) ? -100000 : fxg::FX_S - e, dg);
#pragma unroll
                    for (int t = 0; t < 5; ++t) sA[p][t][r] = dg[t];
                }
                {
                    int c, p;
                    if (!d.tb) { p = idx % GBK; c = idx / GBK; }
                    else       { c = idx % GT; p = idx / GT; }
                    const int64_t gj = j0 + c, gp = kk + p;
                    const double2 v = (gp < k1 && gj < d.n) ? opB_at(d, gp, gj) : make_double2(0.0, 0.0);
                    const int e = s_eb[c];
                    fxg::dd_digits(v, (e <= kNoExp / 2 || e >= 1024) ? -100000 : fxg::FX_S - e, dg);
#pragma unroll
                    for (int t = 0; t < 5; ++t) sB[p][t][c] = dg[t];
                }
            }
            __syncthreads();
#pragma unroll 2
            for (int p = 0; p < GBK; ++p) {
                int da[R][5], db[R][5];
#pragma unroll
                for (int t = 0; t < 5; ++t) {
                    int va[R], vb[R];
                    load_digits<R>(&sA[p][t][R * tx], va);
                    load_digits<R>(&sB[p][t][R * ty], vb);
#pragma unroll
                    for (int u = 0; u < R; ++u) {
                        da[u][t] = va[u];
                        db[u][t] = vb[u];
                    }
                }
#pragma unroll
                for (int a = 0; a < R; ++a)
#pragma unroll
                    for (int b = 0; b < R; ++b) fxg::mac_digits(acc[a][b], da[a], db[b]);
            }
            __syncthreads();
        }

        // the R x R outputs as extended floats (non-finite rows/columns flagged)
        xfp::XF v[R][R];
        bool badv[R][R];
#pragma unroll
        for (int a = 0; a < R; ++a)
#pragma unroll
            for (int b = 0; b < R; ++b) {
                const int ei = s_ea[R * tx + a], ej = s_eb[R * ty + b];
                badv[a][b] = ei >= 1024 || ej >= 1024;
                if (badv[a][b] || ei <= kNoExp / 2 || ej <= kNoExp / 2) {
                    v[a][b].zero = true; v[a][b].neg = false; v[a][b].m = 0; v[a][b].e = 0;
                } else {
                    v[a][b] = fxg::sums_to_xf(acc[a][b], ei, ej);
                }
            }

        if (d.splitk > 1) {
            // write this split's partial tile, then let the last split finish
            fx::XFPod *pt = partials + (d.part_begin + tile * d.splitk + split) * (GT * GT);
#pragma unroll
            for (int a = 0; a < R; ++a)
#pragma unroll
                for (int b = 0; b < R; ++b) pt[(R * ty + b) * GT + R * tx + a] = fx::to_pod(v[a][b], badv[a][b]);
            __threadfence();
            __syncthreads();
            if (tid == 0) {
                int old = atomicAdd(&tile_counters[d.tile_begin + tile], 1);
                s_last = (old == d.splitk - 1);
            }
            __syncthreads();
            if (!s_last) continue;
            __threadfence();
            const fx::XFPod *base = partials + (d.part_begin + tile * d.splitk) * (GT * GT);
#pragma unroll
            for (int a = 0; a < R; ++a)
#pragma unroll
                for (int b = 0; b < R; ++b) {
                    xfp::XF sum;
                    sum.zero = true; sum.neg = false; sum.m = 0; sum.e = 0;
                    bool bad = false;
                    for (int s2 = 0; s2 < d.splitk; ++s2) {
                        // partials written by other CTAs: read through L2
                        const fx::XFPod *q = base + (int64_t)s2 * GT * GT + (R * ty + b) * GT + R * tx + a;
                        fx::XFPod pv;
                        pv.hi = __ldcg(&q->hi);
                        pv.lo = __ldcg(&q->lo);
                        pv.e = __ldcg(&q->e);
                        pv.flags = __ldcg(&q->flags);
                        bad |= (pv.flags & 4) != 0;
                        sum = xfp::xf_add(sum, fx::from_pod(pv));
                    }
                    v[a][b] = sum;
                    badv[a][b] = bad;
                }
            if (tid == 0) tile_counters[d.tile_begin + tile] = 0;   // ready for the next replay
        }
        const dd::real beta = dd::make(d.beta.x, d.beta.y);
        const xfp::XF xa = xfp::xf_from_dd(d.alpha.x, d.alpha.y), xb = xfp::xf_from_dd(d.beta.x, d.beta.y);
        const bool alpha_one = d.alpha.x == 1.0 && d.alpha.y == 0.0;
#pragma unroll
        for (int b = 0; b < R; ++b) {
            const int64_t j = j0 + R * ty + b;
            if (j >= d.n) continue;
#pragma unroll
            for (int a = 0; a < R; ++a) {
                const int64_t i = i0 + R * tx + a;
                if (i >= d.m) continue;
                double2 *pc = d.C + i + j * d.ldc;
                if (badv[a][b]) {
                    const double qnan = __longlong_as_double(0x7ff8000000000000ll);
                    *pc = make_double2(qnan, qnan);
                    continue;
                }
                fxg::store_axpby(pc, v[a][b], xa, alpha_one, xb, beta, d.beta_kind);
            }
        }
    }
}

// ---- grouped TRSM ----------------------------------------------------------------

struct TrsmDesc {
    const double2 *A;
    double2 *B;
    int64_t lda, ldb;
    int m, n;
    double2 alpha;
    int nchunks;          // groups of 32 right-hand sides
    int64_t work_begin;
    int64_t xop_begin;    // this instance's decoded solutions in the scratch array (na * 32 per chunk)
};

constexpr int kTrsmTile = 256;   // entries of a row of op(A) split into digits at a time

__device__ __forceinline__ dd::real dd_recip(dd::real b)
{
    // Hida-Li-Bailey accurate division 1 / b
    double q1 = __ddiv_rn(1.0, b.hi);
    dd::real r = dd::sub_exact(dd::make(1.0, 0.0), dd::mul_exact(dd::make(q1, 0.0), b));
    double q2 = __ddiv_rn(r.hi, b.hi);
    r = dd::sub_exact(r, dd::mul_exact(dd::make(q2, 0.0), b));
    double q3 = __ddiv_rn(r.hi, b.hi);
    dd::real q;
    dd::fast_two_sum(q1, q2, q.hi, q.lo);
    return dd::add_exact(q, dd::make(q3, 0.0));
}

// One work item of the grouped TRSM: instance descs[*] (found by binary
// search on work_begin), right-hand sides [32 chunk, 32 chunk + 32).
__device__ __forceinline__ void trsm_item(const TrsmDesc *__restrict__ descs, int count, int64_t w, int side,
                                          int lower, int trans, int unit, fx::Op *xops, fx::Dig *arow, int lane)
{
    int lo = 0, hi = count - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (descs[mid].work_begin <= w) lo = mid;
        else hi = mid - 1;
    }
    const TrsmDesc d = descs[lo];
    const int chunk = (int)(w - d.work_begin);
    const dd::real alpha = dd::make(d.alpha.x, d.alpha.y);
    const bool alpha1 = (d.alpha.x == 1.0 && d.alpha.y == 0.0);
    const int na = side == 0 ? d.m : d.n;                 // order of the triangle
    const int64_t nr = side == 0 ? d.n : d.m;             // right-hand sides
    const int64_t rhs = (int64_t)chunk * 32 + lane;
    const bool active = rhs < nr;
    fx::Op *xw = xops + d.xop_begin + (int64_t)chunk * na * 32;   // [row][lane]
    const int64_t my = active ? rhs : nr - 1;             // clamped: loads stay in bounds
    // element t of this lane's right-hand side (a column of B for side L, a row for R)
    auto bptr = [&](int t) -> double2 * {
        return side == 0 ? d.B + my * d.ldb + t : d.B + my + (int64_t)t * d.ldb;
    };
#define OPA(i, j) (trans ? d.A[(j) + (int64_t)(i) * d.lda] : d.A[(i) + (int64_t)(j) * d.lda])
    // side L: op(A) X = alpha B, forward if op(A) is lower;
    // side R: X op(A) = alpha B, forward if op(A) is upper.
    const bool forward = side == 0 ? lower : !lower;
    fx::Dig one;
    {
        const fx::Op o = fx::decode(make_double2(1.0, 0.0));
        one = fx::to_dig(o);
    }
    dd::real inv = dd::make(1.0, 0.0);
    for (int s = 0; s < na; ++s) {
        const int r = forward ? s : na - 1 - s;
        if (!unit && (s & 31) == 0) {
            // reciprocals of the next 32 diagonal entries, one per lane
            const int sl = s + lane;
            if (sl < na) {
                const int rl = forward ? sl : na - 1 - sl;
                inv = dd_recip(dd::load(&OPA(rl, rl)));
            }
        }
        fx::Acc acc;
        acc.reset();
        dd::real b0 = dd::load(bptr(r));
        if (!alpha1) b0 = dd::mul_fast(b0, alpha);
        acc.add_dig(fx::decode(make_double2(b0.hi, b0.lo)), one);
        const int p0 = forward ? 0 : r + 1, p1 = forward ? r : na;
        for (int t0 = p0; t0 < p1; t0 += kTrsmTile) {
            const int tl = min(kTrsmTile, p1 - t0);
            // side L: sum_p op(A)(r, p) x_p; side R: sum_p x_p op(A)(p, r)
            for (int q = lane; q < tl; q += 32) {
                const int p = t0 + q;
                arow[q] = fx::to_dig(fx::decode(side == 0 ? OPA(r, p) : OPA(p, r)));
            }
            __syncwarp();
            const fx::Op *xp = xw + (int64_t)t0 * 32 + lane;
            int q = 0;
            // four solutions loaded ahead of their products, so the loads overlap
            for (; q + 4 <= tl; q += 4, xp += 128) {
                fx::Op xo[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) xo[u] = xp[32 * u];
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    xo[u].flags ^= fx::kNeg;
                    acc.add_dig(xo[u], arow[q + u]);
                }
            }
            for (; q < tl; ++q, xp += 32) {
                fx::Op xo = *xp;
                xo.flags ^= fx::kNeg;
                acc.add_dig(xo, arow[q]);
            }
            __syncwarp();
        }
        double h, l;
        xfp::xf_to_dd(acc.finish(), h, l);
        dd::real v = dd::make(h, l);
        if (acc.bad) v = dd::make(__longlong_as_double(0x7ff8000000000000ll), 0.0);
        if (!unit) {
            const double ih = __shfl_sync(0xffffffffu, inv.hi, s & 31);
            const double il = __shfl_sync(0xffffffffu, inv.lo, s & 31);
            v = dd::mul_fast(v, dd::make(ih, il));
        }
        if (active) dd::store(bptr(r), v);
        xw[(int64_t)r * 32 + lane] = fx::decode(make_double2(v.hi, v.lo));
        __syncwarp();
    }
#undef OPA
}

// side: 0 left, 1 right; lower: op(A) lower triangular; trans: op = A^T.
// Warp per (instance, 32 right-hand sides), lane per right-hand side. The
// reciprocals of the diagonal are computed 32 rows at a time, one row per
// lane, and broadcast with shuffles; each row's sum alpha*b - sum_p A x is
// accumulated exactly in fixed point (fixacc.cuh) and rounded once before the
// multiplication by the reciprocal. All lanes stay in the loop (lanes past
// the last right-hand side do the work on a clamped column and store
// nothing) so that the shuffles see the whole warp.
// Persistent: every warp pulls work items (instance, 32 right-hand sides) from
// an atomic counter until none is left; descriptors are sorted longest
// triangle first, so the long solves start first and the short ones fill the
// tail.
__global__ void __launch_bounds__(128, 4) k_trsm_grouped(const TrsmDesc *__restrict__ descs, int count, int64_t total,
                                                     int side, int lower, int trans, int unit, fx::Op *xops,
                                                     unsigned long long *work_counter)
{
    // per warp: a tile of the current row of op(A), split into digits once
    // for all 32 right-hand sides
    __shared__ fx::Dig s_arow[4][kTrsmTile];
    fx::Dig *arow = s_arow[(threadIdx.x >> 5) & 3];
    const int lane = threadIdx.x & 31;
    for (;;) {
        unsigned long long wl = 0;
        if (lane == 0) wl = atomicAdd(work_counter, 1ull);
        const int64_t w = (int64_t)__shfl_sync(0xffffffffu, wl, 0);
        if (w >= total) return;   // whole warp leaves together
        trsm_item(descs, count, w, side, lower, trans, unit, xops, arow, lane);
    }
}

// ---- host: plans, graphs, autotuner ----------------------------------------------

struct Policy {
    int min_k_per_split = 0;   // 0: never split
    int max_tiles_split = 4;   // split only instances with at most this many tiles
    int tile = 32;             // output tile edge: 16, 32 or 64
    int oz_min = 0;            // instances with m, n >= oz_min and k >= 64 run on the tensor cores (0: none)
    int pack_k = 0;            // the other instances with k >= pack_k share tensor-core slots, in pieces of <= 256 x 256 (0: none)
};

struct Plan {
    std::vector<GemmDesc> descs;
    std::vector<OzGroupItem> oz_items;   // instances routed to the tensor-core engine
    OzGroupPlan *oz = nullptr;
    int tile = 32;
    int64_t total = 0, split_tiles = 0, partial_elems = 0;
    // device state
    void *dev = nullptr;
    size_t dev_bytes = 0;
    cudaGraphExec_t exec = nullptr;
    uint64_t key = 0;
};

std::mutex g_batched_mu;
std::map<uint64_t, Policy> g_policy_cache;   // shape class -> tuned policy
Policy g_default_policy{512, 4, 32, 128, 0};
thread_local int t_tuned_tile = 0;   // tile chosen by this thread's most recent tuning
thread_local int t_tuned_oz = -1;    // tensor-core threshold chosen by it (0: none)
std::atomic<int> g_forced_tile{0};   // mwblas_set_grouped_tile: 0 = tuned or default
std::atomic<int> g_forced_oz{-1};    // mwblas_set_grouped_tensor_min: -1 = tuned or default
std::atomic<int> g_forced_pack{-1};  // mwblas_set_grouped_tensor_pack: -1 = tuned or default
thread_local int t_tuned_pack = -1;  // shared-slot depth chosen by this thread's most recent tuning
thread_local Plan t_plan;

uint64_t mix(uint64_t h, uint64_t v)
{
    h ^= v + 0x9e3779b97f4a7c15ull + (h << 6) + (h >> 2);
    return h;
}

// Shape class: count and log-size histogram (the policy depends on shapes, not data).
uint64_t shape_class(int64_t count, const int64_t *m, const int64_t *n, const int64_t *k)
{
    int hist[3][12] = {};
    for (int64_t i = 0; i < count; ++i) {
        int64_t v[3] = {m[i], n[i], k[i]};
        for (int t = 0; t < 3; ++t) {
            int b = 0;
            while (b < 11 && ((int64_t)1 << (b + 1)) <= v[t]) ++b;
            hist[t][b]++;
        }
    }
    uint64_t h = (uint64_t)count;
    for (int t = 0; t < 3; ++t)
        for (int b = 0; b < 12; ++b) h = mix(h, (uint64_t)(hist[t][b] * 16 / (count > 0 ? count : 1)));
    return h;
}

void build_descs(Plan &pl, int64_t count, const char *ta, const char *tb, const int64_t *m, const int64_t *n,
                 const int64_t *k, const mwblas_real64x2 *alpha, const mwblas_real64x2 *const *a, const int64_t *lda,
                 const mwblas_real64x2 *const *b, const int64_t *ldb, const mwblas_real64x2 *beta,
                 mwblas_real64x2 *const *c, const int64_t *ldc, const Policy &pol)
{
    pl.descs.clear();
    pl.descs.reserve((size_t)count);
    pl.oz_items.clear();
    const int oz_min = (pol.oz_min > 0 && ozaki_available()) ? pol.oz_min : 0;
    const int pack_k = (pol.pack_k > 0 && ozaki_available()) ? pol.pack_k : 0;
    const int GT = pol.tile;
    pl.tile = GT;
    int64_t work = 0, stiles = 0, pslots = 0;
    for (int64_t i = 0; i < count; ++i) {
        if (m[i] <= 0 || n[i] <= 0) continue;
        GemmDesc d{};
        d.A = (const double2 *)a[i];
        d.B = (const double2 *)b[i];
        d.C = (double2 *)c[i];
        d.lda = lda[i];
        d.ldb = ldb[i];
        d.ldc = ldc[i];
        d.m = (int)m[i];
        d.n = (int)n[i];
        d.k = (int)k[i];
        char TA = (char)toupper(ta[i]), TB = (char)toupper(tb[i]);
        d.ta = (TA != 'N');
        d.tb = (TB != 'N');
        d.alpha = make_double2(alpha[i].limbs[0], alpha[i].limbs[1]);
        d.beta = make_double2(beta[i].limbs[0], beta[i].limbs[1]);
        const bool alpha0 = (d.alpha.x == 0.0 && d.alpha.y == 0.0);
        d.beta_kind = (d.beta.x == 0.0 && d.beta.y == 0.0) ? 0 : ((d.beta.x == 1.0 && d.beta.y == 0.0) ? 1 : 2);
        const bool own_slot = oz_min > 0 && d.m >= oz_min && d.n >= oz_min && d.k >= 64;
        // the other instances of depth >= pack_k share slots; those with m or
        // n above 256 (the skinny ones) as pieces of at most 256 x 256
        const bool shared_slot = pack_k > 0 && d.k >= pack_k;
        if (!alpha0 && (own_slot || shared_slot) && d.k <= 16384 && d.m <= 8192 && d.n <= 8192) {
            OzGroupItem it;
            memset(&it, 0, sizeof(it));   // the plan key hashes the bytes, padding included
            it.lda = d.lda; it.ldb = d.ldb; it.ldc = d.ldc;
            it.k = d.k;
            it.ta = d.ta != 0; it.tb = d.tb != 0;
            it.alpha = dd_host{d.alpha.x, d.alpha.y};
            it.beta = dd_host{d.beta.x, d.beta.y};
            it.beta_kind = d.beta_kind;
            it.pack = own_slot ? 0 : 1;
            const int pm = own_slot ? d.m : 256, pn = own_slot ? d.n : 256;
            for (int r0 = 0; r0 < d.m; r0 += pm) {
                for (int c0 = 0; c0 < d.n; c0 += pn) {
                    // rows r0.. of op(A), columns c0.. of op(B) and C
                    it.A = d.A + (d.ta ? (int64_t)r0 * d.lda : r0);
                    it.B = d.B + (d.tb ? c0 : (int64_t)c0 * d.ldb);
                    it.C = d.C + r0 + (int64_t)c0 * d.ldc;
                    it.m = std::min(pm, d.m - r0);
                    it.n = std::min(pn, d.n - c0);
                    pl.oz_items.push_back(it);
                }
            }
            continue;
        }
        if (alpha0 || d.k == 0) {
            // only the beta pass: run as a k = 0 product (sigma irrelevant)
            d.k = 0;
        }
        d.tiles_m = (d.m + GT - 1) / GT;
        d.tiles_n = (d.n + GT - 1) / GT;
        const int tiles = d.tiles_m * d.tiles_n;
        d.splitk = 1;
        if (pol.min_k_per_split > 0 && tiles <= pol.max_tiles_split && d.k >= 2 * pol.min_k_per_split)
            d.splitk = std::min(16, d.k / pol.min_k_per_split);
        // the digit column sums hold at most 16384 multiply-adds per split
        const int need_splits = (d.k + 16383) / 16384;
        if (d.splitk < need_splits) d.splitk = need_splits;
        d.klen = d.splitk > 1 ? ((d.k + d.splitk - 1) / d.splitk + GBK - 1) / GBK * GBK : std::max(d.k, 1);
        if (d.k == 0) d.klen = 1;
        d.work_begin = work;
        d.tile_begin = d.splitk > 1 ? stiles : 0;
        d.part_begin = d.splitk > 1 ? pslots : 0;
        if (d.splitk > 1) {
            stiles += tiles;
            pslots += (int64_t)tiles * d.splitk;
        }
        work += (int64_t)tiles * d.splitk;
        pl.descs.push_back(d);
    }
    pl.total = work;
    pl.split_tiles = stiles;
    pl.partial_elems = pslots * GT * GT;   // extended-float partials
}

uint64_t plan_key(const Plan &pl)
{
    // FNV-1a over 64-bit words (GemmDesc is a multiple of 8 bytes)
    static_assert(sizeof(GemmDesc) % 8 == 0, "descriptor size");
    uint64_t h = 1469598103934665603ull;
    const uint64_t *p = (const uint64_t *)pl.descs.data();
    const size_t nw = pl.descs.size() * sizeof(GemmDesc) / 8;
    for (size_t i = 0; i < nw; ++i) h = (h ^ p[i]) * 1099511628211ull;
    static_assert(sizeof(OzGroupItem) % 8 == 0, "item size");
    const uint64_t *q = (const uint64_t *)pl.oz_items.data();
    const size_t nq = pl.oz_items.size() * sizeof(OzGroupItem) / 8;
    for (size_t i = 0; i < nq; ++i) h = (h ^ q[i]) * 1099511628211ull;
    return mix(mix(h, (uint64_t)pl.tile), (uint64_t)pl.oz_items.size());
}

// (Re)creates the device buffers and the graph when the batch layout changed.
// use_graph = false (the library's own calls, whose layouts change from call
// to call): the kernels are enqueued directly instead of capturing a graph.
bool prepare_and_launch(Plan &pl, const char *routine, bool use_graph = true)
{
    if ((pl.descs.empty() || pl.total == 0) && pl.oz_items.empty()) return true;
    const size_t d_bytes = pl.descs.size() * sizeof(GemmDesc);
    const size_t cnt_bytes = 256 + (size_t)(pl.split_tiles + 1) * sizeof(int);
    const size_t part_bytes = (size_t)pl.partial_elems * sizeof(fx::XFPod);
    const size_t need = d_bytes + cnt_bytes + part_bytes + 512;
    const uint64_t key = plan_key(pl);
    cudaStream_t s = stream();
    if (pl.dev_bytes < need) {
        if (pl.exec) {
            cudaGraphExecDestroy(pl.exec);
            pl.exec = nullptr;
        }
        if (pl.dev) cudaFree(pl.dev);
        pl.dev = nullptr;
        pl.dev_bytes = 0;
        if (!cuda_ok(cudaMalloc(&pl.dev, need), routine, "grouped plan buffer")) return false;
        pl.dev_bytes = need;
        if (!cuda_ok(cudaMemset(pl.dev, 0, need), routine, "grouped plan clear")) return false;
    }
    // layout: [descriptors][work counter (256 B) | tile counters][partials],
    // each region starting on a 256-byte boundary
    char *base = (char *)pl.dev;
    const size_t cnt_off = (d_bytes + 255) / 256 * 256;
    const size_t part_off = (cnt_off + cnt_bytes + 255) / 256 * 256;
    GemmDesc *ddesc = (GemmDesc *)base;
    unsigned long long *counter = (unsigned long long *)(base + cnt_off);
    int *tile_counters = (int *)(counter + 32);
    fx::XFPod *partials = (fx::XFPod *)(base + part_off);
    const int sms = device_sm_count();
    const int grid = (int)std::min<int64_t>(pl.total, (int64_t)sms * 16);
    if (pl.key != key) {
        // descriptors change only with the batch layout; upload outside the graph
        if (!pl.descs.empty() &&
            !cuda_ok(cudaMemcpyAsync(ddesc, pl.descs.data(), d_bytes, cudaMemcpyHostToDevice, s), routine,
                     "descriptor upload"))
            return false;
        if (!pl.oz_items.empty() || pl.oz) {
            if (!pl.oz) pl.oz = ozgroup_create();
            if (!ozgroup_prepare(pl.oz, pl.oz_items, routine)) return false;
        }
    }
    if (!use_graph) {
        pl.key = key;
        if (pl.total > 0) {
            cudaMemsetAsync(counter, 0, cnt_bytes, s);
            auto kern = pl.tile == 64 ? k_gemm_grouped<64> : (pl.tile == 16 ? k_gemm_grouped<16> : k_gemm_grouped<32>);
            kern<<<grid, GTHREADS, 0, s>>>(ddesc, (int)pl.descs.size(), pl.total, counter, tile_counters, partials);
            count_launch();
        }
        if (pl.oz && ozgroup_count(pl.oz) > 0) ozgroup_launch(pl.oz, s);
        return cuda_ok(cudaGetLastError(), routine, "grouped launch");
    }
    if (!pl.exec || pl.key != key) {
        if (pl.exec) {
            cudaGraphExecDestroy(pl.exec);
            pl.exec = nullptr;
        }
        cudaStream_t cap;
        if (!cuda_ok(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking), routine, "capture stream")) return false;
        cudaGraph_t graph;
        bool ok = cuda_ok(cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal), routine, "begin capture");
        if (ok) {
            // counters start at zero on every replay
            if (pl.total > 0) {
                cudaMemsetAsync(counter, 0, cnt_bytes, cap);
                auto kern = pl.tile == 64 ? k_gemm_grouped<64> : (pl.tile == 16 ? k_gemm_grouped<16> : k_gemm_grouped<32>);
                kern<<<grid, GTHREADS, 0, cap>>>(ddesc, (int)pl.descs.size(), pl.total, counter, tile_counters,
                                                 partials);
            }
            // the large instances on the tensor cores, in the same graph
            if (pl.oz && ozgroup_count(pl.oz) > 0) ozgroup_launch(pl.oz, cap);
            ok = cuda_ok(cudaStreamEndCapture(cap, &graph), routine, "end capture");
        }
        if (ok) {
            ok = cuda_ok(cudaGraphInstantiate(&pl.exec, graph, 0), routine, "graph instantiate");
            cudaGraphDestroy(graph);
        }
        cudaStreamDestroy(cap);
        if (!ok) return false;
        pl.key = key;
    }
    count_launch();
    return cuda_ok(cudaGraphLaunch(pl.exec, s), routine, "graph launch");
}

// The grouped TRSM's per-thread plan: descriptors, work counter and decoded
// solutions in one device buffer, kept while the batch layout is unchanged,
// and a CUDA graph (counter reset + the persistent kernel) replayed per call.
struct TrsmPlan {
    std::vector<TrsmDesc> descs;
    int64_t total = 0, xop_elems = 0;
    int side = 0, lower = 0, trans = 0, unit = 0;
    void *dev = nullptr;
    size_t dev_bytes = 0;
    cudaGraphExec_t exec = nullptr;
    uint64_t key = 0;
};
thread_local TrsmPlan t_tplan;

bool trsm_prepare_and_launch(TrsmPlan &pl, const char *routine)
{
    if (pl.descs.empty() || pl.total == 0) return true;
    const size_t d_bytes = (pl.descs.size() * sizeof(TrsmDesc) + 255) / 256 * 256;
    const size_t need = d_bytes + 256 + (size_t)pl.xop_elems * sizeof(fx::Op);
    static_assert(sizeof(TrsmDesc) % 8 == 0, "descriptor size");
    uint64_t key = 1469598103934665603ull;
    const uint64_t *w = (const uint64_t *)pl.descs.data();
    for (size_t i = 0; i < pl.descs.size() * sizeof(TrsmDesc) / 8; ++i) key = (key ^ w[i]) * 1099511628211ull;
    key = mix(key, (uint64_t)(pl.side | pl.lower << 1 | pl.trans << 2 | pl.unit << 3));
    cudaStream_t s = stream();
    if (pl.dev_bytes < need) {
        if (pl.exec) {
            cudaGraphExecDestroy(pl.exec);
            pl.exec = nullptr;
        }
        if (pl.dev) cudaFree(pl.dev);
        pl.dev = nullptr;
        pl.dev_bytes = 0;
        pl.key = 0;
        if (!cuda_ok(cudaMalloc(&pl.dev, need), routine, "grouped TRSM plan buffer")) return false;
        pl.dev_bytes = need;
    }
    // layout: [descriptors][work counter (256 B)][decoded solutions]
    TrsmDesc *ddesc = (TrsmDesc *)pl.dev;
    unsigned long long *counter = (unsigned long long *)((char *)pl.dev + d_bytes);
    fx::Op *xops = (fx::Op *)((char *)pl.dev + d_bytes + 256);
    if (pl.key != key) {
        if (pl.exec) {
            cudaGraphExecDestroy(pl.exec);
            pl.exec = nullptr;
        }
        if (!cuda_ok(cudaMemcpyAsync(ddesc, pl.descs.data(), pl.descs.size() * sizeof(TrsmDesc),
                                     cudaMemcpyHostToDevice, s),
                     routine, "descriptor upload"))
            return false;
        // resident blocks: four 4-warp blocks per SM (the kernel's launch bounds)
        const int warps = 4;
        const int64_t grid = std::min<int64_t>((pl.total + warps - 1) / warps, (int64_t)device_sm_count() * 4);
        cudaStream_t cap;
        if (!cuda_ok(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking), routine, "capture stream")) return false;
        cudaGraph_t graph;
        bool ok = cuda_ok(cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal), routine, "begin capture");
        if (ok) {
            cudaMemsetAsync(counter, 0, sizeof(unsigned long long), cap);
            k_trsm_grouped<<<(unsigned)grid, warps * 32, 0, cap>>>(ddesc, (int)pl.descs.size(), pl.total, pl.side,
                                                                 pl.lower, pl.trans, pl.unit, xops, counter);
            ok = cuda_ok(cudaStreamEndCapture(cap, &graph), routine, "end capture");
        }
        if (ok) {
            ok = cuda_ok(cudaGraphInstantiate(&pl.exec, graph, 0), routine, "graph instantiate");
            cudaGraphDestroy(graph);
        }
        cudaStreamDestroy(cap);
        if (!ok) return false;
        pl.key = key;
    }
    count_launch();
    return cuda_ok(cudaGraphLaunch(pl.exec, s), routine, "graph launch");
}

bool grouped_validate(const char *routine, int64_t count, const char *ta, const char *tb, const int64_t *m,
                      const int64_t *n, const int64_t *k, const mwblas_real64x2 *alpha,
                      const mwblas_real64x2 *const *a, const int64_t *lda, const mwblas_real64x2 *const *b,
                      const int64_t *ldb, const mwblas_real64x2 *beta, mwblas_real64x2 *const *c, const int64_t *ldc)
{
    if (count < 0) { set_error(routine, 1, "count < 0"); return false; }
    if (count == 0) return true;
    if (!ta || !tb || !m || !n || !k || !alpha || !a || !lda || !b || !ldb || !beta || !c || !ldc) {
        set_error(routine, 2, "null argument array");
        return false;
    }
    for (int64_t i = 0; i < count; ++i) {
        char TA = (char)toupper(ta[i]), TB = (char)toupper(tb[i]);
        if (TA != 'N' && TA != 'T' && TA != 'C') { set_error(routine, 2, "invalid transa in instance " + std::to_string(i)); return false; }
        if (TB != 'N' && TB != 'T' && TB != 'C') { set_error(routine, 3, "invalid transb in instance " + std::to_string(i)); return false; }
        if (m[i] < 0 || n[i] < 0 || k[i] < 0) { set_error(routine, 4, "negative size in instance " + std::to_string(i)); return false; }
        if (m[i] > (1 << 30) || n[i] > (1 << 30) || k[i] > (1 << 30)) { set_error(routine, 4, "size too large"); return false; }
        int64_t nra = (TA == 'N') ? m[i] : k[i], nrb = (TB == 'N') ? k[i] : n[i];
        if (lda[i] < std::max<int64_t>(1, nra)) { set_error(routine, 9, "lda too small in instance " + std::to_string(i)); return false; }
        if (ldb[i] < std::max<int64_t>(1, nrb)) { set_error(routine, 11, "ldb too small in instance " + std::to_string(i)); return false; }
        if (ldc[i] < std::max<int64_t>(1, m[i])) { set_error(routine, 14, "ldc too small in instance " + std::to_string(i)); return false; }
        if (m[i] > 0 && n[i] > 0 && !is_dd_device_pointer(c[i])) {
            set_error(routine, 13, "grouped calls take 16-byte aligned device (or managed) arrays; C of instance " +
                                       std::to_string(i));
            return false;
        }
        if (m[i] > 0 && n[i] > 0 && k[i] > 0 && !(is_dd_device_pointer(a[i]) && is_dd_device_pointer(b[i]))) {
            set_error(routine, 8, "grouped calls take 16-byte aligned device (or managed) arrays; A or B of instance " +
                                      std::to_string(i));
            return false;
        }
    }
    return true;
}

}  // namespace

// Grouped GEMM for the library's own use (device arrays, arguments already
// valid): its own plan, default split policy, stream-ordered (no sync).
bool grouped_gemm_device(int64_t count, const char *ta, const char *tb, const int64_t *m, const int64_t *n,
                         const int64_t *k, const mwblas_real64x2 *alpha, const mwblas_real64x2 *const *a,
                         const int64_t *lda, const mwblas_real64x2 *const *b, const int64_t *ldb,
                         const mwblas_real64x2 *beta, mwblas_real64x2 *const *c, const int64_t *ldc,
                         int tensor_min, const char *routine)
{
    if (count == 0) return true;
    static thread_local Plan internal;
    Policy pol = g_default_policy;
    pol.oz_min = tensor_min;
    build_descs(internal, count, ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc, pol);
    return prepare_and_launch(internal, routine, false);
}

}  // namespace mw

using mw::Plan;
using mw::Policy;

extern "C" int mgemm_grouped(int64_t count, const char *transa, const char *transb, const int64_t *m,
                             const int64_t *n, const int64_t *k, const mwblas_real64x2 *alpha,
                             const mwblas_real64x2 *const *a, const int64_t *lda, const mwblas_real64x2 *const *b,
                             const int64_t *ldb, const mwblas_real64x2 *beta, mwblas_real64x2 *const *c,
                             const int64_t *ldc)
{
    using namespace mw;
    const char *routine = "mgemm_grouped";
    clear_error();
    if (!grouped_validate(routine, count, transa, transb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc))
        return mwblas_last_error();
    if (count == 0) return 0;
    if (!ensure_device(routine)) return mwblas_last_error();
    Policy pol = g_default_policy;
    {
        std::lock_guard<std::mutex> lk(g_batched_mu);
        auto it = g_policy_cache.find(shape_class(count, m, n, k));
        if (it != g_policy_cache.end()) pol = it->second;
    }
    if (g_forced_tile.load() > 0) pol.tile = g_forced_tile.load();
    if (g_forced_oz.load() >= 0) pol.oz_min = g_forced_oz.load();
    if (g_forced_pack.load() >= 0) pol.pack_k = g_forced_pack.load();
    Plan &pl = t_plan;
    build_descs(pl, count, transa, transb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc, pol);
    if (!prepare_and_launch(pl, routine)) return mwblas_last_error();
    if (!finish(routine)) return mwblas_last_error();
    return 0;
}

// Times the tensor-core size threshold (none, 64, 128, 256), the depth from
// which the remaining small instances share tensor-core slots (none, 16, 32,
// 64), then tile edges (16, 32, 64) and split-K policies for the rest, on the
// caller's batch
// (outputs go to scratch copies of C, the caller's C is not modified)
// and caches the fastest for batches of the same shape class. Returns 0 and
// the chosen minimum K per split in *chosen (0 = no split); the chosen tile
// edge is returned by mwblas_grouped_tuned_tile().
extern "C" int mgemm_grouped_tune(int64_t count, const char *transa, const char *transb, const int64_t *m,
                                  const int64_t *n, const int64_t *k, const mwblas_real64x2 *alpha,
                                  const mwblas_real64x2 *const *a, const int64_t *lda,
                                  const mwblas_real64x2 *const *b, const int64_t *ldb, const mwblas_real64x2 *beta,
                                  mwblas_real64x2 *const *c, const int64_t *ldc, int *chosen)
{
    using namespace mw;
    const char *routine = "mgemm_grouped_tune";
    clear_error();
    if (!grouped_validate(routine, count, transa, transb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc))
        return mwblas_last_error();
    if (count == 0) return 0;
    if (!ensure_device(routine)) return mwblas_last_error();
    // scratch copies of every C
    std::vector<int64_t> off((size_t)count);
    int64_t tot = 0;
    for (int64_t i = 0; i < count; ++i) {
        off[(size_t)i] = tot;
        tot += (m[i] > 0 && n[i] > 0) ? ldc[i] * n[i] : 0;
    }
    double2 *scratch = nullptr;
    if (!cuda_ok(cudaMalloc(&scratch, sizeof(double2) * (size_t)std::max<int64_t>(tot, 1)), routine, "tune scratch"))
        return mwblas_last_error();
    std::vector<mwblas_real64x2 *> cs((size_t)count);
    for (int64_t i = 0; i < count; ++i) {
        cs[(size_t)i] = (mwblas_real64x2 *)(scratch + off[(size_t)i]);
        if (m[i] > 0 && n[i] > 0)
            cudaMemcpyAsync(cs[(size_t)i], c[i], sizeof(double2) * (size_t)(ldc[i] * n[i]), cudaMemcpyDeviceToDevice,
                            stream());
    }
    // two stages: the tile edge at the default split policy, then the split
    // policy at that tile
    const int tiles[] = {16, 32, 64};
    const int cands[] = {0, 2048, 1024, 512, 256, 128};
    Plan pl;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    auto time_policy = [&](const Policy &pol) -> float {
        build_descs(pl, count, transa, transb, m, n, k, alpha, a, lda, b, ldb, beta, cs.data(), ldc, pol);
        if (!prepare_and_launch(pl, routine)) return 1e30f;   // warm + capture
        cudaEventRecord(e0, stream());
        const int reps = 3;
        for (int r = 0; r < reps; ++r) prepare_and_launch(pl, routine);
        cudaEventRecord(e1, stream());
        cudaEventSynchronize(e1);
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, e0, e1);
        return ms;
    };
    // stages: the size from which instances run on the tensor cores, the
    // depth from which the smaller ones share slots there, then the tile edge
    // of the rest (integer pipes), then its split policy
    float best = 1e30f;
    int best_tile = g_default_policy.tile, best_k = g_default_policy.min_k_per_split, best_oz = 0;
    const int ozc[] = {0, 64, 128, 256};
    for (int oz : ozc) {
        if (oz > 0 && !ozaki_available()) break;
        const float ms = time_policy(Policy{best_k, 4, best_tile, oz, 0});
        if (ms < best) {
            best = ms;
            best_oz = oz;
        }
    }
    int best_pack = 0;
    const int packc[] = {16, 32, 64};
    for (int pk : packc) {
        if (!ozaki_available()) break;
        const float ms = time_policy(Policy{best_k, 4, best_tile, best_oz, pk});
        if (ms < best) {
            best = ms;
            best_pack = pk;
        }
    }
    for (int t : tiles) {
        if (t == best_tile) continue;   // timed above
        const float ms = time_policy(Policy{best_k, 4, t, best_oz, best_pack});
        if (ms < best) {
            best = ms;
            best_tile = t;
        }
    }
    for (int cand : cands) {
        if (cand == best_k) continue;   // timed above
        const float ms = time_policy(Policy{cand, 4, best_tile, best_oz, best_pack});
        if (ms < best) {
            best = ms;
            best_k = cand;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (pl.exec) cudaGraphExecDestroy(pl.exec);
    if (pl.dev) cudaFree(pl.dev);
    ozgroup_destroy(pl.oz);
    cudaFree(scratch);
    {
        std::lock_guard<std::mutex> lk(g_batched_mu);
        g_policy_cache[shape_class(count, m, n, k)] = Policy{best_k, 4, best_tile, best_oz, best_pack};
    }
    t_tuned_oz = best_oz;
    t_tuned_pack = best_pack;
    t_tuned_tile = best_tile;
    if (chosen) *chosen = best_k;
    return finish(routine) ? 0 : mwblas_last_error();
}

extern "C" int mtrsm_grouped(int64_t count, char side, char uplo, char transa, char diag, const int64_t *m,
                             const int64_t *n, const mwblas_real64x2 *alpha, const mwblas_real64x2 *const *a,
                             const int64_t *lda, mwblas_real64x2 *const *b, const int64_t *ldb)
{
    using namespace mw;
    const char *routine = "mtrsm_grouped";
    clear_error();
    char S = (char)toupper(side), U = (char)toupper(uplo), T = (char)toupper(transa), D = (char)toupper(diag);
    if (T == 'C') T = 'T';
    if (count < 0) { set_error(routine, 1, "count < 0"); return 1; }
    if (S != 'L' && S != 'R') { set_error(routine, 2, "invalid side"); return 2; }
    if (U != 'U' && U != 'L') { set_error(routine, 3, "invalid uplo"); return 3; }
    if (T != 'N' && T != 'T') { set_error(routine, 4, "invalid transa"); return 4; }
    if (D != 'N' && D != 'U') { set_error(routine, 5, "invalid diag"); return 5; }
    if (count == 0) return 0;
    if (!m || !n || !alpha || !a || !lda || !b || !ldb) { set_error(routine, 6, "null argument array"); return 6; }
    std::vector<TrsmDesc> descs;
    descs.reserve((size_t)count);
    int64_t work = 0;
    for (int64_t i = 0; i < count; ++i) {
        if (m[i] < 0 || n[i] < 0) { set_error(routine, 6, "negative size in instance " + std::to_string(i)); return 6; }
        if (m[i] == 0 || n[i] == 0) continue;
        int64_t na = (S == 'L') ? m[i] : n[i];
        if (lda[i] < std::max<int64_t>(1, na)) { set_error(routine, 10, "lda too small in instance " + std::to_string(i)); return 10; }
        if (ldb[i] < std::max<int64_t>(1, m[i])) { set_error(routine, 12, "ldb too small in instance " + std::to_string(i)); return 12; }
        if (!is_dd_device_pointer(b[i])) {
            set_error(routine, 11, "grouped calls take 16-byte aligned device (or managed) arrays; B of instance " +
                                       std::to_string(i));
            return 11;
        }
        if (!is_dd_device_pointer(a[i])) {
            set_error(routine, 9, "grouped calls take 16-byte aligned device (or managed) arrays; A of instance " +
                                      std::to_string(i));
            return 9;
        }
        TrsmDesc d{};
        d.A = (const double2 *)a[i];
        d.B = (double2 *)b[i];
        d.lda = lda[i];
        d.ldb = ldb[i];
        d.m = (int)m[i];
        d.n = (int)n[i];
        d.alpha = make_double2(alpha[i].limbs[0], alpha[i].limbs[1]);
        const int64_t rhs = (S == 'L') ? n[i] : m[i];
        d.nchunks = (int)((rhs + 31) / 32);
        descs.push_back(d);
    }
    if (descs.empty()) return 0;
    // the longest triangles first, so that they do not form the tail
    std::stable_sort(descs.begin(), descs.end(), [S](const TrsmDesc &x, const TrsmDesc &y) {
        return (S == 'L' ? x.m : x.n) > (S == 'L' ? y.m : y.n);
    });
    int64_t xop_elems = 0;
    for (TrsmDesc &d : descs) {
        d.work_begin = work;
        work += d.nchunks;
        d.xop_begin = xop_elems;
        xop_elems += (int64_t)d.nchunks * (S == 'L' ? d.m : d.n) * 32;
    }
    if (!ensure_device(routine)) return mwblas_last_error();
    const bool trans = (T != 'N');
    const bool lower = ((U == 'L') != trans);
    TrsmPlan &pl = t_tplan;
    pl.descs.swap(descs);
    pl.total = work;
    pl.xop_elems = xop_elems;
    pl.side = S == 'L' ? 0 : 1;
    pl.lower = lower ? 1 : 0;
    pl.trans = trans ? 1 : 0;
    pl.unit = D == 'U' ? 1 : 0;
    if (!trsm_prepare_and_launch(pl, routine)) return mwblas_last_error();
    if (!finish(routine)) return mwblas_last_error();
    return 0;
}

extern "C" int mwblas_grouped_tuned_tile(void) { return mw::t_tuned_tile; }
extern "C" int mwblas_grouped_tuned_tensor_min(void) { return mw::t_tuned_oz; }
extern "C" int mwblas_grouped_tuned_tensor_pack(void) { return mw::t_tuned_pack; }

extern "C" int mwblas_set_grouped_tensor_pack(int kmin)
{
    return mw::g_forced_pack.exchange(kmin < 0 ? -1 : kmin);
}

extern "C" int mwblas_set_grouped_tensor_min(int size)
{
    return mw::g_forced_oz.exchange(size < 0 ? -1 : size);
}

extern "C" int mwblas_set_grouped_tile(int tile)
{
    const int t = (tile == 16 || tile == 32 || tile == 64) ? tile : 0;
    return mw::g_forced_tile.exchange(t);
}
