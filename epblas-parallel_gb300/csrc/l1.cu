// Level-1 double-double kernels: SCAL, AXPY, COPY, SWAP, I*AMAX, DOT and the
// complex twins.
//
// Bit-exactness. The reference's unit-stride SCAL/AXPY run the FMA-fused
// "fast" product on the first (len & ~3) elements of each OpenMP slice and the
// scalar-operator product on the remaining 0..3 (mscal.cpp:42-58,
// maxpy.cpp:42-58, wscal.cpp, wmscal.cpp), where the slices are the balanced
// front-loaded partition of blas_part_bound (common/blas_omp.h:79-84). Every
// element is independent, so a kernel that knows the team size T reproduces
// the same per-element operation sequence on any grid: element i is a "tail"
// element iff its offset inside its slice is >= (slice length & ~3).
// Strided calls use the scalar operators for every element (mscal.cpp:96-100).
// A zero increment on an output makes the reference's loop sequential
// (the same element is updated n times in order); those calls run a
// single-thread kernel that repeats the loop literally.
#include "dd.cuh"
#include "fixacc.cuh"
#include "l1.h"
#include "runtime.h"

namespace mw {

namespace {

constexpr int kThreads = 256;

// Offset of logical element i for a BLAS vector (negative inc starts at the
// far end).
__device__ __forceinline__ int64_t vidx(int64_t i, int64_t n, int64_t inc)
{
    return inc >= 0 ? i * inc : (n - 1 - i) * (-inc);
}

// Position of a thread's elements in the T-way blas_part_bound partition of
// [0, n) (blas_omp.h:79-84): slice t has base + 1 elements for t < rem and
// base after that. An element is in the scalar tail when it lies in the last
// len % 4 elements of its slice. The slice of the thread's first element is
// found with divisions once; after that the grid-stride walk only advances
// the slice (the strided index moves forward), so the per-element test is
// two compares instead of 64-bit divisions.
struct SliceWalk {
    int64_t base, rem, t, lo, len, tmax;

    __device__ __forceinline__ void start(int64_t i, int64_t n, int64_t T)
    {
        tmax = T - 1;
        base = n / T;
        rem = n % T;
        const int64_t big = rem * (base + 1);
        if (i < big) {
            t = i / (base + 1);
            lo = t * (base + 1);
            len = base + 1;
        } else {
            t = rem + (base ? (i - big) / base : 0);
            lo = t * base + rem;
            len = base;
        }
    }
    // i must not decrease between calls
    __device__ __forceinline__ bool tail(int64_t i)
    {
        while (i >= lo + len && t < tmax) {   // every slice before the last is non-empty
            lo += len;
            ++t;
            len = (t < rem) ? base + 1 : base;
        }
        return (i - lo) >= (len & ~(int64_t)3);
    }
};

int grid_for(int64_t n)
{
    int64_t blocks = (n + kThreads - 1) / kThreads;
    int64_t cap = (int64_t)device_sm_count() * 8;
    if (blocks > cap) blocks = cap;
    if (blocks < 1) blocks = 1;
    return (int)blocks;
}

// ---- SCAL ----------------------------------------------------------------

__global__ void k_mscal_unit(int64_t n, dd::real alpha, double2 *x, int64_t T)
{
    const int64_t i0 = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    SliceWalk sw;
    if (i0 < n) sw.start(i0, n, T);
    for (int64_t i = i0; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        dd::real v = dd::load(x + i);
        v = sw.tail(i) ? dd::mul_exact(v, alpha) : dd::mul_fast(v, alpha);
        dd::store(x + i, v);
    }
}

__global__ void k_mscal_strided(int64_t n, dd::real alpha, double2 *x, int64_t inc)
{
    if (inc == 0) {
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            dd::real v = dd::load(x);
            for (int64_t i = 0; i < n; ++i) v = dd::mul_exact(v, alpha);
            dd::store(x, v);
        }
        return;
    }
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double2 *p = x + vidx(i, n, inc);
        dd::store(p, dd::mul_exact(dd::load(p), alpha));
    }
}

__global__ void k_wscal_unit(int64_t n, dd::cplx alpha, double2 *x, int64_t T)
{
    const int64_t i0 = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    SliceWalk sw;
    if (i0 < n) sw.start(i0, n, T);
    for (int64_t i = i0; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        dd::cplx v = dd::cload(x + 2 * i);
        v = sw.tail(i) ? dd::cmul_exact(v, alpha) : dd::cmul_fast(v, alpha);
        dd::cstore(x + 2 * i, v);
    }
}

__global__ void k_wscal_strided(int64_t n, dd::cplx alpha, double2 *x, int64_t inc)
{
    if (inc == 0) {
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            dd::cplx v = dd::cload(x);
            for (int64_t i = 0; i < n; ++i) v = dd::cmul_exact(v, alpha);
            dd::cstore(x, v);
        }
        return;
    }
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double2 *p = x + 2 * vidx(i, n, inc);
        dd::cstore(p, dd::cmul_exact(dd::cload(p), alpha));
    }
}

__global__ void k_wmscal_unit(int64_t n, dd::real alpha, double2 *x, int64_t T)
{
    const int64_t i0 = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    SliceWalk sw;
    if (i0 < n) sw.start(i0, n, T);
    for (int64_t i = i0; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        dd::cplx v = dd::cload(x + 2 * i);
        if (sw.tail(i)) {
            v.re = dd::mul_exact(v.re, alpha);
            v.im = dd::mul_exact(v.im, alpha);
        } else {
            v.re = dd::mul_fast(v.re, alpha);
            v.im = dd::mul_fast(v.im, alpha);
        }
        dd::cstore(x + 2 * i, v);
    }
}

__global__ void k_wmscal_strided(int64_t n, dd::real alpha, double2 *x, int64_t inc)
{
    if (inc == 0) {
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            dd::cplx v = dd::cload(x);
            for (int64_t i = 0; i < n; ++i) {
                v.re = dd::mul_exact(v.re, alpha);
                v.im = dd::mul_exact(v.im, alpha);
            }
            dd::cstore(x, v);
        }
        return;
    }
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double2 *p = x + 2 * vidx(i, n, inc);
        dd::cplx v = dd::cload(p);
        v.re = dd::mul_exact(v.re, alpha);
        v.im = dd::mul_exact(v.im, alpha);
        dd::cstore(p, v);
    }
}

// ---- AXPY ------------------------------------------------------------------

__global__ void k_maxpy_unit(int64_t n, dd::real alpha, const double2 *x, double2 *y, int64_t T)
{
    const int64_t i0 = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    SliceWalk sw;
    if (i0 < n) sw.start(i0, n, T);
    for (int64_t i = i0; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        dd::real xv = dd::load(x + i), yv = dd::load(y + i);
        dd::real r;
        if (sw.tail(i))
            r = dd::add_exact(yv, dd::mul_exact(alpha, xv));
        else
            r = dd::add_fast(yv, dd::mul_fast(alpha, xv));
        dd::store(y + i, r);
    }
}

__global__ void k_maxpy_strided(int64_t n, dd::real alpha, const double2 *x, int64_t incx, double2 *y,
                                int64_t incy)
{
    if (incy == 0) {
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            dd::real yv = dd::load(y);
            for (int64_t i = 0; i < n; ++i)
                yv = dd::add_exact(yv, dd::mul_exact(alpha, dd::load(x + vidx(i, n, incx))));
            dd::store(y, yv);
        }
        return;
    }
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double2 *py = y + vidx(i, n, incy);
        dd::real xv = dd::load(x + vidx(i, n, incx));
        dd::store(py, dd::add_exact(dd::load(py), dd::mul_exact(alpha, xv)));
    }
}

// ---- COPY / SWAP -----------------------------------------------------------

// elem2 = number of double2 words per element (1 real, 2 complex).
__global__ void k_copy(int64_t n, const double2 *x, int64_t incx, double2 *y, int64_t incy, int elem2)
{
    if (incy == 0) {
        // Sequential reference loop: the last logical element wins.
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            const double2 *src = x + elem2 * vidx(n - 1, n, incx);
            for (int w = 0; w < elem2; ++w) y[w] = src[w];
        }
        return;
    }
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double2 *src = x + elem2 * vidx(i, n, incx);
        double2 *dst = y + elem2 * vidx(i, n, incy);
        for (int w = 0; w < elem2; ++w) dst[w] = src[w];
    }
}

__global__ void k_swap(int64_t n, double2 *x, int64_t incx, double2 *y, int64_t incy, int elem2)
{
    if (incx == 0 || incy == 0) {
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            for (int64_t i = 0; i < n; ++i) {
                double2 *px = x + elem2 * vidx(i, n, incx);
                double2 *py = y + elem2 * vidx(i, n, incy);
                for (int w = 0; w < elem2; ++w) {
                    double2 t = px[w];
                    px[w] = py[w];
                    py[w] = t;
                }
            }
        }
        return;
    }
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double2 *px = x + elem2 * vidx(i, n, incx);
        double2 *py = y + elem2 * vidx(i, n, incy);
        for (int w = 0; w < elem2; ++w) {
            double2 t = px[w];
            px[w] = py[w];
            py[w] = t;
        }
    }
}

// ---- I*AMAX ------------------------------------------------------------------
// Order: lexicographic (|hi|, sign-adjusted lo) maximum, lowest index on ties
// (imamax.cpp:43-72, mf_pred.h:60-63). Complex magnitude |re|+|im| uses the
// scalar-operator add (iwamax.cpp:36-76).
//
// The comparison runs on the integer pipe: each magnitude becomes a 128-bit
// unsigned key whose order is the FP64 order of (|hi|, lo). Word 0..1 hold the
// bits of |hi| (monotone for non-negative doubles), words 2..3 the usual
// orderable image of lo (negative: all bits inverted; positive: sign bit set),
// with -0 mapped to +0 so the two zeros tie as they do under FP64 '=='. A NaN
// hi gives the all-zero key and a NaN lo the zero low half, so a NaN never
// beats a number, as with the reference's -inf-seeded vector scan in which
// 'NaN > best' is false; among all-NaN inputs the lowest index wins.

struct AmaxKey {
    uint32_t k[4];   // k[0] most significant
    int64_t idx;     // 0-based; -1 = empty
};

__device__ __forceinline__ AmaxKey amax_key(uint4 v, int64_t idx)
{
    // v = {hi.lo32, hi.hi32, lo.lo32, lo.hi32}
    AmaxKey r;
    const uint32_t ah = v.y & 0x7fffffffu;
    const bool hnan = ah > 0x7ff00000u || (ah == 0x7ff00000u && v.x != 0u);
    const uint32_t lh = v.w ^ (v.y & 0x80000000u);   // lo, sign flipped when hi < 0
    const uint32_t al = lh & 0x7fffffffu;
    const bool lnan = al > 0x7ff00000u || (al == 0x7ff00000u && v.z != 0u);
    const bool lzero = (al | v.z) == 0u;
    const uint32_t m = (uint32_t)((int32_t)lh >> 31);
    uint32_t k2 = lh ^ (m | 0x80000000u), k3 = v.z ^ m;
    if (lzero) { k2 = 0x80000000u; k3 = 0u; }
    if (lnan) { k2 = 0u; k3 = 0u; }
    r.k[0] = hnan ? 0u : ah;
    r.k[1] = hnan ? 0u : v.x;
    r.k[2] = hnan ? 0u : k2;
    r.k[3] = hnan ? 0u : k3;
    r.idx = idx;
    return r;
}

// a.k > b.k as 128-bit unsigned numbers: the borrow out of b - a.
__device__ __forceinline__ bool key_gt(const AmaxKey &a, const AmaxKey &b)
{
    uint32_t borrow;
    asm("{\n\t"
        ".reg .u32 t;\n\t"
        "sub.cc.u32 t, %4, %8;\n\t"
        "subc.cc.u32 t, %3, %7;\n\t"
        "subc.cc.u32 t, %2, %6;\n\t"
        "subc.cc.u32 t, %1, %5;\n\t"
        "subc.u32 %0, 0, 0;\n\t"
        "}"
        : "=r"(borrow)
        : "r"(b.k[0]), "r"(b.k[1]), "r"(b.k[2]), "r"(b.k[3]), "r"(a.k[0]), "r"(a.k[1]), "r"(a.k[2]),
          "r"(a.k[3]));
    return borrow != 0u;
}

__device__ __forceinline__ bool key_eq(const AmaxKey &a, const AmaxKey &b)
{
    return ((a.k[0] ^ b.k[0]) | (a.k[1] ^ b.k[1]) | (a.k[2] ^ b.k[2]) | (a.k[3] ^ b.k[3])) == 0u;
}

// Merge order of two partial results (either may be empty).
__device__ __forceinline__ bool amax_better(const AmaxKey &a, const AmaxKey &b)
{
    if (a.idx < 0) return false;
    if (b.idx < 0) return true;
    return key_gt(a, b) || (key_eq(a, b) && a.idx < b.idx);
}

__device__ __forceinline__ AmaxKey amax_shfl(const AmaxKey &k, int off)
{
    AmaxKey r;
#pragma unroll
    for (int w = 0; w < 4; ++w) r.k[w] = __shfl_down_sync(0xffffffffu, k.k[w], off);
    r.idx = __shfl_down_sync(0xffffffffu, k.idx, off);
    return r;
}

__device__ __forceinline__ AmaxKey amax_empty()
{
    AmaxKey r;
    r.k[0] = r.k[1] = r.k[2] = r.k[3] = 0u;
    r.idx = -1;
    return r;
}

__device__ AmaxKey amax_block_reduce(AmaxKey k)
{
    __shared__ AmaxKey sh[kThreads / 32];
    for (int off = 16; off > 0; off >>= 1) {
        AmaxKey o = amax_shfl(k, off);
        if (amax_better(o, k)) k = o;
    }
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) sh[wid] = k;
    __syncthreads();
    if (wid == 0) {
        k = (lane < (int)(blockDim.x >> 5)) ? sh[lane] : amax_empty();
        for (int off = 16; off > 0; off >>= 1) {
            AmaxKey o = amax_shfl(k, off);
            if (amax_better(o, k)) k = o;
        }
    }
    return k;
}

__device__ __forceinline__ uint4 dd_bits(dd::real m)
{
    const unsigned long long h = (unsigned long long)__double_as_longlong(m.hi);
    const unsigned long long l = (unsigned long long)__double_as_longlong(m.lo);
    return make_uint4((uint32_t)h, (uint32_t)(h >> 32), (uint32_t)l, (uint32_t)(l >> 32));
}

// Within one thread the candidates arrive in increasing index order, so a
// strict '>' keeps the lowest index among equal keys.
template <bool CPLX>
__global__ void k_iamax_partial(int64_t n, const double2 *x, int64_t inc, AmaxKey *part)
{
    AmaxKey best = amax_empty();
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const int64_t i0 = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (!CPLX && inc == 1) {
        // unit stride: two adjacent elements (32 bytes) per thread and step
        const uint4 *v = (const uint4 *)x;
        const int64_t npair = n >> 1;
        for (int64_t p = i0; p < npair; p += stride) {
            const uint4 a = __ldcs(v + 2 * p), b = __ldcs(v + 2 * p + 1);
            const AmaxKey ka = amax_key(a, 2 * p), kb = amax_key(b, 2 * p + 1);
            if (best.idx < 0 || key_gt(ka, best)) best = ka;
            if (key_gt(kb, best)) best = kb;
        }
        if ((n & 1) && i0 == 0) {
            const AmaxKey kl = amax_key(__ldcs(v + n - 1), n - 1);
            if (best.idx < 0 || key_gt(kl, best)) best = kl;   // highest index: strict '>'
        }
    } else {
        for (int64_t i = i0; i < n; i += stride) {
            uint4 bits;
            if (CPLX) {
                const double2 *p = x + 2 * vidx(i, n, inc);
                bits = dd_bits(dd::add_exact(dd::mag(dd::load(p)), dd::mag(dd::load(p + 1))));
            } else {
                bits = __ldcs((const uint4 *)(x + vidx(i, n, inc)));
            }
            const AmaxKey c = amax_key(bits, i);
            if (best.idx < 0 || key_gt(c, best)) best = c;
        }
    }
    best = amax_block_reduce(best);
    if (threadIdx.x == 0) part[blockIdx.x] = best;
}

__global__ void k_iamax_final(int nparts, const AmaxKey *part, int64_t *out)
{
    AmaxKey best = amax_empty();
    for (int i = threadIdx.x; i < nparts; i += blockDim.x)
        if (amax_better(part[i], best)) best = part[i];
    best = amax_block_reduce(best);
    if (threadIdx.x == 0) *out = best.idx;
}

// ---- DOT ---------------------------------------------------------------------
// mdot.cpp:48-87 accumulates TwoProduct + Bailey three-limb sums on the FP64
// pipe. Here the products are accumulated exactly (to 2^-126 of each product)
// in per-thread integer fixed point (fixacc.cuh), the thread sums are added
// as 128-bit extended floats in a fixed order (warp, block, then the grid's
// block partials), and the result is rounded once to double-double. The
// result is deterministic for a given n and device and at least as accurate
// as the reference's.

__device__ fx::XF xf_block_sum(fx::XF v)
{
    __shared__ fx::XFPod sh[kThreads / 32];
    v = fx::xf_warp_sum(v);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
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

__device__ bool block_any(bool b)
{
    return __syncthreads_or(b ? 1 : 0) != 0;
}

__global__ void __launch_bounds__(kThreads, 4) k_mdot_partial(int64_t n, const double2 *__restrict__ x, int64_t incx,
                                                          const double2 *__restrict__ y, int64_t incy,
                                                          fx::XFPod *part)
{
    fx::Acc acc;
    acc.reset();
    fx::XF total;   // accumulators are folded in here every kMaxAdds products
    total.zero = true; total.neg = false; total.m = 0; total.e = 0;
    bool bad = false;
    int cnt = 0;
    auto fold = [&]() {
        bad |= acc.bad;
        total = xfp::xf_add(total, acc.finish());
        acc.reset();
        cnt = 0;
    };
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (incx == 1 && incy == 1) {
        // two elements in flight per thread; the column carries are
        // propagated after each run of 2048 products, outside the inner loop
        while (i + stride < n) {
            const int64_t iend = i + 2 * stride * 1024;
            for (; i + stride < n && i < iend; i += 2 * stride) {
                const double2 x0 = __ldcs(x + i), y0 = __ldcs(y + i);
                const double2 x1 = __ldcs(x + i + stride), y1 = __ldcs(y + i + stride);
                acc.add_core(fx::decode(x0), fx::to_dig(fx::decode(y0)));
                acc.add_core(fx::decode(x1), fx::to_dig(fx::decode(y1)));
            }
            acc.normalize();
            if ((cnt += 2048) >= fx::kMaxAdds) fold();
        }
    }
    for (; i < n; i += stride) {
        acc.add_prod(fx::decode(x[vidx(i, n, incx)]), fx::decode(y[vidx(i, n, incy)]));
        if (++cnt >= fx::kMaxAdds) fold();
    }
    fold();
    bad = block_any(bad);
    fx::XF v = xf_block_sum(total);
    if (threadIdx.x == 0) part[blockIdx.x] = fx::to_pod(v, bad);
}

__global__ void __launch_bounds__(kThreads) k_mdot_final(int nparts, const fx::XFPod *part, double2 *out)
{
    fx::XF acc;
    acc.zero = true; acc.neg = false; acc.m = 0; acc.e = 0;
    bool bad = false;
    for (int i = threadIdx.x; i < nparts; i += blockDim.x) {
        const fx::XFPod p = part[i];
        bad |= (p.flags & 4) != 0;
        acc = xfp::xf_add(acc, fx::from_pod(p));
    }
    bad = block_any(bad);
    acc = xf_block_sum(acc);
    if (threadIdx.x == 0) {
        double h, l;
        xfp::xf_to_dd(acc, h, l);
        if (bad) h = l = __longlong_as_double(0x7ff8000000000000ll);
        *out = make_double2(h, l);
    }
}

}  // namespace

// ---- launchers ---------------------------------------------------------------

void launch_mscal(int64_t n, dd_host alpha, void *x, int64_t inc, bool unit, int64_t team)
{
    dd::real a = dd::make(alpha.hi, alpha.lo);
    if (unit)
        k_mscal_unit<<<grid_for(n), kThreads, 0, stream()>>>(n, a, (double2 *)x, team);
    else
        k_mscal_strided<<<inc == 0 ? 1 : grid_for(n), kThreads, 0, stream()>>>(n, a, (double2 *)x, inc);
    count_launch();
}

void launch_wscal(int64_t n, cdd_host alpha, void *x, int64_t inc, bool unit, int64_t team)
{
    dd::cplx a;
    a.re = dd::make(alpha.re.hi, alpha.re.lo);
    a.im = dd::make(alpha.im.hi, alpha.im.lo);
    if (unit)
        k_wscal_unit<<<grid_for(n), kThreads, 0, stream()>>>(n, a, (double2 *)x, team);
    else
        k_wscal_strided<<<inc == 0 ? 1 : grid_for(n), kThreads, 0, stream()>>>(n, a, (double2 *)x, inc);
    count_launch();
}

void launch_wmscal(int64_t n, dd_host alpha, void *x, int64_t inc, bool unit, int64_t team)
{
    dd::real a = dd::make(alpha.hi, alpha.lo);
    if (unit)
        k_wmscal_unit<<<grid_for(n), kThreads, 0, stream()>>>(n, a, (double2 *)x, team);
    else
        k_wmscal_strided<<<inc == 0 ? 1 : grid_for(n), kThreads, 0, stream()>>>(n, a, (double2 *)x, inc);
    count_launch();
}

void launch_maxpy(int64_t n, dd_host alpha, const void *x, int64_t incx, void *y, int64_t incy, bool unit,
                  int64_t team)
{
    dd::real a = dd::make(alpha.hi, alpha.lo);
    if (unit)
        k_maxpy_unit<<<grid_for(n), kThreads, 0, stream()>>>(n, a, (const double2 *)x, (double2 *)y, team);
    else
        k_maxpy_strided<<<incy == 0 ? 1 : grid_for(n), kThreads, 0, stream()>>>(n, a, (const double2 *)x, incx,
                                                                               (double2 *)y, incy);
    count_launch();
}

void launch_copy(int64_t n, const void *x, int64_t incx, void *y, int64_t incy, int elem2)
{
    k_copy<<<incy == 0 ? 1 : grid_for(n), kThreads, 0, stream()>>>(n, (const double2 *)x, incx, (double2 *)y,
                                                                  incy, elem2);
    count_launch();
}

void launch_swap(int64_t n, void *x, int64_t incx, void *y, int64_t incy, int elem2)
{
    bool seq = (incx == 0 || incy == 0);
    k_swap<<<seq ? 1 : grid_for(n), kThreads, 0, stream()>>>(n, (double2 *)x, incx, (double2 *)y, incy, elem2);
    count_launch();
}

bool launch_iamax(int64_t n, const void *x, int64_t inc, bool cplx, int64_t *result_host, const char *routine)
{
    int g = grid_for(n);
    size_t bytes = (size_t)g * sizeof(AmaxKey) + 64;
    char *scratch = (char *)dev_alloc(bytes, routine);
    if (!scratch) return false;
    AmaxKey *part = (AmaxKey *)scratch;
    int64_t *out = (int64_t *)(scratch + (((size_t)g * sizeof(AmaxKey) + 15) / 16) * 16);
    if (cplx)
        k_iamax_partial<true><<<g, kThreads, 0, stream()>>>(n, (const double2 *)x, inc, part);
    else
        k_iamax_partial<false><<<g, kThreads, 0, stream()>>>(n, (const double2 *)x, inc, part);
    k_iamax_final<<<1, kThreads, 0, stream()>>>(g, part, out);
    count_launch(2);
    bool ok = cuda_ok(cudaMemcpyAsync(result_host, out, sizeof(int64_t), cudaMemcpyDeviceToHost, stream()), routine,
                      "iamax result readback");
    dev_free(scratch);
    if (!ok) return false;
    return cuda_ok(cudaStreamSynchronize(stream()), routine, "iamax sync");
}

bool launch_mdot(int64_t n, const void *x, int64_t incx, const void *y, int64_t incy, dd_host *result_host,
                 const char *routine)
{
    int g = grid_for(n);
    size_t bytes = (size_t)g * sizeof(fx::XFPod) + 256;
    char *buf = (char *)dev_alloc(bytes, routine);
    if (!buf) return false;
    fx::XFPod *part = (fx::XFPod *)buf;
    double2 *res = (double2 *)(buf + ((size_t)g * sizeof(fx::XFPod) + 15) / 16 * 16);
    k_mdot_partial<<<g, kThreads, 0, stream()>>>(n, (const double2 *)x, incx, (const double2 *)y, incy, part);
    k_mdot_final<<<1, kThreads, 0, stream()>>>(g, part, res);
    count_launch(2);
    double2 r;
    bool ok = cuda_ok(cudaMemcpyAsync(&r, res, sizeof(double2), cudaMemcpyDeviceToHost, stream()), routine,
                      "dot result readback");
    dev_free(buf);
    if (!ok) return false;
    if (!cuda_ok(cudaStreamSynchronize(stream()), routine, "dot sync")) return false;
    result_host->hi = r.x;
    result_host->lo = r.y;
    return true;
}

}  // namespace mw
