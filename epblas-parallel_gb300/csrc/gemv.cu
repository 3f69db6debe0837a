// Double-double GEMV: y := alpha*op(A)*x + beta*y (mgemv.cpp:237-275).
//
// beta pre-pass first (mf_kernels.h:63-68: beta == 0 zeroes y, beta == 1
// leaves it), then nothing more when alpha == 0, as in the reference.
//
// NoTrans: thread per row, the columns split into chunks over grid.y so the
// whole GPU streams A once; per-chunk partial sums go to scratch and a second
// kernel folds them in a fixed order and applies y += alpha*s.
// Trans: block per column (A's columns are contiguous), warp-shuffle and
// shared-memory reduction, then y_j += alpha*s (mgemv.cpp:229-233).
// mgemv_ accumulates the products in per-thread integer fixed point
// (fixacc.cuh): x is first split once into 24-bit digit sets (32 bytes per
// entry; it is small and stays in L2), each A(i,j) is decoded from its bits
// and its digits multiplied into the thread's exact column sums; partial sums
// combine as extended floats in a fixed order, and y := y + alpha*s is
// rounded once to double-double. The FP64 pipe, which would bound a
// double-double multiply-add at a fraction of HBM speed, is not used in the
// loop.
// mgemv_n_noalloc keeps the FP64 accumulation (TwoProduct + TwoSum into a
// (sum, error) pair, renormalised every 32 terms, the lo*lo product dropped as
// in mdot.cpp:60-64) so that its partial sums fit its fixed scratch array.
#include <mutex>

#include "dd.cuh"
#include "fixacc.cuh"
#include "level3.h"
#include "runtime.h"

namespace mw {

namespace {

__device__ __forceinline__ int64_t vidx(int64_t i, int64_t n, int64_t inc)
{
    return inc >= 0 ? i * inc : (n - 1 - i) * (-inc);
}

__device__ __forceinline__ void acc_prod(double &s, double &e, double2 a, double2 b)
{
    double p, pe, t;
    dd::two_prod(a.x, b.x, p, pe);
    e = __fma_rn(a.x, b.y, e);
    e = __fma_rn(a.y, b.x, e);
    e = __dadd_rn(e, pe);
    dd::two_sum(s, p, s, t);
    e = __dadd_rn(e, t);
}

__global__ void k_scale_vec(int64_t n, dd::real beta, int beta_kind, double2 *y, int64_t incy)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double2 *p = y + vidx(i, n, incy);
        if (beta_kind == 0) *p = make_double2(0.0, 0.0);
        else dd::store(p, dd::mul_exact(beta, dd::load(p)));
    }
}

__global__ void k_gemv_n_partial(int64_t m, int64_t n, const double2 *A, int64_t lda, const double2 *x, int64_t incx,
                                 int64_t chunk, double2 *part)
{
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= m) return;
    int64_t j0 = blockIdx.y * chunk, j1 = min(n, j0 + chunk);
    double s = 0.0, e = 0.0;
    int cnt = 0;
    for (int64_t j = j0; j < j1; ++j) {
        acc_prod(s, e, A[i + j * lda], x[vidx(j, n, incx)]);
        if (++cnt == 32) {
            dd::fast_two_sum(s, e, s, e);
            cnt = 0;
        }
    }
    double h, l;
    dd::two_sum(s, e, h, l);
    part[blockIdx.y * m + i] = make_double2(h, l);
}

__global__ void k_gemv_n_final(int64_t m, int nchunks, const double2 *part, dd::real alpha, double2 *y,
                               int64_t incy)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
        dd::real s = dd::load(part + i);
        for (int c = 1; c < nchunks; ++c) s = dd::add_fast(s, dd::load(part + (int64_t)c * m + i));
        double2 *py = y + vidx(i, m, incy);
        dd::store(py, dd::add_exact(dd::load(py), dd::mul_exact(alpha, s)));
    }
}

// ---- fixed-point kernels (mgemv_) ------------------------------------------------------

__global__ void k_dig_convert(int64_t n, const double2 *x, int64_t incx, fx::Dig *out)
{
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x)
        out[j] = fx::to_dig(fx::decode(x[vidx(j, n, incx)]));
}

// NoTrans partial sums: row per thread, columns [j0, j1) of chunk blockIdx.y
// (at most fx::kMaxAdds columns per chunk).
__global__ void __launch_bounds__(256, 4) k_gemv_n_fx(int64_t m, int64_t n, const double2 *__restrict__ A,
                                                     int64_t lda, const fx::Dig *__restrict__ xo, int64_t chunk,
                                                     fx::XFPod *__restrict__ part)
{
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= m) return;
    const int64_t j0 = blockIdx.y * chunk, j1 = min(n, j0 + chunk);
    fx::Acc acc;
    acc.reset();
    const double2 *a = A + i;
    int64_t j = j0;
    // four columns in flight; carries propagated after each 2048 columns
    while (j + 4 <= j1) {
        const int64_t jend = min(j1, j + 2048);
        for (; j + 4 <= jend; j += 4) {
            const double2 a0 = __ldcs(a + j * lda), a1 = __ldcs(a + (j + 1) * lda);
            const double2 a2 = __ldcs(a + (j + 2) * lda), a3 = __ldcs(a + (j + 3) * lda);
            const fx::Dig x0 = xo[j], x1 = xo[j + 1], x2 = xo[j + 2], x3 = xo[j + 3];
            if (fx::decode_is_fast(a0) && fx::decode_is_fast(a1) && fx::decode_is_fast(a2) && fx::decode_is_fast(a3) &&
                ((x0.flags | x1.flags | x2.flags | x3.flags) & (fx::kZero | fx::kBad)) == 0) {
                // normal operands (the common case): no per-product flag
                // tests, one block-exponent test per four products
                const fx::Op o0 = fx::decode_fast(a0), o1 = fx::decode_fast(a1);
                const fx::Op o2 = fx::decode_fast(a2), o3 = fx::decode_fast(a3);
                const int e0 = o0.e + x0.e, e1 = o1.e + x1.e, e2 = o2.e + x2.e, e3 = o3.e + x3.e;
                acc.admit(max(max(e0, e1), max(e2, e3)));
                acc.mul_fast(o0, x0, acc.B - e0);
                acc.mul_fast(o1, x1, acc.B - e1);
                acc.mul_fast(o2, x2, acc.B - e2);
                acc.mul_fast(o3, x3, acc.B - e3);
            } else {
                acc.add_core(fx::decode(a0), x0);
                acc.add_core(fx::decode(a1), x1);
                acc.add_core(fx::decode(a2), x2);
                acc.add_core(fx::decode(a3), x3);
            }
        }
        acc.normalize();
    }
    for (; j < j1; ++j) acc.add_dig(fx::decode(a[j * lda]), xo[j]);
    part[blockIdx.y * m + i] = fx::to_pod(acc.finish(), acc.bad);
}

// y(i) := y(i) + alpha * sum_c part(c, i), one rounding to double-double.
__device__ __forceinline__ void fx_update_y(double2 *py, const xfp::XF &xa, xfp::XF s, bool bad)
{
    const double2 y0 = *py;
    if (bad) {
        *py = make_double2(__longlong_as_double(0x7ff8000000000000ll), __longlong_as_double(0x7ff8000000000000ll));
        return;
    }
    xfp::XF t = xfp::xf_mul(xa, s);
    if (!fx::finite_dd(y0)) {
        double h, l;
        xfp::xf_to_dd(t, h, l);
        dd::store(py, dd::add_exact(dd::make(y0.x, y0.y), dd::make(h, l)));
        return;
    }
    t = xfp::xf_add(xfp::xf_from_dd(y0.x, y0.y), t);
    double h, l;
    xfp::xf_to_dd(t, h, l);
    *py = make_double2(h, l);
}

__global__ void k_gemv_n_fx_final(int64_t m, int nchunks, const fx::XFPod *part, dd::real alpha, double2 *y,
                                  int64_t incy)
{
    const xfp::XF xa = xfp::xf_from_dd(alpha.hi, alpha.lo);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
        xfp::XF s;
        s.zero = true; s.neg = false; s.m = 0; s.e = 0;
        bool bad = false;
        for (int c = 0; c < nchunks; ++c) {
            const fx::XFPod p = part[(int64_t)c * m + i];
            bad |= (p.flags & 4) != 0;
            s = xfp::xf_add(s, fx::from_pod(p));
        }
        fx_update_y(y + vidx(i, m, incy), xa, s, bad);
    }
}

// Trans: block per column j of A (contiguous), threads over rows; every
// fx::kMaxAdds products a thread's accumulator is folded into an extended float.
__global__ void __launch_bounds__(256, 3) k_gemv_t_fx(int64_t m, int64_t n, const double2 *__restrict__ A,
                                                     int64_t lda, const fx::Dig *__restrict__ xo, dd::real alpha,
                                                     double2 *y, int64_t incy)
{
    __shared__ fx::XFPod sh[8];
    const int64_t j = blockIdx.x;
    const double2 *col = A + j * lda;
    fx::Acc acc;
    acc.reset();
    xfp::XF total;
    total.zero = true; total.neg = false; total.m = 0; total.e = 0;
    bool bad = false;
    int cnt = 0;
    auto fold = [&]() {
        bad |= acc.bad;
        total = xfp::xf_add(total, acc.finish());
        acc.reset();
        cnt = 0;
    };
    // four rows in flight per thread (GEMV N's flag-free groups of four);
    // carries propagated after each run of 2048 products
    const int64_t bs = blockDim.x;
    int64_t i = threadIdx.x;
    while (i + 3 * bs < m) {
        const int64_t iend = i + 4 * bs * 512;
        for (; i + 3 * bs < m && i < iend; i += 4 * bs) {
            const double2 a0 = __ldcs(col + i), a1 = __ldcs(col + i + bs);
            const double2 a2 = __ldcs(col + i + 2 * bs), a3 = __ldcs(col + i + 3 * bs);
            const fx::Dig x0 = xo[i], x1 = xo[i + bs], x2 = xo[i + 2 * bs], x3 = xo[i + 3 * bs];
            if (fx::decode_is_fast(a0) && fx::decode_is_fast(a1) && fx::decode_is_fast(a2) && fx::decode_is_fast(a3) &&
                ((x0.flags | x1.flags | x2.flags | x3.flags) & (fx::kZero | fx::kBad)) == 0) {
                const fx::Op o0 = fx::decode_fast(a0), o1 = fx::decode_fast(a1);
                const fx::Op o2 = fx::decode_fast(a2), o3 = fx::decode_fast(a3);
                const int e0 = o0.e + x0.e, e1 = o1.e + x1.e, e2 = o2.e + x2.e, e3 = o3.e + x3.e;
                acc.admit(max(max(e0, e1), max(e2, e3)));
                acc.mul_fast(o0, x0, acc.B - e0);
                acc.mul_fast(o1, x1, acc.B - e1);
                acc.mul_fast(o2, x2, acc.B - e2);
                acc.mul_fast(o3, x3, acc.B - e3);
            } else {
                acc.add_core(fx::decode(a0), x0);
                acc.add_core(fx::decode(a1), x1);
                acc.add_core(fx::decode(a2), x2);
                acc.add_core(fx::decode(a3), x3);
            }
        }
        acc.normalize();
        if ((cnt += 2048) >= fx::kMaxAdds) fold();
    }
    for (; i < m; i += bs) {
        acc.add_dig(fx::decode(__ldcs(col + i)), xo[i]);
        if (++cnt >= fx::kMaxAdds) fold();
    }
    bad |= acc.bad;
    total = xfp::xf_add(total, acc.finish());
    bad = __syncthreads_or(bad ? 1 : 0) != 0;
    xfp::XF v = fx::xf_warp_sum(total);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) sh[wid] = fx::to_pod(v, false);
    __syncthreads();
    if (wid == 0) {
        if (lane < (int)(blockDim.x >> 5)) v = fx::from_pod(sh[lane]);
        else { v.zero = true; v.neg = false; v.m = 0; v.e = 0; }
        v = fx::xf_warp_sum(v);
        if (lane == 0) fx_update_y(y + vidx(j, n, incy), xfp::xf_from_dd(alpha.hi, alpha.lo), v, bad);
    }
}

}  // namespace

bool gemv_device(bool trans, int64_t m, int64_t n, dd_host alpha, const void *A, int64_t lda, const void *x,
                 int64_t incx, dd_host beta, int beta_kind, void *y, int64_t incy, const char *routine)
{
    int64_t leny = trans ? n : m;
    int sms = device_sm_count();
    if (beta_kind != 1) {
        int64_t blocks = (leny + 255) / 256;
        if (blocks > sms * 8) blocks = sms * 8;
        k_scale_vec<<<(unsigned)blocks, 256, 0, stream()>>>(leny, dd::make(beta.hi, beta.lo), beta_kind, (double2 *)y,
                                                            incy);
        count_launch();
    }
    if (alpha.hi == 0.0 && alpha.lo == 0.0) return true;
    dd::real al = dd::make(alpha.hi, alpha.lo);
    const int64_t lenx = trans ? m : n;
    // x as digit sets (lenx * 32 bytes), then the partial sums
    const size_t xf_bytes = ((size_t)lenx * sizeof(fx::Dig) + 255) / 256 * 256;
    if (!trans) {
        int64_t rowblocks = (m + 255) / 256;
        int64_t want = 8 * (int64_t)sms;
        int64_t nchunks = (want + rowblocks - 1) / rowblocks;
        if (nchunks < (n + fx::kMaxAdds - 1) / fx::kMaxAdds) nchunks = (n + fx::kMaxAdds - 1) / fx::kMaxAdds;
        if (nchunks > n) nchunks = n;
        if (nchunks < 1) nchunks = 1;
        int64_t chunk = (n + nchunks - 1) / nchunks;
        nchunks = (n + chunk - 1) / chunk;
        if (nchunks > 65535) {
            set_error(routine, MWBLAS_ERR_UNSUPPORTED, "n too large for the no-transpose GEMV grid");
            return false;
        }
        char *buf = (char *)dev_alloc(xf_bytes + sizeof(fx::XFPod) * (size_t)(nchunks * m), routine);
        if (!buf) return false;
        fx::Dig *xf = (fx::Dig *)buf;
        fx::XFPod *part = (fx::XFPod *)(buf + xf_bytes);
        int64_t cb = (n + 255) / 256;
        if (cb > sms * 8) cb = sms * 8;
        k_dig_convert<<<(unsigned)cb, 256, 0, stream()>>>(n, (const double2 *)x, incx, xf);
        dim3 grid((unsigned)rowblocks, (unsigned)nchunks);
        k_gemv_n_fx<<<grid, 256, 0, stream()>>>(m, n, (const double2 *)A, lda, xf, chunk, part);
        int64_t fb = (m + 255) / 256;
        if (fb > sms * 8) fb = sms * 8;
        k_gemv_n_fx_final<<<(unsigned)fb, 256, 0, stream()>>>(m, (int)nchunks, part, al, (double2 *)y, incy);
        count_launch(3);
        dev_free(buf);
    } else {
        fx::Dig *xf = (fx::Dig *)dev_alloc(xf_bytes, routine);
        if (!xf) return false;
        int64_t cb = (m + 255) / 256;
        if (cb > sms * 8) cb = sms * 8;
        k_dig_convert<<<(unsigned)cb, 256, 0, stream()>>>(m, (const double2 *)x, incx, xf);
        k_gemv_t_fx<<<(unsigned)n, 256, 0, stream()>>>(m, n, (const double2 *)A, lda, xf, al, (double2 *)y, incy);
        count_launch(2);
        dev_free(xf);
    }
    return true;
}

}  // namespace mw

// ---- GEMV without device allocation ----------------------------------------------------
//
// For callers that must not allocate device memory on the call path: code whose
// device memory is owned by its own allocator under a fixed budget (cudaMalloc
// there would bypass the budget), and code that cannot afford the driver
// allocator's locking or cudaFree's device-wide synchronisation while other
// work is in flight. mgemv_ itself allocates the per-chunk partial sums of
// the no-transpose kernel (and staging copies of host arrays); this variant
// keeps the partial sums in a file-scope device array instead.
//
// The array below is the only scratch. It is 1 MiB (65536 double-double
// partial sums), every GPU that loads the library holds it until the process
// exits, and all calls share it: two calls whose kernels overlap on the GPU
// (different streams, or different host threads) race on it. Nothing in it
// needs to start at zero: every entry a call reads was written earlier by the
// same call. The host learns its device address once per device, with that
// device current, on the first call made on that device; that first call
// should therefore come before any stream capture. The address is cached
// together with the CUDA context it was looked up in and looked up again
// when the calling thread's current context differs (after cudaDeviceReset,
// or on a context other than the device's primary one).

namespace mw {
namespace {

constexpr int64_t kNoAllocScratch = 65536;   // double2 entries (1 MiB)
static __device__ __align__(256) double2 g_gemv_noalloc_scratch[kNoAllocScratch];

std::mutex g_noalloc_mu;
double2 *g_noalloc_addr[64] = {};
void *g_noalloc_ctx[64] = {};

// The calling thread's current CUDA context (driver entry point, looked up once).
void *current_context()
{
    using Fn = int (*)(void **);
    static Fn fn = [] {
        void *f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            f = nullptr;
        return (Fn)f;
    }();
    void *ctx = nullptr;
    if (!fn || fn(&ctx) != 0) return nullptr;
    return ctx;
}

}  // namespace
}  // namespace mw

extern "C" int mgemv_n_noalloc(int64_t m, int64_t n, const mwblas_real64x2 *alpha, const mwblas_real64x2 *a,
                               int64_t lda, const mwblas_real64x2 *x, int64_t incx, const mwblas_real64x2 *beta,
                               mwblas_real64x2 *y, int64_t incy, void *cuda_stream)
{
    using namespace mw;
    const char *routine = "mgemv_n_noalloc";
    clear_error();
    if (!alpha || !beta) { set_error(routine, 3, "null alpha or beta"); return 3; }
    if (m < 0) { set_error(routine, 1, "m < 0"); return 1; }
    if (n < 0) { set_error(routine, 2, "n < 0"); return 2; }
    if (lda < (m > 1 ? m : 1)) { set_error(routine, 5, "lda too small"); return 5; }
    if (incx == 0) { set_error(routine, 7, "incx == 0"); return 7; }
    if (incy == 0) { set_error(routine, 10, "incy == 0"); return 10; }
    if (m > kNoAllocScratch) {
        set_error(routine, 1, "m exceeds the 65536-row limit of the fixed 1 MiB scratch array");
        return 1;
    }
    if (m == 0 || n == 0) return 0;
    const dd_host al{alpha->limbs[0], alpha->limbs[1]}, be{beta->limbs[0], beta->limbs[1]};
    const bool alpha0 = (al.hi == 0.0 && al.lo == 0.0);
    const int bk = (be.hi == 0.0 && be.lo == 0.0) ? 0 : ((be.hi == 1.0 && be.lo == 0.0) ? 1 : 2);
    if (alpha0 && bk == 1) return 0;
    if (!y || !is_dd_device_pointer(y) ||
        (!alpha0 && (!a || !x || !is_dd_device_pointer(a) || !is_dd_device_pointer(x)))) {
        set_error(routine, 9, "A, x and y must be 16-byte aligned device or managed memory (this entry point stages nothing)");
        return 9;
    }
    int dev = 0;
    if (!cuda_ok(cudaGetDevice(&dev), routine, "cudaGetDevice")) return MWBLAS_ERR_CUDA;
    if (dev < 0 || dev >= 64) { set_error(routine, MWBLAS_ERR_DEVICE, "device ordinal out of range"); return MWBLAS_ERR_DEVICE; }
    double2 *scratch;
    {
        // null before the runtime has initialised a context on this thread; the
        // lookup below initialises it, and the context is read again after it
        void *ctx = current_context();
        std::lock_guard<std::mutex> lk(g_noalloc_mu);
        if (!g_noalloc_addr[dev] || g_noalloc_ctx[dev] != ctx) {
            void *p = nullptr;
            cudaError_t st = cudaGetSymbolAddress(&p, g_gemv_noalloc_scratch);
            if (st != cudaSuccess) {
                g_noalloc_addr[dev] = nullptr;
                cuda_ok(st, routine, "cudaGetSymbolAddress(scratch)");
                return MWBLAS_ERR_CUDA;
            }
            g_noalloc_addr[dev] = (double2 *)p;
            g_noalloc_ctx[dev] = current_context();
        }
        scratch = g_noalloc_addr[dev];
    }
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms <= 0) sms = 148;
    cudaStream_t s = cuda_stream ? (cudaStream_t)cuda_stream : stream();
    if (bk != 1) {
        int64_t blocks = (m + 255) / 256;
        if (blocks > (int64_t)sms * 8) blocks = (int64_t)sms * 8;
        k_scale_vec<<<(unsigned)blocks, 256, 0, s>>>(m, dd::make(be.hi, be.lo), bk, (double2 *)y, incy);
        count_launch();
    }
    if (!alpha0) {
        int64_t rowblocks = (m + 255) / 256;
        int64_t nchunks = (4 * (int64_t)sms + rowblocks - 1) / rowblocks;
        if (nchunks > kNoAllocScratch / m) nchunks = kNoAllocScratch / m;
        if (nchunks > n) nchunks = n;
        if (nchunks < 1) nchunks = 1;
        int64_t chunk = (n + nchunks - 1) / nchunks;
        nchunks = (n + chunk - 1) / chunk;
        dim3 grid((unsigned)rowblocks, (unsigned)nchunks);
        k_gemv_n_partial<<<grid, 256, 0, s>>>(m, n, (const double2 *)a, lda, (const double2 *)x, incx, chunk, scratch);
        int64_t fb = (m + 255) / 256;
        if (fb > (int64_t)sms * 8) fb = (int64_t)sms * 8;
        k_gemv_n_final<<<(unsigned)fb, 256, 0, s>>>(m, (int)nchunks, scratch, dd::make(al.hi, al.lo), (double2 *)y,
                                                     incy);
        count_launch(2);
    }
    cudaError_t st = cudaGetLastError();
    if (st != cudaSuccess) {
        cuda_ok(st, routine, "kernel launch");
        return MWBLAS_ERR_CUDA;
    }
    return 0;
}
