// Host runtime: errors, streams, device scratch and host<->device staging.
#include "runtime.h"

#include <algorithm>
#include <atomic>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <sched.h>
#include <unistd.h>

// OpenMP queries resolved at run time only if the host process has an OpenMP
// runtime loaded (libgomp, libiomp5, ...). The library itself does not depend
// on one.
extern "C" int omp_get_max_threads(void) __attribute__((weak));
extern "C" int omp_in_parallel(void) __attribute__((weak));

namespace mw {

namespace {

struct ThreadErr {
    int info = 0;
    std::string routine;
    std::string message;
};
thread_local ThreadErr t_err;
thread_local cudaStream_t t_stream = nullptr;   // nullptr = cudaStreamPerThread
thread_local bool t_sync = true;

std::atomic<mwblas_error_hook> g_hook{nullptr};
std::atomic<int64_t> g_fail_alloc_after{-1};
std::atomic<int64_t> g_launches{0};
std::atomic<int64_t> g_l1_team{0};

struct DeviceState {
    bool ready = false;
    int sm_count = 0;
    int *status = nullptr;   // device word for bounded-wait timeouts
};
std::mutex g_dev_mu;
DeviceState g_dev[64];

}  // namespace

void set_error(const char *routine, int info, const std::string &message)
{
    t_err.info = info;
    t_err.routine = routine ? routine : "";
    t_err.message = message;
    mwblas_error_hook h = g_hook.load();
    if (h) h(t_err.routine.c_str(), info, t_err.message.c_str());
}

void clear_error()
{
    t_err.info = 0;
    t_err.routine.clear();
    t_err.message.clear();
}

bool cuda_ok(cudaError_t st, const char *routine, const char *what)
{
    if (st == cudaSuccess) return true;
    std::string msg = std::string(what) + ": " + cudaGetErrorString(st);
    int code = (st == cudaErrorMemoryAllocation) ? MWBLAS_ERR_ALLOC : MWBLAS_ERR_CUDA;
    set_error(routine, code, msg);
    return false;
}

cudaStream_t stream() { return t_stream ? t_stream : cudaStreamPerThread; }
bool sync_on_return() { return t_sync; }

bool ensure_device(const char *routine)
{
    int dev = 0;
    cudaError_t st = cudaGetDevice(&dev);
    if (st != cudaSuccess) {
        set_error(routine, MWBLAS_ERR_DEVICE, std::string("no CUDA device: ") + cudaGetErrorString(st));
        return false;
    }
    if (dev < 0 || dev >= 64) {
        set_error(routine, MWBLAS_ERR_DEVICE, "device ordinal out of range");
        return false;
    }
    DeviceState &ds = g_dev[dev];
    if (ds.ready) return true;
    std::lock_guard<std::mutex> lk(g_dev_mu);
    if (ds.ready) return true;
    cudaDeviceProp prop;
    if (!cuda_ok(cudaGetDeviceProperties(&prop, dev), routine, "cudaGetDeviceProperties")) return false;
    if (prop.major < 10) {
        set_error(routine, MWBLAS_ERR_DEVICE, "libmwblas_gb300 needs an sm_100-class (Blackwell) device");
        return false;
    }
    ds.sm_count = prop.multiProcessorCount;
    // Keep freed scratch cached in the pool instead of returning it to the
    // driver after every synchronising call.
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
        uint64_t thresh = UINT64_MAX;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thresh);
    }
    if (!cuda_ok(cudaMalloc(&ds.status, sizeof(int)), routine, "cudaMalloc(status)")) return false;
    if (!cuda_ok(cudaMemset(ds.status, 0, sizeof(int)), routine, "cudaMemset(status)")) return false;
    ds.ready = true;
    return true;
}

int device_sm_count()
{
    int dev = 0;
    cudaGetDevice(&dev);
    return g_dev[dev].sm_count > 0 ? g_dev[dev].sm_count : 148;
}

int *device_status_word()
{
    int dev = 0;
    cudaGetDevice(&dev);
    return g_dev[dev].status;
}

bool check_device_status(const char *routine)
{
    int *w = device_status_word();
    if (!w) return true;
    int v = 0;
    if (!cuda_ok(cudaMemcpyAsync(&v, w, sizeof(int), cudaMemcpyDeviceToHost, stream()), routine,
                 "status readback"))
        return false;
    if (!cuda_ok(cudaStreamSynchronize(stream()), routine, "status sync")) return false;
    if (v != 0) {
        cudaMemsetAsync(w, 0, sizeof(int), stream());
        set_error(routine, MWBLAS_ERR_TIMEOUT, "a bounded device wait gave up (status " + std::to_string(v) + ")");
        return false;
    }
    return true;
}

void *dev_alloc(size_t bytes, const char *routine)
{
    if (bytes == 0) bytes = 16;
    int64_t left = g_fail_alloc_after.load();
    if (left >= 0) {
        if (left == 0) {
            g_fail_alloc_after.store(-1);
            set_error(routine, MWBLAS_ERR_ALLOC, "device allocation failed (injected by test hook)");
            return nullptr;
        }
        g_fail_alloc_after.store(left - 1);
    }
    void *p = nullptr;
    cudaError_t st = cudaMallocAsync(&p, bytes, stream());
    if (st != cudaSuccess) {
        cudaGetLastError();
        set_error(routine, MWBLAS_ERR_ALLOC,
                  "device allocation of " + std::to_string(bytes) + " bytes failed: " + cudaGetErrorString(st));
        return nullptr;
    }
    return p;
}

void dev_free(void *p)
{
    if (p) cudaFreeAsync(p, stream());
}

bool is_device_pointer(const void *p)
{
    if (!p) return false;
    cudaPointerAttributes attr;
    cudaError_t st = cudaPointerGetAttributes(&attr, p);
    if (st != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return attr.type == cudaMemoryTypeDevice || attr.type == cudaMemoryTypeManaged;
}

bool is_aligned16(const void *p) { return ((uintptr_t)p & 15u) == 0; }

bool is_dd_device_pointer(const void *p) { return is_aligned16(p) && is_device_pointer(p); }

void *tensor_map_encoder()
{
    static void *fn = [] {
        cudaDriverEntryPointQueryResult q;
        void *f = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            f = nullptr;
        cudaGetLastError();
        return f;
    }();
    return fn;
}

// Whether kernels of the current device may read pageable host memory through
// the system's page tables (coherent CPU-GPU systems); per device, cached.
bool device_reads_pageable()
{
    static int cached[64];   // 0 unknown, 1 yes, 2 no
    int dev = 0;
    cudaGetDevice(&dev);
    int &c = cached[dev & 63];
    if (c == 0) {
        int v = 0;
        if (cudaDeviceGetAttribute(&v, cudaDevAttrPageableMemoryAccessUsesHostPageTables, dev) != cudaSuccess) {
            cudaGetLastError();
            v = 0;
        }
        c = v ? 1 : 2;
    }
    return c == 1;
}

namespace {

bool is_pageable_host(const void *p)
{
    cudaPointerAttributes attr;
    if (cudaPointerGetAttributes(&attr, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return attr.type == cudaMemoryTypeUnregistered;
}

// Columns of 16-byte words from pageable host memory into device memory, read
// by the kernel in place. Few blocks: it runs beside the product's kernels
// and only needs enough loads in flight to cover the host link.
__global__ void __launch_bounds__(512) k_copy_from_host(const uint4 *__restrict__ src, int64_t spitch,
                                                        uint4 *__restrict__ dst, int64_t dpitch, int64_t words,
                                                        int64_t cols)
{
    for (int64_t c = blockIdx.y; c < cols; c += gridDim.y) {
        const uint4 *s = src + c * spitch;
        uint4 *d = dst + c * dpitch;
        const int64_t step = (int64_t)gridDim.x * blockDim.x;
        int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
        for (; i + 3 * step < words; i += 4 * step) {
            const uint4 a = s[i], b = s[i + step], e = s[i + 2 * step], f = s[i + 3 * step];
            d[i] = a;
            d[i + step] = b;
            d[i + 2 * step] = e;
            d[i + 3 * step] = f;
        }
        for (; i < words; i += step) d[i] = s[i];
    }
}

// Rows [r0, r1) x columns [c0, c1) of a staged matrix from its pageable host
// array on stream cs; false (nothing queued) when the layout is not in
// 16-byte words.
bool copy_block_from_pageable(Staged &s, int64_t r0, int64_t r1, int64_t c0, int64_t c1, cudaStream_t cs,
                              const char *routine)
{
    const size_t pitch = (size_t)s.ld * s.elem, off = (size_t)c0 * pitch + (size_t)r0 * s.elem;
    const size_t wbytes = (size_t)(r1 - r0) * s.elem;
    if ((((uintptr_t)s.host + off) & 15) || (pitch & 15) || (wbytes & 15)) return false;
    const int64_t words = (int64_t)(wbytes / 16), cols = c1 - c0;
    // 128 blocks at most (2 x 8 gave 34.8 ms per 8192^3 call on pageable arrays,
    // 4 x 32 32.7, 8 x 64 36.2: more blocks take SMs from the product)
    const unsigned gx = (unsigned)std::min<int64_t>(4, (words + 511) / 512);
    const unsigned gy = (unsigned)std::min<int64_t>(cols, 32);
    k_copy_from_host<<<dim3(gx, gy), 512, 0, cs>>>((const uint4 *)((const char *)s.host + off), (int64_t)(pitch / 16),
                                                   (uint4 *)((char *)s.dev + off), (int64_t)(pitch / 16), words,
                                                   cols);
    count_launch();
    return cuda_ok(cudaGetLastError(), routine, "copy kernel launch");
}

}  // namespace

bool stage_matrix(Staged &s, const void *host, int64_t rows, int64_t cols, int64_t ld, size_t elem,
                  bool copy_in, const char *routine)
{
    s = Staged();
    s.host = host;
    s.rows = rows;
    s.cols = cols;
    s.ld = ld;
    s.elem = elem;
    if (rows <= 0 || cols <= 0) return true;
    if (is_dd_device_pointer(host)) {   // used in place; anything else is copied
        s.dev = const_cast<void *>(host);
        return true;
    }
    size_t bytes = (size_t)ld * (size_t)cols * elem;
    s.dev = dev_alloc(bytes, routine);
    if (!s.dev) return false;
    s.owned = true;
    s.pageable = device_reads_pageable() && is_pageable_host(host);
    if (copy_in) {
        if (!cuda_ok(cudaMemcpy2DAsync(s.dev, (size_t)ld * elem, host, (size_t)ld * elem, (size_t)rows * elem,
                                       (size_t)cols, cudaMemcpyDefault, stream()),
                     routine, "copy matrix to device"))
            return false;
    }
    return true;
}

bool unstage_matrix(Staged &s, const char *routine)
{
    if (!s.owned || s.rows <= 0 || s.cols <= 0) return true;
    return cuda_ok(cudaMemcpy2DAsync(const_cast<void *>(s.host), (size_t)s.ld * s.elem, s.dev,
                                     (size_t)s.ld * s.elem, (size_t)s.rows * s.elem, (size_t)s.cols,
                                     cudaMemcpyDefault, stream()),
                   routine, "copy matrix to host");
}

namespace {

// Per-thread copy streams, destroyed with the thread.
struct CopyStreams {
    cudaStream_t s[64] = {};
    ~CopyStreams()
    {
        for (cudaStream_t &x : s)
            if (x) cudaStreamDestroy(x);
    }
};
thread_local CopyStreams t_copy, t_side;

// stream `after` waits for the work queued so far on stream `before`
bool order(cudaStream_t before, cudaStream_t after, const char *routine)
{
    cudaEvent_t e;
    if (!cuda_ok(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), routine, "event create")) return false;
    bool ok = cuda_ok(cudaEventRecord(e, before), routine, "event record") &&
              cuda_ok(cudaStreamWaitEvent(after, e, 0), routine, "stream wait");
    cudaEventDestroy(e);
    return ok;
}

}  // namespace

cudaStream_t side_stream()
{
    int d = 0;
    cudaGetDevice(&d);
    if (d < 0 || d >= 64) d = 0;
    if (!t_side.s[d]) cudaStreamCreateWithFlags(&t_side.s[d], cudaStreamNonBlocking);
    return t_side.s[d];
}

StreamOverride::StreamOverride(cudaStream_t s) : prev(t_stream) { t_stream = s; }
StreamOverride::~StreamOverride() { t_stream = prev; }

bool order_streams(cudaStream_t before, cudaStream_t after, const char *routine)
{
    return order(before, after, routine);
}

cudaStream_t copy_stream()
{
    int d = 0;
    cudaGetDevice(&d);
    if (d < 0 || d >= 64) d = 0;
    if (!t_copy.s[d]) cudaStreamCreateWithFlags(&t_copy.s[d], cudaStreamNonBlocking);
    return t_copy.s[d];
}

bool stage_matrix_async(Staged &s, const void *host, int64_t rows, int64_t cols, int64_t ld, size_t elem,
                        bool copy_in, cudaEvent_t &ready, const char *routine)
{
    ready = nullptr;
    if (!copy_in || rows <= 0 || cols <= 0 || is_dd_device_pointer(host))
        return stage_matrix(s, host, rows, cols, ld, elem, copy_in, routine);
    if (!stage_matrix(s, host, rows, cols, ld, elem, false, routine)) return false;   // allocation only
    cudaStream_t cs = copy_stream();
    if (!cs) {
        set_error(routine, MWBLAS_ERR_CUDA, "copy stream unavailable");
        return false;
    }
    if (!order(stream(), cs, routine)) return false;
    const bool direct = s.pageable && copy_block_from_pageable(s, 0, rows, 0, cols, cs, routine);
    if (!direct && !cuda_ok(cudaMemcpy2DAsync(s.dev, (size_t)ld * elem, host, (size_t)ld * elem,
                                              (size_t)rows * elem, (size_t)cols, cudaMemcpyDefault, cs),
                            routine, "copy matrix to device"))
        return false;
    if (!cuda_ok(cudaEventCreateWithFlags(&ready, cudaEventDisableTiming), routine, "event create")) {
        ready = nullptr;
        return false;
    }
    return cuda_ok(cudaEventRecord(ready, cs), routine, "event record");
}

bool unstage_columns_async(Staged &s, int64_t j0, int64_t j1, const char *routine)
{
    if (!s.owned || s.rows <= 0 || j1 <= j0) return true;
    if (s.pageable) {
        cudaEvent_t e = nullptr;
        if (!cuda_ok(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), routine, "event create")) return false;
        if (!cuda_ok(cudaEventRecord(e, stream()), routine, "event record")) {
            cudaEventDestroy(e);
            return false;
        }
        s.deferred.push_back(Staged::Deferred{j0, j1, e});
        return true;
    }
    cudaStream_t cs = copy_stream();
    if (!order(stream(), cs, routine)) return false;
    const size_t pitch = (size_t)s.ld * s.elem;
    return cuda_ok(cudaMemcpy2DAsync((char *)const_cast<void *>(s.host) + (size_t)j0 * pitch, pitch,
                                     (char *)s.dev + (size_t)j0 * pitch, pitch, (size_t)s.rows * s.elem,
                                     (size_t)(j1 - j0), cudaMemcpyDefault, cs),
                   routine, "copy matrix columns to host");
}

bool flush_columns_back(Staged &s, const char *routine)
{
    bool ok = true;
    cudaStream_t cs = copy_stream();
    const size_t pitch = (size_t)s.ld * s.elem;
    for (Staged::Deferred &d : s.deferred) {
        ok = ok && cuda_ok(cudaStreamWaitEvent(cs, d.after, 0), routine, "stream wait") &&
             cuda_ok(cudaMemcpy2DAsync((char *)const_cast<void *>(s.host) + (size_t)d.j0 * pitch, pitch,
                                       (char *)s.dev + (size_t)d.j0 * pitch, pitch, (size_t)s.rows * s.elem,
                                       (size_t)(d.j1 - d.j0), cudaMemcpyDefault, cs),
                     routine, "copy matrix columns to host");
        cudaEventDestroy(d.after);
    }
    s.deferred.clear();
    return ok;
}

bool wait_event(cudaEvent_t e, const char *routine)
{
    return !e || cuda_ok(cudaStreamWaitEvent(stream(), e, 0), routine, "stream wait");
}

bool join_copy_stream(const char *routine) { return order(copy_stream(), stream(), routine); }

HostStage::~HostStage()
{
    for (cudaEvent_t e : {a_ready, b_ready, c_ready})
        if (e) cudaEventDestroy(e);
    for (cudaEvent_t e : a_block)
        if (e) cudaEventDestroy(e);
    for (cudaEvent_t e : b_block)
        if (e) cudaEventDestroy(e);
    for (cudaEvent_t e : c_block)
        if (e) cudaEventDestroy(e);
}

bool upload_block_async(Staged &s, int64_t r0, int64_t r1, int64_t c0, int64_t c1, cudaEvent_t &ready,
                        const char *routine)
{
    ready = nullptr;
    if (!s.owned || r1 <= r0 || c1 <= c0) return true;
    cudaStream_t cs = copy_stream();
    if (!order(stream(), cs, routine)) return false;
    const size_t pitch = (size_t)s.ld * s.elem, off = (size_t)c0 * pitch + (size_t)r0 * s.elem;
    const bool direct = s.pageable && copy_block_from_pageable(s, r0, r1, c0, c1, cs, routine);
    if (!direct && !cuda_ok(cudaMemcpy2DAsync((char *)s.dev + off, pitch, (const char *)s.host + off, pitch,
                                              (size_t)(r1 - r0) * s.elem, (size_t)(c1 - c0), cudaMemcpyDefault, cs),
                            routine, "copy matrix block to device"))
        return false;
    if (!cuda_ok(cudaEventCreateWithFlags(&ready, cudaEventDisableTiming), routine, "event create")) {
        ready = nullptr;
        return false;
    }
    return cuda_ok(cudaEventRecord(ready, cs), routine, "event record");
}

bool stage_vector(Staged &s, const void *host, int64_t n, int64_t inc, size_t elem, bool copy_in,
                  int64_t &dev_inc, const char *routine)
{
    s = Staged();
    s.host = host;
    s.n = n;
    s.inc = inc;
    s.elem = elem;
    s.is_vector = true;
    dev_inc = inc;
    if (n <= 0) return true;
    if (is_dd_device_pointer(host)) {   // used in place; anything else is copied
        s.dev = const_cast<void *>(host);
        return true;
    }
    int64_t ainc = inc < 0 ? -inc : inc;
    int64_t cnt = (inc == 0) ? 1 : n;
    s.dev = dev_alloc((size_t)cnt * elem, routine);
    if (!s.dev) return false;
    s.owned = true;
    dev_inc = (inc > 0) ? 1 : (inc < 0 ? -1 : 0);
    if (copy_in) {
        bool ok;
        if (ainc <= 1)
            ok = cuda_ok(cudaMemcpyAsync(s.dev, host, (size_t)cnt * elem, cudaMemcpyDefault, stream()),
                         routine, "copy vector to device");
        else
            ok = cuda_ok(cudaMemcpy2DAsync(s.dev, elem, host, (size_t)ainc * elem, elem, (size_t)cnt,
                                           cudaMemcpyDefault, stream()),
                         routine, "copy strided vector to device");
        if (!ok) return false;
    }
    return true;
}

bool unstage_vector(Staged &s, const char *routine)
{
    if (!s.owned || s.n <= 0) return true;
    int64_t ainc = s.inc < 0 ? -s.inc : s.inc;
    int64_t cnt = (s.inc == 0) ? 1 : s.n;
    if (ainc <= 1)
        return cuda_ok(cudaMemcpyAsync(const_cast<void *>(s.host), s.dev, (size_t)cnt * s.elem,
                                       cudaMemcpyDefault, stream()),
                       routine, "copy vector to host");
    return cuda_ok(cudaMemcpy2DAsync(const_cast<void *>(s.host), (size_t)ainc * s.elem, s.dev, s.elem, s.elem,
                                     (size_t)cnt, cudaMemcpyDefault, stream()),
                   routine, "copy strided vector to host");
}

void release(Staged &s)
{
    if (s.owned) dev_free(s.dev);
    s.owned = false;
    s.dev = nullptr;
}

bool finish(const char *routine)
{
    cudaError_t st = cudaGetLastError();
    if (st != cudaSuccess) return cuda_ok(st, routine, "kernel launch");
    if (t_sync || t_stream == nullptr) {
        if (!cuda_ok(cudaStreamSynchronize(stream()), routine, "stream synchronize")) return false;
        return check_device_status(routine);   // cheap after the sync
    }
    return true;
}

static int64_t cpu_count()
{
    cpu_set_t set;
    CPU_ZERO(&set);
    if (sched_getaffinity(0, sizeof(set), &set) == 0) {
        int c = CPU_COUNT(&set);
        if (c > 0) return c;
    }
    long c = sysconf(_SC_NPROCESSORS_ONLN);
    return c > 0 ? c : 1;
}

int64_t l1_team(int64_t n, int64_t omp_min)
{
    if (n <= omp_min) return 1;
    int64_t forced = g_l1_team.load();
    if (forced > 0) return forced;
    if (omp_in_parallel && omp_in_parallel()) return 1;
    int64_t t;
    if (omp_get_max_threads) {
        t = omp_get_max_threads();
    } else {
        t = 0;
        const char *e = getenv("OMP_NUM_THREADS");
        if (e && *e) t = strtoll(e, nullptr, 10);
        if (t <= 0) t = cpu_count();
    }
    return t > 1 ? t : 1;
}

void count_launch(int64_t k) { g_launches.fetch_add(k); }

}  // namespace mw

// ---- exported control API ----------------------------------------------------

extern "C" {

mwblas_error_hook mwblas_set_error_hook(mwblas_error_hook hook) { return mw::g_hook.exchange(hook); }
int mwblas_last_error(void) { return mw::t_err.info; }
const char *mwblas_last_error_message(void) { return mw::t_err.message.c_str(); }
const char *mwblas_last_error_routine(void) { return mw::t_err.routine.c_str(); }
void mwblas_clear_error(void) { mw::clear_error(); }
void mwblas_debug_fail_alloc_after(int64_t count) { mw::g_fail_alloc_after.store(count); }
int64_t mwblas_launch_count(void) { return mw::g_launches.load(); }
int64_t mwblas_set_l1_partition(int64_t team) { return mw::g_l1_team.exchange(team < 0 ? 0 : team); }

int mwblas_pageable_direct(void)
{
    mw::clear_error();
    return mw::ensure_device("mwblas_pageable_direct") && mw::device_reads_pageable() ? 1 : 0;
}

int mwblas_set_stream(void *cuda_stream)
{
    mw::t_stream = (cudaStream_t)cuda_stream;
    return 0;
}

int mwblas_set_sync(int sync)
{
    int prev = mw::t_sync ? 1 : 0;
    mw::t_sync = sync != 0;
    return prev;
}

const char *mwblas_version(void) { return "mwblas_gb300 0.1 (sm_103a)"; }

}  // extern "C"
