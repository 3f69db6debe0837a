// Host runtime shared by every entry point of libmwblas_gb300.so.
//
// The reference library is a plain synchronous BLAS over host memory with no
// handles and no argument checking (src/epblas-parallel/common/
// epblas_facade.h:1-56). This runtime keeps that calling model: every entry
// point returns with its outputs complete. Around it, it adds what a GPU
// implementation needs:
//   * per-host-thread stream (cudaStreamPerThread unless the caller set one);
//   * stream-ordered device scratch from the device's default memory pool;
//   * staging of host arrays into device memory and back (pointers the
//     caller already has on the device are used in place);
//   * a thread-local last-error record plus an optional error hook, because
//     a GPU call can fail where the CPU reference could not.
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>
#include <string>
#include <vector>

#include "../../include/mwblas_gb300.h"

namespace mw {

// ---- errors ---------------------------------------------------------------

// Records (routine, info, message) as this thread's last error and calls the
// user hook if one is installed. info > 0: position of a bad argument
// (Netlib convention). info < 0: MWBLAS_ERR_* runtime failure.
void set_error(const char *routine, int info, const std::string &message);
void clear_error();

// Checks a CUDA runtime status; on failure records it against `routine` and
// returns false.
bool cuda_ok(cudaError_t st, const char *routine, const char *what);

// ---- context ----------------------------------------------------------------

cudaStream_t stream();
bool sync_on_return();
int device_sm_count();
// Ensures a CUDA device is present and the per-device runtime is set up.
bool ensure_device(const char *routine);

// ---- device memory ----------------------------------------------------------

// Stream-ordered allocation from the current device's pool. Returns nullptr
// and records MWBLAS_ERR_ALLOC on failure (also when the allocation-failure
// test hook fires).
void *dev_alloc(size_t bytes, const char *routine);
void dev_free(void *p);

// True when the pointer is device or managed memory that kernels may use.
bool is_device_pointer(const void *p);
bool is_aligned16(const void *p);
// Device (or managed) memory at a 16-byte boundary: an array of double-double
// elements that the kernels may read in place with 16-byte loads.
bool is_dd_device_pointer(const void *p);

// The driver's cuTensorMapEncodeTiled (looked up once through the runtime's
// entry-point query; null when unavailable), as an untyped pointer so that
// this header needs no driver types.
void *tensor_map_encoder();

// A device view of a caller array. If the caller's pointer is already device
// memory it is used in place; otherwise a scratch copy is made.
struct Staged {
    void *dev = nullptr;       // device address kernels use
    const void *host = nullptr;
    bool owned = false;        // scratch allocated by us
    size_t elem = 0;
    int64_t rows = 0, cols = 0, ld = 0;   // matrix shape (column-major)
    int64_t n = 0, inc = 0;               // vector shape
    bool is_vector = false;
    // Pageable host memory that the device reads in place (system page
    // tables): uploads run as copy kernels, which never block the host,
    // and the column copies back are queued once the product is enqueued.
    bool pageable = false;
    struct Deferred {
        int64_t j0, j1;
        cudaEvent_t after;
    };
    std::vector<Deferred> deferred;
};

// Matrix rows x cols with leading dimension ld (elements of `elem` bytes).
// copy_in=false allocates without copying (pure outputs).
bool stage_matrix(Staged &s, const void *host, int64_t rows, int64_t cols, int64_t ld,
                  size_t elem, bool copy_in, const char *routine);
// Writes a staged matrix back (only the rows x cols block; padding rows of the
// caller's array are never written).
bool unstage_matrix(Staged &s, const char *routine);

// ---- copies that overlap the kernels -------------------------------------------
// A second stream of the calling thread for host<->device copies (one per
// device, created on first use).
cudaStream_t copy_stream();
// stage_matrix with the copy to the device queued on copy_stream() (after the
// allocation on stream()); `ready`, recorded on copy_stream(), marks its end.
// Device memory used in place, copy_in=false or an empty matrix give no event.
bool stage_matrix_async(Staged &s, const void *host, int64_t rows, int64_t cols, int64_t ld, size_t elem,
                        bool copy_in, cudaEvent_t &ready, const char *routine);
// Queues the copy of columns [j0, j1) of a staged matrix back to the caller's
// array on copy_stream(), after the work queued so far on stream(). For
// pageable host memory (a copy to it returns only when done) the copy is
// noted and queued by flush_columns_back.
bool unstage_columns_async(Staged &s, int64_t j0, int64_t j1, const char *routine);
// Queues the noted copies back, in order (each returns once its columns are
// on the host; the kernels queued before keep the device busy meanwhile).
bool flush_columns_back(Staged &s, const char *routine);
// Whether kernels of the current device read pageable host memory through the
// system page tables (then uploads from pageable arrays run as copy kernels).
bool device_reads_pageable();
// A third per-thread stream, for kernels that run beside those of stream()
// (created on first use, per device).
cudaStream_t side_stream();
// Makes stream() return `s` on this thread until the scope ends.
struct StreamOverride {
    cudaStream_t prev;
    explicit StreamOverride(cudaStream_t s);
    ~StreamOverride();
};
// stream `after` waits for the work queued so far on stream `before`.
bool order_streams(cudaStream_t before, cudaStream_t after, const char *routine);
// stream() waits for `e` (nullptr: nothing to wait for).
bool wait_event(cudaEvent_t e, const char *routine);
// stream() waits for everything queued so far on copy_stream().
bool join_copy_stream(const char *routine);

// Host operands of one call whose uploads run on copy_stream(). An engine that
// understands it waits on each event just before it first reads that operand,
// and may write C back itself in column chunks behind its own kernels.
// With block_cols > 0, op(B) and C arrive instead in blocks of that many
// columns (block j: columns [j * block_cols, ...)), one event per block, so
// that the product of block j can start when its columns are in; with
// a_rows > 0 (only together with column blocks), op(A) arrives in blocks of
// that many rows, and the first `early_blocks` column blocks (uploaded right
// after A's first row block) are multiplied row block by row block while the
// rest of A is still on its way.
struct HostStage {
    cudaEvent_t a_ready = nullptr, b_ready = nullptr, c_ready = nullptr;
    int64_t block_cols = 0, a_rows = 0, early_blocks = 0;
    std::vector<cudaEvent_t> a_block, b_block, c_block;
    Staged *c = nullptr;       // the staged C (target of the write-back)
    bool c_written = false;    // the engine has queued C's copy back and joined
    bool wait_all(const char *routine) const
    {
        bool ok = wait_event(a_ready, routine) && wait_event(b_ready, routine) && wait_event(c_ready, routine);
        for (cudaEvent_t e : a_block) ok = ok && wait_event(e, routine);
        for (cudaEvent_t e : b_block) ok = ok && wait_event(e, routine);
        for (cudaEvent_t e : c_block) ok = ok && wait_event(e, routine);
        return ok;
    }
    ~HostStage();
};
// Queues the copy of rows [r0, r1) x columns [c0, c1) of the caller's matrix
// into a staged (allocated) matrix on copy_stream(); `ready` marks its end.
bool upload_block_async(Staged &s, int64_t r0, int64_t r1, int64_t c0, int64_t c1, cudaEvent_t &ready,
                        const char *routine);

// Vector of n logical elements with increment inc (BLAS convention: a
// negative increment starts at the far end). A staged host vector is
// compacted; the device increment is returned in `dev_inc` (+1, -1 or 0).
bool stage_vector(Staged &s, const void *host, int64_t n, int64_t inc, size_t elem,
                  bool copy_in, int64_t &dev_inc, const char *routine);
bool unstage_vector(Staged &s, const char *routine);

void release(Staged &s);

// Synchronises the library stream when the call is synchronous; records any
// asynchronous error against `routine`.
bool finish(const char *routine);

// ---- reference threading policy --------------------------------------------

// Team size the reference would use for a threaded level-1 sweep of n
// elements with threshold `omp_min` (the *_OMP_MIN constants of the reference
// L1 files). Reproduces blas_omp_should_thread() (common/blas_omp.h:59-65):
// 1 when n <= omp_min, when the OpenMP runtime reports a single thread, or
// when the caller is already inside a parallel region. A value set through
// mwblas_set_l1_partition() overrides the runtime query.
int64_t l1_team(int64_t n, int64_t omp_min);

// ---- launch bookkeeping -----------------------------------------------------

// Counts kernel launches issued by the library (for benchmarking claims).
void count_launch(int64_t k = 1);

// Device-side status word that bounded device waits write to on timeout.
int *device_status_word();
bool check_device_status(const char *routine);

}  // namespace mw
