// Internal interface of the GEMM engines (device pointers only).
#pragma once
#include <vector>
#include <stdint.h>

#include "l1.h"

namespace mw {

struct HostStage;

struct GemmArgs {
    int64_t m = 0, n = 0, k = 0;
    bool ta = false, tb = false;   // op(X) is a transpose
    bool ca = false, cb = false;   // op(X) conjugates (complex only)
    dd_host alpha{1.0, 0.0}, beta{0.0, 0.0};     // real routines
    cdd_host calpha{{1.0, 0.0}, {0.0, 0.0}};     // complex routines
    cdd_host cbeta{{0.0, 0.0}, {0.0, 0.0}};
    int beta_kind = 0;             // 0: beta == 0 (C not read), 1: beta == 1, 2: general
    const void *A = nullptr;
    int64_t lda = 0;
    const void *B = nullptr;
    int64_t ldb = 0;
    void *C = nullptr;
    int64_t ldc = 0;
    int uplo = 0;                  // output triangle: 0 full, 1 upper (i <= j), 2 lower (i >= j)
    bool herm = false;             // complex: force a real diagonal (HERK)
    HostStage *hs = nullptr;       // operands still being uploaded (Ozaki engine only)
    // The tensor-core engine may size its moduli from the operands' significant
    // width (one readback of two integers). Set by the entry points whose
    // product is the whole call (GEMM, the rank-k family, GEMMTR, SYMM), not by
    // the blocked solvers, whose many internal products would each pay it.
    bool width = false;
};

// Plain FP64 error-free-transform engine.
bool gemm_plain_real(const GemmArgs &g, const char *routine);
bool gemm_plain_cplx(const GemmArgs &g, const char *routine);

// Fixed-point engine on the integer pipes (real only).
bool gemm_fixed_real(const GemmArgs &g, const char *routine);

// Integer-exact tensor-core engine (Ozaki scheme II). Returns false with an
// error recorded on failure.
bool gemm_ozaki_real(const GemmArgs &g, int bits, const char *routine);
bool gemm_ozaki_cplx(const GemmArgs &g, int bits, const char *routine);
// Wait limit of the FP64 engine's TMA pipeline (its own copy of the device word).
void set_plain_wait_limit(uint64_t ns);
int ozaki_last_moduli();

// Grouped products on the tensor cores (instances of mgemm_grouped):
// ozgroup_prepare allocates and uploads everything for a list of real
// products (outside any stream capture); ozgroup_launch enqueues the batched
// exponent scan, residue conversion, one residue GEMM per padding class and
// the batched reconstruction on s (capturable: no host round trip).
struct OzGroupItem {
    const void *A, *B;
    void *C;
    int64_t lda, ldb, ldc, m, n, k;
    bool ta, tb;
    dd_host alpha, beta;
    int beta_kind;
    int pack;   // share a 256 x 256 slot with other small instances (m, n <= 256)
};
struct OzGroupPlan;
OzGroupPlan *ozgroup_create();
void ozgroup_destroy(OzGroupPlan *p);
int64_t ozgroup_count(const OzGroupPlan *p);
bool ozgroup_prepare(OzGroupPlan *p, const std::vector<OzGroupItem> &items, const char *routine);
void ozgroup_launch(OzGroupPlan *p, cudaStream_t s);
int ozaki_last_bits(int operand);   // 0: op(A), 1: op(B)

// C := beta*C over an m x n block (beta_kind 0 writes zeros, 1 is a no-op).
// uplo restricts the update to a triangle (0 full, 1 upper, 2 lower); herm
// applies the HERK rules (real beta, real diagonal; beta == 1 still zeroes
// the diagonal's imaginary part).
void launch_scale_matrix(int64_t m, int64_t n, dd_host beta, int beta_kind, void *C, int64_t ldc, int uplo = 0);
void launch_scale_matrix_c(int64_t m, int64_t n, cdd_host beta, int beta_kind, void *C, int64_t ldc, int uplo = 0,
                           bool herm = false);

// Exponent bounds of the rows / columns of op(X) (X column-major
// rows_x x cols_x; elem2 = 1 real, 2 complex); with `low`, also the binary
// exponent of the lowest set bit in each row / column (0x3f3f3f3f when it
// holds no nonzero finite entry).
void launch_exp_rows_of_op(const void *X, int64_t rows_x, int64_t cols_x, int64_t ld, bool trans, int elem2,
                           int *out, int *low = nullptr);
void launch_exp_cols_of_op(const void *X, int64_t rows_x, int64_t cols_x, int64_t ld, bool trans, int elem2,
                           int *out, int *low = nullptr);

}  // namespace mw
