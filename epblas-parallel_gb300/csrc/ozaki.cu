// Integer-exact tensor-core GEMM engine (placeholder until the sm_103a
// kernels land): reports itself unavailable.
#include "level3.h"
#include "runtime.h"

namespace mw {

static int g_last_moduli = 0;

bool ozaki_available() { return false; }
int ozaki_last_moduli() { return g_last_moduli; }

bool gemm_ozaki_real(const GemmArgs &, int, const char *routine)
{
    set_error(routine, MWBLAS_ERR_UNSUPPORTED, "tensor-core engine not built");
    return false;
}

bool gemm_ozaki_cplx(const GemmArgs &, int, const char *routine)
{
    set_error(routine, MWBLAS_ERR_UNSUPPORTED, "tensor-core engine not built");
    return false;
}

}  // namespace mw
