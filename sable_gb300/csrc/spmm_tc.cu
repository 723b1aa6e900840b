// Split-BF16 tensor-core SpMM for the dense blocks (placeholder until the
// tcgen05 kernel lands: returns handled = false so the FP32 path runs).
#include <cuda_runtime.h>
#include "sable.h"
#include "sable_internal.h"
#include "plan_internal.h"

namespace sable {
int spmm_tc_run(sable_plan *p, const float *X, int64_t ldx, float *Y, int64_t ldy, int N, int64_t *cycles,
                void *stream, bool *handled) {
    (void)p; (void)X; (void)ldx; (void)Y; (void)ldy; (void)N; (void)cycles; (void)stream;
    *handled = false;
    return SABLE_OK;
}
void spmm_tc_free(sable_plan *p) { (void)p; }
}  // namespace sable
