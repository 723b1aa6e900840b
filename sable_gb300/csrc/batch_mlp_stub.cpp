// Temporary stubs for the batch and block-model entry points.
#include "sable.h"
#include "plan_internal.h"
using namespace sable;
extern "C" {
int sable_batch_create(sable_plan *const *, int32_t, const int32_t *, const sable_batch_opts *, sable_batch **) { return fail(SABLE_ERR_UNSUPPORTED, "batch not built"); }
int sable_batch_run(sable_batch *, const float *const *, float *const *, void *) { return fail(SABLE_ERR_UNSUPPORTED, "batch not built"); }
int sable_batch_destroy(sable_batch *) { return SABLE_OK; }
int sable_mlp_create(sable_mlp **) { return fail(SABLE_ERR_UNSUPPORTED, "mlp not built"); }
int sable_mlp_destroy(sable_mlp *) { return SABLE_OK; }
int sable_mlp_set_params(sable_mlp *, const float *) { return SABLE_ERR_UNSUPPORTED; }
int sable_mlp_get_params(const sable_mlp *, float *) { return SABLE_ERR_UNSUPPORTED; }
int sable_mlp_set_norm(sable_mlp *, const float *, const float *) { return SABLE_ERR_UNSUPPORTED; }
int sable_mlp_infer(sable_mlp *, const float *, int32_t, float *, void *) { return SABLE_ERR_UNSUPPORTED; }
int sable_mlp_loss_grad(sable_mlp *, const float *, const float *, int32_t, float *, float *, void *) { return SABLE_ERR_UNSUPPORTED; }
int sable_mlp_train_step(sable_mlp *, const float *, const float *, int32_t, float, float *, void *) { return SABLE_ERR_UNSUPPORTED; }
}
