// Temporary stubs for the batch entry points.
#include "sable.h"
#include "plan_internal.h"
using namespace sable;
extern "C" {
int sable_batch_create(sable_plan *const *, int32_t, const int32_t *, const sable_batch_opts *, sable_batch **) { return fail(SABLE_ERR_UNSUPPORTED, "batch not built"); }
int sable_batch_run(sable_batch *, const float *const *, float *const *, void *) { return fail(SABLE_ERR_UNSUPPORTED, "batch not built"); }
int sable_batch_destroy(sable_batch *) { return SABLE_OK; }
}
