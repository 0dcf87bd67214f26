// Placeholder entry points for batched runs and serving until their kernels land.
#include "dispatch.h"

extern "C" {
struct stc_batch { int unused; };
struct stc_server { int unused; };
int stc_batch_create(stc_batch**) { return STC_ERR_UNSUPPORTED; }
int stc_batch_destroy(stc_batch*) { return STC_ERR_UNSUPPORTED; }
int stc_batch_add(stc_batch*, const stc_grid*, const stc_grid*, const stc_stencil*, const stc_op*, const stc_bc*, int64_t) { return STC_ERR_UNSUPPORTED; }
int stc_batch_plan(stc_batch*, int32_t, void*) { return STC_ERR_UNSUPPORTED; }
int stc_batch_run(stc_batch*, void*, uint32_t) { return STC_ERR_UNSUPPORTED; }
int stc_batch_result(const stc_batch*, int32_t, int32_t*) { return STC_ERR_UNSUPPORTED; }
int stc_batch_run_sequential(stc_batch*, void*) { return STC_ERR_UNSUPPORTED; }
int stc_server_create(stc_server**, double, int32_t) { return STC_ERR_UNSUPPORTED; }
int stc_server_destroy(stc_server*) { return STC_ERR_UNSUPPORTED; }
int stc_server_submit(stc_server*, const stc_job*, int64_t*) { return STC_ERR_UNSUPPORTED; }
int stc_server_poll(stc_server*, int64_t) { return STC_ERR_UNSUPPORTED; }
int stc_server_fetch(stc_server*, int64_t, void*, size_t, double*) { return STC_ERR_UNSUPPORTED; }
int stc_server_cancel(stc_server*, int64_t) { return STC_ERR_UNSUPPORTED; }
int stc_server_drain(stc_server*, double) { return STC_ERR_UNSUPPORTED; }
int stc_server_stats(const stc_server*, int64_t*, int64_t*, int64_t*, int64_t*) { return STC_ERR_UNSUPPORTED; }
}
