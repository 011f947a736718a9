// Entry points declared in include/opflow_gpu.h whose kernels live in later translation units of this
// library; until those are linked these return OPFLOW_E_UNSUPPORTED with a clear message.
#include "internal.h"

extern "C" {
int opflow_batch_create(opflow_ctx, const opflow_problem_desc*, int, const opflow_solve_params*, opflow_batch*) {
    return opg::fail(OPFLOW_E_UNSUPPORTED, "batched solves are not available in this build");
}
int opflow_batch_vectors(opflow_batch, int, double**, double**, size_t*) {
    return opg::fail(OPFLOW_E_UNSUPPORTED, "batched solves are not available in this build");
}
int opflow_batch_solve(opflow_batch, opflow_solve_state*) {
    return opg::fail(OPFLOW_E_UNSUPPORTED, "batched solves are not available in this build");
}
int opflow_batch_destroy(opflow_batch) { return OPFLOW_OK; }
}
