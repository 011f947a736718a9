// Entry point declared in include/opflow_gpu.h whose kernel lives in a later translation unit of this
// library; until it is linked it returns OPFLOW_E_UNSUPPORTED with a clear message.
#include "internal.h"

extern "C" {
int opflow_weno_rk3(opflow_ctx, opflow_field, opflow_field, opflow_field, int, int, double, int) {
    return opg::fail(OPFLOW_E_UNSUPPORTED, "fused WENO-RK3 is not available in this build");
}
}
