// Implicit-path entry points not yet linked in this build (see pending.cu).
#include "internal.h"

extern "C" {
void opflow_solve_params_default(opflow_solve_params* p) {
    if (!p) return;
    p->tol = 1e-10;
    p->max_iter = 200;
    p->static_mat = 0;
    p->pin_value = 0;
    p->precision = OPFLOW_PREC_FP64;
    p->pre_sweeps = 2;
    p->post_sweeps = 2;
    p->coarse_max = 512;
    p->zero_guess = 0;
}
int opflow_assemble(opflow_ctx, opflow_field, const opflow_node*, int, const opflow_field*, int, int, int, int*, int*, double*, double*,
                    size_t*) {
    return opg::fail(OPFLOW_E_UNSUPPORTED, "assembly is not available in this build");
}
int opflow_solver_create(opflow_ctx, opflow_field, const opflow_node*, int, const opflow_field*, int, int, const opflow_solve_params*,
                         opflow_solver*) {
    return opg::fail(OPFLOW_E_UNSUPPORTED, "solvers are not available in this build");
}
int opflow_solver_solve(opflow_solver, opflow_solve_state*) { return opg::fail(OPFLOW_E_UNSUPPORTED, "solvers are not available in this build"); }
int opflow_solver_destroy(opflow_solver) { return OPFLOW_OK; }
int opflow_weno_rk3(opflow_ctx, opflow_field, opflow_field, opflow_field, int, int, double, int) {
    return opg::fail(OPFLOW_E_UNSUPPORTED, "fused WENO-RK3 is not available in this build");
}
}
