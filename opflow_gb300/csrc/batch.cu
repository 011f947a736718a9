// Batched solves of many independent problems of uneven sizes: every multigrid operation and every
// Krylov step of the whole batch is one persistent launch over a per-problem chunk (tile) list, and one
// iteration of the batch is recorded once into a CUDA graph and replayed (solver.cu).  Each problem is
//   alpha*u - beta*Lap(u) = f
// written as the OpFlow equation `alpha*e - beta*(d2x(e) + d2y(e) [+ d2z(e)]) == f` and assembled
// with the same StencilPad semantics as a single solve.
#include "solver.h"

#include <chrono>
#include <cmath>

namespace opg {

// alpha*e - beta*(d2<0>(e) + ... ) - f, slots: 0 = e (the unknown), 1 = f
std::vector<opflow_node> helmholtz_tree(int ndim, double alpha, double beta) {
    std::vector<opflow_node> t;
    auto add = [&](int kind, int a, int b, int dim, int field, double v) {
        opflow_node n{kind, a, b, dim, field, v};
        t.push_back(n);
        return (int) t.size() - 1;
    };
    const int ca = add(OPFLOW_NODE_CONST, -1, -1, 0, 0, alpha);
    const int e0 = add(OPFLOW_NODE_FIELD, -1, -1, 0, 0, 0.);
    const int ae = add(OPFLOW_NODE_MUL, ca, e0, 0, 0, 0.);
    int sum = -1;
    for (int d = 0; d < ndim; ++d) {
        const int ed = add(OPFLOW_NODE_FIELD, -1, -1, 0, 0, 0.);
        const int dd = add(OPFLOW_NODE_D2, ed, -1, d, 0, 0.);
        sum = sum < 0 ? dd : add(OPFLOW_NODE_ADD, sum, dd, 0, 0, 0.);
    }
    const int cb = add(OPFLOW_NODE_CONST, -1, -1, 0, 0, beta);
    const int bl = add(OPFLOW_NODE_MUL, cb, sum, 0, 0, 0.);
    const int lhs = add(OPFLOW_NODE_SUB, ae, bl, 0, 0, 0.);
    const int f = add(OPFLOW_NODE_FIELD, -1, -1, 0, 1, 0.);
    add(OPFLOW_NODE_SUB, lhs, f, 0, 0, 0.);
    return t;
}

int batch_problem_fields(opflow_ctx ctx, const opflow_problem_desc& pd, opflow_field* tgt, opflow_field* rhs);

}  // namespace opg

using namespace opg;

struct opflow_batch_s {
    opflow_ctx ctx;
    MGSystem* S = nullptr;
    std::vector<opflow_field> fields;  // targets and right-hand-side fields (owned: problem batches only)
    opflow_solve_params params;
    // equation batches: per problem, whether it is pinned (singular, no Dirichlet side, pin_value)
    std::vector<char> pinned;
};

int opg::batch_problem_fields(opflow_ctx ctx, const opflow_problem_desc& pd, opflow_field* tgt, opflow_field* rhs) {
    if (pd.ndim < 1 || pd.ndim > 3) return fail(OPFLOW_E_INVALID, "problem dimension %d", pd.ndim);
    if (pd.bc != OPFLOW_BC_DIRC && pd.bc != OPFLOW_BC_NEUM) return fail(OPFLOW_E_INVALID, "problem bc must be Dirichlet or Neumann");
    std::vector<double> xs[3], dxs[3];
    opflow_mesh_desc m{};
    m.ndim = pd.ndim;
    m.pad_width = 2;
    for (int d = 0; d < pd.ndim; ++d) {
        if (pd.n[d] < 3 || !(pd.h[d] > 0)) return fail(OPFLOW_E_INVALID, "problem extent / spacing");
        const int nodes = pd.loc == OPFLOW_CENTER ? pd.n[d] + 1 : pd.n[d];
        xs[d].resize(nodes + 4);
        dxs[d].resize(nodes + 3);
        opflow_mesh_uniform(nodes, 0, 2, 0.0, pd.h[d] * (nodes - 1), xs[d].data(), dxs[d].data());
        m.dims[d] = nodes;
        m.x[d] = xs[d].data();
        m.dx[d] = dxs[d].data();
    }
    opflow_field_desc fd{};
    fd.ndim = pd.ndim;
    for (int d = 0; d < pd.ndim; ++d) {
        fd.loc[d] = pd.loc;
        for (int s = 0; s < 2; ++s) {
            fd.bc_type[d][s] = pd.bc;
            fd.bc_value[d][s] = 0.;
            fd.ext[d][s] = (pd.loc == OPFLOW_CENTER || pd.bc == OPFLOW_BC_NEUM) ? 1 : 0;
        }
    }
    OPG_TRY(opflow_field_create(ctx, &m, &fd, tgt));
    int rc = opflow_field_create(ctx, &m, &fd, rhs);
    if (rc) { opflow_field_destroy(*tgt); return rc; }
    return OPFLOW_OK;
}

static MGSystem* new_batch_system(opflow_batch_s* B) {
    B->S = new MGSystem();
    MGSystem* S = B->S;
    S->ctx = B->ctx;
    S->arena.ctx = B->ctx;
    S->precision = B->params.precision;
    S->pre = B->params.pre_sweeps;
    S->post = B->params.post_sweeps;
    S->coarse_max = B->params.coarse_max > 0 ? B->params.coarse_max : 64;
    S->tol = B->params.tol;
    S->max_iter = B->params.max_iter;
    return S;
}

extern "C" {

int opflow_batch_create(opflow_ctx ctx, const opflow_problem_desc* problems, int n_problems, const opflow_solve_params* params, opflow_batch* out) {
    if (!ctx || !problems || n_problems <= 0 || !out) return fail(OPFLOW_E_INVALID, "bad batch arguments");
    auto* B = new opflow_batch_s();
    B->ctx = ctx;
    if (params) B->params = *params;
    else opflow_solve_params_default(&B->params);
    MGSystem* S = new_batch_system(B);
    int rc = OPFLOW_OK;
    for (int p = 0; p < n_problems && rc == OPFLOW_OK; ++p) {
        opflow_field t = nullptr, f = nullptr;
        rc = batch_problem_fields(ctx, problems[p], &t, &f);
        if (rc) break;
        B->fields.push_back(t);
        B->fields.push_back(f);
        std::vector<opflow_node> tree = helmholtz_tree(problems[p].ndim, problems[p].alpha, problems[p].beta);
        opflow_field leaves[2] = {t, f};
        rc = mg_add_problem(S, t, tree.data(), (int) tree.size(), leaves, 2, 0);
    }
    if (rc == OPFLOW_OK) rc = mg_finalize(S);
    if (rc) {
        opflow_batch_destroy(B);
        return rc;
    }
    *out = B;
    return OPFLOW_OK;
}

int opflow_batch_create_eqns(opflow_ctx ctx, const opflow_equation* eqns, int n_eqns, const opflow_solve_params* params, opflow_batch* out) {
    if (!ctx || !eqns || n_eqns <= 0 || !out) return fail(OPFLOW_E_INVALID, "bad batch arguments");
    for (int p = 0; p < n_eqns; ++p) {
        const opflow_equation& e = eqns[p];
        if (!e.nodes || e.n_nodes <= 0 || !e.leaves || e.n_leaves <= 0 || e.unknown < 0 || e.unknown >= e.n_leaves)
            return fail(OPFLOW_E_INVALID, "bad equation %d", p);
        for (int i = 0; i < e.n_leaves; ++i)
            if (!e.leaves[i]) return fail(OPFLOW_E_INVALID, "equation %d: null leaf %d", p, i);
    }
    auto* B = new opflow_batch_s();
    B->ctx = ctx;
    if (params) B->params = *params;
    else opflow_solve_params_default(&B->params);
    MGSystem* S = new_batch_system(B);
    int rc = OPFLOW_OK;
    for (int p = 0; p < n_eqns && rc == OPFLOW_OK; ++p)
        rc = mg_add_problem(S, eqns[p].leaves[eqns[p].unknown], eqns[p].nodes, eqns[p].n_nodes, eqns[p].leaves, eqns[p].n_leaves, eqns[p].unknown);
    if (rc == OPFLOW_OK) rc = mg_finalize(S);
    // initial guesses: the targets' values (initx); singular problems pinned or projected
    for (int p = 0; p < n_eqns && rc == OPFLOW_OK; ++p) {
        ProblemHost& P = S->probs[p];
        rc = mg_gather_target(ctx, P.target, S->kd_host[p].x);
        const bool sing = P.singular && !P.has_dirichlet;
        B->pinned.push_back(sing && B->params.pin_value);
        if (rc == OPFLOW_OK && sing && !B->params.pin_value) {
            const long long N = P.levels[0].N;
            mg_add_scalar(ctx, P.b, N, -mg_sum(ctx, P.b, N) / (double) N);
        }
    }
    if (rc == OPFLOW_OK) rc = cudaStreamSynchronize(ctx->stream) == cudaSuccess ? OPFLOW_OK : fail(OPFLOW_E_CUDA, "batch set-up");
    if (rc) {
        opflow_batch_destroy(B);
        return rc;
    }
    *out = B;
    return OPFLOW_OK;
}

int opflow_batch_vectors(opflow_batch b, int i, double** x, double** f, size_t* n) {
    if (!b || i < 0 || i >= (int) b->S->probs.size()) return fail(OPFLOW_E_INVALID, "bad problem index");
    if (x) *x = b->S->kd_host[i].x;
    if (f) *f = b->S->probs[i].b;
    if (n) *n = (size_t) b->S->probs[i].levels[0].N;
    return OPFLOW_OK;
}

int opflow_batch_set(opflow_batch b, int i, const double* f, const double* x0, size_t n) {
    if (!b || i < 0 || i >= (int) b->S->probs.size() || !f) return fail(OPFLOW_E_INVALID, "bad batch_set arguments");
    const size_t N = (size_t) b->S->probs[i].levels[0].N;
    if (n != N) return fail(OPFLOW_E_INVALID, "problem %d has %zu unknowns, got %zu", i, N, n);
    OPG_CUDA(cudaMemcpyAsync(b->S->probs[i].b, f, N * 8, cudaMemcpyHostToDevice, b->ctx->stream));
    if (x0) OPG_CUDA(cudaMemcpyAsync(b->S->kd_host[i].x, x0, N * 8, cudaMemcpyHostToDevice, b->ctx->stream));
    OPG_CUDA(cudaStreamSynchronize(b->ctx->stream));
    return OPFLOW_OK;
}

int opflow_batch_get(opflow_batch b, int i, double* x, size_t n) {
    if (!b || i < 0 || i >= (int) b->S->probs.size() || !x) return fail(OPFLOW_E_INVALID, "bad batch_get arguments");
    const size_t N = (size_t) b->S->probs[i].levels[0].N;
    if (n != N) return fail(OPFLOW_E_INVALID, "problem %d has %zu unknowns, got %zu", i, N, n);
    OPG_CUDA(cudaMemcpyAsync(x, b->S->kd_host[i].x, N * 8, cudaMemcpyDeviceToHost, b->ctx->stream));
    OPG_CUDA(cudaStreamSynchronize(b->ctx->stream));
    return OPFLOW_OK;
}

int opflow_batch_solve(opflow_batch b, opflow_solve_state* states) {
    if (!b) return fail(OPFLOW_E_INVALID, "null batch");
    MGSystem* S = b->S;
    opflow_ctx ctx = b->ctx;
    auto t0 = std::chrono::steady_clock::now();
    if (b->params.zero_guess) OPG_TRY(kr_launch_zero_x(ctx->stream, ctx->num_sms, S->dL, S->dK, S->dk0, S->nk0));
    // pinned problems (equation batches): the singular system with b[0] := -(sum of the others), then
    // the shift that makes the pinned unknown 0, and b[0] restored (as opflow_solver_solve does)
    const int np0 = (int) S->probs.size();
    std::vector<double> b_pin(np0, 0.);
    for (int p = 0; p < (int) b->pinned.size(); ++p) {
        if (!b->pinned[p]) continue;
        ProblemHost& P = S->probs[p];
        const long long N = P.levels[0].N;
        const double sb = mg_sum(ctx, P.b, N);
        OPG_CUDA(cudaMemcpy(&b_pin[p], P.b, 8, cudaMemcpyDeviceToHost));
        const double nb0 = -(sb - b_pin[p]);
        OPG_CUDA(cudaMemcpy(P.b, &nb0, 8, cudaMemcpyHostToDevice));
    }
    OPG_TRY(mg_solve(S));
    std::vector<Scal> st;
    OPG_TRY(mg_states(S, st));
    for (int p = 0; p < (int) b->pinned.size(); ++p) {
        if (!b->pinned[p]) continue;
        ProblemHost& P = S->probs[p];
        const long long N = P.levels[0].N;
        double shift = 0.;
        OPG_CUDA(cudaMemcpy(&shift, S->kd_host[p].x, 8, cudaMemcpyDeviceToHost));
        mg_add_scalar(ctx, S->kd_host[p].x, N, -shift);
        OPG_CUDA(cudaMemcpy(P.b, &b_pin[p], 8, cudaMemcpyHostToDevice));
    }
    // true residuals of every problem
    const int np = (int) S->probs.size();
    OPG_TRY(kr_launch_apply(ctx->stream, ctx->num_sms, S->dL, S->dK, S->dk0, S->nk0, nullptr, S->partial, 0));
    OPG_TRY(kr_launch_reduce(ctx->stream, ctx->num_sms, S->partial, S->dfirst, S->dcount, np, S->red));
    std::vector<double> red(2 * np);
    OPG_CUDA(cudaMemcpyAsync(red.data(), S->red, red.size() * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    OPG_CUDA(cudaStreamSynchronize(ctx->stream));
    auto t1 = std::chrono::steady_clock::now();
    int all = 1;
    for (int p = 0; p < np; ++p) {
        double bb = red[2 * p], rr = red[2 * p + 1];
        if (p < (int) b->pinned.size() && b->pinned[p]) {
            // a pinned problem's true residual in the singular operator is O(||b||) in its pinned row:
            // its convergence is the flexible PCG's own residual of the pinned system
            bb = st[p].bb;
            rr = st[p].rr;
        }
        const double rel = bb > 0 ? std::sqrt(rr / bb) : std::sqrt(rr);
        if (states) {
            states[p].iterations = st[p].iters;
            states[p].abs_residual = std::sqrt(rr);
            states[p].rel_residual = rel;
            states[p].converged = rel <= S->tol;
            states[p].setup_ms = 0.;
            states[p].solve_ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
        }
        all &= rel <= S->tol;
    }
    return all ? OPFLOW_OK : fail(OPFLOW_E_NOT_CONVERGED, "some problems of the batch did not reach the tolerance");
}

int opflow_batch_destroy(opflow_batch b) {
    if (!b) return OPFLOW_OK;
    if (b->S) mg_destroy(b->S);
    for (auto f : b->fields) opflow_field_destroy(f);
    delete b;
    return OPFLOW_OK;
}

}  // extern "C"
