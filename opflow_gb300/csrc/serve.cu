// Request server: continuous batching of independent solves and stateful heat sessions.
//
// Every admitted request owns a resident single-problem system (its multigrid hierarchy, Krylov
// vectors and fields, in its own arena).  The worker thread composes the active requests into one
// batch table (mg_compose) and replays one recorded flexible-PCG iteration for all of them; a request
// joins at the next iteration boundary (seeded so that its first batched iteration only forms
// z = M r and p = z) and leaves as soon as it converges, so requests of different sizes that arrive at
// different times share every launch while they overlap.  A heat session restarts in place after each
// step (b := x, no recomposition).  Admission is bounded by an HBM budget and a batch size.
//
// Two threads: the admission thread builds each admitted request's system (host-side hierarchy,
// uploads, the seed) on a stream of its own and hands it over ready; the worker only composes and
// iterates, so set-up overlaps the batched iterations instead of stalling them.
#include "solver.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <deque>
#include <mutex>
#include <thread>
#include <unordered_map>

namespace opg {

using Clock = std::chrono::steady_clock;

std::vector<opflow_node> helmholtz_tree(int ndim, double alpha, double beta);
int batch_problem_fields(opflow_ctx ctx, const opflow_problem_desc& pd, opflow_field* tgt, opflow_field* rhs);

struct Req {
    long long id = 0;
    opflow_problem_desc pd{};
    // a user equation (opflow_request.equation): the tree, the caller's fields and the unknown's slot
    bool eqn = false;
    std::vector<opflow_node> nodes;
    std::vector<opflow_field> leaves;
    int unknown = 0;
    size_t est = 0;  // the HBM estimate charged at admission
    int steps = 1;
    const double* f = nullptr;  // the caller's right-hand side, read at admission
    bool f_dev = false;         // f is device memory: checked for non-finite values on the device at admission
    const double* x0 = nullptr;  // the caller's initial guess (or null), read at admission
    long long nf = 0;
    double* x_out = nullptr;
    double* ckpt_out = nullptr;  // a requested checkpoint's buffer
    int ckpt_state = 0;          // 0 none, 1 requested, 2 written (steps in ckpt_steps)
    int ckpt_steps = 0;
    Clock::time_point t_submit, t_admit, t_done;
    MGSystem* sys = nullptr;
    opflow_field t = nullptr, rhs = nullptr;
    size_t bytes = 0;
    size_t admitted_bytes = 0;  // the estimate charged against the budget at admission
    int steps_done = 0;
    int iters = 0;
    double rel = 0.;
    int status = OPFLOW_OK;
    bool pinned = false;
    bool done = false;
    long long N = 0;
    Scal seed{};  // the Krylov scalars after set-up
};

static size_t estimate_bytes(const opflow_problem_desc& pd) {
    double n = 1.;
    for (int d = 0; d < pd.ndim; ++d) n *= (double) (pd.n[d] + 2);
    return (size_t) (n * 240.0) + (8u << 20);
}

// a user equation also keeps float64 and float32 coefficient arrays on every level
static size_t estimate_bytes_eqn(long long cells) { return (size_t) ((double) cells * 420.0) + (8u << 20); }

}  // namespace opg

using namespace opg;

struct opflow_server_s {
    opflow_ctx_s own_ctx;    // the worker's stream and scratch on the caller's device
    opflow_ctx_s setup_ctx;  // the admission thread's
    opflow_solve_params params;
    size_t budget = 0, used = 0;
    int max_active = 64;
    std::thread worker, admitter;
    std::mutex mu;
    std::condition_variable cv, cv_done, cv_admit;
    std::deque<Req*> pending;
    std::deque<Req*> ready;  // set up, joining at the worker's next iteration boundary
    int resident = 0;        // admitted and not finished (in set-up, ready or active)
    int in_setup = 0;
    std::vector<Req*> active;
    std::unordered_map<long long, Req*> reqs;
    bool stop = false;
    long long next_id = 1;
    MGSystem comp;
    double* d_slots = nullptr;  // one float64 per request finishing at a boundary (pinned-shift values)
    bool dirty = true;
    std::vector<Scal> state;  // per active request, host copy
    // stats
    std::vector<double> lat;
    long long submitted = 0, completed = 0, solves = 0, compositions = 0;
    double setup_s = 0, compose_s = 0, iterate_s = 0, retire_s = 0;  // worker wall time per phase
    int max_active_seen = 0;
    Clock::time_point t_first, t_last;
    bool have_first = false;
    std::string error;
};

static void release_req(Req* r) {
    if (r->sys) { mg_destroy(r->sys); r->sys = nullptr; }
    if (r->t) { opflow_field_destroy(r->t); r->t = nullptr; }
    if (r->rhs) { opflow_field_destroy(r->rhs); r->rhs = nullptr; }
}

// flag = 1 when any of the n values is not finite (every offending thread writes the same 1)
__global__ void flag_nonfinite(const double* __restrict__ v, long long n, int* flag) {
    for (long long i = (long long) blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long) gridDim.x * blockDim.x)
        if (!isfinite(v[i])) *flag = 1;
}

// hierarchy, right-hand side, pinning, and the seed of the Krylov scalars
static int setup_req(opflow_server S, Req* r, Scal* seed) {
    opflow_ctx ctx = &S->setup_ctx;
    if (!r->eqn) OPG_TRY(batch_problem_fields(ctx, r->pd, &r->t, &r->rhs));
    r->sys = new MGSystem();
    MGSystem* M = r->sys;
    M->ctx = ctx;
    M->arena.ctx = ctx;
    M->precision = S->params.precision;
    M->pre = S->params.pre_sweeps;
    M->post = S->params.post_sweeps;
    M->coarse_max = S->params.coarse_max > 0 ? S->params.coarse_max : 64;
    M->tol = S->params.tol;
    M->max_iter = S->params.max_iter;
    M->arena.block_hint = 4u << 20;
    // requests take the tuner's cached choices (from earlier solves of the shape or a cache file): timing
    // here would add to the request's latency and run beside the batch, which would skew it
    M->tune_measure = false;
    if (r->eqn) {
        // the caller's equation, assembled from its fields (generateAb); the fields are only read here
        const opflow_field target = r->leaves[r->unknown];
        OPG_TRY(mg_add_problem(M, target, r->nodes.data(), (int) r->nodes.size(), r->leaves.data(), (int) r->leaves.size(), r->unknown));
        OPG_TRY(mg_finalize(M));
        r->N = M->probs[0].levels[0].N;
        if (r->nf != r->N) return fail(OPFLOW_E_INVALID, "request %lld: the equation has %lld unknowns, expected %lld", r->id, r->N, r->nf);
        if (r->x0) OPG_CUDA(cudaMemcpyAsync(M->kd_host[0].x, r->x0, r->N * 8, cudaMemcpyDefault, ctx->stream));
        else OPG_TRY(mg_gather_target(ctx, target, M->kd_host[0].x));  // initx
    } else {
        std::vector<opflow_node> tree = helmholtz_tree(r->pd.ndim, r->pd.alpha, r->pd.beta);
        opflow_field leaves[2] = {r->t, r->rhs};
        OPG_TRY(mg_add_problem(M, r->t, tree.data(), (int) tree.size(), leaves, 2, 0));
        OPG_TRY(mg_finalize(M));
        r->N = M->probs[0].levels[0].N;
        if (r->nf != r->N) return fail(OPFLOW_E_INVALID, "request %lld: f has %lld values, the problem %lld unknowns", r->id, r->nf, r->N);
        // f, x0: host or device memory (unified addressing picks the direction)
        OPG_CUDA(cudaMemcpyAsync(M->probs[0].b, r->f, r->N * 8, cudaMemcpyDefault, ctx->stream));
        if (r->x0) OPG_CUDA(cudaMemcpyAsync(M->kd_host[0].x, r->x0, r->N * 8, cudaMemcpyDefault, ctx->stream));
    }
    if (r->f_dev) {
        // a host f was checked at submission; a device f is checked here, before the request joins a batch
        int* flag = (int*) ctx->scratch;
        int h_flag = 0;
        OPG_CUDA(cudaMemsetAsync(flag, 0, sizeof(int), ctx->stream));
        const long long blk = std::min<long long>((r->N + 255) / 256, (long long) std::max(1, ctx->num_sms) * 8);
        flag_nonfinite<<<(int) std::max<long long>(1, blk), 256, 0, ctx->stream>>>(M->probs[0].b, r->N, flag);
        OPG_LAUNCHED();
        OPG_CUDA(cudaMemcpyAsync(&h_flag, flag, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
        OPG_CUDA(cudaStreamSynchronize(ctx->stream));
        if (h_flag) return fail(OPFLOW_E_NAN, "request %lld: non-finite value in the (device) right-hand side", r->id);
    }
    ProblemHost& P = M->probs[0];
    // a singular problem is pinned (a user equation only when the server's params ask for it, as
    // opflow_solver_solve does; otherwise its right-hand side is projected to zero mean)
    r->pinned = P.singular && !P.has_dirichlet && (!r->eqn || S->params.pin_value);
    if (r->eqn && P.singular && !P.has_dirichlet && !r->pinned) mg_add_scalar(ctx, P.b, r->N, -mg_sum(ctx, P.b, r->N) / (double) r->N);
    if (r->pinned) {
        // the pinned system (first unknown held at 0): singular system with b[0] = -(sum of the others)
        const double sb = mg_sum(ctx, P.b, r->N);
        double b0 = 0.;
        OPG_CUDA(cudaMemcpy(&b0, P.b, 8, cudaMemcpyDeviceToHost));
        const double nb0 = -(sb - b0);
        OPG_CUDA(cudaMemcpy(P.b, &nb0, 8, cudaMemcpyHostToDevice));
    }
    OPG_TRY(mg_prepare_problem(M, S->params.tol, M->dS));
    OPG_CUDA(cudaMemcpyAsync(seed, M->dS, sizeof(Scal), cudaMemcpyDeviceToHost, ctx->stream));
    OPG_CUDA(cudaStreamSynchronize(ctx->stream));
    r->bytes = M->arena.total + (r->t ? (size_t) 2 * r->t->info.count * 8 : 0);
    return OPFLOW_OK;
}

// x -= x[0], with x[0] first copied to `slot` (so no thread reads it while another rewrites it)
__global__ void shift_by_first(double* x, long long n, const double* slot) {
    const double a = -*slot;
    for (long long t = blockIdx.x * (long long) blockDim.x + threadIdx.x; t < n; t += (long long) gridDim.x * blockDim.x) x[t] += a;
}

// Enqueues a finished request's result: the pinned shift and the copy to the caller's buffer
// (completion: after the worker's next stream synchronisation).
static void finish_enqueue(opflow_server S, Req* r, double* slot) {
    opflow_ctx ctx = &S->own_ctx;
    const KrylovDev& K = r->sys->kd_host[0];
    if (r->pinned) {
        cudaMemcpyAsync(slot, K.x, 8, cudaMemcpyDeviceToDevice, ctx->stream);
        const long long blocks = std::min<long long>((r->N + 255) / 256, (long long) ctx->num_sms * 16);
        shift_by_first<<<(int) std::max(1LL, blocks), 256, 0, ctx->stream>>>(K.x, r->N, slot);
        OPG_LAUNCHED();
    }
    if (r->x_out) cudaMemcpyAsync(r->x_out, K.x, r->N * 8, cudaMemcpyDefault, ctx->stream);  // host or device buffer
}

static void finish_mark(opflow_server S, Req* r, int status) {
    r->status = status;
    r->t_done = Clock::now();
    std::lock_guard<std::mutex> lk(S->mu);
    r->done = true;
    S->completed++;
    S->resident--;
    S->used -= std::min(S->used, r->admitted_bytes);
    S->cv_admit.notify_one();
    S->lat.push_back(std::chrono::duration<double, std::milli>(r->t_done - r->t_submit).count());
    S->t_last = r->t_done;
    S->cv_done.notify_all();
}

static void finish_req(opflow_server S, Req* r, int status) {
    opflow_ctx ctx = &S->own_ctx;
    if (status == OPFLOW_OK && r->sys) {
        finish_enqueue(S, r, S->d_slots + S->max_active);
        cudaStreamSynchronize(ctx->stream);
    }
    r->status = status;
    r->t_done = Clock::now();
    std::lock_guard<std::mutex> lk(S->mu);
    r->done = true;
    S->completed++;
    S->resident--;
    S->used -= std::min(S->used, r->admitted_bytes);
    S->cv_admit.notify_one();
    S->lat.push_back(std::chrono::duration<double, std::milli>(r->t_done - r->t_submit).count());
    S->t_last = r->t_done;
    S->cv_done.notify_all();
}

// true when the next pending request fits the batch size and the HBM budget (a request alone is
// always admitted); called with the lock held
static bool can_admit(opflow_server S) {
    if (S->pending.empty() || S->resident >= S->max_active) return false;
    const size_t est = S->pending.front()->est;
    return !S->budget || S->used + est <= S->budget || S->resident == 0;
}

// The admission thread: set-up on its own stream, then the system, its fields and their memory are
// handed to the worker's stream (the set-up stream is synchronised by setup_req).
static void admit_loop(opflow_server S) {
    cudaSetDevice(S->setup_ctx.device);
    for (;;) {
        Req* r = nullptr;
        {
            std::unique_lock<std::mutex> lk(S->mu);
            S->cv_admit.wait(lk, [&] { return (S->stop && S->pending.empty()) || can_admit(S); });
            if (!can_admit(S)) break;  // stopping, nothing left to admit
            r = S->pending.front();
            S->pending.pop_front();
            r->admitted_bytes = r->est;
            S->used += r->admitted_bytes;
            S->resident++;
            S->in_setup++;
        }
        const Clock::time_point t0 = Clock::now();
        r->t_admit = t0;
        const int rc = setup_req(S, r, &r->seed);
        if (rc) {
            const std::string err = opflow_last_error();
            release_req(r);
            finish_req(S, r, rc);
            std::lock_guard<std::mutex> lk(S->mu);
            S->error = err;
            S->in_setup--;
            S->setup_s += std::chrono::duration<double>(Clock::now() - t0).count();
            S->cv.notify_one();
            continue;
        }
        r->sys->ctx = &S->own_ctx;
        r->sys->arena.ctx = &S->own_ctx;
        if (r->t) r->t->ctx = &S->own_ctx;
        if (r->rhs) r->rhs->ctx = &S->own_ctx;
        {
            std::lock_guard<std::mutex> lk(S->mu);
            S->ready.push_back(r);
            S->in_setup--;
            S->setup_s += std::chrono::duration<double>(Clock::now() - t0).count();
        }
        S->cv.notify_one();
    }
}

static void worker_loop(opflow_server S) {
    cudaSetDevice(S->own_ctx.device);
    const int ITERS = 2;
    std::vector<Req*> retired;
    for (;;) {
        std::vector<Req*> admit;
        {
            std::unique_lock<std::mutex> lk(S->mu);
            const auto drained = [&] { return S->stop && S->pending.empty() && S->in_setup == 0 && S->ready.empty(); };
            S->cv.wait(lk, [&] { return drained() || !S->ready.empty() || !S->active.empty(); });
            if (drained() && S->active.empty()) break;
            while (!S->ready.empty()) {
                admit.push_back(S->ready.front());
                S->ready.pop_front();
            }
        }
        auto add_since = [&](double& acc, Clock::time_point t) {
            const double d = std::chrono::duration<double>(Clock::now() - t).count();
            std::lock_guard<std::mutex> lk(S->mu);
            acc += d;
        };
        for (Req* r : admit) {
            S->active.push_back(r);
            S->state.push_back(r->seed);
            S->dirty = true;
        }
        if (S->active.empty()) continue;
        const Clock::time_point t_compose = Clock::now();
        if (S->dirty) {
            std::vector<MGSystem*> parts;
            for (Req* r : S->active) parts.push_back(r->sys);
            if (mg_compose(&S->comp, parts, S->state) != OPFLOW_OK) {
                { std::lock_guard<std::mutex> lk(S->mu); S->error = opflow_last_error(); }
                for (Req* r : S->active) { release_req(r); finish_req(S, r, OPFLOW_E_CUDA); }
                S->active.clear();
                S->state.clear();
                continue;
            }
            S->compositions++;
            S->dirty = false;
            for (Req* r : retired) release_req(r);  // nothing in the new tables points at them
            retired.clear();
            S->max_active_seen = std::max(S->max_active_seen, (int) S->active.size());
        }
        add_since(S->compose_s, t_compose);
        // a few batched iterations, then the per-request scalars
        const Clock::time_point t_iter = Clock::now();
        if (mg_run_iterations(&S->comp, ITERS) != OPFLOW_OK) {
            { std::lock_guard<std::mutex> lk(S->mu); S->error = opflow_last_error(); }
            for (Req* r : S->active) { release_req(r); finish_req(S, r, OPFLOW_E_CUDA); }
            S->active.clear();
            S->state.clear();
            S->dirty = true;
            continue;
        }
        cudaMemcpyAsync(S->state.data(), S->comp.dS, S->state.size() * sizeof(Scal), cudaMemcpyDeviceToHost, S->own_ctx.stream);
        cudaStreamSynchronize(S->own_ctx.stream);
        if (mg_check_error(&S->comp) != OPFLOW_OK) {
            { std::lock_guard<std::mutex> lk(S->mu); S->error = opflow_last_error(); }
            for (Req* r : S->active) { release_req(r); finish_req(S, r, OPFLOW_E_CUDA); }
            S->active.clear();
            S->state.clear();
            S->dirty = true;
            continue;
        }
        add_since(S->iterate_s, t_iter);
        const Clock::time_point t_retire = Clock::now();
        // Every restart and every result of this boundary is enqueued first; one synchronisation
        // then covers them all.
        std::vector<Req*> keep;
        std::vector<Scal> keep_state;
        std::vector<std::pair<size_t, size_t>> restarted;  // (index in keep, index in the composite)
        std::vector<std::pair<Req*, int>> finished;
        std::vector<Req*> checkpointed;
        double* slots = S->d_slots;
        for (size_t i = 0; i < S->active.size(); ++i) {
            Req* r = S->active[i];
            Scal& st = S->state[i];
            if (st.active) { keep.push_back(r); keep_state.push_back(st); continue; }
            r->iters += std::max(0, st.iters);
            r->rel = st.bb > 0 ? std::sqrt(st.rr / st.bb) : std::sqrt(st.rr);
            r->steps_done++;
            { std::lock_guard<std::mutex> lk(S->mu); S->solves++; }
            const bool ok = r->rel <= S->params.tol;
            if (ok && r->steps_done < r->steps) {
                // next backward-Euler step: the solution becomes the right-hand side, same operator
                const KrylovDev& K = r->sys->kd_host[0];
                bool want = false;
                {
                    std::lock_guard<std::mutex> lk(S->mu);
                    want = r->ckpt_state == 1;
                }
                if (want) {  // the state after this step, before the next one changes it
                    cudaMemcpyAsync(r->ckpt_out, K.x, r->N * 8, cudaMemcpyDeviceToHost, S->own_ctx.stream);
                    checkpointed.push_back(r);
                }
                cudaMemcpyAsync(r->sys->probs[0].b, K.x, r->N * 8, cudaMemcpyDeviceToDevice, S->own_ctx.stream);
                mg_prepare_problem(r->sys, S->params.tol, S->comp.dS + i);
                restarted.emplace_back(keep.size(), i);
                keep.push_back(r);
                keep_state.push_back(st);
                continue;
            }
            if (ok) finish_enqueue(S, r, slots + finished.size());
            finished.emplace_back(r, ok ? OPFLOW_OK : OPFLOW_E_NOT_CONVERGED);
            S->dirty = true;
        }
        if (!restarted.empty())
            cudaMemcpyAsync(S->state.data(), S->comp.dS, S->state.size() * sizeof(Scal), cudaMemcpyDeviceToHost, S->own_ctx.stream);
        if (!restarted.empty() || !finished.empty()) cudaStreamSynchronize(S->own_ctx.stream);
        for (auto& q : restarted) keep_state[q.first] = S->state[q.second];
        if (!checkpointed.empty()) {
            std::lock_guard<std::mutex> lk(S->mu);
            for (Req* r : checkpointed) {
                r->ckpt_state = 2;
                r->ckpt_steps = r->steps_done;
            }
            S->cv_done.notify_all();
        }
        for (auto& f : finished) {
            finish_mark(S, f.first, f.second);
            retired.push_back(f.first);
        }
        S->active.swap(keep);
        S->state.swap(keep_state);
        if (S->active.empty() && !retired.empty()) {
            for (Req* r : retired) release_req(r);
            retired.clear();
        }
        add_since(S->retire_s, t_retire);
    }
    for (Req* r : retired) release_req(r);
}

extern "C" {

int opflow_server_create(opflow_ctx ctx, const opflow_solve_params* params, size_t budget, int max_active, opflow_server* out) {
    if (!ctx || !out) return fail(OPFLOW_E_INVALID, "null argument");
    auto* S = new opflow_server_s();
    S->own_ctx.device = ctx->device;
    S->own_ctx.num_sms = ctx->num_sms;
    if (cudaStreamCreateWithFlags(&S->own_ctx.stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete S;
        return fail(OPFLOW_E_CUDA, "stream creation failed");
    }
    S->own_ctx.own_stream = true;
    S->setup_ctx.device = ctx->device;
    S->setup_ctx.num_sms = ctx->num_sms;
    if (cudaStreamCreateWithFlags(&S->setup_ctx.stream, cudaStreamNonBlocking) != cudaSuccess) {
        cudaStreamDestroy(S->own_ctx.stream);
        delete S;
        return fail(OPFLOW_E_CUDA, "stream creation failed");
    }
    S->setup_ctx.own_stream = true;
    if (params) S->params = *params;
    else opflow_solve_params_default(&S->params);
    S->budget = budget;
    S->max_active = max_active > 0 ? max_active : 64;
    S->comp.ctx = &S->own_ctx;
    S->comp.arena.ctx = &S->own_ctx;
    S->comp.precision = S->params.precision;
    S->comp.pre = S->params.pre_sweeps;
    S->comp.post = S->params.post_sweeps;
    S->comp.tol = S->params.tol;
    S->comp.max_iter = S->params.max_iter;
    S->comp.arena.block_hint = 1u << 20;
    if (ensure_scratch(&S->own_ctx, 4096) != OPFLOW_OK || ensure_scratch(&S->setup_ctx, 4096) != OPFLOW_OK ||
        !(S->d_slots = (double*) dev_alloc(&S->own_ctx, (size_t) (S->max_active + 1) * sizeof(double)))) {
        cudaStreamSynchronize(S->own_ctx.stream);
        cudaStreamSynchronize(S->setup_ctx.stream);
        cudaStreamDestroy(S->own_ctx.stream);
        cudaStreamDestroy(S->setup_ctx.stream);
        delete S;
        return OPFLOW_E_NOMEM;
    }
    S->worker = std::thread(worker_loop, S);
    S->admitter = std::thread(admit_loop, S);
    *out = S;
    return OPFLOW_OK;
}

static int submit_equation(opflow_server S, const opflow_request* q, long long* id) {
    const opflow_equation& e = *q->equation;
    if (!e.nodes || e.n_nodes <= 0 || !e.leaves || e.n_leaves <= 0 || e.unknown < 0 || e.unknown >= e.n_leaves)
        return fail(OPFLOW_E_INVALID, "bad equation");
    if (q->steps != 1) return fail(OPFLOW_E_INVALID, "an equation request is one solve (steps must be 1)");
    if (q->f) return fail(OPFLOW_E_INVALID, "an equation request takes its right-hand side from the equation (f must be NULL)");
    for (int i = 0; i < e.n_leaves; ++i)
        if (!e.leaves[i]) return fail(OPFLOW_E_INVALID, "null leaf %d", i);
    const opflow_field target = e.leaves[e.unknown];
    const long long n = assign_box(target->info).count();
    if (n <= 0) return fail(OPFLOW_E_INVALID, "the target has no unknowns");
    // the fields' pending work (uploads, assignments on their contexts' streams) completes first
    for (int i = 0; i < e.n_leaves; ++i) OPG_CUDA(cudaStreamSynchronize(e.leaves[i]->ctx->stream));
    auto* r = new Req();
    r->eqn = true;
    r->nodes.assign(e.nodes, e.nodes + e.n_nodes);
    r->leaves.assign(e.leaves, e.leaves + e.n_leaves);
    r->unknown = e.unknown;
    r->est = estimate_bytes_eqn(n);
    r->steps = 1;
    r->x0 = q->x0;
    r->nf = n;
    r->x_out = q->x_out;
    r->t_submit = Clock::now();
    {
        std::lock_guard<std::mutex> lk(S->mu);
        if (S->stop) { delete r; return fail(OPFLOW_E_INVALID, "server is shutting down"); }
        r->id = S->next_id++;
        S->reqs[r->id] = r;
        S->pending.push_back(r);
        S->submitted++;
        if (!S->have_first) { S->t_first = r->t_submit; S->have_first = true; }
    }
    S->cv_admit.notify_one();
    if (id) *id = r->id;
    return OPFLOW_OK;
}

int opflow_server_submit(opflow_server S, const opflow_request* q, long long* id) {
    if (!S || !q) return fail(OPFLOW_E_INVALID, "null argument");
    if (q->equation) return submit_equation(S, q, id);
    if (!q->f) return fail(OPFLOW_E_INVALID, "null right-hand side");
    if (q->steps < 1) return fail(OPFLOW_E_INVALID, "steps must be >= 1");
    const opflow_problem_desc& pd = q->problem;
    if (pd.ndim < 1 || pd.ndim > 3) return fail(OPFLOW_E_INVALID, "bad problem dimension");
    long long n = 1;
    for (int d = 0; d < pd.ndim; ++d) {
        if (pd.n[d] < 3) return fail(OPFLOW_E_INVALID, "problem extent");
        const int unk = pd.loc == OPFLOW_CENTER ? pd.n[d] : (pd.bc == OPFLOW_BC_DIRC ? pd.n[d] - 2 : pd.n[d]);
        n *= unk;
    }
    // f in device memory is checked on the device at admission; host (or managed) memory here
    cudaPointerAttributes pa{};
    const bool f_dev = cudaPointerGetAttributes(&pa, q->f) == cudaSuccess && pa.type == cudaMemoryTypeDevice;
    cudaGetLastError();  // an unregistered host pointer is not an error for this query
    if (!f_dev)
        for (long long i = 0; i < n; ++i)
            if (!std::isfinite(q->f[i])) return fail(OPFLOW_E_NAN, "non-finite value in the right-hand side at %lld", i);
    auto* r = new Req();
    r->f_dev = f_dev;
    r->pd = pd;
    r->est = estimate_bytes(pd);
    r->steps = q->steps;
    r->f = q->f;
    r->x0 = q->x0;
    r->nf = n;
    r->x_out = q->x_out;
    r->t_submit = Clock::now();
    {
        std::lock_guard<std::mutex> lk(S->mu);
        if (S->stop) { delete r; return fail(OPFLOW_E_INVALID, "server is shutting down"); }
        r->id = S->next_id++;
        S->reqs[r->id] = r;
        S->pending.push_back(r);
        S->submitted++;
        if (!S->have_first) { S->t_first = r->t_submit; S->have_first = true; }
    }
    S->cv_admit.notify_one();
    if (id) *id = r->id;
    return OPFLOW_OK;
}

int opflow_server_result(opflow_server S, long long id, int wait, int* done, opflow_request_result* out) {
    if (!S) return fail(OPFLOW_E_INVALID, "null server");
    std::unique_lock<std::mutex> lk(S->mu);
    auto it = S->reqs.find(id);
    if (it == S->reqs.end()) return fail(OPFLOW_E_INVALID, "unknown request %lld", id);
    Req* r = it->second;
    if (wait) S->cv_done.wait(lk, [&] { return r->done; });
    if (done) *done = r->done;
    if (r->done && out) {
        out->id = r->id;
        out->status = r->status;
        out->iterations = r->iters;
        out->solves = r->steps_done;
        out->rel_residual = r->rel;
        out->queue_ms = std::chrono::duration<double, std::milli>(r->t_admit - r->t_submit).count();
        out->latency_ms = std::chrono::duration<double, std::milli>(r->t_done - r->t_submit).count();
    }
    return OPFLOW_OK;
}

int opflow_server_checkpoint(opflow_server S, long long id, double* x_out, size_t n, int* steps_done) {
    if (!S || !x_out) return fail(OPFLOW_E_INVALID, "null argument");
    std::unique_lock<std::mutex> lk(S->mu);
    auto it = S->reqs.find(id);
    if (it == S->reqs.end()) return fail(OPFLOW_E_INVALID, "unknown request %lld", id);
    Req* r = it->second;
    if (r->steps <= 1) return fail(OPFLOW_E_INVALID, "request %lld is a single solve, not a session", id);
    if ((long long) n != r->nf) return fail(OPFLOW_E_INVALID, "request %lld has %lld unknowns, not %zu", id, r->nf, n);
    if (r->done) return fail(OPFLOW_E_INVALID, "request %lld has finished", id);
    if (r->ckpt_state != 0) return fail(OPFLOW_E_INVALID, "request %lld: a checkpoint is already pending", id);
    r->ckpt_out = x_out;
    r->ckpt_state = 1;
    S->cv_done.wait(lk, [&] { return r->ckpt_state == 2 || r->done; });
    const bool taken = r->ckpt_state == 2;
    r->ckpt_state = 0;
    r->ckpt_out = nullptr;
    if (!taken) return fail(OPFLOW_E_INVALID, "request %lld finished before its next step boundary", id);
    if (steps_done) *steps_done = r->ckpt_steps;
    return OPFLOW_OK;
}

int opflow_server_drain(opflow_server S) {
    if (!S) return fail(OPFLOW_E_INVALID, "null server");
    std::unique_lock<std::mutex> lk(S->mu);
    S->cv_done.wait(lk, [&] { return S->completed == S->submitted; });
    return OPFLOW_OK;
}

int opflow_server_stats(opflow_server S, opflow_serve_stats* o) {
    if (!S || !o) return fail(OPFLOW_E_INVALID, "null argument");
    std::lock_guard<std::mutex> lk(S->mu);
    std::memset(o, 0, sizeof *o);
    o->submitted = S->submitted;
    o->completed = S->completed;
    o->solves = S->solves;
    std::vector<double> l = S->lat;
    if (!l.empty()) {
        std::sort(l.begin(), l.end());
        auto q = [&](double p) { return l[std::min(l.size() - 1, (size_t) std::ceil(p * l.size()) - (p > 0 ? 1 : 0))]; };
        o->p50_ms = q(0.50);
        o->p99_ms = q(0.99);
        double s = 0;
        for (double v : l) s += v;
        o->mean_ms = s / l.size();
        o->max_ms = l.back();
    }
    if (S->have_first && S->completed) {
        o->elapsed_s = std::chrono::duration<double>(S->t_last - S->t_first).count();
        o->solves_per_s = o->elapsed_s > 0 ? S->solves / o->elapsed_s : 0.;
    }
    o->max_active_seen = S->max_active_seen;
    o->graph_launches = S->comp.graph_launches;
    o->compositions = S->compositions;
    o->setup_s = S->setup_s;
    o->compose_s = S->compose_s;
    o->iterate_s = S->iterate_s;
    o->retire_s = S->retire_s;
    return OPFLOW_OK;
}

int opflow_server_destroy(opflow_server S) {
    if (!S) return OPFLOW_OK;
    {
        std::lock_guard<std::mutex> lk(S->mu);
        S->stop = true;
    }
    S->cv_admit.notify_all();
    S->cv.notify_all();
    if (S->admitter.joinable()) S->admitter.join();
    S->cv.notify_all();
    if (S->worker.joinable()) S->worker.join();
    for (auto& kv : S->reqs) {
        release_req(kv.second);
        delete kv.second;
    }
    if (S->comp.exec) cudaGraphExecDestroy(S->comp.exec);
    S->comp.exec = nullptr;
    if (S->comp.solve_exec) cudaGraphExecDestroy(S->comp.solve_exec);
    S->comp.solve_exec = nullptr;
    if (S->comp.rec_stream) cudaStreamDestroy(S->comp.rec_stream);
    S->comp.rec_stream = nullptr;
    S->comp.arena.release();
    if (S->comp.h_active) cudaFreeHost(S->comp.h_active);
    if (S->own_ctx.scratch) dev_free(&S->own_ctx, S->own_ctx.scratch);
    if (S->d_slots) dev_free(&S->own_ctx, S->d_slots);
    cudaStreamSynchronize(S->own_ctx.stream);
    cudaStreamDestroy(S->own_ctx.stream);
    if (S->setup_ctx.scratch) dev_free(&S->setup_ctx, S->setup_ctx.scratch);
    cudaStreamSynchronize(S->setup_ctx.stream);
    cudaStreamDestroy(S->setup_ctx.stream);
    delete S;
    return OPFLOW_OK;
}

}  // extern "C"
