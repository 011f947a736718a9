// Coupled systems of several equations and unknown fields: the reference's SolveEqns /
// makeEqnSolveHandler over an equation set (src/Core/Equation/UnifiedSolve.hpp:69-100,
// AMGCLEqnSolveHandler.hpp:53-190) with the matrix CSRMatrixGenerator builds
// (src/Core/Equation/CSRMatrixGenerator.hpp:25-220).
//
// Equation k is affine in the unknowns, F_k(u_0 .. u_{n-1}) = sum_j A_kj u_j - b_k.  Its block A_kj
// is assembled by the single-unknown StencilPad assembler (assemble.cu) with u_j as the unknown, the
// rows taken from u_k's assignable cells and every other unknown replaced by a zero-valued copy of its
// field (whose padding still carries its boundary values, so each block's right-hand side is the
// same b_k).  Blocks are stored as ELL arrays (one column and value per stencil entry and row),
// numbered like the reference's ColoredMDRangeMapper: equation after equation, x fastest within each
// unknown's assignable range.  A pinned equation's last row becomes an identity row with right-hand
// side 0 (CSRMatrixGenerator::generate, pinValue).
//
// The system is solved by the host-driven Krylov methods (krylov.cu) with one of:
// - smoothed-aggregation AMG over the whole coupled matrix (OPFLOW_PRECOND_AMG, amg.h: AMGCL's
//   amg<smoothed_aggregation, spai0>, the reference's choice), which also coarsens the couplings;
// - a block-diagonal preconditioner: each equation's own geometric multigrid hierarchy on its diagonal
//   block (OPFLOW_PRECOND_MG), leaving the off-diagonal couplings to the Krylov method;
// - Jacobi on the assembled diagonal, or none.
#include "amg.h"
#include "solver.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <vector>

namespace opg {
namespace {

constexpr int EQ_THREADS = 256;

struct Ell {
    int k = 0, j = 0, nk = 0;
    long long rows = 0;
    int* col = nullptr;     // [nk][rows], -1: no entry
    double* val = nullptr;  // [nk][rows]
    int diag_entry = -1;    // entry of offset 0 (diagonal blocks)
};

__global__ void ell_build(Box rows, Box cols, int per0, int per1, int per2, const int* __restrict__ K, int nk, const double* __restrict__ coef,
                          long long col_off, int* __restrict__ col, double* __restrict__ val, int* __restrict__ bad) {
    const long long n = rows.count();
    const int per[3] = {per0, per1, per2};
    for (long long r = blockIdx.x * (long long) blockDim.x + threadIdx.x; r < n; r += (long long) gridDim.x * blockDim.x) {
        int c[3];
        box_index(r, rows, c[0], c[1], c[2]);
        for (int e = 0; e < nk; ++e) {
            const double v = coef[(long long) e * n + r];
            int idx[3];
            bool in = true;
            for (int d = 0; d < 3; ++d) {
                idx[d] = c[d] + K[3 * e + d];
                const int lo = cols.lo[d], len = cols.hi[d] - cols.lo[d];
                if (per[d] && len > 0) idx[d] = lo + (((idx[d] - lo) % len) + len) % len;
                in = in && idx[d] >= cols.lo[d] && idx[d] < cols.hi[d];
            }
            if (!in) {
                if (v != 0.) atomicExch(bad, 1);
                col[(long long) e * n + r] = -1;
                val[(long long) e * n + r] = 0.;
                continue;
            }
            const long long nx = cols.hi[0] - cols.lo[0], ny = cols.hi[1] - cols.lo[1];
            const long long lin = (idx[0] - cols.lo[0]) + nx * ((idx[1] - cols.lo[1]) + ny * (long long) (idx[2] - cols.lo[2]));
            col[(long long) e * n + r] = v != 0. ? (int) (col_off + lin) : -1;
            val[(long long) e * n + r] = v;
        }
    }
}

// y[r] (+)= sum_e val[e][r] * x[col[e][r]]
__global__ void __launch_bounds__(EQ_THREADS) ell_spmv(long long n, int nk, const int* __restrict__ col, const double* __restrict__ val,
                                                       const double* __restrict__ x, double* __restrict__ y, int accumulate) {
    for (long long r = blockIdx.x * (long long) blockDim.x + threadIdx.x; r < n; r += (long long) gridDim.x * blockDim.x) {
        double s = accumulate ? y[r] : 0.;
        for (int e = 0; e < nk; ++e) {
            const int c = col[(long long) e * n + r];
            if (c >= 0) s += val[(long long) e * n + r] * x[c];
        }
        y[r] = s;
    }
}

// a pinned equation's last row: identity in the diagonal block, zero elsewhere
__global__ void ell_pin_row(long long n, int nk, int* col, double* val, int diag_entry, long long self) {
    const int e = threadIdx.x;
    if (e < nk) {
        const long long r = n - 1;
        val[(long long) e * n + r] = e == diag_entry ? 1. : 0.;
        col[(long long) e * n + r] = e == diag_entry ? (int) self : -1;
    }
}

__global__ void ell_diag(long long n, const double* __restrict__ val, double* __restrict__ diag) {
    for (long long r = blockIdx.x * (long long) blockDim.x + threadIdx.x; r < n; r += (long long) gridDim.x * blockDim.x) diag[r] = val[r];
}

// sum of v[0 .. n-1) per block (fixed partition), then the pinned row's consistent value
__global__ void block_sums(long long n, const double* __restrict__ v, double* __restrict__ part) {
    __shared__ double red[EQ_THREADS / 32];
    double s = 0.;
    for (long long r = blockIdx.x * (long long) blockDim.x + threadIdx.x; r < n; r += (long long) gridDim.x * blockDim.x) s += v[r];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.;
        for (int w = 0; w < EQ_THREADS / 32; ++w) t += red[w];
        part[blockIdx.x] = t;
    }
}
// w = v with its last entry replaced by minus the sum of the others (the singular system's consistent
// right-hand side whose solution, shifted, solves the last-row-pinned one)
__global__ void consistent_rhs(long long n, const double* __restrict__ v, const double* __restrict__ part, int nblk, double* __restrict__ w) {
    for (long long r = blockIdx.x * (long long) blockDim.x + threadIdx.x; r < n; r += (long long) gridDim.x * blockDim.x) {
        if (r == n - 1) {
            double s = 0.;
            for (int b = 0; b < nblk; ++b) s += part[b];
            w[r] = -(s - v[r]);
        } else {
            w[r] = v[r];
        }
    }
}
__global__ void shift_to_pin(long long n, const double* __restrict__ v, double* __restrict__ z, double* __restrict__ c) {
    if (blockIdx.x == 0 && threadIdx.x == 0) *c = v[n - 1] - z[n - 1];
}
__global__ void add_dev(long long n, double* __restrict__ z, const double* __restrict__ c) {
    const double a = *c;
    for (long long r = blockIdx.x * (long long) blockDim.x + threadIdx.x; r < n; r += (long long) gridDim.x * blockDim.x) z[r] += a;
}

__global__ void div_by(long long n, const double* __restrict__ v, const double* __restrict__ d, double* __restrict__ z) {
    for (long long r = blockIdx.x * (long long) blockDim.x + threadIdx.x; r < n; r += (long long) gridDim.x * blockDim.x) z[r] = v[r] / d[r];
}

__global__ void box_scatter(FieldView f, Box b, const double* in) {
    for (long long t = blockIdx.x * (long long) blockDim.x + threadIdx.x; t < b.count(); t += (long long) gridDim.x * blockDim.x) {
        int i, j, k;
        box_index(t, b, i, j, k);
        f.data[(i - f.off[0]) + (j - f.off[1]) * f.sy + (k - f.off[2]) * f.sz] = in[t];
    }
}

opflow_mesh_desc mesh_desc_of(const MeshDev* m) {
    opflow_mesh_desc d{};
    d.ndim = m->ndim;
    d.pad_width = m->pad;
    for (int q = 0; q < m->ndim; ++q) {
        d.dims[q] = m->n[q] - 2 * m->pad;
        d.start[q] = m->es[q] + m->pad;
        d.x[q] = const_cast<double*>(m->hx[q].data());
        d.dx[q] = const_cast<double*>(m->hdx[q].data());
    }
    return d;
}

}  // namespace
}  // namespace opg

using namespace opg;

struct opflow_eqnset_s {
    opflow_ctx ctx = nullptr;
    int neq = 0;
    std::vector<opflow_field> targets;
    std::vector<int> slot;  // leaf slot of each target
    std::vector<std::vector<opflow_node>> trees;
    std::vector<opflow_field> leaves;
    std::vector<int> pin;
    opflow_solve_params params{};
    std::vector<opflow_field> zero;  // zero-valued copy of each target
    std::vector<Box> boxes;          // each target's assignable box
    std::vector<long long> off;      // row / column offset of each block
    long long n = 0;
    std::vector<std::vector<int>> deps;  // unknowns each equation reads
    std::vector<Ell> blocks;
    double *b = nullptr, *x = nullptr, *diag = nullptr, *r = nullptr;
    double *tmp = nullptr, *part = nullptr;  // the pinned equations' preconditioner scratch
    Arena arena;        // b, x, diag, the Krylov workspace
    Arena mat;          // the ELL blocks (rebuilt with the matrix)
    KrylovWork* W = nullptr;
    std::vector<MGSystem*> mg;
    AmgDev amg;
    bool amg_built = false;
    bool first = true;
    bool have_matrix = false;
};

namespace {

struct SetOp : KrylovOp {
    opflow_eqnset s;
    int grid;
    int matvec(const double* xin, double* y) override {
        std::vector<bool> touched(s->neq, false);
        for (const Ell& e : s->blocks) {
            ell_spmv<<<grid, EQ_THREADS, 0, stream>>>(e.rows, e.nk, e.col, e.val, xin, y + s->off[e.k], touched[e.k] ? 1 : 0);
            OPG_LAUNCHED();
            touched[e.k] = true;
        }
        return check_launch("ell_spmv");
    }
    int precond(const double* v, double* z) override {
        const int pc = s->params.precond;
        if (pc == OPFLOW_PRECOND_NONE) {
            OPG_CUDA(cudaMemcpyAsync(z, v, s->n * 8, cudaMemcpyDeviceToDevice, stream));
            return OPFLOW_OK;
        }
        if (pc == OPFLOW_PRECOND_JACOBI) {
            div_by<<<grid, EQ_THREADS, 0, stream>>>(s->n, v, s->diag, z);
            OPG_LAUNCHED();
            return check_launch("div_by");
        }
        if (pc == OPFLOW_PRECOND_AMG) return amg_vcycle(s->ctx, stream, s->amg, v, z);
        for (int k = 0; k < s->neq; ++k) {
            const long long Nk = s->boxes[k].count();
            if (!s->pin[k]) {
                OPG_TRY(mg_precond_level0(s->mg[k], v + s->off[k], z + s->off[k]));
                continue;
            }
            // a pinned equation: the V-cycle of the singular operator on the consistent right-hand
            // side, shifted so that the pinned unknown takes the pinned row's value
            const int nblk = 64;
            const double* vk = v + s->off[k];
            double* zk = z + s->off[k];
            block_sums<<<nblk, EQ_THREADS, 0, stream>>>(Nk - 1, vk, s->part);
            consistent_rhs<<<grid, EQ_THREADS, 0, stream>>>(Nk, vk, s->part, nblk, s->tmp);
            OPG_LAUNCHED();
            OPG_TRY(mg_precond_level0(s->mg[k], s->tmp, zk));
            shift_to_pin<<<1, 32, 0, stream>>>(Nk, vk, zk, s->part + nblk);
            add_dev<<<grid, EQ_THREADS, 0, stream>>>(Nk, zk, s->part + nblk);
            OPG_LAUNCHED();
            OPG_TRY(check_launch("pinned preconditioner"));
        }
        return OPFLOW_OK;
    }
};

int grid_of(opflow_ctx ctx, long long n) {
    return (int) std::max<long long>(1, std::min<long long>((n + EQ_THREADS - 1) / EQ_THREADS, (long long) ctx->num_sms * 8));
}

void release_matrix(opflow_eqnset s) {
    s->blocks.clear();
    s->mat.release();
    s->have_matrix = false;
}

void release_mg(opflow_eqnset s) {
    for (MGSystem* S : s->mg) mg_destroy(S);
    s->mg.clear();
}

// the leaves with every unknown but `keep` replaced by its zero copy
std::vector<opflow_field> leaves_for(opflow_eqnset s, int keep) {
    std::vector<opflow_field> L = s->leaves;
    for (int t = 0; t < s->neq; ++t)
        if (t != keep) L[s->slot[t]] = s->zero[t];
    return L;
}

// generateAb: every block and the right-hand side (`rhs_only`: the right-hand side alone, the
// blocks' values are kept)
int assemble(opflow_eqnset s, bool rhs_only) {
    opflow_ctx ctx = s->ctx;
    if (!rhs_only) release_matrix(s);
    for (int k = 0; k < s->neq; ++k) {
        const long long Nk = s->boxes[k].count();
        bool rhs_done = false;
        for (int j : s->deps[k]) {
            if (rhs_only && rhs_done) break;  // generateb: one right-hand-side evaluation per equation
            std::vector<opflow_field> L = leaves_for(s, j);
            AsmPlan plan;
            OPG_TRY(asm_prepare(ctx, s->targets[j], s->trees[k].data(), (int) s->trees[k].size(), L.data(), (int) L.size(), s->slot[j], 0, &plan,
                                s->targets[k]));
            const int nk = plan.P.nk;
            double* coef = rhs_only ? nullptr : (double*) dev_alloc(ctx, (size_t) nk * Nk * 8 + 8);
            double* rhs = (double*) dev_alloc(ctx, (size_t) Nk * 8 + 8);
            int* dK = (int*) dev_alloc(ctx, (size_t) nk * 3 * sizeof(int) + 16);
            if ((!rhs_only && !coef) || !rhs || !dK) return fail(OPFLOW_E_NOMEM, "coupled assembly buffers");
            int rc = asm_run(ctx, &plan, coef, rhs);
            if (rc == OPFLOW_OK && !rhs_done) {
                OPG_CUDA(cudaMemcpyAsync(s->b + s->off[k], rhs, Nk * 8, cudaMemcpyDeviceToDevice, ctx->stream));
                rhs_done = true;
            }
            if (rc == OPFLOW_OK && !rhs_only) {
                Ell E;
                E.k = k;
                E.j = j;
                E.nk = nk;
                E.rows = Nk;
                E.col = (int*) s->mat.alloc((size_t) nk * Nk * sizeof(int));
                E.val = (double*) s->mat.alloc((size_t) nk * Nk * 8);
                if (!E.col || !E.val) rc = fail(OPFLOW_E_NOMEM, "coupled matrix");
                std::vector<int> hK(3 * nk);
                for (int e = 0; e < nk; ++e) {
                    for (int d = 0; d < 3; ++d) hK[3 * e + d] = plan.P.K[e][d];
                    if (!hK[3 * e] && !hK[3 * e + 1] && !hK[3 * e + 2]) E.diag_entry = e;
                }
                int* bad = (int*) ctx->scratch;
                if (rc == OPFLOW_OK) {
                    cudaMemcpyAsync(dK, hK.data(), hK.size() * sizeof(int), cudaMemcpyHostToDevice, ctx->stream);
                    cudaMemsetAsync(bad, 0, sizeof(int), ctx->stream);
                    const opflow_field tj = s->targets[j];
                    int per[3] = {0, 0, 0};
                    for (int d = 0; d < tj->info.ndim; ++d) per[d] = tj->desc.bc_type[d][0] == OPFLOW_BC_PERIODIC;
                    ell_build<<<grid_of(ctx, Nk), EQ_THREADS, 0, ctx->stream>>>(s->boxes[k], s->boxes[j], per[0], per[1], per[2], dK, nk, coef, s->off[j],
                                                                                E.col, E.val, bad);
                    OPG_LAUNCHED();
                    rc = check_launch("ell_build");
                    int hb = 0;
                    cudaMemcpyAsync(&hb, bad, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream);
                    cudaStreamSynchronize(ctx->stream);
                    if (rc == OPFLOW_OK && hb) rc = fail(OPFLOW_E_RANGE, "equation %d: a coefficient on unknown %d falls outside its assignable range", k, j);
                }
                if (rc == OPFLOW_OK) s->blocks.push_back(E);
            }
            cudaStreamSynchronize(ctx->stream);
            dev_free(ctx, coef);
            dev_free(ctx, rhs);
            dev_free(ctx, dK);
            OPG_TRY(rc);
        }
    }
    // pinned equations: identity last row, right-hand side 0
    for (int k = 0; k < s->neq; ++k) {
        if (!s->pin[k]) continue;
        const long long Nk = s->boxes[k].count();
        const double zero = 0.;
        OPG_CUDA(cudaMemcpyAsync(s->b + s->off[k] + Nk - 1, &zero, 8, cudaMemcpyHostToDevice, s->ctx->stream));
        if (rhs_only) continue;
        for (Ell& E : s->blocks) {
            if (E.k != k) continue;
            const int de = E.j == k ? E.diag_entry : -1;
            ell_pin_row<<<1, 128, 0, s->ctx->stream>>>(E.rows, E.nk, E.col, E.val, de, s->off[k] + Nk - 1);
            OPG_LAUNCHED();
        }
    }
    if (!rhs_only) {
        for (const Ell& E : s->blocks)
            if (E.k == E.j && E.diag_entry >= 0) {
                ell_diag<<<grid_of(ctx, E.rows), EQ_THREADS, 0, ctx->stream>>>(E.rows, E.val + (long long) E.diag_entry * E.rows, s->diag + s->off[E.k]);
                OPG_LAUNCHED();
            }
        s->have_matrix = true;
    }
    OPG_CUDA(cudaStreamSynchronize(ctx->stream));
    return check_launch("coupled assembly");
}

// each equation's multigrid hierarchy on its diagonal block (the other unknowns as zero fields)
int build_mg(opflow_eqnset s) {
    release_mg(s);
    for (int k = 0; k < s->neq; ++k) {
        auto* S = new MGSystem();
        S->ctx = s->ctx;
        S->arena.ctx = s->ctx;
        S->precision = s->params.precision;
        S->pre = s->params.pre_sweeps;
        S->post = s->params.post_sweeps;
        S->coarse_max = s->params.coarse_max;
        S->tol = s->params.tol;
        S->max_iter = s->params.max_iter;
        s->mg.push_back(S);
        std::vector<opflow_field> L = leaves_for(s, k);
        OPG_TRY(mg_add_problem(S, s->targets[k], s->trees[k].data(), (int) s->trees[k].size(), L.data(), (int) L.size(), s->slot[k]));
        OPG_TRY(mg_finalize(S));
        OPG_TRY(mg_activate(S));
    }
    return OPFLOW_OK;
}

// the assembled coupled matrix as host CSR (rows sorted by column, entries of one column merged)
int host_csr(opflow_eqnset s, std::vector<std::vector<std::pair<long long, double>>>& R) {
    R.assign((size_t) s->n, {});
    for (const Ell& E : s->blocks) {
        std::vector<int> c((size_t) E.nk * E.rows);
        std::vector<double> v((size_t) E.nk * E.rows);
        OPG_CUDA(cudaMemcpy(c.data(), E.col, c.size() * sizeof(int), cudaMemcpyDeviceToHost));
        OPG_CUDA(cudaMemcpy(v.data(), E.val, v.size() * 8, cudaMemcpyDeviceToHost));
        for (long long r = 0; r < E.rows; ++r)
            for (int e = 0; e < E.nk; ++e) {
                const int cc = c[(size_t) e * E.rows + r];
                if (cc >= 0) R[(size_t) (s->off[E.k] + r)].push_back({cc, v[(size_t) e * E.rows + r]});
            }
    }
    for (auto& row : R) {
        std::sort(row.begin(), row.end(), [](const auto& a, const auto& b) { return a.first < b.first; });
        // entries of several stencil offsets that fold onto one column add up
        std::vector<std::pair<long long, double>> merged;
        for (auto& pr : row) {
            if (!merged.empty() && merged.back().first == pr.first) merged.back().second += pr.second;
            else merged.push_back(pr);
        }
        row.swap(merged);
    }
    return OPFLOW_OK;
}

// the AMG hierarchy of the whole coupled matrix (set up on the host, cycled on the device)
int build_amg(opflow_eqnset s) {
    std::vector<std::vector<std::pair<long long, double>>> R;
    OPG_TRY(host_csr(s, R));
    HostCsr A;
    A.n = A.m = s->n;
    A.ptr.assign((size_t) s->n + 1, 0);
    for (long long r = 0; r < s->n; ++r) {
        for (auto& pr : R[(size_t) r]) {
            A.col.push_back((int) pr.first);
            A.val.push_back(pr.second);
        }
        A.ptr[(size_t) r + 1] = (long long) A.col.size();
    }
    AmgHost H;
    OPG_TRY(amg_build_host(A, AmgParams{}, &H));
    OPG_TRY(amg_upload(s->ctx, H, &s->amg));
    s->amg_built = true;
    return OPFLOW_OK;
}

}  // namespace

extern "C" {

int opflow_eqnset_create(opflow_ctx ctx, int n_eqn, const opflow_field* targets, const opflow_node* const* trees, const int* n_nodes,
                         const opflow_field* leaves, int n_leaves, const int* pin, const opflow_solve_params* params, opflow_eqnset* out) {
    if (!ctx || n_eqn < 1 || !targets || !trees || !n_nodes || !leaves || n_leaves < n_eqn || !out) return fail(OPFLOW_E_INVALID, "bad equation-set arguments");
    if (n_leaves > 8) return fail(OPFLOW_E_INVALID, "at most 8 leaf fields");
    opflow_solve_params p;
    if (params) p = *params;
    else opflow_solve_params_default(&p);
    if (p.krylov < OPFLOW_KRYLOV_PCG || p.krylov > OPFLOW_KRYLOV_NONE || p.precond < OPFLOW_PRECOND_MG || p.precond > OPFLOW_PRECOND_AMG)
        return fail(OPFLOW_E_INVALID, "bad solver parameters");
    if (p.krylov == OPFLOW_KRYLOV_NONE && p.precond == OPFLOW_PRECOND_NONE) return fail(OPFLOW_E_INVALID, "no solver");
    if (p.kdim <= 0) p.kdim = 5;
    auto* s = new opflow_eqnset_s();
    s->ctx = ctx;
    s->neq = n_eqn;
    s->params = p;
    s->leaves.assign(leaves, leaves + n_leaves);
    s->arena.ctx = ctx;
    s->mat.ctx = ctx;
    int rc = OPFLOW_OK;
    for (int k = 0; k < n_eqn && rc == OPFLOW_OK; ++k) {
        s->targets.push_back(targets[k]);
        s->trees.emplace_back(trees[k], trees[k] + n_nodes[k]);
        s->pin.push_back(pin ? pin[k] : 0);
        int sl = -1;
        for (int q = 0; q < n_leaves; ++q)
            if (leaves[q] == targets[k]) sl = q;
        if (sl < 0 || !targets[k] || targets[k]->ctx != ctx) rc = fail(OPFLOW_E_INVALID, "target %d is not among the leaves", k);
        s->slot.push_back(sl);
    }
    for (int k = 0; k < n_eqn && rc == OPFLOW_OK; ++k) {
        // the unknowns equation k reads, in slot order
        std::vector<int> d;
        for (int j = 0; j < n_eqn; ++j)
            for (const opflow_node& nd : s->trees[k])
                if (nd.kind == OPFLOW_NODE_FIELD && nd.field == s->slot[j]) {
                    d.push_back(j);
                    break;
                }
        if (std::find(d.begin(), d.end(), k) == d.end()) rc = fail(OPFLOW_E_INVALID, "equation %d does not involve its own target", k);
        s->deps.push_back(d);
        s->boxes.push_back(assign_box(targets[k]->info));
        s->off.push_back(s->n);
        s->n += s->boxes.back().count();
        opflow_mesh_desc md = mesh_desc_of(targets[k]->mesh);
        opflow_field z = nullptr;
        if (rc == OPFLOW_OK) rc = opflow_field_create(ctx, &md, &targets[k]->desc, &z);
        s->zero.push_back(z);
    }
    if (rc == OPFLOW_OK) {
        s->b = (double*) s->arena.alloc((size_t) s->n * 8);
        s->x = (double*) s->arena.alloc((size_t) s->n * 8);
        s->diag = (double*) s->arena.alloc((size_t) s->n * 8);
        s->r = (double*) s->arena.alloc((size_t) s->n * 8);
        s->tmp = (double*) s->arena.alloc((size_t) s->n * 8);
        s->part = (double*) s->arena.alloc(128 * 8);
        if (!s->b || !s->x || !s->diag || !s->r || !s->tmp || !s->part) rc = fail(OPFLOW_E_NOMEM, "coupled vectors");
        else {
            cudaMemsetAsync(s->x, 0, s->n * 8, ctx->stream);
            cudaMemsetAsync(s->diag, 0, s->n * 8, ctx->stream);
        }
    }
    if (rc) {
        opflow_eqnset_destroy(s);
        return rc;
    }
    *out = s;
    return OPFLOW_OK;
}

int opflow_eqnset_solve(opflow_eqnset s, opflow_solve_state* state) {
    if (!s) return fail(OPFLOW_E_INVALID, "null equation set");
    opflow_ctx ctx = s->ctx;
    using clk = std::chrono::steady_clock;
    const auto t0 = clk::now();
    // AMGCLEqnSolveHandler::solve: generateAb on the first run and whenever the matrix is not static,
    // generateb otherwise; x starts at 0 on the first run and from the previous solution after
    const bool rebuild = s->first || !s->params.static_mat;
    OPG_TRY(assemble(s, !rebuild && s->have_matrix));
    if (s->params.precond == OPFLOW_PRECOND_MG && (rebuild || s->mg.empty())) OPG_TRY(build_mg(s));
    if (s->params.precond == OPFLOW_PRECOND_AMG && (rebuild || !s->amg_built)) OPG_TRY(build_amg(s));
    KrylovParams kp;
    kp.method = s->params.krylov;
    kp.precond = s->params.precond;
    kp.kdim = s->params.kdim;
    kp.max_iter = s->params.max_iter;
    kp.tol = s->params.tol;
    kp.abs_tol = s->params.abs_tol;
    if (!krylov_work_fits(s->W, s->n, kp)) {
        krylov_work_free(s->W);
        s->W = krylov_work(s->arena, ctx, s->n, kp);
        if (!s->W) return fail(OPFLOW_E_NOMEM, "Krylov workspace");
    }
    s->first = false;
    const auto t1 = clk::now();
    SetOp op;
    op.s = s;
    op.grid = grid_of(ctx, s->n);
    int iters = 0;
    OPG_TRY(krylov_run(op, *s->W, ctx, s->n, kp, s->b, s->x, &iters));
    // true residual and the values back into the targets (returnValues)
    double* r = s->r;
    OPG_TRY(op.residual(s->b, s->x, r));
    std::vector<double> hr(s->n), hb(s->n);
    OPG_CUDA(cudaMemcpyAsync(hr.data(), r, s->n * 8, cudaMemcpyDeviceToHost, ctx->stream));
    OPG_CUDA(cudaMemcpyAsync(hb.data(), s->b, s->n * 8, cudaMemcpyDeviceToHost, ctx->stream));
    for (int k = 0; k < s->neq; ++k) {
        opflow_field t = s->targets[k];
        box_scatter<<<grid_of(ctx, s->boxes[k].count()), EQ_THREADS, 0, ctx->stream>>>(t->view(), s->boxes[k], s->x + s->off[k]);
        OPG_LAUNCHED();
        t->bc_fresh[t->cur] = false;
        t->version++;
        OPG_TRY(update_padding_buf(t, t->buf[t->cur]));
    }
    OPG_CUDA(cudaStreamSynchronize(ctx->stream));
    double rr = 0., bb = 0.;
    for (long long q = 0; q < s->n; ++q) {
        rr += hr[q] * hr[q];
        bb += hb[q] * hb[q];
    }
    const auto t2 = clk::now();
    if (state) {
        state->iterations = iters;
        state->abs_residual = std::sqrt(rr);
        state->rel_residual = bb > 0 ? std::sqrt(rr / bb) : std::sqrt(rr);
        state->converged = state->rel_residual <= s->params.tol || (s->params.abs_tol > 0 && state->abs_residual <= s->params.abs_tol);
        state->setup_ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
        state->solve_ms = std::chrono::duration<double, std::milli>(t2 - t1).count();
    }
    if (state && !state->converged && iters >= s->params.max_iter)
        return fail(OPFLOW_E_NOT_CONVERGED, "not converged after %d iterations (relative residual %g)", iters, state->rel_residual);
    return OPFLOW_OK;
}

int opflow_eqnset_csr(opflow_eqnset s, long long* n_rows, long long* nnz, long long* row_ptr, long long* cols, double* vals, double* rhs) {
    if (!s || !n_rows || !nnz) return fail(OPFLOW_E_INVALID, "null argument");
    if (!s->have_matrix) OPG_TRY(assemble(s, false));
    std::vector<std::vector<std::pair<long long, double>>> R;
    OPG_TRY(host_csr(s, R));
    long long total = 0;
    for (auto& row : R) total += (long long) row.size();
    *n_rows = s->n;
    *nnz = total;
    if (row_ptr) {
        long long k = 0;
        for (long long r = 0; r < s->n; ++r) {
            row_ptr[r] = k;
            for (auto& pr : R[(size_t) r]) {
                if (cols) cols[k] = pr.first;
                if (vals) vals[k] = pr.second;
                ++k;
            }
        }
        row_ptr[s->n] = k;
    }
    if (rhs) OPG_CUDA(cudaMemcpy(rhs, s->b, s->n * 8, cudaMemcpyDeviceToHost));
    return OPFLOW_OK;
}

int opflow_eqnset_destroy(opflow_eqnset s) {
    if (!s) return OPFLOW_OK;
    if (s->ctx) cudaStreamSynchronize(s->ctx->stream);
    release_mg(s);
    amg_free(s->ctx, &s->amg);
    release_matrix(s);
    krylov_work_free(s->W);
    s->arena.release();
    for (opflow_field z : s->zero) opflow_field_destroy(z);
    delete s;
    return OPFLOW_OK;
}

}  // extern "C"
