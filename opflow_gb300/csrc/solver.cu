// Path I, steps 2-3: the multigrid hierarchy and the flexible-PCG driver.
//
// Replaces HYPREEqnSolveHandler::solve with StructSolver<PCG> + StructSolver<PFMG>
// (src/Core/Equation/HYPREEqnSolveHandler.hpp:190-209, src/Core/Solvers/Struct/StructSolverPCG.hpp,
// StructSolverPFMG.hpp): a matrix-free geometric multigrid V-cycle preconditions a float64 flexible
// conjugate-gradient iteration.
//
// Coarse levels are rediscretisations of the user's own equation: the same `lhs - rhs` tree is
// assembled (StencilPad semantics) on a mesh of twice the spacing, with the known fields restricted
// (cell averages / node injection).  Levels whose coefficients depend only on the position class of a
// cell (first / interior / last per dim) keep a 27-entry table instead of per-cell arrays, so their
// smoothing sweeps read no coefficients from HBM.
//
// Precision forms: OPFLOW_PREC_FP64 runs the V-cycle in float64; OPFLOW_PREC_MIXED runs it (operator,
// smoother, residual, transfers) in float32 with float32 accumulation, while the outer residual, the
// solution update, the inner products and the coarsest dense solve stay float64.
//
// A singular system (pure Neumann / periodic: zero row sums) with pinValue is solved as the reference
// poses it: the pinned system equals the consistent singular system whose pinned-row right-hand side is
// replaced by minus the sum of the others, followed by a shift that makes the pinned unknown 0.
#include "solver.h"
#include "tune.h"

#include <cstdint>
#include <cstdio>
#include <cstdlib>

#include <chrono>
#include <cmath>
#include <algorithm>
#include <array>
#include <functional>
#include <map>
#include <string>

namespace opg {

// ================================================================================= small kernels
__global__ void gather_box(FieldView f, Box b, double* out) {
    const long long nx = b.hi[0] - b.lo[0], ny = b.hi[1] - b.lo[1], nz = b.hi[2] - b.lo[2];
    for (long long t = blockIdx.x * (long long) blockDim.x + threadIdx.x; t < nx * ny * nz; t += (long long) gridDim.x * blockDim.x) {
        int i, j, k;
        box_index(t, b, i, j, k);
        out[t] = f.data[(i - f.off[0]) + (j - f.off[1]) * f.sy + (k - f.off[2]) * f.sz];
    }
}
__global__ void scatter_box(FieldView f, Box b, const double* in, double shift) {
    const long long nx = b.hi[0] - b.lo[0], ny = b.hi[1] - b.lo[1], nz = b.hi[2] - b.lo[2];
    for (long long t = blockIdx.x * (long long) blockDim.x + threadIdx.x; t < nx * ny * nz; t += (long long) gridDim.x * blockDim.x) {
        int i, j, k;
        box_index(t, b, i, j, k);
        f.data[(i - f.off[0]) + (j - f.off[1]) * f.sy + (k - f.off[2]) * f.sz] = in[t] - shift;
    }
}
// restriction of a known field's data to a coarse field: cell averages along centre-located dims,
// injection along corner-located dims
__global__ void field_restrict(FieldView fine, FieldView coarse, Box cb, int loc0, int loc1, int loc2, int ndim) {
    const long long nx = cb.hi[0] - cb.lo[0], ny = cb.hi[1] - cb.lo[1], nz = cb.hi[2] - cb.lo[2];
    const int locs[3] = {loc0, loc1, loc2};
    for (long long t = blockIdx.x * (long long) blockDim.x + threadIdx.x; t < nx * ny * nz; t += (long long) gridDim.x * blockDim.x) {
        int I[3];
        box_index(t, cb, I[0], I[1], I[2]);
        double acc = 0.;
        int cnt = 0;
        for (int a = 0; a < 2; ++a)
            for (int b = 0; b < 2; ++b)
                for (int c = 0; c < 2; ++c) {
                    const int o[3] = {c, b, a};
                    int f[3];
                    bool ok = true;
                    for (int d = 0; d < 3; ++d) {
                        if (d >= ndim) { if (o[d]) ok = false; f[d] = 0; continue; }
                        if (locs[d] == OPFLOW_CORNER) { if (o[d]) ok = false; f[d] = 2 * I[d]; }
                        else f[d] = 2 * I[d] + o[d];
                        if (f[d] < fine.off[d] || f[d] >= fine.off[d] + fine.dims[d]) ok = false;
                    }
                    if (!ok) continue;
                    acc += fine.data[(f[0] - fine.off[0]) + (f[1] - fine.off[1]) * fine.sy + (f[2] - fine.off[2]) * fine.sz];
                    cnt++;
                }
        coarse.data[(I[0] - coarse.off[0]) + (I[1] - coarse.off[1]) * coarse.sy + (I[2] - coarse.off[2]) * coarse.sz] = cnt ? acc / cnt : 0.;
    }
}
// coefficients from the assembly's K order into the 7 slots; flags entries outside the slots
__global__ void map_slots(const double* coef, long long N, const int* kslot, int nk, double* A, int* bad) {
    for (long long t = blockIdx.x * (long long) blockDim.x + threadIdx.x; t < N; t += (long long) gridDim.x * blockDim.x) {
        for (int s = 0; s < NSLOT; ++s) A[s * N + t] = 0.;
        for (int k = 0; k < nk; ++k) {
            const double v = coef[k * N + t];
            const int s = kslot[k];
            if (s < 0) { if (v != 0.) atomicExch(bad, 1); }
            else A[s * N + t] += v;
        }
    }
}
__global__ void to_f32(const double* a, float* b, long long n) {
    for (long long t = blockIdx.x * (long long) blockDim.x + threadIdx.x; t < n; t += (long long) gridDim.x * blockDim.x) b[t] = (float) a[t];
}
// compare every cell's coefficients with its class representative
__global__ void class_check(const double* A, long long N, int n0, int n1, int n2, int ndim, const double* tab, int* bad) {
    for (long long t = blockIdx.x * (long long) blockDim.x + threadIdx.x; t < N; t += (long long) gridDim.x * blockDim.x) {
        Box b;
        b.lo[0] = b.lo[1] = b.lo[2] = 0;
        b.hi[0] = n0; b.hi[1] = n1; b.hi[2] = n2;
        int i, j, k;
        box_index(t, b, i, j, k);
        auto pc = [](int x, int n) { return x == 0 ? 0 : (x == n - 1 ? 2 : 1); };
        const int cls = pc(i, n0) + 3 * (ndim > 1 ? pc(j, n1) : 0) + 9 * (ndim > 2 ? pc(k, n2) : 0);
        for (int s = 0; s < NSLOT; ++s)
            if (__double_as_longlong(A[s * N + t]) != __double_as_longlong(tab[cls * NSLOT + s])) { atomicExch(bad, 1); return; }
    }
}
// max |row sum| and max |diag| (bit patterns of non-negative doubles)
__global__ void rowsum_stats(const double* A, long long N, int n0, int n1, int n2, int ndim, int p0, int p1, int p2, unsigned long long* out) {
    unsigned long long ms = 0, md = 0;
    for (long long t = blockIdx.x * (long long) blockDim.x + threadIdx.x; t < N; t += (long long) gridDim.x * blockDim.x) {
        Box b;
        b.lo[0] = b.lo[1] = b.lo[2] = 0;
        b.hi[0] = n0; b.hi[1] = n1; b.hi[2] = n2;
        int i, j, k;
        box_index(t, b, i, j, k);
        double s = A[t];
        const int idx[3] = {i, j, k}, n[3] = {n0, n1, n2}, per[3] = {p0, p1, p2};
        for (int d = 0; d < ndim; ++d) {
            if (idx[d] > 0 || per[d]) s += A[(1 + 2 * d) * N + t];
            if (idx[d] < n[d] - 1 || per[d]) s += A[(2 + 2 * d) * N + t];
        }
        const unsigned long long bs = (unsigned long long) __double_as_longlong(fabs(s)), bd = (unsigned long long) __double_as_longlong(fabs(A[t]));
        ms = bs > ms ? bs : ms;
        md = bd > md ? bd : md;
    }
    atomicMax(&out[0], ms);
    atomicMax(&out[1], md);
}
__global__ void sum_partials(const double* v, long long n, double* partial) {
    __shared__ double sh[256];
    double s = 0.;
    for (long long t = blockIdx.x * (long long) blockDim.x + threadIdx.x; t < n; t += (long long) gridDim.x * blockDim.x) s += v[t];
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if ((int) threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = sh[0];
}
__global__ void add_scalar(double* v, long long n, double a) {
    for (long long t = blockIdx.x * (long long) blockDim.x + threadIdx.x; t < n; t += (long long) gridDim.x * blockDim.x) v[t] += a;
}

// The singular right-hand side on the device, without a host round trip: sum[0] = the partial sums
// added in block order (as mg_sum adds them on the host); pinned: b[0] := -(sum - b[0]); else nothing
// (the projection follows in add_scaled_sum)
__global__ void singular_rhs(const double* partial, int nblk, double* b, int pinned, double* sum) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double s = 0.;
    for (int i = 0; i < nblk; ++i) s += partial[i];
    sum[0] = s;
    if (pinned) b[0] = -(s - b[0]);
}
// v += -(*sum) / n (the projection onto zero mean)
__global__ void add_scaled_sum(double* v, long long n, const double* sum) {
    const double a = -*sum / (double) n;
    for (long long t = blockIdx.x * (long long) blockDim.x + threadIdx.x; t < n; t += (long long) gridDim.x * blockDim.x) v[t] += a;
}
// x -= x[0] with x[0] first saved to *slot (so no thread reads it while another rewrites it)
__global__ void save_first(const double* x, double* slot) {
    if (threadIdx.x == 0 && blockIdx.x == 0) slot[0] = x[0];
}
__global__ void sub_slot(double* v, long long n, const double* slot) {
    const double a = -*slot;
    for (long long t = blockIdx.x * (long long) blockDim.x + threadIdx.x; t < n; t += (long long) gridDim.x * blockDim.x) v[t] += a;
}

static int gridN(opflow_ctx ctx, long long n) {
    long long b = (n + 255) / 256;
    return (int) std::max(1LL, std::min(b, (long long) ctx->num_sms * 16));
}

// ================================================================================= arena
void* Arena::alloc(size_t bytes) {
    bytes = (bytes + 255) & ~(size_t) 255;
    if (blocks.empty() || used + bytes > cap) {
        size_t sz = std::max(bytes, block_hint);
        block_hint = std::min(block_hint * 2, (size_t) 256 << 20);
        void* p = nullptr;
        if (ctx) p = dev_alloc(ctx, sz);
        else if (cudaMalloc(&p, sz) != cudaSuccess) p = nullptr;
        if (!p) return nullptr;
        blocks.push_back(p);
        cap = sz;
        used = 0;
    }
    void* r = (char*) blocks.back() + used;
    used += bytes;
    total += bytes;
    return r;
}
void Arena::release() {
    for (void* p : blocks) {
        if (ctx) dev_free(ctx, p);
        else cudaFree(p);
    }
    blocks.clear();
    cap = used = total = 0;
}

// ================================================================================= setup
static int ghost_rule(int bct) {
    switch (bct) {
        case OPFLOW_BC_DIRC: case OPFLOW_BC_ASYMM: return GH_ZERO;
        case OPFLOW_BC_PERIODIC: return GH_WRAP;
        default: return GH_COPY;
    }
}

// Assembles `tree` for `target` (leaves by slot) into level L: slot-ordered FP64 coefficients and,
// when rhs != nullptr, the right-hand side b = -bias.
static int assemble_level(MGSystem* S, opflow_field target, const std::vector<opflow_node>& tree, const std::vector<opflow_field>& leaves,
                          int unknown, LevelHost& L, double* rhs) {
    opflow_ctx ctx = S->ctx;
    AsmPlan plan;
    OPG_TRY(asm_prepare(ctx, target, tree.data(), (int) tree.size(), leaves.data(), (int) leaves.size(), unknown, 0, &plan));
    const long long N = plan.cells;
    const int nk = plan.P.nk;
    double *coef = nullptr, *tmp_rhs = nullptr;
    int* dks = nullptr;
    coef = (double*) dev_alloc(ctx, (size_t) N * nk * sizeof(double));
    if (!coef) return fail(OPFLOW_E_NOMEM, "assembly buffer");
    if (!rhs) {
        tmp_rhs = (double*) dev_alloc(ctx, (size_t) N * sizeof(double));
        if (!tmp_rhs) { dev_free(ctx, coef); return fail(OPFLOW_E_NOMEM, "assembly buffer"); }
    }
    int rc = asm_run(ctx, &plan, coef, rhs ? rhs : tmp_rhs);
    std::vector<int> ks(nk, -1);
    for (int k = 0; k < nk; ++k) {
        const int* o = plan.P.K[k];
        int nz = 0, d = -1;
        for (int q = 0; q < 3; ++q)
            if (o[q]) { nz++; d = q; }
        if (nz == 0) ks[k] = 0;
        else if (nz == 1 && std::abs(o[d]) == 1) ks[k] = 1 + 2 * d + (o[d] > 0 ? 1 : 0);
    }
    if (rc == OPFLOW_OK) {
        L.A64 = (double*) S->arena.alloc((size_t) NSLOT * N * sizeof(double));
        if (!L.A64) rc = fail(OPFLOW_E_NOMEM, "operator arrays");
    }
    if (rc == OPFLOW_OK) {
        dks = (int*) dev_alloc(ctx, nk * sizeof(int));
        if (!dks) return fail(OPFLOW_E_NOMEM, "slot map");
        cudaMemcpyAsync(dks, ks.data(), nk * sizeof(int), cudaMemcpyHostToDevice, ctx->stream);
        int* bad = (int*) ctx->scratch;
        cudaMemsetAsync(bad, 0, sizeof(int), ctx->stream);
        map_slots<<<gridN(ctx, N), 256, 0, ctx->stream>>>(coef, N, dks, nk, L.A64, bad);
        OPG_LAUNCHED();
        int hb = 0;
        cudaMemcpyAsync(&hb, bad, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream);
        cudaStreamSynchronize(ctx->stream);
        if (hb) rc = fail(OPFLOW_E_UNSUPPORTED, "the equation's stencil has entries beyond the (2*dim+1)-point star the multigrid handles");
    }
    dev_free(ctx, coef);
    if (tmp_rhs) dev_free(ctx, tmp_rhs);
    if (dks) dev_free(ctx, dks);
    if (rc) return rc;
    const Box b = plan.P.box;
    L.ndim = target->info.ndim;
    L.N = N;
    for (int d = 0; d < 3; ++d) {
        L.n[d] = b.hi[d] - b.lo[d];
        L.lo[d] = b.lo[d];
        L.per[d] = d < L.ndim && target->desc.bc_type[d][0] == OPFLOW_BC_PERIODIC;
        L.gh_lo[d] = ghost_rule(target->desc.bc_type[d][0]);
        L.gh_hi[d] = ghost_rule(target->desc.bc_type[d][1]);
    }
    return OPFLOW_OK;
}

// gathers the coefficients of the class representatives: tab[cls][slot] = A[slot][rep[cls]]
__global__ void gather_classes(const double* A, long long N, const long long* rep, double* tab) {
    const int t = threadIdx.x;
    if (t < NCLASS * NSLOT) {
        const int cls = t / NSLOT, s = t % NSLOT;
        tab[t] = rep[cls] >= 0 ? A[s * N + rep[cls]] : 0.;
    }
}

// Position-class table if every cell matches its class representative exactly.
static int compress_level(MGSystem* S, LevelHost& L) {
    opflow_ctx ctx = S->ctx;
    const long long N = L.N;
    std::vector<long long> rep(NCLASS, -1);
    auto rp = [&](int c, int n) { return c == 0 ? 0 : (c == 1 ? std::min(1, n - 1) : n - 1); };
    for (int cz = 0; cz < 3; ++cz)
        for (int cy = 0; cy < 3; ++cy)
            for (int cx = 0; cx < 3; ++cx) {
                if ((L.ndim < 2 && cy) || (L.ndim < 3 && cz)) continue;
                const int i = rp(cx, L.n[0]), j = L.ndim > 1 ? rp(cy, L.n[1]) : 0, k = L.ndim > 2 ? rp(cz, L.n[2]) : 0;
                rep[cx + 3 * cy + 9 * cz] = i + (long long) L.n[0] * (j + (long long) L.n[1] * k);
            }
    double* dtab = (double*) S->arena.alloc(NCLASS * NSLOT * sizeof(double));
    long long* drep = (long long*) ((char*) ctx->scratch + 2048);
    if (!dtab) return fail(OPFLOW_E_NOMEM, "class table");
    cudaMemcpyAsync(drep, rep.data(), NCLASS * sizeof(long long), cudaMemcpyHostToDevice, ctx->stream);
    gather_classes<<<1, 256, 0, ctx->stream>>>(L.A64, N, drep, dtab);
    OPG_LAUNCHED();
    int* bad = (int*) ctx->scratch;
    cudaMemsetAsync(bad, 0, sizeof(int), ctx->stream);
    class_check<<<gridN(ctx, N), 256, 0, ctx->stream>>>(L.A64, N, L.n[0], L.n[1], L.n[2], L.ndim, dtab, bad);
    OPG_LAUNCHED();
    std::vector<double> tab(NCLASS * NSLOT);
    int hb = 0;
    cudaMemcpyAsync(tab.data(), dtab, tab.size() * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream);
    cudaMemcpyAsync(&hb, bad, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream);
    OPG_CUDA(cudaStreamSynchronize(ctx->stream));
    // kernel tables: rows of TSTRIDE with the inverse of the centre coefficient appended
    std::vector<double> t8(NCLASS * TSTRIDE, 0.);
    std::vector<float> t8f(NCLASS * TSTRIDE, 0.f);
    for (int c = 0; c < NCLASS; ++c) {
        for (int q = 0; q < NSLOT; ++q) {
            t8[c * TSTRIDE + q] = tab[c * NSLOT + q];
            t8f[c * TSTRIDE + q] = (float) tab[c * NSLOT + q];
        }
        const double c0 = tab[c * NSLOT];
        const float c0f = (float) c0;
        t8[c * TSTRIDE + NSLOT] = c0 != 0. ? 1.0 / c0 : 0.;
        t8f[c * TSTRIDE + NSLOT] = c0f != 0.f ? 1.0f / c0f : 0.f;
    }
    double* dt8 = (double*) S->arena.alloc(NCLASS * TSTRIDE * sizeof(double));
    float* dt8f = (float*) S->arena.alloc(NCLASS * TSTRIDE * sizeof(float));
    if (!dt8 || !dt8f) return fail(OPFLOW_E_NOMEM, "class table");
    cudaMemcpyAsync(dt8, t8.data(), t8.size() * sizeof(double), cudaMemcpyHostToDevice, ctx->stream);
    cudaMemcpyAsync(dt8f, t8f.data(), t8f.size() * sizeof(float), cudaMemcpyHostToDevice, ctx->stream);
    L.T64 = dt8;
    L.T32 = dt8f;
    L.table = hb == 0;
    L.tab = tab;
    if (!L.table) {
        L.A32 = (float*) S->arena.alloc((size_t) NSLOT * N * sizeof(float));
        if (!L.A32) return fail(OPFLOW_E_NOMEM, "float32 operator");
        to_f32<<<gridN(ctx, NSLOT * N), 256, 0, ctx->stream>>>(L.A64, L.A32, NSLOT * N);
        OPG_LAUNCHED();
    }
    OPG_CUDA(cudaStreamSynchronize(ctx->stream));  // t8 / t8f must outlive their copies
    return OPFLOW_OK;
}

// Dense (pseudo-)inverse of the coarsest operator, on the host (N <= a few hundred).
static int coarse_inverse(MGSystem* S, LevelHost& L, bool singular) {
    const int N = (int) L.N;
    std::vector<double> A((size_t) N * N, 0.), coefs((size_t) NSLOT * N);
    OPG_CUDA(cudaMemcpy(coefs.data(), L.A64, coefs.size() * sizeof(double), cudaMemcpyDeviceToHost));
    for (int c = 0; c < N; ++c) {
        const int i = c % L.n[0], j = (c / L.n[0]) % L.n[1], k = c / (L.n[0] * L.n[1]);
        const int idx[3] = {i, j, k};
        A[(size_t) c * N + c] += coefs[c];
        for (int d = 0; d < L.ndim; ++d)
            for (int sd = 0; sd < 2; ++sd) {
                int nb[3] = {i, j, k};
                nb[d] += sd ? 1 : -1;
                if (nb[d] < 0 || nb[d] >= L.n[d]) {
                    if (!L.per[d]) continue;
                    nb[d] = (nb[d] + L.n[d]) % L.n[d];
                }
                (void) idx;
                const int cn = nb[0] + L.n[0] * (nb[1] + L.n[1] * nb[2]);
                A[(size_t) c * N + cn] += coefs[(size_t) (1 + 2 * d + sd) * N + c];
            }
    }
    // singular: pin unknown 0 (row and column), invert the rest
    const int off = singular ? 1 : 0;
    const int M = N - off;
    std::vector<double> B((size_t) M * M), Inv((size_t) M * M, 0.);
    for (int r = 0; r < M; ++r)
        for (int c = 0; c < M; ++c) B[(size_t) r * M + c] = A[(size_t) (r + off) * N + (c + off)];
    for (int r = 0; r < M; ++r) Inv[(size_t) r * M + r] = 1.;
    // Gauss-Jordan with partial pivoting
    for (int col = 0; col < M; ++col) {
        int piv = col;
        for (int r = col + 1; r < M; ++r)
            if (std::fabs(B[(size_t) r * M + col]) > std::fabs(B[(size_t) piv * M + col])) piv = r;
        if (B[(size_t) piv * M + col] == 0.) return fail(OPFLOW_E_INVALID, "singular coarsest operator");
        if (piv != col)
            for (int c = 0; c < M; ++c) {
                std::swap(B[(size_t) piv * M + c], B[(size_t) col * M + c]);
                std::swap(Inv[(size_t) piv * M + c], Inv[(size_t) col * M + c]);
            }
        const double d = B[(size_t) col * M + col];
        for (int c = 0; c < M; ++c) { B[(size_t) col * M + c] /= d; Inv[(size_t) col * M + c] /= d; }
        for (int r = 0; r < M; ++r) {
            if (r == col) continue;
            const double f = B[(size_t) r * M + col];
            if (f == 0.) continue;
            for (int c = 0; c < M; ++c) {
                B[(size_t) r * M + c] -= f * B[(size_t) col * M + c];
                Inv[(size_t) r * M + c] -= f * Inv[(size_t) col * M + c];
            }
        }
    }
    std::vector<double> Full((size_t) N * N, 0.);
    for (int r = 0; r < M; ++r)
        for (int c = 0; c < M; ++c) Full[(size_t) (r + off) * N + (c + off)] = Inv[(size_t) r * M + c];
    L.Ainv64 = (double*) S->arena.alloc(Full.size() * sizeof(double));
    if (!L.Ainv64) return fail(OPFLOW_E_NOMEM, "coarse inverse");
    OPG_CUDA(cudaMemcpy(L.Ainv64, Full.data(), Full.size() * sizeof(double), cudaMemcpyHostToDevice));
    return OPFLOW_OK;
}

// Coarse mesh of the same extent: half the cells (centre) or every other node (corner).
static bool coarse_mesh(const MeshDev* m, const opflow_field_desc& desc, std::vector<std::vector<double>>& xs, std::vector<std::vector<double>>& dxs,
                        opflow_mesh_desc* out) {
    std::memset(out, 0, sizeof *out);
    out->ndim = m->ndim;
    out->pad_width = m->n[0] > 0 ? (int) ((m->n[0] - (int) m->hx[0].size()) / 2) : 0;
    const int pad = (int) (m->hx[0].size() - 0);
    (void) pad;
    xs.assign(m->ndim, {});
    dxs.assign(m->ndim, {});
    for (int d = 0; d < m->ndim; ++d) {
        const int pw = -m->es[d];  // meshes built with start 0: es = -pad_width
        const int nodes = (int) m->hx[d].size() - 2 * pw;
        int nodes_c;
        if (desc.loc[d] == OPFLOW_CENTER) {
            const int cells = nodes - 1;
            if (cells < 4) return false;
            nodes_c = (cells + 1) / 2 + 1;
        } else {
            if (nodes < 5 || (nodes % 2) == 0) return false;
            nodes_c = (nodes + 1) / 2;
        }
        const double x0 = m->hx[d][pw], x1 = m->hx[d][pw + nodes - 1];
        xs[d].resize(nodes_c + 2 * pw);
        dxs[d].resize(nodes_c + 2 * pw - 1);
        opflow_mesh_uniform(nodes_c, 0, pw, x0, x1, xs[d].data(), dxs[d].data());
        out->dims[d] = nodes_c;
        out->start[d] = 0;
        out->x[d] = xs[d].data();
        out->dx[d] = dxs[d].data();
        out->pad_width = pw;
    }
    return true;
}

static void release_level_fields(LevelHost& L) {
    for (auto f : L.owned) opflow_field_destroy(f);
    L.owned.clear();
}

int mg_add_problem(MGSystem* S, opflow_field target, const opflow_node* nodes, int n_nodes, const opflow_field* leaves, int n_leaves,
                   int unknown) {
    opflow_ctx ctx = S->ctx;
    OPG_TRY(ensure_scratch(ctx, 4096));
    ProblemHost P;
    P.target = target;
    P.tree.assign(nodes, nodes + n_nodes);
    P.leaves.assign(leaves, leaves + n_leaves);
    P.unknown = unknown;
    for (int d = 0; d < target->info.ndim; ++d)
        if (target->desc.bc_type[d][0] == OPFLOW_BC_DIRC || target->desc.bc_type[d][1] == OPFLOW_BC_DIRC) P.has_dirichlet = true;
    // level 0
    LevelHost L0;
    const Box box = assign_box(target->info);
    const long long N0 = box.count();
    if (N0 <= 0) return fail(OPFLOW_E_INVALID, "the target has no unknowns");
    P.b = (double*) S->arena.alloc(N0 * sizeof(double));
    if (!P.b) return fail(OPFLOW_E_NOMEM, "right-hand side");
    OPG_TRY(assemble_level(S, target, P.tree, P.leaves, unknown, L0, P.b));
    bool uniform_loc = true;
    for (int d = 1; d < target->info.ndim; ++d) uniform_loc = uniform_loc && target->desc.loc[d] == target->desc.loc[0];
    L0.node = target->desc.loc[0] == OPFLOW_CORNER;
    P.levels.push_back(L0);
    // singularity: zero row sums
    {
        unsigned long long* st = (unsigned long long*) ctx->scratch + 8;
        cudaMemsetAsync(st, 0, 2 * sizeof(unsigned long long), ctx->stream);
        const LevelHost& L = P.levels[0];
        rowsum_stats<<<gridN(ctx, L.N), 256, 0, ctx->stream>>>(L.A64, L.N, L.n[0], L.n[1], L.n[2], L.ndim, L.per[0], L.per[1], L.per[2], st);
        OPG_LAUNCHED();
        unsigned long long h[2];
        cudaMemcpyAsync(h, st, sizeof h, cudaMemcpyDeviceToHost, ctx->stream);
        OPG_CUDA(cudaStreamSynchronize(ctx->stream));
        double ms, md;
        std::memcpy(&ms, &h[0], 8);
        std::memcpy(&md, &h[1], 8);
        P.singular = ms <= 1e-10 * md;
    }
    // coarser levels by rediscretisation
    opflow_field cur_target = target;
    std::vector<opflow_field> cur_leaves = P.leaves;
    while (uniform_loc && (long long) P.levels.back().N > S->coarse_max && (int) P.levels.size() < 24) {
        std::vector<std::vector<double>> xs, dxs;
        opflow_mesh_desc cm;
        if (!coarse_mesh(cur_target->mesh, cur_target->desc, xs, dxs, &cm)) break;
        LevelHost Lc;
        std::vector<opflow_field> nl(cur_leaves.size(), nullptr);
        opflow_field ct = nullptr;
        int rc = OPFLOW_OK;
        for (size_t s = 0; s < cur_leaves.size() && rc == OPFLOW_OK; ++s) {
            if (cur_leaves[s] == cur_target && ct) { nl[s] = ct; continue; }
            opflow_field f = nullptr;
            rc = opflow_field_create(ctx, &cm, &cur_leaves[s]->desc, &f);
            if (rc) break;
            Lc.owned.push_back(f);
            nl[s] = f;
            if (cur_leaves[s] == cur_target) ct = f;
            else {
                const Box cb = assign_box(f->info);
                Box all = cb;
                for (int d = 0; d < 3; ++d) { all.lo[d] = f->info.local[d][0]; all.hi[d] = f->info.local[d][1]; }
                field_restrict<<<gridN(ctx, all.count()), 256, 0, ctx->stream>>>(cur_leaves[s]->view(), f->view(), all, f->desc.loc[0], f->desc.loc[1],
                                                                                  f->desc.loc[2], f->info.ndim);
                OPG_LAUNCHED();
                rc = update_padding_buf(f, f->buf[f->cur]);
            }
        }
        if (rc == OPFLOW_OK && !ct) rc = fail(OPFLOW_E_INVALID, "the target is not among the leaves");
        if (rc == OPFLOW_OK) rc = assemble_level(S, ct, P.tree, nl, unknown, Lc, nullptr);
        if (rc) {
            release_level_fields(Lc);
            for (auto& L : P.levels) release_level_fields(L);
            return rc;
        }
        Lc.node = P.levels[0].node;
        P.levels.push_back(Lc);
        cur_target = ct;
        cur_leaves = nl;
    }
    for (auto& L : P.levels) OPG_TRY(compress_level(S, L));
    // coarsest: direct solve when small enough, else smoothing only
    LevelHost& Lc = P.levels.back();
    if (Lc.N <= std::max(S->coarse_max, 64)) OPG_TRY(coarse_inverse(S, Lc, P.singular && !P.has_dirichlet));
    S->probs.push_back(std::move(P));
    return OPFLOW_OK;
}

// Vectors, device descriptors and chunk lists for every problem added.
static int smooth_z_level(MGSystem* S, int l, int color, const Scal* sc, int zb);
int mg_check_error(MGSystem* S);

// zt_full: per level, whether the staged smoother's tiles cover every level index the z tiles cover
static void zt_coverage(MGSystem* S) {
    S->zt_full.assign(S->nlevels, 0);
    for (int l = 0; l < S->nlevels; ++l) {
        if (S->zt_ch[l].empty()) continue;
        std::vector<int> a, b;
        for (const Chunk& c : S->zsm_ch[l]) a.push_back(c.lvl);
        for (const Chunk& c : S->zt_ch[l]) b.push_back(c.lvl);
        std::sort(a.begin(), a.end());
        a.erase(std::unique(a.begin(), a.end()), a.end());
        std::sort(b.begin(), b.end());
        b.erase(std::unique(b.begin(), b.end()), b.end());
        S->zt_full[l] = a == b;
    }
}

// Device time (ms) of `launch`, run once to warm up and once timed on the system's stream; negative
// when a launch fails.
static float time_launch(MGSystem* S, const std::function<int()>& launch) {
    cudaStream_t s = S->ctx->stream;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    float ms = -1.f;
    if (cudaEventCreate(&e0) == cudaSuccess && cudaEventCreate(&e1) == cudaSuccess && launch() == OPFLOW_OK &&
        cudaEventRecord(e0, s) == cudaSuccess && launch() == OPFLOW_OK && cudaEventRecord(e1, s) == cudaSuccess &&
        cudaEventSynchronize(e1) == cudaSuccess)
        cudaEventElapsedTime(&ms, e0, e1);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    return ms;
}

static std::string level_key(const char* kernel, const MGSystem* S, int l) {
    char buf[160];
    const bool f32 = S->precision == OPFLOW_PREC_MIXED;
    if (S->probs.size() == 1) {
        const LevelHost& H = S->probs[0].levels[l];
        std::snprintf(buf, sizeof buf, "%s/%s/%dx%dx%d/%s/%d,%d", kernel, f32 ? "f32" : "f64", H.n[0], H.ndim > 1 ? H.n[1] : 1,
                      H.ndim > 2 ? H.n[2] : 1, H.node ? "node" : "cell", S->pre, S->post);
    } else {
        long long cells = 0;
        for (const auto& P : S->probs)
            if (l < (int) P.levels.size()) cells += P.levels[l].N;
        std::snprintf(buf, sizeof buf, "%s/%s/batch%zu/%lld/%d/%d,%d", kernel, f32 ? "f32" : "f64", S->probs.size(), cells,
                      (int) S->zsm_ch[l].size(), S->pre, S->post);
    }
    return buf;
}

// The tuner's choices for a finalized system (tune.h): the plane batch of every z-marching level and,
// on single-problem systems, the 2D tile shape of every tiled level, each timed on the level itself.
// The level vectors are zeroed first; every V-cycle rewrites them before reading them.
static int tune_levels(MGSystem* S) {
    if (!tune_enabled()) return OPFLOW_OK;
    bool any = false;
    for (int l = 0; l < S->nlevels; ++l) any = any || S->d_zsm[l].n > 0 || !S->tile_alt[l].empty();
    if (!any) return OPFLOW_OK;
    opflow_ctx ctx = S->ctx;
    const int sms = ctx->num_sms;
    const bool f32 = S->precision == OPFLOW_PREC_MIXED;
    const size_t es = f32 ? 4 : 8;
    auto choose = [&](const std::string& key, const std::vector<int>& cands, const std::function<float(int)>& time_ms) {
        return S->tune_measure ? tune_pick(key, cands, time_ms) : tune_cached(key, cands);
    };
    for (const LvlDev& D : S->lv_host) {
        if (!S->tune_measure) break;
        void* v[3] = {f32 ? (void*) D.x32 : (void*) D.x64, f32 ? (void*) D.b32 : (void*) D.b64, f32 ? (void*) D.r32 : (void*) D.r64};
        for (void* p : v)
            if (p) OPG_CUDA(cudaMemsetAsync(p, 0, (size_t) D.N * es, ctx->stream));
    }
    for (int l = 0; l < S->nlevels; ++l) {
        const ChunkList& Z = S->d_zsm[l];
        if (Z.n > 0) {
            std::vector<int> cands = {4, 2, 8};
            if (S->d_zt[l].n > 0 && S->zt_full[l]) cands.push_back(MG_ZB_TMA);
            S->zb[l] = choose(level_key("mg_smooth_z", S, l), cands, [&](int zb) {
                return time_launch(S, [&] {
                    OPG_TRY(smooth_z_level(S, l, 0, nullptr, zb));
                    return smooth_z_level(S, l, 1, nullptr, zb);
                });
            });
        }
        if (!S->tile_alt[l].empty()) {
            // candidate 0: the list built (the shape the SM-fill rule picked), 1: the other shape
            ChunkList alt{};
            const int pick = choose(level_key("mg_tile", S, l), {0, 1}, [&](int cand) {
                if (cand == 1 && !alt.ptr) {
                    alt.n = (int) S->tile_alt[l].size();
                    alt.ptr = (Chunk*) S->arena.alloc(S->tile_alt[l].size() * sizeof(Chunk));
                    if (!alt.ptr) return -1.f;
                    cudaMemcpyAsync(alt.ptr, S->tile_alt[l].data(), S->tile_alt[l].size() * sizeof(Chunk), cudaMemcpyHostToDevice, ctx->stream);
                }
                const ChunkList& T = cand ? alt : S->d_tiles[l];
                return time_launch(S, [&] {
                    OPG_TRY(mg_launch_tile_down(ctx->stream, sms, f32, S->dL, T.ptr, T.n, nullptr, S->pre));
                    return mg_launch_tile_up(ctx->stream, sms, f32, S->dL, T.ptr, T.n, nullptr, S->post);
                });
            });
            if (pick == 1) {
                if (!alt.ptr) {  // a cached choice: the list is uploaded now
                    alt.n = (int) S->tile_alt[l].size();
                    alt.ptr = (Chunk*) S->arena.alloc(S->tile_alt[l].size() * sizeof(Chunk));
                    if (!alt.ptr) return fail(OPFLOW_E_NOMEM, "tile list");
                    OPG_CUDA(cudaMemcpyAsync(alt.ptr, S->tile_alt[l].data(), S->tile_alt[l].size() * sizeof(Chunk), cudaMemcpyHostToDevice, ctx->stream));
                }
                S->tile_ch[l].swap(S->tile_alt[l]);
                S->d_tiles[l] = alt;
            }
            S->tile_alt[l].clear();
        }
    }
    OPG_CUDA(cudaStreamSynchronize(ctx->stream));
    return OPFLOW_OK;
}

int mg_finalize(MGSystem* S) {
    opflow_ctx ctx = S->ctx;
    const bool f32 = S->precision == OPFLOW_PREC_MIXED;
    std::vector<LvlDev> lv;
    std::vector<KrylovDev> kd;
    S->nlevels = 0;
    for (auto& P : S->probs) S->nlevels = std::max(S->nlevels, (int) P.levels.size());
    S->smooth_ch.assign(S->nlevels, {});
    S->restrict_ch.assign(S->nlevels, {});
    S->prolong_ch.assign(S->nlevels, {});
    S->tile_ch.assign(S->nlevels, {});
    S->zsm_ch.assign(S->nlevels, {});
    S->zb.assign(S->nlevels, 4);
    S->tile_alt.assign(S->nlevels, {});
    S->zt_ch.assign(S->nlevels, {});
    std::map<int, std::array<CUtensorMap, 2>> zt_maps;  // by level index
    S->coarse_sm_ch.clear();
    S->bottom_host.clear();
    S->bottom_cells_host.clear();
    OPG_TRY(mg_bottom_prepare());
    const char* te = getenv("OPFLOW_MG_TILES");
    // tiles for the float32 V-cycle only: the float64 one is bound by float64 issue, where the halo's
    // repeated sweeps cost more than the saved passes over memory (measured)
    bool tiles_on = f32 && !(te && te[0] == '0') && mg_tiles_supported(S->pre) && mg_tiles_supported(S->post);
    if (tiles_on) OPG_TRY(mg_tiles_prepare(std::max(S->pre, S->post)));
    const char* ze = getenv("OPFLOW_MG_ZMARCH");
    const bool zoff = ze && ze[0] == '0';
    std::vector<int> coarse_list;
    std::vector<Chunk> k0;
    std::vector<int> first, count;
    // V-cycle chunks: rows of at least CH cells are split into segments of CH; shorter rows are grouped,
    // whole rows of one plane, into chunks of about CH2 cells (one warp per row in the kernels), as far
    // as the level still has two chunks per SM (a level of few rows keeps one row per chunk)
    const int CH = 1024, CH2 = 2048;
    auto rows = [&](int lvl_index, const LvlDev& L, std::vector<Chunk>& out) {
        const int ny = L.ndim > 1 ? L.n[1] : 1, nz = L.ndim > 2 ? L.n[2] : 1;
        if (L.n[0] >= CH) {
            for (int k = 0; k < nz; ++k)
                for (int j = 0; j < ny; ++j)
                    for (int i0 = 0; i0 < L.n[0]; i0 += CH) out.push_back(Chunk{lvl_index, j, k, i0, std::min(CH, L.n[0] - i0)});
            return;
        }
        const long long all_rows = (long long) ny * nz;
        const int per = (int) std::max<long long>(1, std::min<long long>(CH2 / L.n[0], all_rows / (2LL * ctx->num_sms)));
        for (int k = 0; k < nz; ++k)
            for (int j = 0; j < ny; j += per) {
                Chunk c{lvl_index, j, k, 0, L.n[0]};
                c.nrows = std::min(per, ny - j);
                out.push_back(c);
            }
    };
    if (const char* e = getenv("OPFLOW_MG_BOTTOM")) S->bottom_max = atoll(e);
    // level-0 chunks of the Krylov kernels: whole rows of one plane, about KCH cells each (rows longer
    // than KCH are split), so the per-chunk reduction and its barriers are amortised over many cells.
    // KCH is 8192 for problems of at least 8192 cells per two SMs and halves (down to 1024) for smaller
    // ones, so that a small problem alone still spreads over many SMs; it depends on the problem's size
    // only, so a problem is chunked alike alone and in any batch.
    auto krylov_chunks = [&](int lvl_index, const LvlDev& L, std::vector<Chunk>& out) {
        const long long per_two_sms = L.N / std::max(1, (ctx->num_sms + 1) / 2);
        int KCH = 8192;
        while (KCH > 1024 && KCH > per_two_sms) KCH /= 2;
        const int ny = L.ndim > 1 ? L.n[1] : 1, nz = L.ndim > 2 ? L.n[2] : 1;
        if (L.n[0] >= KCH) {
            for (int k = 0; k < nz; ++k)
                for (int j = 0; j < ny; ++j)
                    for (int i0 = 0; i0 < L.n[0]; i0 += KCH) out.push_back(Chunk{lvl_index, j, k, i0, std::min(KCH, L.n[0] - i0)});
            return;
        }
        const int per = std::max(1, KCH / L.n[0]);
        for (int k = 0; k < nz; ++k)
            for (int j = 0; j < ny; j += per) {
                Chunk c{lvl_index, j, k, 0, L.n[0]};
                c.nrows = std::min(per, ny - j);
                out.push_back(c);
            }
    };
    for (size_t p = 0; p < S->probs.size(); ++p) {
        ProblemHost& P = S->probs[p];
        const int base = (int) lv.size();
        // first level small enough for the one-CTA bottom kernel (levels.size(): none)
        size_t sp = P.levels.size();
        for (size_t l = 0; l < P.levels.size(); ++l)
            if (P.levels[l].N <= S->bottom_max) { sp = l; break; }
        long long bcells = 0;
        for (size_t l = sp; l < P.levels.size(); ++l) bcells += P.levels[l].N;
        if (bcells > MG_BOTTOM_CELLS || P.levels.size() - sp > (size_t) MG_BOTTOM_LEVELS) sp = P.levels.size();  // chunked instead
        // 2D red-black class-table levels above the bottom whose coarse cells all have children in the
        // level run as fused tiles
        auto tileable = [&](size_t l) {
            if (!tiles_on || l >= sp || l + 1 >= P.levels.size()) return false;
            const LevelHost& F = P.levels[l];
            const LevelHost& Cn = P.levels[l + 1];
            if (F.ndim != 2 || !F.table) return false;
            for (int d = 0; d < 2; ++d) {
                if (F.per[d] && (F.n[d] & 1)) return false;  // damped Jacobi level
                if (Cn.node) {
                    if (2 * Cn.lo[d] - F.lo[d] < 0 || 2 * (Cn.lo[d] + Cn.n[d] - 1) - F.lo[d] > F.n[d] - 1) return false;
                } else if (Cn.n[d] != (F.n[d] + 1) / 2) {
                    return false;
                }
            }
            return true;
        };
        for (size_t l = 0; l < P.levels.size(); ++l) {
            LevelHost& H = P.levels[l];
            LvlDev D{};
            D.ndim = H.ndim;
            for (int d = 0; d < 3; ++d) {
                D.n[d] = d < H.ndim ? H.n[d] : 1;
                D.lo[d] = d < H.ndim ? H.lo[d] : 0;
                D.per[d] = H.per[d];
                D.gh_lo[d] = H.gh_lo[d];
                D.gh_hi[d] = H.gh_hi[d];
            }
            D.N = H.N;
            D.node = H.node;
            D.table = H.table;
            bool odd_periodic = false;
            for (int d = 0; d < H.ndim; ++d) odd_periodic = odd_periodic || (H.per[d] && (H.n[d] & 1));
            D.rbgs = !odd_periodic;
            D.problem = (int) p;
            D.coarsest = l + 1 == P.levels.size();
            D.nslot = 2 * H.ndim + 1;
            D.A64 = H.A64;
            D.A32 = H.A32;
            D.T64 = H.T64;
            D.T32 = H.T32;
            D.coarse = D.coarsest ? -1 : base + (int) l + 1;
            D.fine = l == 0 ? -1 : base + (int) l - 1;
            D.tiled = tileable(l) ? 1 : 0;
            D.Ainv64 = H.Ainv64;
            const size_t N = (size_t) H.N;
            if (f32) {
                D.x32 = (float*) S->arena.alloc(N * 4);
                D.b32 = (float*) S->arena.alloc(N * 4);
                D.r32 = (float*) S->arena.alloc(N * 4);
                if (!D.x32 || !D.b32 || !D.r32) return fail(OPFLOW_E_NOMEM, "level vectors");
            } else {
                D.x64 = (double*) S->arena.alloc(N * 8);
                D.b64 = (double*) S->arena.alloc(N * 8);
                D.r64 = (double*) S->arena.alloc(N * 8);
                if (!D.x64 || !D.b64 || !D.r64) return fail(OPFLOW_E_NOMEM, "level vectors");
            }
            lv.push_back(D);
            const int li = base + (int) l;
            if (l == sp) {
                S->bottom_host.push_back(li);
                S->bottom_cells_host.push_back(bcells);
            }
            if (l >= sp) continue;                                   // inside the bottom kernel
            const bool above_tiled = l > 0 && tileable(l - 1);      // restricted by the finer level's tiles
            if (D.tiled) {
                // 54 x 32 tiles, or 22 x 16 where that would leave SMs idle (tile extent: cnt x nrows);
                // a single-problem system also keeps the other shape for the tuner
                const bool small = (long long) ((D.n[0] + MG_TILE_X - 1) / MG_TILE_X) * ((D.n[1] + MG_TILE_Y - 1) / MG_TILE_Y) < 2LL * ctx->num_sms;
                auto tiles = [&](bool sm, std::vector<Chunk>& out) {
                    const int tx = sm ? MG_TILE_X_SMALL : MG_TILE_X, ty = sm ? MG_TILE_Y / 2 : MG_TILE_Y;
                    for (int j0 = 0; j0 < D.n[1]; j0 += ty)
                        for (int i0 = 0; i0 < D.n[0]; i0 += tx) {
                            Chunk c{li, j0, 0, i0, tx};
                            c.nrows = ty;
                            out.push_back(c);
                        }
                };
                tiles(small, S->tile_ch[l]);
                if (S->probs.size() == 1 && tune_enabled()) tiles(!small, S->tile_alt[l]);
            } else {
                const bool zmarch = !zoff && D.ndim == 3 && D.table && D.rbgs && !D.coarsest && D.N >= MG_ZT_MIN && D.n[0] >= 3 && D.n[1] >= 3 &&
                                    D.n[2] >= 3;
                // planes per tile: up to MG_ZT_Z, fewer where the level would otherwise have fewer than
                // four tiles per SM (a short march leaves SMs idle); below 4 planes the chunked kernel
                const long long txy = (long long) ((D.n[0] + MG_ZT_X - 1) / MG_ZT_X) * ((D.n[1] + MG_ZT_Y - 1) / MG_ZT_Y);
                // (even, so that the prolongation's tiles start on whole coarse planes)
                const int zz = (int) std::min<long long>(MG_ZT_Z, (long long) D.n[2] * txy / (4LL * ctx->num_sms)) & ~1;
                const bool ztiles = zmarch && zz >= 4;
                if (ztiles) {
                    for (int k0 = 0; k0 < D.n[2]; k0 += zz)
                        for (int j0 = 0; j0 < D.n[1]; j0 += MG_ZT_Y)
                            for (int i0 = 0; i0 < D.n[0]; i0 += MG_ZT_X) {
                                Chunk c{li, j0, k0, i0, MG_ZT_X};
                                c.nrows = std::min(zz, D.n[2] - k0);
                                S->zsm_ch[l].push_back(c);
                            }
                    // the TMA-staged smoother's tiles: 16-byte aligned rows (float32, a multiple of 4 cells)
                    CUtensorMap two[2];
                    if (f32 && D.n[0] % 4 == 0 && !D.per[0] && !D.per[1] && !D.per[2] && (reinterpret_cast<uintptr_t>(D.x32) & 15) == 0 &&
                        (reinterpret_cast<uintptr_t>(D.b32) & 15) == 0 && mg_encode_zt_maps(D, two) == OPFLOW_OK) {
                        zt_maps[li] = {two[0], two[1]};
                        // planes per tile: the kernel's grid is one wave of resident CTAs striding over
                        // the tiles, so a half sweep takes about (rounds of tiles) x (planes per tile + the
                        // two halo planes); the run count along z that minimises it (at most
                        // MG_ZT2_Z planes per tile); OPFLOW_MG_ZT_PLANES for sweeps
                        const long long txy2 = (long long) ((D.n[0] + MG_ZT2_X - 1) / MG_ZT2_X) * ((D.n[1] + MG_ZT2_Y - 1) / MG_ZT2_Y);
                        const long long R = mg_zt_resident(ctx->num_sms);
                        int zz2 = MG_ZT2_Z;
                        long long best = -1;
                        for (int runs = 1; runs <= D.n[2]; ++runs) {
                            const int zz = (D.n[2] + runs - 1) / runs;
                            if (zz > MG_ZT2_Z) continue;
                            const long long cost = ((txy2 * runs + R - 1) / R) * (zz + 2);
                            if (best < 0 || cost < best) { best = cost; zz2 = zz; }
                        }
                        if (const char* e = getenv("OPFLOW_MG_ZT_PLANES")) zz2 = std::max(2, std::min(MG_ZT2_Z, atoi(e)));
                        for (int k0 = 0; k0 < D.n[2]; k0 += zz2)
                            for (int j0 = 0; j0 < D.n[1]; j0 += MG_ZT2_Y)
                                for (int i0 = 0; i0 < D.n[0]; i0 += MG_ZT2_X) {
                                    Chunk c{li, j0, k0, i0, MG_ZT2_X};
                                    c.nrows = std::min(zz2, D.n[2] - k0);
                                    S->zt_ch[l].push_back(c);
                                }
                    }
                } else if (!D.coarsest) {
                    rows(li, D, S->smooth_ch[l]);  // (also the rows of the residual before restriction)
                }
                // fine rows of level l prolonged from l+1 by the chunked kernel (z levels of cell-centred
                // problems take mg_prolong_z over their tiles)
                if (!D.coarsest && (!ztiles || D.node)) rows(li, D, S->prolong_ch[l]);
            }
            if (l > 0 && !above_tiled) rows(li, D, S->restrict_ch[l]);  // coarse rows of level l (restricted from l-1)
            if (D.coarsest && H.Ainv64) coarse_list.push_back(li);
            if (D.coarsest && !H.Ainv64) rows(li, D, S->coarse_sm_ch);
        }
        KrylovDev K{};
        const size_t N0 = (size_t) P.levels[0].N;
        K.b = P.b;
        K.x = (double*) S->arena.alloc(N0 * 8);
        K.r = (double*) S->arena.alloc(N0 * 8);
        K.p = (double*) S->arena.alloc(N0 * 8);
        K.q = (double*) S->arena.alloc(N0 * 8);
        if (!K.x || !K.r || !K.p || !K.q) return fail(OPFLOW_E_NOMEM, "Krylov vectors");
        cudaMemsetAsync(K.x, 0, N0 * 8, ctx->stream);
        K.lvl0 = base;
        K.pin = -1;
        kd.push_back(K);
        P.lvl0 = base;
        first.push_back((int) k0.size());
        std::vector<Chunk> mine;
        krylov_chunks(base, lv[base], mine);
        k0.insert(k0.end(), mine.begin(), mine.end());
        count.push_back((int) mine.size());
    }
    S->nlv = (int) lv.size();
    S->dL = (LvlDev*) S->arena.alloc(lv.size() * sizeof(LvlDev));
    S->dK = (KrylovDev*) S->arena.alloc(kd.size() * sizeof(KrylovDev));
    S->dS = (Scal*) S->arena.alloc(S->probs.size() * sizeof(Scal));
    S->nk0 = (int) k0.size();
    S->dk0 = (Chunk*) S->arena.alloc(std::max<size_t>(1, k0.size()) * sizeof(Chunk));
    S->dfirst = (int*) S->arena.alloc(first.size() * sizeof(int));
    S->dcount = (int*) S->arena.alloc(count.size() * sizeof(int));
    S->partial = (double*) S->arena.alloc(std::max<size_t>(1, 2 * k0.size()) * sizeof(double));
    S->red = (double*) S->arena.alloc(2 * S->probs.size() * sizeof(double));
    S->dcoarse = (int*) S->arena.alloc(std::max<size_t>(1, coarse_list.size()) * sizeof(int));
    S->d_active = (int*) S->arena.alloc(2 * sizeof(int));  // [0] active count, [1] solve-loop counter
    S->d_done = (int*) S->arena.alloc(S->probs.size() * sizeof(int));
    if (!S->d_done) return fail(OPFLOW_E_NOMEM, "solver tables");
    cudaMemsetAsync(S->d_done, 0, S->probs.size() * sizeof(int), ctx->stream);
    S->ncoarse = (int) coarse_list.size();
    S->coarse_host = coarse_list;
    S->nbottom = (int) S->bottom_host.size();
    S->bottom_cells = 0;
    for (long long c : S->bottom_cells_host) S->bottom_cells = std::max(S->bottom_cells, c);
    S->dbottom = (int*) S->arena.alloc(std::max<size_t>(1, S->bottom_host.size()) * sizeof(int));
    if (!S->dbottom) return fail(OPFLOW_E_NOMEM, "solver tables");
    if (S->nbottom) cudaMemcpyAsync(S->dbottom, S->bottom_host.data(), S->bottom_host.size() * sizeof(int), cudaMemcpyHostToDevice, ctx->stream);
    if (!S->dL || !S->dK || !S->dS || !S->dk0 || !S->partial || !S->red || !S->dcoarse) return fail(OPFLOW_E_NOMEM, "solver tables");
    cudaMemcpyAsync(S->dL, lv.data(), lv.size() * sizeof(LvlDev), cudaMemcpyHostToDevice, ctx->stream);
    cudaMemcpyAsync(S->dK, kd.data(), kd.size() * sizeof(KrylovDev), cudaMemcpyHostToDevice, ctx->stream);
    cudaMemsetAsync(S->dS, 0, S->probs.size() * sizeof(Scal), ctx->stream);
    if (!k0.empty()) cudaMemcpyAsync(S->dk0, k0.data(), k0.size() * sizeof(Chunk), cudaMemcpyHostToDevice, ctx->stream);
    cudaMemcpyAsync(S->dfirst, first.data(), first.size() * sizeof(int), cudaMemcpyHostToDevice, ctx->stream);
    cudaMemcpyAsync(S->dcount, count.data(), count.size() * sizeof(int), cudaMemcpyHostToDevice, ctx->stream);
    if (!coarse_list.empty()) cudaMemcpyAsync(S->dcoarse, coarse_list.data(), coarse_list.size() * sizeof(int), cudaMemcpyHostToDevice, ctx->stream);
    auto upload = [&](std::vector<Chunk>& h, ChunkList& d) {
        d.n = (int) h.size();
        d.ptr = (Chunk*) S->arena.alloc(std::max<size_t>(1, h.size()) * sizeof(Chunk));
        if (!h.empty()) cudaMemcpyAsync(d.ptr, h.data(), h.size() * sizeof(Chunk), cudaMemcpyHostToDevice, ctx->stream);
    };
    S->d_smooth.assign(S->nlevels, {});
    S->d_restrict.assign(S->nlevels, {});
    S->d_prolong.assign(S->nlevels, {});
    S->d_tiles.assign(S->nlevels, {});
    S->d_zsm.assign(S->nlevels, {});
    S->d_zt.assign(S->nlevels, {});
    for (int l = 0; l < S->nlevels; ++l) {
        upload(S->smooth_ch[l], S->d_smooth[l]);
        upload(S->restrict_ch[l], S->d_restrict[l]);
        upload(S->prolong_ch[l], S->d_prolong[l]);
        upload(S->tile_ch[l], S->d_tiles[l]);
        upload(S->zsm_ch[l], S->d_zsm[l]);
        upload(S->zt_ch[l], S->d_zt[l]);
    }
    upload(S->coarse_sm_ch, S->d_coarse_sm);
    S->zt_maps.assign(2 * lv.size(), CUtensorMap{});
    for (auto& m : zt_maps) {
        S->zt_maps[2 * m.first] = m.second[0];
        S->zt_maps[2 * m.first + 1] = m.second[1];
    }
    zt_coverage(S);
    S->d_zt_maps = nullptr;
    if (!zt_maps.empty()) {
        S->d_zt_maps = (CUtensorMap*) S->arena.alloc(S->zt_maps.size() * sizeof(CUtensorMap));
        if (!S->d_zt_maps) return fail(OPFLOW_E_NOMEM, "tensor maps");
        OPG_CUDA(cudaMemcpyAsync(S->d_zt_maps, S->zt_maps.data(), S->zt_maps.size() * sizeof(CUtensorMap), cudaMemcpyHostToDevice, ctx->stream));
    }
    S->kd_host = kd;
    S->lv_host = lv;
    S->k0_host = k0;
    S->nprob = (int) S->probs.size();
    if (!S->h_active) OPG_CUDA(cudaMallocHost(&S->h_active, sizeof(int)));
    OPG_CUDA(cudaStreamSynchronize(ctx->stream));
    return tune_levels(S);
}

// One V-cycle on the level-0 residuals of the active problems: z = M r.  Each problem sees the same
// sequence whatever else is in the batch: pre-smoothing on its levels 0..L-1, the direct solve (or,
// without a dense inverse, pre+post smoothing) on its coarsest level L, prolongation and post-smoothing
// back up.
static cudaStream_t work_stream(const MGSystem* S) { return S->recording ? S->rec_stream : S->ctx->stream; }

// (The level-0 input b = r, x = 0 is written by the Krylov kernel that forms r.)
// one half sweep of level l's z-marching tiles: the TMA-staged smoother where chosen and available,
// else the register kernel with the level's plane batch
static int smooth_z_level(MGSystem* S, int l, int color, const Scal* sc, int zb) {
    cudaStream_t s = work_stream(S);
    const int sms = S->ctx->num_sms;
    if (mg_z_batch(zb) == MG_ZB_TMA && S->d_zt[l].n > 0 && S->zt_full[l])
        return mg_launch_smooth_zt(s, sms, S->dL, S->d_zt[l].ptr, S->d_zt[l].n, color, sc, S->d_zt_maps);
    return mg_launch_smooth_z(s, sms, S->precision == OPFLOW_PREC_MIXED, S->dL, S->d_zsm[l].ptr, S->d_zsm[l].n, color, sc, zb);
}
static int smooth_z_level(MGSystem* S, int l, int color) { return smooth_z_level(S, l, color, S->dS, S->zb[l]); }

static int vcycle(MGSystem* S) {
    cudaStream_t s = work_stream(S);
    const int sms = S->ctx->num_sms;
    const bool f32 = S->precision == OPFLOW_PREC_MIXED;
    const Scal* sc = S->dS;
    for (int l = 0; l < S->nlevels; ++l) {
        if (l > 0) OPG_TRY(mg_launch_restrict(s, sms, f32, S->dL, S->d_restrict[l].ptr, S->d_restrict[l].n, sc));
        OPG_TRY(mg_launch_tile_down(s, sms, f32, S->dL, S->d_tiles[l].ptr, S->d_tiles[l].n, sc, S->pre));
        const ChunkList& C = S->d_smooth[l];
        const ChunkList& Z = S->d_zsm[l];
        for (int it = 0; it < S->pre; ++it) {
            OPG_TRY(mg_launch_smooth(s, sms, f32, S->dL, C.ptr, C.n, 0, sc));
            OPG_TRY(smooth_z_level(S, l, 0));
            OPG_TRY(mg_launch_smooth(s, sms, f32, S->dL, C.ptr, C.n, 1, sc));
            OPG_TRY(smooth_z_level(S, l, 1));
        }
        OPG_TRY(mg_launch_residual(s, sms, f32, S->dL, C.ptr, C.n, sc));
        OPG_TRY(mg_launch_residual_z(s, sms, f32, S->dL, Z.ptr, Z.n, sc, S->zb[l]));
    }
    OPG_TRY(mg_launch_bottom(s, sms, f32, S->dL, S->dbottom, S->nbottom, sc, S->pre, S->post, S->bottom_cells));
    OPG_TRY(mg_launch_coarse(s, sms, f32, S->dL, S->dcoarse, S->ncoarse, sc));
    for (int it = 0; it < S->pre + S->post; ++it) {
        OPG_TRY(mg_launch_smooth(s, sms, f32, S->dL, S->d_coarse_sm.ptr, S->d_coarse_sm.n, 0, sc));
        OPG_TRY(mg_launch_smooth(s, sms, f32, S->dL, S->d_coarse_sm.ptr, S->d_coarse_sm.n, 1, sc));
    }
    for (int l = S->nlevels - 2; l >= 0; --l) {
        OPG_TRY(mg_launch_tile_up(s, sms, f32, S->dL, S->d_tiles[l].ptr, S->d_tiles[l].n, sc, S->post));
        const ChunkList& C = S->d_smooth[l];
        const ChunkList& Z = S->d_zsm[l];
        OPG_TRY(mg_launch_prolong(s, sms, f32, S->dL, S->d_prolong[l].ptr, S->d_prolong[l].n, sc));
        OPG_TRY(mg_launch_prolong_z(s, sms, f32, S->dL, Z.ptr, Z.n, sc, S->zb[l]));
        for (int it = 0; it < S->post; ++it) {
            OPG_TRY(mg_launch_smooth(s, sms, f32, S->dL, C.ptr, C.n, 1, sc));
            OPG_TRY(smooth_z_level(S, l, 1));
            OPG_TRY(mg_launch_smooth(s, sms, f32, S->dL, C.ptr, C.n, 0, sc));
            OPG_TRY(smooth_z_level(S, l, 0));
        }
    }
    return OPFLOW_OK;
}

int mg_vcycle(MGSystem* S) { return vcycle(S); }

// fused per-problem reduction + scalar stage for the Krylov kernels
static Finish finish(MGSystem* S, int stage) {
    Finish F{};
    F.done = S->d_done;
    F.first = S->dfirst;
    F.count = S->dcount;
    F.sc = S->dS;
    F.red = S->red;
    F.stage = stage;
    F.max_iter = S->max_iter;
    F.tol = S->tol;
    return F;
}

// One flexible-PCG iteration (everything after the first direction), recorded into a CUDA graph.
// With `readback` the active count is also copied to the host (for callers that step iterations).
static int iteration(MGSystem* S, bool readback) {
    cudaStream_t s = work_stream(S);
    const int sms = S->ctx->num_sms;
    const bool f32 = S->precision == OPFLOW_PREC_MIXED;
    const int np = S->nprob;
    OPG_TRY(kr_launch_apply(s, sms, S->dL, S->dK, S->dk0, S->nk0, S->dS, S->partial, 1, finish(S, 1)));  // q = A p
    OPG_TRY(kr_launch_update(s, sms, f32, S->dL, S->dK, S->dk0, S->nk0, S->dS, S->partial, finish(S, 2)));
    OPG_TRY(vcycle(S));
    OPG_TRY(kr_launch_from_vcycle(s, sms, f32, S->dL, S->dK, S->dk0, S->nk0, S->dS, S->partial, finish(S, 3)));
    OPG_TRY(kr_launch_pupdate(s, sms, f32, S->dL, S->dK, S->dk0, S->nk0, S->dS, 0));
    OPG_TRY(kr_launch_count(s, S->dS, np, S->d_active));
    if (readback) OPG_CUDA(cudaMemcpyAsync(S->h_active, S->d_active, sizeof(int), cudaMemcpyDeviceToHost, s));
    return OPFLOW_OK;
}

// r = b - A x, the first preconditioned direction and the active count
static int first_direction(MGSystem* S) {
    cudaStream_t s = work_stream(S);
    const int sms = S->ctx->num_sms;
    const bool f32 = S->precision == OPFLOW_PREC_MIXED;
    const int np = S->nprob;
    OPG_TRY(kr_launch_apply(s, sms, S->dL, S->dK, S->dk0, S->nk0, nullptr, S->partial, 0, finish(S, 0), 1, f32));
    OPG_TRY(vcycle(S));
    OPG_TRY(kr_launch_from_vcycle(s, sms, f32, S->dL, S->dK, S->dk0, S->nk0, S->dS, S->partial, finish(S, 4)));
    OPG_TRY(kr_launch_pupdate(s, sms, f32, S->dL, S->dK, S->dk0, S->nk0, S->dS, 1));
    return kr_launch_count(s, S->dS, np, S->d_active);
}

// Loop control of the whole-solve graph.  Before the loop (reset) the counter starts at 0; after each
// body it advances.  The body runs again while some problem is active and fewer than `max_loops`
// bodies have run, so the loop ends even if the active flags never clear.
__global__ void loop_control(cudaGraphConditionalHandle h, int* active_and_counter, int max_loops, int reset) {
    const int c = reset ? 0 : active_and_counter[1] + 1;
    active_and_counter[1] = c;
    cudaGraphSetConditional(h, (active_and_counter[0] > 0 && c < max_loops) ? 1u : 0u);
}

// Records the whole solve - first direction, then a device-side while loop over iterations - as one
// graph, so a solve is one launch with no host round trip per iteration.
static int solve_graph(MGSystem* S) {
    if (S->solve_exec) return OPFLOW_OK;
    if (!S->rec_stream) OPG_CUDA(cudaStreamCreateWithFlags(&S->rec_stream, cudaStreamNonBlocking));
    cudaStream_t s = S->rec_stream;
    const int max_loops = std::max(1, S->max_iter + 1);
    const uint64_t c0 = g_launches.load();
    OPG_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    S->recording = true;
    cudaGraph_t g = nullptr, body = nullptr;
    cudaGraphConditionalHandle h{};
    int rc = first_direction(S);
    cudaError_t e = cudaSuccess;
    if (!rc) {
        cudaStreamCaptureStatus st;
        e = cudaStreamGetCaptureInfo(s, &st, nullptr, &g, nullptr, nullptr, nullptr);
        if (e == cudaSuccess) e = cudaGraphConditionalHandleCreate(&h, g, 0, cudaGraphCondAssignDefault);
        if (e == cudaSuccess) {
            loop_control<<<1, 1, 0, s>>>(h, S->d_active, max_loops, 1);
            OPG_LAUNCHED();
            e = cudaGetLastError();
        }
        const cudaGraphNode_t* deps = nullptr;
        const cudaGraphEdgeData* edata = nullptr;
        size_t ndeps = 0;
        if (e == cudaSuccess) e = cudaStreamGetCaptureInfo(s, &st, nullptr, &g, &deps, &edata, &ndeps);
        cudaGraphNodeParams cp = {};
        cp.type = cudaGraphNodeTypeConditional;
        cp.conditional.handle = h;
        cp.conditional.type = cudaGraphCondTypeWhile;
        cp.conditional.size = 1;
        cudaGraphNode_t cond = nullptr;
        if (e == cudaSuccess) e = cudaGraphAddNode(&cond, g, deps, edata, ndeps, &cp);
        if (e == cudaSuccess) {
            body = cp.conditional.phGraph_out[0];
            e = cudaStreamUpdateCaptureDependencies(s, &cond, nullptr, 1, cudaStreamSetCaptureDependencies);
        }
    }
    S->recording = false;
    const uint64_t c1 = g_launches.load();
    cudaGraph_t outer = nullptr;
    const cudaError_t e_end = cudaStreamEndCapture(s, &outer);
    if (rc || e != cudaSuccess || e_end != cudaSuccess) {
        if (e_end == cudaSuccess && outer) cudaGraphDestroy(outer);
        if (rc) return rc;
        return fail(OPFLOW_E_CUDA, "recording the solve graph failed: %s", cudaGetErrorString(e != cudaSuccess ? e : e_end));
    }
    // the loop body: one iteration and the loop control
    e = cudaStreamBeginCaptureToGraph(s, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) {
        cudaGraphDestroy(outer);
        return fail(OPFLOW_E_CUDA, "recording the solve loop body failed: %s", cudaGetErrorString(e));
    }
    S->recording = true;
    rc = iteration(S, false);
    if (!rc) {
        loop_control<<<1, 1, 0, s>>>(h, S->d_active, max_loops, 0);
        OPG_LAUNCHED();
        e = cudaGetLastError();
    }
    S->recording = false;
    const uint64_t c2 = g_launches.load();
    g_launches.fetch_sub(c2 - c0);
    S->first_kernels = (long long) (c1 - c0);
    S->body_kernels = (long long) (c2 - c1);
    cudaGraph_t body_out = nullptr;
    const cudaError_t e_end2 = cudaStreamEndCapture(s, &body_out);
    if (rc || e != cudaSuccess || e_end2 != cudaSuccess) {
        cudaGraphDestroy(outer);
        if (rc) return rc;
        return fail(OPFLOW_E_CUDA, "recording the solve loop body failed: %s", cudaGetErrorString(e != cudaSuccess ? e : e_end2));
    }
    e = cudaGraphInstantiate(&S->solve_exec, outer, 0);
    cudaGraphDestroy(outer);
    if (e != cudaSuccess) {
        S->solve_exec = nullptr;
        return fail(OPFLOW_E_CUDA, "solve graph instantiation failed: %s", cudaGetErrorString(e));
    }
    return OPFLOW_OK;
}

// OPFLOW_SOLVE_GRAPHS=0 issues the same kernels one by one with a host-side loop (profilers then see
// every kernel as its own launch)
static bool solve_graphs_enabled() {
    const char* e = getenv("OPFLOW_SOLVE_GRAPHS");
    return !(e && e[0] == '0');
}

// Runs the whole solve as one graph launch on the caller's stream; mg_states reads the outcome.
int mg_solve(MGSystem* S) {
    if (!solve_graphs_enabled()) {
        cudaStream_t s = S->ctx->stream;
        OPG_TRY(first_direction(S));
        OPG_CUDA(cudaMemcpyAsync(S->h_active, S->d_active, sizeof(int), cudaMemcpyDeviceToHost, s));
        OPG_CUDA(cudaStreamSynchronize(s));
        for (int it = 0; it < S->max_iter && *S->h_active > 0; ++it) {
            OPG_TRY(iteration(S, true));
            OPG_CUDA(cudaStreamSynchronize(s));
        }
        return OPFLOW_OK;
    }
    OPG_TRY(solve_graph(S));
    OPG_CUDA(cudaGraphLaunch(S->solve_exec, S->ctx->stream));
    S->graph_launches++;
    g_launches.fetch_add((uint64_t) S->first_kernels);
    S->solve_pending = true;
    return OPFLOW_OK;
}

// record one iteration of the whole batch as a CUDA graph (once per table layout)
int mg_iteration_graph(MGSystem* S) {
    if (S->exec) return OPFLOW_OK;
    if (!S->rec_stream) OPG_CUDA(cudaStreamCreateWithFlags(&S->rec_stream, cudaStreamNonBlocking));
    cudaStream_t s = S->rec_stream;
    cudaGraph_t g;
    const uint64_t c0 = g_launches.load();
    OPG_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    S->recording = true;
    int rc = iteration(S, true);
    S->recording = false;
    S->iter_kernels = (long long) (g_launches.load() - c0);
    g_launches.fetch_sub((uint64_t) S->iter_kernels);
    cudaError_t e = cudaStreamEndCapture(s, &g);
    if (rc) {
        if (e == cudaSuccess) cudaGraphDestroy(g);
        return rc;
    }
    if (e != cudaSuccess) return fail(OPFLOW_E_CUDA, "graph capture failed: %s", cudaGetErrorString(e));
    e = cudaGraphInstantiate(&S->exec, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) { S->exec = nullptr; return fail(OPFLOW_E_CUDA, "graph instantiation failed: %s", cudaGetErrorString(e)); }
    return OPFLOW_OK;
}

// `iters` replays without a host synchronisation in between; the active count lands in h_active
int mg_run_iterations(MGSystem* S, int iters) {
    OPG_TRY(mg_iteration_graph(S));
    for (int it = 0; it < iters; ++it) {
        OPG_CUDA(cudaGraphLaunch(S->exec, S->ctx->stream));
        S->graph_launches++;
        g_launches.fetch_add((uint64_t) S->iter_kernels);
    }
    return OPFLOW_OK;
}

__global__ void scal_seed(Scal* out, const double* red, double tol) {
    Scal S{};
    S.bb = red[0];
    S.rr = red[1];
    S.rz = 1.0;   // with p = 0 the next iteration takes alpha = 0 and only forms z = M r, p = z
    S.alpha = 0.;
    S.beta = 0.;
    S.iters = -1;
    S.active = (red[1] > tol * tol * red[0]) && red[0] > 0. ? 1 : 0;
    *out = S;
}

int mg_prepare_problem(MGSystem* S, double tol, Scal* out_dev) {
    cudaStream_t s = S->ctx->stream;
    const int sms = S->ctx->num_sms;
    const KrylovDev& K = S->kd_host[0];
    const long long N = S->probs[0].levels[0].N;
    OPG_TRY(kr_launch_apply(s, sms, S->dL, S->dK, S->dk0, S->nk0, nullptr, S->partial, 0));
    OPG_TRY(kr_launch_reduce(s, sms, S->partial, S->dfirst, S->dcount, 1, S->red));
    OPG_CUDA(cudaMemsetAsync(K.p, 0, N * sizeof(double), s));
    scal_seed<<<1, 1, 0, s>>>(out_dev, S->red, tol);
    OPG_LAUNCHED();
    return check_launch("scal_seed");
}

// Composite tables over resident problems: level / problem indices are renumbered, memory is shared.
int mg_compose(MGSystem* C, const std::vector<MGSystem*>& parts, const std::vector<Scal>& state) {
    opflow_ctx ctx = C->ctx;
    if (C->exec) { cudaGraphExecDestroy(C->exec); C->exec = nullptr; }
    if (C->solve_exec) { cudaGraphExecDestroy(C->solve_exec); C->solve_exec = nullptr; }
    C->arena.release();
    std::vector<LvlDev> lv;
    std::vector<KrylovDev> kd;
    std::vector<Chunk> k0;
    std::vector<int> first, count, coarse_list, bottom_list;
    std::vector<long long> bottom_cells;
    C->bottom_cells = 0;
    C->nlevels = 0;
    for (auto* P : parts) C->nlevels = std::max(C->nlevels, P->nlevels);
    C->smooth_ch.assign(C->nlevels, {});
    C->restrict_ch.assign(C->nlevels, {});
    C->prolong_ch.assign(C->nlevels, {});
    C->tile_ch.assign(C->nlevels, {});
    C->zsm_ch.assign(C->nlevels, {});
    C->zb.assign(C->nlevels, 4);
    C->tile_alt.assign(C->nlevels, {});
    C->zt_ch.assign(C->nlevels, {});
    C->zt_maps.clear();
    bool any_maps = false;
    std::vector<size_t> zb_tiles(C->nlevels, 0);  // each level takes the batch of the part with most tiles there
    C->coarse_sm_ch.clear();
    for (size_t q = 0; q < parts.size(); ++q) {
        MGSystem* P = parts[q];
        const int base = (int) lv.size();
        for (size_t l = 0; l < P->lv_host.size(); ++l) {
            LvlDev D = P->lv_host[l];
            // the part's tensor maps move with its level (they address the part's own vectors)
            const bool has_maps = 2 * l + 1 < P->zt_maps.size();
            C->zt_maps.push_back(has_maps ? P->zt_maps[2 * l] : CUtensorMap{});
            C->zt_maps.push_back(has_maps ? P->zt_maps[2 * l + 1] : CUtensorMap{});
            any_maps = any_maps || (has_maps && P->d_zt_maps);
            D.problem = (int) q;
            if (D.coarse >= 0) D.coarse += base;
            if (D.fine >= 0) D.fine += base;
            lv.push_back(D);
        }
        for (int c : P->coarse_host) coarse_list.push_back(base + c);
        for (int b : P->bottom_host) bottom_list.push_back(base + b);
        for (long long c : P->bottom_cells_host) {
            bottom_cells.push_back(c);
            C->bottom_cells = std::max(C->bottom_cells, c);
        }
        auto shift = [&](const std::vector<Chunk>& src, std::vector<Chunk>& dst) {
            for (Chunk c : src) { c.lvl += base; dst.push_back(c); }
        };
        for (int l = 0; l < P->nlevels; ++l) {
            shift(P->smooth_ch[l], C->smooth_ch[l]);
            shift(P->restrict_ch[l], C->restrict_ch[l]);
            shift(P->prolong_ch[l], C->prolong_ch[l]);
            shift(P->tile_ch[l], C->tile_ch[l]);
            shift(P->zsm_ch[l], C->zsm_ch[l]);
            shift(P->zt_ch[l], C->zt_ch[l]);
            if (P->zsm_ch[l].size() > zb_tiles[l]) {
                zb_tiles[l] = P->zsm_ch[l].size();
                C->zb[l] = P->zb[l];
            }
        }
        shift(P->coarse_sm_ch, C->coarse_sm_ch);
        KrylovDev K = P->kd_host[0];
        K.lvl0 = base;
        kd.push_back(K);
        first.push_back((int) k0.size());
        shift(P->k0_host, k0);
        count.push_back((int) P->k0_host.size());
    }
    C->nprob = (int) parts.size();
    C->nlv = (int) lv.size();
    const size_t np = std::max<size_t>(1, parts.size());
    C->dL = (LvlDev*) C->arena.alloc(std::max<size_t>(1, lv.size()) * sizeof(LvlDev));
    C->dK = (KrylovDev*) C->arena.alloc(np * sizeof(KrylovDev));
    C->dS = (Scal*) C->arena.alloc(np * sizeof(Scal));
    C->nk0 = (int) k0.size();
    C->dk0 = (Chunk*) C->arena.alloc(std::max<size_t>(1, k0.size()) * sizeof(Chunk));
    C->dfirst = (int*) C->arena.alloc(np * sizeof(int));
    C->dcount = (int*) C->arena.alloc(np * sizeof(int));
    C->partial = (double*) C->arena.alloc(std::max<size_t>(1, 2 * k0.size()) * sizeof(double));
    C->red = (double*) C->arena.alloc(2 * np * sizeof(double));
    C->dcoarse = (int*) C->arena.alloc(std::max<size_t>(1, coarse_list.size()) * sizeof(int));
    C->ncoarse = (int) coarse_list.size();
    C->coarse_host = coarse_list;
    C->bottom_host = bottom_list;
    C->bottom_cells_host = bottom_cells;
    C->nbottom = (int) bottom_list.size();
    C->dbottom = (int*) C->arena.alloc(std::max<size_t>(1, bottom_list.size()) * sizeof(int));
    C->d_active = (int*) C->arena.alloc(2 * sizeof(int));
    C->d_done = (int*) C->arena.alloc(np * sizeof(int));
    if (!C->d_done) return fail(OPFLOW_E_NOMEM, "batch tables");
    cudaMemsetAsync(C->d_done, 0, np * sizeof(int), ctx->stream);
    if (!C->dL || !C->dK || !C->dS || !C->dk0 || !C->dfirst || !C->dcount || !C->partial || !C->red || !C->dcoarse || !C->d_active || !C->dbottom)
        return fail(OPFLOW_E_NOMEM, "batch tables");
    cudaStream_t s = ctx->stream;
    if (!lv.empty()) cudaMemcpyAsync(C->dL, lv.data(), lv.size() * sizeof(LvlDev), cudaMemcpyHostToDevice, s);
    if (!kd.empty()) cudaMemcpyAsync(C->dK, kd.data(), kd.size() * sizeof(KrylovDev), cudaMemcpyHostToDevice, s);
    if (!state.empty()) cudaMemcpyAsync(C->dS, state.data(), state.size() * sizeof(Scal), cudaMemcpyHostToDevice, s);
    if (!k0.empty()) cudaMemcpyAsync(C->dk0, k0.data(), k0.size() * sizeof(Chunk), cudaMemcpyHostToDevice, s);
    if (!first.empty()) cudaMemcpyAsync(C->dfirst, first.data(), first.size() * sizeof(int), cudaMemcpyHostToDevice, s);
    if (!count.empty()) cudaMemcpyAsync(C->dcount, count.data(), count.size() * sizeof(int), cudaMemcpyHostToDevice, s);
    if (!coarse_list.empty()) cudaMemcpyAsync(C->dcoarse, coarse_list.data(), coarse_list.size() * sizeof(int), cudaMemcpyHostToDevice, s);
    if (!bottom_list.empty()) cudaMemcpyAsync(C->dbottom, bottom_list.data(), bottom_list.size() * sizeof(int), cudaMemcpyHostToDevice, s);
    auto upload = [&](std::vector<Chunk>& h, ChunkList& d) {
        d.n = (int) h.size();
        d.ptr = (Chunk*) C->arena.alloc(std::max<size_t>(1, h.size()) * sizeof(Chunk));
        if (!h.empty()) cudaMemcpyAsync(d.ptr, h.data(), h.size() * sizeof(Chunk), cudaMemcpyHostToDevice, s);
    };
    C->d_smooth.assign(C->nlevels, {});
    C->d_restrict.assign(C->nlevels, {});
    C->d_prolong.assign(C->nlevels, {});
    C->d_tiles.assign(C->nlevels, {});
    C->d_zsm.assign(C->nlevels, {});
    C->d_zt.assign(C->nlevels, {});
    for (int l = 0; l < C->nlevels; ++l) {
        upload(C->smooth_ch[l], C->d_smooth[l]);
        upload(C->restrict_ch[l], C->d_restrict[l]);
        upload(C->prolong_ch[l], C->d_prolong[l]);
        upload(C->tile_ch[l], C->d_tiles[l]);
        upload(C->zsm_ch[l], C->d_zsm[l]);
        upload(C->zt_ch[l], C->d_zt[l]);
    }
    zt_coverage(C);
    C->d_zt_maps = nullptr;
    if (any_maps) {
        C->d_zt_maps = (CUtensorMap*) C->arena.alloc(C->zt_maps.size() * sizeof(CUtensorMap));
        if (!C->d_zt_maps) return fail(OPFLOW_E_NOMEM, "tensor maps");
        OPG_CUDA(cudaMemcpyAsync(C->d_zt_maps, C->zt_maps.data(), C->zt_maps.size() * sizeof(CUtensorMap), cudaMemcpyHostToDevice, ctx->stream));
    } else {
        for (auto& z : C->zt_ch) z.clear();
        for (auto& z : C->d_zt) z.n = 0;
    }
    upload(C->coarse_sm_ch, C->d_coarse_sm);
    C->kd_host = kd;
    C->lv_host = lv;
    C->k0_host = k0;
    C->composite = true;
    if (!C->h_active) OPG_CUDA(cudaMallocHost(&C->h_active, sizeof(int)));
    OPG_CUDA(cudaStreamSynchronize(s));  // the host vectors above must outlive their copies
    return OPFLOW_OK;
}

int mg_states(MGSystem* S, std::vector<Scal>& out) {
    out.resize(S->probs.size());
    OPG_CUDA(cudaMemcpyAsync(out.data(), S->dS, out.size() * sizeof(Scal), cudaMemcpyDeviceToHost, S->ctx->stream));
    int ac[2] = {0, 0};
    if (S->solve_pending) OPG_CUDA(cudaMemcpyAsync(ac, S->d_active, sizeof ac, cudaMemcpyDeviceToHost, S->ctx->stream));
    OPG_CUDA(cudaStreamSynchronize(S->ctx->stream));
    if (S->solve_pending) {
        g_launches.fetch_add((uint64_t) ((long long) ac[1] * S->body_kernels));
        S->solve_pending = false;
    }
    return mg_check_error(S);
}

// the TMA-staged smoother's failure flag (a bounded wait that gave up), for systems that use it
int mg_check_error(MGSystem* S) {
    bool uses = false;
    for (const ChunkList& z : S->d_zt) uses = uses || z.n > 0;
    if (!uses) return OPFLOW_OK;
    int err = 0;
    OPG_TRY(mg_take_error(S->ctx->stream, &err));
    if (err) return fail(OPFLOW_E_CUDA, "the staged 3D smoother gave up waiting for an asynchronous copy; results are invalid");
    return OPFLOW_OK;
}

void mg_destroy(MGSystem* S) {
    if (!S) return;
    // memory goes back to the stream-ordered pool after the work already enqueued; only recorded
    // graphs need the stream idle before they are destroyed
    if (S->exec || S->solve_exec) cudaStreamSynchronize(S->ctx->stream);
    if (S->exec) cudaGraphExecDestroy(S->exec);
    S->exec = nullptr;
    if (S->solve_exec) cudaGraphExecDestroy(S->solve_exec);
    S->solve_exec = nullptr;
    if (S->rec_stream) cudaStreamDestroy(S->rec_stream);
    S->rec_stream = nullptr;
    for (auto& P : S->probs)
        for (auto& L : P.levels) release_level_fields(L);
    krylov_release(S);
    S->arena.release();
    if (S->h_active) cudaFreeHost(S->h_active);
    delete S;
}

// ================================================================================= single-problem API
int mg_gather_target(opflow_ctx ctx, opflow_field target, double* x) {
    const Box box = assign_box(target->info);
    gather_box<<<gridN(ctx, box.count()), 256, 0, ctx->stream>>>(target->view(), box, x);
    OPG_LAUNCHED();
    return check_launch("gather_box");
}

void mg_add_scalar(opflow_ctx ctx, double* v, long long n, double a) {
    add_scalar<<<gridN(ctx, n), 256, 0, ctx->stream>>>(v, n, a);
    OPG_LAUNCHED();
}

double mg_sum(opflow_ctx ctx, const double* v, long long n);

double mg_sum(opflow_ctx ctx, const double* v, long long n) {
    double* part = (double*) ctx->scratch + 64;
    const int blocks = 256;
    sum_partials<<<blocks, 256, 0, ctx->stream>>>(v, n, part);
    OPG_LAUNCHED();
    double h[256];
    cudaMemcpyAsync(h, part, sizeof h, cudaMemcpyDeviceToHost, ctx->stream);
    cudaStreamSynchronize(ctx->stream);
    double s = 0.;
    for (int i = 0; i < blocks; ++i) s += h[i];
    return s;
}

}  // namespace opg

using namespace opg;

struct opflow_solver_s {
    opflow_ctx ctx;
    opflow_field target;
    std::vector<opflow_node> tree;
    std::vector<opflow_field> leaves;
    int unknown;
    opflow_solve_params params;
    MGSystem* S = nullptr;
    bool first = true;
    // write counters of the leaves when the system was last assembled (the target's after its solve)
    std::vector<unsigned long long> assembled_versions;
    // generateb's compiled plan (staticMat), made on the first re-solve
    AsmPlan rhs_plan;
    bool rhs_plan_ok = false;
};

// (the unknown's own values only seed the iteration, so its slot is left out)
static std::vector<unsigned long long> leaf_versions(opflow_solver s) {
    std::vector<unsigned long long> v;
    for (size_t k = 0; k < s->leaves.size(); ++k) v.push_back((int) k == s->unknown ? 0ull : s->leaves[k]->version);
    return v;
}

static int build_system(opflow_solver s) {
    if (s->S) mg_destroy(s->S);
    s->S = new MGSystem();
    s->S->ctx = s->ctx;
    s->S->arena.ctx = s->ctx;
    s->S->precision = s->params.precision;
    s->S->pre = s->params.pre_sweeps;
    s->S->post = s->params.post_sweeps;
    s->S->coarse_max = s->params.coarse_max;
    s->S->tol = s->params.tol;
    s->S->max_iter = s->params.max_iter;
    OPG_TRY(mg_add_problem(s->S, s->target, s->tree.data(), (int) s->tree.size(), s->leaves.data(), (int) s->leaves.size(), s->unknown));
    return mg_finalize(s->S);
}

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
    p->coarse_max = 64;
    p->zero_guess = 0;
    p->krylov = OPFLOW_KRYLOV_PCG;
    p->precond = OPFLOW_PRECOND_MG;
    p->kdim = 5;
    p->abs_tol = 0.;
}

int opflow_solver_create(opflow_ctx ctx, opflow_field target, const opflow_node* nodes, int n_nodes, const opflow_field* leaves, int n_leaves,
                         int unknown_slot, const opflow_solve_params* params, opflow_solver* out) {
    if (!ctx || !target || !nodes || !leaves || !out) return fail(OPFLOW_E_INVALID, "null argument");
    opflow_solve_params p;
    if (params) p = *params;
    else opflow_solve_params_default(&p);
    if (!(p.tol > 0) || p.max_iter < 0 || p.pre_sweeps < 0 || p.post_sweeps < 0) return fail(OPFLOW_E_INVALID, "bad solver parameters");
    if (p.precision != OPFLOW_PREC_FP64 && p.precision != OPFLOW_PREC_MIXED) return fail(OPFLOW_E_INVALID, "bad precision");
    if (p.krylov < OPFLOW_KRYLOV_PCG || p.krylov > OPFLOW_KRYLOV_NONE) return fail(OPFLOW_E_INVALID, "bad Krylov method %d", p.krylov);
    if (p.precond == OPFLOW_PRECOND_AMG) return fail(OPFLOW_E_UNSUPPORTED, "AMG preconditioning is for equation sets (opflow_eqnset_*)");
    if (p.precond < OPFLOW_PRECOND_MG || p.precond > OPFLOW_PRECOND_NONE) return fail(OPFLOW_E_INVALID, "bad preconditioner %d", p.precond);
    if (p.krylov == OPFLOW_KRYLOV_NONE && p.precond == OPFLOW_PRECOND_NONE) return fail(OPFLOW_E_INVALID, "no solver: neither a Krylov method nor a preconditioner");
    if (p.kdim <= 0) p.kdim = 5;
    if (p.kdim > 60) return fail(OPFLOW_E_INVALID, "kdim must be at most 60");
    if (p.abs_tol < 0) return fail(OPFLOW_E_INVALID, "negative abs_tol");
    if (p.coarse_max <= 0) p.coarse_max = 64;
    auto* s = new opflow_solver_s();
    s->ctx = ctx;
    s->target = target;
    s->tree.assign(nodes, nodes + n_nodes);
    s->leaves.assign(leaves, leaves + n_leaves);
    s->unknown = unknown_slot;
    s->params = p;
    int rc = build_system(s);
    s->assembled_versions = leaf_versions(s);
    if (rc) {
        if (s->S) mg_destroy(s->S);
        delete s;
        return rc;
    }
    *out = s;
    return OPFLOW_OK;
}

int opflow_solver_solve(opflow_solver s, opflow_solve_state* state) {
    if (!s) return fail(OPFLOW_E_INVALID, "null solver");
    using clk = std::chrono::steady_clock;
    auto t0 = clk::now();
    opflow_ctx ctx = s->ctx;
    // generateAb on the first solve and on every later one, generateb only when staticMat
    // (HYPREEqnSolveHandler.hpp:190-209).  The first solve reuses the system assembled at creation
    // unless a field of the equation was written since.
    if (s->first && leaf_versions(s) != s->assembled_versions) OPG_TRY(build_system(s));
    else if (!s->first) {
        if (s->params.static_mat) {
            // generateb: the right-hand side alone, from a plan compiled once (the leaves' current buffers)
            if (!s->rhs_plan_ok) {
                OPG_TRY(asm_prepare(ctx, s->target, s->tree.data(), (int) s->tree.size(), s->leaves.data(), (int) s->leaves.size(), s->unknown, 0,
                                    &s->rhs_plan));
                s->rhs_plan_ok = true;
            }
            for (size_t k = 0; k < s->leaves.size(); ++k) s->rhs_plan.P.leaves[k] = s->leaves[k]->view();
            OPG_TRY(asm_run(ctx, &s->rhs_plan, nullptr, s->S->probs[0].b));
        } else {
            OPG_TRY(build_system(s));
        }
    }
    s->first = false;
    MGSystem* S = s->S;
    ProblemHost& P = S->probs[0];
    const KrylovDev& K = S->kd_host[0];
    const long long N = P.levels[0].N;
    const Box box = assign_box(s->target->info);
    // initial guess: the target's current values (initx)
    if (s->params.zero_guess) cudaMemsetAsync(K.x, 0, N * 8, ctx->stream);
    else {
        gather_box<<<gridN(ctx, N), 256, 0, ctx->stream>>>(s->target->view(), box, K.x);
        OPG_LAUNCHED();
    }
    const bool pinned = P.singular && !P.has_dirichlet && s->params.pin_value;
    OPG_TRY(ensure_scratch(ctx, 4096));
    double* dsc = (double*) ctx->scratch;  // [40]: sum of b, [41]: pinned shift; [64..320): partial sums
    if (P.singular && !P.has_dirichlet) {
        // the pinned system equals the singular one with b[0] := -(sum of the others), shifted after
        sum_partials<<<256, 256, 0, ctx->stream>>>(P.b, N, dsc + 64);
        singular_rhs<<<1, 32, 0, ctx->stream>>>(dsc + 64, 256, P.b, pinned ? 1 : 0, dsc + 40);
        if (!pinned) add_scaled_sum<<<gridN(ctx, N), 256, 0, ctx->stream>>>(P.b, N, dsc + 40);
        OPG_LAUNCHED();
    }
    auto t1 = clk::now();
    int iters = 0;
    if (s->params.krylov == OPFLOW_KRYLOV_PCG && s->params.precond == OPFLOW_PRECOND_MG) {
        OPG_TRY(mg_solve(S));
        std::vector<Scal> st;
        OPG_TRY(mg_states(S, st));
        iters = st[0].iters;
    } else {
        KrylovParams kp;
        kp.method = s->params.krylov;
        kp.precond = s->params.precond;
        kp.kdim = s->params.kdim;
        kp.max_iter = s->params.max_iter;
        kp.tol = s->params.tol;
        kp.abs_tol = s->params.abs_tol;
        OPG_TRY(krylov_solve(S, kp, &iters));
    }
    if (pinned) {
        // the reference's b (the pinned row's right-hand side is 0) and x shifted so that x[0] = 0
        OPG_CUDA(cudaMemsetAsync(P.b, 0, 8, ctx->stream));
        save_first<<<1, 32, 0, ctx->stream>>>(K.x, dsc + 41);
        sub_slot<<<gridN(ctx, N), 256, 0, ctx->stream>>>(K.x, N, dsc + 41);
        OPG_LAUNCHED();
    }
    // true residual of the reference's system (a pinned system's first row, the identity with b = 0, is
    // satisfied exactly after the shift and is left out of r.r instead of being subtracted afterwards,
    // which would cancel catastrophically: that row's residual in the singular operator is O(||b||))
    OPG_TRY(kr_launch_apply(ctx->stream, ctx->num_sms, S->dL, S->dK, S->dk0, S->nk0, nullptr, S->partial, 0, Finish{}, 0, false, pinned));
    OPG_TRY(kr_launch_reduce(ctx->stream, ctx->num_sms, S->partial, S->dfirst, S->dcount, 1, S->red));
    double red[2];
    OPG_CUDA(cudaMemcpyAsync(red, S->red, sizeof red, cudaMemcpyDeviceToHost, ctx->stream));
    OPG_CUDA(cudaStreamSynchronize(ctx->stream));
    const double rr = red[1], bb = red[0];
    scatter_box<<<gridN(ctx, N), 256, 0, ctx->stream>>>(s->target->view(), box, K.x, 0.);
    OPG_LAUNCHED();
    s->target->bc_fresh[s->target->cur] = false;
    s->target->version++;
    s->assembled_versions = leaf_versions(s);
    OPG_TRY(update_padding_buf(s->target, s->target->buf[s->target->cur]));
    OPG_CUDA(cudaStreamSynchronize(ctx->stream));
    auto t2 = clk::now();
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

int opflow_solver_destroy(opflow_solver s) {
    if (!s) return OPFLOW_OK;
    mg_destroy(s->S);
    delete s;
    return OPFLOW_OK;
}

}  // extern "C"
