// Host-side multigrid hierarchy and flexible-PCG driver (solver.cu); used by the single-problem
// solver, the batched solves and the request server.
#pragma once
#include "assemble.h"
#include "mg_kernels.h"

namespace opg {

struct KrylovWork;  // krylov.cu

// Bump allocator over large device blocks (one solver / batch owns one).
struct Arena {
    opflow_ctx ctx = nullptr;  // blocks come from the context's stream-ordered pool (cudaMalloc if null)
    std::vector<void*> blocks;
    size_t cap = 0, used = 0, total = 0;
    size_t block_hint = (size_t) 256 << 20;  // size of the next block (grows x2 up to 256 MiB)
    void* alloc(size_t bytes);
    void release();
};

struct LevelHost {
    int ndim = 0;
    int n[3] = {1, 1, 1}, lo[3] = {0, 0, 0};
    long long N = 0;
    int node = 0;
    int per[3] = {0, 0, 0};
    int gh_lo[3] = {GH_COPY, GH_COPY, GH_COPY}, gh_hi[3] = {GH_COPY, GH_COPY, GH_COPY};
    bool table = false;
    std::vector<double> tab;
    double* A64 = nullptr;
    float* A32 = nullptr;
    double* T64 = nullptr;
    float* T32 = nullptr;
    double* Ainv64 = nullptr;
    std::vector<opflow_field> owned;  // coarse-level fields created for the rediscretisation
};

struct ProblemHost {
    opflow_field target = nullptr;
    std::vector<opflow_node> tree;
    std::vector<opflow_field> leaves;
    int unknown = 0;
    std::vector<LevelHost> levels;
    double* b = nullptr;  // level-0 right-hand side (assembly output)
    bool singular = false;
    bool has_dirichlet = false;
    int lvl0 = 0;
};

struct ChunkList {
    Chunk* ptr = nullptr;
    int n = 0;
};

struct MGSystem {
    opflow_ctx ctx = nullptr;
    int precision = OPFLOW_PREC_FP64;
    int pre = 2, post = 2;
    int coarse_max = 256;
    double tol = 1e-10;
    int max_iter = 200;
    Arena arena;
    std::vector<ProblemHost> probs;
    int nlevels = 0, nlv = 0;
    // smooth_ch[l]: rows of level l of the problems for which l is not the coarsest level;
    // coarse_sm: rows of coarsest levels that have no dense inverse (they are smoothed instead)
    std::vector<std::vector<Chunk>> smooth_ch, restrict_ch, prolong_ch;
    std::vector<ChunkList> d_smooth, d_restrict, d_prolong;
    // tiles of the levels run by the fused 2D tile kernels (such levels are in none of the lists above)
    std::vector<std::vector<Chunk>> tile_ch;
    std::vector<ChunkList> d_tiles;
    // tiles of the 3D levels smoothed by the z-marching kernel (such levels are not in smooth_ch)
    std::vector<std::vector<Chunk>> zsm_ch;
    std::vector<ChunkList> d_zsm;
    std::vector<int> zb;  // planes per load batch of the z-marching kernels, per level (tuned; MG_ZB_TMA: mg_smooth_zt)
    // tiles of the TMA-staged smoother (float32 levels whose rows hold a multiple of 4 cells)
    std::vector<std::vector<Chunk>> zt_ch;
    std::vector<ChunkList> d_zt;
    std::vector<CUtensorMap> zt_maps;  // the x and b maps of level index l at [2 l], [2 l + 1] (levels with zt tiles)
    // per level: every problem with z tiles there also has zt tiles (only then may the level take the
    // staged smoother, which visits nothing else)
    std::vector<char> zt_full;
    CUtensorMap* d_zt_maps = nullptr;
    bool tune_measure = true;  // false: cached tuner choices only, nothing timed (the request server)
    // the other 2D tile shape of a tiled level, when the tuner is to time it against tile_ch
    std::vector<std::vector<Chunk>> tile_alt;
    std::vector<Chunk> coarse_sm_ch;
    ChunkList d_coarse_sm;
    LvlDev* dL = nullptr;
    KrylovDev* dK = nullptr;
    Scal* dS = nullptr;
    Chunk* dk0 = nullptr;
    int nk0 = 0;
    int *dfirst = nullptr, *dcount = nullptr;
    double* partial = nullptr;
    double* red = nullptr;
    int* dcoarse = nullptr;
    int ncoarse = 0;
    // Levels of at most bottom_max cells run inside one CTA per problem (mg_bottom): bottom_host lists
    // each problem's first such level, coarse_host the coarsest levels above that size (chunked path);
    // both in this system's level numbering
    long long bottom_max = 1024;
    std::vector<int> coarse_host, bottom_host;
    int* dbottom = nullptr;
    int nbottom = 0;
    long long bottom_cells = 0;  // largest cell total of a problem's bottom levels (shared memory of mg_bottom)
    std::vector<long long> bottom_cells_host;  // per entry of bottom_host
    std::vector<KrylovDev> kd_host;
    int* h_active = nullptr;
    int* d_active = nullptr;  // device count of active problems (owned, so a recorded graph never dangles)
    int* d_done = nullptr;    // per-problem chunk counters of the fused reductions (zero between launches)
    cudaGraphExec_t exec = nullptr;        // one iteration (stepped by the request server)
    cudaGraphExec_t solve_exec = nullptr;  // a whole solve: first direction + device-side while loop
    // private stream the iteration graph is recorded on: the caller's stream may be the legacy default
    // stream, which cannot be captured; the recorded graph is then launched on the caller's stream
    cudaStream_t rec_stream = nullptr;
    bool recording = false;
    long long graph_launches = 0;
    // kernels per recorded graph, added to the library's launch counter on every replay (capture itself
    // launches nothing): one stepped iteration, the whole-solve prologue, one whole-solve loop body
    long long iter_kernels = 0, first_kernels = 0, body_kernels = 0;
    bool solve_pending = false;   // a whole-solve launch whose loop count is not yet counted
    int nprob = 0;                       // problems the device tables describe
    // host copies of the device tables (for composing batches out of resident problems)
    std::vector<LvlDev> lv_host;
    std::vector<Chunk> k0_host;
    bool composite = false;              // tables reference other systems' memory
    KrylovWork* kwork = nullptr;         // workspace of the host-driven Krylov methods (arena memory)
};

// The host-driven Krylov methods of krylov.cu (every method but the fused flexible PCG with the
// multigrid preconditioner).
struct KrylovParams {
    int method = OPFLOW_KRYLOV_GMRES;  // enum opflow_krylov
    int precond = OPFLOW_PRECOND_MG;   // enum opflow_precond
    int kdim = 5;
    int max_iter = 100;
    double tol = 1e-10, abs_tol = 0.;
};
// A linear operator with its preconditioner for the host-driven methods.  `residual` defaults to
// matvec + r = b - A x; stream / grid_hint / n are set by krylov_run.
struct KrylovOp {
    cudaStream_t stream = nullptr;
    int grid_hint = 1;
    long long n = 0;
    virtual ~KrylovOp() = default;
    virtual int matvec(const double* x, double* y) = 0;
    virtual int residual(const double* b, const double* x, double* r);
    virtual int precond(const double* v, double* z) = 0;
};
// Workspace sized for P's method (carved from `arena`), and the method itself: x holds the initial
// guess and receives the solution of A x = b.
KrylovWork* krylov_work(Arena& arena, opflow_ctx ctx, long long N, const KrylovParams& P);
bool krylov_work_fits(const KrylovWork* W, long long N, const KrylovParams& P);
void krylov_work_free(KrylovWork* W);
int krylov_run(KrylovOp& op, KrylovWork& W, opflow_ctx ctx, long long N, const KrylovParams& P, double* b, double* x, int* iters);
// Solves the single problem of S in place (K.x holds the initial guess, K.b the right-hand side).
int krylov_solve(MGSystem* S, const KrylovParams& P, int* iters);
void krylov_release(MGSystem* S);
// z = one V-cycle of S's single problem applied to v (level-0 vectors); mg_activate marks the
// problem active for the V-cycle kernels first
int mg_precond_level0(MGSystem* S, const double* v, double* z);
int mg_activate(MGSystem* S);
// one V-cycle on the level-0 input already written (b, x = 0)
int mg_vcycle(MGSystem* S);

// Device tables of a batch assembled from single-problem systems (the problems stay where they are);
// state[i] seeds problem i's Krylov scalars.
int mg_compose(MGSystem* C, const std::vector<MGSystem*>& parts, const std::vector<Scal>& state);
int mg_iteration_graph(MGSystem* S);
int mg_run_iterations(MGSystem* S, int iters);
// r = b - A x, p = 0 and scalars for one problem so that the next batched iteration starts it
int mg_prepare_problem(MGSystem* single, double tol, Scal* out);
int mg_add_problem(MGSystem* S, opflow_field target, const opflow_node* nodes, int n_nodes, const opflow_field* leaves, int n_leaves, int unknown);
// x[0..N) := the target's values over its assignable box, x fastest (HYPREEqnSolveHandler::initx)
int mg_gather_target(opflow_ctx ctx, opflow_field target, double* x);
// sum of v[0..n) (synchronises ctx's stream); v[0..n) += a
double mg_sum(opflow_ctx ctx, const double* v, long long n);
void mg_add_scalar(opflow_ctx ctx, double* v, long long n, double a);
int mg_finalize(MGSystem* S);
int mg_solve(MGSystem* S);
int mg_states(MGSystem* S, std::vector<Scal>& out);
// OPFLOW_E_CUDA when a bounded wait of the staged 3D smoother gave up since the last check
int mg_check_error(MGSystem* S);
void mg_destroy(MGSystem* S);

}  // namespace opg
