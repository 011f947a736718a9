// Host-side multigrid hierarchy and flexible-PCG driver (solver.cu); used by the single-problem
// solver, the batched solves and the request server.
#pragma once
#include "assemble.h"
#include "mg_kernels.h"

namespace opg {

// Bump allocator over large device blocks (one solver / batch owns one).
struct Arena {
    std::vector<void*> blocks;
    size_t cap = 0, used = 0, total = 0;
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
    std::vector<std::vector<Chunk>> smooth_ch, restrict_ch, prolong_ch;
    std::vector<ChunkList> d_smooth, d_restrict, d_prolong;
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
    std::vector<KrylovDev> kd_host;
    int* h_active = nullptr;
    int* d_active = nullptr;  // device count of active problems (owned, so a recorded graph never dangles)
    cudaGraphExec_t exec = nullptr;
    long long graph_launches = 0;
};

int mg_add_problem(MGSystem* S, opflow_field target, const opflow_node* nodes, int n_nodes, const opflow_field* leaves, int n_leaves, int unknown);
int mg_finalize(MGSystem* S);
int mg_solve(MGSystem* S);
int mg_states(MGSystem* S, std::vector<Scal>& out);
void mg_destroy(MGSystem* S);

}  // namespace opg
