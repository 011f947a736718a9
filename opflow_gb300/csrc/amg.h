// Algebraic multigrid by smoothed aggregation: the preconditioner of coupled equation sets
// (OPFLOW_PRECOND_AMG), in place of AMGCL's amg<smoothed_aggregation, spai0> that the reference's
// SolveEqns / AMGCLEqnSolveHandler use (src/Core/Equation/AMGCLEqnSolveHandler.hpp:53-172;
// test/Core/Equation/EqnSetTest.cpp:79-81).
//
// The hierarchy is built on the host from the assembled CSR matrix (amg.cpp) and moved to the device
// once, where every V-cycle runs (amg.cu) - the split AMGCL itself makes for its GPU back ends.
#pragma once
#include "internal.h"

#include <vector>

namespace opg {

// Host CSR matrix, 32-bit column indices.
struct HostCsr {
    long long n = 0, m = 0;  // rows, columns
    std::vector<long long> ptr;
    std::vector<int> col;
    std::vector<double> val;
};

struct AmgParams {
    double eps_strong = 0.08;  // strong connection: a_ij^2 > eps^2 |a_ii a_jj| (halved on every level)
    double relax = 1.0;        // prolongator smoothing weight: omega = relax * 4/3 / rho(D^-1 A_f)
    long long coarse_enough = 500;  // the coarsest level is solved directly (dense inverse)
    int max_levels = 20;
};

struct AmgLevelHost {
    HostCsr A, P, R;          // operator; prolongation to this level from the next; restriction
    std::vector<double> M;    // SPAI-0 smoother: m_i = a_ii / sum_j a_ij^2
};

struct AmgHost {
    std::vector<AmgLevelHost> levels;  // the last level has no P / R
    std::vector<double> coarse_inv;     // dense inverse of the coarsest operator, row-major
};

// The smoothed-aggregation hierarchy of A (square, host CSR).
int amg_build_host(const HostCsr& A, const AmgParams& prm, AmgHost* out);

struct AmgLevelDev {
    long long n = 0, nc = 0;
    long long *Ap = nullptr, *Pp = nullptr, *Rp = nullptr;
    int *Ac = nullptr, *Pc = nullptr, *Rc = nullptr;
    double *Av = nullptr, *Pv = nullptr, *Rv = nullptr;
    double *M = nullptr, *x = nullptr, *b = nullptr, *r = nullptr;
};

struct AmgDev {
    std::vector<AmgLevelDev> levels;
    double* coarse_inv = nullptr;
    long long nc = 0;
    std::vector<void*> allocs;
};

// Moves a host hierarchy to the device (allocations through ctx's pool).
int amg_upload(opflow_ctx ctx, const AmgHost& H, AmgDev* D);
// z = one V-cycle applied to v (level-0 vectors of D.levels[0].n values), on `stream`.
int amg_vcycle(opflow_ctx ctx, cudaStream_t stream, AmgDev& D, const double* v, double* z);
void amg_free(opflow_ctx ctx, AmgDev* D);

}  // namespace opg
