// Multigrid / Krylov data structures shared by the kernels (mg.cu) and the host drivers (solver.cu).
#pragma once
#include "internal.h"

namespace opg {

// operator slots: centre, x-, x+, y-, y+, z-, z+
constexpr int NSLOT = 7;
constexpr int NCLASS = 27;  // position classes (first / interior / last cell per dim)
constexpr int TSTRIDE = 8;  // class-table row: the NSLOT coefficients, then the inverse of the centre one

enum GhostRule { GH_ZERO = 0, GH_COPY = 1, GH_WRAP = 2 };

// One level of one problem, as the kernels see it.
struct LvlDev {
    int ndim;
    int n[3];            // unknowns per dim
    int lo[3];           // absolute index of the first unknown (for node-centred transfers)
    long long N;
    int per[3];          // periodic dims (neighbours wrap)
    int gh_lo[3], gh_hi[3];  // prolongation ghost rule per side (GhostRule)
    int node;            // 1: node-centred transfers (coarse I <-> fine 2I), 0: cell-centred (I <-> 2I, 2I+1)
    int table;           // 1: coefficients from the class table, 0: SoA arrays
    int rbgs;            // 1: red-black Gauss-Seidel, 0: damped Jacobi
    int problem;         // owning problem
    int coarsest;        // 1 if no coarser level
    int tiled;           // 1: smoothed by the fused tile kernels (which also restrict into the next level)
    int nslot;           // 2*ndim + 1
    const double* A64;   // [NSLOT][N]
    const float* A32;
    const double* T64;   // [NCLASS][TSTRIDE]
    const float* T32;
    double *x64, *b64, *r64;
    float *x32, *b32, *r32;
    int coarse;          // index of the next coarser level descriptor, -1 if none
    int fine;            // index of the next finer level descriptor, -1 if none
    const double* Ainv64;  // coarsest only: dense (pseudo-)inverse [N][N]
    const float* Ainv32;
};

// A row segment of one level: cells (i0 .. i0+cnt-1, j, k) of level `lvl`.
// The Krylov kernels' chunks on level 0 span `nrows` consecutive rows (j .. j+nrows-1 of plane k).
struct Chunk {
    int lvl;
    int j, k;
    int i0, cnt;
    int nrows = 1;
};

// Per-problem Krylov state (FP64).
struct KrylovDev {
    double *x, *r, *p, *q, *b;  // level-0 vectors of the problem (z is read from the V-cycle's level-0 x)
    int lvl0;                        // descriptor of level 0
    int pin;                         // pinned unknown index (-1 none)
};

struct Scal {
    double rz, pq, zq, rr, bb, alpha, beta;
    double sum_b;   // for the pinned / projected right-hand side
    int active;
    int iters;
    int singular;
    int pad_;
};

// Per-problem reduction of chunk partials fused into the kernel that produces them: the CTA that
// completes a problem's last chunk sums the problem's partials (the fixed order of the separate reduce
// kernel), writes them to red[2p], red[2p+1] and applies scalar stage `stage` (none if stage < 0).
struct Finish {
    int* done;          // [nprob] completed-chunk counters, 0 between launches; nullptr: no fused finish
    const int* first;   // [nprob] first chunk of each problem
    const int* count;   // [nprob] chunks of each problem
    Scal* sc;
    double* red;
    int stage;
    int max_iter;
    double tol;
};

}  // namespace opg
