// Runs OpFlow's own implicit path -- HYPREEqnSolveHandler (generateAb, initx, setup, solve, returnValues)
// driving the vendored HYPRE Struct PCG preconditioned by PFMG -- on small seeded Poisson problems and
// dumps the right-hand side, the coefficient field and the solution it returns, with HYPRE's iteration
// count and final relative residual.  Test infrastructure only: compiled by oracle/build_ref.sh (with
// HYPRE's struct solvers built from their sources by oracle/build_hypre.sh) into oracle/_ref/ and used
// to generate the tests/golden/hypre_*.npz fixtures that pin the GPU solves to the reference's answer.
//
// The call sequence is the one `Solve<PCG, PFMG>(eqn, p, params, pparams)` makes
// (src/Core/Equation/UnifiedSolve.hpp:36-43): a PrecondStructSolver, makeEqnSolveHandler
// (HYPREEqnSolveHandler.hpp:44-48) and one handler->solve() (HYPREEqnSolveHandler.hpp:190-209).
// UnifiedSolve.hpp itself is not included because it pulls in the AMGCL backend (Boost).
//
// Output: the dump format of ref_driver.cpp, plus one "SOLVE <json>\n" record without payload.
#include "OpFlowCoreHYPRE.hpp"
#include "DataStructures/StencilPad.hpp"
#include "Math/Function/Numeric.hpp"

#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

using namespace OpFlow;

#include "ref_common.hpp"

struct SolveOpts {
    double tol = 1e-10;
    int max_iter = 100;
    int two_norm = 1;        // stop on ||r||_2 / ||b||_2 (HYPRE's default is the C-norm r.z)
    int precond_cycles = 0;  // 0: PFMG with HYPRE's defaults (the reference tests' usage); k: k V-cycles, tol 0
};

template <typename Field, typename Getter>
static int solve_and_dump(Field& p, Getter&& getter, bool pin, const SolveOpts& o) {
    StructSolverParams<StructSolverType::PCG> params;
    params.tol = o.tol;
    params.maxIter = o.max_iter;
    params.pinValue = pin;
    if (o.two_norm) params.twoNorm = 1;
    StructSolverParams<StructSolverType::PFMG> pparams;
    if (o.precond_cycles > 0) {
        pparams.maxIter = o.precond_cycles;
        pparams.tol = 0.0;
    }
    auto solver = PrecondStructSolver<StructSolverType::PCG, StructSolverType::PFMG>(params, pparams);
    auto t0 = std::chrono::steady_clock::now();
    auto handler = makeEqnSolveHandler(getter, p, solver);
    auto st = handler->solve();
    auto t1 = std::chrono::steady_clock::now();
    fprintf(g_out, "SOLVE {\"niter\":%d,\"relres\":%.17g,\"seconds\":%.6f,\"pin\":%d,\"two_norm\":%d,\"precond_cycles\":%d}\n",
            st.niter, st.relerr, std::chrono::duration<double>(t1 - t0).count(), pin ? 1 : 0, o.two_norm,
            o.precond_cycles);
    dump_field(p, "x");
    return 0;
}

// Cell-centred 2D Poisson in the SPD form f == d2x(e) + d2y(e) (A = -L, b = -f) on n x n cells of [0,1]^2.
// bc: "neum" (homogeneous Neumann, f projected to zero mean, pinned) or "dirc" (homogeneous Dirichlet).
static int run_poisson2d(const std::string& bc, int n, uint64_t seed, const SolveOpts& o) {
    using Mesh = CartesianMesh<Meta::int_<2>>;
    using Field = CartesianField<Real, Mesh>;
    auto m = MeshBuilder<Mesh>().newMesh(n + 1, n + 1).setMeshOfDim(0, 0., 1.).setMeshOfDim(1, 0., 1.).build();
    auto b = ExprBuilder<Field>().setMesh(m).setName("p").setLoc(LocOnMesh::Center).setExt(1);
    for (int d = 0; d < 2; ++d)
        for (auto pos : {DimPos::start, DimPos::end}) {
            if (bc == "dirc") b.setBC(d, pos, BCType::Dirc, 0.);
            else b.setBC(d, pos, BCType::Neum, 0.);
        }
    auto p = b.build();
    auto f = p;
    rangeFor_s(f.assignableRange, [&](auto&& i) { f[i] = u01(seed, (uint64_t) i[1] * n + i[0]) - 0.5; });
    if (bc != "dirc") {
        double s = 0.;
        rangeFor_s(f.assignableRange, [&](auto&& i) { s += f[i]; });
        s /= (double) f.assignableRange.count();
        rangeFor_s(f.assignableRange, [&](auto&& i) { f[i] -= s; });
    }
    f.updatePadding();
    p = 0.;
    dump_field(f, "f");
    return solve_and_dump(
            p, [&](auto&& e) { return f == d2x<D2SecondOrderCentered>(e) + d2y<D2SecondOrderCentered>(e); },
            bc != "dirc", o);
}

// 3D flux form with a face coefficient interpolated from a cell field K = exp(g), g smooth:
// f == sum_d dd(intp_d(K) * dd(e)), homogeneous Neumann, pinned, on n^3 cells of [0,1]^3.
static int run_var3d(int n, uint64_t seed, const SolveOpts& o) {
    using Mesh = CartesianMesh<Meta::int_<3>>;
    using Field = CartesianField<Real, Mesh>;
    auto m = MeshBuilder<Mesh>()
                     .newMesh(n + 1, n + 1, n + 1)
                     .setMeshOfDim(0, 0., 1.)
                     .setMeshOfDim(1, 0., 1.)
                     .setMeshOfDim(2, 0., 1.)
                     .build();
    auto b = ExprBuilder<Field>().setMesh(m).setName("p").setLoc(LocOnMesh::Center).setExt(1);
    for (int d = 0; d < 3; ++d)
        for (auto pos : {DimPos::start, DimPos::end}) b.setBC(d, pos, BCType::Neum, 0.);
    auto p = b.build();
    auto K = p, f = p;
    K.initBy([](auto&& x) { return std::exp(std::sin(6.0 * x[0]) * std::cos(4.0 * x[1]) + 0.5 * x[2]); });
    rangeFor_s(f.assignableRange,
               [&](auto&& i) { f[i] = u01(seed, ((uint64_t) i[2] * n + i[1]) * n + i[0]) - 0.5; });
    double s = 0.;
    rangeFor_s(f.assignableRange, [&](auto&& i) { s += f[i]; });
    s /= (double) f.assignableRange.count();
    rangeFor_s(f.assignableRange, [&](auto&& i) { f[i] -= s; });
    f.updatePadding();
    p = 0.;
    dump_field(K, "K");
    dump_field(f, "f");
    return solve_and_dump(
            p,
            [&](auto&& e) {
                return f
                       == dx<D1FirstOrderCentered>(d1IntpCenterToCorner<0>(K) * dx<D1FirstOrderCentered>(e))
                                  + dy<D1FirstOrderCentered>(d1IntpCenterToCorner<1>(K) * dy<D1FirstOrderCentered>(e))
                                  + dz<D1FirstOrderCentered>(d1IntpCenterToCorner<2>(K) * dz<D1FirstOrderCentered>(e));
            },
            true, o);
}

// The program tests/adapter/poisson_solve.cpp (OpFlow's own API) on the reference itself: -Lap(p) = f,
// f = sin(3x) cos(2y), on n x n cells, Dirichlet 0, PCG (tol, maxIter; HYPRE's default norm) + PFMG with
// its defaults; one Solve (UnifiedSolve.hpp:36-43: a handler and one solve), then one handler solved
// twice.  Each solve starts from p's current values (HYPREEqnSolveHandler::initx).
static int run_program2d(int n, const SolveOpts& o) {
    using Mesh = CartesianMesh<Meta::int_<2>>;
    using Field = CartesianField<Real, Mesh>;
    auto m = MeshBuilder<Mesh>().newMesh(n + 1, n + 1).setMeshOfDim(0, 0., 1.).setMeshOfDim(1, 0., 1.).build();
    auto b = ExprBuilder<Field>().setMesh(m).setName("p").setLoc(LocOnMesh::Center).setExt(1);
    for (int d = 0; d < 2; ++d) {
        b.setBC(d, DimPos::start, BCType::Dirc, 0.);
        b.setBC(d, DimPos::end, BCType::Dirc, 0.);
    }
    auto p = b.build();
    auto f = p;
    f.initBy([](auto&& x) { return std::sin(3.0 * x[0]) * std::cos(2.0 * x[1]); });
    p = 0.;
    StructSolverParams<StructSolverType::PCG> params;
    params.tol = o.tol;
    params.maxIter = o.max_iter;
    StructSolverParams<StructSolverType::PFMG> pp;
    auto eqn = [&](auto&& e) { return f == d2x<D2SecondOrderCentered>(e) + d2y<D2SecondOrderCentered>(e); };
    auto record = [&](const EqnSolveState& st) {
        fprintf(g_out, "SOLVE {\"niter\":%d,\"relres\":%.17g}\n", st.niter, st.relerr);
    };
    {
        auto solver = PrecondStructSolver<StructSolverType::PCG, StructSolverType::PFMG>(params, pp);
        record(makeEqnSolveHandler(eqn, p, solver)->solve());
    }
    dump_field(p, "x_solve");
    auto solver = PrecondStructSolver<StructSolverType::PCG, StructSolverType::PFMG>(params, pp);
    auto handler = makeEqnSolveHandler(eqn, p, solver);
    for (int k = 0; k < 2; ++k) record(handler->solve());
    dump_field(p, "x");
    return 0;
}

int main(int argc, char** argv) {
    if (argc < 5) {
        fprintf(stderr,
                "usage: ref_solve <out.bin> neum2d|dirc2d|var3d|program2d <n> <seed> [tol] [maxIter] [twoNorm] [pfmgCycles]\n");
        return 2;
    }
    g_out = fopen(argv[1], "wb");
    if (!g_out) return 1;
    std::string cmd = argv[2];
    int n = std::atoi(argv[3]);
    uint64_t seed = std::strtoull(argv[4], nullptr, 10);
    SolveOpts o;
    if (argc > 5) o.tol = std::atof(argv[5]);
    if (argc > 6) o.max_iter = std::atoi(argv[6]);
    if (argc > 7) o.two_norm = std::atoi(argv[7]);
    if (argc > 8) o.precond_cycles = std::atoi(argv[8]);
    int rc;
    if (cmd == "neum2d") rc = run_poisson2d("neum", n, seed, o);
    else if (cmd == "dirc2d") rc = run_poisson2d("dirc", n, seed, o);
    else if (cmd == "var3d") rc = run_var3d(n, seed, o);
    else if (cmd == "program2d") rc = run_program2d(n, o);
    else {
        fprintf(stderr, "unknown case %s\n", cmd.c_str());
        rc = 2;
    }
    fclose(g_out);
    return rc;
}
