// Variable-coefficient Poisson problem solved through makeEqnSolveHandler, in the form of the reference's
// DircEqnTest (test/Core/Equation/DircEqnTest.cpp): dx(dx(p)/intp(r)) + dy(dy(p)/intp(r)) == b with
// b the discrete operator applied to p_true, so the solve recovers p_true.
//
//   poisson <n> <fp64|mixed>
//
// Prints the iteration count, the relative residual and the max relative error against p_true.
#include <opflow_gb300/OpFlowGPU.hpp>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>

using namespace OpFlow;

int main(int argc, char** argv) {
    const int n = argc > 1 ? std::atoi(argv[1]) : 64;
    const bool mixed = argc > 2 && std::strcmp(argv[2], "mixed") == 0;
    EnvironmentGardian _(&argc, &argv);
    using Mesh = CartesianMesh<Meta::int_<2>>;
    using Field = CartesianField<Real, Mesh>;
    auto mesh = MeshBuilder<Mesh>().newMesh(n + 1, n + 1).setMeshOfDim(0, 0., 1.).setMeshOfDim(1, 0., 1.).build();
    auto make = [&](Real v) {
        return ExprBuilder<Field>()
                .setMesh(mesh)
                .setLoc(std::array {LocOnMesh::Center, LocOnMesh::Center})
                .setExt(1)
                .setBC(0, DimPos::start, BCType::Dirc, v)
                .setBC(0, DimPos::end, BCType::Dirc, v)
                .setBC(1, DimPos::start, BCType::Dirc, v)
                .setBC(1, DimPos::end, BCType::Dirc, v)
                .build();
    };
    auto p = make(0.), ptrue = make(0.), b = make(0.), r = make(1.);
    ptrue.initBy([](const std::array<Real, 2>& x) { return x[0] * (1. - x[0]) * x[1] * (1. - x[1]); });
    const Real h = 1.0 / n;
    r.initBy([&](const std::array<Real, 2>& x) {
        const Real dist = std::sqrt((x[0] - 0.5) * (x[0] - 0.5) + (x[1] - 0.5) * (x[1] - 0.5)), w = 8 * h;
        const Real t = dist - 0.2;
        const Real hev = t < -w ? 0. : (t > w ? 1. : 0.5 * (1 + t / w + std::sin(M_PI * t / w) / M_PI));
        return hev + (1. - hev) * 1000.;
    });
    auto op = [&](auto&& e) {
        return dx<D1FirstOrderCentered>(dx<D1FirstOrderCentered>(e) / d1IntpCenterToCorner<0>(r))
               + dy<D1FirstOrderCentered>(dy<D1FirstOrderCentered>(e) / d1IntpCenterToCorner<1>(r));
    };
    b = op(ptrue);
    p = 0.;
    StructSolverParams<StructSolverType::PCG> params;
    params.tol = 1e-10;
    params.maxIter = 200;
    params.gpuMixedPrecision = mixed;
    StructSolverParams<StructSolverType::PFMG> p_params;
    auto handler = makeEqnSolveHandler([&](auto&& e) { return b == op(e); }, p, PrecondStructSolver<StructSolverType::PCG, StructSolverType::PFMG>(params, p_params));
    const EqnSolveState st = handler->solve();
    Real err = 0., mx = 0.;
    DS::MDIndex<2> i;
    for (i[1] = p.assignableRange.start[1]; i[1] < p.assignableRange.end[1]; ++i[1])
        for (i[0] = p.assignableRange.start[0]; i[0] < p.assignableRange.end[0]; ++i[0]) {
            err = std::max(err, std::abs(p.evalAt(i) - ptrue.evalAt(i)));
            mx = std::max(mx, std::abs(ptrue.evalAt(i)));
        }
    std::printf("niter %d relerr %.3e converged %d error %.3e\n", st.niter, st.relerr, st.converged ? 1 : 0, err / mx);
    return st.converged && err / mx < 1e-6 ? 0 : 1;
}
