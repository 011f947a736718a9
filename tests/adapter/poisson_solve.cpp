// A program written against OpFlow's own API (the style of test/Core/Equation/DircEqnTest.cpp and
// NeumEqnTest.cpp): -Lap(p) = f on 64 x 64 cells, Dirichlet 0, in the SPD form f == d2x(p) + d2y(p),
// solved with PCG + PFMG through Solve and again through makeEqnSolveHandler (two solves of one
// handler).  tests/golden/make_adapter_golden.py compiles it against OpFlow's headers with the GB300
// adapter ahead of them, so its solves run on the engine's solver.
#include <OpFlow>
using namespace OpFlow;
int main() {
    using Mesh = CartesianMesh<Meta::int_<2>>;
    using Field = CartesianField<Real, Mesh>;
    const int n = 64;
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
    params.tol = 1e-10;
    params.maxIter = 100;
    StructSolverParams<StructSolverType::PFMG> pp;
    auto eqn = [&](auto&& e) { return f == d2x<D2SecondOrderCentered>(e) + d2y<D2SecondOrderCentered>(e); };
    auto st = Solve(eqn, p, params, pp);
    std::printf("Solve: niter %d relerr %.3e\n", st.niter, st.relerr);
    auto solver = PrecondStructSolver<StructSolverType::PCG, StructSolverType::PFMG>(params, pp);
    auto handler = makeEqnSolveHandler(eqn, p, solver);
    for (int k = 0; k < 2; ++k) {
        st = handler->solve();
        std::printf("handler solve %d: niter %d relerr %.3e\n", k, st.niter, st.relerr);
    }
    Utils::RawBinaryOStream os("./p");
    os << p;
    return 0;
}
