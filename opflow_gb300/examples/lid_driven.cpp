// Lid-driven cavity, written with OpFlow's user API as in the reference's examples/LidDriven/LidDriven2D.cpp
// and compiled against the GB300 engine's front end: staggered velocities (u on x faces, v on y faces),
// Crank-Nicolson diffusion with semi-implicit convection solved by GMRES + PFMG, a pinned
// pressure-correction Poisson equation with a static matrix, and the projection.
//
//   lid_driven <n> <steps> <out.bin>
//
// Prints per step the iteration counts of the three solves and the largest |div u| after the
// projection; writes u, v and p (each field's data array, float64) to out.bin.
#include <opflow_gb300/OpFlowGPU.hpp>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>

using namespace OpFlow;

int main(int argc, char** argv) {
    if (argc < 4) {
        std::fprintf(stderr, "usage: lid_driven n steps out.bin\n");
        return 2;
    }
    const int n = std::atoi(argv[1]), steps = std::atoi(argv[2]);
    EnvironmentGardian env(&argc, &argv);
    using Mesh = CartesianMesh<Meta::int_<2>>;
    using Field = CartesianField<Real, Mesh>;

    auto mesh = MeshBuilder<Mesh>().newMesh(n, n).setMeshOfDim(0, 0., 1.).setMeshOfDim(1, 0., 1.).build();
    auto walls = ExprBuilder<Field>().setMesh(mesh).setExt(1);
    for (int d = 0; d < 2; ++d) walls.setBC(d, DimPos::start, BCType::Dirc, 0.).setBC(d, DimPos::end, BCType::Dirc, 0.);
    // the lid moves the top of the u field
    auto u = walls.setName("u").setLoc({LocOnMesh::Corner, LocOnMesh::Center}).setBC(1, DimPos::end, BCType::Dirc, 1.).build();
    auto du = walls.setName("du").setBC(1, DimPos::end, BCType::Dirc, 0.).build();
    auto v = walls.setName("v").setLoc({LocOnMesh::Center, LocOnMesh::Corner}).build();
    auto dv = v;
    for (int d = 0; d < 2; ++d) walls.setBC(d, DimPos::start, BCType::Neum, 0.).setBC(d, DimPos::end, BCType::Neum, 0.);
    auto p = walls.setName("p").setLoc(LocOnMesh::Center).build();
    auto dp = p;
    auto divu = p;
    u = 0; du = 0; v = 0; dv = 0; p = 0; dp = 0;

    // convective fluxes on the staggered grid
    auto cxx = [](auto&& a, auto&& b) { return dx<D1FirstOrderCentered>(d1IntpCornerToCenter<0>(a) * d1IntpCornerToCenter<0>(b)); };
    auto cxy = [](auto&& a, auto&& b) { return dy<D1FirstOrderCentered>(d1IntpCenterToCorner<1>(a) * d1IntpCenterToCorner<0>(b)); };
    auto cyx = [](auto&& a, auto&& b) { return dx<D1FirstOrderCentered>(d1IntpCenterToCorner<1>(a) * d1IntpCenterToCorner<0>(b)); };
    auto cyy = [](auto&& a, auto&& b) { return dy<D1FirstOrderCentered>(d1IntpCornerToCenter<1>(a) * d1IntpCornerToCenter<1>(b)); };
    auto lap = [](auto&& e) { return d2x<D2SecondOrderCentered>(e) + d2y<D2SecondOrderCentered>(e); };

    const Real dt = 0.5e-2, nu = 1.0e-2;
    StructSolverParams<StructSolverType::GMRES> gm;
    gm.tol = 1e-10;
    gm.maxIter = 100;
    StructSolverParams<StructSolverType::PFMG> mg;
    mg.useZeroGuess = true;
    mg.numPreRelax = mg.numPostRelax = 1;
    auto momentum = PrecondStructSolver<StructSolverType::GMRES, StructSolverType::PFMG>(gm, mg);
    auto gp = gm;
    gp.staticMat = true;
    gp.pinValue = true;
    auto pressure = PrecondStructSolver<StructSolverType::GMRES, StructSolverType::PFMG>(gp, mg);

    auto hu = makeEqnSolveHandler(
            [&](auto&& e) {
                return e / dt + cxx(u, e) + 0.5 * cxy(e, v)
                       == nu * lap(u) + 0.5 * nu * lap(e) - (cxx(u, u) + cxy(u, v)) - dx<D1FirstOrderCentered>(p);
            },
            du, momentum);
    auto hv = makeEqnSolveHandler(
            [&](auto&& e) {
                return e / dt + cyy(v, e) + cyy(v, v) + cyx(u, v) + 0.5 * cyx(u, e) + 0.5 * cyx(du, v)
                       == nu * lap(v) + 0.5 * nu * lap(e) - dy<D1FirstOrderCentered>(p);
            },
            dv, momentum);
    auto hp = makeEqnSolveHandler(
            [&](auto&& e) { return lap(e) == (dx<D1FirstOrderCentered>(du) + dy<D1FirstOrderCentered>(dv)) / dt; }, dp, pressure);

    int worst = 0;
    for (int step = 0; step < steps; ++step) {
        const EqnSolveState su = hu->solve();
        const EqnSolveState sv = hv->solve();
        du = du - 0.5 * dt * cxy(u, dv);
        u = u + du;
        v = v + dv;
        const EqnSolveState sp = hp->solve();
        u = u - dt * dx<D1FirstOrderCentered>(dp);
        v = v - dt * dy<D1FirstOrderCentered>(dp);
        p = p + dp;
        divu = dx<D1FirstOrderCentered>(u) + dy<D1FirstOrderCentered>(v);
        Real dmax = 0.;
        const auto& dd = divu.data();
        DS::MDIndex<2> i;
        for (i[1] = divu.assignableRange.start[1]; i[1] < divu.assignableRange.end[1]; ++i[1])
            for (i[0] = divu.assignableRange.start[0]; i[0] < divu.assignableRange.end[0]; ++i[0]) dmax = std::max(dmax, std::fabs(dd[divu.linear(i)]));
        std::printf("step %d iters %d %d %d relerr %.3g %.3g %.3g div %.3g\n", step, su.niter, sv.niter, sp.niter, su.relerr, sv.relerr,
                    sp.relerr, dmax);
        if (!su.converged || !sv.converged || !sp.converged) worst = 1;
    }
    FILE* f = std::fopen(argv[3], "wb");
    if (!f) return 1;
    for (const Field* q : {&u, &v, &p}) {
        const std::vector<Real>& a = q->data();
        if (std::fwrite(a.data(), sizeof(Real), a.size(), f) != a.size()) return 1;
    }
    std::fclose(f);
    return worst;
}
