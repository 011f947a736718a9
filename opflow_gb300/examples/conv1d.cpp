// 1D linear convection, written against OpFlow's user API (examples/CONV1D/CONV1D.cpp of the
// reference) and compiled against the GB300 engine's front end.
//
//   conv1d <n> <steps> <scheme> <out.bin>
//
// n nodes on [0,1], Dirichlet 0 at both ends, a square pulse on [0.2, 0.4], c = 1, dt = 0.005.
// scheme:
//   upwind   u = u - dt*c*dx<D1FirstOrderBiasedDownwind>(u)              (the reference example)
//   cond     u = u - dt*c*conditional(c > 0, dx<Downwind>(u), dx<Upwind>(u)), with a cell field c
//   minmod   u = u - dt*dx<D1FirstOrderCentered>(c*d1Intp<0, Cor2Cen, D1Minmod>(c, u)): a limited
//            flux at the cell centres, differenced back to the nodes
// Writes the final data array (padded layout, float64) to out.bin.
#include <opflow_gb300/OpFlowGPU.hpp>

#include <cstdio>
#include <cstdlib>
#include <cstring>

using namespace OpFlow;

int main(int argc, char** argv) {
    if (argc < 5) {
        std::fprintf(stderr, "usage: conv1d n steps upwind|cond|minmod out.bin\n");
        return 2;
    }
    const int n = std::atoi(argv[1]), steps = std::atoi(argv[2]);
    const char* scheme = argv[3];
    EnvironmentGardian _(&argc, &argv);
    using Mesh = CartesianMesh<Meta::int_<1>>;
    using Field = CartesianField<Real, Mesh>;
    auto mesh = MeshBuilder<Mesh>().newMesh(n).setMeshOfDim(0, 0., 1.).build();
    auto u = ExprBuilder<Field>()
                     .setMesh(mesh)
                     .setName("u")
                     .setBC(0, DimPos::start, BCType::Dirc, 0.)
                     .setBC(0, DimPos::end, BCType::Dirc, 0.)
                     .setLoc(LocOnMesh::Corner)
                     .setExt(2)
                     .build();
    u.initBy([](auto&& x) { return 0.2 <= x[0] && x[0] <= 0.4 ? 1.0 : 0.0; });
    auto c = ExprBuilder<Field>()
                     .setMesh(mesh)
                     .setName("c")
                     .setBC(0, DimPos::start, BCType::Neum, 0.)
                     .setBC(0, DimPos::end, BCType::Neum, 0.)
                     .setLoc(LocOnMesh::Center)
                     .setExt(1)
                     .build();
    c = 1.0;
    const Real dt = 0.5e-2, cv = 1.0;
    for (int i = 0; i < steps; ++i) {
        if (!std::strcmp(scheme, "upwind")) u = u - dt * cv * dx<D1FirstOrderBiasedDownwind>(u);
        else if (!std::strcmp(scheme, "cond"))
            u = u - dt * cv * conditional(cv > 0., dx<D1FirstOrderBiasedDownwind>(u), dx<D1FirstOrderBiasedUpwind>(u));
        else u = u - dt * dx<D1FirstOrderCentered>(c * d1Intp<0, IntpDirection::Cor2Cen, D1Minmod>(c, u));
    }
    const std::vector<Real>& out = u.data();
    FILE* f = std::fopen(argv[4], "wb");
    if (!f || std::fwrite(out.data(), sizeof(Real), out.size(), f) != out.size()) return 1;
    std::fclose(f);
    return 0;
}
