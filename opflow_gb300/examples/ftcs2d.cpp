// FTCS heat equation in 2D, written against OpFlow's user API (examples/FTCS2D/FTCS-OMP.cpp of the
// reference) and compiled against the GB300 engine's front end.
//
//   ftcs2d <n> <steps> <seed> <out.bin> [fast]
//
// n x n node grid on [0,1]^2, Dirichlet 0 on all sides, u0 ~ U[0,1) on the interior from a counter-based
// splitmix64 stream (value k = j*n + i), alpha = 1, dt = 0.2*h^2; writes the final data array (padded
// layout, float64) to out.bin.
#include <opflow_gb300/OpFlowGPU.hpp>

#include <cstdint>
#include <cstdio>
#include <cstdlib>

using namespace OpFlow;

static uint64_t mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
static double u01(uint64_t seed, uint64_t k) { return (double) (mix64(seed + (k + 1) * 0x9E3779B97F4A7C15ull) >> 11) * 0x1.0p-53; }

int main(int argc, char** argv) {
    if (argc < 5) {
        std::fprintf(stderr, "usage: ftcs2d n steps seed out.bin [fast]\n");
        return 2;
    }
    const int n = std::atoi(argv[1]), steps = std::atoi(argv[2]);
    const uint64_t seed = std::strtoull(argv[3], nullptr, 10);
    if (argc > 5) GPU::setEvalMode(OPFLOW_EVAL_FAST);
    EnvironmentGardian _(&argc, &argv);
    using Mesh = CartesianMesh<Meta::int_<2>>;
    using Field = CartesianField<Real, Mesh>;
    auto mesh = MeshBuilder<Mesh>().newMesh(n, n).setMeshOfDim(0, 0., 1.).setMeshOfDim(1, 0., 1.).build();
    auto u = ExprBuilder<Field>()
                     .setName("u")
                     .setMesh(mesh)
                     .setBC(0, DimPos::start, BCType::Dirc, 0.)
                     .setBC(0, DimPos::end, BCType::Dirc, 0.)
                     .setBC(1, DimPos::start, BCType::Dirc, 0.)
                     .setBC(1, DimPos::end, BCType::Dirc, 0.)
                     .build();
    u = 0;
    std::vector<Real> v = u.data();
    DS::MDIndex<2> i;
    for (i[1] = u.assignableRange.start[1]; i[1] < u.assignableRange.end[1]; ++i[1])
        for (i[0] = u.assignableRange.start[0]; i[0] < u.assignableRange.end[0]; ++i[0])
            v[u.linear(i)] = u01(seed, (uint64_t) i[1] * (uint64_t) n + (uint64_t) i[0]);
    u.setData(v);
    const Real h = 1.0 / (n - 1), dt = 0.2 * h * h, alpha = 1.0;
    for (int s = 0; s < steps; ++s) u = u + dt * alpha * (d2x<D2SecondOrderCentered>(u) + d2y<D2SecondOrderCentered>(u));
    const std::vector<Real>& out = u.data();
    FILE* f = std::fopen(argv[4], "wb");
    if (!f || std::fwrite(out.data(), sizeof(Real), out.size(), f) != out.size()) return 1;
    std::fclose(f);
    std::printf("center %.17g\n", u.evalAt(DS::MDIndex<2> {n / 2, n / 2}));
    return 0;
}
