// Runs OpFlow's own CPU implementation of the explicit-evaluation and stencil-assembly paths on small
// cases and writes raw dumps, so that the restated oracle (oracle/oracle.c) and the CUDA library can be
// checked against the reference's actual output.  Test infrastructure only: it is compiled by
// oracle/build_ref.sh into oracle/_ref/ and used to (re)generate tests/golden/ fixtures.
//
// Output format (little-endian, one file per run): a sequence of records, each a text line
// "FIELD <json>\n" or "STENCIL <json>\n" followed by the raw float64 payload the json describes.
#include "OpFlowCoreNoSolvers.hpp"
#include "DataStructures/StencilPad.hpp"
#include "Math/Function/Numeric.hpp"
// The reference's raw binary writer calls CartesianField::evalSafeAt, which its CartesianField no
// longer declares; for the indices it visits (the local range) evalAt returns the same stored value.
#define evalSafeAt evalAt
#include "Utils/Writers/RawBinaryStream.hpp"
#undef evalSafeAt

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

using namespace OpFlow;

#include "ref_common.hpp"

// ---------------------------------------------------------------------------------------------------
// Explicit path
// ---------------------------------------------------------------------------------------------------
static int run_ftcs2d(int n, int steps, uint64_t seed, double bcv, double cfl) {
    using Mesh = CartesianMesh<Meta::int_<2>>;
    using Field = CartesianField<Real, Mesh>;
    auto mesh = MeshBuilder<Mesh>().newMesh(n, n).setMeshOfDim(0, 0., 1.).setMeshOfDim(1, 0., 1.).build();
    auto u = ExprBuilder<Field>()
                     .setName("u")
                     .setMesh(mesh)
                     .setBC(0, DimPos::start, BCType::Dirc, bcv)
                     .setBC(0, DimPos::end, BCType::Dirc, bcv)
                     .setBC(1, DimPos::start, BCType::Dirc, bcv)
                     .setBC(1, DimPos::end, BCType::Dirc, bcv)
                     .build();
    rangeFor_s(u.assignableRange, [&](auto&& i) { u[i] = u01(seed, (uint64_t) i[1] * n + i[0]); });
    u.updatePadding();
    const Real h = 1.0 / (n - 1);
    const Real dt = cfl * h * h, alpha = 1.0;
    for (int s = 0; s < steps; ++s)
        u = u + dt * alpha * (d2x<D2SecondOrderCentered>(u) + d2y<D2SecondOrderCentered>(u));
    dump_field(u, "u");
    return 0;
}

static int run_ftcs3d(int n, int steps, uint64_t seed, double cfl) {
    using Mesh = CartesianMesh<Meta::int_<3>>;
    using Field = CartesianField<Real, Mesh>;
    auto mesh = MeshBuilder<Mesh>()
                        .newMesh(n, n, n)
                        .setMeshOfDim(0, 0., 1.)
                        .setMeshOfDim(1, 0., 1.)
                        .setMeshOfDim(2, 0., 1.)
                        .build();
    auto b = ExprBuilder<Field>().setName("u").setMesh(mesh);
    for (int d = 0; d < 3; ++d) {
        b.setBC(d, DimPos::start, BCType::Dirc, 0.);
        b.setBC(d, DimPos::end, BCType::Dirc, 0.);
    }
    auto u = b.build();
    // 8 Gaussians: centre in [0.2,0.8]^3, width in [0.03,0.1], amplitude in [0.5,1]
    double c[8][3], w[8], a[8];
    for (int g = 0; g < 8; ++g) {
        for (int d = 0; d < 3; ++d) c[g][d] = 0.2 + 0.6 * u01(seed, 5 * g + d);
        w[g] = 0.03 + 0.07 * u01(seed, 5 * g + 3);
        a[g] = 0.5 + 0.5 * u01(seed, 5 * g + 4);
    }
    u.initBy([&](auto&& x) {
        double s = 0.;
        for (int g = 0; g < 8; ++g) {
            double r2 = (x[0] - c[g][0]) * (x[0] - c[g][0]) + (x[1] - c[g][1]) * (x[1] - c[g][1])
                        + (x[2] - c[g][2]) * (x[2] - c[g][2]);
            s += a[g] * std::exp(-r2 / (w[g] * w[g]));
        }
        return s;
    });
    dump_field(u, "u0");
    const Real h = 1.0 / (n - 1);
    const Real dt = cfl * h * h, alpha = 1.0;
    for (int s = 0; s < steps; ++s)
        u = u
            + dt * alpha
                      * (d2x<D2SecondOrderCentered>(u) + d2y<D2SecondOrderCentered>(u)
                         + d2z<D2SecondOrderCentered>(u));
    dump_field(u, "u");
    return 0;
}

// Periodic WENO5-JS + Shu-Osher RK3 on a 2D cell-centred field, derivative along dim 0 only.
static int run_weno(int nx, int ny, int steps, uint64_t seed, int upwind_kernel) {
    using Mesh = CartesianMesh<Meta::int_<2>>;
    using Field = CartesianField<Real, Mesh>;
    const double Lx = 1.0, Ly = 1.0;
    auto mesh = MeshBuilder<Mesh>().newMesh(nx + 1, ny + 1).setMeshOfDim(0, 0., Lx).setMeshOfDim(1, 0., Ly).build();
    auto u = ExprBuilder<Field>()
                     .setName("u")
                     .setMesh(mesh)
                     .setLoc(LocOnMesh::Center)
                     .setBC(0, DimPos::start, BCType::Periodic)
                     .setBC(0, DimPos::end, BCType::Periodic)
                     .setBC(1, DimPos::start, BCType::Periodic)
                     .setBC(1, DimPos::end, BCType::Periodic)
                     .setExt(3)
                     .build();
    // per line: a square pulse [x0, x0+wd) of height A plus a sine of amplitude B and wave number m
    rangeFor_s(u.assignableRange, [&](auto&& i) {
        uint64_t line = (uint64_t) i[1];
        double x0 = 0.6 * u01(seed, 4 * line), wd = 0.1 + 0.2 * u01(seed, 4 * line + 1);
        double A = 0.5 + u01(seed, 4 * line + 2);
        double B = 0.5 * u01(seed, 4 * line + 3);
        int m = 1 + (int) (line % 4);
        double x = (i[0] + 0.5) / nx;
        u[i] = (x >= x0 && x < x0 + wd ? A : 0.0) + B * std::sin(2.0 * 3.141592653589793 * m * x);
    });
    u.updatePadding();
    dump_field(u, "u0");
    auto u1 = u, u2 = u;
    const Real h = Lx / nx, dt = 0.5 * h;
    for (int s = 0; s < steps; ++s) {
        if (upwind_kernel) {
            u1 = u - dt * d1<D1WENO53Upwind<0>>(u);
            u2 = 0.75 * u + 0.25 * (u1 - dt * d1<D1WENO53Upwind<0>>(u1));
            u = 1.0 / 3.0 * u + 2.0 / 3.0 * (u2 - dt * d1<D1WENO53Upwind<0>>(u2));
        } else {
            u1 = u - dt * d1<D1WENO53Downwind<0>>(u);
            u2 = 0.75 * u + 0.25 * (u1 - dt * d1<D1WENO53Downwind<0>>(u1));
            u = 1.0 / 3.0 * u + 2.0 / 3.0 * (u2 - dt * d1<D1WENO53Downwind<0>>(u2));
        }
    }
    dump_field(u, "u");
    return 0;
}

// One-sided first differences and corner-to-centre interpolation on a stretched 2D mesh.
static double stretched(int i, int n) {
    const double t = (double) i / (double) (n - 1);
    return t + 0.25 * t * (1.0 - t);
}
static int run_ops(int nx, int ny, uint64_t seed) {
    using Mesh = CartesianMesh<Meta::int_<2>>;
    using Field = CartesianField<Real, Mesh>;
    auto mesh = MeshBuilder<Mesh>()
                        .newMesh(nx + 1, ny + 1)
                        .setMeshOfDim(0, [&](int i) { return stretched(i, nx + 1); })
                        .setMeshOfDim(1, [&](int i) { return stretched(i, ny + 1) * 2.0; })
                        .build();
    // the mesh itself (extended range), so that the restated MeshBuilder is pinned too
    for (int d = 0; d < 2; ++d) {
        auto er = mesh.getExtRange();
        std::vector<double> xs, dxs;
        for (int i = er.start[d]; i < er.end[d]; ++i) xs.push_back(mesh.x(d, i));
        for (int i = er.start[d]; i < er.end[d] - 1; ++i) dxs.push_back(mesh.dx(d, i));
        fprintf(g_out, "FIELD {\"name\":\"mesh_x%d\",\"count\":%zu}\n", d, xs.size());
        put(xs);
        fprintf(g_out, "FIELD {\"name\":\"mesh_dx%d\",\"count\":%zu}\n", d, dxs.size());
        put(dxs);
    }
    // c: cell-centred, Dirc 0.5 / Neum -1 along x, periodic along y
    auto c = ExprBuilder<Field>()
                     .setName("c")
                     .setMesh(mesh)
                     .setLoc(LocOnMesh::Center)
                     .setBC(0, DimPos::start, BCType::Dirc, 0.5)
                     .setBC(0, DimPos::end, BCType::Neum, -1.0)
                     .setBC(1, DimPos::start, BCType::Periodic)
                     .setBC(1, DimPos::end, BCType::Periodic)
                     .setExt(1)
                     .build();
    rangeFor_s(c.assignableRange, [&](auto&& i) { c[i] = u01(seed, (uint64_t) i[1] * nx + i[0]); });
    c.updatePadding();
    // v: nodal, Dirc 0.25 / Dirc -0.75 along x, Neum 0 / Dirc 1 along y
    auto v = ExprBuilder<Field>()
                     .setName("v")
                     .setMesh(mesh)
                     .setLoc(LocOnMesh::Corner)
                     .setBC(0, DimPos::start, BCType::Dirc, 0.25)
                     .setBC(0, DimPos::end, BCType::Dirc, -0.75)
                     .setBC(1, DimPos::start, BCType::Neum, 0.)
                     .setBC(1, DimPos::end, BCType::Dirc, 1.0)
                     .setExt(1)
                     .build();
    rangeFor_s(v.assignableRange, [&](auto&& i) { v[i] = u01(seed + 1, (uint64_t) i[1] * (nx + 1) + i[0]); });
    v.updatePadding();
    dump_field(c, "c");
    dump_field(v, "v");
    auto c_up0 = c, c_dn1 = c, c_mix = c;
    c_up0 = d1<D1FirstOrderBiasedUpwind<0>>(c);
    c_dn1 = d1<D1FirstOrderBiasedDownwind<1>>(c);
    c_mix = c + 0.25 * d1IntpCornerToCenter<1>(d1IntpCornerToCenter<0>(v)) - 0.3 * dx<D1FirstOrderBiasedDownwind>(c);
    dump_field(c_up0, "c_up0");
    dump_field(c_dn1, "c_dn1");
    dump_field(c_mix, "c_mix");
    auto v_up1 = v, v_dn0 = v;
    v_up1 = dy<D1FirstOrderBiasedUpwind>(v);
    v_dn0 = dx<D1FirstOrderBiasedDownwind>(v);
    dump_field(v_up1, "v_up1");
    dump_field(v_dn0, "v_dn0");
    // corner -> centre along one dim: destinations with the mixed locations
    auto w0 = ExprBuilder<Field>()
                      .setName("w0")
                      .setMesh(mesh)
                      .setLoc({LocOnMesh::Center, LocOnMesh::Corner})
                      .setBC(0, DimPos::start, BCType::Dirc, 0.)
                      .setBC(0, DimPos::end, BCType::Dirc, 0.)
                      .setBC(1, DimPos::start, BCType::Neum, 0.)
                      .setBC(1, DimPos::end, BCType::Dirc, 0.)
                      .build();
    auto w1 = ExprBuilder<Field>()
                      .setName("w1")
                      .setMesh(mesh)
                      .setLoc({LocOnMesh::Corner, LocOnMesh::Center})
                      .setBC(0, DimPos::start, BCType::Dirc, 0.)
                      .setBC(0, DimPos::end, BCType::Dirc, 0.)
                      .setBC(1, DimPos::start, BCType::Neum, 0.)
                      .setBC(1, DimPos::end, BCType::Dirc, 0.)
                      .build();
    w0 = d1IntpCornerToCenter<0>(v);
    w1 = d1IntpCornerToCenter<1>(v);
    dump_field(w0, "w0");
    dump_field(w1, "w1");
    return 0;
}

// Comparisons, logic, conditionals, per-element functions and flux-limiter interpolation on the
// stretched mesh of run_ops.
template <typename K>
using FL = typename D1FluxLimiterGen<K>::template Op<0, IntpDirection::Cen2Cor>;
static int run_logic(int nx, int ny, uint64_t seed) {
    using Mesh = CartesianMesh<Meta::int_<2>>;
    using Field = CartesianField<Real, Mesh>;
    auto mesh = MeshBuilder<Mesh>()
                        .newMesh(nx + 1, ny + 1)
                        .setMeshOfDim(0, [&](int i) { return stretched(i, nx + 1); })
                        .setMeshOfDim(1, [&](int i) { return stretched(i, ny + 1) * 2.0; })
                        .build();
    // the x faces / nodes of the flux-limiter targets are Dirichlet at both ends, so that no target
    // point needs a value beyond the operand's one-cell padding
    auto mk = [&](const char* name, LocOnMesh l0, LocOnMesh l1, bool periodic_y) {
        auto b = ExprBuilder<Field>().setName(name).setMesh(mesh).setLoc({l0, l1}).setExt(1);
        b.setBC(0, DimPos::start, BCType::Dirc, 0.5);
        if (l0 == LocOnMesh::Corner && l1 == LocOnMesh::Center) b.setBC(0, DimPos::end, BCType::Dirc, -1.0);
        else b.setBC(0, DimPos::end, BCType::Neum, -1.0);
        if (periodic_y) b.setBC(1, DimPos::start, BCType::Periodic).setBC(1, DimPos::end, BCType::Periodic);
        else b.setBC(1, DimPos::start, BCType::Neum, 0.).setBC(1, DimPos::end, BCType::Dirc, 1.0);
        return b.build();
    };
    auto fill = [&](auto& f, uint64_t s, double shift) {
        auto r = f.assignableRange;
        rangeFor_s(r, [&](auto&& i) { f[i] = u01(s, (uint64_t) i[1] * 1000 + i[0]) - shift; });
        f.updatePadding();
    };
    const auto Cn = LocOnMesh::Center, Co = LocOnMesh::Corner;
    auto c = mk("c", Cn, Cn, true), g = mk("g", Cn, Cn, true);
    auto v = mk("v", Co, Co, false);
    auto ux = mk("ux", Co, Cn, true);  // velocity on the x faces of the cells
    auto uy = mk("uy", Co, Cn, false); // velocity at the y-cell centres of the x nodes
    fill(c, seed, 0.0);
    fill(g, seed + 1, 0.5);
    fill(v, seed + 2, 0.25);
    fill(ux, seed + 3, 0.5);
    fill(uy, seed + 4, 0.5);
    for (auto* f : {&c, &g, &v, &ux, &uy}) dump_field(*f, f->getName().c_str());
    auto out_c = c;
    out_c = conditional(g > 0., dx<D1FirstOrderBiasedDownwind>(c), dx<D1FirstOrderBiasedUpwind>(c));
    dump_field(out_c, "cond");
    out_c = (g > 0.25 && c < 0.5) || !(g >= -0.1);
    dump_field(out_c, "logic");
    out_c = conditional(g != c, max(c, g) - min(g, c), abs(g)) + sqrt(c) * floor(g * 4.) - ceil(c * 3.)
            + round(g * 7.) + trunc(c * 5.) + fdim(c, g) + copysign(c, g) + fmod(c * 7., g + 1.);
    dump_field(out_c, "exactfn");
    out_c = exp(c) * sin(g) + log(g + 1.5) - pow(c, g + 1.) + tanh(g) + atan2(g, c) + hypot(c, g) + erf(g)
            + cbrt(g) + log1p(c) + expm1(g) + cos(c) + sqrt(c * c + g * g);
    dump_field(out_c, "transfn");
    // flux-limiter interpolation: centres -> x faces (c, upwinded by ux) and nodes -> y centres
    // (v, upwinded by uy), one dump per limiter kernel
    auto fx = ux, fy = uy;
    auto both = [&](auto kern, const char* name) {
        using K = decltype(kern);
        fx = d1Intp<0, IntpDirection::Cen2Cor, D1FluxLimiterGen<K>::template Op>(ux, c);
        fy = d1Intp<1, IntpDirection::Cor2Cen, D1FluxLimiterGen<K>::template Op>(uy, v);
        dump_field(fx, (std::string("fx_") + name).c_str());
        dump_field(fy, (std::string("fy_") + name).c_str());
    };
    both(KappaKernel<KappaScheme::CDS> {}, "CDS");
    both(KappaKernel<KappaScheme::QUICK> {}, "QUICK");
    both(KappaKernel<KappaScheme::CUI> {}, "CUI");
    both(KappaKernel<KappaScheme::Fromm> {}, "Fromm");
    both(KappaKernel<KappaScheme::LUI> {}, "LUI");
    both(MinmodKernel {}, "Minmod");
    both(SuperbeeKernel {}, "Superbee");
    both(MUSCLKernel {}, "MUSCL");
    both(HarmonicKernel {}, "Harmonic");
    both(vanAlbadaKernel {}, "vanAlbada");
    both(UMISTKernel {}, "UMIST");
    both(SPL13Kernel {}, "SPL13");
    both(SPLMax12Kernel {}, "SPLMax12");
    both(SPLMax13Kernel {}, "SPLMax13");
    both(KorenLimitedCUIKernel {}, "Koren");
    both(SMARTKernel {}, "SMART");
    both(BSOUKernel {}, "BSOU");
    return 0;
}

// examples/FTCS2D/FTCS-OMP.cpp's computation: n x n nodes on [0,1]^2, Dirichlet 1 on every side, u = 0,
// dt = 0.1 / (n-1)^2, alpha = 1, `steps` updates u = u + dt*alpha*(d2x(u) + d2y(u)).
static int run_ftcs_omp(int n, int steps) {
    using Mesh = CartesianMesh<Meta::int_<2>>;
    using Field = CartesianField<Real, Mesh>;
    auto mesh = MeshBuilder<Mesh>().newMesh(n, n).setMeshOfDim(0, 0., 1.).setMeshOfDim(1, 0., 1.).build();
    auto u = ExprBuilder<Field>()
                     .setName("u")
                     .setMesh(mesh)
                     .setBC(0, DimPos::start, BCType::Dirc, 1.)
                     .setBC(0, DimPos::end, BCType::Dirc, 1.)
                     .setBC(1, DimPos::start, BCType::Dirc, 1.)
                     .setBC(1, DimPos::end, BCType::Dirc, 1.)
                     .build();
    u = 0;
    const Real dt = 0.1 / Math::pow2(n - 1), alpha = 1.0;
    for (int i = 1; i <= steps; ++i) u = u + dt * alpha * (d2x<D2SecondOrderCentered>(u) + d2y<D2SecondOrderCentered>(u));
    dump_field(u, "u");
    return 0;
}

// examples/CONV1D: first-order upwind convection of a square pulse, u = u - dt*c*dx<Downwind>(u).
static int run_conv1d(int n, int steps) {
    using Mesh = CartesianMesh<Meta::int_<1>>;
    using Field = CartesianField<Real, Mesh>;
    auto mesh = MeshBuilder<Mesh>().newMesh(n).setMeshOfDim(0, 0., 1.).build();
    auto u = ExprBuilder<Field>()
                     .setMesh(mesh)
                     .setName("u")
                     .setBC(0, DimPos::start, BCType::Dirc, 0.)
                     .setBC(0, DimPos::end, BCType::Dirc, 0.)
                     .setLoc(LocOnMesh::Corner)
                     .build();
    u.initBy([](auto&& x) { return 0.2 <= x[0] && x[0] <= 0.4 ? 1.0 : 0.0; });
    dump_field(u, "u0");
    const Real dt = 0.5e-2, cc = 1.0;
    for (int s = 0; s < steps; ++s) u = u - dt * cc * dx<D1FirstOrderBiasedDownwind>(u);
    dump_field(u, "u");
    return 0;
}

// Utils::RawBinaryOStream (src/Utils/Writers/RawBinaryStream.hpp:80-152): the two fields of the raw binary
// tests (a cell-centred and a nodal field on a stretched 7 x 6-node mesh) written as
// << TimeStamp(0.25) << c << v << TimeStamp(1.5) << c into <dir>/c_0.cart, v_1.cart, c_2.cart.
static int run_rawbinary(const char* dir, uint64_t seed) {
    using Mesh = CartesianMesh<Meta::int_<2>>;
    using Field = CartesianField<Real, Mesh>;
    const int nx = 6, ny = 5;
    auto mesh = MeshBuilder<Mesh>()
                        .newMesh(nx + 1, ny + 1)
                        .setMeshOfDim(0, [&](int i) { return stretched(i, nx + 1); })
                        .setMeshOfDim(1, [&](int i) { return stretched(i, ny + 1) * 2.0; })
                        .build();
    auto c = ExprBuilder<Field>()
                     .setName("c")
                     .setMesh(mesh)
                     .setLoc(LocOnMesh::Center)
                     .setBC(0, DimPos::start, BCType::Dirc, 0.5)
                     .setBC(0, DimPos::end, BCType::Neum, -1.0)
                     .setBC(1, DimPos::start, BCType::Periodic)
                     .setBC(1, DimPos::end, BCType::Periodic)
                     .setExt(1)
                     .build();
    rangeFor_s(c.assignableRange, [&](auto&& i) { c[i] = u01(seed, (uint64_t) i[1] * (nx + 1) + i[0]); });
    c.updatePadding();
    auto v = ExprBuilder<Field>()
                     .setName("v")
                     .setMesh(mesh)
                     .setLoc(LocOnMesh::Corner)
                     .setBC(0, DimPos::start, BCType::Dirc, 0.25)
                     .setBC(0, DimPos::end, BCType::Dirc, -0.75)
                     .setBC(1, DimPos::start, BCType::Neum, 0.)
                     .setBC(1, DimPos::end, BCType::Dirc, 1.0)
                     .build();
    rangeFor_s(v.assignableRange, [&](auto&& i) { v[i] = u01(seed + 1, (uint64_t) i[1] * (nx + 1) + i[0]); });
    v.updatePadding();
    dump_field(c, "c");
    dump_field(v, "v");
    Utils::RawBinaryOStream os(std::string(dir) + "/snap");
    os << Utils::TimeStamp(0.25) << c << v;
    os << Utils::TimeStamp(1.5) << c;
    return 0;
}

// Field construction + padding rules: one field per (loc, bc) combination, initialised by a smooth
// function of the coordinates, dumped over its readable range.
static int run_padding(int nx, int ny, int loc_i, int bc_lo, int bc_hi, int ext) {
    using Mesh = CartesianMesh<Meta::int_<2>>;
    using Field = CartesianField<Real, Mesh>;
    auto mesh = MeshBuilder<Mesh>().newMesh(nx, ny).setMeshOfDim(0, 0., 1.).setMeshOfDim(1, 0., 2.).build();
    auto b = ExprBuilder<Field>().setName("f").setMesh(mesh).setLoc(loc_i ? LocOnMesh::Center : LocOnMesh::Corner);
    auto setbc = [&](int d, DimPos pos, int t, double v) {
        switch (t) {
            case 0: b.setBC(d, pos, BCType::Dirc, v); break;
            case 1: b.setBC(d, pos, BCType::Neum, v); break;
            case 2: b.setBC(d, pos, BCType::Periodic); break;
            case 3: b.setBC(d, pos, BCType::Symm); break;
            case 4: b.setBC(d, pos, BCType::ASymm); break;
        }
    };
    // dim 0 uses (bc_lo, bc_hi); dim 1 uses the same types swapped, with different constants
    setbc(0, DimPos::start, bc_lo, 0.25);
    setbc(0, DimPos::end, bc_hi, -0.5);
    setbc(1, DimPos::start, bc_hi, 0.75);
    setbc(1, DimPos::end, bc_lo, 1.5);
    b.setExt(ext);
    auto f = b.build();
    f.initBy([](auto&& x) { return 1.0 + x[0] * x[0] - 0.5 * x[1] + 0.25 * x[0] * x[1]; });
    dump_field(f, "f");
    return 0;
}

// ---------------------------------------------------------------------------------------------------
// Implicit path: the assembly HYPREEqnSolveHandler::generateAb performs, without HYPRE.
// ---------------------------------------------------------------------------------------------------
template <typename Field, typename Getter>
static void assemble_dump(Field& target, Getter&& getter, bool pin) {
    constexpr int dim = internal::CartesianFieldExprTrait<Field>::dim;
    auto st = target.getStencilField();
    st.pin(pin);
    auto stf = std::make_unique<StencilField<Field>>(std::move(st));
    stf->ignorePeriodicBC();
    auto eqn = getter(*stf);
    auto t = eqn.lhs - eqn.rhs;
    t.prepare();
    DS::MDIndex<dim> middle;
    for (int i = 0; i < dim; ++i) middle[i] = (target.assignableRange.start[i] + target.assignableRange.end[i]) / 2;
    auto comm = getOffsetStencil(t.evalAt(middle), middle);
    auto rr = DS::commonRange(target.assignableRange, target.localRange);
    std::string js = std::format("{{\"dim\":{},\"nent\":{},\"range\":[", dim, comm.pad.size());
    for (int d = 0; d < dim; ++d) js += std::format("{}[{},{}]", d ? "," : "", rr.start[d], rr.end[d]);
    js += "],\"offsets\":[";
    int e = 0;
    for (const auto& [k, v] : comm.pad) {
        js += e++ ? ",[" : "[";
        for (int d = 0; d < dim; ++d) js += std::format("{}{}", d ? "," : "", k[d]);
        js += "]";
    }
    js += std::format("],\"count\":{}}}", rr.count());
    fprintf(g_out, "STENCIL %s\n", js.c_str());
    std::vector<double> vals, rhs;
    rangeFor_s(rr, [&](auto&& k) {
        auto cur = getOffsetStencil(t.evalAt(k), k);
        auto ext = commonStencil(cur, comm);
        for (const auto& [key, val] : comm.pad) vals.push_back(ext.pad[key]);
        rhs.push_back(-ext.bias);
    });
    if (pin) {
        // the first unknown's row becomes the identity and its rhs 0
        int e2 = 0;
        for (const auto& [key, val] : comm.pad) {
            bool centre = true;
            for (int d = 0; d < dim; ++d) centre &= key[d] == 0;
            vals[e2++] = centre ? 1.0 : 0.0;
        }
        rhs[0] = 0.0;
    }
    put(vals);
    put(rhs);
}

static int run_assemble(const std::string& which, int n) {
    using Mesh2 = CartesianMesh<Meta::int_<2>>;
    using Field2 = CartesianField<Real, Mesh2>;
    using Mesh3 = CartesianMesh<Meta::int_<3>>;
    using Field3 = CartesianField<Real, Mesh3>;
    if (which == "csr_dirc" || which == "csr_neum" || which == "csr_periodic") {
        // the CSRMatrixGeneratorTest cases: 4x4 cells, h = 1, 1.0 == d2x(e) + d2y(e)
        auto m = MeshBuilder<Mesh2>().newMesh(5, 5).setMeshOfDim(0, 0., 4.).setMeshOfDim(1, 0., 4.).build();
        auto b = ExprBuilder<Field2>().setMesh(m).setName("p").setLoc(LocOnMesh::Center).setExt(1);
        for (int d = 0; d < 2; ++d)
            for (auto pos : {DimPos::start, DimPos::end}) {
                if (which == "csr_dirc") b.setBC(d, pos, BCType::Dirc, 0.);
                else if (which == "csr_neum") b.setBC(d, pos, BCType::Neum, 0.);
                else b.setBC(d, pos, BCType::Periodic);
            }
        auto p = b.build();
        assemble_dump(p, [](auto&& e) { return 1.0 == d2x<D2SecondOrderCentered>(e) + d2y<D2SecondOrderCentered>(e); },
                      which == "csr_neum");
        return 0;
    }
    if (which == "neum2d" || which == "dirc2d" || which == "periodic2d") {
        // -Lap(p) = f in the SPD form f == d2x(e) + d2y(e): A = -L, b = -f
        auto m = MeshBuilder<Mesh2>().newMesh(n + 1, n + 1).setMeshOfDim(0, 0., 1.).setMeshOfDim(1, 0., 1.).build();
        auto b = ExprBuilder<Field2>().setMesh(m).setName("p").setLoc(LocOnMesh::Center).setExt(1);
        for (int d = 0; d < 2; ++d)
            for (auto pos : {DimPos::start, DimPos::end}) {
                if (which == "dirc2d") b.setBC(d, pos, BCType::Dirc, 0.);
                else if (which == "neum2d") b.setBC(d, pos, BCType::Neum, 0.);
                else b.setBC(d, pos, BCType::Periodic);
            }
        auto p = b.build();
        auto f = p;
        rangeFor_s(f.assignableRange, [&](auto&& i) { f[i] = u01(7, (uint64_t) i[1] * n + i[0]) - 0.5; });
        f.updatePadding();
        assemble_dump(p, [&](auto&& e) { return f == d2x<D2SecondOrderCentered>(e) + d2y<D2SecondOrderCentered>(e); },
                      which != "dirc2d");
        return 0;
    }
    if (which == "var2d") {
        // the DircEqnTest operator: dx(dx(e)/intp(r)) + dy(dy(e)/intp(r)), r with a 1000:1 jump
        auto m = MeshBuilder<Mesh2>().newMesh(n + 1, n + 1).setMeshOfDim(0, 0., 1.).setMeshOfDim(1, 0., 1.).build();
        auto mk = [&](double bcv) {
            return ExprBuilder<Field2>()
                    .setMesh(m)
                    .setName("p")
                    .setBC(0, DimPos::start, BCType::Dirc, bcv)
                    .setBC(0, DimPos::end, BCType::Dirc, bcv)
                    .setBC(1, DimPos::start, BCType::Dirc, bcv)
                    .setBC(1, DimPos::end, BCType::Dirc, bcv)
                    .setExt(1)
                    .setLoc({LocOnMesh::Center, LocOnMesh::Center})
                    .build();
        };
        auto p = mk(0.);
        auto r = mk(1.);
        auto bb = mk(0.);
        r.initBy([&](auto&& x) {
            auto dist = Math::norm2(x[0] - 0.5, x[1] - 0.5);
            auto hevi = Math::smoothHeviside(r.getMesh().dx(0, 0) * 8, dist - 0.2);
            return 1. * hevi + (1. - hevi) * 1000;
        });
        rangeFor_s(bb.assignableRange, [&](auto&& i) { bb[i] = u01(11, (uint64_t) i[1] * n + i[0]) - 0.5; });
        bb.updatePadding();
        dump_field(r, "r");
        dump_field(bb, "b");
        assemble_dump(p,
                      [&](auto&& e) {
                          return bb
                                 == dx<D1FirstOrderCentered>(dx<D1FirstOrderCentered>(e) / d1IntpCenterToCorner<0>((r)))
                                            + dy<D1FirstOrderCentered>(dy<D1FirstOrderCentered>(e)
                                                                       / d1IntpCenterToCorner<1>(r));
                      },
                      false);
        return 0;
    }
    if (which == "biased2d") {
        // flux form from one-sided differences on a stretched mesh, Dirichlet cells:
        // f == d1<Down<0>>(K * d1<Up<0>>(e)) + d1<Down<1>>(d1<Up<1>>(e)) - 0.5 * e
        auto m = MeshBuilder<Mesh2>()
                         .newMesh(n + 1, n + 1)
                         .setMeshOfDim(0, [&](int i) { return stretched(i, n + 1); })
                         .setMeshOfDim(1, [&](int i) { return stretched(i, n + 1) * 2.0; })
                         .build();
        auto mk = [&](double bcv) {
            return ExprBuilder<Field2>()
                    .setMesh(m)
                    .setName("p")
                    .setBC(0, DimPos::start, BCType::Dirc, bcv)
                    .setBC(0, DimPos::end, BCType::Dirc, bcv)
                    .setBC(1, DimPos::start, BCType::Dirc, bcv)
                    .setBC(1, DimPos::end, BCType::Dirc, bcv)
                    .setExt(1)
                    .setLoc({LocOnMesh::Center, LocOnMesh::Center})
                    .build();
        };
        auto p = mk(0.25);
        auto K = mk(1.0);
        auto f = mk(0.);
        rangeFor_s(K.assignableRange, [&](auto&& i) { K[i] = 1.0 + u01(17, (uint64_t) i[1] * n + i[0]); });
        K.updatePadding();
        rangeFor_s(f.assignableRange, [&](auto&& i) { f[i] = u01(19, (uint64_t) i[1] * n + i[0]) - 0.5; });
        f.updatePadding();
        dump_field(K, "K");
        dump_field(f, "f");
        assemble_dump(p,
                      [&](auto&& e) {
                          return f
                                 == d1<D1FirstOrderBiasedDownwind<0>>(K * d1<D1FirstOrderBiasedUpwind<0>>(e))
                                            + d1<D1FirstOrderBiasedDownwind<1>>(d1<D1FirstOrderBiasedUpwind<1>>(e))
                                            - 0.5 * e;
                      },
                      false);
        return 0;
    }
    if (which == "funcs2d") {
        // coefficients built from comparisons, conditionals and per-element functions of known fields:
        // f == dx(max(intp0(K), 1.25) * dx(e)) + dy(conditional(intp1(K) > 1.5, sqrt(intp1(K)), intp1(K)) * dy(e))
        //      - (abs(g) + 0.5) * e
        auto m = MeshBuilder<Mesh2>().newMesh(n + 1, n + 1).setMeshOfDim(0, 0., 1.).setMeshOfDim(1, 0., 1.).build();
        auto mk = [&](double bcv) {
            return ExprBuilder<Field2>()
                    .setMesh(m)
                    .setName("p")
                    .setBC(0, DimPos::start, BCType::Dirc, bcv)
                    .setBC(0, DimPos::end, BCType::Dirc, bcv)
                    .setBC(1, DimPos::start, BCType::Neum, 0.)
                    .setBC(1, DimPos::end, BCType::Neum, 0.)
                    .setExt(1)
                    .setLoc({LocOnMesh::Center, LocOnMesh::Center})
                    .build();
        };
        auto p = mk(0.5);
        auto K = mk(1.0);
        auto g = mk(0.);
        auto f = mk(0.);
        rangeFor_s(K.assignableRange, [&](auto&& i) { K[i] = 1.0 + u01(23, (uint64_t) i[1] * n + i[0]); });
        K.updatePadding();
        rangeFor_s(g.assignableRange, [&](auto&& i) { g[i] = u01(29, (uint64_t) i[1] * n + i[0]) - 0.5; });
        g.updatePadding();
        rangeFor_s(f.assignableRange, [&](auto&& i) { f[i] = u01(31, (uint64_t) i[1] * n + i[0]) - 0.5; });
        f.updatePadding();
        dump_field(K, "K");
        dump_field(g, "g");
        dump_field(f, "f");
        assemble_dump(p,
                      [&](auto&& e) {
                          return f
                                 == dx<D1FirstOrderCentered>(max(d1IntpCenterToCorner<0>(K), 1.25)
                                                             * dx<D1FirstOrderCentered>(e))
                                            + dy<D1FirstOrderCentered>(
                                                    conditional(d1IntpCenterToCorner<1>(K) > 1.5,
                                                                sqrt(d1IntpCenterToCorner<1>(K)),
                                                                d1IntpCenterToCorner<1>(K))
                                                    * dy<D1FirstOrderCentered>(e))
                                            - (abs(g) + 0.5) * e;
                      },
                      false);
        return 0;
    }
    if (which == "helm_corner") {
        // (I - k Lap) u = f on a node grid with Dirichlet nodes: e - k*(d2x(e)+d2y(e)) == f
        auto m = MeshBuilder<Mesh2>().newMesh(n, n).setMeshOfDim(0, 0., 1.).setMeshOfDim(1, 0., 1.).build();
        auto b = ExprBuilder<Field2>().setMesh(m).setName("u").setLoc(LocOnMesh::Corner);
        for (int d = 0; d < 2; ++d)
            for (auto pos : {DimPos::start, DimPos::end}) b.setBC(d, pos, BCType::Dirc, 0.125);
        auto u = b.build();
        auto f = u;
        rangeFor_s(f.assignableRange, [&](auto&& i) { f[i] = u01(13, (uint64_t) i[1] * n + i[0]); });
        const double k = 0.0123;
        assemble_dump(u, [&](auto&& e) { return e - k * (d2x<D2SecondOrderCentered>(e) + d2y<D2SecondOrderCentered>(e)) == f; },
                      false);
        return 0;
    }
    if (which == "var3d") {
        // flux form with face coefficient intp(K): f == sum_d dd(intp_d(K) * dd(e)), Neumann, pinned
        auto m = MeshBuilder<Mesh3>()
                         .newMesh(n + 1, n + 1, n + 1)
                         .setMeshOfDim(0, 0., 1.)
                         .setMeshOfDim(1, 0., 1.)
                         .setMeshOfDim(2, 0., 1.)
                         .build();
        auto b = ExprBuilder<Field3>().setMesh(m).setName("p").setLoc(LocOnMesh::Center).setExt(1);
        for (int d = 0; d < 3; ++d)
            for (auto pos : {DimPos::start, DimPos::end}) b.setBC(d, pos, BCType::Neum, 0.);
        auto p = b.build();
        auto K = p, f = p;
        K.initBy([](auto&& x) { return std::exp(std::sin(6.0 * x[0]) * std::cos(4.0 * x[1]) + 0.5 * x[2]); });
        rangeFor_s(f.assignableRange, [&](auto&& i) { f[i] = u01(17, ((uint64_t) i[2] * n + i[1]) * n + i[0]) - 0.5; });
        f.updatePadding();
        dump_field(K, "K");
        dump_field(f, "f");
        assemble_dump(p,
                      [&](auto&& e) {
                          return f
                                 == dx<D1FirstOrderCentered>(d1IntpCenterToCorner<0>(K) * dx<D1FirstOrderCentered>(e))
                                            + dy<D1FirstOrderCentered>(d1IntpCenterToCorner<1>(K)
                                                                       * dy<D1FirstOrderCentered>(e))
                                            + dz<D1FirstOrderCentered>(d1IntpCenterToCorner<2>(K)
                                                                       * dz<D1FirstOrderCentered>(e));
                      },
                      true);
        return 0;
    }
    fprintf(stderr, "unknown assemble case %s\n", which.c_str());
    return 2;
}

int main(int argc, char** argv) {
    if (argc < 3) {
        fprintf(stderr, "usage: ref_driver <out.bin> <cmd> args...\n");
        return 2;
    }
    g_out = fopen(argv[1], "wb");
    if (!g_out) return 3;
    std::string cmd = argv[2];
    auto I = [&](int k) { return std::atoi(argv[k]); };
    auto D = [&](int k) { return std::atof(argv[k]); };
    int rc = 2;
    if (cmd == "ftcs2d") rc = run_ftcs2d(I(3), I(4), std::strtoull(argv[5], nullptr, 10), D(6), D(7));
    else if (cmd == "ftcs3d") rc = run_ftcs3d(I(3), I(4), std::strtoull(argv[5], nullptr, 10), D(6));
    else if (cmd == "weno") rc = run_weno(I(3), I(4), I(5), std::strtoull(argv[6], nullptr, 10), I(7));
    else if (cmd == "padding") rc = run_padding(I(3), I(4), I(5), I(6), I(7), I(8));
    else if (cmd == "ops") rc = run_ops(I(3), I(4), std::strtoull(argv[5], nullptr, 10));
    else if (cmd == "rawbinary") rc = run_rawbinary(argv[3], std::strtoull(argv[4], nullptr, 10));
    else if (cmd == "ftcs_omp") rc = run_ftcs_omp(I(3), I(4));
    else if (cmd == "conv1d") rc = run_conv1d(I(3), I(4));
    else if (cmd == "logic") rc = run_logic(I(3), I(4), std::strtoull(argv[5], nullptr, 10));
    else if (cmd == "assemble") rc = run_assemble(argv[3], argc > 4 ? I(4) : 0);
    fclose(g_out);
    return rc;
}
