// GB300 engine behind OpFlow's own types: the adapter that makes a program written against OpFlow
// (#include <OpFlow>, CartesianMesh / CartesianField / expressions) run its explicit assignments on
// the GPU through the C ABI of libopflow_gpu (include/opflow_gpu.h), with OpFlow's headers unchanged.
//
// How it plugs in.  Every assignment of a CartesianField - Expr::operator=, +=, -=, *=, /=
// (src/Core/Expr/Expr.hpp:53-81) - ends in internal::FieldAssigner::assign<Op>(src, dst), called from
// CartesianField::assignImpl_final (src/Core/Field/MeshBased/Structured/CartesianField.hpp:179-234) and
// defined in src/Core/Loops/FieldAssigner.hpp:27-84 behind the include guard OPFLOW_FIELDASSIGNER_HPP.
// This header defines that guard and its own FieldAssigner before OpFlow's field headers are read, so
// CartesianField calls this engine instead of the CPU loop.  A program switches to the engine by
// putting include/opflow_gb300/adapter first on its include path: its `#include <OpFlow>` then finds
// the umbrella next to this file, which includes this header and, through it, OpFlow's own headers.
//
// What an assignment does here.  The expression type (Expression<Op, Args...> over CartesianField
// leaves, ScalarExpr and plain numbers) is lowered at compile time into the engine's node program
// (opflow_node, postorder); every field the expression reads and the destination get a device mirror
// (created on first use with the field's mesh, location, boundary conditions, extension and padding;
// its ranges are checked against the field's own); the host data of those fields is uploaded, the
// program runs on the device (opflow_assign, which also refreshes the destination's padding), and the
// destination's data array is downloaded into the field.  Host code therefore sees OpFlow's layout and
// values after every assignment, exactly as with the CPU loop (evaluation mode EXACT: bit-identical to
// the reference; OPFLOW_GB300_EVAL=fast selects the fixed-point mode).
//
// What a solve does here.  makeEqnSolveHandler(getter, target, solver) with a Struct solver and a
// CartesianField target, and Solve(...), return a handler whose solve() runs on the engine's Krylov +
// multigrid solver (the section "the implicit path" below); the equation is lowered like an
// assignment's expression.  The relative tolerance is tested on ||b - Ax||_2 / ||b||_2 (HYPRE PCG's
// default test is the preconditioned norm unless twoNorm is set).
//
// Pieces of OpFlow that need libraries this engine does not use are left out by defining their include
// guards first: the AMGCL back end and UnifiedSolve.hpp (Boost), the CSR matrix generation of the
// AMGCL path (CSRMatrixGenerator, EquationHolder, StencilHolder, DS::CSRMatrix: oneTBB's parallel
// algorithms; the engine assembles coupled sets itself, opflow_eqnset_*), the HDF5 writer (libhdf5)
// and the Tecplot binary / SZPLT writers (TecIO), VTK AMR and IOGroup.  Utils::H5Stream is provided here as a
// stand-in that writes each field as RawBinaryOStream does (<dir>/<name>_<count>.cart next to the given
// path).  RawBinaryStream.hpp still calls CartesianField::evalSafeAt, which OpFlow's field no longer
// declares; it is included with that call renamed to evalAt (the same stored value over the local
// range it visits).
//
// Errors of the C ABI end the program with the library's message and exit(1), as OP_ABORT does.
#pragma once

#include <opflow_gpu.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <type_traits>
#include <unordered_map>
#include <vector>

#include "Core/Macros.hpp"
#include "Core/Constants.hpp"

namespace opflow_gb300::adapter {
template <OpFlow::BasicArithOp Op, typename S, typename D>
D& assign(const S& src, D& dst);
}

// ---- internal::FieldAssigner, replaced (OpFlow's definition: src/Core/Loops/FieldAssigner.hpp) ----
#define OPFLOW_FIELDASSIGNER_HPP
namespace OpFlow::internal {
struct FieldAssigner {
    template <BasicArithOp Op = BasicArithOp::Eq>
    static auto& assign(auto&& src, auto&& dst) {
        return opflow_gb300::adapter::assign<Op>(src, dst);
    }
};
}  // namespace OpFlow::internal

// ---- OpFlow's headers, without the parts that need libraries the engine does not use ----
#define OPFLOW_AMGCLEQNSOLVEHANDLER_HPP
#define OPFLOW_AMGCLBACKEND_HPP
#define OPFLOW_UNIFIEDSOLVE_HPP
#define OPFLOW_CSRMATRIXGENERATOR_HPP
#define OPFLOW_EQUATIONHOLDER_HPP
#define OPFLOW_STENCILHOLDER_HPP
#define OPFLOW_CSRMATRIX_HPP
#define OPFLOW_HDF5STREAM_HPP
#define OPFLOW_TECPLOTSZPLTSTREAM_HPP
#define OPFLOW_TECPLOTBINARYSTREAM_HPP
#define OPFLOW_VTKAMRSTREAM_HPP
#define OPFLOW_IOGROUP_HPP
#include "Core"
#include "DS"
#include "Math"
#define evalSafeAt evalAt
#include "Utils/Writers/RawBinaryStream.hpp"
#undef evalSafeAt
#include "Utils"

namespace opflow_gb300::adapter {

[[noreturn]] inline void die(const char* what) {
    std::fprintf(stderr, "[opflow_gb300] %s: %s\n", what, opflow_last_error());
    std::exit(1);
}
inline void check(int rc, const char* what) {
    if (rc != 0) die(what);
}

// One engine context for the process: device OPFLOW_GB300_DEVICE (default 0).
inline opflow_ctx context() {
    static opflow_ctx ctx = [] {
        opflow_ctx c = nullptr;
        const char* e = std::getenv("OPFLOW_GB300_DEVICE");
        check(opflow_ctx_create(e ? std::atoi(e) : 0, &c), "opflow_ctx_create");
        return c;
    }();
    return ctx;
}

inline int eval_mode() {
    const char* e = std::getenv("OPFLOW_GB300_EVAL");
    return e && std::strcmp(e, "fast") == 0 ? OPFLOW_EVAL_FAST : OPFLOW_EVAL_EXACT;
}

// ---- device mirrors of CartesianFields ------------------------------------------------------------
struct Mirror {
    opflow_field f = nullptr;
    opflow_field_info info{};
    const void* data0 = nullptr;  // address of the field's first data element when the mirror was made
    std::vector<double> x[3], dx[3];
};

inline std::unordered_map<const void*, Mirror>& registry() {
    static std::unordered_map<const void*, Mirror> r;
    return r;
}

template <typename F>
constexpr int dim_of() {
    return OpFlow::internal::CartesianFieldExprTrait<F>::dim;
}

// Address of the field's data element 0 (the padded local range, x fastest: the PlainTensor layout).
template <typename F>
double* host_data(const F& f, const opflow_field_info& info) {
    constexpr int D = dim_of<F>();
    OpFlow::DS::MDIndex<D> i0;
    for (int d = 0; d < D; ++d) i0[d] = info.data_offset[d];
    return &const_cast<F&>(f)[i0];
}

inline int bc_code(OpFlow::BCType t) {
    switch (t) {
        case OpFlow::BCType::Dirc: return OPFLOW_BC_DIRC;
        case OpFlow::BCType::Neum: return OPFLOW_BC_NEUM;
        case OpFlow::BCType::Periodic: return OPFLOW_BC_PERIODIC;
        case OpFlow::BCType::Symm: return OPFLOW_BC_SYMM;
        case OpFlow::BCType::ASymm: return OPFLOW_BC_ASYMM;
        default: return OPFLOW_BC_UNDEFINED;
    }
}

// The mirror of `f`, made on first use (and again if the field's storage or shape changed).
template <typename F>
Mirror& mirror(const F& f) {
    constexpr int D = dim_of<F>();
    auto& reg = registry();
    auto it = reg.find(&f);
    if (it != reg.end()) {
        Mirror& m = it->second;
        if (host_data(f, m.info) == m.data0) return m;
        opflow_field_destroy(m.f);
        reg.erase(it);
    }
    Mirror m;
    const auto& mesh = f.getMesh();
    const auto& rg = mesh.getRange();
    const auto& er = mesh.getExtRange();
    opflow_mesh_desc md{};
    md.ndim = D;
    md.pad_width = rg.start[0] - er.start[0];
    for (int d = 0; d < D; ++d) {
        md.dims[d] = rg.end[d] - rg.start[d];
        md.start[d] = rg.start[d];
        if (rg.start[d] - er.start[d] != md.pad_width || er.end[d] - rg.end[d] != md.pad_width)
            die("the mesh's extension differs between dimensions or sides, which the engine's mesh does not take");
        for (int i = er.start[d]; i < er.end[d]; ++i) m.x[d].push_back(mesh.x(d, i));
        for (int i = er.start[d]; i < er.end[d] - 1; ++i) m.dx[d].push_back(mesh.dx(d, i));
        md.x[d] = m.x[d].data();
        md.dx[d] = m.dx[d].data();
    }
    opflow_field_desc fd{};
    fd.ndim = D;
    fd.padding = f.padding;
    for (int d = 0; d < D; ++d) {
        fd.loc[d] = f.loc[d] == OpFlow::LocOnMesh::Corner ? OPFLOW_CORNER : OPFLOW_CENTER;
        fd.ext[d][0] = f.accessibleRange.start[d] - f.logicalRange.start[d];
        fd.ext[d][1] = f.logicalRange.end[d] - f.accessibleRange.end[d];
        using BCPtr = decltype(f.bc[d].start.get());
        const BCPtr sides[2] = {f.bc[d].start.get(), f.bc[d].end.get()};
        for (int s = 0; s < 2; ++s) {
            if (!sides[s]) die("a field without a boundary condition on some side");
            fd.bc_type[d][s] = bc_code(sides[s]->getBCType());
            fd.bc_value[d][s] = 0.;
            const std::string tn = sides[s]->getTypeName();
            if (tn == "ConstDircBC" || tn == "ConstNeumBC") {
                OpFlow::DS::MDIndex<D> at;
                for (int q = 0; q < D; ++q) at[q] = f.accessibleRange.start[q];
                at[d] = s == 0 ? f.accessibleRange.start[d] : f.accessibleRange.end[d] - 1;
                fd.bc_value[d][s] = sides[s]->evalAt(at);
            } else if (fd.bc_type[d][s] == OPFLOW_BC_DIRC || fd.bc_type[d][s] == OPFLOW_BC_NEUM) {
                die(("boundary condition " + tn + ": the engine takes constant Dirichlet / Neumann values").c_str());
            } else if (fd.bc_type[d][s] == OPFLOW_BC_UNDEFINED) {
                die(("boundary condition " + tn + " is not taken by the engine").c_str());
            }
        }
    }
    check(opflow_field_create(context(), &md, &fd, &m.f), "opflow_field_create");
    check(opflow_field_get_info(m.f, &m.info), "opflow_field_get_info");
    // the engine's ranges must be the field's own (ExprBuilder::calculateRanges restated)
    for (int d = 0; d < D; ++d) {
        const bool same = m.info.logical[d][0] == f.logicalRange.start[d] && m.info.logical[d][1] == f.logicalRange.end[d] &&
                          m.info.accessible[d][0] == f.accessibleRange.start[d] && m.info.accessible[d][1] == f.accessibleRange.end[d] &&
                          m.info.assignable[d][0] == f.assignableRange.start[d] && m.info.assignable[d][1] == f.assignableRange.end[d] &&
                          m.info.local[d][0] == f.localRange.start[d] && m.info.local[d][1] == f.localRange.end[d];
        if (!same) die("the engine's ranges of a field differ from the field's own");
    }
    m.data0 = host_data(f, m.info);
    return reg.emplace(&f, std::move(m)).first->second;
}

// ---- lowering of OpFlow's expression types to the engine's node program ---------------------------
template <typename T, template <typename...> class Tmpl>
struct is_inst : std::false_type {};
template <template <typename...> class Tmpl, typename... A>
struct is_inst<Tmpl<A...>, Tmpl> : std::true_type {};

template <typename T>
struct is_cfield : std::false_type {};
template <typename Dt, typename M, typename C>
struct is_cfield<OpFlow::CartesianField<Dt, M, C>> : std::true_type {};

template <typename Op>
struct op_kind {
    static constexpr int kind = 0;
    static constexpr int dim = 0;
};
#define OPG_ADAPT_BIN(OpT, K)                  \
    template <>                                \
    struct op_kind<OpFlow::OpT> {              \
        static constexpr int kind = K;         \
        static constexpr int dim = 0;          \
    };
OPG_ADAPT_BIN(AddOp, OPFLOW_NODE_ADD)
OPG_ADAPT_BIN(SubOp, OPFLOW_NODE_SUB)
OPG_ADAPT_BIN(MulOp, OPFLOW_NODE_MUL)
OPG_ADAPT_BIN(DivOp, OPFLOW_NODE_DIV)
OPG_ADAPT_BIN(NegOp, OPFLOW_NODE_NEG)
OPG_ADAPT_BIN(GreaterThanOp, OPFLOW_NODE_GT)
OPG_ADAPT_BIN(GreaterThanOrEqualOp, OPFLOW_NODE_GE)
OPG_ADAPT_BIN(LessThanOp, OPFLOW_NODE_LT)
OPG_ADAPT_BIN(LessThanOrEqualOp, OPFLOW_NODE_LE)
OPG_ADAPT_BIN(NotEqualToOp, OPFLOW_NODE_NE)
#undef OPG_ADAPT_BIN
#define OPG_ADAPT_DIM(OpT, K)                  \
    template <std::size_t d>                   \
    struct op_kind<OpFlow::OpT<d>> {           \
        static constexpr int kind = K;         \
        static constexpr int dim = (int) d;    \
    };
OPG_ADAPT_DIM(D2SecondOrderCentered, OPFLOW_NODE_D2)
OPG_ADAPT_DIM(D1FirstOrderCentered, OPFLOW_NODE_D1)
OPG_ADAPT_DIM(D1FirstOrderBiasedUpwind, OPFLOW_NODE_D1_BIASED_UP)
OPG_ADAPT_DIM(D1FirstOrderBiasedDownwind, OPFLOW_NODE_D1_BIASED_DOWN)
OPG_ADAPT_DIM(D1WENO53Downwind, OPFLOW_NODE_WENO53_DOWN)
OPG_ADAPT_DIM(D1WENO53Upwind, OPFLOW_NODE_WENO53_UP)
#undef OPG_ADAPT_DIM
template <std::size_t d>
struct op_kind<OpFlow::D1Linear<d, OpFlow::IntpDirection::Cen2Cor>> {
    static constexpr int kind = OPFLOW_NODE_INTP_C2C;
    static constexpr int dim = (int) d;
};
template <std::size_t d>
struct op_kind<OpFlow::D1Linear<d, OpFlow::IntpDirection::Cor2Cen>> {
    static constexpr int kind = OPFLOW_NODE_INTP_COR2CEN;
    static constexpr int dim = (int) d;
};

template <typename>
inline constexpr bool always_false = false;

struct Lowering {
    std::vector<opflow_node> nodes;
    std::vector<const void*> leaf_keys;
    std::vector<opflow_field> leaves;

    int add(int kind, int a, int b, int dim, int field, double value) {
        opflow_node n{};
        n.kind = kind;
        n.a = a;
        n.b = b;
        n.dim = dim;
        n.field = field;
        n.value = value;
        n.c = -1;
        nodes.push_back(n);
        return (int) nodes.size() - 1;
    }
    template <typename F>
    int slot(const F& f) {
        for (size_t i = 0; i < leaf_keys.size(); ++i)
            if (leaf_keys[i] == (const void*) &f) return (int) i;
        leaf_keys.push_back(&f);
        leaves.push_back(mirror(f).f);
        return (int) leaves.size() - 1;
    }

    template <typename E>
    int lower(const E& e) {
        using T = std::remove_cvref_t<E>;
        if constexpr (std::is_arithmetic_v<T>) {
            return add(OPFLOW_NODE_CONST, -1, -1, 0, 0, (double) e);
        } else if constexpr (is_inst<T, OpFlow::ScalarExpr>::value) {
            return add(OPFLOW_NODE_CONST, -1, -1, 0, 0, (double) e.get());
        } else if constexpr (is_cfield<T>::value) {
            return add(OPFLOW_NODE_FIELD, -1, -1, 0, slot(e), 0.);
        } else if constexpr (is_inst<T, OpFlow::Expression>::value) {
            return lower_expr(e);
        } else {
            static_assert(always_false<T>, "this expression leaf has no GPU form (CartesianField, ScalarExpr and numbers do)");
            return -1;
        }
    }

    template <typename Op, typename... A>
    int lower_expr(const OpFlow::Expression<Op, A...>& e) {
        constexpr int K = op_kind<Op>::kind;
        static_assert(K != 0, "this operator has no GPU form in the engine");
        if constexpr (sizeof...(A) == 1) {
            if constexpr (std::is_same_v<Op, OpFlow::PosOp>) return lower(e.arg1);
            const int a = lower(e.arg1);
            return add(K, a, -1, op_kind<Op>::dim, 0, 0.);
        } else if constexpr (sizeof...(A) == 2) {
            const int a = lower(e.arg1);
            const int b = lower(e.arg2);
            return add(K, a, b, op_kind<Op>::dim, 0, 0.);
        } else {
            static_assert(always_false<Op>, "operators of three or more operands have no GPU form in the adapter");
            return -1;
        }
    }
};
template <>
struct op_kind<OpFlow::PosOp> {
    static constexpr int kind = -1;
    static constexpr int dim = 0;
};

template <OpFlow::BasicArithOp Op>
constexpr int arith_code() {
    if constexpr (Op == OpFlow::BasicArithOp::Eq) return OPFLOW_ASSIGN_EQ;
    else if constexpr (Op == OpFlow::BasicArithOp::Add) return OPFLOW_ASSIGN_ADD;
    else if constexpr (Op == OpFlow::BasicArithOp::Minus) return OPFLOW_ASSIGN_SUB;
    else if constexpr (Op == OpFlow::BasicArithOp::Mul) return OPFLOW_ASSIGN_MUL;
    else if constexpr (Op == OpFlow::BasicArithOp::Div) return OPFLOW_ASSIGN_DIV;
    else return -1;
}

template <typename F>
void upload(const F& f) {
    Mirror& m = mirror(f);
    check(opflow_field_upload(m.f, host_data(f, m.info), m.info.count), "opflow_field_upload");
}

template <OpFlow::BasicArithOp Op, typename S, typename D>
D& assign(const S& src, D& dst) {
    using DT = std::remove_cvref_t<D>;
    static_assert(is_cfield<DT>::value, "the GPU engine assigns CartesianFields (AMR fields are not on its path)");
    static_assert(arith_code<Op>() >= 0, "the GPU engine takes =, +=, -=, *= and /=");
    Lowering L;
    L.lower(src);
    Mirror& md = mirror(dst);
    // every field the expression reads, and the destination, from the host (host code may have written
    // any of them since the last assignment)
    std::vector<const void*> done;
    auto up = [&](const void* key, const Mirror& m, double* host) {
        for (auto* k : done)
            if (k == key) return;
        done.push_back(key);
        check(opflow_field_upload(m.f, host, m.info.count), "opflow_field_upload");
    };
    for (size_t i = 0; i < L.leaf_keys.size(); ++i) {
        const Mirror& m = registry().at(L.leaf_keys[i]);
        up(L.leaf_keys[i], m, const_cast<double*>(static_cast<const double*>(m.data0)));
    }
    up(&dst, md, host_data(dst, md.info));
    check(opflow_assign(context(), md.f, arith_code<Op>(), L.nodes.data(), (int) L.nodes.size(), L.leaves.data(), (int) L.leaves.size(),
                        eval_mode()),
          "opflow_assign");
    check(opflow_field_download(md.f, host_data(dst, md.info), md.info.count), "opflow_field_download");
    return dst;
}

// ---- the implicit path: makeEqnSolveHandler / Solve over the engine's solver ----------------------
// makeEqnSolveHandler(getter, target, solver) (HYPREEqnSolveHandler.hpp:44-48) with a Struct solver
// (StructSolver<T> or PrecondStructSolver<T, P>) and a CartesianField target returns this handler
// instead of OpFlow's HYPREEqnSolveHandler: the overload below has the reference's signature and a
// constraint, so overload resolution prefers it.  The getter is called with the target itself; the
// equation's lhs - rhs is lowered like an assignment's expression, with the target as the unknown,
// and opflow_solver_create assembles it with StencilPad semantics (the reference's generateAb).
// solve() uploads the fields the equation reads and the target (initial guess), solves on the device
// (re-assembling only b under staticMat) and downloads the solution (HYPREEqnSolveHandler::solve,
// returnValues).  The solver parameters map onto the engine's: tol, maxIter, staticMat, pinValue,
// absTol, kDim; the outer iteration (PCG, GMRES, FGMRES, LGMRES, BiCGSTAB, or the preconditioner
// alone) and the preconditioner (PFMG / SMG / CycRed: the engine's multigrid V-cycle; Jacobi; none).
template <typename S>
struct struct_solver : std::false_type {};
template <OpFlow::StructSolverType T>
struct struct_solver<OpFlow::StructSolver<T>> : std::true_type {
    static constexpr OpFlow::StructSolverType outer = T, pre = OpFlow::StructSolverType::None;
};
template <OpFlow::StructSolverType T, OpFlow::StructSolverType P>
struct struct_solver<OpFlow::PrecondStructSolver<T, P>> : std::true_type {
    static constexpr OpFlow::StructSolverType outer = T, pre = P;
};

inline int krylov_code(OpFlow::StructSolverType t) {
    using ST = OpFlow::StructSolverType;
    switch (t) {
        case ST::PCG: return OPFLOW_KRYLOV_PCG;
        case ST::GMRES: return OPFLOW_KRYLOV_GMRES;
        case ST::FGMRES: return OPFLOW_KRYLOV_FGMRES;
        case ST::LGMRES: return OPFLOW_KRYLOV_LGMRES;
        case ST::BICGSTAB: return OPFLOW_KRYLOV_BICGSTAB;
        default: return OPFLOW_KRYLOV_NONE;  // a preconditioner used as the solver
    }
}
inline int precond_code(OpFlow::StructSolverType t) {
    using ST = OpFlow::StructSolverType;
    switch (t) {
        case ST::PFMG: case ST::SMG: case ST::CYCRED: return OPFLOW_PRECOND_MG;
        case ST::Jacobi: return OPFLOW_PRECOND_JACOBI;
        default: return OPFLOW_PRECOND_NONE;
    }
}

template <typename Getter, typename T, typename S>
struct GpuEqnSolveHandler : virtual public OpFlow::EqnSolveHandler {
    GpuEqnSolveHandler(const Getter& g, T& target, const S& s) : getter(g), target(&target), solver(s) { this->init(); }
    ~GpuEqnSolveHandler() override {
        if (h) opflow_solver_destroy(h);
    }
    void init() override {
        auto eqn = getter(*target);
        const int l = L.lower(eqn.lhs);
        const int r = L.lower(eqn.rhs);
        L.add(OPFLOW_NODE_SUB, l, r, 0, 0, 0.);
        unknown = L.slot(*target);
        opflow_solve_params_default(&p);
        using K = struct_solver<S>;
        const auto& sp = solver.params;
        if (sp.tol) p.tol = sp.tol.value();
        if (sp.maxIter) p.max_iter = sp.maxIter.value();
        p.static_mat = sp.staticMat ? 1 : 0;
        p.pin_value = sp.pinValue ? 1 : 0;
        if constexpr (requires { sp.absTol; })
            if (sp.absTol) p.abs_tol = sp.absTol.value();
        if constexpr (requires { sp.kDim; })
            if (sp.kDim) p.kdim = sp.kDim.value();
        if constexpr (K::pre == OpFlow::StructSolverType::None) {
            // a solver alone: a preconditioner type iterates itself, a Krylov method runs unpreconditioned
            const int kc = krylov_code(K::outer);
            p.krylov = kc;
            p.precond = kc == OPFLOW_KRYLOV_NONE ? precond_code(K::outer) : OPFLOW_PRECOND_NONE;
        } else {
            p.krylov = krylov_code(K::outer);
            p.precond = precond_code(K::pre);
        }
        if (const char* e = std::getenv("OPFLOW_GB300_PRECISION")) p.precision = std::strcmp(e, "mixed") == 0 ? OPFLOW_PREC_MIXED : p.precision;
    }
    OpFlow::EqnSolveState solve() override {
        for (size_t i = 0; i < L.leaf_keys.size(); ++i) {
            const Mirror& m = registry().at(L.leaf_keys[i]);
            check(opflow_field_upload(m.f, const_cast<double*>(static_cast<const double*>(m.data0)), m.info.count), "opflow_field_upload");
        }
        if (!h) check(opflow_solver_create(context(), L.leaves[unknown], L.nodes.data(), (int) L.nodes.size(), L.leaves.data(),
                                           (int) L.leaves.size(), unknown, &p, &h),
                      "opflow_solver_create");
        opflow_solve_state st{};
        const int rc = opflow_solver_solve(h, &st);
        if (rc != 0 && rc != OPFLOW_E_NOT_CONVERGED) die("opflow_solver_solve");
        const Mirror& mt = registry().at(L.leaf_keys[unknown]);
        check(opflow_field_download(mt.f, host_data(*target, mt.info), mt.info.count), "opflow_field_download");
        return OpFlow::EqnSolveState(st.iterations, st.rel_residual, st.abs_residual);
    }
    void generateAb() override {}

private:
    Getter getter;
    T* target;
    S solver;
    Lowering L;
    int unknown = 0;
    opflow_solve_params p{};
    opflow_solver h = nullptr;
};

template <typename T, typename S>
concept GpuSolvable = is_cfield<std::remove_cvref_t<T>>::value && struct_solver<std::remove_cvref_t<S>>::value;

}  // namespace opflow_gb300::adapter

namespace OpFlow {
template <typename F, typename T, typename S>
    requires opflow_gb300::adapter::GpuSolvable<T, S>
std::unique_ptr<EqnSolveHandler> makeEqnSolveHandler(F&& f, T&& t, S&& s) {
    return std::make_unique<opflow_gb300::adapter::GpuEqnSolveHandler<std::remove_cvref_t<F>, std::remove_cvref_t<T>, std::remove_cvref_t<S>>>(
            f, t, s);
}

// Solve (UnifiedSolve.hpp:36-43, left out with the AMGCL back end it includes): one handler, one solve.
template <StructSolverType type = StructSolverType::GMRES, StructSolverType pType = StructSolverType::None, typename F,
          StructuredFieldExprType T>
auto Solve(const F& func, T&& target, StructSolverParams<type> params = StructSolverParams<type> {},
           StructSolverParams<pType> precParams = StructSolverParams<pType> {}) {
    auto solver = PrecondStructSolver<type, pType>(params, precParams);
    auto handler = makeEqnSolveHandler(func, target, solver);
    return handler->solve();
}
}  // namespace OpFlow


// ---- Utils::H5Stream stand-in (OpFlow's HDF5 writer needs libhdf5) -----------------------------------
namespace OpFlow::Utils {
// The calls FTCS-style programs make on H5Stream (fixedMesh, << TimeStamp, << field, close), writing
// each field through RawBinaryOStream into the directory of the given path.
struct H5Stream {
    H5Stream() = default;
    explicit H5Stream(const std::string& path) : os(path) {}
    H5Stream& fixedMesh() { return *this; }
    H5Stream& operator<<(const TimeStamp& t) {
        os << t;
        return *this;
    }
    template <typename F>
    H5Stream& operator<<(const F& f) {
        os << f;
        return *this;
    }
    void close() {}

private:
    RawBinaryOStream os;
};
}  // namespace OpFlow::Utils
