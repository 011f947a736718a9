// OpFlowGPU.hpp -- C++ front end of the GB300 engine with the names of OpFlow's user API.
//
// User code written against OpFlow's CartesianMesh / CartesianField / expression / EqnSolveHandler API
// (src/Core/Mesh/Structured/CartesianMesh.hpp, src/Core/Field/MeshBased/Structured/CartesianField.hpp,
// src/Core/Operator/FDMOperators/DiffsInterface.hpp, src/Core/Equation/HYPREEqnSolveHandler.hpp,
// src/Core/Solvers/Struct/UnifiedSolve.hpp) recompiles against this header: meshes, fields, the
// expression operators, assignment and Solve / makeEqnSolveHandler keep their spelling, and every
// assignment or solve runs on the GPU through the C ABI in opflow_gpu.h (link -lopflow_gpu).
//
// What differs from the reference, by design:
//   - Expressions are runtime trees (one node per operator) rather than compile-time expression
//     templates; they are lowered to device kernels when assigned.
//   - Field data lives in device memory.  Host reads (evalAt, operator[], data()) download a host
//     mirror on demand; host writes go through initBy / setData / operator[] + upload().
//   - The implicit solve runs the requested PrecondStructSolver<Solver, Precond> pair on the GPU:
//     PCG, GMRES / FlexGMRES / LGMRES (restarted flexible GMRES with kDim), BICGSTAB, or the
//     preconditioner alone, with the engine's geometric-multigrid V-cycle standing in for PFMG, SMG and
//     CycRed, or Jacobi, or none.  tol, absTol, maxIter, kDim, staticMat and pinValue keep their
//     meaning; `gpuMixedPrecision` selects the FP32 V-cycle inside the FP64 outer iteration.
//   - Failures print the engine's message and exit(1), the reference's OP_ABORT behaviour
//     (src/Core/Macros.hpp:146-151); set OpFlow::GPU::throwOnError(true) to get exceptions instead.
#ifndef OPFLOW_GB300_OPFLOWGPU_HPP
#define OPFLOW_GB300_OPFLOWGPU_HPP

#include "../opflow_gpu.h"

#include <array>
#include <cstdio>
#include <cstdlib>
#include <functional>
#include <memory>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <unordered_map>
#include <utility>
#include <vector>

namespace OpFlow {

using Real = double;

namespace Meta {
    template <int N>
    struct int_ {
        static constexpr int value = N;
    };
}// namespace Meta

enum class LocOnMesh { Corner = OPFLOW_CORNER, Center = OPFLOW_CENTER };
enum class BCType {
    Undefined = OPFLOW_BC_UNDEFINED,
    Dirc = OPFLOW_BC_DIRC,
    Neum = OPFLOW_BC_NEUM,
    Periodic = OPFLOW_BC_PERIODIC,
    Symm = OPFLOW_BC_SYMM,
    ASymm = OPFLOW_BC_ASYMM
};
enum class DimPos { start = 0, end = 1 };

namespace DS {
    template <int d>
    struct MDIndex {
        std::array<int, d> idx {};
        MDIndex() = default;
        MDIndex(std::initializer_list<int> l) {
            int k = 0;
            for (int v : l)
                if (k < d) idx[k++] = v;
        }
        int& operator[](int k) { return idx[k]; }
        int operator[](int k) const { return idx[k]; }
    };
    template <int d>
    struct Range {
        std::array<int, d> start {}, end {};
        long long count() const {
            long long n = 1;
            for (int k = 0; k < d; ++k) n *= end[k] > start[k] ? end[k] - start[k] : 0;
            return n;
        }
    };
}// namespace DS

// ------------------------------------------------------------------------------------- engine glue
namespace GPU {
    inline bool& throwOnError(bool set = false, bool value = false) {
        static bool t = false;
        if (set) t = value;
        return t;
    }
    inline void throwOnError(bool v) { throwOnError(true, v); }

    inline void check(int rc, const char* what) {
        if (rc == OPFLOW_OK) return;
        std::string msg = std::string("OpFlow GPU: ") + what + ": " + opflow_last_error();
        if (throwOnError()) throw std::runtime_error(msg);
        std::fprintf(stderr, "%s\n", msg.c_str());
        std::exit(1);
    }

    // The process-wide engine context on device 0 (the reference's global environment).
    inline opflow_ctx& contextSlot() {
        static opflow_ctx c = nullptr;
        return c;
    }
    inline opflow_ctx context() {
        opflow_ctx& c = contextSlot();
        if (!c) check(opflow_ctx_create(0, &c), "opflow_ctx_create");
        return c;
    }

    // Arithmetic of explicit assignments: EXACT (bit-identical to the reference) or FAST (fixed point,
    // normwise relative error <= 1e-14; linear constant-coefficient stencils only).
    inline int& evalMode() {
        static int m = OPFLOW_EVAL_EXACT;
        return m;
    }
    inline void setEvalMode(int m) { evalMode() = m; }

    struct FieldHandle {
        opflow_field f = nullptr;
        opflow_field_info info {};
        std::vector<double> host;  // host mirror
        bool host_valid = false;   // mirror equals device data
        ~FieldHandle() {
            if (f) opflow_field_destroy(f);
        }
    };

    struct Node;
    using NodeP = std::shared_ptr<const Node>;
    struct Node {
        int kind = 0;
        NodeP a, b, c;  // c: the false branch of a conditional
        int dim = 0;
        int param = 0;  // function or flux limiter id
        double value = 0.;
        std::shared_ptr<FieldHandle> field;  // leaves
    };

    // Postfix node list (children first, root last) and the leaf fields in slot order.
    struct Program {
        std::vector<opflow_node> nodes;
        std::vector<std::shared_ptr<FieldHandle>> leaves;
        int slotOf(const std::shared_ptr<FieldHandle>& h) {
            for (std::size_t i = 0; i < leaves.size(); ++i)
                if (leaves[i].get() == h.get()) return (int) i;
            leaves.push_back(h);
            return (int) leaves.size() - 1;
        }
        int add(const NodeP& n, std::unordered_map<const Node*, int>& memo) {
            auto it = memo.find(n.get());
            if (it != memo.end()) return it->second;
            opflow_node o {};
            o.kind = n->kind;
            o.a = n->a ? add(n->a, memo) : -1;
            o.b = n->b ? add(n->b, memo) : -1;
            o.c = n->c ? add(n->c, memo) : -1;
            o.dim = n->dim;
            o.value = n->value;
            o.field = n->kind == OPFLOW_NODE_FIELD ? slotOf(n->field) : n->param;
            nodes.push_back(o);
            return memo[n.get()] = (int) nodes.size() - 1;
        }
        static Program of(const NodeP& root, const std::shared_ptr<FieldHandle>& first_leaf = nullptr) {
            Program p;
            if (first_leaf) p.slotOf(first_leaf);
            std::unordered_map<const Node*, int> memo;
            p.add(root, memo);
            return p;
        }
        std::vector<opflow_field> handles() const {
            std::vector<opflow_field> h;
            for (auto& l : leaves) h.push_back(l->f);
            return h;
        }
    };
}// namespace GPU

// ------------------------------------------------------------------------------------------ mesh
template <typename Dim>
struct CartesianMesh {
    static constexpr int dim = Dim::value;
    std::array<int, dim> dims {}, start {};
    int padWidth = 5;
    std::array<std::vector<Real>, dim> xs, dxs;

    int getDimOf(int d) const { return dims[d]; }
    Real x(int d, int i) const { return xs[d][i - start[d] + padWidth]; }
    Real dx(int d, int i) const { return dxs[d][i - start[d] + padWidth]; }
    opflow_mesh_desc desc() const {
        opflow_mesh_desc m {};
        m.ndim = dim;
        for (int d = 0; d < dim; ++d) {
            m.dims[d] = dims[d];
            m.start[d] = start[d];
            m.x[d] = xs[d].data();
            m.dx[d] = dxs[d].data();
        }
        m.pad_width = padWidth;
        return m;
    }
};

template <typename M>
struct MeshBuilder;

template <typename Dim>
struct MeshBuilder<CartesianMesh<Dim>> {
    static constexpr int dim = Dim::value;
    CartesianMesh<Dim> m;
    std::array<Real, dim> lo {}, hi {};

    template <typename... I>
    MeshBuilder& newMesh(I... n) {
        static_assert(sizeof...(I) == dim, "newMesh takes one extent per dimension");
        int k = 0;
        ((m.dims[k++] = (int) n), ...);
        for (int d = 0; d < dim; ++d) hi[d] = (Real) (m.dims[d] - 1);
        return *this;
    }
    MeshBuilder& setMeshOfDim(int k, Real min, Real max) {
        lo[k] = min;
        hi[k] = max;
        return *this;
    }
    MeshBuilder& setPadWidth(int w) {
        m.padWidth = w;
        return *this;
    }
    MeshBuilder& setStart(const std::array<int, dim>& s) {
        m.start = s;
        return *this;
    }
    CartesianMesh<Dim> build() {
        for (int d = 0; d < dim; ++d) {
            m.xs[d].assign(m.dims[d] + 2 * m.padWidth, 0.);
            m.dxs[d].assign(m.dims[d] + 2 * m.padWidth - 1, 0.);
            GPU::check(opflow_mesh_uniform(m.dims[d], m.start[d], m.padWidth, lo[d], hi[d], m.xs[d].data(), m.dxs[d].data()),
                       "MeshBuilder::build");
        }
        return m;
    }
};

// ------------------------------------------------------------------------------------ expressions
class Expr {
public:
    GPU::NodeP node;
    Expr() = default;
    explicit Expr(GPU::NodeP n) : node(std::move(n)) {}
    Expr(Real v) {
        auto n = std::make_shared<GPU::Node>();
        n->kind = OPFLOW_NODE_CONST;
        n->value = v;
        node = n;
    }
};

template <typename Real_, typename Mesh>
class CartesianField;

template <typename T>
struct is_field : std::false_type {};
template <typename R, typename M>
struct is_field<CartesianField<R, M>> : std::true_type {};

template <typename T>
constexpr bool is_operand_v = std::is_same_v<std::decay_t<T>, Expr> || is_field<std::decay_t<T>>::value || std::is_arithmetic_v<std::decay_t<T>>;
template <typename A, typename B>
constexpr bool is_binary_v = is_operand_v<A> && is_operand_v<B> && !(std::is_arithmetic_v<std::decay_t<A>> && std::is_arithmetic_v<std::decay_t<B>>);

inline Expr toExpr(const Expr& e) { return e; }
template <typename T, std::enable_if_t<std::is_arithmetic_v<T>, int> = 0>
inline Expr toExpr(T v) {
    return Expr((Real) v);
}
template <typename R, typename M>
inline Expr toExpr(const CartesianField<R, M>& f) {
    return f.asExpr();
}

namespace GPU {
    inline Expr makeNode(int kind, const Expr& a, const Expr* b = nullptr, int dim = 0, int param = 0, const Expr* c = nullptr) {
        auto n = std::make_shared<Node>();
        n->kind = kind;
        n->a = a.node;
        if (b) n->b = b->node;
        if (c) n->c = c->node;
        n->dim = dim;
        n->param = param;
        return Expr(n);
    }
}// namespace GPU

template <typename A, typename B, std::enable_if_t<is_binary_v<A, B>, int> = 0>
Expr operator+(const A& a, const B& b) {
    Expr y = toExpr(b);
    return GPU::makeNode(OPFLOW_NODE_ADD, toExpr(a), &y);
}
template <typename A, typename B, std::enable_if_t<is_binary_v<A, B>, int> = 0>
Expr operator-(const A& a, const B& b) {
    Expr y = toExpr(b);
    return GPU::makeNode(OPFLOW_NODE_SUB, toExpr(a), &y);
}
template <typename A, typename B, std::enable_if_t<is_binary_v<A, B>, int> = 0>
Expr operator*(const A& a, const B& b) {
    Expr y = toExpr(b);
    return GPU::makeNode(OPFLOW_NODE_MUL, toExpr(a), &y);
}
template <typename A, typename B, std::enable_if_t<is_binary_v<A, B>, int> = 0>
Expr operator/(const A& a, const B& b) {
    Expr y = toExpr(b);
    return GPU::makeNode(OPFLOW_NODE_DIV, toExpr(a), &y);
}
template <typename A, std::enable_if_t<is_operand_v<A> && !std::is_arithmetic_v<A>, int> = 0>
Expr operator-(const A& a) {
    return GPU::makeNode(OPFLOW_NODE_NEG, toExpr(a));
}

// comparisons and logic (src/Core/Operator/Logical/Compare.hpp, Boolean.hpp): 1.0 / 0.0 valued
#define OPFLOW_GPU_BINOP(op, kind)                                                                           \
    template <typename A, typename B, std::enable_if_t<is_binary_v<A, B>, int> = 0>                           \
    Expr operator op(const A& a, const B& b) {                                                                \
        Expr y = toExpr(b);                                                                                  \
        return GPU::makeNode(kind, toExpr(a), &y);                                                           \
    }
OPFLOW_GPU_BINOP(>, OPFLOW_NODE_GT)
OPFLOW_GPU_BINOP(>=, OPFLOW_NODE_GE)
OPFLOW_GPU_BINOP(<, OPFLOW_NODE_LT)
OPFLOW_GPU_BINOP(<=, OPFLOW_NODE_LE)
OPFLOW_GPU_BINOP(!=, OPFLOW_NODE_NE)
OPFLOW_GPU_BINOP(&&, OPFLOW_NODE_AND)
OPFLOW_GPU_BINOP(||, OPFLOW_NODE_OR)
#undef OPFLOW_GPU_BINOP
template <typename A, std::enable_if_t<is_operand_v<A> && !std::is_arithmetic_v<A>, int> = 0>
Expr operator!(const A& a) {
    return GPU::makeNode(OPFLOW_NODE_NOT, toExpr(a));
}

// conditional(c, a, b) = c ? a : b (src/Core/Operator/Conditional.hpp)
template <typename C, typename A, typename B>
Expr conditional(const C& c, const A& a, const B& b) {
    Expr ya = toExpr(a), yb = toExpr(b);
    return GPU::makeNode(OPFLOW_NODE_COND, toExpr(c), &ya, 0, 0, &yb);
}

// per-element functions (src/Core/Operator/Arithmetic/AMDS.hpp, MinMax.hpp)
#define OPFLOW_GPU_FUNC1(name, id)                                                                           \
    template <typename A, std::enable_if_t<is_operand_v<A> && !std::is_arithmetic_v<A>, int> = 0>             \
    Expr name(const A& a) {                                                                                  \
        return GPU::makeNode(OPFLOW_NODE_FUNC1, toExpr(a), nullptr, 0, id);                                  \
    }
OPFLOW_GPU_FUNC1(abs, OPFLOW_F_ABS)
OPFLOW_GPU_FUNC1(sqrt, OPFLOW_F_SQRT)
OPFLOW_GPU_FUNC1(ceil, OPFLOW_F_CEIL)
OPFLOW_GPU_FUNC1(floor, OPFLOW_F_FLOOR)
OPFLOW_GPU_FUNC1(trunc, OPFLOW_F_TRUNC)
OPFLOW_GPU_FUNC1(round, OPFLOW_F_ROUND)
OPFLOW_GPU_FUNC1(rint, OPFLOW_F_RINT)
OPFLOW_GPU_FUNC1(exp, OPFLOW_F_EXP)
OPFLOW_GPU_FUNC1(exp2, OPFLOW_F_EXP2)
OPFLOW_GPU_FUNC1(expm1, OPFLOW_F_EXPM1)
OPFLOW_GPU_FUNC1(log, OPFLOW_F_LOG)
OPFLOW_GPU_FUNC1(log10, OPFLOW_F_LOG10)
OPFLOW_GPU_FUNC1(log2, OPFLOW_F_LOG2)
OPFLOW_GPU_FUNC1(log1p, OPFLOW_F_LOG1P)
OPFLOW_GPU_FUNC1(cbrt, OPFLOW_F_CBRT)
OPFLOW_GPU_FUNC1(sin, OPFLOW_F_SIN)
OPFLOW_GPU_FUNC1(cos, OPFLOW_F_COS)
OPFLOW_GPU_FUNC1(tan, OPFLOW_F_TAN)
OPFLOW_GPU_FUNC1(asin, OPFLOW_F_ASIN)
OPFLOW_GPU_FUNC1(acos, OPFLOW_F_ACOS)
OPFLOW_GPU_FUNC1(atan, OPFLOW_F_ATAN)
OPFLOW_GPU_FUNC1(sinh, OPFLOW_F_SINH)
OPFLOW_GPU_FUNC1(cosh, OPFLOW_F_COSH)
OPFLOW_GPU_FUNC1(tanh, OPFLOW_F_TANH)
OPFLOW_GPU_FUNC1(asinh, OPFLOW_F_ASINH)
OPFLOW_GPU_FUNC1(acosh, OPFLOW_F_ACOSH)
OPFLOW_GPU_FUNC1(atanh, OPFLOW_F_ATANH)
OPFLOW_GPU_FUNC1(erf, OPFLOW_F_ERF)
OPFLOW_GPU_FUNC1(erfc, OPFLOW_F_ERFC)
OPFLOW_GPU_FUNC1(tgamma, OPFLOW_F_TGAMMA)
OPFLOW_GPU_FUNC1(lgamma, OPFLOW_F_LGAMMA)
#undef OPFLOW_GPU_FUNC1
#define OPFLOW_GPU_FUNC2(name, id)                                                                           \
    template <typename A, typename B, std::enable_if_t<is_binary_v<A, B>, int> = 0>                           \
    Expr name(const A& a, const B& b) {                                                                      \
        Expr y = toExpr(b);                                                                                  \
        return GPU::makeNode(OPFLOW_NODE_FUNC2, toExpr(a), &y, 0, id);                                       \
    }
OPFLOW_GPU_FUNC2(max, OPFLOW_F2_MAX)
OPFLOW_GPU_FUNC2(min, OPFLOW_F2_MIN)
OPFLOW_GPU_FUNC2(fdim, OPFLOW_F2_FDIM)
OPFLOW_GPU_FUNC2(copysign, OPFLOW_F2_COPYSIGN)
OPFLOW_GPU_FUNC2(fmod, OPFLOW_F2_FMOD)
OPFLOW_GPU_FUNC2(remainder, OPFLOW_F2_REMAINDER)
OPFLOW_GPU_FUNC2(pow, OPFLOW_F2_POW)
OPFLOW_GPU_FUNC2(hypot, OPFLOW_F2_HYPOT)
OPFLOW_GPU_FUNC2(atan2, OPFLOW_F2_ATAN2)
#undef OPFLOW_GPU_FUNC2

// `lhs == rhs` (src/Core/Equation/Equation.hpp:41-55); the solver works on lhs - rhs.
struct Equation {
    Expr lhs, rhs;
    Expr residual() const { return lhs - rhs; }
};
template <typename A, typename B, std::enable_if_t<is_binary_v<A, B>, int> = 0>
Equation operator==(const A& a, const B& b) {
    return Equation {toExpr(a), toExpr(b)};
}

// Operator kernels: tags with the reference's names (the arithmetic lives in the engine).
template <std::size_t d>
struct D2SecondOrderCentered {
    static constexpr int kind = OPFLOW_NODE_D2, dim = (int) d;
};
template <std::size_t d>
struct D1FirstOrderCentered {
    static constexpr int kind = OPFLOW_NODE_D1, dim = (int) d;
};
template <std::size_t d>
struct D1WENO53Downwind {
    static constexpr int kind = OPFLOW_NODE_WENO53_DOWN, dim = (int) d;
};
template <std::size_t d>
struct D1WENO53Upwind {
    static constexpr int kind = OPFLOW_NODE_WENO53_UP, dim = (int) d;
};
template <std::size_t d>
struct D1FirstOrderBiasedUpwind {
    static constexpr int kind = OPFLOW_NODE_D1_BIASED_UP, dim = (int) d;
};
template <std::size_t d>
struct D1FirstOrderBiasedDownwind {
    static constexpr int kind = OPFLOW_NODE_D1_BIASED_DOWN, dim = (int) d;
};

// d1 / d2 / dx..dz / d2x..d2z as in src/Core/Operator/FDMOperators/DiffsInterface.hpp
template <typename Kernel, typename E>
Expr d1(const E& e) {
    return GPU::makeNode(Kernel::kind, toExpr(e), nullptr, Kernel::dim);
}
template <typename Kernel, typename E>
Expr d2(const E& e) {
    return GPU::makeNode(Kernel::kind, toExpr(e), nullptr, Kernel::dim);
}
#define OPFLOW_GPU_AXIS_OP(name, base, d)                                                                   \
    template <template <std::size_t> typename Kernel, typename E>                                            \
    Expr name(const E& e) {                                                                                  \
        return base<Kernel<d>>(e);                                                                           \
    }
OPFLOW_GPU_AXIS_OP(dx, d1, 0)
OPFLOW_GPU_AXIS_OP(dy, d1, 1)
OPFLOW_GPU_AXIS_OP(dz, d1, 2)
OPFLOW_GPU_AXIS_OP(d2x, d2, 0)
OPFLOW_GPU_AXIS_OP(d2y, d2, 1)
OPFLOW_GPU_AXIS_OP(d2z, d2, 2)
#undef OPFLOW_GPU_AXIS_OP

// d1IntpCenterToCorner<dim> with the default D1Linear kernel (src/Core/Operator/Interpolator/IntpInterface.hpp:26-29)
template <std::size_t dim, typename E>
Expr d1IntpCenterToCorner(const E& e) {
    return GPU::makeNode(OPFLOW_NODE_INTP_C2C, toExpr(e), nullptr, (int) dim);
}
// d1IntpCornerToCenter<dim> with the default D1Linear kernel (IntpInterface.hpp:31-34)
template <std::size_t dim, typename E>
Expr d1IntpCornerToCenter(const E& e) {
    return GPU::makeNode(OPFLOW_NODE_INTP_COR2CEN, toExpr(e), nullptr, (int) dim);
}

// Flux-limiter interpolation (Interpolator/D1FluxLimiter.hpp, FluxLimiterKernels.hpp,
// D1FluxLimiterBasedIntpOp.hpp): d1Intp<d, IntpDirection::Cen2Cor, D1QUICK>(u, e) interpolates e to
// the faces along d, upwinded by the sign of u at the target point.
enum class IntpDirection { Cor2Cen, Cen2Cor };
enum class KappaScheme { CDS, QUICK, CUI, Fromm, LUI };
template <KappaScheme s>
struct KappaKernel {
    static constexpr int id = (int) s;  // OPFLOW_FL_CDS .. OPFLOW_FL_LUI
};
#define OPFLOW_GPU_LIMITER(name, id_)                                                                        \
    struct name {                                                                                            \
        static constexpr int id = id_;                                                                       \
    };
OPFLOW_GPU_LIMITER(MinmodKernel, OPFLOW_FL_MINMOD)
OPFLOW_GPU_LIMITER(SuperbeeKernel, OPFLOW_FL_SUPERBEE)
OPFLOW_GPU_LIMITER(MUSCLKernel, OPFLOW_FL_MUSCL)
OPFLOW_GPU_LIMITER(HarmonicKernel, OPFLOW_FL_HARMONIC)
OPFLOW_GPU_LIMITER(vanAlbadaKernel, OPFLOW_FL_VANALBADA)
OPFLOW_GPU_LIMITER(UMISTKernel, OPFLOW_FL_UMIST)
OPFLOW_GPU_LIMITER(SPL13Kernel, OPFLOW_FL_SPL13)
OPFLOW_GPU_LIMITER(SPLMax12Kernel, OPFLOW_FL_SPLMAX12)
OPFLOW_GPU_LIMITER(SPLMax13Kernel, OPFLOW_FL_SPLMAX13)
OPFLOW_GPU_LIMITER(KorenLimitedCUIKernel, OPFLOW_FL_KOREN)
OPFLOW_GPU_LIMITER(SMARTKernel, OPFLOW_FL_SMART)
OPFLOW_GPU_LIMITER(BSOUKernel, OPFLOW_FL_BSOU)
#undef OPFLOW_GPU_LIMITER
template <typename K>
struct D1FluxLimiterGen {
    template <std::size_t d, IntpDirection dir>
    struct Op {
        static constexpr int limiter = K::id;
    };
};
template <std::size_t d, IntpDirection dir> using D1Central = D1FluxLimiterGen<KappaKernel<KappaScheme::CDS>>::Op<d, dir>;
template <std::size_t d, IntpDirection dir> using D1QUICK = D1FluxLimiterGen<KappaKernel<KappaScheme::QUICK>>::Op<d, dir>;
template <std::size_t d, IntpDirection dir> using D1CUI = D1FluxLimiterGen<KappaKernel<KappaScheme::CUI>>::Op<d, dir>;
template <std::size_t d, IntpDirection dir> using D1Fromm = D1FluxLimiterGen<KappaKernel<KappaScheme::Fromm>>::Op<d, dir>;
template <std::size_t d, IntpDirection dir> using D1LinearUpwind = D1FluxLimiterGen<KappaKernel<KappaScheme::LUI>>::Op<d, dir>;
template <std::size_t d, IntpDirection dir> using D1Minmod = D1FluxLimiterGen<MinmodKernel>::Op<d, dir>;
template <std::size_t d, IntpDirection dir> using D1Superbee = D1FluxLimiterGen<SuperbeeKernel>::Op<d, dir>;
template <std::size_t d, IntpDirection dir> using D1MUSCL = D1FluxLimiterGen<MUSCLKernel>::Op<d, dir>;
template <std::size_t d, IntpDirection dir> using D1Harmonic = D1FluxLimiterGen<HarmonicKernel>::Op<d, dir>;
template <std::size_t d, IntpDirection dir> using D1Albada = D1FluxLimiterGen<vanAlbadaKernel>::Op<d, dir>;
// d1Intp<dim, dir, Kernel>(u, e) (IntpInterface.hpp:36-40) for the flux-limiter kernels
template <std::size_t d, IntpDirection dir, template <std::size_t, IntpDirection> typename Kernel, typename U, typename E>
Expr d1Intp(const U& u, const E& e) {
    Expr ye = toExpr(e);
    return GPU::makeNode(dir == IntpDirection::Cen2Cor ? OPFLOW_NODE_INTP_FL_CEN2COR : OPFLOW_NODE_INTP_FL_COR2CEN, toExpr(u), &ye,
                         (int) d, Kernel<d, dir>::limiter);
}
// d1IntpCenterToCorner<dim, Kernel>(u, e) / d1IntpCornerToCenter<dim, Kernel>(u, e) with a flux-limiter kernel
template <std::size_t d, template <std::size_t, IntpDirection> typename Kernel, typename U, typename E>
Expr d1IntpCenterToCorner(const U& u, const E& e) {
    return d1Intp<d, IntpDirection::Cen2Cor, Kernel>(u, e);
}
template <std::size_t d, template <std::size_t, IntpDirection> typename Kernel, typename U, typename E>
Expr d1IntpCornerToCenter(const U& u, const E& e) {
    return d1Intp<d, IntpDirection::Cor2Cen, Kernel>(u, e);
}

// ------------------------------------------------------------------------------------------ field
template <typename Real_, typename Mesh>
class CartesianField {
public:
    static constexpr int dim = Mesh::dim;
    using index_type = DS::MDIndex<dim>;
    std::string name;
    Mesh mesh;
    opflow_field_desc desc {};
    DS::Range<dim> logicalRange, accessibleRange, assignableRange, localRange;
    std::shared_ptr<GPU::FieldHandle> h;

    CartesianField() = default;
    CartesianField(const CartesianField& o) : name(o.name), mesh(o.mesh), desc(o.desc) {
        if (!o.h) return;  // a copy of a field that was never built is unbuilt too
        create();
        GPU::check(opflow_field_copy(h->f, o.h->f), "CartesianField copy");
    }
    CartesianField(CartesianField&&) noexcept = default;
    CartesianField& operator=(CartesianField&& o) noexcept = default;

    // the reference's value assignment between fields
    CartesianField& operator=(const CartesianField& o) {
        if (this == &o) return *this;
        if (!o.h) GPU::check(OPFLOW_E_INVALID, "assignment from a field that was never built");
        if (!h) {
            name = o.name;
            mesh = o.mesh;
            desc = o.desc;
            create();
        }
        GPU::check(opflow_field_copy(h->f, o.h->f), "CartesianField::operator=");
        h->host_valid = false;
        return *this;
    }
    CartesianField& operator=(const Expr& e) { return assign(e, OPFLOW_ASSIGN_EQ); }
    CartesianField& operator+=(const Expr& e) { return assign(e, OPFLOW_ASSIGN_ADD); }
    CartesianField& operator-=(const Expr& e) { return assign(e, OPFLOW_ASSIGN_SUB); }
    CartesianField& operator*=(const Expr& e) { return assign(e, OPFLOW_ASSIGN_MUL); }
    CartesianField& operator/=(const Expr& e) { return assign(e, OPFLOW_ASSIGN_DIV); }
    template <typename T, std::enable_if_t<std::is_arithmetic_v<T>, int> = 0>
    CartesianField& operator=(T c) {
        GPU::check(opflow_field_fill(h->f, OPFLOW_ASSIGN_EQ, (double) c), "CartesianField::operator=(scalar)");
        h->host_valid = false;
        return *this;
    }

    Expr asExpr() const {
        auto n = std::make_shared<GPU::Node>();
        n->kind = OPFLOW_NODE_FIELD;
        n->field = h;
        return Expr(n);
    }

    // ---- host access (downloads a mirror on demand)
    const std::vector<Real>& data() const {
        if (!h->host_valid) {
            h->host.resize(h->info.count);
            GPU::check(opflow_field_download(h->f, h->host.data(), h->host.size()), "CartesianField download");
            h->host_valid = true;
        }
        return h->host;
    }
    long long linear(const index_type& i) const {
        long long off = 0, stride = 1;
        for (int d = 0; d < dim; ++d) {
            off += (long long) (i[d] - h->info.data_offset[d]) * stride;
            stride *= h->info.data_dims[d];
        }
        return off;
    }
    Real evalAt(const index_type& i) const { return data()[linear(i)]; }
    Real operator[](const index_type& i) const { return evalAt(i); }
    // write a host array in the data layout, then refresh the padding
    void setData(const std::vector<Real>& v) {
        GPU::check(opflow_field_upload(h->f, v.data(), v.size()), "CartesianField upload");
        GPU::check(opflow_field_update_padding(h->f), "CartesianField updatePadding");
        h->host_valid = false;
    }
    // CartesianField::initBy (CartesianField.hpp:282-294): f(x) at every assignable point's coordinates
    template <typename F>
    void initBy(F&& f) {
        std::vector<Real> v = data();
        const DS::Range<dim>& r = assignableRange;
        if (r.count() > 0) {
            index_type i;
            for (int d = 0; d < dim; ++d) i[d] = r.start[d];
            for (;;) {
                std::array<Real, dim> X;
                for (int q = 0; q < dim; ++q)
                    X[q] = desc.loc[q] == OPFLOW_CENTER ? mesh.x(q, i[q]) + .5 * mesh.dx(q, i[q]) : mesh.x(q, i[q]);
                v[linear(i)] = f(X);
                int d = 0;
                while (d < dim && ++i[d] == r.end[d]) {
                    i[d] = r.start[d];
                    ++d;
                }
                if (d == dim) break;
            }
        }
        setData(v);
    }
    void updatePadding() {
        GPU::check(opflow_field_update_padding(h->f), "CartesianField::updatePadding");
        h->host_valid = false;
    }
    opflow_field handle() const { return h->f; }

    void create() {
        h = std::make_shared<GPU::FieldHandle>();
        opflow_mesh_desc md = mesh.desc();
        GPU::check(opflow_field_create(GPU::context(), &md, &desc, &h->f), "ExprBuilder::build");
        GPU::check(opflow_field_get_info(h->f, &h->info), "field info");
        auto cp = [&](DS::Range<dim>& r, const int (*src)[2]) {
            for (int d = 0; d < dim; ++d) {
                r.start[d] = src[d][0];
                r.end[d] = src[d][1];
            }
        };
        cp(logicalRange, h->info.logical);
        cp(accessibleRange, h->info.accessible);
        cp(assignableRange, h->info.assignable);
        cp(localRange, h->info.local);
    }

private:
    CartesianField& assign(const Expr& e, int arith) {
        GPU::Program p = GPU::Program::of(e.node);
        std::vector<opflow_field> leaves = p.handles();
        GPU::check(opflow_assign(GPU::context(), h->f, arith, p.nodes.data(), (int) p.nodes.size(), leaves.data(), (int) leaves.size(),
                                 GPU::evalMode()),
                   "CartesianField assignment");
        h->host_valid = false;
        return *this;
    }
};

template <typename F>
struct ExprBuilder;

template <typename R, typename Mesh>
struct ExprBuilder<CartesianField<R, Mesh>> {
    static constexpr int dim = Mesh::dim;
    using Field = CartesianField<R, Mesh>;
    // plain settings (copying a builder copies no device data); one builder makes several fields,
    // as OpFlow's does
    std::string name;
    Mesh mesh;
    opflow_field_desc desc {};
    bool ext_set = false;

    ExprBuilder() {
        desc.ndim = dim;
        for (int d = 0; d < dim; ++d) desc.loc[d] = OPFLOW_CORNER;
    }
    ExprBuilder& setName(const std::string& n) {
        name = n;
        return *this;
    }
    ExprBuilder& setMesh(const Mesh& m) {
        mesh = m;
        return *this;
    }
    ExprBuilder& setLoc(const std::array<LocOnMesh, dim>& loc) {
        for (int d = 0; d < dim; ++d) desc.loc[d] = (int) loc[d];
        return *this;
    }
    ExprBuilder& setLoc(LocOnMesh loc) {
        for (int d = 0; d < dim; ++d) desc.loc[d] = (int) loc;
        return *this;
    }
    ExprBuilder& setBC(int d, DimPos pos, BCType type, Real value = 0.) {
        desc.bc_type[d][(int) pos] = (int) type;
        desc.bc_value[d][(int) pos] = value;
        return *this;
    }
    ExprBuilder& setExt(int e) {
        for (int d = 0; d < dim; ++d) desc.ext[d][0] = desc.ext[d][1] = e;
        ext_set = true;
        return *this;
    }
    ExprBuilder& setExt(int d, DimPos pos, int e) {
        desc.ext[d][(int) pos] = e;
        ext_set = true;
        return *this;
    }
    ExprBuilder& setPadding(int p) {
        desc.padding = p;
        return *this;
    }
    Field build() const {
        Field out;
        out.name = name;
        out.mesh = mesh;
        out.desc = desc;
        out.create();
        return out;
    }
};

// ------------------------------------------------------------------------------------ implicit path
enum class StructSolverType { GMRES, FlexGMRES, LGMRES, BICGSTAB, PCG, PFMG, SMG, CYCRED, Jacobi, None };

// StructSolverParamsBase (src/Core/Solvers/Struct/StructSolver.hpp:39-51) with the PFMG knobs
// (StructSolverPFMG.hpp:23-33) and the engine's precision switch.
template <StructSolverType T>
struct StructSolverParams {
    Real tol = 1e-10;
    int maxIter = 100;
    bool staticMat = false;
    bool pinValue = false;
    bool useZeroGuess = false;
    std::string dumpPath;
    int printLevel = 0, logging = 0;
    int rapType = 0, relaxType = 1, numPreRelax = 1, numPostRelax = 1, skipRelax = 0;
    int kDim = 5;                    // GMRES restart length (StructSolverGMRES.hpp:20-23)
    Real absTol = 0.;
    bool gpuMixedPrecision = false;  // FP32 V-cycle inside the FP64 flexible outer iteration
};

template <StructSolverType Solver, StructSolverType Precond = StructSolverType::None>
struct PrecondStructSolver {
    StructSolverParams<Solver> params;
    StructSolverParams<Precond> p_params;
    PrecondStructSolver() = default;
    PrecondStructSolver(const StructSolverParams<Solver>& p, const StructSolverParams<Precond>& pp = {}) : params(p), p_params(pp) {}
};

template <StructSolverType T>
struct StructSolver {
    StructSolverParams<T> params;
    StructSolver() = default;
    explicit StructSolver(const StructSolverParams<T>& p) : params(p) {}
};

// EqnSolveState (src/Core/Equation/EqnSolveHandler.hpp:17-25)
struct EqnSolveState {
    int niter = 0;
    Real relerr = 0.;
    bool converged = false;
};

// EqnSolveHandler (EqnSolveHandler.hpp:28-33)
struct EqnSolveHandler {
    virtual ~EqnSolveHandler() = default;
    virtual void init() = 0;
    virtual EqnSolveState solve() = 0;
    virtual void generateAb() {}
};

namespace GPU {
    template <typename Target>
    struct Handler : EqnSolveHandler {
        Target* target;
        Program prog;
        opflow_solve_params prm {};
        opflow_solver s = nullptr;
        Handler(const Equation& eq, Target& t, const opflow_solve_params& p) : target(&t), prm(p) {
            prog = Program::of(eq.residual().node, t.h);  // the unknown is slot 0
            init();
        }
        ~Handler() override {
            if (s) opflow_solver_destroy(s);
        }
        void init() override {
            if (s) opflow_solver_destroy(s);
            s = nullptr;
            std::vector<opflow_field> leaves = prog.handles();
            check(opflow_solver_create(context(), target->h->f, prog.nodes.data(), (int) prog.nodes.size(), leaves.data(), (int) leaves.size(), 0,
                                       &prm, &s),
                  "makeEqnSolveHandler");
        }
        EqnSolveState solve() override {
            opflow_solve_state st {};
            const int rc = opflow_solver_solve(s, &st);
            if (rc != OPFLOW_E_NOT_CONVERGED) check(rc, "EqnSolveHandler::solve");
            target->h->host_valid = false;
            return EqnSolveState {st.iterations, st.rel_residual, st.converged != 0};
        }
    };

    template <StructSolverType T, StructSolverType P>
    opflow_solve_params toParams(const StructSolverParams<T>& p, const StructSolverParams<P>& pp) {
        opflow_solve_params o;
        opflow_solve_params_default(&o);
        o.tol = p.tol;
        o.max_iter = p.maxIter;
        o.static_mat = p.staticMat ? 1 : 0;
        o.pin_value = p.pinValue ? 1 : 0;
        o.zero_guess = p.useZeroGuess ? 1 : 0;
        o.precision = (p.gpuMixedPrecision || pp.gpuMixedPrecision) ? OPFLOW_PREC_MIXED : OPFLOW_PREC_FP64;
        o.kdim = p.kDim;
        o.abs_tol = p.absTol;
        // PrecondStructSolver<T, P>: T the outer iteration, P its preconditioner; a preconditioner type
        // as T without P (StructSolver<PFMG> etc.) iterates it alone
        auto pre = [](StructSolverType t) {
            switch (t) {
                case StructSolverType::PFMG: case StructSolverType::SMG: case StructSolverType::CYCRED: return (int) OPFLOW_PRECOND_MG;
                case StructSolverType::Jacobi: return (int) OPFLOW_PRECOND_JACOBI;
                default: return (int) OPFLOW_PRECOND_NONE;
            }
        };
        switch (T) {
            case StructSolverType::PCG: o.krylov = OPFLOW_KRYLOV_PCG; o.precond = pre(P); break;
            case StructSolverType::GMRES: o.krylov = OPFLOW_KRYLOV_GMRES; o.precond = pre(P); break;
            case StructSolverType::FlexGMRES: o.krylov = OPFLOW_KRYLOV_FGMRES; o.precond = pre(P); break;
            case StructSolverType::LGMRES: o.krylov = OPFLOW_KRYLOV_LGMRES; o.precond = pre(P); break;
            case StructSolverType::BICGSTAB: o.krylov = OPFLOW_KRYLOV_BICGSTAB; o.precond = pre(P); break;
            default: o.krylov = OPFLOW_KRYLOV_NONE; o.precond = pre(T); break;
        }
        return o;
    }
}// namespace GPU

// makeEqnSolveHandler(getter, target, solver) (src/Core/Equation/HYPREEqnSolveHandler.hpp:44-48)
template <typename F, typename Target, StructSolverType S, StructSolverType P>
std::unique_ptr<EqnSolveHandler> makeEqnSolveHandler(F&& getter, Target& target, const PrecondStructSolver<S, P>& solver) {
    Equation eq = getter(target);
    return std::make_unique<GPU::Handler<Target>>(eq, target, GPU::toParams(solver.params, solver.p_params));
}
template <typename F, typename Target, StructSolverType S>
std::unique_ptr<EqnSolveHandler> makeEqnSolveHandler(F&& getter, Target& target, const StructSolver<S>& solver) {
    Equation eq = getter(target);
    return std::make_unique<GPU::Handler<Target>>(eq, target, GPU::toParams(solver.params, StructSolverParams<StructSolverType::None> {}));
}

// Solve<S, P>(getter, target, params, p_params) (src/Core/Solvers/Struct/UnifiedSolve.hpp:36-43)
template <StructSolverType S, StructSolverType P, typename F, typename Target>
EqnSolveState Solve(F&& getter, Target& target, const StructSolverParams<S>& params, const StructSolverParams<P>& p_params) {
    auto h = makeEqnSolveHandler(std::forward<F>(getter), target, PrecondStructSolver<S, P>(params, p_params));
    return h->solve();
}
template <StructSolverType S = StructSolverType::PCG, StructSolverType P = StructSolverType::PFMG, typename F, typename Target>
EqnSolveState Solve(F&& getter, Target& target) {
    return Solve<S, P>(std::forward<F>(getter), target, StructSolverParams<S> {}, StructSolverParams<P> {});
}

// ------------------------------------------------------------------------------------ snapshots
namespace Utils {
    // TimeStamp (src/Utils/Writers/Streams.hpp:31-45)
    struct TimeStamp {
        double time {};
        TimeStamp() = default;
        explicit TimeStamp(double t) : time(t) {}
        explicit operator double() const { return time; }
    };
    // the directory part of a stream path (std::filesystem::path::parent_path of a plain path)
    inline std::string parentDir(const std::string& p) {
        const auto k = p.find_last_of('/');
        return k == std::string::npos ? std::string(".") : (k == 0 ? std::string("/") : p.substr(0, k));
    }
    // RawBinaryOStream (src/Utils/Writers/RawBinaryStream.hpp:42-62, 97-150): `s << TimeStamp(t) << u`
    // writes <dir>/<name>_<count>.cart and advances the counter
    struct RawBinaryOStream {
        std::string dir = ".";
        double time = 0.;
        int count = 0;
        RawBinaryOStream() = default;
        explicit RawBinaryOStream(const std::string& path) : dir(parentDir(path)) {}
        void setCounterTo(int c) { count = c; }
        RawBinaryOStream& operator<<(const TimeStamp& t) {
            time = t.time;
            return *this;
        }
        template <typename R, typename M>
        RawBinaryOStream& operator<<(const CartesianField<R, M>& f) {
            GPU::check(opflow_field_write_raw(f.handle(), dir.c_str(), f.name.c_str(), count, time), "RawBinaryOStream");
            ++count;
            return *this;
        }
    };
    // RawBinaryIStream (RawBinaryStream.hpp:64-77, 152-224): `s >> u` reads <dir>/<name>_<count>.cart
    struct RawBinaryIStream {
        std::string dir = ".";
        int count = 0;
        double time = 0.;
        RawBinaryIStream() = default;
        explicit RawBinaryIStream(const std::string& path) : dir(parentDir(path)) {}
        void setCounterTo(int c) { count = c; }
        template <typename R, typename M>
        RawBinaryIStream& operator>>(CartesianField<R, M>& f) {
            GPU::check(opflow_field_read_raw(f.handle(), dir.c_str(), f.name.c_str(), count, &time), "RawBinaryIStream");
            f.h->host_valid = false;
            ++count;
            return *this;
        }
    };
}// namespace Utils

// EnvironmentGardian (src/Core/Environment.hpp): brings the engine up and releases it at scope exit.
struct EnvironmentGardian {
    EnvironmentGardian() { GPU::context(); }
    EnvironmentGardian(int*, char***) { GPU::context(); }
    ~EnvironmentGardian() {
        opflow_ctx& c = GPU::contextSlot();
        if (c) {
            opflow_ctx_synchronize(c);
        }
    }
};

}// namespace OpFlow

#endif// OPFLOW_GB300_OPFLOWGPU_HPP
