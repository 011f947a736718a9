// Path E: expression trees -> device programs and stencil kernels.
//
// An assignment `dst <op>= expr` (internal::FieldAssigner::assign, src/Core/Loops/FieldAssigner.hpp:27-84)
// is lowered in one of three ways:
//   1. FTCS-shaped trees  u + s*(d2<0>(u) + d2<1>(u) [+ d2<2>(u)])  on a uniform mesh go to a fused
//      exact kernel that performs the reference's IEEE operations in its order
//      (D2SecondOrderCentered::eval, D2SecondOrderCentered.hpp:160-171).
//   2. In OPFLOW_EVAL_FAST mode, a tree that is a linear constant-coefficient stencil of one field goes
//      to a fixed-point kernel (exact 64-bit integer sums, one product per weight group, one rounding
//      back to float64 per point) that runs on the integer pipes instead of GB300's narrow FP64 pipe.
//   3. Everything else runs in a generic interpreter kernel over a postfix program expanded from the
//      tree, again in the reference's operation order.
#include "internal.h"
#include "stencil.h"
#include "pointwise.h"

#include <algorithm>
#include <array>
#include <cmath>
#include <map>
#include <unordered_map>

namespace opg {

// ======================================================================================== program format
enum POp : int {
    P_LOAD = 0, P_CONST, P_ADD, P_SUB, P_MUL, P_DIV, P_NEG, P_DX, P_X, P_WENO,
    P_GT, P_GE, P_LT, P_LE, P_NE, P_AND, P_OR, P_NOT,  // 1.0 / 0.0 results
    P_SEL,  // c ? a : b with (c, a, b) on the stack, c true when non-zero
    P_F1,   // slot: enum opflow_func1
    P_F2,   // slot: enum opflow_func2
    P_LIM   // slot: enum opflow_flux_limiter (a non-linear limiter K(r))
};
struct Instr {
    int op;
    int slot;    // P_LOAD: leaf slot; P_DX/P_X: dim; P_WENO: 1 for the upwind variant; P_F1/P_F2/P_LIM: function
    int off[3];  // P_LOAD: offset; P_DX/P_X: off[0] = index offset along dim
    double v;    // P_CONST
};

static bool is_pow2(double h) {
    if (!(h > 0) || !std::isfinite(h)) return false;
    int e;
    double m = std::frexp(h, &e);
    return m == 0.5;
}

static bool func1_known(int f) { return (f >= OPFLOW_F_ABS && f <= OPFLOW_F_RINT) || (f >= OPFLOW_F_EXP && f <= OPFLOW_F_LGAMMA); }
static bool func2_known(int f) { return (f >= OPFLOW_F2_MAX && f <= OPFLOW_F2_REMAINDER) || (f >= OPFLOW_F2_POW && f <= OPFLOW_F2_ATAN2); }

// Host compiler: expands the tree into postfix with per-leaf offsets, mirroring the recursion of
// Expression::evalAtImpl_final (Expression.hpp:51-88); operands of binary operators keep their order.
struct Compiler {
    const opflow_node* nodes;
    int n;
    const opflow_field* leaves;
    int nleaves;
    const MeshDev* mesh;
    std::vector<std::array<int, 3>> loc;  // per node, -1 = scalar
    std::vector<Instr> prog;
    int max_off[3][2] = {{0, 0}, {0, 0}, {0, 0}};  // per dim min/max offset touched, per slot merged
    std::vector<std::array<int, 6>> slot_extent;   // per slot: min/max offset per dim
    int err = OPFLOW_OK;
    size_t limit = 1 << 16;

    int locs() {
        loc.assign(n, {-1, -1, -1});
        for (int k = 0; k < n; ++k) {
            const opflow_node& nd = nodes[k];
            if (nd.a >= k || nd.b >= k) return fail(OPFLOW_E_INVALID, "node %d: children must precede parents", k);
            if (nd.kind == OPFLOW_NODE_COND && (nd.c < 0 || nd.c >= k)) return fail(OPFLOW_E_INVALID, "node %d: bad third operand", k);
            auto& L = loc[k];
            switch (nd.kind) {
                case OPFLOW_NODE_FIELD:
                    if (nd.field < 0 || nd.field >= nleaves || !leaves[nd.field]) return fail(OPFLOW_E_INVALID, "node %d: bad leaf slot %d", k, nd.field);
                    for (int d = 0; d < 3; ++d) L[d] = leaves[nd.field]->desc.loc[d];
                    break;
                case OPFLOW_NODE_CONST: break;
                case OPFLOW_NODE_ADD: case OPFLOW_NODE_SUB: case OPFLOW_NODE_MUL: case OPFLOW_NODE_DIV:
                case OPFLOW_NODE_GT: case OPFLOW_NODE_GE: case OPFLOW_NODE_LT: case OPFLOW_NODE_LE: case OPFLOW_NODE_NE:
                case OPFLOW_NODE_AND: case OPFLOW_NODE_OR: case OPFLOW_NODE_FUNC2:
                    // initPropsFrom(arg1), or arg2 when arg1 is a scalar (BinOpDefMacros.hpp.in)
                    if (nd.a < 0 || nd.b < 0) return fail(OPFLOW_E_INVALID, "node %d: missing operand", k);
                    if (nd.kind == OPFLOW_NODE_FUNC2 && !func2_known(nd.field)) return fail(OPFLOW_E_INVALID, "node %d: unknown function %d", k, nd.field);
                    L = loc[nd.a][0] >= 0 ? loc[nd.a] : loc[nd.b];
                    break;
                case OPFLOW_NODE_NOT: case OPFLOW_NODE_FUNC1:
                    if (nd.a < 0) return fail(OPFLOW_E_INVALID, "node %d: missing operand", k);
                    if (nd.kind == OPFLOW_NODE_FUNC1 && !func1_known(nd.field)) return fail(OPFLOW_E_INVALID, "node %d: unknown function %d", k, nd.field);
                    L = loc[nd.a];
                    break;
                case OPFLOW_NODE_COND:
                    // CondOp::prepare: initPropsFrom(arg2), or arg3 when arg2 is a scalar (Conditional.hpp:41-115)
                    if (nd.a < 0 || nd.b < 0) return fail(OPFLOW_E_INVALID, "node %d: missing operand", k);
                    L = loc[nd.b][0] >= 0 ? loc[nd.b] : (loc[nd.c][0] >= 0 ? loc[nd.c] : loc[nd.a]);
                    break;
                case OPFLOW_NODE_INTP_FL_CEN2COR: case OPFLOW_NODE_INTP_FL_COR2CEN: {
                    // D1FluxLimiterImpl::prepare (D1FluxLimiter.hpp:152-166, 182-201)
                    if (nd.a < 0 || nd.b < 0) return fail(OPFLOW_E_INVALID, "node %d: missing operand", k);
                    if (nd.dim < 0 || nd.dim >= mesh->ndim) return fail(OPFLOW_E_INVALID, "node %d: operator dim %d", k, nd.dim);
                    if (nd.field < OPFLOW_FL_CDS || nd.field > OPFLOW_FL_BSOU) return fail(OPFLOW_E_INVALID, "node %d: unknown flux limiter %d", k, nd.field);
                    if (loc[nd.b][0] < 0) return fail(OPFLOW_E_INVALID, "node %d: interpolation of a scalar", k);
                    const bool c2c = nd.kind == OPFLOW_NODE_INTP_FL_CEN2COR;
                    if (loc[nd.b][nd.dim] != (c2c ? OPFLOW_CENTER : OPFLOW_CORNER))
                        return fail(OPFLOW_E_INVALID, "node %d: flux-limiter interpolation of an expression located at the %s along dim %d", k,
                                    c2c ? "corner" : "centre", nd.dim);
                    L = loc[nd.b];
                    L[nd.dim] = c2c ? OPFLOW_CORNER : OPFLOW_CENTER;
                    break;
                }
                case OPFLOW_NODE_NEG: case OPFLOW_NODE_D2: case OPFLOW_NODE_WENO53_DOWN: case OPFLOW_NODE_WENO53_UP:
                case OPFLOW_NODE_D1: case OPFLOW_NODE_INTP_C2C: case OPFLOW_NODE_INTP_COR2CEN:
                case OPFLOW_NODE_D1_BIASED_UP: case OPFLOW_NODE_D1_BIASED_DOWN:
                    if (nd.a < 0) return fail(OPFLOW_E_INVALID, "node %d: missing operand", k);
                    L = loc[nd.a];
                    if (nd.kind != OPFLOW_NODE_NEG) {
                        if (nd.dim < 0 || nd.dim >= mesh->ndim) return fail(OPFLOW_E_INVALID, "node %d: operator dim %d", k, nd.dim);
                        if (loc[nd.a][0] < 0) return fail(OPFLOW_E_INVALID, "node %d: differential operator on a scalar", k);
                    }
                    if (nd.kind == OPFLOW_NODE_D1) L[nd.dim] = L[nd.dim] == OPFLOW_CENTER ? OPFLOW_CORNER : OPFLOW_CENTER;
                    if (nd.kind == OPFLOW_NODE_INTP_C2C) L[nd.dim] = OPFLOW_CORNER;
                    if (nd.kind == OPFLOW_NODE_INTP_COR2CEN) L[nd.dim] = OPFLOW_CENTER;
                    break;
                default: return fail(OPFLOW_E_UNSUPPORTED, "node %d: unknown kind %d", k, nd.kind);
            }
        }
        return OPFLOW_OK;
    }

    void push(const Instr& in) {
        if (prog.size() >= limit) { err = fail(OPFLOW_E_UNSUPPORTED, "expression expands beyond %zu instructions", limit); return; }
        prog.push_back(in);
    }
    void cst(double v) { push(Instr{P_CONST, 0, {0, 0, 0}, v}); }
    // binary op with constant folding when both operands are constants (host IEEE arithmetic, no
    // contraction: this file's host code is compiled with -ffp-contract=off)
    void bin(int op) {
        size_t s = prog.size();
        if (s >= 2 && prog[s - 1].op == P_CONST && prog[s - 2].op == P_CONST) {
            double a = prog[s - 2].v, b = prog[s - 1].v, r = 0;
            switch (op) {
                case P_ADD: r = a + b; break;
                case P_SUB: r = a - b; break;
                case P_MUL: r = a * b; break;
                case P_DIV: r = a / b; break;
            }
            prog.pop_back();
            prog.back().v = r;
            return;
        }
        // division by a constant power of two is an exact multiplication by its reciprocal
        if (op == P_DIV && s >= 1 && prog[s - 1].op == P_CONST && is_pow2(prog[s - 1].v)) {
            prog[s - 1].v = 1.0 / prog[s - 1].v;
            op = P_MUL;
        }
        push(Instr{op, 0, {0, 0, 0}, 0.});
    }
    void mesh_dx(int d, int o) {
        if (mesh->uniform[d]) cst(mesh->h[d]);
        else push(Instr{P_DX, d, {o, 0, 0}, 0.});
    }
    void mesh_x(int d, int o) { push(Instr{P_X, d, {o, 0, 0}, 0.}); }

    void emit(int k, const int* off) {
        if (err) return;
        const opflow_node& nd = nodes[k];
        switch (nd.kind) {
            case OPFLOW_NODE_FIELD: {
                Instr in{P_LOAD, nd.field, {off[0], off[1], off[2]}, 0.};
                auto& e = slot_extent[nd.field];
                for (int d = 0; d < 3; ++d) { e[2 * d] = std::min(e[2 * d], off[d]); e[2 * d + 1] = std::max(e[2 * d + 1], off[d]); }
                push(in);
                break;
            }
            case OPFLOW_NODE_CONST: cst(nd.value); break;
            case OPFLOW_NODE_ADD: emit(nd.a, off); emit(nd.b, off); bin(P_ADD); break;
            case OPFLOW_NODE_SUB: emit(nd.a, off); emit(nd.b, off); bin(P_SUB); break;
            case OPFLOW_NODE_MUL: emit(nd.a, off); emit(nd.b, off); bin(P_MUL); break;
            case OPFLOW_NODE_DIV: emit(nd.a, off); emit(nd.b, off); bin(P_DIV); break;
            case OPFLOW_NODE_NEG:
                emit(nd.a, off);
                if (!prog.empty() && prog.back().op == P_CONST) prog.back().v = -prog.back().v;
                else push(Instr{P_NEG, 0, {0, 0, 0}, 0.});
                break;
            case OPFLOW_NODE_D2: {
                // ((r - c)/dx_r - (c - l)/dx_l)/dx_c
                const int d = nd.dim, corner = loc[nd.a][d] == OPFLOW_CORNER, o = off[d];
                int op_[3] = {off[0], off[1], off[2]}, om[3] = {off[0], off[1], off[2]};
                op_[d]++; om[d]--;
                auto dxl = [&] { if (corner) mesh_dx(d, o - 1); else { mesh_dx(d, o - 1); mesh_dx(d, o); bin(P_ADD); cst(0.5); bin(P_MUL); } };
                auto dxr = [&] { if (corner) mesh_dx(d, o); else { mesh_dx(d, o); mesh_dx(d, o + 1); bin(P_ADD); cst(0.5); bin(P_MUL); } };
                emit(nd.a, op_); emit(nd.a, off); bin(P_SUB); dxr(); bin(P_DIV);
                emit(nd.a, off); emit(nd.a, om); bin(P_SUB); dxl(); bin(P_DIV);
                bin(P_SUB);
                dxl(); dxr(); bin(P_ADD); cst(0.5); bin(P_MUL);
                bin(P_DIV);
                break;
            }
            case OPFLOW_NODE_D1: {
                const int d = nd.dim, o = off[d];
                int op_[3] = {off[0], off[1], off[2]}, om[3] = {off[0], off[1], off[2]};
                op_[d]++; om[d]--;
                if (loc[nd.a][d] == OPFLOW_CENTER) {
                    emit(nd.a, off); emit(nd.a, om); bin(P_SUB);
                    mesh_dx(d, o - 1); mesh_dx(d, o); bin(P_ADD); bin(P_DIV);
                    cst(2.0); bin(P_MUL);
                } else {
                    emit(nd.a, op_); emit(nd.a, off); bin(P_SUB); mesh_dx(d, o); bin(P_DIV);
                }
                break;
            }
            case OPFLOW_NODE_WENO53_DOWN: case OPFLOW_NODE_WENO53_UP: {
                const int d = nd.dim, up = nd.kind == OPFLOW_NODE_WENO53_UP;
                for (int s = 0; s < 6; ++s) {
                    int j[3] = {off[0], off[1], off[2]};
                    j[d] += up ? (3 - s) : (s - 3);
                    emit(nd.a, j);
                }
                mesh_dx(d, off[d]);
                push(Instr{P_WENO, up, {0, 0, 0}, 0.});
                break;
            }
            case OPFLOW_NODE_INTP_C2C: {
                // intp(x1 - x, y1, x2 - x, y2) with x1 = x(i-1) + 0.5*dx(i-1), x2 = x(i) + 0.5*dx(i), x = x(i):
                // (a*y2 - b*y1) / (a - b), a = x1 - x, b = x2 - x
                const int d = nd.dim, o = off[d];
                int om[3] = {off[0], off[1], off[2]};
                om[d]--;
                auto A = [&] { mesh_x(d, o - 1); cst(0.5); mesh_dx(d, o - 1); bin(P_MUL); bin(P_ADD); mesh_x(d, o); bin(P_SUB); };
                auto B = [&] { mesh_x(d, o); cst(0.5); mesh_dx(d, o); bin(P_MUL); bin(P_ADD); mesh_x(d, o); bin(P_SUB); };
                A(); emit(nd.a, off); bin(P_MUL);
                B(); emit(nd.a, om); bin(P_MUL);
                bin(P_SUB);
                A(); B(); bin(P_SUB);
                bin(P_DIV);
                break;
            }
            case OPFLOW_NODE_INTP_COR2CEN: {
                // Math::mid(e(i), e(i + 1)) = (x1 + x2) * 0.5
                int op_[3] = {off[0], off[1], off[2]};
                op_[nd.dim]++;
                emit(nd.a, off); emit(nd.a, op_); bin(P_ADD); cst(0.5); bin(P_MUL);
                break;
            }
            case OPFLOW_NODE_D1_BIASED_UP: case OPFLOW_NODE_D1_BIASED_DOWN: {
                // upwind:   (e(i+1) - e(i)) / (Corner ? dx(i)   : (dx(i)   + dx(i+1)) * 0.5)
                // downwind: (e(i) - e(i-1)) / (Corner ? dx(i-1) : (dx(i-1) + dx(i))   * 0.5)
                const int d = nd.dim, up = nd.kind == OPFLOW_NODE_D1_BIASED_UP, o = off[d] - (up ? 0 : 1);
                int hi[3] = {off[0], off[1], off[2]}, lo[3] = {off[0], off[1], off[2]};
                if (up) hi[d]++; else lo[d]--;
                emit(nd.a, hi); emit(nd.a, lo); bin(P_SUB);
                if (loc[nd.a][d] == OPFLOW_CORNER) mesh_dx(d, o);
                else { mesh_dx(d, o); mesh_dx(d, o + 1); bin(P_ADD); cst(0.5); bin(P_MUL); }
                bin(P_DIV);
                break;
            }
            case OPFLOW_NODE_GT: case OPFLOW_NODE_GE: case OPFLOW_NODE_LT: case OPFLOW_NODE_LE: case OPFLOW_NODE_NE:
            case OPFLOW_NODE_AND: case OPFLOW_NODE_OR: {
                static const int ops[] = {P_GT, P_GE, P_LT, P_LE, P_NE, P_AND, P_OR};
                emit(nd.a, off); emit(nd.b, off);
                push(Instr{ops[nd.kind - OPFLOW_NODE_GT], 0, {0, 0, 0}, 0.});
                break;
            }
            case OPFLOW_NODE_NOT: emit(nd.a, off); push(Instr{P_NOT, 0, {0, 0, 0}, 0.}); break;
            case OPFLOW_NODE_FUNC1: emit(nd.a, off); push(Instr{P_F1, nd.field, {0, 0, 0}, 0.}); break;
            case OPFLOW_NODE_FUNC2: emit(nd.a, off); emit(nd.b, off); push(Instr{P_F2, nd.field, {0, 0, 0}, 0.}); break;
            case OPFLOW_NODE_COND:
                // both branches are evaluated; the reference evaluates only the taken one, with the same value
                emit(nd.a, off); emit(nd.b, off); emit(nd.c, off);
                push(Instr{P_SEL, 0, {0, 0, 0}, 0.});
                break;
            case OPFLOW_NODE_INTP_FL_CEN2COR: case OPFLOW_NODE_INTP_FL_COR2CEN: {
                // u(i) > 0. ? upwind : downwind (D1FluxLimiterImpl::eval)
                emit(nd.a, off); cst(0.); push(Instr{P_GT, 0, {0, 0, 0}, 0.});
                flux_side(nd, off, true);
                flux_side(nd, off, false);
                push(Instr{P_SEL, 0, {0, 0, 0}, 0.});
                break;
            }
        }
    }

    // One side of D1FluxLimiterUpwindImpl / D1FluxLimiterDownwindImpl (D1FluxLimiter.hpp:36-133).
    // Points p1, p2, p3 along dim (offsets from i); positions are cell centres x + 0.5*dx (Cen2Cor) or
    // nodes x (Cor2Cen); su, sf the upwind and face slopes; the value is y2 +- (dx(o)*0.5)*K(su, sf)
    // for the kappa kernels and y2 +- ((dx(o)*0.5)*K(sf/(su + 1e-16)))*su for the limiters.
    void flux_side(const opflow_node& nd, const int* off, bool up) {
        const int d = nd.dim, c2c = nd.kind == OPFLOW_NODE_INTP_FL_CEN2COR;
        int p1, hoff;  // offset of the first point and of the dx factor
        if (c2c) { p1 = up ? -2 : -1; hoff = up ? -1 : 0; }
        else { p1 = up ? -1 : 0; hoff = 0; }
        auto pos = [&](int q) {
            const int o = off[d] + p1 + q;
            if (c2c) {
                if (up) { mesh_x(d, o); cst(0.5); mesh_dx(d, o); bin(P_MUL); bin(P_ADD); }  // x + 0.5*dx
                else { mesh_x(d, o); mesh_dx(d, o); cst(0.5); bin(P_MUL); bin(P_ADD); }     // x + dx*0.5
            } else mesh_x(d, o);
        };
        auto val = [&](int q) { int j[3] = {off[0], off[1], off[2]}; j[d] += p1 + q; emit(nd.b, j); };
        // slope between points q and q+1: (y(q+1) - y(q)) / (x(q+1) - x(q))
        auto slope = [&](int q) { val(q + 1); val(q); bin(P_SUB); pos(q + 1); pos(q); bin(P_SUB); bin(P_DIV); };
        auto su = [&] { slope(up ? 0 : 1); };
        auto sf = [&] { slope(up ? 1 : 0); };
        val(1);                                             // y2
        mesh_dx(d, off[d] + hoff); cst(0.5); bin(P_MUL);    // dx*0.5
        const int K = nd.field;
        if (K <= OPFLOW_FL_LUI) {
            // KappaKernel::eval(slop_u, slop_f) = (1 + kappa) / 2. * slop_f + (1 - kappa) / 2. * slop_u
            static const double kap[] = {1., 0.5, 1. / 3., 0., -1.};
            cst((1 + kap[K]) / 2.); sf(); bin(P_MUL);
            cst((1 - kap[K]) / 2.); su(); bin(P_MUL);
            bin(P_ADD);
            bin(P_MUL);
        } else {
            sf(); su(); cst(1e-16); bin(P_ADD); bin(P_DIV);  // r
            push(Instr{P_LIM, K, {0, 0, 0}, 0.});
            bin(P_MUL);
            su(); bin(P_MUL);
        }
        bin(up ? P_ADD : P_SUB);
    }

    int run() {
        OPG_TRY(locs());
        slot_extent.assign(nleaves, {0, 0, 0, 0, 0, 0});
        int off[3] = {0, 0, 0};
        emit(n - 1, off);
        if (err) return err;
        // stack depth check
        int sp = 0, maxsp = 0;
        for (auto& in : prog) {
            switch (in.op) {
                case P_LOAD: case P_CONST: case P_DX: case P_X: sp++; break;
                case P_NEG: case P_NOT: case P_F1: case P_LIM: break;
                case P_WENO: sp -= 6; break;
                case P_SEL: sp -= 2; break;
                default: sp--; break;
            }
            maxsp = std::max(maxsp, sp);
        }
        if (sp != 1) return fail(OPFLOW_E_INVALID, "malformed expression");
        if (maxsp > 24) return fail(OPFLOW_E_UNSUPPORTED, "expression needs a stack of %d values (limit 24)", maxsp);
        return OPFLOW_OK;
    }
};

// ======================================================================================== device helpers
struct LeafViews {
    FieldView v[8];
    int n;
};
struct MeshPtrs {
    const double* x[3];
    const double* dx[3];
    int es[3];
};

__device__ __forceinline__ double ld(const FieldView& f, int i, int j, int k) {
    return f.data[(i - f.off[0]) + (j - f.off[1]) * f.sy + (k - f.off[2]) * f.sz];
}

// D1WENO53Downwind::kernel (D1WENO53Downwind.hpp:136-154) with every operation spelled as an IEEE
// intrinsic so that no multiply-add is contracted; std::max over an initializer list keeps the first
// maximal element.
__device__ double weno_kernel(double pm3, double pm2, double pm1, double p0, double pp1, double pp2, double h) {
    const double d1 = __ddiv_rn(__dsub_rn(pm2, pm3), h), d2 = __ddiv_rn(__dsub_rn(pm1, pm2), h), d3 = __ddiv_rn(__dsub_rn(p0, pm1), h),
                 d4 = __ddiv_rn(__dsub_rn(pp1, p0), h), d5 = __ddiv_rn(__dsub_rn(pp2, pp1), h);
    const double ddx1 = __dadd_rn(__dsub_rn(__ddiv_rn(d1, 3.), __ddiv_rn(__dmul_rn(7., d2), 6.)), __ddiv_rn(__dmul_rn(11., d3), 6.));
    const double ddx2 = __dadd_rn(__dadd_rn(__ddiv_rn(-d2, 6.), __ddiv_rn(__dmul_rn(5., d3), 6.)), __ddiv_rn(d4, 3.));
    const double ddx3 = __dsub_rn(__dadd_rn(__ddiv_rn(d3, 3.), __ddiv_rn(__dmul_rn(5., d4), 6.)), __ddiv_rn(d5, 6.));
    const double c1312 = 13. / 12.;
    double t1 = __dadd_rn(__dsub_rn(d1, __dmul_rn(2., d2)), d3);
    double t2 = __dadd_rn(__dsub_rn(d1, __dmul_rn(4., d2)), __dmul_rn(3., d3));
    const double s1 = __dadd_rn(__dmul_rn(c1312, __dmul_rn(t1, t1)), __ddiv_rn(__dmul_rn(t2, t2), 4.));
    t1 = __dadd_rn(__dsub_rn(d2, __dmul_rn(2., d3)), d4);
    t2 = __dsub_rn(d2, d4);
    const double s2 = __dadd_rn(__dmul_rn(c1312, __dmul_rn(t1, t1)), __ddiv_rn(__dmul_rn(t2, t2), 4.));
    t1 = __dadd_rn(__dsub_rn(d3, __dmul_rn(2., d4)), d5);
    t2 = __dadd_rn(__dsub_rn(__dmul_rn(3., d3), __dmul_rn(4., d4)), d5);
    const double s3 = __dadd_rn(__dmul_rn(c1312, __dmul_rn(t1, t1)), __ddiv_rn(__dmul_rn(t2, t2), 4.));
    double mx = __dmul_rn(d1, d1), t;
    t = __dmul_rn(d2, d2); if (mx < t) mx = t;
    t = __dmul_rn(d3, d3); if (mx < t) mx = t;
    t = __dmul_rn(d4, d4); if (mx < t) mx = t;
    t = __dmul_rn(d5, d5); if (mx < t) mx = t;
    const double eps = __dadd_rn(__dmul_rn(1e-6, mx), 1e-99);
    double q;
    q = __dadd_rn(s1, eps); const double a1 = __ddiv_rn(.1, __dmul_rn(q, q));
    q = __dadd_rn(s2, eps); const double a2 = __ddiv_rn(.6, __dmul_rn(q, q));
    q = __dadd_rn(s3, eps); const double a3 = __ddiv_rn(.3, __dmul_rn(q, q));
    const double sum = __dadd_rn(__dadd_rn(a1, a2), a3);
    const double w1 = __ddiv_rn(a1, sum), w2 = __ddiv_rn(a2, sum), w3 = __ddiv_rn(a3, sum);
    return __dadd_rn(__dadd_rn(__dmul_rn(w1, ddx1), __dmul_rn(w2, ddx2)), __dmul_rn(w3, ddx3));
}

__device__ __forceinline__ double apply_arith(int arith, double o, double v) {
    switch (arith) {
        case OPFLOW_ASSIGN_ADD: return __dadd_rn(o, v);
        case OPFLOW_ASSIGN_SUB: return __dsub_rn(o, v);
        case OPFLOW_ASSIGN_MUL: return __dmul_rn(o, v);
        case OPFLOW_ASSIGN_DIV: return __ddiv_rn(o, v);
        default: return v;
    }
}

// ======================================================================================== generic kernel
#define STACK_MAX 24
// one cell (box-relative index t) of the postfix program: out = value, or cur op value
__device__ __forceinline__ void interp_cell(const Instr* __restrict__ prog, int nprog, const LeafViews& leaves, const MeshPtrs& mesh,
                                            const Box& box, const FieldView& out, const FieldView& cur, int arith, long long t) {
    int i, j, k;
    box_index(t, box, i, j, k);
    const int idx[3] = {i, j, k};
    double st[STACK_MAX];
    int sp = 0;
    for (int p = 0; p < nprog; ++p) {
        const Instr in = prog[p];
        switch (in.op) {
            case P_LOAD: st[sp++] = ld(leaves.v[in.slot], i + in.off[0], j + in.off[1], k + in.off[2]); break;
            case P_CONST: st[sp++] = in.v; break;
            case P_ADD: sp--; st[sp - 1] = __dadd_rn(st[sp - 1], st[sp]); break;
            case P_SUB: sp--; st[sp - 1] = __dsub_rn(st[sp - 1], st[sp]); break;
            case P_MUL: sp--; st[sp - 1] = __dmul_rn(st[sp - 1], st[sp]); break;
            case P_DIV: sp--; st[sp - 1] = __ddiv_rn(st[sp - 1], st[sp]); break;
            case P_NEG: st[sp - 1] = -st[sp - 1]; break;
            case P_DX: st[sp++] = mesh.dx[in.slot][idx[in.slot] + in.off[0] - mesh.es[in.slot]]; break;
            case P_X: st[sp++] = mesh.x[in.slot][idx[in.slot] + in.off[0] - mesh.es[in.slot]]; break;
            case P_WENO: {
                sp -= 6;
                const double* a = &st[sp - 1];
                const double h = st[sp + 5];
                const double w = weno_kernel(a[0], a[1], a[2], a[3], a[4], a[5], h);
                // D1WENO53Upwind: the mirrored stencil's result, negated (exact)
                st[sp - 1] = in.slot ? -w : w;
                break;
            }
            case P_GT: sp--; st[sp - 1] = st[sp - 1] > st[sp] ? 1. : 0.; break;
            case P_GE: sp--; st[sp - 1] = st[sp - 1] >= st[sp] ? 1. : 0.; break;
            case P_LT: sp--; st[sp - 1] = st[sp - 1] < st[sp] ? 1. : 0.; break;
            case P_LE: sp--; st[sp - 1] = st[sp - 1] <= st[sp] ? 1. : 0.; break;
            case P_NE: sp--; st[sp - 1] = st[sp - 1] != st[sp] ? 1. : 0.; break;
            case P_AND: sp--; st[sp - 1] = (st[sp - 1] != 0. && st[sp] != 0.) ? 1. : 0.; break;
            case P_OR: sp--; st[sp - 1] = (st[sp - 1] != 0. || st[sp] != 0.) ? 1. : 0.; break;
            case P_NOT: st[sp - 1] = st[sp - 1] == 0. ? 1. : 0.; break;
            case P_SEL: sp -= 2; st[sp - 1] = st[sp - 1] != 0. ? st[sp] : st[sp + 1]; break;
            case P_F1: st[sp - 1] = func1_eval(in.slot, st[sp - 1]); break;
            case P_F2: sp--; st[sp - 1] = func2_eval(in.slot, st[sp - 1], st[sp]); break;
            case P_LIM: st[sp - 1] = flux_limiter(in.slot, st[sp - 1]); break;
        }
    }
    const long long o = (i - out.off[0]) + (j - out.off[1]) * out.sy + (k - out.off[2]) * out.sz;
    out.data[o] = arith == OPFLOW_ASSIGN_EQ ? st[0] : apply_arith(arith, cur.data[o], st[0]);
}

__global__ void __launch_bounds__(128) interp_kernel(const Instr* __restrict__ prog, int nprog, LeafViews leaves, MeshPtrs mesh,
                                                     Box box, FieldView out, FieldView cur, int arith) {
    const long long nx = box.hi[0] - box.lo[0], ny = box.hi[1] - box.lo[1], nz = box.hi[2] - box.lo[2];
    const long long total = nx * ny * nz;
    for (long long t = blockIdx.x * (long long) blockDim.x + threadIdx.x; t < total; t += (long long) gridDim.x * blockDim.x)
        interp_cell(prog, nprog, leaves, mesh, box, out, cur, arith, t);
}

// ======================================================================================== exact FTCS kernel
// u_out = u + s * (d2<d0>(u) + d2<d1>(u) [+ d2<d2>(u)]) on a uniform mesh, each d2 being
// ((r - c)/h - (c - l)/h)/h (D2SecondOrderCentered.hpp:160-171 with dx_l = dx_r = dx_c = h; for a
// cell-centred field (h + h)*0.5 == h exactly).  Division by h is
//   - an exact multiplication by 1/h when h is a power of two,
//   - otherwise Markstein's correctly rounded division by a constant (q = x*y, r = fma(-q, h, x),
//     q' = fma(r, y, q) with y = RN(1/h)), which returns the IEEE quotient; each divisor is checked
//     against __ddiv_rn on the device before it is used (markstein_ok).
struct FtcsParams {
    int ndim;
    int dims_order[3];  // dim of the k-th d2 term, in tree order
    double h[3], inv_h[3];
    int pow2[3];
    double s;
};

__device__ __forceinline__ double div_h(double x, double h, double y, int p2) {
    if (p2) return __dmul_rn(x, y);
    const double q = __dmul_rn(x, y);
    const double r = __fma_rn(-q, h, x);
    return __fma_rn(r, y, q);
}

// one cell (box-relative index t) of the exact FTCS update, D terms (D <= 3; a compile-time D unrolls)
__device__ __forceinline__ void ftcs_cell(const FieldView& in, const FieldView& out, const Box& box, const FtcsParams& P, long long t, int D) {
    int i, j, k;
    box_index(t, box, i, j, k);
    const long long o = (i - in.off[0]) + (j - in.off[1]) * in.sy + (k - in.off[2]) * in.sz;
    const double c = in.data[o];
    double sum = 0.;
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        if (q >= D) break;
        const int d = P.dims_order[q];
        const long long st = d == 0 ? 1 : (d == 1 ? in.sy : in.sz);
        const double l = in.data[o - st], r = in.data[o + st];
        const double h = P.h[d], y = P.inv_h[d];
        const int p2 = P.pow2[d];
        const double a = div_h(__dsub_rn(r, c), h, y, p2);
        const double b = div_h(__dsub_rn(c, l), h, y, p2);
        const double d2 = div_h(__dsub_rn(a, b), h, y, p2);
        sum = q == 0 ? d2 : __dadd_rn(sum, d2);
    }
    const long long oo = (i - out.off[0]) + (j - out.off[1]) * out.sy + (k - out.off[2]) * out.sz;
    out.data[oo] = __dadd_rn(c, __dmul_rn(P.s, sum));
}

template <int D>
__global__ void __launch_bounds__(256) ftcs_exact_kernel(FieldView in, FieldView out, Box box, FtcsParams P) {
    const long long nx = box.hi[0] - box.lo[0], ny = box.hi[1] - box.lo[1], nz = box.hi[2] - box.lo[2];
    const long long total = nx * ny * nz;
    for (long long t = blockIdx.x * (long long) blockDim.x + threadIdx.x; t < total; t += (long long) gridDim.x * blockDim.x)
        ftcs_cell(in, out, box, P, t, D);
}

// Many assignments in one launch (opflow_assign_batch): a persistent grid takes tiles of every
// assignment's box from one work queue (an atomic counter over the tile table), so grids of uneven
// sizes and expressions of uneven cost share the launch.  An FTCS-shaped item takes the exact FTCS
// cell (the values of the specialised kernels), any other the interpreter.
struct BatchItem {
    const Instr* prog;
    int nprog, arith;
    int ftcs;          // 1: the exact FTCS update of `src`
    FtcsParams fp;
    FieldView src;
    LeafViews leaves;
    MeshPtrs mesh;
    Box box;
    FieldView out, cur;
};
struct BatchTile {
    int item;
    int n;           // cells
    long long t0;    // first box-relative cell
};
constexpr int BATCH_TILE = 4096;

__global__ void __launch_bounds__(128) interp_batch_kernel(const BatchItem* __restrict__ items, const BatchTile* __restrict__ tiles, int ntiles,
                                                           int* next) {
    __shared__ int tile;
    for (;;) {
        if (threadIdx.x == 0) tile = atomicAdd(next, 1);
        __syncthreads();
        const int c = tile;
        __syncthreads();  // every thread has read `tile` before thread 0 takes the next one
        if (c >= ntiles) return;
        const BatchTile T = tiles[c];
        const BatchItem& I = items[T.item];
        if (I.ftcs) {
            for (long long t = T.t0 + threadIdx.x; t < T.t0 + T.n; t += blockDim.x) ftcs_cell(I.src, I.out, I.box, I.fp, t, I.fp.ndim);
        } else {
            for (long long t = T.t0 + threadIdx.x; t < T.t0 + T.n; t += blockDim.x)
                interp_cell(I.prog, I.nprog, I.leaves, I.mesh, I.box, I.out, I.cur, I.arith, t);
        }
    }
}

// Markstein self-check: compares the three-operation quotient with __ddiv_rn on seeded operands that
// span many binades (both signs), including values right next to multiples of h.
__global__ void markstein_check_kernel(double h, double y, unsigned long long seed, long long n, int* bad) {
    for (long long t = blockIdx.x * (long long) blockDim.x + threadIdx.x; t < n; t += (long long) gridDim.x * blockDim.x) {
        unsigned long long z = seed + (unsigned long long) (t + 1) * 0x9E3779B97F4A7C15ull;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        // mantissa random, exponent in [-60, 60], random sign
        const unsigned long long mant = z & 0xFFFFFFFFFFFFFull;
        const int ex = (int) ((z >> 52) % 121) - 60;
        double x = __longlong_as_double((long long) ((unsigned long long) (1023 + ex) << 52 | mant));
        if (z >> 63) x = -x;
        if (t % 4 == 1) x = __dmul_rn(__ddiv_rn(x, h), h);  // near multiples of h
        const double q = __dmul_rn(x, y);
        const double r = __fma_rn(-q, h, x);
        const double m = __fma_rn(r, y, q);
        if (__double_as_longlong(m) != __double_as_longlong(__ddiv_rn(x, h))) atomicAdd(bad, 1);
    }
}

static std::map<double, bool> g_markstein_cache;

static int markstein_ok(opflow_ctx ctx, double h, bool* ok) {
    auto it = g_markstein_cache.find(h);
    if (it != g_markstein_cache.end()) { *ok = it->second; return OPFLOW_OK; }
    OPG_TRY(ensure_scratch(ctx, 64));
    int* bad = (int*) ctx->scratch;
    OPG_CUDA(cudaMemsetAsync(bad, 0, sizeof(int), ctx->stream));
    markstein_check_kernel<<<ctx->num_sms * 4, 256, 0, ctx->stream>>>(h, 1.0 / h, 0x5eedull, 1LL << 22, bad);
    OPG_LAUNCHED();
    OPG_TRY(check_launch("markstein_check_kernel"));
    int hb = 0;
    OPG_CUDA(cudaMemcpyAsync(&hb, bad, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    OPG_CUDA(cudaStreamSynchronize(ctx->stream));
    *ok = hb == 0;
    g_markstein_cache[h] = *ok;
    return OPFLOW_OK;
}

int markstein_ok_public(opflow_ctx ctx, double h, bool* ok) { return markstein_ok(ctx, h, ok); }

// ======================================================================================== fast fixed point
// Linear constant-coefficient stencil of one field in difference form:
//   out = c + sum_g sigma_g * sum_{k in g} (u(i + o_k) - c),   c = u(i)
// Values are converted to 64-bit fixed point q = RN(u * 2^(58 - E)) with max|u| < 2^E, the sums of
// differences are exact integer sums, each weight group costs one 64x53-bit product rounded to the
// fixed grid, and the result is rounded once back to float64.  The running maximum that sets E for
// the next step is reduced by the same kernel (atomicMax on the bit pattern of |out|).
struct FastParams {
    int ndim;
    int nnb;                 // neighbours
    int off[12][3];
    int group[12];           // weight group of each neighbour
    int ngroups;
    unsigned long long wm[4];  // weight mantissas (53 bits) per group
    int wshift[4];           // product >> wshift gives fixed-point units
    int wneg[4];
    unsigned long long bound_bits;  // |value| bound of fixed boundary values read by the stencil
};

__device__ __forceinline__ long long to_fixed(double x, int E) {
    const unsigned long long b = (unsigned long long) __double_as_longlong(x);
    const int e = (int) ((b >> 52) & 0x7FF);
    unsigned long long m = b & 0xFFFFFFFFFFFFFull;
    int ex;
    if (e == 0) ex = 1 - 1075;
    else { m |= 1ull << 52; ex = e - 1075; }
    const int sh = ex + 58 - E;
    unsigned long long q;
    if (sh >= 0) q = m << sh;  // sh <= 5 because |x| < 2^E
    else if (sh > -64) q = (m + (1ull << (-sh - 1))) >> (-sh);
    else q = 0;
    return (b >> 63) ? -(long long) q : (long long) q;
}

__device__ __forceinline__ double from_fixed(long long q, int E) {
    if (q == 0) return 0.0;
    const unsigned long long sign = q < 0 ? 1ull : 0ull;
    unsigned long long a = q < 0 ? (unsigned long long) (-q) : (unsigned long long) q;
    const int bl = 64 - __clzll((long long) a);
    unsigned long long mant;
    int exp2 = bl - 1 + E - 58;  // unbiased exponent of the result
    if (bl <= 53) {
        mant = a << (53 - bl);
    } else {
        const int sh = bl - 53;
        mant = a >> sh;
        const unsigned long long rem = a & ((1ull << sh) - 1), half = 1ull << (sh - 1);
        if (rem > half || (rem == half && (mant & 1ull))) {
            mant++;
            if (mant == (1ull << 53)) { mant >>= 1; exp2++; }
        }
    }
    const unsigned long long bits = (sign << 63) | ((unsigned long long) (exp2 + 1023) << 52) | (mant & 0xFFFFFFFFFFFFFull);
    return __longlong_as_double((long long) bits);
}

// signed 64-bit value times an unsigned 53-bit weight mantissa, shifted right with rounding
__device__ __forceinline__ long long mul_shift(long long z, unsigned long long w, int sh, int neg) {
    const bool zn = z < 0;
    const unsigned long long a = zn ? (unsigned long long) (-z) : (unsigned long long) z;
    const unsigned long long lo = a * w, hi = __umul64hi(a, w);
    unsigned long long r;
    if (sh >= 64) r = hi >> (sh - 64);  // sh - 64 < 64 by construction
    else if (sh == 0) r = lo;
    else {
        // round half up on the dropped bits
        const unsigned long long add = 1ull << (sh - 1);
        unsigned long long lo2 = lo + add;
        unsigned long long hi2 = hi + (lo2 < lo ? 1ull : 0ull);
        r = (lo2 >> sh) | (hi2 << (64 - sh));
    }
    return (zn != (neg != 0)) ? -(long long) r : (long long) r;
}

template <int D>
__global__ void __launch_bounds__(256) fast_stencil_kernel(FieldView in, FieldView out, Box box, FastParams P,
                                                           unsigned long long* maxslots, int step) {
    const unsigned long long mx_in = maxslots[step % 3] > P.bound_bits ? maxslots[step % 3] : P.bound_bits;
    // E: smallest exponent with max|u| < 2^E
    int E = (int) ((mx_in >> 52) & 0x7FF) - 1023 + 1;
    if (mx_in == 0) E = -1000;
    const long long nx = box.hi[0] - box.lo[0], ny = box.hi[1] - box.lo[1], nz = box.hi[2] - box.lo[2];
    const long long total = nx * ny * nz;
    unsigned long long local_max = 0;
    if (blockIdx.x == 0 && threadIdx.x == 0) maxslots[(step + 2) % 3] = 0ull;
    for (long long t = blockIdx.x * (long long) blockDim.x + threadIdx.x; t < total; t += (long long) gridDim.x * blockDim.x) {
        int i, j, k;
        box_index(t, box, i, j, k);
        const long long o = (i - in.off[0]) + (j - in.off[1]) * in.sy + (k - in.off[2]) * in.sz;
        const long long qc = to_fixed(in.data[o], E);
        long long z[4] = {0, 0, 0, 0};
#pragma unroll 6
        for (int n = 0; n < P.nnb; ++n) {
            const long long on = o + P.off[n][0] + P.off[n][1] * in.sy + P.off[n][2] * in.sz;
            z[P.group[n]] += to_fixed(in.data[on], E) - qc;
        }
        long long q = qc;
        for (int g = 0; g < P.ngroups; ++g) q += mul_shift(z[g], P.wm[g], P.wshift[g], P.wneg[g]);
        const double v = from_fixed(q, E);
        const long long oo = (i - out.off[0]) + (j - out.off[1]) * out.sy + (k - out.off[2]) * out.sz;
        out.data[oo] = v;
        const unsigned long long ab = (unsigned long long) __double_as_longlong(v) & 0x7FFFFFFFFFFFFFFFull;
        local_max = ab > local_max ? ab : local_max;
    }
    // block max -> one atomic
    for (int s = 16; s > 0; s >>= 1) {
        const unsigned long long o2 = __shfl_xor_sync(0xffffffffu, local_max, s);
        local_max = o2 > local_max ? o2 : local_max;
    }
    __shared__ unsigned long long wmax[8];
    if ((threadIdx.x & 31) == 0) wmax[threadIdx.x >> 5] = local_max;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long m = 0;
        for (int w = 0; w < (int) (blockDim.x >> 5); ++w) m = wmax[w] > m ? wmax[w] : m;
        atomicMax(&maxslots[(step + 1) % 3], m);
    }
}

// max |u| over a box, as the bit pattern of a non-negative double
__global__ void maxabs_kernel(FieldView in, Box box, unsigned long long* slot) {
    const long long nx = box.hi[0] - box.lo[0], ny = box.hi[1] - box.lo[1], nz = box.hi[2] - box.lo[2];
    const long long total = nx * ny * nz;
    unsigned long long m = 0;
    for (long long t = blockIdx.x * (long long) blockDim.x + threadIdx.x; t < total; t += (long long) gridDim.x * blockDim.x) {
        int i, j, k;
        box_index(t, box, i, j, k);
        const unsigned long long b = (unsigned long long) __double_as_longlong(ld(in, i, j, k)) & 0x7FFFFFFFFFFFFFFFull;
        m = b > m ? b : m;
    }
    for (int s = 16; s > 0; s >>= 1) {
        const unsigned long long o2 = __shfl_xor_sync(0xffffffffu, m, s);
        m = o2 > m ? o2 : m;
    }
    if ((threadIdx.x & 31) == 0) atomicMax(slot, m);
}

// ======================================================================================== small kernels
__global__ void fill_kernel(FieldView f, Box box, int arith, double c) {
    const long long nx = box.hi[0] - box.lo[0], ny = box.hi[1] - box.lo[1], nz = box.hi[2] - box.lo[2];
    const long long total = nx * ny * nz;
    for (long long t = blockIdx.x * (long long) blockDim.x + threadIdx.x; t < total; t += (long long) gridDim.x * blockDim.x) {
        int i, j, k;
        box_index(t, box, i, j, k);
        const long long o = (i - f.off[0]) + (j - f.off[1]) * f.sy + (k - f.off[2]) * f.sz;
        f.data[o] = arith == OPFLOW_ASSIGN_EQ ? c : apply_arith(arith, f.data[o], c);
    }
}

static int grid_for(opflow_ctx ctx, long long n, int threads) {
    long long b = (n + threads - 1) / threads;
    const long long cap = (long long) ctx->num_sms * 16;
    if (b > cap) b = cap;
    if (b < 1) b = 1;
    return (int) b;
}

// ======================================================================================== planning
enum PlanKind { PLAN_INTERP = 0, PLAN_FTCS_EXACT = 1, PLAN_FAST = 2, PLAN_AXIS_EXACT = 3, PLAN_AXIS_FAST = 4 };
struct Plan {
    int kind = PLAN_INTERP;
    bool aliased = false;
    Box box;
    std::vector<Instr> prog;
    Instr* dprog = nullptr;
    LeafViews leaves{};
    MeshPtrs mesh{};
    FtcsParams ftcs{};
    FastParams fast{};
    AxisParams axis{};
    int src_slot = -1;  // field read by the specialised kernels
};

// The fixed-point form as per-dim weights of (u(i-e_d) - u) + (u(i+e_d) - u), if it has that shape.
static bool fast_to_axis(const FastParams& F, int ndim, AxisParams* A) {
    if (ndim < 2 || F.nnb != 2 * ndim) return false;
    int g_of_dim[3] = {-1, -1, -1};
    int seen[3][2] = {{0, 0}, {0, 0}, {0, 0}};
    for (int n = 0; n < F.nnb; ++n) {
        int d = -1, sgn = 0;
        for (int q = 0; q < 3; ++q)
            if (F.off[n][q]) { d = q; sgn = F.off[n][q] > 0; }
        if (d < 0 || d >= ndim) return false;
        if (seen[d][sgn]) return false;
        seen[d][sgn] = 1;
        if (g_of_dim[d] >= 0 && g_of_dim[d] != F.group[n]) return false;  // x- and x+ weights differ
        g_of_dim[d] = F.group[n];
    }
    std::memset(A, 0, sizeof *A);
    A->ndim = ndim;
    A->iso = F.ngroups == 1;
    for (int d = 0; d < ndim; ++d) {
        const int g = g_of_dim[d];
        A->wm[d] = F.wm[g];
        A->wshift[d] = F.wshift[g];
        A->wneg[d] = F.wneg[g];
    }
    A->bound_bits = F.bound_bits;
    return true;
}

// Checks that every read of the program at every point of the box stays inside the leaf's data array.
static int check_reads(const Compiler& C, const Box& box, const opflow_field* leaves, int nleaves) {
    for (int s = 0; s < nleaves; ++s) {
        const auto& e = C.slot_extent[s];
        bool used = false;
        for (auto& in : C.prog) used |= in.op == P_LOAD && in.slot == s;
        if (!used) continue;
        const opflow_field_info& r = leaves[s]->info;
        for (int d = 0; d < 3; ++d) {
            const int lo = box.lo[d] + e[2 * d], hi = box.hi[d] - 1 + e[2 * d + 1];
            if (lo < r.data_offset[d] || hi >= r.data_offset[d] + r.data_dims[d])
                return fail(OPFLOW_E_RANGE, "stencil reads leaf %d at index %d..%d along dim %d, outside its data [%d, %d)", s, lo, hi, d,
                            r.data_offset[d], r.data_offset[d] + r.data_dims[d]);
        }
    }
    for (auto& in : C.prog) {
        if (in.op != P_DX && in.op != P_X) continue;
        const int d = in.slot;
        const int lo = box.lo[d] + in.off[0], hi = box.hi[d] - 1 + in.off[0];
        const int n = C.mesh->n[d] - (in.op == P_DX ? 1 : 0);
        if (lo < C.mesh->es[d] || hi >= C.mesh->es[d] + n) return fail(OPFLOW_E_RANGE, "mesh read outside the extended mesh along dim %d", d);
    }
    return OPFLOW_OK;
}

// Recognises u + s*(d2<a>(u) + d2<b>(u) [+ d2<c>(u)]) with a uniform mesh along every used dim.
static bool match_ftcs(const opflow_node* nodes, int n, const MeshDev* mesh, FtcsParams* P, int* slot) {
    const opflow_node& root = nodes[n - 1];
    if (root.kind != OPFLOW_NODE_ADD) return false;
    const opflow_node& u = nodes[root.a];
    if (u.kind != OPFLOW_NODE_FIELD) return false;
    const opflow_node& mul = nodes[root.b];
    if (mul.kind != OPFLOW_NODE_MUL) return false;
    int sidx, tidx;
    if (nodes[mul.a].kind == OPFLOW_NODE_CONST) { sidx = mul.a; tidx = mul.b; }
    else if (nodes[mul.b].kind == OPFLOW_NODE_CONST) { sidx = mul.b; tidx = mul.a; }
    else return false;
    // left-associated sum of d2 terms
    std::vector<int> terms;
    int cur = tidx;
    while (nodes[cur].kind == OPFLOW_NODE_ADD) {
        terms.insert(terms.begin(), nodes[cur].b);
        cur = nodes[cur].a;
    }
    terms.insert(terms.begin(), cur);
    if ((int) terms.size() != mesh->ndim) return false;
    int used = 0;
    for (size_t q = 0; q < terms.size(); ++q) {
        const opflow_node& t = nodes[terms[q]];
        if (t.kind != OPFLOW_NODE_D2) return false;
        const opflow_node& leaf = nodes[t.a];
        if (leaf.kind != OPFLOW_NODE_FIELD || leaf.field != u.field) return false;
        if (used & (1 << t.dim)) return false;
        used |= 1 << t.dim;
        if (!mesh->uniform[t.dim]) return false;
        P->dims_order[q] = t.dim;
    }
    P->ndim = mesh->ndim;
    for (int d = 0; d < 3; ++d) {
        P->h[d] = d < mesh->ndim ? mesh->h[d] : 1.0;
        P->inv_h[d] = 1.0 / P->h[d];
        P->pow2[d] = is_pow2(P->h[d]);
    }
    P->s = nodes[sidx].value;
    *slot = u.field;
    return true;
}

// Affine form of the tree over (slot, offset) leaves with uniform-mesh constants; true when it is
// linear in a single field with offsets in {0, +-e_d}.
struct Lin {
    bool ok = true;
    bool isconst = true;
    double c = 0.;
    std::map<std::array<int, 4>, double> w;
};
static Lin lin_eval(const Compiler& C, int k, const int* off) {
    const opflow_node& nd = C.nodes[k];
    Lin r;
    auto bin = [&](Lin a, Lin b, int op) {
        Lin o;
        o.ok = a.ok && b.ok;
        if (!o.ok) return o;
        if (op == P_ADD || op == P_SUB) {
            const double sg = op == P_ADD ? 1. : -1.;
            o = a;
            o.isconst = a.isconst && b.isconst;
            o.c = a.c + sg * b.c;
            for (auto& kv : b.w) o.w[kv.first] += sg * kv.second;
            return o;
        }
        if (op == P_MUL) {
            if (!a.isconst && !b.isconst) { o.ok = false; return o; }
            const Lin& s = a.isconst ? a : b;
            const Lin& v = a.isconst ? b : a;
            o = v;
            o.c = v.c * s.c;
            for (auto& kv : o.w) kv.second *= s.c;
            return o;
        }
        if (!b.isconst) { o.ok = false; return o; }
        o = a;
        o.c = a.c / b.c;
        for (auto& kv : o.w) kv.second /= b.c;
        return o;
    };
    auto cstv = [](double v) { Lin l; l.c = v; return l; };
    switch (nd.kind) {
        case OPFLOW_NODE_FIELD: r.isconst = false; r.w[{nd.field, off[0], off[1], off[2]}] = 1.0; return r;
        case OPFLOW_NODE_CONST: r.c = nd.value; return r;
        case OPFLOW_NODE_ADD: return bin(lin_eval(C, nd.a, off), lin_eval(C, nd.b, off), P_ADD);
        case OPFLOW_NODE_SUB: return bin(lin_eval(C, nd.a, off), lin_eval(C, nd.b, off), P_SUB);
        case OPFLOW_NODE_MUL: return bin(lin_eval(C, nd.a, off), lin_eval(C, nd.b, off), P_MUL);
        case OPFLOW_NODE_DIV: return bin(lin_eval(C, nd.a, off), lin_eval(C, nd.b, off), P_DIV);
        case OPFLOW_NODE_NEG: return bin(cstv(-1.), lin_eval(C, nd.a, off), P_MUL);
        case OPFLOW_NODE_D2: {
            const int d = nd.dim;
            if (!C.mesh->uniform[d]) { r.ok = false; return r; }
            const double h = C.mesh->h[d];
            int op_[3] = {off[0], off[1], off[2]}, om[3] = {off[0], off[1], off[2]};
            op_[d]++; om[d]--;
            Lin a = bin(bin(lin_eval(C, nd.a, op_), lin_eval(C, nd.a, off), P_SUB), cstv(h), P_DIV);
            Lin b = bin(bin(lin_eval(C, nd.a, off), lin_eval(C, nd.a, om), P_SUB), cstv(h), P_DIV);
            return bin(bin(a, b, P_SUB), cstv(h), P_DIV);
        }
        case OPFLOW_NODE_D1_BIASED_UP: case OPFLOW_NODE_D1_BIASED_DOWN: {
            // on a uniform mesh both locations divide by h ((h + h) * 0.5 == h)
            const int d = nd.dim;
            if (!C.mesh->uniform[d]) { r.ok = false; return r; }
            int hi[3] = {off[0], off[1], off[2]}, lo[3] = {off[0], off[1], off[2]};
            if (nd.kind == OPFLOW_NODE_D1_BIASED_UP) hi[d]++; else lo[d]--;
            return bin(bin(lin_eval(C, nd.a, hi), lin_eval(C, nd.a, lo), P_SUB), cstv(C.mesh->h[d]), P_DIV);
        }
        default: r.ok = false; return r;
    }
}

static bool match_fast(const Compiler& C, int* slot, FastParams* P) {
    int off[3] = {0, 0, 0};
    Lin L = lin_eval(C, C.n - 1, off);
    if (!L.ok || L.isconst || L.c != 0.) return false;
    int s = -1;
    double wsum = 0.;
    std::vector<std::pair<std::array<int, 3>, double>> nb;
    for (auto& kv : L.w) {
        if (s < 0) s = kv.first[0];
        if (kv.first[0] != s) return false;
        std::array<int, 3> o = {kv.first[1], kv.first[2], kv.first[3]};
        int nz = 0, mag = 0;
        for (int d = 0; d < 3; ++d) { nz += o[d] != 0; mag = std::max(mag, std::abs(o[d])); }
        if (nz > 1 || mag > 1) return false;
        wsum += kv.second;
        if (nz != 0) nb.push_back({o, kv.second});
    }
    if (std::fabs(wsum - 1.0) > 1e-12 || nb.empty() || nb.size() > 12) return false;
    std::vector<double> gw;
    P->nnb = (int) nb.size();
    for (size_t q = 0; q < nb.size(); ++q) {
        for (int d = 0; d < 3; ++d) P->off[q][d] = nb[q].first[d];
        int g = -1;
        for (size_t h = 0; h < gw.size(); ++h)
            if (gw[h] == nb[q].second) g = (int) h;
        if (g < 0) {
            if (gw.size() >= 4) return false;
            gw.push_back(nb[q].second);
            g = (int) gw.size() - 1;
        }
        P->group[q] = g;
    }
    P->ngroups = (int) gw.size();
    for (size_t g = 0; g < gw.size(); ++g) {
        // w = m * 2^(e - 53) with m a 53-bit integer: product (z * m) >> (53 - e)
        int e;
        double mf = std::frexp(std::fabs(gw[g]), &e);  // |w| = mf * 2^e, mf in [0.5, 1)
        unsigned long long m = (unsigned long long) std::ldexp(mf, 53);
        int sh = 53 - e;
        if (gw[g] == 0.0) { m = 0; sh = 0; }
        if (sh < 0 || sh >= 127) return false;
        P->wm[g] = m;
        P->wshift[g] = sh;
        P->wneg[g] = gw[g] < 0;
    }
    P->ndim = C.mesh->ndim;
    *slot = s;
    return true;
}

static int build_plan(opflow_ctx ctx, opflow_field dst, int arith, const opflow_node* nodes, int n, const opflow_field* leaves, int nleaves,
                      int mode, Plan* plan) {
    if (!ctx || !dst || !nodes || n < 1 || nleaves < 0 || nleaves > 8) return fail(OPFLOW_E_INVALID, "bad assign arguments (at most 8 leaves)");
    if (arith < OPFLOW_ASSIGN_EQ || arith > OPFLOW_ASSIGN_DIV) return fail(OPFLOW_E_INVALID, "bad arith op");
    for (int s = 0; s < nleaves; ++s) {
        if (!leaves[s]) return fail(OPFLOW_E_INVALID, "null leaf %d", s);
        if (!mesh_equal(leaves[s]->mesh, dst->mesh)) return fail(OPFLOW_E_INVALID, "leaf %d lives on another mesh", s);
        if (leaves[s]->ctx != ctx) return fail(OPFLOW_E_INVALID, "leaf %d belongs to another context", s);
    }
    Compiler C{nodes, n, leaves, nleaves, dst->mesh};
    OPG_TRY(C.run());
    plan->box = assign_box(dst->info);
    OPG_TRY(check_reads(C, plan->box, leaves, nleaves));
    for (int s = 0; s < nleaves; ++s) plan->aliased |= leaves[s] == dst;
    plan->prog = C.prog;
    plan->leaves.n = nleaves;
    for (int d = 0; d < 3; ++d) {
        plan->mesh.x[d] = dst->mesh->x[d];
        plan->mesh.dx[d] = dst->mesh->dx[d];
        plan->mesh.es[d] = dst->mesh->es[d];
    }
    // specialised kernels need the whole read footprint to be one field and EQ semantics
    if (arith == OPFLOW_ASSIGN_EQ) {
        int slot = -1;
        FastParams fp{};
        bool fast_bcs = true;  // boundary values must be constants or copies of interior values
        double bcmax = 0.;
        if (mode == OPFLOW_EVAL_FAST && match_fast(C, &slot, &fp)) {
            const opflow_field src = leaves[slot];
            for (int d = 0; d < src->info.ndim; ++d)
                for (int sd = 0; sd < 2; ++sd) {
                    const int t = src->desc.bc_type[d][sd];
                    if (t == OPFLOW_BC_DIRC && src->desc.loc[d] == OPFLOW_CORNER) bcmax = std::max(bcmax, std::fabs(src->desc.bc_value[d][sd]));
                    else if (t != OPFLOW_BC_PERIODIC) fast_bcs = false;
                }
            fp.bound_bits = (unsigned long long) __builtin_bit_cast(long long, bcmax);
        }
        if (mode == OPFLOW_EVAL_FAST && fast_bcs && slot >= 0) {
            plan->kind = PLAN_FAST;
            plan->fast = fp;
            plan->src_slot = slot;
            if (fast_to_axis(fp, dst->mesh->ndim, &plan->axis)) plan->kind = PLAN_AXIS_FAST;
        } else {
            FtcsParams P{};
            if (match_ftcs(nodes, n, dst->mesh, &P, &slot)) {
                bool ok = true;
                for (int d = 0; d < P.ndim; ++d)
                    if (!P.pow2[d]) {
                        bool good = false;
                        OPG_TRY(markstein_ok(ctx, P.h[d], &good));
                        ok = ok && good;
                    }
                if (ok) {
                    plan->kind = PLAN_FTCS_EXACT;
                    plan->ftcs = P;
                    plan->src_slot = slot;
                    if (P.ndim >= 2) {
                        AxisParams& A = plan->axis;
                        std::memset(&A, 0, sizeof A);
                        A.ndim = P.ndim;
                        for (int d = 0; d < 3; ++d) {
                            A.h[d] = P.h[d];
                            A.inv_h[d] = P.inv_h[d];
                            A.pow2[d] = P.pow2[d];
                            A.order[d] = d < P.ndim ? P.dims_order[d] : 0;
                        }
                        A.s = P.s;
                        plan->kind = PLAN_AXIS_EXACT;
                    }
                }
            }
        }
    }
    if (plan->kind == PLAN_INTERP && !plan->prog.empty()) {
        OPG_CUDA(cudaMalloc(&plan->dprog, plan->prog.size() * sizeof(Instr)));
        OPG_CUDA(cudaMemcpyAsync(plan->dprog, plan->prog.data(), plan->prog.size() * sizeof(Instr), cudaMemcpyHostToDevice, ctx->stream));
    }
    return OPFLOW_OK;
}

static void free_plan(Plan* p) {
    if (p->dprog) cudaFree(p->dprog);
    p->dprog = nullptr;
}

// A run of fixed-point steps can keep the field in fixed point between its steps when the update reads
// only the destination (u = u + sum_d w_d (u(i-e_d) + u(i+e_d) - 2u), 2D or 3D), the values outside the
// update box are constants (node-centred Dirichlet on every side, no ghost layer: updatePadding rewrites
// only those constants) and the weights obey the maximum principle (w_d >= 0, 1 - 2 sum w_d >= 0), so
// that the initial bound on |u| holds for every step.  OPFLOW_FX_RESIDENT=0 turns it off.
static bool resident_eligible(const Plan& plan, opflow_field dst, const opflow_field* leaves, int steps) {
    if (plan.kind != PLAN_AXIS_FAST || !plan.aliased || steps < 2 || plan.axis.ndim < 2 || plan.axis.ndim != dst->info.ndim) return false;
    if (leaves[plan.src_slot] != dst || !dst->padding_is_step0_only()) return false;
    const char* e = getenv("OPFLOW_FX_RESIDENT");
    if (e && e[0] == '0') return false;
    const int D = plan.axis.ndim;
    for (int d = 0; d < D; ++d)
        for (int sd = 0; sd < 2; ++sd)
            if (dst->desc.loc[d] != OPFLOW_CORNER || dst->desc.bc_type[d][sd] != OPFLOW_BC_DIRC) return false;
    double sum = 0.;
    for (int d = 0; d < D; ++d) {
        const int g = plan.axis.iso ? 0 : d;
        if (plan.axis.wneg[g]) return false;
        sum += std::ldexp((double) plan.axis.wm[g], -plan.axis.wshift[g]);
    }
    return 1.0 - 2.0 * sum >= 0.0 && axis_resident_ok(plan.axis);
}

// The scale of a fixed-point run (the exponent scale_exp gives on the device) and a float64 constant in
// that fixed point, rounded as fx_from rounds (to nearest even; half away from zero at extreme scales).
static int host_scale_exp(unsigned long long mx, unsigned long long bound_bits) {
    const unsigned long long m = mx > bound_bits ? mx : bound_bits;
    if (m == 0) return -1000;
    return (int) ((m >> 52) & 0x7FF) - 1023 + 1;
}
static long long host_fx(double v, int E) {
    const double x = std::ldexp(v, 58 - E);
    if (E > -900 && E < 1000) return (long long) std::nearbyint(x);
    return (long long) std::round(x);
}

// `reps` replays of a graph of RES_GRAPH_STEPS steady-state resident steps (fixed point in and out),
// captured from the field's current buffers; the field's buffer index ends where it started.
constexpr int RES_GRAPH_STEPS = 32;
static_assert(RES_GRAPH_STEPS % 2 == 0, "a replay returns the field to the buffer it started from");
static int run_resident_graph(opflow_ctx ctx, opflow_field dst, Plan& plan, unsigned long long* maxslots, int reps) {
    cudaGraph_t g = nullptr;
    cudaGraphExec_t exec = nullptr;
    OPG_CUDA(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    int rc = OPFLOW_OK;
    FieldView a = dst->view(), b = dst->view_back();
    for (int q = 0; q < RES_GRAPH_STEPS && rc == OPFLOW_OK; ++q) {
        rc = axis_launch_resident(ctx, a, b, plan.box, plan.axis, maxslots, false, false);
        std::swap(a, b);
    }
    // a 2D resident step is one launch: the captured ones are counted once per replay instead
    g_launches.fetch_sub((uint64_t) RES_GRAPH_STEPS);
    const cudaError_t e_end = cudaStreamEndCapture(ctx->stream, &g);
    if (rc == OPFLOW_OK && e_end != cudaSuccess) rc = fail(OPFLOW_E_CUDA, "resident-step graph capture failed: %s", cudaGetErrorString(e_end));
    if (rc == OPFLOW_OK && cudaGraphInstantiate(&exec, g, 0) != cudaSuccess) rc = fail(OPFLOW_E_CUDA, "resident-step graph instantiation failed");
    for (int r = 0; r < reps && rc == OPFLOW_OK; ++r) {
        if (cudaGraphLaunch(exec, ctx->stream) != cudaSuccess) rc = fail(OPFLOW_E_CUDA, "resident-step graph launch failed");
        g_launches.fetch_add((uint64_t) RES_GRAPH_STEPS);
        dst->version += RES_GRAPH_STEPS;
    }
    if (exec) cudaGraphExecDestroy(exec);
    if (g) cudaGraphDestroy(g);
    if (rc != OPFLOW_OK) cudaGetLastError();
    return rc;
}

// K >= 2 steps with the field in fixed point between them: step 1 reads float64; then the boundary
// nodes of both buffers take their constants' fixed-point bit patterns; the last step writes float64
// and the boundary constants are written back as float64 into both buffers.
static int run_resident(opflow_ctx ctx, opflow_field dst, Plan& plan, unsigned long long* maxslots, int steps) {
    OPG_TRY(ensure_back(dst));
    unsigned long long mx = 0;
    OPG_CUDA(cudaMemcpyAsync(&mx, maxslots, sizeof mx, cudaMemcpyDeviceToHost, ctx->stream));
    OPG_CUDA(cudaStreamSynchronize(ctx->stream));
    const int E = host_scale_exp(mx, plan.axis.bound_bits);
    double fxv[3][2] = {{0., 0.}, {0., 0.}, {0., 0.}};
    for (int d = 0; d < dst->info.ndim; ++d)
        for (int sd = 0; sd < 2; ++sd) fxv[d][sd] = __builtin_bit_cast(double, host_fx(dst->desc.bc_value[d][sd], E));
    int rc = OPFLOW_OK;
    for (int s = 0; s < steps && rc == OPFLOW_OK; ++s) {
        if (s == 1 && dst->info.ndim == 2 && steps - 2 >= 2 * RES_GRAPH_STEPS) {
            // a long run of short (2D) steady-state steps: replays of one graph of RES_GRAPH_STEPS launches
            // (an even count: every replay starts from the same buffer)
            const int reps = (steps - 2) / RES_GRAPH_STEPS;
            rc = run_resident_graph(ctx, dst, plan, maxslots, reps);
            s += reps * RES_GRAPH_STEPS - 1;
            continue;
        }
        rc = axis_launch_resident(ctx, dst->view(), dst->view_back(), plan.box, plan.axis, maxslots, s == 0, s == steps - 1);
        dst->cur = 1 - dst->cur;
        dst->version++;
        if (rc == OPFLOW_OK && s == 0) {
            dst->bc_fresh[0] = dst->bc_fresh[1] = false;
            rc = fill_dirichlet_nodes(dst, dst->buf[0], fxv);
            if (rc == OPFLOW_OK) rc = fill_dirichlet_nodes(dst, dst->buf[1], fxv);
        }
    }
    if (rc == OPFLOW_OK) rc = update_padding_full(dst, dst->buf[0]);
    if (rc == OPFLOW_OK) rc = update_padding_full(dst, dst->buf[1]);
    if (rc == OPFLOW_OK) dst->bc_fresh[0] = dst->bc_fresh[1] = true;
    if (rc == OPFLOW_OK && steps > 2 && dst->info.ndim == 3) {  // a TMA-staged step whose copy never completed
        int err = 0;
        rc = stencil_take_error(ctx->stream, &err);
        if (rc == OPFLOW_OK && err) rc = fail(OPFLOW_E_CUDA, "a TMA-staged stencil step gave up waiting for its plane copies");
    }
    return rc;
}

// One assignment step: evaluates into the back buffer when the expression reads dst (out-of-place, as
// FieldAssigner does through its temporary copy), otherwise into dst directly; then the padding.
static int run_plan(opflow_ctx ctx, opflow_field dst, int arith, const opflow_field* leaves, Plan* plan, unsigned long long* maxslots, int step) {
    const bool oop = plan->aliased;
    if (oop) OPG_TRY(ensure_back(dst));
    for (int s = 0; s < plan->leaves.n; ++s) plan->leaves.v[s] = leaves[s]->view();
    FieldView out = oop ? dst->view_back() : dst->view();
    FieldView cur = dst->view();
    const long long total = plan->box.count();
    if (total > 0) {
        switch (plan->kind) {
            case PLAN_FTCS_EXACT: {
                const FieldView in = leaves[plan->src_slot]->view();
                const int g = grid_for(ctx, total, 256);
                if (plan->ftcs.ndim == 1) ftcs_exact_kernel<1><<<g, 256, 0, ctx->stream>>>(in, out, plan->box, plan->ftcs);
                else if (plan->ftcs.ndim == 2) ftcs_exact_kernel<2><<<g, 256, 0, ctx->stream>>>(in, out, plan->box, plan->ftcs);
                else ftcs_exact_kernel<3><<<g, 256, 0, ctx->stream>>>(in, out, plan->box, plan->ftcs);
                OPG_LAUNCHED();
                OPG_TRY(check_launch("ftcs_exact_kernel"));
                break;
            }
            case PLAN_AXIS_EXACT: case PLAN_AXIS_FAST:
                OPG_TRY(axis_launch(ctx, leaves[plan->src_slot]->view(), out, plan->box, plan->axis, plan->kind == PLAN_AXIS_FAST, maxslots, step));
                break;
            case PLAN_FAST: {
                const FieldView in = leaves[plan->src_slot]->view();
                const int g = grid_for(ctx, total, 256);
                if (plan->fast.ndim == 1) fast_stencil_kernel<1><<<g, 256, 0, ctx->stream>>>(in, out, plan->box, plan->fast, maxslots, step);
                else if (plan->fast.ndim == 2) fast_stencil_kernel<2><<<g, 256, 0, ctx->stream>>>(in, out, plan->box, plan->fast, maxslots, step);
                else fast_stencil_kernel<3><<<g, 256, 0, ctx->stream>>>(in, out, plan->box, plan->fast, maxslots, step);
                OPG_LAUNCHED();
                OPG_TRY(check_launch("fast_stencil_kernel"));
                break;
            }
            default: {
                const int g = grid_for(ctx, total, 128);
                interp_kernel<<<g, 128, 0, ctx->stream>>>(plan->dprog, (int) plan->prog.size(), plan->leaves, plan->mesh, plan->box, out, cur, arith);
                OPG_LAUNCHED();
                OPG_TRY(check_launch("interp_kernel"));
            }
        }
    }
    if (oop) dst->cur = 1 - dst->cur;  // (the interpreter applied `cur op value` while writing the back buffer)
    dst->version++;
    return update_padding_assign(dst);
}

}  // namespace opg

using namespace opg;

extern "C" {

int opflow_assign_repeat(opflow_ctx ctx, opflow_field dst, int arith, const opflow_node* nodes, int n_nodes, const opflow_field* leaves,
                         int n_leaves, int mode, int steps) {
    if (steps < 0) return fail(OPFLOW_E_INVALID, "negative step count");
    if (steps == 0) return OPFLOW_OK;
    Plan plan;
    int rc = build_plan(ctx, dst, arith, nodes, n_nodes, leaves, n_leaves, mode, &plan);
    if (rc) { free_plan(&plan); return rc; }
    unsigned long long* maxslots = nullptr;
    if (plan.kind == PLAN_FAST || plan.kind == PLAN_AXIS_FAST) {
        rc = ensure_scratch(ctx, 256);
        if (rc) { free_plan(&plan); return rc; }
        maxslots = (unsigned long long*) ctx->scratch;
        cudaMemsetAsync(maxslots, 0, 3 * sizeof(unsigned long long), ctx->stream);
        // the source's readable values bound the fixed-point scale of the first step
        const opflow_field src = leaves[plan.src_slot];
        Box all;
        for (int d = 0; d < 3; ++d) { all.lo[d] = src->info.data_offset[d]; all.hi[d] = all.lo[d] + src->info.data_dims[d]; }
        maxabs_kernel<<<grid_for(ctx, all.count(), 256), 256, 0, ctx->stream>>>(src->view(), all, maxslots);
        OPG_LAUNCHED();
        rc = check_launch("maxabs_kernel");
        if (rc) { free_plan(&plan); return rc; }
    }
    if (resident_eligible(plan, dst, leaves, steps)) {
        // fixed point kept in the field's buffers between the steps of the run (axis3d_fxres_kernel)
        rc = run_resident(ctx, dst, plan, maxslots, steps);
    } else {
        for (int s = 0; s < steps && rc == OPFLOW_OK; ++s) rc = run_plan(ctx, dst, arith, leaves, &plan, maxslots, s);
    }
    if (rc == OPFLOW_OK && cudaStreamSynchronize(ctx->stream) != cudaSuccess) rc = fail(OPFLOW_E_CUDA, "assign failed: %s", cudaGetErrorString(cudaGetLastError()));
    free_plan(&plan);
    return rc;
}

int opflow_assign(opflow_ctx ctx, opflow_field dst, int arith, const opflow_node* nodes, int n_nodes, const opflow_field* leaves, int n_leaves,
                  int mode) {
    return opflow_assign_repeat(ctx, dst, arith, nodes, n_nodes, leaves, n_leaves, mode, 1);
}

int opflow_assign_batch(opflow_ctx ctx, int n, const opflow_field* dsts, const int* arith, const opflow_node* const* nodes, const int* n_nodes,
                        const opflow_field* const* leaves, const int* n_leaves, int steps) {
    if (!ctx || n < 0 || (n > 0 && (!dsts || !arith || !nodes || !n_nodes || !leaves || !n_leaves))) return fail(OPFLOW_E_INVALID, "bad batch arguments");
    if (steps < 0) return fail(OPFLOW_E_INVALID, "negative step count");
    if (n == 0 || steps == 0) return OPFLOW_OK;
    for (int i = 0; i < n; ++i) {
        if (!dsts[i]) return fail(OPFLOW_E_INVALID, "null destination %d", i);
        if (dsts[i]->ctx != ctx) return fail(OPFLOW_E_INVALID, "destination %d belongs to another context", i);
        for (int q = 0; q < i; ++q)
            if (dsts[q] == dsts[i]) return fail(OPFLOW_E_INVALID, "destinations %d and %d are the same field", q, i);
    }
    // the assignments run concurrently: none may read another one's destination
    for (int i = 0; i < n; ++i)
        for (int s = 0; s < n_leaves[i]; ++s)
            for (int q = 0; q < n; ++q)
                if (q != i && leaves[i][s] == dsts[q]) return fail(OPFLOW_E_INVALID, "assignment %d reads the destination of assignment %d", i, q);
    std::vector<Plan> plans(n);
    std::vector<int> prog_at(n);
    std::vector<Instr> progs;
    int rc = OPFLOW_OK;
    for (int i = 0; i < n && rc == OPFLOW_OK; ++i) {
        // exact mode for every item: the FTCS cell where the expression has that shape, else the interpreter
        rc = build_plan(ctx, dsts[i], arith[i], nodes[i], n_nodes[i], leaves[i], n_leaves[i], OPFLOW_EVAL_EXACT, &plans[i]);
        free_plan(&plans[i]);
        if (rc == OPFLOW_OK && plans[i].aliased) rc = ensure_back(dsts[i]);
        prog_at[i] = (int) progs.size();
        progs.insert(progs.end(), plans[i].prog.begin(), plans[i].prog.end());
    }
    if (rc) return rc;
    // tiles of every box; items for even and odd steps (aliased destinations swap buffers every step)
    std::vector<BatchTile> tiles;
    for (int i = 0; i < n; ++i) {
        const long long total = plans[i].box.count();
        for (long long t0 = 0; t0 < total; t0 += BATCH_TILE) tiles.push_back(BatchTile{i, (int) std::min<long long>(BATCH_TILE, total - t0), t0});
    }
    if (tiles.size() > (size_t) 0x7fffffff) return fail(OPFLOW_E_INVALID, "too many tiles");
    std::vector<BatchItem> items(2 * (size_t) n);
    for (int par = 0; par < 2; ++par)
        for (int i = 0; i < n; ++i) {
            opflow_field d = dsts[i];
            const bool flip = par == 1 && plans[i].aliased;
            const FieldView front = flip ? d->view_back() : d->view(), back = flip ? d->view() : d->view_back();
            BatchItem& I = items[(size_t) par * n + i];
            I.nprog = (int) plans[i].prog.size();
            I.arith = arith[i];
            I.leaves = plans[i].leaves;
            for (int s = 0; s < n_leaves[i]; ++s) I.leaves.v[s] = leaves[i][s] == d ? front : leaves[i][s]->view();
            I.mesh = plans[i].mesh;
            I.box = plans[i].box;
            I.out = plans[i].aliased ? back : front;
            I.cur = front;
            I.ftcs = plans[i].kind == PLAN_FTCS_EXACT || plans[i].kind == PLAN_AXIS_EXACT;
            I.fp = plans[i].ftcs;
            if (I.ftcs) I.src = I.leaves.v[plans[i].src_slot];
        }
    const size_t bytes_items = items.size() * sizeof(BatchItem), bytes_tiles = std::max<size_t>(1, tiles.size()) * sizeof(BatchTile);
    const size_t bytes_prog = std::max<size_t>(1, progs.size()) * sizeof(Instr);
    char* blob = (char*) dev_alloc(ctx, bytes_items + bytes_tiles + bytes_prog + 256);
    if (!blob) return fail(OPFLOW_E_NOMEM, "batch tables");
    auto align = [](size_t v) { return (v + 15) & ~(size_t) 15; };
    BatchItem* d_items = (BatchItem*) blob;
    BatchTile* d_tiles = (BatchTile*) (blob + align(bytes_items));
    Instr* d_prog = (Instr*) (blob + align(bytes_items) + align(bytes_tiles));
    int* d_next = (int*) (blob + align(bytes_items) + align(bytes_tiles) + align(bytes_prog));
    for (size_t q = 0; q < items.size(); ++q) items[q].prog = d_prog + prog_at[q % n];
    rc = OPFLOW_OK;
    if (cudaMemcpyAsync(d_items, items.data(), bytes_items, cudaMemcpyHostToDevice, ctx->stream) != cudaSuccess ||
        (!tiles.empty() && cudaMemcpyAsync(d_tiles, tiles.data(), tiles.size() * sizeof(BatchTile), cudaMemcpyHostToDevice, ctx->stream) != cudaSuccess) ||
        (!progs.empty() && cudaMemcpyAsync(d_prog, progs.data(), progs.size() * sizeof(Instr), cudaMemcpyHostToDevice, ctx->stream) != cudaSuccess))
        rc = fail(OPFLOW_E_CUDA, "batch tables upload failed");
    const int grid = (int) std::max<long long>(1, std::min<long long>((long long) tiles.size(), (long long) ctx->num_sms * 8));
    for (int s = 0; s < steps && rc == OPFLOW_OK; ++s) {
        if (!tiles.empty()) {
            if (cudaMemsetAsync(d_next, 0, sizeof(int), ctx->stream) != cudaSuccess) { rc = fail(OPFLOW_E_CUDA, "batch queue reset failed"); break; }
            interp_batch_kernel<<<grid, 128, 0, ctx->stream>>>(d_items + (size_t) (s & 1) * n, d_tiles, (int) tiles.size(), d_next);
            OPG_LAUNCHED();
            rc = check_launch("interp_batch_kernel");
        }
        for (int i = 0; i < n && rc == OPFLOW_OK; ++i) {
            if (plans[i].aliased) dsts[i]->cur = 1 - dsts[i]->cur;
            dsts[i]->version++;
            rc = update_padding_assign(dsts[i]);
        }
    }
    dev_free(ctx, blob);
    if (rc == OPFLOW_OK && cudaStreamSynchronize(ctx->stream) != cudaSuccess) rc = fail(OPFLOW_E_CUDA, "batched assign failed: %s", cudaGetErrorString(cudaGetLastError()));
    return rc;
}

int opflow_field_fill(opflow_field f, int arith, double c) {
    if (!f) return fail(OPFLOW_E_INVALID, "null field");
    f->version++;
    Box b = assign_box(f->info);
    if (b.count() > 0) {
        fill_kernel<<<grid_for(f->ctx, b.count(), 256), 256, 0, f->ctx->stream>>>(f->view(), b, arith, c);
        OPG_LAUNCHED();
        OPG_TRY(check_launch("fill_kernel"));
    }
    OPG_TRY(update_padding_buf(f, f->buf[f->cur]));
    OPG_CUDA(cudaStreamSynchronize(f->ctx->stream));
    return OPFLOW_OK;
}

int opflow_field_copy(opflow_field dst, opflow_field src) {
    if (!dst || !src) return fail(OPFLOW_E_INVALID, "null field");
    if (dst->info.count != src->info.count) return fail(OPFLOW_E_INVALID, "field shapes differ");
    dst->bc_fresh[0] = dst->bc_fresh[1] = false;
    dst->version++;
    OPG_CUDA(cudaMemcpyAsync(dst->buf[dst->cur], src->buf[src->cur], src->info.count * sizeof(double), cudaMemcpyDeviceToDevice, dst->ctx->stream));
    OPG_TRY(update_padding_buf(dst, dst->buf[dst->cur]));
    OPG_CUDA(cudaStreamSynchronize(dst->ctx->stream));
    return OPFLOW_OK;
}

}  // extern "C"
