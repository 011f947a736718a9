// Path I, step 1: stencil generation.  Replaces HYPREEqnSolveHandler::initStencil / generateAb
// (src/Core/Equation/HYPREEqnSolveHandler.hpp:79-166): the tree of `lhs - rhs` is evaluated per cell
// with StencilPad arithmetic (src/DataStructures/StencilPad.hpp:137-298) in which the unknown's leaves
// are StencilField values with the reference's boundary folding (src/Core/Field/MeshBased/
// StencilField.hpp:123-350).  The device keeps each pad dense over the fixed offset set K that the
// program can reach; "absent" and "zero" coincide there, which changes no value.
#include "assemble.h"
#include "pointwise.h"

#include <cmath>
#include <map>
#include <set>

namespace opg {

// ================================================================================== program compiler
static bool is_pow2_h(double h) {
    if (!(h > 0) || !std::isfinite(h)) return false;
    int e;
    return std::frexp(h, &e) == 0.5;
}

struct PadCompiler {
    const opflow_node* nodes;
    int n;
    const opflow_field* leaves;
    int nleaves;
    int unknown;
    const MeshDev* mesh;
    std::vector<std::array<int, 3>> loc;
    std::vector<PInstr> prog;
    std::vector<int> kinds;  // static value kind per emitted stack value: 0 scalar, 1 pad
    std::vector<std::array<int, 3>> uoffs;
    std::vector<std::array<int, 6>> slot_extent;
    int err = OPFLOW_OK;

    int locs() {
        loc.assign(n, {-1, -1, -1});
        for (int k = 0; k < n; ++k) {
            const opflow_node& nd = nodes[k];
            if (nd.a >= k || nd.b >= k) return fail(OPFLOW_E_INVALID, "node %d: children must precede parents", k);
            auto& L = loc[k];
            switch (nd.kind) {
                case OPFLOW_NODE_FIELD:
                    if (nd.field < 0 || nd.field >= nleaves || !leaves[nd.field]) return fail(OPFLOW_E_INVALID, "node %d: bad leaf slot", k);
                    for (int d = 0; d < 3; ++d) L[d] = leaves[nd.field]->desc.loc[d];
                    break;
                case OPFLOW_NODE_CONST: break;
                case OPFLOW_NODE_ADD: case OPFLOW_NODE_SUB: case OPFLOW_NODE_MUL: case OPFLOW_NODE_DIV:
                    if (nd.a < 0 || nd.b < 0) return fail(OPFLOW_E_INVALID, "node %d: missing operand", k);
                    L = loc[nd.a][0] >= 0 ? loc[nd.a] : loc[nd.b];
                    break;
                case OPFLOW_NODE_NEG: case OPFLOW_NODE_D2: case OPFLOW_NODE_D1: case OPFLOW_NODE_INTP_C2C:
                case OPFLOW_NODE_INTP_COR2CEN: case OPFLOW_NODE_D1_BIASED_UP: case OPFLOW_NODE_D1_BIASED_DOWN:
                    if (nd.a < 0) return fail(OPFLOW_E_INVALID, "node %d: missing operand", k);
                    L = loc[nd.a];
                    if (nd.kind != OPFLOW_NODE_NEG && (nd.dim < 0 || nd.dim >= mesh->ndim)) return fail(OPFLOW_E_INVALID, "node %d: bad dim", k);
                    if (nd.kind == OPFLOW_NODE_D1) L[nd.dim] = L[nd.dim] == OPFLOW_CENTER ? OPFLOW_CORNER : OPFLOW_CENTER;
                    if (nd.kind == OPFLOW_NODE_INTP_C2C) L[nd.dim] = OPFLOW_CORNER;
                    if (nd.kind == OPFLOW_NODE_INTP_COR2CEN) L[nd.dim] = OPFLOW_CENTER;
                    break;
                case OPFLOW_NODE_WENO53_DOWN: case OPFLOW_NODE_WENO53_UP:
                    return fail(OPFLOW_E_UNSUPPORTED, "WENO operators are nonlinear and have no StencilPad form");
                case OPFLOW_NODE_GT: case OPFLOW_NODE_GE: case OPFLOW_NODE_LT: case OPFLOW_NODE_LE: case OPFLOW_NODE_NE:
                case OPFLOW_NODE_AND: case OPFLOW_NODE_OR: case OPFLOW_NODE_FUNC2:
                    if (nd.a < 0 || nd.b < 0) return fail(OPFLOW_E_INVALID, "node %d: missing operand", k);
                    L = loc[nd.a][0] >= 0 ? loc[nd.a] : loc[nd.b];
                    break;
                case OPFLOW_NODE_NOT: case OPFLOW_NODE_FUNC1:
                    if (nd.a < 0) return fail(OPFLOW_E_INVALID, "node %d: missing operand", k);
                    L = loc[nd.a];
                    break;
                case OPFLOW_NODE_COND:
                    if (nd.a < 0 || nd.b < 0 || nd.c < 0 || nd.c >= k) return fail(OPFLOW_E_INVALID, "node %d: bad conditional operands", k);
                    L = loc[nd.b][0] >= 0 ? loc[nd.b] : (loc[nd.c][0] >= 0 ? loc[nd.c] : loc[nd.a]);
                    break;
                case OPFLOW_NODE_INTP_FL_CEN2COR: case OPFLOW_NODE_INTP_FL_COR2CEN:
                    return fail(OPFLOW_E_UNSUPPORTED, "flux-limiter interpolation has no StencilPad form in this engine");
                default: return fail(OPFLOW_E_UNSUPPORTED, "node %d: unknown kind", k);
            }
        }
        return OPFLOW_OK;
    }
    void push(const PInstr& in, int kind) {
        if (prog.size() >= (1u << 15)) { err = fail(OPFLOW_E_UNSUPPORTED, "equation expands beyond 32768 instructions"); return; }
        prog.push_back(in);
        kinds.push_back(kind);
    }
    void cst(double v) { push(PInstr{Q_CONST, 0, {0, 0, 0}, v}, 0); }
    void bin(int op) {
        if (err) return;
        const size_t s = prog.size(), ks = kinds.size();
        const int kb = kinds[ks - 1], ka = kinds[ks - 2];
        if (!ka && !kb && prog[s - 1].op == Q_CONST && prog[s - 2].op == Q_CONST) {
            double a = prog[s - 2].v, b = prog[s - 1].v, r = 0;
            switch (op) {
                case Q_ADD: r = a + b; break;
                case Q_SUB: r = a - b; break;
                case Q_MUL: r = a * b; break;
                case Q_DIV: r = a / b; break;
            }
            prog.pop_back();
            kinds.pop_back();
            prog.back().v = r;
            return;
        }
        if (ka && kb && op == Q_MUL) { err = fail(OPFLOW_E_UNSUPPORTED, "product of two unknown-dependent terms: the equation is not linear"); return; }
        if (kb && op == Q_DIV) { err = fail(OPFLOW_E_UNSUPPORTED, "division by an unknown-dependent term: the equation is not linear"); return; }
        // scalar / power-of-two constant is an exact multiplication (pads divide through 1./b anyway)
        if (!ka && op == Q_DIV && prog[s - 1].op == Q_CONST && is_pow2_h(prog[s - 1].v)) {
            prog[s - 1].v = 1.0 / prog[s - 1].v;
            op = Q_MUL;
        }
        PInstr in{op, 0, {0, 0, 0}, 0.};
        in.ta = ka;
        in.tb = kb;
        kinds.pop_back();
        kinds.pop_back();
        prog.push_back(in);
        kinds.push_back(ka | kb);
    }
    void dxm(int d, int o) {
        if (mesh->uniform[d]) cst(mesh->h[d]);
        else push(PInstr{Q_DX, d, {o, 0, 0}, 0.}, 0);
    }
    void xm(int d, int o) { push(PInstr{Q_X, d, {o, 0, 0}, 0.}, 0); }

    void emit(int k, const int* off) {
        if (err) return;
        const opflow_node& nd = nodes[k];
        switch (nd.kind) {
            case OPFLOW_NODE_FIELD:
                if (nd.field == unknown) {
                    uoffs.push_back({off[0], off[1], off[2]});
                    push(PInstr{Q_LOADU, nd.field, {off[0], off[1], off[2]}, 0.}, 1);
                } else {
                    auto& e = slot_extent[nd.field];
                    for (int d = 0; d < 3; ++d) { e[2 * d] = std::min(e[2 * d], off[d]); e[2 * d + 1] = std::max(e[2 * d + 1], off[d]); }
                    push(PInstr{Q_LOADS, nd.field, {off[0], off[1], off[2]}, 0.}, 0);
                }
                break;
            case OPFLOW_NODE_CONST: cst(nd.value); break;
            case OPFLOW_NODE_ADD: emit(nd.a, off); emit(nd.b, off); bin(Q_ADD); break;
            case OPFLOW_NODE_SUB: emit(nd.a, off); emit(nd.b, off); bin(Q_SUB); break;
            case OPFLOW_NODE_MUL: emit(nd.a, off); emit(nd.b, off); bin(Q_MUL); break;
            case OPFLOW_NODE_DIV: emit(nd.a, off); emit(nd.b, off); bin(Q_DIV); break;
            case OPFLOW_NODE_NEG:
                emit(nd.a, off);
                if (!kinds.back() && prog.back().op == Q_CONST) prog.back().v = -prog.back().v;
                else { PInstr in{Q_NEG, 0, {0, 0, 0}, 0.}; in.ta = kinds.back(); prog.push_back(in); }
                break;
            case OPFLOW_NODE_D2: {
                const int d = nd.dim, corner = loc[nd.a][d] == OPFLOW_CORNER, o = off[d];
                int op_[3] = {off[0], off[1], off[2]}, om[3] = {off[0], off[1], off[2]};
                op_[d]++; om[d]--;
                auto dxl = [&] { if (corner) dxm(d, o - 1); else { dxm(d, o - 1); dxm(d, o); bin(Q_ADD); cst(0.5); bin(Q_MUL); } };
                auto dxr = [&] { if (corner) dxm(d, o); else { dxm(d, o); dxm(d, o + 1); bin(Q_ADD); cst(0.5); bin(Q_MUL); } };
                emit(nd.a, op_); emit(nd.a, off); bin(Q_SUB); dxr(); bin(Q_DIV);
                emit(nd.a, off); emit(nd.a, om); bin(Q_SUB); dxl(); bin(Q_DIV);
                bin(Q_SUB);
                dxl(); dxr(); bin(Q_ADD); cst(0.5); bin(Q_MUL);
                bin(Q_DIV);
                break;
            }
            case OPFLOW_NODE_D1: {
                const int d = nd.dim, o = off[d];
                int op_[3] = {off[0], off[1], off[2]}, om[3] = {off[0], off[1], off[2]};
                op_[d]++; om[d]--;
                if (loc[nd.a][d] == OPFLOW_CENTER) {
                    emit(nd.a, off); emit(nd.a, om); bin(Q_SUB);
                    dxm(d, o - 1); dxm(d, o); bin(Q_ADD); bin(Q_DIV);
                    cst(2.0); bin(Q_MUL);
                } else {
                    emit(nd.a, op_); emit(nd.a, off); bin(Q_SUB); dxm(d, o); bin(Q_DIV);
                }
                break;
            }
            case OPFLOW_NODE_INTP_C2C: {
                const int d = nd.dim, o = off[d];
                int om[3] = {off[0], off[1], off[2]};
                om[d]--;
                auto A = [&] { xm(d, o - 1); cst(0.5); dxm(d, o - 1); bin(Q_MUL); bin(Q_ADD); xm(d, o); bin(Q_SUB); };
                auto B = [&] { xm(d, o); cst(0.5); dxm(d, o); bin(Q_MUL); bin(Q_ADD); xm(d, o); bin(Q_SUB); };
                // (a*y2 - b*y1)/(a - b): with a pad y the products are y*a (StencilPad scalar product)
                A(); emit(nd.a, off); bin(Q_MUL);
                B(); emit(nd.a, om); bin(Q_MUL);
                bin(Q_SUB);
                A(); B(); bin(Q_SUB);
                bin(Q_DIV);
                break;
            }
            case OPFLOW_NODE_INTP_COR2CEN: {
                // Math::mid(e(i), e(i + 1)) = (x1 + x2) * 0.5
                int op_[3] = {off[0], off[1], off[2]};
                op_[nd.dim]++;
                emit(nd.a, off); emit(nd.a, op_); bin(Q_ADD); cst(0.5); bin(Q_MUL);
                break;
            }
            case OPFLOW_NODE_D1_BIASED_UP: case OPFLOW_NODE_D1_BIASED_DOWN: {
                const int d = nd.dim, up = nd.kind == OPFLOW_NODE_D1_BIASED_UP, o = off[d] - (up ? 0 : 1);
                int hi[3] = {off[0], off[1], off[2]}, lo[3] = {off[0], off[1], off[2]};
                if (up) hi[d]++; else lo[d]--;
                emit(nd.a, hi); emit(nd.a, lo); bin(Q_SUB);
                if (loc[nd.a][d] == OPFLOW_CORNER) dxm(d, o);
                else { dxm(d, o); dxm(d, o + 1); bin(Q_ADD); cst(0.5); bin(Q_MUL); }
                bin(Q_DIV);
                break;
            }
            case OPFLOW_NODE_GT: case OPFLOW_NODE_GE: case OPFLOW_NODE_LT: case OPFLOW_NODE_LE: case OPFLOW_NODE_NE:
            case OPFLOW_NODE_AND: case OPFLOW_NODE_OR: case OPFLOW_NODE_FUNC2: {
                static const int ops[] = {Q_GT, Q_GE, Q_LT, Q_LE, Q_NE, Q_AND, Q_OR};
                emit(nd.a, off); emit(nd.b, off);
                scalar_op(nd.kind == OPFLOW_NODE_FUNC2 ? Q_F2 : ops[nd.kind - OPFLOW_NODE_GT], 2, nd.field);
                break;
            }
            case OPFLOW_NODE_NOT: emit(nd.a, off); scalar_op(Q_NOT, 1, 0); break;
            case OPFLOW_NODE_FUNC1: emit(nd.a, off); scalar_op(Q_F1, 1, nd.field); break;
            case OPFLOW_NODE_COND: emit(nd.a, off); emit(nd.b, off); emit(nd.c, off); scalar_op(Q_SEL, 3, 0); break;
            default: err = fail(OPFLOW_E_UNSUPPORTED, "operator without a StencilPad form");
        }
    }
    // A comparison, logic operator, conditional or per-element function of values that do not depend
    // on the unknown; applied to a StencilPad it has no linear form.
    void scalar_op(int op, int arity, int fn) {
        if (err) return;
        for (int q = 0; q < arity; ++q)
            if (kinds[kinds.size() - 1 - q]) {
                err = fail(OPFLOW_E_UNSUPPORTED, "comparison, conditional or function of the unknown: no StencilPad form");
                return;
            }
        for (int q = 0; q < arity; ++q) kinds.pop_back();
        PInstr in{op, fn, {0, 0, 0}, 0.};
        prog.push_back(in);
        kinds.push_back(0);
    }

    int run(std::vector<std::array<int, 3>>& K) {
        OPG_TRY(locs());
        if (unknown < 0 || unknown >= nleaves) return fail(OPFLOW_E_INVALID, "bad unknown slot %d", unknown);
        slot_extent.assign(nleaves, {0, 0, 0, 0, 0, 0});
        int off[3] = {0, 0, 0};
        emit(n - 1, off);
        if (err) return err;
        if (kinds.size() != 1 || !kinds[0]) return fail(OPFLOW_E_INVALID, "the equation does not depend on the unknown");
        // depths of the evaluator's two stacks (StencilPads and numbers)
        int sp = 0, psp = 0, maxsp = 0, maxpsp = 0;
        for (auto& in : prog) {
            switch (in.op) {
                case Q_LOADU: psp++; break;
                case Q_LOADS: case Q_CONST: case Q_DX: case Q_X: sp++; break;
                case Q_NEG: case Q_NOT: case Q_F1: break;
                case Q_SEL: sp -= 2; break;
                case Q_GT: case Q_GE: case Q_LT: case Q_LE: case Q_NE: case Q_AND: case Q_OR: case Q_F2: sp--; break;
                default:
                    if (in.ta && in.tb) psp--;
                    else sp--;
            }
            maxsp = std::max(maxsp, sp);
            maxpsp = std::max(maxpsp, psp);
        }
        if (psp != 1 || sp != 0) return fail(OPFLOW_E_INVALID, "malformed equation");
        if (maxpsp > PAD_STACK) return fail(OPFLOW_E_UNSUPPORTED, "equation needs %d StencilPads at once (limit %d)", maxpsp, PAD_STACK);
        if (maxsp > SCAL_STACK) return fail(OPFLOW_E_UNSUPPORTED, "equation needs a stack of %d numbers (limit %d)", maxsp, SCAL_STACK);
        // K: every offset a folded unknown leaf can land on (box hull of each loaded offset)
        std::set<std::array<int, 3>> ks;
        for (auto& o : uoffs) {
            for (int a = -std::abs(o[0]); a <= std::abs(o[0]); ++a)
                for (int b = -std::abs(o[1]); b <= std::abs(o[1]); ++b)
                    for (int c = -std::abs(o[2]); c <= std::abs(o[2]); ++c) ks.insert({a, b, c});
        }
        K.assign(ks.begin(), ks.end());
        if ((int) K.size() > PAD_KMAX) return fail(OPFLOW_E_UNSUPPORTED, "stencil of %zu entries (limit %d)", K.size(), PAD_KMAX);
        return OPFLOW_OK;
    }
};

// ================================================================================== device evaluation
struct PadVal {
    double c[PAD_KMAX];
    double b;
};

// StencilField::evalAtImpl_final, iteratively: follow the chain of mirror folds (one per out-of-range
// dim, outermost first), then apply the affine transforms innermost-first.  Returns the K index of the
// single coefficient (-1 if none) and its value / the bias.
struct FoldStep {
    int kind;  // 0 dirichlet-intp, 1 neumann, 2 symm, 3 asymm
    double x1, x2, bcv, dist;
};

__device__ bool st_leaf(const AsmParams& P, const int* cell, const int* off, int* kidx, double* coef, double* bias) {
    int idx[3] = {cell[0] + off[0], cell[1] + off[1], cell[2] + off[2]};
    FoldStep chain[3];
    int nch = 0;
    double cbias = 0.;
    bool has = true;
    for (int guard = 0; guard < 4; ++guard) {
        bool inA = true, inL = true;
        for (int d = 0; d < P.ndim; ++d) {
            inA = inA && P.st_asg[d][0] <= idx[d] && idx[d] < P.st_asg[d][1];
            inL = inL && P.st_log[d][0] <= idx[d] && idx[d] < P.st_log[d][1];
        }
        if (inA) {
            bool pinned = P.pin != 0;
            for (int d = 0; d < P.ndim; ++d) pinned = pinned && idx[d] == P.pin_index[d];
            has = !pinned;
            break;
        }
        if (!inL) return false;
        int i = -1;
        for (int d = 0; d < P.ndim && i < 0; ++d)
            if (!(P.st_acc[d][0] <= idx[d] && idx[d] < P.st_acc[d][1])) i = d;
        if (i < 0) {
            // case 2: a Dirichlet node of a corner-located field
            for (int d = 0; d < P.ndim; ++d) {
                if (P.loc[d] == OPFLOW_CORNER && P.bct[d][0] == OPFLOW_BC_DIRC && idx[d] == P.st_acc[d][0]) { cbias = P.bcv[d][0]; has = false; goto done_chain; }
                if (P.loc[d] == OPFLOW_CORNER && P.bct[d][1] == OPFLOW_BC_DIRC && idx[d] == P.st_acc[d][1] - 1) { cbias = P.bcv[d][1]; has = false; goto done_chain; }
            }
            return false;
        }
        {
            const int lower = idx[i] < P.st_acc[i][0];
            const int bct = P.bct[i][lower ? 0 : 1];
            const double bcv = P.bcv[i][lower ? 0 : 1];
            const int as = P.st_acc[i][0], ae = P.st_acc[i][1];
            const double* X = P.mx[i];
            const double* DX = P.mdx[i];
            const int es = P.es[i];
            int mi = idx[i];
            FoldStep st{};
            if (P.loc[i] == OPFLOW_CORNER) {
                mi = lower ? 2 * as - idx[i] : 2 * ae - 2 - idx[i];
                if (bct == OPFLOW_BC_DIRC) {
                    st.kind = 0;
                    st.x1 = __dsub_rn(X[(lower ? as : ae - 1) - es], X[idx[i] - es]);
                    st.x2 = __dsub_rn(X[mi - es], X[idx[i] - es]);
                    st.bcv = bcv;
                } else if (bct == OPFLOW_BC_NEUM) {
                    st.kind = 1;
                    st.bcv = bcv;
                    st.dist = __dsub_rn(X[idx[i] - es], X[mi - es]);
                } else if (bct == OPFLOW_BC_SYMM) st.kind = 2;
                else if (bct == OPFLOW_BC_ASYMM) st.kind = 3;
                else return false;
            } else {
                mi = lower ? 2 * as - 1 - idx[i] : 2 * ae - 1 - idx[i];
                if (bct == OPFLOW_BC_DIRC) {
                    const double xb = X[(lower ? as : ae) - es];
                    const double xmv = __dadd_rn(X[mi - es], __ddiv_rn(DX[mi - es], 2.));
                    const double xg = __dadd_rn(X[idx[i] - es], __ddiv_rn(DX[idx[i] - es], 2.));
                    st.kind = 0;
                    st.x1 = __dsub_rn(xb, xg);
                    st.x2 = __dsub_rn(xmv, xg);
                    st.bcv = bcv;
                } else if (bct == OPFLOW_BC_NEUM) {
                    st.kind = 1;
                    st.bcv = bcv;
                    double t = __dadd_rn(X[idx[i] - es], __ddiv_rn(DX[idx[i] - es], 2.));
                    t = __dsub_rn(t, X[mi - es]);
                    st.dist = __dsub_rn(t, __ddiv_rn(DX[mi - es], 2.));
                } else if (bct == OPFLOW_BC_SYMM) st.kind = 2;
                else if (bct == OPFLOW_BC_ASYMM) st.kind = 3;
                else return false;
            }
            if (nch >= 3) return false;
            chain[nch++] = st;
            idx[i] = mi;
        }
    }
done_chain:
    // innermost value: identity pad at idx (unless pinned / a Dirichlet node), then the transforms
    double c = has ? 1.0 : 0.0, b = cbias;
    for (int s = nch - 1; s >= 0; --s) {
        const FoldStep& st = chain[s];
        switch (st.kind) {
            case 0: {
                // (y2*x1) + ((y1*x2) * -1.0), then * (1./(x1 - x2)); y1 = bias-only pad(bcv)
                const double r = __ddiv_rn(1., __dsub_rn(st.x1, st.x2));
                c = __dmul_rn(__dmul_rn(c, st.x1), r);
                b = __dmul_rn(__dadd_rn(__dmul_rn(b, st.x1), __dmul_rn(__dmul_rn(st.bcv, st.x2), -1.0)), r);
                break;
            }
            case 1: b = __dadd_rn(b, __dmul_rn(st.bcv, st.dist)); break;  // mirror + bc_v * dist
            case 2: break;
            case 3: c = __dmul_rn(c, -1.); b = __dmul_rn(b, -1.); break;
        }
    }
    *coef = c;
    *bias = b;
    *kidx = -1;
    if (has) {
        const int o[3] = {idx[0] - cell[0], idx[1] - cell[1], idx[2] - cell[2]};
        for (int k = 0; k < P.nk; ++k)
            if (P.K[k][0] == o[0] && P.K[k][1] == o[1] && P.K[k][2] == o[2]) *kidx = k;
        if (*kidx < 0) return false;
    }
    return true;
}

// RHS_ONLY: the right-hand side alone (generateb): the same program on the pads' bias parts, which no
// coefficient ever feeds, so b is bit-identical to the full assembly's
template <bool RHS_ONLY>
__global__ void __launch_bounds__(128) assemble_kernel(const PInstr* __restrict__ prog, int nprog, AsmParams P, double* __restrict__ coef,
                                                       double* __restrict__ rhs, int* __restrict__ err) {
    const int NK = RHS_ONLY ? 0 : P.nk;
    const long long nx = P.box.hi[0] - P.box.lo[0], ny = P.box.hi[1] - P.box.lo[1], nz = P.box.hi[2] - P.box.lo[2];
    const long long total = nx * ny * nz;
    // the last divisor of a pad / num step and its reciprocal RN(1 / num): on a uniform mesh the same
    // spacing divides every difference, so the float64 division runs once per thread, not per use
    double last_div = 0., last_rec = __ddiv_rn(1., 0.);
    for (long long t = blockIdx.x * (long long) blockDim.x + threadIdx.x; t < total; t += (long long) gridDim.x * blockDim.x) {
        int cell[3];
        box_index(t, P.box, cell[0], cell[1], cell[2]);
        // two stacks: StencilPad values (operands that depend on the unknown) and plain numbers; every
        // instruction knows statically which of its operands are pads (ta, tb)
        PadVal st[PAD_STACK];
        double sv[SCAL_STACK];
        int psp = 0, sp = 0;
        bool ok = true;
        for (int p = 0; p < nprog && ok; ++p) {
            const PInstr in = prog[p];
            switch (in.op) {
                case Q_LOADS: {
                    const FieldView& f = P.leaves[in.slot];
                    const int i = cell[0] + in.off[0], j = cell[1] + in.off[1], k = cell[2] + in.off[2];
                    sv[sp++] = f.data[(i - f.off[0]) + (j - f.off[1]) * f.sy + (k - f.off[2]) * f.sz];
                    break;
                }
                case Q_LOADU: {
                    int ki;
                    double c, b;
                    ok = st_leaf(P, cell, in.off, &ki, &c, &b);
                    for (int q = 0; q < NK; ++q) st[psp].c[q] = 0.;
                    if (!RHS_ONLY && ki >= 0) st[psp].c[ki] = c;
                    st[psp].b = b;
                    psp++;
                    break;
                }
                case Q_CONST: sv[sp++] = in.v; break;
                case Q_DX: sv[sp++] = P.mdx[in.slot][cell[in.slot] + in.off[0] - P.es[in.slot]]; break;
                case Q_X: sv[sp++] = P.mx[in.slot][cell[in.slot] + in.off[0] - P.es[in.slot]]; break;
                case Q_NEG:
                    if (in.ta) {
                        for (int q = 0; q < NK; ++q) st[psp - 1].c[q] = -st[psp - 1].c[q];
                        st[psp - 1].b = -st[psp - 1].b;
                    } else sv[sp - 1] = -sv[sp - 1];
                    break;
                case Q_GT: sp--; sv[sp - 1] = sv[sp - 1] > sv[sp] ? 1. : 0.; break;
                case Q_GE: sp--; sv[sp - 1] = sv[sp - 1] >= sv[sp] ? 1. : 0.; break;
                case Q_LT: sp--; sv[sp - 1] = sv[sp - 1] < sv[sp] ? 1. : 0.; break;
                case Q_LE: sp--; sv[sp - 1] = sv[sp - 1] <= sv[sp] ? 1. : 0.; break;
                case Q_NE: sp--; sv[sp - 1] = sv[sp - 1] != sv[sp] ? 1. : 0.; break;
                case Q_AND: sp--; sv[sp - 1] = (sv[sp - 1] != 0. && sv[sp] != 0.) ? 1. : 0.; break;
                case Q_OR: sp--; sv[sp - 1] = (sv[sp - 1] != 0. || sv[sp] != 0.) ? 1. : 0.; break;
                case Q_NOT: sv[sp - 1] = sv[sp - 1] == 0. ? 1. : 0.; break;
                case Q_SEL: sp -= 2; sv[sp - 1] = sv[sp - 1] != 0. ? sv[sp] : sv[sp + 1]; break;
                case Q_F1: sv[sp - 1] = func1_eval(in.slot, sv[sp - 1]); break;
                case Q_F2: sp--; sv[sp - 1] = func2_eval(in.slot, sv[sp - 1], sv[sp]); break;
                default: {
                    if (!in.ta && !in.tb) {
                        sp--;
                        const double a = sv[sp - 1], b = sv[sp];
                        double r;
                        switch (in.op) {
                            case Q_ADD: r = __dadd_rn(a, b); break;
                            case Q_SUB: r = __dsub_rn(a, b); break;
                            case Q_MUL: r = __dmul_rn(a, b); break;
                            default: r = __ddiv_rn(a, b);
                        }
                        sv[sp - 1] = r;
                        break;
                    }
                    // pad (op) pad: A = st[psp-2], B = st[psp-1]; pad (op) num: A = st[psp-1], b = sv[sp-1];
                    // num (op) pad: a = sv[sp-1], B = st[psp-1]; the result is a pad on top of st
                    double a = 0., b = 0.;
                    if (in.ta && in.tb) psp--;
                    else if (in.ta) b = sv[--sp];
                    else a = sv[--sp];
                    PadVal& A = st[psp - 1];
                    const PadVal& B = st[psp - (in.ta && in.tb ? 0 : 1)];
                    if (in.op == Q_ADD) {
                        if (in.ta && in.tb) { for (int q = 0; q < NK; ++q) A.c[q] = __dadd_rn(A.c[q], B.c[q]); A.b = __dadd_rn(A.b, B.b); }
                        else if (in.ta) A.b = __dadd_rn(A.b, b);
                        else A.b = __dadd_rn(B.b, a);
                    } else if (in.op == Q_SUB) {
                        // pad - pad = a + (b * -1.0); pad - num = a + (-b); num - pad = StencilPad(a) + (b * -1.0)
                        if (in.ta && in.tb) { for (int q = 0; q < NK; ++q) A.c[q] = __dadd_rn(A.c[q], __dmul_rn(B.c[q], -1.0)); A.b = __dadd_rn(A.b, __dmul_rn(B.b, -1.0)); }
                        else if (in.ta) A.b = __dadd_rn(A.b, -b);
                        else { for (int q = 0; q < NK; ++q) A.c[q] = __dmul_rn(A.c[q], -1.0); A.b = __dadd_rn(a, __dmul_rn(A.b, -1.0)); }
                    } else if (in.op == Q_MUL) {
                        const double s = in.ta ? b : a;
                        for (int q = 0; q < NK; ++q) A.c[q] = __dmul_rn(A.c[q], s);
                        A.b = __dmul_rn(A.b, s);
                    } else {  // pad / num = pad * (1. / num)
                        if (__double_as_longlong(b) != __double_as_longlong(last_div)) {  // bit patterns: -0 is not +0
                            last_div = b;
                            last_rec = __ddiv_rn(1., b);
                        }
                        const double r = last_rec;
                        for (int q = 0; q < NK; ++q) A.c[q] = __dmul_rn(A.c[q], r);
                        A.b = __dmul_rn(A.b, r);
                    }
                }
            }
        }
        if (!ok) {
            atomicExch(err, 1);
            continue;
        }
        for (int q = 0; q < NK; ++q) {
            const double v = st[0].c[q];
            coef[(long long) q * total + t] = v == 0. ? 0. : v;  // +0 for -0
        }
        rhs[t] = -st[0].b;
    }
}

// ======================================================================== host structural evaluation
// Key order of the middle cell's StencilPad (fake_map insertion order): the recursion of the
// reference with only the keys tracked.
struct KeyPad {
    std::vector<std::array<int, 3>> keys;
    bool pad = false;
};
static void kmerge(KeyPad& a, const KeyPad& b) {
    for (auto& k : b.keys)
        if (std::find(a.keys.begin(), a.keys.end(), k) == a.keys.end()) a.keys.push_back(k);
    a.pad = a.pad || b.pad;
}

struct KeyEval {
    const PadCompiler& C;
    const AsmParams& P;
    KeyPad leaf(const int* idx0) const {
        int idx[3] = {idx0[0], idx0[1], idx0[2]};
        for (int guard = 0; guard < 4; ++guard) {
            bool inA = true;
            for (int d = 0; d < P.ndim; ++d) inA = inA && P.st_asg[d][0] <= idx[d] && idx[d] < P.st_asg[d][1];
            KeyPad r;
            r.pad = true;
            if (inA) {
                bool pinned = P.pin != 0;
                for (int d = 0; d < P.ndim; ++d) pinned = pinned && idx[d] == P.pin_index[d];
                if (!pinned) r.keys.push_back({idx[0], idx[1], idx[2]});
                return r;
            }
            int i = -1;
            for (int d = 0; d < P.ndim && i < 0; ++d)
                if (!(P.st_acc[d][0] <= idx[d] && idx[d] < P.st_acc[d][1])) i = d;
            if (i < 0) return r;  // Dirichlet node: bias only
            const int lower = idx[i] < P.st_acc[i][0];
            const int as = P.st_acc[i][0], ae = P.st_acc[i][1];
            if (P.loc[i] == OPFLOW_CORNER) idx[i] = lower ? 2 * as - idx[i] : 2 * ae - 2 - idx[i];
            else idx[i] = lower ? 2 * as - 1 - idx[i] : 2 * ae - 1 - idx[i];
        }
        return KeyPad{{}, true};
    }
    KeyPad ev(int k, const int* i) const {
        const opflow_node& nd = C.nodes[k];
        KeyPad r;
        auto sh = [&](int d, int o) { std::array<int, 3> j = {i[0], i[1], i[2]}; j[d] += o; return j; };
        switch (nd.kind) {
            case OPFLOW_NODE_FIELD:
                if (nd.field == C.unknown) return leaf(i);
                return r;
            case OPFLOW_NODE_CONST: return r;
            case OPFLOW_NODE_ADD: case OPFLOW_NODE_SUB: case OPFLOW_NODE_MUL: case OPFLOW_NODE_DIV: {
                KeyPad a = ev(nd.a, i), b = ev(nd.b, i);
                if (!a.pad) return b;
                kmerge(a, b);
                return a;
            }
            case OPFLOW_NODE_NEG: return ev(nd.a, i);
            case OPFLOW_NODE_D2: {
                auto jp = sh(nd.dim, 1), jm = sh(nd.dim, -1);
                KeyPad l = ev(nd.a, jm.data()), c = ev(nd.a, i), rr = ev(nd.a, jp.data());
                KeyPad t1 = rr; kmerge(t1, c);
                KeyPad t2 = c; kmerge(t2, l);
                kmerge(t1, t2);
                return t1;
            }
            case OPFLOW_NODE_D1: {
                auto jp = sh(nd.dim, 1), jm = sh(nd.dim, -1);
                if (C.loc[nd.a][nd.dim] == OPFLOW_CENTER) { KeyPad a = ev(nd.a, i), b = ev(nd.a, jm.data()); kmerge(a, b); return a; }
                KeyPad a = ev(nd.a, jp.data()), b = ev(nd.a, i);
                kmerge(a, b);
                return a;
            }
            case OPFLOW_NODE_INTP_C2C: {
                auto jm = sh(nd.dim, -1);
                KeyPad y2 = ev(nd.a, i), y1 = ev(nd.a, jm.data());
                if (!y2.pad) return y1;
                kmerge(y2, y1);
                return y2;
            }
            case OPFLOW_NODE_GT: case OPFLOW_NODE_GE: case OPFLOW_NODE_LT: case OPFLOW_NODE_LE: case OPFLOW_NODE_NE:
            case OPFLOW_NODE_AND: case OPFLOW_NODE_OR: case OPFLOW_NODE_NOT: case OPFLOW_NODE_COND:
            case OPFLOW_NODE_FUNC1: case OPFLOW_NODE_FUNC2:
                return r;  // scalar-valued (the compiler refuses them on the unknown)
            case OPFLOW_NODE_INTP_COR2CEN: {
                auto jp = sh(nd.dim, 1);
                KeyPad a = ev(nd.a, i), b = ev(nd.a, jp.data());
                if (!a.pad) return b;
                kmerge(a, b);
                return a;
            }
            case OPFLOW_NODE_D1_BIASED_UP: case OPFLOW_NODE_D1_BIASED_DOWN: {
                const bool up = nd.kind == OPFLOW_NODE_D1_BIASED_UP;
                auto j = sh(nd.dim, up ? 1 : -1);
                KeyPad a = up ? ev(nd.a, j.data()) : ev(nd.a, i), b = up ? ev(nd.a, i) : ev(nd.a, j.data());
                if (!a.pad) return b;
                kmerge(a, b);
                return a;
            }
        }
        return r;
    }
};

// ================================================================================== public helpers
int asm_prepare(opflow_ctx ctx, opflow_field target, const opflow_node* nodes, int n, const opflow_field* leaves, int nleaves, int unknown,
                int pin, AsmPlan* plan, opflow_field rows) {
    if (!ctx || !target || !nodes || n < 1 || nleaves < 1 || nleaves > 8) return fail(OPFLOW_E_INVALID, "bad assembly arguments (1..8 leaves)");
    for (int s = 0; s < nleaves; ++s) {
        if (!leaves[s]) return fail(OPFLOW_E_INVALID, "null leaf %d", s);
        if (!mesh_equal(leaves[s]->mesh, target->mesh)) return fail(OPFLOW_E_INVALID, "leaf %d lives on another mesh", s);
    }
    if (unknown < 0 || unknown >= nleaves || leaves[unknown] != target)
        return fail(OPFLOW_E_INVALID, "leaf slot %d must be the target field (the StencilField's base)", unknown);
    PadCompiler C{nodes, n, leaves, nleaves, unknown, target->mesh};
    std::vector<std::array<int, 3>> K;
    OPG_TRY(C.run(K));
    AsmParams& P = plan->P;
    std::memset(&P, 0, sizeof P);
    const opflow_field_info& R = target->info;
    P.ndim = R.ndim;
    P.pin = pin;
    for (int d = 0; d < 3; ++d) {
        for (int s = 0; s < 2; ++s) {
            P.st_asg[d][s] = R.assignable[d][s];
            P.st_acc[d][s] = R.accessible[d][s];
            P.st_log[d][s] = R.logical[d][s];
            P.bct[d][s] = target->desc.bc_type[d][s];
            P.bcv[d][s] = target->desc.bc_value[d][s];
        }
        P.loc[d] = target->desc.loc[d];
        P.pin_index[d] = R.assignable[d][0];
        // ignorePeriodicBC (StencilField.hpp:112-121)
        if (d < R.ndim && target->desc.bc_type[d][0] == OPFLOW_BC_PERIODIC)
            for (int s = 0; s < 2; ++s) P.st_asg[d][s] = P.st_acc[d][s] = R.logical[d][s];
        P.mx[d] = target->mesh->x[d];
        P.mdx[d] = target->mesh->dx[d];
        P.es[d] = target->mesh->es[d];
    }
    P.box = assign_box(rows ? rows->info : R);
    if (rows && (rows->info.ndim != R.ndim || !mesh_equal(rows->mesh, target->mesh))) return fail(OPFLOW_E_INVALID, "row field on another mesh");
    P.nk = (int) K.size();
    for (int k = 0; k < P.nk; ++k)
        for (int d = 0; d < 3; ++d) P.K[k][d] = K[k][d];
    for (int s = 0; s < nleaves; ++s) P.leaves[s] = leaves[s]->view();
    // every known-field read must stay in its data array; unknown reads must stay in the logical range
    for (int s = 0; s < nleaves; ++s) {
        if (s == unknown) continue;
        const auto& e = C.slot_extent[s];
        const opflow_field_info& r = leaves[s]->info;
        for (int d = 0; d < R.ndim; ++d) {
            const int lo = P.box.lo[d] + e[2 * d], hi = P.box.hi[d] - 1 + e[2 * d + 1];
            if (lo < r.data_offset[d] || hi >= r.data_offset[d] + r.data_dims[d])
                return fail(OPFLOW_E_RANGE, "equation reads leaf %d outside its data along dim %d", s, d);
        }
    }
    for (auto& in : C.prog) {
        if (in.op != Q_DX && in.op != Q_X) continue;
        const int d = in.slot;
        const int lo = P.box.lo[d] + in.off[0], hi = P.box.hi[d] - 1 + in.off[0];
        const int nn = target->mesh->n[d] - (in.op == Q_DX ? 1 : 0);
        if (lo < target->mesh->es[d] || hi >= target->mesh->es[d] + nn) return fail(OPFLOW_E_RANGE, "mesh read outside the extended mesh");
    }
    for (auto& o : C.uoffs)
        for (int d = 0; d < R.ndim; ++d) {
            const int lo = P.box.lo[d] + o[d], hi = P.box.hi[d] - 1 + o[d];
            if (lo < P.st_log[d][0] || hi >= P.st_log[d][1]) return fail(OPFLOW_E_RANGE, "unknown read outside its logical range along dim %d", d);
        }
    plan->prog = C.prog;
    // middle cell's key order (HYPREEqnSolveHandler.hpp:97-107)
    int mid[3] = {0, 0, 0};
    for (int d = 0; d < R.ndim; ++d) mid[d] = (R.assignable[d][0] + R.assignable[d][1]) / 2;
    KeyEval KE{C, P};
    KeyPad kp = KE.ev(n - 1, mid);
    plan->comm.clear();
    for (auto& k : kp.keys) plan->comm.push_back({k[0] - mid[0], k[1] - mid[1], k[2] - mid[2]});
    plan->cells = P.box.count();
    return OPFLOW_OK;
}

int asm_run(opflow_ctx ctx, AsmPlan* plan, double* coef, double* rhs) {
    if (!coef && !rhs) return fail(OPFLOW_E_INVALID, "assembly: no output");
    const long long N = plan->cells;
    if (N <= 0) return OPFLOW_OK;
    OPG_TRY(ensure_scratch(ctx, 64));
    PInstr* dprog = (PInstr*) dev_alloc(ctx, plan->prog.size() * sizeof(PInstr));
    if (!dprog) return fail(OPFLOW_E_NOMEM, "assembly program");
    int* err = (int*) ctx->scratch;
    cudaMemsetAsync(err, 0, sizeof(int), ctx->stream);
    cudaMemcpyAsync(dprog, plan->prog.data(), plan->prog.size() * sizeof(PInstr), cudaMemcpyHostToDevice, ctx->stream);
    long long blocks = (N + 127) / 128;
    if (blocks > (long long) ctx->num_sms * 32) blocks = (long long) ctx->num_sms * 32;
    if (coef) assemble_kernel<false><<<(int) blocks, 128, 0, ctx->stream>>>(dprog, (int) plan->prog.size(), plan->P, coef, rhs, err);
    else assemble_kernel<true><<<(int) blocks, 128, 0, ctx->stream>>>(dprog, (int) plan->prog.size(), plan->P, coef, rhs, err);
    OPG_LAUNCHED();
    int rc = check_launch("assemble_kernel");
    int herr = 0;
    cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream);
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    dev_free(ctx, dprog);
    if (rc) return rc;
    if (e != cudaSuccess) return fail(OPFLOW_E_CUDA, "assembly failed: %s", cudaGetErrorString(e));
    if (herr) return fail(OPFLOW_E_RANGE, "a folded unknown leaf left the stencil offset set or the logical range");
    return OPFLOW_OK;
}

}  // namespace opg

using namespace opg;

extern "C" int opflow_assemble(opflow_ctx ctx, opflow_field target, const opflow_node* nodes, int n_nodes, const opflow_field* leaves,
                               int n_leaves, int unknown_slot, int pin, int* n_entries, int* offsets_out, double* coef_out,
                               double* rhs_out, size_t* n_cells) {
    AsmPlan plan;
    OPG_TRY(asm_prepare(ctx, target, nodes, n_nodes, leaves, n_leaves, unknown_slot, pin, &plan));
    const int ne = (int) plan.comm.size();
    const int D = target->info.ndim;
    if (n_entries) *n_entries = ne;
    if (n_cells) *n_cells = (size_t) plan.cells;
    if (!coef_out && !rhs_out && !offsets_out) return OPFLOW_OK;
    if (offsets_out)
        for (int e = 0; e < ne; ++e)
            for (int d = 0; d < D; ++d) offsets_out[e * D + d] = plan.comm[e][d];
    const long long N = plan.cells;
    const int nk = plan.P.nk;
    double *dc = nullptr, *dr = nullptr;
    if (cudaMalloc(&dc, (size_t) N * nk * sizeof(double)) != cudaSuccess || cudaMalloc(&dr, (size_t) N * sizeof(double)) != cudaSuccess) {
        if (dc) cudaFree(dc);
        return fail(OPFLOW_E_NOMEM, "assembly buffers");
    }
    int rc = asm_run(ctx, &plan, dc, dr);
    std::vector<double> hc, hr;
    if (rc == OPFLOW_OK) {
        hc.resize((size_t) N * nk);
        hr.resize(N);
        cudaMemcpy(hc.data(), dc, hc.size() * sizeof(double), cudaMemcpyDeviceToHost);
        cudaMemcpy(hr.data(), dr, hr.size() * sizeof(double), cudaMemcpyDeviceToHost);
    }
    cudaFree(dc);
    cudaFree(dr);
    if (rc) return rc;
    // comm entry -> K index
    std::vector<int> map(ne, -1);
    for (int e = 0; e < ne; ++e)
        for (int k = 0; k < nk; ++k)
            if (plan.P.K[k][0] == plan.comm[e][0] && plan.P.K[k][1] == plan.comm[e][1] && plan.P.K[k][2] == plan.comm[e][2]) map[e] = k;
    for (long long c = 0; c < N; ++c) {
        if (coef_out)
            for (int e = 0; e < ne; ++e) coef_out[c * ne + e] = map[e] >= 0 ? hc[(size_t) map[e] * N + c] : 0.;
        if (rhs_out) rhs_out[c] = hr[c];
    }
    if (pin && N > 0) {
        // the first unknown's row becomes the identity with rhs 0 (HYPREEqnSolveHandler.hpp:145-163)
        for (int e = 0; e < ne; ++e) {
            bool centre = plan.comm[e][0] == 0 && plan.comm[e][1] == 0 && plan.comm[e][2] == 0;
            if (coef_out) coef_out[e] = centre ? 1.0 : 0.0;
        }
        if (rhs_out) rhs_out[0] = 0.;
    }
    return OPFLOW_OK;
}
