// StencilPad-program assembly shared by opflow_assemble and the solvers.
#pragma once
#include "internal.h"

namespace opg {

enum QOp : int {
    Q_LOADS = 0, Q_LOADU, Q_CONST, Q_ADD, Q_SUB, Q_MUL, Q_DIV, Q_NEG, Q_DX, Q_X,
    // scalar-only operators (no operand depends on the unknown)
    Q_GT, Q_GE, Q_LT, Q_LE, Q_NE, Q_AND, Q_OR, Q_NOT, Q_SEL, Q_F1, Q_F2
};
struct PInstr {
    int op;
    int slot;     // Q_LOADS/Q_LOADU: leaf slot; Q_DX/Q_X: dim; Q_F1/Q_F2: function
    int off[3];   // load offset; Q_DX/Q_X: off[0]
    double v;     // Q_CONST
    int ta = 0, tb = 0;  // operand kinds (0 scalar, 1 pad) for arithmetic
};

constexpr int PAD_KMAX = 9;   // stencil entries a pad may hold (up to 3x3 in 2D / 7 in 3D)
constexpr int PAD_STACK = 8;    // StencilPad values live at once during an evaluation
constexpr int SCAL_STACK = 24;  // plain numbers live at once

struct AsmParams {
    int ndim;
    Box box;                    // cells evaluated: commonRange(assignable, local)
    int st_asg[3][2], st_acc[3][2], st_log[3][2];  // StencilField ranges after ignorePeriodicBC
    int loc[3];
    int bct[3][2];
    double bcv[3][2];
    int pin, pin_index[3];
    const double* mx[3];
    const double* mdx[3];
    int es[3];
    int nk;
    int K[PAD_KMAX][3];
    FieldView leaves[8];
};

struct AsmPlan {
    AsmParams P;
    std::vector<PInstr> prog;
    std::vector<std::array<int, 3>> comm;  // middle cell's stencil keys, offset form, insertion order
    long long cells = 0;
};

// `rows`: the field whose assignable cells are the equations' rows when they are not the unknown's own
// (a coupled system's off-diagonal block); the unknown's StencilField rules still come from `target`.
int asm_prepare(opflow_ctx ctx, opflow_field target, const opflow_node* nodes, int n, const opflow_field* leaves, int nleaves, int unknown,
                int pin, AsmPlan* plan, opflow_field rows = nullptr);
// coef: [nk][cells] (SoA over the plan's K order), rhs: [cells] = -bias
// coef == nullptr: the right-hand side alone (generateb), bit-identical to the full assembly's
int asm_run(opflow_ctx ctx, AsmPlan* plan, double* coef, double* rhs);

}  // namespace opg
