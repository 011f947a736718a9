/* opflow_gpu.h -- C ABI of the GB300 engine for OpFlow's two data-parallel paths on structured
 * Cartesian grids:
 *   (E) explicit evaluation of a stencil expression into a field  (`u = u + dt*a*(d2x(u)+d2y(u))`),
 *   (I) implicit solve of a stencil-generated linear equation      (`Solve(f, p, PCG, PFMG)`).
 *
 * OpFlow itself is a header-only C++ template library with no FFI; the entry points below are what a
 * C++ adapter (include/opflow_gb300/OpFlowGPU.hpp) or any FFI (ctypes, cgo, JNI) binds in place of
 * the reference's template machinery.  Each declaration names the reference interface it replaces
 * (paths relative to the OpFlow source tree).
 *
 * Conventions
 *   - Every call returns an int status (OPFLOW_OK == 0).  The library never aborts; the message of the
 *     last failure on the calling thread is returned by opflow_last_error().
 *   - No torch or CUDA types appear in signatures: handles are opaque pointers, buffers are plain
 *     pointers with element counts.  CUDA streams are passed as void*.
 *   - Field data layout is the reference's PlainTensor layout (src/DataStructures/Arrays/Tensor/
 *     PlainTensor.hpp:204-213): x fastest, over the padded local range
 *     localRange.getInnerRange(-padding), float64.
 */
#ifndef OPFLOW_GPU_H
#define OPFLOW_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define OPFLOW_GPU_ABI_VERSION 3

/* ---- status codes ---------------------------------------------------------------------------- */
enum opflow_status {
    OPFLOW_OK = 0,
    OPFLOW_E_INVALID = 1,       /* bad argument / inconsistent description (reference: OP_ABORT)      */
    OPFLOW_E_NOMEM = 2,         /* device allocation or HBM admission budget exhausted               */
    OPFLOW_E_CUDA = 3,          /* a CUDA runtime call failed                                        */
    OPFLOW_E_TIMEOUT = 4,       /* a bounded device-side wait expired                                */
    OPFLOW_E_NOT_CONVERGED = 5, /* maxIter reached before the tolerance                              */
    OPFLOW_E_UNSUPPORTED = 6,   /* expression / stencil shape outside what the engine lowers         */
    OPFLOW_E_RANGE = 7,         /* a stencil read would leave the field's readable range             */
    OPFLOW_E_NAN = 8            /* non-finite input (e.g. NaN in a right-hand side)                  */
};

/* Reference enums: LocOnMesh (src/Core/Field/MeshBased/StructuredFieldExpr*), BCType (src/Core/BC/BCBase.hpp) */
enum opflow_loc { OPFLOW_CORNER = 0, OPFLOW_CENTER = 1 };
enum opflow_bc {
    OPFLOW_BC_UNDEFINED = 0,
    OPFLOW_BC_DIRC = 1,
    OPFLOW_BC_NEUM = 2,
    OPFLOW_BC_PERIODIC = 3,
    OPFLOW_BC_SYMM = 4,
    OPFLOW_BC_ASYMM = 5
};

/* BasicArithOp of FieldAssigner::assign<Op> (src/Core/Loops/FieldAssigner.hpp:26-84) */
enum opflow_arith { OPFLOW_ASSIGN_EQ = 0, OPFLOW_ASSIGN_ADD = 1, OPFLOW_ASSIGN_SUB = 2, OPFLOW_ASSIGN_MUL = 3, OPFLOW_ASSIGN_DIV = 4 };

typedef struct opflow_ctx_s* opflow_ctx;
typedef struct opflow_field_s* opflow_field;
typedef struct opflow_solver_s* opflow_solver;
typedef struct opflow_batch_s* opflow_batch;
typedef struct opflow_server_s* opflow_server;
typedef struct opflow_eqnset_s* opflow_eqnset;

/* ---- context --------------------------------------------------------------------------------- */
/* Replaces EnvironmentGardian / the global ParallelPlan (src/Core/Environment.hpp:41-62): one context
 * per device, owning one CUDA stream. */
int opflow_ctx_create(int device, opflow_ctx* out);
int opflow_ctx_destroy(opflow_ctx ctx);
int opflow_ctx_set_stream(opflow_ctx ctx, void* cuda_stream);
int opflow_ctx_get_stream(opflow_ctx ctx, void** cuda_stream);
int opflow_ctx_synchronize(opflow_ctx ctx);
/* Message of the last failed call on this thread ("" if none). */
const char* opflow_last_error(void);
/* Number of kernels this library has launched in this process (for launch accounting). */
int opflow_kernel_launch_count(uint64_t* out);
int opflow_abi_version(void);

/* ---- mesh + field ---------------------------------------------------------------------------- */
/* Replaces MeshBuilder<CartesianMesh<Dim>> (src/Core/Mesh/Structured/CartesianMesh.hpp:122-305) and
 * ExprBuilder<CartesianField> (src/Core/Field/MeshBased/Structured/CartesianField.hpp:796-1033).
 * The mesh is given by its node coordinates over the extended range
 * [start-pad_width, start+dims+pad_width) per dimension (what MeshBuilder::build produces);
 * opflow_mesh_uniform() fills that from setMeshOfDim(d, min, max). */
typedef struct {
    int ndim;
    int dims[3];      /* nodes per dimension                                        */
    int start[3];     /* first node index (MeshBuilder::setStart, default 0)        */
    int pad_width;    /* mesh ghost extension (MeshBuilder padding_width, default 5) */
    const double* x[3];  /* dims[d] + 2*pad_width node coordinates (CartesianMesh::_x)  */
    const double* dx[3]; /* dims[d] + 2*pad_width - 1 spacings (CartesianMesh::_dx)      */
} opflow_mesh_desc;

typedef struct {
    int ndim;
    int loc[3];             /* enum opflow_loc                                       */
    int bc_type[3][2];      /* [dim][start/end], enum opflow_bc                      */
    double bc_value[3][2];  /* constant Dirichlet value / Neumann gradient           */
    int ext[3][2];          /* ExprBuilder::setExt widths                           */
    int padding;            /* ExprBuilder::setPadding (final padding = max(padding, ext)) */
} opflow_field_desc;

typedef struct {
    int ndim;
    int padding;
    int data_dims[3];        /* extents of the data array (padded local range)          */
    int data_offset[3];      /* index of data element 0 (CartesianField::offset)        */
    int logical[3][2], accessible[3][2], assignable[3][2], local[3][2];
    size_t count;            /* data_dims product                                       */
} opflow_field_info;

/* Node coordinates and spacings of MeshBuilder::set1DMesh(min, max) including its Symm ghost extension
 * (CartesianMesh.hpp:209-303).  x_out holds dims + 2*pad_width values, dx_out one fewer. */
int opflow_mesh_uniform(int dims, int start, int pad_width, double min, double max, double* x_out, double* dx_out);

/* The ranges and data extents ExprBuilder<CartesianField>::calculateRanges / validateRanges compute
 * (CartesianField.hpp:941-1029), without allocating anything (no GPU needed). */
int opflow_field_describe(const opflow_mesh_desc* mesh, const opflow_field_desc* desc, opflow_field_info* out);

/* ExprBuilder<CartesianField>::build (CartesianField.hpp:929-1029): computes the ranges, allocates the
 * device data array (zero-filled) and applies updatePadding. */
int opflow_field_create(opflow_ctx ctx, const opflow_mesh_desc* mesh, const opflow_field_desc* desc, opflow_field* out);
int opflow_field_destroy(opflow_field f);
int opflow_field_get_info(opflow_field f, opflow_field_info* out);
/* Full data array (layout above); count must equal info.count.  Upload is followed by nothing: call
 * opflow_field_update_padding if the host data's padding is stale. */
int opflow_field_upload(opflow_field f, const double* host, size_t count);
int opflow_field_download(opflow_field f, double* host, size_t count);
/* Device pointer of the current data array (it alternates between two buffers across aliased
 * assignments, so re-query after each assign). */
int opflow_field_device_ptr(opflow_field f, double** dptr);
/* CartesianField::updatePaddingImpl_final (CartesianField.hpp:349-629), single-rank branch. */
int opflow_field_update_padding(opflow_field f);
/* Field snapshots in OpFlow's raw binary format: Utils::RawBinaryOStream << field
 * (src/Utils/Writers/RawBinaryStream.hpp:97-150) writes <dir>/<name>_<count>.cart with the time stamp,
 * the mesh range and coordinates, the field's accessible and local ranges and the local-range values;
 * RawBinaryIStream >> field (RawBinaryStream.hpp:152-224) reads one back after checking the mesh and
 * ranges against the field's, then updates the padding.  The streams' counters live in the caller. */
int opflow_field_write_raw(opflow_field f, const char* dir, const char* name, int count, double time);
int opflow_field_read_raw(opflow_field f, const char* dir, const char* name, int count, double* time_out);
/* `f = c` for a constant (CartesianField::assignImpl_final(const D&), CartesianField.hpp:236-280). */
int opflow_field_fill(opflow_field f, int arith, double c);
/* `dst = src` between two fields of identical shape (data copy, then padding). */
int opflow_field_copy(opflow_field dst, opflow_field src);

/* ---- expressions (path E) ---------------------------------------------------------------------- */
/* One node of an expression tree, children before parents; the root is the last node.
 * Mirrors Expression<Op, Args...> (src/Core/Expr/Expression.hpp) with the operators of
 * src/Core/Operator/{Arithmetic/AMDS.hpp, FDMOperators, Interpolator/D1Linear.hpp}. */
enum opflow_node_kind {
    OPFLOW_NODE_FIELD = 1,      /* leaf: field slot `field`                                        */
    OPFLOW_NODE_CONST = 2,      /* ScalarExpr<double> `value`                                     */
    OPFLOW_NODE_ADD = 3,        /* AddOp                                                          */
    OPFLOW_NODE_SUB = 4,        /* SubOp                                                          */
    OPFLOW_NODE_MUL = 5,        /* MulOp                                                          */
    OPFLOW_NODE_DIV = 6,        /* DivOp                                                          */
    OPFLOW_NODE_NEG = 7,        /* unary minus                                                    */
    OPFLOW_NODE_D2 = 8,         /* D2SecondOrderCentered<dim>   (D2SecondOrderCentered.hpp:160-171) */
    OPFLOW_NODE_D1 = 9,         /* D1FirstOrderCentered<dim>    (D1FirstOrderCentered.hpp:31-36)    */
    OPFLOW_NODE_WENO53_DOWN = 10,/* D1WENO53Downwind<dim>       (D1WENO53Downwind.hpp:136-154)      */
    OPFLOW_NODE_WENO53_UP = 11, /* D1WENO53Upwind<dim>          (D1WENO53Upwind.hpp:133-151)        */
    OPFLOW_NODE_INTP_C2C = 12,  /* D1Linear Cen2Cor, d1IntpCenterToCorner<dim> (D1Linear.hpp:35-45) */
    OPFLOW_NODE_INTP_COR2CEN = 13,/* D1Linear Cor2Cen, d1IntpCornerToCenter<dim> (D1Linear.hpp:43-45) */
    OPFLOW_NODE_D1_BIASED_UP = 14,  /* D1FirstOrderBiasedUpwind<dim>   (D1FirstOrderBiasedUpwind.hpp:53-58)   */
    OPFLOW_NODE_D1_BIASED_DOWN = 15,/* D1FirstOrderBiasedDownwind<dim> (D1FirstOrderBiasedDownwind.hpp:52-57) */
    /* comparisons (Logical/Compare.hpp:27-31): 1.0 when true, 0.0 when false */
    OPFLOW_NODE_GT = 16,        /* a > b   GreaterThan                                             */
    OPFLOW_NODE_GE = 17,        /* a >= b  GreaterThanOrEqual                                      */
    OPFLOW_NODE_LT = 18,        /* a < b   LessThan                                                */
    OPFLOW_NODE_LE = 19,        /* a <= b  LessThanOrEqual                                         */
    OPFLOW_NODE_NE = 20,        /* a != b  NotEqualTo                                              */
    /* logic (Logical/Boolean.hpp:24-26): operands are true when non-zero                           */
    OPFLOW_NODE_AND = 21,       /* a && b                                                          */
    OPFLOW_NODE_OR = 22,        /* a || b                                                          */
    OPFLOW_NODE_NOT = 23,       /* !a                                                              */
    OPFLOW_NODE_COND = 24,      /* conditional(a, b, c): a ? b : c   (Conditional.hpp:22-40)       */
    OPFLOW_NODE_FUNC1 = 25,     /* per-element function `field` (enum opflow_func1) of a (AMDS.hpp:54-91) */
    OPFLOW_NODE_FUNC2 = 26,     /* per-element function `field` (enum opflow_func2) of a, b (AMDS.hpp:39-50, MinMax.hpp) */
    OPFLOW_NODE_INTP_FL_CEN2COR = 27, /* d1Intp<D1FluxLimiterGen<K>::Op, dim, Cen2Cor>(a, b): b interpolated
                                         to faces, upwinded by the sign of a (D1FluxLimiter.hpp:36-133, 136-166);
                                         `field` is the limiter K (enum opflow_flux_limiter) */
    OPFLOW_NODE_INTP_FL_COR2CEN = 28  /* the same, corners to centres (D1FluxLimiter.hpp:61-150, 168-201) */
};

/* Per-element functions of OPFLOW_NODE_FUNC1 (std:: functions of the same name).  ABS .. RINT are
 * exact in IEEE arithmetic and bit-identical to the reference; the others are CUDA's double-precision
 * math functions (a few ulp from the host C library's). */
enum opflow_func1 {
    OPFLOW_F_ABS = 0, OPFLOW_F_SQRT, OPFLOW_F_CEIL, OPFLOW_F_FLOOR, OPFLOW_F_TRUNC, OPFLOW_F_ROUND, OPFLOW_F_RINT,
    OPFLOW_F_EXP = 16, OPFLOW_F_EXP2, OPFLOW_F_EXPM1, OPFLOW_F_LOG, OPFLOW_F_LOG10, OPFLOW_F_LOG2, OPFLOW_F_LOG1P,
    OPFLOW_F_CBRT, OPFLOW_F_SIN, OPFLOW_F_COS, OPFLOW_F_TAN, OPFLOW_F_ASIN, OPFLOW_F_ACOS, OPFLOW_F_ATAN,
    OPFLOW_F_SINH, OPFLOW_F_COSH, OPFLOW_F_TANH, OPFLOW_F_ASINH, OPFLOW_F_ACOSH, OPFLOW_F_ATANH, OPFLOW_F_ERF,
    OPFLOW_F_ERFC, OPFLOW_F_TGAMMA, OPFLOW_F_LGAMMA
};
/* Per-element functions of OPFLOW_NODE_FUNC2.  MAX, MIN (std::max / std::min: a < b ? b : a and
 * b < a ? b : a), FDIM, COPYSIGN, FMOD and REMAINDER are exact; POW, HYPOT and ATAN2 are CUDA's. */
enum opflow_func2 {
    OPFLOW_F2_MAX = 0, OPFLOW_F2_MIN, OPFLOW_F2_FDIM, OPFLOW_F2_COPYSIGN, OPFLOW_F2_FMOD, OPFLOW_F2_REMAINDER,
    OPFLOW_F2_POW = 16, OPFLOW_F2_HYPOT, OPFLOW_F2_ATAN2
};
/* Flux limiters K of OPFLOW_NODE_INTP_FL_* (Interpolator/FluxLimiterKernels.hpp, the aliases of
 * D1FluxLimiterBasedIntpOp.hpp).  The kappa schemes are the linear kernels K(slope_u, slope_f). */
enum opflow_flux_limiter {
    OPFLOW_FL_CDS = 0,      /* D1Central:      KappaKernel<CDS>,   kappa = 1     */
    OPFLOW_FL_QUICK = 1,    /* D1QUICK:        KappaKernel<QUICK>, kappa = 1/2   */
    OPFLOW_FL_CUI = 2,      /* D1CUI:          KappaKernel<CUI>,   kappa = 1/3   */
    OPFLOW_FL_FROMM = 3,    /* D1Fromm:        KappaKernel<Fromm>, kappa = 0     */
    OPFLOW_FL_LUI = 4,      /* D1LinearUpwind: KappaKernel<LUI>,   kappa = -1    */
    OPFLOW_FL_MINMOD = 5,   /* D1Minmod                                          */
    OPFLOW_FL_SUPERBEE = 6, /* D1Superbee                                        */
    OPFLOW_FL_MUSCL = 7,    /* D1MUSCL                                           */
    OPFLOW_FL_HARMONIC = 8, /* D1Harmonic                                        */
    OPFLOW_FL_VANALBADA = 9,/* D1Albada                                          */
    OPFLOW_FL_UMIST = 10,   /* SPLMinKernel<2, 1/2>                              */
    OPFLOW_FL_SPL13 = 11,   /* SPLMinKernel<2, 1/3>                              */
    OPFLOW_FL_SPLMAX12 = 12,/* SPLMaxKernel<2, 1/2>                              */
    OPFLOW_FL_SPLMAX13 = 13,/* SPLMaxKernel<2, 1/3>                              */
    OPFLOW_FL_KOREN = 14,   /* GPLKappaKernel<2, 0, 1/3> (Koren's limited CUI)   */
    OPFLOW_FL_SMART = 15,   /* GPLKappaKernel<4, 0, 1/2>                         */
    OPFLOW_FL_BSOU = 16     /* GPLKappaKernel<1, 0, -1>                          */
};

typedef struct {
    int kind;     /* enum opflow_node_kind                                                     */
    int a, b;     /* child node indices, -1 if unused                                          */
    int dim;      /* operator direction                                                        */
    int field;    /* leaf slot for OPFLOW_NODE_FIELD; function for FUNC1/FUNC2; limiter for INTP_FL_* */
    double value; /* constant for OPFLOW_NODE_CONST                                            */
    int c;        /* third child (OPFLOW_NODE_COND's false branch), -1 if unused               */
} opflow_node;

/* Evaluation modes of the explicit path. */
enum opflow_eval_mode {
    OPFLOW_EVAL_EXACT = 0, /* IEEE float64 in the reference's operation order: bit-identical results */
    OPFLOW_EVAL_FAST = 1   /* linear constant-coefficient stencils in exact 64-bit fixed point with one
                              rounding per point (normwise relative error <= 1e-14 per 1000 steps);
                              falls back to EXACT for anything else                                 */
};

/* `dst <op>= expr` for a Cartesian field: replaces internal::FieldAssigner::assign<Op>
 * (src/Core/Loops/FieldAssigner.hpp:27-36) reached from Expr::operator= / += / -= / *= / /=
 * (src/Core/Expr/Expr.hpp:53-81) through CartesianField::assignImpl_final (CartesianField.hpp:195-234).
 * Evaluates over commonRange(dst.assignableRange, dst.localRange) and then updates dst's padding.
 * An expression that reads dst itself is evaluated out of place, as the reference does. */
int opflow_assign(opflow_ctx ctx, opflow_field dst, int arith, const opflow_node* nodes, int n_nodes,
                  const opflow_field* leaves, int n_leaves, int mode);
/* Many explicit assignments in one launch, each `dsts[i] <arith[i]>= expr_i` over its own field and
 * grid (sizes may differ), `steps` times: a persistent grid takes tiles of every assignment's box from
 * one work queue.  Each expression is evaluated in exact mode (the FTCS update where it has that
 * shape, else the interpreter), so the values equal
 * opflow_assign_repeat's in OPFLOW_EVAL_EXACT mode, step for step.  The destinations must differ and no
 * assignment may read another one's destination (they run concurrently); an assignment may read its own
 * destination (u = u + ...), as in opflow_assign.  No counterpart in the reference, which evaluates one
 * field per FieldAssigner::assign call. */
int opflow_assign_batch(opflow_ctx ctx, int n, const opflow_field* dsts, const int* arith, const opflow_node* const* nodes, const int* n_nodes,
                        const opflow_field* const* leaves, const int* n_leaves, int steps);

/* Runs `steps` repetitions of the same assignment (one fused kernel per step where the expression has
 * a specialised kernel).  In OPFLOW_EVAL_FAST mode, steps >= 2 of u = u + sum_d w_d (u(i-e_d) + u(i+e_d)
 * - 2u) on a 2D or 3D node grid with Dirichlet sides and no ghost layer, with w_d >= 0 and
 * 1 - 2 sum_d w_d >= 0, keep the field in 64-bit fixed point between the steps (one scale for the run;
 * float64 again after the last step), within 1e-14 of the EXACT run.  OPFLOW_FX_RESIDENT=0 in the
 * environment turns that off. */
int opflow_assign_repeat(opflow_ctx ctx, opflow_field dst, int arith, const opflow_node* nodes, int n_nodes,
                         const opflow_field* leaves, int n_leaves, int mode, int steps);

/* Shu-Osher RK3 step of u_t + L(u) = 0 with L = dt * d1<WENO53 kind, dim>(.), the three stages
 *   u1 = u - dt*L(u);  u2 = 0.75*u + 0.25*(u1 - dt*L(u1));  u = 1/3*u + 2/3*(u2 - dt*L(u2))
 * fused into one pass (stages in shared memory), bit-identical to three reference assignments.
 * `kind` is OPFLOW_NODE_WENO53_DOWN or OPFLOW_NODE_WENO53_UP.  u1 and u2 receive the stage fields. */
int opflow_weno_rk3(opflow_ctx ctx, opflow_field u, opflow_field u1, opflow_field u2, int kind, int dim, double dt, int steps);

/* opflow_weno_rk3 with an evaluation mode.  OPFLOW_EVAL_EXACT is opflow_weno_rk3.  OPFLOW_EVAL_FAST
 * evaluates the same scheme with contracted (fused multiply-add) arithmetic and the nonlinear weights
 * w_k = (c_k / q_k^2) / sum_j (c_j / q_j^2) through one reciprocal instead of six divisions; it is not
 * bit-identical: max |u_fast - u_exact| <= 4 ulps of max |u| after one RK3 step and <= 1e-14 * max |u|
 * after 20 on periodic lines with square and cosine pulses (the tested bounds).  Over longer runs the
 * scheme's own sensitivity dominates: WENO5-JS moves the exact result by up to 1e-8 after 100 steps
 * when its input moves by one ulp, and FAST stays within that spread. */
int opflow_weno_rk3_mode(opflow_ctx ctx, opflow_field u, opflow_field u1, opflow_field u2, int kind, int dim, double dt, int steps,
                         int mode);

/* ---- implicit path (path I) -------------------------------------------------------------------- */
/* The equation `lhs == rhs` is given as the tree of `lhs - rhs` (Equation.hpp:41-55) in which the
 * unknown appears as the leaf slot `unknown_slot`; the other leaves are known fields.  This replaces
 * HYPREEqnSolveHandler::initStencil/generateAb (src/Core/Equation/HYPREEqnSolveHandler.hpp:79-166),
 * i.e. StencilField evaluation with StencilPad arithmetic (StencilField.hpp:123-350,
 * StencilPad.hpp:137-336). */

/* Assembly for parity checks: writes, for every cell of commonRange(target.assignable, target.local)
 * in x-fastest order, the coefficients of the stencil entries and the right-hand side b = -bias,
 * exactly as generateAb hands them to HYPRE_StructMatrixSetValues / HYPRE_StructVectorSetValues,
 * including the pinned first row when pin != 0.  offsets_out receives n_entries*ndim ints in the
 * order of the middle cell's StencilPad (commStencil).  Pass NULL buffers to query sizes. */
int opflow_assemble(opflow_ctx ctx, opflow_field target, const opflow_node* nodes, int n_nodes,
                    const opflow_field* leaves, int n_leaves, int unknown_slot, int pin,
                    int* n_entries, int* offsets_out, double* coef_out, double* rhs_out, size_t* n_cells);

/* Solver parameters: StructSolverParamsBase (src/Core/Solvers/Struct/StructSolver.hpp:39-51) plus the
 * PFMG preconditioner knobs (StructSolverPFMG.hpp:23-33) and the GPU extensions. */
enum opflow_precision { OPFLOW_PREC_FP64 = 0, OPFLOW_PREC_MIXED = 1 };
/* Outer iterations (src/Core/Solvers/Struct/StructSolver.hpp:23-34).  PCG with the multigrid
 * preconditioner is the fused device-side flexible PCG; every other combination runs host-driven
 * (one host read of the step's scalars per step).  GMRES, FGMRES and LGMRES all run as restarted
 * flexible GMRES(kdim); NONE iterates the preconditioner alone (PFMG, SMG or Jacobi as the solver). */
enum opflow_krylov {
    OPFLOW_KRYLOV_PCG = 0,
    OPFLOW_KRYLOV_GMRES = 1,
    OPFLOW_KRYLOV_FGMRES = 2,
    OPFLOW_KRYLOV_LGMRES = 3,
    OPFLOW_KRYLOV_BICGSTAB = 4,
    OPFLOW_KRYLOV_NONE = 5
};
/* Preconditioners: the geometric multigrid V-cycle stands in for PFMG, SMG and CycRed; JACOBI is one
 * diagonal step z = D^-1 v; NONE the identity. */
enum opflow_precond {
    OPFLOW_PRECOND_MG = 0,
    OPFLOW_PRECOND_JACOBI = 1,
    OPFLOW_PRECOND_NONE = 2,
    OPFLOW_PRECOND_AMG = 3 /* equation sets only: smoothed-aggregation AMG over the whole coupled matrix
                              (AMGCL's amg<smoothed_aggregation, spai0>, AMGCLEqnSolveHandler.hpp) */
};

typedef struct {
    double tol;           /* relative residual ||b-Ax||_2/||b||_2 target (reference: tol)        */
    int max_iter;         /* reference: maxIter                                                  */
    int static_mat;       /* reference: staticMat (reuse A, regenerate b only)                   */
    int pin_value;        /* reference: pinValue (pin the first unknown to 0)                    */
    int precision;        /* enum opflow_precision                                               */
    int pre_sweeps;       /* V-cycle smoothing sweeps (red-black Gauss-Seidel), default 2        */
    int post_sweeps;      /* default 2                                                           */
    int coarse_max;       /* coarsest level size bound for the dense direct solve, default 64    */
    int zero_guess;       /* 1: start from x = 0 instead of the target's values                  */
    int krylov;           /* enum opflow_krylov: the outer iteration (reference: StructSolverType) */
    int precond;          /* enum opflow_precond: its preconditioner                             */
    int kdim;             /* GMRES restart length (reference: kDim, HYPRE's default 5)           */
    double abs_tol;       /* also stop once ||b - A x||_2 <= abs_tol (reference: absTol); 0 off  */
} opflow_solve_params;

typedef struct {
    int iterations;       /* EqnSolveState::niter (EqnSolveHandler.hpp:17-25)                    */
    double rel_residual;  /* ||b - A x||_2 / ||b||_2 of the reference's system (pinned if pinned) */
    double abs_residual;
    int converged;
    double setup_ms, solve_ms;
} opflow_solve_state;

void opflow_solve_params_default(opflow_solve_params* p);

/* makeEqnSolveHandler(f, target, PrecondStructSolver<PCG,PFMG>) (HYPREEqnSolveHandler.hpp:44-48):
 * assembles the operator on the device and builds the multigrid hierarchy. */
int opflow_solver_create(opflow_ctx ctx, opflow_field target, const opflow_node* nodes, int n_nodes,
                         const opflow_field* leaves, int n_leaves, int unknown_slot,
                         const opflow_solve_params* params, opflow_solver* out);
/* EqnSolveHandler::solve (HYPREEqnSolveHandler.hpp:190-209): regenerates A and b (or only b when
 * static_mat), solves, writes the solution into the target field and updates its padding. */
int opflow_solver_solve(opflow_solver s, opflow_solve_state* state);
int opflow_solver_destroy(opflow_solver s);

/* ---- coupled equation sets (the reference's SolveEqns / AMGCL path) ------------------------------
 * SolveEqns(getter_0, ..., getter_{n-1}, targets..., mapper, params) (src/Core/Equation/UnifiedSolve.hpp:69-100,
 * AMGCLEqnSolveHandler.hpp:53-190): equation k (the tree trees[k], the lhs - rhs of getter k) is solved
 * for targets[k] jointly with the others.  All trees index one leaf list in which every target
 * appears; pin[k] pins equation k's last unknown (CSRMatrixGenerator.hpp:57-75); params (one set for
 * the whole system) choose the outer iteration and the block-diagonal preconditioner (each equation's
 * multigrid, Jacobi, none).  The first solve assembles the matrix; later ones re-assemble it unless
 * static_mat, in which case only the right-hand side is regenerated.  x starts at 0 on the first solve
 * and from the previous solution afterwards; the solution is written back into the targets. */
int opflow_eqnset_create(opflow_ctx ctx, int n_eqn, const opflow_field* targets, const opflow_node* const* trees, const int* n_nodes,
                         const opflow_field* leaves, int n_leaves, const int* pin, const opflow_solve_params* params, opflow_eqnset* out);
int opflow_eqnset_solve(opflow_eqnset s, opflow_solve_state* state);
/* The assembled system as CSR (CSRMatrixGenerator::generate): rows and columns numbered equation after
 * equation, x fastest within each target's assignable range; columns ascending within a row; exact
 * zeros left out.  Call with null arrays to get n_rows and nnz; row_ptr has n_rows + 1 entries. */
int opflow_eqnset_csr(opflow_eqnset s, long long* n_rows, long long* nnz, long long* row_ptr, long long* cols, double* vals, double* rhs);
int opflow_eqnset_destroy(opflow_eqnset s);

/* ---- batched uneven solves ------------------------------------------------------------------- */
/* Many independent 2D/3D problems of different sizes in one persistent launch per multigrid
 * operation.  The description is a compact physics form (no expression trees), one per problem:
 *   alpha*u - beta*Lap(u) = f   on an n[0] x n[1] (x n[2]) grid of cells (loc CENTER) or nodes (CORNER),
 * Dirichlet (value 0) or Neumann (gradient 0) on every side. */
typedef struct {
    int ndim;
    int n[3];           /* cells (CENTER) or nodes (CORNER) per dimension              */
    int loc;            /* enum opflow_loc                                             */
    int bc;             /* OPFLOW_BC_DIRC or OPFLOW_BC_NEUM on all sides               */
    double h[3];        /* grid spacing                                                */
    double alpha, beta; /* alpha*u - beta*Lap(u)                                       */
} opflow_problem_desc;

int opflow_batch_create(opflow_ctx ctx, const opflow_problem_desc* problems, int n_problems,
                        const opflow_solve_params* params, opflow_batch* out);

/* A user equation, as opflow_solver_create takes it (the equation of a makeEqnSolveHandler,
 * HYPREEqnSolveHandler.hpp:44-108): the tree of lhs - rhs over `leaves`, the unknown as leaf slot
 * `unknown` (its field is the target).  Any StencilPad-generated equation whose stencil is the
 * (2*dim+1)-point star: variable coefficients, mixed boundary conditions, Helmholtz terms. */
typedef struct {
    const opflow_node* nodes;
    int n_nodes;
    const opflow_field* leaves;
    int n_leaves;
    int unknown;
} opflow_equation;

/* A batch of user equations (any sizes, any mix of operators) solved together like
 * opflow_batch_create's problems.  Each problem is assembled from its fields at creation (generateAb);
 * its right-hand side is the equation's (opflow_batch_set may replace it) and its initial guess the
 * target's values (HYPREEqnSolveHandler::initx).  A singular problem (zero row sums, no Dirichlet
 * side) is pinned as opflow_solver_solve pins it when params->pin_value, else its right-hand side is
 * projected to zero mean.  The solution stays in the batch (opflow_batch_get / opflow_batch_vectors);
 * the target fields are not written. */
int opflow_batch_create_eqns(opflow_ctx ctx, const opflow_equation* eqns, int n_eqns, const opflow_solve_params* params,
                             opflow_batch* out);
/* Device pointers of problem i's unknown vector and right-hand side (x fastest over the unknowns). */
int opflow_batch_vectors(opflow_batch b, int i, double** x, double** f, size_t* n_unknowns);
/* Host copies: set problem i's right-hand side (and, unless x0 is NULL, its initial guess); read its
 * solution.  n must equal the problem's number of unknowns. */
int opflow_batch_set(opflow_batch b, int i, const double* f_host, const double* x0_host, size_t n);
int opflow_batch_get(opflow_batch b, int i, double* x_host, size_t n);
int opflow_batch_solve(opflow_batch b, opflow_solve_state* states /* n_problems */);
int opflow_batch_destroy(opflow_batch b);

/* ---- serving ---------------------------------------------------------------------------------- */
/* A request loop that keeps problems resident on the device and batches whatever is active into one
 * persistent launch per multigrid operation (continuous batching: requests join at the next iteration
 * boundary once HBM budget and a slot are free, and leave as soon as they converge).  No counterpart
 * in the reference, which solves one equation per call (HYPREEqnSolveHandler::solve). */
typedef struct {
    opflow_problem_desc problem; /* alpha*u - beta*Lap(u) = f                                          */
    int steps;                   /* 1: one solve; k > 1: a session of k solves, each taking the previous
                                    solution as its right-hand side (backward-Euler heat steps)        */
    const double* f;             /* right-hand side / initial state, n unknowns, in host or device memory
                                    (unified addressing): read when the request is admitted, so it must
                                    stay valid and unchanged until the request's result is available
                                    (pinned host memory gives the fastest host copy).  Non-finite values
                                    are refused with OPFLOW_E_NAN: by submit for host memory, as the
                                    request's result status for device memory (checked at admission)   */
    double* x_out;               /* buffer for the final solution, n unknowns, host or device (may be NULL) */
    const double* x0;            /* initial guess of the first solve, n unknowns, host or device (NULL: zero);
                                    a session restored from a checkpoint passes the checkpoint here and as f */
    const opflow_equation* equation; /* NULL: the request is `problem`.  Otherwise a user equation (the
                                    problem is ignored): it is assembled from its fields at admission, so
                                    the fields must stay alive and unchanged until the request's result is
                                    available.  steps must be 1 and f NULL (the right-hand side is the
                                    equation's); x0 NULL starts from the target's values (initx); x_out
                                    receives the solution over the target's assignable cells (x fastest);
                                    the target field itself is not written.  A singular equation is pinned
                                    when the server's params->pin_value, else projected to zero mean. */
} opflow_request;

typedef struct {
    long long id;
    int status;                  /* OPFLOW_OK, OPFLOW_E_NOT_CONVERGED, ...                           */
    int iterations;              /* flexible-PCG iterations summed over the request's solves          */
    int solves;
    double rel_residual;         /* of the last solve                                                */
    double queue_ms, latency_ms; /* submit -> admission, submit -> result on the host                 */
} opflow_request_result;

typedef struct {
    long long submitted, completed, solves;
    double p50_ms, p99_ms, mean_ms, max_ms;
    double elapsed_s, solves_per_s;
    int max_active_seen;
    long long graph_launches, compositions;
    double setup_s, compose_s, iterate_s, retire_s; /* worker wall time: admitting requests (hierarchy
                                                       setup), composing batch tables, batched iterations
                                                       with their state read-back, retiring results     */
} opflow_serve_stats;

/* hbm_budget_bytes bounds the resident problems' memory (0: unbounded); max_active bounds the batch
 * (1 gives one-request-at-a-time serving). */
int opflow_server_create(opflow_ctx ctx, const opflow_solve_params* params, size_t hbm_budget_bytes, int max_active, opflow_server* out);
int opflow_server_submit(opflow_server s, const opflow_request* req, long long* id);
/* wait != 0 blocks until the request is done; otherwise *done tells whether `out` was filled */
int opflow_server_result(opflow_server s, long long id, int wait, int* done, opflow_request_result* out);
int opflow_server_drain(opflow_server s);
/* Checkpoint of a running session (steps > 1) at its next step boundary: x_out (n values) receives the
 * solver state after *steps_done steps (for a pinned problem, before the final shift).  Submitting the
 * same problem with f = x0 = that state and steps - *steps_done steps continues the session bit for bit
 * (the state can go to disk through a field and opflow_field_write_raw).  OPFLOW_E_INVALID for an
 * unknown request, a single solve, a wrong n, or a session that finishes before its next boundary. */
int opflow_server_checkpoint(opflow_server s, long long id, double* x_out, size_t n, int* steps_done);
int opflow_server_stats(opflow_server s, opflow_serve_stats* out);
int opflow_server_destroy(opflow_server s);

/* ---- autotuner ---------------------------------------------------------------------------------- */
/* No counterpart in the reference (HYPRE and the OpenMP evaluators have no launch configurations).
 * Where a kernel has equivalent launch configurations - the z-marching 3D multigrid kernels' plane
 * batch, the 2D tile shape of the fused multigrid tile kernels, the 3D explicit kernels' tiling - the
 * engine times them on the device the first time a (kernel, shape, stencil) key is met and keeps the
 * fastest; results are identical whichever is chosen.  OPFLOW_TUNE=0 turns tuning off (the measured
 * defaults); the explicit OPFLOW_MG_ZB / OPFLOW_AXIS_TILING switches override it.
 * set_cache: choices are loaded from `path` (when it exists) and new ones appended to it; NULL keeps
 * them in memory only (the default; OPFLOW_TUNE_CACHE names a file for the process instead).
 * lookup: the cached choice for a key (OPFLOW_E_INVALID when there is none).  stats: choices measured
 * by this process, cache hits, and entries held.  clear: forget every choice (the file is kept). */
int opflow_tune_set_cache(const char* path);
int opflow_tune_lookup(const char* key, int* value);
int opflow_tune_stats(long long* tuned, long long* hits, long long* entries);
int opflow_tune_clear(void);

/* ---- residual norms without device allocation ------------------------------------------------- */
/* No counterpart in the reference.  For callers that cannot allocate device memory where they need the
 * answer - code running inside a CUDA stream capture (cudaMalloc/cudaFree cannot be captured), hosts
 * whose device memory belongs to their own pool allocator, latency-critical loops that must not
 * synchronise the device: computes r = b - A x and norms[0] = ||b||_2, norms[1] = ||b - A x||_2 with no
 * allocation at all.  For a system with nonzero b, norms[1]/norms[0] is the residual the solvers report
 * as EqnSolveState::relerr (with b = 0 they report norms[1]).  For a pinned system (pinValue) pass the
 * reference's system: the first unknown's row the identity (centre 1, other slots 0) with b[0] = 0 and
 * the solution with x[0] = 0, as the solvers return it; that row's residual is then exactly 0.
 * Every pointer is device memory the caller owns: coef is the (2*ndim+1)-point operator as seven
 * float64 slot arrays [7][N] (centre, x-, x+, y-, y+, z-, z+; unused slots ignored), b/x/r hold N
 * values x fastest, norms two values.  Work is enqueued on `stream` (results valid after it completes).
 * The partial sums live in one static 1 MiB device array per device: grids needing more than 65536
 * chunks (one per 1024 cells of every x-row) are rejected with OPFLOW_E_INVALID; calls that overlap on
 * the GPU race on that array.  Every call looks up the array's address in the current device's
 * context (no allocation); the first call on a device may load the module, so make it before any
 * stream capture begins. */
int opflow_residual_norms_noalloc(void* stream, int ndim, const int* n, const int* periodic, const double* coef, const double* b,
                                  const double* x, double* r, double* norms);

#ifdef __cplusplus
}
#endif
#endif /* OPFLOW_GPU_H */
