/* oracle.c -- CPU restatement of OpFlow's explicit-evaluation and stencil-assembly paths.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker the tests, __graft_entry__.smoke() and the
 * CPU-baseline leg of bench.py compare the CUDA library against.  It is never linked into, loaded by or
 * called from the product path (opflow_gb300/).
 *
 * Parity is pinned: tests/test_oracle_golden.py checks this restatement bit-for-bit against dumps of
 * the reference itself (oracle/_ref/ref_driver built from the OpFlow sources by oracle/build_ref.sh,
 * stored under tests/golden/) and against the literal CSR matrices of the reference's
 * test/Core/Equation/CSRMatrixGeneratorTest.cpp.
 *
 * Everything follows the reference's evaluation order operation by operation and is compiled with
 * -ffp-contract=off, so no multiply-add is fused that the reference (built for x86-64, no FMA) keeps
 * separate.  File:line citations are relative to the OpFlow source tree.
 */
#include "../include/opflow_gpu.h"

#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif
#define MAXD 3
int or_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
    return omp_get_max_threads();
#else
    (void) n;
    return 1;
#endif
}
static char g_err[512];
const char* or_last_error(void) { return g_err; }
static int fail(int code, const char* msg) {
    snprintf(g_err, sizeof g_err, "%s", msg);
    return code;
}

/* ------------------------------------------------------------------------------------------------ */
/* seeded inputs (counter-based splitmix64), identical to the generator used by the tests           */
/* ------------------------------------------------------------------------------------------------ */
static inline uint64_t mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
double or_u01(uint64_t seed, uint64_t k) {
    return (double) (mix64(seed + (k + 1) * 0x9E3779B97F4A7C15ull) >> 11) * 0x1.0p-53;
}

/* ------------------------------------------------------------------------------------------------ */
/* mesh: MeshBuilder<CartesianMesh>::set1DRange / set1DMesh(min,max) / setExtMesh (Symm)             */
/* CartesianMesh.hpp:209-217, 219-237, 268-276, 292-303                                              */
/* ------------------------------------------------------------------------------------------------ */
static void ext_symm(int dims, int start, int pad, double* x, double* dx);

int or_mesh_uniform(int dims, int start, int pad, double min, double max, double* x, double* dx) {
    if (dims < 2 || pad < 0) return fail(OPFLOW_E_INVALID, "mesh needs >= 2 nodes");
    const int es = start - pad, end = start + dims;
    for (int i = start; i < end; ++i) x[i - es] = (max - min) / (double) (dims - 1) * (double) (i - start) + min;
    for (int j = start; j < end - 1; ++j) dx[j - es] = (max - min) / (double) (dims - 1);
    ext_symm(dims, start, pad, x, dx);
    return OPFLOW_OK;
}

/* set1DMesh(const MeshSetter& f, k) (CartesianMesh.hpp:279-290): pts[i - start] = f(i) for the dims
 * nodes, dx(j) = x(j + 1) - x(j), then the same Symm extension. */
int or_mesh_points(int dims, int start, int pad, const double* pts, double* x, double* dx) {
    if (dims < 2 || pad < 0) return fail(OPFLOW_E_INVALID, "mesh needs >= 2 nodes");
    const int es = start - pad, end = start + dims;
    for (int i = start; i < end; ++i) x[i - es] = pts[i - start];
    for (int j = start; j < end - 1; ++j) dx[j - es] = x[j + 1 - es] - x[j - es];
    ext_symm(dims, start, pad, x, dx);
    return OPFLOW_OK;
}

static void ext_symm(int dims, int start, int pad, double* x, double* dx) {
    const int es = start - pad, end = start + dims, ee = end + pad;
    /* Symm extension of dx (the default MeshExtMode) */
    for (int i = es; i < start; ++i) dx[i - es] = dx[2 * start - 1 - i - es];
    for (int i = end - 1; i < ee - 1; ++i) dx[i - es] = dx[2 * end - 3 - i - es];
    /* integrate x into the ghost extension */
    for (int i = start - 1; i >= es; --i) x[i - es] = x[i + 1 - es] - dx[i - es];
    for (int i = end; i < ee; ++i) x[i - es] = x[i - 1 - es] + dx[i - 1 - es];
}

typedef struct {
    const opflow_mesh_desc* m;
} Mesh;
static inline double mesh_x(const opflow_mesh_desc* m, int d, int i) { return m->x[d][i - (m->start[d] - m->pad_width)]; }
static inline double mesh_dx(const opflow_mesh_desc* m, int d, int i) { return m->dx[d][i - (m->start[d] - m->pad_width)]; }

/* ------------------------------------------------------------------------------------------------ */
/* field ranges: ExprBuilder::calculateRanges / validateRanges / build (CartesianField.hpp:929-1029) */
/* ------------------------------------------------------------------------------------------------ */
static inline int imax(int a, int b) { return a > b ? a : b; }
static inline int imin(int a, int b) { return a < b ? a : b; }

int or_field_info(const opflow_mesh_desc* m, const opflow_field_desc* f, opflow_field_info* o) {
    if (!m || !f || !o || f->ndim != m->ndim || f->ndim < 1 || f->ndim > 3) return fail(OPFLOW_E_INVALID, "bad field description");
    memset(o, 0, sizeof *o);
    const int D = f->ndim;
    o->ndim = D;
    int pad = f->padding;
    for (int d = 0; d < D; ++d) pad = imax(pad, imax(f->ext[d][0], f->ext[d][1]));
    o->padding = pad;
    for (int d = 0; d < D; ++d) {
        int s = m->start[d], e = m->start[d] + m->dims[d];
        o->logical[d][0] = o->assignable[d][0] = o->local[d][0] = o->accessible[d][0] = s;
        o->logical[d][1] = o->assignable[d][1] = o->local[d][1] = o->accessible[d][1] = e;
    }
    for (int d = 0; d < D; ++d) {
        const int loc = f->loc[d];
        switch (f->bc_type[d][0]) {
            case OPFLOW_BC_DIRC:
                if (loc == OPFLOW_CORNER) o->assignable[d][0]++;
                break;
            case OPFLOW_BC_NEUM: case OPFLOW_BC_UNDEFINED: case OPFLOW_BC_SYMM: case OPFLOW_BC_ASYMM: case OPFLOW_BC_PERIODIC:
                break;
            default: return fail(OPFLOW_E_INVALID, "unknown bc type");
        }
        switch (f->bc_type[d][1]) {
            case OPFLOW_BC_DIRC:
                if (loc == OPFLOW_CORNER) o->assignable[d][1]--;
                else { o->accessible[d][1]--; o->assignable[d][1]--; }
                break;
            case OPFLOW_BC_NEUM: case OPFLOW_BC_UNDEFINED: case OPFLOW_BC_SYMM: case OPFLOW_BC_ASYMM:
                if (loc == OPFLOW_CENTER) { o->accessible[d][1]--; o->assignable[d][1]--; }
                break;
            case OPFLOW_BC_PERIODIC:
                o->accessible[d][1]--; o->assignable[d][1]--;
                break;
            default: return fail(OPFLOW_E_INVALID, "unknown bc type");
        }
        o->logical[d][0] = o->accessible[d][0] - f->ext[d][0];
        o->logical[d][1] = o->accessible[d][1] + f->ext[d][1];
    }
    for (int d = 0; d < D; ++d) {
        o->local[d][0] = o->accessible[d][0];
        o->local[d][1] = o->accessible[d][1];
        /* validateRanges */
        o->accessible[d][0] = imax(o->accessible[d][0], o->logical[d][0]);
        o->accessible[d][1] = imin(o->accessible[d][1], o->logical[d][1]);
        o->local[d][0] = imax(o->local[d][0], o->logical[d][0]);
        o->local[d][1] = imin(o->local[d][1], o->logical[d][1]);
        o->assignable[d][0] = imax(o->assignable[d][0], o->accessible[d][0]);
        o->assignable[d][1] = imin(o->assignable[d][1], o->accessible[d][1]);
    }
    o->count = 1;
    for (int d = 0; d < 3; ++d) {
        if (d < D) {
            o->data_offset[d] = o->local[d][0] - pad;
            o->data_dims[d] = o->local[d][1] - o->local[d][0] + 2 * pad;
        } else {
            o->data_offset[d] = 0;
            o->data_dims[d] = 1;
            o->logical[d][1] = o->accessible[d][1] = o->assignable[d][1] = o->local[d][1] = 1;
        }
        o->count *= (size_t) o->data_dims[d];
    }
    return OPFLOW_OK;
}

/* ------------------------------------------------------------------------------------------------ */
/* a field = description + ranges + host data                                                       */
/* ------------------------------------------------------------------------------------------------ */
typedef struct {
    const opflow_field_desc* d;
    opflow_field_info r;
    double* data;
} Field;

static int g_range_err;
static inline int in_data(const Field* f, const int* i) {
    for (int d = 0; d < f->r.ndim; ++d)
        if (i[d] < f->r.data_offset[d] || i[d] >= f->r.data_offset[d] + f->r.data_dims[d]) return 0;
    return 1;
}
/* PlainTensor::getOffset (PlainTensor.hpp:204-213): x fastest */
static inline size_t lin(const Field* f, const int* i) {
    size_t o = 0;
    for (int d = f->r.ndim - 1; d >= 0; --d) o = o * (size_t) f->r.data_dims[d] + (size_t) (i[d] - f->r.data_offset[d]);
    return o;
}
static inline double fget(const Field* f, const int* i) {
    if (!in_data(f, i)) { g_range_err = 1; return NAN; }
    return f->data[lin(f, i)];
}
static inline void fset(Field* f, const int* i, double v) {
    if (!in_data(f, i)) { g_range_err = 1; return; }
    f->data[lin(f, i)] = v;
}

/* iterate a box [lo, hi) x fastest */
#define BOX_FOR(D, lo, hi, idx)                                                                               \
    for (idx[2] = (D > 2 ? lo[2] : 0); idx[2] < (D > 2 ? hi[2] : 1); ++idx[2])                              \
        for (idx[1] = (D > 1 ? lo[1] : 0); idx[1] < (D > 1 ? hi[1] : 1); ++idx[1])                          \
            for (idx[0] = lo[0]; idx[0] < hi[0]; ++idx[0])

/* Interpolator1D::intp(x1, y1, x2, y2, x) (src/Math/Interpolator/Interpolator.hpp:21-23,38-40) */
static inline double intp_d(double x1, double y1, double x2, double y2, double x) {
    double a = x1 - x, b = x2 - x;
    return (a * y2 - b * y1) / (a - b);
}

/* ------------------------------------------------------------------------------------------------ */
/* CartesianField::updatePaddingImpl_final, single-rank branch (CartesianField.hpp:349-629)         */
/* ------------------------------------------------------------------------------------------------ */
static void update_padding(const opflow_mesh_desc* m, Field* f) {
    const int D = f->r.ndim;
    const opflow_field_info* R = &f->r;
    int idx[3], lo[3], hi[3];
    /* step 0: Dirichlet values on corner-located boundary nodes (lines 350-364) */
    for (int i = 0; i < D; ++i) {
        if (R->local[i][0] == R->accessible[i][0] && f->d->bc_type[i][0] == OPFLOW_BC_DIRC && f->d->loc[i] == OPFLOW_CORNER) {
            for (int k = 0; k < 3; ++k) { lo[k] = R->local[k][0]; hi[k] = R->local[k][1]; }
            lo[i] = R->local[i][0]; hi[i] = lo[i] + 1;
            BOX_FOR(D, lo, hi, idx) fset(f, idx, f->d->bc_value[i][0]);
        }
        if (R->local[i][1] == R->accessible[i][1] && f->d->bc_type[i][1] == OPFLOW_BC_DIRC && f->d->loc[i] == OPFLOW_CORNER) {
            for (int k = 0; k < 3; ++k) { lo[k] = R->local[k][0]; hi[k] = R->local[k][1]; }
            lo[i] = R->local[i][1] - 1; hi[i] = lo[i] + 1;
            BOX_FOR(D, lo, hi, idx) fset(f, idx, f->d->bc_value[i][1]);
        }
    }
    /* step 1: padding zones by BC extension (lines 365-606) */
    int st[3] = {0, 0, 0}, en[3] = {0, 0, 0};
    for (int i = 0; i < D; ++i) {
        for (int side = 0; side < 2; ++side) {
            const int bct = f->d->bc_type[i][side];
            const double bcv = f->d->bc_value[i][side];
            const int at_bound = side == 0 ? R->local[i][0] == R->accessible[i][0] : R->local[i][1] == R->accessible[i][1];
            if (!(at_bound && bct != OPFLOW_BC_UNDEFINED && bct != OPFLOW_BC_PERIODIC)) {
                if (side == 0) st[i] = R->local[i][0];
                else en[i] = R->local[i][1];
                continue;
            }
            if (side == 0) st[i] = R->logical[i][0];
            else en[i] = R->logical[i][1];
            for (int k = 0; k < 3; ++k) { lo[k] = R->local[k][0]; hi[k] = R->local[k][1]; }
            for (int j = 0; j < i; ++j) { lo[j] = st[j]; hi[j] = en[j]; }
            if (side == 0) { lo[i] = st[i]; hi[i] = R->local[i][0]; }
            else { lo[i] = R->local[i][1]; hi[i] = R->logical[i][1]; }
            const int corner = f->d->loc[i] == OPFLOW_CORNER;
            BOX_FOR(D, lo, hi, idx) {
                int mi[3] = {idx[0], idx[1], idx[2]};
                if (corner) mi[i] = side == 0 ? 2 * R->local[i][0] - idx[i] : 2 * R->local[i][1] - 2 - idx[i];
                else mi[i] = side == 0 ? 2 * R->local[i][0] - 1 - idx[i] : 2 * R->local[i][1] - 1 - idx[i];
                double v = 0.;
                switch (bct) {
                    case OPFLOW_BC_DIRC:
                        if (corner) {
                            double xb = mesh_x(m, i, side == 0 ? R->local[i][0] : R->local[i][1] - 1);
                            v = intp_d(xb, bcv, mesh_x(m, i, mi[i]), fget(f, mi), mesh_x(m, i, idx[i]));
                        } else {
                            double xb = mesh_x(m, i, side == 0 ? R->local[i][0] : R->local[i][1]);
                            v = intp_d(xb, bcv, mesh_x(m, i, mi[i]) + mesh_dx(m, i, mi[i]) / 2., fget(f, mi),
                                       mesh_x(m, i, idx[i]) + mesh_dx(m, i, idx[i]) / 2.);
                        }
                        break;
                    case OPFLOW_BC_NEUM:
                        if (corner) v = fget(f, mi) + bcv * (mesh_x(m, i, idx[i]) - mesh_x(m, i, mi[i]));
                        else
                            v = fget(f, mi) + bcv * (mesh_x(m, i, idx[i]) + mesh_dx(m, i, idx[i]) / 2. - mesh_x(m, i, mi[i])
                                                     - mesh_dx(m, i, mi[i]) / 2.);
                        break;
                    case OPFLOW_BC_SYMM: v = fget(f, mi); break;
                    case OPFLOW_BC_ASYMM: v = -fget(f, mi); break;
                }
                fset(f, idx, v);
            }
        }
    }
    /* step 2: periodic copies over the logical range (lines 609-629) */
    for (int i = 0; i < D; ++i) {
        if (f->d->bc_type[i][0] != OPFLOW_BC_PERIODIC) continue;
        const int period = R->accessible[i][1] - R->accessible[i][0];
        for (int k = 0; k < 3; ++k) { lo[k] = R->logical[k][0]; hi[k] = R->logical[k][1]; }
        lo[i] = R->logical[i][0]; hi[i] = R->accessible[i][0];
        BOX_FOR(D, lo, hi, idx) {
            int mi[3] = {idx[0], idx[1], idx[2]};
            mi[i] += period;
            fset(f, idx, fget(f, mi));
        }
        for (int k = 0; k < 3; ++k) { lo[k] = R->logical[k][0]; hi[k] = R->logical[k][1]; }
        lo[i] = R->accessible[i][1]; hi[i] = R->logical[i][1];
        BOX_FOR(D, lo, hi, idx) {
            int mi[3] = {idx[0], idx[1], idx[2]};
            mi[i] -= period;
            fset(f, idx, fget(f, mi));
        }
    }
}

int or_update_padding(const opflow_mesh_desc* m, const opflow_field_desc* fd, double* data) {
    Field f = {fd, {0}, data};
    int rc = or_field_info(m, fd, &f.r);
    if (rc) return rc;
    g_range_err = 0;
    update_padding(m, &f);
    return g_range_err ? fail(OPFLOW_E_RANGE, "padding read outside the data array") : OPFLOW_OK;
}

/* ------------------------------------------------------------------------------------------------ */
/* expression trees: location propagation (the operators' prepare())                                */
/* ------------------------------------------------------------------------------------------------ */
typedef struct {
    const opflow_mesh_desc* m;
    const opflow_node* nodes;
    int n;
    Field* fields;
    int nf;
    int loc[64][3]; /* loc per node, -1 for scalar-valued nodes */
    int unknown;    /* leaf slot of the unknown for stencil evaluation, -1 otherwise */
    int pin;
    /* StencilField ranges (after ignorePeriodicBC, StencilField.hpp:112-121) */
    int st_assignable[3][2], st_accessible[3][2], st_logical[3][2];
    int pin_index[3];
} Ctx;

static int compute_locs(Ctx* c) {
    if (c->n > 64) return fail(OPFLOW_E_UNSUPPORTED, "expression too large");
    for (int k = 0; k < c->n; ++k) {
        const opflow_node* nd = &c->nodes[k];
        int* L = c->loc[k];
        L[0] = L[1] = L[2] = -1;
        if ((nd->a >= k) || (nd->b >= k)) return fail(OPFLOW_E_INVALID, "children must precede parents");
        switch (nd->kind) {
            case OPFLOW_NODE_FIELD:
                if (nd->field < 0 || nd->field >= c->nf) return fail(OPFLOW_E_INVALID, "bad leaf slot");
                for (int d = 0; d < 3; ++d) L[d] = c->fields[nd->field].d->loc[d];
                break;
            case OPFLOW_NODE_CONST: break;
            case OPFLOW_NODE_ADD: case OPFLOW_NODE_SUB: case OPFLOW_NODE_MUL: case OPFLOW_NODE_DIV: {
                /* initPropsFrom(arg1), or arg2 when arg1 is a scalar (BinOpDefMacros.hpp.in:18-71) */
                const int* La = c->loc[nd->a];
                const int* Lb = c->loc[nd->b];
                for (int d = 0; d < 3; ++d) L[d] = La[0] >= 0 ? La[d] : Lb[d];
                break;
            }
            case OPFLOW_NODE_NEG: case OPFLOW_NODE_D2: case OPFLOW_NODE_WENO53_DOWN: case OPFLOW_NODE_WENO53_UP:
                for (int d = 0; d < 3; ++d) L[d] = c->loc[nd->a][d];
                break;
            case OPFLOW_NODE_D1: /* D1FirstOrderCentered.hpp:38-56: the location flips along dim */
                for (int d = 0; d < 3; ++d) L[d] = c->loc[nd->a][d];
                L[nd->dim] = L[nd->dim] == OPFLOW_CENTER ? OPFLOW_CORNER : OPFLOW_CENTER;
                break;
            case OPFLOW_NODE_INTP_C2C: /* D1Linear.hpp:48-58 */
                for (int d = 0; d < 3; ++d) L[d] = c->loc[nd->a][d];
                L[nd->dim] = OPFLOW_CORNER;
                break;
            case OPFLOW_NODE_INTP_COR2CEN: /* D1Linear.hpp:60-69 */
                for (int d = 0; d < 3; ++d) L[d] = c->loc[nd->a][d];
                L[nd->dim] = OPFLOW_CENTER;
                break;
            case OPFLOW_NODE_D1_BIASED_UP: case OPFLOW_NODE_D1_BIASED_DOWN:
                /* D1FirstOrderBiasedUpwind.hpp:68-84, D1FirstOrderBiasedDownwind.hpp:67-83: loc kept */
                for (int d = 0; d < 3; ++d) L[d] = c->loc[nd->a][d];
                break;
            case OPFLOW_NODE_GT: case OPFLOW_NODE_GE: case OPFLOW_NODE_LT: case OPFLOW_NODE_LE: case OPFLOW_NODE_NE:
            case OPFLOW_NODE_AND: case OPFLOW_NODE_OR: case OPFLOW_NODE_FUNC2: {
                /* binary operators and functions: initPropsFrom(arg1), or arg2 when arg1 is a scalar */
                if (nd->b < 0) return fail(OPFLOW_E_INVALID, "missing operand");
                const int* La = c->loc[nd->a];
                const int* Lb = c->loc[nd->b];
                for (int d = 0; d < 3; ++d) L[d] = La[0] >= 0 ? La[d] : Lb[d];
                break;
            }
            case OPFLOW_NODE_NOT: case OPFLOW_NODE_FUNC1:
                for (int d = 0; d < 3; ++d) L[d] = c->loc[nd->a][d];
                break;
            case OPFLOW_NODE_COND: { /* CondOp::prepare: initPropsFrom(arg2), or arg3 (Conditional.hpp:41-115) */
                if (nd->b < 0 || nd->c < 0 || nd->c >= k) return fail(OPFLOW_E_INVALID, "bad conditional operands");
                const int* Lt = c->loc[nd->b];
                const int* Lf = c->loc[nd->c];
                for (int d = 0; d < 3; ++d) L[d] = Lt[0] >= 0 ? Lt[d] : (Lf[0] >= 0 ? Lf[d] : c->loc[nd->a][d]);
                break;
            }
            case OPFLOW_NODE_INTP_FL_CEN2COR: case OPFLOW_NODE_INTP_FL_COR2CEN: {
                /* D1FluxLimiterImpl::prepare (D1FluxLimiter.hpp:152-166, 182-201): the location of arg2 */
                const int c2c = nd->kind == OPFLOW_NODE_INTP_FL_CEN2COR;
                if (nd->b < 0) return fail(OPFLOW_E_INVALID, "missing operand");
                if (nd->field < OPFLOW_FL_CDS || nd->field > OPFLOW_FL_BSOU) return fail(OPFLOW_E_INVALID, "unknown flux limiter");
                if (nd->dim < 0 || nd->dim >= c->m->ndim) return fail(OPFLOW_E_INVALID, "bad operator dim");
                if (c->loc[nd->b][nd->dim] != (c2c ? OPFLOW_CENTER : OPFLOW_CORNER)) return fail(OPFLOW_E_INVALID, "flux-limiter operand at the wrong location");
                for (int d = 0; d < 3; ++d) L[d] = c->loc[nd->b][d];
                L[nd->dim] = c2c ? OPFLOW_CORNER : OPFLOW_CENTER;
                break;
            }
            default: return fail(OPFLOW_E_UNSUPPORTED, "unknown node kind");
        }
        if (nd->kind >= OPFLOW_NODE_D2 && nd->kind <= OPFLOW_NODE_D1_BIASED_DOWN && (nd->dim < 0 || nd->dim >= c->m->ndim))
            return fail(OPFLOW_E_INVALID, "bad operator dim");
        if (nd->kind != OPFLOW_NODE_FIELD && nd->kind != OPFLOW_NODE_CONST && nd->a < 0) return fail(OPFLOW_E_INVALID, "missing operand");
        if (nd->kind >= OPFLOW_NODE_ADD && nd->kind <= OPFLOW_NODE_DIV && nd->b < 0) return fail(OPFLOW_E_INVALID, "missing operand");
    }
    return OPFLOW_OK;
}

/* ------------------------------------------------------------------------------------------------ */
/* double-valued evaluation: Expression::evalAtImpl_final recursion (Expression.hpp:51-88)          */
/* ------------------------------------------------------------------------------------------------ */
static inline double pow2d(double a) { return a * a; } /* Math::pow2 (Numeric.hpp:104) */

/* D1WENO53Downwind::kernel (D1WENO53Downwind.hpp:136-154); D1WENO53Upwind::kernel has the same body
 * (D1WENO53Upwind.hpp:133-151) with its arguments taken from the other side. */
static double weno_kernel(double pm3, double pm2, double pm1, double p0, double pp1, double pp2, double h) {
    double d1 = (pm2 - pm3) / h, d2 = (pm1 - pm2) / h, d3 = (p0 - pm1) / h, d4 = (pp1 - p0) / h, d5 = (pp2 - pp1) / h;
    double ddx1 = d1 / 3. - 7. * d2 / 6. + 11. * d3 / 6.;
    double ddx2 = -d2 / 6. + 5 * d3 / 6 + d4 / 3;
    double ddx3 = d3 / 3 + 5 * d4 / 6 - d5 / 6;
    double s1 = 13. / 12. * pow2d(d1 - 2 * d2 + d3) + pow2d(d1 - 4 * d2 + 3 * d3) / 4;
    double s2 = 13. / 12. * pow2d(d2 - 2 * d3 + d4) + pow2d(d2 - d4) / 4.;
    double s3 = 13. / 12. * pow2d(d3 - 2 * d4 + d5) + pow2d(3 * d3 - 4 * d4 + d5) / 4.;
    /* std::max({...}) over an initializer list: first maximal element, compared with < */
    double mx = d1 * d1, t;
    t = d2 * d2; if (mx < t) mx = t;
    t = d3 * d3; if (mx < t) mx = t;
    t = d4 * d4; if (mx < t) mx = t;
    t = d5 * d5; if (mx < t) mx = t;
    const double eps = 1e-6 * mx + 1e-99;
    double a1 = .1 / pow2d(s1 + eps);
    double a2 = .6 / pow2d(s2 + eps);
    double a3 = .3 / pow2d(s3 + eps);
    double w1 = a1 / (a1 + a2 + a3);
    double w2 = a2 / (a1 + a2 + a3);
    double w3 = a3 / (a1 + a2 + a3);
    return w1 * ddx1 + w2 * ddx2 + w3 * ddx3;
}

/* std::max(a, b) = (a < b) ? b : a; std::min(a, b) = (b < a) ? b : a; the initializer-list forms
 * (std::max_element / std::min_element) keep the first extreme element. */
static double std_max(double a, double b) { return a < b ? b : a; }
static double std_min(double a, double b) { return b < a ? b : a; }

/* FluxLimiterKernels.hpp: MinmodKernel, SuperbeeKernel, MUSCLKernel, HarmonicKernel, vanAlbadaKernel,
 * SPLMinKernel, SPLMaxKernel and GPLKappaKernel with the aliases' parameters.  `m`, `kappa` and
 * `alpha` are computed as the reference does, `M::num / M::den` in integer arithmetic. */
static double ratio_int(long num, long den) { return (double) (num / den); }
static double spl_min(double m, double kappa, double r) {
    const double v[4] = {m * r, 0.5 * (1 + kappa) * r + 0.5 * (1 - kappa), 0.5 * (1 - kappa) * r + 0.5 * (1 + kappa), m};
    double cur = v[0];
    for (int q = 1; q < 4; ++q) if (v[q] < cur) cur = v[q];
    return std_max(0., cur);
}
static double spl_max(double m, double kappa, double r) {
    double mx = 0.5 * (1 + kappa) * r + 0.5 * (1 - kappa);
    const double l2 = 0.5 * (1 - kappa) * r + 0.5 * (1 + kappa);
    if (mx < l2) mx = l2;
    double cur = m * r;
    if (mx < cur) cur = mx;
    if (m < cur) cur = m;
    return std_max(0., cur);
}
static double gpl(double m, double alpha, double kappa, double r) {
    double cur = (2 + alpha) * r;
    const double t = 0.5 * (1 + kappa) * r + 0.5 * (1 - kappa);
    if (t < cur) cur = t;
    if (m < cur) cur = m;
    return std_max(0., cur);
}
static double limiter(int K, double r) {
    switch (K) {
        case OPFLOW_FL_MINMOD: return std_max(0., std_min(r, 1.));
        case OPFLOW_FL_SUPERBEE: {
            double m = 0., t = std_min(2. * r, 1.);
            if (m < t) m = t;
            t = std_min(r, 2.);
            if (m < t) m = t;
            return m;
        }
        case OPFLOW_FL_MUSCL: {
            double m = 2 * r, t = (r + 1) / 2.;
            if (t < m) m = t;
            if (2. < m) m = 2.;
            return std_max(0., m);
        }
        case OPFLOW_FL_HARMONIC: return (r + fabs(r)) / (r + 1);
        case OPFLOW_FL_VANALBADA: return r * (r + 1) / (r * r + 1);
        case OPFLOW_FL_UMIST: return spl_min(ratio_int(2, 1), ratio_int(1, 2), r);
        case OPFLOW_FL_SPL13: return spl_min(ratio_int(2, 1), ratio_int(1, 3), r);
        case OPFLOW_FL_SPLMAX12: return spl_max(ratio_int(2, 1), ratio_int(1, 2), r);
        case OPFLOW_FL_SPLMAX13: return spl_max(ratio_int(2, 1), ratio_int(1, 3), r);
        case OPFLOW_FL_KOREN: return gpl(ratio_int(2, 1), ratio_int(0, 1), ratio_int(1, 3), r);
        case OPFLOW_FL_SMART: return gpl(ratio_int(4, 1), ratio_int(0, 1), ratio_int(1, 2), r);
        default: return gpl(ratio_int(1, 1), ratio_int(0, 1), ratio_int(-1, 1), r); /* BSOU */
    }
}
/* KappaKernel<s>::eval(slop_u, slop_f) (FluxLimiterKernels.hpp:31-44) */
static double kappa_kernel(int K, double su, double sf) {
    static const double kap[] = {1., 0.5, 1. / 3., 0., -1.};
    const double kappa = kap[K];
    return (1 + kappa) / 2. * sf + (1 - kappa) / 2. * su;
}

static double func1(int f, double x) {
    switch (f) {
        case OPFLOW_F_ABS: return fabs(x);
        case OPFLOW_F_SQRT: return sqrt(x);
        case OPFLOW_F_CEIL: return ceil(x);
        case OPFLOW_F_FLOOR: return floor(x);
        case OPFLOW_F_TRUNC: return trunc(x);
        case OPFLOW_F_ROUND: return round(x);
        case OPFLOW_F_RINT: return rint(x);
        case OPFLOW_F_EXP: return exp(x);
        case OPFLOW_F_EXP2: return exp2(x);
        case OPFLOW_F_EXPM1: return expm1(x);
        case OPFLOW_F_LOG: return log(x);
        case OPFLOW_F_LOG10: return log10(x);
        case OPFLOW_F_LOG2: return log2(x);
        case OPFLOW_F_LOG1P: return log1p(x);
        case OPFLOW_F_CBRT: return cbrt(x);
        case OPFLOW_F_SIN: return sin(x);
        case OPFLOW_F_COS: return cos(x);
        case OPFLOW_F_TAN: return tan(x);
        case OPFLOW_F_ASIN: return asin(x);
        case OPFLOW_F_ACOS: return acos(x);
        case OPFLOW_F_ATAN: return atan(x);
        case OPFLOW_F_SINH: return sinh(x);
        case OPFLOW_F_COSH: return cosh(x);
        case OPFLOW_F_TANH: return tanh(x);
        case OPFLOW_F_ASINH: return asinh(x);
        case OPFLOW_F_ACOSH: return acosh(x);
        case OPFLOW_F_ATANH: return atanh(x);
        case OPFLOW_F_ERF: return erf(x);
        case OPFLOW_F_ERFC: return erfc(x);
        case OPFLOW_F_TGAMMA: return tgamma(x);
        case OPFLOW_F_LGAMMA: return lgamma(x);
    }
    return NAN;
}
static double func2(int f, double a, double b) {
    switch (f) {
        case OPFLOW_F2_MAX: return std_max(a, b);
        case OPFLOW_F2_MIN: return std_min(a, b);
        case OPFLOW_F2_FDIM: return fdim(a, b);
        case OPFLOW_F2_COPYSIGN: return copysign(a, b);
        case OPFLOW_F2_FMOD: return fmod(a, b);
        case OPFLOW_F2_REMAINDER: return remainder(a, b);
        case OPFLOW_F2_POW: return pow(a, b);
        case OPFLOW_F2_HYPOT: return hypot(a, b);
        case OPFLOW_F2_ATAN2: return atan2(a, b);
    }
    return NAN;
}

static double ev(Ctx* c, int k, const int* i);

/* D1FluxLimiterUpwindImpl / D1FluxLimiterDownwindImpl::eval (D1FluxLimiter.hpp:36-133) */
static double flux_side(Ctx* c, const opflow_node* nd, const int* i, int up) {
    const opflow_mesh_desc* m = c->m;
    const int d = nd->dim, c2c = nd->kind == OPFLOW_NODE_INTP_FL_CEN2COR;
    double x[3], y[3];
    int p1, hoff;
    if (c2c) { p1 = up ? -2 : -1; hoff = up ? -1 : 0; }
    else { p1 = up ? -1 : 0; hoff = 0; }
    for (int q = 0; q < 3; ++q) {
        const int o = i[d] + p1 + q;
        if (c2c) x[q] = up ? mesh_x(m, d, o) + 0.5 * mesh_dx(m, d, o) : mesh_x(m, d, o) + mesh_dx(m, d, o) * 0.5;
        else x[q] = mesh_x(m, d, o);
        int j[3] = {i[0], i[1], i[2]};
        j[d] = o;
        y[q] = ev(c, nd->b, j);
    }
    double su, sf;
    if (up) { su = (y[1] - y[0]) / (x[1] - x[0]); sf = (y[2] - y[1]) / (x[2] - x[1]); }
    else { su = (y[2] - y[1]) / (x[2] - x[1]); sf = (y[1] - y[0]) / (x[1] - x[0]); }
    const double h = mesh_dx(m, d, i[d] + hoff);
    double t;
    if (nd->field <= OPFLOW_FL_LUI) t = h * 0.5 * kappa_kernel(nd->field, su, sf);
    else {
        const double r = sf / (su + 1e-16);
        t = h * 0.5 * limiter(nd->field, r) * su;
    }
    return up ? y[1] + t : y[1] - t;
}

static double ev(Ctx* c, int k, const int* i) {
    const opflow_node* nd = &c->nodes[k];
    switch (nd->kind) {
        case OPFLOW_NODE_FIELD: return fget(&c->fields[nd->field], i);
        case OPFLOW_NODE_CONST: return nd->value;
        case OPFLOW_NODE_ADD: return ev(c, nd->a, i) + ev(c, nd->b, i);
        case OPFLOW_NODE_SUB: return ev(c, nd->a, i) - ev(c, nd->b, i);
        case OPFLOW_NODE_MUL: return ev(c, nd->a, i) * ev(c, nd->b, i);
        case OPFLOW_NODE_DIV: return ev(c, nd->a, i) / ev(c, nd->b, i);
        case OPFLOW_NODE_NEG: return -ev(c, nd->a, i);
        case OPFLOW_NODE_D2: { /* D2SecondOrderCentered::eval (D2SecondOrderCentered.hpp:160-171) */
            const int d = nd->dim, corner = c->loc[nd->a][d] == OPFLOW_CORNER;
            int ip[3] = {i[0], i[1], i[2]}, im[3] = {i[0], i[1], i[2]};
            ip[d]++; im[d]--;
            double l = ev(c, nd->a, im), ce = ev(c, nd->a, i), r = ev(c, nd->a, ip);
            const opflow_mesh_desc* m = c->m;
            double dxl = corner ? mesh_dx(m, d, i[d] - 1) : (mesh_dx(m, d, i[d] - 1) + mesh_dx(m, d, i[d])) * 0.5;
            double dxr = corner ? mesh_dx(m, d, i[d]) : (mesh_dx(m, d, i[d]) + mesh_dx(m, d, i[d] + 1)) * 0.5;
            double dxc = (dxl + dxr) * 0.5;
            return ((r - ce) / dxr - (ce - l) / dxl) / dxc;
        }
        case OPFLOW_NODE_D1: { /* D1FirstOrderCentered::eval (D1FirstOrderCentered.hpp:31-36) */
            const int d = nd->dim;
            int ip[3] = {i[0], i[1], i[2]}, im[3] = {i[0], i[1], i[2]};
            ip[d]++; im[d]--;
            if (c->loc[nd->a][d] == OPFLOW_CENTER)
                return (ev(c, nd->a, i) - ev(c, nd->a, im)) / (mesh_dx(c->m, d, i[d] - 1) + mesh_dx(c->m, d, i[d])) * 2;
            return (ev(c, nd->a, ip) - ev(c, nd->a, i)) / (mesh_dx(c->m, d, i[d]));
        }
        case OPFLOW_NODE_WENO53_DOWN: case OPFLOW_NODE_WENO53_UP: {
            const int d = nd->dim, up = nd->kind == OPFLOW_NODE_WENO53_UP;
            double v[6];
            for (int o = 0; o < 6; ++o) {
                int j[3] = {i[0], i[1], i[2]};
                j[d] += up ? (3 - o) : (o - 3); /* Upwind passes (pp3..pm2) in the kernel's pm3..pp2 slots */
                v[o] = ev(c, nd->a, j);
            }
            double h = mesh_dx(c->m, d, i[d]);
            /* Upwind's differences are the negated Downwind differences of the mirrored stencil, and
             * every operation of the kernel is odd in them, so the result is the exact negation. */
            double r = weno_kernel(v[0], v[1], v[2], v[3], v[4], v[5], h);
            return up ? -r : r;
        }
        case OPFLOW_NODE_INTP_C2C: { /* D1Linear<Cen2Cor>::eval (D1Linear.hpp:35-45) */
            const int d = nd->dim;
            int im[3] = {i[0], i[1], i[2]};
            im[d]--;
            double x1 = mesh_x(c->m, d, i[d] - 1) + 0.5 * mesh_dx(c->m, d, i[d] - 1);
            double x2 = mesh_x(c->m, d, i[d]) + 0.5 * mesh_dx(c->m, d, i[d]);
            double y1 = ev(c, nd->a, im), y2 = ev(c, nd->a, i);
            return intp_d(x1, y1, x2, y2, mesh_x(c->m, d, i[d]));
        }
        case OPFLOW_NODE_INTP_COR2CEN: { /* D1Linear<Cor2Cen>::eval: Math::mid(e(i), e(i+1)) (D1Linear.hpp:43-45) */
            int ip[3] = {i[0], i[1], i[2]};
            ip[nd->dim]++;
            return (ev(c, nd->a, i) + ev(c, nd->a, ip)) * 0.5;
        }
        case OPFLOW_NODE_D1_BIASED_UP: { /* D1FirstOrderBiasedUpwind::eval (D1FirstOrderBiasedUpwind.hpp:53-58) */
            const int d = nd->dim;
            int ip[3] = {i[0], i[1], i[2]};
            ip[d]++;
            const double h = c->loc[nd->a][d] == OPFLOW_CORNER ? mesh_dx(c->m, d, i[d])
                                                                : (mesh_dx(c->m, d, i[d]) + mesh_dx(c->m, d, i[d] + 1)) * 0.5;
            return (ev(c, nd->a, ip) - ev(c, nd->a, i)) / h;
        }
        case OPFLOW_NODE_D1_BIASED_DOWN: { /* D1FirstOrderBiasedDownwind::eval (D1FirstOrderBiasedDownwind.hpp:52-57) */
            const int d = nd->dim;
            int im[3] = {i[0], i[1], i[2]};
            im[d]--;
            const double h = c->loc[nd->a][d] == OPFLOW_CORNER ? mesh_dx(c->m, d, i[d] - 1)
                                                                : (mesh_dx(c->m, d, i[d] - 1) + mesh_dx(c->m, d, i[d])) * 0.5;
            return (ev(c, nd->a, i) - ev(c, nd->a, im)) / h;
        }
        case OPFLOW_NODE_GT: return ev(c, nd->a, i) > ev(c, nd->b, i) ? 1. : 0.;
        case OPFLOW_NODE_GE: return ev(c, nd->a, i) >= ev(c, nd->b, i) ? 1. : 0.;
        case OPFLOW_NODE_LT: return ev(c, nd->a, i) < ev(c, nd->b, i) ? 1. : 0.;
        case OPFLOW_NODE_LE: return ev(c, nd->a, i) <= ev(c, nd->b, i) ? 1. : 0.;
        case OPFLOW_NODE_NE: return ev(c, nd->a, i) != ev(c, nd->b, i) ? 1. : 0.;
        case OPFLOW_NODE_AND: return (ev(c, nd->a, i) != 0. && ev(c, nd->b, i) != 0.) ? 1. : 0.;
        case OPFLOW_NODE_OR: return (ev(c, nd->a, i) != 0. || ev(c, nd->b, i) != 0.) ? 1. : 0.;
        case OPFLOW_NODE_NOT: return ev(c, nd->a, i) == 0. ? 1. : 0.;
        case OPFLOW_NODE_COND: /* CondOp::eval (Conditional.hpp:35-40): only the taken branch */
            return ev(c, nd->a, i) != 0. ? ev(c, nd->b, i) : ev(c, nd->c, i);
        case OPFLOW_NODE_FUNC1: return func1(nd->field, ev(c, nd->a, i));
        case OPFLOW_NODE_FUNC2: { double a = ev(c, nd->a, i); return func2(nd->field, a, ev(c, nd->b, i)); }
        case OPFLOW_NODE_INTP_FL_CEN2COR: case OPFLOW_NODE_INTP_FL_COR2CEN: /* D1FluxLimiterImpl::eval */
            return ev(c, nd->a, i) > 0. ? flux_side(c, nd, i, 1) : flux_side(c, nd, i, 0);
    }
    return NAN;
}

static int setup_ctx(Ctx* c, const opflow_mesh_desc* m, const opflow_field_desc* descs, double** datas, int nf,
                     const opflow_node* nodes, int n, Field* fields) {
    memset(c, 0, sizeof *c);
    c->m = m; c->nodes = nodes; c->n = n; c->fields = fields; c->nf = nf; c->unknown = -1;
    if (n < 1) return fail(OPFLOW_E_INVALID, "empty expression");
    for (int k = 0; k < nf; ++k) {
        fields[k].d = &descs[k];
        fields[k].data = datas[k];
        int rc = or_field_info(m, &descs[k], &fields[k].r);
        if (rc) return rc;
    }
    return compute_locs(c);
}

/* dst[i] = expr(i) over a box; rows are independent, so the outer loop may run on several host threads
 * (the values do not depend on the thread count). */
static void eval_box(Ctx* c, int D, const int* lo, const int* hi, Field* dst) {
    const int outer = D == 3 ? 2 : (D == 2 ? 1 : 0);
#pragma omp parallel for schedule(static)
    for (int o = lo[outer]; o < hi[outer]; ++o) {
        int l2[3] = {lo[0], lo[1], lo[2]}, h2[3] = {hi[0], hi[1], hi[2]}, idx[3];
        l2[outer] = o;
        h2[outer] = o + 1;
        BOX_FOR(D, l2, h2, idx) fset(dst, idx, ev(c, c->n - 1, idx));
    }
}

/* internal::FieldAssigner::assign<Op> (FieldAssigner.hpp:27-84) followed by the updatePadding of
 * CartesianField::assignImpl_final (CartesianField.hpp:195-234).  `dst` is a slot of `datas`; when the
 * expression reads it, the evaluation goes to a temporary copy first, as the reference does. */
int or_assign(const opflow_mesh_desc* m, const opflow_field_desc* descs, double** datas, int nf, int dst, int arith,
              const opflow_node* nodes, int n) {
    Field fields[16];
    Ctx c;
    if (nf > 16 || dst < 0 || dst >= nf) return fail(OPFLOW_E_INVALID, "bad field slots");
    int rc = setup_ctx(&c, m, descs, datas, nf, nodes, n, fields);
    if (rc) return rc;
    Field* out = &fields[dst];
    int aliased = 0;
    for (int k = 0; k < n; ++k) aliased |= nodes[k].kind == OPFLOW_NODE_FIELD && nodes[k].field == dst;
    const opflow_field_info* R = &out->r;
    int lo[3], hi[3], idx[3];
    for (int d = 0; d < 3; ++d) {
        lo[d] = imax(R->assignable[d][0], R->local[d][0]);
        hi[d] = imin(R->assignable[d][1], R->local[d][1]);
    }
    double* tmp = NULL;
    g_range_err = 0;
    if (aliased) {
        /* temp = dst; assign_impl<Eq>(src, temp); assign_impl<Op>(temp, dst) */
        tmp = (double*) malloc(R->count * sizeof(double));
        if (!tmp) return fail(OPFLOW_E_NOMEM, "host allocation failed");
        memcpy(tmp, out->data, R->count * sizeof(double));
        Field t = *out;
        t.data = tmp;
        eval_box(&c, R->ndim, lo, hi, &t);
        update_padding(m, &t);
        BOX_FOR(R->ndim, lo, hi, idx) {
            double v = fget(&t, idx), o = fget(out, idx);
            switch (arith) {
                case OPFLOW_ASSIGN_EQ: o = v; break;
                case OPFLOW_ASSIGN_ADD: o += v; break;
                case OPFLOW_ASSIGN_SUB: o -= v; break;
                case OPFLOW_ASSIGN_MUL: o *= v; break;
                case OPFLOW_ASSIGN_DIV: o /= v; break;
            }
            fset(out, idx, o);
        }
        free(tmp);
    } else if (arith == OPFLOW_ASSIGN_EQ) {
        eval_box(&c, R->ndim, lo, hi, out);
    } else {
        BOX_FOR(R->ndim, lo, hi, idx) {
            double v = ev(&c, n - 1, idx), o = fget(out, idx);
            switch (arith) {
                case OPFLOW_ASSIGN_EQ: o = v; break;
                case OPFLOW_ASSIGN_ADD: o += v; break;
                case OPFLOW_ASSIGN_SUB: o -= v; break;
                case OPFLOW_ASSIGN_MUL: o *= v; break;
                case OPFLOW_ASSIGN_DIV: o /= v; break;
            }
            fset(out, idx, o);
        }
    }
    update_padding(m, out); /* assign_impl's dst.updatePadding() */
    update_padding(m, out); /* assignImpl_final's this->updatePadding() (idempotent) */
    return g_range_err ? fail(OPFLOW_E_RANGE, "stencil read outside a field's data array") : OPFLOW_OK;
}

/* ------------------------------------------------------------------------------------------------ */
/* StencilPad arithmetic (StencilPad.hpp:137-298) with fake_map insertion order (StencilPad.hpp:26-134) */
/* ------------------------------------------------------------------------------------------------ */
#define PADMAX 16
typedef struct {
    int n;
    int key[PADMAX][3];
    double val[PADMAX];
    double bias;
} Pad;
typedef struct {
    int is_pad;
    double v;
    Pad p;
} Val;

static int g_pad_err;
static int pad_find(const Pad* p, const int* k) {
    for (int e = 0; e < p->n; ++e)
        if (p->key[e][0] == k[0] && p->key[e][1] == k[1] && p->key[e][2] == k[2]) return e;
    return -1;
}
static double* pad_at(Pad* p, const int* k) { /* fake_map::operator[] (appends a missing key) */
    int e = pad_find(p, k);
    if (e >= 0) return &p->val[e];
    if (p->n >= PADMAX) { g_pad_err = 1; return &p->val[0]; }
    e = p->n++;
    memcpy(p->key[e], k, sizeof(int) * 3);
    p->val[e] = 0.;
    return &p->val[e];
}
static void pad_scale(Pad* p, double r) { /* operator*(pad, num) */
    for (int e = 0; e < p->n; ++e) p->val[e] *= r;
    p->bias *= r;
}
static void pad_add_assign(Pad* a, const Pad* b) { /* operator+=(pad) */
    for (int e = 0; e < b->n; ++e) {
        int f = pad_find(a, b->key[e]);
        if (f >= 0) a->val[f] += b->val[e];
        else *pad_at(a, b->key[e]) = b->val[e];
    }
    a->bias += b->bias;
}
static Val vnum(double v) { Val r; r.is_pad = 0; r.v = v; r.p.n = 0; r.p.bias = 0.; return r; }
static Val vpad_bias(double b) { Val r; r.is_pad = 1; r.v = 0.; r.p.n = 0; r.p.bias = b; return r; }

static Val v_add(Val a, Val b) {
    if (!a.is_pad && !b.is_pad) return vnum(a.v + b.v);
    if (a.is_pad && b.is_pad) { Val r = a; pad_add_assign(&r.p, &b.p); return r; }
    if (a.is_pad) { Val r = a; r.p.bias += b.v; return r; }       /* pad + num */
    Val r = b; r.p.bias += a.v; return r;                           /* num + pad: ret = b; ret += a */
}
static Val v_neg_scale(Val b) { Val r = b; pad_scale(&r.p, -1.0); return r; }
static Val v_sub(Val a, Val b) {
    if (!a.is_pad && !b.is_pad) return vnum(a.v - b.v);
    if (a.is_pad && b.is_pad) return v_add(a, v_neg_scale(b));      /* a + (b * -1.0) */
    if (a.is_pad) { Val r = a; r.p.bias += -b.v; return r; }      /* a + (-b) */
    return v_add(vpad_bias(a.v), v_neg_scale(b));                   /* StencilPad(a) - b */
}
static Val v_mul(Val a, Val b) {
    if (!a.is_pad && !b.is_pad) return vnum(a.v * b.v);
    if (a.is_pad && b.is_pad) { g_pad_err = 2; return a; }          /* nonlinear: not a linear equation */
    if (a.is_pad) { Val r = a; pad_scale(&r.p, b.v); return r; }
    Val r = b; pad_scale(&r.p, a.v); return r;
}
static Val v_div(Val a, Val b) {
    if (!a.is_pad && !b.is_pad) return vnum(a.v / b.v);
    if (b.is_pad) { g_pad_err = 2; return a; }
    Val r = a; pad_scale(&r.p, 1. / b.v); return r;                 /* a * (1. / b) */
}
static Val v_neg(Val a) { /* unary operator-: v = -v, bias = -bias */
    if (!a.is_pad) return vnum(-a.v);
    Val r = a;
    for (int e = 0; e < r.p.n; ++e) r.p.val[e] = -r.p.val[e];
    r.p.bias = -r.p.bias;
    return r;
}
static Val v_scal(Val a, double s) { /* double * pad or pad * double */
    if (!a.is_pad) return vnum(a.v * s);
    Val r = a; pad_scale(&r.p, s); return r;
}

/* StencilField::evalAtImpl_final (StencilField.hpp:123-350) */
static Val st_eval(Ctx* c, const int* idx) {
    const int D = c->m->ndim;
    const Field* base = &c->fields[c->unknown];
    int inA = 1, inL = 1;
    for (int d = 0; d < D; ++d) {
        inA &= c->st_assignable[d][0] <= idx[d] && idx[d] < c->st_assignable[d][1];
        inL &= c->st_logical[d][0] <= idx[d] && idx[d] < c->st_logical[d][1];
    }
    if (inA) {
        Val r = vpad_bias(0.);
        int pinned = c->pin;
        for (int d = 0; d < D; ++d) pinned &= idx[d] == c->pin_index[d];
        if (!pinned) {
            int k[3] = {idx[0], idx[1], idx[2]};
            *pad_at(&r.p, k) = 1.0;
        }
        return r;
    }
    if (!inL) { g_pad_err = 3; return vpad_bias(NAN); }
    const opflow_mesh_desc* m = c->m;
    /* case 1: fold an index outside the accessible range back into it */
    for (int i = 0; i < D; ++i) {
        if (c->st_accessible[i][0] <= idx[i] && idx[i] < c->st_accessible[i][1]) continue;
        const int lower = idx[i] < c->st_accessible[i][0];
        const int bct = base->d->bc_type[i][lower ? 0 : 1];
        const double bcv = base->d->bc_value[i][lower ? 0 : 1];
        int mi[3] = {idx[0], idx[1], idx[2]};
        const int as = c->st_accessible[i][0], ae = c->st_accessible[i][1];
        if (base->d->loc[i] == OPFLOW_CORNER) {
            mi[i] = lower ? 2 * as - idx[i] : 2 * ae - 2 - idx[i];
            switch (bct) {
                case OPFLOW_BC_DIRC: {
                    /* intp(x1, y1=bc pad, x2, y2=mirror pad, x): (x1'*y2 - x2'*y1) / (x1' - x2') in pad arithmetic */
                    double x1 = mesh_x(m, i, lower ? as : ae - 1) - mesh_x(m, i, idx[i]);
                    double x2 = mesh_x(m, i, mi[i]) - mesh_x(m, i, idx[i]);
                    Val y1 = vpad_bias(bcv), y2 = st_eval(c, mi);
                    return v_div(v_sub(v_scal(y2, x1), v_scal(y1, x2)), vnum(x1 - x2));
                }
                case OPFLOW_BC_NEUM:
                    return v_add(st_eval(c, mi), v_scal(vpad_bias(bcv), mesh_x(m, i, idx[i]) - mesh_x(m, i, mi[i])));
                case OPFLOW_BC_SYMM: return st_eval(c, mi);
                case OPFLOW_BC_ASYMM: return v_scal(st_eval(c, mi), -1.);
                case OPFLOW_BC_PERIODIC:
                    mi[i] = idx[i] + (lower ? (ae - as) : -(ae - as));
                    return st_eval(c, mi);
                default: g_pad_err = 4; return vpad_bias(NAN);
            }
        } else {
            mi[i] = lower ? 2 * as - 1 - idx[i] : 2 * ae - 1 - idx[i];
            switch (bct) {
                case OPFLOW_BC_DIRC: {
                    double xb = mesh_x(m, i, lower ? as : ae);
                    double xm = mesh_x(m, i, mi[i]) + mesh_dx(m, i, mi[i]) / 2.;
                    double xg = mesh_x(m, i, idx[i]) + mesh_dx(m, i, idx[i]) / 2.;
                    double x1 = xb - xg, x2 = xm - xg;
                    Val y1 = vpad_bias(bcv), y2 = st_eval(c, mi);
                    return v_div(v_sub(v_scal(y2, x1), v_scal(y1, x2)), vnum(x1 - x2));
                }
                case OPFLOW_BC_NEUM:
                    return v_add(st_eval(c, mi),
                                 v_scal(vpad_bias(bcv), mesh_x(m, i, idx[i]) + mesh_dx(m, i, idx[i]) / 2. - mesh_x(m, i, mi[i])
                                                                - mesh_dx(m, i, mi[i]) / 2.));
                case OPFLOW_BC_SYMM: return st_eval(c, mi);
                case OPFLOW_BC_ASYMM: return v_scal(st_eval(c, mi), -1.0);
                case OPFLOW_BC_PERIODIC:
                    mi[i] = idx[i] + (lower ? (ae - as) : -(ae - as));
                    return st_eval(c, mi);
                default: g_pad_err = 4; return vpad_bias(NAN);
            }
        }
    }
    /* case 2: the index sits on a Dirichlet boundary node */
    for (int i = 0; i < D; ++i) {
        if (base->d->loc[i] == OPFLOW_CORNER && base->d->bc_type[i][0] == OPFLOW_BC_DIRC && idx[i] == c->st_accessible[i][0])
            return vpad_bias(base->d->bc_value[i][0]);
        if (base->d->loc[i] == OPFLOW_CORNER && base->d->bc_type[i][1] == OPFLOW_BC_DIRC && idx[i] == c->st_accessible[i][1] - 1)
            return vpad_bias(base->d->bc_value[i][1]);
    }
    g_pad_err = 5;
    return vpad_bias(NAN);
}

static Val evp(Ctx* c, int k, const int* i) {
    const opflow_node* nd = &c->nodes[k];
    switch (nd->kind) {
        case OPFLOW_NODE_FIELD:
            if (nd->field == c->unknown) return st_eval(c, i);
            return vnum(fget(&c->fields[nd->field], i));
        case OPFLOW_NODE_CONST: return vnum(nd->value);
        case OPFLOW_NODE_ADD: { Val a = evp(c, nd->a, i); return v_add(a, evp(c, nd->b, i)); }
        case OPFLOW_NODE_SUB: { Val a = evp(c, nd->a, i); return v_sub(a, evp(c, nd->b, i)); }
        case OPFLOW_NODE_MUL: { Val a = evp(c, nd->a, i); return v_mul(a, evp(c, nd->b, i)); }
        case OPFLOW_NODE_DIV: { Val a = evp(c, nd->a, i); return v_div(a, evp(c, nd->b, i)); }
        case OPFLOW_NODE_NEG: return v_neg(evp(c, nd->a, i));
        case OPFLOW_NODE_D2: {
            const int d = nd->dim, corner = c->loc[nd->a][d] == OPFLOW_CORNER;
            int ip[3] = {i[0], i[1], i[2]}, im[3] = {i[0], i[1], i[2]};
            ip[d]++; im[d]--;
            Val l = evp(c, nd->a, im), ce = evp(c, nd->a, i), r = evp(c, nd->a, ip);
            const opflow_mesh_desc* m = c->m;
            double dxl = corner ? mesh_dx(m, d, i[d] - 1) : (mesh_dx(m, d, i[d] - 1) + mesh_dx(m, d, i[d])) * 0.5;
            double dxr = corner ? mesh_dx(m, d, i[d]) : (mesh_dx(m, d, i[d]) + mesh_dx(m, d, i[d] + 1)) * 0.5;
            double dxc = (dxl + dxr) * 0.5;
            return v_div(v_sub(v_div(v_sub(r, ce), vnum(dxr)), v_div(v_sub(ce, l), vnum(dxl))), vnum(dxc));
        }
        case OPFLOW_NODE_D1: {
            const int d = nd->dim;
            int ip[3] = {i[0], i[1], i[2]}, im[3] = {i[0], i[1], i[2]};
            ip[d]++; im[d]--;
            if (c->loc[nd->a][d] == OPFLOW_CENTER) {
                Val a = evp(c, nd->a, i), b = evp(c, nd->a, im);
                return v_mul(v_div(v_sub(a, b), vnum(mesh_dx(c->m, d, i[d] - 1) + mesh_dx(c->m, d, i[d]))), vnum(2));
            }
            Val a = evp(c, nd->a, ip), b = evp(c, nd->a, i);
            return v_div(v_sub(a, b), vnum(mesh_dx(c->m, d, i[d])));
        }
        case OPFLOW_NODE_INTP_C2C: {
            const int d = nd->dim;
            int im[3] = {i[0], i[1], i[2]};
            im[d]--;
            double x1 = mesh_x(c->m, d, i[d] - 1) + 0.5 * mesh_dx(c->m, d, i[d] - 1);
            double x2 = mesh_x(c->m, d, i[d]) + 0.5 * mesh_dx(c->m, d, i[d]);
            double x = mesh_x(c->m, d, i[d]);
            Val y1 = evp(c, nd->a, im), y2 = evp(c, nd->a, i);
            double a = x1 - x, b = x2 - x;
            return v_div(v_sub(v_scal(y2, a), v_scal(y1, b)), vnum(a - b));
        }
        case OPFLOW_NODE_INTP_COR2CEN: {
            int ip[3] = {i[0], i[1], i[2]};
            ip[nd->dim]++;
            Val a = evp(c, nd->a, i);
            return v_mul(v_add(a, evp(c, nd->a, ip)), vnum(0.5));
        }
        case OPFLOW_NODE_D1_BIASED_UP: case OPFLOW_NODE_D1_BIASED_DOWN: {
            const int d = nd->dim, up = nd->kind == OPFLOW_NODE_D1_BIASED_UP, o = up ? i[d] : i[d] - 1;
            int j[3] = {i[0], i[1], i[2]};
            j[d] += up ? 1 : -1;
            const double h = c->loc[nd->a][d] == OPFLOW_CORNER ? mesh_dx(c->m, d, o) : (mesh_dx(c->m, d, o) + mesh_dx(c->m, d, o + 1)) * 0.5;
            Val a = up ? evp(c, nd->a, j) : evp(c, nd->a, i);
            Val b = up ? evp(c, nd->a, i) : evp(c, nd->a, j);
            return v_div(v_sub(a, b), vnum(h));
        }
        case OPFLOW_NODE_GT: case OPFLOW_NODE_GE: case OPFLOW_NODE_LT: case OPFLOW_NODE_LE: case OPFLOW_NODE_NE:
        case OPFLOW_NODE_AND: case OPFLOW_NODE_OR: case OPFLOW_NODE_NOT: case OPFLOW_NODE_COND:
        case OPFLOW_NODE_FUNC1: case OPFLOW_NODE_FUNC2: {
            /* scalar-valued operators: defined on numbers only (a StencilPad operand has no linear form) */
            Val a = evp(c, nd->a, i);
            Val b = nd->b >= 0 ? evp(c, nd->b, i) : vnum(0.);
            Val t = nd->kind == OPFLOW_NODE_COND ? evp(c, nd->c, i) : vnum(0.);
            if (a.is_pad || b.is_pad || t.is_pad) { g_pad_err = 2; return vnum(NAN); }
            switch (nd->kind) {
                case OPFLOW_NODE_GT: return vnum(a.v > b.v ? 1. : 0.);
                case OPFLOW_NODE_GE: return vnum(a.v >= b.v ? 1. : 0.);
                case OPFLOW_NODE_LT: return vnum(a.v < b.v ? 1. : 0.);
                case OPFLOW_NODE_LE: return vnum(a.v <= b.v ? 1. : 0.);
                case OPFLOW_NODE_NE: return vnum(a.v != b.v ? 1. : 0.);
                case OPFLOW_NODE_AND: return vnum((a.v != 0. && b.v != 0.) ? 1. : 0.);
                case OPFLOW_NODE_OR: return vnum((a.v != 0. || b.v != 0.) ? 1. : 0.);
                case OPFLOW_NODE_NOT: return vnum(a.v == 0. ? 1. : 0.);
                case OPFLOW_NODE_COND: return a.v != 0. ? b : t;
                case OPFLOW_NODE_FUNC1: return vnum(func1(nd->field, a.v));
                default: return vnum(func2(nd->field, a.v, b.v));
            }
        }
        default:
            /* WENO and the other nonlinear operators have no StencilPad form */
            g_pad_err = 2;
            return vnum(NAN);
    }
}

/* HYPREEqnSolveHandler::initStencil + generateAb (HYPREEqnSolveHandler.hpp:79-166) with the
 * HYPRE_Struct*SetValues calls replaced by writes into coef[cell][entry] / rhs[cell]. */
int or_assemble(const opflow_mesh_desc* m, const opflow_field_desc* descs, double** datas, int nf, int target,
                const opflow_node* nodes, int n, int pin, int* n_entries, int* offsets, double* coef, double* rhs,
                size_t* n_cells) {
    Field fields[16];
    Ctx c;
    if (nf > 16 || target < 0 || target >= nf) return fail(OPFLOW_E_INVALID, "bad field slots");
    int rc = setup_ctx(&c, m, descs, datas, nf, nodes, n, fields);
    if (rc) return rc;
    c.unknown = target;
    c.pin = pin;
    const Field* T = &fields[target];
    const int D = m->ndim;
    for (int d = 0; d < 3; ++d) {
        for (int s = 0; s < 2; ++s) {
            c.st_assignable[d][s] = T->r.assignable[d][s];
            c.st_accessible[d][s] = T->r.accessible[d][s];
            c.st_logical[d][s] = T->r.logical[d][s];
        }
        c.pin_index[d] = T->r.assignable[d][0];
        /* ignorePeriodicBC (StencilField.hpp:112-121) */
        if (d < D && T->d->bc_type[d][0] == OPFLOW_BC_PERIODIC)
            for (int s = 0; s < 2; ++s) c.st_assignable[d][s] = c.st_accessible[d][s] = T->r.logical[d][s];
    }
    int lo[3], hi[3], mid[3] = {0, 0, 0}, idx[3];
    size_t cells = 1;
    for (int d = 0; d < 3; ++d) {
        lo[d] = imax(T->r.assignable[d][0], T->r.local[d][0]);
        hi[d] = imin(T->r.assignable[d][1], T->r.local[d][1]);
        if (d < D) mid[d] = (T->r.assignable[d][0] + T->r.assignable[d][1]) / 2;
        cells *= (size_t) (hi[d] - lo[d]);
    }
    g_pad_err = 0;
    g_range_err = 0;
    /* commStencil: the middle cell's pad, offset to the middle (lines 97-107) */
    Val vm = evp(&c, n - 1, mid);
    if (!vm.is_pad) return fail(OPFLOW_E_INVALID, "the equation does not contain the unknown");
    Pad comm = vm.p;
    for (int e = 0; e < comm.n; ++e)
        for (int d = 0; d < 3; ++d) comm.key[e][d] -= mid[d];
    *n_entries = comm.n;
    *n_cells = cells;
    if (g_pad_err) return fail(OPFLOW_E_UNSUPPORTED, "equation is not linear in the unknown or leaves the logical range");
    if (!coef) return OPFLOW_OK;
    if (offsets)
        for (int e = 0; e < comm.n; ++e)
            for (int d = 0; d < D; ++d) offsets[e * D + d] = comm.key[e][d];
    /* cells are independent: the outermost dimension's slabs run on several host threads (the values
     * do not depend on the thread count; each slab writes its own rows of coef and rhs) */
    const int outer = D - 1;
    size_t slab = 1;
    for (int d = 0; d < outer; ++d) slab *= (size_t) (hi[d] - lo[d]);
#pragma omp parallel for schedule(static)
    for (int o = lo[outer]; o < hi[outer]; ++o) {
        int l2[3] = {lo[0], lo[1], lo[2]}, h2[3] = {hi[0], hi[1], hi[2]}, ix[3];
        l2[outer] = o;
        h2[outer] = o + 1;
        size_t cell = (size_t) (o - lo[outer]) * slab;
        BOX_FOR(D, l2, h2, ix) {
            Val v = evp(&c, n - 1, ix);
            Pad cur = v.p;
            for (int e = 0; e < cur.n; ++e)
                for (int d = 0; d < 3; ++d) cur.key[e][d] -= ix[d];
            for (int e = 0; e < comm.n; ++e) {
                int f = pad_find(&cur, comm.key[e]);
                double x = f >= 0 ? cur.val[f] : 0.;
                coef[cell * comm.n + e] = x == 0. ? 0. : x; /* +0 for -0 */
            }
            rhs[cell] = -cur.bias;
            ++cell;
        }
    }
    (void) idx;
    if (pin) {
        /* the first unknown's row: identity, rhs 0 (lines 145-163) */
        for (int e = 0; e < comm.n; ++e) {
            int centre = comm.key[e][0] == 0 && comm.key[e][1] == 0 && comm.key[e][2] == 0;
            coef[e] = centre ? 1.0 : 0.0;
        }
        rhs[0] = 0.;
    }
    if (g_pad_err || g_range_err) return fail(OPFLOW_E_UNSUPPORTED, "assembly failed (nonlinear term or out-of-range read)");
    return OPFLOW_OK;
}

/* ------------------------------------------------------------------------------------------------ */
/* FP64 reference solve of an assembled structured system (the checker for the GPU solvers):        */
/* conjugate gradients with a Jacobi preconditioner, periodic offsets wrapped like HYPRE's periodic  */
/* grid.  coef is [cell][entry] over the box `dims`, x fastest.                                      */
/* ------------------------------------------------------------------------------------------------ */
static void or_matvec(int D, const int* dims, const int* periodic, int ne, const int* off, const double* coef,
                      const double* x, double* y) {
    size_t n = (size_t) dims[0] * dims[1] * dims[2];
    for (size_t c = 0; c < n; ++c) {
        int i[3] = {(int) (c % dims[0]), (int) ((c / dims[0]) % dims[1]), (int) (c / ((size_t) dims[0] * dims[1]))};
        double s = 0.;
        for (int e = 0; e < ne; ++e) {
            int j[3] = {i[0], i[1], i[2]}, ok = 1;
            for (int d = 0; d < D; ++d) {
                j[d] += off[e * D + d];
                if (j[d] < 0 || j[d] >= dims[d]) {
                    if (periodic[d]) j[d] = (j[d] % dims[d] + dims[d]) % dims[d];
                    else ok = 0;
                }
            }
            if (!ok) continue;
            s += coef[c * ne + e] * x[((size_t) j[2] * dims[1] + j[1]) * dims[0] + j[0]];
        }
        y[c] = s;
    }
}

double or_residual(int D, const int* dims, const int* periodic, int ne, const int* off, const double* coef,
                   const double* rhs, const double* x, double* bnorm_out) {
    size_t n = (size_t) dims[0] * dims[1] * dims[2];
    double* y = (double*) malloc(n * sizeof(double));
    or_matvec(D, dims, periodic, ne, off, coef, x, y);
    double rr = 0., bb = 0.;
    for (size_t c = 0; c < n; ++c) {
        double r = rhs[c] - y[c];
        rr += r * r;
        bb += rhs[c] * rhs[c];
    }
    free(y);
    if (bnorm_out) *bnorm_out = sqrt(bb);
    return sqrt(rr);
}

int or_pcg(int D, const int* dims_in, const int* periodic, int ne, const int* off, const double* coef, const double* rhs,
           double* x, double tol, int maxit, int* iters, double* relres) {
    int dims[3] = {dims_in[0], D > 1 ? dims_in[1] : 1, D > 2 ? dims_in[2] : 1};
    size_t n = (size_t) dims[0] * dims[1] * dims[2];
    int ci = -1;
    for (int e = 0; e < ne; ++e) {
        int z = 1;
        for (int d = 0; d < D; ++d) z &= off[e * D + d] == 0;
        if (z) ci = e;
    }
    if (ci < 0) return fail(OPFLOW_E_INVALID, "stencil has no centre entry");
    double *r = malloc(n * 8), *z = malloc(n * 8), *p = malloc(n * 8), *q = malloc(n * 8);
    or_matvec(D, dims, periodic, ne, off, coef, x, q);
    double bb = 0., rz = 0.;
    for (size_t c = 0; c < n; ++c) {
        r[c] = rhs[c] - q[c];
        bb += rhs[c] * rhs[c];
    }
    double bn = sqrt(bb) > 0 ? sqrt(bb) : 1.;
    for (size_t c = 0; c < n; ++c) { z[c] = r[c] / coef[c * ne + ci]; p[c] = z[c]; rz += r[c] * z[c]; }
    int it = 0;
    double rn = 0.;
    for (; it < maxit; ++it) {
        rn = 0.;
        for (size_t c = 0; c < n; ++c) rn += r[c] * r[c];
        if (sqrt(rn) / bn <= tol) break;
        or_matvec(D, dims, periodic, ne, off, coef, p, q);
        double pq = 0.;
        for (size_t c = 0; c < n; ++c) pq += p[c] * q[c];
        double al = rz / pq;
        for (size_t c = 0; c < n; ++c) { x[c] += al * p[c]; r[c] -= al * q[c]; }
        double rz2 = 0.;
        for (size_t c = 0; c < n; ++c) { z[c] = r[c] / coef[c * ne + ci]; rz2 += r[c] * z[c]; }
        double be = rz2 / rz;
        rz = rz2;
        for (size_t c = 0; c < n; ++c) p[c] = z[c] + be * p[c];
    }
    *iters = it;
    *relres = or_residual(D, dims, periodic, ne, off, coef, rhs, x, NULL) / bn;
    free(r); free(z); free(p); free(q);
    return OPFLOW_OK;
}

/* ------------------------------------------------------------------------------------------------ */
/* The reference's CPU solve of an assembled structured system, restated: HYPRE Struct PCG           */
/* (external/hypre/src/krylov/pcg.c:318-830, two-norm stopping test) preconditioned by PFMG          */
/* (struct_ls/pfmg_setup.c:63-720, pfmg_setup_interp.c:290-410, pfmg_setup_rap.c (Galerkin R A P    */
/* with R = P^T, pfmg_setup.c:416-427), pfmg_solve.c:31-340, pfmg_relax.c (weighted Jacobi),        */
/* semi_restrict.c, semi_interp.c).  It is the CPU baseline the benchmark times when the reference    */
/* itself (OpFlow + vendored HYPRE) is not built on the host, and the tests check it against the      */
/* fixtures HYPRE produced (iteration counts, residuals, solutions).                                  */
/*                                                                                                    */
/* PFMG as restated: semicoarsening by 2 in one direction per level (coarse points at even indices),  */
/* the direction with the smallest "dxyz" (from the operator's mean off-diagonal couplings,           */
/* pfmg_setup.c:765-895), dxyz doubled in that direction per level, until every extent is 1;         */
/* operator-dependent 1D interpolation at the fine (odd) points, P = -(A_left|A_right collapsed) /    */
/* (A collapsed centre), set to 0 where the direct neighbour coefficient is 0; restriction P^T;      */
/* coarse operator P^T A P; weighted Jacobi with the weight 2/(3 - beta/alpha) (2/3 when the          */
/* coefficients vary by more than 10 % or in 1D), one pre- and one post-sweep, relaxation skipped on */
/* levels not coarsened before in the same direction (skip_relax = 1); the coarsest level: plain     */
/* Jacobi, min(4 * levels, extent) sweeps.  Stencils of radius 1 only; no periodic directions.       */
/* Reentrant (no globals); `threads` host threads share each loop (the sums of a dot product are     */
/* then split by thread, so the last bits may depend on the thread count, as in HYPRE with OpenMP).   */
/* ------------------------------------------------------------------------------------------------ */
typedef struct {
    int n[3];          /* points per dim (1 beyond ndim)                                  */
    int g[3];          /* ghosted extents n + 2 (dims < ndim), 1 otherwise                */
    size_t G;          /* ghosted vector length                                           */
    int ne;            /* stencil entries                                                 */
    int off[27][3];    /* their offsets                                                   */
    long long lo[27];  /* their linear offsets in the ghosted layout                      */
    double* A;         /* [interior cell][ne], interior cells x fastest                   */
    double* diag;      /* centre coefficient per interior cell                            */
    double *x, *b, *r; /* ghosted vectors (ghosts stay 0)                                 */
    double *p0, *p1;   /* interpolation weights per interior cell (used at odd cdir index) */
    int cdir, active;
    double w;
    int nt;            /* host threads for this level's loops                             */
} PfLvl;

typedef struct {
    int D, nl;
    PfLvl L[64];
    double* t; /* scratch for Jacobi, ghosted, level 0 size */
} Pfmg;

static inline long long pf_lin(const PfLvl* l, int i, int j, int k) {
    return ((long long) (k + (l->g[2] > 1)) * l->g[1] + (j + (l->g[1] > 1))) * l->g[0] + (i + 1);
}

static void pf_geom(PfLvl* l, int D, const int* n) {
    l->G = 1;
    for (int d = 0; d < 3; ++d) {
        l->n[d] = d < D ? n[d] : 1;
        l->g[d] = d < D ? n[d] + 2 : 1;
        l->G *= (size_t) l->g[d];
    }
}

static void pf_set_offsets(PfLvl* l) {
    for (int e = 0; e < l->ne; ++e)
        l->lo[e] = ((long long) l->off[e][2] * l->g[1] + l->off[e][1]) * l->g[0] + l->off[e][0];
}

/* y = A x over the interior (ghost x are 0, so boundary rows need no test) */
static void pf_matvec(const PfLvl* l, const double* x, double* y) {
    const long long rows = (long long) l->n[1] * l->n[2];
#pragma omp parallel for schedule(static) num_threads(l->nt) if (l->nt > 1)
    for (long long row = 0; row < rows; ++row) {
        const int j = (int) (row % l->n[1]), k = (int) (row / l->n[1]);
        size_t c = (size_t) row * l->n[0];
        long long q = pf_lin(l, 0, j, k);
        for (int i = 0; i < l->n[0]; ++i, ++q, ++c) {
            const double* a = l->A + c * l->ne;
            double s = 0.;
            for (int e = 0; e < l->ne; ++e) s += a[e] * x[q + l->lo[e]];
            y[q] = s;
        }
    }
}

/* r = b - A x */
static void pf_residual(const PfLvl* l, const double* x, const double* b, double* r) {
    const long long rows = (long long) l->n[1] * l->n[2];
#pragma omp parallel for schedule(static) num_threads(l->nt) if (l->nt > 1)
    for (long long row = 0; row < rows; ++row) {
        const int j = (int) (row % l->n[1]), k = (int) (row / l->n[1]);
        size_t c = (size_t) row * l->n[0];
        long long q = pf_lin(l, 0, j, k);
        for (int i = 0; i < l->n[0]; ++i, ++q, ++c) {
            const double* a = l->A + c * l->ne;
            double s = 0.;
            for (int e = 0; e < l->ne; ++e) s += a[e] * x[q + l->lo[e]];
            r[q] = b[q] - s;
        }
    }
}

/* weighted Jacobi (pfmg_relax.c / point_relax.c): x += w D^-1 (b - A x); zero guess: x = w D^-1 b */
static void pf_relax(const PfLvl* l, double* x, const double* b, double* t, double w, int sweeps, int zero_guess) {
    const long long rows = (long long) l->n[1] * l->n[2];
    for (int s = 0; s < sweeps; ++s) {
        if (zero_guess && s == 0) {
#pragma omp parallel for schedule(static) num_threads(l->nt) if (l->nt > 1)
            for (long long row = 0; row < rows; ++row) {
                const int j = (int) (row % l->n[1]), k = (int) (row / l->n[1]);
                size_t c = (size_t) row * l->n[0];
                long long q = pf_lin(l, 0, j, k);
                for (int i = 0; i < l->n[0]; ++i, ++q, ++c) x[q] = l->diag[c] != 0. ? w * b[q] / l->diag[c] : 0.;
            }
            continue;
        }
        pf_residual(l, x, b, t);
#pragma omp parallel for schedule(static) num_threads(l->nt) if (l->nt > 1)
        for (long long row = 0; row < rows; ++row) {
            const int j = (int) (row % l->n[1]), k = (int) (row / l->n[1]);
            size_t c = (size_t) row * l->n[0];
            long long q = pf_lin(l, 0, j, k);
            for (int i = 0; i < l->n[0]; ++i, ++q, ++c)
                if (l->diag[c] != 0.) x[q] += w * t[q] / l->diag[c];
        }
    }
}

static int pf_find(const PfLvl* l, int ox, int oy, int oz) {
    for (int e = 0; e < l->ne; ++e)
        if (l->off[e][0] == ox && l->off[e][1] == oy && l->off[e][2] == oz) return e;
    return -1;
}

/* interpolation weights at every point (pfmg_setup_interp.c:325-410): collapse the stencil onto the
 * coarsening direction; p0 weighs the coarse point below, p1 the one above */
static void pf_interp_weights(PfLvl* l, int cdir) {
    int dn[3] = {0, 0, 0}, up[3] = {0, 0, 0};
    dn[cdir] = -1;
    up[cdir] = 1;
    const int s0 = pf_find(l, dn[0], dn[1], dn[2]), s1 = pf_find(l, up[0], up[1], up[2]);
    const long long N = (long long) l->n[0] * l->n[1] * l->n[2];
#pragma omp parallel for schedule(static) num_threads(l->nt) if (l->nt > 1)
    for (long long c = 0; c < N; ++c) {
        const double* a = l->A + c * l->ne;
        double center = 0., w0 = 0., w1 = 0.;
        for (int e = 0; e < l->ne; ++e) {
            const int o = l->off[e][cdir];
            if (o == 0) center += a[e];
            else if (o == -1) w0 -= a[e];
            else w1 -= a[e];
        }
        if (center == 0.) w0 = w1 = 0.;
        else {
            w0 /= center;
            w1 /= center;
        }
        if (s0 < 0 || a[s0] == 0.) w0 = 0.;
        if (s1 < 0 || a[s1] == 0.) w1 = 0.;
        l->p0[c] = w0;
        l->p1[c] = w1;
    }
}

static inline size_t pf_cell(const PfLvl* l, int i, int j, int k) { return ((size_t) k * l->n[1] + j) * l->n[0] + i; }

/* coarse operator R A P with R = P^T (the Galerkin product of pfmg_setup_rap.c for rap_type 0) */
static int pf_rap(const PfLvl* f, PfLvl* c, int cdir, int D) {
    /* the coarse pattern: offsets reachable through R (cdir -1..1), A (f's offsets) and P */
    int mark[27] = {0};
    for (int a = -1; a <= 1; ++a)
        for (int e = 0; e < f->ne; ++e) {
            const int t = a + f->off[e][cdir];
            int ks[2], nk = 0;
            if ((t & 1) == 0) ks[nk++] = t / 2;
            else {
                ks[nk++] = (t - 1) / 2;
                ks[nk++] = (t + 1) / 2;
            }
            for (int q = 0; q < nk; ++q) {
                int o[3] = {f->off[e][0], f->off[e][1], f->off[e][2]};
                o[cdir] = ks[q];
                if (o[cdir] < -1 || o[cdir] > 1) continue;
                mark[((o[2] + 1) * 3 + (o[1] + 1)) * 3 + (o[0] + 1)] = 1;
            }
        }
    c->ne = 0;
    int slot[27];
    for (int m = 0; m < 27; ++m) {
        slot[m] = -1;
        if (!mark[m]) continue;
        const int ox = m % 3 - 1, oy = (m / 3) % 3 - 1, oz = m / 9 - 1;
        if ((D < 2 && oy) || (D < 3 && oz)) continue;
        slot[m] = c->ne;
        c->off[c->ne][0] = ox;
        c->off[c->ne][1] = oy;
        c->off[c->ne][2] = oz;
        c->ne++;
    }
    pf_set_offsets(c);
    const size_t Nc = (size_t) c->n[0] * c->n[1] * c->n[2];
    c->A = (double*) calloc(Nc * c->ne, sizeof(double));
    if (!c->A) return 1;
    const long long crows = (long long) c->n[1] * c->n[2];
#pragma omp parallel for schedule(static) num_threads(f->nt) if (f->nt > 1)
    for (long long row = 0; row < crows; ++row)
        for (int i0 = 0; i0 < c->n[0]; ++i0) {
                const int I[3] = {i0, (int) (row % c->n[1]), (int) (row / c->n[1])};
                double* ac = c->A + pf_cell(c, I[0], I[1], I[2]) * c->ne;
                for (int a = -1; a <= 1; ++a) {
                    int f1[3] = {I[0], I[1], I[2]};
                    f1[cdir] = 2 * I[cdir] + a;
                    if (f1[cdir] < 0 || f1[cdir] >= f->n[cdir]) continue;
                    const size_t c1 = pf_cell(f, f1[0], f1[1], f1[2]);
                    /* R(I, f1): 1 at the coarse point; the F point's weight towards I otherwise */
                    const double ra = a == 0 ? 1. : (a == 1 ? f->p0[c1] : f->p1[c1]);
                    if (ra == 0.) continue;
                    const double* af = f->A + c1 * f->ne;
                    for (int e = 0; e < f->ne; ++e) {
                        if (af[e] == 0.) continue;
                        int f2[3] = {f1[0] + f->off[e][0], f1[1] + f->off[e][1], f1[2] + f->off[e][2]};
                        int out = 0;
                        for (int d = 0; d < 3; ++d) out |= f2[d] < 0 || f2[d] >= f->n[d];
                        if (out) continue;
                        const int t = f2[cdir];
                        int ks[2], nk = 0;
                        double wk[2];
                        if ((t & 1) == 0) {
                            ks[nk] = t / 2;
                            wk[nk++] = 1.;
                        } else {
                            const size_t c2 = pf_cell(f, f2[0], f2[1], f2[2]);
                            ks[nk] = (t - 1) / 2;
                            wk[nk++] = f->p0[c2];
                            ks[nk] = (t + 1) / 2;
                            wk[nk++] = f->p1[c2];
                        }
                        for (int q = 0; q < nk; ++q) {
                            if (wk[q] == 0.) continue;
                            int o[3] = {f2[0] - I[0], f2[1] - I[1], f2[2] - I[2]};
                            o[cdir] = ks[q] - I[cdir];
                            const int m = ((o[2] + 1) * 3 + (o[1] + 1)) * 3 + (o[0] + 1);
                            ac[slot[m]] += ra * af[e] * wk[q];
                        }
                    }
                }
            }
    return 0;
}

static void pf_free(Pfmg* P) {
    for (int l = 0; l < P->nl; ++l) {
        free(P->L[l].A);
        free(P->L[l].diag);
        free(P->L[l].x);
        free(P->L[l].b);
        free(P->L[l].r);
        free(P->L[l].p0);
        free(P->L[l].p1);
    }
    free(P->t);
}

static int pf_alloc_vectors(PfLvl* l) {
    const size_t N = (size_t) l->n[0] * l->n[1] * l->n[2];
    l->x = (double*) calloc(l->G, 8);
    l->b = (double*) calloc(l->G, 8);
    l->r = (double*) calloc(l->G, 8);
    l->p0 = (double*) calloc(N, 8);
    l->p1 = (double*) calloc(N, 8);
    l->diag = (double*) calloc(N, 8);
    if (!l->x || !l->b || !l->r || !l->p0 || !l->p1 || !l->diag) return 1;
    const int ce = pf_find(l, 0, 0, 0);
    for (size_t c = 0; c < N; ++c) l->diag[c] = ce >= 0 ? l->A[c * l->ne + ce] : 0.;
    return 0;
}

/* hypre_PFMGComputeDxyz (pfmg_setup.c:765-895, the 5/7-point branches generalised to any radius-1
 * stencil): per direction the mean and mean square of -sign(diag) * (sum of the couplings along it) */
static int pf_dxyz(const PfLvl* l, int D, double* dxyz) {
    double cx[3] = {0, 0, 0}, sq[3] = {0, 0, 0};
    const size_t N = (size_t) l->n[0] * l->n[1] * l->n[2];
    for (size_t c = 0; c < N; ++c) {
        const double* a = l->A + c * l->ne;
        const double sg = l->diag[c] < 0. ? -1. : 1.;
        for (int d = 0; d < D; ++d) {
            double t = 0.;
            for (int e = 0; e < l->ne; ++e) {
                int only = l->off[e][d] != 0;
                for (int q = 0; q < 3; ++q)
                    if (q != d && l->off[e][q] != 0) only = 0;
                if (only) t += a[e];
            }
            t = -sg * t;
            cx[d] += t;
            sq[d] += t * t;
        }
    }
    int flag = 0;
    for (int d = 0; d < D; ++d) {
        const double mean = cx[d] / (double) N, dev = sq[d] / (double) N - mean * mean;
        if (dev > 0.1 * mean * mean) flag = 1;
    }
    double mx = 0.;
    for (int d = 0; d < D; ++d) mx = cx[d] > mx ? cx[d] : mx;
    if (mx == 0.) {
        for (int d = 0; d < D; ++d) cx[d] = 1.;
        mx = 1.;
    }
    for (int d = 0; d < 3; ++d) {
        if (d >= D) {
            dxyz[d] = 1.;
            continue;
        }
        const double maxan = 1.7976931348623157e308 / 1000.;
        if (cx[d] > mx / maxan) dxyz[d] = sqrt(1. / (cx[d] / mx));
        else dxyz[d] = sqrt(maxan);
    }
    return flag;
}

static int pf_setup(Pfmg* P, int D, const int* dims, int ne, const int* off, const double* coef, int nt) {
    memset(P, 0, sizeof *P);
    P->D = D;
    for (int l = 0; l < 64; ++l) P->L[l].nt = nt;
    PfLvl* l0 = &P->L[0];
    pf_geom(l0, D, dims);
    l0->ne = ne;
    for (int e = 0; e < ne; ++e)
        for (int d = 0; d < 3; ++d) {
            l0->off[e][d] = d < D ? off[e * D + d] : 0;
            if (l0->off[e][d] < -1 || l0->off[e][d] > 1) return 2;
        }
    pf_set_offsets(l0);
    const size_t N0 = (size_t) l0->n[0] * l0->n[1] * l0->n[2];
    l0->A = (double*) malloc(N0 * ne * 8);
    if (!l0->A) return 1;
    memcpy(l0->A, coef, N0 * ne * 8);
    P->nl = 1;
    if (pf_alloc_vectors(l0)) return 1;
    P->t = (double*) calloc(l0->G, 8);
    if (!P->t) return 1;
    double dxyz[3];
    const int dflag = pf_dxyz(l0, D, dxyz);
    int coarsen[3] = {1, 1, 1};
    for (int l = 0;; ++l) {
        PfLvl* L = &P->L[l];
        double mn = dxyz[0] + dxyz[1] + dxyz[2] + 1, alpha = 0., beta = 0.;
        int cdir = -1;
        for (int d = 0; d < D; ++d) {
            if (L->n[d] > 1 && dxyz[d] < mn) {
                mn = dxyz[d];
                cdir = d;
            }
            alpha += 1. / (dxyz[d] * dxyz[d]);
        }
        L->w = 1.;
        if (cdir != -1) {
            if (dflag) L->w = 2. / 3.;
            else {
                for (int d = 0; d < D; ++d)
                    if (d != cdir) beta += 1. / (dxyz[d] * dxyz[d]);
                alpha = beta == alpha ? 0. : beta / alpha;
                L->w = D > 1 ? 2. / (3. - alpha) : 2. / 3.;
            }
        }
        if (cdir != -1 && l == 63) cdir = -1;
        if (cdir == -1) {
            L->active = 1;
            L->cdir = -1;
            break;
        }
        L->cdir = cdir;
        if (coarsen[cdir]) {
            L->active = 1;
            coarsen[0] = coarsen[1] = coarsen[2] = 0;
            coarsen[cdir] = 1;
        } else {
            L->active = 0;
            coarsen[cdir] = 1;
        }
        dxyz[cdir] *= 2;
        pf_interp_weights(L, cdir);
        PfLvl* C = &P->L[l + 1];
        int nc[3] = {L->n[0], L->n[1], L->n[2]};
        nc[cdir] = (L->n[cdir] + 1) / 2;
        pf_geom(C, D, nc);
        P->nl = l + 2;
        if (pf_rap(L, C, cdir, D)) return 1;
        if (pf_alloc_vectors(C)) return 1;
    }
    return 0;
}

/* semi_restrict.c: b_c(I) = r(2I) + p0(2I+1) r(2I+1) + p1(2I-1) r(2I-1) along cdir */
static void pf_restrict(const PfLvl* f, PfLvl* c, int cdir) {
    const long long crows = (long long) c->n[1] * c->n[2];
#pragma omp parallel for schedule(static) num_threads(f->nt) if (f->nt > 1)
    for (long long row = 0; row < crows; ++row)
        for (int i0 = 0; i0 < c->n[0]; ++i0) {
                const int I[3] = {i0, (int) (row % c->n[1]), (int) (row / c->n[1])};
                int F[3] = {I[0], I[1], I[2]};
                F[cdir] = 2 * I[cdir];
                double s = f->r[pf_lin(f, F[0], F[1], F[2])];
                if (F[cdir] + 1 < f->n[cdir]) {
                    int G[3] = {F[0], F[1], F[2]};
                    G[cdir] += 1;
                    s += f->p0[pf_cell(f, G[0], G[1], G[2])] * f->r[pf_lin(f, G[0], G[1], G[2])];
                }
                if (F[cdir] - 1 >= 0) {
                    int G[3] = {F[0], F[1], F[2]};
                    G[cdir] -= 1;
                    s += f->p1[pf_cell(f, G[0], G[1], G[2])] * f->r[pf_lin(f, G[0], G[1], G[2])];
                }
                c->b[pf_lin(c, I[0], I[1], I[2])] = s;
            }
}

/* semi_interp.c + the correction: x(2I) += x_c(I); x(2I+1) += p0 x_c(I) + p1 x_c(I+1) */
static void pf_interp_add(PfLvl* f, const PfLvl* c, int cdir) {
    const long long frows = (long long) f->n[1] * f->n[2];
#pragma omp parallel for schedule(static) num_threads(f->nt) if (f->nt > 1)
    for (long long row = 0; row < frows; ++row)
        for (int i0 = 0; i0 < f->n[0]; ++i0) {
                const int F[3] = {i0, (int) (row % f->n[1]), (int) (row / f->n[1])};
                int I[3] = {F[0], F[1], F[2]};
                const int t = F[cdir];
                double e;
                if ((t & 1) == 0) {
                    I[cdir] = t / 2;
                    e = c->x[pf_lin(c, I[0], I[1], I[2])];
                } else {
                    const size_t cf = pf_cell(f, F[0], F[1], F[2]);
                    I[cdir] = (t - 1) / 2;
                    e = f->p0[cf] * c->x[pf_lin(c, I[0], I[1], I[2])];
                    if ((t + 1) / 2 < c->n[cdir]) {
                        I[cdir] = (t + 1) / 2;
                        e += f->p1[cf] * c->x[pf_lin(c, I[0], I[1], I[2])];
                    }
                }
                f->x[pf_lin(f, F[0], F[1], F[2])] += e;
            }
}

static double pf_dot(const PfLvl* l, const double* u, const double* v) {
    double s = 0.;
    const long long rows = (long long) l->n[1] * l->n[2];
#pragma omp parallel for schedule(static) reduction(+ : s) num_threads(l->nt) if (l->nt > 1)
    for (long long row = 0; row < rows; ++row) {
        const int j = (int) (row % l->n[1]), k = (int) (row / l->n[1]);
        long long q = pf_lin(l, 0, j, k);
        for (int i = 0; i < l->n[0]; ++i, ++q) s += u[q] * v[q];
    }
    return s;
}

static void pf_zero(const PfLvl* l, double* v) { memset(v, 0, l->G * 8); }

/* one PFMG V-cycle from x = 0 on level 0 (pfmg_solve.c:120-330) */
static void pf_vcycle(Pfmg* P) {
    PfLvl* L = P->L;
    const int nl = P->nl;
    pf_zero(&L[0], L[0].x);
    pf_relax(&L[0], L[0].x, L[0].b, P->t, L[0].w, 1, 1);
    if (nl == 1) return;
    pf_residual(&L[0], L[0].x, L[0].b, L[0].r);
    pf_restrict(&L[0], &L[1], L[0].cdir);
    int l = 1;
    for (; l <= nl - 2; ++l) {
        if (L[l].active) {
            pf_relax(&L[l], L[l].x, L[l].b, P->t, L[l].w, 1, 1);
            pf_residual(&L[l], L[l].x, L[l].b, L[l].r);
        } else {
            pf_zero(&L[l], L[l].x);
            memcpy(L[l].r, L[l].b, L[l].G * 8);
        }
        pf_restrict(&L[l], &L[l + 1], L[l].cdir);
    }
    /* the coarsest level: Jacobi (weight 1), min(4 * levels, largest extent) sweeps */
    {
        int mx = 1;
        for (int d = 0; d < 3; ++d) mx = L[l].n[d] > mx ? L[l].n[d] : mx;
        const int sweeps = 4 * nl < mx ? 4 * nl : mx;
        pf_relax(&L[l], L[l].x, L[l].b, P->t, 1.0, sweeps, 1);
    }
    for (l = nl - 2; l >= 1; --l) {
        pf_interp_add(&L[l], &L[l + 1], L[l].cdir);
        if (L[l].active) pf_relax(&L[l], L[l].x, L[l].b, P->t, L[l].w, 1, 0);
    }
    pf_interp_add(&L[0], &L[1], L[0].cdir);
    pf_relax(&L[0], L[0].x, L[0].b, P->t, L[0].w, 1, 0);
}

/* z = M r: `cycles` V-cycles (0: PFMG's defaults, V-cycles until ||b - A z|| < 1e-6 ||b||, at most
 * 200, always at least one) */
static void pf_precond(Pfmg* P, const double* r, double* z, int cycles, double* tmp) {
    PfLvl* L0 = &P->L[0];
    memcpy(L0->b, r, L0->G * 8);
    if (cycles > 0 && cycles == 1) {
        pf_vcycle(P);
        memcpy(z, L0->x, L0->G * 8);
        return;
    }
    /* iterate x += V(b - A x) */
    const int maxc = cycles > 0 ? cycles : 200;
    const double bb = pf_dot(L0, r, r);
    memset(z, 0, L0->G * 8);
    for (int it = 0; it < maxc; ++it) {
        if (it == 0) memcpy(L0->b, r, L0->G * 8);
        else {
            pf_residual(L0, z, r, tmp);
            if (cycles == 0 && pf_dot(L0, tmp, tmp) < 1e-12 * bb) break;
            memcpy(L0->b, tmp, L0->G * 8);
        }
        pf_vcycle(P);
        for (size_t q = 0; q < L0->G; ++q) z[q] += L0->x[q];
    }
}

int or_pfmg_pcg_x0(int D, const int* dims_in, int ne, const int* off, const double* coef, const double* rhs, const double* x0,
                   double* x_out, double tol, int maxit, int precond_cycles, int threads, int* iters, double* relres, int* levels);

int or_pfmg_pcg(int D, const int* dims_in, int ne, const int* off, const double* coef, const double* rhs, double* x_out, double tol,
                int maxit, int precond_cycles, int threads, int* iters, double* relres, int* levels) {
    return or_pfmg_pcg_x0(D, dims_in, ne, off, coef, rhs, NULL, x_out, tol, maxit, precond_cycles, threads, iters, relres, levels);
}

/* As or_pfmg_pcg, from the initial guess x0 (NULL: zero).  HYPREEqnSolveHandler::initx
 * (src/Core/Equation/HYPREEqnSolveHandler.hpp:119) loads the target's values into x before every
 * solve; hypre_PCGSolve (external/hypre/src/krylov/pcg.c) then starts from r = b - A x0 and runs at
 * least one iteration before its first convergence test. */
int or_pfmg_pcg_x0(int D, const int* dims_in, int ne, const int* off, const double* coef, const double* rhs, const double* x0,
                   double* x_out, double tol, int maxit, int precond_cycles, int threads, int* iters, double* relres, int* levels) {
    Pfmg* P = (Pfmg*) calloc(1, sizeof(Pfmg));
    if (!P) return OPFLOW_E_NOMEM;
    const int nt = threads > 0 ? threads : 1;
    int rc = pf_setup(P, D, dims_in, ne, off, coef, nt);
    if (rc) {
        pf_free(P);
        free(P);
        return rc == 2 ? OPFLOW_E_UNSUPPORTED : OPFLOW_E_NOMEM;
    }
    PfLvl* L0 = &P->L[0];
    const size_t G = L0->G;
    double *x = calloc(G, 8), *b = calloc(G, 8), *r = calloc(G, 8), *p = calloc(G, 8), *s = calloc(G, 8), *tmp = calloc(G, 8);
    if (!x || !b || !r || !p || !s || !tmp) {
        free(x); free(b); free(r); free(p); free(s); free(tmp);
        pf_free(P);
        free(P);
        return OPFLOW_E_NOMEM;
    }
    size_t c = 0;
    for (int k = 0; k < L0->n[2]; ++k)
        for (int j = 0; j < L0->n[1]; ++j) {
            long long q = pf_lin(L0, 0, j, k);
            for (int i = 0; i < L0->n[0]; ++i, ++q, ++c) {
                b[q] = rhs[c];
                if (x0) x[q] = x0[c];
            }
        }
    /* PCG (pcg.c), two-norm test <r,r>/<b,b> < tol^2 */
    const double bi = pf_dot(L0, b, b);
    int it = 0;
    if (bi > 0.) {
        const double eps = tol * tol;
        if (x0) pf_residual(L0, x, b, r);
        else memcpy(r, b, G * 8);
        pf_precond(P, r, p, precond_cycles, tmp);
        double gamma = pf_dot(L0, r, p);
        while (it < maxit) {
            ++it;
            pf_matvec(L0, p, s);
            const double alpha = gamma / pf_dot(L0, s, p);
#pragma omp parallel for schedule(static) num_threads(nt) if (nt > 1)
            for (size_t q = 0; q < G; ++q) {
                x[q] += alpha * p[q];
                r[q] -= alpha * s[q];
            }
            pf_precond(P, r, s, precond_cycles, tmp);
            const double gold = gamma;
            gamma = pf_dot(L0, r, s);
            const double ip = pf_dot(L0, r, r);
            if (ip / bi < eps) break;
            const double beta = gamma / gold;
#pragma omp parallel for schedule(static) num_threads(nt) if (nt > 1)
            for (size_t q = 0; q < G; ++q) p[q] = s[q] + beta * p[q];
        }
    }
    c = 0;
    for (int k = 0; k < L0->n[2]; ++k)
        for (int j = 0; j < L0->n[1]; ++j) {
            long long q = pf_lin(L0, 0, j, k);
            for (int i = 0; i < L0->n[0]; ++i, ++q, ++c) x_out[c] = x[q];
        }
    pf_residual(L0, x, b, r);
    const double rr = pf_dot(L0, r, r);
    if (iters) *iters = it;
    if (relres) *relres = bi > 0. ? sqrt(rr / bi) : sqrt(rr);
    if (levels) *levels = P->nl;
    free(x); free(b); free(r); free(p); free(s); free(tmp);
    pf_free(P);
    free(P);
    return OPFLOW_OK;
}
