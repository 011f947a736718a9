/* abi_double.c -- a stand-in for the slice of libopflow_gpu's C ABI that the OpFlow adapter
 * (include/opflow_gb300/adapter) calls, computed on the host by the oracle.
 *
 * TEST INFRASTRUCTURE ONLY.  It lets a program compiled unchanged against OpFlow's own headers and the
 * adapter run where there is no GPU (here, where the OpFlow tree is), so that the adapter's lowering of
 * OpFlow's expression types, its field mirrors and its host synchronisation are checked end to end
 * against the reference's own output.  With OPFLOW_ABI_RECORD=<file> it also records every field it is
 * given and every assignment program the adapter builds (JSON lines), which the GPU tests replay
 * through the real library.  Never linked into the product.
 *
 * Entry points: opflow_ctx_create, opflow_last_error, opflow_field_create / _destroy / _get_info /
 * _upload / _download, opflow_assign (all fields of an assignment share one mesh, as the oracle
 * assumes). */
#include "../include/opflow_gpu.h"

#include <stdio.h>
#include <stdlib.h>
#include <string.h>

int or_field_info(const opflow_mesh_desc* m, const opflow_field_desc* f, opflow_field_info* o);
int or_update_padding(const opflow_mesh_desc* m, const opflow_field_desc* fd, double* data);
int or_assign(const opflow_mesh_desc* m, const opflow_field_desc* descs, double** datas, int nf, int dst, int arith,
              const opflow_node* nodes, int n);
const char* or_last_error(void);

struct opflow_ctx_s {
    int device;
};
struct opflow_field_s {
    int id;
    opflow_mesh_desc mesh;
    double* x[3];
    double* dx[3];
    opflow_field_desc desc;
    opflow_field_info info;
    double* data;
    int uploaded;
};

static char g_msg[512];
static int g_next_id = 0;
static FILE* g_rec = NULL;
static int g_rec_checked = 0;

static FILE* rec(void) {
    if (!g_rec_checked) {
        const char* p = getenv("OPFLOW_ABI_RECORD");
        if (p && *p) g_rec = fopen(p, "w");
        g_rec_checked = 1;
    }
    return g_rec;
}

static int failm(int code, const char* m) {
    snprintf(g_msg, sizeof g_msg, "%s", m);
    return code;
}

const char* opflow_last_error(void) { return g_msg; }

int opflow_ctx_create(int device, opflow_ctx* out) {
    if (!out) return failm(OPFLOW_E_INVALID, "null argument");
    *out = (opflow_ctx) calloc(1, sizeof(struct opflow_ctx_s));
    (*out)->device = device;
    return OPFLOW_OK;
}

static void put_doubles(FILE* f, const double* v, size_t n) {
    fputc('[', f);
    for (size_t i = 0; i < n; ++i) fprintf(f, "%s%.17g", i ? "," : "", v[i]);
    fputc(']', f);
}

int opflow_field_create(opflow_ctx ctx, const opflow_mesh_desc* mesh, const opflow_field_desc* desc, opflow_field* out) {
    (void) ctx;
    if (!mesh || !desc || !out) return failm(OPFLOW_E_INVALID, "null argument");
    struct opflow_field_s* f = (struct opflow_field_s*) calloc(1, sizeof *f);
    f->id = g_next_id++;
    f->mesh = *mesh;
    for (int d = 0; d < mesh->ndim; ++d) {
        const size_t nx = (size_t) mesh->dims[d] + 2 * (size_t) mesh->pad_width;
        f->x[d] = (double*) malloc(nx * sizeof(double));
        f->dx[d] = (double*) malloc((nx - 1) * sizeof(double));
        memcpy(f->x[d], mesh->x[d], nx * sizeof(double));
        memcpy(f->dx[d], mesh->dx[d], (nx - 1) * sizeof(double));
        f->mesh.x[d] = f->x[d];
        f->mesh.dx[d] = f->dx[d];
    }
    f->desc = *desc;
    int rc = or_field_info(&f->mesh, &f->desc, &f->info);
    if (rc) return failm(rc, or_last_error());
    f->data = (double*) calloc(f->info.count, sizeof(double));
    rc = or_update_padding(&f->mesh, &f->desc, f->data);
    if (rc) return failm(rc, or_last_error());
    FILE* r = rec();
    if (r) {
        fprintf(r, "{\"op\":\"field\",\"id\":%d,\"ndim\":%d,\"dims\":[%d,%d,%d],\"start\":[%d,%d,%d],\"pad_width\":%d", f->id, mesh->ndim,
                mesh->dims[0], mesh->dims[1], mesh->dims[2], mesh->start[0], mesh->start[1], mesh->start[2], mesh->pad_width);
        for (int d = 0; d < mesh->ndim; ++d) {
            const size_t nx = (size_t) mesh->dims[d] + 2 * (size_t) mesh->pad_width;
            fprintf(r, ",\"x%d\":", d);
            put_doubles(r, f->x[d], nx);
            fprintf(r, ",\"dx%d\":", d);
            put_doubles(r, f->dx[d], nx - 1);
        }
        fprintf(r, ",\"loc\":[%d,%d,%d],\"bc_type\":[[%d,%d],[%d,%d],[%d,%d]],\"bc_value\":[[%.17g,%.17g],[%.17g,%.17g],[%.17g,%.17g]],"
                   "\"ext\":[[%d,%d],[%d,%d],[%d,%d]],\"padding\":%d}\n",
                desc->loc[0], desc->loc[1], desc->loc[2], desc->bc_type[0][0], desc->bc_type[0][1], desc->bc_type[1][0], desc->bc_type[1][1],
                desc->bc_type[2][0], desc->bc_type[2][1], desc->bc_value[0][0], desc->bc_value[0][1], desc->bc_value[1][0], desc->bc_value[1][1],
                desc->bc_value[2][0], desc->bc_value[2][1], desc->ext[0][0], desc->ext[0][1], desc->ext[1][0], desc->ext[1][1], desc->ext[2][0],
                desc->ext[2][1], desc->padding);
        fflush(r);
    }
    *out = f;
    return OPFLOW_OK;
}

int opflow_field_destroy(opflow_field f) {
    if (!f) return OPFLOW_OK;
    for (int d = 0; d < 3; ++d) {
        free(f->x[d]);
        free(f->dx[d]);
    }
    free(f->data);
    free(f);
    return OPFLOW_OK;
}

int opflow_field_get_info(opflow_field f, opflow_field_info* out) {
    if (!f || !out) return failm(OPFLOW_E_INVALID, "null argument");
    *out = f->info;
    return OPFLOW_OK;
}

int opflow_field_upload(opflow_field f, const double* host, size_t count) {
    if (!f || !host || count != f->info.count) return failm(OPFLOW_E_INVALID, "bad upload");
    FILE* r = rec();
    /* recorded: the first state a field is given, and later uploads that differ from what the field
     * holds (host code wrote it); values for fields of up to 65536 doubles, otherwise only whether the
     * data is the zero field with its padding applied (what the replay rebuilds) */
    if (r && (!f->uploaded || memcmp(f->data, host, count * sizeof(double)) != 0)) {
        fprintf(r, "{\"op\":\"upload\",\"id\":%d,\"count\":%zu,\"data\":", f->id, count);
        if (count <= 65536) {
            put_doubles(r, host, count);
        } else {
            double* z = (double*) calloc(count, sizeof(double));
            or_update_padding(&f->mesh, &f->desc, z);
            const int zp = memcmp(z, host, count * sizeof(double)) == 0;
            free(z);
            fprintf(r, "null,\"zero_padded\":%d", zp);
        }
        fputs("}\n", r);
        fflush(r);
    }
    memcpy(f->data, host, count * sizeof(double));
    f->uploaded = 1;
    return OPFLOW_OK;
}

int opflow_field_download(opflow_field f, double* host, size_t count) {
    if (!f || !host || count != f->info.count) return failm(OPFLOW_E_INVALID, "bad download");
    memcpy(host, f->data, count * sizeof(double));
    return OPFLOW_OK;
}

int opflow_assign(opflow_ctx ctx, opflow_field dst, int arith, const opflow_node* nodes, int n_nodes, const opflow_field* leaves,
                  int n_leaves, int mode) {
    (void) ctx;
    if (!dst || !nodes || n_nodes <= 0 || n_leaves < 0 || n_leaves > 15) return failm(OPFLOW_E_INVALID, "bad assign arguments");
    opflow_field_desc descs[16];
    double* datas[16];
    int slot = -1;
    for (int i = 0; i < n_leaves; ++i) {
        descs[i] = leaves[i]->desc;
        datas[i] = leaves[i]->data;
        if (leaves[i] == dst) slot = i;
    }
    int nf = n_leaves;
    if (slot < 0) {
        descs[nf] = dst->desc;
        datas[nf] = dst->data;
        slot = nf++;
    }
    FILE* r = rec();
    if (r) {
        fprintf(r, "{\"op\":\"assign\",\"dst\":%d,\"arith\":%d,\"mode\":%d,\"leaves\":[", dst->id, arith, mode);
        for (int i = 0; i < n_leaves; ++i) fprintf(r, "%s%d", i ? "," : "", leaves[i]->id);
        fputs("],\"nodes\":[", r);
        for (int k = 0; k < n_nodes; ++k)
            fprintf(r, "%s[%d,%d,%d,%d,%d,%.17g,%d]", k ? "," : "", nodes[k].kind, nodes[k].a, nodes[k].b, nodes[k].dim, nodes[k].field,
                    nodes[k].value, nodes[k].c);
        fputs("]}\n", r);
        fflush(r);
    }
    int rc = or_assign(&dst->mesh, descs, datas, nf, slot, arith, nodes, n_nodes);
    if (rc) return failm(rc, or_last_error());
    return OPFLOW_OK;
}

/* ---- the implicit path: the oracle's assembly (generateAb restated) and its restated PCG + PFMG ---- */
int or_assemble(const opflow_mesh_desc* m, const opflow_field_desc* descs, double** datas, int nf, int target, const opflow_node* nodes,
                int n, int pin, int* n_entries, int* offsets, double* coef, double* rhs, size_t* n_cells);
int or_pfmg_pcg_x0(int D, const int* dims_in, int ne, const int* off, const double* coef, const double* rhs, const double* x0,
                   double* x_out, double tol, int maxit, int precond_cycles, int threads, int* iters, double* relres, int* levels);

/* the data index of the c-th assignable cell (x fastest) */
static size_t assignable_index(const opflow_field_info* R, const int* dims, size_t c) {
    const int D = R->ndim;
    const long long i = (long long) (c % dims[0]), j = (long long) ((c / dims[0]) % dims[1]), k = (long long) (c / ((size_t) dims[0] * dims[1]));
    const long long ii = R->assignable[0][0] + i - R->data_offset[0];
    const long long jj = D > 1 ? R->assignable[1][0] + j - R->data_offset[1] : 0;
    const long long kk = D > 2 ? R->assignable[2][0] + k - R->data_offset[2] : 0;
    return (size_t) ((kk * (D > 1 ? R->data_dims[1] : 1) + jj) * R->data_dims[0] + ii);
}

void opflow_solve_params_default(opflow_solve_params* p) {
    memset(p, 0, sizeof *p);
    p->tol = 1e-8;
    p->max_iter = 100;
    p->pre_sweeps = p->post_sweeps = 2;
    p->coarse_max = 64;
    p->kdim = 5;
}

struct opflow_solver_s {
    opflow_field target;
    opflow_node* nodes;
    int n_nodes;
    opflow_field leaves[16];
    int n_leaves, unknown;
    opflow_solve_params params;
};

int opflow_solver_create(opflow_ctx ctx, opflow_field target, const opflow_node* nodes, int n_nodes, const opflow_field* leaves, int n_leaves,
                         int unknown_slot, const opflow_solve_params* params, opflow_solver* out) {
    (void) ctx;
    if (!target || !nodes || n_nodes <= 0 || n_leaves <= 0 || n_leaves > 16 || unknown_slot < 0 || unknown_slot >= n_leaves || !params || !out)
        return failm(OPFLOW_E_INVALID, "bad solver arguments");
    struct opflow_solver_s* s = (struct opflow_solver_s*) calloc(1, sizeof *s);
    s->target = target;
    s->nodes = (opflow_node*) malloc(n_nodes * sizeof(opflow_node));
    memcpy(s->nodes, nodes, n_nodes * sizeof(opflow_node));
    s->n_nodes = n_nodes;
    memcpy(s->leaves, leaves, n_leaves * sizeof(opflow_field));
    s->n_leaves = n_leaves;
    s->unknown = unknown_slot;
    s->params = *params;
    FILE* r = rec();
    if (r) {
        fprintf(r, "{\"op\":\"solver\",\"target\":%d,\"unknown\":%d,\"leaves\":[", target->id, unknown_slot);
        for (int i = 0; i < n_leaves; ++i) fprintf(r, "%s%d", i ? "," : "", leaves[i]->id);
        fprintf(r, "],\"params\":{\"tol\":%.17g,\"max_iter\":%d,\"static_mat\":%d,\"pin_value\":%d,\"precision\":%d,\"krylov\":%d,"
                   "\"precond\":%d,\"kdim\":%d,\"abs_tol\":%.17g,\"zero_guess\":%d},\"nodes\":[",
                params->tol, params->max_iter, params->static_mat, params->pin_value, params->precision, params->krylov, params->precond,
                params->kdim, params->abs_tol, params->zero_guess);
        for (int k = 0; k < n_nodes; ++k)
            fprintf(r, "%s[%d,%d,%d,%d,%d,%.17g,%d]", k ? "," : "", nodes[k].kind, nodes[k].a, nodes[k].b, nodes[k].dim, nodes[k].field,
                    nodes[k].value, nodes[k].c);
        fputs("]}\n", r);
        fflush(r);
    }
    *out = s;
    return OPFLOW_OK;
}

int opflow_solver_solve(opflow_solver s, opflow_solve_state* state) {
    if (!s) return failm(OPFLOW_E_INVALID, "null solver");
    FILE* r = rec();
    if (r) {
        fprintf(r, "{\"op\":\"solve\",\"target\":%d}\n", s->target->id);
        fflush(r);
    }
    opflow_field_desc descs[16];
    double* datas[16];
    for (int i = 0; i < s->n_leaves; ++i) {
        descs[i] = s->leaves[i]->desc;
        datas[i] = s->leaves[i]->data;
    }
    opflow_field t = s->leaves[s->unknown];
    int ne = 0;
    size_t nc = 0;
    int rc = or_assemble(&t->mesh, descs, datas, s->n_leaves, s->unknown, s->nodes, s->n_nodes, s->params.pin_value, &ne, NULL, NULL, NULL, &nc);
    if (rc) return failm(rc, or_last_error());
    const int D = t->info.ndim;
    int* off = (int*) malloc((size_t) ne * D * sizeof(int));
    double* coef = (double*) malloc(nc * ne * sizeof(double));
    double* rhs = (double*) malloc(nc * sizeof(double));
    double* x = (double*) calloc(nc, sizeof(double));
    rc = or_assemble(&t->mesh, descs, datas, s->n_leaves, s->unknown, s->nodes, s->n_nodes, s->params.pin_value, &ne, off, coef, rhs, &nc);
    int dims[3] = {1, 1, 1}, it = 0, nl = 0;
    double rel = 0.;
    for (int d = 0; d < D; ++d) dims[d] = t->info.assignable[d][1] - t->info.assignable[d][0];
    /* initial guess: the target's values (HYPREEqnSolveHandler::initx), unless zero_guess */
    double* x0 = s->params.zero_guess ? NULL : (double*) malloc(nc * sizeof(double));
    if (x0)
        for (size_t c = 0; c < nc; ++c) x0[c] = t->data[assignable_index(&t->info, dims, c)];
    if (!rc) rc = or_pfmg_pcg_x0(D, dims, ne, off, coef, rhs, x0, x, s->params.tol, s->params.max_iter, 1, 1, &it, &rel, &nl);
    free(x0);
    if (!rc) {
        /* the solution into the target's assignable cells, then its padding */
        for (size_t c = 0; c < nc; ++c) t->data[assignable_index(&t->info, dims, c)] = x[c];
        rc = or_update_padding(&t->mesh, &t->desc, t->data);
    }
    free(off);
    free(coef);
    free(rhs);
    free(x);
    if (rc) return failm(rc, or_last_error());
    if (state) {
        memset(state, 0, sizeof *state);
        state->iterations = it;
        state->rel_residual = rel;
        state->converged = rel <= s->params.tol;
    }
    return OPFLOW_OK;
}

int opflow_solver_destroy(opflow_solver s) {
    if (!s) return OPFLOW_OK;
    free(s->nodes);
    free(s);
    return OPFLOW_OK;
}
