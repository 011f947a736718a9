// Context, mesh, field storage and the padding (ghost-cell) update of OpFlow's CartesianField.
#include "internal.h"

#include <cstdarg>
#include <cstdlib>
#include <mutex>

namespace opg {

static thread_local char t_err[1024] = "";
std::atomic<uint64_t> g_launches{0};

void set_error(const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(t_err, sizeof t_err, fmt, ap);
    va_end(ap);
}
int fail(int code, const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(t_err, sizeof t_err, fmt, ap);
    va_end(ap);
    return code;
}
int check_launch(const char* what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(OPFLOW_E_CUDA, "launch of %s failed: %s", what, cudaGetErrorString(e));
    return OPFLOW_OK;
}

static std::mutex g_pool_mu;
static cudaMemPool_t g_pool[64] = {};

static cudaMemPool_t device_pool(int dev) {
    if (dev < 0 || dev >= 64) return nullptr;
    std::lock_guard<std::mutex> lk(g_pool_mu);
    if (!g_pool[dev]) {
        cudaMemPoolProps props{};
        props.allocType = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = dev;
        cudaMemPool_t p = nullptr;
        if (cudaMemPoolCreate(&p, &props) != cudaSuccess) return nullptr;
        uint64_t keep = ~0ull;  // never hand memory back at synchronisation points
        cudaMemPoolSetAttribute(p, cudaMemPoolAttrReleaseThreshold, &keep);
        g_pool[dev] = p;
    }
    return g_pool[dev];
}

void* dev_alloc(opflow_ctx ctx, size_t bytes) {
    void* p = nullptr;
    cudaMemPool_t pool = device_pool(ctx->device);
    if (!pool || cudaMallocFromPoolAsync(&p, bytes, pool, ctx->stream) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return p;
}

void dev_free(opflow_ctx ctx, void* p) {
    if (p) cudaFreeAsync(p, ctx->stream);
}

int ensure_scratch(opflow_ctx ctx, size_t bytes) {
    if (ctx->scratch_bytes >= bytes) return OPFLOW_OK;
    if (ctx->scratch) dev_free(ctx, ctx->scratch);
    ctx->scratch = nullptr;
    ctx->scratch_bytes = 0;
    ctx->scratch = dev_alloc(ctx, bytes);
    if (!ctx->scratch) return fail(OPFLOW_E_NOMEM, "cannot allocate %zu bytes of scratch", bytes);
    ctx->scratch_bytes = bytes;
    return OPFLOW_OK;
}

// ---- mesh ---------------------------------------------------------------------------------------------
int mesh_create(opflow_ctx ctx, const opflow_mesh_desc* m, MeshDev** out) {
    if (!m || m->ndim < 1 || m->ndim > 3 || m->pad_width < 0) return fail(OPFLOW_E_INVALID, "bad mesh description");
    auto* md = new MeshDev();
    md->ndim = m->ndim;
    md->pad = m->pad_width;
    for (int d = 0; d < 3; ++d) {
        md->x[d] = md->dx[d] = nullptr;
        md->uniform[d] = true;
        md->h[d] = 0.;
        md->es[d] = 0;
        md->n[d] = 1;
    }
    for (int d = 0; d < m->ndim; ++d) {
        if (m->dims[d] < 2 || !m->x[d] || !m->dx[d]) {
            mesh_destroy(ctx, md);
            return fail(OPFLOW_E_INVALID, "mesh dim %d needs >= 2 nodes and coordinate arrays", d);
        }
        const int n = m->dims[d] + 2 * m->pad_width;
        md->es[d] = m->start[d] - m->pad_width;
        md->n[d] = n;
        md->hx[d].assign(m->x[d], m->x[d] + n);
        md->hdx[d].assign(m->dx[d], m->dx[d] + n - 1);
        md->h[d] = md->hdx[d][0];
        for (int i = 0; i < n - 1; ++i) md->uniform[d] = md->uniform[d] && md->hdx[d][i] == md->h[d];
        md->x[d] = (double*) dev_alloc(ctx, n * sizeof(double));
        md->dx[d] = (double*) dev_alloc(ctx, n * sizeof(double));
        if (!md->x[d] || !md->dx[d]) {
            cudaStreamSynchronize(ctx->stream);  // copies of earlier dims still read md's host arrays
            mesh_destroy(ctx, md);
            return fail(OPFLOW_E_NOMEM, "mesh allocation failed");
        }
        // the host arrays live in md: the copies may complete after this call returns
        cudaMemcpyAsync(md->x[d], md->hx[d].data(), n * sizeof(double), cudaMemcpyHostToDevice, ctx->stream);
        cudaMemcpyAsync(md->dx[d], md->hdx[d].data(), (n - 1) * sizeof(double), cudaMemcpyHostToDevice, ctx->stream);
    }
    *out = md;
    return OPFLOW_OK;
}
void mesh_destroy(opflow_ctx ctx, MeshDev* m) {
    if (!m) return;
    for (int d = 0; d < 3; ++d) {
        if (m->x[d]) dev_free(ctx, m->x[d]);
        if (m->dx[d]) dev_free(ctx, m->dx[d]);
    }
    delete m;
}
bool mesh_equal(const MeshDev* a, const MeshDev* b) {
    if (a == b) return true;
    if (a->ndim != b->ndim) return false;
    for (int d = 0; d < a->ndim; ++d)
        if (a->es[d] != b->es[d] || a->hx[d] != b->hx[d] || a->hdx[d] != b->hdx[d]) return false;
    return true;
}

// ---- ranges: ExprBuilder::calculateRanges / validateRanges (CartesianField.hpp:941-1029) ---------------
int compute_info(const opflow_mesh_desc* m, const opflow_field_desc* f, opflow_field_info* o) {
    if (!m || !f || !o || f->ndim != m->ndim || f->ndim < 1 || f->ndim > 3) return fail(OPFLOW_E_INVALID, "field/mesh dimension mismatch");
    std::memset(o, 0, sizeof *o);
    const int D = f->ndim;
    o->ndim = D;
    int pad = f->padding < 0 ? 0 : f->padding;
    for (int d = 0; d < D; ++d) {
        if (f->ext[d][0] < 0 || f->ext[d][1] < 0) return fail(OPFLOW_E_INVALID, "negative ext width");
        pad = std::max(pad, std::max(f->ext[d][0], f->ext[d][1]));
        if (f->loc[d] != OPFLOW_CORNER && f->loc[d] != OPFLOW_CENTER) return fail(OPFLOW_E_INVALID, "bad loc");
        for (int s = 0; s < 2; ++s)
            if (f->bc_type[d][s] < OPFLOW_BC_UNDEFINED || f->bc_type[d][s] > OPFLOW_BC_ASYMM) return fail(OPFLOW_E_INVALID, "bad bc type");
        if ((f->bc_type[d][0] == OPFLOW_BC_PERIODIC) != (f->bc_type[d][1] == OPFLOW_BC_PERIODIC))
            return fail(OPFLOW_E_INVALID, "periodic bc must be set on both sides of dim %d", d);
    }
    if (pad > m->pad_width) return fail(OPFLOW_E_INVALID, "field padding %d exceeds the mesh ghost extension %d", pad, m->pad_width);
    o->padding = pad;
    for (int d = 0; d < D; ++d) {
        const int s = m->start[d], e = m->start[d] + m->dims[d];
        o->logical[d][0] = o->assignable[d][0] = o->local[d][0] = o->accessible[d][0] = s;
        o->logical[d][1] = o->assignable[d][1] = o->local[d][1] = o->accessible[d][1] = e;
        const int loc = f->loc[d];
        if (f->bc_type[d][0] == OPFLOW_BC_DIRC && loc == OPFLOW_CORNER) o->assignable[d][0]++;
        switch (f->bc_type[d][1]) {
            case OPFLOW_BC_DIRC:
                if (loc == OPFLOW_CORNER) o->assignable[d][1]--;
                else { o->accessible[d][1]--; o->assignable[d][1]--; }
                break;
            case OPFLOW_BC_PERIODIC: o->accessible[d][1]--; o->assignable[d][1]--; break;
            default:
                if (loc == OPFLOW_CENTER) { o->accessible[d][1]--; o->assignable[d][1]--; }
        }
        o->logical[d][0] = o->accessible[d][0] - f->ext[d][0];
        o->logical[d][1] = o->accessible[d][1] + f->ext[d][1];
        o->local[d][0] = std::max(o->accessible[d][0], o->logical[d][0]);
        o->local[d][1] = std::min(o->accessible[d][1], o->logical[d][1]);
        o->accessible[d][0] = std::max(o->accessible[d][0], o->logical[d][0]);
        o->accessible[d][1] = std::min(o->accessible[d][1], o->logical[d][1]);
        o->assignable[d][0] = std::max(o->assignable[d][0], o->accessible[d][0]);
        o->assignable[d][1] = std::min(o->assignable[d][1], o->accessible[d][1]);
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
        if (o->data_dims[d] <= 0) return fail(OPFLOW_E_INVALID, "empty field range in dim %d", d);
        o->count *= (size_t) o->data_dims[d];
    }
    return OPFLOW_OK;
}

Box assign_box(const opflow_field_info& r) {
    Box b;
    for (int d = 0; d < 3; ++d) {
        b.lo[d] = std::max(r.assignable[d][0], r.local[d][0]);
        b.hi[d] = std::min(r.assignable[d][1], r.local[d][1]);
    }
    return b;
}

// ---- padding kernels: CartesianField::updatePaddingImpl_final (CartesianField.hpp:349-629) -------------
enum PadKind { PAD_FILL = 0, PAD_MIRROR = 1, PAD_PERIODIC = 2 };
struct PadOp {
    int kind, dim, side, bct, corner;
    double bcv;
    int lo[3], hi[3];
    int lstart, lend;  // localRange start/end along dim
    int period;
    int es;            // mesh extended-range start along dim
};

__device__ __forceinline__ double intp_exact(double x1, double y1, double x2, double y2, double x) {
    // Interpolator1D::intp(x1, y1, x2, y2, x) (Interpolator.hpp:21-23, 38-40), no contraction
    const double a = __dsub_rn(x1, x), b = __dsub_rn(x2, x);
    return __ddiv_rn(__dsub_rn(__dmul_rn(a, y2), __dmul_rn(b, y1)), __dsub_rn(a, b));
}

__global__ void pad_kernel(FieldView f, PadOp op, const double* __restrict__ mx, const double* __restrict__ mdx) {
    const long long nx = op.hi[0] - op.lo[0], ny = op.hi[1] - op.lo[1], nz = op.hi[2] - op.lo[2];
    const long long total = nx * ny * nz;
    for (long long t = blockIdx.x * (long long) blockDim.x + threadIdx.x; t < total; t += (long long) gridDim.x * blockDim.x) {
        Box bx;
        for (int d = 0; d < 3; ++d) { bx.lo[d] = op.lo[d]; bx.hi[d] = op.hi[d]; }
        int idx[3];
        box_index(t, bx, idx[0], idx[1], idx[2]);
        const long long o = (idx[0] - f.off[0]) + (idx[1] - f.off[1]) * f.sy + (idx[2] - f.off[2]) * f.sz;
        if (op.kind == PAD_FILL) {
            f.data[o] = op.bcv;
            continue;
        }
        int mi[3] = {idx[0], idx[1], idx[2]};
        const int i = op.dim;
        if (op.kind == PAD_PERIODIC) {
            mi[i] += op.side == 0 ? op.period : -op.period;
        } else if (op.corner) {
            mi[i] = op.side == 0 ? 2 * op.lstart - idx[i] : 2 * op.lend - 2 - idx[i];
        } else {
            mi[i] = op.side == 0 ? 2 * op.lstart - 1 - idx[i] : 2 * op.lend - 1 - idx[i];
        }
        const long long om = (mi[0] - f.off[0]) + (mi[1] - f.off[1]) * f.sy + (mi[2] - f.off[2]) * f.sz;
        const double vm = f.data[om];
        double v = vm;
        if (op.kind == PAD_MIRROR) {
            const double xi = mx[idx[i] - op.es], xm = mx[mi[i] - op.es];
            switch (op.bct) {
                case OPFLOW_BC_DIRC:
                    if (op.corner) {
                        const double xb = mx[(op.side == 0 ? op.lstart : op.lend - 1) - op.es];
                        v = intp_exact(xb, op.bcv, xm, vm, xi);
                    } else {
                        const double xb = mx[(op.side == 0 ? op.lstart : op.lend) - op.es];
                        v = intp_exact(xb, op.bcv, __dadd_rn(xm, __ddiv_rn(mdx[mi[i] - op.es], 2.)), vm,
                                       __dadd_rn(xi, __ddiv_rn(mdx[idx[i] - op.es], 2.)));
                    }
                    break;
                case OPFLOW_BC_NEUM:
                    if (op.corner) v = __dadd_rn(vm, __dmul_rn(op.bcv, __dsub_rn(xi, xm)));
                    else {
                        // x(idx) + dx(idx)/2 - x(mirror) - dx(mirror)/2, left to right
                        double t = __dadd_rn(xi, __ddiv_rn(mdx[idx[i] - op.es], 2.));
                        t = __dsub_rn(t, xm);
                        t = __dsub_rn(t, __ddiv_rn(mdx[mi[i] - op.es], 2.));
                        v = __dadd_rn(vm, __dmul_rn(op.bcv, t));
                    }
                    break;
                case OPFLOW_BC_SYMM: v = vm; break;
                case OPFLOW_BC_ASYMM: v = -vm; break;
            }
        }
        f.data[o] = v;
    }
}

static int launch_pad_box(opflow_field f, double* data, const PadOp& op) {
    Box b;
    for (int d = 0; d < 3; ++d) { b.lo[d] = op.lo[d]; b.hi[d] = op.hi[d]; }
    const long long n = b.count();
    if (n <= 0) return OPFLOW_OK;
    FieldView v = f->view();
    v.data = data;
    const int threads = 256;
    long long blocks = (n + threads - 1) / threads;
    if (blocks > 4096) blocks = 4096;
    pad_kernel<<<(int) blocks, threads, 0, f->ctx->stream>>>(v, op, f->mesh->x[op.dim], f->mesh->dx[op.dim]);
    OPG_LAUNCHED();
    return check_launch("pad_kernel");
}

// The reference fills a padding zone in one x-fastest pass.  A periodic zone wider than the period
// copies from cells of the same zone, so such a zone is filled layer by layer along `dim` in the
// reference's order.  (Mirror zones read the interior or the other side's zone, never their own.)
static int launch_pad(opflow_field f, double* data, const PadOp& op) {
    const int i = op.dim;
    const int width = op.hi[i] - op.lo[i];
    const bool overlap = op.kind == PAD_PERIODIC && op.period < width;
    if (!overlap) return launch_pad_box(f, data, op);
    for (int l = op.lo[i]; l < op.hi[i]; ++l) {
        PadOp layer = op;
        layer.lo[i] = l;
        layer.hi[i] = l + 1;
        OPG_TRY(launch_pad_box(f, data, layer));
    }
    return OPFLOW_OK;
}

int update_padding_full(opflow_field f, double* data);

// Step 0 (Dirichlet values on corner-located boundary nodes) is idempotent with what the kernels write,
// step 1 mirrors, step 2 periodic copies, in the reference's order.
int update_padding_buf(opflow_field f, double* data) {
    const int which = data == f->buf[0] ? 0 : 1;
    if (f->padding_is_step0_only() && f->bc_fresh[which]) return OPFLOW_OK;
    OPG_TRY(update_padding_full(f, data));
    f->bc_fresh[which] = true;
    return OPFLOW_OK;
}

// The corner-located Dirichlet boundary nodes of `data` (the writes updatePadding makes for a field
// without a ghost layer, in its order) filled with values[d][side] instead of the boundary values: a
// resident fixed-point run stores the boundary constants there as fixed-point bit patterns between its
// steps, and update_padding_full puts the float64 constants back afterwards.
int fill_dirichlet_nodes(opflow_field f, double* data, const double values[3][2]) {
    const opflow_field_info& R = f->info;
    const opflow_field_desc& F = f->desc;
    for (int i = 0; i < R.ndim; ++i)
        for (int side = 0; side < 2; ++side) {
            const bool at = side == 0 ? R.local[i][0] == R.accessible[i][0] : R.local[i][1] == R.accessible[i][1];
            if (at && F.bc_type[i][side] == OPFLOW_BC_DIRC && F.loc[i] == OPFLOW_CORNER) {
                PadOp op{};
                op.kind = PAD_FILL;
                op.dim = i;
                op.bcv = values[i][side];
                for (int k = 0; k < 3; ++k) { op.lo[k] = R.local[k][0]; op.hi[k] = R.local[k][1]; }
                op.lo[i] = side == 0 ? R.local[i][0] : R.local[i][1] - 1;
                op.hi[i] = op.lo[i] + 1;
                OPG_TRY(launch_pad(f, data, op));
            }
        }
    return OPFLOW_OK;
}

int update_padding_full(opflow_field f, double* data) {
    const opflow_field_info& R = f->info;
    const opflow_field_desc& F = f->desc;
    const int D = R.ndim;
    for (int i = 0; i < D; ++i) {
        for (int side = 0; side < 2; ++side) {
            const bool at = side == 0 ? R.local[i][0] == R.accessible[i][0] : R.local[i][1] == R.accessible[i][1];
            if (at && F.bc_type[i][side] == OPFLOW_BC_DIRC && F.loc[i] == OPFLOW_CORNER) {
                PadOp op{};
                op.kind = PAD_FILL;
                op.dim = i;
                op.bcv = F.bc_value[i][side];
                for (int k = 0; k < 3; ++k) { op.lo[k] = R.local[k][0]; op.hi[k] = R.local[k][1]; }
                op.lo[i] = side == 0 ? R.local[i][0] : R.local[i][1] - 1;
                op.hi[i] = op.lo[i] + 1;
                OPG_TRY(launch_pad(f, data, op));
            }
        }
    }
    int st[3] = {0, 0, 0}, en[3] = {0, 0, 0};
    for (int i = 0; i < D; ++i) {
        for (int side = 0; side < 2; ++side) {
            const int bct = F.bc_type[i][side];
            const bool at = side == 0 ? R.local[i][0] == R.accessible[i][0] : R.local[i][1] == R.accessible[i][1];
            if (!(at && bct != OPFLOW_BC_UNDEFINED && bct != OPFLOW_BC_PERIODIC)) {
                if (side == 0) st[i] = R.local[i][0];
                else en[i] = R.local[i][1];
                continue;
            }
            if (side == 0) st[i] = R.logical[i][0];
            else en[i] = R.logical[i][1];
            PadOp op{};
            op.kind = PAD_MIRROR;
            op.dim = i;
            op.side = side;
            op.bct = bct;
            op.corner = F.loc[i] == OPFLOW_CORNER;
            op.bcv = F.bc_value[i][side];
            op.lstart = R.local[i][0];
            op.lend = R.local[i][1];
            op.es = f->mesh->es[i];
            for (int k = 0; k < 3; ++k) { op.lo[k] = R.local[k][0]; op.hi[k] = R.local[k][1]; }
            for (int j = 0; j < i; ++j) { op.lo[j] = st[j]; op.hi[j] = en[j]; }
            if (side == 0) { op.lo[i] = st[i]; op.hi[i] = R.local[i][0]; }
            else { op.lo[i] = R.local[i][1]; op.hi[i] = R.logical[i][1]; }
            OPG_TRY(launch_pad(f, data, op));
        }
    }
    for (int i = 0; i < D; ++i) {
        if (F.bc_type[i][0] != OPFLOW_BC_PERIODIC) continue;
        for (int side = 0; side < 2; ++side) {
            PadOp op{};
            op.kind = PAD_PERIODIC;
            op.dim = i;
            op.side = side;
            op.period = R.accessible[i][1] - R.accessible[i][0];
            for (int k = 0; k < 3; ++k) { op.lo[k] = R.logical[k][0]; op.hi[k] = R.logical[k][1]; }
            if (side == 0) { op.lo[i] = R.logical[i][0]; op.hi[i] = R.accessible[i][0]; }
            else { op.lo[i] = R.accessible[i][1]; op.hi[i] = R.logical[i][1]; }
            OPG_TRY(launch_pad(f, data, op));
        }
    }
    return OPFLOW_OK;
}

bool padding_self_overlaps(opflow_field f) {
    for (int d = 0; d < f->info.ndim; ++d) {
        if (f->desc.bc_type[d][0] != OPFLOW_BC_PERIODIC) continue;
        const int period = f->info.accessible[d][1] - f->info.accessible[d][0];
        if (period < f->desc.ext[d][0] || period < f->desc.ext[d][1]) return true;
    }
    return false;
}

int update_padding_assign(opflow_field f) {
    OPG_TRY(update_padding_buf(f, f->buf[f->cur]));
    if (padding_self_overlaps(f)) OPG_TRY(update_padding_full(f, f->buf[f->cur]));
    return OPFLOW_OK;
}

int ensure_back(opflow_field f) {
    if (f->buf[1 - f->cur]) return OPFLOW_OK;
    double* p = (double*) dev_alloc(f->ctx, f->info.count * sizeof(double));
    if (!p) return fail(OPFLOW_E_NOMEM, "cannot allocate the second buffer of a field (%zu doubles)", f->info.count);
    OPG_CUDA(cudaMemcpyAsync(p, f->buf[f->cur], f->info.count * sizeof(double), cudaMemcpyDeviceToDevice, f->ctx->stream));
    f->buf[1 - f->cur] = p;
    f->bc_fresh[1 - f->cur] = f->bc_fresh[f->cur];
    return OPFLOW_OK;
}

}  // namespace opg

// With no ghost layer (padding 0, all ext 0) updatePadding can only write corner-located Dirichlet
// nodes (step 0), whose values are constants.
bool opflow_field_s::padding_is_step0_only() const {
    if (info.padding != 0) return false;
    for (int d = 0; d < info.ndim; ++d)
        if (desc.ext[d][0] != 0 || desc.ext[d][1] != 0) return false;
    return true;
}

opg::FieldView opflow_field_s::view() const {
    opg::FieldView v;
    v.data = buf[cur];
    for (int d = 0; d < 3; ++d) { v.off[d] = info.data_offset[d]; v.dims[d] = info.data_dims[d]; }
    v.sy = info.data_dims[0];
    v.sz = (long long) info.data_dims[0] * info.data_dims[1];
    return v;
}
opg::FieldView opflow_field_s::view_back() const {
    opg::FieldView v = view();
    v.data = buf[1 - cur];
    return v;
}

using namespace opg;

// ===================================================================================================== C ABI
extern "C" {

const char* opflow_last_error(void) { return opg::t_err; }
int opflow_abi_version(void) { return OPFLOW_GPU_ABI_VERSION; }
int opflow_kernel_launch_count(uint64_t* out) {
    if (!out) return fail(OPFLOW_E_INVALID, "null out");
    *out = g_launches.load();
    return OPFLOW_OK;
}

int opflow_ctx_create(int device, opflow_ctx* out) {
    if (!out) return fail(OPFLOW_E_INVALID, "null out");
    int n = 0;
    OPG_CUDA(cudaGetDeviceCount(&n));
    if (device < 0 || device >= n) return fail(OPFLOW_E_INVALID, "device %d not present (%d devices)", device, n);
    OPG_CUDA(cudaSetDevice(device));
    auto* c = new opflow_ctx_s();
    c->device = device;
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete c;
        return fail(OPFLOW_E_CUDA, "stream creation failed");
    }
    c->own_stream = true;
    cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device);
    *out = c;
    return OPFLOW_OK;
}

int opflow_ctx_destroy(opflow_ctx ctx) {
    if (!ctx) return OPFLOW_OK;
    if (ctx->scratch) dev_free(ctx, ctx->scratch);
    cudaStreamSynchronize(ctx->stream);
    if (ctx->own_stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return OPFLOW_OK;
}

int opflow_ctx_set_stream(opflow_ctx ctx, void* s) {
    if (!ctx) return fail(OPFLOW_E_INVALID, "null ctx");
    if (ctx->own_stream) {
        cudaStreamSynchronize(ctx->stream);
        cudaStreamDestroy(ctx->stream);
    }
    ctx->stream = (cudaStream_t) s;
    ctx->own_stream = false;
    return OPFLOW_OK;
}
int opflow_ctx_get_stream(opflow_ctx ctx, void** s) {
    if (!ctx || !s) return fail(OPFLOW_E_INVALID, "null argument");
    *s = (void*) ctx->stream;
    return OPFLOW_OK;
}
int opflow_ctx_synchronize(opflow_ctx ctx) {
    if (!ctx) return fail(OPFLOW_E_INVALID, "null ctx");
    OPG_CUDA(cudaStreamSynchronize(ctx->stream));
    return OPFLOW_OK;
}

// MeshBuilder::set1DRange / set1DMesh(min,max) / setExtMesh, Symm mode (CartesianMesh.hpp:209-303).
int opflow_mesh_uniform(int dims, int start, int pad, double min, double max, double* x, double* dx) {
    if (dims < 2 || pad < 0 || !x || !dx) return fail(OPFLOW_E_INVALID, "mesh needs >= 2 nodes");
    const int es = start - pad, end = start + dims, ee = end + pad;
    for (int i = start; i < end; ++i) x[i - es] = (max - min) / (double) (dims - 1) * (double) (i - start) + min;
    for (int j = start; j < end - 1; ++j) dx[j - es] = (max - min) / (double) (dims - 1);
    for (int i = es; i < start; ++i) dx[i - es] = dx[2 * start - 1 - i - es];
    for (int i = end - 1; i < ee - 1; ++i) dx[i - es] = dx[2 * end - 3 - i - es];
    for (int i = start - 1; i >= es; --i) x[i - es] = x[i + 1 - es] - dx[i - es];
    for (int i = end; i < ee; ++i) x[i - es] = x[i - 1 - es] + dx[i - 1 - es];
    return OPFLOW_OK;
}

int opflow_field_describe(const opflow_mesh_desc* mesh, const opflow_field_desc* desc, opflow_field_info* out) {
    return compute_info(mesh, desc, out);
}

int opflow_field_create(opflow_ctx ctx, const opflow_mesh_desc* mesh, const opflow_field_desc* desc, opflow_field* out) {
    if (!ctx || !mesh || !desc || !out) return fail(OPFLOW_E_INVALID, "null argument");
    opflow_field_info info;
    OPG_TRY(compute_info(mesh, desc, &info));
    OPG_CUDA(cudaSetDevice(ctx->device));
    MeshDev* md = nullptr;
    OPG_TRY(mesh_create(ctx, mesh, &md));
    auto* f = new opflow_field_s();
    f->ctx = ctx;
    f->desc = *desc;
    f->info = info;
    f->mesh = md;
    f->buf[0] = (double*) dev_alloc(ctx, info.count * sizeof(double));
    if (!f->buf[0]) {
        mesh_destroy(ctx, md);
        delete f;
        return fail(OPFLOW_E_NOMEM, "cannot allocate %zu doubles", info.count);
    }
    cudaMemsetAsync(f->buf[0], 0, info.count * sizeof(double), ctx->stream);
    int rc = update_padding_buf(f, f->buf[0]);
    if (rc) {
        opflow_field_destroy(f);
        return rc;
    }
    // the data array is usable from any stream once created
    OPG_CUDA(cudaStreamSynchronize(ctx->stream));
    *out = f;
    return OPFLOW_OK;
}

int opflow_field_destroy(opflow_field f) {
    if (!f) return OPFLOW_OK;
    // freed in the order of the context's stream, after the work already enqueued on it
    for (int k = 0; k < 2; ++k)
        if (f->buf[k]) dev_free(f->ctx, f->buf[k]);
    mesh_destroy(f->ctx, f->mesh);
    delete f;
    return OPFLOW_OK;
}

int opflow_field_get_info(opflow_field f, opflow_field_info* out) {
    if (!f || !out) return fail(OPFLOW_E_INVALID, "null argument");
    *out = f->info;
    return OPFLOW_OK;
}

int opflow_field_upload(opflow_field f, const double* host, size_t count) {
    if (!f || !host) return fail(OPFLOW_E_INVALID, "null argument");
    if (count != f->info.count) return fail(OPFLOW_E_INVALID, "upload of %zu values into a field of %zu", count, f->info.count);
    f->bc_fresh[0] = f->bc_fresh[1] = false;
    f->version++;
    OPG_CUDA(cudaMemcpyAsync(f->buf[f->cur], host, count * sizeof(double), cudaMemcpyHostToDevice, f->ctx->stream));
    if (f->buf[1 - f->cur])
        OPG_CUDA(cudaMemcpyAsync(f->buf[1 - f->cur], f->buf[f->cur], count * sizeof(double), cudaMemcpyDeviceToDevice, f->ctx->stream));
    OPG_CUDA(cudaStreamSynchronize(f->ctx->stream));
    return OPFLOW_OK;
}

int opflow_field_download(opflow_field f, double* host, size_t count) {
    if (!f || !host) return fail(OPFLOW_E_INVALID, "null argument");
    if (count != f->info.count) return fail(OPFLOW_E_INVALID, "download of %zu values from a field of %zu", count, f->info.count);
    OPG_CUDA(cudaMemcpyAsync(host, f->buf[f->cur], count * sizeof(double), cudaMemcpyDeviceToHost, f->ctx->stream));
    OPG_CUDA(cudaStreamSynchronize(f->ctx->stream));
    return OPFLOW_OK;
}

int opflow_field_device_ptr(opflow_field f, double** p) {
    if (!f || !p) return fail(OPFLOW_E_INVALID, "null argument");
    *p = f->buf[f->cur];
    f->bc_fresh[0] = f->bc_fresh[1] = false;  // the caller may write through the pointer
    f->version++;
    return OPFLOW_OK;
}

int opflow_field_update_padding(opflow_field f) {
    if (!f) return fail(OPFLOW_E_INVALID, "null field");
    OPG_TRY(update_padding_full(f, f->buf[f->cur]));
    f->bc_fresh[f->cur] = true;
    return OPFLOW_OK;
}

}  // extern "C"
