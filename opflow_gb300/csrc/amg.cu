// The device side of the smoothed-aggregation AMG (amg.h): the hierarchy in CSR form in HBM and the
// V-cycle as AMGCL's amg::cycle runs it with one pre- and one post-smoothing SPAI-0 sweep:
//   x_l = M_l b_l;  b_{l+1} = R_l (b_l - A_l x_l);  (recurse)  x_l += P_l x_{l+1};  x_l += M_l (b_l - A_l x_l)
// and x = A^-1 b (dense inverse) on the coarsest level.  Every kernel is a streaming pass over one
// level's CSR arrays (HBM or L2 bound); a V-cycle is about 6 launches per level.
#include "amg.h"

namespace opg {
namespace {

constexpr int AMG_THREADS = 256;

int amg_grid(opflow_ctx ctx, long long n) {
    return (int) std::max<long long>(1, std::min<long long>((n + AMG_THREADS - 1) / AMG_THREADS, (long long) ctx->num_sms * 8));
}

// r = b - A x
__global__ void csr_residual(long long n, const long long* __restrict__ p, const int* __restrict__ c, const double* __restrict__ v,
                             const double* __restrict__ x, const double* __restrict__ b, double* __restrict__ r) {
    for (long long i = blockIdx.x * (long long) blockDim.x + threadIdx.x; i < n; i += (long long) gridDim.x * blockDim.x) {
        double s = 0.;
        for (long long q = p[i]; q < p[i + 1]; ++q) s += v[q] * x[c[q]];
        r[i] = b[i] - s;
    }
}

// y = A x, or y += A x
__global__ void csr_spmv(long long n, const long long* __restrict__ p, const int* __restrict__ c, const double* __restrict__ v,
                         const double* __restrict__ x, double* __restrict__ y, int accumulate) {
    for (long long i = blockIdx.x * (long long) blockDim.x + threadIdx.x; i < n; i += (long long) gridDim.x * blockDim.x) {
        double s = 0.;
        for (long long q = p[i]; q < p[i + 1]; ++q) s += v[q] * x[c[q]];
        y[i] = accumulate ? y[i] + s : s;
    }
}

// x = M b (accumulate = 0) or x += M b
__global__ void diag_apply(long long n, const double* __restrict__ M, const double* __restrict__ b, double* __restrict__ x, int accumulate) {
    for (long long i = blockIdx.x * (long long) blockDim.x + threadIdx.x; i < n; i += (long long) gridDim.x * blockDim.x)
        x[i] = accumulate ? x[i] + M[i] * b[i] : M[i] * b[i];
}

// x = Ainv b, one warp per row of the row-major dense inverse
__global__ void dense_apply(long long n, const double* __restrict__ inv, const double* __restrict__ b, double* __restrict__ x) {
    const int lane = threadIdx.x & 31;
    const long long warps = (long long) gridDim.x * (blockDim.x >> 5);
    for (long long i = (blockIdx.x * (long long) blockDim.x + threadIdx.x) >> 5; i < n; i += warps) {
        double s = 0.;
        for (long long j = lane; j < n; j += 32) s += inv[i * n + j] * b[j];
        for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
        if (lane == 0) x[i] = s;
    }
}

template <typename T>
T* up(opflow_ctx ctx, AmgDev* D, const std::vector<T>& h) {
    if (h.empty()) return nullptr;
    T* d = (T*) dev_alloc(ctx, h.size() * sizeof(T));
    if (!d) return nullptr;
    D->allocs.push_back(d);
    cudaMemcpyAsync(d, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, ctx->stream);
    return d;
}

double* vec(opflow_ctx ctx, AmgDev* D, long long n) {
    double* d = (double*) dev_alloc(ctx, (size_t) std::max<long long>(n, 1) * sizeof(double));
    if (d) D->allocs.push_back(d);
    return d;
}

}  // namespace

int amg_upload(opflow_ctx ctx, const AmgHost& H, AmgDev* D) {
    amg_free(ctx, D);
    for (size_t l = 0; l < H.levels.size(); ++l) {
        const AmgLevelHost& L = H.levels[l];
        AmgLevelDev d;
        d.n = L.A.n;
        d.nc = L.P.m;
        d.Ap = up(ctx, D, L.A.ptr);
        d.Ac = up(ctx, D, L.A.col);
        d.Av = up(ctx, D, L.A.val);
        d.M = up(ctx, D, L.M);
        if (!d.Ap || (!L.A.col.empty() && (!d.Ac || !d.Av)) || !d.M) return fail(OPFLOW_E_NOMEM, "AMG level %zu", l);
        if (l + 1 < H.levels.size()) {
            d.Pp = up(ctx, D, L.P.ptr);
            d.Pc = up(ctx, D, L.P.col);
            d.Pv = up(ctx, D, L.P.val);
            d.Rp = up(ctx, D, L.R.ptr);
            d.Rc = up(ctx, D, L.R.col);
            d.Rv = up(ctx, D, L.R.val);
            if (!d.Pp || !d.Pc || !d.Pv || !d.Rp || !d.Rc || !d.Rv) return fail(OPFLOW_E_NOMEM, "AMG transfer operators %zu", l);
        }
        d.r = vec(ctx, D, d.n);
        if (l > 0) {
            d.x = vec(ctx, D, d.n);
            d.b = vec(ctx, D, d.n);
        }
        if (!d.r || (l > 0 && (!d.x || !d.b))) return fail(OPFLOW_E_NOMEM, "AMG vectors %zu", l);
        D->levels.push_back(d);
    }
    D->nc = H.levels.back().A.n;
    D->coarse_inv = up(ctx, D, H.coarse_inv);
    if (!D->coarse_inv) return fail(OPFLOW_E_NOMEM, "AMG coarse inverse");
    OPG_CUDA(cudaStreamSynchronize(ctx->stream));
    return OPFLOW_OK;
}

int amg_vcycle(opflow_ctx ctx, cudaStream_t s, AmgDev& D, const double* v, double* z) {
    const int nl = (int) D.levels.size();
    // down: pre-smoothing from zero, residual, restriction
    for (int l = 0; l < nl - 1; ++l) {
        AmgLevelDev& L = D.levels[l];
        const double* b = l == 0 ? v : L.b;
        double* x = l == 0 ? z : L.x;
        const int g = amg_grid(ctx, L.n);
        diag_apply<<<g, AMG_THREADS, 0, s>>>(L.n, L.M, b, x, 0);
        csr_residual<<<g, AMG_THREADS, 0, s>>>(L.n, L.Ap, L.Ac, L.Av, x, b, L.r);
        AmgLevelDev& C = D.levels[l + 1];
        csr_spmv<<<amg_grid(ctx, C.n), AMG_THREADS, 0, s>>>(C.n, L.Rp, L.Rc, L.Rv, L.r, C.b, 0);
        OPG_LAUNCHED();
    }
    {
        AmgLevelDev& L = D.levels[nl - 1];
        const double* b = nl == 1 ? v : L.b;
        double* x = nl == 1 ? z : L.x;
        dense_apply<<<amg_grid(ctx, L.n * 32), AMG_THREADS, 0, s>>>(L.n, D.coarse_inv, b, x);
        OPG_LAUNCHED();
    }
    // up: prolongation, post-smoothing
    for (int l = nl - 2; l >= 0; --l) {
        AmgLevelDev& L = D.levels[l];
        const double* b = l == 0 ? v : L.b;
        double* x = l == 0 ? z : L.x;
        const int g = amg_grid(ctx, L.n);
        csr_spmv<<<g, AMG_THREADS, 0, s>>>(L.n, L.Pp, L.Pc, L.Pv, D.levels[l + 1].x, x, 1);
        csr_residual<<<g, AMG_THREADS, 0, s>>>(L.n, L.Ap, L.Ac, L.Av, x, b, L.r);
        diag_apply<<<g, AMG_THREADS, 0, s>>>(L.n, L.M, L.r, x, 1);
        OPG_LAUNCHED();
    }
    return check_launch("amg_vcycle");
}

void amg_free(opflow_ctx ctx, AmgDev* D) {
    for (void* p : D->allocs) dev_free(ctx, p);
    D->allocs.clear();
    D->levels.clear();
    D->coarse_inv = nullptr;
    D->nc = 0;
}

}  // namespace opg
