// Krylov methods besides the fused flexible PCG of solver.cu, for the single-problem solver:
//   - restarted flexible GMRES (the reference's StructSolverType::GMRES / FGMRES / LGMRES,
//     src/Core/Solvers/Struct/StructSolverGMRES.hpp, FGMRES.hpp, LGMRES.hpp: HYPRE GMRES with k_dim),
//   - BiCGSTAB (StructSolverBiCGSTAB.hpp),
//   - PCG with a Jacobi preconditioner or none (StructSolverPCG.hpp with a non-PFMG preconditioner),
//   - the preconditioner iterated on its own (StructSolverPFMG / SMG / Jacobi used as the solver),
// each preconditioned by the multigrid V-cycle (the PFMG / SMG stand-in), one Jacobi step
// (z = D^-1 v) or nothing.  The preconditioner is applied on the right, and every method stops on the
// relative residual ||b - A x||_2 / ||b||_2 <= tol (or an absolute residual <= abs_tol), the
// reference's criterion.
//
// These run host-driven: one short host read of the step's scalars per step.  The vector work is in
// the kernels below, on the level-0 vectors of the problem (dense over the unknown box, float64), with
// inner products reduced per CTA and then across CTAs in a fixed order, so results do not depend on
// timing.
#include "mg_device.h"
#include "solver.h"

#include <cmath>
#include <vector>

namespace opg {

int mg_vcycle(MGSystem* S);  // solver.cu

namespace {

constexpr int KV_BLOCKS_PER_SM = 2;
constexpr int KV_THREADS = 256;
constexpr int KV_MAXDOT = 8;  // inner products per launch

__device__ __forceinline__ void cell_ijk(const LvlDev& L, long long c, int& i, int& j, int& k) {
    const long long n0 = L.n[0], n1 = L.n[1];
    i = (int) (c % n0);
    const long long r = c / n0;
    j = (int) (r % n1);
    k = (int) (r / n1);
}

// y = A x
__global__ void __launch_bounds__(KV_THREADS) kv_matvec(LvlDev L, const double* __restrict__ x, double* __restrict__ y) {
    for (long long c = blockIdx.x * (long long) blockDim.x + threadIdx.x; c < L.N; c += (long long) gridDim.x * blockDim.x) {
        int i, j, k;
        cell_ijk(L, c, i, j, k);
        double c0, offd;
        stencil_parts<double>(L, x, i, j, k, c, c0, offd);
        y[c] = c0 * x[c] + offd;
    }
}

// r = b - A x
__global__ void __launch_bounds__(KV_THREADS) kv_residual(LvlDev L, const double* __restrict__ b, const double* __restrict__ x,
                                                          double* __restrict__ r) {
    for (long long c = blockIdx.x * (long long) blockDim.x + threadIdx.x; c < L.N; c += (long long) gridDim.x * blockDim.x) {
        int i, j, k;
        cell_ijk(L, c, i, j, k);
        double c0, offd;
        stencil_parts<double>(L, x, i, j, k, c, c0, offd);
        r[c] = b[c] - (c0 * x[c] + offd);
    }
}

// z = v / diag(A)  (one Jacobi step from a zero guess)
__global__ void __launch_bounds__(KV_THREADS) kv_jacobi(LvlDev L, const double* __restrict__ v, double* __restrict__ z) {
    for (long long c = blockIdx.x * (long long) blockDim.x + threadIdx.x; c < L.N; c += (long long) gridDim.x * blockDim.x) {
        int i, j, k;
        cell_ijk(L, c, i, j, k);
        const int cls = pos_class(i, L.n[0]) + 3 * (L.ndim > 1 ? pos_class(j, L.n[1]) : 0) + 9 * (L.ndim > 2 ? pos_class(k, L.n[2]) : 0);
        const double d = L.table ? L.T64[cls * TSTRIDE] : L.A64[c];
        z[c] = v[c] / d;
    }
}

// the V-cycle's level-0 input: b = v (in the V-cycle's precision), x = 0
template <typename T>
__global__ void kv_to_vcycle(long long n, const double* __restrict__ v, T* __restrict__ b, T* __restrict__ x) {
    for (long long c = blockIdx.x * (long long) blockDim.x + threadIdx.x; c < n; c += (long long) gridDim.x * blockDim.x) {
        b[c] = (T) v[c];
        x[c] = (T) 0;
    }
}
template <typename T>
__global__ void kv_from_vcycle(long long n, const T* __restrict__ x, double* __restrict__ z) {
    for (long long c = blockIdx.x * (long long) blockDim.x + threadIdx.x; c < n; c += (long long) gridDim.x * blockDim.x) z[c] = (double) x[c];
}

// part[blk * NV + q] = sum over the block's cells of w * v_q, v_q = base + (q0 + q) * stride
template <int NV>
__global__ void __launch_bounds__(KV_THREADS) kv_dots(const double* __restrict__ base, long long stride, int q0, const double* __restrict__ w,
                                                     long long n, double* __restrict__ part) {
    double acc[NV];
#pragma unroll
    for (int q = 0; q < NV; ++q) acc[q] = 0.;
    for (long long c = blockIdx.x * (long long) blockDim.x + threadIdx.x; c < n; c += (long long) gridDim.x * blockDim.x) {
        const double wc = w[c];
#pragma unroll
        for (int q = 0; q < NV; ++q) acc[q] += wc * base[(q0 + q) * stride + c];
    }
    __shared__ double red[KV_THREADS / 32][NV];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < NV; ++q) {
        double v = acc[q];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) red[warp][q] = v;
    }
    __syncthreads();
    if (threadIdx.x < NV) {
        double s = 0.;
        for (int wi = 0; wi < KV_THREADS / 32; ++wi) s += red[wi][threadIdx.x];
        part[blockIdx.x * NV + threadIdx.x] = s;
    }
}

// out[q] = sum over blocks (in order) of part[blk * nv + q]
__global__ void kv_reduce(const double* __restrict__ part, int nblk, int nv, double* __restrict__ out) {
    const int q = threadIdx.x;
    if (q < nv) {
        double s = 0.;
        for (int b = 0; b < nblk; ++b) s += part[b * nv + q];
        out[q] = s;
    }
}

// w += sign * sum_q coef[q] * v_q (v_q = base + (q0 + q) * stride), coefficients on the device
__global__ void __launch_bounds__(KV_THREADS) kv_maxpy(double* __restrict__ w, const double* __restrict__ base, long long stride, int q0, int nv,
                                                      const double* __restrict__ coef, double sign, long long n) {
    for (long long c = blockIdx.x * (long long) blockDim.x + threadIdx.x; c < n; c += (long long) gridDim.x * blockDim.x) {
        double s = 0.;
        for (int q = 0; q < nv; ++q) s += coef[q] * base[(q0 + q) * stride + c];
        w[c] += sign * s;
    }
}

// y = a*x + b*y (+ c*z when z is set); with b == 0 the old y is not read
__global__ void __launch_bounds__(KV_THREADS) kv_axpby(long long n, double a, const double* __restrict__ x, double b, double* __restrict__ y,
                                                      double c, const double* __restrict__ z) {
    for (long long t = blockIdx.x * (long long) blockDim.x + threadIdx.x; t < n; t += (long long) gridDim.x * blockDim.x) {
        double v = a * x[t];
        if (b != 0.) v += b * y[t];
        if (z) v += c * z[t];
        y[t] = v;
    }
}

}  // namespace

// Workspace of the host-driven methods, carved from the system's arena once.
struct KrylovWork {
    int kdim = 0;
    long long N = 0;
    double* vec = nullptr;  // nvec vectors of N
    int nvec = 0;
    double* part = nullptr;  // blocks x KV_MAXDOT
    double* dred = nullptr;  // reduced inner products (64)
    double* dcoef = nullptr; // coefficients of kv_maxpy (64)
    int blocks = 0;
    double* v(int q) const { return vec + (long long) q * N; }
};

namespace {

struct Ctx {
    KrylovOp* op;
    KrylovWork* W;
    cudaStream_t s;
    int grid;
    long long N;
};

int launch_ok(const char* what) { return check_launch(what); }

int matvec(Ctx& c, const double* x, double* y) { return c.op->matvec(x, y); }
int residual(Ctx& c, const double* b, const double* x, double* r) { return c.op->residual(b, x, r); }
int precond(Ctx& c, const double* v, double* z) { return c.op->precond(v, z); }

// dred[0..nv) = <w, v_{q0..q0+nv}> (device only)
int dots_dev(Ctx& c, const double* base, long long stride, int q0, int nv, const double* w) {
    for (int done = 0; done < nv;) {
        const int m = std::min(KV_MAXDOT, nv - done);
        switch (m) {
            case 1: kv_dots<1><<<c.W->blocks, KV_THREADS, 0, c.s>>>(base, stride, q0 + done, w, c.N, c.W->part); break;
            case 2: kv_dots<2><<<c.W->blocks, KV_THREADS, 0, c.s>>>(base, stride, q0 + done, w, c.N, c.W->part); break;
            case 3: kv_dots<3><<<c.W->blocks, KV_THREADS, 0, c.s>>>(base, stride, q0 + done, w, c.N, c.W->part); break;
            case 4: kv_dots<4><<<c.W->blocks, KV_THREADS, 0, c.s>>>(base, stride, q0 + done, w, c.N, c.W->part); break;
            case 5: kv_dots<5><<<c.W->blocks, KV_THREADS, 0, c.s>>>(base, stride, q0 + done, w, c.N, c.W->part); break;
            case 6: kv_dots<6><<<c.W->blocks, KV_THREADS, 0, c.s>>>(base, stride, q0 + done, w, c.N, c.W->part); break;
            case 7: kv_dots<7><<<c.W->blocks, KV_THREADS, 0, c.s>>>(base, stride, q0 + done, w, c.N, c.W->part); break;
            default: kv_dots<8><<<c.W->blocks, KV_THREADS, 0, c.s>>>(base, stride, q0 + done, w, c.N, c.W->part); break;
        }
        OPG_LAUNCHED();
        kv_reduce<<<1, 32, 0, c.s>>>(c.W->part, c.W->blocks, m, c.W->dred + done);
        OPG_LAUNCHED();
        done += m;
    }
    return launch_ok("kv_dots");
}

// <a, b> on the host
int dot(Ctx& c, const double* a, const double* b, double* out) {
    OPG_TRY(dots_dev(c, a, 0, 0, 1, b));
    OPG_CUDA(cudaMemcpyAsync(out, c.W->dred, 8, cudaMemcpyDeviceToHost, c.s));
    OPG_CUDA(cudaStreamSynchronize(c.s));
    return OPFLOW_OK;
}

int axpby(Ctx& c, double a, const double* x, double b, double* y, double cc = 0., const double* z = nullptr) {
    kv_axpby<<<c.grid, KV_THREADS, 0, c.s>>>(c.N, a, x, b, y, cc, z);
    OPG_LAUNCHED();
    return launch_ok("kv_axpby");
}

bool reached(double rnorm, double bnorm, const KrylovParams& P) {
    if (P.abs_tol > 0 && rnorm <= P.abs_tol) return true;
    return bnorm > 0 ? rnorm <= P.tol * bnorm : rnorm == 0.;
}

// ---------------------------------------------------------------------------------------- FGMRES(m)
// Right-preconditioned restarted GMRES with the preconditioned vectors kept (flexible form, so a
// float32 V-cycle is safe); classical Gram-Schmidt applied twice; Givens rotations on the host.
int fgmres(Ctx& c, const KrylovParams& P, double* b, double* x, int* iters) {
    KrylovWork& W = *c.W;
    const int m = W.kdim;
    // vectors: V_0..V_m at 0..m, Z_0..Z_{m-1} at m+1..2m, w at 2m+1
    double* Vb = W.v(0);
    double* Zb = W.v(m + 1);
    double* w = W.v(2 * m + 1);
    double bnorm2;
    OPG_TRY(dot(c, b, b, &bnorm2));
    const double bnorm = std::sqrt(bnorm2);
    std::vector<double> H((size_t) (m + 1) * m), cs(m), sn(m), g(m + 1), y(m);
    int it = 0;
    for (;;) {
        OPG_TRY(residual(c, b, x, Vb));
        double beta2;
        OPG_TRY(dot(c, Vb, Vb, &beta2));
        const double beta = std::sqrt(beta2);
        if (reached(beta, bnorm, P) || it >= P.max_iter) break;
        OPG_TRY(axpby(c, 0., Vb, 1. / beta, Vb));
        std::fill(g.begin(), g.end(), 0.);
        g[0] = beta;
        int j = 0;
        for (; j < m && it < P.max_iter; ++j) {
            ++it;
            OPG_TRY(precond(c, W.v(j), W.v(m + 1 + j)));
            OPG_TRY(matvec(c, W.v(m + 1 + j), w));
            // h = V^T w, w -= V h, twice
            double h[64] = {0};
            for (int pass = 0; pass < 2; ++pass) {
                OPG_TRY(dots_dev(c, Vb, W.N, 0, j + 1, w));
                kv_maxpy<<<c.grid, KV_THREADS, 0, c.s>>>(w, Vb, W.N, 0, j + 1, W.dred, -1., c.N);
                OPG_LAUNCHED();
                double hp[64];
                OPG_CUDA(cudaMemcpyAsync(hp, W.dred, (j + 1) * 8, cudaMemcpyDeviceToHost, c.s));
                OPG_CUDA(cudaStreamSynchronize(c.s));
                for (int q = 0; q <= j; ++q) h[q] += hp[q];
            }
            double hn2;
            OPG_TRY(dot(c, w, w, &hn2));
            const double hn = std::sqrt(hn2);
            if (hn > 0) OPG_TRY(axpby(c, 1. / hn, w, 0., W.v(j + 1)));  // v_{j+1} = w / |w|
            // previous rotations, then a new one that annihilates hn
            for (int q = 0; q < j; ++q) {
                const double t = cs[q] * h[q] + sn[q] * h[q + 1];
                h[q + 1] = -sn[q] * h[q] + cs[q] * h[q + 1];
                h[q] = t;
            }
            const double den = std::hypot(h[j], hn);
            cs[j] = den > 0 ? h[j] / den : 1.;
            sn[j] = den > 0 ? hn / den : 0.;
            h[j] = den;
            g[j + 1] = -sn[j] * g[j];
            g[j] = cs[j] * g[j];
            for (int q = 0; q <= j; ++q) H[(size_t) q * m + j] = h[q];
            if (reached(std::fabs(g[j + 1]), bnorm, P) || hn == 0.) {
                ++j;
                break;
            }
        }
        // y = H^-1 g (upper triangular), x += Z y
        for (int q = j - 1; q >= 0; --q) {
            double s = g[q];
            for (int r = q + 1; r < j; ++r) s -= H[(size_t) q * m + r] * y[r];
            y[q] = H[(size_t) q * m + q] != 0 ? s / H[(size_t) q * m + q] : 0.;
        }
        if (j > 0) {
            OPG_CUDA(cudaMemcpyAsync(W.dcoef, y.data(), j * 8, cudaMemcpyHostToDevice, c.s));
            kv_maxpy<<<c.grid, KV_THREADS, 0, c.s>>>(x, Zb, W.N, 0, j, W.dcoef, 1., c.N);
            OPG_LAUNCHED();
        }
    }
    *iters = it;
    return launch_ok("fgmres");
}

// ---------------------------------------------------------------------------------------- BiCGSTAB
int bicgstab(Ctx& c, const KrylovParams& P, double* b, double* x, int* iters) {
    KrylovWork& W = *c.W;
    double *r = W.v(0), *rh = W.v(1), *p = W.v(2), *v = W.v(3), *ph = W.v(4), *s = W.v(5), *sh = W.v(6), *t = W.v(7);
    double bnorm2;
    OPG_TRY(dot(c, b, b, &bnorm2));
    const double bnorm = std::sqrt(bnorm2);
    OPG_TRY(residual(c, b, x, r));
    double rho_old = 1., alpha = 1., omega = 1., rr;
    OPG_TRY(dot(c, r, r, &rr));
    int it = 0;
    // The recurrence residual drifts from b - A x on ill-conditioned systems (a pinned row): when it
    // reports convergence the true residual is formed, and the iteration restarts from it (shadow
    // residual reset) until the true residual meets the tolerance (at most four restarts).
    for (int restarts = 0;; ++restarts) {
        OPG_CUDA(cudaMemcpyAsync(rh, r, c.N * 8, cudaMemcpyDeviceToDevice, c.s));
        OPG_CUDA(cudaMemsetAsync(p, 0, c.N * 8, c.s));
        OPG_CUDA(cudaMemsetAsync(v, 0, c.N * 8, c.s));
        rho_old = alpha = omega = 1.;
        while (!reached(std::sqrt(rr), bnorm, P) && it < P.max_iter) {
            ++it;
            double rho;
            OPG_TRY(dot(c, rh, r, &rho));
            if (rho == 0.) {  // breakdown: restart the shadow residual
                OPG_CUDA(cudaMemcpyAsync(rh, r, c.N * 8, cudaMemcpyDeviceToDevice, c.s));
                OPG_CUDA(cudaMemsetAsync(p, 0, c.N * 8, c.s));
                OPG_CUDA(cudaMemsetAsync(v, 0, c.N * 8, c.s));
                rho_old = alpha = omega = 1.;
                OPG_TRY(dot(c, rh, r, &rho));
                if (rho == 0.) break;
            }
            const double beta = (rho / rho_old) * (alpha / omega);
            OPG_TRY(axpby(c, 1., r, beta, p, -beta * omega, v));  // p = r + beta (p - omega v)
            OPG_TRY(precond(c, p, ph));
            OPG_TRY(matvec(c, ph, v));
            double rv;
            OPG_TRY(dot(c, rh, v, &rv));
            alpha = rv != 0. ? rho / rv : 0.;
            OPG_CUDA(cudaMemcpyAsync(s, r, c.N * 8, cudaMemcpyDeviceToDevice, c.s));
            OPG_TRY(axpby(c, -alpha, v, 1., s));  // s = r - alpha v
            double ss;
            OPG_TRY(dot(c, s, s, &ss));
            if (reached(std::sqrt(ss), bnorm, P)) {
                OPG_TRY(axpby(c, alpha, ph, 1., x));
                rr = ss;
                break;
            }
            OPG_TRY(precond(c, s, sh));
            OPG_TRY(matvec(c, sh, t));
            double ts, tt;
            OPG_TRY(dot(c, t, s, &ts));
            OPG_TRY(dot(c, t, t, &tt));
            omega = tt != 0. ? ts / tt : 0.;
            OPG_TRY(axpby(c, alpha, ph, 1., x, omega, sh));  // x += alpha ph + omega sh
            OPG_CUDA(cudaMemcpyAsync(r, s, c.N * 8, cudaMemcpyDeviceToDevice, c.s));
            OPG_TRY(axpby(c, -omega, t, 1., r));  // r = s - omega t
            OPG_TRY(dot(c, r, r, &rr));
            rho_old = rho;
            if (omega == 0.) break;
        }
        if (it >= P.max_iter || restarts >= 4) break;
        OPG_TRY(residual(c, b, x, r));
        OPG_TRY(dot(c, r, r, &rr));
        if (reached(std::sqrt(rr), bnorm, P)) break;
    }
    *iters = it;
    return OPFLOW_OK;
}

// ---------------------------------------------------------------------------------------- PCG
int pcg(Ctx& c, const KrylovParams& P, double* b, double* x, int* iters) {
    KrylovWork& W = *c.W;
    double *r = W.v(0), *z = W.v(1), *p = W.v(2), *q = W.v(3);
    double bnorm2;
    OPG_TRY(dot(c, b, b, &bnorm2));
    const double bnorm = std::sqrt(bnorm2);
    OPG_TRY(residual(c, b, x, r));
    double rr;
    OPG_TRY(dot(c, r, r, &rr));
    OPG_TRY(precond(c, r, z));
    OPG_CUDA(cudaMemcpyAsync(p, z, c.N * 8, cudaMemcpyDeviceToDevice, c.s));
    double rz;
    OPG_TRY(dot(c, r, z, &rz));
    int it = 0;
    while (!reached(std::sqrt(rr), bnorm, P) && it < P.max_iter) {
        ++it;
        OPG_TRY(matvec(c, p, q));
        double pq;
        OPG_TRY(dot(c, p, q, &pq));
        if (pq == 0.) break;
        const double alpha = rz / pq;
        OPG_TRY(axpby(c, alpha, p, 1., x));
        OPG_TRY(axpby(c, -alpha, q, 1., r));
        OPG_TRY(dot(c, r, r, &rr));
        if (reached(std::sqrt(rr), bnorm, P)) break;
        OPG_TRY(precond(c, r, z));
        double rz_new;
        OPG_TRY(dot(c, r, z, &rz_new));
        const double beta = rz != 0. ? rz_new / rz : 0.;
        rz = rz_new;
        OPG_TRY(axpby(c, 1., z, beta, p));  // p = z + beta p
    }
    *iters = it;
    return OPFLOW_OK;
}

// ---------------------------------------------------------------------------------------- stationary
// x += M (b - A x) until converged: the multigrid V-cycle (PFMG / SMG as the solver) or Jacobi
int stationary(Ctx& c, const KrylovParams& P, double* b, double* x, int* iters) {
    KrylovWork& W = *c.W;
    double *r = W.v(0), *z = W.v(1);
    double bnorm2;
    OPG_TRY(dot(c, b, b, &bnorm2));
    const double bnorm = std::sqrt(bnorm2);
    int it = 0;
    for (;;) {
        OPG_TRY(residual(c, b, x, r));
        double rr;
        OPG_TRY(dot(c, r, r, &rr));
        if (reached(std::sqrt(rr), bnorm, P) || it >= P.max_iter) break;
        ++it;
        OPG_TRY(precond(c, r, z));
        OPG_TRY(axpby(c, 1., z, 1., x));
    }
    *iters = it;
    return OPFLOW_OK;
}

// The operator of one multigrid system's level 0 with its preconditioners.
struct MgOp : KrylovOp {
    MGSystem* S;
    LvlDev L0;
    cudaStream_t s;
    int grid;
    long long N;
    int pc;
    bool f32;
    int matvec(const double* x, double* y) override {
        kv_matvec<<<grid, KV_THREADS, 0, s>>>(L0, x, y);
        OPG_LAUNCHED();
        return launch_ok("kv_matvec");
    }
    int residual(const double* b, const double* x, double* r) override {
        kv_residual<<<grid, KV_THREADS, 0, s>>>(L0, b, x, r);
        OPG_LAUNCHED();
        return launch_ok("kv_residual");
    }
    int precond(const double* v, double* z) override {
        if (pc == OPFLOW_PRECOND_NONE) {
            OPG_CUDA(cudaMemcpyAsync(z, v, N * 8, cudaMemcpyDeviceToDevice, s));
            return OPFLOW_OK;
        }
        if (pc == OPFLOW_PRECOND_JACOBI) {
            kv_jacobi<<<grid, KV_THREADS, 0, s>>>(L0, v, z);
            OPG_LAUNCHED();
            return launch_ok("kv_jacobi");
        }
        return mg_precond_level0(S, v, z);
    }
};

}  // namespace

int KrylovOp::residual(const double* b, const double* x, double* r) {
    OPG_TRY(matvec(x, r));
    kv_axpby<<<grid_hint, KV_THREADS, 0, stream>>>(n, 1., b, -1., r, 0., nullptr);  // r = b - A x
    OPG_LAUNCHED();
    return launch_ok("kv_axpby");
}

// z = V-cycle(v) on S's level 0 (its single problem must be active)
int mg_precond_level0(MGSystem* S, const double* v, double* z) {
    const ProblemHost& Pr = S->probs[0];
    const LvlDev& L0 = S->lv_host[Pr.lvl0];
    const long long N = Pr.levels[0].N;
    cudaStream_t s = S->ctx->stream;
    const int grid = (int) std::max<long long>(1, std::min<long long>((N + KV_THREADS - 1) / KV_THREADS, (long long) S->ctx->num_sms * 8));
    if (S->precision == OPFLOW_PREC_MIXED) kv_to_vcycle<float><<<grid, KV_THREADS, 0, s>>>(N, v, L0.b32, L0.x32);
    else kv_to_vcycle<double><<<grid, KV_THREADS, 0, s>>>(N, v, L0.b64, L0.x64);
    OPG_LAUNCHED();
    OPG_TRY(mg_vcycle(S));
    if (S->precision == OPFLOW_PREC_MIXED) kv_from_vcycle<float><<<grid, KV_THREADS, 0, s>>>(N, L0.x32, z);
    else kv_from_vcycle<double><<<grid, KV_THREADS, 0, s>>>(N, L0.x64, z);
    OPG_LAUNCHED();
    return launch_ok("kv_from_vcycle");
}

// marks S's single problem active for the V-cycle kernels (they skip inactive problems)
int mg_activate(MGSystem* S) {
    Scal sc{};
    sc.active = 1;
    OPG_CUDA(cudaMemcpyAsync(S->dS, &sc, sizeof sc, cudaMemcpyHostToDevice, S->ctx->stream));
    return OPFLOW_OK;
}

int krylov_vectors(const KrylovParams& P) {
    return (P.method == OPFLOW_KRYLOV_GMRES || P.method == OPFLOW_KRYLOV_FGMRES || P.method == OPFLOW_KRYLOV_LGMRES) ? 2 * P.kdim + 2 : 8;
}

KrylovWork* krylov_work(Arena& arena, opflow_ctx ctx, long long N, const KrylovParams& P) {
    auto* W = new KrylovWork();
    W->N = N;
    W->nvec = krylov_vectors(P);
    W->kdim = P.kdim;
    W->blocks = std::max(1, ctx->num_sms * KV_BLOCKS_PER_SM);
    W->vec = (double*) arena.alloc((size_t) W->nvec * N * 8);
    W->part = (double*) arena.alloc((size_t) W->blocks * KV_MAXDOT * 8);
    W->dred = (double*) arena.alloc(64 * 8);
    W->dcoef = (double*) arena.alloc(64 * 8);
    if (!W->vec || !W->part || !W->dred || !W->dcoef) {
        delete W;
        return nullptr;
    }
    return W;
}

void krylov_work_free(KrylovWork* W) { delete W; }

bool krylov_work_fits(const KrylovWork* W, long long N, const KrylovParams& P) {
    return W && W->N == N && W->nvec >= krylov_vectors(P) && W->kdim == P.kdim;
}

int krylov_run(KrylovOp& op, KrylovWork& W, opflow_ctx ctx, long long N, const KrylovParams& P, double* b, double* x, int* iters) {
    if (P.kdim < 1 || P.kdim > 60) return fail(OPFLOW_E_INVALID, "GMRES restart length must be 1..60");
    Ctx c{};
    c.op = &op;
    c.W = &W;
    c.s = ctx->stream;
    c.N = N;
    c.grid = (int) std::max<long long>(1, std::min<long long>((N + KV_THREADS - 1) / KV_THREADS, (long long) ctx->num_sms * 8));
    op.stream = c.s;
    op.grid_hint = c.grid;
    op.n = N;
    switch (P.method) {
        case OPFLOW_KRYLOV_GMRES: case OPFLOW_KRYLOV_FGMRES: case OPFLOW_KRYLOV_LGMRES: return fgmres(c, P, b, x, iters);
        case OPFLOW_KRYLOV_BICGSTAB: return bicgstab(c, P, b, x, iters);
        case OPFLOW_KRYLOV_PCG: return pcg(c, P, b, x, iters);
        case OPFLOW_KRYLOV_NONE: return stationary(c, P, b, x, iters);
    }
    return fail(OPFLOW_E_INVALID, "unknown Krylov method %d", P.method);
}

void krylov_release(MGSystem* S) {
    delete S->kwork;
    S->kwork = nullptr;
}

int krylov_solve(MGSystem* S, const KrylovParams& P, int* iters) {
    if (S->probs.size() != 1) return fail(OPFLOW_E_INVALID, "the host-driven Krylov methods solve one problem");
    opflow_ctx ctx = S->ctx;
    const ProblemHost& Pr = S->probs[0];
    const KrylovDev& K = S->kd_host[0];
    const long long N = Pr.levels[0].N;
    if (!krylov_work_fits(S->kwork, N, P)) {
        krylov_release(S);
        S->kwork = krylov_work(S->arena, ctx, N, P);
        if (!S->kwork) return fail(OPFLOW_E_NOMEM, "Krylov workspace");
    }
    MgOp op;
    op.S = S;
    op.L0 = S->lv_host[Pr.lvl0];
    op.s = ctx->stream;
    op.N = N;
    op.grid = (int) std::max<long long>(1, std::min<long long>((N + KV_THREADS - 1) / KV_THREADS, (long long) ctx->num_sms * 8));
    op.pc = P.precond;
    op.f32 = S->precision == OPFLOW_PREC_MIXED;
    if (op.pc == OPFLOW_PRECOND_MG) OPG_TRY(mg_activate(S));
    return krylov_run(op, *S->kwork, ctx, N, P, K.b, K.x, iters);
}

}  // namespace opg
