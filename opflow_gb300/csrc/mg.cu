// Multigrid V-cycle and flexible-PCG kernels over chunk lists.
//
// Every kernel walks a list of row segments ("chunks") that may belong to many problems and levels, so
// one launch serves a single solve or a batch of uneven problems alike (a persistent grid strides over
// the list).  Inner products are formed per chunk inside one CTA in a fixed order and then reduced per
// problem in a fixed order, so a problem's iterates are bit-identical whether it runs alone or in a
// batch.  T selects the precision of the V-cycle (float for the mixed form, double for the plain one);
// the Krylov vectors, their updates and all inner products are float64.
#include "mg_kernels.h"

namespace opg {

template <typename T> struct Sel;
template <> struct Sel<double> {
    __device__ static double* x(const LvlDev& L) { return L.x64; }
    __device__ static double* b(const LvlDev& L) { return L.b64; }
    __device__ static double* r(const LvlDev& L) { return L.r64; }
    __device__ static const double* A(const LvlDev& L) { return L.A64; }
    __device__ static const double* Tb(const LvlDev& L) { return L.T64; }
};
template <> struct Sel<float> {
    __device__ static float* x(const LvlDev& L) { return L.x32; }
    __device__ static float* b(const LvlDev& L) { return L.b32; }
    __device__ static float* r(const LvlDev& L) { return L.r32; }
    __device__ static const float* A(const LvlDev& L) { return L.A32; }
    __device__ static const float* Tb(const LvlDev& L) { return L.T32; }
};

__device__ __forceinline__ int pos_class(int i, int n) { return i == 0 ? 0 : (i == n - 1 ? 2 : 1); }

// A x at (i, j, k) with the level's coefficients; neighbours outside a non-periodic box carry no
// coupling (the assembly folded them).  Returns the off-diagonal part in `offd` and the centre in c0.
template <typename T, typename V>
__device__ __forceinline__ void stencil_parts(const LvlDev& L, const V* __restrict__ x, int i, int j, int k, long long cell, T& c0, T& offd) {
    const int cls = pos_class(i, L.n[0]) + 3 * (L.ndim > 1 ? pos_class(j, L.n[1]) : 0) + 9 * (L.ndim > 2 ? pos_class(k, L.n[2]) : 0);
    const T* A = Sel<T>::A(L);
    const T* Tb = Sel<T>::Tb(L);
    auto cf = [&](int s) -> T { return L.table ? Tb[cls * NSLOT + s] : A[(long long) s * L.N + cell]; };
    c0 = cf(0);
    T acc = 0;
    const int n0 = L.n[0];
    // x direction
    {
        int im = i - 1, ip = i + 1;
        if (im < 0 && L.per[0]) im += n0;
        if (ip >= n0 && L.per[0]) ip -= n0;
        if (im >= 0) acc += cf(1) * (T) x[cell - i + im];
        if (ip < n0) acc += cf(2) * (T) x[cell - i + ip];
    }
    if (L.ndim > 1) {
        const int n1 = L.n[1];
        const long long sy = n0;
        int jm = j - 1, jp = j + 1;
        if (jm < 0 && L.per[1]) jm += n1;
        if (jp >= n1 && L.per[1]) jp -= n1;
        if (jm >= 0) acc += cf(3) * (T) x[cell + (jm - j) * sy];
        if (jp < n1) acc += cf(4) * (T) x[cell + (jp - j) * sy];
    }
    if (L.ndim > 2) {
        const int n2 = L.n[2];
        const long long sz = (long long) n0 * L.n[1];
        int km = k - 1, kp = k + 1;
        if (km < 0 && L.per[2]) km += n2;
        if (kp >= n2 && L.per[2]) kp -= n2;
        if (km >= 0) acc += cf(5) * (T) x[cell + (km - k) * sz];
        if (kp < n2) acc += cf(6) * (T) x[cell + (kp - k) * sz];
    }
    offd = acc;
}

__device__ __forceinline__ long long cell_of(const LvlDev& L, int i, int j, int k) {
    return (long long) i + (long long) L.n[0] * ((long long) j + (long long) L.n[1] * k);
}

__device__ __forceinline__ bool active(const LvlDev* L, const Chunk& c, const Scal* sc) {
    return !sc || sc[L[c.lvl].problem].active;
}

// ------------------------------------------------------------------------------------ V-cycle pieces
// Per-cell bodies, shared by the chunked kernels (large levels, a grid strides over row segments) and
// the bottom kernel (small levels, one CTA walks every cell of a problem's level), so both give
// bit-identical values.

// r = b - A x
template <typename T>
__device__ __forceinline__ void cell_residual(const LvlDev& L, int i, int j, int k) {
    const long long cell = cell_of(L, i, j, k);
    const T* x = Sel<T>::x(L);
    T c0, offd;
    stencil_parts<T>(L, x, i, j, k, cell, c0, offd);
    Sel<T>::r(L)[cell] = Sel<T>::b(L)[cell] - (c0 * x[cell] + offd);
}

// Gauss-Seidel update of one cell: x = (b - offd) / c0
template <typename T>
__device__ __forceinline__ void cell_gs(const LvlDev& L, int i, int j, int k) {
    const long long cell = cell_of(L, i, j, k);
    T* x = Sel<T>::x(L);
    T c0, offd;
    stencil_parts<T>(L, x, i, j, k, cell, c0, offd);
    x[cell] = (Sel<T>::b(L)[cell] - offd) / c0;
}

// damped Jacobi in two phases: 0 forms r = b - A x, 1 applies x += 0.8 r / diag
template <typename T>
__device__ __forceinline__ void cell_jacobi(const LvlDev& L, int i, int j, int k, int phase) {
    const long long cell = cell_of(L, i, j, k);
    T* x = Sel<T>::x(L);
    T* r = Sel<T>::r(L);
    T c0, offd;
    stencil_parts<T>(L, x, i, j, k, cell, c0, offd);
    if (phase == 0) r[cell] = Sel<T>::b(L)[cell] - (c0 * x[cell] + offd);
    else x[cell] += (T) 0.8 * r[cell] / c0;
}

// coarse b = R r_fine at coarse cell I, coarse x = 0
template <typename T>
__device__ __forceinline__ void cell_restrict(const LvlDev* __restrict__ Ls, const LvlDev& Lc, int I0, int I1, int I2) {
    const LvlDev& Lf = Ls[Lc.fine];
    const T* rf = Sel<T>::r(Lf);
    const int I[3] = {I0, I1, I2};
    const long long cc = cell_of(Lc, I[0], I[1], I[2]);
    T acc = 0;
    if (!Lc.node) {
        // average of the children that exist
        int cnt = 0;
        for (int dz = 0; dz < (Lc.ndim > 2 ? 2 : 1); ++dz)
            for (int dy = 0; dy < (Lc.ndim > 1 ? 2 : 1); ++dy)
                for (int dx = 0; dx < 2; ++dx) {
                    const int fi = 2 * I[0] + dx, fj = 2 * I[1] + dy, fk = 2 * I[2] + dz;
                    if (fi < Lf.n[0] && fj < Lf.n[1] && fk < Lf.n[2]) {
                        acc += rf[cell_of(Lf, fi, fj, fk)];
                        cnt++;
                    }
                }
        acc = acc / (T) cnt;
    } else {
        // full weighting on absolute node indices: coarse node I <-> fine node 2I
        const int ga[3] = {Lc.lo[0] + I[0], Lc.lo[1] + I[1], Lc.lo[2] + I[2]};
        const int rz = Lc.ndim > 2 ? 1 : 0, ry = Lc.ndim > 1 ? 1 : 0;
        for (int dz = -rz; dz <= rz; ++dz)
            for (int dy = -ry; dy <= ry; ++dy)
                for (int dx = -1; dx <= 1; ++dx) {
                    T w = dx == 0 ? (T) 0.5 : (T) 0.25;
                    if (ry) w *= dy == 0 ? (T) 0.5 : (T) 0.25;
                    if (rz) w *= dz == 0 ? (T) 0.5 : (T) 0.25;
                    const int fi = 2 * ga[0] + dx - Lf.lo[0], fj = 2 * ga[1] + dy - Lf.lo[1], fk = 2 * ga[2] + dz - Lf.lo[2];
                    if (fi >= 0 && fi < Lf.n[0] && fj >= 0 && fj < Lf.n[1] && fk >= 0 && fk < Lf.n[2]) acc += w * rf[cell_of(Lf, fi, fj, fk)];
                }
    }
    Sel<T>::b(Lc)[cc] = acc;
    Sel<T>::x(Lc)[cc] = 0;
}

// value of a coarse unknown for interpolation, with the boundary ghost rules
template <typename T>
__device__ __forceinline__ T coarse_at(const LvlDev& Lc, const T* xc, int I0, int I1, int I2, T& sign_out) {
    int I[3] = {I0, I1, I2};
    T sgn = 1;
    for (int d = 0; d < Lc.ndim; ++d) {
        if (I[d] < 0) {
            if (Lc.gh_lo[d] == GH_WRAP) I[d] += Lc.n[d];
            else if (Lc.gh_lo[d] == GH_COPY) I[d] = 0;
            else { sgn = -sgn; I[d] = 0; }
        } else if (I[d] >= Lc.n[d]) {
            if (Lc.gh_hi[d] == GH_WRAP) I[d] -= Lc.n[d];
            else if (Lc.gh_hi[d] == GH_COPY) I[d] = Lc.n[d] - 1;
            else { sgn = -sgn; I[d] = Lc.n[d] - 1; }
        }
    }
    sign_out = sgn;
    return xc[cell_of(Lc, I[0], I[1], I[2])];
}

// fine x += P x_coarse at fine cell f
template <typename T>
__device__ __forceinline__ void cell_prolong(const LvlDev* __restrict__ Ls, const LvlDev& Lf, int f0, int f1, int f2) {
    const LvlDev& Lc = Ls[Lf.coarse];
    T* xf = Sel<T>::x(Lf);
    const T* xc = Sel<T>::x(Lc);
    const int f[3] = {f0, f1, f2};
    T acc = 0;
    if (!Lc.node) {
        // bilinear / trilinear on cell centres: 3/4 nearest coarse cell, 1/4 the next one
        int I[3], J[3];
        for (int d = 0; d < 3; ++d) {
            I[d] = f[d] >> 1;
            J[d] = (f[d] & 1) ? I[d] + 1 : I[d] - 1;
        }
        const int nz = Lc.ndim > 2 ? 2 : 1, ny = Lc.ndim > 1 ? 2 : 1;
        for (int a = 0; a < nz; ++a)
            for (int bb = 0; bb < ny; ++bb)
                for (int e = 0; e < 2; ++e) {
                    const T w = (e ? (T) 0.25 : (T) 0.75) * (Lc.ndim > 1 ? (bb ? (T) 0.25 : (T) 0.75) : (T) 1) *
                                (Lc.ndim > 2 ? (a ? (T) 0.25 : (T) 0.75) : (T) 1);
                    T s;
                    const T v = coarse_at<T>(Lc, xc, e ? J[0] : I[0], Lc.ndim > 1 ? (bb ? J[1] : I[1]) : 0, Lc.ndim > 2 ? (a ? J[2] : I[2]) : 0, s);
                    acc += w * s * v;
                }
    } else {
        // linear interpolation on nodes: absolute fine node g <-> coarse node g/2
        const int g[3] = {Lf.lo[0] + f[0], Lf.lo[1] + f[1], Lf.lo[2] + f[2]};
        int c0[3], c1[3];
        T w0[3], w1[3];
        for (int d = 0; d < 3; ++d) {
            if (d >= Lc.ndim) { c0[d] = c1[d] = 0; w0[d] = 1; w1[d] = 0; continue; }
            if ((g[d] & 1) == 0) { c0[d] = c1[d] = g[d] / 2 - Lc.lo[d]; w0[d] = 1; w1[d] = 0; }
            else { c0[d] = (g[d] - 1) / 2 - Lc.lo[d]; c1[d] = c0[d] + 1; w0[d] = w1[d] = (T) 0.5; }
        }
        for (int a = 0; a < 2; ++a)
            for (int bb = 0; bb < 2; ++bb)
                for (int e = 0; e < 2; ++e) {
                    const T w = (e ? w1[0] : w0[0]) * (bb ? w1[1] : w0[1]) * (a ? w1[2] : w0[2]);
                    if (w == (T) 0) continue;
                    const int I0 = e ? c1[0] : c0[0], I1 = bb ? c1[1] : c0[1], I2 = a ? c1[2] : c0[2];
                    bool in = I0 >= 0 && I0 < Lc.n[0] && I1 >= 0 && I1 < Lc.n[1] && I2 >= 0 && I2 < Lc.n[2];
                    if (in) acc += w * xc[cell_of(Lc, I0, I1, I2)];
                    else {
                        T s;
                        const T v = coarse_at<T>(Lc, xc, I0, I1, I2, s);
                        // outside a Dirichlet boundary the coarse correction is 0
                        bool zero = false;
                        const int II[3] = {I0, I1, I2};
                        for (int d = 0; d < Lc.ndim; ++d)
                            if ((II[d] < 0 && Lc.gh_lo[d] == GH_ZERO) || (II[d] >= Lc.n[d] && Lc.gh_hi[d] == GH_ZERO)) zero = true;
                        if (!zero) acc += w * s * v;
                    }
                }
    }
    xf[cell_of(Lf, f[0], f[1], f[2])] += acc;
}

// coarsest level: x = Ainv b (dense, accumulated in float64), rows t0, t0+dt, ...
template <typename T>
__device__ __forceinline__ void coarse_rows(const LvlDev& L, int t0, int dt) {
    const T* b = Sel<T>::b(L);
    T* x = Sel<T>::x(L);
    const int N = (int) L.N;
    for (int row = t0; row < N; row += dt) {
        double acc = 0.;
        const double* Ar = L.Ainv64 + (long long) row * N;
        for (int col = 0; col < N; ++col) acc = fma(Ar[col], (double) b[col], acc);
        x[row] = (T) acc;
    }
}

// ---- chunked kernels (large levels)
template <typename T>
__global__ void __launch_bounds__(256) mg_residual(const LvlDev* __restrict__ Ls, const Chunk* __restrict__ ch, int nch, const Scal* sc) {
    for (int c = blockIdx.x; c < nch; c += gridDim.x) {
        const Chunk C = ch[c];
        if (!active(Ls, C, sc)) continue;
        const LvlDev& L = Ls[C.lvl];
        for (int t = threadIdx.x; t < C.cnt; t += blockDim.x) cell_residual<T>(L, C.i0 + t, C.j, C.k);
    }
}

// Red-black Gauss-Seidel half sweep (cells with (i+j+k)%2 == color), or for Jacobi levels:
// color 0 computes r = b - A x, color 1 applies x += omega r / diag.
template <typename T>
__global__ void __launch_bounds__(256) mg_smooth(const LvlDev* __restrict__ Ls, const Chunk* __restrict__ ch, int nch, int color, const Scal* sc) {
    for (int c = blockIdx.x; c < nch; c += gridDim.x) {
        const Chunk C = ch[c];
        if (!active(Ls, C, sc)) continue;
        const LvlDev& L = Ls[C.lvl];
        if (L.rbgs) {
            const int first = (C.i0 + C.j + C.k + color) & 1;  // offset of the first cell of this color
            for (int t = 2 * threadIdx.x + first; t < C.cnt; t += 2 * blockDim.x) cell_gs<T>(L, C.i0 + t, C.j, C.k);
        } else {
            for (int t = threadIdx.x; t < C.cnt; t += blockDim.x) cell_jacobi<T>(L, C.i0 + t, C.j, C.k, color);
        }
    }
}

// coarse b = R r_fine, coarse x = 0; chunks are coarse rows
template <typename T>
__global__ void __launch_bounds__(256) mg_restrict(const LvlDev* __restrict__ Ls, const Chunk* __restrict__ ch, int nch, const Scal* sc) {
    for (int c = blockIdx.x; c < nch; c += gridDim.x) {
        const Chunk C = ch[c];
        if (!active(Ls, C, sc)) continue;
        const LvlDev& Lc = Ls[C.lvl];
        for (int t = threadIdx.x; t < C.cnt; t += blockDim.x) cell_restrict<T>(Ls, Lc, C.i0 + t, C.j, C.k);
    }
}

// fine x += P x_coarse; chunks are fine rows
template <typename T>
__global__ void __launch_bounds__(256) mg_prolong(const LvlDev* __restrict__ Ls, const Chunk* __restrict__ ch, int nch, const Scal* sc) {
    for (int c = blockIdx.x; c < nch; c += gridDim.x) {
        const Chunk C = ch[c];
        if (!active(Ls, C, sc)) continue;
        const LvlDev& Lf = Ls[C.lvl];
        for (int t = threadIdx.x; t < C.cnt; t += blockDim.x) cell_prolong<T>(Ls, Lf, C.i0 + t, C.j, C.k);
    }
}

// coarsest level: x = Ainv b (dense, accumulated in float64); one CTA per listed level
template <typename T>
__global__ void __launch_bounds__(256) mg_coarse(const LvlDev* __restrict__ Ls, const int* __restrict__ lv, int nlv, const Scal* sc) {
    for (int q = blockIdx.x; q < nlv; q += gridDim.x) {
        const LvlDev& L = Ls[lv[q]];
        if (sc && !sc[L.problem].active) continue;
        coarse_rows<T>(L, threadIdx.x, blockDim.x);
    }
}

// ---- bottom kernel (small levels)
// Walks every cell of level L in x-fastest order; for a red-black color only the cells of that color.
template <typename T, typename F>
__device__ __forceinline__ void for_cells(const LvlDev& L, int color, F&& f) {
    const int n0 = L.n[0], n1 = L.n[1];
    for (int c = threadIdx.x; c < (int) L.N; c += blockDim.x) {
        const int i = c % n0, jk = c / n0, j = jk % n1, k = jk / n1;
        if (color >= 0 && ((i + j + k) & 1) != color) continue;
        f(i, j, k);
    }
}

template <typename T>
__device__ __forceinline__ void bottom_smooth(const LvlDev& L, int color) {
    if (L.rbgs) for_cells<T>(L, color, [&](int i, int j, int k) { cell_gs<T>(L, i, j, k); });
    else for_cells<T>(L, -1, [&](int i, int j, int k) { cell_jacobi<T>(L, i, j, k, color); });
    __syncthreads();
}

// The V-cycle below (and including) a problem's first small level, one CTA per problem: the
// restriction into that level, pre-smoothing, residuals and restrictions down to the coarsest level,
// the coarsest solve, then prolongation and post-smoothing back up - the same operations in the same
// order as the chunked kernels, with a CTA barrier where those have a launch boundary.
template <typename T>
__global__ void __launch_bounds__(512) mg_bottom(const LvlDev* __restrict__ Ls, const int* __restrict__ top, int ntop, const Scal* sc, int pre,
                                                 int post) {
    for (int q = blockIdx.x; q < ntop; q += gridDim.x) {
        const int s = top[q];
        if (sc && !sc[Ls[s].problem].active) continue;
        if (Ls[s].fine >= 0) {
            const LvlDev& L = Ls[s];
            for_cells<T>(L, -1, [&](int i, int j, int k) { cell_restrict<T>(Ls, L, i, j, k); });
            __syncthreads();
        }
        int l = s;
        while (!Ls[l].coarsest) {
            const LvlDev& L = Ls[l];
            for (int it = 0; it < pre; ++it) {
                bottom_smooth<T>(L, 0);
                bottom_smooth<T>(L, 1);
            }
            for_cells<T>(L, -1, [&](int i, int j, int k) { cell_residual<T>(L, i, j, k); });
            __syncthreads();
            const LvlDev& Lc = Ls[L.coarse];
            for_cells<T>(Lc, -1, [&](int i, int j, int k) { cell_restrict<T>(Ls, Lc, i, j, k); });
            __syncthreads();
            l = L.coarse;
        }
        {
            const LvlDev& L = Ls[l];
            if (L.Ainv64) {
                coarse_rows<T>(L, threadIdx.x, blockDim.x);
                __syncthreads();
            } else {
                for (int it = 0; it < pre + post; ++it) {
                    bottom_smooth<T>(L, 0);
                    bottom_smooth<T>(L, 1);
                }
            }
        }
        while (l != s) {
            const LvlDev& Lf = Ls[Ls[l].fine];
            for_cells<T>(Lf, -1, [&](int i, int j, int k) { cell_prolong<T>(Ls, Lf, i, j, k); });
            __syncthreads();
            for (int it = 0; it < post; ++it) {
                bottom_smooth<T>(Lf, 1);
                bottom_smooth<T>(Lf, 0);
            }
            l = Ls[l].fine;
        }
        __syncthreads();
    }
}

// ------------------------------------------------------------------------------------ Krylov (FP64)
__device__ __forceinline__ double block_sum(double v, double* sh) {
    // fixed-order reduction: warp tree, then warp 0 over the warp sums
    for (int s = 16; s > 0; s >>= 1) v += __shfl_xor_sync(0xffffffffu, v, s);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) sh[w] = v;
    __syncthreads();
    double t = 0.;
    if (w == 0) {
        t = l < (int) (blockDim.x >> 5) ? sh[l] : 0.;
        for (int s = 16; s > 0; s >>= 1) t += __shfl_xor_sync(0xffffffffu, t, s);
    }
    return t;  // valid in thread 0
}

// mode 0: r = b - A x, partial (b.b, r.r)        mode 1: q = A p, partial (p.q)
__global__ void __launch_bounds__(256) kr_apply(const LvlDev* __restrict__ Ls, const KrylovDev* __restrict__ K, const Chunk* __restrict__ ch, int nch,
                                                const Scal* sc, double* partial, int mode) {
    __shared__ double sh[32];
    for (int c = blockIdx.x; c < nch; c += gridDim.x) {
        const Chunk C = ch[c];
        const LvlDev& L = Ls[C.lvl];
        const int pb = L.problem;
        const bool act = !sc || sc[pb].active;
        const KrylovDev& Kp = K[pb];
        double s0 = 0., s1 = 0.;
        if (act) {
            const double* in = mode == 0 ? Kp.x : Kp.p;
            for (int t = threadIdx.x; t < C.cnt; t += blockDim.x) {
                const int i = C.i0 + t;
                const long long cell = cell_of(L, i, C.j, C.k);
                double c0, offd;
                stencil_parts<double>(L, in, i, C.j, C.k, cell, c0, offd);
                const double ax = fma(c0, in[cell], offd);
                if (mode == 0) {
                    const double r = Kp.b[cell] - ax;
                    Kp.r[cell] = r;
                    s0 = fma(Kp.b[cell], Kp.b[cell], s0);
                    s1 = fma(r, r, s1);
                } else {
                    Kp.q[cell] = ax;
                    s0 = fma(in[cell], ax, s0);
                }
            }
        }
        const double a = block_sum(s0, sh);
        const double b = block_sum(s1, sh);
        if (threadIdx.x == 0) {
            partial[2 * c] = act ? a : 0.;
            partial[2 * c + 1] = act ? b : 0.;
        }
    }
}

// x += alpha p, r -= alpha q, partial (r.r)
__global__ void __launch_bounds__(256) kr_update(const LvlDev* __restrict__ Ls, const KrylovDev* __restrict__ K, const Chunk* __restrict__ ch, int nch,
                                                 const Scal* sc, double* partial) {
    __shared__ double sh[32];
    for (int c = blockIdx.x; c < nch; c += gridDim.x) {
        const Chunk C = ch[c];
        const LvlDev& L = Ls[C.lvl];
        const int pb = L.problem;
        const bool act = sc[pb].active;
        const KrylovDev& Kp = K[pb];
        double s = 0.;
        if (act) {
            const double al = sc[pb].alpha;
            for (int t = threadIdx.x; t < C.cnt; t += blockDim.x) {
                const long long cell = cell_of(L, C.i0 + t, C.j, C.k);
                Kp.x[cell] = fma(al, Kp.p[cell], Kp.x[cell]);
                const double r = fma(-al, Kp.q[cell], Kp.r[cell]);
                Kp.r[cell] = r;
                s = fma(r, r, s);
            }
        }
        const double a = block_sum(s, sh);
        if (threadIdx.x == 0) { partial[2 * c] = act ? a : 0.; partial[2 * c + 1] = 0.; }
    }
}

// level-0 V-cycle input from r (float64 -> T) and zero initial guess
template <typename T>
__global__ void __launch_bounds__(256) kr_to_vcycle(const LvlDev* __restrict__ Ls, const KrylovDev* __restrict__ K, const Chunk* __restrict__ ch, int nch,
                                                    const Scal* sc) {
    for (int c = blockIdx.x; c < nch; c += gridDim.x) {
        const Chunk C = ch[c];
        const LvlDev& L = Ls[C.lvl];
        if (sc && !sc[L.problem].active) continue;
        const KrylovDev& Kp = K[L.problem];
        T* b = Sel<T>::b(L);
        T* x = Sel<T>::x(L);
        for (int t = threadIdx.x; t < C.cnt; t += blockDim.x) {
            const long long cell = cell_of(L, C.i0 + t, C.j, C.k);
            b[cell] = (T) Kp.r[cell];
            x[cell] = 0;
        }
    }
}

// z = V-cycle result; partial (z.r, z.q)
template <typename T>
__global__ void __launch_bounds__(256) kr_from_vcycle(const LvlDev* __restrict__ Ls, const KrylovDev* __restrict__ K, const Chunk* __restrict__ ch,
                                                      int nch, const Scal* sc, double* partial) {
    __shared__ double sh[32];
    for (int c = blockIdx.x; c < nch; c += gridDim.x) {
        const Chunk C = ch[c];
        const LvlDev& L = Ls[C.lvl];
        const bool act = !sc || sc[L.problem].active;
        const KrylovDev& Kp = K[L.problem];
        const T* x = Sel<T>::x(L);
        double s0 = 0., s1 = 0.;
        if (act) {
            for (int t = threadIdx.x; t < C.cnt; t += blockDim.x) {
                const long long cell = cell_of(L, C.i0 + t, C.j, C.k);
                const double z = (double) x[cell];
                Kp.z[cell] = z;
                s0 = fma(z, Kp.r[cell], s0);
                s1 = fma(z, Kp.q[cell], s1);
            }
        }
        const double a = block_sum(s0, sh);
        const double b = block_sum(s1, sh);
        if (threadIdx.x == 0) { partial[2 * c] = act ? a : 0.; partial[2 * c + 1] = act ? b : 0.; }
    }
}

// p = z + beta p   (beta = 0 for the first direction)
__global__ void __launch_bounds__(256) kr_pupdate(const LvlDev* __restrict__ Ls, const KrylovDev* __restrict__ K, const Chunk* __restrict__ ch, int nch,
                                                  const Scal* sc, int first) {
    for (int c = blockIdx.x; c < nch; c += gridDim.x) {
        const Chunk C = ch[c];
        const LvlDev& L = Ls[C.lvl];
        if (!sc[L.problem].active) continue;
        const KrylovDev& Kp = K[L.problem];
        const double be = first ? 0. : sc[L.problem].beta;
        for (int t = threadIdx.x; t < C.cnt; t += blockDim.x) {
            const long long cell = cell_of(L, C.i0 + t, C.j, C.k);
            Kp.p[cell] = first ? Kp.z[cell] : fma(be, Kp.p[cell], Kp.z[cell]);
        }
    }
}

// per-problem sums of the chunk partials, in chunk order: out[2*p + s] = sum over the problem's chunks
__global__ void __launch_bounds__(256) kr_reduce(const double* __restrict__ partial, const int* __restrict__ first, const int* __restrict__ count,
                                                 int nprob, double* out) {
    __shared__ double sh[32];
    for (int p = blockIdx.x; p < nprob; p += gridDim.x) {
        for (int s = 0; s < 2; ++s) {
            double v = 0.;
            for (int c = threadIdx.x; c < count[p]; c += blockDim.x) v += partial[2 * (first[p] + c) + s];
            const double t = block_sum(v, sh);
            if (threadIdx.x == 0) out[2 * p + s] = t;
        }
    }
}

// scalar steps: stage 0 after init (bb, rr), 1 after A p (pq -> alpha), 2 after the update (rr ->
// convergence), 3 after the preconditioner (zr, zq -> beta)
__global__ void kr_scalars(Scal* sc, const double* red, int nprob, int stage, double tol, int max_iter, int flexible) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= nprob) return;
    Scal& S = sc[p];
    const double a = red[2 * p], b = red[2 * p + 1];
    if (stage == 0) {
        S.bb = a;
        S.rr = b;
        S.iters = 0;
        S.active = (b > tol * tol * a) && a > 0. ? 1 : 0;
        if (max_iter <= 0) S.active = 0;
        return;
    }
    if (!S.active) return;
    if (stage == 1) {
        S.pq = a;
        S.alpha = a != 0. ? S.rz / a : 0.;
    } else if (stage == 2) {
        S.rr = a;
        S.iters++;
        if (a <= tol * tol * S.bb || S.iters >= max_iter || !(a == a)) S.active = 0;
    } else if (stage == 3) {
        const double zr = a, zq = b;
        S.beta = flexible ? (S.rz != 0. ? -S.alpha * zq / S.rz : 0.) : (S.rz != 0. ? zr / S.rz : 0.);
        S.rz = zr;
    } else if (stage == 4) {  // first preconditioned residual
        S.rz = a;
    }
}

__global__ void count_active(const Scal* sc, int nprob, int* out) {
    int c = 0;
    for (int p = threadIdx.x; p < nprob; p += blockDim.x) c += sc[p].active;
    for (int s = 16; s > 0; s >>= 1) c += __shfl_xor_sync(0xffffffffu, c, s);
    __shared__ int sh[32];
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        int t = 0;
        for (int w = 0; w < (int) (blockDim.x >> 5); ++w) t += sh[w];
        *out = t;
    }
}

// ------------------------------------------------------------------------------------ launchers
static int grid_of(int nch, int sms) { return std::max(1, std::min(nch, sms * 8)); }

int mg_launch_residual(cudaStream_t s, int sms, bool f32, const LvlDev* L, const Chunk* ch, int nch, const Scal* sc) {
    if (nch <= 0) return OPFLOW_OK;
    if (f32) mg_residual<float><<<grid_of(nch, sms), 256, 0, s>>>(L, ch, nch, sc);
    else mg_residual<double><<<grid_of(nch, sms), 256, 0, s>>>(L, ch, nch, sc);
    OPG_LAUNCHED();
    return check_launch("mg_residual");
}
int mg_launch_smooth(cudaStream_t s, int sms, bool f32, const LvlDev* L, const Chunk* ch, int nch, int color, const Scal* sc) {
    if (nch <= 0) return OPFLOW_OK;
    if (f32) mg_smooth<float><<<grid_of(nch, sms), 256, 0, s>>>(L, ch, nch, color, sc);
    else mg_smooth<double><<<grid_of(nch, sms), 256, 0, s>>>(L, ch, nch, color, sc);
    OPG_LAUNCHED();
    return check_launch("mg_smooth");
}
int mg_launch_restrict(cudaStream_t s, int sms, bool f32, const LvlDev* L, const Chunk* ch, int nch, const Scal* sc) {
    if (nch <= 0) return OPFLOW_OK;
    if (f32) mg_restrict<float><<<grid_of(nch, sms), 256, 0, s>>>(L, ch, nch, sc);
    else mg_restrict<double><<<grid_of(nch, sms), 256, 0, s>>>(L, ch, nch, sc);
    OPG_LAUNCHED();
    return check_launch("mg_restrict");
}
int mg_launch_prolong(cudaStream_t s, int sms, bool f32, const LvlDev* L, const Chunk* ch, int nch, const Scal* sc) {
    if (nch <= 0) return OPFLOW_OK;
    if (f32) mg_prolong<float><<<grid_of(nch, sms), 256, 0, s>>>(L, ch, nch, sc);
    else mg_prolong<double><<<grid_of(nch, sms), 256, 0, s>>>(L, ch, nch, sc);
    OPG_LAUNCHED();
    return check_launch("mg_prolong");
}
int mg_launch_coarse(cudaStream_t s, int sms, bool f32, const LvlDev* L, const int* lv, int nlv, const Scal* sc) {
    if (nlv <= 0) return OPFLOW_OK;
    if (f32) mg_coarse<float><<<std::min(nlv, sms * 4), 256, 0, s>>>(L, lv, nlv, sc);
    else mg_coarse<double><<<std::min(nlv, sms * 4), 256, 0, s>>>(L, lv, nlv, sc);
    OPG_LAUNCHED();
    return check_launch("mg_coarse");
}
int mg_launch_bottom(cudaStream_t s, int sms, bool f32, const LvlDev* L, const int* top, int ntop, const Scal* sc, int pre, int post) {
    if (ntop <= 0) return OPFLOW_OK;
    const int g = std::min(ntop, sms * 4);
    if (f32) mg_bottom<float><<<g, 512, 0, s>>>(L, top, ntop, sc, pre, post);
    else mg_bottom<double><<<g, 512, 0, s>>>(L, top, ntop, sc, pre, post);
    OPG_LAUNCHED();
    return check_launch("mg_bottom");
}
int kr_launch_apply(cudaStream_t s, int sms, const LvlDev* L, const KrylovDev* K, const Chunk* ch, int nch, const Scal* sc, double* partial, int mode) {
    if (nch <= 0) return OPFLOW_OK;
    kr_apply<<<grid_of(nch, sms), 256, 0, s>>>(L, K, ch, nch, sc, partial, mode);
    OPG_LAUNCHED();
    return check_launch("kr_apply");
}
int kr_launch_update(cudaStream_t s, int sms, const LvlDev* L, const KrylovDev* K, const Chunk* ch, int nch, const Scal* sc, double* partial) {
    if (nch <= 0) return OPFLOW_OK;
    kr_update<<<grid_of(nch, sms), 256, 0, s>>>(L, K, ch, nch, sc, partial);
    OPG_LAUNCHED();
    return check_launch("kr_update");
}
int kr_launch_to_vcycle(cudaStream_t s, int sms, bool f32, const LvlDev* L, const KrylovDev* K, const Chunk* ch, int nch, const Scal* sc) {
    if (nch <= 0) return OPFLOW_OK;
    if (f32) kr_to_vcycle<float><<<grid_of(nch, sms), 256, 0, s>>>(L, K, ch, nch, sc);
    else kr_to_vcycle<double><<<grid_of(nch, sms), 256, 0, s>>>(L, K, ch, nch, sc);
    OPG_LAUNCHED();
    return check_launch("kr_to_vcycle");
}
int kr_launch_from_vcycle(cudaStream_t s, int sms, bool f32, const LvlDev* L, const KrylovDev* K, const Chunk* ch, int nch, const Scal* sc,
                          double* partial) {
    if (nch <= 0) return OPFLOW_OK;
    if (f32) kr_from_vcycle<float><<<grid_of(nch, sms), 256, 0, s>>>(L, K, ch, nch, sc, partial);
    else kr_from_vcycle<double><<<grid_of(nch, sms), 256, 0, s>>>(L, K, ch, nch, sc, partial);
    OPG_LAUNCHED();
    return check_launch("kr_from_vcycle");
}
int kr_launch_pupdate(cudaStream_t s, int sms, const LvlDev* L, const KrylovDev* K, const Chunk* ch, int nch, const Scal* sc, int first) {
    if (nch <= 0) return OPFLOW_OK;
    kr_pupdate<<<grid_of(nch, sms), 256, 0, s>>>(L, K, ch, nch, sc, first);
    OPG_LAUNCHED();
    return check_launch("kr_pupdate");
}
int kr_launch_reduce(cudaStream_t s, int sms, const double* partial, const int* first, const int* count, int nprob, double* out) {
    kr_reduce<<<std::min(nprob, sms * 8), 256, 0, s>>>(partial, first, count, nprob, out);
    OPG_LAUNCHED();
    return check_launch("kr_reduce");
}
int kr_launch_scalars(cudaStream_t s, Scal* sc, const double* red, int nprob, int stage, double tol, int max_iter, int flexible) {
    kr_scalars<<<(nprob + 127) / 128, 128, 0, s>>>(sc, red, nprob, stage, tol, max_iter, flexible);
    OPG_LAUNCHED();
    return check_launch("kr_scalars");
}
int kr_launch_count(cudaStream_t s, const Scal* sc, int nprob, int* out) {
    count_active<<<1, 256, 0, s>>>(sc, nprob, out);
    OPG_LAUNCHED();
    return check_launch("count_active");
}

}  // namespace opg
