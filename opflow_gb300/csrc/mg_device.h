// Device-side pieces of the multigrid V-cycle shared by the chunked kernels (mg.cu), the bottom kernel
// (mg.cu) and the tile kernels (mg_tiles.cu): operator access and the per-cell bodies of smoothing,
// residual, restriction and prolongation.
#pragma once
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
__device__ __forceinline__ void stencil_parts(const LvlDev& L, const V* __restrict__ x, int i, int j, int k, long long cell, T& c0, T& offd,
                                              int* cls_out = nullptr) {
    const int cls = pos_class(i, L.n[0]) + 3 * (L.ndim > 1 ? pos_class(j, L.n[1]) : 0) + 9 * (L.ndim > 2 ? pos_class(k, L.n[2]) : 0);
    const T* A = Sel<T>::A(L);
    const T* Tb = Sel<T>::Tb(L);
    if (cls_out) *cls_out = cls;
    auto cf = [&](int s) -> T { return L.table ? Tb[cls * TSTRIDE + s] : A[(long long) s * L.N + cell]; };
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

// Gauss-Seidel update of one cell: x = (b - offd) / c0, as a product with the tabulated inverse of c0
// on class-table levels (no division in the sweep)
template <typename T>
__device__ __forceinline__ void cell_gs(const LvlDev& L, int i, int j, int k) {
    const long long cell = cell_of(L, i, j, k);
    T* x = Sel<T>::x(L);
    T c0, offd;
    int cls;
    stencil_parts<T>(L, x, i, j, k, cell, c0, offd, &cls);
    const T num = Sel<T>::b(L)[cell] - offd;
    x[cell] = L.table ? num * Sel<T>::Tb(L)[cls * TSTRIDE + NSLOT] : num / c0;
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

// fine x += P x_coarse at fine cell f.  FAST adds a path for cell-centred fine cells whose coarse
// neighbours are all inside the box (the same terms in the same order, sign 1); the chunked
// float32 prolongation uses it, the tile and bottom kernels (tight on registers) do not.
template <typename T, bool FAST = false>
__device__ __forceinline__ T prolong_acc(const LvlDev* __restrict__ Ls, const LvlDev& Lf, int f0, int f1, int f2) {
    const LvlDev& Lc = Ls[Lf.coarse];
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
        bool inside = FAST;
        for (int d = 0; FAST && d < Lc.ndim; ++d) inside = inside && I[d] >= 0 && I[d] < Lc.n[d] && J[d] >= 0 && J[d] < Lc.n[d];
        if (FAST && inside) {
            // every coarse neighbour inside the box: the terms below with sign 1, in their order
            for (int a = 0; a < nz; ++a)
                for (int bb = 0; bb < ny; ++bb)
                    for (int e = 0; e < 2; ++e) {
                        const T w = (e ? (T) 0.25 : (T) 0.75) * (Lc.ndim > 1 ? (bb ? (T) 0.25 : (T) 0.75) : (T) 1) *
                                    (Lc.ndim > 2 ? (a ? (T) 0.25 : (T) 0.75) : (T) 1);
                        const T v = xc[cell_of(Lc, e ? J[0] : I[0], Lc.ndim > 1 ? (bb ? J[1] : I[1]) : 0, Lc.ndim > 2 ? (a ? J[2] : I[2]) : 0)];
                        acc += w * (T) 1 * v;
                    }
            return acc;
        }
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
    return acc;
}

template <typename T, bool FAST = false>
__device__ __forceinline__ void cell_prolong(const LvlDev* __restrict__ Ls, const LvlDev& Lf, int f0, int f1, int f2) {
    const T acc = prolong_acc<T, FAST>(Ls, Lf, f0, f1, f2);
    Sel<T>::x(Lf)[cell_of(Lf, f0, f1, f2)] += acc;
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

}  // namespace opg
