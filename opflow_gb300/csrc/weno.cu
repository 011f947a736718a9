// Fused Shu-Osher RK3 step of periodic WENO5-JS advection along one dimension:
//   u1 = u - dt*d1<WENO53>(u);  u2 = 0.75*u + 0.25*(u1 - dt*d1<WENO53>(u1));
//   u  = 1/3*u + 2/3*(u2 - dt*d1<WENO53>(u2))
// exactly as three reference assignments compute it (D1WENO53Downwind::kernel,
// D1WENO53Downwind.hpp:136-154; D1WENO53Upwind.hpp:133-151), with every stage of a line kept in shared
// memory: one HBM read and one write of u per point per RK3 step (plus the optional stage fields).
//
// The periodic padding the reference refreshes between stages is the same line wrapped around, so
// the stages read u[(i + o) mod n].  Divisions by the constants 3 and 6 use Markstein's correctly
// rounded division by a constant (checked against IEEE division on the device before use); division
// by a power-of-two h is an exact multiplication; everything else is the reference's operation.
//
// The kernel is float64-issue-bound: this GPU retires about two float64 instructions per clock per SM,
// 1/64 of its float32 rate, so every float64 operation saved is time saved and integer work is nearly
// free.  EXACT mode shares the terms that neighbouring points have in common (below) and keeps the
// reference's six IEEE divisions per point.  FAST mode (not bit-identical) contracts the arithmetic and
// forms the three nonlinear weights with one reciprocal.
#include "internal.h"

#include <cmath>

namespace opg {

struct WenoParams {
    int n;            // line length (cells)
    int dim;          // direction
    int up;           // 1: D1WENO53Upwind (mirrored stencil, negated)
    double dt, h, inv_h;
    int h_pow2;
    int mk3, mk6;     // Markstein usable for /3 and /6
    double r3, r6;    // RN(1/3), RN(1/6)
    double c1312, third, two_third;
    // FAST mode only: RN(5/6), RN(7/6), RN(11/6); differences are taken in units of dt/h (fdx) and the
    // smoothness indicators multiplied by 4, which leaves the weights unchanged and makes the stage
    // derivative come out as dt * L directly
    double c5_6, c7_6, c11_6, fdx, c1312x4, eps_floor4;
};

__device__ __forceinline__ double divc(double x, double c, double y, int mk) {
    if (!mk) return __ddiv_rn(x, c);
    const double q = __dmul_rn(x, y);
    const double r = __fma_rn(-q, c, x);
    return __fma_rn(r, y, q);
}

// ---- per-point arithmetic, with the terms that neighbouring points share computed once ----------------
// A thread evaluates K consecutive points of a line.  For Downwind the point i reads the six values
// g[p..p+5] = u[i-3..i+2] (p = i - i0); for Upwind the mirrored values u[i+3..i-2] (the line read
// backwards, p = i0 + K - 1 - i), negated at the end.  Point p's differences d1..d5 are D[p..p+4] with
// D[k] = (g[k+1] - g[k]) / h, so point p + 1 reuses four of them, and with them every term the
// reference forms from one difference alone: d/3, d/6, 5d/6, 7d/6, 11d/6, 2d, 3d, 4d, d*d, and the
// smoothness sub-term (13/12) * ((d_k - 2 d_{k+1}) + d_{k+2})^2 that s1, s2 and s3 of three consecutive
// points share.  Each shared term is the same IEEE operation on the same operands as in the reference's
// kernel (D1WENO53Downwind.hpp:136-154), so EXACT results stay bit-identical; divc(-d, 6) = -divc(d, 6)
// exactly, since every step of divc is odd in its argument.  The largest of d1^2..d5^2 is taken on the
// bit patterns (non-negative doubles order like their bits), which equals the reference's comparisons
// for non-NaN values.
struct DiffTerms {
    double D, D3, D6, D56, D76, D116, M2, M3, M4;
    long long SQ;  // bits of D * D
    double A;      // FAST: D / 3
};

__device__ __forceinline__ double dh_of(double a, const WenoParams& P) { return P.h_pow2 ? __dmul_rn(a, P.inv_h) : __ddiv_rn(a, P.h); }

template <bool FAST>
__device__ __forceinline__ DiffTerms diff_terms(double lo, double hi, const WenoParams& P) {
    DiffTerms t;
    t.D = FAST ? __dmul_rn(__dsub_rn(hi, lo), P.fdx) : dh_of(__dsub_rn(hi, lo), P);
    t.SQ = __double_as_longlong(__dmul_rn(t.D, t.D));
    if constexpr (FAST) t.A = __dmul_rn(P.r3, t.D);
    if constexpr (!FAST) {
        t.D3 = divc(t.D, 3., P.r3, P.mk3);
        t.D6 = divc(t.D, 6., P.r6, P.mk6);
        t.D56 = divc(__dmul_rn(5., t.D), 6., P.r6, P.mk6);
        t.D76 = divc(__dmul_rn(7., t.D), 6., P.r6, P.mk6);
        t.D116 = divc(__dmul_rn(11., t.D), 6., P.r6, P.mk6);
        t.M2 = __dmul_rn(2., t.D);
        t.M3 = __dmul_rn(3., t.D);
        t.M4 = __dmul_rn(4., t.D);
    }
    return t;
}

// (13/12) * t1^2 with t1 = (d_k - 2 d_{k+1}) + d_{k+2} (FAST: 4 times that)
template <bool FAST>
__device__ __forceinline__ double smooth_p1(const DiffTerms& a, const DiffTerms& b, const DiffTerms& c, const WenoParams& P) {
    if constexpr (FAST) {
        const double t1 = __dadd_rn(__fma_rn(-2., b.D, a.D), c.D);
        return __dmul_rn(__dmul_rn(P.c1312x4, t1), t1);
    } else {
        const double t1 = __dadd_rn(__dsub_rn(a.D, b.M2), c.D);
        return __dmul_rn(P.c1312, __dmul_rn(t1, t1));
    }
}

__device__ __forceinline__ long long max_bits(long long a, long long b) { return a < b ? b : a; }

// 1/x for x in the normal range: the hardware's approximate reciprocal refined by the cubic Newton step
// y = r + r*(e + e^2), e = 1 - x*r (Newton-Raphson iteration for 1/x with the second-order term; the
// relative error goes from eps to about eps^3).
__device__ __forceinline__ double recip_fast(double x) {
    double r;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(x));
    const double e = __fma_rn(-x, r, 1.0);
    return __fma_rn(__fma_rn(e, e, e), r, r);
}

// the WENO5-JS derivative at point p from the five difference windows X0..X4 (= D[p..p+4]) and the three
// smoothness sub-terms of windows p, p+1, p+2 (FAST: dt times the derivative)
template <bool FAST>
__device__ __forceinline__ double weno_point(const DiffTerms& X0, const DiffTerms& X1, const DiffTerms& X2, const DiffTerms& X3,
                                             const DiffTerms& X4, double p0, double p1, double p2, const WenoParams& P) {
    long long mb = max_bits(max_bits(max_bits(X0.SQ, X1.SQ), max_bits(X2.SQ, X3.SQ)), X4.SQ);
    const double mx = __longlong_as_double(mb);
    if constexpr (!FAST) {
        const double ddx1 = __dadd_rn(__dsub_rn(X0.D3, X1.D76), X2.D116);
        const double ddx2 = __dadd_rn(__dadd_rn(-X1.D6, X2.D56), X3.D3);
        const double ddx3 = __dsub_rn(__dadd_rn(X2.D3, X3.D56), X4.D6);
        double t2 = __dadd_rn(__dsub_rn(X0.D, X1.M4), X2.M3);
        const double s1 = __dadd_rn(p0, __dmul_rn(__dmul_rn(t2, t2), 0.25));
        t2 = __dsub_rn(X1.D, X3.D);
        const double s2 = __dadd_rn(p1, __dmul_rn(__dmul_rn(t2, t2), 0.25));
        t2 = __dadd_rn(__dsub_rn(X2.M3, X3.M4), X4.D);
        const double s3 = __dadd_rn(p2, __dmul_rn(__dmul_rn(t2, t2), 0.25));
        const double eps = __dadd_rn(__dmul_rn(1e-6, mx), 1e-99);
        double q;
        q = __dadd_rn(s1, eps); const double a1 = __ddiv_rn(.1, __dmul_rn(q, q));
        q = __dadd_rn(s2, eps); const double a2 = __ddiv_rn(.6, __dmul_rn(q, q));
        q = __dadd_rn(s3, eps); const double a3 = __ddiv_rn(.3, __dmul_rn(q, q));
        const double sum = __dadd_rn(__dadd_rn(a1, a2), a3);
        const double w1 = __ddiv_rn(a1, sum), w2 = __ddiv_rn(a2, sum), w3 = __ddiv_rn(a3, sum);
        return __dadd_rn(__dadd_rn(__dmul_rn(w1, ddx1), __dmul_rn(w2, ddx2)), __dmul_rn(w3, ddx3));
    } else {
        // The same quantities with contracted arithmetic, in the scaled units above, and one reciprocal:
        //   w_k = c_k / q_k^2 / sum_j c_j / q_j^2 = c_k prod_{j != k} q_j^2 / sum_j c_j prod_{i != j} q_i^2,
        // with the q's first scaled by a power of two that brings the largest into [1, 2).  The q's lie
        // within a factor 3.4e7 of each other (eps >= 1e-6 max d^2 and s_k <= 33.4 max d^2), so the
        // products neither overflow nor underflow.
        const double ddx1 = __fma_rn(P.c11_6, X2.D, __fma_rn(-P.c7_6, X1.D, X0.A));
        const double ddx2 = __fma_rn(P.r3, X3.D, __fma_rn(P.c5_6, X2.D, __dmul_rn(-P.r6, X1.D)));
        const double ddx3 = __fma_rn(-P.r6, X4.D, __fma_rn(P.c5_6, X3.D, X2.A));
        double t2 = __fma_rn(3., X2.D, __fma_rn(-4., X1.D, X0.D));
        const double s1 = __fma_rn(t2, t2, p0);
        t2 = __dsub_rn(X1.D, X3.D);
        const double s2 = __fma_rn(t2, t2, p1);
        t2 = __fma_rn(3., X2.D, __fma_rn(-4., X3.D, X4.D));
        const double s3 = __fma_rn(t2, t2, p2);
        const double eps = __fma_rn(4e-6, mx, P.eps_floor4);
        double q1 = __dadd_rn(s1, eps), q2 = __dadd_rn(s2, eps), q3 = __dadd_rn(s3, eps);
        const long long qb = max_bits(max_bits(__double_as_longlong(q1), __double_as_longlong(q2)), __double_as_longlong(q3));
        const int e = (int) (qb >> 52);
        if (e <= 0 || e >= 2046) {
            // q out of the scaled form's range (an overflowed or NaN smoothness indicator): the
            // reference's weights
            const double a1 = __ddiv_rn(.1, __dmul_rn(q1, q1)), a2 = __ddiv_rn(.6, __dmul_rn(q2, q2)), a3 = __ddiv_rn(.3, __dmul_rn(q3, q3));
            const double sum = __dadd_rn(__dadd_rn(a1, a2), a3);
            return __dadd_rn(__dadd_rn(__dmul_rn(__ddiv_rn(a1, sum), ddx1), __dmul_rn(__ddiv_rn(a2, sum), ddx2)),
                             __dmul_rn(__ddiv_rn(a3, sum), ddx3));
        }
        const double sc = __longlong_as_double((long long) (2046 - e) << 52);  // 2^(1023 - e): exact scaling
        q1 = __dmul_rn(q1, sc);
        q2 = __dmul_rn(q2, sc);
        q3 = __dmul_rn(q3, sc);
        const double Q1 = __dmul_rn(q1, q1), Q2 = __dmul_rn(q2, q2), Q3 = __dmul_rn(q3, q3);
        const double n1 = __dmul_rn(.1, __dmul_rn(Q2, Q3)), n2 = __dmul_rn(.6, __dmul_rn(Q1, Q3)), n3 = __dmul_rn(.3, __dmul_rn(Q1, Q2));
        const double den = __dadd_rn(__dadd_rn(n1, n2), n3);
        const double num = __fma_rn(n3, ddx3, __fma_rn(n2, ddx2, __dmul_rn(n1, ddx1)));
        return __dmul_rn(num, recip_fast(den));
    }
}

__device__ __forceinline__ int wrap_index(int j, int n) {
    j += j < 0 ? n : 0;
    j -= j >= n ? n : 0;
    j -= j >= n ? n : 0;
    return j;
}

// One stage over a line held in shared memory: out[i] = combine(i, src-derivative at i).
//   STAGE 0: s1 = u - dt*L(u)                         (src = u)
//   STAGE 1: s2 = 0.75*u + 0.25*(s1 - dt*L(s1))       (src = s1)
//   STAGE 2: u' = 1/3*u + 2/3*(s2 - dt*L(s2))         (src = s2)
// Chunks of K consecutive points per thread; requires n >= K and n >= 6.
template <int K, bool UP, bool FAST, int STAGE>
__device__ __forceinline__ void weno_stage(const double* __restrict__ u, const double* __restrict__ src, double* __restrict__ out, int n,
                                           const WenoParams& P) {
    const int nchunks = (n + K - 1) / K;
    for (int c = threadIdx.x; c < nchunks; c += blockDim.x) {
        int i0 = c * K;
        // a partial last chunk is shifted back so that it ends at the line's end (points computed twice
        // give the same values and are stored by both threads)
        if (i0 + K > n) i0 = n - K;
        double g[K + 5];
#pragma unroll
        for (int t = 0; t < K + 5; ++t) g[t] = src[wrap_index(UP ? i0 + K + 2 - t : i0 - 3 + t, n)];
        DiffTerms X[5];
#pragma unroll
        for (int k = 0; k < 4; ++k) X[k] = diff_terms<FAST>(g[k], g[k + 1], P);
        double p0 = smooth_p1<FAST>(X[0], X[1], X[2], P), p1 = smooth_p1<FAST>(X[1], X[2], X[3], P);
#pragma unroll
        for (int p = 0; p < K; ++p) {
            X[4] = diff_terms<FAST>(g[p + 4], g[p + 5], P);
            const double p2 = smooth_p1<FAST>(X[2], X[3], X[4], P);
            double r = weno_point<FAST>(X[0], X[1], X[2], X[3], X[4], p0, p1, p2, P);
            if (UP) r = -r;
            const int i = UP ? i0 + K - 1 - p : i0 + p;
            const double L = FAST ? r : __dmul_rn(P.dt, r);
            double v;
            if constexpr (STAGE == 0) v = __dsub_rn(u[i], L);
            else if constexpr (STAGE == 1) v = __dadd_rn(__dmul_rn(0.75, u[i]), __dmul_rn(0.25, __dsub_rn(src[i], L)));
            else v = __dadd_rn(__dmul_rn(P.third, u[i]), __dmul_rn(P.two_third, __dsub_rn(src[i], L)));
            out[i] = v;
            X[0] = X[1];
            X[1] = X[2];
            X[2] = X[3];
            X[3] = X[4];
            p0 = p1;
            p1 = p2;
        }
    }
}

// One CTA per line: the line and its two stage fields in shared memory, `steps` RK3 steps, one HBM read
// and one write of u per point (plus the last step's stage fields when asked for).  u/u1/u2 views
// address the line's first cell, `stride` between its cells.
constexpr int kWenoThreads = 256;

// A line between global and shared memory.  A contiguous line (x lines) moves in 16-byte pairs from its
// first 16-byte aligned cell, with a lone cell at either end taken by thread 0; other lines cell by
// cell.  Plain copies: the values are the same whichever way they move.
__device__ __forceinline__ void line_load(double* __restrict__ dst, const double* __restrict__ src, int n, long long stride) {
    if (stride == 1) {
        const int head = (reinterpret_cast<unsigned long long>(src) & 15ull) != 0 ? 1 : 0;  // (cells are 8-byte aligned)
        const int np = (n - head) / 2;
        const double2* __restrict__ s2 = reinterpret_cast<const double2*>(src + head);
        for (int t = threadIdx.x; t < np; t += blockDim.x) {
            const double2 v = s2[t];
            dst[head + 2 * t] = v.x;
            dst[head + 2 * t + 1] = v.y;
        }
        if (threadIdx.x == 0) {
            if (head) dst[0] = src[0];
            if (head + 2 * np < n) dst[n - 1] = src[n - 1];
        }
    } else {
        for (int i = threadIdx.x; i < n; i += blockDim.x) dst[i] = src[i * stride];
    }
}
__device__ __forceinline__ void line_store(double* __restrict__ dst, const double* __restrict__ src, int n, long long stride) {
    if (stride == 1) {
        const int head = (reinterpret_cast<unsigned long long>(dst) & 15ull) != 0 ? 1 : 0;
        const int np = (n - head) / 2;
        double2* __restrict__ d2 = reinterpret_cast<double2*>(dst + head);
        for (int t = threadIdx.x; t < np; t += blockDim.x) d2[t] = make_double2(src[head + 2 * t], src[head + 2 * t + 1]);
        if (threadIdx.x == 0) {
            if (head) dst[0] = src[0];
            if (head + 2 * np < n) dst[n - 1] = src[n - 1];
        }
    } else {
        for (int i = threadIdx.x; i < n; i += blockDim.x) dst[i * stride] = src[i];
    }
}

template <int K, bool UP, bool FAST, int MINB>
__global__ void __launch_bounds__(kWenoThreads, MINB) weno_rk3_kernel(FieldView u, FieldView u1, FieldView u2, int write_stages, Box lines, WenoParams P,
                                                          int steps) {
    extern __shared__ double sm[];
    const int n = P.n;
    double* s0 = sm;
    double* s1 = sm + n;
    double* s2 = sm + 2 * n;
    const long long nlines = lines.count();
    for (long long ln = blockIdx.x; ln < nlines; ln += gridDim.x) {
        int a, b, c;
        box_index(ln, lines, a, b, c);  // line start: (a, b, c) with the `dim` coordinate at 0
        int idx0[3] = {a, b, c};
        const long long stride = P.dim == 0 ? 1 : (P.dim == 1 ? u.sy : u.sz);
        const long long base = (idx0[0] - u.off[0]) + (idx0[1] - u.off[1]) * u.sy + (idx0[2] - u.off[2]) * u.sz;
        line_load(s0, u.data + base, n, stride);
        __syncthreads();
        for (int st = 0; st < steps; ++st) {
            weno_stage<K, UP, FAST, 0>(s0, s0, s1, n, P);
            __syncthreads();
            weno_stage<K, UP, FAST, 1>(s0, s1, s2, n, P);
            __syncthreads();
            if (write_stages && st == steps - 1) {
                line_store(u1.data + base, s1, n, stride);
                __syncthreads();
            }
            // the third stage reads u and s2 only: its result replaces s1, which then becomes u
            weno_stage<K, UP, FAST, 2>(s0, s2, s1, n, P);
            __syncthreads();
            double* t = s0;
            s0 = s1;
            s1 = t;
        }
        line_store(u.data + base, s0, n, stride);
        if (write_stages) line_store(u2.data + base, s2, n, stride);
        __syncthreads();
        // the next line starts from the shared buffers' original order
        if (steps & 1) {
            double* t = s0;
            s0 = s1;
            s1 = t;
        }
    }
}

extern int markstein_ok_public(opflow_ctx ctx, double h, bool* ok);

}  // namespace opg

using namespace opg;

template <int K, bool UP, bool FAST, int MINB>
static int launch_weno(opflow_ctx ctx, int blocks, size_t smem, FieldView u, FieldView v1, FieldView v2, int stages, const Box& lines,
                       const WenoParams& P, int steps) {
    static bool attr_set = false;  // per instantiation
    if (!attr_set) {
        OPG_CUDA(cudaFuncSetAttribute(weno_rk3_kernel<K, UP, FAST, MINB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      3 * 8192 * (int) sizeof(double)));
        attr_set = true;
    }
    weno_rk3_kernel<K, UP, FAST, MINB><<<blocks, kWenoThreads, smem, ctx->stream>>>(u, v1, v2, stages, lines, P, steps);
    OPG_LAUNCHED();
    return check_launch("weno_rk3_kernel");
}

template <int K, int MINB>
static int launch_weno_k(opflow_ctx ctx, bool up, bool fast, int blocks, size_t smem, FieldView u, FieldView v1, FieldView v2, int stages,
                         const Box& lines, const WenoParams& P, int steps) {
    if (up) return fast ? launch_weno<K, true, true, MINB>(ctx, blocks, smem, u, v1, v2, stages, lines, P, steps)
                        : launch_weno<K, true, false, MINB>(ctx, blocks, smem, u, v1, v2, stages, lines, P, steps);
    return fast ? launch_weno<K, false, true, MINB>(ctx, blocks, smem, u, v1, v2, stages, lines, P, steps)
                : launch_weno<K, false, false, MINB>(ctx, blocks, smem, u, v1, v2, stages, lines, P, steps);
}

extern "C" int opflow_weno_rk3(opflow_ctx ctx, opflow_field u, opflow_field u1, opflow_field u2, int kind, int dim, double dt, int steps) {
    return opflow_weno_rk3_mode(ctx, u, u1, u2, kind, dim, dt, steps, OPFLOW_EVAL_EXACT);
}

extern "C" int opflow_weno_rk3_mode(opflow_ctx ctx, opflow_field u, opflow_field u1, opflow_field u2, int kind, int dim, double dt, int steps,
                                    int mode) {
    if (!ctx || !u) return fail(OPFLOW_E_INVALID, "null argument");
    if (kind != OPFLOW_NODE_WENO53_DOWN && kind != OPFLOW_NODE_WENO53_UP) return fail(OPFLOW_E_INVALID, "kind must be a WENO53 node kind");
    if (mode != OPFLOW_EVAL_EXACT && mode != OPFLOW_EVAL_FAST) return fail(OPFLOW_E_INVALID, "bad evaluation mode");
    if (dim < 0 || dim >= u->info.ndim) return fail(OPFLOW_E_INVALID, "bad dim");
    if (steps < 0) return fail(OPFLOW_E_INVALID, "negative steps");
    if (u->desc.bc_type[dim][0] != OPFLOW_BC_PERIODIC) return fail(OPFLOW_E_UNSUPPORTED, "the fused WENO-RK3 step needs a periodic direction");
    if (!u->mesh->uniform[dim]) return fail(OPFLOW_E_UNSUPPORTED, "the fused WENO-RK3 step needs a uniform mesh along its direction");
    const bool stages = u1 && u2;
    if (stages && (u1->info.count != u->info.count || u2->info.count != u->info.count)) return fail(OPFLOW_E_INVALID, "stage fields differ in shape");
    const opflow_field_info& R = u->info;
    const int n = R.accessible[dim][1] - R.accessible[dim][0];
    if (n < 6) return fail(OPFLOW_E_UNSUPPORTED, "WENO5 needs at least 6 cells along its direction");
    if (n > 8192) return fail(OPFLOW_E_UNSUPPORTED, "lines longer than 8192 cells do not fit the shared-memory stages");
    if (steps == 0) return OPFLOW_OK;
    WenoParams P{};
    P.n = n;
    P.dim = dim;
    P.up = kind == OPFLOW_NODE_WENO53_UP;
    P.dt = dt;
    P.h = u->mesh->h[dim];
    P.inv_h = 1.0 / P.h;
    {
        int e;
        P.h_pow2 = std::frexp(P.h, &e) == 0.5;
    }
    bool ok3 = false, ok6 = false;
    OPG_TRY(markstein_ok_public(ctx, 3.0, &ok3));
    OPG_TRY(markstein_ok_public(ctx, 6.0, &ok6));
    P.mk3 = ok3;
    P.mk6 = ok6;
    P.r3 = 1.0 / 3.0;
    P.r6 = 1.0 / 6.0;
    P.c1312 = 13. / 12.;
    P.third = 1.0 / 3.0;
    P.two_third = 2.0 / 3.0;
    P.c5_6 = 5.0 / 6.0;
    P.c7_6 = 7.0 / 6.0;
    P.c11_6 = 11.0 / 6.0;
    P.fdx = dt / P.h;
    P.c1312x4 = 13.0 / 3.0;
    P.eps_floor4 = 4e-99 * P.fdx * P.fdx;
    // the scaled form needs the scaled eps floor to be a normal number (dt = 0 or |dt/h| outside about
    // 1e-104..1e150 take the EXACT evaluation)
    if (!(std::fabs(P.eps_floor4) >= 2.2250738585072014e-308 && std::isfinite(P.eps_floor4 * 1e50))) mode = OPFLOW_EVAL_EXACT;
    // lines: the assignable box with the `dim` extent collapsed to its first cell
    Box lines = assign_box(R);
    lines.hi[dim] = lines.lo[dim] + 1;
    const size_t smem = 3 * (size_t) n * sizeof(double);
    const long long nl = lines.count();
    const int blocks = (int) std::min<long long>(nl, (long long) ctx->num_sms * 2);
    FieldView v1 = stages ? u1->view() : u->view(), v2 = stages ? u2->view() : u->view();
    const bool up = P.up, fast = mode == OPFLOW_EVAL_FAST;
    // 16 points per thread (4 on lines shorter than 16 cells); measured at 4096-cell lines, 8 or 16
    // points and one or two CTAs per SM are within 2% of each other
    if (n < 16) OPG_TRY((launch_weno_k<4, 2>(ctx, up, fast, blocks, smem, u->view(), v1, v2, stages ? 1 : 0, lines, P, steps)));
    else OPG_TRY((launch_weno_k<16, 2>(ctx, up, fast, blocks, smem, u->view(), v1, v2, stages ? 1 : 0, lines, P, steps)));
    u->version++;
    OPG_TRY(update_padding_assign(u));
    if (stages) {
        u1->bc_fresh[0] = u1->bc_fresh[1] = false;
        u2->bc_fresh[0] = u2->bc_fresh[1] = false;
        u1->version++;
        u2->version++;
        OPG_TRY(update_padding_assign(u1));
        OPG_TRY(update_padding_assign(u2));
    }
    OPG_CUDA(cudaStreamSynchronize(ctx->stream));
    return OPFLOW_OK;
}
