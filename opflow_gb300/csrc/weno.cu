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
#include "internal.h"

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
};

__device__ __forceinline__ double divc(double x, double c, double y, int mk) {
    if (!mk) return __ddiv_rn(x, c);
    const double q = __dmul_rn(x, y);
    const double r = __fma_rn(-q, c, x);
    return __fma_rn(r, y, q);
}

// the WENO5-JS derivative from six line values (pm3..pp2 for Downwind; the mirrored sequence, negated
// at the end, for Upwind)
__device__ __forceinline__ double weno_val(const double* v, const WenoParams& P) {
    const double h = P.h;
    auto dh = [&](double a) { return P.h_pow2 ? __dmul_rn(a, P.inv_h) : __ddiv_rn(a, h); };
    const double d1 = dh(__dsub_rn(v[1], v[0])), d2 = dh(__dsub_rn(v[2], v[1])), d3 = dh(__dsub_rn(v[3], v[2])),
                 d4 = dh(__dsub_rn(v[4], v[3])), d5 = dh(__dsub_rn(v[5], v[4]));
    const double ddx1 = __dadd_rn(__dsub_rn(divc(d1, 3., P.r3, P.mk3), divc(__dmul_rn(7., d2), 6., P.r6, P.mk6)),
                                  divc(__dmul_rn(11., d3), 6., P.r6, P.mk6));
    const double ddx2 = __dadd_rn(__dadd_rn(divc(-d2, 6., P.r6, P.mk6), divc(__dmul_rn(5., d3), 6., P.r6, P.mk6)), divc(d4, 3., P.r3, P.mk3));
    const double ddx3 = __dsub_rn(__dadd_rn(divc(d3, 3., P.r3, P.mk3), divc(__dmul_rn(5., d4), 6., P.r6, P.mk6)), divc(d5, 6., P.r6, P.mk6));
    double t1 = __dadd_rn(__dsub_rn(d1, __dmul_rn(2., d2)), d3);
    double t2 = __dadd_rn(__dsub_rn(d1, __dmul_rn(4., d2)), __dmul_rn(3., d3));
    const double s1 = __dadd_rn(__dmul_rn(P.c1312, __dmul_rn(t1, t1)), __dmul_rn(__dmul_rn(t2, t2), 0.25));
    t1 = __dadd_rn(__dsub_rn(d2, __dmul_rn(2., d3)), d4);
    t2 = __dsub_rn(d2, d4);
    const double s2 = __dadd_rn(__dmul_rn(P.c1312, __dmul_rn(t1, t1)), __dmul_rn(__dmul_rn(t2, t2), 0.25));
    t1 = __dadd_rn(__dsub_rn(d3, __dmul_rn(2., d4)), d5);
    t2 = __dadd_rn(__dsub_rn(__dmul_rn(3., d3), __dmul_rn(4., d4)), d5);
    const double s3 = __dadd_rn(__dmul_rn(P.c1312, __dmul_rn(t1, t1)), __dmul_rn(__dmul_rn(t2, t2), 0.25));
    double mx = __dmul_rn(d1, d1), t;
    t = __dmul_rn(d2, d2); if (mx < t) mx = t;
    t = __dmul_rn(d3, d3); if (mx < t) mx = t;
    t = __dmul_rn(d4, d4); if (mx < t) mx = t;
    t = __dmul_rn(d5, d5); if (mx < t) mx = t;
    const double eps = __dadd_rn(__dmul_rn(1e-6, mx), 1e-99);
    double q;
    q = __dadd_rn(s1, eps); const double a1 = __ddiv_rn(.1, __dmul_rn(q, q));
    q = __dadd_rn(s2, eps); const double a2 = __ddiv_rn(.6, __dmul_rn(q, q));
    q = __dadd_rn(s3, eps); const double a3 = __ddiv_rn(.3, __dmul_rn(q, q));
    const double sum = __dadd_rn(__dadd_rn(a1, a2), a3);
    const double w1 = __ddiv_rn(a1, sum), w2 = __ddiv_rn(a2, sum), w3 = __ddiv_rn(a3, sum);
    const double r = __dadd_rn(__dadd_rn(__dmul_rn(w1, ddx1), __dmul_rn(w2, ddx2)), __dmul_rn(w3, ddx3));
    return P.up ? -r : r;
}

__device__ __forceinline__ double weno_at(const double* s, int i, int n, const WenoParams& P) {
    double v[6];
#pragma unroll
    for (int o = 0; o < 6; ++o) {
        int j = P.up ? i + 3 - o : i + o - 3;
        j += j < 0 ? n : 0;
        j -= j >= n ? n : 0;
        v[o] = s[j];
    }
    return weno_val(v, P);
}

// one CTA per line; u/u1/u2 views address the line's first cell, `stride` between its cells
__global__ void __launch_bounds__(512) weno_rk3_kernel(FieldView u, FieldView u1, FieldView u2, int write_stages, Box lines, WenoParams P,
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
        for (int i = threadIdx.x; i < n; i += blockDim.x) s0[i] = u.data[base + i * stride];
        __syncthreads();
        for (int st = 0; st < steps; ++st) {
            for (int i = threadIdx.x; i < n; i += blockDim.x) s1[i] = __dsub_rn(s0[i], __dmul_rn(P.dt, weno_at(s0, i, n, P)));
            __syncthreads();
            for (int i = threadIdx.x; i < n; i += blockDim.x)
                s2[i] = __dadd_rn(__dmul_rn(0.75, s0[i]), __dmul_rn(0.25, __dsub_rn(s1[i], __dmul_rn(P.dt, weno_at(s1, i, n, P)))));
            __syncthreads();
            // the last stage overwrites s0 in place only after every thread has read its stencil
            double nv[16];
            int cnt = 0;
            for (int i = threadIdx.x; i < n; i += blockDim.x)
                nv[cnt++] = __dadd_rn(__dmul_rn(P.third, s0[i]), __dmul_rn(P.two_third, __dsub_rn(s2[i], __dmul_rn(P.dt, weno_at(s2, i, n, P)))));
            __syncthreads();
            cnt = 0;
            for (int i = threadIdx.x; i < n; i += blockDim.x) s0[i] = nv[cnt++];
            __syncthreads();
        }
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
            u.data[base + i * stride] = s0[i];
            if (write_stages) {
                u1.data[base + i * stride] = s1[i];
                u2.data[base + i * stride] = s2[i];
            }
        }
        __syncthreads();
    }
}

extern int markstein_ok_public(opflow_ctx ctx, double h, bool* ok);

}  // namespace opg

using namespace opg;

extern "C" int opflow_weno_rk3(opflow_ctx ctx, opflow_field u, opflow_field u1, opflow_field u2, int kind, int dim, double dt, int steps) {
    if (!ctx || !u) return fail(OPFLOW_E_INVALID, "null argument");
    if (kind != OPFLOW_NODE_WENO53_DOWN && kind != OPFLOW_NODE_WENO53_UP) return fail(OPFLOW_E_INVALID, "kind must be a WENO53 node kind");
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
    // lines: the assignable box with the `dim` extent collapsed to its first cell
    Box lines = assign_box(R);
    lines.hi[dim] = lines.lo[dim] + 1;
    const size_t smem = 3 * (size_t) n * sizeof(double);
    static bool attr_set = false;
    if (!attr_set) {
        cudaFuncSetAttribute(weno_rk3_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 3 * 8192 * (int) sizeof(double));
        attr_set = true;
    }
    const int threads = 512;
    if ((n + threads - 1) / threads > 16) return fail(OPFLOW_E_UNSUPPORTED, "line too long");
    long long nl = lines.count();
    int blocks = (int) std::min<long long>(nl, (long long) ctx->num_sms * 2);
    FieldView v1 = stages ? u1->view() : u->view(), v2 = stages ? u2->view() : u->view();
    weno_rk3_kernel<<<blocks, threads, smem, ctx->stream>>>(u->view(), v1, v2, stages ? 1 : 0, lines, P, steps);
    OPG_LAUNCHED();
    OPG_TRY(check_launch("weno_rk3_kernel"));
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
