// Per-element device functions shared by the expression interpreter (expr.cu) and the stencil
// assembler (assemble.cu): std::max / std::min, the flux-limiter kernels K(r) and the per-element
// math functions of the reference's expression operators.
#pragma once

#include "../../include/opflow_gpu.h"

namespace opg {

// std::max(a, b) / std::min(a, b): (a < b) ? b : a and (b < a) ? b : a, NaN and signed-zero behaviour
// included; the initializer-list forms keep the first extreme element.
static __device__ __forceinline__ double std_max(double a, double b) { return a < b ? b : a; }
static __device__ __forceinline__ double std_min(double a, double b) { return b < a ? b : a; }

// Flux-limiter kernels K(r) of FluxLimiterKernels.hpp.  The SPL / GPL parameters are what the reference
// computes: `static constexpr double m = M::num / M::den` divides the std::ratio's integers, so
// kappa = 1/2 and 1/3 become 0 (and alpha = 0/1 = 0).
static __device__ __noinline__ double flux_limiter(int K, double r) {
    switch (K) {
        case OPFLOW_FL_MINMOD: return std_max(0., std_min(r, 1.));
        case OPFLOW_FL_SUPERBEE: {
            double m = 0., t = std_min(__dmul_rn(2., r), 1.);
            if (m < t) m = t;
            t = std_min(r, 2.);
            if (m < t) m = t;
            return m;
        }
        case OPFLOW_FL_MUSCL: {
            double m = __dmul_rn(2., r), t = __dmul_rn(__dadd_rn(r, 1.), 0.5);  // (r + 1) / 2. is exact as * 0.5
            if (t < m) m = t;
            if (2. < m) m = 2.;
            return std_max(0., m);
        }
        case OPFLOW_FL_HARMONIC: return __ddiv_rn(__dadd_rn(r, fabs(r)), __dadd_rn(r, 1.));
        case OPFLOW_FL_VANALBADA: return __ddiv_rn(__dmul_rn(r, __dadd_rn(r, 1.)), __dadd_rn(__dmul_rn(r, r), 1.));
        case OPFLOW_FL_UMIST: case OPFLOW_FL_SPL13: case OPFLOW_FL_SPLMAX12: case OPFLOW_FL_SPLMAX13: {
            const double m = 2., kappa = 0.;  // std::ratio<2,1>, std::ratio<1,2> or <1,3> by integer division
            const double a = 0.5 * (1 + kappa), b = 0.5 * (1 - kappa);
            const double l1 = __dadd_rn(__dmul_rn(a, r), b), l2 = __dadd_rn(__dmul_rn(b, r), a);
            double cur = __dmul_rn(m, r);
            if (K == OPFLOW_FL_UMIST || K == OPFLOW_FL_SPL13) {  // min({m r, l1, l2, m})
                if (l1 < cur) cur = l1;
                if (l2 < cur) cur = l2;
            } else {  // min({m r, max({l1, l2}), m})
                double mx = l1;
                if (mx < l2) mx = l2;
                if (mx < cur) cur = mx;
            }
            if (m < cur) cur = m;
            return 0. < cur ? cur : 0.;
        }
        default: {  // GPLKappaKernel: max({0., min({(2 + alpha) r, 0.5 (1 + kappa) r + 0.5 (1 - kappa), m})})
            const double m = K == OPFLOW_FL_SMART ? 4. : (K == OPFLOW_FL_KOREN ? 2. : 1.);
            const double kappa = K == OPFLOW_FL_BSOU ? -1. : 0., alpha = 0.;
            double cur = __dmul_rn(2 + alpha, r);
            const double t = __dadd_rn(__dmul_rn(0.5 * (1 + kappa), r), 0.5 * (1 - kappa));
            if (t < cur) cur = t;
            if (m < cur) cur = m;
            return 0. < cur ? cur : 0.;
        }
    }
}

// Per-element functions (AMDS.hpp, MinMax.hpp).  The first group of each is exact IEEE arithmetic;
// the transcendental ones are CUDA's double-precision math library.
static __device__ __noinline__ double func1_eval(int f, double x) {
    switch (f) {
        case OPFLOW_F_ABS: return fabs(x);
        case OPFLOW_F_SQRT: return __dsqrt_rn(x);
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
        default: return lgamma(x);
    }
}
static __device__ __noinline__ double func2_eval(int f, double a, double b) {
    switch (f) {
        case OPFLOW_F2_MAX: return std_max(a, b);
        case OPFLOW_F2_MIN: return std_min(a, b);
        case OPFLOW_F2_FDIM: return fdim(a, b);
        case OPFLOW_F2_COPYSIGN: return copysign(a, b);
        case OPFLOW_F2_FMOD: return fmod(a, b);
        case OPFLOW_F2_REMAINDER: return remainder(a, b);
        case OPFLOW_F2_POW: return pow(a, b);
        case OPFLOW_F2_HYPOT: return hypot(a, b);
        default: return atan2(a, b);
    }
}

}  // namespace opg
