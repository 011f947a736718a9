// Tiled stencil kernels for the axis-aligned (2*D+1)-point updates of path E.
//
// 3D: a CTA owns a 32x8 column of the xy plane and marches along z through a chunk of planes.  The
// z-1 / z / z+1 values of its own column stay in registers; the plane z (with a one-cell halo) is staged
// in shared memory, so every grid value is read from HBM once per step (8 B read + 8 B written per
// lattice update).  2D: a CTA owns 128 x-points and marches along y.
//
// Two arithmetic modes share the tiling:
//   EXACT - the reference's IEEE operations per point (D2SecondOrderCentered::eval,
//           D2SecondOrderCentered.hpp:160-171, summed in tree order, then u + s*sum);
//   FAST  - exact 64-bit fixed point: values are converted once when staged, the second differences
//           are exact integer sums, one 64x53-bit product per weight group, one rounding back.
//
// A run of FAST steps on a Dirichlet node grid can keep the field in fixed point between its steps
// (the resident kernels below): in 3D its steady-state steps stream their planes into shared memory
// by TMA (axis3d_fxtma_kernel), in 2D a warp updates 30 columns x 8 rows with every load in flight.
#include "stencil.h"
#include "tma.h"
#include "tune.h"

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

namespace opg {

__device__ __forceinline__ double ld3(const FieldView& f, int i, int j, int k) {
    return f.data[(long long) (i - f.off[0]) + (long long) (j - f.off[1]) * f.sy + (long long) (k - f.off[2]) * f.sz];
}

// x * y for y a power of two, exactly: when x and the product are normal numbers the product is x
// with its exponent field moved, an integer add (no float64 instruction); zeros are returned as they
// are; everything else (subnormal operand or product, infinities, NaN) takes the float64 multiply.
__device__ __forceinline__ double mul_pow2(double x, double y) {
    const int k = (int) ((__double_as_longlong(y) >> 52) & 0x7FF) - 1023;
    const long long b = __double_as_longlong(x);
    const int e = (int) ((b >> 52) & 0x7FF);
    if (e > 0 && e < 2047 && e + k > 0 && e + k < 2047) return __longlong_as_double(b + ((long long) k << 52));
    if ((b & 0x7FFFFFFFFFFFFFFFll) == 0) return x;
    return __dmul_rn(x, y);
}

// correctly rounded x / h: an exact multiply for a power-of-two h, else Markstein's three operations
__device__ __forceinline__ double tdiv(double x, double h, double y, int p2) {
    if (p2) return mul_pow2(x, y);
    const double q = __dmul_rn(x, y);
    const double r = __fma_rn(-q, h, x);
    return __fma_rn(r, y, q);
}

__device__ __forceinline__ double d2_exact(double l, double c, double r, double h, double y, int p2) {
    const double a = tdiv(__dsub_rn(r, c), h, y, p2);
    const double b = tdiv(__dsub_rn(c, l), h, y, p2);
    return tdiv(__dsub_rn(a, b), h, y, p2);
}

// x * 2^(58-E) rounded to an integer.  For moderate E the scaling is an exact exponent add and the
// rounding is the hardware's float64 -> int64 conversion (round to nearest even); values whose scaled
// magnitude is below 2^-1022 (zeros and subnormals) give 0.  Extreme E take the integer path below
// (round half away from zero).
__device__ __forceinline__ long long fx_from(double x, int E) {
    if (E > -900 && E < 1000) {
        const int hi = __double2hiint(x), lo = __double2loint(x);
        const int emin = max(0, E - 58);
        if ((hi & 0x7FF00000) <= emin * (1 << 20)) return 0;
        return __double2ll_rn(__hiloint2double(hi + (58 - E) * (1 << 20), lo));
    }
    const unsigned long long b = (unsigned long long) __double_as_longlong(x);
    const int e = (int) ((b >> 52) & 0x7FF);
    unsigned long long m = b & 0xFFFFFFFFFFFFFull;
    int ex;
    if (e == 0) ex = 1 - 1075;
    else { m |= 1ull << 52; ex = e - 1075; }
    const int sh = ex + 58 - E;
    unsigned long long q;
    if (sh >= 0) q = m << sh;
    else if (sh > -64) q = (m + (1ull << (-sh - 1))) >> (-sh);
    else q = 0;
    return (b >> 63) ? -(long long) q : (long long) q;
}

// q * 2^(E-58) rounded to float64 (nearest even): the hardware int64 -> float64 conversion, then an
// exact exponent add; extreme E take the integer path.
__device__ __forceinline__ double fx_to(long long q, int E) {
    if (q == 0) return 0.0;
    if (E > -900 && E < 1000) {
        const double d = __ll2double_rn(q);
        return __hiloint2double(__double2hiint(d) + (E - 58) * (1 << 20), __double2loint(d));
    }
    const unsigned long long sign = q < 0 ? 1ull : 0ull;
    const unsigned long long a = q < 0 ? (unsigned long long) (-q) : (unsigned long long) q;
    const int bl = 64 - __clzll((long long) a);
    unsigned long long mant;
    int exp2 = bl - 1 + E - 58;
    if (bl <= 53) {
        mant = a << (53 - bl);
    } else {
        const int sh = bl - 53;
        mant = a >> sh;
        const unsigned long long rem = a & ((1ull << sh) - 1), half = 1ull << (sh - 1);
        if (rem > half || (rem == half && (mant & 1ull))) {
            mant++;
            if (mant == (1ull << 53)) { mant >>= 1; exp2++; }
        }
    }
    return __longlong_as_double((long long) ((sign << 63) | ((unsigned long long) (exp2 + 1023) << 52) | (mant & 0xFFFFFFFFFFFFFull)));
}

__device__ __forceinline__ long long fx_mul(long long z, unsigned long long w, int sh, int neg) {
    const bool zn = z < 0;
    const unsigned long long a = zn ? (unsigned long long) (-z) : (unsigned long long) z;
    const unsigned long long lo = a * w, hi = __umul64hi(a, w);
    unsigned long long r;
    if (sh >= 64) r = hi >> (sh - 64);
    else if (sh == 0) r = lo;
    else {
        const unsigned long long lo2 = lo + (1ull << (sh - 1));
        const unsigned long long hi2 = hi + (lo2 < lo ? 1ull : 0ull);
        r = (lo2 >> sh) | (hi2 << (64 - sh));
    }
    return (zn != (neg != 0)) ? -(long long) r : (long long) r;
}

__device__ __forceinline__ int scale_exp(const unsigned long long* maxslots, int step, unsigned long long bound_bits) {
    unsigned long long m = maxslots[step % 3];
    if (bound_bits > m) m = bound_bits;
    if (m == 0) return -1000;
    return (int) ((m >> 52) & 0x7FF) - 1023 + 1;
}

__device__ __forceinline__ void block_max_commit(unsigned long long v, unsigned long long* slot) {
    for (int s = 16; s > 0; s >>= 1) {
        const unsigned long long o = __shfl_xor_sync(0xffffffffu, v, s);
        v = o > v ? o : v;
    }
    if ((threadIdx.x & 31) == 0 && v) atomicMax(slot, v);
}

// ------------------------------------------------------------------------------------------------ 3D
constexpr int TX = 32, TY = 8;

template <bool FAST>
__global__ void __launch_bounds__(TX * TY) axis3d_kernel(FieldView in, FieldView out, Box box, AxisParams P, unsigned long long* maxslots,
                                                          int step, int zchunk) {
    using T = typename std::conditional<FAST, long long, double>::type;
    __shared__ T tile[TY + 2][TX + 2];
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int x0 = box.lo[0] + blockIdx.x * TX, y0 = box.lo[1] + blockIdx.y * TY;
    const int i = x0 + tx, j = y0 + ty;
    const bool valid = i < box.hi[0] && j < box.hi[1];
    const int ic = min(i, box.hi[0]), jc = min(j, box.hi[1]);
    const int zs = box.lo[2] + blockIdx.z * zchunk;
    const int ze = min(zs + zchunk, box.hi[2]);
    if (zs >= ze) return;
    int E = 0;
    if (FAST) {
        E = scale_exp(maxslots, step, P.bound_bits);
        if (blockIdx.x == 0 && blockIdx.y == 0 && blockIdx.z == 0 && tx == 0 && ty == 0) maxslots[(step + 2) % 3] = 0ull;
    }
    auto conv = [&](double v) -> T {
        if constexpr (FAST) return fx_from(v, E);
        else return v;
    };
    T below = conv(ld3(in, ic, jc, zs - 1));
    T cur = conv(ld3(in, ic, jc, zs));
    unsigned long long vmax = 0;
    for (int k = zs; k < ze; ++k) {
        const T above = conv(ld3(in, ic, jc, k + 1));
        tile[ty + 1][tx + 1] = cur;
        if (tx == 0) tile[ty + 1][0] = conv(ld3(in, x0 - 1, jc, k));
        if (tx == TX - 1) tile[ty + 1][TX + 1] = conv(ld3(in, min(x0 + TX, box.hi[0]), jc, k));
        if (ty == 0) tile[0][tx + 1] = conv(ld3(in, ic, y0 - 1, k));
        if (ty == TY - 1) tile[TY + 1][tx + 1] = conv(ld3(in, ic, min(y0 + TY, box.hi[1]), k));
        __syncthreads();
        if (valid) {
            const T l = tile[ty + 1][tx], r = tile[ty + 1][tx + 2];
            const T b = tile[ty][tx + 1], t = tile[ty + 2][tx + 1];
            double v;
            if constexpr (FAST) {
                long long q = cur;
                if (P.iso) {
                    const long long z = (l - cur) + (r - cur) + (b - cur) + (t - cur) + (below - cur) + (above - cur);
                    q += fx_mul(z, P.wm[0], P.wshift[0], P.wneg[0]);
                } else {
                    q += fx_mul((l - cur) + (r - cur), P.wm[0], P.wshift[0], P.wneg[0]);
                    q += fx_mul((b - cur) + (t - cur), P.wm[1], P.wshift[1], P.wneg[1]);
                    q += fx_mul((below - cur) + (above - cur), P.wm[2], P.wshift[2], P.wneg[2]);
                }
                v = fx_to(q, E);
                const unsigned long long ab = (unsigned long long) __double_as_longlong(v) & 0x7FFFFFFFFFFFFFFFull;
                vmax = ab > vmax ? ab : vmax;
            } else {
                double d2v[3];
                d2v[0] = d2_exact(l, cur, r, P.h[0], P.inv_h[0], P.pow2[0]);
                d2v[1] = d2_exact(b, cur, t, P.h[1], P.inv_h[1], P.pow2[1]);
                d2v[2] = d2_exact(below, cur, above, P.h[2], P.inv_h[2], P.pow2[2]);
                double sum = d2v[P.order[0]];
                sum = __dadd_rn(sum, d2v[P.order[1]]);
                sum = __dadd_rn(sum, d2v[P.order[2]]);
                v = __dadd_rn(cur, __dmul_rn(P.s, sum));
            }
            out.data[(long long) (i - out.off[0]) + (long long) (j - out.off[1]) * out.sy + (long long) (k - out.off[2]) * out.sz] = v;
        }
        __syncthreads();
        below = cur;
        cur = above;
    }
    if (FAST) block_max_commit(vmax, &maxslots[(step + 1) % 3]);
}

// ------------------------------------------------------------------------------------------------ 2D
constexpr int TX2 = 128;

template <bool FAST>
__global__ void __launch_bounds__(TX2) axis2d_kernel(FieldView in, FieldView out, Box box, AxisParams P, unsigned long long* maxslots, int step,
                                                     int ychunk) {
    using T = typename std::conditional<FAST, long long, double>::type;
    __shared__ T row[TX2 + 2];
    const int tx = threadIdx.x;
    const int x0 = box.lo[0] + blockIdx.x * TX2;
    const int i = x0 + tx;
    const bool vx = i < box.hi[0];
    const int ic = min(i, box.hi[0]);
    const int ys = box.lo[1] + blockIdx.y * ychunk;
    const int ye = min(ys + ychunk, box.hi[1]);
    if (ys >= ye) return;
    int E = 0;
    if (FAST) {
        E = scale_exp(maxslots, step, P.bound_bits);
        if (blockIdx.x == 0 && blockIdx.y == 0 && tx == 0) maxslots[(step + 2) % 3] = 0ull;
    }
    auto conv = [&](double v) -> T {
        if constexpr (FAST) return fx_from(v, E);
        else return v;
    };
    const int k = box.lo[2];
    T below = conv(ld3(in, ic, ys - 1, k));
    T cur = conv(ld3(in, ic, ys, k));
    unsigned long long vmax = 0;
    for (int j = ys; j < ye; ++j) {
        const T above = conv(ld3(in, ic, j + 1, k));
        row[tx + 1] = cur;
        if (tx == 0) row[0] = conv(ld3(in, x0 - 1, j, k));
        if (tx == TX2 - 1) row[TX2 + 1] = conv(ld3(in, min(x0 + TX2, box.hi[0]), j, k));
        __syncthreads();
        if (vx) {
            const T l = row[tx], r = row[tx + 2];
            double v;
            if constexpr (FAST) {
                long long q = cur;
                if (P.iso) {
                    q += fx_mul((l - cur) + (r - cur) + (below - cur) + (above - cur), P.wm[0], P.wshift[0], P.wneg[0]);
                } else {
                    q += fx_mul((l - cur) + (r - cur), P.wm[0], P.wshift[0], P.wneg[0]);
                    q += fx_mul((below - cur) + (above - cur), P.wm[1], P.wshift[1], P.wneg[1]);
                }
                v = fx_to(q, E);
                const unsigned long long ab = (unsigned long long) __double_as_longlong(v) & 0x7FFFFFFFFFFFFFFFull;
                vmax = ab > vmax ? ab : vmax;
            } else {
                double d2v[2];
                d2v[0] = d2_exact(l, cur, r, P.h[0], P.inv_h[0], P.pow2[0]);
                d2v[1] = d2_exact(below, cur, above, P.h[1], P.inv_h[1], P.pow2[1]);
                double sum = __dadd_rn(d2v[P.order[0]], d2v[P.order[1]]);
                v = __dadd_rn(cur, __dmul_rn(P.s, sum));
            }
            out.data[(long long) (i - out.off[0]) + (long long) (j - out.off[1]) * out.sy + (long long) (k - out.off[2]) * out.sz] = v;
        }
        __syncthreads();
        below = cur;
        cur = above;
    }
    if (FAST) block_max_commit(vmax, &maxslots[(step + 1) % 3]);
}

// ------------------------------------------------------------------------- 3D, register-blocked
// One warp covers 32 consecutive x-columns and computes the 30 inner ones (lanes 1..30; lanes 0 and 31
// only supply the x neighbours) for RB consecutive y-rows, marching along z.  The planes z-1, z, z+1
// of those rows stay in registers (z and z+1 with one halo row on each side), plane z+2 is loaded
// while z is computed, and x neighbours come from warp shuffles.  No shared memory, no CTA barrier.
constexpr int RB = 8;
constexpr int RB_WARPS = 4;
constexpr int RB_COLS = 30;

template <bool FAST>
__global__ void __launch_bounds__(32 * RB_WARPS, 4) axis3d_rb_kernel(FieldView in, FieldView out, Box box, AxisParams P, unsigned long long* maxslots,
                                                                  int step, int zchunk, int tiles_x, int tiles_y) {
    using T = typename std::conditional<FAST, long long, double>::type;
    const int lane = threadIdx.x & 31;
    const int warp = blockIdx.x * RB_WARPS + (threadIdx.x >> 5);
    if (warp >= tiles_x * tiles_y) return;
    const int tx = warp % tiles_x, ty = warp / tiles_x;
    const int x0 = box.lo[0] + tx * RB_COLS, y0 = box.lo[1] + ty * RB;
    const int i = x0 - 1 + lane;
    const bool vx = lane >= 1 && lane <= RB_COLS && i < box.hi[0];
    const int ic = min(i, box.hi[0]);
    const int zs = box.lo[2] + blockIdx.y * zchunk;
    const int ze = min(zs + zchunk, box.hi[2]);
    if (zs >= ze) return;
    int E = 0;
    if (FAST) {
        E = scale_exp(maxslots, step, P.bound_bits);
        if (blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0) maxslots[(step + 2) % 3] = 0ull;
    }
    auto conv = [&](double v) -> T {
        if constexpr (FAST) return fx_from(v, E);
        else return v;
    };
    // row offsets of y0-1 .. y0+RB, clamped to the box edge + 1 (the farthest row the stencil reads)
    long long roff[RB + 2];
#pragma unroll
    for (int r = 0; r < RB + 2; ++r) roff[r] = (long long) (min(y0 - 1 + r, box.hi[1]) - in.off[1]) * in.sy;
    const double* col = in.data + (ic - in.off[0]) - (long long) in.off[2] * in.sz;
    T below[RB], cur[RB + 2], above[RB + 2];
    double nxt[RB + 2];
    {
        const double* pm = col + (long long) (zs - 1) * in.sz;
        const double* p0 = col + (long long) zs * in.sz;
        const double* p1 = col + (long long) min(zs + 1, box.hi[2]) * in.sz;
#pragma unroll
        for (int r = 0; r < RB; ++r) below[r] = conv(pm[roff[r + 1]]);
#pragma unroll
        for (int r = 0; r < RB + 2; ++r) cur[r] = conv(p0[roff[r]]);
#pragma unroll
        for (int r = 0; r < RB + 2; ++r) above[r] = conv(p1[roff[r]]);
    }
    unsigned long long vmax = 0;
    double* const ocol = out.data + (i - out.off[0]) - (long long) out.off[1] * out.sy - (long long) out.off[2] * out.sz;
    for (int k = zs; k < ze; ++k) {
        {
            const double* pn = col + (long long) min(k + 2, box.hi[2]) * in.sz;
#pragma unroll
            for (int r = 0; r < RB + 2; ++r) nxt[r] = pn[roff[r]];
        }
#pragma unroll
        for (int r = 0; r < RB; ++r) {
            const T c = cur[r + 1];
            const T l = __shfl_up_sync(0xffffffffu, c, 1);
            const T rr = __shfl_down_sync(0xffffffffu, c, 1);
            const int j = y0 + r;
            if (vx && j < box.hi[1]) {
                const T b = cur[r], t = cur[r + 2], zb = below[r], za = above[r + 1];
                double v;
                if constexpr (FAST) {
                    long long q = c;
                    if (P.iso) {
                        const long long z = (l - c) + (rr - c) + (b - c) + (t - c) + (zb - c) + (za - c);
                        q += fx_mul(z, P.wm[0], P.wshift[0], P.wneg[0]);
                    } else {
                        q += fx_mul((l - c) + (rr - c), P.wm[0], P.wshift[0], P.wneg[0]);
                        q += fx_mul((b - c) + (t - c), P.wm[1], P.wshift[1], P.wneg[1]);
                        q += fx_mul((zb - c) + (za - c), P.wm[2], P.wshift[2], P.wneg[2]);
                    }
                    v = fx_to(q, E);
                    const unsigned long long ab = (unsigned long long) __double_as_longlong(v) & 0x7FFFFFFFFFFFFFFFull;
                    vmax = ab > vmax ? ab : vmax;
                } else {
                    const double d0 = d2_exact(l, c, rr, P.h[0], P.inv_h[0], P.pow2[0]);
                    const double d1 = d2_exact(b, c, t, P.h[1], P.inv_h[1], P.pow2[1]);
                    const double d2 = d2_exact(zb, c, za, P.h[2], P.inv_h[2], P.pow2[2]);
                    auto pick = [&](int a) { return a == 0 ? d0 : (a == 1 ? d1 : d2); };
                    double sum = pick(P.order[0]);
                    sum = __dadd_rn(sum, pick(P.order[1]));
                    sum = __dadd_rn(sum, pick(P.order[2]));
                    v = __dadd_rn(c, __dmul_rn(P.s, sum));
                }
                ocol[(long long) (j) * out.sy + (long long) k * out.sz] = v;
            }
        }
#pragma unroll
        for (int r = 0; r < RB; ++r) below[r] = cur[r + 1];
#pragma unroll
        for (int r = 0; r < RB + 2; ++r) cur[r] = above[r];
#pragma unroll
        for (int r = 0; r < RB + 2; ++r) above[r] = conv(nxt[r]);
    }
    if (FAST) block_max_commit(vmax, &maxslots[(step + 1) % 3]);
}

// ------------------------------------------------------------- 3D, fixed point kept between steps
// A run of K >= 2 fixed-point steps of a field whose update box is surrounded by constant boundary
// nodes (node-centred Dirichlet, no ghost layer) and whose weights obey the maximum principle
// (w_d >= 0, 1 - 2 sum_d w_d >= 0): then |u| never exceeds its initial bound 2^E, one scale serves every
// step, and the field's two buffers hold 64-bit fixed-point integers between the steps instead of
// values rounded to float64 and converted back at every step.  The first step reads float64 (MODE bit
// 0) and converts as it loads; after it the boundary nodes of both buffers hold the fixed-point bit
// patterns of their constants (fill_dirichlet_nodes), so the steady state converts nothing; the last
// step writes float64 (MODE bit 1) and the float64 constants are put back.  Per update: the six
// neighbours' sum minus six times the centre (exact), one 64 x 64-bit high product, one add - no
// float64 instruction.  Same register blocking as axis3d_rb_kernel, 6 rows per warp.

// (z * w + 2^(sh-1)) >> sh (floor, on the exact 128-bit product) for a weight 0 <= w < 2^53 given as
// ws = w * 2^(64 - sh) (exact, ws < 2^63, so 54 <= sh <= 64): the product's high word plus the carry of
// adding 2^63 to its low word.
__device__ __forceinline__ long long fx_mul_hi(long long z, long long ws) {
    const unsigned long long lo = (unsigned long long) z * (unsigned long long) ws;
    return __mul64hi(z, ws) + (long long) (lo >> 63);
}

template <int MODE, int RBX>
__global__ void __launch_bounds__(32 * RB_WARPS, RBX <= 4 ? 6 : (RBX <= 6 ? 5 : 4)) axis3d_fxres_kernel(FieldView in, FieldView out, Box box, AxisParams P, long long ws0,
                                                                     long long ws1, long long ws2, const unsigned long long* maxslots,
                                                                     int zchunk, int tiles_x, int tiles_y) {
    constexpr bool IN_F64 = (MODE & 1) != 0, OUT_F64 = (MODE & 2) != 0;
    const int lane = threadIdx.x & 31;
    const int warp = blockIdx.x * RB_WARPS + (threadIdx.x >> 5);
    if (warp >= tiles_x * tiles_y) return;
    const int tx = warp % tiles_x, ty = warp / tiles_x;
    const int x0 = box.lo[0] + tx * RB_COLS, y0 = box.lo[1] + ty * RBX;
    const int i = x0 - 1 + lane;
    const bool vx = lane >= 1 && lane <= RB_COLS && i < box.hi[0];
    const int ic = min(i, box.hi[0]);
    const int zs = box.lo[2] + blockIdx.y * zchunk;
    const int ze = min(zs + zchunk, box.hi[2]);
    if (zs >= ze) return;
    const int E = scale_exp(maxslots, 0, P.bound_bits);
    long long roff[RBX + 2];
#pragma unroll
    for (int r = 0; r < RBX + 2; ++r) roff[r] = (long long) (min(y0 - 1 + r, box.hi[1]) - in.off[1]) * in.sy;
    const double* col = in.data + (ic - in.off[0]) - (long long) in.off[2] * in.sz;
    auto ldq = [&](double v) -> long long {
        if constexpr (IN_F64) return fx_from(v, E);
        else return __double_as_longlong(v);
    };
    long long below[RBX], cur[RBX + 2], above[RBX + 2];
    double nxt[RBX + 2];
    {
        const double* pm = col + (long long) (zs - 1) * in.sz;
        const double* p0 = col + (long long) zs * in.sz;
        const double* p1 = col + (long long) min(zs + 1, box.hi[2]) * in.sz;
#pragma unroll
        for (int r = 0; r < RBX; ++r) below[r] = ldq(pm[roff[r + 1]]);
#pragma unroll
        for (int r = 0; r < RBX + 2; ++r) cur[r] = ldq(p0[roff[r]]);
#pragma unroll
        for (int r = 0; r < RBX + 2; ++r) above[r] = ldq(p1[roff[r]]);
    }
    double* const ocol = out.data + (i - out.off[0]) - (long long) out.off[1] * out.sy - (long long) out.off[2] * out.sz;
    for (int k = zs; k < ze; ++k) {
        {
            const double* pn = col + (long long) min(k + 2, box.hi[2]) * in.sz;
#pragma unroll
            for (int r = 0; r < RBX + 2; ++r) nxt[r] = pn[roff[r]];
        }
#pragma unroll
        for (int r = 0; r < RBX; ++r) {
            const long long c = cur[r + 1];
            const long long l = __shfl_up_sync(0xffffffffu, c, 1);
            const long long rr = __shfl_down_sync(0xffffffffu, c, 1);
            if (vx && y0 + r < box.hi[1]) {
                const long long b = cur[r], t = cur[r + 2], zb = below[r], za = above[r + 1];
                long long q = c;
                if (P.iso) {
                    q += fx_mul_hi(((l + rr) + (b + t)) + ((zb + za) - 6 * c), ws0);
                } else {
                    q += fx_mul_hi((l + rr) - 2 * c, ws0);
                    q += fx_mul_hi((b + t) - 2 * c, ws1);
                    q += fx_mul_hi((zb + za) - 2 * c, ws2);
                }
                ocol[(long long) (y0 + r) * out.sy + (long long) k * out.sz] = OUT_F64 ? fx_to(q, E) : __longlong_as_double(q);
            }
        }
#pragma unroll
        for (int r = 0; r < RBX; ++r) below[r] = cur[r + 1];
#pragma unroll
        for (int r = 0; r < RBX + 2; ++r) cur[r] = above[r];
#pragma unroll
        for (int r = 0; r < RBX + 2; ++r) above[r] = ldq(nxt[r]);
    }
}

// -------------------------------------------------------------------------- 2D resident fixed point
// One step of a resident fixed-point run on a 2D grid (u + w_x (u(i-1) + u(i+1) - 2u) + w_y (...), or
// one weight times the four neighbours' sum minus four times the centre): a warp covers 32 consecutive
// x-columns and updates the 30 inner ones over R2 rows, loading its R2 + 2 rows at once (every load in
// flight together: a 2D grid of this kind is usually L2-resident, so a step is one round trip plus the
// bandwidth time), x neighbours by warp shuffles.  MODE bit 0: float64 in (converted as loaded), bit 1:
// float64 out; the steady state converts nothing.
constexpr int R2ROWS = 8;

template <int MODE>
__global__ void __launch_bounds__(32 * RB_WARPS) axis2d_fxres_kernel(FieldView in, FieldView out, Box box, int iso, long long ws0, long long ws1,
                                                                   const unsigned long long* maxslots, unsigned long long bound_bits,
                                                                   int tiles_x, int tiles_y) {
    constexpr bool IN_F64 = (MODE & 1) != 0, OUT_F64 = (MODE & 2) != 0;
    const int lane = threadIdx.x & 31;
    const int warp = blockIdx.x * RB_WARPS + (threadIdx.x >> 5);
    if (warp >= tiles_x * tiles_y) return;
    const int tx = warp % tiles_x, ty = warp / tiles_x;
    const int x0 = box.lo[0] + tx * RB_COLS, y0 = box.lo[1] + ty * R2ROWS;
    const int i = x0 - 1 + lane;
    const bool vx = lane >= 1 && lane <= RB_COLS && i < box.hi[0];
    const int ic = min(i, box.hi[0]);
    const int k = box.lo[2];
    const int E = (MODE != 0) ? scale_exp(maxslots, 0, bound_bits) : 0;
    long long v[R2ROWS + 2];
#pragma unroll
    for (int r = 0; r < R2ROWS + 2; ++r) {
        const double d = ld3(in, ic, min(y0 - 1 + r, box.hi[1]), k);
        if constexpr (IN_F64) v[r] = fx_from(d, E);
        else v[r] = __double_as_longlong(d);
    }
    double* const orow = out.data + (i - out.off[0]) - (long long) out.off[1] * out.sy + (long long) (k - out.off[2]) * out.sz;
#pragma unroll
    for (int r = 0; r < R2ROWS; ++r) {
        const long long c = v[r + 1];
        const long long l = __shfl_up_sync(0xffffffffu, c, 1);
        const long long rr = __shfl_down_sync(0xffffffffu, c, 1);
        if (vx && y0 + r < box.hi[1]) {
            const long long b = v[r], t = v[r + 2];
            long long q = c;
            if (iso) {
                q += fx_mul_hi((l + rr) + (b + t) - 4 * c, ws0);
            } else {
                q += fx_mul_hi((l + rr) - 2 * c, ws0);
                q += fx_mul_hi((b + t) - 2 * c, ws1);
            }
            orow[(long long) (y0 + r) * out.sy] = OUT_F64 ? fx_to(q, E) : __longlong_as_double(q);
        }
    }
}

// ------------------------------------------------------- 3D resident fixed point, TMA-staged planes
// The steady-state step of a resident run (fixed point in, fixed point out) with its planes staged in
// shared memory by TMA: a CTA owns FT_X x FT_Y points of the xy plane and a run of zchunk planes.  One
// thread streams each plane's FT_W x FT_H box (the tile and its one-point halo, from (x origin - 1,
// y origin - 1), an x coordinate on a 16-byte boundary) into a ring of FT_RING slots, up to
// FT_RING - 2 planes ahead of the plane being updated; each slot's mbarrier counts the box's bytes.
// One CTA barrier per plane: past it, the slot of the previous plane is refilled.
// A thread updates FT_ROWS consecutive rows of one x-column: the centre values of planes k - 1 and k
// stay in registers, the x and y neighbours and plane k + 1 come from shared memory, the results go
// straight to global memory (64-bit coalesced stores).  The integer operations are those of
// axis3d_fxres_kernel<0, *>, so the two give bit-identical fields.
constexpr int FT_X = 64, FT_Y = 16, FT_ROWS = 4, FT_RING = 5;
constexpr int FT_W = FT_X + 2, FT_H = FT_Y + 2;
constexpr int FT_THREADS = FT_X * FT_Y / FT_ROWS;
constexpr int FT_SLOT = ((FT_W * FT_H * 8 + 127) / 128) * 16;  // int64 per slot (a 128-byte multiple)
constexpr unsigned FT_BYTES = FT_W * FT_H * 8;                  // bytes per plane box
struct FtStage {
    long long v[FT_RING][FT_SLOT];
    unsigned long long bar[FT_RING];
};
static_assert((FT_W * 8) % 16 == 0, "box rows are 16-byte multiples");
static_assert(FT_RING >= 3, "planes k and k + 1 are read while k + 2 is in flight");

// set when a wait of axis3d_fxtma_kernel gave up
__device__ int g_st_err;

__global__ void __launch_bounds__(FT_THREADS, 4) axis3d_fxtma_kernel(const __grid_constant__ CUtensorMap map, FieldView in, FieldView out,
                                                                   Box box, int iso, long long ws0, long long ws1, long long ws2, int zchunk,
                                                                   int tiles_x) {
    __shared__ __align__(128) FtStage St;
    const int tx = blockIdx.x % tiles_x, ty = blockIdx.x / tiles_x;
    const int x0 = box.lo[0] + tx * FT_X, y0 = box.lo[1] + ty * FT_Y;
    const int zs = box.lo[2] + blockIdx.y * zchunk;
    const int ze = min(zs + zchunk, box.hi[2]);
    if (zs >= ze) return;  // (the whole CTA)
    const int lx = threadIdx.x % FT_X, ly0 = (threadIdx.x / FT_X) * FT_ROWS;
    const int i = x0 + lx;
    const bool vx = i < box.hi[0];
    if (threadIdx.x == 0) {
        for (int s = 0; s < FT_RING; ++s) mbar_init(&St.bar[s], 1);
        mbar_fence_init();
    }
    __syncthreads();
    // plane p (zs - 1 .. ze) is this tile's plane number q = p - zs + 1: slot q % FT_RING, phase (q / FT_RING) & 1
    auto slot_of = [&](int p) { return (p - zs + 1) % FT_RING; };
    auto phase_of = [&](int p) { return (unsigned) ((p - zs + 1) / FT_RING) & 1u; };
    const int cx = x0 - 1 - in.off[0], cy = y0 - 1 - in.off[1];
    const bool producer = threadIdx.x == 0;
    auto issue = [&](int p) {
        const int s = slot_of(p);
        mbar_arrive_expect(&St.bar[s], FT_BYTES);
        tma_load_3d(&St.v[s][0], &map, cx, cy, p - in.off[2], &St.bar[s]);
    };
    const int last = ze;
    int issued = min(zs - 1 + FT_RING - 1, last);  // planes zs - 1 .. issued fill every slot
    if (producer)
        for (int p = zs - 1; p <= issued; ++p) issue(p);
    bool ok = mbar_wait(&St.bar[slot_of(zs - 1)], phase_of(zs - 1));
    ok = ok && mbar_wait(&St.bar[slot_of(zs)], phase_of(zs));
    long long below[FT_ROWS], cur[FT_ROWS];
    const int at0 = (ly0 + 1) * FT_W + lx + 1;  // the thread's first point in a slot
    if (ok) {
        const long long* Sb = St.v[slot_of(zs - 1)];
        const long long* Sc = St.v[slot_of(zs)];
#pragma unroll
        for (int r = 0; r < FT_ROWS; ++r) {
            below[r] = Sb[at0 + r * FT_W];
            cur[r] = Sc[at0 + r * FT_W];
        }
    }
    double* const ocol = out.data + (i - out.off[0]) - (long long) out.off[1] * out.sy - (long long) out.off[2] * out.sz;
    bool failed = false;
    for (int k = zs; k < ze; ++k) {
        ok = ok && mbar_wait(&St.bar[slot_of(k + 1)], phase_of(k + 1));
        if (__syncthreads_or(!ok)) {  // (the same answer in every thread)
            failed = true;
            break;
        }
        if (issued < last) {  // every thread is past step k - 1: plane k - 1's slot takes plane k + FT_RING - 1
            ++issued;
            if (producer) issue(issued);
        }
        const long long* S = St.v[slot_of(k)];
        const long long* A = St.v[slot_of(k + 1)];
        long long above[FT_ROWS];
#pragma unroll
        for (int r = 0; r < FT_ROWS; ++r) above[r] = A[at0 + r * FT_W];
#pragma unroll
        for (int r = 0; r < FT_ROWS; ++r) {
            const int at = at0 + r * FT_W;
            const long long c = cur[r];
            const long long l = S[at - 1], rr = S[at + 1];
            const long long b = r == 0 ? S[at - FT_W] : cur[r - 1];
            const long long t = r == FT_ROWS - 1 ? S[at + FT_W] : cur[r + 1];
            const long long zb = below[r], za = above[r];
            const int j = y0 + ly0 + r;
            if (vx && j < box.hi[1]) {
                long long q = c;
                if (iso) {
                    q += fx_mul_hi(((l + rr) + (b + t)) + ((zb + za) - 6 * c), ws0);
                } else {
                    q += fx_mul_hi((l + rr) - 2 * c, ws0);
                    q += fx_mul_hi((b + t) - 2 * c, ws1);
                    q += fx_mul_hi((zb + za) - 2 * c, ws2);
                }
                ocol[(long long) j * out.sy + (long long) k * out.sz] = __longlong_as_double(q);
            }
        }
#pragma unroll
        for (int r = 0; r < FT_ROWS; ++r) {
            below[r] = cur[r];
            cur[r] = above[r];
        }
    }
    if (failed) {
        // a copy never completed: record it, wait (bounded) for every copy this tile issued, stop
        // (the last fill of each slot: the earlier ones have completed)
        if (producer) {
            for (int p = max(zs - 1, issued - FT_RING + 1); p <= issued; ++p) mbar_wait(&St.bar[slot_of(p)], phase_of(p));
            atomicExch(&g_st_err, 1);
        }
    }
}

// The TMA-staged steady-state step (default) or the register-blocked one: OPFLOW_FXRES_TMA=0|1, read at
// every launch.
static bool fxtma_enabled() {
    const char* e = getenv("OPFLOW_FXRES_TMA");
    return !(e && e[0] == '0');
}

int stencil_take_error(cudaStream_t s, int* err) {
    int zero = 0;
    OPG_CUDA(cudaMemcpyFromSymbolAsync(err, g_st_err, sizeof(int), 0, cudaMemcpyDeviceToHost, s));
    OPG_CUDA(cudaStreamSynchronize(s));
    if (*err) OPG_CUDA(cudaMemcpyToSymbolAsync(g_st_err, &zero, sizeof(int), 0, cudaMemcpyHostToDevice, s));
    return OPFLOW_OK;
}

// Whether the TMA-staged steady-state step takes this box of this buffer: rows and planes on 16-byte
// strides, a 16-byte aligned buffer, the tiles' x origins minus one on even indices (16-byte boundaries)
// and the box's halo inside the buffer.
static bool fxtma_ok(const FieldView& in, const Box& box) {
    if (((unsigned long long) in.data & 15ull) != 0 || (in.sy & 1) != 0 || (in.sz & 1) != 0) return false;
    if (((box.lo[0] - 1 - in.off[0]) & 1) != 0) return false;
    for (int d = 0; d < 3; ++d)
        if (box.lo[d] - 1 < in.off[d] || box.hi[d] + 1 > in.off[d] + in.dims[d]) return false;
    return in.dims[0] <= in.sy && (long long) in.dims[1] * in.sy <= in.sz;
}

bool axis_resident_ok(const AxisParams& P) {
    for (int d = 0; d < P.ndim; ++d) {
        const int g = P.iso ? 0 : d;
        if (P.wneg[g] || P.wshift[g] < 54 || P.wshift[g] > 64) return false;
        if (P.wm[g] >= (1ull << 53)) return false;
        if (P.wshift[g] < 64 && (P.wm[g] >> (P.wshift[g] - 1)) != 0) return false;  // w * 2^(64 - sh) < 2^63
    }
    return true;
}

int axis_launch_resident(opflow_ctx ctx, const FieldView& in, const FieldView& out, const Box& box, const AxisParams& P,
                         const unsigned long long* maxslots, bool first, bool last) {
    if (!axis_resident_ok(P)) return fail(OPFLOW_E_UNSUPPORTED, "weights outside the resident fixed-point kernel's range");
    const int nx = box.hi[0] - box.lo[0], ny = box.hi[1] - box.lo[1], nz = box.hi[2] - box.lo[2];
    if (nx <= 0 || ny <= 0 || nz <= 0) return OPFLOW_OK;
    if (P.ndim == 2) {
        const int tiles_x = (nx + RB_COLS - 1) / RB_COLS, tiles_y = (ny + R2ROWS - 1) / R2ROWS;
        const int g = (int) (((long long) tiles_x * tiles_y + RB_WARPS - 1) / RB_WARPS);
        const int gi1 = P.iso ? 0 : 1;
        const long long w0 = (long long) (P.wm[0] << (64 - P.wshift[0])), w1 = (long long) (P.wm[gi1] << (64 - P.wshift[gi1]));
        const int mode = (first ? 1 : 0) | (last ? 2 : 0);
        switch (mode) {
            case 0: axis2d_fxres_kernel<0><<<g, 32 * RB_WARPS, 0, ctx->stream>>>(in, out, box, P.iso, w0, w1, maxslots, P.bound_bits, tiles_x, tiles_y); break;
            case 1: axis2d_fxres_kernel<1><<<g, 32 * RB_WARPS, 0, ctx->stream>>>(in, out, box, P.iso, w0, w1, maxslots, P.bound_bits, tiles_x, tiles_y); break;
            case 2: axis2d_fxres_kernel<2><<<g, 32 * RB_WARPS, 0, ctx->stream>>>(in, out, box, P.iso, w0, w1, maxslots, P.bound_bits, tiles_x, tiles_y); break;
            default: axis2d_fxres_kernel<3><<<g, 32 * RB_WARPS, 0, ctx->stream>>>(in, out, box, P.iso, w0, w1, maxslots, P.bound_bits, tiles_x, tiles_y); break;
        }
        OPG_LAUNCHED();
        return check_launch("axis2d_fxres_kernel");
    }
    if (P.ndim != 3) return fail(OPFLOW_E_UNSUPPORTED, "the resident fixed-point kernels cover 2D and 3D grids");
    // rows per warp: 6 (the measured best at 512^3); OPFLOW_FXRES_RB=4|6|8 for sweeps
    int rbx = 6;
    if (const char* e = getenv("OPFLOW_FXRES_RB")) rbx = atoi(e) == 4 ? 4 : (atoi(e) == 8 ? 8 : 6);
    const int tiles_x = (nx + RB_COLS - 1) / RB_COLS, tiles_y = (ny + rbx - 1) / rbx;
    const int bx = (tiles_x * tiles_y + RB_WARPS - 1) / RB_WARPS;
    const int per_sm = rbx == 4 ? 6 : (rbx == 6 ? 5 : 4);
    int zchunks = (ctx->num_sms * per_sm * 3 / 2 + bx - 1) / bx;
    zchunks = std::max(1, std::min(zchunks, (nz + 15) / 16));
    const int zchunk = (nz + zchunks - 1) / zchunks;
    zchunks = (nz + zchunk - 1) / zchunk;
    dim3 g(bx, zchunks), b(32 * RB_WARPS);
    // the weights as w * 2^(64 - wshift), exact and below 2^63 (checked by axis_resident_ok)
    long long ws[3];
    for (int d = 0; d < 3; ++d) {
        const int gi = P.iso ? 0 : d;
        ws[d] = (long long) (P.wm[gi] << (64 - P.wshift[gi]));
    }
    if (!first && !last && fxtma_enabled() && fxtma_ok(in, box)) {
        const PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
        CUtensorMap map;
        const cuuint64_t dims[3] = {(cuuint64_t) in.dims[0], (cuuint64_t) in.dims[1], (cuuint64_t) in.dims[2]};
        const cuuint64_t strides[2] = {(cuuint64_t) in.sy * 8, (cuuint64_t) in.sz * 8};
        const cuuint32_t boxd[3] = {FT_W, FT_H, 1}, ones[3] = {1, 1, 1};
        if (enc && enc(&map, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 3, (void*) in.data, dims, strides, boxd, ones, CU_TENSOR_MAP_INTERLEAVE_NONE,
                       CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS) {
            // planes per CTA: OPFLOW_FXTMA_Z for sweeps
            int zc = 32;
            if (const char* e = getenv("OPFLOW_FXTMA_Z")) zc = std::max(4, std::min(1024, atoi(e)));
            const int ftx = (nx + FT_X - 1) / FT_X, fty = (ny + FT_Y - 1) / FT_Y;
            const int zch = (nz + zc - 1) / zc;
            long long ws[3];
            for (int d = 0; d < 3; ++d) {
                const int gi = P.iso ? 0 : d;
                ws[d] = (long long) (P.wm[gi] << (64 - P.wshift[gi]));
            }
            axis3d_fxtma_kernel<<<dim3(ftx * fty, zch), FT_THREADS, 0, ctx->stream>>>(map, in, out, box, P.iso, ws[0], ws[1], ws[2], zc, ftx);
            OPG_LAUNCHED();
            return check_launch("axis3d_fxtma_kernel");
        }
    }
    const int mode = (first ? 1 : 0) | (last ? 2 : 0);
    auto go = [&](auto rb_tag) {
        constexpr int R = decltype(rb_tag)::value;
        switch (mode) {
            case 0: axis3d_fxres_kernel<0, R><<<g, b, 0, ctx->stream>>>(in, out, box, P, ws[0], ws[1], ws[2], maxslots, zchunk, tiles_x, tiles_y); break;
            case 1: axis3d_fxres_kernel<1, R><<<g, b, 0, ctx->stream>>>(in, out, box, P, ws[0], ws[1], ws[2], maxslots, zchunk, tiles_x, tiles_y); break;
            case 2: axis3d_fxres_kernel<2, R><<<g, b, 0, ctx->stream>>>(in, out, box, P, ws[0], ws[1], ws[2], maxslots, zchunk, tiles_x, tiles_y); break;
            default: axis3d_fxres_kernel<3, R><<<g, b, 0, ctx->stream>>>(in, out, box, P, ws[0], ws[1], ws[2], maxslots, zchunk, tiles_x, tiles_y); break;
        }
    };
    if (rbx == 4) go(std::integral_constant<int, 4>{});
    else if (rbx == 8) go(std::integral_constant<int, 8>{});
    else go(std::integral_constant<int, 6>{});
    OPG_LAUNCHED();
    return check_launch("axis3d_fxres_kernel");
}

// 3D tiling: register-blocked warps (the measured default for the fixed-point mode: integer-issue
// bound, gains from the absent barriers) or shared-memory tiles (the default for the exact mode:
// float64-pipe bound).  Both give the same values; the tuner times the two on the first launch of a
// (mode, box, stencil) key (a repeated launch rewrites `out` and the max slot with the same values),
// and OPFLOW_AXIS_TILING=register|smem overrides it, read at every launch.
static int axis_launch_tiling(opflow_ctx ctx, const FieldView& in, const FieldView& out, const Box& box, const AxisParams& P, bool fast,
                              unsigned long long* maxslots, int step, bool reg);

static bool use_register_tiles(opflow_ctx ctx, const FieldView& in, const FieldView& out, const Box& box, const AxisParams& P, bool fast,
                               unsigned long long* maxslots, int step) {
    const char* e = getenv("OPFLOW_AXIS_TILING");
    if (e && strcmp(e, "smem") == 0) return false;
    if (e && strcmp(e, "register") == 0) return true;
    if (!tune_enabled()) return fast;
    unsigned long long h = tune_hash(&P.ndim, sizeof P.ndim);
    h = tune_hash(P.h, sizeof P.h, h);
    h = tune_hash(P.inv_h, sizeof P.inv_h, h);
    h = tune_hash(P.pow2, sizeof P.pow2, h);
    h = tune_hash(P.order, sizeof P.order, h);
    h = tune_hash(&P.s, sizeof P.s, h);
    h = tune_hash(&P.iso, sizeof P.iso, h);
    h = tune_hash(P.wm, sizeof P.wm, h);
    h = tune_hash(P.wshift, sizeof P.wshift, h);
    h = tune_hash(P.wneg, sizeof P.wneg, h);
    h = tune_hash(&P.bound_bits, sizeof P.bound_bits, h);
    char key[160];
    std::snprintf(key, sizeof key, "axis3d/%s/%dx%dx%d/%016llx", fast ? "fixed" : "exact", box.hi[0] - box.lo[0], box.hi[1] - box.lo[1],
                  box.hi[2] - box.lo[2], h);
    const std::vector<int> cands = fast ? std::vector<int>{1, 0} : std::vector<int>{0, 1};
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(ctx->stream, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) return tune_cached(key, cands) == 1;
    return tune_pick(key, cands, [&](int reg) {
        cudaEvent_t e0 = nullptr, e1 = nullptr;
        float ms = -1.f;
        if (cudaEventCreate(&e0) == cudaSuccess && cudaEventCreate(&e1) == cudaSuccess &&
            axis_launch_tiling(ctx, in, out, box, P, fast, maxslots, step, reg) == OPFLOW_OK && cudaEventRecord(e0, ctx->stream) == cudaSuccess &&
            axis_launch_tiling(ctx, in, out, box, P, fast, maxslots, step, reg) == OPFLOW_OK && cudaEventRecord(e1, ctx->stream) == cudaSuccess &&
            cudaEventSynchronize(e1) == cudaSuccess)
            cudaEventElapsedTime(&ms, e0, e1);
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
        return ms;
    }) == 1;
}

int axis_launch(opflow_ctx ctx, const FieldView& in, const FieldView& out, const Box& box, const AxisParams& P, bool fast,
                unsigned long long* maxslots, int step) {
    const int nx = box.hi[0] - box.lo[0], ny = box.hi[1] - box.lo[1], nz = box.hi[2] - box.lo[2];
    if (nx <= 0 || ny <= 0 || nz <= 0) return OPFLOW_OK;
    const bool reg = P.ndim == 3 && use_register_tiles(ctx, in, out, box, P, fast, maxslots, step);
    return axis_launch_tiling(ctx, in, out, box, P, fast, maxslots, step, reg);
}

static int axis_launch_tiling(opflow_ctx ctx, const FieldView& in, const FieldView& out, const Box& box, const AxisParams& P, bool fast,
                              unsigned long long* maxslots, int step, bool reg) {
    const int nx = box.hi[0] - box.lo[0], ny = box.hi[1] - box.lo[1], nz = box.hi[2] - box.lo[2];
    if (P.ndim == 3 && reg) {
        const int tiles_x = (nx + RB_COLS - 1) / RB_COLS, tiles_y = (ny + RB - 1) / RB;
        const int bx = (tiles_x * tiles_y + RB_WARPS - 1) / RB_WARPS;
        int zchunks = (ctx->num_sms * 6 + bx - 1) / bx;
        zchunks = std::max(1, std::min(zchunks, (nz + 15) / 16));
        const int zchunk = (nz + zchunks - 1) / zchunks;
        zchunks = (nz + zchunk - 1) / zchunk;
        dim3 g(bx, zchunks), b(32 * RB_WARPS);
        if (fast) axis3d_rb_kernel<true><<<g, b, 0, ctx->stream>>>(in, out, box, P, maxslots, step, zchunk, tiles_x, tiles_y);
        else axis3d_rb_kernel<false><<<g, b, 0, ctx->stream>>>(in, out, box, P, maxslots, step, zchunk, tiles_x, tiles_y);
        OPG_LAUNCHED();
        return check_launch("axis3d_rb_kernel");
    }
    if (P.ndim == 3) {
        const int bx = (nx + TX - 1) / TX, by = (ny + TY - 1) / TY;
        // enough CTAs for ~8 per SM, each marching at least 16 planes
        int zchunks = (ctx->num_sms * 8 + bx * by - 1) / (bx * by);
        zchunks = std::max(1, std::min(zchunks, (nz + 15) / 16));
        const int zchunk = (nz + zchunks - 1) / zchunks;
        zchunks = (nz + zchunk - 1) / zchunk;
        dim3 g(bx, by, zchunks), b(TX, TY);
        if (fast) axis3d_kernel<true><<<g, b, 0, ctx->stream>>>(in, out, box, P, maxslots, step, zchunk);
        else axis3d_kernel<false><<<g, b, 0, ctx->stream>>>(in, out, box, P, maxslots, step, zchunk);
        OPG_LAUNCHED();
        return check_launch("axis3d_kernel");
    }
    if (P.ndim == 2) {
        const int bx = (nx + TX2 - 1) / TX2;
        int ychunks = (ctx->num_sms * 8 + bx - 1) / bx;
        ychunks = std::max(1, std::min(ychunks, (ny + 7) / 8));
        const int ychunk = (ny + ychunks - 1) / ychunks;
        ychunks = (ny + ychunk - 1) / ychunk;
        dim3 g(bx, ychunks), b(TX2);
        if (fast) axis2d_kernel<true><<<g, b, 0, ctx->stream>>>(in, out, box, P, maxslots, step, ychunk);
        else axis2d_kernel<false><<<g, b, 0, ctx->stream>>>(in, out, box, P, maxslots, step, ychunk);
        OPG_LAUNCHED();
        return check_launch("axis2d_kernel");
    }
    return fail(OPFLOW_E_UNSUPPORTED, "tiled stencil kernels cover 2D and 3D grids");
}

}  // namespace opg
