// Multigrid V-cycle and flexible-PCG kernels over chunk lists.
//
// Every kernel walks a list of row segments ("chunks") that may belong to many problems and levels, so
// one launch serves a single solve or a batch of uneven problems alike (a persistent grid strides over
// the list).  Inner products are formed per chunk inside one CTA in a fixed order and then reduced per
// problem in a fixed order, so a problem's iterates are bit-identical whether it runs alone or in a
// batch.  T selects the precision of the V-cycle (float for the mixed form, double for the plain one);
// the Krylov vectors, their updates and all inner products are float64.
#include "mg_device.h"
#include "tma.h"

#include <cstdlib>
#include <type_traits>

namespace opg {

// ---- chunked kernels (large levels)
// A chunk is one row segment (nrows == 1: the CTA's threads stride along it) or several whole rows of
// one plane (one warp per row, lanes along the row), so short rows still fill the CTA.  `color` >= 0
// visits only the cells of that red-black color.
template <typename F>
__device__ __forceinline__ void chunk_cells(const Chunk& C, int color, F&& f) {
    if (C.nrows == 1) {
        if (color < 0) {
            for (int t = threadIdx.x; t < C.cnt; t += blockDim.x) f(C.i0 + t, C.j);
        } else {
            const int first = (C.i0 + C.j + C.k + color) & 1;
            for (int t = 2 * threadIdx.x + first; t < C.cnt; t += 2 * blockDim.x) f(C.i0 + t, C.j);
        }
        return;
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    for (int r = warp; r < C.nrows; r += nw) {
        const int j = C.j + r;
        if (color < 0) {
            for (int t = lane; t < C.cnt; t += 32) f(C.i0 + t, j);
        } else {
            const int first = (C.i0 + j + C.k + color) & 1;
            for (int t = first + 2 * lane; t < C.cnt; t += 64) f(C.i0 + t, j);
        }
    }
}

template <typename T>
__global__ void __launch_bounds__(256, 4) mg_residual(const LvlDev* __restrict__ Ls, const Chunk* __restrict__ ch, int nch, const Scal* sc) {
    for (int c = blockIdx.x; c < nch; c += gridDim.x) {
        const Chunk C = ch[c];
        if (!active(Ls, C, sc)) continue;
        const LvlDev& L = Ls[C.lvl];
        chunk_cells(C, -1, [&](int i, int j) { cell_residual<T>(L, i, j, C.k); });
    }
}

// Red-black Gauss-Seidel half sweep (cells with (i+j+k)%2 == color), or for Jacobi levels:
// color 0 computes r = b - A x, color 1 applies x += omega r / diag.
template <typename T>
__global__ void __launch_bounds__(256, 4) mg_smooth(const LvlDev* __restrict__ Ls, const Chunk* __restrict__ ch, int nch, int color, const Scal* sc) {
    for (int c = blockIdx.x; c < nch; c += gridDim.x) {
        const Chunk C = ch[c];
        if (!active(Ls, C, sc)) continue;
        const LvlDev& L = Ls[C.lvl];
        if (L.rbgs) chunk_cells(C, color, [&](int i, int j) { cell_gs<T>(L, i, j, C.k); });
        else chunk_cells(C, -1, [&](int i, int j) { cell_jacobi<T>(L, i, j, C.k, color); });
    }
}

// Cells of a z tile that take the general per-cell path (boundary faces), queued during the march and
// updated by the whole CTA after it: a boundary column would otherwise hold its warp for every plane
// of the tile.  Deferring them is exact for the three z kernels: a half sweep's cells only read cells
// of the other colour, and the residual and prolongation write nothing they read.
struct ZQueue {
    unsigned n;
    unsigned short cell[MG_ZT_X * MG_ZT_Y * MG_ZT_Z];  // (plane offset << 8) | (row << 5) | lane
};
static_assert(MG_ZT_Y <= 8 && MG_ZT_Z <= 256, "queue entries hold the row in 3 bits and the plane offset in 8");

__device__ __forceinline__ void zq_push(ZQueue& Q, unsigned planes, int koff, int warp, int lane) {
    if (!planes) return;
    unsigned slot = atomicAdd(&Q.n, (unsigned) __popc(planes));
    for (; planes; planes &= planes - 1) Q.cell[slot++] = (unsigned short) (((koff + __ffs(planes) - 1) << 8) | (warp << 5) | lane);
}

// after the march: every thread of the CTA takes queued cells; leaves the queue empty (x of lane 0 of a
// queued cell: C.i0 + x0)
template <typename F>
__device__ __forceinline__ void zq_drain(ZQueue& Q, const Chunk& C, F&& fn, int x0 = -1) {
    __syncthreads();
    const unsigned n = Q.n;
    __syncthreads();
    if (threadIdx.x == 0) Q.n = 0;
    for (unsigned e = threadIdx.x; e < n; e += blockDim.x) {
        const unsigned v = Q.cell[e];
        fn(C.i0 + x0 + (int) (v & 31), C.j + (int) ((v >> 5) & 7), C.k + (int) (v >> 8));
    }
    __syncthreads();
}

// Red-black Gauss-Seidel half sweep of a 3D class-table level, marching along z: a CTA owns a tile of
// MG_ZT_X computed x-columns (lanes 1..30 of each warp; lanes 0 and 31 only hold the neighbouring
// columns) by MG_ZT_Y rows (one warp each) and a run of planes.  Each thread walks its column upward
// in batches of ZB planes: it first issues every load of the batch (x at the next ZB planes, and b and
// the two y-neighbours of the cells it updates), then updates the batch's cells with the x-neighbours
// taken from the adjacent lanes, so x is streamed once per half sweep with ZB planes of loads in
// flight per thread.  The cells of one colour only read cells of the other, so values loaded ahead
// are never stale and the in-place update needs no barrier.  Interior cells use the interior class's
// coefficients with the chunked kernel's operations in its order (bit-identical results); boundary
// cells take the general per-cell path, queued (ZQueue).  (Levels with coefficient arrays stay on the chunked kernel:
// with seven more streams per cell the march was measured slower.)  Tiles: Chunk{lvl, j = y origin,
// k = first plane, i0 = x origin, cnt = MG_ZT_X, nrows = planes}.
template <typename T, int ZB>
__global__ void __launch_bounds__(32 * MG_ZT_Y) mg_smooth_z(const LvlDev* __restrict__ Ls, const Chunk* __restrict__ ch, int nch, int color,
                                                           const Scal* sc) {
    static_assert(ZB % 2 == 0, "every batch starts on the same colour");
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    __shared__ ZQueue Q;
    if (threadIdx.x == 0) Q.n = 0;
    __syncthreads();
    for (int c = blockIdx.x; c < nch; c += gridDim.x) {
        const Chunk C = ch[c];
        if (!active(Ls, C, sc)) continue;
        const LvlDev& L = Ls[C.lvl];
        const int n0 = L.n[0], n1 = L.n[1], n2 = L.n[2];
        const long long sy = n0, sz = (long long) n0 * n1;
        const int i = C.i0 - 1 + lane, j = C.j + warp;
        const bool col_ok = i >= 0 && i < n0 && j < n1;
        const bool computes = col_ok && lane >= 1 && lane <= MG_ZT_X;
        T* x = Sel<T>::x(L);
        const T* b = Sel<T>::b(L);
        const T* t = Sel<T>::Tb(L) + 13 * TSTRIDE;  // the interior class (1 + 3 + 9)
        const T c1 = t[1], c2 = t[2], c3 = t[3], c4 = t[4], c5 = t[5], c6 = t[6], cinv = t[NSLOT];
        const long long col = col_ok ? (long long) i + sy * j : 0;
        const int k0 = C.k, k1 = min(C.k + C.nrows, n2);
        const bool ij_inner = i > 0 && i < n0 - 1 && j > 0 && j < n1 - 1;
        const int p0 = (i + j + k0 + color) & 1;  // 0: the cells at planes k0, k0 + 2, ... are updated
        T* xk = x + col + sz * k0;                // this column at the batch's first plane (dereferenced only where col_ok)
        const T* bk = b + col + sz * k0;
        T xm = (col_ok && k0 > 0) ? xk[-sz] : (T) 0;
        T xc = col_ok ? *xk : (T) 0;
        for (int kb = k0; kb < k1; kb += ZB) {
            T xs[ZB + 2], bv[ZB], ys[ZB], yn[ZB];  // xs[q + 1]: x at plane kb + q
            unsigned general = 0;                  // planes of the batch whose cell takes the per-cell path
            xs[0] = xm;
            xs[1] = xc;
#pragma unroll
            for (int q = 0; q < ZB; ++q) {
                const int k = kb + q;
                const bool upd = computes && k < k1 && ((q + p0) & 1) == 0;
                xs[q + 2] = (col_ok && k + 1 < n2) ? xk[(q + 1) * sz] : (T) 0;
                bv[q] = upd ? bk[q * sz] : (T) 0;
                ys[q] = (upd && ij_inner) ? xk[q * sz - sy] : (T) 0;
                yn[q] = (upd && ij_inner) ? xk[q * sz + sy] : (T) 0;
            }
#pragma unroll
            for (int q = 0; q < ZB; ++q) {
                const int k = kb + q;
                const T xw = __shfl_up_sync(0xffffffffu, xs[q + 1], 1), xe = __shfl_down_sync(0xffffffffu, xs[q + 1], 1);
                if (computes && k < k1 && ((q + p0) & 1) == 0) {
                    if (ij_inner && k > 0 && k < n2 - 1) {
                        T acc = 0;
                        acc += c1 * xw;
                        acc += c2 * xe;
                        acc += c3 * ys[q];
                        acc += c4 * yn[q];
                        acc += c5 * xs[q];
                        acc += c6 * xs[q + 2];
                        xk[q * sz] = (bv[q] - acc) * cinv;
                    } else {
                        general |= 1u << q;
                    }
                }
            }
            zq_push(Q, general, kb - k0, warp, lane);
            xm = xs[ZB];
            xc = xs[ZB + 1];
            xk += ZB * sz;
            bk += ZB * sz;
        }
        zq_drain(Q, C, [&](int ci, int cj, int ck) { cell_gs<T>(L, ci, cj, ck); });
    }
}

// r = b - A x over the z-marching tiles of a 3D class-table level (every cell; the same batches,
// register window and lane shuffles as mg_smooth_z, and cell_residual's operations in its order)
template <typename T, int ZB>
__global__ void __launch_bounds__(32 * MG_ZT_Y) mg_residual_z(const LvlDev* __restrict__ Ls, const Chunk* __restrict__ ch, int nch, const Scal* sc) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    __shared__ ZQueue Q;
    if (threadIdx.x == 0) Q.n = 0;
    __syncthreads();
    for (int c = blockIdx.x; c < nch; c += gridDim.x) {
        const Chunk C = ch[c];
        if (!active(Ls, C, sc)) continue;
        const LvlDev& L = Ls[C.lvl];
        const int n0 = L.n[0], n1 = L.n[1], n2 = L.n[2];
        const long long sy = n0, sz = (long long) n0 * n1;
        const int i = C.i0 - 1 + lane, j = C.j + warp;
        const bool col_ok = i >= 0 && i < n0 && j < n1;
        const bool computes = col_ok && lane >= 1 && lane <= MG_ZT_X;
        const T* t = Sel<T>::Tb(L) + 13 * TSTRIDE;
        const T c0 = t[0], c1 = t[1], c2 = t[2], c3 = t[3], c4 = t[4], c5 = t[5], c6 = t[6];
        const long long col = col_ok ? (long long) i + sy * j : 0;
        const int k0 = C.k, k1 = min(C.k + C.nrows, n2);
        const bool ij_inner = i > 0 && i < n0 - 1 && j > 0 && j < n1 - 1;
        const T* xk = Sel<T>::x(L) + col + sz * k0;
        const T* bk = Sel<T>::b(L) + col + sz * k0;
        T* rk = Sel<T>::r(L) + col + sz * k0;
        T xm = (col_ok && k0 > 0) ? xk[-sz] : (T) 0;
        T xc = col_ok ? *xk : (T) 0;
        for (int kb = k0; kb < k1; kb += ZB) {
            T xs[ZB + 2], bv[ZB], ys[ZB], yn[ZB];
            unsigned general = 0;
            xs[0] = xm;
            xs[1] = xc;
#pragma unroll
            for (int q = 0; q < ZB; ++q) {
                const int k = kb + q;
                const bool in = computes && k < k1;
                xs[q + 2] = (col_ok && k + 1 < n2) ? xk[(q + 1) * sz] : (T) 0;
                bv[q] = in ? bk[q * sz] : (T) 0;
                ys[q] = (in && ij_inner) ? xk[q * sz - sy] : (T) 0;
                yn[q] = (in && ij_inner) ? xk[q * sz + sy] : (T) 0;
            }
#pragma unroll
            for (int q = 0; q < ZB; ++q) {
                const int k = kb + q;
                const T xw = __shfl_up_sync(0xffffffffu, xs[q + 1], 1), xe = __shfl_down_sync(0xffffffffu, xs[q + 1], 1);
                if (computes && k < k1) {
                    if (ij_inner && k > 0 && k < n2 - 1) {
                        T acc = 0;
                        acc += c1 * xw;
                        acc += c2 * xe;
                        acc += c3 * ys[q];
                        acc += c4 * yn[q];
                        acc += c5 * xs[q];
                        acc += c6 * xs[q + 2];
                        rk[q * sz] = bv[q] - (c0 * xs[q + 1] + acc);
                    } else {
                        general |= 1u << q;
                    }
                }
            }
            zq_push(Q, general, kb - k0, warp, lane);
            xm = xs[ZB];
            xc = xs[ZB + 1];
            xk += ZB * sz;
            bk += ZB * sz;
            rk += ZB * sz;
        }
        zq_drain(Q, C, [&](int ci, int cj, int ck) { cell_residual<T>(L, ci, cj, ck); });
    }
}

// x += P x_coarse over the z-marching tiles of a 3D level whose coarse level is cell-centred: each
// thread walks its fine column upward, ZB fine planes (ZB / 2 coarse planes) per batch.  Fine plane
// 2K + e interpolates coarse planes K and K - 1 + 2e, so a batch reads coarse planes K0 - 1 .. K0 + ZB/2
// of which the first two come from the previous batch: each coarse value a thread needs is loaded once
// per tile instead of once per fine cell.  Interior cells sum the eight trilinear terms in
// prolong_acc's order and weights (bit-identical to the chunked kernel); cells with a coarse
// neighbour outside the box take cell_prolong (queued).  Levels whose coarse level is node-centred are
// skipped here (they stay on the chunked kernel).  Tiles start at even planes.
template <typename T, int ZB>
__global__ void __launch_bounds__(32 * MG_ZT_Y) mg_prolong_z(const LvlDev* __restrict__ Ls, const Chunk* __restrict__ ch, int nch, const Scal* sc) {
    static_assert(ZB % 2 == 0, "whole coarse planes per batch");
    constexpr bool FAST = std::is_same<T, float>::value;  // the chunked kernel's instance
    constexpr int NP = ZB / 2 + 2;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    __shared__ ZQueue Q;
    if (threadIdx.x == 0) Q.n = 0;
    __syncthreads();
    for (int c = blockIdx.x; c < nch; c += gridDim.x) {
        const Chunk C = ch[c];
        if (!active(Ls, C, sc)) continue;
        const LvlDev& L = Ls[C.lvl];
        const LvlDev& Lc = Ls[L.coarse];
        const int n0 = L.n[0], n1 = L.n[1], n2 = L.n[2];
        const long long sy = n0, sz = (long long) n0 * n1;
        const int i = C.i0 - 1 + lane, j = C.j + warp;
        const bool computes = i >= 0 && i < n0 && j < n1 && lane >= 1 && lane <= MG_ZT_X;
        const int k0 = C.k, k1 = min(C.k + C.nrows, n2);
        if (Lc.node || (k0 & 1)) continue;  // node-centred levels take the chunked kernel; tiles start at even planes
        const int nc0 = Lc.n[0], nc1 = Lc.n[1], nc2 = Lc.n[2];
        const int I0 = i >> 1, J0 = (i & 1) ? I0 + 1 : I0 - 1;
        const int I1 = j >> 1, J1 = (j & 1) ? I1 + 1 : I1 - 1;
        const bool in_xy = computes && I0 < nc0 && J0 >= 0 && J0 < nc0 && I1 < nc1 && J1 >= 0 && J1 < nc1;
        const long long csz = (long long) nc0 * nc1;
        // the four coarse columns, in prolong_acc's order (x fastest, then y)
        const long long o0 = in_xy ? I0 + (long long) nc0 * I1 : 0, o1 = in_xy ? J0 + (long long) nc0 * I1 : 0;
        const long long o2 = in_xy ? I0 + (long long) nc0 * J1 : 0, o3 = in_xy ? J0 + (long long) nc0 * J1 : 0;
        const T* xcr = Sel<T>::x(Lc);
        T cv[NP][4];  // cv[p]: coarse plane K0 - 1 + p of the current batch
        auto load_plane = [&](int K, T* v) {
            const bool ok = in_xy && K >= 0 && K < nc2;
            const T* pl = xcr + csz * (ok ? K : 0);
            v[0] = ok ? pl[o0] : (T) 0;
            v[1] = ok ? pl[o1] : (T) 0;
            v[2] = ok ? pl[o2] : (T) 0;
            v[3] = ok ? pl[o3] : (T) 0;
        };
        load_plane((k0 >> 1) - 1, cv[0]);
        load_plane(k0 >> 1, cv[1]);
        T* xf = Sel<T>::x(L) + (computes ? (long long) i + sy * j : 0) + sz * k0;
        const T w[2] = {(T) 0.75, (T) 0.25};
        for (int kb = k0; kb < k1; kb += ZB) {
            const int K0 = kb >> 1;
#pragma unroll
            for (int p = 2; p < NP; ++p) load_plane(K0 + p - 1, cv[p]);
            T xv[ZB];
            unsigned general = 0;
#pragma unroll
            for (int q = 0; q < ZB; ++q) xv[q] = (computes && kb + q < k1) ? xf[q * sz] : (T) 0;
#pragma unroll
            for (int q = 0; q < ZB; ++q) {
                const int k = kb + q;
                if (!computes || k >= k1) continue;
                const int KI = K0 + q / 2, KJ = (q & 1) ? KI + 1 : KI - 1;
                if (in_xy && KI < nc2 && KJ >= 0 && KJ < nc2) {
                    const int pI = q / 2 + 1, pJ = (q & 1) ? pI + 1 : pI - 1;
                    T acc = 0;
#pragma unroll
                    for (int a = 0; a < 2; ++a)
#pragma unroll
                        for (int bb = 0; bb < 2; ++bb)
#pragma unroll
                            for (int e = 0; e < 2; ++e) {
                                const T wt = w[e] * w[bb] * w[a];
                                acc += wt * (T) 1 * cv[a ? pJ : pI][2 * bb + e];
                            }
                    xf[q * sz] = xv[q] + acc;
                } else {
                    general |= 1u << q;
                }
            }
            zq_push(Q, general, kb - k0, warp, lane);
#pragma unroll
            for (int v = 0; v < 4; ++v) {
                cv[0][v] = cv[NP - 2][v];
                cv[1][v] = cv[NP - 1][v];
            }
            xf += ZB * sz;
        }
        zq_drain(Q, C, [&](int ci, int cj, int ck) { cell_prolong<T, FAST>(Ls, L, ci, cj, ck); });
    }
}

// ---------------------------------------------------------------- TMA-staged z-marching smoother
// set by mg_smooth_zt when one of its bounded mbarrier waits (tma.h) gave up
__device__ int g_mg_err;

// Red-black half sweep of a non-periodic float32 class-table 3D level whose rows hold a multiple of 4
// cells, the planes staged in shared memory by TMA.  A CTA of 256 threads owns MG_ZT2_X x-columns (x
// origin a multiple of MG_ZT2_X) by MG_ZT2_Y rows and a run of planes.  Thread (p, q) = (tid % 32,
// tid / 32) holds the column pair 2p, 2p + 1 of rows 2q, 2q + 1 and updates, on every plane, the cell of
// the colour in each of its two rows, so every thread updates two cells per plane.  One thread streams
// each plane as two tensor-map boxes - x: (MG_ZT2_X + 8) x (MG_ZT2_Y + 2) cells from (x origin - 4,
// y origin - 1), the halo, its x coordinate on a 16-byte boundary; b: MG_ZT2_X x MG_ZT2_Y - into a ring
// of ZT_RING slots; each slot's mbarrier counts both boxes' bytes.  The planes k - 1, k, k + 1 are read
// at step k while k + 2 .. k + 4 are in flight; past step k's barrier the slot of plane k - 2 takes
// plane k + 4.  Updates go straight to global memory: a half sweep reads only the other colour, which
// it never writes.  Interior cells use the interior class's coefficients in the other kernels' operation
// order; cells on the level's faces take their class's coefficients and skip the absent neighbours, as
// the per-cell path (stencil_parts) does, also from shared memory: bit-identical results.
// maps[2 * level] and maps[2 * level + 1] are the level's x and b maps.
constexpr int ZT_RING = 6, ZT_W = MG_ZT2_X + 8, ZT_H = MG_ZT2_Y + 2;
constexpr int ZT_XSLOT = ((ZT_W * ZT_H * 4 + 127) / 128) * 32;    // floats per x slot (128-byte multiple)
constexpr int ZT_BSLOT = MG_ZT2_X * MG_ZT2_Y;                      // floats per b slot (128-byte multiple)
constexpr unsigned ZT_BYTES = (ZT_W * ZT_H + MG_ZT2_X * MG_ZT2_Y) * 4;  // bytes per plane (both boxes)
struct ZtStage {
    float x[ZT_RING][ZT_XSLOT];
    float b[ZT_RING][ZT_BSLOT];
    float cls[NCLASS * TSTRIDE];  // the tile's level's class table (face cells read their class's row)
    unsigned long long bar[ZT_RING];
};
static_assert(MG_ZT2_X == 64 && MG_ZT2_Y == 16, "the thread layout covers 64 x 16 cells with 256 threads");
static_assert((ZT_BSLOT * 4) % 128 == 0 && (ZT_W * 4) % 16 == 0, "slots on 128-byte boundaries, box rows 16-byte multiples");
constexpr size_t ZT_SMEM = sizeof(ZtStage) + 128;  // (+ alignment of the dynamic shared memory to 128 bytes)
// four CTAs per SM: 4 x (ZT_SMEM + the 1 KB the hardware reserves per CTA) within an SM's 228 KB
static_assert(4 * (ZT_SMEM + 1024) <= 228 * 1024, "four resident CTAs per SM");

__global__ void __launch_bounds__(256) mg_smooth_zt(const LvlDev* __restrict__ Ls, const Chunk* __restrict__ ch, int nch, int color,
                                                   const Scal* sc, const CUtensorMap* __restrict__ maps) {
    extern __shared__ unsigned char zt_raw[];
    ZtStage& St = *reinterpret_cast<ZtStage*>(zt_raw + ((128 - (smem_addr(zt_raw) & 127)) & 127));
    const int px = threadIdx.x & 31, ry = threadIdx.x >> 5;
    if (threadIdx.x == 0) {
        for (int s = 0; s < ZT_RING; ++s) mbar_init(&St.bar[s], 1);
        mbar_fence_init();
    }
    __syncthreads();
    unsigned seq = 0;  // planes issued by this CTA so far: plane number q uses slot q % ZT_RING, phase (q / ZT_RING) & 1
    for (int c = blockIdx.x; c < nch; c += gridDim.x) {
        const Chunk C = ch[c];
        if (!active(Ls, C, sc)) continue;
        const LvlDev& L = Ls[C.lvl];
        const int n0 = L.n[0], n1 = L.n[1], n2 = L.n[2];
        const long long sy = n0, sz = (long long) n0 * n1;
        const int i0 = C.i0, j0 = C.j, k0 = C.k, k1 = min(C.k + C.nrows, n2);
        float* x = L.x32;
        const float* t = L.T32 + 13 * TSTRIDE;
        const float c1 = t[1], c2 = t[2], c3 = t[3], c4 = t[4], c5 = t[5], c6 = t[6], cinv = t[NSLOT];
        for (int e = threadIdx.x; e < NCLASS * TSTRIDE; e += blockDim.x) St.cls[e] = L.T32[e];  // (read after the first step's barrier)
        const CUtensorMap* mx = maps + 2 * C.lvl;
        const CUtensorMap* mb = mx + 1;
        const unsigned base = seq;  // plane k0 - 1 is plane number base
        const int last = k1;        // planes k0 - 1 .. k1 are read
        auto slot_of = [&](int p) { return (int) ((base + (unsigned) (p - k0 + 1)) % ZT_RING); };
        auto phase_of = [&](int p) { return ((base + (unsigned) (p - k0 + 1)) / ZT_RING) & 1u; };
        const bool producer = threadIdx.x == 0;
        auto issue = [&](int p) {  // the producer thread: plane p's two boxes into its slot
            const int s = slot_of(p);
            mbar_arrive_expect(&St.bar[s], ZT_BYTES);
            tma_load_3d(&St.x[s][0], mx, i0 - 4, j0 - 1, p, &St.bar[s]);
            tma_load_3d(&St.b[s][0], mb, i0, j0, p, &St.bar[s]);
        };
        int issued = min(k0 - 1 + ZT_RING - 1, last);  // planes k0 - 1 .. issued fill every slot
        if (producer) {
            tensormap_acquire(mx);
            tensormap_acquire(mb);
            for (int p = k0 - 1; p <= issued; ++p) issue(p);
        }
        bool ok = mbar_wait(&St.bar[slot_of(k0 - 1)], phase_of(k0 - 1));
        ok = ok && mbar_wait(&St.bar[slot_of(k0)], phase_of(k0));
        bool failed = false;
        // the slots of planes k - 1, k, k + 1 and the phase of plane k + 1's fill, advanced step by step
        int sd = slot_of(k0 - 1), sc = slot_of(k0), su = slot_of(k0 + 1);
        unsigned phu = phase_of(k0 + 1);
        // per thread: whether its two candidate columns (even, odd) and its two rows are inside the
        // level's faces, and its rows' global offsets
        const int ia = i0 + 2 * px;
        const bool xin0 = ia > 0 && ia < n0 - 1, xin1 = ia + 1 > 0 && ia + 1 < n0 - 1;
        const bool xok0 = ia < n0, xok1 = ia + 1 < n0;
        float* xrow[2];
        bool yin[2], yok[2];
#pragma unroll
        for (int r = 0; r < 2; ++r) {
            const int j = j0 + 2 * ry + r;
            yin[r] = j > 0 && j < n1 - 1;
            yok[r] = j < n1;
            xrow[r] = x + (long long) k0 * sz + (long long) j * sy + ia;
        }
        for (int k = k0; k < k1; ++k) {
            ok = ok && mbar_wait(&St.bar[su], phu);
            if (__syncthreads_or(!ok)) {  // (the same answer in every thread)
                failed = true;
                break;
            }
            if (k > k0 && issued < last) {  // every thread is past step k - 1: plane k - 2's slot takes plane k + 4
                ++issued;
                if (producer) issue(issued);
            }
            const float* Xd = St.x[sd];
            const float* Xc = St.x[sc];
            const float* Xu = St.x[su];
            const float* Bc = St.b[sc];
            const bool kin = k > 0 && k < n2 - 1;
#pragma unroll
            for (int r = 0; r < 2; ++r) {
                const int ly = 2 * ry + r, j = j0 + ly;
                const int e = (j + k + color) & 1;  // the colour's column of the pair (i0 is even)
                const int lx = 2 * px + e, i = ia + e;
                if ((e ? xok1 : xok0) && yok[r]) {
                    const int at = (ly + 1) * ZT_W + lx + 4;
                    const float bv = Bc[ly * MG_ZT2_X + lx];
                    float v;
                    if ((e ? xin1 : xin0) && yin[r] && kin) {
                        float acc = 0;
                        acc += c1 * Xc[at - 1];
                        acc += c2 * Xc[at + 1];
                        acc += c3 * Xc[at - ZT_W];
                        acc += c4 * Xc[at + ZT_W];
                        acc += c5 * Xd[at];
                        acc += c6 * Xu[at];
                        v = (bv - acc) * cinv;
                    } else {
                        // a face cell: its class's coefficients, the neighbours inside the level only
                        const float* tc = St.cls + (pos_class(i, n0) + 3 * pos_class(j, n1) + 9 * pos_class(k, n2)) * TSTRIDE;
                        float acc = 0;
                        if (i > 0) acc += tc[1] * Xc[at - 1];
                        if (i < n0 - 1) acc += tc[2] * Xc[at + 1];
                        if (j > 0) acc += tc[3] * Xc[at - ZT_W];
                        if (j < n1 - 1) acc += tc[4] * Xc[at + ZT_W];
                        if (k > 0) acc += tc[5] * Xd[at];
                        if (k < n2 - 1) acc += tc[6] * Xu[at];
                        v = (bv - acc) * tc[NSLOT];
                    }
                    xrow[r][e] = v;
                }
                xrow[r] += sz;
            }
            sd = sc;
            sc = su;
            if (++su == ZT_RING) {
                su = 0;
                phu ^= 1u;
            }
        }
        seq = base + (unsigned) (last - k0 + 2);
        if (failed) {
            // a copy never completed: record it, wait (bounded) for the last copy of each slot, stop
            for (int p = max(k0 - 1, issued - ZT_RING + 1); p <= issued; ++p) mbar_wait(&St.bar[slot_of(p)], phase_of(p));
            if (threadIdx.x == 0) atomicExch(&g_mg_err, 1);
            return;
        }
        __syncthreads();  // every thread is past the tile's last step before the next tile's planes refill the ring
    }
}

// coarse b = R r_fine, coarse x = 0; chunks are coarse rows
template <typename T>
__global__ void __launch_bounds__(256) mg_restrict(const LvlDev* __restrict__ Ls, const Chunk* __restrict__ ch, int nch, const Scal* sc) {
    for (int c = blockIdx.x; c < nch; c += gridDim.x) {
        const Chunk C = ch[c];
        if (!active(Ls, C, sc)) continue;
        const LvlDev& Lc = Ls[C.lvl];
        chunk_cells(C, -1, [&](int i, int j) { cell_restrict<T>(Ls, Lc, i, j, C.k); });
    }
}

// fine x += P x_coarse; chunks are fine rows
template <typename T>
__global__ void __launch_bounds__(256) mg_prolong(const LvlDev* __restrict__ Ls, const Chunk* __restrict__ ch, int nch, const Scal* sc) {
    for (int c = blockIdx.x; c < nch; c += gridDim.x) {
        const Chunk C = ch[c];
        if (!active(Ls, C, sc)) continue;
        const LvlDev& Lf = Ls[C.lvl];
        chunk_cells(C, -1, [&](int i, int j) { cell_prolong<T, std::is_same<T, float>::value>(Ls, Lf, i, j, C.k); });
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
// Walks every cell of level L (for a red-black color only the cells of that color): warps take rows,
// lanes take columns, so no thread divides a cell index.
template <typename T, typename F>
__device__ __forceinline__ void for_cells(const LvlDev& L, int color, F&& f) {
    const int n0 = L.n[0], n1 = L.n[1], rows = L.n[1] * L.n[2];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    for (int row = warp; row < rows; row += nw) {
        const int j = row % n1, k = row / n1;
        if (color < 0) {
            for (int i = lane; i < n0; i += 32) f(i, j, k);
        } else {
            for (int i = ((j + k + color) & 1) + 2 * lane; i < n0; i += 64) f(i, j, k);
        }
    }
}

template <typename T>
__device__ __forceinline__ void bottom_smooth(const LvlDev& L, int color) {
    if (L.rbgs) for_cells<T>(L, color, [&](int i, int j, int k) { cell_gs<T>(L, i, j, k); });
    else for_cells<T>(L, -1, [&](int i, int j, int k) { cell_jacobi<T>(L, i, j, k, color); });
    __syncthreads();
}

// Points the level's V-cycle vectors (of precision T) at x, b, r.
template <typename T>
__device__ __forceinline__ void set_vectors(LvlDev& L, T* x, T* b, T* r);
template <>
__device__ __forceinline__ void set_vectors<float>(LvlDev& L, float* x, float* b, float* r) {
    L.x32 = x;
    L.b32 = b;
    L.r32 = r;
}
template <>
__device__ __forceinline__ void set_vectors<double>(LvlDev& L, double* x, double* b, double* r) {
    L.x64 = x;
    L.b64 = b;
    L.r64 = r;
}

// The V-cycle below (and including) a problem's first small level, one CTA per problem, with the
// levels' x, b and r in shared memory: the restriction into that level (unless a tiled finer level
// did it), pre-smoothing, residuals and restrictions down to the coarsest level, the coarsest solve,
// then prolongation and post-smoothing back up - the chunked kernels' operations in their order, with
// a CTA barrier where those have a launch boundary - and the first level's x written back.
template <typename T>
__global__ void __launch_bounds__(512) mg_bottom(const LvlDev* __restrict__ Ls, const int* __restrict__ top, int ntop, const Scal* sc, int pre,
                                                 int post) {
    extern __shared__ __align__(16) unsigned char bottom_smem[];
    __shared__ LvlDev Lsm[MG_BOTTOM_LEVELS];
    for (int q = blockIdx.x; q < ntop; q += gridDim.x) {
        const int s = top[q];
        if (sc && !sc[Ls[s].problem].active) continue;
        if (Ls[s].fine >= 0 && !Ls[Ls[s].fine].tiled) {  // a tiled finer level restricted into s already
            const LvlDev& L = Ls[s];
            for_cells<T>(L, -1, [&](int i, int j, int k) { cell_restrict<T>(Ls, L, i, j, k); });
            __syncthreads();
        }
        if (threadIdx.x == 0) {
            T* p = (T*) bottom_smem;
            int l = s;
            for (int i = 0; i < MG_BOTTOM_LEVELS; ++i) {
                Lsm[i] = Ls[l];
                Lsm[i].fine = i - 1;
                Lsm[i].coarse = Ls[l].coarsest ? -1 : i + 1;
                const long long N = Ls[l].N;
                set_vectors<T>(Lsm[i], p, p + N, p + 2 * N);
                p += 3 * N;
                if (Ls[l].coarsest) break;
                l = Ls[l].coarse;
            }
        }
        __syncthreads();
        {
            const T* bg = Sel<T>::b(Ls[s]);
            T* bs = Sel<T>::b(Lsm[0]);
            T* xs = Sel<T>::x(Lsm[0]);
            for (int c = threadIdx.x; c < (int) Lsm[0].N; c += blockDim.x) {
                bs[c] = bg[c];
                xs[c] = 0;
            }
        }
        __syncthreads();
        int l = 0;
        while (!Lsm[l].coarsest) {
            const LvlDev& L = Lsm[l];
            for (int it = 0; it < pre; ++it) {
                bottom_smooth<T>(L, 0);
                bottom_smooth<T>(L, 1);
            }
            for_cells<T>(L, -1, [&](int i, int j, int k) { cell_residual<T>(L, i, j, k); });
            __syncthreads();
            const LvlDev& Lc = Lsm[L.coarse];
            for_cells<T>(Lc, -1, [&](int i, int j, int k) { cell_restrict<T>(Lsm, Lc, i, j, k); });
            __syncthreads();
            l = L.coarse;
        }
        {
            const LvlDev& L = Lsm[l];
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
        while (l != 0) {
            const LvlDev& Lf = Lsm[Lsm[l].fine];
            for_cells<T>(Lf, -1, [&](int i, int j, int k) { cell_prolong<T>(Lsm, Lf, i, j, k); });
            __syncthreads();
            for (int it = 0; it < post; ++it) {
                bottom_smooth<T>(Lf, 1);
                bottom_smooth<T>(Lf, 0);
            }
            l = Lsm[l].fine;
        }
        {
            T* xg = Sel<T>::x(Ls[s]);
            const T* xs = Sel<T>::x(Lsm[0]);
            for (int c = threadIdx.x; c < (int) Lsm[0].N; c += blockDim.x) xg[c] = xs[c];
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

// scalar steps: stage 0 after init (bb, rr), 1 after A p (pq -> alpha), 2 after the update (rr ->
// convergence), 3 after the preconditioner (zr, zq -> beta), 4 first preconditioned residual (zr)
__device__ __forceinline__ void scalars_stage(Scal& S, double a, double b, int stage, double tol, int max_iter, int flexible) {
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
    } else if (stage == 4) {
        S.rz = a;
    }
}

// Called by every thread of the CTA after thread 0 has stored chunk c's partials for problem p: the CTA
// that completes the problem's last chunk reduces and applies the scalar stage.
__device__ __forceinline__ void chunk_finish(const Finish& F, int p, const double* partial, double* sh, int* flag) {
    if (!F.done) return;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        const int old = atomicAdd(&F.done[p], 1);
        *flag = old == F.count[p] - 1;
    }
    __syncthreads();
    if (!*flag) return;
    __threadfence();
    const int f0 = F.first[p], n = F.count[p];
    double sums[2];
    for (int s = 0; s < 2; ++s) {
        double v = 0.;
        for (int c = threadIdx.x; c < n; c += blockDim.x) v += __ldcg(&partial[2 * (f0 + c) + s]);
        sums[s] = block_sum(v, sh);
    }
    if (threadIdx.x == 0) {
        F.red[2 * p] = sums[0];
        F.red[2 * p + 1] = sums[1];
        if (F.stage >= 0) scalars_stage(F.sc[p], sums[0], sums[1], F.stage, F.tol, F.max_iter, 1);
        F.done[p] = 0;
    }
}

// mode 0: r = b - A x, partial (b.b, r.r)        mode 1: q = A p, partial (p.q)
// With to_vc (mode 0) the V-cycle's level-0 input is written as well: b = (T) r, x = 0.
// With skip0 (mode 0) the first unknown's r is left out of r.r: the true residual of a pinned system,
// whose first row is the identity with b = 0 (satisfied exactly once the solution is shifted to x[0] = 0).
template <typename T, int mode>
__global__ void __launch_bounds__(256, 4) kr_apply(const LvlDev* __restrict__ Ls, const KrylovDev* __restrict__ K, const Chunk* __restrict__ ch, int nch,
                                                   const Scal* sc, double* partial, int to_vc, Finish F, int skip0) {
    __shared__ double sh[32];
    __shared__ int flag;
    for (int c = blockIdx.x; c < nch; c += gridDim.x) {
        const Chunk C = ch[c];
        const LvlDev& L = Ls[C.lvl];
        const int pb = L.problem;
        const bool act = !sc || sc[pb].active;
        const KrylovDev& Kp = K[pb];
        double s0 = 0., s1 = 0.;
        if (act) {
            const double* __restrict__ in = mode == 0 ? Kp.x : Kp.p;
            const double* __restrict__ bp = Kp.b;
            double* __restrict__ rp = Kp.r;
            double* __restrict__ qp = Kp.q;
            T* __restrict__ vb = Sel<T>::b(L);
            T* __restrict__ vx = Sel<T>::x(L);
            for (int rw = 0; rw < C.nrows; ++rw)
#pragma unroll 2
                for (int t = threadIdx.x; t < C.cnt; t += blockDim.x) {
                    const int i = C.i0 + t, j = C.j + rw;
                    const long long cell = cell_of(L, i, j, C.k);
                    double c0, offd;
                    stencil_parts<double>(L, in, i, j, C.k, cell, c0, offd);
                    const double ax = fma(c0, in[cell], offd);
                    if constexpr (mode == 0) {
                        const double bv = bp[cell];
                        const double r = bv - ax;
                        rp[cell] = r;
                        s0 = fma(bv, bv, s0);
                        if (!(skip0 && cell == 0)) s1 = fma(r, r, s1);
                        if (to_vc) {
                            vb[cell] = (T) r;
                            vx[cell] = 0;
                        }
                    } else {
                        qp[cell] = ax;
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
        chunk_finish(F, pb, partial, sh, &flag);
    }
}

// A chunk whose cells form one contiguous run of an even number of cells from an even cell (full rows
// of a level, or a row segment): the Krylov vector kernels then move two cells per access (16-byte
// float64 and 8-byte float32 pairs; every vector is 256-byte aligned), which keeps twice the bytes in
// flight per instruction on these latency-bound streaming passes.
__device__ __forceinline__ bool chunk_pairs(const LvlDev& L, const Chunk& C, long long& start, long long& n) {
    if (!(C.nrows == 1 || (C.i0 == 0 && C.cnt == L.n[0]))) return false;
    start = cell_of(L, C.i0, C.j, C.k);
    n = (long long) C.cnt * C.nrows;
    return true;
}
// Splits the contiguous run [start, start + n) into an odd head cell (start odd), the aligned pairs
// [a, a + 2 np) and an odd tail cell; single(cell) is called by thread 0 for the head and the last
// thread for the tail, pair(t) for pair t (cells a + 2t, a + 2t + 1) by the CTA's threads.
__device__ __forceinline__ void split_run(long long start, long long n, long long& a, long long& np, long long& head, long long& tail) {
    head = (start & 1) && n > 0 ? start : -1;
    a = start + (head >= 0 ? 1 : 0);
    const long long rest = n - (head >= 0 ? 1 : 0);
    np = rest / 2;
    tail = (rest & 1) ? a + 2 * np : -1;
}
template <typename T>
struct Pair;
template <>
struct Pair<float> {
    using V = float2;
    __device__ static V make(double a, double b) { return make_float2((float) a, (float) b); }
};
template <>
struct Pair<double> {
    using V = double2;
    __device__ static V make(double a, double b) { return make_double2(a, b); }
};

// x += alpha p, r -= alpha q, partial (r.r); the V-cycle's level-0 input b = (T) r, x = 0 alongside
template <typename T>
__global__ void __launch_bounds__(256, 4) kr_update(const LvlDev* __restrict__ Ls, const KrylovDev* __restrict__ K, const Chunk* __restrict__ ch, int nch,
                                                 const Scal* sc, double* partial, Finish F) {
    __shared__ double sh[32];
    __shared__ int flag;
    for (int c = blockIdx.x; c < nch; c += gridDim.x) {
        const Chunk C = ch[c];
        const LvlDev& L = Ls[C.lvl];
        const int pb = L.problem;
        const bool act = sc[pb].active;
        const KrylovDev& Kp = K[pb];
        double s = 0.;
        if (act) {
            const double al = sc[pb].alpha;
            double* __restrict__ xp = Kp.x;
            const double* __restrict__ pp = Kp.p;
            double* __restrict__ rp = Kp.r;
            const double* __restrict__ qp = Kp.q;
            T* __restrict__ vb = Sel<T>::b(L);
            T* __restrict__ vx = Sel<T>::x(L);
            long long st, n;
            if (chunk_pairs(L, C, st, n)) {
                using V = typename Pair<T>::V;
                long long a0, np, head, tail;
                split_run(st, n, a0, np, head, tail);
                auto one = [&](long long cell) {
                    xp[cell] = fma(al, pp[cell], xp[cell]);
                    const double r = fma(-al, qp[cell], rp[cell]);
                    rp[cell] = r;
                    s = fma(r, r, s);
                    vb[cell] = (T) r;
                    vx[cell] = 0;
                };
                if (head >= 0 && threadIdx.x == 0) one(head);
                if (tail >= 0 && threadIdx.x == blockDim.x - 1) one(tail);
                double2* __restrict__ x2 = (double2*) (xp + a0);
                const double2* __restrict__ p2 = (const double2*) (pp + a0);
                double2* __restrict__ r2 = (double2*) (rp + a0);
                const double2* __restrict__ q2 = (const double2*) (qp + a0);
                V* __restrict__ b2 = (V*) (vb + a0);
                V* __restrict__ z2 = (V*) (vx + a0);
#pragma unroll 4
                for (long long t = threadIdx.x; t < np; t += blockDim.x) {
                    double2 xv = x2[t];
                    const double2 pv = p2[t], qv = q2[t];
                    double2 rv = r2[t];
                    xv.x = fma(al, pv.x, xv.x);
                    xv.y = fma(al, pv.y, xv.y);
                    rv.x = fma(-al, qv.x, rv.x);
                    rv.y = fma(-al, qv.y, rv.y);
                    x2[t] = xv;
                    r2[t] = rv;
                    s = fma(rv.x, rv.x, s);
                    s = fma(rv.y, rv.y, s);
                    b2[t] = Pair<T>::make(rv.x, rv.y);
                    z2[t] = Pair<T>::make(0., 0.);
                }
            } else {
                for (int rw = 0; rw < C.nrows; ++rw)
#pragma unroll 4
                    for (int t = threadIdx.x; t < C.cnt; t += blockDim.x) {
                        const long long cell = cell_of(L, C.i0 + t, C.j + rw, C.k);
                        xp[cell] = fma(al, pp[cell], xp[cell]);
                        const double r = fma(-al, qp[cell], rp[cell]);
                        rp[cell] = r;
                        s = fma(r, r, s);
                        vb[cell] = (T) r;
                        vx[cell] = 0;
                    }
            }
        }
        const double a = block_sum(s, sh);
        if (threadIdx.x == 0) { partial[2 * c] = act ? a : 0.; partial[2 * c + 1] = 0.; }
        chunk_finish(F, pb, partial, sh, &flag);
    }
}

// z = V-cycle result (read where it lies, never stored); partial (z.r, z.q)
template <typename T>
__global__ void __launch_bounds__(256, 4) kr_from_vcycle(const LvlDev* __restrict__ Ls, const KrylovDev* __restrict__ K, const Chunk* __restrict__ ch,
                                                      int nch, const Scal* sc, double* partial, Finish F) {
    __shared__ double sh[32];
    __shared__ int flag;
    for (int c = blockIdx.x; c < nch; c += gridDim.x) {
        const Chunk C = ch[c];
        const LvlDev& L = Ls[C.lvl];
        const bool act = !sc || sc[L.problem].active;
        const KrylovDev& Kp = K[L.problem];
        const T* __restrict__ x = Sel<T>::x(L);
        double s0 = 0., s1 = 0.;
        if (act) {
            const double* __restrict__ rp = Kp.r;
            const double* __restrict__ qp = Kp.q;
            long long st, n;
            if (chunk_pairs(L, C, st, n)) {
                using V = typename Pair<T>::V;
                long long a0, np, head, tail;
                split_run(st, n, a0, np, head, tail);
                auto one = [&](long long cell) {
                    const double z = (double) x[cell];
                    s0 = fma(z, rp[cell], s0);
                    s1 = fma(z, qp[cell], s1);
                };
                if (head >= 0 && threadIdx.x == 0) one(head);
                if (tail >= 0 && threadIdx.x == blockDim.x - 1) one(tail);
                const V* __restrict__ z2 = (const V*) (x + a0);
                const double2* __restrict__ r2 = (const double2*) (rp + a0);
                const double2* __restrict__ q2 = (const double2*) (qp + a0);
#pragma unroll 4
                for (long long t = threadIdx.x; t < np; t += blockDim.x) {
                    const V zv = z2[t];
                    const double2 rv = r2[t], qv = q2[t];
                    const double za = (double) zv.x, zb = (double) zv.y;
                    s0 = fma(za, rv.x, s0);
                    s1 = fma(za, qv.x, s1);
                    s0 = fma(zb, rv.y, s0);
                    s1 = fma(zb, qv.y, s1);
                }
            } else {
                for (int rw = 0; rw < C.nrows; ++rw)
#pragma unroll 4
                    for (int t = threadIdx.x; t < C.cnt; t += blockDim.x) {
                        const long long cell = cell_of(L, C.i0 + t, C.j + rw, C.k);
                        const double z = (double) x[cell];
                        s0 = fma(z, rp[cell], s0);
                        s1 = fma(z, qp[cell], s1);
                    }
            }
        }
        const double a = block_sum(s0, sh);
        const double b = block_sum(s1, sh);
        if (threadIdx.x == 0) { partial[2 * c] = act ? a : 0.; partial[2 * c + 1] = act ? b : 0.; }
        chunk_finish(F, L.problem, partial, sh, &flag);
    }
}

// x = 0 for every problem (zero initial guess), one launch for the whole batch
__global__ void __launch_bounds__(256) kr_zero_x(const LvlDev* __restrict__ Ls, const KrylovDev* __restrict__ K, const Chunk* __restrict__ ch, int nch) {
    for (int c = blockIdx.x; c < nch; c += gridDim.x) {
        const Chunk C = ch[c];
        const LvlDev& L = Ls[C.lvl];
        const KrylovDev& Kp = K[L.problem];
        for (int rw = 0; rw < C.nrows; ++rw)
            for (int t = threadIdx.x; t < C.cnt; t += blockDim.x) Kp.x[cell_of(L, C.i0 + t, C.j + rw, C.k)] = 0.;
    }
}

// p = z + beta p with z the V-cycle result (beta = 0 for the first direction)
template <typename T>
__global__ void __launch_bounds__(256) kr_pupdate(const LvlDev* __restrict__ Ls, const KrylovDev* __restrict__ K, const Chunk* __restrict__ ch, int nch,
                                                  const Scal* sc, int first) {
    for (int c = blockIdx.x; c < nch; c += gridDim.x) {
        const Chunk C = ch[c];
        const LvlDev& L = Ls[C.lvl];
        if (!sc[L.problem].active) continue;
        const KrylovDev& Kp = K[L.problem];
        const double be = first ? 0. : sc[L.problem].beta;
        const T* __restrict__ x = Sel<T>::x(L);
        double* __restrict__ pp = Kp.p;
        long long st, n;
        if (chunk_pairs(L, C, st, n)) {
            using V = typename Pair<T>::V;
            long long a0, np, head, tail;
            split_run(st, n, a0, np, head, tail);
            auto one = [&](long long cell) {
                const double z = (double) x[cell];
                pp[cell] = first ? z : fma(be, pp[cell], z);
            };
            if (head >= 0 && threadIdx.x == 0) one(head);
            if (tail >= 0 && threadIdx.x == blockDim.x - 1) one(tail);
            const V* __restrict__ z2 = (const V*) (x + a0);
            double2* __restrict__ p2 = (double2*) (pp + a0);
#pragma unroll 4
            for (long long t = threadIdx.x; t < np; t += blockDim.x) {
                const V zv = z2[t];
                double2 pv;
                if (first) pv = make_double2((double) zv.x, (double) zv.y);
                else {
                    pv = p2[t];
                    pv.x = fma(be, pv.x, (double) zv.x);
                    pv.y = fma(be, pv.y, (double) zv.y);
                }
                p2[t] = pv;
            }
        } else {
            for (int rw = 0; rw < C.nrows; ++rw)
#pragma unroll 4
                for (int t = threadIdx.x; t < C.cnt; t += blockDim.x) {
                    const long long cell = cell_of(L, C.i0 + t, C.j + rw, C.k);
                    const double z = (double) x[cell];
                    pp[cell] = first ? z : fma(be, pp[cell], z);
                }
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

__global__ void kr_scalars(Scal* sc, const double* red, int nprob, int stage, double tol, int max_iter, int flexible) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= nprob) return;
    scalars_stage(sc[p], red[2 * p], red[2 * p + 1], stage, tol, max_iter, flexible);
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
// the z-marching variant: the system's (tuned) choice unless OPFLOW_MG_ZB = 2, 4, 8 (plane batch of the
// register kernels) or 16 (the TMA-staged smoother where a level has its tiles)
int mg_z_batch(int zb) {
    // (read at every call: a process may switch it between solves)
    const char* e = getenv("OPFLOW_MG_ZB");
    const int v = e ? atoi(e) : 0;
    const int forced = v == 2 || v == 4 || v == 8 || v == MG_ZB_TMA ? v : 0;
    return forced ? forced : zb;
}
// the register kernels' plane batch
static int z_batch(int zb) {
    const int v = mg_z_batch(zb);
    return v == 2 || v == 8 ? v : 4;
}
#define OPG_ZB_LAUNCH(KERNEL, T, ...)                                                                   \
    switch (z_batch(zb)) {                                                                             \
        case 2: KERNEL<T, 2><<<grid_of(nch, sms), 32 * MG_ZT_Y, 0, s>>>(__VA_ARGS__); break;           \
        case 8: KERNEL<T, 8><<<grid_of(nch, sms), 32 * MG_ZT_Y, 0, s>>>(__VA_ARGS__); break;           \
        default: KERNEL<T, 4><<<grid_of(nch, sms), 32 * MG_ZT_Y, 0, s>>>(__VA_ARGS__); break;          \
    }
int mg_launch_smooth_z(cudaStream_t s, int sms, bool f32, const LvlDev* L, const Chunk* ch, int nch, int color, const Scal* sc, int zb) {
    if (nch <= 0) return OPFLOW_OK;
    if (f32) { OPG_ZB_LAUNCH(mg_smooth_z, float, L, ch, nch, color, sc) }
    else { OPG_ZB_LAUNCH(mg_smooth_z, double, L, ch, nch, color, sc) }
    OPG_LAUNCHED();
    return check_launch("mg_smooth_z");
}
int mg_launch_residual_z(cudaStream_t s, int sms, bool f32, const LvlDev* L, const Chunk* ch, int nch, const Scal* sc, int zb) {
    if (nch <= 0) return OPFLOW_OK;
    if (f32) { OPG_ZB_LAUNCH(mg_residual_z, float, L, ch, nch, sc) }
    else { OPG_ZB_LAUNCH(mg_residual_z, double, L, ch, nch, sc) }
    OPG_LAUNCHED();
    return check_launch("mg_residual_z");
}
int mg_zt_resident(int sms) {
    static const int per_sm = [] {
        int b = 0;
        if (cudaFuncSetAttribute(mg_smooth_zt, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) ZT_SMEM) != cudaSuccess ||
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, mg_smooth_zt, 256, ZT_SMEM) != cudaSuccess) {
            cudaGetLastError();
            b = 0;
        }
        return std::max(1, b);
    }();
    return per_sm * sms;
}
int mg_launch_smooth_zt(cudaStream_t s, int sms, const LvlDev* L, const Chunk* ch, int nch, int color, const Scal* sc, const CUtensorMap* maps) {
    if (nch <= 0) return OPFLOW_OK;
    mg_smooth_zt<<<std::max(1, std::min(nch, mg_zt_resident(sms))), 256, ZT_SMEM, s>>>(L, ch, nch, color, sc, maps);
    OPG_LAUNCHED();
    return check_launch("mg_smooth_zt");
}
int mg_encode_zt_maps(const LvlDev& D, CUtensorMap* two) {
    const PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
    if (!enc) return fail(OPFLOW_E_UNSUPPORTED, "cuTensorMapEncodeTiled is not available");
    const cuuint64_t dims[3] = {(cuuint64_t) D.n[0], (cuuint64_t) D.n[1], (cuuint64_t) D.n[2]};
    const cuuint64_t strides[2] = {(cuuint64_t) D.n[0] * 4, (cuuint64_t) D.n[0] * D.n[1] * 4};
    const cuuint32_t box_x[3] = {ZT_W, ZT_H, 1}, box_b[3] = {MG_ZT2_X, MG_ZT2_Y, 1}, ones[3] = {1, 1, 1};
    // (the kernel's ring and queue take more than the default 48 KB of dynamic shared memory; set once,
    // outside any stream capture)
    static const bool smem_ok = cudaFuncSetAttribute(mg_smooth_zt, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) ZT_SMEM) == cudaSuccess;
    if (!smem_ok) return fail(OPFLOW_E_UNSUPPORTED, "mg_smooth_zt: %zu bytes of shared memory", ZT_SMEM);
    for (int q = 0; q < 2; ++q) {
        const CUresult r = enc(&two[q], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, q == 0 ? (void*) D.x32 : (void*) D.b32, dims, strides,
                               q == 0 ? box_x : box_b, ones, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                               CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        if (r != CUDA_SUCCESS) return fail(OPFLOW_E_UNSUPPORTED, "tensor map of a %dx%dx%d level: error %d", D.n[0], D.n[1], D.n[2], (int) r);
    }
    return OPFLOW_OK;
}
int mg_take_error(cudaStream_t s, int* err) {
    int zero = 0;
    OPG_CUDA(cudaMemcpyFromSymbolAsync(err, g_mg_err, sizeof(int), 0, cudaMemcpyDeviceToHost, s));
    OPG_CUDA(cudaStreamSynchronize(s));
    if (*err) OPG_CUDA(cudaMemcpyToSymbolAsync(g_mg_err, &zero, sizeof(int), 0, cudaMemcpyHostToDevice, s));
    return OPFLOW_OK;
}
int mg_launch_prolong_z(cudaStream_t s, int sms, bool f32, const LvlDev* L, const Chunk* ch, int nch, const Scal* sc, int zb) {
    if (nch <= 0) return OPFLOW_OK;
    if (f32) { OPG_ZB_LAUNCH(mg_prolong_z, float, L, ch, nch, sc) }
    else { OPG_ZB_LAUNCH(mg_prolong_z, double, L, ch, nch, sc) }
    OPG_LAUNCHED();
    return check_launch("mg_prolong_z");
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
int mg_bottom_prepare() {
    const size_t need[2] = {3 * MG_BOTTOM_CELLS * sizeof(float), 3 * MG_BOTTOM_CELLS * sizeof(double)};
    const void* fn[2] = {(const void*) mg_bottom<float>, (const void*) mg_bottom<double>};
    for (int q = 0; q < 2; ++q) {
        const cudaError_t e = cudaFuncSetAttribute(fn[q], cudaFuncAttributeMaxDynamicSharedMemorySize, (int) need[q]);
        if (e != cudaSuccess) return fail(OPFLOW_E_CUDA, "bottom kernel: shared memory %zu B: %s", need[q], cudaGetErrorString(e));
    }
    return OPFLOW_OK;
}

int mg_launch_bottom(cudaStream_t s, int sms, bool f32, const LvlDev* L, const int* top, int ntop, const Scal* sc, int pre, int post,
                     long long cells) {
    if (ntop <= 0) return OPFLOW_OK;
    if (cells > MG_BOTTOM_CELLS) return fail(OPFLOW_E_INVALID, "bottom levels hold %lld cells (limit %d)", cells, MG_BOTTOM_CELLS);
    const int g = std::min(ntop, sms * 2);
    const size_t smem = (size_t) (3 * cells) * (f32 ? sizeof(float) : sizeof(double));
    if (f32) mg_bottom<float><<<g, 512, smem, s>>>(L, top, ntop, sc, pre, post);
    else mg_bottom<double><<<g, 512, smem, s>>>(L, top, ntop, sc, pre, post);
    OPG_LAUNCHED();
    return check_launch("mg_bottom");
}
int kr_launch_apply(cudaStream_t s, int sms, const LvlDev* L, const KrylovDev* K, const Chunk* ch, int nch, const Scal* sc, double* partial, int mode,
                    const Finish& F, int to_vc, bool f32, bool skip_first) {
    if (nch <= 0) return OPFLOW_OK;
    const int sk = skip_first ? 1 : 0;
    if (mode == 0 && f32) kr_apply<float, 0><<<grid_of(nch, sms), 256, 0, s>>>(L, K, ch, nch, sc, partial, to_vc, F, sk);
    else if (mode == 0) kr_apply<double, 0><<<grid_of(nch, sms), 256, 0, s>>>(L, K, ch, nch, sc, partial, to_vc, F, sk);
    else kr_apply<double, 1><<<grid_of(nch, sms), 256, 0, s>>>(L, K, ch, nch, sc, partial, 0, F, 0);
    OPG_LAUNCHED();
    return check_launch("kr_apply");
}
int kr_launch_update(cudaStream_t s, int sms, bool f32, const LvlDev* L, const KrylovDev* K, const Chunk* ch, int nch, const Scal* sc, double* partial,
                     const Finish& F) {
    if (nch <= 0) return OPFLOW_OK;
    if (f32) kr_update<float><<<grid_of(nch, sms), 256, 0, s>>>(L, K, ch, nch, sc, partial, F);
    else kr_update<double><<<grid_of(nch, sms), 256, 0, s>>>(L, K, ch, nch, sc, partial, F);
    OPG_LAUNCHED();
    return check_launch("kr_update");
}
int kr_launch_from_vcycle(cudaStream_t s, int sms, bool f32, const LvlDev* L, const KrylovDev* K, const Chunk* ch, int nch, const Scal* sc,
                          double* partial, const Finish& F) {
    if (nch <= 0) return OPFLOW_OK;
    if (f32) kr_from_vcycle<float><<<grid_of(nch, sms), 256, 0, s>>>(L, K, ch, nch, sc, partial, F);
    else kr_from_vcycle<double><<<grid_of(nch, sms), 256, 0, s>>>(L, K, ch, nch, sc, partial, F);
    OPG_LAUNCHED();
    return check_launch("kr_from_vcycle");
}
int kr_launch_pupdate(cudaStream_t s, int sms, bool f32, const LvlDev* L, const KrylovDev* K, const Chunk* ch, int nch, const Scal* sc, int first) {
    if (nch <= 0) return OPFLOW_OK;
    if (f32) kr_pupdate<float><<<grid_of(nch, sms), 256, 0, s>>>(L, K, ch, nch, sc, first);
    else kr_pupdate<double><<<grid_of(nch, sms), 256, 0, s>>>(L, K, ch, nch, sc, first);
    OPG_LAUNCHED();
    return check_launch("kr_pupdate");
}
int kr_launch_zero_x(cudaStream_t s, int sms, const LvlDev* L, const KrylovDev* K, const Chunk* ch, int nch) {
    if (nch <= 0) return OPFLOW_OK;
    kr_zero_x<<<grid_of(nch, sms), 256, 0, s>>>(L, K, ch, nch);
    OPG_LAUNCHED();
    return check_launch("kr_zero_x");
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
