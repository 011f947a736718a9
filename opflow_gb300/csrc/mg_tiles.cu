// Fused 2D multigrid tile kernels for the large red-black levels with a class-table operator.
//
// The chunked kernels make one pass over a level per half-sweep, residual, restriction and
// prolongation: 2*(pre+post) + 3 launches and as many passes over memory per level.  Here one CTA takes
// a TX x TY tile plus a halo into shared memory and runs the whole down-leg step of the level in it -
// pre-smoothing, residual, restriction into the next level - or the whole up-leg step - prolongation
// and post-smoothing.  Red-black Gauss-Seidel only couples a half-sweep to its neighbours' previous
// half-sweep, so every half-sweep shrinks the region that is still exact by one cell: with a halo of
// (half-sweeps + 1 + restriction reach) cells the tile's own cells end exactly as in the global sweeps.
// The per-cell arithmetic is the chunked kernels' (same operation order), so the two paths give
// bit-identical iterates; only the tile's own cells are written back.
//
// Tiles of one launch read their halos from the level's arrays while other tiles write their results,
// so a launch never writes the array it reads: the down step reads x and leaves the smoothed x in the
// level's r array (the residual itself stays in shared memory), the up step reads that array and
// writes x.
//
// Work layout: warps take rows of the tile region, lanes take columns (a colour's cells with a stride
// of two), so no thread divides an index.  Tiles whose region lies inside the level away from its
// boundary take the interior form: constant coefficients, no wrap-around or existence tests.  The tile
// extent is chosen per level (Chunk.cnt x Chunk.nrows, even widths) so that small levels still spread
// over the SMs.
#include "mg_device.h"

namespace opg {

constexpr int TILE_THREADS = 256;
constexpr int TILE_WARPS = TILE_THREADS / 32;

// global index of a tile position along one dim: wrapped for a periodic dim, -1 outside otherwise
__device__ __forceinline__ int tile_wrap(int g, int n, int per) {
    if (g >= 0 && g < n) return g;
    if (!per) return -1;
    g %= n;
    return g < 0 ? g + n : g;
}

// The tile's geometry in registers.  (Kernels read level data through `const LvlDev&` into global
// memory; inside loops that store through generic pointers the compiler must reload such fields after
// every store, so the loops below only use these copies.)
template <typename T>
struct TileView {
    T* x;        // [SY][SX] smem
    T* b;
    int SX, SY, H;
    int TX, TY;  // tile extent (without halo)
    int i0, j0;  // global origin of the tile (without halo)
    int n0, n1;  // level extent
    int per0, per1;
    bool interior;
};

// One red-black update of smem position s mirroring global (gi, gj), general form.
template <typename T>
__device__ __forceinline__ void tile_gs(const LvlDev& L, const T* __restrict__ tab, const TileView<T>& V, int s, int gi, int gj) {
    const int n0 = V.n0, n1 = V.n1;
    const int cls = pos_class(gi, n0) + 3 * pos_class(gj, n1);
    const T* cf = tab + cls * TSTRIDE;
    T acc = 0;
    if (V.per0 || gi - 1 >= 0) acc += cf[1] * V.x[s - 1];
    if (V.per0 || gi + 1 < n0) acc += cf[2] * V.x[s + 1];
    if (V.per1 || gj - 1 >= 0) acc += cf[3] * V.x[s - V.SX];
    if (V.per1 || gj + 1 < n1) acc += cf[4] * V.x[s + V.SX];
    V.x[s] = (V.b[s] - acc) * cf[NSLOT];
}

template <typename T>
__device__ __forceinline__ T tile_res(const LvlDev& L, const T* __restrict__ tab, const TileView<T>& V, int s, int gi, int gj) {
    const int n0 = V.n0, n1 = V.n1;
    const int cls = pos_class(gi, n0) + 3 * pos_class(gj, n1);
    const T* cf = tab + cls * TSTRIDE;
    T acc = 0;
    if (V.per0 || gi - 1 >= 0) acc += cf[1] * V.x[s - 1];
    if (V.per0 || gi + 1 < n0) acc += cf[2] * V.x[s + 1];
    if (V.per1 || gj - 1 >= 0) acc += cf[3] * V.x[s - V.SX];
    if (V.per1 || gj + 1 < n1) acc += cf[4] * V.x[s + V.SX];
    return V.b[s] - (cf[0] * V.x[s] + acc);
}

// interior coefficients (class 1 + 3*1): the same operations as tile_gs / tile_res with every
// neighbour present
template <typename T>
struct Interior {
    T c0, c1, c2, c3, c4, inv;
};

template <typename T>
__device__ __forceinline__ void int_gs(const Interior<T>& K, const TileView<T>& V, int s) {
    T acc = 0;
    acc += K.c1 * V.x[s - 1];
    acc += K.c2 * V.x[s + 1];
    acc += K.c3 * V.x[s - V.SX];
    acc += K.c4 * V.x[s + V.SX];
    V.x[s] = (V.b[s] - acc) * K.inv;
}

template <typename T>
__device__ __forceinline__ T int_res(const Interior<T>& K, const TileView<T>& V, int s) {
    T acc = 0;
    acc += K.c1 * V.x[s - 1];
    acc += K.c2 * V.x[s + 1];
    acc += K.c3 * V.x[s - V.SX];
    acc += K.c4 * V.x[s + V.SX];
    return V.b[s] - (K.c0 * V.x[s] + acc);
}

// Asynchronous global -> shared copy of one element (cp.async: the copy needs no register and every
// copy a thread issues is in flight at once); completed by async_wait_all + a CTA barrier.
template <typename T>
__device__ __forceinline__ void async_copy(T* smem, const T* gmem) {
    const unsigned sa = (unsigned) __cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], %2;\n" ::"r"(sa), "l"(gmem), "n"(sizeof(T)) : "memory");
}
__device__ __forceinline__ void async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// Issues the copies of x (from `x`) and b of the tile + halo (positions outside a non-periodic level
// get 0 and are never used); the caller waits (async_wait_all + __syncthreads).
template <typename T>
__device__ __forceinline__ void tile_load_issue(const TileView<T>& V, const T* __restrict__ x, const T* __restrict__ b) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int ly = warp; ly < V.SY; ly += TILE_WARPS) {
        const int gjr = V.j0 - V.H + ly;
        const int gj = V.interior ? gjr : tile_wrap(gjr, V.n1, V.per1);
        for (int lx = lane; lx < V.SX; lx += 32) {
            const int gir = V.i0 - V.H + lx;
            const int gi = V.interior ? gir : tile_wrap(gir, V.n0, V.per0);
            const int s = ly * V.SX + lx;
            if (gi >= 0 && gj >= 0) {
                const long long c = (long long) gj * V.n0 + gi;
                async_copy(V.x + s, x + c);
                async_copy(V.b + s, b + c);
            } else {
                V.x[s] = 0;
                V.b[s] = 0;
            }
        }
    }
}

template <typename T>
__device__ __forceinline__ void tile_load(const TileView<T>& V, const T* __restrict__ x, const T* __restrict__ b) {
    tile_load_issue<T>(V, x, b);
    async_wait_all();
    __syncthreads();
}

// Half-sweep of `color` over the positions at distance >= d from the region's edge.
template <typename T>
__device__ __forceinline__ void tile_sweep(const LvlDev& L, const T* __restrict__ tab, const Interior<T>& K, const TileView<T>& V, int color, int d) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int ly = d + warp; ly < V.SY - d; ly += TILE_WARPS) {
        const int gjr = V.j0 - V.H + ly;
        // first position >= d of this colour: (gi + gj) & 1 == color with gi = i0 - H + lx (wrapping by an
        // even period keeps the parity)
        const int lx0 = d + ((color - (V.i0 - V.H + d) - gjr) & 1);
        if (V.interior) {
            for (int lx = lx0 + 2 * lane; lx < V.SX - d; lx += 64) int_gs<T>(K, V, ly * V.SX + lx);
        } else {
            const int gj = tile_wrap(gjr, V.n1, V.per1);
            if (gj < 0) continue;
            for (int lx = lx0 + 2 * lane; lx < V.SX - d; lx += 64) {
                const int gi = tile_wrap(V.i0 - V.H + lx, V.n0, V.per0);
                if (gi >= 0) tile_gs<T>(L, tab, V, ly * V.SX + lx, gi, gj);
            }
        }
    }
    __syncthreads();
}

template <typename T>
__device__ __forceinline__ void tile_store(const TileView<T>& V, T* __restrict__ x) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int ty = warp; ty < V.TY; ty += TILE_WARPS) {
        const int gj = V.j0 + ty;
        if (gj >= V.n1) break;
        for (int tx = lane; tx < V.TX; tx += 32) {
            const int gi = V.i0 + tx;
            if (gi < V.n0) x[(long long) gj * V.n0 + gi] = V.x[(ty + V.H) * V.SX + tx + V.H];
        }
    }
}

template <typename T>
__device__ __forceinline__ void tile_setup(const LvlDev& L, const Chunk& C, int H, T* sm, T* tab, Interior<T>& K, TileView<T>& V) {
    V.TX = C.cnt;
    V.TY = C.nrows;
    V.H = H;
    V.SX = V.TX + 2 * H;
    V.SY = V.TY + 2 * H;
    V.i0 = C.i0;
    V.j0 = C.j;
    V.x = sm;
    V.b = sm + V.SX * V.SY;
    V.n0 = L.n[0];
    V.n1 = L.n[1];
    V.per0 = L.per[0];
    V.per1 = L.per[1];
    // inside the level with a cell to spare on each side: every position is an interior-class cell
    V.interior = V.i0 - H >= 1 && V.i0 + V.TX + H <= V.n0 - 1 && V.j0 - H >= 1 && V.j0 + V.TY + H <= V.n1 - 1;
    for (int q = threadIdx.x; q < NCLASS * TSTRIDE; q += blockDim.x) tab[q] = Sel<T>::Tb(L)[q];
    const T* ti = Sel<T>::Tb(L) + 4 * TSTRIDE;
    K.c0 = ti[0];
    K.c1 = ti[1];
    K.c2 = ti[2];
    K.c3 = ti[3];
    K.c4 = ti[4];
    K.inv = ti[NSLOT];
}

// Down-leg step of a 2D level: `pre` red-black sweeps, residual, restriction into the next level (its
// x set to 0).  reach = 1 for node-centred full weighting (residual needed one cell beyond the tile).
template <typename T>
__global__ void __launch_bounds__(TILE_THREADS, 8) mg_tile_down(const LvlDev* __restrict__ Ls, const Chunk* __restrict__ tiles, int ntiles, const Scal* sc,
                                                                int pre) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* sm = (T*) smem_raw;
    __shared__ T tab[NCLASS * TSTRIDE];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const Chunk C = tiles[t];
        const LvlDev& L = Ls[C.lvl];
        if (sc && !sc[L.problem].active) continue;
        const LvlDev& Lc = Ls[L.coarse];
        const int reach = Lc.node ? 1 : 0;
        TileView<T> V;
        Interior<T> K;
        tile_setup<T>(L, C, 2 * pre + 1 + reach, sm, tab, K, V);
        T* rs = V.b + V.SX * V.SY;  // residual over the tile + reach: RX x RY
        const int RX = V.TX + 2 * reach, RY = V.TY + 2 * reach;
        tile_load<T>(V, Sel<T>::x(L), Sel<T>::b(L));
        for (int it = 0; it < pre; ++it) {
            tile_sweep<T>(L, tab, K, V, 0, 2 * it + 1);
            tile_sweep<T>(L, tab, K, V, 1, 2 * it + 2);
        }
        // residual over the tile + reach (positions outside the level are never read by the restriction)
        const int d = V.H - reach;
        for (int ry = warp; ry < RY; ry += TILE_WARPS) {
            const int ly = d + ry;
            const int gjr = V.j0 - V.H + ly;
            const int gj = V.interior ? gjr : tile_wrap(gjr, V.n1, V.per1);
            for (int rx = lane; rx < RX; rx += 32) {
                const int lx = d + rx;
                const int s = ly * V.SX + lx;
                T r;
                if (V.interior) {
                    r = int_res<T>(K, V, s);
                } else {
                    const int gi = tile_wrap(V.i0 - V.H + lx, V.n0, V.per0);
                    r = (gi >= 0 && gj >= 0) ? tile_res<T>(L, tab, V, s, gi, gj) : (T) 0;
                }
                rs[ry * RX + rx] = r;
            }
        }
        __syncthreads();
        tile_store<T>(V, Sel<T>::r(L));
        // restriction: the coarse cells whose children / centre node lie in this tile
        T* __restrict__ bc = Sel<T>::b(Lc);
        T* __restrict__ xc = Sel<T>::x(Lc);
        const int cnode = Lc.node, cn0 = Lc.n[0], cn1 = Lc.n[1], clo0 = Lc.lo[0], clo1 = Lc.lo[1], flo0 = L.lo[0], flo1 = L.lo[1];
        int Ilo[2], Ihi[2];
        const int o[2] = {V.i0, V.j0}, ext[2] = {V.TX, V.TY};
        {
            const int cn[2] = {cn0, cn1}, clo[2] = {clo0, clo1}, flo[2] = {flo0, flo1};
            for (int q = 0; q < 2; ++q) {
                if (!cnode) {
                    Ilo[q] = o[q] / 2;
                    Ihi[q] = min((o[q] + ext[q]) / 2, cn[q]);
                } else {
                    // fine f <-> coarse I with f = 2 (Lc.lo + I) - L.lo
                    const int a = o[q] + flo[q], e = o[q] + ext[q] + flo[q];
                    Ilo[q] = max(0, (a + 1) / 2 - clo[q]);
                    Ihi[q] = min(cn[q], (e + 1) / 2 - clo[q]);
                }
            }
        }
        for (int I1 = Ilo[1] + warp; I1 < Ihi[1]; I1 += TILE_WARPS) {
            for (int I0 = Ilo[0] + lane; I0 < Ihi[0]; I0 += 32) {
                T acc = 0;
                if (!cnode) {
                    int cnt = 0;
                    for (int dy = 0; dy < 2; ++dy)
                        for (int dx = 0; dx < 2; ++dx) {
                            const int fi = 2 * I0 + dx, fj = 2 * I1 + dy;
                            if (fi < V.n0 && fj < V.n1) {
                                acc += rs[(fj - V.j0) * RX + (fi - V.i0)];
                                cnt++;
                            }
                        }
                    acc = acc / (T) cnt;
                } else {
                    const int ga0 = clo0 + I0, ga1 = clo1 + I1;
                    for (int dy = -1; dy <= 1; ++dy)
                        for (int dx = -1; dx <= 1; ++dx) {
                            T w = dx == 0 ? (T) 0.5 : (T) 0.25;
                            w *= dy == 0 ? (T) 0.5 : (T) 0.25;
                            const int fi = 2 * ga0 + dx - flo0, fj = 2 * ga1 + dy - flo1;
                            if (fi >= 0 && fi < V.n0 && fj >= 0 && fj < V.n1) acc += w * rs[(fj - V.j0 + 1) * RX + (fi - V.i0 + 1)];
                        }
                }
                const long long cc = (long long) I1 * cn0 + I0;
                bc[cc] = acc;
                xc[cc] = 0;
            }
        }
        __syncthreads();
    }
}

// Up-leg step of a 2D level: x += P x_coarse, then `post` red-black sweeps (color 1 first).
template <typename T>
__global__ void __launch_bounds__(TILE_THREADS, 8) mg_tile_up(const LvlDev* __restrict__ Ls, const Chunk* __restrict__ tiles, int ntiles, const Scal* sc,
                                                              int post) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* sm = (T*) smem_raw;
    __shared__ T tab[NCLASS * TSTRIDE];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const Chunk C = tiles[t];
        const LvlDev& L = Ls[C.lvl];
        if (sc && !sc[L.problem].active) continue;
        TileView<T> V;
        Interior<T> K;
        tile_setup<T>(L, C, 2 * post, sm, tab, K, V);
        const LvlDev& Lc = Ls[L.coarse];
        // cell-centred interior tile whose coarse neighbours (I = f/2 and I +- 1) all exist: bilinear
        // interpolation without ghost rules, in the generic form's operation order, from a copy of the
        // coarse block [cx0, cx0 + CW) x [cy0, cy0 + CH) in shared memory
        const int cx0 = ((V.i0 - V.H) >> 1) - 1, cy0 = ((V.j0 - V.H) >> 1) - 1;
        const int CW = ((V.i0 + V.TX + V.H - 1) >> 1) + 2 - cx0, CH = ((V.j0 + V.TY + V.H - 1) >> 1) + 2 - cy0;
        const bool cint = V.interior && !Lc.node && cx0 >= 0 && cx0 + CW <= Lc.n[0] && cy0 >= 0 && cy0 + CH <= Lc.n[1];
        const T* __restrict__ xc = Sel<T>::x(Lc);
        const int nc0 = Lc.n[0];
        T* cs = V.b + V.SX * V.SY;
        tile_load_issue<T>(V, Sel<T>::r(L), Sel<T>::b(L));
        if (cint)
            for (int cy = warp; cy < CH; cy += TILE_WARPS)
                for (int cx = lane; cx < CW; cx += 32) async_copy(cs + cy * CW + cx, xc + (long long) (cy0 + cy) * nc0 + cx0 + cx);
        async_wait_all();
        __syncthreads();
        for (int ly = warp; ly < V.SY; ly += TILE_WARPS) {
            const int gjr = V.j0 - V.H + ly;
            if (cint) {
                const int I1 = gjr >> 1, J1 = (gjr & 1) ? I1 + 1 : I1 - 1;
                const T* r0 = cs + (I1 - cy0) * CW - cx0;
                const T* r1 = cs + (J1 - cy0) * CW - cx0;
                for (int lx = lane; lx < V.SX; lx += 32) {
                    const int gi = V.i0 - V.H + lx;
                    const int I0 = gi >> 1, J0 = (gi & 1) ? I0 + 1 : I0 - 1;
                    T acc = 0;
                    acc += (T) 0.75 * (T) 0.75 * (T) 1 * r0[I0];
                    acc += (T) 0.25 * (T) 0.75 * (T) 1 * r0[J0];
                    acc += (T) 0.75 * (T) 0.25 * (T) 1 * r1[I0];
                    acc += (T) 0.25 * (T) 0.25 * (T) 1 * r1[J0];
                    V.x[ly * V.SX + lx] += acc;
                }
                continue;
            }
            const int gj = tile_wrap(gjr, V.n1, V.per1);
            if (gj < 0) continue;
            for (int lx = lane; lx < V.SX; lx += 32) {
                const int gi = tile_wrap(V.i0 - V.H + lx, V.n0, V.per0);
                if (gi >= 0) {
                    const T acc = prolong_acc<T>(Ls, L, gi, gj, 0);
                    V.x[ly * V.SX + lx] += acc;
                }
            }
        }
        __syncthreads();
        for (int it = 0; it < post; ++it) {
            tile_sweep<T>(L, tab, K, V, 1, 2 * it + 1);
            tile_sweep<T>(L, tab, K, V, 0, 2 * it + 2);
        }
        tile_store<T>(V, Sel<T>::x(L));
        __syncthreads();
    }
}

static size_t tile_smem(bool f32, int sweeps, bool down) {
    const int H = down ? 2 * sweeps + 2 : 2 * sweeps;  // down: + residual + node reach (upper bound)
    const size_t cells = (size_t) (MG_TILE_X + 2 * H) * (MG_TILE_Y + 2 * H);
    // down: the residual over the tile + reach; up: the coarse block of the prolongation
    const size_t extra = down ? (size_t) (MG_TILE_X + 2) * (MG_TILE_Y + 2) : (size_t) ((MG_TILE_X + 2 * H) / 2 + 4) * ((MG_TILE_Y + 2 * H) / 2 + 4);
    return (2 * cells + extra) * (f32 ? 4 : 8);
}

bool mg_tiles_supported(int sweeps) { return sweeps >= 1 && tile_smem(false, sweeps, true) + NCLASS * TSTRIDE * 8 <= 200 * 1024; }

// Raises the kernels' dynamic shared-memory limit for `sweeps` (called while setting a system up, never
// during graph recording).
int mg_tiles_prepare(int sweeps) {
    const size_t need[4] = {tile_smem(true, sweeps, true), tile_smem(false, sweeps, true), tile_smem(true, sweeps, false),
                            tile_smem(false, sweeps, false)};
    const void* fn[4] = {(const void*) mg_tile_down<float>, (const void*) mg_tile_down<double>, (const void*) mg_tile_up<float>,
                         (const void*) mg_tile_up<double>};
    for (int q = 0; q < 4; ++q) {
        const cudaError_t e = cudaFuncSetAttribute(fn[q], cudaFuncAttributeMaxDynamicSharedMemorySize, (int) std::max<size_t>(need[q], 48 * 1024));
        if (e != cudaSuccess) return fail(OPFLOW_E_CUDA, "tile kernels: shared memory %zu B: %s", need[q], cudaGetErrorString(e));
    }
    return OPFLOW_OK;
}

template <typename K>
static int launch_tiles(K kernel, cudaStream_t s, int sms, size_t smem, const LvlDev* L, const Chunk* tiles, int ntiles, const Scal* sc, int sweeps,
                        const char* name) {
    // 256 threads x 32 registers: eight CTAs per SM (measured faster than four CTAs without spilling,
    // the extra tiles in flight hiding each tile's barrier-separated phases)
    const int g = std::max(1, std::min(ntiles, sms * 8));
    kernel<<<g, TILE_THREADS, smem, s>>>(L, tiles, ntiles, sc, sweeps);
    OPG_LAUNCHED();
    return check_launch(name);
}

int mg_launch_tile_down(cudaStream_t s, int sms, bool f32, const LvlDev* L, const Chunk* tiles, int ntiles, const Scal* sc, int pre) {
    if (ntiles <= 0) return OPFLOW_OK;
    const size_t smem = tile_smem(f32, pre, true);
    if (f32) return launch_tiles(mg_tile_down<float>, s, sms, smem, L, tiles, ntiles, sc, pre, "mg_tile_down");
    return launch_tiles(mg_tile_down<double>, s, sms, smem, L, tiles, ntiles, sc, pre, "mg_tile_down");
}

int mg_launch_tile_up(cudaStream_t s, int sms, bool f32, const LvlDev* L, const Chunk* tiles, int ntiles, const Scal* sc, int post) {
    if (ntiles <= 0) return OPFLOW_OK;
    const size_t smem = tile_smem(f32, post, false);
    if (f32) return launch_tiles(mg_tile_up<float>, s, sms, smem, L, tiles, ntiles, sc, post, "mg_tile_up");
    return launch_tiles(mg_tile_up<double>, s, sms, smem, L, tiles, ntiles, sc, post, "mg_tile_up");
}

}  // namespace opg
