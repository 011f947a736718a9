// Fused 2D multigrid tile kernels for the large red-black levels with a class-table operator.
//
// The chunked kernels make one pass over a level per half-sweep, residual, restriction and
// prolongation: 2*(pre+post) + 3 launches and as many HBM passes per level.  Here one CTA takes a
// TX x TY tile plus a halo into shared memory and runs the whole down-leg step of the level in it -
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
#include "mg_device.h"

namespace opg {

constexpr int TILE_X = MG_TILE_X, TILE_Y = MG_TILE_Y, TILE_THREADS = 512;

// global index of a tile position along one dim: wrapped for a periodic dim, -1 outside otherwise
__device__ __forceinline__ int tile_wrap(int g, int n, int per) {
    if (g >= 0 && g < n) return g;
    if (!per) return -1;
    g %= n;
    return g < 0 ? g + n : g;
}

template <typename T>
struct TileView {
    T* x;        // [SY][SX] smem
    T* b;
    int SX, SY, H;
    int i0, j0;  // global origin of the tile (without halo)
};

// One red-black update of smem cell (lx, ly) mirroring global (gi, gj) (both inside the level).
template <typename T>
__device__ __forceinline__ void tile_gs(const LvlDev& L, const T* __restrict__ tab, const TileView<T>& V, int lx, int ly, int gi, int gj) {
    const int n0 = L.n[0], n1 = L.n[1];
    const int cls = pos_class(gi, n0) + 3 * pos_class(gj, n1);
    const T* cf = tab + cls * TSTRIDE;
    const int s = ly * V.SX + lx;
    T acc = 0;
    if (L.per[0] || gi - 1 >= 0) acc += cf[1] * V.x[s - 1];
    if (L.per[0] || gi + 1 < n0) acc += cf[2] * V.x[s + 1];
    if (L.per[1] || gj - 1 >= 0) acc += cf[3] * V.x[s - V.SX];
    if (L.per[1] || gj + 1 < n1) acc += cf[4] * V.x[s + V.SX];
    V.x[s] = (V.b[s] - acc) * cf[NSLOT];
}

template <typename T>
__device__ __forceinline__ T tile_residual(const LvlDev& L, const T* __restrict__ tab, const TileView<T>& V, int lx, int ly, int gi, int gj) {
    const int n0 = L.n[0], n1 = L.n[1];
    const int cls = pos_class(gi, n0) + 3 * pos_class(gj, n1);
    const T* cf = tab + cls * TSTRIDE;
    const int s = ly * V.SX + lx;
    T acc = 0;
    if (L.per[0] || gi - 1 >= 0) acc += cf[1] * V.x[s - 1];
    if (L.per[0] || gi + 1 < n0) acc += cf[2] * V.x[s + 1];
    if (L.per[1] || gj - 1 >= 0) acc += cf[3] * V.x[s - V.SX];
    if (L.per[1] || gj + 1 < n1) acc += cf[4] * V.x[s + V.SX];
    return V.b[s] - (cf[0] * V.x[s] + acc);
}

// Loads x (from `x`) and b of the tile + halo (positions outside a non-periodic level hold 0 and are
// never used).
template <typename T>
__device__ __forceinline__ void tile_load(const LvlDev& L, const TileView<T>& V, const T* __restrict__ x) {
    const T* b = Sel<T>::b(L);
    for (int idx = threadIdx.x; idx < V.SX * V.SY; idx += blockDim.x) {
        const int lx = idx % V.SX, ly = idx / V.SX;
        const int gi = tile_wrap(V.i0 - V.H + lx, L.n[0], L.per[0]), gj = tile_wrap(V.j0 - V.H + ly, L.n[1], L.per[1]);
        if (gi >= 0 && gj >= 0) {
            const long long c = (long long) gj * L.n[0] + gi;
            V.x[idx] = x[c];
            V.b[idx] = b[c];
        } else {
            V.x[idx] = 0;
            V.b[idx] = 0;
        }
    }
    __syncthreads();
}

// Half-sweep of `color` over the positions at distance >= d from the region's edge.
template <typename T>
__device__ __forceinline__ void tile_sweep(const LvlDev& L, const T* __restrict__ tab, const TileView<T>& V, int color, int d) {
    const int w = V.SX - 2 * d, h = V.SY - 2 * d;
    for (int idx = threadIdx.x; idx < w * h; idx += blockDim.x) {
        const int lx = d + idx % w, ly = d + idx / w;
        const int gi = tile_wrap(V.i0 - V.H + lx, L.n[0], L.per[0]), gj = tile_wrap(V.j0 - V.H + ly, L.n[1], L.per[1]);
        if (gi < 0 || gj < 0 || ((gi + gj) & 1) != color) continue;
        tile_gs<T>(L, tab, V, lx, ly, gi, gj);
    }
    __syncthreads();
}

template <typename T>
__device__ __forceinline__ void tile_store(const LvlDev& L, const TileView<T>& V, T* __restrict__ x) {
    for (int idx = threadIdx.x; idx < TILE_X * TILE_Y; idx += blockDim.x) {
        const int tx = idx % TILE_X, ty = idx / TILE_X;
        const int gi = V.i0 + tx, gj = V.j0 + ty;
        if (gi < L.n[0] && gj < L.n[1]) x[(long long) gj * L.n[0] + gi] = V.x[(ty + V.H) * V.SX + tx + V.H];
    }
}

// Down-leg step of a 2D level: `pre` red-black sweeps, residual, restriction into the next level (its
// x set to 0).  reach = 1 for node-centred full weighting (residual needed one cell beyond the tile).
template <typename T>
__global__ void __launch_bounds__(TILE_THREADS) mg_tile_down(const LvlDev* __restrict__ Ls, const Chunk* __restrict__ tiles, int ntiles, const Scal* sc,
                                                             int pre) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* sm = (T*) smem_raw;
    __shared__ T tab[NCLASS * TSTRIDE];
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const Chunk C = tiles[t];
        const LvlDev& L = Ls[C.lvl];
        if (sc && !sc[L.problem].active) continue;
        const LvlDev& Lc = Ls[L.coarse];
        const int reach = Lc.node ? 1 : 0;
        TileView<T> V;
        V.H = 2 * pre + 1 + reach;
        V.SX = TILE_X + 2 * V.H;
        V.SY = TILE_Y + 2 * V.H;
        V.i0 = C.i0;
        V.j0 = C.j;
        V.x = sm;
        V.b = sm + V.SX * V.SY;
        T* rs = V.b + V.SX * V.SY;  // residual over the tile + reach: (TILE_X + 2 reach) x (TILE_Y + 2 reach)
        const int RX = TILE_X + 2 * reach;
        for (int q = threadIdx.x; q < NCLASS * TSTRIDE; q += blockDim.x) tab[q] = Sel<T>::Tb(L)[q];
        tile_load<T>(L, V, Sel<T>::x(L));
        for (int it = 0; it < pre; ++it) {
            tile_sweep<T>(L, tab, V, 0, 2 * it + 1);
            tile_sweep<T>(L, tab, V, 1, 2 * it + 2);
        }
        // residual over the tile + reach (positions outside the level are never read by the restriction)
        const int d = V.H - reach;
        for (int idx = threadIdx.x; idx < RX * (TILE_Y + 2 * reach); idx += blockDim.x) {
            const int lx = d + idx % RX, ly = d + idx / RX;
            const int gi = tile_wrap(V.i0 - V.H + lx, L.n[0], L.per[0]), gj = tile_wrap(V.j0 - V.H + ly, L.n[1], L.per[1]);
            rs[idx] = (gi >= 0 && gj >= 0) ? tile_residual<T>(L, tab, V, lx, ly, gi, gj) : (T) 0;
        }
        __syncthreads();
        tile_store<T>(L, V, Sel<T>::r(L));
        // restriction: the coarse cells whose children / centre node lie in this tile
        T* bc = Sel<T>::b(Lc);
        T* xc = Sel<T>::x(Lc);
        int Ilo[2], Ihi[2];
        const int o[2] = {V.i0, V.j0};
        for (int q = 0; q < 2; ++q) {
            if (!Lc.node) {
                Ilo[q] = o[q] / 2;
                Ihi[q] = min((o[q] + (q ? TILE_Y : TILE_X)) / 2, Lc.n[q]);
            } else {
                // fine f <-> coarse I with f = 2 (Lc.lo + I) - L.lo
                const int a = o[q] + L.lo[q], e = o[q] + (q ? TILE_Y : TILE_X) + L.lo[q];
                Ilo[q] = max(0, (a + 1) / 2 - Lc.lo[q]);
                Ihi[q] = min(Lc.n[q], (e + 1) / 2 - Lc.lo[q]);
            }
        }
        const int cw = Ihi[0] - Ilo[0], ch = Ihi[1] - Ilo[1];
        for (int idx = threadIdx.x; idx < cw * ch; idx += blockDim.x) {
            const int I0 = Ilo[0] + idx % cw, I1 = Ilo[1] + idx / cw;
            T acc = 0;
            if (!Lc.node) {
                int cnt = 0;
                for (int dy = 0; dy < 2; ++dy)
                    for (int dx = 0; dx < 2; ++dx) {
                        const int fi = 2 * I0 + dx, fj = 2 * I1 + dy;
                        if (fi < L.n[0] && fj < L.n[1]) {
                            acc += rs[(fj - V.j0) * RX + (fi - V.i0)];
                            cnt++;
                        }
                    }
                acc = acc / (T) cnt;
            } else {
                const int ga0 = Lc.lo[0] + I0, ga1 = Lc.lo[1] + I1;
                for (int dy = -1; dy <= 1; ++dy)
                    for (int dx = -1; dx <= 1; ++dx) {
                        T w = dx == 0 ? (T) 0.5 : (T) 0.25;
                        w *= dy == 0 ? (T) 0.5 : (T) 0.25;
                        const int fi = 2 * ga0 + dx - L.lo[0], fj = 2 * ga1 + dy - L.lo[1];
                        if (fi >= 0 && fi < L.n[0] && fj >= 0 && fj < L.n[1]) acc += w * rs[(fj - V.j0 + 1) * RX + (fi - V.i0 + 1)];
                    }
            }
            const long long cc = (long long) I1 * Lc.n[0] + I0;
            bc[cc] = acc;
            xc[cc] = 0;
        }
        __syncthreads();
    }
}

// Up-leg step of a 2D level: x += P x_coarse, then `post` red-black sweeps (color 1 first).
template <typename T>
__global__ void __launch_bounds__(TILE_THREADS) mg_tile_up(const LvlDev* __restrict__ Ls, const Chunk* __restrict__ tiles, int ntiles, const Scal* sc,
                                                           int post) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* sm = (T*) smem_raw;
    __shared__ T tab[NCLASS * TSTRIDE];
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const Chunk C = tiles[t];
        const LvlDev& L = Ls[C.lvl];
        if (sc && !sc[L.problem].active) continue;
        TileView<T> V;
        V.H = 2 * post;
        V.SX = TILE_X + 2 * V.H;
        V.SY = TILE_Y + 2 * V.H;
        V.i0 = C.i0;
        V.j0 = C.j;
        V.x = sm;
        V.b = sm + V.SX * V.SY;
        for (int q = threadIdx.x; q < NCLASS * TSTRIDE; q += blockDim.x) tab[q] = Sel<T>::Tb(L)[q];
        tile_load<T>(L, V, Sel<T>::r(L));
        for (int idx = threadIdx.x; idx < V.SX * V.SY; idx += blockDim.x) {
            const int lx = idx % V.SX, ly = idx / V.SX;
            const int gi = tile_wrap(V.i0 - V.H + lx, L.n[0], L.per[0]), gj = tile_wrap(V.j0 - V.H + ly, L.n[1], L.per[1]);
            if (gi >= 0 && gj >= 0) {
                const T acc = prolong_acc<T>(Ls, L, gi, gj, 0);
                V.x[idx] += acc;
            }
        }
        __syncthreads();
        for (int it = 0; it < post; ++it) {
            tile_sweep<T>(L, tab, V, 1, 2 * it + 1);
            tile_sweep<T>(L, tab, V, 0, 2 * it + 2);
        }
        tile_store<T>(L, V, Sel<T>::x(L));
        __syncthreads();
    }
}

static size_t tile_smem(bool f32, int sweeps, bool down) {
    const int H = down ? 2 * sweeps + 2 : 2 * sweeps;  // down: + residual + node reach (upper bound)
    const size_t cells = (size_t) (TILE_X + 2 * H) * (TILE_Y + 2 * H);
    const size_t res = down ? (size_t) (TILE_X + 2) * (TILE_Y + 2) : 0;
    return (2 * cells + res) * (f32 ? 4 : 8);
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
    const int g = std::max(1, std::min(ntiles, sms * 2));  // 512 threads x <= 64 registers: two CTAs per SM
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
