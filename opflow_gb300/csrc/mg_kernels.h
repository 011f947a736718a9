// Launchers of the multigrid / Krylov kernels (mg.cu).
#pragma once

#include <cuda.h>
#include "mg.h"

namespace opg {
int mg_launch_residual(cudaStream_t s, int sms, bool f32, const LvlDev* L, const Chunk* ch, int nch, const Scal* sc);
int mg_launch_smooth(cudaStream_t s, int sms, bool f32, const LvlDev* L, const Chunk* ch, int nch, int color, const Scal* sc);
// red-black half sweep of 3D class-table levels marching along z (tiles: Chunk{lvl, j = y origin,
// k = first plane, i0 = x origin, cnt = MG_ZT_X, nrows = planes}); used for 3D levels of at least
// MG_ZT_MIN cells with at least 3 cells along every dim
constexpr int MG_ZT_X = 30, MG_ZT_Y = 8, MG_ZT_Z = 32;
constexpr long long MG_ZT_MIN = 32768;
// (zb: planes per load batch, 2, 4 or 8; OPFLOW_MG_ZB overrides)
int mg_launch_smooth_z(cudaStream_t s, int sms, bool f32, const LvlDev* L, const Chunk* ch, int nch, int color, const Scal* sc, int zb);
// r = b - A x over the same tiles
int mg_launch_residual_z(cudaStream_t s, int sms, bool f32, const LvlDev* L, const Chunk* ch, int nch, const Scal* sc, int zb);
// the TMA-staged float32 smoother of non-periodic levels over its own tiles (Chunk{lvl, j = a multiple
// of MG_ZT2_Y, k, i0 = a multiple of MG_ZT2_X, MG_ZT2_X, planes <= MG_ZT2_Z}); maps: device array, the x
// and b tensor maps of level index l at [2 l] and [2 l + 1]
constexpr int MG_ZT2_X = 64, MG_ZT2_Y = 16, MG_ZT2_Z = 64;
int mg_launch_smooth_zt(cudaStream_t s, int sms, const LvlDev* L, const Chunk* ch, int nch, int color, const Scal* sc, const CUtensorMap* maps);
// CTAs of mg_smooth_zt resident at once on `sms` SMs (its grid)
int mg_zt_resident(int sms);
// encodes the x and b tensor maps of a float32 level for mg_smooth_zt (boxes (MG_ZT2_X + 8) x
// (MG_ZT2_Y + 2) and MG_ZT2_X x MG_ZT2_Y)
int mg_encode_zt_maps(const LvlDev& D, CUtensorMap* two);
// reads (and clears) the kernels' failure flag: 1 after a bounded wait of mg_smooth_zt gave up
int mg_take_error(cudaStream_t s, int* err);
// plane-batch value that selects mg_smooth_zt in the tuner and OPFLOW_MG_ZB
constexpr int MG_ZB_TMA = 16;
// a level's z-marching choice after the OPFLOW_MG_ZB override
int mg_z_batch(int zb);
// x += P x_coarse over the same tiles (the tiles' first planes are even)
int mg_launch_prolong_z(cudaStream_t s, int sms, bool f32, const LvlDev* L, const Chunk* ch, int nch, const Scal* sc, int zb);
int mg_launch_restrict(cudaStream_t s, int sms, bool f32, const LvlDev* L, const Chunk* ch, int nch, const Scal* sc);
int mg_launch_prolong(cudaStream_t s, int sms, bool f32, const LvlDev* L, const Chunk* ch, int nch, const Scal* sc);
// fused 2D tile steps of a level (mg_tiles.cu): down = pre-smoothing + residual + restriction,
// up = prolongation + post-smoothing; tiles are Chunk{lvl, j = tile y origin, k = 0, i0 = tile x origin}
// 54 columns: with the down step's 5-cell halo a region row is 64 positions, one colour of it one
// warp-wide pass; small levels use MG_TILE_X_SMALL x MG_TILE_Y / 2 (32-position rows)
constexpr int MG_TILE_X = 54, MG_TILE_Y = 32, MG_TILE_X_SMALL = 22;
bool mg_tiles_supported(int sweeps);
int mg_tiles_prepare(int sweeps);
int mg_launch_tile_down(cudaStream_t s, int sms, bool f32, const LvlDev* L, const Chunk* tiles, int ntiles, const Scal* sc, int pre);
int mg_launch_tile_up(cudaStream_t s, int sms, bool f32, const LvlDev* L, const Chunk* tiles, int ntiles, const Scal* sc, int post);
// the whole V-cycle below each listed level (a problem's first small level), one CTA per problem with
// those levels' vectors in shared memory: at most MG_BOTTOM_LEVELS levels and MG_BOTTOM_CELLS cells
// in all (`cells`: the largest such total of the listed problems)
constexpr int MG_BOTTOM_LEVELS = 12;
constexpr int MG_BOTTOM_CELLS = 8192;
int mg_bottom_prepare();
int mg_launch_bottom(cudaStream_t s, int sms, bool f32, const LvlDev* L, const int* top, int ntop, const Scal* sc, int pre, int post,
                     long long cells);
int mg_launch_coarse(cudaStream_t s, int sms, bool f32, const LvlDev* L, const int* lv, int nlv, const Scal* sc);
// The Krylov kernels write per-chunk partial sums; with F.done set they also reduce them per problem
// and apply a scalar stage (see Finish), otherwise kr_launch_reduce / kr_launch_scalars do that.
// to_vc (mode 0): also write the V-cycle's level-0 input (precision f32 ? float : double) from r.
int kr_launch_apply(cudaStream_t s, int sms, const LvlDev* L, const KrylovDev* K, const Chunk* ch, int nch, const Scal* sc, double* partial, int mode,
                    const Finish& F = Finish{}, int to_vc = 0, bool f32 = false, bool skip_first = false);
// x += alpha p, r -= alpha q and the V-cycle's level-0 input from the new r
int kr_launch_update(cudaStream_t s, int sms, bool f32, const LvlDev* L, const KrylovDev* K, const Chunk* ch, int nch, const Scal* sc, double* partial,
                     const Finish& F = Finish{});
int kr_launch_from_vcycle(cudaStream_t s, int sms, bool f32, const LvlDev* L, const KrylovDev* K, const Chunk* ch, int nch, const Scal* sc,
                          double* partial, const Finish& F = Finish{});
int kr_launch_pupdate(cudaStream_t s, int sms, bool f32, const LvlDev* L, const KrylovDev* K, const Chunk* ch, int nch, const Scal* sc, int first);
int kr_launch_zero_x(cudaStream_t s, int sms, const LvlDev* L, const KrylovDev* K, const Chunk* ch, int nch);
int kr_launch_reduce(cudaStream_t s, int sms, const double* partial, const int* first, const int* count, int nprob, double* out);
int kr_launch_scalars(cudaStream_t s, Scal* sc, const double* red, int nprob, int stage, double tol, int max_iter, int flexible);
int kr_launch_count(cudaStream_t s, const Scal* sc, int nprob, int* out);
}  // namespace opg
