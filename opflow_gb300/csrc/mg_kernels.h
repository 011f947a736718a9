// Launchers of the multigrid / Krylov kernels (mg.cu).
#pragma once
#include "mg.h"

namespace opg {
int mg_launch_residual(cudaStream_t s, int sms, bool f32, const LvlDev* L, const Chunk* ch, int nch, const Scal* sc);
int mg_launch_smooth(cudaStream_t s, int sms, bool f32, const LvlDev* L, const Chunk* ch, int nch, int color, const Scal* sc);
int mg_launch_restrict(cudaStream_t s, int sms, bool f32, const LvlDev* L, const Chunk* ch, int nch, const Scal* sc);
int mg_launch_prolong(cudaStream_t s, int sms, bool f32, const LvlDev* L, const Chunk* ch, int nch, const Scal* sc);
// the whole V-cycle below each listed level (a problem's first small level), one CTA per problem
int mg_launch_bottom(cudaStream_t s, int sms, bool f32, const LvlDev* L, const int* top, int ntop, const Scal* sc, int pre, int post);
int mg_launch_coarse(cudaStream_t s, int sms, bool f32, const LvlDev* L, const int* lv, int nlv, const Scal* sc);
int kr_launch_apply(cudaStream_t s, int sms, const LvlDev* L, const KrylovDev* K, const Chunk* ch, int nch, const Scal* sc, double* partial, int mode);
int kr_launch_update(cudaStream_t s, int sms, const LvlDev* L, const KrylovDev* K, const Chunk* ch, int nch, const Scal* sc, double* partial);
int kr_launch_to_vcycle(cudaStream_t s, int sms, bool f32, const LvlDev* L, const KrylovDev* K, const Chunk* ch, int nch, const Scal* sc);
int kr_launch_from_vcycle(cudaStream_t s, int sms, bool f32, const LvlDev* L, const KrylovDev* K, const Chunk* ch, int nch, const Scal* sc,
                          double* partial);
int kr_launch_pupdate(cudaStream_t s, int sms, const LvlDev* L, const KrylovDev* K, const Chunk* ch, int nch, const Scal* sc, int first);
int kr_launch_reduce(cudaStream_t s, int sms, const double* partial, const int* first, const int* count, int nprob, double* out);
int kr_launch_scalars(cudaStream_t s, Scal* sc, const double* red, int nprob, int stage, double tol, int max_iter, int flexible);
int kr_launch_count(cudaStream_t s, const Scal* sc, int nprob, int* out);
}  // namespace opg
