// Residual norms without any device allocation.
//
// Some callers of this library cannot allocate device memory at the point where they need the answer:
// code running while a CUDA stream is being captured into a graph (cudaMalloc / cudaFree are not
// capturable and break the capture), hosts whose device memory is owned by their own pool allocator
// and hand this library only buffers they allocated, and latency-critical loops where a cudaMalloc or
// cudaFree would synchronise the whole device.  For them this file offers the solver's residual
// computation (r = b - A x with float64 norms of b and r, the kernel the flexible-PCG driver uses to
// report EqnSolveState::relerr) with its scratch - the per-chunk partial sums - in a fixed,
// file-scope device array instead of memory allocated per solver.
//
// Limits and sharing rules:
//   - The array holds OPFLOW_NOALLOC_MAX_CHUNKS chunk partials (1 MiB); a grid needs one chunk per
//     1024 cells of every x-row, and calls needing more are rejected with OPFLOW_E_INVALID.
//   - Every GPU that loads the library keeps the array for the life of the process.
//   - All calls on one device share the array.  Each call writes every partial it later reads, so no
//     entry has to start at zero; but calls whose kernels overlap on the GPU (different streams, or
//     different host threads) race on the array: serialise them.
//   - Every call looks up the array's device address in the current device's context
//     (cudaGetSymbolAddress, no allocation).  The first call on a device may load the module: make it
//     before any stream capture begins.
#include "internal.h"

#define OPFLOW_NOALLOC_MAX_CHUNKS 65536
#define OPFLOW_NOALLOC_CHUNK 1024

namespace opg {

// two float64 partial sums (b.b, r.r) per chunk
static __device__ __align__(256) double g_noalloc_partials[2 * OPFLOW_NOALLOC_MAX_CHUNKS];

struct NaGrid {
    int ndim, n[3], per[3];
    long long N;
    int segs;  // chunks per x-row
};

__device__ __forceinline__ double na_block_sum(double v, double* sh) {
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
    return t;
}

// r = b - A x over chunks of x-rows (same operation order as the solver's residual kernel), one pair
// of partial sums per chunk, reduced inside the CTA in a fixed order
__global__ void __launch_bounds__(256) na_residual_partials(NaGrid G, const double* __restrict__ A, const double* __restrict__ b,
                                                            const double* __restrict__ x, double* __restrict__ r, double* __restrict__ part,
                                                            int nchunks) {
    __shared__ double sh[32];
    for (int c = blockIdx.x; c < nchunks; c += gridDim.x) {
        const int row = c / G.segs, seg = c % G.segs;
        const int j = G.ndim > 1 ? row % G.n[1] : 0, k = G.ndim > 2 ? row / G.n[1] : 0;
        const int i0 = seg * OPFLOW_NOALLOC_CHUNK, cnt = min(OPFLOW_NOALLOC_CHUNK, G.n[0] - i0);
        double sb = 0., sr = 0.;
        for (int t = threadIdx.x; t < cnt; t += blockDim.x) {
            const int i = i0 + t;
            const long long cell = (long long) i + (long long) G.n[0] * ((long long) j + (long long) G.n[1] * k);
            double acc = 0.;
            const int n0 = G.n[0];
            int im = i - 1, ip = i + 1;
            if (im < 0 && G.per[0]) im += n0;
            if (ip >= n0 && G.per[0]) ip -= n0;
            if (im >= 0) acc += A[1 * G.N + cell] * x[cell - i + im];
            if (ip < n0) acc += A[2 * G.N + cell] * x[cell - i + ip];
            if (G.ndim > 1) {
                int jm = j - 1, jp = j + 1;
                if (jm < 0 && G.per[1]) jm += G.n[1];
                if (jp >= G.n[1] && G.per[1]) jp -= G.n[1];
                if (jm >= 0) acc += A[3 * G.N + cell] * x[cell + (long long) (jm - j) * n0];
                if (jp < G.n[1]) acc += A[4 * G.N + cell] * x[cell + (long long) (jp - j) * n0];
            }
            if (G.ndim > 2) {
                const long long sz = (long long) n0 * G.n[1];
                int km = k - 1, kp = k + 1;
                if (km < 0 && G.per[2]) km += G.n[2];
                if (kp >= G.n[2] && G.per[2]) kp -= G.n[2];
                if (km >= 0) acc += A[5 * G.N + cell] * x[cell + (km - k) * sz];
                if (kp < G.n[2]) acc += A[6 * G.N + cell] * x[cell + (kp - k) * sz];
            }
            const double rv = b[cell] - fma(A[cell], x[cell], acc);
            r[cell] = rv;
            sb = fma(b[cell], b[cell], sb);
            sr = fma(rv, rv, sr);
        }
        const double tb = na_block_sum(sb, sh);
        const double tr = na_block_sum(sr, sh);
        if (threadIdx.x == 0) {
            part[2 * c] = tb;
            part[2 * c + 1] = tr;
        }
    }
}

// norms[0] = ||b||_2, norms[1] = ||b - A x||_2 from the chunk partials, summed in chunk order
__global__ void __launch_bounds__(256) na_reduce(const double* __restrict__ part, int nchunks, double* norms) {
    __shared__ double sh[32];
    double sb = 0., sr = 0.;
    for (int c = threadIdx.x; c < nchunks; c += blockDim.x) {
        sb += part[2 * c];
        sr += part[2 * c + 1];
    }
    const double tb = na_block_sum(sb, sh);
    const double tr = na_block_sum(sr, sh);
    if (threadIdx.x == 0) {
        norms[0] = sqrt(tb);
        norms[1] = sqrt(tr);
    }
}

// Device address of the static partial-sum array in the current device's context, looked up on every
// call (no allocation once the module is loaded, and never stale after a device reset).
static int noalloc_scratch(double** out) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_partials);
    if (e != cudaSuccess || !p) return fail(OPFLOW_E_CUDA, "cudaGetSymbolAddress of the static residual scratch failed: %s", cudaGetErrorString(e));
    *out = (double*) p;
    return OPFLOW_OK;
}

}  // namespace opg

using namespace opg;

extern "C" int opflow_residual_norms_noalloc(void* stream, int ndim, const int* n, const int* periodic, const double* coef, const double* b,
                                             const double* x, double* r, double* norms) {
    if (ndim < 1 || ndim > 3 || !n || !coef || !b || !x || !r || !norms) return fail(OPFLOW_E_INVALID, "null or bad argument");
    NaGrid G{};
    G.ndim = ndim;
    G.N = 1;
    for (int d = 0; d < 3; ++d) {
        G.n[d] = d < ndim ? n[d] : 1;
        G.per[d] = d < ndim && periodic ? (periodic[d] != 0) : 0;
        if (G.n[d] < 1) return fail(OPFLOW_E_INVALID, "empty grid along dim %d", d);
        G.N *= G.n[d];
    }
    G.segs = (G.n[0] + OPFLOW_NOALLOC_CHUNK - 1) / OPFLOW_NOALLOC_CHUNK;
    const long long rows = (long long) G.n[1] * G.n[2];
    const long long nchunks = rows * G.segs;
    if (nchunks > OPFLOW_NOALLOC_MAX_CHUNKS)
        return fail(OPFLOW_E_INVALID,
                    "grid needs %lld partial-sum chunks (one per %d cells of each x-row); the static scratch holds %d: use the allocating solver",
                    nchunks, OPFLOW_NOALLOC_CHUNK, OPFLOW_NOALLOC_MAX_CHUNKS);
    double* part = nullptr;
    OPG_TRY(noalloc_scratch(&part));
    int sms = 0, dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int blocks = (int) std::max<long long>(1, std::min<long long>(nchunks, (long long) sms * 8));
    cudaStream_t s = (cudaStream_t) stream;
    na_residual_partials<<<blocks, 256, 0, s>>>(G, coef, b, x, r, part, (int) nchunks);
    OPG_LAUNCHED();
    OPG_TRY(check_launch("na_residual_partials"));
    na_reduce<<<1, 256, 0, s>>>(part, (int) nchunks, norms);
    OPG_LAUNCHED();
    return check_launch("na_reduce");
}
