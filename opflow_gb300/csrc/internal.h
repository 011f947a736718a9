// Internal declarations shared by the translation units of libopflow_gpu.so.
#pragma once
#include "../../include/opflow_gpu.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <atomic>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

namespace opg {

// ---- errors -----------------------------------------------------------------------------------------
void set_error(const char* fmt, ...);
int fail(int code, const char* fmt, ...);
#define OPG_CUDA(call)                                                                                         \
    do {                                                                                                       \
        cudaError_t e_ = (call);                                                                               \
        if (e_ != cudaSuccess) return ::opg::fail(OPFLOW_E_CUDA, "%s failed: %s (%s:%d)", #call,              \
                                                  cudaGetErrorString(e_), __FILE__, __LINE__);                \
    } while (0)
#define OPG_TRY(call)                                                                                          \
    do {                                                                                                       \
        int rc_ = (call);                                                                                      \
        if (rc_ != OPFLOW_OK) return rc_;                                                                      \
    } while (0)

// Every kernel launch goes through this counter (gpu_launches accounting in the bench).
extern std::atomic<uint64_t> g_launches;
#define OPG_LAUNCHED() (::opg::g_launches.fetch_add(1, std::memory_order_relaxed))
int check_launch(const char* what);

// ---- geometry ---------------------------------------------------------------------------------------
struct Box {
    int lo[3] = {0, 0, 0}, hi[3] = {1, 1, 1};
    __host__ __device__ long long count() const {
        long long c = 1;
        for (int d = 0; d < 3; ++d) c *= (hi[d] > lo[d] ? hi[d] - lo[d] : 0);
        return c;
    }
    __host__ __device__ bool empty() const { return count() == 0; }
};

// Device view of a field's data array and the ranges the kernels need.
struct FieldView {
    double* data;
    int off[3];      // index of element 0
    int dims[3];     // data extents
    long long sy, sz;  // strides (x fastest)
};

struct MeshDev {
    int ndim;
    int es[3];          // first index of the extended mesh range (start - pad_width)
    int n[3];           // number of nodes in the extended range
    int pad = 0;        // pad_width: the mesh range is [es + pad, es + n - pad)
    double* x[3];       // device arrays
    double* dx[3];
    // host copies
    std::vector<double> hx[3], hdx[3];
    bool uniform[3];
    double h[3];        // uniform spacing (valid when uniform[d])
};

#ifdef __CUDACC__
// Grid-stride linear index -> box index (x fastest), with 32-bit division when the box allows.
__device__ __forceinline__ void box_index(long long t, const Box& b, int& i, int& j, int& k) {
    const unsigned nx = (unsigned) (b.hi[0] - b.lo[0]), ny = (unsigned) (b.hi[1] - b.lo[1]);
    if (t < 0xFFFFFFFFll) {
        const unsigned tt = (unsigned) t, q = tt / nx, r = q / ny;
        i = b.lo[0] + (int) (tt - q * nx);
        j = b.lo[1] + (int) (q - r * ny);
        k = b.lo[2] + (int) r;
    } else {
        const long long q = t / nx, r = q / ny;
        i = b.lo[0] + (int) (t - q * nx);
        j = b.lo[1] + (int) (q - r * ny);
        k = b.lo[2] + (int) r;
    }
}
#endif

}  // namespace opg

struct opflow_ctx_s {
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    int num_sms = 0;
    // scratch for reductions (grown on demand)
    void* scratch = nullptr;
    size_t scratch_bytes = 0;
};

struct opflow_field_s {
    opflow_ctx ctx = nullptr;
    opflow_field_desc desc{};
    opflow_field_info info{};
    opg::MeshDev* mesh = nullptr;  // shared (reference counted by owner fields)
    int mesh_refs_owner = 1;
    double* buf[2] = {nullptr, nullptr};  // front = buf[cur]; back allocated on the first aliased assign
    int cur = 0;
    // buffer k already holds this field's boundary values (set by a padding update, cleared whenever
    // the caller may have written the buffer); lets a padding update that can only rewrite constant
    // Dirichlet nodes be skipped
    bool bc_fresh[2] = {false, false};
    // bumped by every write of the values (assign, fill, copy, upload, device pointer, solve, WENO
    // step): a solve handler compares it to decide whether its assembled system is still current
    unsigned long long version = 0;
    bool padding_is_step0_only() const;
    opg::FieldView view() const;
    opg::FieldView view_back() const;
};

namespace opg {
int mesh_create(opflow_ctx ctx, const opflow_mesh_desc* m, MeshDev** out);
void mesh_destroy(opflow_ctx ctx, MeshDev* m);
bool mesh_equal(const MeshDev* a, const MeshDev* b);
int ensure_back(opflow_field f);
int update_padding_buf(opflow_field f, double* data);
int update_padding_full(opflow_field f, double* data);
int fill_dirichlet_nodes(opflow_field f, double* data, const double values[3][2]);
// updatePadding as an assignment does it (assign_impl and assignImpl_final each run one pass; a second
// pass only changes a periodic zone wider than its period)
int update_padding_assign(opflow_field f);
bool padding_self_overlaps(opflow_field f);
int ensure_scratch(opflow_ctx ctx, size_t bytes);
// Device memory of a context: stream-ordered allocations on the context's stream from a per-device
// pool that keeps its memory (no device-wide synchronisation on free, cheap reuse).  Memory returned
// by dev_alloc is usable on the context's stream at once and on other streams after that stream
// has been synchronised.
void* dev_alloc(opflow_ctx ctx, size_t bytes);
void dev_free(opflow_ctx ctx, void* p);
int compute_info(const opflow_mesh_desc* m, const opflow_field_desc* f, opflow_field_info* o);
Box assign_box(const opflow_field_info& r);
}  // namespace opg
