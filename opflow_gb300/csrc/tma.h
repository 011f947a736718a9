// TMA copies (global -> shared, completing on an mbarrier), bounded mbarrier waits and the host-side
// tensor-map encoder, shared by the TMA-staged kernels (the multigrid smoother mg_smooth_zt and the
// resident fixed-point FTCS step axis3d_fxtma_kernel).
//
// Every wait gives up after MBAR_SPINS polls of mbarrier.try_wait, each of which suspends the thread
// for at most MBAR_SUSPEND_NS (about a second in all); the kernel then records the failure in a device
// flag of its own, waits (bounded again) for the copies it issued and returns.
#pragma once
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

namespace opg {

constexpr int MBAR_SPINS = 1 << 20;
constexpr unsigned MBAR_SUSPEND_NS = 1000;

__device__ __forceinline__ unsigned smem_addr(const void* p) { return (unsigned) __cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_fence_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void mbar_arrive_expect(unsigned long long* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
}
// true once the phase of the given parity has completed; the thread is suspended (not spinning) while it
// waits, for at most MBAR_SUSPEND_NS
__device__ __forceinline__ bool mbar_test(unsigned long long* bar, unsigned parity) {
    unsigned done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(smem_addr(bar)), "r"(parity), "r"(MBAR_SUSPEND_NS)
        : "memory");
    return done != 0;
}
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, unsigned parity) {
    for (int it = 0; it < MBAR_SPINS; ++it)
        if (mbar_test(bar, parity)) return true;
    return false;
}

// 3D tiled copy of a tensor map's box at (x, y, z) into shared memory, completing on `bar`
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, int x, int y, int z, unsigned long long* bar) {
    asm volatile("cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_addr(dst)),
                 "l"(map), "r"(x), "r"(y), "r"(z), "r"(smem_addr(bar))
                 : "memory");
}
__device__ __forceinline__ void tensormap_acquire(const CUtensorMap* map) {
    asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"(map) : "memory");
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (null when the driver has none)
inline PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
    static const PFN_cuTensorMapEncodeTiled_v12000 enc = [] {
        void* fn = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess) {
            cudaGetLastError();
            fn = nullptr;
        }
        return (PFN_cuTensorMapEncodeTiled_v12000) fn;
    }();
    return enc;
}

}  // namespace opg
