// gmi_common.cuh -- shared definitions for the GB300 mobility library:
// status codes, the CUDA error check, and the inline-PTX primitives the
// pair kernels use (mbarrier, TMA tensor loads, bounded waits).
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/gmi.h"

namespace gmi {

constexpr double kPi = 3.14159265358979323846264338327950288;

// Device-side error bits, OR-ed into the context's device error word.
// (Non-finite values are not flagged here: the host checks every residual it
// reads -- GMRES's, the refinement's, Broyden's -- and a NaN residual also
// ends the device-side Arnoldi loop, whose convergence test fails for it.)
enum : unsigned {
    kDevErrWaitTimeout = 1u << 0,  // an mbarrier wait ran past its deadline
};

// Programmatic dependent launch.  A kernel launched with the programmatic
// stream-serialization attribute may start while the previous kernel on its
// stream still runs.  griddepcontrol.wait blocks until that kernel has
// completed and its memory is visible (a no-op after an ordinary launch);
// launch_dependents then lets the next kernel start launching, so kernel
// boundaries in a chain of short kernels overlap the launch latency.  The
// kernels of the graph-replayed Arnoldi step call this first.  The pair
// kernels only wait (pdl_wait): their many CTAs keep the SMs, and the next
// kernel launches when they exit.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

__device__ __forceinline__ void pdl_wait_then_release()
{
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// Upper bound for any spin on an mbarrier: by default 2 s of %globaltimer
// (a context can set its own, gmi_context_set_wait_deadline; a launch passes
// it by value, 0 meaning the default).  A wait that runs past it records
// kDevErrWaitTimeout and the kernel returns.
constexpr unsigned long long kWaitDeadlineNs = 2000000000ull;

#define GMI_CUDA_TRY(expr)                                        \
    do {                                                          \
        cudaError_t gmi_e_ = (expr);                              \
        if (gmi_e_ != cudaSuccess) {                              \
            gmi::set_last_error(cudaGetErrorString(gmi_e_), #expr, __FILE__, __LINE__); \
            return GMI_ERR_CUDA;                                  \
        }                                                         \
    } while (0)

// Return the status of a gmi call that failed.
#define GMI_TRY(expr)                        \
    do {                                     \
        gmi_status gmi_s_ = (expr);          \
        if (gmi_s_ != GMI_OK) return gmi_s_; \
    } while (0)

void set_last_error(const char *what, const char *expr, const char *file, int line);
void set_last_error_msg(const char *msg);

// ---------------------------------------------------------------------------
// PTX helpers
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned smem_u32(const void *p)
{
    return static_cast<unsigned>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_mbar_init()
{
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void fence_proxy_async_smem()
{
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, unsigned bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t *bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, unsigned parity)
{
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ unsigned long long global_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
    return t;
}

// Wait for the mbarrier phase with the given parity to complete, giving up
// after deadline_ns (kWaitDeadlineNs when 0).  Returns false on timeout.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, unsigned parity,
                                                  unsigned long long deadline_ns = 0)
{
    if (mbar_try_wait(bar, parity)) return true;
    const unsigned long long limit = deadline_ns ? deadline_ns : kWaitDeadlineNs;
    const unsigned long long t0 = global_ns();
    for (unsigned it = 0;; ++it) {
        if (mbar_try_wait(bar, parity)) return true;
        if ((it & 255u) == 255u && global_ns() - t0 > limit) return false;
    }
}

// 2-D tiled TMA load of one box into shared memory, completing on `bar`.
// c0 is the innermost coordinate (always 0 here: whole records are loaded),
// c1 the row (source index).
__device__ __forceinline__ void tma_load_2d(void *smem_dst, const CUtensorMap *map, int c0, int c1,
                                            uint64_t *bar)
{
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3}], [%4];" ::"r"(smem_u32(smem_dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ void prefetch_tensormap(const CUtensorMap *map)
{
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(map)) : "memory");
}

}  // namespace gmi
