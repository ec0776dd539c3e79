// gmi_context.hpp -- per-GPU execution context: stream, grow-only scratch,
// launch-shape cache, device error word.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include <map>
#include <mutex>
#include <tuple>

#include "gmi_common.cuh"

namespace gmi {

// Grow-only device buffer.  Scratch never shrinks during a context's life,
// so a steady-state solve performs no allocation.
struct DeviceBuffer {
    void *ptr = nullptr;
    size_t bytes = 0;
    gmi_status reserve(size_t need);
    void release();
};

// Launch shape of one tiled pair kernel.
struct PairShape {
    int tpb = 128;     // threads per CTA
    int tt = 2;        // targets per thread
    int splits = 0;    // source splits; 0 = choose from the SM count
    int packed = -1;   // two sources per thread step (FP32, no wall): 1 yes, 0 no, -1 where available
};

enum PairKind : int { kSS = 0, kSSWall = 1, kBB = 2, kSB = 3, kBS = 4 };

using TuneKey = std::tuple<int, int, int, int>;  // kind, precision, n_tgt, n_src

}  // namespace gmi

struct gmi_context {
    int device = 0;
    int sm_count = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    int precision = GMI_FP64;
    unsigned *d_err = nullptr;       // device error word (kDevErr* bits)
    unsigned *h_err = nullptr;       // pinned mirror for the synchronising read
    long long launches = 0;          // kernels this context has launched
    gmi::DeviceBuffer rec_src, rec_tgt, partial;
    gmi::DeviceBuffer cells;  // the barrier's cell list
    std::map<gmi::TuneKey, gmi::PairShape> tuned;
    int last_splits = 1;  // source splits of the last tiled pair launch (the autotuner reads it)
    void *encode_tiled = nullptr;    // cuTensorMapEncodeTiled from the driver
    unsigned long long wait_ns = 0;  // deadline of the pair kernels' bounded waits (0: kWaitDeadlineNs)
};

namespace gmi {
gmi_status context_init(gmi_context *ctx, int device);
gmi_status context_check_device_errors(gmi_context *ctx);

// Make fn's dynamic shared-memory limit on the current device at least
// bytes.  The limit belongs to the function, not to a context or a stream,
// so solvers of different sizes driven from different host threads share
// it: it is only ever raised, under a lock, and a launch sized for one
// solver never finds it lowered by another.
cudaError_t raise_dynamic_smem_limit(const void *fn, size_t bytes);
// cudaOccupancyMaxActiveBlocksPerMultiprocessor for this device, function,
// block size and dynamic shared memory, asked once and remembered (a pair
// launch sizes its grid by it on every call).
cudaError_t max_active_blocks(int *blocks, const void *fn, int threads, size_t smem);

// One process-wide lock over every stream capture and every call that
// synchronises the whole device (cudaFree, cudaFreeHost, and cudaMalloc,
// which may).  A device-wide synchronisation on one host thread invalidates
// a capture in progress on another, so solvers stepped from several threads
// (independent swimmers) allocate, free and capture one at a time; their
// kernels still overlap.  Recursive: a capture may allocate.
std::recursive_mutex &device_sync_mutex();
cudaError_t dev_malloc_bytes(void **p, size_t bytes);
cudaError_t dev_free(void *p);
cudaError_t host_alloc_bytes(void **p, size_t bytes, unsigned flags);
cudaError_t host_free(void *p);

template <class T>
cudaError_t dev_malloc(T **p, size_t bytes)
{
    return dev_malloc_bytes(reinterpret_cast<void **>(p), bytes);
}

template <class T>
cudaError_t host_alloc(T **p, size_t bytes, unsigned flags = cudaHostAllocDefault)
{
    return host_alloc_bytes(reinterpret_cast<void **>(p), bytes, flags);
}
}  // namespace gmi
