// gmi_context.hpp -- per-GPU execution context: stream, grow-only scratch,
// launch-shape cache, device error word.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include <map>
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
    std::map<gmi::TuneKey, gmi::PairShape> tuned;
    int last_splits = 1;  // source splits of the last tiled pair launch (the autotuner reads it)
    void *encode_tiled = nullptr;    // cuTensorMapEncodeTiled from the driver
};

namespace gmi {
gmi_status context_init(gmi_context *ctx, int device);
gmi_status context_check_device_errors(gmi_context *ctx);
}  // namespace gmi
