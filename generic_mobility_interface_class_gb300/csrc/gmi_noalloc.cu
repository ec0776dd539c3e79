// gmi_noalloc.cu -- an allocation-free form of the segment<-segment mobility
// apply (gmi_Mss_mult).
//
// Who needs it: a caller that cannot call cudaMalloc.  Some host programs
// fix their device-memory budget at start-up and hand every byte to their
// own allocator, so a plug-in may not allocate; others call in from a place
// where the implicit device-wide synchronisation of cudaMalloc/cudaFree is
// not acceptable.  gmi_Mss_mult needs scratch memory (packed source records
// and per-split partial sums), which it grows with cudaMalloc through a
// gmi_context; this variant takes its scratch from a fixed array compiled
// into the library instead, so the caller supplies only its inputs and
// outputs.
//
// The array, kScratchBytes (16 MiB), is a file-scope __device__ variable:
// every GPU that loads the library holds it until the process exits.  It
// bounds the problem to kMaxSegs segments.  All calls share it and it keeps
// the contents of the last call, so two calls that overlap on the GPU
// (different streams, or different host threads on one device) race on it.
#include <map>
#include <mutex>

#include "gmi_context.hpp"
#include "gmi_pair_kernels.hpp"

namespace {

constexpr size_t kScratchBytes = size_t(16) << 20;
constexpr int kMaxSegs = 32768;
constexpr size_t kErrBytes = 256;  // the device error word, then records, then partial sums

__device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

// Per-context set-up, done on the first call in a CUDA context with that
// context current: the device address of g_noalloc_scratch (in host code the
// name g_noalloc_scratch is only a host-side stand-in, not a device
// address), the SM count, and the driver's tensor-map encoder.  The address
// belongs to the context the module was loaded into, so the table is keyed
// by the current driver context (the device's primary context for runtime
// API callers; a context of the caller's own made current with
// cuCtxSetCurrent gets its own entry).
struct DeviceSetup {
    unsigned char *scratch = nullptr;
    int sm_count = 0;
    void *encode_tiled = nullptr;
    bool ready = false;
};

std::map<CUcontext, DeviceSetup> g_setup;
std::mutex g_setup_mutex;
using CtxGetCurrentFn = CUresult (*)(CUcontext *);

gmi_status current_driver_context(CUcontext *ctx)
{
    static CtxGetCurrentFn get_current = nullptr;
    if (get_current == nullptr) {
        cudaDriverEntryPointQueryResult q;
        void *fn = nullptr;
        GMI_CUDA_TRY(cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &fn, 12000, cudaEnableDefault, &q));
        if (q != cudaDriverEntryPointSuccess || fn == nullptr) {
            gmi::set_last_error_msg("driver does not provide cuCtxGetCurrent");
            return GMI_ERR_CUDA;
        }
        get_current = reinterpret_cast<CtxGetCurrentFn>(fn);
    }
    *ctx = nullptr;
    if (get_current(ctx) != CUDA_SUCCESS || *ctx == nullptr) {
        gmi::set_last_error_msg("gmi_Mss_mult_noalloc: no current CUDA context");
        return GMI_ERR_CUDA;
    }
    return GMI_OK;
}

gmi_status scratch_address(void **p)
{
    *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(p, g_noalloc_scratch);
    if (e != cudaSuccess || *p == nullptr) {
        gmi::set_last_error(cudaGetErrorString(e), "cudaGetSymbolAddress(g_noalloc_scratch)", __FILE__, __LINE__);
        return GMI_ERR_CUDA;
    }
    return GMI_OK;
}

gmi_status setup_current_device(DeviceSetup **out)
{
    int dev = 0;
    GMI_CUDA_TRY(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    CUcontext cu = nullptr;
    void *p = nullptr;
    if (current_driver_context(&cu) != GMI_OK) {
        // no context is current on this thread yet: the symbol lookup makes
        // the runtime bind the device's primary context, which is then current
        gmi_status ps = scratch_address(&p);
        if (ps != GMI_OK) return ps;
        ps = current_driver_context(&cu);
        if (ps != GMI_OK) return ps;
    }
    DeviceSetup &d = g_setup[cu];
    if (!d.ready) {
        if (p == nullptr) {
            gmi_status ps = scratch_address(&p);
            if (ps != GMI_OK) return ps;
        }
        int sms = 0;
        GMI_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        cudaDriverEntryPointQueryResult q;
        void *fn = nullptr;
        GMI_CUDA_TRY(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q));
        if (q != cudaDriverEntryPointSuccess || fn == nullptr) {
            gmi::set_last_error_msg("driver does not provide cuTensorMapEncodeTiled");
            return GMI_ERR_CUDA;
        }
        d.scratch = static_cast<unsigned char *>(p);
        d.sm_count = sms;
        d.encode_tiled = fn;
        d.ready = true;
    }
    *out = &d;
    return GMI_OK;
}

}  // namespace

extern "C" gmi_status gmi_Mss_mult_noalloc(double *V_d, const double *F_d, const double *X_d, int start_seg,
                                           int num_segs, int total_segs, double rseg, double mu, int precision,
                                           void *cuda_stream)
{
    using namespace gmi;
    if (num_segs == 0) return GMI_OK;
    if (!(V_d && F_d && X_d)) {
        set_last_error_msg("gmi_Mss_mult_noalloc: null argument");
        return GMI_ERR_ARG;
    }
    if (!(start_seg >= 0 && num_segs >= 0 && (long long)start_seg + num_segs <= (long long)total_segs)) {
        set_last_error_msg("gmi_Mss_mult_noalloc: target range outside [0, total_segs)");
        return GMI_ERR_ARG;
    }
    if (total_segs > kMaxSegs) {
        set_last_error_msg("gmi_Mss_mult_noalloc: total_segs exceeds the fixed scratch limit of 32768 segments; "
                           "use gmi_Mss_mult");
        return GMI_ERR_ARG;
    }
    if (!(rseg > 0 && mu > 0) || (precision != GMI_FP64 && precision != GMI_FP32C)) {
        set_last_error_msg("gmi_Mss_mult_noalloc: bad radius, viscosity or precision");
        return GMI_ERR_ARG;
    }
    DeviceSetup *d = nullptr;
    gmi_status st = setup_current_device(&d);
    if (st != GMI_OK) return st;
    const bool f64 = precision == GMI_FP64;
    cudaStream_t stream = static_cast<cudaStream_t>(cuda_stream);
    unsigned *err = reinterpret_cast<unsigned *>(d->scratch);
    unsigned char *records = d->scratch + kErrBytes;
    const size_t rec_bytes = (size_t)total_segs * record_bytes(f64);
    const size_t part_off = (kErrBytes + rec_bytes + 255) / 256 * 256;
    double *partial = reinterpret_cast<double *>(d->scratch + part_off);
    // the error word must start at zero; records and partials are fully
    // rewritten before they are read
    GMI_CUDA_TRY(cudaMemsetAsync(err, 0, sizeof(unsigned), stream));
    st = pack_records_into(stream, f64, X_d, F_d, 6, total_segs, records);
    if (st != GMI_OK) return st;
    PairConsts k;
    fill_consts(k, rseg, rseg, rseg, mu);
    ExplicitPairEnv env{};
    env.stream = stream;
    env.partial = partial;
    env.partial_bytes = kScratchBytes - part_off;
    env.err = err;
    env.encode_tiled = d->encode_tiled;
    env.sm_count = d->sm_count;
    const bool small = (long long)num_segs * 2 < (long long)d->sm_count * 256;
    env.tpb = small ? 64 : 128;
    env.tt = (small || !f64) ? 1 : 2;  // FP32: the packed kernel, one target per thread
    st = launch_pair_into(env, kSS, f64, records, start_seg, num_segs, records, total_segs, k, V_d, 0);
    if (st != GMI_OK) return st;
    // V is complete when this returns; report a bounded-wait timeout, if any
    unsigned h_err = 0;
    GMI_CUDA_TRY(cudaMemcpyAsync(&h_err, err, sizeof(unsigned), cudaMemcpyDeviceToHost, stream));
    GMI_CUDA_TRY(cudaStreamSynchronize(stream));
    if (h_err & kDevErrWaitTimeout) {
        set_last_error_msg("gmi_Mss_mult_noalloc: a bounded mbarrier wait timed out; V is invalid");
        return GMI_ERR_DEVICE_TIMEOUT;
    }
    return GMI_OK;
}
