// gmi_context.cu -- context lifetime, scratch buffers, error reporting.
#include <cstdio>
#include <cstring>
#include <map>
#include <tuple>
#include <mutex>
#include <string>
#include <utility>

#include "gmi_context.hpp"

namespace gmi {

static thread_local std::string g_last_error;

void set_last_error(const char *what, const char *expr, const char *file, int line)
{
    char buf[512];
    snprintf(buf, sizeof buf, "%s (%s at %s:%d)", what, expr, file, line);
    g_last_error = buf;
}

void set_last_error_msg(const char *msg) { g_last_error = msg; }

const char *last_error() { return g_last_error.c_str(); }

std::recursive_mutex &device_sync_mutex()
{
    static std::recursive_mutex mu;
    return mu;
}

cudaError_t dev_malloc_bytes(void **p, size_t bytes)
{
    std::lock_guard<std::recursive_mutex> lock(device_sync_mutex());
    return cudaMalloc(p, bytes);
}

cudaError_t dev_free(void *p)
{
    std::lock_guard<std::recursive_mutex> lock(device_sync_mutex());
    return cudaFree(p);
}

cudaError_t host_alloc_bytes(void **p, size_t bytes, unsigned flags)
{
    std::lock_guard<std::recursive_mutex> lock(device_sync_mutex());
    return cudaHostAlloc(p, bytes, flags);
}

cudaError_t host_free(void *p)
{
    std::lock_guard<std::recursive_mutex> lock(device_sync_mutex());
    return cudaFreeHost(p);
}

cudaError_t raise_dynamic_smem_limit(const void *fn, size_t bytes)
{
    static std::mutex mu;
    static std::map<std::pair<int, const void *>, size_t> limits;  // (device, function) -> limit set
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lock(mu);
    size_t &have = limits[{dev, fn}];
    if (bytes <= have) return cudaSuccess;
    e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (e == cudaSuccess) have = bytes;
    return e;
}

cudaError_t max_active_blocks(int *blocks, const void *fn, int threads, size_t smem)
{
    static std::mutex mu;
    static std::map<std::tuple<int, const void *, int, size_t>, int> known;  // (device, function, threads, smem)
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lock(mu);
    const auto key = std::make_tuple(dev, fn, threads, smem);
    const auto it = known.find(key);
    if (it != known.end()) {
        *blocks = it->second;
        return cudaSuccess;
    }
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, fn, threads, smem);
    if (e == cudaSuccess) known[key] = *blocks;
    return e;
}

gmi_status DeviceBuffer::reserve(size_t need)
{
    if (need <= bytes) return GMI_OK;
    if (ptr) {
        cudaError_t e = dev_free(ptr);
        ptr = nullptr;
        bytes = 0;
        if (e != cudaSuccess) {
            set_last_error(cudaGetErrorString(e), "cudaFree", __FILE__, __LINE__);
            return GMI_ERR_CUDA;
        }
    }
    // round up to 2 MiB so that small growth steps do not reallocate
    const size_t grain = size_t(2) << 20;
    const size_t alloc = (need + grain - 1) / grain * grain;
    cudaError_t e = dev_malloc(&ptr, alloc);
    if (e != cudaSuccess) {
        ptr = nullptr;
        set_last_error(cudaGetErrorString(e), "cudaMalloc", __FILE__, __LINE__);
        return GMI_ERR_CUDA;
    }
    bytes = alloc;
    return GMI_OK;
}

void DeviceBuffer::release()
{
    if (ptr) dev_free(ptr);
    ptr = nullptr;
    bytes = 0;
}

gmi_status context_init(gmi_context *ctx, int device)
{
    int count = 0;
    GMI_CUDA_TRY(cudaGetDeviceCount(&count));
    if (device < 0 || device >= count) {
        set_last_error_msg("device index out of range");
        return GMI_ERR_ARG;
    }
    ctx->device = device;
    GMI_CUDA_TRY(cudaSetDevice(device));
    GMI_CUDA_TRY(cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, device));
    GMI_CUDA_TRY(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
    ctx->own_stream = true;
    GMI_CUDA_TRY(dev_malloc(&ctx->d_err, sizeof(unsigned)));
    // stream-ordered and complete before the caller can launch anything
    GMI_CUDA_TRY(cudaMemsetAsync(ctx->d_err, 0, sizeof(unsigned), ctx->stream));
    GMI_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    GMI_CUDA_TRY(host_alloc(&ctx->h_err, sizeof(unsigned)));
    *ctx->h_err = 0;
    cudaDriverEntryPointQueryResult q;
    void *fn = nullptr;
    GMI_CUDA_TRY(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q));
    if (q != cudaDriverEntryPointSuccess || fn == nullptr) {
        set_last_error_msg("driver does not provide cuTensorMapEncodeTiled");
        return GMI_ERR_CUDA;
    }
    ctx->encode_tiled = fn;
    return GMI_OK;
}

gmi_status context_check_device_errors(gmi_context *ctx)
{
    GMI_CUDA_TRY(cudaMemcpyAsync(ctx->h_err, ctx->d_err, sizeof(unsigned), cudaMemcpyDeviceToHost, ctx->stream));
    GMI_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    const unsigned e = *ctx->h_err;
    if (e != 0) {
        GMI_CUDA_TRY(cudaMemsetAsync(ctx->d_err, 0, sizeof(unsigned), ctx->stream));
        GMI_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
        if (e & kDevErrWaitTimeout) {
            set_last_error_msg("a kernel's bounded mbarrier wait timed out; its results are invalid");
            return GMI_ERR_DEVICE_TIMEOUT;
        }
        set_last_error_msg("a kernel reported a non-finite value");
        return GMI_ERR_NONFINITE;
    }
    return GMI_OK;
}

}  // namespace gmi
