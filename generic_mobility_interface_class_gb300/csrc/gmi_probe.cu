// gmi_probe.cu -- FMA-pipe throughput probe, and the check of the bounded
// mbarrier wait.  The pair kernels are bound by the FP32 (or FP64) FMA pipe,
// not by HBM or the tensor cores, so their roofline denominator is measured
// on the running GPU with fma_probe_kernel: eight independent FMA chains per
// thread, enough CTAs to fill every SM.
#include "gmi_context.hpp"

namespace gmi {

template <class R>
__global__ void __launch_bounds__(256) fma_probe_kernel(R seed, int iters, R *sink)
{
    R a0 = seed + threadIdx.x, a1 = a0 + R(1), a2 = a0 + R(2), a3 = a0 + R(3);
    R a4 = a0 + R(4), a5 = a0 + R(5), a6 = a0 + R(6), a7 = a0 + R(7);
    const R m = R(0.999999), c = R(1e-7);
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int u = 0; u < 16; ++u) {
            a0 = fma(a0, m, c); a1 = fma(a1, m, c); a2 = fma(a2, m, c); a3 = fma(a3, m, c);
            a4 = fma(a4, m, c); a5 = fma(a5, m, c); a6 = fma(a6, m, c); a7 = fma(a7, m, c);
        }
    }
    const R s = ((a0 + a1) + (a2 + a3)) + ((a4 + a5) + (a6 + a7));
    if (s == R(-12345.0)) sink[0] = s;  // never true; keeps the chains live
}

// One CTA waits on an mbarrier that expects two arrivals, through the same
// bounded wait (mbar_wait_bounded) as the pair kernels' source-tile waits.
// With withhold == 0 both arrivals come and the wait completes; with
// withhold == 1 the second never comes (a flag nothing sets), the wait gives
// up after deadline_ns and records kDevErrWaitTimeout, and the kernel
// returns.  No asynchronous copy is involved.
__global__ void bounded_wait_check_kernel(int withhold, unsigned long long deadline_ns, unsigned *err)
{
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 2);
        fence_mbar_init();
    }
    __syncthreads();
    if (threadIdx.x == 0) mbar_arrive(&bar);
    if (threadIdx.x == 1 && withhold == 0) mbar_arrive(&bar);
    if (threadIdx.x == 0 && !mbar_wait_bounded(&bar, 0, deadline_ns)) atomicOr(err, kDevErrWaitTimeout);
}

}  // namespace gmi

using namespace gmi;

extern "C" gmi_status gmi_context_set_wait_deadline(gmi_context *ctx, long long nanoseconds)
{
    if (ctx == nullptr || nanoseconds < 0 || (nanoseconds != 0 && nanoseconds < 1000) ||
        nanoseconds > 60000000000ll) {
        set_last_error_msg("gmi_context_set_wait_deadline: null context, or a deadline outside [1 us, 60 s] "
                           "(0 restores the default of 2 s)");
        return GMI_ERR_ARG;
    }
    ctx->wait_ns = (unsigned long long)nanoseconds;
    return GMI_OK;
}

extern "C" gmi_status gmi_context_check_bounded_wait(gmi_context *ctx, int withhold_arrival)
{
    if (ctx == nullptr || (withhold_arrival != 0 && withhold_arrival != 1)) {
        set_last_error_msg("gmi_context_check_bounded_wait: null context or withhold_arrival not 0/1");
        return GMI_ERR_ARG;
    }
    GMI_CUDA_TRY(cudaSetDevice(ctx->device));
    bounded_wait_check_kernel<<<1, 32, 0, ctx->stream>>>(withhold_arrival, ctx->wait_ns, ctx->d_err);
    GMI_CUDA_TRY(cudaGetLastError());
    ctx->launches++;
    return context_check_device_errors(ctx);
}

extern "C" gmi_status gmi_measure_fma_peak(gmi_context *ctx, int precision, double *flops_per_s)
{
    if (ctx == nullptr || flops_per_s == nullptr) {
        set_last_error_msg("gmi_measure_fma_peak: null argument");
        return GMI_ERR_ARG;
    }
    GMI_CUDA_TRY(cudaSetDevice(ctx->device));
    const bool f64 = precision == GMI_FP64;
    const int blocks = ctx->sm_count * 8, tpb = 256;
    const int iters = f64 ? 64 : 2048;
    gmi_status st = ctx->partial.reserve(64);
    if (st != GMI_OK) return st;
    cudaEvent_t e0, e1;
    GMI_CUDA_TRY(cudaEventCreate(&e0));
    GMI_CUDA_TRY(cudaEventCreate(&e1));
    float best = 1e30f;
    for (int rep = 0; rep < 4; ++rep) {
        GMI_CUDA_TRY(cudaEventRecord(e0, ctx->stream));
        if (f64)
            fma_probe_kernel<double><<<blocks, tpb, 0, ctx->stream>>>(1.0, iters, (double *)ctx->partial.ptr);
        else
            fma_probe_kernel<float><<<blocks, tpb, 0, ctx->stream>>>(1.0f, iters, (float *)ctx->partial.ptr);
        GMI_CUDA_TRY(cudaEventRecord(e1, ctx->stream));
        GMI_CUDA_TRY(cudaEventSynchronize(e1));
        float ms = 0.f;
        GMI_CUDA_TRY(cudaEventElapsedTime(&ms, e0, e1));
        if (rep > 0 && ms < best) best = ms;  // first launch is a warm-up
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    const double fmas = (double)blocks * tpb * iters * 16 * 8;
    *flops_per_s = 2.0 * fmas / (best * 1e-3);
    return GMI_OK;
}
