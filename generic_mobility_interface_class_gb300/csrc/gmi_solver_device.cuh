// gmi_solver_device.cuh -- device helpers shared by the linear-solver
// kernels (the graph-replayed Arnoldi step and the persistent solve).
#pragma once

#include <cuda_runtime.h>

namespace gmi {

__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// Warp sums of six values per lane by recursive halving: each level swaps
// half of the remaining values with the partner lane and adds the other
// half, so the six totals cost 9 FP64 adds per lane instead of the 30 of six
// shuffle trees (a warp FP64 instruction costs the same on one lane as on
// 32).  Lanes 4c .. 4c+3 return the total of value c (c < 6); lanes 24..31
// return the zero padding's.
__device__ __forceinline__ double warp_sum6_scatter(const double v[6])
{
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const bool h16 = (lane & 16) != 0, h8 = (lane & 8) != 0, h4 = (lane & 4) != 0;
    const double a[8] = {v[0], v[1], v[2], v[3], v[4], v[5], 0.0, 0.0};
    double b[4], c[2];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const double keep = h16 ? a[j + 4] : a[j], send = h16 ? a[j] : a[j + 4];
        b[j] = keep + __shfl_xor_sync(full, send, 16);
    }
#pragma unroll
    for (int j = 0; j < 2; ++j) {
        const double keep = h8 ? b[j + 2] : b[j], send = h8 ? b[j] : b[j + 2];
        c[j] = keep + __shfl_xor_sync(full, send, 8);
    }
    double d = (h4 ? c[1] : c[0]) + __shfl_xor_sync(full, h4 ? c[0] : c[1], 4);
    d += __shfl_xor_sync(full, d, 2);
    d += __shfl_xor_sync(full, d, 1);
    return d;
}

// True in every thread of the CTA that arrives last (of `total`) at *ticket;
// that CTA re-arms the ticket for the next launch.  Partials written before
// the call are visible to the last CTA through L2 (__ldcg).
// The block barrier orders the CTA's writes before thread 0's release fence
// (a CTA barrier synchronises, and a release is cumulative over what
// precedes it), so one thread fences for the whole CTA; the last CTA's
// acquire fence, then its block barrier, make every partial visible to all
// of its threads.
__device__ __forceinline__ bool last_cta(int *ticket, int total)
{
    __shared__ int is_last;
    __syncthreads();
    if (threadIdx.x == 0) {
        asm volatile("fence.acq_rel.gpu;" ::: "memory");
        const int t = atomicAdd(ticket, 1);
        is_last = (t == total - 1);
        if (is_last) {
            *ticket = 0;
            asm volatile("fence.acq_rel.gpu;" ::: "memory");
        }
    }
    __syncthreads();
    return is_last;
}

// o = R v, R row-major 3x3
__device__ __forceinline__ void rot_apply(const double *R, const double *v, double *o)
{
    o[0] = R[0] * v[0] + R[1] * v[1] + R[2] * v[2];
    o[1] = R[3] * v[0] + R[4] * v[1] + R[5] * v[2];
    o[2] = R[6] * v[0] + R[7] * v[1] + R[8] * v[2];
}

// The pair kernels' 12-scalar record of blob i (position x, force f): FP64
// [x y z fx fy fz 0 0 0 0 0 0]; FP32C [xh yh zh fx][xl yl zl fy][fz 0 0 0]
// with the position as a double-float (hi, lo) pair.
__device__ __forceinline__ void pack_record(void *rec, int i, const double *x, const double *f, int f64)
{
    if (f64) {
        double2 *r = static_cast<double2 *>(rec) + 6 * (size_t)i;
        r[0] = make_double2(x[0], x[1]);
        r[1] = make_double2(x[2], f[0]);
        r[2] = make_double2(f[1], f[2]);
        r[3] = make_double2(0.0, 0.0);
        r[4] = make_double2(0.0, 0.0);
        r[5] = make_double2(0.0, 0.0);
    } else {
        const float hx = (float)x[0], hy = (float)x[1], hz = (float)x[2];
        float4 *r = static_cast<float4 *>(rec) + 3 * (size_t)i;
        r[0] = make_float4(hx, hy, hz, (float)f[0]);
        r[1] = make_float4((float)(x[0] - (double)hx), (float)(x[1] - (double)hy), (float)(x[2] - (double)hz),
                           (float)f[1]);
        r[2] = make_float4((float)f[2], 0.f, 0.f, 0.f);
    }
}

}  // namespace gmi
