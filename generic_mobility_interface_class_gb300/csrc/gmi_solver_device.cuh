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
