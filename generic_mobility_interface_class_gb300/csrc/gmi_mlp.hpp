// gmi_mlp.hpp -- the MLP object and its GEMM, shared by the training entry
// points (gmi_mlp.cu) and the time step that runs the network for its
// learned initial inverse Jacobian (gmi_sim.cu).
#pragma once

#include <cuda_bf16.h>

#include <vector>

#include "gmi_context.hpp"

namespace gmi {

// C = A B with bf16 operands addressed through strides (element (m, k) of A
// at A[m sam + k sak], (k, n) of B at B[k sbk + n sbn]), FP32 accumulation;
// epilogue in this order: + bias[n], relu, times [mask(m, n) > 0]; stored to
// C32 (FP32) and/or C16 (bf16, round to nearest even) through strides.
struct GemmArgs {
    int M = 0, N = 0, K = 0;
    const __nv_bfloat16 *A = nullptr;
    long long sam = 0, sak = 0;
    const __nv_bfloat16 *B = nullptr;
    long long sbk = 0, sbn = 0;
    const float *bias = nullptr;
    int relu = 0;
    const __nv_bfloat16 *mask = nullptr;
    long long smm = 0, smn = 0;
    float *C32 = nullptr;
    long long scm = 0, scn = 0;
    __nv_bfloat16 *C16 = nullptr;
    long long s16m = 0, s16n = 0;
};

gmi_status gemm_bf16(cudaStream_t stream, const GemmArgs &g);

}  // namespace gmi

struct gmi_mlp {
    int device = 0;
    int n_in = 0, n_hidden = 0, n_out = 0;
    cudaStream_t stream = nullptr;
    // flat parameters W1 b1 W2 b2 W3 b3 (off[] in elements; W row-major [out x in])
    long long off[6] = {0, 0, 0, 0, 0, 0};
    long long nparam = 0;
    float *p32 = nullptr, *grad = nullptr, *m1 = nullptr, *m2 = nullptr;
    __nv_bfloat16 *p16 = nullptr;
    int adam_t = 0;
    long long train_steps = 0;
    long long launches = 0;
    // batch workspace of the training entry points (grown on demand)
    int cap_batch = 0;
    __nv_bfloat16 *X16 = nullptr, *H1 = nullptr, *H2 = nullptr, *dO16 = nullptr, *dZ2 = nullptr, *dZ1 = nullptr;
    float *X32 = nullptr, *O = nullptr, *dO = nullptr, *loss = nullptr, *loss_mean = nullptr;
    int *idx = nullptr;
    std::vector<void *> allocs, batch_allocs;
};

namespace gmi {
// Forward with caller-owned activations (the weights are only read, so
// several time steps on several streams may share one network).
gmi_status mlp_forward_ws(const gmi_mlp *m, cudaStream_t st, const __nv_bfloat16 *X16, int batch, __nv_bfloat16 *H1,
                          __nv_bfloat16 *H2, float *O);
}  // namespace gmi
