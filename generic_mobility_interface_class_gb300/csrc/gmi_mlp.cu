// gmi_mlp.cu -- the learned initial inverse Jacobian: a 3-layer MLP with
// bf16 weights and activations and FP32 accumulation, its training kernels,
// and the secant-pair loss that fits it.  No counterpart in the reference.
//
// Network: X [B x n_in] -> H1 = relu(X W1^T + b1) -> H2 = relu(H1 W2^T + b2)
// -> O = H2 W3^T + b3.  W_l is [n_out_l x n_in_l] row-major; X, H1, H2 are
// stored in bf16 (round to nearest even), O in FP32.  Every product runs on
// the tensor cores as mma.sync m16n8k16 bf16 x bf16 -> f32: these GEMMs are a
// few hundred MFLOP (batches of a few hundred filaments, width 256), far too
// small for tcgen05's 128-row tiles and TMEM staging to pay for themselves.
//
// Backward (the exact gradient of that bf16-rounded forward):
//   dO16 = bf16(dO)                  db3 = colsum(dO16)   dW3 = dO16^T H2
//   dZ2  = bf16((dO16 W3) * [H2>0])  db2 = colsum(dZ2)    dW2 = dZ2^T H1
//   dZ1  = bf16((dZ2 W2) * [H1>0])   db1 = colsum(dZ1)    dW1 = dZ1^T X
// with FP32 accumulation and FP32 gradients; Adam keeps FP32 master weights
// and rewrites their bf16 copies.
//
// Secant-pair head.  For one filament of nseg segments (n6 = 6 nseg Broyden
// unknowns, nblk = 2 nseg three-vectors) the output row holds
//   s[nblk]      log-scales, sigma = exp(clamp(s, -3, 3)), one per 3-vector
//   U[n6 x r]    row-major, then V[n6 x r]
// and the learned initial inverse Jacobian of that filament is
//   H0 d = sigma (.) b + U (V^T d),   b = conf Jinv_approx d,
// in the filament's local frame.  A training record (FP32) is
//   [phi (n_in) | d (n6) | b (n6) | t (n6)]
// with d = the change of the Broyden error over one iteration, b = conf
// Jinv_approx d, t = the update that produced it (the secant pair of that
// iteration), all rotated into the filament's local frame.  The loss of a
// record is |H0 d - t|^2 / (|t|^2 + eps), averaged over the batch.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "gmi_mlp.hpp"

namespace gmi {

// ---------------------------------------------------------------------------
// GEMM: C[M x N] = sum_k A(m, k) B(k, n), bf16 operands through strides,
// FP32 accumulation on mma.sync m16n8k16; epilogue: + bias[n], relu, times
// [mask(m, n) > 0], stored as FP32 and/or bf16 through strides.
// 64 x 64 CTA tile, K step 32, four warps of 32 x 32.
// ---------------------------------------------------------------------------
constexpr int kGBM = 64, kGBN = 64, kGBK = 32, kGTpb = 128;
constexpr int kGPad = 8;  // bf16 padding of a shared row (conflict-free fragment loads)

__device__ __forceinline__ void mma_bf16_16816(float *c, const unsigned *a, const unsigned *b)
{
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

__global__ void __launch_bounds__(kGTpb) gemm_bf16_kernel(GemmArgs g)
{
    __shared__ __align__(16) __nv_bfloat16 As[kGBM][kGBK + kGPad];
    __shared__ __align__(16) __nv_bfloat16 Bs[kGBN][kGBK + kGPad];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int m0 = blockIdx.y * kGBM, n0 = blockIdx.x * kGBN;
    const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;
    const int gq = lane >> 2, tq = lane & 3;
    float acc[2][4][4];
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int e = 0; e < 4; ++e) acc[i][j][e] = 0.f;
    const __nv_bfloat16 zero = __float2bfloat16_rn(0.f);
    for (int k0 = 0; k0 < g.K; k0 += kGBK) {
        // tiles: the index that is contiguous in memory runs fastest over threads
        for (int e = tid; e < kGBM * kGBK; e += kGTpb) {
            int r, c;
            if (g.sak == 1) { r = e / kGBK; c = e % kGBK; } else { r = e % kGBM; c = e / kGBM; }
            const int m = m0 + r, k = k0 + c;
            As[r][c] = (m < g.M && k < g.K) ? g.A[(long long)m * g.sam + (long long)k * g.sak] : zero;
        }
        for (int e = tid; e < kGBN * kGBK; e += kGTpb) {
            int r, c;
            if (g.sbk == 1) { r = e / kGBK; c = e % kGBK; } else { r = e % kGBN; c = e / kGBN; }
            const int n = n0 + r, k = k0 + c;
            Bs[r][c] = (n < g.N && k < g.K) ? g.B[(long long)k * g.sbk + (long long)n * g.sbn] : zero;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < kGBK; kk += 16) {
            unsigned a[2][4], b[4][2];
#pragma unroll
            for (int i = 0; i < 2; ++i) {
                const int r = wm + 16 * i + gq;
                a[i][0] = *reinterpret_cast<const unsigned *>(&As[r][kk + 2 * tq]);
                a[i][1] = *reinterpret_cast<const unsigned *>(&As[r + 8][kk + 2 * tq]);
                a[i][2] = *reinterpret_cast<const unsigned *>(&As[r][kk + 2 * tq + 8]);
                a[i][3] = *reinterpret_cast<const unsigned *>(&As[r + 8][kk + 2 * tq + 8]);
            }
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int r = wn + 8 * j + gq;
                b[j][0] = *reinterpret_cast<const unsigned *>(&Bs[r][kk + 2 * tq]);
                b[j][1] = *reinterpret_cast<const unsigned *>(&Bs[r][kk + 2 * tq + 8]);
            }
#pragma unroll
            for (int i = 0; i < 2; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) mma_bf16_16816(acc[i][j], a[i], b[j]);
        }
        __syncthreads();
    }
    // epilogue: c0, c1 at (row g, cols 2t, 2t+1); c2, c3 at (row g+8, ...)
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                const int m = m0 + wm + 16 * i + gq + (e >= 2 ? 8 : 0);
                const int n = n0 + wn + 8 * j + 2 * tq + (e & 1);
                if (m >= g.M || n >= g.N) continue;
                float v = acc[i][j][e];
                if (g.bias) v += g.bias[n];
                if (g.relu) v = fmaxf(v, 0.f);
                if (g.mask && !(__bfloat162float(g.mask[(long long)m * g.smm + (long long)n * g.smn]) > 0.f))
                    v = 0.f;
                if (g.C32) g.C32[(long long)m * g.scm + (long long)n * g.scn] = v;
                if (g.C16) g.C16[(long long)m * g.s16m + (long long)n * g.s16n] = __float2bfloat16_rn(v);
            }
}

gmi_status gemm_bf16(cudaStream_t stream, const GemmArgs &g)
{
    if (g.M <= 0 || g.N <= 0) return GMI_OK;
    const dim3 grid((g.N + kGBN - 1) / kGBN, (g.M + kGBM - 1) / kGBM);
    gemm_bf16_kernel<<<grid, kGTpb, 0, stream>>>(g);
    GMI_CUDA_TRY(cudaGetLastError());
    return GMI_OK;
}

// ---------------------------------------------------------------------------
// small kernels
// ---------------------------------------------------------------------------
__global__ void to_bf16_kernel(const float *__restrict__ x, long long n, __nv_bfloat16 *__restrict__ y)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        y[i] = __float2bfloat16_rn(x[i]);
}

// db[n] = sum over rows of G[m, n] (bf16), FP32, rows in order
__global__ void colsum_bf16_kernel(const __nv_bfloat16 *__restrict__ G, int M, int N, float *__restrict__ db)
{
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= N) return;
    float s = 0.f;
    for (int m = 0; m < M; ++m) s += __bfloat162float(G[(long long)m * N + n]);
    db[n] = s;
}

// Adam over the flat FP32 parameter array, rewriting the bf16 copy.
__global__ void adam_kernel(float *__restrict__ p, const float *__restrict__ g, float *__restrict__ m1,
                            float *__restrict__ m2, __nv_bfloat16 *__restrict__ p16, long long n, float lr, float b1,
                            float b2, float eps, float c1, float c2)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float a = b1 * m1[i] + (1.f - b1) * gi;
        const float v = b2 * m2[i] + (1.f - b2) * gi * gi;
        m1[i] = a;
        m2[i] = v;
        const float w = p[i] - lr * (a * c1) / (sqrtf(v * c2) + eps);
        p[i] = w;
        p16[i] = __float2bfloat16_rn(w);
    }
}

// The minibatch of a training step: record indices drawn with replacement by
// a counter-based hash (splitmix64) of (seed, step, row); the features are
// rounded to bf16 for the first GEMM.
__device__ __forceinline__ unsigned long long splitmix64(unsigned long long z)
{
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

__global__ void gather_batch_kernel(const float *__restrict__ rec, long long nrec, int rec_len, int n_in,
                                    unsigned long long seed, long long step, int batch, int *__restrict__ idx,
                                    __nv_bfloat16 *__restrict__ X)
{
    const int row = blockIdx.x;
    if (row >= batch) return;
    __shared__ long long r;
    if (threadIdx.x == 0) {
        const unsigned long long h = splitmix64(seed ^ splitmix64((unsigned long long)step * 1000003ull + row));
        r = (long long)(h % (unsigned long long)nrec);
        idx[row] = (int)r;
    }
    __syncthreads();
    for (int c = threadIdx.x; c < n_in; c += blockDim.x)
        X[(long long)row * n_in + c] = __float2bfloat16_rn(rec[r * rec_len + c]);
}

// Secant-pair loss and its gradient with respect to the output row, one CTA
// per record (see the file comment).  dO is written in full (zeros past the
// head's outputs); loss[row] receives the record's loss.
template <int R>
__global__ void __launch_bounds__(128) secant_head_kernel(const float *__restrict__ O, int n_out,
                                                          const float *__restrict__ rec, int rec_len, int n_in,
                                                          const int *__restrict__ idx, int nseg, int batch,
                                                          float *__restrict__ dO, float *__restrict__ loss)
{
    const int row = blockIdx.x, tid = threadIdx.x;
    const int n6 = 6 * nseg, nblk = 2 * nseg;
    extern __shared__ float sh[];
    float *d = sh, *b = d + n6, *t = b + n6, *gp = t + n6;  // gp: dL/dpred
    __shared__ float y[R], dy[R], red[4][R + 1];
    const float *o = O + (long long)row * n_out;
    const float *U = o + nblk, *V = U + n6 * R;
    const float *r0 = rec + (long long)(idx ? idx[row] : row) * rec_len + n_in;
    for (int i = tid; i < n6; i += 128) {
        d[i] = r0[i];
        b[i] = r0[n6 + i];
        t[i] = r0[2 * n6 + i];
    }
    __syncthreads();
    // y = V^T d
    float yp[R];
#pragma unroll
    for (int j = 0; j < R; ++j) yp[j] = 0.f;
    for (int i = tid; i < n6; i += 128)
#pragma unroll
        for (int j = 0; j < R; ++j) yp[j] += V[i * R + j] * d[i];
    const int lane = tid & 31, w = tid >> 5;
#pragma unroll
    for (int j = 0; j < R; ++j) {
        float v = yp[j];
        for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
        if (lane == 0) red[w][j] = v;
    }
    __syncthreads();
    if (tid < R) y[tid] = red[0][tid] + red[1][tid] + red[2][tid] + red[3][tid];
    __syncthreads();
    // residual e = sigma b + U y - t, and |t|^2
    float ee = 0.f, tt = 0.f;
    for (int i = tid; i < n6; i += 128) {
        const float s = fminf(fmaxf(o[i / 3], -3.f), 3.f);
        float p = expf(s) * b[i];
#pragma unroll
        for (int j = 0; j < R; ++j) p += U[i * R + j] * y[j];
        const float e = p - t[i];
        gp[i] = e;
        ee += e * e;
        tt += t[i] * t[i];
    }
    for (int off = 16; off > 0; off >>= 1) {
        ee += __shfl_xor_sync(0xffffffffu, ee, off);
        tt += __shfl_xor_sync(0xffffffffu, tt, off);
    }
    __shared__ float sums[2][4];
    if (lane == 0) {
        sums[0][w] = ee;
        sums[1][w] = tt;
    }
    __syncthreads();
    const float E = sums[0][0] + sums[0][1] + sums[0][2] + sums[0][3];
    const float T = sums[1][0] + sums[1][1] + sums[1][2] + sums[1][3] + 1e-30f;
    if (tid == 0) loss[row] = E / T;
    const float scale = 2.f / (T * (float)batch);
    for (int i = tid; i < n6; i += 128) gp[i] *= scale;
    __syncthreads();
    // dy = U^T gp
#pragma unroll
    for (int j = 0; j < R; ++j) yp[j] = 0.f;
    for (int i = tid; i < n6; i += 128)
#pragma unroll
        for (int j = 0; j < R; ++j) yp[j] += U[i * R + j] * gp[i];
#pragma unroll
    for (int j = 0; j < R; ++j) {
        float v = yp[j];
        for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
        if (lane == 0) red[w][j] = v;
    }
    __syncthreads();
    if (tid < R) dy[tid] = red[0][tid] + red[1][tid] + red[2][tid] + red[3][tid];
    __syncthreads();
    float *dr = dO + (long long)row * n_out;
    // d/ds: sum over the 3-vector of gp b sigma (zero where clamped)
    for (int k = tid; k < nblk; k += 128) {
        const float sr = o[k];
        const float s = fminf(fmaxf(sr, -3.f), 3.f);
        float a = 0.f;
        for (int c = 0; c < 3; ++c) a += gp[3 * k + c] * b[3 * k + c];
        dr[k] = (sr > -3.f && sr < 3.f) ? a * expf(s) : 0.f;
    }
    for (int e = tid; e < n6 * R; e += 128) {
        const int i = e / R, j = e % R;
        dr[nblk + e] = gp[i] * y[j];           // dU
        dr[nblk + n6 * R + e] = d[i] * dy[j];  // dV
    }
    for (int e = nblk + 2 * n6 * R + tid; e < n_out; e += 128) dr[e] = 0.f;
}

__global__ void sum_kernel(const float *__restrict__ x, int n, float *__restrict__ out)
{
    __shared__ float red[256];
    float s = 0.f;
    for (int i = threadIdx.x; i < n; i += 256) s += x[i];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = red[0] / (float)n;
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
static gmi_status mlp_alloc(gmi_mlp *m, void **p, size_t bytes)
{
    GMI_CUDA_TRY(dev_malloc(p, bytes < 16 ? 16 : bytes));
    m->allocs.push_back(*p);
    GMI_CUDA_TRY(cudaMemsetAsync(*p, 0, bytes < 16 ? 16 : bytes, m->stream));
    return GMI_OK;
}

gmi_status mlp_reserve_batch(gmi_mlp *m, int batch)
{
    if (batch <= m->cap_batch) return GMI_OK;
    for (void *p : m->batch_allocs) dev_free(p);
    m->batch_allocs.clear();
    auto al = [&](void **p, size_t bytes) -> gmi_status {
        GMI_CUDA_TRY(dev_malloc(p, bytes < 16 ? 16 : bytes));
        m->batch_allocs.push_back(*p);
        return GMI_OK;
    };
    const size_t B = (size_t)batch;
    GMI_TRY(al((void **)&m->X16, B * m->n_in * 2));
    GMI_TRY(al((void **)&m->X32, B * m->n_in * 4));
    GMI_TRY(al((void **)&m->H1, B * m->n_hidden * 2));
    GMI_TRY(al((void **)&m->H2, B * m->n_hidden * 2));
    GMI_TRY(al((void **)&m->O, B * m->n_out * 4));
    GMI_TRY(al((void **)&m->dO, B * m->n_out * 4));
    GMI_TRY(al((void **)&m->dO16, B * m->n_out * 2));
    GMI_TRY(al((void **)&m->dZ2, B * m->n_hidden * 2));
    GMI_TRY(al((void **)&m->dZ1, B * m->n_hidden * 2));
    GMI_TRY(al((void **)&m->idx, B * 4));
    GMI_TRY(al((void **)&m->loss, B * 4));
    m->cap_batch = batch;
    return GMI_OK;
}

gmi_status mlp_forward_ws(const gmi_mlp *m, cudaStream_t st, const __nv_bfloat16 *X16, int batch,
                          __nv_bfloat16 *H1, __nv_bfloat16 *H2, float *O)
{
    GemmArgs g{};
    // H1 = relu(X W1^T + b1)
    g.M = batch; g.N = m->n_hidden; g.K = m->n_in;
    g.A = X16; g.sam = m->n_in; g.sak = 1;
    g.B = m->p16 + m->off[0]; g.sbk = 1; g.sbn = m->n_in;
    g.bias = m->p32 + m->off[1]; g.relu = 1;
    g.C16 = H1; g.s16m = m->n_hidden; g.s16n = 1;
    GMI_TRY(gemm_bf16(st, g));
    // H2 = relu(H1 W2^T + b2)
    g.K = m->n_hidden; g.A = H1; g.sam = m->n_hidden;
    g.B = m->p16 + m->off[2]; g.sbn = m->n_hidden;
    g.bias = m->p32 + m->off[3];
    g.C16 = H2;
    GMI_TRY(gemm_bf16(st, g));
    // O = H2 W3^T + b3 (FP32)
    GemmArgs h{};
    h.M = batch; h.N = m->n_out; h.K = m->n_hidden;
    h.A = H2; h.sam = m->n_hidden; h.sak = 1;
    h.B = m->p16 + m->off[4]; h.sbk = 1; h.sbn = m->n_hidden;
    h.bias = m->p32 + m->off[5];
    h.C32 = O; h.scm = m->n_out; h.scn = 1;
    return gemm_bf16(st, h);
}

// gradients of the last forward (m->X16, H1, H2) for upstream dO (FP32,
// already holding the 1/B of a mean) into m->grad
static gmi_status mlp_backward_ws(gmi_mlp *m, int batch, const float *dO)
{
    cudaStream_t st = m->stream;
    const int B = batch, nh = m->n_hidden, ni = m->n_in, no = m->n_out;
    const long long ndo = (long long)B * no;
    to_bf16_kernel<<<(int)std::min<long long>((ndo + 255) / 256, 4096), 256, 0, st>>>(dO, ndo, m->dO16);
    colsum_bf16_kernel<<<(no + 127) / 128, 128, 0, st>>>(m->dO16, B, no, m->grad + m->off[5]);
    GMI_CUDA_TRY(cudaGetLastError());
    GemmArgs g{};
    // dW3 = dO16^T H2  [no x nh]
    g.M = no; g.N = nh; g.K = B;
    g.A = m->dO16; g.sam = 1; g.sak = no;
    g.B = m->H2; g.sbk = nh; g.sbn = 1;
    g.C32 = m->grad + m->off[4]; g.scm = nh; g.scn = 1;
    GMI_TRY(gemm_bf16(st, g));
    // dZ2 = bf16((dO16 W3) * [H2 > 0])  [B x nh]
    GemmArgs h{};
    h.M = B; h.N = nh; h.K = no;
    h.A = m->dO16; h.sam = no; h.sak = 1;
    h.B = m->p16 + m->off[4]; h.sbk = nh; h.sbn = 1;
    h.mask = m->H2; h.smm = nh; h.smn = 1;
    h.C16 = m->dZ2; h.s16m = nh; h.s16n = 1;
    GMI_TRY(gemm_bf16(st, h));
    colsum_bf16_kernel<<<(nh + 127) / 128, 128, 0, st>>>(m->dZ2, B, nh, m->grad + m->off[3]);
    GMI_CUDA_TRY(cudaGetLastError());
    // dW2 = dZ2^T H1
    g.M = nh; g.N = nh; g.K = B;
    g.A = m->dZ2; g.sam = 1; g.sak = nh;
    g.B = m->H1; g.sbk = nh; g.sbn = 1;
    g.C32 = m->grad + m->off[2]; g.scm = nh;
    GMI_TRY(gemm_bf16(st, g));
    // dZ1 = bf16((dZ2 W2) * [H1 > 0])
    h.M = B; h.N = nh; h.K = nh;
    h.A = m->dZ2; h.sam = nh;
    h.B = m->p16 + m->off[2]; h.sbk = nh; h.sbn = 1;
    h.mask = m->H1;
    h.C16 = m->dZ1;
    GMI_TRY(gemm_bf16(st, h));
    colsum_bf16_kernel<<<(nh + 127) / 128, 128, 0, st>>>(m->dZ1, B, nh, m->grad + m->off[1]);
    GMI_CUDA_TRY(cudaGetLastError());
    // dW1 = dZ1^T X
    g.M = nh; g.N = ni; g.K = B;
    g.A = m->dZ1; g.sam = 1; g.sak = nh;
    g.B = m->X16; g.sbk = ni; g.sbn = 1;
    g.C32 = m->grad + m->off[0]; g.scm = ni;
    GMI_TRY(gemm_bf16(st, g));
    m->launches += 10;
    return GMI_OK;
}

static int head_outputs(int nseg, int rank) { return 2 * nseg + 2 * 6 * nseg * rank; }

static gmi_status launch_head(cudaStream_t st, const float *O, int n_out, const float *rec, int rec_len, int n_in,
                              const int *idx, int nseg, int rank, int batch, float *dO, float *loss)
{
    const size_t smem = 4 * (size_t)6 * nseg * sizeof(float);
    switch (rank) {
    case 2: secant_head_kernel<2><<<batch, 128, smem, st>>>(O, n_out, rec, rec_len, n_in, idx, nseg, batch, dO, loss); break;
    case 4: secant_head_kernel<4><<<batch, 128, smem, st>>>(O, n_out, rec, rec_len, n_in, idx, nseg, batch, dO, loss); break;
    case 8: secant_head_kernel<8><<<batch, 128, smem, st>>>(O, n_out, rec, rec_len, n_in, idx, nseg, batch, dO, loss); break;
    default: set_last_error_msg("secant head: rank must be 2, 4 or 8"); return GMI_ERR_ARG;
    }
    GMI_CUDA_TRY(cudaGetLastError());
    return GMI_OK;
}

// Kaiming-uniform weights from a seeded splitmix64 stream; the last layer
// scaled by last_scale (small: the network starts near sigma = 1, U V^T = 0,
// i.e. the plain initial inverse Jacobian).
static void init_params(std::vector<float> &p, const gmi_mlp *m, unsigned long long seed, float last_scale)
{
    unsigned long long z = seed;
    auto next = [&]() {
        z += 0x9E3779B97F4A7C15ull;
        unsigned long long x = z;
        x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
        x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
        x ^= x >> 31;
        return (double)(x >> 11) * (1.0 / 9007199254740992.0);  // [0, 1)
    };
    const int fan_in[3] = {m->n_in, m->n_hidden, m->n_hidden};
    const int rows[3] = {m->n_hidden, m->n_hidden, m->n_out};
    for (int l = 0; l < 3; ++l) {
        const double bound = std::sqrt(6.0 / fan_in[l]) * (l == 2 ? last_scale : 1.0);
        float *W = p.data() + m->off[2 * l];
        for (long long i = 0; i < (long long)rows[l] * fan_in[l]; ++i) W[i] = (float)((2.0 * next() - 1.0) * bound);
        float *b = p.data() + m->off[2 * l + 1];
        for (int i = 0; i < rows[l]; ++i) b[i] = 0.f;
    }
}

static gmi_status upload_params(gmi_mlp *m, const float *host)
{
    GMI_CUDA_TRY(cudaMemcpyAsync(m->p32, host, (size_t)m->nparam * 4, cudaMemcpyHostToDevice, m->stream));
    to_bf16_kernel<<<(int)std::min<long long>((m->nparam + 255) / 256, 4096), 256, 0, m->stream>>>(m->p32, m->nparam,
                                                                                                  m->p16);
    GMI_CUDA_TRY(cudaGetLastError());
    GMI_CUDA_TRY(cudaMemsetAsync(m->m1, 0, (size_t)m->nparam * 4, m->stream));
    GMI_CUDA_TRY(cudaMemsetAsync(m->m2, 0, (size_t)m->nparam * 4, m->stream));
    m->adam_t = 0;
    GMI_CUDA_TRY(cudaStreamSynchronize(m->stream));
    return GMI_OK;
}

}  // namespace gmi

using namespace gmi;

#define MLP_ARG_CHECK(cond, msg)     \
    do {                             \
        if (!(cond)) {               \
            set_last_error_msg(msg); \
            return GMI_ERR_ARG;      \
        }                            \
    } while (0)

extern "C" {

gmi_status gmi_mlp_create(int device, int n_in, int n_hidden, int n_out, unsigned long long seed, gmi_mlp **out)
{
    MLP_ARG_CHECK(out != nullptr, "gmi_mlp_create: null out");
    *out = nullptr;
    MLP_ARG_CHECK(n_in > 0 && n_hidden > 0 && n_out > 0 && n_in % 8 == 0 && n_hidden % 8 == 0 && n_out % 8 == 0 &&
                      n_in <= 4096 && n_hidden <= 4096 && n_out <= 16384,
                  "gmi_mlp_create: layer widths must be positive multiples of 8 (n_in, n_hidden <= 4096)");
    GMI_CUDA_TRY(cudaSetDevice(device));
    gmi_mlp *m = new gmi_mlp();
    m->device = device;
    m->n_in = n_in;
    m->n_hidden = n_hidden;
    m->n_out = n_out;
    const long long sizes[6] = {(long long)n_hidden * n_in, n_hidden, (long long)n_hidden * n_hidden, n_hidden,
                                (long long)n_out * n_hidden, n_out};
    long long o = 0;
    for (int l = 0; l < 6; ++l) {
        m->off[l] = o;
        o += (sizes[l] + 7) / 8 * 8;  // 16-byte aligned bf16 and FP32 segments
    }
    m->nparam = o;
    cudaError_t e = cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete m;
        set_last_error(cudaGetErrorString(e), "cudaStreamCreateWithFlags", __FILE__, __LINE__);
        return GMI_ERR_CUDA;
    }
    gmi_status st;
    if ((st = mlp_alloc(m, (void **)&m->p32, (size_t)o * 4)) != GMI_OK ||
        (st = mlp_alloc(m, (void **)&m->p16, (size_t)o * 2)) != GMI_OK ||
        (st = mlp_alloc(m, (void **)&m->grad, (size_t)o * 4)) != GMI_OK ||
        (st = mlp_alloc(m, (void **)&m->m1, (size_t)o * 4)) != GMI_OK ||
        (st = mlp_alloc(m, (void **)&m->m2, (size_t)o * 4)) != GMI_OK ||
        (st = mlp_alloc(m, (void **)&m->loss_mean, 64)) != GMI_OK) {
        gmi_mlp_destroy(m);
        return st;
    }
    std::vector<float> p((size_t)o, 0.f);
    init_params(p, m, seed, 0.05f);
    if ((st = upload_params(m, p.data())) != GMI_OK) {
        gmi_mlp_destroy(m);
        return st;
    }
    *out = m;
    return GMI_OK;
}

gmi_status gmi_mlp_destroy(gmi_mlp *m)
{
    if (m == nullptr) return GMI_OK;
    cudaSetDevice(m->device);
    if (m->stream) cudaStreamSynchronize(m->stream);
    for (void *p : m->batch_allocs) dev_free(p);
    for (void *p : m->allocs) dev_free(p);
    if (m->stream) cudaStreamDestroy(m->stream);
    delete m;
    return GMI_OK;
}

gmi_status gmi_mlp_param_count(const gmi_mlp *m, long long *count)
{
    MLP_ARG_CHECK(m && count, "gmi_mlp_param_count: null argument");
    *count = m->nparam;
    return GMI_OK;
}

gmi_status gmi_mlp_param_offsets(const gmi_mlp *m, long long *offsets6)
{
    MLP_ARG_CHECK(m && offsets6, "gmi_mlp_param_offsets: null argument");
    for (int l = 0; l < 6; ++l) offsets6[l] = m->off[l];
    return GMI_OK;
}

gmi_status gmi_mlp_get_params(gmi_mlp *m, float *host, long long count)
{
    MLP_ARG_CHECK(m && host && count == m->nparam, "gmi_mlp_get_params: null argument or wrong count");
    GMI_CUDA_TRY(cudaSetDevice(m->device));
    GMI_CUDA_TRY(cudaMemcpyAsync(host, m->p32, (size_t)count * 4, cudaMemcpyDeviceToHost, m->stream));
    GMI_CUDA_TRY(cudaStreamSynchronize(m->stream));
    return GMI_OK;
}

gmi_status gmi_mlp_set_params(gmi_mlp *m, const float *host, long long count)
{
    MLP_ARG_CHECK(m && host && count == m->nparam, "gmi_mlp_set_params: null argument or wrong count");
    GMI_CUDA_TRY(cudaSetDevice(m->device));
    return upload_params(m, host);
}

gmi_status gmi_mlp_forward(gmi_mlp *m, const float *X_d, int batch, float *O_d)
{
    MLP_ARG_CHECK(m && X_d && O_d && batch > 0, "gmi_mlp_forward: bad argument");
    GMI_CUDA_TRY(cudaSetDevice(m->device));
    GMI_TRY(mlp_reserve_batch(m, batch));
    const long long nx = (long long)batch * m->n_in;
    to_bf16_kernel<<<(int)std::min<long long>((nx + 255) / 256, 4096), 256, 0, m->stream>>>(X_d, nx, m->X16);
    GMI_CUDA_TRY(cudaGetLastError());
    GMI_TRY(mlp_forward_ws(m, m->stream, m->X16, batch, m->H1, m->H2, m->O));
    GMI_CUDA_TRY(cudaMemcpyAsync(O_d, m->O, (size_t)batch * m->n_out * 4, cudaMemcpyDeviceToDevice, m->stream));
    GMI_CUDA_TRY(cudaStreamSynchronize(m->stream));
    m->launches += 4;
    return GMI_OK;
}

gmi_status gmi_mlp_backward(gmi_mlp *m, const float *dO_d, int batch, float *grad_h)
{
    MLP_ARG_CHECK(m && dO_d && batch > 0 && batch <= m->cap_batch, "gmi_mlp_backward: bad argument (forward first)");
    GMI_CUDA_TRY(cudaSetDevice(m->device));
    GMI_TRY(mlp_backward_ws(m, batch, dO_d));
    if (grad_h)
        GMI_CUDA_TRY(cudaMemcpyAsync(grad_h, m->grad, (size_t)m->nparam * 4, cudaMemcpyDeviceToHost, m->stream));
    GMI_CUDA_TRY(cudaStreamSynchronize(m->stream));
    return GMI_OK;
}

gmi_status gmi_mlp_secant_loss(gmi_mlp *m, const float *records_d, long long nrec, int nseg, int rank,
                               float *O_scratch_d, double *mean_loss, float *dO_d)
{
    MLP_ARG_CHECK(m && records_d && nrec > 0 && nrec <= (1 << 20) && mean_loss && O_scratch_d,
                  "gmi_mlp_secant_loss: bad argument");
    MLP_ARG_CHECK(m->n_in == 6 * nseg && head_outputs(nseg, rank) <= m->n_out,
                  "gmi_mlp_secant_loss: network widths do not match nseg and rank");
    GMI_CUDA_TRY(cudaSetDevice(m->device));
    const int rec_len = m->n_in + 18 * nseg;
    double total = 0.0;
    const int chunk = 4096;
    std::vector<float> lh(chunk);
    for (long long r0 = 0; r0 < nrec; r0 += chunk) {
        const int b = (int)std::min<long long>(chunk, nrec - r0);
        GMI_TRY(mlp_reserve_batch(m, b));
        // features of records r0 .. r0 + b (in order) to bf16
        const float *rec = records_d + r0 * rec_len;
        GMI_CUDA_TRY(cudaMemcpy2DAsync(m->X32, (size_t)m->n_in * 4, rec, (size_t)rec_len * 4, (size_t)m->n_in * 4, b,
                                       cudaMemcpyDeviceToDevice, m->stream));
        const long long nx = (long long)b * m->n_in;
        to_bf16_kernel<<<(int)std::min<long long>((nx + 255) / 256, 4096), 256, 0, m->stream>>>(m->X32, nx, m->X16);
        GMI_CUDA_TRY(cudaGetLastError());
        GMI_TRY(mlp_forward_ws(m, m->stream, m->X16, b, m->H1, m->H2, O_scratch_d));
        GMI_TRY(launch_head(m->stream, O_scratch_d, m->n_out, rec, rec_len, m->n_in, nullptr, nseg, rank, b,
                            dO_d ? dO_d + r0 * m->n_out : m->dO, m->loss));
        GMI_CUDA_TRY(cudaMemcpyAsync(lh.data(), m->loss, (size_t)b * 4, cudaMemcpyDeviceToHost, m->stream));
        GMI_CUDA_TRY(cudaStreamSynchronize(m->stream));
        for (int i = 0; i < b; ++i) total += lh[i];
    }
    *mean_loss = total / (double)nrec;
    return GMI_OK;
}

gmi_status gmi_mlp_train_secant(gmi_mlp *m, const float *records_d, long long nrec, int nseg, int rank, int steps,
                                int batch, float lr, unsigned long long seed, float *loss_h)
{
    MLP_ARG_CHECK(m && records_d && nrec > 0 && steps >= 0 && batch > 0 && batch <= 8192 && lr > 0.f,
                  "gmi_mlp_train_secant: bad argument");
    MLP_ARG_CHECK(m->n_in == 6 * nseg && head_outputs(nseg, rank) <= m->n_out,
                  "gmi_mlp_train_secant: network widths do not match nseg and rank");
    GMI_CUDA_TRY(cudaSetDevice(m->device));
    GMI_TRY(mlp_reserve_batch(m, batch));
    const int rec_len = m->n_in + 18 * nseg;
    cudaStream_t st = m->stream;
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    for (int s = 0; s < steps; ++s) {
        gather_batch_kernel<<<batch, 128, 0, st>>>(records_d, nrec, rec_len, m->n_in, seed, m->train_steps, batch,
                                                   m->idx, m->X16);
        GMI_CUDA_TRY(cudaGetLastError());
        GMI_TRY(mlp_forward_ws(m, st, m->X16, batch, m->H1, m->H2, m->O));
        GMI_TRY(launch_head(st, m->O, m->n_out, records_d, rec_len, m->n_in, m->idx, nseg, rank, batch, m->dO,
                            m->loss));
        GMI_TRY(mlp_backward_ws(m, batch, m->dO));
        ++m->adam_t;
        const float c1 = 1.f / (1.f - std::pow(b1, (float)m->adam_t));
        const float c2 = 1.f / (1.f - std::pow(b2, (float)m->adam_t));
        adam_kernel<<<(int)std::min<long long>((m->nparam + 255) / 256, 4096), 256, 0, st>>>(
            m->p32, m->grad, m->m1, m->m2, m->p16, m->nparam, lr, b1, b2, eps, c1, c2);
        sum_kernel<<<1, 256, 0, st>>>(m->loss, batch, m->loss_mean + (s & 7));
        GMI_CUDA_TRY(cudaGetLastError());
        m->launches += 7;
        ++m->train_steps;
        if (loss_h && ((s & 7) == 7 || s == steps - 1)) {
            const int k0 = s & ~7, nk = s - k0 + 1;
            GMI_CUDA_TRY(cudaMemcpyAsync(loss_h + k0, m->loss_mean, (size_t)nk * 4, cudaMemcpyDeviceToHost, st));
            GMI_CUDA_TRY(cudaStreamSynchronize(st));
        }
    }
    GMI_CUDA_TRY(cudaStreamSynchronize(st));
    return GMI_OK;
}

long long gmi_mlp_launch_count(const gmi_mlp *m) { return m ? m->launches : -1; }

void gmi_learned_policy_init(gmi_learned_policy *p)
{
    if (p == nullptr) return;
    std::memset(p, 0, sizeof *p);
    p->calibration_steps = 3;
    p->window = 8;
    p->max_regressions = 2;
    p->margin = 0.05;
    p->cap_factor = 2.0;
}

int gmi_learned_policy_use_learned(const gmi_learned_policy *p)
{
    if (p == nullptr || p->mode == 2) return 0;
    return (p->mode == 1 || p->steps_plain >= p->calibration_steps) ? 1 : 0;
}

int gmi_learned_policy_iteration_cap(const gmi_learned_policy *p, int max_broyden_iter)
{
    if (p == nullptr || p->steps_plain == 0) return max_broyden_iter;
    const double mean = p->plain_iters_sum / p->steps_plain;
    const int cap = (int)std::ceil(p->cap_factor * mean) + 2;
    return std::max(1, std::min(cap, max_broyden_iter));
}

void gmi_learned_policy_record(gmi_learned_policy *p, int used_learned, int converged, int broyden_iters)
{
    if (p == nullptr) return;
    if (!used_learned) {
        p->steps_plain++;
        p->plain_iters_sum += broyden_iters;
        if (p->mode == 0 && p->steps_plain >= p->calibration_steps) p->mode = 1;
        return;
    }
    p->mode = p->mode == 0 ? 1 : p->mode;
    p->steps_learned++;
    if (!converged) {
        if (++p->regressions >= p->max_regressions) p->mode = 2;
        return;
    }
    p->recent[p->recent_count % 64] = broyden_iters;
    p->recent_count++;
    const int w = std::max(1, std::min(p->window, 64));
    if (p->recent_count >= w && p->steps_plain > 0) {
        double sum = 0.0;
        for (int k = 0; k < w; ++k) sum += p->recent[(p->recent_count - 1 - k) % 64];
        const double plain_mean = p->plain_iters_sum / p->steps_plain;
        if (sum / w > (1.0 + p->margin) * plain_mean) p->mode = 2;
    }
}

}  // extern "C"
