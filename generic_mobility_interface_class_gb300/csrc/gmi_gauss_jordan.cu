// gmi_gauss_jordan.cu -- in-place inverses of the filament Jacobians
// (column-major n x n FP64 matrices), standing in for the reference's LAPACK
// dgetrf + dgetri (matrix.cpp:538-566).
//
// Gauss-Jordan with partial (row) pivoting: at step k the pivot row p (the
// largest |A(i, k)|, i >= k, lowest i on ties) is swapped into row k, every
// other row is eliminated with column k, and column k becomes the inverse's
// column; the row swaps are undone at the end as a column permutation.  A
// zero pivot sets flags[2] and leaves the matrix unspecified.
//
// The FP64 unit is the bound (a warp FP64 instruction occupies a scheduler's
// FP64 pipe for the same time on one lane as on 32), so a step spends FP64
// instructions only on the elimination itself:
//   * the pivot search compares magnitudes as integers (the bit pattern with
//     the sign cleared orders finite doubles like fabs does);
//   * the pivot column is published once per step already swapped, scaled by
//     -1/pivot, so that every other column is one FMA per row,
//     A(i, j) += A(p, j) * (-A(i, k) / pivot), and the pivot row entry is the
//     same FMA with the multiplier 1/pivot and a zero addend;
//   * the row swap is folded into that pass (each warp swaps rows k and p of
//     its own column as it reads them);
//   * the search for step k + 1 runs inside step k, in the warp that owns
//     column k + 1, right after it has eliminated that column first, so a step
//     needs one barrier;
//   * for n <= 256 a warp holds several of its columns in registers at once
//     (rows lane + 32 t) and takes the pivot-row entries by shuffle, so their
//     FMAs are all in flight together; larger n steps one column at a time
//     through shared memory (the same arithmetic).
// Two kernels share that step: one CTA per matrix (many filaments), and one
// thread-block cluster per matrix with the columns sliced over the CTAs and
// the published pivot column read through distributed shared memory (few
// filaments, where one CTA per matrix would leave most SMs idle).  Both are
// templates on the element type: FP64 for the reference's arithmetic, FP32
// for the mixed-precision time step, whose approximate inverse only starts
// the Broyden iteration (on the FMA pipe a step is latency-bound, not
// FP64-bound).
#include <cooperative_groups.h>

#include "gmi_context.hpp"
#include "gmi_gauss_jordan.hpp"

namespace cg = cooperative_groups;

namespace gmi {

constexpr int kGjTpb = 512;  // one CTA per matrix: 16 warps, four per scheduler keep the FP64 unit busy
constexpr int kGjWarps = kGjTpb / 32;
constexpr int kGcTpb = 256;  // cluster kernel: 8 warps per CTA (few columns each; a step is latency-bound)
constexpr int kGcWarps = kGcTpb / 32;

// Warp-wide pivot of column Ac (global column index c) among rows i >= c.
// Writes the step's multiplier column ncol[i] = -A'(i, c) / pivot, A' the
// column with rows c and p swapped, 1/pivot to *pinv and p to *piv (-1 when
// the column is zero there).
// |x| as an unsigned integer that orders finite values like fabs does
__device__ __forceinline__ unsigned long long gj_mag(double x)
{
    return (unsigned long long)__double_as_longlong(x) & 0x7fffffffffffffffull;
}
__device__ __forceinline__ unsigned long long gj_mag(float x) { return __float_as_uint(x) & 0x7fffffffu; }
__device__ __forceinline__ double gj_fma(double a, double b, double c) { return fma(a, b, c); }
__device__ __forceinline__ float gj_fma(float a, float b, float c) { return fmaf(a, b, c); }

template <typename T>
static __device__ void gj_pivot_warp(const T *Ac, int n, int c, T *ncol, T *pinv, int *piv, int lane)
{
    unsigned long long best = 0ull;
    int bi = c;
    for (int i = c + lane; i < n; i += 32) {
        const unsigned long long m = gj_mag(Ac[i]);
        if (m > best) {
            best = m;
            bi = i;
        }
    }
    for (int o = 16; o > 0; o >>= 1) {  // butterfly: every lane ends with the same (best, bi)
        const unsigned long long ob = __shfl_xor_sync(0xffffffffu, best, o);
        const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
        if (ob > best || (ob == best && oi < bi)) {
            best = ob;
            bi = oi;
        }
    }
    if (best == 0ull) {
        if (lane == 0) *piv = -1;
        return;
    }
    const T pivinv = T(1) / Ac[bi];
    for (int i = lane; i < n; i += 32) {
        const int src = (i == c) ? bi : ((i == bi) ? c : i);
        ncol[i] = -(Ac[src] * pivinv);
    }
    if (lane == 0) {
        *piv = bi;
        *pinv = pivinv;
    }
}

// Step k on up to C columns jl[0..cnt) held in registers (row
// i = lane + 32 t, RPL rows per lane): the pivot row entries come from the
// owning lanes by shuffle, so a lane touches only its own rows in shared
// memory and the columns' FMAs (RPL each) are all in flight together.
template <int RPL> struct GjColsPerPass {
    static constexpr int value = RPL >= 8 ? 2 : 4;
};

template <typename T, int RPL, int C = GjColsPerPass<RPL>::value>
static __device__ __forceinline__ void gj_cols(T *A, int n, int j0, const int (&jl)[C], int cnt, int k, int p,
                                               T pivinv, const T (&ncr)[RPL], int lane)
{
    T v[C][RPL];
#pragma unroll
    for (int c = 0; c < C; ++c)
#pragma unroll
        for (int t = 0; t < RPL; ++t) {
            const int i = lane + 32 * t;
            v[c][t] = (c < cnt && i < n) ? A[(size_t)n * jl[c] + i] : T(0);
        }
    const int pq = p >> 5, pl = p & 31, kq = k >> 5, kl = k & 31;
#pragma unroll
    for (int c = 0; c < C; ++c) {
        if (c >= cnt) continue;  // warp-uniform
        if (j0 + jl[c] == k) {
#pragma unroll
            for (int t = 0; t < RPL; ++t) {
                const int i = lane + 32 * t;
                v[c][t] = (i == k) ? pivinv : ncr[t];
            }
            continue;
        }
        T sp = v[c][0], sk = v[c][0];
#pragma unroll
        for (int t = 1; t < RPL; ++t) {
            if (pq == t) sp = v[c][t];
            if (kq == t) sk = v[c][t];
        }
        const T akj = __shfl_sync(0xffffffffu, sp, pl);  // row p, swapped into row k
        const T apj = __shfl_sync(0xffffffffu, sk, kl);  // row k, swapped into row p
        if constexpr (sizeof(T) == 8) {
            // FP64: the FP64 pipe bounds the step, so rows k and p are
            // selected inside the one FMA per row (the selects are free)
#pragma unroll
            for (int t = 0; t < RPL; ++t) {
                const int i = lane + 32 * t;
                const T a = (i == k) ? T(0) : ((i == p) ? apj : v[c][t]);
                v[c][t] = gj_fma(akj, (i == k) ? pivinv : ncr[t], a);
            }
        } else {
            // FP32: the per-row selects, not the FMAs, bound the step (ALU
            // pipe 86 % busy, FMA pipe 7 %), so every row takes one FMA as if
            // it were neither k nor p, and the lanes that hold rows p and k
            // redo theirs: row p from the old row k, row k as akj / pivot (a
            // zero addend; when p == k the second fix wins, as in the
            // swap-free case).  1.77 -> 1.57 ms for 640 matrices of 120 x 120.
#pragma unroll
            for (int t = 0; t < RPL; ++t) v[c][t] = gj_fma(akj, ncr[t], v[c][t]);
            if (lane == pl) {
#pragma unroll
                for (int t = 0; t < RPL; ++t)
                    if (t == pq) v[c][t] = gj_fma(akj, ncr[t], apj);
            }
            if (lane == kl) {
#pragma unroll
                for (int t = 0; t < RPL; ++t)
                    if (t == kq) v[c][t] = gj_fma(akj, pivinv, T(0));
            }
        }
    }
#pragma unroll
    for (int c = 0; c < C; ++c)
#pragma unroll
        for (int t = 0; t < RPL; ++t) {
            const int i = lane + 32 * t;
            if (c < cnt && i < n) A[(size_t)n * jl[c] + i] = v[c][t];
        }
}

// Step k on the ncl columns at A (local column jl is global column j0 + jl),
// warp wid taking columns wid, wid + NW, ...: the owner of column k + 1
// eliminates it first and then searches it for the next pivot.  RPL > 0:
// rows in registers (n <= 32 RPL), several columns at a time; RPL == 0: any
// n, one column at a time through shared memory.
template <typename T, int RPL, int NW>
static __device__ __forceinline__ void gj_step(T *A, int n, int ncl, int j0, int k, int p, T pivinv, const T *nc,
                                               T *next_ncol, T *next_pinv, int *next_piv, int wid, int lane)
{
    const int la = k + 1 - j0;
    const int nt = (ncl > wid) ? (ncl - wid + NW - 1) / NW : 0;
    const bool own_la = k + 1 < n && la >= 0 && la < ncl && la % NW == wid;
    if constexpr (RPL > 0) {
        T ncr[RPL];
#pragma unroll
        for (int t = 0; t < RPL; ++t) {
            const int i = lane + 32 * t;
            ncr[t] = i < n ? nc[i] : T(0);
        }
        constexpr int C = GjColsPerPass<RPL>::value;
        int jj[C] = {};
        if (own_la) {
            jj[0] = la;
            gj_cols<T, RPL>(A, n, j0, jj, 1, k, p, pivinv, ncr, lane);
            __syncwarp();
            gj_pivot_warp(A + (size_t)n * la, n, k + 1, next_ncol, next_pinv, next_piv, lane);
        }
        int t = 0;
        while (t < nt) {
            // the next columns in slots 0 .. cnt-1 (a slot is empty only
            // once the warp's columns have run out)
            int cnt = 0;
#pragma unroll
            for (int c = 0; c < C; ++c) {
                int jl = -1;
                while (jl < 0 && t < nt) {
                    const int cand = wid + NW * t++;
                    if (!(own_la && cand == la)) jl = cand;
                }
                jj[c] = jl < 0 ? 0 : jl;
                cnt += jl >= 0 ? 1 : 0;
            }
            if (cnt > 0) gj_cols<T, RPL>(A, n, j0, jj, cnt, k, p, pivinv, ncr, lane);
        }
    } else {
        const int t0 = own_la ? la / NW : 0;
        for (int tt = 0; tt < nt; ++tt) {
            const int t = (tt + t0 < nt) ? tt + t0 : tt + t0 - nt;
            const int jl = wid + NW * t;
            T *Aj = A + (size_t)n * jl;
            if (j0 + jl == k) {
                for (int i = lane; i < n; i += 32) Aj[i] = (i == k) ? pivinv : nc[i];
            } else {
                const T akj = Aj[p], apj = Aj[k];  // rows p and k, swapped
                __syncwarp();
#pragma unroll 4
                for (int i = lane; i < n; i += 32) {
                    const T a = (i == k) ? T(0) : ((i == p) ? apj : Aj[i]);
                    Aj[i] = gj_fma(akj, (i == k) ? pivinv : nc[i], a);
                }
            }
            if (jl == la && own_la) {
                __syncwarp();
                gj_pivot_warp(Aj, n, k + 1, next_ncol, next_pinv, next_piv, lane);
            }
        }
    }
}

// position j of the inverse holds the eliminated column where[j]: the swaps
// (k, perm[k]), k = n-1 .. 0, applied to the column positions
static __device__ void gj_unpivot_map(const int *perm, int n, int *where)
{
    for (int j = 0; j < n; ++j) where[j] = j;
    for (int k = n - 1; k >= 0; --k) {
        const int q = perm[k];
        if (q != k) {
            const int t = where[k];
            where[k] = where[q];
            where[q] = t;
        }
    }
}

// one CTA per matrix; the matrix in shared memory when use_smem, else
// worked on in place in global memory
template <typename T, int RPL>
__global__ void __launch_bounds__(kGjTpb) gj_invert_kernel(T *mats, int n, int use_smem, int *flags)
{
    extern __shared__ __align__(16) double sh[];
    T *Mg = mats + (size_t)blockIdx.x * n * n;
    T *ncol = reinterpret_cast<T *>(sh);              // [2][n], by step parity
    T *pinv = ncol + 2 * (size_t)n;                   // [2]
    int *perm = reinterpret_cast<int *>(pinv + 2);    // [n]
    T *A = use_smem ? reinterpret_cast<T *>(perm + ((n + 1) & ~1)) : Mg;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    if (use_smem)
        for (int e = tid; e < n * n; e += kGjTpb) A[e] = Mg[e];
    __syncthreads();
    if (wid == 0) gj_pivot_warp(A, n, 0, ncol, pinv, perm, lane);
    __syncthreads();
    for (int k = 0; k < n; ++k) {
        const int par = k & 1, p = perm[k];
        if (p < 0) {  // the same in every thread
            if (tid == 0) atomicOr(flags + 2, 1);
            return;
        }
        gj_step<T, RPL, kGjWarps>(A, n, n, 0, k, p, pinv[par], ncol + par * (size_t)n,
                                  ncol + (par ^ 1) * (size_t)n, pinv + (par ^ 1), perm + k + 1, wid, lane);
        __syncthreads();
    }
    if (use_smem) {
        int *where = reinterpret_cast<int *>(ncol);
        if (tid == 0) gj_unpivot_map(perm, n, where);
        __syncthreads();
        for (int j = wid; j < n; j += kGjWarps)
            for (int i = lane; i < n; i += 32) Mg[(size_t)n * j + i] = A[(size_t)n * where[j] + i];
    } else {
        for (int k = n - 1; k >= 0; --k) {
            const int q = perm[k];
            if (q != k)
                for (int i = tid; i < n; i += kGjTpb) {
                    const T t = A[i + (size_t)n * k];
                    A[i + (size_t)n * k] = A[i + (size_t)n * q];
                    A[i + (size_t)n * q] = t;
                }
            __syncthreads();
        }
    }
}

// One cluster of C CTAs per matrix; CTA r owns columns [r nc, r nc + nc).
// Per step: one cluster barrier, after which every CTA copies the step's
// multiplier column, pivot row and 1/pivot from the owner of column k (who
// found them during the previous step) and runs the step on its columns.
// The inverse is gathered at the end straight from the CTAs' shared memory.
template <typename T, int RPL>
__global__ void __launch_bounds__(kGcTpb) gj_cluster_kernel(T *mats, int n, int nc, int *flags)
{
    cg::cluster_group cl = cg::this_cluster();
    const int C = (int)cl.num_blocks(), r = (int)cl.block_rank(), tid = threadIdx.x;
    const int lane = tid & 31, wid = tid >> 5;
    T *Mg = mats + (size_t)(blockIdx.x / C) * n * n;
    const int j0 = r * nc, ncl = max(0, min(n, j0 + nc) - j0);
    extern __shared__ __align__(16) double sh[];
    T *A = reinterpret_cast<T *>(sh);                 // [nc][n]
    T *ncol = A + (size_t)n * nc;                     // [2][n]: published by the pivot column's owner
    T *cur = ncol + 2 * (size_t)n;                    // [n]: this step's copy
    T *pinv = cur + n;                                // [2], published
    T *pv = pinv + 2;                                 // [2]: this step's copy of 1/pivot
    int *piv = reinterpret_cast<int *>(pv + 2);       // [2], published
    int *pk = piv + 2;                                // [2]: this step's pivot row
    int *perm = pk + 2;                               // [n]
    for (int e = tid; e < n * ncl; e += kGcTpb) A[e] = Mg[(size_t)n * j0 + e];
    __syncthreads();
    if (r == 0 && wid == 0) gj_pivot_warp(A, n, 0, ncol, pinv, piv, lane);
    bool singular = false;
    for (int k = 0; k < n; ++k) {
        const int owner = k / nc, par = k & 1;
        cl.sync();  // step k's pivot is published, and step k - 1 is done everywhere
        const T *src = cl.map_shared_rank(ncol, owner) + par * (size_t)n;
        for (int i = tid; i < n; i += kGcTpb) cur[i] = src[i];
        if (tid == 0) {
            pk[0] = cl.map_shared_rank(piv, owner)[par];
            pv[0] = cl.map_shared_rank(pinv, owner)[par];
            perm[k] = pk[0];
        }
        __syncthreads();
        const int p = pk[0];
        if (p < 0) {
            singular = true;
            break;
        }
        gj_step<T, RPL, kGcWarps>(A, n, ncl, j0, k, p, pv[0], cur, ncol + (par ^ 1) * (size_t)n, pinv + (par ^ 1),
                                  piv + (par ^ 1), wid, lane);
    }
    if (singular) {
        if (r == 0 && tid == 0) atomicOr(flags + 2, 1);
        cl.sync();  // no CTA leaves while another may still read its shared memory
        return;
    }
    int *where = reinterpret_cast<int *>(cur);
    if (tid == 0) gj_unpivot_map(perm, n, where);
    cl.sync();  // the last step is done in every CTA
    for (int jl = wid; jl < ncl; jl += kGcWarps) {
        const int w = where[j0 + jl];
        const T *srcc = cl.map_shared_rank(A, w / nc) + (size_t)n * (w % nc);
        for (int i = lane; i < n; i += 32) Mg[(size_t)n * (j0 + jl) + i] = srcc[i];
    }
    cl.sync();  // every CTA has read the columns it needs
}

int gj_cluster_size(int nmat, int n, int sm_count)
{
    if (nmat <= 0 || n < 16) return 1;
    int cs = 8;
    while (cs > 1 && (long long)nmat * cs > sm_count) cs >>= 1;
    return cs;
}

// rows per lane of the register path for n (0: the shared-memory path)
static int gj_rows_per_lane(int n)
{
    return n <= 32 ? 1 : n <= 64 ? 2 : n <= 128 ? 4 : n <= 256 ? 8 : 0;
}

template <typename T, int RPL>
static gmi_status gj_launch(cudaStream_t stream, T *mats, int nmat, int n, int csize, int dev_max, int *flags)
{
    if (csize > 1) {
        const int nc = (n + csize - 1) / csize;
        const size_t smem = ((size_t)n * nc + 3 * (size_t)n + 4) * sizeof(T) + (6 + (size_t)n) * sizeof(int);
        if (smem <= (size_t)dev_max) {
            const void *fn = reinterpret_cast<const void *>(&gj_cluster_kernel<T, RPL>);
            GMI_CUDA_TRY(raise_dynamic_smem_limit(fn, smem));
            cudaLaunchConfig_t cfg{};
            cudaLaunchAttribute attr[1];
            attr[0].id = cudaLaunchAttributeClusterDimension;
            attr[0].val.clusterDim.x = csize;
            attr[0].val.clusterDim.y = 1;
            attr[0].val.clusterDim.z = 1;
            cfg.gridDim = dim3(nmat * csize);
            cfg.blockDim = dim3(kGcTpb);
            cfg.dynamicSmemBytes = smem;
            cfg.stream = stream;
            cfg.attrs = attr;
            cfg.numAttrs = 1;
            GMI_CUDA_TRY(cudaLaunchKernelEx(&cfg, gj_cluster_kernel<T, RPL>, mats, n, nc, flags));
            return GMI_OK;
        }
    }
    const size_t base = (2 * (size_t)n + 2) * sizeof(T) + (size_t)((n + 1) & ~1) * sizeof(int);
    const size_t mat = (size_t)n * n * sizeof(T);
    const int use_smem = (base + mat <= (size_t)dev_max) ? 1 : 0;
    const size_t smem = use_smem ? base + mat : base;
    GMI_CUDA_TRY(raise_dynamic_smem_limit(reinterpret_cast<const void *>(&gj_invert_kernel<T, RPL>), smem));
    gj_invert_kernel<T, RPL><<<nmat, kGjTpb, smem, stream>>>(mats, n, use_smem, flags);
    GMI_CUDA_TRY(cudaGetLastError());
    return GMI_OK;
}

template <typename T>
static gmi_status gj_invert_t(cudaStream_t stream, T *mats, int nmat, int n, int csize, bool registers, int device,
                              int *flags)
{
    if (nmat <= 0) return GMI_OK;
    int dev_max = 0;
    GMI_CUDA_TRY(cudaDeviceGetAttribute(&dev_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, device));
    switch (registers ? gj_rows_per_lane(n) : 0) {
    case 1: return gj_launch<T, 1>(stream, mats, nmat, n, csize, dev_max, flags);
    case 2: return gj_launch<T, 2>(stream, mats, nmat, n, csize, dev_max, flags);
    case 4: return gj_launch<T, 4>(stream, mats, nmat, n, csize, dev_max, flags);
    case 8: return gj_launch<T, 8>(stream, mats, nmat, n, csize, dev_max, flags);
    default: return gj_launch<T, 0>(stream, mats, nmat, n, csize, dev_max, flags);
    }
}

gmi_status gj_invert(cudaStream_t stream, double *mats, int nmat, int n, int csize, bool registers, int device,
                     int *flags)
{
    return gj_invert_t(stream, mats, nmat, n, csize, registers, device, flags);
}

gmi_status gj_invert(cudaStream_t stream, float *mats, int nmat, int n, int csize, bool registers, int device,
                     int *flags)
{
    return gj_invert_t(stream, mats, nmat, n, csize, registers, device, flags);
}

}  // namespace gmi
