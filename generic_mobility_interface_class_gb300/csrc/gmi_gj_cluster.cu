// gmi_gj_cluster.cu -- in-place inverse of n x n column-major matrices with
// each matrix spread over one thread-block cluster: the reference's LAPACK
// dgetrf + dgetri (matrix.cpp:538-566) for the filament Jacobians, when there
// are too few filaments to occupy the GPU with one CTA each.
//
// Gauss-Jordan with partial (row) pivoting, the same arithmetic as the
// one-CTA kernel in gmi_sim.cu: CTA r of a cluster owns a contiguous slice
// of columns in shared memory.  Per pivot step k the owner of column k finds
// the pivot row (largest |A(i, k)|, lowest i on ties), swaps it into row k
// in its columns and publishes the pivot index and the swapped column
// (double-buffered by step parity); after one cluster barrier every CTA
// reads them through DSMEM, swaps the same rows in its own columns and
// eliminates.  At the end the columns are written back and the pivot
// swaps are undone as a column permutation through global memory.  A zero
// pivot sets flags[2] and leaves the matrix unspecified.
#include <cooperative_groups.h>

#include "gmi_context.hpp"
#include "gmi_gj_cluster.hpp"

namespace cg = cooperative_groups;

namespace gmi {

constexpr int kGcTpb = 256;
constexpr int kGcWarps = kGcTpb / 32;

// shared memory: A slice [n][nc] column-major, col[2][n], piv[2] (pivot index
// per parity, -1 = singular), pinv, where[n]
static size_t gc_smem(int n, int nc)
{
    return (size_t)n * nc * sizeof(double) + 2 * (size_t)n * sizeof(double) + 2 * sizeof(double) +
           4 * sizeof(int) + (size_t)n * sizeof(int) + 64;
}

__global__ void __launch_bounds__(kGcTpb) gj_cluster_kernel(double *mats, int n, int nc, int *flags)
{
    cg::cluster_group cl = cg::this_cluster();
    const int C = (int)cl.num_blocks(), r = (int)cl.block_rank(), tid = threadIdx.x;
    const int lane = tid & 31, wid = tid >> 5;
    const int mat = blockIdx.x / C;
    double *Mg = mats + (size_t)mat * n * n;
    const int j0 = r * nc, ncl = max(0, min(n, j0 + nc) - j0);  // this CTA's columns [j0, j0 + ncl)
    extern __shared__ __align__(16) unsigned char sm[];
    double *A = reinterpret_cast<double *>(sm);          // [ncl][n]
    double *col = A + (size_t)n * nc;                      // [2][n]
    double *pinv = col + 2 * (size_t)n;                    // [2]
    int *piv = reinterpret_cast<int *>(pinv + 2);          // [2], then perm flag slots
    int *where = piv + 4;                                  // [n]
    int *perm = where;                                     // the pivot rows, reused as `where` at the end

    for (int e = tid; e < n * ncl; e += kGcTpb) A[e] = Mg[(size_t)n * j0 + e];
    __syncthreads();

    bool singular = false;
    for (int k = 0; k < n; ++k) {
        const int owner = k / nc, par = k & 1;
        if (r == owner) {
            const int kl = k - j0;
            if (wid == 0) {
                double best = -1.0;
                int bi = k;
                for (int i = k + lane; i < n; i += 32) {
                    const double a = fabs(A[i + (size_t)n * kl]);
                    if (a > best) {
                        best = a;
                        bi = i;
                    }
                }
                for (int o = 16; o > 0; o >>= 1) {
                    const double ob = __shfl_down_sync(0xffffffffu, best, o);
                    const int oi = __shfl_down_sync(0xffffffffu, bi, o);
                    if (ob > best || (ob == best && oi < bi)) {
                        best = ob;
                        bi = oi;
                    }
                }
                if (lane == 0) piv[par] = (best > 0.0) ? bi : -1;
            }
            __syncthreads();
            const int p = piv[par];
            if (p > k)
                for (int jl = tid; jl < ncl; jl += kGcTpb) {
                    const double t = A[k + (size_t)n * jl];
                    A[k + (size_t)n * jl] = A[p + (size_t)n * jl];
                    A[p + (size_t)n * jl] = t;
                }
            __syncthreads();
            for (int i = tid; i < n; i += kGcTpb) col[par * n + i] = A[i + (size_t)n * kl];
        }
        cl.sync();  // the pivot row and the swapped pivot column of step k are published
        const int p = cl.map_shared_rank(piv, owner)[par];
        if (p < 0) {
            singular = true;
            break;  // the same in every CTA
        }
        double *cl_col = col + par * n;
        if (r != owner) {
            const double *src = cl.map_shared_rank(col, owner) + par * n;
            for (int i = tid; i < n; i += kGcTpb) cl_col[i] = src[i];
            if (p > k)
                for (int jl = tid; jl < ncl; jl += kGcTpb) {
                    const double t = A[k + (size_t)n * jl];
                    A[k + (size_t)n * jl] = A[p + (size_t)n * jl];
                    A[p + (size_t)n * jl] = t;
                }
        }
        __syncthreads();  // the copied pivot column is complete before thread 0 reads its pivot
        if (tid == 0) {
            perm[k] = p;
            pinv[par] = 1.0 / ((r == owner) ? col[par * n + k] : cl_col[k]);
        }
        __syncthreads();
        const double pivinv = pinv[par];
        for (int jl = wid; jl < ncl; jl += kGcWarps) {
            double *Aj = A + (size_t)n * jl;
            if (j0 + jl == k) {
                for (int i = lane; i < n; i += 32) Aj[i] = (i == k) ? pivinv : -cl_col[i] * pivinv;
            } else {
                const double akj = Aj[k] * pivinv;
                for (int i = lane; i < n; i += 32)
                    if (i != k) Aj[i] = Aj[i] - akj * cl_col[i];
                __syncwarp();
                if (lane == 0) Aj[k] = akj;
            }
        }
        __syncthreads();
    }
    if (singular) {
        if (r == 0 && tid == 0) atomicOr(flags + 2, 1);
        cl.sync();
        return;
    }
    // undo the row pivoting as a column permutation: position j of the
    // inverse holds the eliminated column where[j] (the swaps (k, perm[k]),
    // k = n-1 .. 0, applied to the column positions)
    for (int e = tid; e < n * ncl; e += kGcTpb) Mg[(size_t)n * j0 + e] = A[e];
    __syncthreads();
    if (tid == 0) {
        // perm and where share storage: build where in col (free now) first
        int *wtmp = reinterpret_cast<int *>(col);
        for (int j = 0; j < n; ++j) wtmp[j] = j;
        for (int k = n - 1; k >= 0; --k) {
            const int q = perm[k];
            if (q != k) {
                const int t = wtmp[k];
                wtmp[k] = wtmp[q];
                wtmp[q] = t;
            }
        }
        for (int j = 0; j < n; ++j) where[j] = wtmp[j];
    }
    cl.sync();  // every CTA's columns are in global memory
    for (int e = tid; e < n * ncl; e += kGcTpb) {
        const int jl = e / n, i = e % n;
        A[e] = Mg[(size_t)n * where[j0 + jl] + i];
    }
    cl.sync();  // every CTA has read the columns it needs
    for (int e = tid; e < n * ncl; e += kGcTpb) Mg[(size_t)n * j0 + e] = A[e];
}

int gj_cluster_size(int nmat, int n, int sm_count)
{
    if (nmat <= 0 || n < 16) return 1;
    int cs = 8;
    while (cs > 1 && (long long)nmat * cs > sm_count) cs >>= 1;
    return cs;
}

gmi_status gj_invert_cluster(cudaStream_t stream, double *mats, int nmat, int n, int csize, int *flags)
{
    const int nc = (n + csize - 1) / csize;
    const size_t smem = gc_smem(n, nc);
    const void *fn = reinterpret_cast<const void *>(&gj_cluster_kernel);
    GMI_CUDA_TRY(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
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
    GMI_CUDA_TRY(cudaLaunchKernelEx(&cfg, gj_cluster_kernel, mats, n, nc, flags));
    return GMI_OK;
}

}  // namespace gmi
