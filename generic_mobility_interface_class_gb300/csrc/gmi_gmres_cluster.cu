// gmi_gmres_cluster.cu -- the FP32C GMRES solve of a small free-swimmer
// saddle-point system (mobility_solver.cpp:970-1354, the CILIA_TYPE != 3
// branches of apply_preconditioner :651-721 and system_matrix_mult
// :905-962) run to completion by ONE thread-block cluster.
//
// At small sizes (a few hundred to two thousand blobs) the graph-replayed
// Arnoldi step is bound by latency: six dependent kernels whose cross-CTA
// sums go through L2 (fence, atomic ticket, reload).  Here the whole Arnoldi
// loop is one launch of C CTAs (16 where the GPU allows non-portable
// clusters, else 8).  Each CTA owns a contiguous slice of the blobs and their
// rows (the last CTA also owns the 6W body rows).  Every cross-CTA sum is a
// cluster barrier followed by one DSMEM load per lane (lane r reads CTA r)
// and a fixed shuffle tree, so all CTAs hold bit-identical copies of h,
// ||w|| and the Givens state and take the same stop decision.
//
// Per Arnoldi iteration k (the phases of the multi-kernel step):
//   A  q = w / ||w|| into Q[:, k-1]; body moments of q  -> barrier 1
//      z_body from the summed moments (every CTA)
//   B  blob block of the preconditioner; the CTA's blob loads (z, FP32,
//      pair-interleaved) into its shared memory  -> barrier 2
//      copy the other CTAs' loads; w_body = -K^T z by linearity from the
//      moments of q and K^T K (last CTA)
//   C  blob-blob RPY sum over all blobs, packed FP32 (gmi_pairs2.cuh), from
//      shared memory; meanwhile one reserved warp finishes the Givens step
//      of iteration k-1, whose stop flag is read right after this phase
//      (iteration k then ends unused: it has written only scratch and
//      Q[:, k-1], a column past the solution)
//      w_blob = M_bb z - K z_body
//   D  first classical Gram-Schmidt projections  -> barrier 3, h
//   E  w -= Q h; second projections and ||w||^2  -> barrier 4, h2
//   F  w -= Q h2 on the CTA's rows; ||w - Q h2||^2 = ||w||^2 - ||h2||^2
//      (no barrier)
// All arithmetic except the pair sum is FP64, as in the multi-kernel step.
#include <cooperative_groups.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>

#include "gmi_context.hpp"
#include "gmi_gmres_cluster.hpp"
#include "gmi_pair_kernels.hpp"
#include "gmi_pairs2.cuh"
#include "gmi_solver_device.cuh"
#include "gmi_solver_internal.hpp"

namespace cg = cooperative_groups;

namespace gmi {

constexpr int kCgTpb = 512;
constexpr int kCgWarps = kCgTpb / 32;
constexpr int kCgPairThreads = kCgTpb - 32;  // the last warp runs the Givens step during phase C
constexpr int kCgMaxK = 160;                 // H rows and Givens state (>= max_iter + 1)
constexpr int kCgMaxBlobs = 2048;
constexpr int kCgMaxSwimmers = 16;
constexpr int kCgFold = 64;                  // source pairs summed in FP32 before an FP64 add

struct ClusterGmresArgs {
    int W, nblob, nb, n, ldh, max_iter, bpc;
    size_t ld;
    double *Q, *H, *beta, *cs, *sn;
    double *Qr;                       // the basis again, row-major with ldr columns (projections)
    int ldr;
    int kq, kqs;                      // basis columns [0, kq) of the CTA's rows cached in shared memory, row stride kqs
    const double *w0;                 // r0, all n rows
    const double *R, *refs, *ktk_rot, *mob_rot, *ktkf_rot, *xb;
    double minv, beta0, tol, norm_ref, inv_norm_ref;
    double eta2;                      // conditional re-orthogonalisation threshold (0: two passes always)
    GmresCtl *ctl;
    EqualK<float> kbb;
};

// Shared-memory layout (offsets in bytes), fixed by nb, W and bpc.
struct CgLayout {
    size_t ipos, iload, wl, ql, av, dl, kt, mb, kf, mom1, sums, zb, hp1, hp2, h, h2, np, pp, csh, snh, bet,
        col, red, flag, qs, total;
};

__host__ __device__ inline CgLayout cg_layout(int nb, int W, int bpc, int kqs = 0)
{
    CgLayout L;
    const size_t npairs = (size_t)(nb + 1) / 2, rows = 3 * (size_t)bpc + 6 * (size_t)W;
    size_t o = 0;
    auto take = [&](size_t bytes) {
        const size_t at = o;
        o += (bytes + 15) / 16 * 16;
        return at;
    };
    L.ipos = take(npairs * 3 * sizeof(float4));   // -x hi / lo of every source pair
    L.iload = take(npairs * 2 * sizeof(float4));  // loads of every source pair
    L.wl = take(rows * sizeof(double));
    L.ql = take(rows * sizeof(double));
    L.av = take((size_t)bpc * 6 * sizeof(double));
    L.dl = take((size_t)bpc * 3 * sizeof(double));  // R refs of the CTA's blobs
    L.kt = take(36 * (size_t)W * sizeof(double));
    L.mb = take(36 * (size_t)W * sizeof(double));
    L.kf = take(36 * (size_t)W * sizeof(double));  // K^T K itself, rotated
    L.mom1 = take(6 * (size_t)W * sizeof(double));
    L.sums = take(6 * (size_t)W * sizeof(double));
    L.zb = take(6 * (size_t)W * sizeof(double));
    L.hp1 = take((kCgMaxK + 1) * sizeof(double));
    L.hp2 = take((kCgMaxK + 1) * sizeof(double));
    L.h = take((kCgMaxK + 1) * sizeof(double));
    L.h2 = take((kCgMaxK + 1) * sizeof(double));
    L.np = take(4 * sizeof(double));
    L.pp = take((size_t)kCgTpb * 3 * sizeof(double));
    L.csh = take(kCgMaxK * sizeof(double));
    L.snh = take(kCgMaxK * sizeof(double));
    L.bet = take((kCgMaxK + 1) * sizeof(double));
    L.col = take((kCgMaxK + 1) * sizeof(double));
    L.red = take(kCgWarps * sizeof(double));
    L.flag = take(4 * sizeof(int));
    L.qs = take(rows * (size_t)kqs * sizeof(double));  // cached basis rows
    L.total = o;
    return L;
}

// Deterministic block sum of values held by threads [0, nthreads) (fixed
// shuffle tree in each of their warps, then one over the warp sums held by
// lanes of warp 0); the result is returned to thread 0 only.
__device__ __forceinline__ double cg_block_sum(double v, double *red, int nthreads)
{
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (wid * 32 < nthreads) v = warp_sum(v);  // warps without values skip the FP64 tree
    else v = 0.0;
    if (lane == 0) red[wid] = v;
    __syncthreads();
    double t = 0.0;
    if (wid == 0) {
        t = lane < kCgWarps ? red[lane] : 0.0;
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    }
    __syncthreads();
    return t;
}

// out[e] = sum over the cluster's CTAs of arr[e] (e < count), for every
// thread of the CTA.  Each element has kCrLanes adjacent lanes; lane r adds
// the elements of CTAs r, r + kCrLanes, ... in that order, then an
// xor-shuffle tree adds the lanes (every lane ends with the same bits, in
// every CTA).  Only warps holding elements run FP64 instructions (a warp
// FP64 instruction costs the same with any number of active lanes).
constexpr int kCrLanes = 4;

__device__ __forceinline__ void cluster_reduce(cg::cluster_group &cl, double *arr, int count, double *out, int C,
                                               int /*G*/)
{
    constexpr int groups = kCgTpb / kCrLanes;
    const int gid = threadIdx.x / kCrLanes, r = threadIdx.x % kCrLanes;
    for (int base = 0; base < count; base += groups) {
        const int warps = (min(groups, count - base) * kCrLanes + 31) / 32;
        if ((int)(threadIdx.x >> 5) >= warps) continue;
        const int e = base + gid;
        double v = 0.0;
        if (e < count) {
#pragma unroll 4
            for (int q = r; q < C; q += kCrLanes) v += cl.map_shared_rank(arr, q)[e];
        }
        for (int o = kCrLanes >> 1; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (e < count && r == 0) out[e] = v;
    }
}

// mom[6 s + j] = sum over the CTA's blobs t of swimmer s of av[6 t + j], one
// warp per (s, j): lanes stride over t, then a warp sum.
__device__ __forceinline__ void swimmer_moments(const double *av, int W, int nblob, int b0, int bl, double *mom)
{
    const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int task = wid; task < 6 * W; task += kCgWarps) {
        const int sw = task / 6, j = task % 6;
        const int t0 = max(0, sw * nblob - b0), t1 = min(bl, (sw + 1) * nblob - b0);
        double v = 0.0;
        for (int t = t0 + lane; t < t1; t += 32) v += av[6 * t + j];
        v = warp_sum(v);
        if (lane == 0) mom[task] = v;
    }
}

__global__ void __launch_bounds__(kCgTpb) gmres_cluster_kernel(const ClusterGmresArgs a)
{
    cg::cluster_group cl = cg::this_cluster();
    const int C = (int)cl.num_blocks(), c = (int)cl.block_rank(), tid = threadIdx.x;
    const int G = C <= 8 ? 8 : (C <= 16 ? 16 : 32);
    extern __shared__ __align__(16) unsigned char sm[];
    const CgLayout L = cg_layout(a.nb, a.W, a.bpc, a.kqs);
    float4 *ipos = reinterpret_cast<float4 *>(sm + L.ipos);
    float4 *iload = reinterpret_cast<float4 *>(sm + L.iload);
    double *wl = reinterpret_cast<double *>(sm + L.wl), *ql = reinterpret_cast<double *>(sm + L.ql);
    double *av = reinterpret_cast<double *>(sm + L.av), *dl = reinterpret_cast<double *>(sm + L.dl);
    double *kt = reinterpret_cast<double *>(sm + L.kt), *mb = reinterpret_cast<double *>(sm + L.mb);
    double *mom1 = reinterpret_cast<double *>(sm + L.mom1), *kf = reinterpret_cast<double *>(sm + L.kf);
    double *sums = reinterpret_cast<double *>(sm + L.sums), *zb = reinterpret_cast<double *>(sm + L.zb);
    double *hp1 = reinterpret_cast<double *>(sm + L.hp1), *hp2 = reinterpret_cast<double *>(sm + L.hp2);
    double *h = reinterpret_cast<double *>(sm + L.h), *h2 = reinterpret_cast<double *>(sm + L.h2);
    double *np = reinterpret_cast<double *>(sm + L.np);
    float *pp = reinterpret_cast<float *>(sm + L.pp);  // pair-sum partials, [split][target][3]
    double *csh = reinterpret_cast<double *>(sm + L.csh), *snh = reinterpret_cast<double *>(sm + L.snh);
    double *bet = reinterpret_cast<double *>(sm + L.bet), *col = reinterpret_cast<double *>(sm + L.col);
    double *red = reinterpret_cast<double *>(sm + L.red);
    int *flag = reinterpret_cast<int *>(sm + L.flag);
    double *qs = reinterpret_cast<double *>(sm + L.qs);
    const int kq = a.kq, kqs = a.kqs;

    const int W = a.W, nb = a.nb, nblob = a.nblob, bpc = a.bpc;
    const int npairs = (nb + 1) / 2;
    const int b0 = c * bpc, bl = max(0, min(nb, b0 + bpc) - b0);
    const int bl_last = max(0, nb - (C - 1) * bpc);           // blobs of the last CTA
    const int nr = 3 * bl + (c == C - 1 ? 6 * W : 0);
    const int nw6 = 6 * W;
    const float load_scale = a.kbb.f8pm;
    auto row_of = [&](int lr) { return lr < 3 * bl ? 3 * b0 + lr : 3 * nb + (lr - 3 * bl); };

    // ---- setup: r0 rows, fixed geometry (positions, R refs, 6x6 blocks) ----
    for (int lr = tid; lr < nr; lr += kCgTpb) wl[lr] = a.w0[row_of(lr)];
    for (int t = tid; t < bl; t += kCgTpb) {
        const int i = b0 + t;
        rot_apply(a.R + 9 * (i / nblob), a.refs + 3 * (i % nblob), dl + 3 * t);
    }
    for (int e = tid; e < 36 * W; e += kCgTpb) {
        kt[e] = a.ktk_rot[e];
        mb[e] = a.mob_rot[e];
        kf[e] = a.ktkf_rot[e];
    }
    for (int p = tid; p < npairs; p += kCgTpb) {
        float hp[2][3], lp[2][3];
#pragma unroll
        for (int l = 0; l < 2; ++l) {
            const int j = 2 * p + l;
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                const double x = j < nb ? a.xb[3 * (size_t)j + d] : 0.0;
                const float hi = (float)x;
                hp[l][d] = -hi;
                lp[l][d] = -(float)(x - (double)hi);
            }
        }
        ipos[3 * p] = make_float4(hp[0][0], hp[1][0], hp[0][1], hp[1][1]);
        ipos[3 * p + 1] = make_float4(hp[0][2], hp[1][2], lp[0][0], lp[1][0]);
        ipos[3 * p + 2] = make_float4(lp[0][1], lp[1][1], lp[0][2], lp[1][2]);
        iload[2 * p] = make_float4(0.f, 0.f, 0.f, 0.f);
        iload[2 * p + 1] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    if (tid == 0) {
        bet[0] = a.beta0;
        flag[0] = 0;
        np[2] = a.beta0;        // ||w||, computed once per CTA (np[1] holds ||w||^2)
        np[3] = 1.0 / a.beta0;  // and its reciprocal
    }
    // pair-phase thread map: bl target lanes x S source splits
    const int S = bl > 0 ? kCgPairThreads / bl : 0;
    const int pt = bl > 0 ? tid % bl : 0, ps = bl > 0 ? tid / bl : 0;
    const int pc = S > 0 ? (npairs + S - 1) / S : 0;
    float2 th[3], tlo[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const double x = bl > 0 ? a.xb[3 * (size_t)(b0 + pt) + d] : 0.0;
        const float hi = (float)x;
        th[d] = bc2(hi);
        tlo[d] = bc2((float)(x - (double)hi));
    }
    __syncthreads();

    for (int k = 1; k <= a.max_iter + 1; ++k) {
        double *qcol = a.Q + a.ld * (size_t)(k - 1);
        // ---- A: q_{k-1}, body moments ------------------------------------
        const double nrm = np[2], inrm = np[3];
        for (int lr = tid; lr < nr; lr += kCgTpb) {
            const double q = wl[lr] * inrm;
            const int row = row_of(lr);
            ql[lr] = q;
            qcol[row] = q;
            if (k - 1 < kq)
                qs[lr * kqs + (k - 1)] = q;
            else
                a.Qr[(size_t)row * a.ldr + (k - 1)] = q;
        }
        __syncthreads();
        // per (blob, component): q and (R ref) x q
        for (int e = tid; e < 3 * bl; e += kCgTpb) {
            const int t = e / 3, cc = e % 3, i1 = (cc + 1) % 3, i2 = (cc + 2) % 3;
            const double *d = dl + 3 * t, *f = ql + 3 * t;
            av[6 * t + cc] = f[cc];
            av[6 * t + 3 + cc] = d[i1] * f[i2] - d[i2] * f[i1];
        }
        __syncthreads();
        swimmer_moments(av, W, nblob, b0, bl, mom1);
        cl.sync();  // barrier 1
        cluster_reduce(cl, mom1, nw6, sums, C, G);
        {
            const double *qb_remote = cl.map_shared_rank(ql, C - 1) + 3 * bl_last;
            for (int e = tid; e < nw6; e += kCgTpb) col[e] = qb_remote[e];  // q body rows (col is free here)
        }
        __syncthreads();
        for (int e = tid; e < nw6; e += kCgTpb) {
            const int sw = e / 6, i = e % 6;
            const double *Kt = kt + 36 * sw, *Mb = mb + 36 * sw;
            double x = 0.0, y = 0.0;
            for (int j = 0; j < 6; ++j) {
                x += Kt[i + 6 * j] * (-sums[6 * sw + j]);
                y += Mb[i + 6 * j] * col[6 * sw + j];
            }
            zb[e] = x - y;
        }
        __syncthreads();
        // ---- B: blob preconditioner, loads, w_body -------------------------
        // per (blob, component): z = the blob block applied to q + U + U_rot x (R ref)
        for (int e = tid; e < 3 * bl; e += kCgTpb) {
            const int t = e / 3, cc = e % 3, i1 = (cc + 1) % 3, i2 = (cc + 2) % 3;
            const int i = b0 + t, sw = i / nblob;
            const double *U = zb + 6 * sw, *d = dl + 3 * t;
            double o = ql[3 * t + cc] + U[cc];
            o += U[3 + i1] * d[i2] - U[3 + i2] * d[i1];
            for (int q = sw; q < W; ++q) o *= a.minv;
            float *ld = reinterpret_cast<float *>(iload + 2 * (i >> 1));
            ld[cc == 0 ? (i & 1) : (cc == 1 ? 2 + (i & 1) : 4 + (i & 1))] = (float)o * load_scale;
        }
        cl.sync();  // barrier 2
        // the other CTAs' loads (bpc is even: a source pair has one owner)
        for (int e = tid; e < 2 * npairs; e += kCgTpb) {
            const int owner = (2 * (e >> 1)) / bpc;
            if (owner != c) iload[e] = cl.map_shared_rank(iload, owner)[e];
        }
        if (c == C - 1) {
            // w body rows = -K^T z for z = Minv^(W-n) (q + K z_body): by
            // linearity -Minv^(W-n) (K^T q + (K^T K) z_body), K^T q being
            // phase A's summed moments (still in sums)
            for (int e = tid; e < nw6; e += kCgTpb) {
                const int sw = e / 6, i = e % 6;
                const double *Kf = kf + 36 * sw + i, *zz = zb + 6 * sw;
                double x0 = 0.0, x1 = 0.0;
#pragma unroll
                for (int j = 0; j < 6; j += 2) {
                    x0 += Kf[6 * j] * zz[j];
                    x1 += Kf[6 * (j + 1)] * zz[j + 1];
                }
                double v = sums[e] + (x0 + x1);
                for (int q = sw; q < W; ++q) v *= a.minv;
                wl[3 * bl + e] = -v;
            }
        }
        __syncthreads();
        // ---- C: blob-blob sum (packed FP32); Givens step of iteration k-1 ---
        if (tid < S * bl) {
            // two accumulator sets, one per source pair of an unrolled step,
            // so that their chains overlap: a thread has only a few dozen
            // steps and a few warps share each scheduler
            float2 pacc[3] = {make_float2(0.f, 0.f), make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
            float2 pacc2[3] = {make_float2(0.f, 0.f), make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
            double acc[3] = {0.0, 0.0, 0.0};
            const int p0 = ps * pc, p1 = min(npairs, p0 + pc);
            int cnt = 0;
            auto step = [&](int p, float2 *acc2) {
                const float4 q0 = ipos[3 * p], q1 = ipos[3 * p + 1], q2 = ipos[3 * p + 2];
                const float4 f0 = iload[2 * p], f1 = iload[2 * p + 1];
                const float2 dx = add2(add2(th[0], make_float2(q0.x, q0.y)), add2(tlo[0], make_float2(q1.z, q1.w)));
                const float2 dy = add2(add2(th[1], make_float2(q0.z, q0.w)), add2(tlo[1], make_float2(q2.x, q2.y)));
                const float2 dz = add2(add2(th[2], make_float2(q1.x, q1.y)), add2(tlo[2], make_float2(q2.z, q2.w)));
                const float2 F[3] = {make_float2(f0.x, f0.y), make_float2(f0.z, f0.w), make_float2(f1.x, f1.y)};
                pair2_bb(dx, dy, dz, F, a.kbb, acc2);
            };
            int p = p0;
            for (; p + 1 < p1; p += 2) {
                step(p, pacc);
                step(p + 1, pacc2);
                if ((cnt += 2) >= kCgFold) {
#pragma unroll
                    for (int d = 0; d < 3; ++d) {
                        acc[d] += (double)((pacc[d].x + pacc[d].y) + (pacc2[d].x + pacc2[d].y));
                        pacc[d] = pacc2[d] = make_float2(0.f, 0.f);
                    }
                    cnt = 0;
                }
            }
            if (p < p1) step(p, pacc);
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                pacc[d].x += pacc2[d].x;
                pacc[d].y += pacc2[d].y;
            }
            if (pc <= kCgFold) {  // no fold happened: the partial is an FP32 sum (no FP64 work)
#pragma unroll
                for (int d = 0; d < 3; ++d) pp[3 * tid + d] = pacc[d].x + pacc[d].y;
            } else {
#pragma unroll
                for (int d = 0; d < 3; ++d) pp[3 * tid + d] = (float)(acc[d] + (double)(pacc[d].x + pacc[d].y));
            }
        } else if (tid >= kCgPairThreads && k > 1) {
            // Givens step of iteration k - 1 by the last warp: the H column
            // h + h2 through the previous rotations.  Entry i after rotation
            // i is x_i = -s_{i-1} x_{i-1} + c_{i-1} (h + h2)_i, a first-order
            // linear recurrence, evaluated 32 entries at a time by a
            // Kogge-Stone scan over (a, b) pairs (x -> a x + b); the rotated
            // H entries are then c_{i-1} x_{i-1} + s_{i-1} (h + h2)_i.
            const int iter = k - 1, lane = tid & 31;
            double xin = 0.0;  // x just before the chunk
            for (int base = 0; base < iter; base += 32) {
                const int i = base + lane;
                double aa = 1.0, bb = 0.0, cur = 0.0;
                if (i < iter) {
                    cur = h[i] + h2[i];
                    if (i == 0) {
                        aa = 0.0;
                        bb = cur;
                    } else {
                        aa = -snh[i - 1];
                        bb = csh[i - 1] * cur;
                    }
                }
                for (int o = 1; o < 32; o <<= 1) {
                    const double ap = __shfl_up_sync(0xffffffffu, aa, o), bp = __shfl_up_sync(0xffffffffu, bb, o);
                    if (lane >= o) {
                        bb = fma(aa, bp, bb);
                        aa = aa * ap;
                    }
                }
                const double xi = fma(aa, xin, bb);
                double xm1 = __shfl_up_sync(0xffffffffu, xi, 1);
                if (lane == 0) xm1 = xin;
                if (i >= 1 && i < iter) col[i - 1] = csh[i - 1] * xm1 + snh[i - 1] * cur;
                xin = __shfl_sync(0xffffffffu, xi, 31);  // lanes past the column repeat its last entry
            }
            __syncwarp();
          if (lane == 0) {
            const double hk = nrm, hd = xin;
            double cc, ss;
            if (hk == 0.0) {
                cc = 1.0;
                ss = 0.0;
            } else if (fabs(hk) > fabs(hd)) {  // the reference's scaled form; rsqrt saves a division
                const double u = hd / hk;
                ss = (2.0 * (double)(hk > 0) - 1.0) * rsqrt(1.0 + u * u);
                cc = u * ss;
            } else {
                const double u = hk / hd;
                cc = (2.0 * (double)(hd > 0) - 1.0) * rsqrt(1.0 + u * u);
                ss = u * cc;
            }
            csh[iter - 1] = cc;
            snh[iter - 1] = ss;
            col[iter - 1] = cc * hd + ss * hk;
            col[iter] = 0.0;
            bet[iter] = -ss * bet[iter - 1];
            bet[iter - 1] = cc * bet[iter - 1];
            const double resid = fabs(bet[iter]) * a.inv_norm_ref;
            const int done = !(resid > a.tol) || iter >= a.max_iter;
            flag[0] = done;
            if (c == 0) {
                a.cs[iter - 1] = cc;
                a.sn[iter - 1] = ss;
                a.beta[iter - 1] = bet[iter - 1];
                a.beta[iter] = bet[iter];
                if (done) {
                    a.ctl->k = iter;
                    a.ctl->resid = resid;
                    a.ctl->done = 1;
                    a.ctl->replays = iter;
                }
            }
          }
            __syncwarp();
            if (c == 0) {
                double *gcol = a.H + (size_t)a.ldh * (iter - 1);
                for (int i = lane; i <= iter; i += 32) gcol[i] = col[i];
            }
        }
        __syncthreads();
        if (flag[0]) break;  // the same in every CTA
        for (int e = tid; e < 3 * bl; e += kCgTpb) {
            // component d of blob t: the S split partials (FP32 sums of at
            // most kCgFold source pairs each, added in FP32), then
            // w = M_bb z - (K z_body) in FP64
            const int t = e / 3, d = e % 3, i1 = (d + 1) % 3, i2 = (d + 2) % 3;
            float m0 = 0.f, m1 = 0.f;
            int sp = 0;
            for (; sp + 1 < S; sp += 2) {
                m0 += pp[3 * (sp * bl + t) + d];
                m1 += pp[3 * ((sp + 1) * bl + t) + d];
            }
            if (sp < S) m0 += pp[3 * (sp * bl + t) + d];
            const double *U = zb + 6 * ((b0 + t) / nblob), *dd = dl + 3 * t;
            wl[e] = -(U[d] - dd[i1] * U[3 + i2] + dd[i2] * U[3 + i1]) + (double)(m0 + m1);
        }
        __syncthreads();
        // ---- D..F: CGS2 and ||w|| ------------------------------------------
        // With eta2 > 0 the first pass also sums ||w||^2 (entry k), and the
        // second pass is skipped when ||w - Q h||^2 = ||w||^2 - ||h||^2 keeps
        // at least eta2 of ||w||^2 (Daniel, Gragg, Kaufman and Stewart): every
        // CTA holds the same h, so every CTA takes the same branch.
        const bool dgks = a.eta2 > 0.0;
        for (int pass = 0; pass < 2; ++pass) {
            double *hp = pass == 0 ? hp1 : hp2, *hs = pass == 0 ? h : h2;
            // items (column i, row group g), PG groups per column on adjacent
            // lanes (PG a power of two, k PG <= the CTA's threads): every lane
            // of a warp has FP64 work, and a segmented shuffle tree adds a
            // column's groups
            int PG = 16;
            while (PG > 1 && k * PG > kCgTpb) PG >>= 1;
            {
                const int t = tid, i = t / PG, g = t % PG;
                double s0 = 0.0, s1 = 0.0;
                if (i < k) {
                    int lr = g;
                    if (i < kq) {
                        for (; lr + PG < nr; lr += 2 * PG) {
                            s0 += qs[lr * kqs + i] * wl[lr];
                            s1 += qs[(lr + PG) * kqs + i] * wl[lr + PG];
                        }
                        if (lr < nr) s0 += qs[lr * kqs + i] * wl[lr];
                    } else {
                        for (; lr + PG < nr; lr += 2 * PG) {
                            s0 += a.Qr[(size_t)row_of(lr) * a.ldr + i] * wl[lr];
                            s1 += a.Qr[(size_t)row_of(lr + PG) * a.ldr + i] * wl[lr + PG];
                        }
                        if (lr < nr) s0 += a.Qr[(size_t)row_of(lr) * a.ldr + i] * wl[lr];
                    }
                }
                double sg = s0 + s1;
                for (int o = PG >> 1; o > 0; o >>= 1) sg += __shfl_xor_sync(0xffffffffu, sg, o);
                if (i < k && g == 0) hp[i] = sg;
            }
            if (pass == 1 || dgks) {  // ||w||^2 of the CTA's rows rides along as entry k
                double v2 = 0.0;
                for (int lr = tid; lr < nr; lr += kCgTpb) v2 += wl[lr] * wl[lr];
                v2 = cg_block_sum(v2, red, nr);
                if (tid == 0) hp[k] = v2;
            }
            cl.sync();  // barriers 3 and 4
            cluster_reduce(cl, hp, (pass == 0 && !dgks) ? k : k + 1, hs, C, G);
            __syncthreads();
            for (int lr = tid; lr < nr; lr += kCgTpb) {
                const int row = row_of(lr);
                // (Q h)_row in four interleaved partial sums
                double p0 = 0.0, p1 = 0.0, p2 = 0.0, p3 = 0.0;
                const double *qr = qs + lr * kqs;
                const int kc = min(k, kq);
                int i = 0;
                for (; i + 3 < kc; i += 4) {
                    p0 += hs[i] * qr[i];
                    p1 += hs[i + 1] * qr[i + 1];
                    p2 += hs[i + 2] * qr[i + 2];
                    p3 += hs[i + 3] * qr[i + 3];
                }
                for (; i < kc; ++i) p0 += hs[i] * qr[i];
                for (; i < k; ++i) p0 += hs[i] * a.Q[a.ld * (size_t)i + row];
                wl[lr] -= (p0 + p1) + (p2 + p3);
            }
            __syncthreads();
            if (pass == 0 && dgks) {
                // ||h||^2 by one warp (fixed tree: the same bits in every CTA)
                if (tid < 32) {
                    double t = 0.0;
                    for (int i = tid; i < k; i += 32) t += h[i] * h[i];
                    t = warp_sum(t);
                    if (tid == 0) {
                        const double w2 = h[k], after = w2 - t;
                        const int skip = (w2 > 0.0 && after >= a.eta2 * w2 && after < INFINITY) ? 1 : 0;
                        flag[1] = skip;
                        if (skip) h2[k] = after;  // the norm below: ||w||^2 - ||h2||^2 with h2 = 0
                    }
                }
                __syncthreads();
                if (flag[1]) {
                    for (int i = tid; i < k; i += kCgTpb) h2[i] = 0.0;
                    __syncthreads();
                    break;
                }
            }
        }
        // ||w - Q h2||^2 = ||w||^2 - ||h2||^2 (Q orthonormal; h2 is the second
        // pass's small correction, so nothing cancels), from the same
        // cluster sum as h2: every CTA computes the same bits
        if (tid < 32) {
            double t = 0.0;
            if (!(dgks && flag[1])) {  // a skipped second pass left h2 = 0
                for (int i = tid; i < k; i += 32) t += h2[i] * h2[i];
                t = warp_sum(t);
            }
            if (tid == 0) {
                // an exact breakdown (the new vector cancelled to nothing)
                // gives ||w|| = 0, which the next Givens step takes as
                // convergence; 0 * rsqrt(0) would be NaN
                np[1] = fmax(h2[k] - t, 0.0);
                const double ir = np[1] > 0.0 ? rsqrt(np[1]) : 0.0;
                np[2] = np[1] * ir;  // ||w||
                np[3] = ir;          // 1 / ||w|| (0 after a breakdown: the unused next column is zero)
            }
        }
        __syncthreads();
    }
    // no CTA leaves while another may still read its shared memory
    cl.sync();
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
namespace {
struct ClusterChoice {
    int csize = 0;  // 0: not usable
    int bpc = 0;
    int kq = 0, kqs = 0;
    size_t smem = 0;
};
}  // namespace

static ClusterChoice choose_cluster_uncached(gmi_solver *s);

// The launch shape of this solver's cluster solve: chosen on its first solve
// and kept (the shared-memory limit, the cluster-size attribute and the
// occupancy query are driver calls that would otherwise sit between the
// kernels of every linear solve).
static ClusterChoice choose_cluster(gmi_solver *s)
{
    ClusterChoice ch;
    if (s->cluster_state == 0) {
        ch = choose_cluster_uncached(s);
        s->cluster_state = ch.csize > 0 ? 1 : -1;
        s->cluster_csize = ch.csize;
        s->cluster_bpc = ch.bpc;
        s->cluster_kq = ch.kq;
        s->cluster_kqs = ch.kqs;
        s->cluster_smem = ch.smem;
        return ch;
    }
    if (s->cluster_state > 0) {
        ch.csize = s->cluster_csize;
        ch.bpc = s->cluster_bpc;
        ch.kq = s->cluster_kq;
        ch.kqs = s->cluster_kqs;
        ch.smem = s->cluster_smem;
    }
    return ch;
}

static ClusterChoice choose_cluster_uncached(gmi_solver *s)
{
    ClusterChoice ch;
    const int nb = s->B, W = s->W;
    if (nb <= 0 || nb > kCgMaxBlobs || W <= 0 || W > kCgMaxSwimmers || s->m + 1 > kCgMaxK) return ch;
    const void *fn = reinterpret_cast<const void *>(&gmres_cluster_kernel);
    for (int csize : {16, 8}) {
        int bpc = (nb + csize - 1) / csize;
        bpc += bpc & 1;  // even: a source pair never straddles two CTAs
        // cache as many basis columns of the CTA's rows as fit next to the rest
        const CgLayout L0 = cg_layout(nb, W, bpc, 0);
        if (L0.total > 200 * 1024) continue;
        const size_t rows = 3 * (size_t)bpc + 6 * (size_t)W;
        int kq = (int)((200 * 1024 - L0.total) / (rows * sizeof(double))) - 1;
        kq = std::min(kq, s->m + 1);
        if (kq < 8) kq = 0;
        const int kqs = kq > 0 ? (kq | 1) : 0;  // odd row stride: the per-row update loop avoids bank conflicts
        const CgLayout L = cg_layout(nb, W, bpc, kqs);
        if (raise_dynamic_smem_limit(fn, L.total) != cudaSuccess) {
            cudaGetLastError();
            continue;
        }
        if (csize > 8 &&
            cudaFuncSetAttribute(fn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess) {
            cudaGetLastError();
            continue;
        }
        cudaLaunchConfig_t cfg{};
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = csize;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        cfg.gridDim = dim3(csize);
        cfg.blockDim = dim3(kCgTpb);
        cfg.dynamicSmemBytes = L.total;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        int clusters = 0;
        if (cudaOccupancyMaxActiveClusters(&clusters, fn, &cfg) != cudaSuccess) {
            cudaGetLastError();
            continue;
        }
        if (clusters < 1) continue;
        ch.csize = csize;
        ch.bpc = bpc;
        ch.kq = kq;
        ch.kqs = kqs;
        ch.smem = L.total;
        return ch;
    }
    return ch;
}

bool cluster_gmres_usable(gmi_solver *s)
{
    if (s->ctx->precision != GMI_FP32C) return false;
    const char *env = std::getenv("GMI_GMRES_CLUSTER");
    if (env && env[0] == '0') return false;
    return choose_cluster(s).csize > 0;
}

gmi_status cluster_gmres_launch(gmi_solver *s, double beta0, double norm_ref, double tol, int max_iter)
{
    const ClusterChoice ch = choose_cluster(s);
    if (ch.csize == 0) {
        set_last_error_msg("the cluster GMRES solve does not fit this system");
        return GMI_ERR_STATE;
    }
    // row-major copy of the Krylov basis (n rows of ldr >= max_iter + 1 entries)
    const int ldr = s->m + 1;
    if (s->Qr == nullptr) {
        GMI_CUDA_TRY(dev_malloc(&s->Qr, (size_t)s->n * ldr * sizeof(double)));
        s->allocs.push_back(s->Qr);
    }
    double *Qr = s->Qr;
    ClusterGmresArgs a{};
    a.W = s->W;
    a.nblob = s->cfg.nblob;
    a.nb = s->B;
    a.n = s->n;
    a.ldh = s->m + 1;
    a.max_iter = max_iter;
    a.bpc = ch.bpc;
    a.ld = (size_t)s->n;
    a.Q = s->Q;
    a.Qr = Qr;
    a.ldr = ldr;
    a.kq = ch.kq;
    a.kqs = ch.kqs;
    a.H = s->H;
    a.beta = s->beta;
    a.cs = s->cs;
    a.sn = s->sn;
    a.w0 = s->w;
    a.R = s->R;
    a.refs = s->refs;
    a.ktk_rot = s->ktk_rot;
    a.mob_rot = s->mob_rot;
    a.ktkf_rot = s->ktkf_rot;
    a.xb = s->x_blobs;
    a.minv = 6.0 * kPi * s->cfg.mu * s->cfg.rblob;
    a.beta0 = beta0;
    a.tol = tol;
    a.norm_ref = norm_ref;
    a.inv_norm_ref = 1.0 / norm_ref;
    a.eta2 = reorth_eta2(false);  // the cluster solve is FP32C only
    a.ctl = s->ctl;
    PairConsts k;
    fill_consts(k, s->cfg.rblob, s->cfg.rblob, s->cfg.rblob, s->cfg.mu);
    a.kbb.four_a2 = (float)k.eq[0];
    a.kbb.two_a2 = (float)k.eq[1];
    a.kbb.f8pm = (float)k.eq[2];
    a.kbb.f6pma = (float)k.eq[3];
    a.kbb.q32 = (float)k.eq[4];
    a.kbb.inv_a = (float)k.eq[5];
    a.kbb.f8pma3 = (float)k.eq[6];
    a.kbb.f16pma3 = (float)k.eq[7];
    a.kbb.q8 = (float)k.eq[8];
    cudaLaunchConfig_t cfg{};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = ch.csize;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3(ch.csize);
    cfg.blockDim = dim3(kCgTpb);
    cfg.dynamicSmemBytes = ch.smem;
    cfg.stream = s->ctx->stream;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    GMI_CUDA_TRY(cudaLaunchKernelEx(&cfg, gmres_cluster_kernel, a));
    s->ctx->launches++;
    return GMI_OK;
}

}  // namespace gmi
