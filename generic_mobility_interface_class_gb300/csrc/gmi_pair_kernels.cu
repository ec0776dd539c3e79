// gmi_pair_kernels.cu -- the O(N^2) RPY pair sums on sm_103a.
//
// Data path of one apply (all on the context stream):
//   1. pack: the reference's AoS FP64 arrays (X[3n], F[3n|6n]) become
//      12-scalar records per particle.  FP32C records hold the position as a
//      double-float (hi, lo) pair so differences keep ~FP64 accuracy:
//        [xh yh zh fx] [xl yl zl fy] [fz tx ty tz]
//      FP64 records:  [x y z fx fy fz tx ty tz 0 0 0]
//   2. pair kernel: each CTA owns TPB*TT targets and one contiguous slice
//      ("split") of the sources.  Source tiles of kTile records are staged
//      into shared memory by TMA (cp.async.bulk.tensor.2d, one elected
//      thread, kStages-deep ring of mbarriers); every thread then walks the
//      tile (broadcast reads, no bank conflicts) for its TT targets.  FP32C
//      accumulates each tile in plain FP32 and folds the tile sum into a
//      (hi, lo) two-sum accumulator, so the error does not grow with N.
//   3. with more than one split, per-split partial sums (FP64) go to scratch
//      and a reduce kernel adds them in split order into the output (= or +=).
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <type_traits>
#include <vector>

#include "gmi_context.hpp"
#include "gmi_pairs.cuh"
#include "gmi_pairs2.cuh"
#include "gmi_df.cuh"
#include "gmi_pair_kernels.hpp"

namespace gmi {

constexpr int kRecLen = 12;
constexpr int kTile = 128;   // sources per TMA box (box rows <= 256)
constexpr int kStages = 4;   // depth of the shared-memory ring

// ---------------------------------------------------------------------------
// 1. pack kernels
// ---------------------------------------------------------------------------
__global__ void pack_records_f32(const double *__restrict__ x, const double *__restrict__ f, int nf, int n,
                                 float4 *__restrict__ rec)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double px = x[3 * i], py = x[3 * i + 1], pz = x[3 * i + 2];
    const float hx = (float)px, hy = (float)py, hz = (float)pz;
    const float lx = (float)(px - (double)hx), ly = (float)(py - (double)hy), lz = (float)(pz - (double)hz);
    float f0 = 0.f, f1 = 0.f, f2 = 0.f, t0 = 0.f, t1 = 0.f, t2 = 0.f;
    if (f != nullptr) {
        f0 = (float)f[nf * i];
        f1 = (float)f[nf * i + 1];
        f2 = (float)f[nf * i + 2];
        if (nf == 6) {
            t0 = (float)f[6 * i + 3];
            t1 = (float)f[6 * i + 4];
            t2 = (float)f[6 * i + 5];
        }
    }
    float4 *r = rec + 3 * (size_t)i;
    r[0] = make_float4(hx, hy, hz, f0);
    r[1] = make_float4(lx, ly, lz, f1);
    r[2] = make_float4(f2, t0, t1, t2);
}

// Double-float records (precision GMI_DF64, blob forces only):
// [xh yh zh fxh][xl yl zl fyh][fzh fxl fyl fzl], every value an FP32
// (hi, lo) pair.  Positions are taken relative to the first blob (in FP64),
// so their 48 bits resolve the cloud, not its distance from the origin.
__global__ void pack_records_df(const double *__restrict__ x, const double *__restrict__ f, int n,
                                float4 *__restrict__ rec)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const df2 px = df_from_double(x[3 * i] - x[0]), py = df_from_double(x[3 * i + 1] - x[1]),
              pz = df_from_double(x[3 * i + 2] - x[2]);
    df2 f0 = df2{0.f, 0.f}, f1 = f0, f2 = f0;
    if (f != nullptr) {
        f0 = df_from_double(f[3 * i]);
        f1 = df_from_double(f[3 * i + 1]);
        f2 = df_from_double(f[3 * i + 2]);
    }
    float4 *r = rec + 3 * (size_t)i;
    r[0] = make_float4(px.h, py.h, pz.h, f0.h);
    r[1] = make_float4(px.l, py.l, pz.l, f1.h);
    r[2] = make_float4(f2.h, f0.l, f1.l, f2.l);
}

__global__ void pack_records_f64(const double *__restrict__ x, const double *__restrict__ f, int nf, int n,
                                 double2 *__restrict__ rec)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double f0 = 0, f1 = 0, f2 = 0, t0 = 0, t1 = 0, t2 = 0;
    if (f != nullptr) {
        f0 = f[nf * i];
        f1 = f[nf * i + 1];
        f2 = f[nf * i + 2];
        if (nf == 6) {
            t0 = f[6 * i + 3];
            t1 = f[6 * i + 4];
            t2 = f[6 * i + 5];
        }
    }
    double2 *r = rec + 6 * (size_t)i;
    r[0] = make_double2(x[3 * i], x[3 * i + 1]);
    r[1] = make_double2(x[3 * i + 2], f0);
    r[2] = make_double2(f1, f2);
    r[3] = make_double2(t0, t1);
    r[4] = make_double2(t2, 0.0);
    r[5] = make_double2(0.0, 0.0);
}

// ---------------------------------------------------------------------------
// record access
// ---------------------------------------------------------------------------
template <class R> struct Pos {
    R x, y, z, lx, ly, lz;
};

// Source record from shared memory: position and the 6 load components.
__device__ __forceinline__ void load_src(const float *p, Pos<float> &s, float *F)
{
    const float4 a = reinterpret_cast<const float4 *>(p)[0];
    const float4 b = reinterpret_cast<const float4 *>(p)[1];
    const float4 c = reinterpret_cast<const float4 *>(p)[2];
    s.x = a.x; s.y = a.y; s.z = a.z; s.lx = b.x; s.ly = b.y; s.lz = b.z;
    F[0] = a.w; F[1] = b.w; F[2] = c.x; F[3] = c.y; F[4] = c.z; F[5] = c.w;
}
__device__ __forceinline__ void load_src(const double *p, Pos<double> &s, double *F)
{
    const double2 a = reinterpret_cast<const double2 *>(p)[0];
    const double2 b = reinterpret_cast<const double2 *>(p)[1];
    const double2 c = reinterpret_cast<const double2 *>(p)[2];
    const double2 d = reinterpret_cast<const double2 *>(p)[3];
    const double2 e = reinterpret_cast<const double2 *>(p)[4];
    s.x = a.x; s.y = a.y; s.z = b.x; s.lx = s.ly = s.lz = 0.0;
    F[0] = b.y; F[1] = c.x; F[2] = c.y; F[3] = d.x; F[4] = d.y; F[5] = e.x;
}
__device__ __forceinline__ Pos<float> load_tgt(const float *rec, int i)
{
    const float4 a = reinterpret_cast<const float4 *>(rec)[3 * (size_t)i];
    const float4 b = reinterpret_cast<const float4 *>(rec)[3 * (size_t)i + 1];
    return Pos<float>{a.x, a.y, a.z, b.x, b.y, b.z};
}
__device__ __forceinline__ Pos<double> load_tgt(const double *rec, int i)
{
    const double2 a = reinterpret_cast<const double2 *>(rec)[6 * (size_t)i];
    const double2 b = reinterpret_cast<const double2 *>(rec)[6 * (size_t)i + 1];
    return Pos<double>{a.x, a.y, b.x, 0.0, 0.0, 0.0};
}

// d = x_i - x_j with the low words folded in (they are zero for FP64).
template <class R> __device__ __forceinline__ R diff(R hi_i, R hi_j, R lo_i, R lo_j)
{
    return (hi_i - hi_j) + (lo_i - lo_j);
}
template <> __device__ __forceinline__ double diff<double>(double hi_i, double hi_j, double, double)
{
    return hi_i - hi_j;
}

// Per-target accumulator.  FP32: tile sum + (hi, lo) compensated total.
template <class R, int NOUT> struct Acc;
template <int NOUT> struct Acc<double, NOUT> {
    double t[NOUT];
    __device__ void zero() {
#pragma unroll
        for (int c = 0; c < NOUT; ++c) t[c] = 0.0;
    }
    __device__ void fold() {}
    __device__ double total(int c) const { return t[c]; }
};
template <int NOUT> struct Acc<float, NOUT> {
    float t[NOUT], hi[NOUT], lo[NOUT];
    __device__ void zero() {
#pragma unroll
        for (int c = 0; c < NOUT; ++c) t[c] = hi[c] = lo[c] = 0.f;
    }
    // Knuth two-sum of the tile sum into the running total.
    __device__ void fold() {
#pragma unroll
        for (int c = 0; c < NOUT; ++c) {
            const float s = hi[c] + t[c];
            const float bp = s - hi[c];
            const float e = (hi[c] - (s - bp)) + (t[c] - bp);
            hi[c] = s;
            lo[c] += e;
            t[c] = 0.f;
        }
    }
    __device__ double total(int c) const { return (double)hi[c] + (double)lo[c]; }
};

template <int KIND> struct KindTraits;
template <> struct KindTraits<kSS> { static constexpr int nout = 6; };
template <> struct KindTraits<kSSWall> { static constexpr int nout = 6; };
template <> struct KindTraits<kBB> { static constexpr int nout = 3; };
template <> struct KindTraits<kSB> { static constexpr int nout = 6; };
template <> struct KindTraits<kBS> { static constexpr int nout = 3; };

// ---------------------------------------------------------------------------
// 2. tiled pair kernel
// ---------------------------------------------------------------------------
template <class R> struct KernelConsts {
    EqualK<R> eq;
    UnequalK<R> uq;
};

template <class R> __device__ __forceinline__ KernelConsts<R> convert_consts(const PairConsts &c)
{
    KernelConsts<R> k;
    k.eq.four_a2 = (R)c.eq[0]; k.eq.two_a2 = (R)c.eq[1]; k.eq.f8pm = (R)c.eq[2]; k.eq.f6pma = (R)c.eq[3];
    k.eq.q32 = (R)c.eq[4]; k.eq.inv_a = (R)c.eq[5]; k.eq.f8pma3 = (R)c.eq[6]; k.eq.f16pma3 = (R)c.eq[7];
    k.eq.q8 = (R)c.eq[8];
    k.uq.sum2 = (R)c.uq[0]; k.uq.dmin2 = (R)c.uq[1]; k.uq.far_c = (R)c.uq[2]; k.uq.half_sum = (R)c.uq[3];
    k.uq.f8pm = (R)c.uq[4]; k.uq.f6pmab = (R)c.uq[5]; k.uq.fmax = (R)c.uq[6]; k.uq.c_mid_den = (R)c.uq[7];
    k.uq.ab = (R)c.uq[8]; k.uq.as = (R)c.uq[9]; k.uq.ab2 = (R)c.uq[10]; k.uq.inner_c = (R)c.uq[11];
    k.uq.dmin = (R)c.uq[12];
    return k;
}

// One source's contribution to one target's accumulator (self: the target
// and the source are the same particle; only the wall formula needs it).
template <int KIND, class R>
__device__ __forceinline__ void pair_apply(const Pos<R> &t, const Pos<R> &sp, const R *F, const KernelConsts<R> &K,
                                           bool self, R *acc)
{
    const R dx = diff<R>(t.x, sp.x, t.lx, sp.lx);
    const R dy = diff<R>(t.y, sp.y, t.ly, sp.ly);
    const R dz = diff<R>(t.z, sp.z, t.lz, sp.lz);
    if constexpr (KIND == kSSWall) {
        const R zi = t.z + t.lz, zj = sp.z + sp.lz;
        const R zs = (t.z + sp.z) + (t.lz + sp.lz);
        pair_ss_wall<R>(dx, dy, dz, zs, zi, zj, self, F, acc, acc + 3);
    }
    if constexpr (KIND == kSS) pair_ss<R>(dx, dy, dz, F, K.eq, acc, acc + 3);
    if constexpr (KIND == kBB) pair_bb<R>(dx, dy, dz, F, K.eq, acc);
    if constexpr (KIND == kSB) pair_sb<R>(dx, dy, dz, F, K.uq, acc, acc + 3);
    if constexpr (KIND == kBS) pair_bs<R>(dx, dy, dz, F, K.uq, acc);
}

template <int KIND, class R, int TPB, int TT>
__global__ void __launch_bounds__(TPB) rpy_pair_kernel(const __grid_constant__ CUtensorMap src_map,
                                                       const PairLaunch args)
{
    constexpr int NOUT = KindTraits<KIND>::nout;
    constexpr int kStageScalars = kTile * kRecLen;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    R *ring = reinterpret_cast<R *>(smem_raw);
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem_raw + kStages * kStageScalars * sizeof(R));

    pdl_wait();
    if (args.skip != nullptr && *args.skip != 0) return;
    const int tid = threadIdx.x;
    const int j_begin = blockIdx.y * args.chunk;
    const int j_end = min(j_begin + args.chunk, args.n_src);
    const int ntiles = j_end > j_begin ? (j_end - j_begin + kTile - 1) / kTile : 0;
    constexpr unsigned kBoxBytes = kStageScalars * sizeof(R);

    if (tid == 0) {
        prefetch_tensormap(&src_map);
#pragma unroll
        for (int s = 0; s < kStages; ++s) mbar_init(&bars[s], 1);
        fence_mbar_init();
    }
    __syncthreads();
    int issued = 0;  // tiles requested so far (meaningful on thread 0)
    if (tid == 0) {
        for (; issued < kStages && issued < ntiles; ++issued) {
            mbar_arrive_expect_tx(&bars[issued], kBoxBytes);
            tma_load_2d(ring + issued * kStageScalars, &src_map, 0, j_begin + issued * kTile, &bars[issued]);
        }
    }

    const KernelConsts<R> K = convert_consts<R>(args.k);
    const R *tgt_rec = reinterpret_cast<const R *>(args.tgt_rec);
    Pos<R> tp[TT];
    int ti[TT];
    Acc<R, NOUT> acc[TT];
#pragma unroll
    for (int k = 0; k < TT; ++k) {
        ti[k] = blockIdx.x * (TPB * TT) + k * TPB + tid;
        const int gi = args.tgt_start + min(ti[k], args.n_tgt - 1);
        tp[k] = load_tgt(tgt_rec, gi);
        acc[k].zero();
    }

    bool timed_out = false;
    int t = 0;
    for (; t < ntiles; ++t) {
        const int s = t % kStages;
        const bool ok = mbar_wait_bounded(&bars[s], (t / kStages) & 1, args.wait_ns);
        if (__syncthreads_or(!ok)) {
            timed_out = true;
            break;
        }
        // Every thread has finished tile t-1: its stage can be refilled.
        if (tid == 0 && t >= 1 && issued < ntiles) {
            const int sp = (t - 1) % kStages;
            mbar_arrive_expect_tx(&bars[sp], kBoxBytes);
            tma_load_2d(ring + sp * kStageScalars, &src_map, 0, j_begin + issued * kTile, &bars[sp]);
            ++issued;
        }
        const R *tile = ring + s * kStageScalars;
        const int j0 = j_begin + t * kTile;
        const int jn = min(kTile, j_end - j0);
#pragma unroll 4
        for (int jj = 0; jj < jn; ++jj) {
            Pos<R> sp;
            R F[6];
            load_src(tile + jj * kRecLen, sp, F);
#pragma unroll
            for (int k = 0; k < TT; ++k)
                pair_apply<KIND, R>(tp[k], sp, F, K, (args.tgt_start + ti[k]) == (j0 + jj), acc[k].t);
        }
#pragma unroll
        for (int k = 0; k < TT; ++k) acc[k].fold();
    }

    if (timed_out) {
        if (tid == 0) {
            atomicOr(args.err, kDevErrWaitTimeout);
            // Let the copies still in flight land (bounded) before the CTA exits.
            for (int u = t; u < issued; ++u) (void)mbar_wait_bounded(&bars[u % kStages], (u / kStages) & 1);
        }
        return;
    }

#pragma unroll
    for (int k = 0; k < TT; ++k) {
        if (ti[k] >= args.n_tgt) continue;
        if (args.partial != nullptr) {
            double *p = args.partial + ((size_t)blockIdx.y * args.n_tgt + ti[k]) * NOUT;
#pragma unroll
            for (int c = 0; c < NOUT; ++c) p[c] = acc[k].total(c);
        } else {
            double *o = args.out + (size_t)ti[k] * NOUT;
#pragma unroll
            for (int c = 0; c < NOUT; ++c) o[c] = args.accumulate ? o[c] + acc[k].total(c) : acc[k].total(c);
        }
    }
}

// ---------------------------------------------------------------------------
// 2''. double-float blob-blob sum (precision GMI_DF64): the FP64 operator's
// accuracy (about 1e-13 per pair) on the FP32 pipe, for the residuals of the
// mixed-precision refinement.  The scalar kernel's TMA ring on the records
// of pack_records_df; per target three double-float accumulators; the pair
// formulas of pair_bb (cuda_functions.cu:429-539) step by step in
// double-float.
// ---------------------------------------------------------------------------
struct DfBBConsts {
    df2 four_a2, two_a2, f8pm, f6pma, q32, third;
};

// a - b for double-float positions
__device__ __forceinline__ df2 df_diff(df2 a, df2 b)
{
    const df2 s = df_two_sum(a.h, -b.h);
    return df_fast_two_sum(s.h, __fadd_rn(s.l, __fsub_rn(a.l, b.l)));
}

__device__ __forceinline__ void pair_bb_df(const df2 *d, const df2 *F, const DfBBConsts &K, df2 *v)
{
    const df2 r2 = df_add(df_add(df_sqr(d[0]), df_sqr(d[1])), df_sqr(d[2]));
    const df2 dF = df_add(df_add(df_mul(d[0], F[0]), df_mul(d[1], F[1])), df_mul(d[2], F[2]));
    df2 At, Bt;
    if (r2.h == 0.0f) {  // coincident blobs (the self term): the near-field limit r -> 0
        At = K.f6pma;
        Bt = df_make(0.0f);
    } else {
        const df2 ir = df_rsqrt(r2);
        const df2 ir2 = df_sqr(ir);
        if (r2.h > K.four_a2.h || (r2.h == K.four_a2.h && r2.l > K.four_a2.l)) {
            const df2 s = df_mul(K.two_a2, ir2);
            const df2 ik = df_mul(ir, K.f8pm);
            At = df_mul(ik, df_add(df_make(1.0f), df_mul(s, K.third)));
            const df2 c3dF = df_mul(df_mul(ik, ir2), dF);
            Bt = df_sub(c3dF, df_mul(s, c3dF));
        } else {
            const df2 q = df_mul(df_mul(r2, ir), K.q32);
            At = df_mul(df_sub(df_make(1.0f), df_mul_f(q, 3.0f)), K.f6pma);
            Bt = df_mul(df_mul(df_mul(q, K.f6pma), ir2), dF);
        }
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) v[c] = df_add(v[c], df_add(df_mul(At, F[c]), df_mul(Bt, d[c])));
}

template <int TPB>
__global__ void __launch_bounds__(TPB) rpy_bb_df_kernel(const __grid_constant__ CUtensorMap src_map,
                                                        const PairLaunch args, const DfBBConsts K)
{
    constexpr int kStageScalars = kTile * kRecLen;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    float *ring = reinterpret_cast<float *>(smem_raw);
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem_raw + kStages * kStageScalars * sizeof(float));

    pdl_wait();
    if (args.skip != nullptr && *args.skip != 0) return;
    const int tid = threadIdx.x;
    const int j_begin = blockIdx.y * args.chunk;
    const int j_end = min(j_begin + args.chunk, args.n_src);
    const int ntiles = j_end > j_begin ? (j_end - j_begin + kTile - 1) / kTile : 0;
    constexpr unsigned kBoxBytes = kStageScalars * sizeof(float);

    if (tid == 0) {
        prefetch_tensormap(&src_map);
#pragma unroll
        for (int s = 0; s < kStages; ++s) mbar_init(&bars[s], 1);
        fence_mbar_init();
    }
    __syncthreads();
    int issued = 0;  // tiles requested so far (meaningful on thread 0)
    if (tid == 0) {
        for (; issued < kStages && issued < ntiles; ++issued) {
            mbar_arrive_expect_tx(&bars[issued], kBoxBytes);
            tma_load_2d(ring + issued * kStageScalars, &src_map, 0, j_begin + issued * kTile, &bars[issued]);
        }
    }

    const int ti = blockIdx.x * TPB + tid;
    const float4 *tr = reinterpret_cast<const float4 *>(args.tgt_rec) +
                       3 * (size_t)(args.tgt_start + min(ti, args.n_tgt - 1));
    const float4 t0 = tr[0], t1 = tr[1];
    const df2 xi[3] = {df2{t0.x, t1.x}, df2{t0.y, t1.y}, df2{t0.z, t1.z}};
    df2 v[3] = {df2{0.f, 0.f}, df2{0.f, 0.f}, df2{0.f, 0.f}};

    bool timed_out = false;
    int t = 0;
    for (; t < ntiles; ++t) {
        const int s = t % kStages;
        const bool ok = mbar_wait_bounded(&bars[s], (t / kStages) & 1, args.wait_ns);
        if (__syncthreads_or(!ok)) {
            timed_out = true;
            break;
        }
        // Every thread has finished tile t-1: its stage can be refilled.
        if (tid == 0 && t >= 1 && issued < ntiles) {
            const int sp = (t - 1) % kStages;
            mbar_arrive_expect_tx(&bars[sp], kBoxBytes);
            tma_load_2d(ring + sp * kStageScalars, &src_map, 0, j_begin + issued * kTile, &bars[sp]);
            ++issued;
        }
        const float4 *tile = reinterpret_cast<const float4 *>(ring + s * kStageScalars);
        const int jn = min(kTile, j_end - (j_begin + t * kTile));
#pragma unroll 2
        for (int jj = 0; jj < jn; ++jj) {
            const float4 b0 = tile[3 * jj], b1 = tile[3 * jj + 1], b2 = tile[3 * jj + 2];
            const df2 d[3] = {df_diff(xi[0], df2{b0.x, b1.x}), df_diff(xi[1], df2{b0.y, b1.y}),
                              df_diff(xi[2], df2{b0.z, b1.z})};
            const df2 F[3] = {df2{b0.w, b2.y}, df2{b1.w, b2.z}, df2{b2.x, b2.w}};
            pair_bb_df(d, F, K, v);
        }
    }

    if (timed_out) {
        if (tid == 0) {
            atomicOr(args.err, kDevErrWaitTimeout);
            for (int u = t; u < issued; ++u) (void)mbar_wait_bounded(&bars[u % kStages], (u / kStages) & 1);
        }
        return;
    }
    if (ti >= args.n_tgt) return;
    if (args.partial != nullptr) {
        double *p = args.partial + ((size_t)blockIdx.y * args.n_tgt + ti) * 3;
#pragma unroll
        for (int c = 0; c < 3; ++c) p[c] = df_to_double(v[c]);
    } else {
        double *o = args.out + (size_t)ti * 3;
#pragma unroll
        for (int c = 0; c < 3; ++c) o[c] = args.accumulate ? o[c] + df_to_double(v[c]) : df_to_double(v[c]);
    }
}

// Small systems (up to kPairWarpMaxSources sources): one warp per target,
// its 32 lanes striding over the sources read straight from the records
// (they stay in L1), then the lanes' double-float sums added by a fixed
// butterfly.  The TMA kernel gives such a system a few dozen CTAs, each a
// serial chain of 128 double-float pair evaluations per thread; here every
// lane has about n / 32.
__global__ void __launch_bounds__(128) rpy_bb_df_warp_kernel(const PairLaunch args, const float4 *__restrict__ src,
                                                             const DfBBConsts K)
{
    const int t = (int)((blockIdx.x * 128u + threadIdx.x) >> 5), lane = threadIdx.x & 31;
    if (t >= args.n_tgt) return;
    const float4 *tr = reinterpret_cast<const float4 *>(args.tgt_rec) + 3 * (size_t)(args.tgt_start + t);
    const float4 t0 = tr[0], t1 = tr[1];
    const df2 xi[3] = {df2{t0.x, t1.x}, df2{t0.y, t1.y}, df2{t0.z, t1.z}};
    df2 v[3] = {df2{0.f, 0.f}, df2{0.f, 0.f}, df2{0.f, 0.f}};
    for (int j = lane; j < args.n_src; j += 32) {
        const float4 b0 = src[3 * (size_t)j], b1 = src[3 * (size_t)j + 1], b2 = src[3 * (size_t)j + 2];
        const df2 d[3] = {df_diff(xi[0], df2{b0.x, b1.x}), df_diff(xi[1], df2{b0.y, b1.y}),
                          df_diff(xi[2], df2{b0.z, b1.z})};
        const df2 F[3] = {df2{b0.w, b2.y}, df2{b1.w, b2.z}, df2{b2.x, b2.w}};
        pair_bb_df(d, F, K, v);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
#pragma unroll
        for (int c = 0; c < 3; ++c)
            v[c] = df_add(v[c], df2{__shfl_xor_sync(0xffffffffu, v[c].h, o), __shfl_xor_sync(0xffffffffu, v[c].l, o)});
    if (lane != 0) return;
    double *o = args.out + (size_t)t * 3;
#pragma unroll
    for (int c = 0; c < 3; ++c) o[c] = args.accumulate ? o[c] + df_to_double(v[c]) : df_to_double(v[c]);
}

// ---------------------------------------------------------------------------
// 2'. packed FP32 variant (kinds SS, BB, SB, BS): each thread takes two
// sources per step, one per lane of the packed f32x2 instructions.  After a
// tile lands, the CTA rewrites it into a pair-interleaved buffer (every
// record component as {source 2p, source 2p+1}, positions negated so that
// differences are additions); the TMA stage is free again right after that
// pass, so a 2-deep ring suffices, and the interleaved buffer is double
// buffered so that one barrier per tile orders everything:
//   wait(stage) -> interleave into ibuf[t&1] -> barrier -> refill stage
//   -> compute on ibuf[t&1]
// (a thread interleaves tile t+1 into ibuf[(t+1)&1] only after the barrier
// of tile t, which every thread reaches after finishing tile t-1).
// Accumulation: per target, plus and minus parts per lane (gmi_pairs2.cuh),
// added up at the end of each tile and folded into the (hi, lo) total.
// ---------------------------------------------------------------------------
constexpr int kStagesP = 2;
constexpr int kTilePairs = kTile / 2;

template <int KIND>
__device__ __forceinline__ void pair2_apply(float2 dx, float2 dy, float2 dz, const float2 *F,
                                            const KernelConsts<float> &K, float2 *p, float2 *m)
{
    if constexpr (KIND == kSS) pair2_ss(dx, dy, dz, F, K.eq, p, m);
    if constexpr (KIND == kBB) pair2_bb(dx, dy, dz, F, K.eq, p);
    if constexpr (KIND == kSB) pair2_sb(dx, dy, dz, F, K.uq, p, m);
    if constexpr (KIND == kBS) pair2_bs(dx, dy, dz, F, K.uq, p, m);
}

template <int KIND, int TPB, int TT>
__global__ void __launch_bounds__(TPB) rpy_pair2_kernel(const __grid_constant__ CUtensorMap src_map,
                                                        const PairLaunch args)
{
    constexpr int NOUT = KindTraits<KIND>::nout;
    constexpr int kStageScalars = kTile * kRecLen;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    // a launch whose splits are one tile each (chunk <= kTile) uses ring
    // stage 0 and interleave buffer 0 only, and the launcher allocates just
    // those (half the shared memory: twice the CTAs per SM)
    const bool single = args.chunk <= kTile;
    float *ring = reinterpret_cast<float *>(smem_raw);
    float4 *ibuf = reinterpret_cast<float4 *>(smem_raw + (single ? 1 : kStagesP) * kStageScalars * sizeof(float));
    uint64_t *bars =
        reinterpret_cast<uint64_t *>(smem_raw + (single ? 2 : kStagesP + 2) * kStageScalars * sizeof(float));

    pdl_wait();
    if (args.skip != nullptr && *args.skip != 0) return;
    const int tid = threadIdx.x;
    const int j_begin = blockIdx.y * args.chunk;
    const int j_end = min(j_begin + args.chunk, args.n_src);
    const int ntiles = j_end > j_begin ? (j_end - j_begin + kTile - 1) / kTile : 0;
    constexpr unsigned kBoxBytes = kStageScalars * sizeof(float);

    if (tid == 0) {
        prefetch_tensormap(&src_map);
#pragma unroll
        for (int s = 0; s < kStagesP; ++s) mbar_init(&bars[s], 1);
        fence_mbar_init();
    }
    __syncthreads();
    int issued = 0;  // tiles requested so far (meaningful on thread 0)
    if (tid == 0) {
        for (; issued < kStagesP && issued < ntiles; ++issued) {
            mbar_arrive_expect_tx(&bars[issued], kBoxBytes);
            tma_load_2d(ring + issued * kStageScalars, &src_map, 0, j_begin + issued * kTile, &bars[issued]);
        }
    }

    const KernelConsts<float> K = convert_consts<float>(args.k);
    // loads enter the packed formulas times 1/(8 pi mu) (gmi_pairs2.cuh)
    const float load_scale = (KIND == kSB || KIND == kBS) ? K.uq.f8pm : K.eq.f8pm;
    const float *tgt_rec = reinterpret_cast<const float *>(args.tgt_rec);
    float2 th[TT][3], tl[TT][3];  // target position (hi, lo), both lanes
    int ti[TT];
    float2 p[TT][NOUT], m[TT][NOUT];
    float hi[TT][NOUT], lo[TT][NOUT];
#pragma unroll
    for (int k = 0; k < TT; ++k) {
        ti[k] = blockIdx.x * (TPB * TT) + k * TPB + tid;
        const Pos<float> tp = load_tgt(tgt_rec, args.tgt_start + min(ti[k], args.n_tgt - 1));
        th[k][0] = bc2(tp.x); th[k][1] = bc2(tp.y); th[k][2] = bc2(tp.z);
        tl[k][0] = bc2(tp.lx); tl[k][1] = bc2(tp.ly); tl[k][2] = bc2(tp.lz);
#pragma unroll
        for (int c = 0; c < NOUT; ++c) {
            p[k][c] = m[k][c] = make_float2(0.f, 0.f);
            hi[k][c] = lo[k][c] = 0.f;
        }
    }

    bool timed_out = false;
    int t = 0;
    for (; t < ntiles; ++t) {
        const int s = t % kStagesP;
        const bool ok = mbar_wait_bounded(&bars[s], (t / kStagesP) & 1, args.wait_ns);
        const int j0 = j_begin + t * kTile;
        const int jn = min(kTile, j_end - j0);
        const int npair = (jn + 1) >> 1;
        float4 *ib = ibuf + (t & 1) * (kTilePairs * 6);
        if (ok) {
            // interleave: item (pair pp, quarter q) turns float4 q of records
            // 2pp and 2pp+1 into two float4 of {a, b} lanes; a missing odd
            // source (jn odd) is all zeros and contributes nothing
            const float4 *st = reinterpret_cast<const float4 *>(ring + s * kStageScalars);
            for (int it = tid; it < 3 * npair; it += TPB) {
                const int pp = it / 3, q = it - 3 * pp;
                float4 a = st[6 * pp + q];
                float4 b = 2 * pp + 1 < jn ? st[6 * pp + 3 + q] : make_float4(0.f, 0.f, 0.f, 0.f);
                if (q < 2) {  // .xyz are positions (hi for q = 0, lo for q = 1), .w a load
                    a.x = -a.x; a.y = -a.y; a.z = -a.z;
                    b.x = -b.x; b.y = -b.y; b.z = -b.z;
                    a.w *= load_scale; b.w *= load_scale;
                } else {
                    a.x *= load_scale; a.y *= load_scale; a.z *= load_scale; a.w *= load_scale;
                    b.x *= load_scale; b.y *= load_scale; b.z *= load_scale; b.w *= load_scale;
                }
                ib[6 * pp + 2 * q] = make_float4(a.x, b.x, a.y, b.y);
                ib[6 * pp + 2 * q + 1] = make_float4(a.z, b.z, a.w, b.w);
            }
        }
        if (__syncthreads_or(!ok)) {
            timed_out = true;
            break;
        }
        // every thread has interleaved tile t: its stage can be refilled
        if (tid == 0 && issued < ntiles) {
            mbar_arrive_expect_tx(&bars[s], kBoxBytes);
            tma_load_2d(ring + s * kStageScalars, &src_map, 0, j_begin + issued * kTile, &bars[s]);
            ++issued;
        }
#pragma unroll 2
        for (int pp = 0; pp < npair; ++pp) {
            // record order: [xh yh zh f0][xl yl zl f1][f2 f3 f4 f5], lanes paired
            const float4 q0 = ib[6 * pp], q1 = ib[6 * pp + 1], q2 = ib[6 * pp + 2];
            const float4 q3 = ib[6 * pp + 3], q4 = ib[6 * pp + 4], q5 = ib[6 * pp + 5];
            const float2 nxh = make_float2(q0.x, q0.y), nyh = make_float2(q0.z, q0.w);
            const float2 nzh = make_float2(q1.x, q1.y);
            const float2 nxl = make_float2(q2.x, q2.y), nyl = make_float2(q2.z, q2.w);
            const float2 nzl = make_float2(q3.x, q3.y);
            const float2 F[6] = {make_float2(q1.z, q1.w), make_float2(q3.z, q3.w), make_float2(q4.x, q4.y),
                                 make_float2(q4.z, q4.w), make_float2(q5.x, q5.y), make_float2(q5.z, q5.w)};
#pragma unroll
            for (int k = 0; k < TT; ++k) {
                const float2 dx = add2(add2(th[k][0], nxh), add2(tl[k][0], nxl));
                const float2 dy = add2(add2(th[k][1], nyh), add2(tl[k][1], nyl));
                const float2 dz = add2(add2(th[k][2], nzh), add2(tl[k][2], nzl));
                pair2_apply<KIND>(dx, dy, dz, F, K, p[k], m[k]);
            }
        }
        // tile sum of both lanes, plus minus minus, folded by two-sum
#pragma unroll
        for (int k = 0; k < TT; ++k) {
#pragma unroll
            for (int c = 0; c < NOUT; ++c) {
                const float v = (p[k][c].x + p[k][c].y) - (m[k][c].x + m[k][c].y);
                const float sum = hi[k][c] + v;
                const float bp = sum - hi[k][c];
                lo[k][c] += (hi[k][c] - (sum - bp)) + (v - bp);
                hi[k][c] = sum;
                p[k][c] = m[k][c] = make_float2(0.f, 0.f);
            }
        }
    }

    if (timed_out) {
        if (tid == 0) {
            atomicOr(args.err, kDevErrWaitTimeout);
            for (int u = t; u < issued; ++u) (void)mbar_wait_bounded(&bars[u % kStagesP], (u / kStagesP) & 1);
        }
        return;
    }

#pragma unroll
    for (int k = 0; k < TT; ++k) {
        if (ti[k] >= args.n_tgt) continue;
        if (args.partial != nullptr) {
            double *o = args.partial + ((size_t)blockIdx.y * args.n_tgt + ti[k]) * NOUT;
#pragma unroll
            for (int c = 0; c < NOUT; ++c) o[c] = (double)hi[k][c] + (double)lo[k][c];
        } else {
            double *o = args.out + (size_t)ti[k] * NOUT;
#pragma unroll
            for (int c = 0; c < NOUT; ++c) {
                const double v = (double)hi[k][c] + (double)lo[k][c];
                o[c] = args.accumulate ? o[c] + v : v;
            }
        }
    }
}

// 3. split reduction: out[i] (=|+=) sum over splits, in split order.
__global__ void reduce_splits(const double *__restrict__ partial, int splits, int count,
                              double *__restrict__ out, int accumulate, const int *skip)
{
    if (skip != nullptr && *skip != 0) return;
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= count) return;
    double s = accumulate ? out[e] : 0.0;
    for (int p = 0; p < splits; ++p) s += partial[(size_t)p * count + e];
    out[e] = s;
}

// ---------------------------------------------------------------------------
// 2b. small problems (up to a few thousand sources): one warp per TPW
// targets, its 32 lanes stride over the sources with direct vector loads
// (records stay in L1/L2), each lane sums its share (FP32C folds its tile
// sum every kWarpFold sources), and the warp adds the lane sums in FP64.
// At these sizes the tiled kernel cannot field enough threads to fill the
// GPU; this one runs N/TPW warps with no split reduction.
// ---------------------------------------------------------------------------
constexpr int kWarpCta = 128;  // threads per CTA of the warp kernel
constexpr int kWarpFold = 32;

__device__ __forceinline__ double warp_sum_d(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

template <int KIND, class R, int TPW>
__global__ void __launch_bounds__(kWarpCta) rpy_pair_warp_kernel(const PairLaunch args, const R *__restrict__ src)
{
    constexpr int NOUT = KindTraits<KIND>::nout;
    pdl_wait();
    if (args.skip != nullptr && *args.skip != 0) return;
    const int lane = threadIdx.x & 31;
    const int t0 = ((blockIdx.x * kWarpCta + threadIdx.x) >> 5) * TPW;
    if (t0 >= args.n_tgt) return;  // whole warp
    const KernelConsts<R> K = convert_consts<R>(args.k);
    const R *tgt_rec = reinterpret_cast<const R *>(args.tgt_rec);
    Pos<R> tp[TPW];
    int gi[TPW];
    Acc<R, NOUT> acc[TPW];
#pragma unroll
    for (int k = 0; k < TPW; ++k) {
        gi[k] = args.tgt_start + min(t0 + k, args.n_tgt - 1);
        tp[k] = load_tgt(tgt_rec, gi[k]);
        acc[k].zero();
    }
    int cnt = 0;
    for (int j = lane; j < args.n_src; j += 32) {
        Pos<R> sp;
        R F[6];
        load_src(src + (size_t)j * kRecLen, sp, F);
#pragma unroll
        for (int k = 0; k < TPW; ++k) pair_apply<KIND, R>(tp[k], sp, F, K, gi[k] == j, acc[k].t);
        if (++cnt == kWarpFold) {
#pragma unroll
            for (int k = 0; k < TPW; ++k) acc[k].fold();
            cnt = 0;
        }
    }
#pragma unroll
    for (int k = 0; k < TPW; ++k) {
        acc[k].fold();
        double v[NOUT];
#pragma unroll
        for (int c = 0; c < NOUT; ++c) v[c] = warp_sum_d(acc[k].total(c));
        if (lane == 0 && t0 + k < args.n_tgt) {
            double *o = args.out + (size_t)(t0 + k) * NOUT;
#pragma unroll
            for (int c = 0; c < NOUT; ++c) o[c] = args.accumulate ? o[c] + v[c] : v[c];
        }
    }
}

// ---------------------------------------------------------------------------
// barrier forces: cuda_functions.cu:961-1157.  Positions are screened in
// FP32; pairs that can be inside the cutoff are re-evaluated in FP64 from
// the original arrays, so the force arithmetic is the reference's FP64.
// Targets: segments [0,S) then blobs [S, S+B) (of the requested ranges);
// sources: all S segments then all B blobs.
//
// The screen positions are FP32 offsets from the first particle, one float4
// each; a rounding margin from the largest offset (the pack kernel's
// extent) keeps every pair that is inside the cutoff in FP64 inside the
// screen.  Each lane screens its target against eight sources at a time
// (independent arithmetic, one warp vote per eight), and only then looks at
// the candidates one by one.
//
// The FP64 path (sqrt, divide) is slow on this GPU and rare per lane, so the
// lanes of a warp do not each run it for their own candidates: every warp
// queues its candidates (lane, j) in shared memory in screening order,
// evaluates them 32 at a time, one per lane, and each lane then adds its own
// entries in queue order, which is ascending j: the reference's summation
// order per target.  Sources are split over blockIdx.y (for occupancy); each
// split sums in j order and the splits are added in order by barrier_reduce.
// ---------------------------------------------------------------------------
constexpr int kBarrierTpb = 64;
constexpr int kBarrierWarps = kBarrierTpb / 32;
constexpr int kBarrierQ = 64;     // queue entries per warp (flushed at >= 32)
constexpr int kBarrierGroup = 8;  // sources per warp vote

// out[i] = x_i - x_0 in FP32; *extent = max |coordinate| (FP32 bits, which
// order like the values for non-negative floats; zeroed by the launcher)
__global__ void pack_screen_positions(const double *__restrict__ xs, int S, const double *__restrict__ xb, int B,
                                      float4 *__restrict__ out, unsigned *__restrict__ extent)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const double *p0 = S > 0 ? xs : xb;
    float m = 0.0f;
    if (i < S + B) {
        const double *p = i < S ? xs + 3 * (size_t)i : xb + 3 * (size_t)(i - S);
        const float rx = (float)(p[0] - p0[0]), ry = (float)(p[1] - p0[1]), rz = (float)(p[2] - p0[2]);
        out[i] = make_float4(rx, ry, rz, 0.f);
        m = fmaxf(fabsf(rx), fmaxf(fabsf(ry), fabsf(rz)));
    }
    const unsigned mb = __reduce_max_sync(0xffffffffu, __float_as_uint(m));
    if ((threadIdx.x & 31) == 0 && mb != 0u) atomicMax(extent, mb);
}

struct BarrierQueue {
    int j[kBarrierQ];
    int lane[kBarrierQ];
    double v[3][kBarrierQ];
};

// Evaluate the warp's queued candidates in FP64 and add them, in queue order,
// to the owning lanes' accumulators.
__device__ __forceinline__ void barrier_flush(const BarrierLaunch &a, BarrierQueue &q, int count, double xi,
                                              double yi, double zi, double a_tgt, double &g0, double &g1, double &g2)
{
    const int lane = threadIdx.x & 31;
    for (int base = 0; base < count; base += 32) {
        const int e = base + lane;
        const int src = e < count ? q.lane[e] : lane;
        const double tx = __shfl_sync(0xffffffffu, xi, src);
        const double ty = __shfl_sync(0xffffffffu, yi, src);
        const double tz = __shfl_sync(0xffffffffu, zi, src);
        const double ta = __shfl_sync(0xffffffffu, a_tgt, src);
        if (e < count) {
            const int j = q.j[e];
            const bool src_seg = j < a.S;
            const double asum = ta + (src_seg ? a.rseg : a.rblob);
            const double *pj = src_seg ? a.xs + 3 * (size_t)j : a.xb + 3 * (size_t)(j - a.S);
            const double ddx = tx - pj[0], ddy = ty - pj[1], ddz = tz - pj[2];
            const double dist = sqrt(ddx * ddx + ddy * ddy + ddz * ddz);
            double v0 = 0.0, v1 = 0.0, v2 = 0.0;
            if (dist < 1.1 * asum) {
                double c = fmin(1.0, 1.0 - (10.0 / asum) * (dist - asum));
                c = a.scale * c * c * c * c;
                const double idist = 1.0 / dist;
                v0 = c * ddx * idist;
                v1 = c * ddy * idist;
                v2 = c * ddz * idist;
            }
            q.v[0][e] = v0;
            q.v[1][e] = v1;
            q.v[2][e] = v2;
        }
    }
    __syncwarp();
    for (int e = 0; e < count; ++e) {
        if (q.lane[e] == lane) {
            g0 += q.v[0][e];
            g1 += q.v[1][e];
            g2 += q.v[2][e];
        }
    }
    __syncwarp();
}

__global__ void __launch_bounds__(kBarrierTpb) barrier_kernel(BarrierLaunch a)
{
    __shared__ float4 tile[kBarrierTpb];
    __shared__ BarrierQueue queues[kBarrierWarps];
    BarrierQueue &q = queues[threadIdx.x >> 5];
    const int lane = threadIdx.x & 31;
    const int N = a.S + a.B;
    const int local = blockIdx.x * blockDim.x + threadIdx.x;  // over [0, num_segs + num_blobs)
    const bool is_seg_target = local < a.num_segs;
    const bool valid = local < a.num_segs + (a.wall ? 0 : a.num_blobs);
    const int gi = is_seg_target ? a.start_seg + local : a.S + a.start_blob + (local - a.num_segs);
    double xi = 0, yi = 0, zi = 0;
    float4 pf = make_float4(0.f, 0.f, 0.f, 0.f);
    if (valid) {
        const double *p = is_seg_target ? a.xs + 3 * (size_t)gi : a.xb + 3 * (size_t)(gi - a.S);
        xi = p[0]; yi = p[1]; zi = p[2];
        pf = a.screen[gi];
    }
    const int fil_i = gi / a.nseg;
    double g0 = 0, g1 = 0, g2 = 0;
    const double DL = 2.2 * a.rseg;
    const int j_begin = blockIdx.y * a.chunk, j_end = min(N, j_begin + a.chunk);
    if (blockIdx.y == 0 && valid && is_seg_target && a.wall && zi < 0.5 * DL) {
        const double fz = fmin(1.0, 1.0 - (zi - a.rseg) / (0.5 * DL - a.rseg));
        g2 = a.scale * fz * fz * fz * fz;
    }
    const double a_tgt = is_seg_target ? a.rseg : a.rblob;
    // squared screen cutoffs against segment and blob sources: the FP32
    // cutoff plus the rounding of the offsets (each within 2^-24 of the
    // extent, their difference within 2^-23 of it) and of the separation
    const float margin = 1.0e-6f * __uint_as_float(*a.extent);
    const float cs = (is_seg_target ? a.cut_ss : a.cut_sb) + margin;
    const float cb = (is_seg_target ? a.cut_sb : a.cut_bb) + margin;
    const float c2_s = cs * cs, c2_b = cb * cb;
    int count = 0;  // warp-uniform
    for (int j0 = j_begin; j0 < j_end; j0 += kBarrierTpb) {
        const int jl = j0 + threadIdx.x;
        if (jl < j_end) tile[threadIdx.x] = a.screen[jl];
        __syncthreads();
        const int jn = min(kBarrierTpb, j_end - j0);
        for (int u0 = 0; u0 < jn; u0 += kBarrierGroup) {
            unsigned bits = 0u;
#pragma unroll
            for (int u = 0; u < kBarrierGroup; ++u) {
                const int jj = u0 + u;
                const float4 s = tile[jj < jn ? jj : jn - 1];
                const float dx = pf.x - s.x, dy = pf.y - s.y, dz = pf.z - s.z;
                const float d2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
                const bool in = jj < jn && d2 < ((j0 + jj) < a.S ? c2_s : c2_b);
                bits |= in ? (1u << u) : 0u;
            }
            if (!valid) bits = 0u;
            if (!__any_sync(0xffffffffu, bits != 0u)) continue;
            for (int u = 0; u < kBarrierGroup; ++u) {
                const int j = j0 + u0 + u;
                bool cand = ((bits >> u) & 1u) != 0u;
                if (cand) {
                    if (is_seg_target) {
                        const int di = gi - j;
                        cand = !((fil_i == j / a.nseg) && (di <= 1 && di >= -1));
                    } else {
                        cand = (j != gi);
                    }
                }
                const unsigned mask = __ballot_sync(0xffffffffu, cand);
                if (mask) {
                    if (cand) {
                        const int pos = count + __popc(mask & ((1u << lane) - 1u));
                        q.j[pos] = j;
                        q.lane[pos] = lane;
                    }
                    count += __popc(mask);
                    __syncwarp();
                    if (count >= 32) {
                        barrier_flush(a, q, count, xi, yi, zi, a_tgt, g0, g1, g2);
                        count = 0;
                    }
                }
            }
        }
        __syncthreads();
    }
    if (count > 0) barrier_flush(a, q, count, xi, yi, zi, a_tgt, g0, g1, g2);
    if (!valid) return;
    if (a.partial != nullptr) {
        const int ntg = a.num_segs + (a.wall ? 0 : a.num_blobs);
        double *p = a.partial + ((size_t)blockIdx.y * ntg + local) * 3;
        p[0] = g0;
        p[1] = g1;
        p[2] = g2;
        return;
    }
    if (is_seg_target) {
        double *f = a.f_segs + 6 * (size_t)gi;
        f[0] += g0;
        f[1] += g1;
        f[2] += g2;
    } else {
        double *f = a.f_blobs_rep + 3 * (size_t)(local - a.num_segs);
        f[0] = g0;
        f[1] = g1;
        f[2] = g2;
    }
}

// Barrier split sums, in split order: segment targets add into f_segs,
// blob targets overwrite their repulsion force.
__global__ void barrier_reduce(BarrierLaunch a, int splits)
{
    const int ntg = a.num_segs + (a.wall ? 0 : a.num_blobs);
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= 3 * ntg) return;
    const int local = e / 3, c = e % 3;
    double g = 0.0;
    for (int p = 0; p < splits; ++p) g += a.partial[((size_t)p * ntg + local) * 3 + c];
    if (local < a.num_segs)
        a.f_segs[6 * (size_t)(a.start_seg + local) + c] += g;
    else
        a.f_blobs_rep[3 * (size_t)(local - a.num_segs) + c] = g;
}

// ---------------------------------------------------------------------------
// Barrier forces through a hashed cell list.
//
// The barrier force is short-ranged: a pair contributes only inside
// 1.1 (a_i + a_j) (cuda_functions.cu:1031-1046, 1121-1135).  With cells at
// least as wide as the widest screen cutoff, a target's candidates lie in
// the 27 cells around its own.  Cell (cx, cy, cz) of a particle's FP32 screen
// position hashes to one of T = 2^k buckets, and a counting sort (count,
// bucket offsets, scatter) lists each bucket's particles.  Each target
// screens the particles of its 27 buckets exactly as barrier_kernel does
// (the same FP32 test and exclusions), keeps its candidates in shared
// memory, sorts them by index, drops repeats (two of its cells can share a
// bucket), and adds their FP64 forces in ascending j in one accumulator: the
// reference's per-target order, so each force is the reference's bit for
// bit.  A target with more than kCellCand candidates goes to an overflow
// list, which a warp-per-target all-pairs kernel finishes in the same order.
// ---------------------------------------------------------------------------
constexpr int kCellTpb = 128;
constexpr int kCellCand = 40;          // candidates per target kept in shared memory
constexpr int kCellScanTpb = 1024;
constexpr int kCellScanTile = 4 * kCellScanTpb;  // buckets per CTA of the offset scan
constexpr int kCellMinParticles = 8192;          // fewer particles: the all-pairs kernel

struct CellList {
    int T;              // buckets (a power of two, a multiple of kCellScanTile)
    float cut_max;      // widest FP32 screen cutoff before the rounding margin
    const unsigned *extent;
    int *count;         // [T] particles per bucket (counted down again by the scatter)
    int *local;         // [T] exclusive scan of count within its scan tile
    int *tile_prefix;   // [T / kCellScanTile] particles before each scan tile
    int *order;         // [N] particles by bucket
    int *key;           // [N] each particle's bucket
    int *overflow;      // [1 + targets]: count, then the overflowed targets (launch-local indices)
    int *ticket;        // [1] the scan's last-CTA ticket (zero between launches)
};

// cell width: the widest screen cutoff plus the rounding margin of the
// screen (as barrier_kernel) with 1 % to spare, so that any pair the screen
// can accept lies in adjacent cells whatever the rounding of x / h
__device__ __forceinline__ float cell_inv_width(const CellList &c)
{
    const float margin = 1.0e-6f * __uint_as_float(*c.extent);
    return 1.0f / ((c.cut_max + margin) * 1.01f);
}
__device__ __forceinline__ int cell_coord(float x, float inv_h) { return (int)floorf(x * inv_h); }
__device__ __forceinline__ int cell_bucket(int cx, int cy, int cz, int T)
{
    const unsigned h = ((unsigned)cx * 73856093u) ^ ((unsigned)cy * 19349663u) ^ ((unsigned)cz * 83492791u);
    return (int)(h & (unsigned)(T - 1));
}
__device__ __forceinline__ int cell_offset(const CellList &c, int b)
{
    return __ldcg(c.local + b) + __ldcg(c.tile_prefix + b / kCellScanTile);
}

__global__ void cell_keys_kernel(CellList c, const float4 *__restrict__ screen, int N)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    const float inv_h = cell_inv_width(c);
    const float4 p = screen[i];
    const int b = cell_bucket(cell_coord(p.x, inv_h), cell_coord(p.y, inv_h), cell_coord(p.z, inv_h), c.T);
    c.key[i] = b;
    atomicAdd(c.count + b, 1);
}

// Exclusive scan of the bucket counts: each CTA scans one tile of
// kCellScanTile buckets (four per thread) into local[] and writes its total;
// the last CTA to finish scans the totals into tile_prefix[].
__global__ void __launch_bounds__(kCellScanTpb) cell_scan_kernel(CellList c)
{
    __shared__ int warp_tot[kCellScanTpb / 32];
    __shared__ int is_last;
    const int t = threadIdx.x, lane = t & 31, wid = t >> 5;
    const int base = blockIdx.x * kCellScanTile + 4 * t;
    const int4 v = *reinterpret_cast<const int4 *>(c.count + base);
    const int own = v.x + v.y + v.z + v.w;
    int incl = own;
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
    }
    if (lane == 31) warp_tot[wid] = incl;
    __syncthreads();
    if (wid == 0) {
        int w = warp_tot[lane];
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        warp_tot[lane] = w;  // inclusive over warps
    }
    __syncthreads();
    const int before = incl - own + (wid > 0 ? warp_tot[wid - 1] : 0);
    int4 e;
    e.x = before;
    e.y = before + v.x;
    e.z = e.y + v.y;
    e.w = e.z + v.z;
    *reinterpret_cast<int4 *>(c.local + base) = e;
    if (t == kCellScanTpb - 1) {
        c.tile_prefix[blockIdx.x] = before + own;  // the tile's total, scanned below
        __threadfence();
        is_last = atomicAdd(c.ticket, 1) == (int)gridDim.x - 1;
    }
    __syncthreads();
    if (!is_last) return;
    __threadfence();
    // the last CTA: exclusive scan of the gridDim.x (<= kCellScanTpb) tile totals
    const int n = gridDim.x;
    const int tot = t < n ? __ldcg(c.tile_prefix + t) : 0;
    int x = tot;
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    __syncthreads();
    if (lane == 31) warp_tot[wid] = x;
    __syncthreads();
    if (wid == 0) {
        int w = warp_tot[lane];
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        warp_tot[lane] = w;
    }
    __syncthreads();
    if (t < n) c.tile_prefix[t] = x - tot + (wid > 0 ? warp_tot[wid - 1] : 0);
    if (t == 0) *c.ticket = 0;
}

__global__ void cell_scatter_kernel(CellList c, int N)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    const int b = c.key[i];
    const int slot = atomicSub(c.count + b, 1) - 1;
    c.order[cell_offset(c, b) + slot] = i;
}

// The FP64 force of one accepted pair, as barrier_flush: zero outside the
// exact cutoff.
__device__ __forceinline__ void barrier_pair(const BarrierLaunch &a, int j, double xi, double yi, double zi,
                                             double a_tgt, double &g0, double &g1, double &g2)
{
    const bool src_seg = j < a.S;
    const double asum = a_tgt + (src_seg ? a.rseg : a.rblob);
    const double *pj = src_seg ? a.xs + 3 * (size_t)j : a.xb + 3 * (size_t)(j - a.S);
    const double ddx = xi - pj[0], ddy = yi - pj[1], ddz = zi - pj[2];
    const double dist = sqrt(ddx * ddx + ddy * ddy + ddz * ddz);
    if (dist < 1.1 * asum) {
        double cc = fmin(1.0, 1.0 - (10.0 / asum) * (dist - asum));
        cc = a.scale * cc * cc * cc * cc;
        const double idist = 1.0 / dist;
        g0 += cc * ddx * idist;
        g1 += cc * ddy * idist;
        g2 += cc * ddz * idist;
    }
}

// a target's launch-local index -> its global particle index, position and
// the store of its force (segment targets add, blob targets overwrite)
struct BarrierTarget {
    int gi;
    bool seg;
    double x, y, z;
};
__device__ __forceinline__ BarrierTarget barrier_target(const BarrierLaunch &a, int local)
{
    BarrierTarget t;
    t.seg = local < a.num_segs;
    t.gi = t.seg ? a.start_seg + local : a.S + a.start_blob + (local - a.num_segs);
    const double *p = t.seg ? a.xs + 3 * (size_t)t.gi : a.xb + 3 * (size_t)(t.gi - a.S);
    t.x = p[0];
    t.y = p[1];
    t.z = p[2];
    return t;
}
__device__ __forceinline__ double barrier_wall_z(const BarrierLaunch &a, const BarrierTarget &t)
{
    const double DL = 2.2 * a.rseg;
    if (!(t.seg && a.wall && t.z < 0.5 * DL)) return 0.0;
    const double fz = fmin(1.0, 1.0 - (t.z - a.rseg) / (0.5 * DL - a.rseg));
    return a.scale * fz * fz * fz * fz;
}
__device__ __forceinline__ void barrier_store(const BarrierLaunch &a, const BarrierTarget &t, int local, double g0,
                                              double g1, double g2)
{
    if (t.seg) {
        double *f = a.f_segs + 6 * (size_t)t.gi;
        f[0] += g0;
        f[1] += g1;
        f[2] += g2;
    } else {
        double *f = a.f_blobs_rep + 3 * (size_t)(local - a.num_segs);
        f[0] = g0;
        f[1] = g1;
        f[2] = g2;
    }
}
// the screen and exclusions of barrier_kernel for target t (screen position
// pf, squared cutoffs c2_s / c2_b against segment / blob sources) and source j
__device__ __forceinline__ bool barrier_candidate(const BarrierLaunch &a, const BarrierTarget &t, float4 pf,
                                                  float c2_s, float c2_b, int j, float4 s)
{
    const float dx = pf.x - s.x, dy = pf.y - s.y, dz = pf.z - s.z;
    const float d2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
    if (!(d2 < (j < a.S ? c2_s : c2_b))) return false;
    if (t.seg) {
        const int di = t.gi - j;
        return !((t.gi / a.nseg == j / a.nseg) && (di <= 1 && di >= -1));
    }
    return j != t.gi;
}
__device__ __forceinline__ void barrier_cutoffs(const BarrierLaunch &a, bool seg, float &c2_s, float &c2_b)
{
    const float margin = 1.0e-6f * __uint_as_float(*a.extent);
    const float cs = (seg ? a.cut_ss : a.cut_sb) + margin;
    const float cb = (seg ? a.cut_sb : a.cut_bb) + margin;
    c2_s = cs * cs;
    c2_b = cb * cb;
}

__global__ void __launch_bounds__(kCellTpb) barrier_cell_kernel(BarrierLaunch a, CellList c)
{
    __shared__ int cand[kCellCand * kCellTpb];  // candidate e of thread t at [e * kCellTpb + t]
    const int ntg = a.num_segs + (a.wall ? 0 : a.num_blobs);
    const int local = blockIdx.x * blockDim.x + threadIdx.x;
    if (local >= ntg) return;
    const int N = a.S + a.B;
    const BarrierTarget t = barrier_target(a, local);
    const float4 pf = a.screen[t.gi];
    float c2_s, c2_b;
    barrier_cutoffs(a, t.seg, c2_s, c2_b);
    const float inv_h = cell_inv_width(c);
    const int cx = cell_coord(pf.x, inv_h), cy = cell_coord(pf.y, inv_h), cz = cell_coord(pf.z, inv_h);
    int n = 0;
    bool over = false;
    for (int dz = -1; dz <= 1; ++dz)
        for (int dy = -1; dy <= 1; ++dy)
            for (int dx = -1; dx <= 1; ++dx) {
                const int b = cell_bucket(cx + dx, cy + dy, cz + dz, c.T);
                const int beg = cell_offset(c, b), end = b + 1 < c.T ? cell_offset(c, b + 1) : N;
                for (int p = beg; p < end; ++p) {
                    const int j = __ldcg(c.order + p);
                    if (!barrier_candidate(a, t, pf, c2_s, c2_b, j, a.screen[j])) continue;
                    if (n < kCellCand)
                        cand[n * kCellTpb + threadIdx.x] = j;
                    else
                        over = true;
                    ++n;
                }
            }
    if (over) {
        const int pos = atomicAdd(c.overflow, 1);
        c.overflow[1 + pos] = local;
        return;
    }
    // ascending j (insertion sort of a handful), repeats dropped below
    for (int e = 1; e < n; ++e) {
        const int v = cand[e * kCellTpb + threadIdx.x];
        int f = e - 1;
        while (f >= 0 && cand[f * kCellTpb + threadIdx.x] > v) {
            cand[(f + 1) * kCellTpb + threadIdx.x] = cand[f * kCellTpb + threadIdx.x];
            --f;
        }
        cand[(f + 1) * kCellTpb + threadIdx.x] = v;
    }
    const double a_tgt = t.seg ? a.rseg : a.rblob;
    double g0 = 0.0, g1 = 0.0, g2 = barrier_wall_z(a, t);
    int prev = -1;
    for (int e = 0; e < n; ++e) {
        const int j = cand[e * kCellTpb + threadIdx.x];
        if (j == prev) continue;
        prev = j;
        barrier_pair(a, j, t.x, t.y, t.z, a_tgt, g0, g1, g2);
    }
    barrier_store(a, t, local, g0, g1, g2);
}

// Targets with more candidates than the cell kernel keeps: one warp each,
// all sources screened 32 at a time and the accepted ones added in
// ascending j by lane 0 (the lanes evaluate their own source's force).
__global__ void __launch_bounds__(128) barrier_overflow_kernel(BarrierLaunch a, CellList c)
{
    const int lane = threadIdx.x & 31;
    const int warps = gridDim.x * (blockDim.x >> 5);
    const int N = a.S + a.B;
    const int todo = __ldcg(c.overflow);
    for (int w = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); w < todo; w += warps) {
        const int local = __ldcg(c.overflow + 1 + w);
        const BarrierTarget t = barrier_target(a, local);
        const float4 pf = a.screen[t.gi];
        float c2_s, c2_b;
        barrier_cutoffs(a, t.seg, c2_s, c2_b);
        const double a_tgt = t.seg ? a.rseg : a.rblob;
        double g0 = 0.0, g1 = 0.0, g2 = barrier_wall_z(a, t);
        for (int j0 = 0; j0 < N; j0 += 32) {
            const int j = j0 + lane;
            const bool cand = j < N && barrier_candidate(a, t, pf, c2_s, c2_b, j, a.screen[j]);
            unsigned mask = __ballot_sync(0xffffffffu, cand);
            double v0 = 0.0, v1 = 0.0, v2 = 0.0;
            if (cand) barrier_pair(a, j, t.x, t.y, t.z, a_tgt, v0, v1, v2);
            while (mask) {
                const int src = __ffs(mask) - 1;
                mask &= mask - 1;
                const double u0 = __shfl_sync(0xffffffffu, v0, src);
                const double u1 = __shfl_sync(0xffffffffu, v1, src);
                const double u2 = __shfl_sync(0xffffffffu, v2, src);
                g0 += u0;
                g1 += u1;
                g2 += u2;
            }
        }
        if (lane == 0) barrier_store(a, t, local, g0, g1, g2);
    }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
void fill_consts(PairConsts &c, double a_eq, double as, double ab, double mu)
{
    const double pi = kPi;
    c.eq[0] = 4.0 * a_eq * a_eq;
    c.eq[1] = 2.0 * a_eq * a_eq;
    c.eq[2] = 1.0 / (8.0 * pi * mu);
    c.eq[3] = 1.0 / (6.0 * pi * mu * a_eq);
    c.eq[4] = 3.0 / (32.0 * a_eq);
    c.eq[5] = 1.0 / a_eq;
    c.eq[6] = 1.0 / (8.0 * pi * mu * a_eq * a_eq * a_eq);
    c.eq[7] = 1.0 / (16.0 * pi * mu * a_eq * a_eq * a_eq);
    c.eq[8] = 3.0 / (8.0 * a_eq);
    const double dmin = fabs(as - ab);
    c.uq[0] = (as + ab) * (as + ab);
    c.uq[1] = dmin * dmin;
    c.uq[2] = (as * as + ab * ab) / 3.0;
    c.uq[3] = 0.5 * (as + ab);
    c.uq[4] = 1.0 / (8.0 * pi * mu);
    c.uq[5] = 1.0 / (6.0 * pi * mu * as * ab);
    c.uq[6] = 1.0 / (6.0 * pi * mu * (as > ab ? as : ab));
    c.uq[7] = 1.0 / (128.0 * pi * mu * ab * as * as * as);
    c.uq[8] = ab;
    c.uq[9] = as;
    c.uq[10] = ab * ab;
    c.uq[11] = (as > ab ? 1.0 : 0.0) / (8.0 * pi * mu * as * as * as);
    c.uq[12] = dmin;
}

gmi_status pack_records(gmi_context *ctx, const double *x, const double *f, int nf, int n, DeviceBuffer &buf)
{
    if (ctx->precision == GMI_DF64) {
        if (nf != 3) {
            set_last_error_msg("double-float pair sums exist for the blob-blob sum only");
            return GMI_ERR_ARG;
        }
        gmi_status st = buf.reserve(n > 0 ? (size_t)n * kRecLen * sizeof(float) : 16);
        if (st != GMI_OK) return st;
        if (n == 0) return GMI_OK;
        pack_records_df<<<(n + 255) / 256, 256, 0, ctx->stream>>>(x, f, n, static_cast<float4 *>(buf.ptr));
        ctx->launches++;
        GMI_CUDA_TRY(cudaGetLastError());
        return GMI_OK;
    }
    const bool f64 = ctx->precision == GMI_FP64;
    const size_t bytes = (size_t)n * kRecLen * (f64 ? sizeof(double) : sizeof(float));
    gmi_status st = buf.reserve(bytes > 0 ? bytes : 16);
    if (st != GMI_OK) return st;
    if (n == 0) return GMI_OK;
    const int tpb = 256;
    const int grid = (n + tpb - 1) / tpb;
    if (f64)
        pack_records_f64<<<grid, tpb, 0, ctx->stream>>>(x, f, nf, n, static_cast<double2 *>(buf.ptr));
    else
        pack_records_f32<<<grid, tpb, 0, ctx->stream>>>(x, f, nf, n, static_cast<float4 *>(buf.ptr));
    ctx->launches++;
    GMI_CUDA_TRY(cudaGetLastError());
    return GMI_OK;
}

static gmi_status make_record_map(gmi_context *ctx, CUtensorMap *map, const void *base, int n, bool f64)
{
    using EncodeFn = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
    auto encode = reinterpret_cast<EncodeFn>(ctx->encode_tiled);
    if (encode == nullptr) {
        set_last_error_msg("cuTensorMapEncodeTiled is unavailable from the driver");
        return GMI_ERR_CUDA;
    }
    const cuuint64_t esize = f64 ? 8 : 4;
    cuuint64_t dims[2] = {(cuuint64_t)kRecLen, (cuuint64_t)(n > 0 ? n : 1)};
    cuuint64_t strides[1] = {kRecLen * esize};
    cuuint32_t box[2] = {(cuuint32_t)kRecLen, (cuuint32_t)kTile};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = encode(map, f64 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2,
                        const_cast<void *>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                        CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        char msg[128];
        snprintf(msg, sizeof msg, "cuTensorMapEncodeTiled failed (CUresult %d)", (int)r);
        set_last_error_msg(msg);
        return GMI_ERR_CUDA;
    }
    return GMI_OK;
}

// Kernel table: (kind, precision, tpb, tt, packed) -> kernel.  Packed
// entries exist for FP32 and the kinds without a wall.
using KernelFn = void (*)(CUtensorMap, PairLaunch);

template <int KIND, class R, int TPB, int TT> struct Inst {
    static void *fn() { return reinterpret_cast<void *>(&rpy_pair_kernel<KIND, R, TPB, TT>); }
};
template <int KIND, class R, int TPB, int TT> struct Inst2 {
    static void *fn()
    {
        if constexpr (std::is_same<R, float>::value && KIND != kSSWall)
            return reinterpret_cast<void *>(&rpy_pair2_kernel<KIND, TPB, TT>);
        else
            return nullptr;
    }
};

struct ShapeEntry {
    int tpb, tt, packed;
};
static const ShapeEntry kShapes[] = {{128, 1, 0}, {128, 2, 0}, {256, 1, 0}, {256, 2, 0}, {128, 4, 0},
                                     {64, 1, 0},  {64, 2, 0},  {64, 1, 1},  {64, 2, 1},  {128, 1, 1},
                                     {128, 2, 1}, {256, 1, 1}};
constexpr int kNumShapes = sizeof(kShapes) / sizeof(kShapes[0]);

template <int KIND, class R> static void *kernel_for_shape(int idx)
{
    switch (idx) {
        case 0: return Inst<KIND, R, 128, 1>::fn();
        case 1: return Inst<KIND, R, 128, 2>::fn();
        case 2: return Inst<KIND, R, 256, 1>::fn();
        case 3: return Inst<KIND, R, 256, 2>::fn();
        case 4: return Inst<KIND, R, 128, 4>::fn();
        case 5: return Inst<KIND, R, 64, 1>::fn();
        case 6: return Inst<KIND, R, 64, 2>::fn();
        case 7: return Inst2<KIND, R, 64, 1>::fn();
        case 8: return Inst2<KIND, R, 64, 2>::fn();
        case 9: return Inst2<KIND, R, 128, 1>::fn();
        case 10: return Inst2<KIND, R, 128, 2>::fn();
        default: return Inst2<KIND, R, 256, 1>::fn();
    }
}

static void *kernel_ptr(int kind, bool f64, int shape_idx)
{
    switch (kind) {
        case kSS: return f64 ? kernel_for_shape<kSS, double>(shape_idx) : kernel_for_shape<kSS, float>(shape_idx);
        case kSSWall:
            return f64 ? kernel_for_shape<kSSWall, double>(shape_idx) : kernel_for_shape<kSSWall, float>(shape_idx);
        case kBB: return f64 ? kernel_for_shape<kBB, double>(shape_idx) : kernel_for_shape<kBB, float>(shape_idx);
        case kSB: return f64 ? kernel_for_shape<kSB, double>(shape_idx) : kernel_for_shape<kSB, float>(shape_idx);
        default: return f64 ? kernel_for_shape<kBS, double>(shape_idx) : kernel_for_shape<kBS, float>(shape_idx);
    }
}

static bool packed_available(int kind, bool f64) { return !f64 && kind != kSSWall; }

constexpr int kWarpShapeTpb = kPairWarpShapeTpb;
constexpr int kWarpMaxSources = kPairWarpMaxSources;

template <int KIND> static void *warp_kernel_for(bool f64, int tpw)
{
    if (f64) return tpw >= 2 ? reinterpret_cast<void *>(&rpy_pair_warp_kernel<KIND, double, 2>)
                              : reinterpret_cast<void *>(&rpy_pair_warp_kernel<KIND, double, 1>);
    return tpw >= 2 ? reinterpret_cast<void *>(&rpy_pair_warp_kernel<KIND, float, 2>)
                    : reinterpret_cast<void *>(&rpy_pair_warp_kernel<KIND, float, 1>);
}

static void *warp_kernel_ptr(int kind, bool f64, int tpw)
{
    switch (kind) {
        case kSS: return warp_kernel_for<kSS>(f64, tpw);
        case kSSWall: return warp_kernel_for<kSSWall>(f64, tpw);
        case kBB: return warp_kernel_for<kBB>(f64, tpw);
        case kSB: return warp_kernel_for<kSB>(f64, tpw);
        default: return warp_kernel_for<kBS>(f64, tpw);
    }
}

// cudaLaunchKernel, or with pdl the same launch marked for programmatic
// dependent launch (the kernel may start while the previous one on the
// stream finishes; it waits in pdl_wait_then_release)
static cudaError_t launch_fn(const void *fn, dim3 grid, dim3 block, void **params, size_t smem, cudaStream_t stream,
                             bool pdl)
{
    if (!pdl) return cudaLaunchKernel(fn, grid, block, params, smem, stream);
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelExC(&cfg, fn, params);
}

static gmi_status launch_warp(cudaStream_t stream, int kind, bool f64, int tpw, const PairLaunch &a,
                              const void *src_rec, bool pdl = false)
{
    tpw = tpw >= 2 ? 2 : 1;
    void *fn = warp_kernel_ptr(kind, f64, tpw);
    const long long warps = ((long long)a.n_tgt + tpw - 1) / tpw;
    const int ctas = (int)((warps * 32 + kWarpCta - 1) / kWarpCta);
    PairLaunch la = a;
    la.partial = nullptr;
    void *params[] = {&la, const_cast<void **>(&src_rec)};
    GMI_CUDA_TRY(launch_fn(fn, dim3(ctas), dim3(kWarpCta), params, 0, stream, pdl));
    return GMI_OK;
}

// Index of the table entry for (tpb, tt); packed < 0 picks the packed
// variant where it exists.  Falls back to the scalar (tpb, tt) entry, then to
// 128 x 2.
static int shape_index(int tpb, int tt, int packed, int kind, bool f64)
{
    const int want = packed < 0 ? (packed_available(kind, f64) ? 1 : 0) : (packed_available(kind, f64) ? packed : 0);
    for (int i = 0; i < kNumShapes; ++i)
        if (kShapes[i].tpb == tpb && kShapes[i].tt == tt && kShapes[i].packed == want) return i;
    for (int i = 0; i < kNumShapes; ++i)
        if (kShapes[i].tpb == tpb && kShapes[i].tt == tt && kShapes[i].packed == 0) return i;
    return 1;
}

bool pair_shape_exists(const PairShape &s, int kind, bool f64)
{
    if (s.tpb == kWarpShapeTpb) return (s.tt == 1 || s.tt == 2) && s.packed != 1;
    for (int i = 0; i < kNumShapes; ++i)
        if (kShapes[i].tpb == s.tpb && kShapes[i].tt == s.tt &&
            (s.packed < 0 || kShapes[i].packed == s.packed) && (!kShapes[i].packed || packed_available(kind, f64)))
            return true;
    return false;
}

bool pair_shape_is_packed(const PairShape &s, int kind, bool f64)
{
    if (s.tpb == kWarpShapeTpb) return false;
    return kShapes[shape_index(s.tpb, s.tt, s.packed, kind, f64)].packed != 0;
}

static size_t ring_bytes(bool f64, bool packed)
{
    if (packed) return (size_t)(kStagesP + 2) * kTile * kRecLen * sizeof(float) + kStagesP * 8;
    return (size_t)kStages * kTile * kRecLen * (f64 ? 8 : 4) + kStages * 8;
}

// the packed kernel's shared memory when every split is one tile: ring
// stage 0, interleave buffer 0 and the barriers (rpy_pair2_kernel)
static size_t ring_bytes_single_tile() { return (size_t)2 * kTile * kRecLen * sizeof(float) + kStagesP * 8; }

static int nout_of(int kind) { return (kind == kBB || kind == kBS) ? 3 : 6; }

// Source splits: enough CTAs for ~2 full waves when the target tiles alone
// cannot fill the GPU; every split keeps at least one tile of sources.
static int choose_splits(const gmi_context *ctx, int n_tgt_ctas, int n_src, int occ)
{
    const int slots = ctx->sm_count * (occ > 0 ? occ : 1);
    const int max_splits = (n_src + kTile - 1) / kTile;
    if (n_tgt_ctas >= 2 * slots) return 1;
    int s = (2 * slots + n_tgt_ctas - 1) / n_tgt_ctas;
    return s < max_splits ? s : max_splits;
}

// The double-float blob-blob sum: the warp kernel for small systems, else
// 128 targets per CTA, the sources split over enough CTAs for two waves, the
// splits added in order.
constexpr int kDfTpb = 128;
static gmi_status launch_bb_df(gmi_context *ctx, const void *tgt_rec, int tgt_start, int n_tgt, const void *src_rec,
                               int n_src, const PairConsts &k, double *out, int accumulate)
{
    DfBBConsts K;
    K.four_a2 = df_from_double(k.eq[0]);
    K.two_a2 = df_from_double(k.eq[1]);
    K.f8pm = df_from_double(k.eq[2]);
    K.f6pma = df_from_double(k.eq[3]);
    K.q32 = df_from_double(k.eq[4]);
    K.third = df_from_double(1.0 / 3.0);
    if (n_src <= kPairWarpMaxSources) {
        PairLaunch a{};
        a.tgt_rec = tgt_rec;
        a.tgt_start = tgt_start;
        a.n_tgt = n_tgt;
        a.n_src = n_src;
        a.out = out;
        a.accumulate = accumulate;
        const unsigned ctas = (unsigned)(((long long)n_tgt * 32 + 127) / 128);
        rpy_bb_df_warp_kernel<<<ctas, 128, 0, ctx->stream>>>(a, static_cast<const float4 *>(src_rec), K);
        ctx->launches++;
        GMI_CUDA_TRY(cudaGetLastError());
        return GMI_OK;
    }
    void *fn = reinterpret_cast<void *>(&rpy_bb_df_kernel<kDfTpb>);
    const size_t smem = ring_bytes(false, false);
    GMI_CUDA_TRY(raise_dynamic_smem_limit(fn, smem));
    int occ = 0;
    GMI_CUDA_TRY(max_active_blocks(&occ, fn, kDfTpb, smem));
    const int n_tgt_ctas = (n_tgt + kDfTpb - 1) / kDfTpb;
    const int slots = ctx->sm_count * (occ > 0 ? occ : 1);
    int splits = 1;
    if (n_tgt_ctas < 2 * slots) splits = (2 * slots + n_tgt_ctas - 1) / n_tgt_ctas;
    const int max_by_src = (n_src + kTile - 1) / kTile;
    if (splits > max_by_src) splits = max_by_src;
    int chunk = (n_src + splits - 1) / splits;
    chunk = (chunk + kTile - 1) / kTile * kTile;
    splits = (n_src + chunk - 1) / chunk;
    PairLaunch a{};
    a.tgt_rec = tgt_rec;
    a.tgt_start = tgt_start;
    a.n_tgt = n_tgt;
    a.n_src = n_src;
    a.chunk = chunk;
    a.k = k;
    a.out = out;
    a.accumulate = accumulate;
    a.err = ctx->d_err;
    a.wait_ns = ctx->wait_ns;
    a.partial = nullptr;
    if (splits > 1) {
        gmi_status st = ctx->partial.reserve((size_t)splits * n_tgt * 3 * sizeof(double));
        if (st != GMI_OK) return st;
        a.partial = static_cast<double *>(ctx->partial.ptr);
    }
    CUtensorMap map;
    gmi_status st = make_record_map(ctx, &map, src_rec, n_src, false);
    if (st != GMI_OK) return st;
    void *params[] = {&map, &a, &K};
    GMI_CUDA_TRY(cudaLaunchKernel(fn, dim3(n_tgt_ctas, splits), dim3(kDfTpb), params, smem, ctx->stream));
    ctx->launches++;
    if (splits > 1) {
        const int count = n_tgt * 3;
        reduce_splits<<<(count + 255) / 256, 256, 0, ctx->stream>>>(a.partial, splits, count, out, accumulate,
                                                                    nullptr);
        ctx->launches++;
        GMI_CUDA_TRY(cudaGetLastError());
    }
    return GMI_OK;
}

gmi_status launch_pair(gmi_context *ctx, int kind, const void *tgt_rec, int tgt_start, int n_tgt, const void *src_rec,
                       int n_src, const PairConsts &k, double *out, int accumulate, const PairShape *force_shape)
{
    if (n_tgt <= 0) return GMI_OK;
    if (ctx->precision == GMI_DF64) {
        if (kind != kBB) {
            set_last_error_msg("double-float pair sums exist for the blob-blob sum only");
            return GMI_ERR_ARG;
        }
        if (n_src <= 0) {
            if (!accumulate) GMI_CUDA_TRY(cudaMemsetAsync(out, 0, (size_t)n_tgt * 3 * sizeof(double), ctx->stream));
            return GMI_OK;
        }
        return launch_bb_df(ctx, tgt_rec, tgt_start, n_tgt, src_rec, n_src, k, out, accumulate);
    }
    const bool f64 = ctx->precision == GMI_FP64;
    const int nout = nout_of(kind);
    if (n_src <= 0) {
        if (!accumulate) GMI_CUDA_TRY(cudaMemsetAsync(out, 0, (size_t)n_tgt * nout * sizeof(double), ctx->stream));
        return GMI_OK;
    }
    PairShape shape;
    if (force_shape) {
        shape = *force_shape;
    } else {
        auto it = ctx->tuned.find(TuneKey{kind, ctx->precision, n_tgt, n_src});
        if (it != ctx->tuned.end()) {
            shape = it->second;
        } else if (n_src <= kWarpMaxSources) {
            shape = PairShape{kWarpShapeTpb, 2, 0};  // few sources: warp per two targets
        } else if ((long long)n_tgt * 2 < (long long)ctx->sm_count * 256) {
            shape = PairShape{64, 1, 0};  // small target sets: more, smaller CTAs
        } else if (packed_available(kind, f64)) {
            shape = PairShape{128, 1, 0};
        }
    }
    if (shape.tpb == kWarpShapeTpb) {
        PairLaunch a{};
        a.tgt_rec = tgt_rec;
        a.tgt_start = tgt_start;
        a.n_tgt = n_tgt;
        a.n_src = n_src;
        a.k = k;
        a.out = out;
        a.accumulate = accumulate;
        a.err = ctx->d_err;
        a.wait_ns = ctx->wait_ns;
        const gmi_status ws = launch_warp(ctx->stream, kind, f64, shape.tt, a, src_rec);
        if (ws == GMI_OK) ctx->launches++;
        return ws;
    }
    const int sidx = shape_index(shape.tpb, shape.tt, shape.packed, kind, f64);
    const int tpb = kShapes[sidx].tpb, tt = kShapes[sidx].tt;
    void *fn = kernel_ptr(kind, f64, sidx);
    const size_t smem = ring_bytes(f64, kShapes[sidx].packed != 0);
    GMI_CUDA_TRY(raise_dynamic_smem_limit(fn, smem));
    int occ = 0;
    GMI_CUDA_TRY(max_active_blocks(&occ, fn, tpb, smem));
    const int n_tgt_ctas = (n_tgt + tpb * tt - 1) / (tpb * tt);
    int splits = shape.splits > 0 ? shape.splits : choose_splits(ctx, n_tgt_ctas, n_src, occ);
    int chunk = (n_src + splits - 1) / splits;
    chunk = (chunk + kTile - 1) / kTile * kTile;
    splits = (n_src + chunk - 1) / chunk;
    ctx->last_splits = splits;

    PairLaunch a{};
    a.tgt_rec = tgt_rec;
    a.tgt_start = tgt_start;
    a.n_tgt = n_tgt;
    a.n_src = n_src;
    a.chunk = chunk;
    a.k = k;
    a.out = out;
    a.accumulate = accumulate;
    a.err = ctx->d_err;
    a.wait_ns = ctx->wait_ns;
    a.partial = nullptr;
    if (splits > 1) {
        gmi_status st = ctx->partial.reserve((size_t)splits * n_tgt * nout * sizeof(double));
        if (st != GMI_OK) return st;
        a.partial = static_cast<double *>(ctx->partial.ptr);
    }
    CUtensorMap map;
    gmi_status st = make_record_map(ctx, &map, src_rec, n_src, f64);
    if (st != GMI_OK) return st;
    void *params[] = {&map, &a};
    dim3 grid(n_tgt_ctas, splits);
    const size_t smem_run = (kShapes[sidx].packed != 0 && chunk <= kTile) ? ring_bytes_single_tile() : smem;
    GMI_CUDA_TRY(cudaLaunchKernel(fn, grid, dim3(tpb), params, smem_run, ctx->stream));
    ctx->launches++;
    if (splits > 1) {
        const int count = n_tgt * nout;
        reduce_splits<<<(count + 255) / 256, 256, 0, ctx->stream>>>(a.partial, splits, count, out, accumulate,
                                                                    nullptr);
        ctx->launches++;
        GMI_CUDA_TRY(cudaGetLastError());
    }
    return GMI_OK;
}

gmi_status launch_barrier(gmi_context *ctx, const BarrierLaunch &in)
{
    BarrierLaunch a = in;
    const int N = a.S + a.B;
    const int ntg = a.num_segs + (a.wall ? 0 : a.num_blobs);
    if (ntg <= 0) return GMI_OK;
    gmi_status st = ctx->rec_tgt.reserve((size_t)(N > 0 ? N : 1) * sizeof(float4) + sizeof(float4));
    if (st != GMI_OK) return st;
    a.screen = static_cast<float4 *>(ctx->rec_tgt.ptr);
    a.extent = reinterpret_cast<unsigned *>(a.screen + (N > 0 ? N : 1));
    // screen cutoffs 1.1 (a_i + a_j) with a relative margin of 1e-3 (FP32
    // rounding of the separation and of the cutoff); the kernel adds the
    // offsets' rounding; pairs inside are re-evaluated in FP64
    auto cut = [](double asum) { return (float)(1.1 * asum) * 1.001f; };
    a.cut_ss = cut(2.0 * a.rseg);
    a.cut_sb = cut(a.rseg + a.rblob);
    a.cut_bb = cut(2.0 * a.rblob);
    // source splits: enough CTAs for ~8 per SM, at least 64 sources each
    const int tgt_ctas = (ntg + kBarrierTpb - 1) / kBarrierTpb;
    int splits = (8 * ctx->sm_count + tgt_ctas - 1) / tgt_ctas;
    splits = std::max(1, std::min(splits, N / 64));
    a.chunk = (N + splits - 1) / splits;
    splits = (N + a.chunk - 1) / a.chunk;
    a.partial = nullptr;
    if (splits > 1) {
        st = ctx->partial.reserve((size_t)splits * ntg * 3 * sizeof(double));
        if (st != GMI_OK) return st;
        a.partial = static_cast<double *>(ctx->partial.ptr);
    }
    GMI_CUDA_TRY(cudaMemsetAsync(a.extent, 0, sizeof(unsigned), ctx->stream));
    pack_screen_positions<<<(N + 255) / 256, 256, 0, ctx->stream>>>(a.xs, a.S, a.xb, a.B, a.screen, a.extent);
    ctx->launches++;
    // the cell list from kCellMinParticles particles (GMI_BARRIER_CELLS=0
    // never, =1 always), up to the scan's 4 M buckets
    const char *cells_env = std::getenv("GMI_BARRIER_CELLS");
    const bool cells = cells_env ? cells_env[0] != '0' : N >= kCellMinParticles;
    int T = kCellScanTile;
    while (T < 2 * N) T *= 2;
    if (cells && T / kCellScanTile <= kCellScanTpb) {
        a.partial = nullptr;
        const size_t tiles = (size_t)T / kCellScanTile;
        const size_t ints = 4 + 2 * (size_t)T + ((tiles + 3) & ~(size_t)3) + 2 * (size_t)N + 1 + (size_t)ntg;
        st = ctx->cells.reserve(ints * sizeof(int));
        if (st != GMI_OK) return st;
        CellList c{};
        int *base = static_cast<int *>(ctx->cells.ptr);
        c.T = T;
        c.cut_max = std::max(a.cut_ss, std::max(a.cut_sb, a.cut_bb));
        c.extent = a.extent;
        c.ticket = base;
        c.count = base + 4;
        c.local = c.count + T;
        c.tile_prefix = c.local + T;
        c.key = c.tile_prefix + ((tiles + 3) & ~(size_t)3);
        c.order = c.key + N;
        c.overflow = c.order + N;
        GMI_CUDA_TRY(cudaMemsetAsync(base, 0, (4 + (size_t)T) * sizeof(int), ctx->stream));
        GMI_CUDA_TRY(cudaMemsetAsync(c.overflow, 0, sizeof(int), ctx->stream));
        cell_keys_kernel<<<(N + 255) / 256, 256, 0, ctx->stream>>>(c, a.screen, N);
        cell_scan_kernel<<<(unsigned)tiles, kCellScanTpb, 0, ctx->stream>>>(c);
        cell_scatter_kernel<<<(N + 255) / 256, 256, 0, ctx->stream>>>(c, N);
        barrier_cell_kernel<<<(ntg + kCellTpb - 1) / kCellTpb, kCellTpb, 0, ctx->stream>>>(a, c);
        barrier_overflow_kernel<<<ctx->sm_count, 128, 0, ctx->stream>>>(a, c);
        ctx->launches += 5;
        GMI_CUDA_TRY(cudaGetLastError());
        return GMI_OK;
    }
    barrier_kernel<<<dim3(tgt_ctas, splits), kBarrierTpb, 0, ctx->stream>>>(a);
    ctx->launches++;
    if (splits > 1) {
        barrier_reduce<<<(3 * ntg + 255) / 256, 256, 0, ctx->stream>>>(a, splits);
        ctx->launches++;
    }
    GMI_CUDA_TRY(cudaGetLastError());
    return GMI_OK;
}

// Autotuner: time each candidate shape (with the automatic split choice and
// with a few explicit split counts) on the records already packed for this
// problem.  Among the candidates within 1 % of the fastest it keeps the one
// with the fewest source splits: the split partial sums (FP64, one set per
// split) are the kernel's only DRAM traffic beyond the records, and fewer
// of them stay in L2.
gmi_status autotune_pair(gmi_context *ctx, int kind, const void *tgt_rec, int n_tgt, const void *src_rec, int n_src,
                         const PairConsts &k, double *out)
{
    cudaEvent_t e0, e1;
    GMI_CUDA_TRY(cudaEventCreate(&e0));
    GMI_CUDA_TRY(cudaEventCreate(&e1));
    struct Timed {
        PairShape shape;
        float ms;
        int splits;  // the split count the launch used (automatic choices resolved)
    };
    std::vector<Timed> timed;
    const bool f64 = ctx->precision == GMI_FP64;
    for (int si = 0; si < kNumShapes + 2; ++si) {
        const bool warp = si >= kNumShapes;
        if (!warp && kShapes[si].packed && !packed_available(kind, f64)) continue;
        if (warp && n_src > 4 * kWarpMaxSources) continue;  // the warp kernel is for small source sets
        for (int sp : {0, 1, 2, 4, 8, 16, 32}) {
            if (warp && sp != 0) continue;
            PairShape s = warp ? PairShape{kWarpShapeTpb, si - kNumShapes + 1, 0}
                               : PairShape{kShapes[si].tpb, kShapes[si].tt, sp, kShapes[si].packed};
            gmi_status st = launch_pair(ctx, kind, tgt_rec, 0, n_tgt, src_rec, n_src, k, out, 0, &s);
            if (st != GMI_OK) return st;
            GMI_CUDA_TRY(cudaEventRecord(e0, ctx->stream));
            for (int rep = 0; rep < 3; ++rep) {
                st = launch_pair(ctx, kind, tgt_rec, 0, n_tgt, src_rec, n_src, k, out, 0, &s);
                if (st != GMI_OK) return st;
            }
            GMI_CUDA_TRY(cudaEventRecord(e1, ctx->stream));
            GMI_CUDA_TRY(cudaEventSynchronize(e1));
            float ms = 0.f;
            GMI_CUDA_TRY(cudaEventElapsedTime(&ms, e0, e1));
            timed.push_back(Timed{s, ms, warp ? 1 : ctx->last_splits});
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    float best = 1e30f;
    for (const Timed &t : timed) best = std::min(best, t.ms);
    const Timed *pick = nullptr;
    for (const Timed &t : timed)
        if (t.ms <= 1.01f * best && (pick == nullptr || t.splits < pick->splits ||
                                     (t.splits == pick->splits && t.ms < pick->ms)))
            pick = &t;
    if (pick != nullptr) ctx->tuned[TuneKey{kind, ctx->precision, n_tgt, n_src}] = pick->shape;
    return context_check_device_errors(ctx);
}

}  // namespace gmi

// ---------------------------------------------------------------------------
// Launchers on caller-provided buffers (no gmi_context): used by the
// allocation-free entry point in gmi_noalloc.cu.
// ---------------------------------------------------------------------------
namespace gmi {

gmi_status pack_records_into(cudaStream_t stream, bool f64, const double *x, const double *f, int nf, int n,
                             void *dst)
{
    if (n == 0) return GMI_OK;
    const int tpb = 256, grid = (n + tpb - 1) / tpb;
    if (f64)
        pack_records_f64<<<grid, tpb, 0, stream>>>(x, f, nf, n, static_cast<double2 *>(dst));
    else
        pack_records_f32<<<grid, tpb, 0, stream>>>(x, f, nf, n, static_cast<float4 *>(dst));
    GMI_CUDA_TRY(cudaGetLastError());
    return GMI_OK;
}

size_t record_bytes(bool f64) { return (size_t)kRecLen * (f64 ? sizeof(double) : sizeof(float)); }

// The record tensor map of make_record_map, from an explicit encoder.
static gmi_status encode_record_map(void *encode_tiled, CUtensorMap *map, const void *base, int n, bool f64)
{
    using EncodeFn = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
    auto encode = reinterpret_cast<EncodeFn>(encode_tiled);
    if (encode == nullptr) {
        set_last_error_msg("cuTensorMapEncodeTiled is unavailable from the driver");
        return GMI_ERR_CUDA;
    }
    const cuuint64_t esize = f64 ? 8 : 4;
    cuuint64_t dims[2] = {(cuuint64_t)kRecLen, (cuuint64_t)(n > 0 ? n : 1)};
    cuuint64_t strides[1] = {kRecLen * esize};
    cuuint32_t box[2] = {(cuuint32_t)kRecLen, (cuuint32_t)kTile};
    cuuint32_t estr[2] = {1, 1};
    const CUresult r = encode(map, f64 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2,
                              const_cast<void *>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                              CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        set_last_error_msg("cuTensorMapEncodeTiled failed");
        return GMI_ERR_CUDA;
    }
    return GMI_OK;
}

gmi_status launch_pair_into(const ExplicitPairEnv &env, int kind, bool f64, const void *tgt_rec, int tgt_start,
                            int n_tgt, const void *src_rec, int n_src, const PairConsts &k, double *out,
                            int accumulate)
{
    if (env.splits_out) *env.splits_out = 1;
    if (n_tgt <= 0) return GMI_OK;
    const int nout = nout_of(kind);
    if (n_src <= 0) {
        if (!accumulate) GMI_CUDA_TRY(cudaMemsetAsync(out, 0, (size_t)n_tgt * nout * sizeof(double), env.stream));
        return GMI_OK;
    }
    if (env.tpb == kWarpShapeTpb) {
        PairLaunch a{};
        a.tgt_rec = tgt_rec;
        a.tgt_start = tgt_start;
        a.n_tgt = n_tgt;
        a.n_src = n_src;
        a.k = k;
        a.out = out;
        a.accumulate = accumulate;
        a.err = env.err;
        a.wait_ns = env.wait_ns;
        a.skip = env.skip;
        return launch_warp(env.stream, kind, f64, env.tt, a, src_rec, env.pdl != 0);
    }
    const int sidx = shape_index(env.tpb, env.tt, env.scalar_only ? 0 : -1, kind, f64);
    const int tpb = kShapes[sidx].tpb, tt = kShapes[sidx].tt;
    void *fn = kernel_ptr(kind, f64, sidx);
    const size_t smem = ring_bytes(f64, kShapes[sidx].packed != 0);
    GMI_CUDA_TRY(raise_dynamic_smem_limit(fn, smem));
    int occ = 0;
    GMI_CUDA_TRY(max_active_blocks(&occ, fn, tpb, smem));
    const int n_tgt_ctas = (n_tgt + tpb * tt - 1) / (tpb * tt);
    const int slots = env.sm_count * (occ > 0 ? occ : 1);
    int splits = 1;
    if (n_tgt_ctas < 2 * slots) splits = (2 * slots + n_tgt_ctas - 1) / n_tgt_ctas;
    const int max_by_src = (n_src + kTile - 1) / kTile;
    if (splits > max_by_src) splits = max_by_src;
    const size_t per_split = (size_t)n_tgt * nout * sizeof(double);
    const int max_by_scratch = env.partial_bytes / per_split > 0 ? (int)(env.partial_bytes / per_split) : 1;
    if (splits > max_by_scratch) splits = max_by_scratch;
    if (env.max_splits > 0 && splits > env.max_splits) splits = env.max_splits;
    if (splits < 1) splits = 1;
    int chunk = (n_src + splits - 1) / splits;
    chunk = (chunk + kTile - 1) / kTile * kTile;
    splits = (n_src + chunk - 1) / chunk;

    PairLaunch a{};
    a.tgt_rec = tgt_rec;
    a.tgt_start = tgt_start;
    a.n_tgt = n_tgt;
    a.n_src = n_src;
    a.chunk = chunk;
    a.k = k;
    a.out = out;
    a.accumulate = accumulate;
    a.err = env.err;
    a.wait_ns = env.wait_ns;
    a.partial = splits > 1 ? env.partial : nullptr;
    a.skip = env.skip;
    CUtensorMap map;
    gmi_status st = encode_record_map(env.encode_tiled, &map, src_rec, n_src, f64);
    if (st != GMI_OK) return st;
    void *params[] = {&map, &a};
    const size_t smem_run = (kShapes[sidx].packed != 0 && chunk <= kTile) ? ring_bytes_single_tile() : smem;
    GMI_CUDA_TRY(launch_fn(fn, dim3(n_tgt_ctas, splits), dim3(tpb), params, smem_run, env.stream, env.pdl != 0));
    if (env.splits_out) {
        *env.splits_out = splits;
        return GMI_OK;
    }
    if (splits > 1) {
        const int count = n_tgt * nout;
        reduce_splits<<<(count + 255) / 256, 256, 0, env.stream>>>(a.partial, splits, count, out, accumulate,
                                                                   env.skip);
        GMI_CUDA_TRY(cudaGetLastError());
    }
    return GMI_OK;
}

}  // namespace gmi
