// gmi_pair_kernels.hpp -- host interface of the tiled pair kernels.
#pragma once

#include "gmi_context.hpp"

namespace gmi {

// Physical constants of one pair kind, precomputed on the host in FP64
// (converted to the kernel's scalar type on the device).
struct PairConsts {
    double eq[9];   // equal radii: see EqualK
    double uq[13];  // segment/blob radii: see UnequalK
};

struct PairLaunch {
    const void *tgt_rec;  // records of the target set
    int tgt_start, n_tgt; // targets [tgt_start, tgt_start + n_tgt)
    int n_src, chunk;     // sources, sources per split (multiple of the tile)
    PairConsts k;
    double *out;          // direct output when there is one split
    double *partial;      // [splits][n_tgt][nout] when there are several
    int accumulate;
    unsigned *err;
    const int *skip;      // if non-null and *skip != 0 the launch does nothing (converged GMRES)
    unsigned long long wait_ns;  // deadline of the source-tile waits (0: kWaitDeadlineNs)
    int max_splits;              // cap on the source splits (0: none beyond the automatic choice)
};

struct BarrierLaunch {
    double *f_segs;
    double *f_blobs_rep;
    const double *xs;
    const double *xb;
    float4 *screen;   // FP32 positions of all S + B particles relative to the first (filled by the launcher)
    unsigned *extent;  // largest |coordinate| of `screen`, as FP32 bits (filled by the launcher)
    int S, B;
    int start_seg, num_segs, start_blob, num_blobs;
    int nseg;
    double rseg, rblob, scale;
    int wall;
    float cut_ss, cut_sb, cut_bb;  // FP32 screen cutoffs before the rounding margin (filled by the launcher)
    int chunk;            // sources per split (filled by the launcher)
    double *partial;      // [splits][targets][3] when there are several splits (filled by the launcher)
};

// Launch shape with tpb == kPairWarpShapeTpb: the warp-per-target kernel for
// small source sets (tt = targets per warp, 1 or 2).  Chosen by default for
// up to kPairWarpMaxSources sources.
constexpr int kPairWarpShapeTpb = 32;
constexpr int kPairWarpMaxSources = 2048;

void fill_consts(PairConsts &c, double a_eq, double a_seg, double a_blob, double mu);

// Pack AoS FP64 positions (and forces with nf = 3 or 6 components, or none
// when f == nullptr) into the context's record format for its precision.
gmi_status pack_records(gmi_context *ctx, const double *x, const double *f, int nf, int n, DeviceBuffer &buf);

// One pair sum: out[nout*(i)] (=|+=) sum_j M(i, j) F_j for targets
// [tgt_start, tgt_start + n_tgt).  force_shape overrides the tuned shape.
gmi_status launch_pair(gmi_context *ctx, int kind, const void *tgt_rec, int tgt_start, int n_tgt, const void *src_rec,
                       int n_src, const PairConsts &k, double *out, int accumulate,
                       const PairShape *force_shape = nullptr);

gmi_status launch_barrier(gmi_context *ctx, const BarrierLaunch &a);

// Whether a kernel exists for this shape, kind and precision, and whether the
// shape resolves to the packed (two sources per step) kernel.
bool pair_shape_exists(const PairShape &s, int kind, bool f64);
bool pair_shape_is_packed(const PairShape &s, int kind, bool f64);

gmi_status autotune_pair(gmi_context *ctx, int kind, const void *tgt_rec, int n_tgt, const void *src_rec, int n_src,
                         const PairConsts &k, double *out);

// Everything a pair launch needs, supplied by the caller instead of a context.
struct ExplicitPairEnv {
    cudaStream_t stream;
    double *partial;       // split partial sums
    size_t partial_bytes;  // capacity of `partial`; bounds the number of splits
    unsigned *err;         // device error word
    void *encode_tiled;    // cuTensorMapEncodeTiled
    int sm_count;
    int tpb, tt;           // launch shape
    int scalar_only;       // non-zero: one source per thread step even where the packed kernel exists
    const int *skip;       // optional device flag: non-zero turns the launch into a no-op
    int *splits_out;       // optional: the caller adds the per-split partials (partial[p * 3 n_tgt + e],
                           // p < *splits_out) itself; 1 means the kernel wrote `out` directly
    int pdl;               // non-zero: launch for programmatic dependent launch (the pair kernel
                           // waits for the previous kernel in pdl_wait_then_release)
    unsigned long long wait_ns;  // deadline of the source-tile waits (0: kWaitDeadlineNs)
    int max_splits;              // cap on the source splits (0: none beyond the automatic choice)
};

size_t record_bytes(bool f64);
gmi_status pack_records_into(cudaStream_t stream, bool f64, const double *x, const double *f, int nf, int n,
                             void *dst);
gmi_status launch_pair_into(const ExplicitPairEnv &env, int kind, bool f64, const void *tgt_rec, int tgt_start,
                            int n_tgt, const void *src_rec, int n_src, const PairConsts &k, double *out,
                            int accumulate);

}  // namespace gmi
