// gmi_capi_pairs.cu -- extern "C" entry points for the context and the
// reference-shaped pair sums (include/gmi.h).
#include <cmath>
#include <new>

#include "gmi_context.hpp"
#include "gmi_pair_kernels.hpp"

namespace gmi {
const char *last_error();
}

using namespace gmi;

#define GMI_ARG_CHECK(cond, msg)         \
    do {                                 \
        if (!(cond)) {                   \
            set_last_error_msg(msg);     \
            return GMI_ERR_ARG;          \
        }                                \
    } while (0)

static gmi_status select_device(gmi_context *ctx)
{
    GMI_CUDA_TRY(cudaSetDevice(ctx->device));
    return GMI_OK;
}

static bool range_ok(int start, int num, int total) { return start >= 0 && num >= 0 && total >= 0 && start + num <= total; }

extern "C" {

const char *gmi_last_error(void) { return gmi::last_error(); }

int gmi_version(void) { return 100; }

gmi_status gmi_context_create(int device, gmi_context **out)
{
    GMI_ARG_CHECK(out != nullptr, "gmi_context_create: out is null");
    *out = nullptr;
    gmi_context *ctx = new (std::nothrow) gmi_context();
    GMI_ARG_CHECK(ctx != nullptr, "gmi_context_create: out of host memory");
    gmi_status st = context_init(ctx, device);
    if (st != GMI_OK) {
        gmi_context_destroy(ctx);
        return st;
    }
    *out = ctx;
    return GMI_OK;
}

gmi_status gmi_context_destroy(gmi_context *ctx)
{
    if (ctx == nullptr) return GMI_OK;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    ctx->rec_src.release();
    ctx->rec_tgt.release();
    ctx->partial.release();
    ctx->cells.release();
    if (ctx->d_err) gmi::dev_free(ctx->d_err);
    if (ctx->h_err) gmi::host_free(ctx->h_err);
    if (ctx->own_stream && ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return GMI_OK;
}

gmi_status gmi_context_set_stream(gmi_context *ctx, void *cuda_stream)
{
    GMI_ARG_CHECK(ctx != nullptr, "null context");
    GMI_CUDA_TRY(cudaSetDevice(ctx->device));
    if (cuda_stream == nullptr) {
        if (!ctx->own_stream) {
            GMI_CUDA_TRY(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
            ctx->own_stream = true;
        }
        return GMI_OK;
    }
    if (ctx->own_stream && ctx->stream) {
        GMI_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
        GMI_CUDA_TRY(cudaStreamDestroy(ctx->stream));
    }
    ctx->stream = static_cast<cudaStream_t>(cuda_stream);
    ctx->own_stream = false;
    return GMI_OK;
}

gmi_status gmi_context_set_precision(gmi_context *ctx, int precision)
{
    GMI_ARG_CHECK(ctx != nullptr, "null context");
    GMI_ARG_CHECK(precision == GMI_FP64 || precision == GMI_FP32C || precision == GMI_DF64,
                  "precision must be GMI_FP64, GMI_FP32C or GMI_DF64");
    ctx->precision = precision;
    return GMI_OK;
}

int gmi_context_precision(const gmi_context *ctx) { return ctx ? ctx->precision : -1; }

gmi_status gmi_context_synchronize(gmi_context *ctx)
{
    GMI_ARG_CHECK(ctx != nullptr, "null context");
    GMI_CUDA_TRY(cudaSetDevice(ctx->device));
    return context_check_device_errors(ctx);
}

long long gmi_context_launch_count(const gmi_context *ctx) { return ctx ? ctx->launches : -1; }

gmi_status gmi_Mss_mult(gmi_context *ctx, double *V_d, const double *F_d, const double *X_d, int start_seg,
                        int num_segs, int total_segs, double rseg, double mu)
{
    GMI_ARG_CHECK(ctx != nullptr, "gmi_Mss_mult: null context");
    if (num_segs == 0) return GMI_OK;
    GMI_ARG_CHECK(ctx && V_d && F_d && X_d, "gmi_Mss_mult: null argument");
    GMI_ARG_CHECK(range_ok(start_seg, num_segs, total_segs), "gmi_Mss_mult: target range outside [0, total_segs)");
    GMI_ARG_CHECK(rseg > 0 && mu > 0, "gmi_Mss_mult: radius and viscosity must be positive");
    gmi_status st = select_device(ctx);
    if (st != GMI_OK) return st;
    st = pack_records(ctx, X_d, F_d, 6, total_segs, ctx->rec_src);
    if (st != GMI_OK) return st;
    PairConsts k;
    fill_consts(k, rseg, rseg, rseg, mu);
    return launch_pair(ctx, kSS, ctx->rec_src.ptr, start_seg, num_segs, ctx->rec_src.ptr, total_segs, k, V_d, 0);
}

gmi_status gmi_Mss_mult_wall(gmi_context *ctx, double *V_d, const double *F_d, const double *X_d, int start_seg,
                             int num_segs, int total_segs)
{
    GMI_ARG_CHECK(ctx != nullptr, "gmi_Mss_mult_wall: null context");
    if (num_segs == 0) return GMI_OK;
    GMI_ARG_CHECK(ctx && V_d && F_d && X_d, "gmi_Mss_mult_wall: null argument");
    GMI_ARG_CHECK(range_ok(start_seg, num_segs, total_segs),
                  "gmi_Mss_mult_wall: target range outside [0, total_segs)");
    gmi_status st = select_device(ctx);
    if (st != GMI_OK) return st;
    st = pack_records(ctx, X_d, F_d, 6, total_segs, ctx->rec_src);
    if (st != GMI_OK) return st;
    PairConsts k;
    fill_consts(k, 1.0, 1.0, 1.0, 1.0);
    return launch_pair(ctx, kSSWall, ctx->rec_src.ptr, start_seg, num_segs, ctx->rec_src.ptr, total_segs, k, V_d, 0);
}

gmi_status gmi_Mbb_mult(gmi_context *ctx, double *V_d, const double *F_d, const double *X_d, int start_blob,
                        int num_blobs, int total_blobs, double rblob, double mu)
{
    GMI_ARG_CHECK(ctx != nullptr, "gmi_Mbb_mult: null context");
    if (num_blobs == 0) return GMI_OK;
    GMI_ARG_CHECK(ctx && V_d && F_d && X_d, "gmi_Mbb_mult: null argument");
    GMI_ARG_CHECK(range_ok(start_blob, num_blobs, total_blobs), "gmi_Mbb_mult: target range outside [0, total_blobs)");
    GMI_ARG_CHECK(rblob > 0 && mu > 0, "gmi_Mbb_mult: radius and viscosity must be positive");
    gmi_status st = select_device(ctx);
    if (st != GMI_OK) return st;
    st = pack_records(ctx, X_d, F_d, 3, total_blobs, ctx->rec_src);
    if (st != GMI_OK) return st;
    PairConsts k;
    fill_consts(k, rblob, rblob, rblob, mu);
    return launch_pair(ctx, kBB, ctx->rec_src.ptr, start_blob, num_blobs, ctx->rec_src.ptr, total_blobs, k, V_d, 0);
}

gmi_status gmi_Msb_mult(gmi_context *ctx, double *V_d, const double *F_blobs_d, const double *Xs_d,
                        const double *Xb_d, int start_seg, int num_segs, int total_segs, int total_blobs,
                        double rseg, double rblob, double mu)
{
    GMI_ARG_CHECK(ctx != nullptr, "gmi_Msb_mult: null context");
    if (num_segs == 0) return GMI_OK;
    GMI_ARG_CHECK(ctx && V_d && Xs_d, "gmi_Msb_mult: null argument");
    GMI_ARG_CHECK(total_blobs == 0 || (F_blobs_d && Xb_d), "gmi_Msb_mult: null blob arrays");
    GMI_ARG_CHECK(range_ok(start_seg, num_segs, total_segs), "gmi_Msb_mult: target range outside [0, total_segs)");
    GMI_ARG_CHECK(total_blobs >= 0 && rseg > 0 && rblob > 0 && mu > 0, "gmi_Msb_mult: bad size or radius");
    gmi_status st = select_device(ctx);
    if (st != GMI_OK) return st;
    st = pack_records(ctx, Xs_d, nullptr, 0, total_segs, ctx->rec_tgt);
    if (st != GMI_OK) return st;
    st = pack_records(ctx, Xb_d, F_blobs_d, 3, total_blobs, ctx->rec_src);
    if (st != GMI_OK) return st;
    PairConsts k;
    fill_consts(k, rseg, rseg, rblob, mu);
    return launch_pair(ctx, kSB, ctx->rec_tgt.ptr, start_seg, num_segs, ctx->rec_src.ptr, total_blobs, k, V_d, 1);
}

gmi_status gmi_Mbs_mult(gmi_context *ctx, double *V_d, const double *F_segs_d, const double *Xb_d,
                        const double *Xs_d, int start_blob, int num_blobs, int total_blobs, int total_segs,
                        double rseg, double rblob, double mu)
{
    GMI_ARG_CHECK(ctx != nullptr, "gmi_Mbs_mult: null context");
    if (num_blobs == 0) return GMI_OK;
    GMI_ARG_CHECK(ctx && V_d && Xb_d, "gmi_Mbs_mult: null argument");
    GMI_ARG_CHECK(total_segs == 0 || (F_segs_d && Xs_d), "gmi_Mbs_mult: null segment arrays");
    GMI_ARG_CHECK(range_ok(start_blob, num_blobs, total_blobs), "gmi_Mbs_mult: target range outside [0, total_blobs)");
    GMI_ARG_CHECK(total_segs >= 0 && rseg > 0 && rblob > 0 && mu > 0, "gmi_Mbs_mult: bad size or radius");
    gmi_status st = select_device(ctx);
    if (st != GMI_OK) return st;
    st = pack_records(ctx, Xb_d, nullptr, 0, total_blobs, ctx->rec_tgt);
    if (st != GMI_OK) return st;
    st = pack_records(ctx, Xs_d, F_segs_d, 6, total_segs, ctx->rec_src);
    if (st != GMI_OK) return st;
    PairConsts k;
    fill_consts(k, rseg, rseg, rblob, mu);
    return launch_pair(ctx, kBS, ctx->rec_tgt.ptr, start_blob, num_blobs, ctx->rec_src.ptr, total_segs, k, V_d, 0);
}

gmi_status gmi_barrier_forces(gmi_context *ctx, double *f_segs_d, double *f_blobs_repulsion_d, const double *x_segs_d,
                              const double *x_blobs_d, int start_seg, int num_segs, int start_blob, int num_blobs,
                              int total_segs, int total_blobs, int nseg_per_filament, double rseg, double rblob,
                              double force_scale, int wall)
{
    GMI_ARG_CHECK(ctx != nullptr, "gmi_barrier_forces: null context");
    GMI_ARG_CHECK(total_segs == 0 || (f_segs_d && x_segs_d), "gmi_barrier_forces: null segment arrays");
    GMI_ARG_CHECK(total_blobs == 0 || x_blobs_d, "gmi_barrier_forces: null blob positions");
    GMI_ARG_CHECK(wall || num_blobs == 0 || f_blobs_repulsion_d, "gmi_barrier_forces: null blob repulsion output");
    GMI_ARG_CHECK(range_ok(start_seg, num_segs, total_segs) && range_ok(start_blob, num_blobs, total_blobs),
                  "gmi_barrier_forces: target range outside the particle sets");
    GMI_ARG_CHECK(nseg_per_filament > 0 && rseg > 0 && rblob > 0, "gmi_barrier_forces: bad segment count or radius");
    gmi_status st = select_device(ctx);
    if (st != GMI_OK) return st;
    BarrierLaunch a{};
    a.f_segs = f_segs_d;
    a.f_blobs_rep = f_blobs_repulsion_d;
    a.xs = x_segs_d;
    a.xb = x_blobs_d;
    a.S = total_segs;
    a.B = total_blobs;
    a.start_seg = start_seg;
    a.num_segs = num_segs;
    a.start_blob = start_blob;
    a.num_blobs = num_blobs;
    a.nseg = nseg_per_filament;
    a.rseg = rseg;
    a.rblob = rblob;
    a.scale = force_scale;
    a.wall = wall;
    return launch_barrier(ctx, a);
}

gmi_status gmi_tuned_shape(const gmi_context *ctx, int kind, int num_targets, int num_sources, int *threads_per_cta,
                           int *targets_per_thread, int *source_splits)
{
    GMI_ARG_CHECK(ctx && threads_per_cta && targets_per_thread && source_splits, "gmi_tuned_shape: null argument");
    PairShape s;
    auto it = ctx->tuned.find(TuneKey{kind, ctx->precision, num_targets, num_sources});
    const bool found = it != ctx->tuned.end();
    if (found) s = it->second;
    *threads_per_cta = s.tpb;
    *targets_per_thread = s.tt;
    *source_splits = s.splits;
    return found ? GMI_OK : GMI_ERR_STATE;
}

gmi_status gmi_tuned_sources_per_step(const gmi_context *ctx, int kind, int num_targets, int num_sources,
                                      int *sources_per_step)
{
    GMI_ARG_CHECK(ctx && sources_per_step, "gmi_tuned_sources_per_step: null argument");
    PairShape s;
    auto it = ctx->tuned.find(TuneKey{kind, ctx->precision, num_targets, num_sources});
    const bool found = it != ctx->tuned.end();
    if (found) s = it->second;
    *sources_per_step = pair_shape_is_packed(s, kind, ctx->precision == GMI_FP64) ? 2 : 1;
    return found ? GMI_OK : GMI_ERR_STATE;
}

gmi_status gmi_set_shape(gmi_context *ctx, int kind, int num_targets, int num_sources, int threads_per_cta,
                         int targets_per_thread, int source_splits, int sources_per_step)
{
    GMI_ARG_CHECK(ctx != nullptr, "gmi_set_shape: null context");
    GMI_ARG_CHECK(kind >= 0 && kind <= 4, "gmi_set_shape: kind must be 0..4");
    GMI_ARG_CHECK(source_splits >= 0, "gmi_set_shape: source_splits must be >= 0");
    GMI_ARG_CHECK(sources_per_step == 1 || sources_per_step == 2, "gmi_set_shape: sources_per_step must be 1 or 2");
    const bool f64 = ctx->precision == GMI_FP64;
    PairShape s{threads_per_cta, targets_per_thread, source_splits, sources_per_step == 2 ? 1 : 0};
    GMI_ARG_CHECK(pair_shape_exists(s, kind, f64), "gmi_set_shape: no kernel for this shape, kind and precision");
    ctx->tuned[TuneKey{kind, ctx->precision, num_targets, num_sources}] = s;
    return GMI_OK;
}

gmi_status gmi_autotune(gmi_context *ctx, int kind, int num_targets, int num_sources)
{
    GMI_ARG_CHECK(ctx != nullptr, "gmi_autotune: null context");
    GMI_ARG_CHECK(kind >= 0 && kind <= 4, "gmi_autotune: kind must be 0..4");
    GMI_ARG_CHECK(num_targets > 0 && num_sources > 0, "gmi_autotune: sizes must be positive");
    gmi_status st = select_device(ctx);
    if (st != GMI_OK) return st;
    // synthetic problem on a jittered lattice with unit-scale loads
    DeviceBuffer xt, xsrc, fsrc, out, rt, rs;
    const int nf = (kind == kBB || kind == kSB) ? 3 : 6;
    const int nout = (kind == kBB || kind == kBS) ? 3 : 6;
    st = xt.reserve((size_t)num_targets * 3 * sizeof(double));
    if (st == GMI_OK) st = xsrc.reserve((size_t)num_sources * 3 * sizeof(double));
    if (st == GMI_OK) st = fsrc.reserve((size_t)num_sources * nf * sizeof(double));
    if (st == GMI_OK) st = out.reserve((size_t)num_targets * nout * sizeof(double));
    if (st != GMI_OK) return st;
    {
        const size_t nbytes_max = (size_t)(num_targets > num_sources ? num_targets : num_sources) * 6;
        double *h = nullptr;
        GMI_CUDA_TRY(gmi::host_alloc(&h, nbytes_max * sizeof(double)));
        auto fill_pos = [&](int n, double *dst) -> gmi_status {
            const int side = (int)std::ceil(std::cbrt((double)n));
            for (int i = 0; i < n; ++i) {
                const int a = i % side, b = (i / side) % side, c = i / (side * side);
                h[3 * i] = 2.5 * a + 0.1 * std::sin(1.0 + i);
                h[3 * i + 1] = 2.5 * b + 0.1 * std::sin(2.0 + i);
                h[3 * i + 2] = 2.5 * c + 1.5 + 0.1 * std::sin(3.0 + i);
            }
            GMI_CUDA_TRY(cudaMemcpyAsync(dst, h, (size_t)n * 3 * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
            GMI_CUDA_TRY(cudaStreamSynchronize(ctx->stream));  // h is refilled next
            return GMI_OK;
        };
        st = fill_pos(num_targets, static_cast<double *>(xt.ptr));
        if (st == GMI_OK) st = fill_pos(num_sources, static_cast<double *>(xsrc.ptr));
        if (st == GMI_OK) {
            for (size_t i = 0; i < (size_t)num_sources * nf; ++i) h[i] = std::cos(0.7 * (double)i);
            cudaError_t e = cudaMemcpyAsync(fsrc.ptr, h, (size_t)num_sources * nf * sizeof(double),
                                            cudaMemcpyHostToDevice, ctx->stream);
            if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);  // before h is freed
            if (e != cudaSuccess) st = GMI_ERR_CUDA;
        }
        gmi::host_free(h);
        if (st != GMI_OK) return st;
    }
    st = pack_records(ctx, static_cast<double *>(xt.ptr), nullptr, 0, num_targets, rt);
    if (st == GMI_OK)
        st = pack_records(ctx, static_cast<double *>(xsrc.ptr), static_cast<double *>(fsrc.ptr), nf, num_sources, rs);
    if (st != GMI_OK) return st;
    PairConsts k;
    fill_consts(k, 1.0, 1.0, 1.0, 1.0);
    st = autotune_pair(ctx, kind, rt.ptr, num_targets, rs.ptr, num_sources, k, static_cast<double *>(out.ptr));
    cudaStreamSynchronize(ctx->stream);
    xt.release();
    xsrc.release();
    fsrc.release();
    out.release();
    rt.release();
    rs.release();
    return st;
}

}  // extern "C"
