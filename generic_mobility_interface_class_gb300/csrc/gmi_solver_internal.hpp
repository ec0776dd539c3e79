// gmi_solver_internal.hpp -- the mobility solver object, shared by the
// C-ABI solver entry points (gmi_solver.cu) and the implicit time step
// (gmi_sim.cu), which drives the solver on device-resident state.
#pragma once

#include <vector>

#include "gmi_context.hpp"

struct PrescribedWork;  // workspace of the prescribed-shape cilia solve (gmi_prescribed.cu)

struct gmi_solver {
    gmi_context *ctx = nullptr;
    gmi_solver_config cfg{};
    int S = 0, B = 0, W = 0, n = 0, m = 0;
    gmi_host_arrays h{};
    double *h_stage = nullptr;   // pinned staging: body x, q, f, scalars
    // device state
    double *x_segs = nullptr, *f_segs = nullptr, *v_segs = nullptr;
    double *x_blobs = nullptr, *f_blobs = nullptr, *v_blobs = nullptr, *f_rep = nullptr;
    double *body_x = nullptr, *body_q = nullptr, *body_f = nullptr, *v_bodies = nullptr;
    double *R = nullptr, *ktk_ref = nullptr, *mob_ref = nullptr, *ktk_rot = nullptr, *mob_rot = nullptr;
    double *ktkf_ref = nullptr, *ktkf_rot = nullptr;  // K^T K itself (not inverted), reference and rotated
    double *refs = nullptr, *sums = nullptr, *kt_part = nullptr;  // K^T sums and their per-CTA partials
    double *rhs = nullptr, *soln = nullptr, *Q = nullptr, *H = nullptr, *beta = nullptr, *cs = nullptr, *sn = nullptr;
    double *z = nullptr, *w = nullptr, *tmp = nullptr, *mbb = nullptr, *partial = nullptr, *yv = nullptr;
    double *b64 = nullptr, *xacc = nullptr;  // refinement: FP64 right-hand side, accumulated solution
    double *scal = nullptr;  // device scalars: [0] norm, [1] resid
    bool refs_set = false;
    // the last linear solve: its relative residual (GMRES's estimate |beta|/||b||
    // in FP64; the FP64-grade refinement residual in FP32C) and whether it met
    // the tolerance; strict makes compute_velocities report a solve that did not
    double last_rel_resid = 0.0;
    int last_iters = 0;
    bool strict = false;
    double gm_resid = 0.0;  // relative residual estimate at the end of the last gmres_run
    std::vector<void *> allocs;
    // device-controlled Arnoldi iterations replayed from a CUDA graph
    struct GmresCtl *ctl = nullptr;   // device control block
    struct GmresCtl *h_ctl = nullptr; // pinned mirror
    bool ctl_pending = false;          // a GMRES solve's control block is on its way to h_ctl, unchecked
    long long ctl_pending_nodes = 0;   // launches per pass of that solve's device loop (0: cluster kernel)
    void *gm_rec = nullptr;           // blob records of the GMRES operator (own buffer: fixed address)
    size_t partial_count = 0;         // doubles in partial
    double *st_scal = nullptr;        // Arnoldi step scalars: projections h, ||w||
    int *st_tickets = nullptr;        // Arnoldi step arrival tickets (zero between launches)
    int *aux_tickets = nullptr;       // the same for norm_kernel [0] and kt_kernel [1]
    size_t st_ticket_count = 0;
    double *gm_partial = nullptr;     // split partial sums of the GMRES operator
    size_t gm_partial_bytes = 0;
    cudaGraphExec_t graph[2] = {nullptr, nullptr};  // per precision: the Arnoldi loop (or one step)
    size_t graph_nodes[2] = {0, 0};
    bool graph_loops[2] = {false, false};           // graph holds the whole device-side loop
    bool use_graphs = true;
    bool use_cluster = true;  // FP32C solves of small systems in one thread-block cluster
    bool use_pdl = true;      // Arnoldi-step kernels launched for programmatic dependent launch (GMI_PDL=0: off;
                              // also off if a graph with programmatic edges fails to capture or instantiate)
    double *Qr = nullptr;     // the cluster solve's row-major copy of Q (allocated by its first launch)
    // the cluster solve's launch shape, chosen once (it depends only on the
    // sizes): 0 not chosen yet, 1 chosen (cluster_* below), -1 unusable
    int cluster_state = 0;
    int cluster_csize = 0, cluster_bpc = 0, cluster_kq = 0, cluster_kqs = 0;
    size_t cluster_smem = 0;
    PrescribedWork *prescribed = nullptr;  // allocated by the first prescribed-cilia solve
    // generalised forces of the prescribed beat over one period, for solves
    // with the phase speeds as unknowns; serial counts the setter's calls
    std::vector<double> gen_force_refs;
    unsigned gen_force_serial = 0;
};


// Iteration state of a GMRES solve that the device advances by itself.
struct GmresCtl {
    int k;         // current Arnoldi iteration (1-based)
    int done;      // set by the Givens step when converged or at max_iter
    int max_iter;
    int replays;   // Arnoldi steps completed by the norm kernel in this solve
    int guard;     // passes of the device-side loop (counted by its guard kernel)
    int pass2;     // set by S3: 1 = this step runs the second Gram-Schmidt pass (S4), 0 = skipped
    double tol;    // relative residual target
    double norm_ref;
    double resid;  // |beta(k)| / norm_ref after the last Givens step
    double inv_norm_ref;  // 1 / norm_ref (the Givens step multiplies: no division on its serial path)
};
static_assert(sizeof(GmresCtl) <= 64, "GmresCtl lives in an 8-double device block");

namespace gmi {

// mobility_solver::compute_velocities on inputs already on the device
// (x_segs, f_segs, body_x, body_q, body_f): blob positions, barrier forces
// (their blob part added into body_f), M_ss, M_bs, the right-hand side, the
// linear solve, M_sb.  Leaves v_segs, f_blobs, v_bodies on the device.
gmi_status solver_compute_velocities_device(gmi_solver *s, int *iters);

// Body state from the host (x[3W], q[4W]), rotation matrices and blob
// positions on the device.
gmi_status solver_place_blobs(gmi_solver *s, const double *body_x, const double *body_q);

// eta^2 of the conditional re-orthogonalisation of the device Arnoldi steps
// (GMI_REORTH_ETA; 0: the second Gram-Schmidt pass always runs).
double reorth_eta2(bool fp64);

// Frees the prescribed-cilia workspace (gmi_solver_destroy).
void prescribed_release(gmi_solver *s);

// make_body_reference_matrices on the device-resident x_segs/f_segs and
// body state; the outputs (may be null) are column-major 6x6.
gmi_status solver_make_body_reference_matrices_device(gmi_solver *s, double *ktkinv_out, double *mob_out);

}  // namespace gmi
