// gmi_gmres_cluster.hpp -- the FP32C free-swimmer GMRES solve inside one
// thread-block cluster (gmi_gmres_cluster.cu).
#pragma once

#include "gmi_context.hpp"

struct gmi_solver;

namespace gmi {

// True when the solver's context is FP32C and the system is small enough for
// one cluster (at most 2048 blobs, 16 swimmers); GMI_GMRES_CLUSTER=0 turns
// the path off.
bool cluster_gmres_usable(gmi_solver *s);

// Enqueues the whole Arnoldi loop (Q[:, 0] = w / beta0 onward) on the solver
// stream: on return from the stream, ctl holds the iteration count and
// residual, and H, beta, cs, sn and Q the same quantities as after the
// multi-kernel steps.
gmi_status cluster_gmres_launch(gmi_solver *s, double beta0, double norm_ref, double tol, int max_iter);

}  // namespace gmi
