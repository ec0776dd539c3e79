// gmi_gmres.hpp -- a device-resident GMRES for any operator given as host
// callbacks that enqueue kernels: the reference's solve_linear_system
// (mobility_solver.cpp:970-1354) for systems other than the free-swimmer
// saddle point (which has its own graph-replayed Arnoldi step).
#pragma once

#include <functional>

#include "gmi_context.hpp"

namespace gmi {

// Device workspace of one GMRES size: n unknowns, at most m iterations.
struct KrylovSpace {
    int n = 0, m = 0;
    double *Q = nullptr, *H = nullptr, *beta = nullptr, *cs = nullptr, *sn = nullptr, *yv = nullptr;
    double *w = nullptr, *z = nullptr, *tmp = nullptr, *partial = nullptr, *scal = nullptr;
    double *h_scal = nullptr;  // pinned
};

gmi_status krylov_alloc(KrylovSpace &K, int n, int m, cudaStream_t stream);
void krylov_free(KrylovSpace &K);

// out = Op(in), enqueued on the context stream
using DeviceApply = std::function<gmi_status(const double *in, double *out)>;

// Right-preconditioned GMRES with classical Gram-Schmidt and one
// re-orthogonalisation, Givens rotations and back substitution in FP64.
// soln holds the warm start on entry (rejected, as the reference does, when
// its residual exceeds ||rhs||) and the solution on return; stops when the
// residual falls to tol * ||rhs||.  One host read per iteration.
gmi_status krylov_gmres(gmi_context *ctx, KrylovSpace &K, const DeviceApply &precond, const DeviceApply &matvec,
                        const double *rhs, double *soln, double tol, int *iters);

}  // namespace gmi
