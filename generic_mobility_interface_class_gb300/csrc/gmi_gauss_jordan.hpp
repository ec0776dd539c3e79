// gmi_gauss_jordan.hpp -- Gauss-Jordan inversion of the filament Jacobians
// (gmi_gauss_jordan.cu): one CTA per matrix, or one thread-block cluster per
// matrix when there are few of them.
#pragma once

#include "gmi_context.hpp"

namespace gmi {

// CTAs per matrix (a power of two <= 8) that keep nmat matrices within the
// GPU's SMs; 1 means the one-CTA kernel is the better choice.
int gj_cluster_size(int nmat, int n, int sm_count);

// In-place inverse of nmat column-major n x n FP64 matrices on `stream`,
// csize CTAs per matrix (1: one CTA each); registers = false steps the
// columns through shared memory even where they fit in registers (the same
// arithmetic).  A zero pivot sets flags[2].
gmi_status gj_invert(cudaStream_t stream, double *mats, int nmat, int n, int csize, bool registers, int device,
                     int *flags);
// The same in FP32 (the mixed-precision time step's approximate inverse).
gmi_status gj_invert(cudaStream_t stream, float *mats, int nmat, int n, int csize, bool registers, int device,
                     int *flags);

}  // namespace gmi
