// gmi_gj_cluster.hpp -- Gauss-Jordan inversion of small matrices spread over
// thread-block clusters (gmi_gj_cluster.cu).
#pragma once

#include "gmi_context.hpp"

namespace gmi {

// CTAs per matrix (a power of two <= 8) that keep nmat matrices within the
// GPU's SMs; 1 means the one-CTA kernel is the better choice.
int gj_cluster_size(int nmat, int n, int sm_count);

// In-place inverse of nmat column-major n x n matrices, csize CTAs each; a
// zero pivot sets flags[2].
gmi_status gj_invert_cluster(cudaStream_t stream, double *mats, int nmat, int n, int csize, int *flags);

}  // namespace gmi
