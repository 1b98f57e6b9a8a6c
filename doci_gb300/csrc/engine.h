// engine.h -- the batch engine (engine.cu): block Davidson for many
// Hamiltonians at once, device-resident, one graph-captured iteration for
// the whole batch.
#pragma once

#include <cuda_runtime.h>

#include "internal.h"

namespace doci {

// Device bytes the engine holds for one problem of shape (L, N) with opts o
// (vectors of both phases, Ritz vectors, the handle's diagonals and tables).
int64_t engine_footprint(int L, int N, const doci_batch_opts &o);

// Solve the o.nroots lowest eigenpairs of hams[0..n) on stream st (a created
// stream: the iteration is captured as a CUDA graph).  res[i] receives the
// energies, residuals and counts of problem i; vecs[i] (host, D x nroots,
// may be null, as may vecs) its Ritz vectors.  A problem's result does not
// depend on the other problems of the batch.
int engine_solve(int n, doci_ham *const *hams, const doci_batch_opts &o, cudaStream_t st, doci_root_result *res,
                 double *const *vecs);

// Time the engine's sigma tile shapes (1, 2 or 4 determinants per thread)
// on this handle with nv vectors and keep the fastest for every problem of
// the same (device, L, N) in the process; *dpt receives it.
int engine_tune(doci_ham *h, int nv, int *dpt);

}  // namespace doci
