// vec.h -- launchers of the device vector layer (vec.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstddef>

namespace doci {

// Partial-sum buffer of the reductions below (doubles): a block counter, the
// results, one row per block.  Every reduction pass finishes its own sum (in
// a fixed order) into the results; initialise a new buffer's counter once
// with vec_partials_init.
int vec_partials_capacity();
int vec_partials_init(double *partials, cudaStream_t st);
// the results of the last reduction pass on `partials` (device pointer)
const double *vec_results(const double *partials);
// the default number of blocks of a reduction pass (the largest is twice it)
int vec_reduction_blocks();
// out[k] = result k of the last pass, k < nk (device to device copy)
int vec_reduce(const double *partials, int nk, double *out, cudaStream_t st);

template <typename S>
int vec_multidot(const S *V, size_t ld, int m, const S *w, size_t n, double *partials, cudaStream_t st,
                 bool fp64_products = false,  // FP32 storage: true = exact products, FP64 sums
                 bool mixed = false);         // FP64 storage: column 0 in FP64, the rest in FP32 arithmetic
template <typename S>
int vec_residual(const S *V, const S *VA, size_t ld, int m, const double *y, double theta, const double *diag,
                 size_t n, S *t, double *x, double *partials, cudaStream_t st, double diag_shift = 0.0,
                 bool mixed = false);
// index of the smallest element (first on ties), synchronous
int vec_argmin(const double *d, size_t n, int64_t *idx, cudaStream_t st);
// bytes from src to dst by a kernel (both device-accessible: device memory or
// pinned host memory mapped into the device's address space)
int vec_copy(void *dst, const void *src, size_t bytes, cudaStream_t st);
// y += a x (FP64)
int vec_axpy(double a, const double *x, double *y, size_t n, cudaStream_t st);
// out[j] = (float)(d[j] - shift): the FP32 diagonal of the shifted operator H - shift
int vec_shifted_diag32(const double *d, double shift, float *out, size_t n, cudaStream_t st);
template <typename S>
int vec_gs_update(const S *V, size_t ld, int m, const double *c, size_t n, S *t, double *partials, cudaStream_t st,
                  bool mixed = false);
template <typename S>
int vec_gs_finish(const S *V, size_t ld, int m, const double *c, double scale, size_t n, const S *t, S *out,
                  double *partials, cudaStream_t st, bool mixed = false);
template <typename S>
int vec_deflate(S *V, size_t ld, int mv, int keep, const double *Y, int ldy, size_t n, cudaStream_t st);
template <typename S>
int vec_combine(const S *V, size_t ld, int m, const double *y, size_t n, double *x, cudaStream_t st);
template <typename A, typename B>
int vec_convert(const A *a, B *b, size_t n, cudaStream_t st);

int cg_gram(const double *x, const double *p, const double *Ax, const double *Ap, size_t n, double *partials,
            cudaStream_t st);
int cg_update(double a, double b, int first, double rho, double *x, const double *p, double *Ax, const double *Ap,
              double *g, const double *pinv, size_t n, double *partials, cudaStream_t st);
int cg_direction(double beta, int first, double *p, const double *g, size_t n, cudaStream_t st);
int precond_inverse(const double *diag, double *pinv, size_t n, cudaStream_t st);

// host-side dense symmetric eigensolver (cyclic Jacobi), ascending order;
// A column-major n x n (leading dimension lda, upper triangle read),
// eigenvectors to V (same leading dimension)
void jacobi_eig(int n, const double *A, int lda, double *w, double *V);
// lowest eigenpair of A v = lambda B v for 2x2 symmetric A, B (upper
// triangles, column-major), B-normalised as LAPACK's dsygv returns it
int gen_eig_2x2(const double *A, const double *B, double *lambda, double *v);

}  // namespace doci
