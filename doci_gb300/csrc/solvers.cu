// solvers.cu -- device-resident Davidson (davidson.c:33-128) and Rayleigh-
// quotient CG (CG.c:13-164).
//
// The iteration structure, stopping rules, preconditioner quirks (|D-theta|
// with a 1e-12 cutoff; 1/diag for CGP), deflation and return codes are the
// reference's.  The basis, residual and search vectors live in HBM; only the
// subspace matrix (<= 32 x 32) and a handful of reduction results cross to
// the host each iteration.  The matvec is either the device sigma of a
// doci_ham or, for a foreign matvec function, a call on host buffers.
#include <cuda_runtime.h>

#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "internal.h"
#include "solvers.h"
#include "vec.h"

namespace doci {

namespace {

// Stream-ordered device buffer (cudaMallocAsync / cudaFreeAsync): freeing
// does not synchronise the device, so concurrent solves on other streams keep
// running.
struct DevMem {
  void *p = nullptr;
  cudaStream_t st = nullptr;
  DevMem() = default;
  DevMem(const DevMem &) = delete;
  DevMem &operator=(const DevMem &) = delete;
  ~DevMem() {
    if (p) cudaFreeAsync(p, st);
  }
  int alloc(size_t bytes, cudaStream_t s) {
    if (p) cudaFreeAsync(p, st);
    p = nullptr;
    st = s;
    if (bytes == 0) bytes = 16;
    DOCI_CUDA(cudaMallocAsync(&p, bytes, s));
    return DOCI_OK;
  }
  template <typename T>
  T *as() const {
    return static_cast<T *>(p);
  }
};

#define DOCI_TRY(expr)          \
  do {                          \
    int _s = (expr);            \
    if (_s != DOCI_OK) return _s; \
  } while (0)

}  // namespace

double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

int ShiftedView::make(const doci_ham *h, cudaStream_t s) {
  st = s;
  view = *h;
  int64_t idx = 0;
  DOCI_TRY(vec_argmin(h->d_diag, h->D, &idx, s));
  DOCI_CUDA(cudaMemcpyAsync(&shift, h->d_diag + idx, sizeof(double), cudaMemcpyDeviceToHost, s));
  DOCI_CUDA(cudaStreamSynchronize(s));
  DOCI_CUDA(cudaMallocAsync(&d_diag32, sizeof(float) * h->D, s));
  DOCI_TRY(vec_shifted_diag32(h->d_diag, shift, d_diag32, h->D, s));
  view.d_diag32 = d_diag32;
  return DOCI_OK;
}

ShiftedView::~ShiftedView() {
  if (d_diag32) cudaFreeAsync(d_diag32, st);
}

int MatvecOp::apply(const void *d_x, void *d_y, int precision, cudaStream_t st) {
  if (ham) {
    if (events_on) cudaEventRecord(ev0, st);
    int s;
    if (ham32 && precision == DOCI_FP64 && !anchor_next) {
      const double *x = static_cast<const double *>(d_x);
      s = vec_convert<double, float>(x, x32, n, st);
      if (s == DOCI_OK) s = launch_sigma(ham32, x32, y32, DOCI_FP32, st);
      if (s == DOCI_OK) s = vec_convert<float, double>(y32, static_cast<double *>(d_y), n, st);
    } else {
      s = launch_sigma(ham, d_x, d_y, precision, st);
      if (s == DOCI_OK && ham32 && precision == DOCI_FP64)
        s = vec_axpy(-shift32, static_cast<const double *>(d_x), static_cast<double *>(d_y), n, st);
    }
    anchor_next = false;
    if (events_on) {
      cudaEventRecord(ev1, st);
      cudaEventSynchronize(ev1);
      float ms = 0;
      cudaEventElapsedTime(&ms, ev0, ev1);
      sigma_seconds += ms * 1e-3;
    }
    return s;
  }
  if (precision != DOCI_FP64 || !host_fn) return DOCI_ERR_INVALID;
  hx.resize(n);
  hy.resize(n);
  DOCI_CUDA(cudaMemcpyAsync(hx.data(), d_x, n * sizeof(double), cudaMemcpyDeviceToHost, st));
  DOCI_CUDA(cudaStreamSynchronize(st));
  host_fn(hx.data(), hy.data(), host_dat);
  DOCI_CUDA(cudaMemcpyAsync(d_y, hy.data(), n * sizeof(double), cudaMemcpyHostToDevice, st));
  DOCI_CUDA(cudaStreamSynchronize(st));
  return DOCI_OK;
}

void MatvecOp::enable_timing() {
  if (!events_on && ham) {
    cudaEventCreate(&ev0);
    cudaEventCreate(&ev1);
    events_on = true;
  }
}

MatvecOp::~MatvecOp() {
  if (events_on) {
    cudaEventDestroy(ev0);
    cudaEventDestroy(ev1);
  }
}

// Davidson on storage type S (double: FP64 mode; float: FP32 phase of the
// mixed mode).  d_t holds the start vector (it is the search-vector buffer).
template <typename S>
int davidson_run(MatvecOp &op, size_t D, const double *d_diag, S *d_t, const DavidsonArgs &a, cudaStream_t st,
                 DavidsonOut *out, double *d_x_out) {
  const int maxv = a.max_vectors, keep = a.keep;
  if (maxv < 2 || maxv > 32 || keep < 1 || keep >= maxv) return DOCI_ERR_INVALID;
  const int precision = sizeof(S) == 8 ? DOCI_FP64 : DOCI_FP32;
  DevMem V, VA, part, small;
  DOCI_TRY(V.alloc(sizeof(S) * D * maxv, st));
  DOCI_TRY(VA.alloc(sizeof(S) * D * maxv, st));
  DOCI_TRY(part.alloc(sizeof(double) * vec_partials_capacity(), st));
  DOCI_TRY(vec_partials_init(part.as<double>(), st));
  // small device scratch: [0,64) reduction output, [64,96) y/c, [96, 96+32*32) Y
  DOCI_TRY(small.alloc(sizeof(double) * (96 + 32 * 32), st));
  double *d_red = small.as<double>(), *d_vec = d_red + 64, *d_Y = d_red + 96;
  S *Vp = V.as<S>(), *VAp = VA.as<S>();
  double *dp = part.as<double>();
  std::vector<double> Sm(maxv * maxv, 0.0), Y(maxv * maxv, 0.0), w(maxv, 0.0), red(64), c(32, 0.0);

  auto fetch = [&](int nk) -> int {
    DOCI_CUDA(cudaMemcpyAsync(red.data(), vec_results(dp), sizeof(double) * nk, cudaMemcpyDeviceToHost, st));
    DOCI_CUDA(cudaStreamSynchronize(st));
    return DOCI_OK;
  };

  int its = 0, m = 0;
  double res = a.tol * 10, energy = 0, d_energy = a.tol * 10;
  const double t0 = now_s();
  if (a.print_table) std::printf("IT\tINFO\tRESIDUE\tENERGY\n");
  int stall = 0;
  double best = 1e300;
  double t_norm2 = 0, proj2 = 0;  // ||t||^2 and ||V^T t||^2 from the residual pass
  // Mixed sigma precisions (FP64 phase with FP32 correction sigmas): werr[i]
  // weighs the rounding error of VA_i (0 for the FP64 anchor).  The entry
  // S[i][j] = v_i . H v_j is taken from the more accurate side, VA_i . v_j
  // or v_i . VA_j: the anchor's cross terms then carry no FP32 error, which
  // would otherwise enter the Ritz vector at full size.
  const bool mixed_sigmas = op.ham32 != nullptr && sizeof(S) == 8;
  std::vector<double> werr(maxv, 0.0);
  auto column = [&](int j) -> int {
    DOCI_TRY(vec_multidot<S>(Vp, D, j + 1, VAp + static_cast<size_t>(j) * D, D, dp, st, false, mixed_sigmas));
    DOCI_TRY(fetch(j + 1));
    for (int i = 0; i <= j; ++i) Sm[j * maxv + i] = red[i];
    bool other = false;
    for (int i = 0; i < j; ++i) other = other || werr[i] < werr[j];
    if (!other) return DOCI_OK;
    std::vector<double> a(red.begin(), red.begin() + j + 1);
    DOCI_TRY(vec_multidot<S>(VAp, D, j + 1, Vp + static_cast<size_t>(j) * D, D, dp, st, false, mixed_sigmas));
    DOCI_TRY(fetch(j + 1));
    for (int i = 0; i < j; ++i) Sm[j * maxv + i] = werr[i] < werr[j] ? red[i] : a[i];
    return DOCI_OK;
  };
  while (res > a.tol && its++ < a.max_its) {
    // ---- new search vector: orthogonalise t against V, normalise (davidson.c:133-176)
    S *Vm = Vp + static_cast<size_t>(m) * D;
    if (m == 0) {
      DOCI_TRY(vec_multidot<S>(d_t, D, 1, d_t, D, dp, st));
      DOCI_TRY(fetch(1));
      DOCI_TRY(vec_gs_finish<S>(Vp, D, 0, nullptr, 1.0 / std::sqrt(red[0]), D, d_t, Vm, dp, st));
    } else if ((sizeof(S) == 4 || mixed_sigmas) && t_norm2 - proj2 > 0.5 * t_norm2) {
      // FP32 basis: t keeps more than half of its norm after one projection,
      // so one classical Gram-Schmidt pass is enough (the Daniel-Gragg-
      // Kaufman-Stewart criterion); the residual pass already gave V^T t
      DOCI_CUDA(cudaMemcpyAsync(d_vec, c.data(), sizeof(double) * m, cudaMemcpyHostToDevice, st));
      DOCI_TRY(vec_gs_finish<S>(Vp, D, m, d_vec, 1.0 / std::sqrt(t_norm2 - proj2), D, d_t, Vm, dp, st, mixed_sigmas));
    } else {
      DOCI_CUDA(cudaMemcpyAsync(d_vec, c.data(), sizeof(double) * m, cudaMemcpyHostToDevice, st));
      DOCI_TRY(vec_gs_update<S>(Vp, D, m, d_vec, D, d_t, dp, st, mixed_sigmas));
      DOCI_TRY(fetch(m + 1));
      double n2 = red[0];
      for (int i = 0; i < m; ++i) {
        c[i] = red[1 + i];
        n2 -= c[i] * c[i];
      }
      if (!(n2 > 0)) n2 = red[0] > 0 ? red[0] : 1.0;
      DOCI_CUDA(cudaMemcpyAsync(d_vec, c.data(), sizeof(double) * m, cudaMemcpyHostToDevice, st));
      DOCI_TRY(vec_gs_finish<S>(Vp, D, m, d_vec, 1.0 / std::sqrt(n2), D, d_t, Vm, dp, st, mixed_sigmas));
    }
    // ---- the one matvec of the iteration (davidson.c:76)
    DOCI_TRY(op.apply(Vm, VAp + static_cast<size_t>(m) * D, precision, st));
    // ---- subspace column S[m][i] = V_i . VA_m (davidson.c:178-193)
    werr[m] = mixed_sigmas && m > 0 ? 1.0 : 0.0;  // only the run's first sigma is FP64 (the anchor)
    DOCI_TRY(column(m));
    ++m;
    jacobi_eig(m, Sm.data(), maxv, w.data(), Y.data());
    if (m == maxv) {  // ---- deflation (davidson.c:83-89, :229-255)
      DOCI_CUDA(cudaMemcpyAsync(d_Y, Y.data(), sizeof(double) * maxv * keep, cudaMemcpyHostToDevice, st));
      DOCI_TRY(vec_deflate<S>(Vp, D, maxv, keep, d_Y, maxv, D, st));
      DOCI_TRY(vec_deflate<S>(VAp, D, maxv, keep, d_Y, maxv, D, st));
      if (mixed_sigmas) {  // error weight of a kept vector: sum_k |Y[k][c]| werr[k]
        std::vector<double> wn(keep, 0.0);
        for (int cc = 0; cc < keep; ++cc)
          for (int k = 0; k < maxv; ++k) wn[cc] += std::fabs(Y[cc * maxv + k]) * werr[k];
        for (int cc = 0; cc < keep; ++cc) werr[cc] = wn[cc];
      }
      for (int cc = 0; cc < keep; ++cc) DOCI_TRY(column(cc));
      m = keep;
      jacobi_eig(m, Sm.data(), maxv, w.data(), Y.data());
    }
    // ---- residual, preconditioner, first GS projections (davidson.c:90, :98)
    const double theta = w[0];
    DOCI_CUDA(cudaMemcpyAsync(d_vec, Y.data(), sizeof(double) * m, cudaMemcpyHostToDevice, st));
    DOCI_TRY(vec_residual<S>(Vp, VAp, D, m, d_vec, theta, d_diag, D, d_t, nullptr, dp, st, a.shift, mixed_sigmas));
    DOCI_TRY(fetch(m + 2));
    res = std::sqrt(red[0]);
    t_norm2 = red[1];
    proj2 = 0;
    for (int i = 0; i < m; ++i) {
      c[i] = red[2 + i];
      proj2 += c[i] * c[i];
    }
    d_energy = energy - theta;
    energy = theta;
    if (a.print_table) std::printf("%d\t%d\t%e\t%f\n", its, 0, res, theta + a.shift);
    if (a.trace && a.trace_count && *a.trace_count < a.trace_len) {
      double *r = a.trace + 4 * (*a.trace_count)++;
      r[0] = a.trace_phase;
      r[1] = res;
      r[2] = theta + a.shift;
      r[3] = now_s() - a.trace_t0;
    }
    // mixed mode (FP32 phase, and the FP64 phase with FP32 corrections): stop
    // once the residual has not reached a new minimum for stall_window
    // iterations (the FP32 noise floor; restarted Davidson residuals are not
    // monotone, so a short window would stop early)
    if (a.stall_window > 0) {
      if (res < best) {
        best = res;
        stall = 0;
      } else if (++stall >= a.stall_window) {
        break;
      }
    }
  }
  const double t1 = now_s();
  if (a.print_table) {
    if (its <= a.max_its)
      std::printf("Davidson converged in %d iterations with %e residue and d_energy %e.\n", its, res, d_energy);
    else
      std::printf("Davidson didn't converge within %d iterations! d_energy is %e.\n", a.max_its, d_energy);
    std::printf("elapsed time : %lf sec\n", t1 - t0);
    std::printf("average time per matvec : %lf sec\n", (t1 - t0) / (its > 0 ? its : 1));
  } else if (a.print_summary) {
    std::printf("\t\t ** DAVIDSON ITERATIONS : %d\n", its);
  }
  std::fflush(stdout);
  // the eigenvector x = V y of the last Ritz pair
  if (d_x_out) {
    DOCI_CUDA(cudaMemcpyAsync(d_vec, Y.data(), sizeof(double) * m, cudaMemcpyHostToDevice, st));
    DOCI_TRY(vec_combine<S>(Vp, D, m, d_vec, D, d_x_out, st));
  }
  DOCI_CUDA(cudaStreamSynchronize(st));
  out->energy = w[0] + a.shift;
  out->residual = res;
  out->iterations = its;
  out->converged = res <= a.tol;
  out->return_code = its >= a.max_its;
  out->seconds = t1 - t0;
  return DOCI_OK;
}

template int davidson_run<double>(MatvecOp &, size_t, const double *, double *, const DavidsonArgs &, cudaStream_t,
                                  DavidsonOut *, double *);
template int davidson_run<float>(MatvecOp &, size_t, const double *, float *, const DavidsonArgs &, cudaStream_t,
                                 DavidsonOut *, double *);


// RQ-CG (CG.c:13-164).  d_x holds the start vector and receives the result.
int ray_q_run(MatvecOp &op, size_t D, const double *d_diag_or_null, double *d_x, const CgArgs &a, cudaStream_t st,
              CgOut *out) {
  DevMem buf, part, small;
  DOCI_TRY(buf.alloc(sizeof(double) * D * 5, st));
  DOCI_TRY(part.alloc(sizeof(double) * vec_partials_capacity(), st));
  DOCI_TRY(vec_partials_init(part.as<double>(), st));
  DOCI_TRY(small.alloc(sizeof(double) * 64, st));
  double *p = buf.as<double>(), *Ax = p + D, *Ap = Ax + D, *g = Ap + D, *pinv = g + D;
  double *dp = part.as<double>(), *d_red = small.as<double>();
  double red[8];
  auto fetch = [&](int nk) -> int {
    DOCI_CUDA(cudaMemcpyAsync(red, vec_results(dp), sizeof(double) * nk, cudaMemcpyDeviceToHost, st));
    DOCI_CUDA(cudaStreamSynchronize(st));
    return DOCI_OK;
  };
  const double *use_pinv = nullptr;
  if (d_diag_or_null) {
    DOCI_TRY(precond_inverse(d_diag_or_null, pinv, D, st));
    use_pinv = pinv;
  }
  const double t0 = now_s();
  if (a.print) std::printf("\nIT\tINFO\tRESIDUE\tENERGY\n");
  int its = 0;
  DOCI_TRY(op.apply(d_x, Ax, DOCI_FP64, st));
  // rho = Ax . x, g = 2 (Ax - rho x)  (CG.c:75-86)
  DOCI_CUDA(cudaMemsetAsync(p, 0, sizeof(double) * D, st));
  DOCI_CUDA(cudaMemsetAsync(Ap, 0, sizeof(double) * D, st));
  DOCI_TRY(cg_gram(d_x, p, Ax, Ap, D, dp, st));
  DOCI_TRY(fetch(7));
  double rho = red[0], d_energy = 0;
  DOCI_TRY(cg_update(1.0, 0.0, 1, rho, d_x, p, Ax, Ap, g, use_pinv, D, dp, st));
  DOCI_TRY(fetch(2));
  double normq = red[0], ng = red[1], ng_prev = red[1];
  if (a.print) std::printf("%d\t%d\t%e\t%f\n", its, 0, ng, rho);
  int info = 0;
  while (normq > a.tol && its < a.max_its) {
    DOCI_TRY(cg_direction(its != 0 ? ng / ng_prev : 0.0, its == 0, p, g, D, st));
    DOCI_TRY(op.apply(p, Ap, DOCI_FP64, st));
    DOCI_TRY(cg_gram(d_x, p, Ax, Ap, D, dp, st));
    DOCI_TRY(fetch(7));
    const double A[4] = {red[0], red[1], red[2], red[3]};
    const double B[4] = {red[4], red[5], red[5], red[6]};
    double lam, v[2];
    info = gen_eig_2x2(A, B, &lam, v);
    if (info) break;
    d_energy = rho - lam;
    rho = lam;
    DOCI_TRY(cg_update(v[0], v[1], 0, rho, d_x, p, Ax, Ap, g, use_pinv, D, dp, st));
    DOCI_TRY(fetch(2));
    normq = red[0];
    ng_prev = ng;
    ng = red[1];
    if (a.print) std::printf("%d\t%d\t%e\t%f\n", its, info, ng, rho);
    if (a.trace && its < a.trace_len) {
      a.trace[2 * its] = ng;
      a.trace[2 * its + 1] = rho;
    }
    its++;
  }
  const double t1 = now_s();
  if (a.print) {
    if (its <= a.max_its)
      std::printf("CG converged in %d iterations with %e residue and d_energy %e.\n", its, ng, d_energy);
    else
      std::printf("CG didn't converge within %d iterations! d_energy is %e.\n", a.max_its, d_energy);
    std::printf("elapsed time : %lf sec\n", t1 - t0);
    std::printf("average time per matvec : %lf sec\n", (t1 - t0) / (its + 1));
    std::fflush(stdout);
  }
  out->energy = rho;
  out->normq = normq;
  out->normq_g = ng;
  out->iterations = its;
  out->converged = !(normq > a.tol);
  out->return_code = its <= a.max_its;
  out->seconds = t1 - t0;
  return DOCI_OK;
}

// ---------------------------------------------------------------------------
// Dense helpers
// ---------------------------------------------------------------------------
void jacobi_eig(int n, const double *A, int lda, double *w, double *Vout) {
  std::vector<double> a(n * n), v(n * n);
  for (int c = 0; c < n; ++c)
    for (int r = 0; r < n; ++r) {
      a[r + c * n] = r <= c ? A[r + c * lda] : A[c + r * lda];
      v[r + c * n] = r == c ? 1.0 : 0.0;
    }
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0, tot = 0;
    for (int c = 0; c < n; ++c)
      for (int r = 0; r < n; ++r) {
        const double e = a[r + c * n] * a[r + c * n];
        tot += e;
        if (r != c) off += e;
      }
    if (off == 0 || off <= 1e-30 * tot) break;
    for (int p = 0; p < n - 1; ++p)
      for (int q = p + 1; q < n; ++q) {
        const double apq = a[p + q * n];
        if (apq == 0) continue;
        const double theta = (a[q + q * n] - a[p + p * n]) / (2 * apq);
        const double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1));
        const double cs = 1 / std::sqrt(t * t + 1), sn = t * cs;
        for (int k = 0; k < n; ++k) {
          const double akp = a[k + p * n], akq = a[k + q * n];
          a[k + p * n] = cs * akp - sn * akq;
          a[k + q * n] = sn * akp + cs * akq;
        }
        for (int k = 0; k < n; ++k) {
          const double apk = a[p + k * n], aqk = a[q + k * n];
          a[p + k * n] = cs * apk - sn * aqk;
          a[q + k * n] = sn * apk + cs * aqk;
        }
        for (int k = 0; k < n; ++k) {
          const double vkp = v[k + p * n], vkq = v[k + q * n];
          v[k + p * n] = cs * vkp - sn * vkq;
          v[k + q * n] = sn * vkp + cs * vkq;
        }
      }
  }
  std::vector<int> idx(n);
  for (int i = 0; i < n; ++i) idx[i] = i;
  for (int i = 0; i < n; ++i)
    for (int j = i + 1; j < n; ++j)
      if (a[idx[j] * (n + 1)] < a[idx[i] * (n + 1)]) std::swap(idx[i], idx[j]);
  for (int i = 0; i < n; ++i) {
    w[i] = a[idx[i] * (n + 1)];
    for (int r = 0; r < n; ++r) Vout[r + i * lda] = v[r + idx[i] * n];
  }
}

int gen_eig_2x2(const double *A, const double *B, double *lam, double *vec) {
  /* dsygv_ (ITYPE=1, UPLO='U'): B = U^T U, C = U^-T A U^-1, dsyev_(C), v = U^-1 z.
   * For n = 2 dsyev_ reduces to LAPACK's dlaev2 (published netlib algorithm)
   * applied to (c11, c12, c22) inside dsteqr, which stores the eigenvector
   * (cs1, sn1) of the larger-magnitude eigenvalue rt1 in column 1 and
   * (-sn1, cs1) in column 2, then sorts ascending.  The sign of that
   * eigenvector matters: CG.c:106-113 updates x but keeps p, so a flipped
   * x changes the next search direction (CG.c:92-94). */
  const double b11 = B[0], b12 = B[2], b22 = B[3];
  if (!(b11 > 0)) return 1;
  const double u11 = std::sqrt(b11), u12 = b12 / u11, s = b22 - u12 * u12;
  if (!(s > 0)) return 2;
  const double u22 = std::sqrt(s);
  const double i11 = 1 / u11, i12 = -u12 / (u11 * u22), i22 = 1 / u22;
  const double a11 = A[0], a12 = A[2], a22 = A[3];
  const double c11 = i11 * i11 * a11;
  const double c12 = i11 * (a11 * i12 + a12 * i22);
  const double c22 = i12 * i12 * a11 + 2 * i12 * i22 * a12 + i22 * i22 * a22;
  /* dlaev2(c11, c12, c22) */
  const double sm = c11 + c22, df = c11 - c22, adf = std::fabs(df), tb = c12 + c12, ab = std::fabs(tb);
  const double acmx = std::fabs(c11) > std::fabs(c22) ? c11 : c22, acmn = std::fabs(c11) > std::fabs(c22) ? c22 : c11;
  double rt, rt1, rt2, cs, cs1, sn1;
  int sgn1, sgn2;
  if (adf > ab) rt = adf * std::sqrt(1 + (ab / adf) * (ab / adf));
  else if (adf < ab) rt = ab * std::sqrt(1 + (adf / ab) * (adf / ab));
  else rt = ab * std::sqrt(2.0);
  if (sm < 0) { rt1 = 0.5 * (sm - rt); sgn1 = -1; rt2 = (acmx / rt1) * acmn - (c12 / rt1) * c12; }
  else if (sm > 0) { rt1 = 0.5 * (sm + rt); sgn1 = 1; rt2 = (acmx / rt1) * acmn - (c12 / rt1) * c12; }
  else { rt1 = 0.5 * rt; rt2 = -0.5 * rt; sgn1 = 1; }
  if (df >= 0) { cs = df + rt; sgn2 = 1; } else { cs = df - rt; sgn2 = -1; }
  if (std::fabs(cs) > ab) { const double ct = -tb / cs; sn1 = 1 / std::sqrt(1 + ct * ct); cs1 = ct * sn1; }
  else if (ab == 0) { cs1 = 1; sn1 = 0; }
  else { const double tn = -cs / tb; cs1 = 1 / std::sqrt(1 + tn * tn); sn1 = tn * cs1; }
  if (sgn1 == sgn2) { const double tn = cs1; cs1 = -sn1; sn1 = tn; }
  /* dsteqr: column 1 = (cs1, sn1) for rt1, column 2 = (-sn1, cs1) for rt2;
   * ascending selection sort swaps them when rt2 < rt1 */
  double z0, z1, l0;
  if (rt2 < rt1) { l0 = rt2; z0 = -sn1; z1 = cs1; } else { l0 = rt1; z0 = cs1; z1 = sn1; }
  *lam = l0;
  vec[0] = i11 * z0 + i12 * z1;
  vec[1] = i22 * z1;
  return 0;
}

}  // namespace doci
