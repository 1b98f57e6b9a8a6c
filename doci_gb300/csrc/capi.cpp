// capi.cpp -- the C ABI of libdoci_gb300.so (include/doci_gb300.h).
#include <cuda_runtime.h>

#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <new>
#include <set>
#include <string>

#include "internal.h"
#include "solvers.h"
#include "vec.h"

namespace doci {
const char *last_cuda_error();
int vec_argmin(const double *d, size_t n, int64_t *idx, cudaStream_t st);
int vec_fill_random(double *t, size_t n, uint64_t seed, cudaStream_t st);
int vec_set_unit(double *t, size_t n, int64_t idx, cudaStream_t st);
}  // namespace doci

using namespace doci;

namespace {

std::mutex g_reg_mu;
std::set<const void *> g_live;  // handles created by this library

void reg_add(const void *h) {
  std::lock_guard<std::mutex> g(g_reg_mu);
  g_live.insert(h);
}
void reg_del(const void *h) {
  std::lock_guard<std::mutex> g(g_reg_mu);
  g_live.erase(h);
}
bool reg_has(const void *h) {
  std::lock_guard<std::mutex> g(g_reg_mu);
  return g_live.count(h) != 0;
}

// Streams are used as given, as everywhere in CUDA: NULL is the default
// stream, so work queued by the caller on it is ordered before ours.
cudaStream_t pick(doci_ham *, void *stream) { return static_cast<cudaStream_t>(stream); }

// stream-ordered device buffer (freeing does not synchronise the device)
struct DevBuf {
  void *p = nullptr;
  cudaStream_t st = nullptr;
  ~DevBuf() {
    if (p) cudaFreeAsync(p, st);
  }
};

// fatal-error convention of the reference's entry points
[[noreturn]] void die_cuda(const char *where, int st) {
  std::fprintf(stderr, "%s: %s (%s)\n", where, doci_status_string(st), last_cuda_error());
  std::printf("Exiting...\n");
  std::exit(EXIT_FAILURE);
}

int build_from_integrals(const Integrals &in, doci_ham **out) {
  doci_ham *h = new (std::nothrow) doci_ham();
  if (!h) return DOCI_ERR_OUT_OF_MEMORY;
  const int st = ham_build(h, in);
  if (st != DOCI_OK) {
    ham_release(h);
    delete h;
    return st;
  }
  reg_add(h);
  *out = h;
  return DOCI_OK;
}

// Start vector of executable.c:270-299 on the device: HF_INIT=1 puts 1 at the
// lowest diagonal element (first index on ties); HF_INIT=0 draws positive
// uniform numbers (the reference seeds rand() with time(NULL); here the seed
// is explicit so runs repeat).
int make_start(doci_ham *h, int hf_init, uint64_t seed, double *d_t, cudaStream_t st) {
  if (hf_init) {
    int64_t idx = 0;
    int s = vec_argmin(h->d_diag, h->D, &idx, st);
    if (s) return s;
    return vec_set_unit(d_t, h->D, idx, st);
  }
  return vec_fill_random(d_t, h->D, seed, st);
}

// Device address of a pinned (page-locked, mapped) host buffer, or null for
// pageable memory.
const void *mapped_host(const void *p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();  // pageable memory on older drivers reports an error
    return nullptr;
  }
  return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

// One FP64 sigma y = H x (through op, as an anchor), theta = x.y / x.x and
// the residual norm ||y - theta x|| / ||x||.  dp: partial-sum scratch of
// vec_partials_capacity() + 64 doubles; r: D doubles of scratch.
int fp64_check(MatvecOp &op, const double *d_x, size_t D, double *d_y, double *d_r, double *dp, cudaStream_t st,
               double *theta, double *rnorm) {
  op.anchor_next = true;
  int s = op.apply(d_x, d_y, DOCI_FP64, st);
  if (s) return s;
  double *d_red = dp + vec_partials_capacity();
  double h_red[3];
  if ((s = vec_multidot<double>(d_x, D, 1, d_y, D, dp, st))) return s;
  if ((s = vec_reduce(dp, 1, d_red, st))) return s;
  if ((s = vec_multidot<double>(d_x, D, 1, d_x, D, dp, st))) return s;
  if ((s = vec_reduce(dp, 1, d_red + 1, st))) return s;
  DOCI_CUDA(cudaMemcpyAsync(h_red, d_red, 2 * sizeof(double), cudaMemcpyDeviceToHost, st));
  DOCI_CUDA(cudaStreamSynchronize(st));
  const double xx = h_red[1] > 0 ? h_red[1] : 1.0;
  *theta = h_red[0] / xx;
  // r = y - theta x with the residual pass (coefficient 1 on x and y)
  const double one = 1.0;
  DOCI_CUDA(cudaMemcpyAsync(d_red + 8, &one, sizeof(double), cudaMemcpyHostToDevice, st));
  if ((s = vec_residual<double>(d_x, d_y, D, 1, d_red + 8, *theta, op.ham->d_diag, D, d_r, nullptr, dp, st,
                                op.ham32 ? op.shift32 : 0.0)))
    return s;
  if ((s = vec_reduce(dp, 3, d_red + 16, st))) return s;
  DOCI_CUDA(cudaMemcpyAsync(h_red, d_red + 16, sizeof(double), cudaMemcpyDeviceToHost, st));
  DOCI_CUDA(cudaStreamSynchronize(st));
  *rnorm = std::sqrt(h_red[0] / xx);
  return DOCI_OK;
}

}  // namespace

// ===========================================================================
// Part 2: status API
// ===========================================================================
extern "C" {

const char *doci_status_string(int s) {
  switch (s) {
    case DOCI_OK: return "ok";
    case DOCI_ERR_OPEN: return "cannot open FCIDUMP file";
    case DOCI_ERR_FORMAT: return "FCIDUMP file is wrongly formatted";
    case DOCI_ERR_NALPHA_NBETA: return "number of up and down electrons not equal (obligatory for DOCI)";
    case DOCI_ERR_TOO_MANY_ORBITALS: return "too many orbitals (L > 32)";
    case DOCI_ERR_INVALID: return "invalid argument";
    case DOCI_ERR_CUDA: return "CUDA error";
    case DOCI_ERR_OUT_OF_MEMORY: return "out of memory";
    case DOCI_ERR_NO_DEVICE: return "no CUDA device";
    case DOCI_ERR_ADMISSION: return "request exceeds the HBM budget";
    case DOCI_ERR_NOT_FOUND: return "unknown ticket";
    case DOCI_ERR_PENDING: return "not finished";
    case DOCI_ERR_DEVICE_TIMEOUT: return "device wait timed out";
    case DOCI_ERR_UNKNOWN_SOLVER: return "unknown solver";
    case DOCI_ERR_SCRATCH_LIMIT: return "request exceeds the fixed scratch of the allocation-free entry point";
    default: return "unknown status";
  }
}

int doci_ham_from_fcidump(const char *path, doci_ham **out) {
  if (!path || !out) return DOCI_ERR_INVALID;
  *out = nullptr;
  Integrals in;
  int bad = 0;
  const int st = read_fcidump_file(path, &in, &bad);
  if (st) return st;
  return build_from_integrals(in, out);
}

int doci_ham_from_fcidump_relaxed(const char *path, doci_ham **out) {
  if (!path || !out) return DOCI_ERR_INVALID;
  *out = nullptr;
  Integrals in;
  int bad = 0;
  const int st = read_fcidump_relaxed(path, &in, &bad);
  if (st) return st;
  return build_from_integrals(in, out);
}

int doci_fcidump_integrals(const char *path, int relaxed, int *L, int *n_alpha, int *n_beta, double *core,
                           double *one, double *two, int *bad_line) {
  if (!path) return DOCI_ERR_INVALID;
  Integrals in;
  int bad = 0;
  const int st = relaxed ? read_fcidump_relaxed(path, &in, &bad) : read_fcidump_file(path, &in, &bad);
  if (bad_line) *bad_line = bad;
  if (st) return st;
  if (L) *L = in.L;
  if (n_alpha) *n_alpha = in.Na;
  if (n_beta) *n_beta = in.Nb;
  if (core) *core = in.core;
  if (one) std::memcpy(one, in.one.data(), in.one.size() * sizeof(double));
  if (two) std::memcpy(two, in.two.data(), in.two.size() * sizeof(double));
  return DOCI_OK;
}

int doci_ham_from_integrals(int L, int n_pairs, double core, const double *one, const double *two,
                            doci_ham **out) {
  if (!out || !one || !two || L < 1 || n_pairs < 0) return DOCI_ERR_INVALID;
  *out = nullptr;
  if (L > kMaxOrbitals) return DOCI_ERR_TOO_MANY_ORBITALS;
  Integrals in;
  in.L = L;
  in.Na = in.Nb = n_pairs;
  in.core = core;
  const size_t n2 = static_cast<size_t>(L) * L;
  in.one.assign(one, one + n2);
  in.two.assign(two, two + n2 * n2);
  return build_from_integrals(in, out);
}

void doci_ham_destroy(doci_ham *h) {
  if (!h || !reg_has(h)) return;
  reg_del(h);
  cudaStreamSynchronize(h->stream);
  ham_release(h);
  delete h;
}

int doci_ham_dims(const doci_ham *h, int *L, int *n_pairs, int64_t *dim) {
  if (!h) return DOCI_ERR_INVALID;
  if (L) *L = h->L;
  if (n_pairs) *n_pairs = h->N;
  if (dim) *dim = h->D;
  return DOCI_OK;
}

int doci_ham_diagonal(const doci_ham *h, double *out) {
  if (!h || !out) return DOCI_ERR_INVALID;
  DOCI_CUDA(cudaMemcpy(out, h->d_diag, sizeof(double) * h->D, cudaMemcpyDeviceToHost));
  return DOCI_OK;
}

const double *doci_ham_diagonal_device(const doci_ham *h) { return h ? h->d_diag : nullptr; }

int doci_sigma(doci_ham *h, const void *d_x, void *d_y, int precision, void *stream) {
  if (!h || !d_x || !d_y || d_x == d_y) return DOCI_ERR_INVALID;
  return launch_sigma(h, d_x, d_y, precision, pick(h, stream));
}

int doci_sigma_block(doci_ham *h, const void *d_X, int64_t ldx, void *d_Y, int64_t ldy, int nv, int precision,
                     void *stream) {
  if (!h || !d_X || !d_Y || nv < 1 || ldx < h->D || ldy < h->D) return DOCI_ERR_INVALID;
  if (precision != DOCI_FP64 && precision != DOCI_FP32) return DOCI_ERR_INVALID;
  const size_t es = precision == DOCI_FP64 ? 8 : 4;
  const char *x = static_cast<const char *>(d_X);
  char *y = static_cast<char *>(d_Y);
  // the output block must not overlap the input block
  const char *xe = x + ((nv - 1) * static_cast<size_t>(ldx) + h->D) * es;
  const char *ye = y + ((nv - 1) * static_cast<size_t>(ldy) + h->D) * es;
  if (x < ye && y < xe) return DOCI_ERR_INVALID;
  const cudaStream_t st = pick(h, stream);
  for (int v0 = 0; v0 < nv; v0 += 4) {
    const int k = nv - v0 < 4 ? nv - v0 : 4;
    const int r = launch_sigma_multi(h, x + v0 * static_cast<size_t>(ldx) * es, ldx,
                                     y + v0 * static_cast<size_t>(ldy) * es, ldy, k, precision, st);
    if (r != DOCI_OK) return r;
  }
  return DOCI_OK;
}

int doci_sigma_plan(const doci_ham *h, int precision, int *kind, int *launches) {
  if (!h || (precision != DOCI_FP64 && precision != DOCI_FP32)) return DOCI_ERR_INVALID;
  const SigmaPlan p = plan_sigma(h, precision);
  if (kind) *kind = p.kind;
  if (launches) *launches = p.launches;
  return DOCI_OK;
}

int doci_ham_autotune(doci_ham *h, int precision, int nvec, int *choice) {
  if (!h || nvec < 1 || nvec > 4) return DOCI_ERR_INVALID;
  return autotune_sigma(h, precision, nvec, h->stream, choice);
}

int doci_ham_set_sigma_kernel(doci_ham *h, int kind) {
  if (!h || !(kind == 0 || kind == 1 || kind == 3 || kind == 4 || kind == 6 || kind == 8 || kind == 9))
    return DOCI_ERR_INVALID;
  h->sigma_kernel = kind;
  return DOCI_OK;
}

int doci_sigma_host(doci_ham *h, const void *x, void *y, int precision) {
  if (!h || !x || !y || x == y) return DOCI_ERR_INVALID;
  if (precision != DOCI_FP64 && precision != DOCI_FP32) return DOCI_ERR_INVALID;
  const size_t bytes = static_cast<size_t>(h->D) * (precision == DOCI_FP64 ? 8 : 4);
  int st = ham_stage(h, bytes);
  if (st) return st;
  // pinned host buffers are read and written by copy kernels through their
  // device mapping or by the copy engines (both at the host link's rate);
  // pageable ones go through cudaMemcpyAsync
  // (the copy kernels move 4-byte words: a pinned buffer that is not 4-byte
  // aligned takes the cudaMemcpyAsync path too)
  const bool words = (reinterpret_cast<uintptr_t>(x) | reinterpret_cast<uintptr_t>(y)) % 4 == 0;
  const void *dx = words ? mapped_host(x) : nullptr;
  void *dy = words ? const_cast<void *>(mapped_host(y)) : nullptr;
  const int kind = plan_sigma(h, precision).kind;
  const bool sched = h->d_pblocks_host && !h->host_steps.empty();
  if (sched && ((precision == DOCI_FP32 && kind == 6 && pair_fits(h)) ||
                (precision == DOCI_FP64 && kind == 9 && pair_ff_fits(h)))) {
    // the pair forms overlap the copies with the sigma: pieces of x go up and
    // pieces of y come down on the copy engines while the unit groups run (a
    // pageable y is copied after the sigma: a copy into pageable memory can
    // hold the calling thread until it is done)
    const bool y_pinned = mapped_host(y) != nullptr;
    if (precision == DOCI_FP32)
      st = launch_pair_host(h, static_cast<const float *>(x), static_cast<float *>(h->d_stage_x),
                            static_cast<float *>(h->d_stage_y), y_pinned ? static_cast<float *>(y) : nullptr,
                            h->stream);
    else
      st = launch_pair_ff_host(h, static_cast<const double *>(x), static_cast<double *>(h->d_stage_x),
                               static_cast<double *>(h->d_stage_y), y_pinned ? static_cast<double *>(y) : nullptr,
                               h->stream);
    if (st) return st;
    if (y_pinned) {
      DOCI_CUDA(cudaStreamSynchronize(h->stream));
      return ham_device_error(h, h->stream);
    }
  } else {
    if (dx) {
      if ((st = vec_copy(h->d_stage_x, dx, bytes, h->stream))) return st;
    } else {
      DOCI_CUDA(cudaMemcpyAsync(h->d_stage_x, x, bytes, cudaMemcpyHostToDevice, h->stream));
    }
    st = launch_sigma(h, h->d_stage_x, h->d_stage_y, precision, h->stream);
    if (st) return st;
  }
  if (dy) {
    if ((st = vec_copy(dy, h->d_stage_y, bytes, h->stream))) return st;
  } else {
    DOCI_CUDA(cudaMemcpyAsync(y, h->d_stage_y, bytes, cudaMemcpyDeviceToHost, h->stream));
  }
  DOCI_CUDA(cudaStreamSynchronize(h->stream));
  return ham_device_error(h, h->stream);
}

int doci_bitstrings(doci_ham *h, int64_t first, int64_t count, uint32_t *d_bits, void *stream) {
  if (!h || (!d_bits && count > 0)) return DOCI_ERR_INVALID;
  return launch_bitstrings(h, first, count, d_bits, pick(h, stream));
}

int doci_ranks(doci_ham *h, const uint32_t *d_bits, int64_t count, int64_t *d_ranks, void *stream) {
  if (!h || ((!d_bits || !d_ranks) && count > 0)) return DOCI_ERR_INVALID;
  return launch_ranks(h, d_bits, count, d_ranks, pick(h, stream));
}

int doci_multidot(const void *d_V, int64_t ld, int m, const void *d_w, int64_t n, int precision, double *d_out,
                  void *stream) {
  if (!d_V || !d_w || !d_out || m < 1 || m > 32 || n < 0 || ld < n) return DOCI_ERR_INVALID;
  if (precision != DOCI_FP64 && precision != DOCI_FP32) return DOCI_ERR_INVALID;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  double *partials = nullptr;
  DOCI_CUDA(cudaMallocAsync(&partials, sizeof(double) * vec_partials_capacity(), st));
  int s = vec_partials_init(partials, st);
  if (s == DOCI_OK)
    s = precision == DOCI_FP64
              ? vec_multidot<double>(static_cast<const double *>(d_V), static_cast<size_t>(ld), m,
                                     static_cast<const double *>(d_w), static_cast<size_t>(n), partials, st)
              : vec_multidot<float>(static_cast<const float *>(d_V), static_cast<size_t>(ld), m,
                                    static_cast<const float *>(d_w), static_cast<size_t>(n), partials, st, true);
  if (s == DOCI_OK) s = vec_reduce(partials, m, d_out, st);
  const cudaError_t e = cudaFreeAsync(partials, st);  // on every path after the allocation
  if (s != DOCI_OK) return s;
  DOCI_CUDA(e);
  return DOCI_OK;
}

void doci_solve_opts_default(doci_solve_opts *o) {
  if (!o) return;
  std::memset(o, 0, sizeof *o);
  o->solver = DOCI_SOLVER_D;
  o->max_its = 200;         // options.h:7
  o->tol = 1e-8;            // options.h:6
  o->davidson_keep = 2;     // options.h:5
  o->davidson_max_vec = 30; // options.h:4
  o->hf_init = 1;
  o->mode = DOCI_MODE_FP64;
  o->mixed_tol = 1e-5;
  o->fp32_corrections = 1;
  o->print_level = 0;
  o->seed = 1;
}

int64_t doci_solve_footprint(int L, int n_pairs, const doci_solve_opts *o, int nroots) {
  if (L < 1 || L > 32 || n_pairs < 0 || n_pairs > L) return -1;
  doci_solve_opts d;
  if (!o) {
    doci_solve_opts_default(&d);
    o = &d;
  }
  (void)nroots;
  const int64_t D = static_cast<int64_t>(binom64(L, n_pairs));
  const int64_t mv = o->davidson_max_vec;
  const int64_t ham = D * 12;  // FP64 + FP32 diagonal
  int64_t solver;
  if (o->solver != DOCI_SOLVER_D) {
    solver = D * 8 * 7;  // x, p, Ax, Ap, g, pinv + start
  } else if (o->mode == DOCI_MODE_MIXED) {
    // FP32 phase: basis, start, x, shifted FP32 diagonal; FP64 phase: basis,
    // start, x, and with FP32 corrections the shifted diagonal, two FP32 and
    // two FP64 scratch vectors
    const int64_t p32 = D * (2 * mv * 4 + 4 + 8 + 4);
    const int64_t p64 = D * (2 * mv * 8 + 8 + 8 + (o->fp32_corrections ? 4 + 8 + 16 : 0));
    solver = p32 > p64 ? p32 : p64;
  } else {
    solver = D * (2 * mv * 8 + 8 + 8);
  }
  return ham + solver + (1 << 20);
}

int doci_solve(doci_ham *h, const doci_solve_opts *opts, double *vec, doci_solve_result *res) {
  return doci_solve_trace(h, opts, vec, res, nullptr, 0, nullptr);
}

int doci_solve_trace(doci_ham *h, const doci_solve_opts *opts, double *vec, doci_solve_result *res, double *trace,
                     int trace_len, int *trace_count) {
  if (!h || !res) return DOCI_ERR_INVALID;
  int count_local = 0;
  if (!trace_count) trace_count = &count_local;
  *trace_count = 0;
  const double trace_t0 = now_s();
  doci_solve_opts o;
  if (opts) o = *opts; else doci_solve_opts_default(&o);
  std::memset(res, 0, sizeof *res);
  const size_t D = h->D;
  cudaStream_t st = h->stream;
  DevBuf x;
  x.st = st;
  DOCI_CUDA(cudaMallocAsync(&x.p, sizeof(double) * D, st));
  double *d_x = static_cast<double *>(x.p);
  int s;
  if (o.hf_init < 0) {
    if (!vec) return DOCI_ERR_INVALID;
    DOCI_CUDA(cudaMemcpyAsync(d_x, vec, sizeof(double) * D, cudaMemcpyHostToDevice, st));
  } else if ((s = make_start(h, o.hf_init, o.seed, d_x, st))) {
    return s;
  }
  MatvecOp op;
  op.ham = h;
  op.n = D;
  op.enable_timing();
  const auto t0 = std::chrono::steady_clock::now();
  if (o.solver == DOCI_SOLVER_D) {
    DavidsonArgs a;
    a.max_vectors = o.davidson_max_vec;
    a.keep = o.davidson_keep;
    a.max_its = o.max_its;
    a.tol = o.tol;
    a.print_table = o.print_level >= 2;
    a.print_summary = o.print_level == 1;
    a.trace = trace;
    a.trace_len = trace_len;
    a.trace_t0 = trace_t0;
    a.trace_count = trace_count;
    a.trace_phase = 1;
    DavidsonOut out;
    int its_left = o.max_its;
    if (o.mode == DOCI_MODE_MIXED) {
      DevBuf t32;
      t32.st = st;
  DOCI_CUDA(cudaMallocAsync(&t32.p, sizeof(float) * D, st));
      if ((s = vec_convert<double, float>(d_x, static_cast<float *>(t32.p), D, st))) return s;
      DavidsonArgs a32 = a;
      a32.tol = o.mixed_tol > o.tol ? o.mixed_tol : o.tol;
      a32.stall_window = 15;
      a32.print_summary = 0;
      a32.trace_phase = 0;
      // the FP32 phase runs on H - (lowest diagonal element)
      ShiftedView sv;
      if ((s = sv.make(h, st))) return s;
      a32.shift = sv.shift;
      MatvecOp op32;
      op32.ham = &sv.view;
      op32.n = D;
      op32.enable_timing();
      s = davidson_run<float>(op32, D, h->d_diag, static_cast<float *>(t32.p), a32, st, &out, d_x);
      op.sigma_seconds += op32.sigma_seconds;
      if (s) return s;
      res->iterations_fp32 = out.iterations;
      res->energy_fp32 = out.energy;
      its_left -= out.iterations;
      if (its_left < 1) its_left = 1;
    }
    a.max_its = its_left;
    DevBuf t;
    t.st = st;
    DOCI_CUDA(cudaMallocAsync(&t.p, sizeof(double) * D, st));
    DOCI_CUDA(cudaMemcpyAsync(t.p, d_x, sizeof(double) * D, cudaMemcpyDeviceToDevice, st));
    // mixed mode: the FP64 phase computes the correction vectors' sigmas in
    // FP32 on the shifted view (each run's first sigma, the anchor, and a
    // closing verification sigma are FP64); plain FP64 mode: FP64 throughout
    const bool corr32 = o.mode == DOCI_MODE_MIXED && o.fp32_corrections;
    ShiftedView sv64;
    DevBuf x32, y32, scratch;
    x32.st = y32.st = scratch.st = st;
    if (corr32) {
      if ((s = sv64.make(h, st))) return s;
      DOCI_CUDA(cudaMallocAsync(&x32.p, sizeof(float) * D, st));
      DOCI_CUDA(cudaMallocAsync(&y32.p, sizeof(float) * D, st));
      DOCI_CUDA(cudaMallocAsync(&scratch.p, sizeof(double) * (2 * D + vec_partials_capacity() + 64), st));
      if ((s = vec_partials_init(static_cast<double *>(scratch.p) + 2 * D, st))) return s;
      op.ham32 = &sv64.view;
      op.shift32 = sv64.shift;
      op.x32 = static_cast<float *>(x32.p);
      op.y32 = static_cast<float *>(y32.p);
      a.shift = sv64.shift;  // the FP64 phase works on H - shift as well
      // the FP32 corrections leave a noise floor in the run's residual: a run
      // whose residual has not reached a new minimum for 25 iterations stops,
      // and the next round re-anchors it from its vector with an FP64 sigma
      a.stall_window = 25;
    }
    int its64 = 0;
    for (int round = 0;; ++round) {
      op.anchor_next = true;
      if ((s = davidson_run<double>(op, D, h->d_diag, static_cast<double *>(t.p), a, st, &out, d_x))) return s;
      its64 += out.iterations;
      if (!corr32) break;
      // verification: one FP64 sigma of the result, its Rayleigh quotient and
      // true residual (what the result reports)
      double theta = 0, rnorm = 0;
      double *d_y = static_cast<double *>(scratch.p), *d_r = d_y + D, *dp = d_r + D;
      if ((s = fp64_check(op, d_x, D, d_y, d_r, dp, st, &theta, &rnorm))) return s;
      theta += sv64.shift;  // op's operator is H - shift
      ++its64;
      out.energy = theta;
      out.residual = rnorm;
      out.converged = rnorm <= o.tol;
      if (trace && trace_count && *trace_count < trace_len) {
        double *r = trace + 4 * (*trace_count)++;
        r[0] = 1;
        r[1] = rnorm;
        r[2] = theta;
        r[3] = now_s() - trace_t0;
      }
      if (out.converged || round >= 3 || res->iterations_fp32 + its64 >= o.max_its) break;
      a.max_its = o.max_its - res->iterations_fp32 - its64;
      DOCI_CUDA(cudaMemcpyAsync(t.p, d_x, sizeof(double) * D, cudaMemcpyDeviceToDevice, st));
    }
    res->energy = out.energy;
    res->residual = out.residual;
    res->iterations = its64 + res->iterations_fp32;
    res->converged = out.converged;
    res->status_code = out.return_code;
  } else if (o.solver == DOCI_SOLVER_CG || o.solver == DOCI_SOLVER_CGP) {
    CgArgs a;
    a.max_its = o.max_its;
    a.tol = o.tol;
    a.print = o.print_level >= 1;
    CgOut out;
    if ((s = ray_q_run(op, D, o.solver == DOCI_SOLVER_CGP ? h->d_diag : nullptr, d_x, a, st, &out))) return s;
    res->energy = out.energy;
    res->residual = out.normq;
    res->iterations = out.iterations;
    res->converged = out.converged;
    res->status_code = out.return_code;
  } else {
    return DOCI_ERR_UNKNOWN_SOLVER;
  }
  res->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  res->sigma_seconds = op.sigma_seconds;
  if (vec) DOCI_CUDA(cudaMemcpyAsync(vec, d_x, sizeof(double) * D, cudaMemcpyDeviceToHost, st));
  DOCI_CUDA(cudaStreamSynchronize(st));
  return ham_device_error(h, st);
}

// ===========================================================================
// Part 1: reference-compatible drop-in
// ===========================================================================

void read_fcidump(char *filename, unsigned int *NORB, unsigned int *NALPHA, unsigned int *NBETA,
                  double *core_energy, double **one_p_int, double **two_p_int) {
  Integrals in;
  int bad = 0;
  const int st = read_fcidump_file(filename, &in, &bad);
  if (st == DOCI_ERR_OPEN) {
    std::fprintf(stderr, "Error reading fcidump file\n");
    std::exit(EXIT_FAILURE);
  }
  if (st == DOCI_ERR_FORMAT && bad <= 1) {
    std::fprintf(stderr, "Error in reading %s. File is wrongly formatted.\n", filename);
    std::exit(EXIT_FAILURE);
  }
  if (st != DOCI_OK) {
    std::fprintf(stderr, "Whilst reading the integrals, an error occured, wrong formatting at line %d!\n", bad);
    std::exit(EXIT_FAILURE);
  }
  const size_t n2 = static_cast<size_t>(in.L) * in.L;
  *NORB = static_cast<unsigned>(in.L);
  *NALPHA = static_cast<unsigned>(in.Na);
  *NBETA = static_cast<unsigned>(in.Nb);
  *core_energy = in.core;
  *one_p_int = static_cast<double *>(std::malloc(sizeof(double) * n2));
  *two_p_int = static_cast<double *>(std::malloc(sizeof(double) * n2 * n2));
  if (!*one_p_int || !*two_p_int) {
    std::fprintf(stderr, "read_fcidump: out of memory\n");
    std::exit(EXIT_FAILURE);
  }
  std::memcpy(*one_p_int, in.one.data(), sizeof(double) * n2);
  std::memcpy(*two_p_int, in.two.data(), sizeof(double) * n2 * n2);
}

void fill_doci_data(char *dumpfil, void **dat) {
  Integrals in;
  int bad = 0;
  int st = read_fcidump_file(dumpfil, &in, &bad);
  if (st == DOCI_ERR_OPEN) {
    std::fprintf(stderr, "Error reading fcidump file\n");
    std::exit(EXIT_FAILURE);
  }
  if (st == DOCI_ERR_FORMAT && bad <= 1) {
    std::fprintf(stderr, "Error in reading %s. File is wrongly formatted.\n", dumpfil);
    std::exit(EXIT_FAILURE);
  }
  if (st != DOCI_OK && st != DOCI_ERR_TOO_MANY_ORBITALS) {
    std::fprintf(stderr, "Whilst reading the integrals, an error occured, wrong formatting at line %d!\n", bad);
    std::exit(EXIT_FAILURE);
  }
  if (st == DOCI_OK && in.Na != in.Nb) {  // doci.c:76-82
    std::fprintf(stderr, "Number of up and down electrons not equal in FCIDUMP-file.\n");
    std::fprintf(stderr, "This is obligatory for DOCI.\n");
    std::printf("Exiting...\n");
    std::exit(EXIT_FAILURE);
  }
  if (st == DOCI_ERR_TOO_MANY_ORBITALS || in.L > kMaxOrbitals) {  // doci.c:84-89
    std::fprintf(stderr, "Too many orbitals.\n");
    std::printf("Exiting...\n");
    std::exit(EXIT_FAILURE);
  }
  doci_ham *h = nullptr;
  st = build_from_integrals(in, &h);
  if (st) die_cuda("fill_doci_data", st);
  h->from_fill = true;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaDeviceProp prop;
  cudaGetDeviceProperties(&prop, dev);
  std::printf(
      "----------\n"
      "\t** executing DOCI (GPU %d: %s, %d SMs)\n"
      "\t** N = (%u,%u)\n"
      "\t** L = %u\n"
      "\t** basis size : %u\n"
      "----------\n",
      dev, prop.name, sms, h->N, h->N, h->L, h->D);
  std::fflush(stdout);
  *dat = h;
}

double *doci_get_diagonal(void *vdat) {
  doci_ham *h = static_cast<doci_ham *>(vdat);
  if (!h->h_diag) {
    if (cudaMallocHost(&h->h_diag, sizeof(double) * h->D) != cudaSuccess) die_cuda("doci_get_diagonal", DOCI_ERR_OUT_OF_MEMORY);
    if (cudaMemcpy(h->h_diag, h->d_diag, sizeof(double) * h->D, cudaMemcpyDeviceToHost) != cudaSuccess)
      die_cuda("doci_get_diagonal", DOCI_ERR_CUDA);
  }
  return h->h_diag;
}

int doci_get_basis_size(void *vdat) { return static_cast<int>(static_cast<doci_ham *>(vdat)->D); }

void doci_cleanup_data(void **vdat) {
  doci_ham_destroy(static_cast<doci_ham *>(*vdat));
  *vdat = nullptr;
}

void doci_matvec(double *vec, double *result, void *vdat) {
  const int st = doci_sigma_host(static_cast<doci_ham *>(vdat), vec, result, DOCI_FP64);
  if (st) die_cuda("doci_matvec", st);
}

namespace {

// Resolve the (matvec, dat, diagonal) triple of the reference's solver API:
// our own matvec on our own handle runs the device sigma; anything else is
// called on host buffers.  A host diagonal other than the handle's is
// uploaded.
struct SolverContext {
  MatvecOp op;
  doci_ham *h = nullptr;
  DevBuf diag_buf;
  const double *d_diag = nullptr;
  cudaStream_t st = nullptr;
  cudaStream_t own = nullptr;
  ~SolverContext() {
    // members are destroyed after this body: free the diagonal copy while its
    // stream still exists, then retire the stream
    if (diag_buf.p) cudaFreeAsync(diag_buf.p, diag_buf.st);
    diag_buf.p = nullptr;
    if (own) {
      cudaStreamSynchronize(own);
      cudaStreamDestroy(own);
    }
  }
  int init(void (*matvec)(double *, double *, void *), void *vdat, const double *diagonal, size_t n) {
    op.n = n;
    if (matvec == doci_matvec && reg_has(vdat)) {
      h = static_cast<doci_ham *>(vdat);
      if (static_cast<size_t>(h->D) != n) return DOCI_ERR_INVALID;
      op.ham = h;
      st = h->stream;
    } else {
      op.host_fn = matvec;
      op.host_dat = vdat;
      DOCI_CUDA(cudaStreamCreateWithFlags(&own, cudaStreamNonBlocking));
      st = own;
    }
    if (diagonal) {
      if (h && diagonal == h->h_diag) {
        d_diag = h->d_diag;
      } else {
        diag_buf.st = st;
  DOCI_CUDA(cudaMallocAsync(&diag_buf.p, sizeof(double) * n, st));
        DOCI_CUDA(cudaMemcpyAsync(diag_buf.p, diagonal, sizeof(double) * n, cudaMemcpyHostToDevice, st));
        d_diag = static_cast<const double *>(diag_buf.p);
      }
    }
    return DOCI_OK;
  }
};

bool env_flag(const char *name) {
  const char *v = std::getenv(name);
  return v && *v && std::strcmp(v, "0") != 0;
}

}  // namespace

int davidson(double *result, double *energy, int max_vectors, int keep_deflate, double davidson_tol,
             void (*matvec)(double *, double *, void *), double *diagonal, int basis_size, int max_its,
             void *vdat) {
  const size_t n = static_cast<size_t>(basis_size);
  SolverContext ctx;
  int st = ctx.init(matvec, vdat, diagonal, n);
  if (st) die_cuda("davidson", st);
  if (!ctx.d_diag) die_cuda("davidson (no diagonal)", DOCI_ERR_INVALID);
  DevBuf t, x;
  t.st = x.st = ctx.st;
  if (cudaMallocAsync(&t.p, sizeof(double) * n, ctx.st) || cudaMallocAsync(&x.p, sizeof(double) * n, ctx.st))
    die_cuda("davidson", DOCI_ERR_OUT_OF_MEMORY);
  cudaMemcpyAsync(t.p, result, sizeof(double) * n, cudaMemcpyHostToDevice, ctx.st);
  DavidsonArgs a;
  a.max_vectors = max_vectors;
  a.keep = keep_deflate;
  a.tol = davidson_tol;
  a.max_its = max_its;
  a.print_table = env_flag("DOCI_DAVIDIT");
  a.print_summary = !a.print_table;
  DavidsonOut out;
  st = davidson_run<double>(ctx.op, n, ctx.d_diag, static_cast<double *>(t.p), a, ctx.st, &out,
                            static_cast<double *>(x.p));
  if (st) die_cuda("davidson", st);
  if (cudaMemcpy(result, x.p, sizeof(double) * n, cudaMemcpyDeviceToHost) != cudaSuccess)
    die_cuda("davidson", DOCI_ERR_CUDA);
  *energy = out.energy;
  return out.return_code;
}

int ray_q(void (*matvec)(double *, double *, void *), double *M, double *vec, int size, double *energy,
          double cg_tol, int max_its, double *precond, void *vdat) {
  if (M != nullptr) {  // CG.c:26-29
    std::fprintf(stderr, "%s:%d @ %s :: Wrong M!\n", __FILE__, __LINE__, __func__);
    std::exit(EXIT_FAILURE);
  }
  const size_t n = static_cast<size_t>(size);
  SolverContext ctx;
  int st = ctx.init(matvec, vdat, precond, n);
  if (st) die_cuda("ray_q", st);
  DevBuf x;
  x.st = ctx.st;
  if (cudaMallocAsync(&x.p, sizeof(double) * n, ctx.st)) die_cuda("ray_q", DOCI_ERR_OUT_OF_MEMORY);
  cudaMemcpyAsync(x.p, vec, sizeof(double) * n, cudaMemcpyHostToDevice, ctx.st);
  CgArgs a;
  a.max_its = max_its;
  a.tol = cg_tol;
  a.print = 1;
  CgOut out;
  st = ray_q_run(ctx.op, n, precond ? ctx.d_diag : nullptr, static_cast<double *>(x.p), a, ctx.st, &out);
  if (st) die_cuda("ray_q", st);
  if (cudaMemcpy(vec, x.p, sizeof(double) * n, cudaMemcpyDeviceToHost) != cudaSuccess) die_cuda("ray_q", DOCI_ERR_CUDA);
  *energy = out.energy;
  return out.return_code;
}

int sparse_eigensolve(double *vec, int dims, double *energy, void (*matvec)(double *, double *, void *),
                      double *diagonal, double *M, double tol, int max_its, char solver[], int davidson_keep,
                      int davidson_max_vec, void *dat) {
  int res = -1;  // wrapper_solvers.c:14-23
  if (std::strcmp(solver, "D") == 0)
    res = davidson(vec, energy, davidson_max_vec, davidson_keep, tol, matvec, diagonal, dims, max_its, dat);
  else if (std::strcmp(solver, "CG") == 0)
    res = ray_q(matvec, M, vec, dims, energy, tol, max_its, nullptr, dat);
  else if (std::strcmp(solver, "CGP") == 0)
    res = ray_q(matvec, M, vec, dims, energy, tol, max_its, diagonal, dat);
  return res;
}

}  // extern "C"
