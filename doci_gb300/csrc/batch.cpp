// batch.cpp -- multi-root solves, batched solves of many Hamiltonians, and the
// request server (continuous batching with HBM-footprint admission).
//
// No counterpart in the reference (single Hamiltonian, single root,
// davidson.c:90 / :117 use the lowest eigenvalue only).  Every solve runs the
// device-resident block Davidson (solvers.cu) on its own CUDA stream; a pool
// of host workers keeps several solves in flight so that their kernels
// overlap on the GPU.  A solve's arithmetic does not depend on what else runs
// (fixed grids, fixed-order reductions, no atomics), so a result is the same
// alone and in the mix.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include "internal.h"
#include "solvers.h"
#include "vec.h"

namespace doci {
int vec_argmin(const double *d, size_t n, int64_t *idx, cudaStream_t st);
int vec_set_unit(double *t, size_t n, int64_t idx, cudaStream_t st);
}  // namespace doci

using namespace doci;

namespace {

struct StreamBuf {
  void *p = nullptr;
  cudaStream_t st = nullptr;
  StreamBuf() = default;
  StreamBuf(const StreamBuf &) = delete;
  StreamBuf &operator=(const StreamBuf &) = delete;
  ~StreamBuf() {
    if (p) cudaFreeAsync(p, st);
  }
  int alloc(size_t bytes, cudaStream_t s) {
    st = s;
    DOCI_CUDA(cudaMallocAsync(&p, bytes ? bytes : 16, s));
    return DOCI_OK;
  }
};

#define DOCI_TRY_B(expr)            \
  do {                              \
    const int _st = (expr);         \
    if (_st != DOCI_OK) return _st; \
  } while (0)

// nroots start vectors: unit vectors on the nroots lowest diagonal elements
// (the HF start of executable.c:276-288, extended to several roots)
int start_vectors(doci_ham *h, int R, double *d_T, cudaStream_t st) {
  const size_t D = h->D;
  StreamBuf tmp;
  DOCI_TRY_B(tmp.alloc(sizeof(double) * D, st));
  double *d = static_cast<double *>(tmp.p);
  DOCI_CUDA(cudaMemcpyAsync(d, h->d_diag, sizeof(double) * D, cudaMemcpyDeviceToDevice, st));
  const double inf = 1e308;
  for (int r = 0; r < R; ++r) {
    int64_t idx = 0;
    DOCI_TRY_B(vec_argmin(d, D, &idx, st));
    DOCI_TRY_B(vec_set_unit(d_T + static_cast<size_t>(r) * D, D, idx, st));
    DOCI_CUDA(cudaMemcpyAsync(d + idx, &inf, sizeof(double), cudaMemcpyHostToDevice, st));
    DOCI_CUDA(cudaStreamSynchronize(st));
  }
  return DOCI_OK;
}

double clock_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// The solve of one Hamiltonian for the nroots lowest eigenpairs, on stream st.
int solve_roots(doci_ham *h, const doci_batch_opts &o, cudaStream_t st, doci_root_result *res, double *vecs) {
  const int R = o.nroots;
  if (R < 1 || R > 8 || static_cast<uint64_t>(R) > h->D) return DOCI_ERR_INVALID;
  const size_t D = h->D;
  MatvecOp op;
  op.ham = h;
  op.n = D;
  StreamBuf X, T;
  DOCI_TRY_B(X.alloc(sizeof(double) * D * R, st));
  DOCI_TRY_B(T.alloc(sizeof(double) * D * R, st));
  double *d_X = static_cast<double *>(X.p), *d_T = static_cast<double *>(T.p);
  DOCI_TRY_B(start_vectors(h, R, d_T, st));
  BlockArgs a;
  a.nroots = R;
  a.max_vectors = o.max_vec < 2 * R ? 2 * R : o.max_vec;
  if (a.max_vectors > 32) a.max_vectors = 32;
  // thick restart: by default keep 2 nroots Ritz vectors, at least a quarter
  // of the basis (keeping only the nroots wanted ones restarts every few
  // blocks and stalls the higher roots: measured on 40 of the batch
  // workload's problems, 4 roots, 30/40 converged within 200 iterations with
  // keep = 4 against 40/40 with keep = 8)
  a.keep = o.keep > 0 ? o.keep : std::max(2 * R, a.max_vectors / 4);
  if (a.keep < R) a.keep = R;
  if (a.keep > a.max_vectors - R) a.keep = a.max_vectors - R;
  a.max_its = o.max_its;
  a.tol = o.tol;
  BlockOut out;
  int its32 = 0;
  if (o.mode == DOCI_MODE_MIXED) {
    StreamBuf T32;
    DOCI_TRY_B(T32.alloc(sizeof(float) * D * R, st));
    DOCI_TRY_B((vec_convert<double, float>(d_T, static_cast<float *>(T32.p), D * R, st)));
    BlockArgs a32 = a;
    a32.tol = o.mixed_tol > o.tol ? o.mixed_tol : o.tol;
    a32.stall_window = 15;
    // the FP32 phase runs on H - (lowest diagonal element)
    ShiftedView sv;
    DOCI_TRY_B(sv.make(h, st));
    a32.shift = sv.shift;
    MatvecOp op32;
    op32.ham = &sv.view;
    op32.n = D;
    BlockOut o32;
    DOCI_TRY_B(block_davidson_run<float>(op32, D, h->d_diag, static_cast<float *>(T32.p), a32, st, &o32, d_X));
    its32 = o32.iterations;
    for (int r = 0; r < R; ++r) res->energy_fp32[r] = o32.energy[r];
    DOCI_CUDA(cudaMemcpyAsync(d_T, d_X, sizeof(double) * D * R, cudaMemcpyDeviceToDevice, st));
    a.max_its = o.max_its - its32 > 1 ? o.max_its - its32 : 1;
    out.sigmas = o32.sigmas;
  }
  DOCI_TRY_B(block_davidson_run<double>(op, D, h->d_diag, d_T, a, st, &out, d_X));
  res->nroots = R;
  for (int r = 0; r < R; ++r) {
    res->energy[r] = out.energy[r];
    res->residual[r] = out.residual[r];
  }
  res->iterations = out.iterations + its32;
  res->iterations_fp32 = its32;
  res->sigmas = out.sigmas;
  res->converged = out.converged;
  if (vecs) {
    DOCI_CUDA(cudaMemcpyAsync(vecs, d_X, sizeof(double) * D * R, cudaMemcpyDeviceToHost, st));
  }
  DOCI_CUDA(cudaStreamSynchronize(st));
  return DOCI_OK;
}

int64_t roots_footprint(int L, int N, const doci_batch_opts &o) {
  if (L < 1 || L > 32 || N < 0 || N > L) return -1;
  const int64_t D = static_cast<int64_t>(binom64(L, N));
  const int64_t R = o.nroots, mv = std::min(32, std::max(o.max_vec, 2 * o.nroots));
  const int64_t ham = D * 12 + (16ll << 20);  // diagonals, tables
  const int64_t common = D * R * 8 * 2 + D * 8;  // X, T, start-vector scratch
  const int64_t p64 = 2 * mv * D * 8 + R * D * 8;
  // FP32 phase: basis, start and correction blocks, shifted FP32 diagonal
  const int64_t p32 = o.mode == DOCI_MODE_MIXED ? 2 * mv * D * 4 + R * D * 4 * 2 + D * 4 : 0;
  return ham + common + std::max(p64, p32) + (4ll << 20);
}

}  // namespace

// ===========================================================================
// Request server
// ===========================================================================
struct doci_server {
  doci_batch_opts opts{};
  double t0 = 0;
  int64_t budget = 0;
  std::mutex mu;
  std::condition_variable cv_work, cv_done, cv_mem;
  struct Req {
    int64_t ticket;
    int L = 0, N = 0;
    double core = 0;
    std::vector<double> one, two;  // integrals (read_fcidump layout)
    std::string path;              // or an FCIDUMP file
    doci_ham *ham = nullptr;       // or a caller-owned handle (batch mode)
    double queued = 0;
  };
  std::deque<Req> queue;
  std::map<int64_t, doci_root_result> done;
  std::vector<std::thread> workers;
  int64_t next_ticket = 1, in_use = 0, running = 0, submitted = 0, finished = 0;
  bool stop = false;
  int device = 0;  // the device current when the server was created: every worker solves on it

  void worker_main() {
    cudaStream_t st = nullptr;
    // a worker without its device or stream still takes requests and completes
    // them with DOCI_ERR_CUDA, so that no ticket stays pending
    bool usable = cudaSetDevice(device) == cudaSuccess &&
                  cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) == cudaSuccess;
    if (!usable) cudaGetLastError();
    for (;;) {
      Req r;
      {
        std::unique_lock<std::mutex> lk(mu);
        cv_work.wait(lk, [&] { return stop || !queue.empty(); });
        if (stop && queue.empty()) break;
        r = std::move(queue.front());
        queue.pop_front();
      }
      doci_root_result res;
      std::memset(&res, 0, sizeof res);
      res.queued_s = r.queued;
      res.status = usable ? run(r, st, &res) : DOCI_ERR_CUDA;
      res.end_s = clock_s() - t0;
      {
        std::lock_guard<std::mutex> lk(mu);
        done[r.ticket] = res;
        ++finished;
      }
      cv_done.notify_all();
    }
    if (st) cudaStreamDestroy(st);
  }

  int run(Req &r, cudaStream_t st, doci_root_result *res) {
    // size of the request, for admission
    int L = r.L, N = r.N;
    Integrals in;
    if (r.ham) {
      L = r.ham->L;
      N = r.ham->N;
    } else if (!r.path.empty()) {
      int bad = 0;
      const int s = read_fcidump_file(r.path.c_str(), &in, &bad);
      if (s) return s;
      if (in.Na != in.Nb) return DOCI_ERR_NALPHA_NBETA;
      L = in.L;
      N = in.Na;
    } else {
      in.L = r.L;
      in.Na = in.Nb = r.N;
      in.core = r.core;
      in.one = std::move(r.one);
      in.two = std::move(r.two);
    }
    const int64_t fp = roots_footprint(L, N, opts);
    if (fp < 0) return DOCI_ERR_INVALID;
    if (fp > budget) return DOCI_ERR_ADMISSION;
    {
      std::unique_lock<std::mutex> lk(mu);
      cv_mem.wait(lk, [&] { return in_use + fp <= budget; });
      in_use += fp;
      ++running;
    }
    res->start_s = clock_s() - t0;
    int s = DOCI_OK;
    doci_ham *h = r.ham;
    bool own = false;
    if (!h) {
      h = new doci_ham();
      s = ham_build(h, in);
      own = true;
    }
    if (s == DOCI_OK) s = solve_roots(h, opts, st, res, nullptr);
    if (own) {
      ham_release(h);
      delete h;
    }
    {
      std::lock_guard<std::mutex> lk(mu);
      in_use -= fp;
      --running;
    }
    cv_mem.notify_all();
    return s;
  }

  int64_t submit(Req &&r) {
    int64_t t;
    {
      std::lock_guard<std::mutex> lk(mu);
      t = next_ticket++;
      r.ticket = t;
      r.queued = clock_s() - t0;
      queue.push_back(std::move(r));
      ++submitted;
    }
    cv_work.notify_one();
    return t;
  }
};

extern "C" {

void doci_batch_opts_default(doci_batch_opts *o) {
  if (!o) return;
  std::memset(o, 0, sizeof *o);
  o->nroots = 1;
  o->max_vec = 16;
  o->max_its = 200;
  o->tol = 1e-6;
  o->mode = DOCI_MODE_MIXED;
  o->mixed_tol = 1e-4;
  o->workers = 8;
  o->hbm_budget = 0;
}

int64_t doci_roots_footprint(int L, int n_pairs, const doci_batch_opts *o) {
  doci_batch_opts d;
  if (!o) {
    doci_batch_opts_default(&d);
    o = &d;
  }
  return roots_footprint(L, n_pairs, *o);
}

int doci_solve_roots(doci_ham *h, const doci_batch_opts *opts, doci_root_result *res, double *vecs) {
  if (!h || !res) return DOCI_ERR_INVALID;
  doci_batch_opts o;
  if (opts) o = *opts; else doci_batch_opts_default(&o);
  std::memset(res, 0, sizeof *res);
  const double t0 = clock_s();
  const int s = solve_roots(h, o, h->stream, res, vecs);
  res->end_s = clock_s() - t0;
  res->status = s;
  return s;
}

int doci_server_create(const doci_batch_opts *opts, doci_server **out) {
  if (!out) return DOCI_ERR_INVALID;
  auto *srv = new (std::nothrow) doci_server();
  if (!srv) return DOCI_ERR_OUT_OF_MEMORY;
  if (opts) srv->opts = *opts; else doci_batch_opts_default(&srv->opts);
  if (srv->opts.workers < 1) srv->opts.workers = 1;
  if (cudaGetDevice(&srv->device) != cudaSuccess) {
    cudaGetLastError();
    delete srv;
    return DOCI_ERR_NO_DEVICE;
  }
  srv->budget = srv->opts.hbm_budget;
  if (srv->budget <= 0) {
    size_t fr = 0, tot = 0;
    if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) {
      cudaGetLastError();
      delete srv;
      return DOCI_ERR_NO_DEVICE;
    }
    srv->budget = static_cast<int64_t>(fr * 0.85);
  }
  srv->t0 = clock_s();
  for (int w = 0; w < srv->opts.workers; ++w) srv->workers.emplace_back([srv] { srv->worker_main(); });
  *out = srv;
  return DOCI_OK;
}

int doci_server_submit(doci_server *srv, int L, int n_pairs, double core, const double *one, const double *two,
                       int64_t *ticket) {
  if (!srv || !one || !two || !ticket || L < 1 || L > 32 || n_pairs < 0 || n_pairs > L) return DOCI_ERR_INVALID;
  doci_server::Req r;
  r.L = L;
  r.N = n_pairs;
  r.core = core;
  const size_t n2 = static_cast<size_t>(L) * L;
  r.one.assign(one, one + n2);
  r.two.assign(two, two + n2 * n2);
  *ticket = srv->submit(std::move(r));
  return DOCI_OK;
}

int doci_server_submit_fcidump(doci_server *srv, const char *path, int64_t *ticket) {
  if (!srv || !path || !ticket) return DOCI_ERR_INVALID;
  doci_server::Req r;
  r.path = path;
  *ticket = srv->submit(std::move(r));
  return DOCI_OK;
}

int doci_server_poll(doci_server *srv, int64_t ticket, doci_root_result *out) {
  if (!srv || !out) return DOCI_ERR_INVALID;
  std::lock_guard<std::mutex> lk(srv->mu);
  auto it = srv->done.find(ticket);
  if (it == srv->done.end()) return ticket > 0 && ticket < srv->next_ticket ? DOCI_ERR_PENDING : DOCI_ERR_NOT_FOUND;
  *out = it->second;
  return DOCI_OK;
}

int doci_server_wait(doci_server *srv, int64_t ticket, doci_root_result *out) {
  if (!srv || !out) return DOCI_ERR_INVALID;
  std::unique_lock<std::mutex> lk(srv->mu);
  if (ticket <= 0 || ticket >= srv->next_ticket) return DOCI_ERR_NOT_FOUND;
  srv->cv_done.wait(lk, [&] { return srv->done.count(ticket) != 0; });
  *out = srv->done[ticket];
  return DOCI_OK;
}

int doci_server_stats(doci_server *srv, int64_t *submitted, int64_t *finished, int64_t *running,
                      int64_t *bytes_in_use) {
  if (!srv) return DOCI_ERR_INVALID;
  std::lock_guard<std::mutex> lk(srv->mu);
  if (submitted) *submitted = srv->submitted;
  if (finished) *finished = srv->finished;
  if (running) *running = srv->running;
  if (bytes_in_use) *bytes_in_use = srv->in_use;
  return DOCI_OK;
}

void doci_server_destroy(doci_server *srv) {
  if (!srv) return;
  {
    std::lock_guard<std::mutex> lk(srv->mu);
    srv->stop = true;
  }
  srv->cv_work.notify_all();
  for (auto &t : srv->workers) t.join();
  delete srv;
}

int doci_batch_solve(int n, doci_ham *const *hams, const doci_batch_opts *opts, doci_root_result *results) {
  if (n < 0 || (n > 0 && (!hams || !results))) return DOCI_ERR_INVALID;
  doci_server *srv = nullptr;
  int s = doci_server_create(opts, &srv);
  if (s) return s;
  std::vector<int64_t> tickets(n);
  for (int i = 0; i < n; ++i) {
    doci_server::Req r;
    r.ham = hams[i];
    tickets[i] = srv->submit(std::move(r));
  }
  int first_err = DOCI_OK;
  for (int i = 0; i < n; ++i) {
    doci_server_wait(srv, tickets[i], &results[i]);
    if (results[i].status != DOCI_OK && first_err == DOCI_OK) first_err = results[i].status;
  }
  doci_server_destroy(srv);
  return first_err;
}

}  // extern "C"
