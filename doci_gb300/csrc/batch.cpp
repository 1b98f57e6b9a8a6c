// batch.cpp -- multi-root solves, batched solves of many Hamiltonians, and the
// request server (continuous batching with HBM-footprint admission).
//
// No counterpart in the reference (single Hamiltonian, single root,
// davidson.c:90 / :117 use the lowest eigenvalue only).  Every solve runs on
// the batch engine (engine.cu): doci_batch_solve hands it the whole batch
// (in groups that fit the HBM budget), one lockstep iteration for all
// problems; doci_solve_roots and the request server's workers hand it one
// problem each, and the server keeps several such solves in flight on their
// own streams so that their kernels overlap on the GPU.  A problem's
// arithmetic in the engine does not depend on the other problems (fixed
// chunks, fixed-order reductions, no atomics), so a result is the same alone,
// in a batch and in the server's mix.
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

#include "engine.h"
#include "internal.h"

using namespace doci;

namespace {

double clock_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// The solve of one Hamiltonian for the nroots lowest eigenpairs, on stream st:
// the batch engine with a batch of one (the same arithmetic as in any batch).
int solve_roots(doci_ham *h, const doci_batch_opts &o, cudaStream_t st, doci_root_result *res, double *vecs) {
  if (o.nroots < 1 || o.nroots > 8 || static_cast<uint64_t>(o.nroots) > h->D) return DOCI_ERR_INVALID;
  double *const v[1] = {vecs};
  return engine_solve(1, &h, o, st, res, v);
}

int64_t roots_footprint(int L, int N, const doci_batch_opts &o) {
  const int64_t e = engine_footprint(L, N, o);
  if (o.nroots != 1 || e < 0) return e;
  doci_solve_opts so;
  doci_solve_opts_default(&so);
  so.mode = o.mode;
  so.davidson_max_vec = o.max_vec;
  const int64_t d = doci_solve_footprint(L, N, &so, 1);
  return d > e ? d : e;
}

// A one-root request of the server: the single-root device Davidson
// (doci_solve on the request's own handle and stream; mixed or FP64 as the
// options say), which needs fewer vector passes per iteration than the
// block engine.
int solve_single(doci_ham *h, const doci_batch_opts &o, doci_root_result *res) {
  doci_solve_opts so;
  doci_solve_opts_default(&so);
  so.solver = DOCI_SOLVER_D;
  so.max_its = o.max_its;
  so.tol = o.tol;
  so.mode = o.mode;
  so.mixed_tol = o.mixed_tol;
  so.davidson_max_vec = o.max_vec;
  so.davidson_keep = 2;
  so.print_level = 0;
  doci_solve_result r;
  const int s = doci_solve(h, &so, nullptr, &r);
  if (s != DOCI_OK) return s;
  res->nroots = 1;
  res->energy[0] = r.energy;
  res->residual[0] = r.residual;
  res->energy_fp32[0] = r.energy_fp32;
  res->iterations = r.iterations;
  res->iterations_fp32 = r.iterations_fp32;
  res->sigmas = r.iterations;
  res->converged = r.converged;
  return DOCI_OK;
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
    if (s == DOCI_OK) s = opts.nroots == 1 ? solve_single(h, opts, res) : solve_roots(h, opts, st, res, nullptr);
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

int doci_engine_autotune(doci_ham *h, int nvec, int *dets_per_thread) {
  if (!h) return DOCI_ERR_INVALID;
  return engine_tune(h, nvec, dets_per_thread);
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
  if (n == 0) return DOCI_OK;
  doci_batch_opts o;
  if (opts) o = *opts; else doci_batch_opts_default(&o);
  for (int i = 0; i < n; ++i) {
    if (!hams[i]) return DOCI_ERR_INVALID;
    std::memset(&results[i], 0, sizeof results[i]);
  }
  int64_t budget = o.hbm_budget;
  if (budget <= 0) {
    size_t fr = 0, tot = 0;
    if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) {
      cudaGetLastError();
      return DOCI_ERR_NO_DEVICE;
    }
    budget = static_cast<int64_t>(fr * 0.85);
  }
  cudaStream_t st = nullptr;
  DOCI_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  const double t0 = clock_s();
  int first_err = DOCI_OK;
  // groups of consecutive problems whose engine footprint fits the budget
  // (the handles' own memory is already allocated: count the solve's share)
  for (int i = 0; i < n;) {
    int64_t used = 0;
    int j = i;
    while (j < n) {
      const int64_t f = engine_footprint(hams[j]->L, hams[j]->N, o) - static_cast<int64_t>(hams[j]->D) * 12;
      if (j > i && used + f > budget) break;
      used += f;
      ++j;
    }
    const double ts = clock_s() - t0;
    int s = (used > budget) ? DOCI_ERR_ADMISSION : engine_solve(j - i, hams + i, o, st, results + i, nullptr);
    const double te = clock_s() - t0;
    for (int k = i; k < j; ++k) {
      results[k].status = s;
      results[k].queued_s = 0;
      results[k].start_s = ts;
      results[k].end_s = te;
    }
    if (s != DOCI_OK && first_err == DOCI_OK) first_err = s;
    i = j;
  }
  cudaStreamDestroy(st);
  return first_err;
}

}  // extern "C"
