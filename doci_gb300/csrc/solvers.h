// solvers.h -- device-resident Davidson and RQ-CG drivers (solvers.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <vector>

#include "internal.h"

namespace doci {

// The matvec a solver calls once per iteration: the device sigma of `ham`
// (in the solver's storage precision), or a host function on FP64 buffers.
struct MatvecOp {
  doci_ham *ham = nullptr;
  void (*host_fn)(double *, double *, void *) = nullptr;
  void *host_dat = nullptr;
  size_t n = 0;
  std::vector<double> hx, hy;
  double sigma_seconds = 0;
  bool events_on = false;
  cudaEvent_t ev0{}, ev1{};
  // FP64 phase of the mixed mode: the first FP64 sigma after `anchor_next`
  // is a true FP64 sigma (the anchor vector); the later ones (correction
  // vectors, whose coefficients in the Ritz vector are of the size of the
  // residual) run on the shifted FP32 view: y = sigma32((float)x) + shift x.
  // Their FP32 rounding enters the Ritz vector scaled by those coefficients.
  // With ham32 set the operator is the shifted H - shift32 (both paths): the
  // anchor's FP64 sigma gets -shift32 x added, the FP32 sigma of the view is
  // already shifted.  The FP64 phase then works, like the FP32 phase, with
  // quantities of the size of H - shift32, so its FP32-arithmetic correction
  // terms stay accurate.
  const doci_ham *ham32 = nullptr;
  double shift32 = 0;
  float *x32 = nullptr, *y32 = nullptr;  // D-element scratch, owned by the caller
  bool anchor_next = true;
  int apply(const void *d_x, void *d_y, int precision, cudaStream_t st);
  void enable_timing();
  ~MatvecOp();
};

struct DavidsonArgs {
  int max_vectors = 30, keep = 2, max_its = 200;
  double tol = 1e-8;
  int print_table = 0;    // the -DDAVIDIT table of davidson.c:47-112
  int print_summary = 0;  // "** DAVIDSON ITERATIONS" (davidson.c:114)
  int stall_window = 0;   // > 0: stop when the residual stops reaching new minima (mixed mode)
  // the operator is H - shift (energies are reported + shift; the
  // preconditioner's diagonal is the unshifted FP64 one)
  double shift = 0;
  // optional per-iteration records {phase, residual, energy, seconds since
  // trace_t0} (4 doubles each), trace_len records at most
  double *trace = nullptr;
  int trace_len = 0;
  double trace_t0 = 0;
  double trace_phase = 0;
  int *trace_count = nullptr;  // records written so far (shared across phases)
};

struct DavidsonOut {
  double energy = 0, residual = 0, seconds = 0;
  int iterations = 0, converged = 0, return_code = 0;
};

struct CgArgs {
  int max_its = 200;
  double tol = 1e-8;
  int print = 1;  // CG.c prints its table unconditionally
  double *trace = nullptr;
  int trace_len = 0;
};

struct CgOut {
  double energy = 0, normq = 0, normq_g = 0, seconds = 0;
  int iterations = 0, converged = 0, return_code = 0;
};

double now_s();  // steady clock, seconds

// The FP32 phase of the mixed mode runs on H - s, s = the lowest diagonal
// element (the reference determinant's energy): the FP32 rounding of sigma
// then scales with |H - s| on the determinants that carry the ground state
// (a few Ha) instead of with |E| (hundreds of Ha at L = 32).  `view` is a copy
// of the handle whose FP32 diagonal is diag - s (owned here, freed on st).
struct ShiftedView {
  doci_ham view;
  double shift = 0;
  float *d_diag32 = nullptr;
  cudaStream_t st = nullptr;
  int make(const doci_ham *h, cudaStream_t s);
  ShiftedView() = default;
  ShiftedView(const ShiftedView &) = delete;
  ShiftedView &operator=(const ShiftedView &) = delete;
  ~ShiftedView();
};

template <typename S>
int davidson_run(MatvecOp &op, size_t D, const double *d_diag, S *d_t, const DavidsonArgs &a, cudaStream_t st,
                 DavidsonOut *out, double *d_x_out);

int ray_q_run(MatvecOp &op, size_t D, const double *d_diag_or_null, double *d_x, const CgArgs &a, cudaStream_t st,
              CgOut *out);

}  // namespace doci
