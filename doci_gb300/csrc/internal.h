// internal.h -- shared definitions of libdoci_gb300 (not part of the C ABI).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

#include "../../include/doci_gb300.h"
#include "host_plan.h"

namespace doci {

constexpr int kMaxOrbitals = 32;
// binomial table C(n, k) for n = 0..32 and k = 0..34 (k up to N + 2 is read
// by the neighbour-rank prefix sums)
constexpr int kBinomRows = 33;
constexpr int kBinomCols = 35;

// Integrals after the reference's transform (doci.c:630-665), reduced to the
// L x L tables the DOCI Hamiltonian needs.
struct Integrals {
  int L = 0, Na = 0, Nb = 0;
  double core = 0;
  std::vector<double> one;  // h' (L*L), after the transform
  std::vector<double> two;  // (ij|kl) (L^4), after the transform
};

// FCIDUMP reader restating read_fcidump.c:18-82; returns a doci_status and
// the offending line number on a format error.
int read_fcidump_file(const char *path, Integrals *out, int *bad_line);
// relaxed reader (fcidump.cpp): multi-line namelist, any key order, other
// keys ignored, any integral index order (stored canonically)
int read_fcidump_relaxed(const char *path, Integrals *out, int *bad_line);
// doci.c:630-665 (in place)
void transform_integrals(double *one, double *two, int L);
// doci.c:687-701
uint32_t combination(unsigned n, unsigned m);
uint64_t binom64(unsigned n, unsigned k);
void fill_binom_table(uint32_t *t);  // kBinomRows x kBinomCols

// cached device properties
int device_sm_count();

// CUDA error plumbing: every CUDA call goes through check(); the first
// failure is remembered per thread for doci_status_string.
int cuda_status(cudaError_t e, const char *what);
#define DOCI_CUDA(call)                                       \
  do {                                                        \
    cudaError_t _e = (call);                                  \
    if (_e != cudaSuccess) return ::doci::cuda_status(_e, #call); \
  } while (0)

}  // namespace doci

// The opaque handle of the C ABI.
struct doci_ham {
  int L = 0, N = 0;
  uint32_t D = 0;
  int nh = 0;  // holes per determinant, L - N
  double core = 0;
  int device = 0;
  cudaStream_t stream = nullptr;

  // host tables (L x L, row-major by first orbital)
  std::vector<double> h2;   // 2 h'_ii
  std::vector<double> J2;   // 2 (ii|jj)
  std::vector<double> Kx;   // (ij|ji)
  std::vector<double> Kp;   // (ia|ia), zero diagonal (Viikk, doci.c:667-683)

  // device tables
  uint32_t *d_binom = nullptr;   // kBinomRows x kBinomCols
  double *d_Kmir64 = nullptr;    // 32 x 32, mirrored orbitals: [m][q] = K[L-1-m][L-1-q]
  float *d_Kmir32 = nullptr;
  double *d_tab64 = nullptr;     // h2 | J2 | Kx for the diagonal kernel
  double *d_diag = nullptr;      // D, FP64 diagonal
  float *d_diag32 = nullptr;     // D, FP32 copy

  // Row tiling of the rank space used by the row sigma kernel: mirrored
  // orbitals [0, split) are the "column" part, [split, L) the "row" part.
  // All determinants with the same row-part occupation form one contiguous
  // rank range (a row) of C(split, j) columns, j = N - |row part|.
  int split = 0;                  // columns' orbitals; 0 = row kernel unused
  int nrows = 0;
  int max_row = 0;                // largest row length
  uint32_t *d_rows = nullptr;     // nrows x {rowstart, mask | k << 24}
  int sigma_kernel = 0;           // doci_ham_set_sigma_kernel's kind (0 automatic)
  uint32_t *d_rowstart = nullptr; // 2^(L - split) entries: row start by row-part mask
  // cross-hop index tables of the phase-ordered row pass (addressing.cuh,
  // build_cross_tables)
  uint32_t *d_rem = nullptr, *d_ins = nullptr, *d_tab_off = nullptr;
  // the insertion table in quads (entries 4q..4q+3 of column position c of
  // size j at tab_off[j] + 4 (q C(split, j) + c)): a warp's 16-byte loads of
  // one quad are consecutive (the pair kernels)
  uint32_t *d_ins_t = nullptr;
  // pair form (sigma_pair.cu): one block per (N-1)-pair set's row part R',
  // {own row start or ~0, mask | k' << 24}, largest first; the K matrix split
  // into TF32 high and low parts (2 x 32 x 32 floats, mirrored orbitals; also
  // the B operand of the tensor-core pair form, sigma_tc.cu)
  uint32_t *d_pblocks = nullptr;
  int npblocks = 0;
  void *d_kfrag = nullptr;
  // doci_sigma_host on the pair forms: x and sigma cross the host link in
  // pieces (chunk_off) on copy_stream while the pair units run in groups,
  // alternately on the handle's stream and side_stream (host_plan.h):
  // d_pblocks_host holds the units in group order, host_steps what each
  // group's launch waits for and which pieces go down after it.
  static constexpr int kHostChunks = doci::hostplan::kPieces;
  uint32_t *d_pblocks_host = nullptr;
  std::vector<doci::hostplan::Group> host_groups;
  std::vector<doci::hostplan::Step> host_steps;
  uint64_t chunk_off[kHostChunks + 1] = {};
  cudaStream_t copy_stream = nullptr, side_stream = nullptr;
  cudaEvent_t up_ev[kHostChunks] = {}, init_ev[kHostChunks] = {}, start_ev = nullptr, end_ev = nullptr,
              side_ev = nullptr;
  std::vector<cudaEvent_t> group_ev;  // one per host group

  // error word of the tensor-core sigma's bounded waits (0 = none)
  int *d_tc_err = nullptr;
  // host diagonal for doci_get_diagonal (lazy)
  double *h_diag = nullptr;
  // device staging for the host-buffer entry points (lazy)
  void *d_stage_x = nullptr, *d_stage_y = nullptr;
  size_t stage_bytes = 0;
  // the reference-compatible handle prints its banner once
  bool from_fill = false;
};

namespace doci {
// ham.cu
int ham_build(doci_ham *h, const Integrals &in);
void ham_release(doci_ham *h);
int ham_stage(doci_ham *h, size_t bytes);
int ham_device_error(doci_ham *h, cudaStream_t st);
// sigma.cu
// The kernel path of a sigma: kind as doci_ham_set_sigma_kernel (1, 3, 4, 6,
// 8) and the number of kernel launches it takes.
struct SigmaPlan {
  int kind, launches;
};
SigmaPlan plan_sigma(const doci_ham *h, int precision, bool allow_pair = true);
// Time the sigma paths that fit this handle's shape (nv = 1: single sigma,
// with and without the pair form; 2..4: the block paths) and keep the
// fastest for every handle of the same (device, L, N, precision) in this
// process; *choice gets the pick (a kind for nv = 1, a block method else).
int autotune_sigma(doci_ham *h, int precision, int nv, cudaStream_t s, int *choice);
bool sigma_tuned(const doci_ham *h, int precision, int nv);
// allow_pair = false keeps the FP32 result run-to-run reproducible (the pair
// form adds with atomics)
int launch_sigma(const doci_ham *h, const void *x, void *y, int precision, cudaStream_t s, bool allow_pair = true);
// nv <= 4 vectors x + v ldx -> y + v ldy with the neighbour work shared;
// never the pair form
int launch_sigma_multi(const doci_ham *h, const void *x, size_t ldx, void *y, size_t ldy, int nv, int precision,
                       cudaStream_t s);
// resident blocks per SM of a kernel with `dyn` bytes of dynamic shared
// memory (raises the kernel's dynamic shared-memory limit on first use)
int kernel_blocks(const void *kernel, int threads, size_t dyn, int *blocks);
// pair-form sigma (sigma_pair.cu), FP32 only
bool pair_fits(const doci_ham *h);
int launch_pair(const doci_ham *h, const float *x, float *y, cudaStream_t s);
// the same sigma from a pinned host x: the upload into dx in pieces,
// overlapped with the unit groups; y = dy on stream s, and, for a pinned hy,
// the pieces of dy copied to hy as they become final (all done when s is)
int launch_pair_host(doci_ham *h, const float *hx, float *dx, float *dy, float *hy, cudaStream_t s);
// FP64-accurate pair form in float-float arithmetic (sigma_pair.cu)
bool pair_ff_fits(const doci_ham *h);
int launch_pair_ff(const doci_ham *h, const double *x, double *y, cudaStream_t s);
// its host-buffer form on the same piece and group schedule as launch_pair_host
int launch_pair_ff_host(doci_ham *h, const double *hx, double *dx, double *dy, double *hy, cudaStream_t s);
// tensor-core pair form (sigma_tc.cu), FP32 only, sm_103a; x 16-byte aligned.
// A device wait that runs out writes a nonzero code to *d_err (spin_limit:
// try_wait iterations per wait).
constexpr long kTcSpinLimit = 1L << 20;  // try_wait polls per wait (seconds at most)
bool tc_fits(const doci_ham *h);
int tc_launches(const doci_ham *h);
int launch_tc(const doci_ham *h, const float *x, float *y, cudaStream_t s, int *d_err, long spin_limit);
int ham_build_pairs(doci_ham *h, const std::vector<uint32_t> &row_start);
int launch_bitstrings(const doci_ham *h, int64_t first, int64_t count, uint32_t *out, cudaStream_t s);
int launch_ranks(const doci_ham *h, const uint32_t *bits, int64_t count, int64_t *out, cudaStream_t s);
int launch_diagonal(doci_ham *h, cudaStream_t s);
int ham_build_rows(doci_ham *h);
}  // namespace doci
