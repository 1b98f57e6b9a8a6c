/*
 * doci_gb300.h -- C ABI of libdoci_gb300.so, the GB300 (sm_103a) DOCI engine.
 *
 * Part 1 exports the reference's own entry points (klgunst/doci) with the same
 * names, signatures and semantics, so that its C host code (executable.c,
 * davidson.c, CG.c) links against this library unchanged:
 *   - the Hamiltonian / matvec plug-in of include/doci.h,
 *   - the solver dispatch of include/wrapper_solvers.h,
 *   - the solvers of include/davidson.h and include/CG.h,
 *   - the FCIDUMP reader of include/read_fcidump.h.
 * Like the reference they print the reference's messages and exit on fatal
 * input errors.
 *
 * Part 2 is the status-returning API: device Hamiltonian handles, sigma on
 * device or host buffers, the device-resident solvers (FP64 and mixed
 * FP32/FP64), batched solves and the request server.  Every call returns a
 * doci_status; none exits.  Streams are passed as void* (a cudaStream_t;
 * NULL is CUDA's default stream, as in the CUDA API itself).  No CUDA or
 * torch types appear here.
 */
#ifndef DOCI_GB300_H
#define DOCI_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ======================================================================== */
/* Part 1: reference-compatible drop-in                                      */
/* ======================================================================== */

/* include/doci.h:14, src/doci.c:69-134.  Reads the FCIDUMP, checks
 * N_alpha == N_beta and L <= 32, builds the device Hamiltonian (addressing
 * tables, K_ia, diagonal) and returns it through *dat.  Prints the
 * reference's banner (doci.c:122-131). */
void fill_doci_data(char *dumpfil, void **dat);

/* include/doci.h:12, src/doci.c:136-140.  Borrowed host pointer to the D
 * diagonal elements (owned by dat). */
double *doci_get_diagonal(void *dat);

/* include/doci.h:16, src/doci.c:142-146 */
int doci_get_basis_size(void *dat);

/* include/doci.h:18, src/doci.c:148-159.  Frees everything, sets *dat = NULL. */
void doci_cleanup_data(void **dat);

/* include/doci.h:31, src/doci.c:164-238.  result = H vec for host arrays of D
 * doubles (they must not alias); result is overwritten.  FP64 on the GPU,
 * host<->device copies inside the call. */
void doci_matvec(double *vec, double *result, void *dat);

/* include/wrapper_solvers.h:36-38, src/wrapper_solvers.c:10-24.
 * solver "D" (Davidson), "CG", "CGP" (CG, diagonal preconditioner); M must be
 * NULL.  When matvec == doci_matvec and dat came from fill_doci_data the whole
 * solve stays on the device; any other matvec is called on host buffers once
 * per iteration while the vector layer runs on the device.  Returns -1 for an
 * unknown solver, else the solver's return value. */
int sparse_eigensolve(double *vec, int dims, double *energy,
                      void (*matvec)(double *, double *, void *), double *diagonal,
                      double *M, double tol, int max_its, char solver[],
                      int davidson_keep, int davidson_max_vec, void *dat);

/* include/davidson.h:25-27, src/davidson.c:33-128.  Returns its >= max_its. */
int davidson(double *result, double *energy, int max_vectors, int keep_deflate,
             double davidson_tol, void (*matvec)(double *, double *, void *),
             double *diagonal, int basis_size, int max_its, void *vdat);

/* include/CG.h:4-5, src/CG.c:13-164.  Returns its <= max_its (as the
 * reference, this is 1 even when MAX_ITS was reached). */
int ray_q(void (*matvec)(double *, double *, void *), double *M, double *vec, int size,
          double *energy, double cg_tol, int max_its, double *precond, void *vdat);

/* include/read_fcidump.h:4, src/read_fcidump.c:18-82.  Allocates one_p_int
 * (L*L) and two_p_int (L^4) with malloc; the caller frees them. */
void read_fcidump(char *filename, unsigned int *NORB, unsigned int *NALPHA,
                  unsigned int *NBETA, double *core_energy, double **one_p_int,
                  double **two_p_int);

/* ======================================================================== */
/* Part 2: status-returning GB300 API                                        */
/* ======================================================================== */

typedef enum doci_status {
  DOCI_OK = 0,
  DOCI_ERR_OPEN = 1,              /* FCIDUMP cannot be opened (read_fcidump.c:27-30) */
  DOCI_ERR_FORMAT = 2,            /* malformed header or integral line (:33-42, :63-67) */
  DOCI_ERR_NALPHA_NBETA = 3,      /* N_alpha != N_beta (doci.c:76-82) */
  DOCI_ERR_TOO_MANY_ORBITALS = 4, /* L > 32 (doci.c:84-89) */
  DOCI_ERR_INVALID = 5,           /* bad argument */
  DOCI_ERR_CUDA = 6,              /* a CUDA call failed */
  DOCI_ERR_OUT_OF_MEMORY = 7,     /* device or host allocation failed */
  DOCI_ERR_NO_DEVICE = 8,         /* no CUDA device */
  DOCI_ERR_ADMISSION = 9,         /* request larger than the server's HBM budget */
  DOCI_ERR_NOT_FOUND = 10,        /* unknown ticket */
  DOCI_ERR_PENDING = 11,          /* ticket not finished yet */
  DOCI_ERR_DEVICE_TIMEOUT = 12,   /* a bounded device wait ran out */
  DOCI_ERR_UNKNOWN_SOLVER = 13,
  DOCI_ERR_SCRATCH_LIMIT = 14     /* request exceeds the fixed scratch of doci_multidot_noalloc */
} doci_status;

typedef enum doci_precision {
  DOCI_FP64 = 0, /* FP64 storage and arithmetic */
  DOCI_FP32 = 1  /* FP32 storage, FP32 sigma with FP32 accumulation */
} doci_precision;

/* Opaque device Hamiltonian: integrals, addressing tables and diagonal,
 * resident on one GPU. */
typedef struct doci_ham doci_ham;

const char *doci_status_string(int status);

/* Build from an FCIDUMP file (same parser and integral transform as the
 * reference: read_fcidump.c:18-82, doci.c:630-665). */
int doci_ham_from_fcidump(const char *path, doci_ham **out);

/* Build from an FCIDUMP file read by the relaxed reader (no counterpart in
 * the reference, whose reader wants the header on one line in a fixed order
 * and propagates the 8-fold symmetry only from canonically ordered entries):
 * the &FCI ... &END (or /) namelist over any number of lines, keys in any
 * order and case, other keys (ORBSYM, ISYM, UHF, ...) ignored, MS2 optional
 * (0), Fortran D exponents, blank lines; every integral entry is stored at
 * its canonical slot whatever its index order, so the transform sees it.
 * Two entries naming the same integral with different values are a format
 * error.  On canonically ordered files it gives the reference's integrals. */
int doci_ham_from_fcidump_relaxed(const char *path, doci_ham **out);

/* Host-only: the raw integrals of an FCIDUMP (before the transform, layout of
 * doci_ham_from_integrals) by the reference's reader (relaxed = 0) or the
 * relaxed one (1).  one/two may be NULL (dimensions only); else they hold
 * L*L and L^4 doubles.  *bad_line gets the offending line of a format error. */
int doci_fcidump_integrals(const char *path, int relaxed, int *L, int *n_alpha, int *n_beta, double *core,
                           double *one, double *two, int *bad_line);

/* Build from integrals laid out as read_fcidump returns them (before the
 * transform): one[L*L], two[L^4] with two[i + j L + k L^2 + l L^3] = (ij|kl),
 * 0-based, canonical entries at least (the transform mirrors them). */
int doci_ham_from_integrals(int L, int n_pairs, double core, const double *one,
                            const double *two, doci_ham **out);

void doci_ham_destroy(doci_ham *ham);

/* L, N (pairs), D = C(L, N) */
int doci_ham_dims(const doci_ham *ham, int *L, int *n_pairs, int64_t *dim);

/* Copy the FP64 diagonal (doci.c:550-628, bit-identical summation order) to
 * host memory out[D]. */
int doci_ham_diagonal(const doci_ham *ham, double *out);

/* Device pointer to the FP64 diagonal (borrowed). */
const double *doci_ham_diagonal_device(const doci_ham *ham);

/* sigma = H x on device buffers of D elements (double for DOCI_FP64, float
 * for DOCI_FP32).  y is overwritten; x and y must not alias.  Asynchronous on
 * stream (NULL = the default stream). */
int doci_sigma(doci_ham *ham, const void *d_x, void *d_y, int precision, void *stream);

/* Block sigma Y_v = H X_v for v < nv on device buffers: X and Y column-major
 * with leading dimensions ldx, ldy >= D (elements).  The neighbour ranks and
 * hop weights of each determinant are computed once per launch for up to
 * four vectors (larger nv runs in groups of four), so a block of vectors
 * costs much less than nv doci_sigma calls.  Results agree with doci_sigma to
 * rounding (identical when both use the same kernel).  No counterpart in the
 * reference, whose matvec (doci.c:164-238) takes one vector; used by the
 * block Davidson of doci_solve_roots.  Asynchronous on stream (NULL = the
 * default stream). */
int doci_sigma_block(doci_ham *ham, const void *d_X, int64_t ldx, void *d_Y, int64_t ldy, int nv, int precision,
                     void *stream);

/* Sigma kernel selection for a handle: 0 automatic (default: with a row
 * tiling that gives every SM work, kind 6 for FP32 and kind 9 for FP64; else
 * with a row tiling kind 3 for FP32 and kind 4 for FP64; else kind 1),
 * 1 the per-determinant gather kernel, 3 the row pass doing all hops, 4 the
 * phase-ordered row pass (cross hops staged one source row at a time), 6 the
 * (N-1)-pair form on the warp-level tensor-core path (FP32 only: gather the
 * neighbours of every (N-1)-pair set, multiply by K, scatter with atomic
 * adds), 8 the (N-1)-pair form on the 5th-generation tensor cores (FP32
 * only: the own row of a set's row part staged in shared memory, the other
 * rows streamed by TMA, the product in TMEM, each own row written once;
 * needs a 16-byte aligned x, else kind 6 runs), 9 the (N-1)-pair form in
 * float-float arithmetic (FP64 only: FP64 accuracy from pairs of FP32
 * values on the FP32 units, x converted once per call into stream-ordered
 * scratch of D x 8 bytes, FP64 atomic adds into sigma; the phase-ordered row
 * pass in the same arithmetic where the pair tiling does not fit; FP32
 * requests for it use the automatic choice).  Kinds 6, 8 and 9 reduce into
 * sigma with atomic adds, so their last bits vary between runs; FP64
 * requests for them use the automatic choice.  3-9 fall back to 1 when the
 * handle has no row tiling.  Other values: DOCI_ERR_INVALID.  A device wait
 * of kind 8 that runs out (it never should) is reported as
 * DOCI_ERR_DEVICE_TIMEOUT by the handle's next synchronous call
 * (doci_sigma_host, doci_solve).  For tests and tuning. */
int doci_ham_set_sigma_kernel(doci_ham *ham, int kind);

/* Autotuning: time the sigma paths that fit this handle's shape and keep
 * the fastest for every handle of the same (device, L, N, precision) in the
 * process (used when the handle's kind is 0, automatic).  nvec = 1 tunes the
 * single sigma (doci_sigma, doci_solve; *choice = the kind picked, with the
 * pair form allowed) and the pair-free path of the block solves; nvec = 2..4
 * tunes the block sigma of nvec vectors (doci_sigma_block, doci_solve_roots
 * with that many roots; *choice = 1 row pass in groups, 2 gather, 3 one
 * vector at a time).  Synchronous; a few sigma calls per candidate.  The
 * choices change which kernels run, so results computed before and after a
 * tuning may differ in their last bits; tune before a batch whose results
 * are compared to single solves.  No counterpart in the reference. */
int doci_ham_autotune(doci_ham *ham, int precision, int nvec, int *choice);

/* The path doci_sigma takes for this handle and precision: *kind as in
 * doci_ham_set_sigma_kernel (1, 3, 4, 6, 8 or 9; the automatic choice resolved) and
 * *launches, the number of kernel launches of one call.  Host-only query. */
int doci_sigma_plan(const doci_ham *ham, int precision, int *kind, int *launches);

/* Same on host buffers; copies in and out inside the call, synchronous.  On
 * the pair forms (kinds 6 and 9) x is uploaded, and a pinned (page-locked) y
 * downloaded, in pieces on the handle's own copy stream, overlapped with the
 * sigma (whose unit groups alternate between the handle's stream and a
 * second stream of its own).  The staging buffers and these streams belong
 * to the handle: calls on one handle from several host threads must be
 * serialised by the caller. */
int doci_sigma_host(doci_ham *ham, const void *x, void *y, int precision);

/* Lexical addressing on the device: bitstrings of determinants
 * [first, first+count) (bit o = orbital o, order of doci.c:472-548), and the
 * inverse map from bitstrings to ranks. */
int doci_bitstrings(doci_ham *ham, int64_t first, int64_t count, uint32_t *d_bits, void *stream);
int doci_ranks(doci_ham *ham, const uint32_t *d_bits, int64_t count, int64_t *d_ranks, void *stream);

/* Projections out[i] = V_i . w for i < m (m <= 32) on device buffers: V is
 * column-major with leading dimension ld >= n (element type double for
 * DOCI_FP64, float for DOCI_FP32), w has n elements, out is m doubles on the
 * device.  Products are accumulated in FP64 in a fixed order (per-block
 * partial sums, then one block adding them), so repeated calls give identical
 * results.  This is the subspace-column / Gram-Schmidt reduction of the
 * Davidson vector layer (davidson.c:139-143, :178-193: m ddot_ calls in the
 * reference), for callers that run their own solver around doci_sigma.
 * Allocates its partial-sum scratch on `stream` (stream-ordered). */
int doci_multidot(const void *d_V, int64_t ld, int m, const void *d_w, int64_t n, int precision, double *d_out,
                  void *stream);

/* doci_multidot without any device allocation.  No counterpart in the
 * reference: it serves callers that cannot let a library allocate GPU
 * memory -- processes that keep the device's memory in their own
 * pre-reserved pool (a serving loop holding many resident Davidson states,
 * a framework's caching allocator), where an extra cudaMalloc can fail or
 * fragment the pool, and latency-critical loops that cannot afford the
 * synchronisation an allocation or free may cause.  Same arguments and
 * results as doci_multidot; the per-block partial sums live in a fixed
 * 256 KiB array in the library's device image, held on every GPU that loads
 * the library until the process exits.  Limit: m <= 32 (larger m returns
 * DOCI_ERR_SCRATCH_LIMIT).  The first call on a device looks up that
 * array's device address (cudaGetSymbolAddress), so make it before any
 * stream capture.  All calls share the array: calls that overlap on the GPU
 * (other streams, other host threads) race and must be serialised by the
 * caller.  The looked-up address is kept for the life of the process: after
 * cudaDeviceReset on a device (which unloads the library's device image
 * there, as it invalidates every handle) do not call it on that device
 * again.  Allocates nothing, frees nothing. */
int doci_multidot_noalloc(const void *d_V, int64_t ld, int m, const void *d_w, int64_t n, int precision,
                          double *d_out, void *stream);

typedef enum doci_solver_kind { DOCI_SOLVER_D = 0, DOCI_SOLVER_CG = 1, DOCI_SOLVER_CGP = 2 } doci_solver_kind;

typedef enum doci_solve_mode {
  DOCI_MODE_FP64 = 0,  /* FP64 sigma and FP64 basis throughout */
  DOCI_MODE_MIXED = 1  /* FP32 phase: FP32 sigma and FP32 basis on the shifted
                          operator H - (lowest diagonal element), FP32 vector
                          arithmetic with FP64 accumulation of the reductions,
                          FP64 subspace eigenproblem; it ends at mixed_tol or
                          when the residual stops improving.  Then FP64
                          Davidson steps from that vector to tol. */
} doci_solve_mode;

typedef struct doci_solve_opts {
  int solver;            /* doci_solver_kind (input key SOLVER) */
  int max_its;           /* MAX_ITS, default 200 (options.h:7) */
  double tol;            /* TOL, default 1e-8 (options.h:6) */
  int davidson_keep;     /* DAVIDSON_KEEP, default 2 (options.h:5) */
  int davidson_max_vec;  /* DAVIDSON_MAX_VEC, default 30 (options.h:4) */
  int hf_init;           /* HF_INIT, default 1; 0 = seeded random start */
  int mode;              /* doci_solve_mode (Davidson only) */
  double mixed_tol;      /* residual at which the FP32 phase hands over (mixed) */
  int print_level;       /* 0 silent, 1 reference summary lines, 2 per-iteration table */
  uint64_t seed;         /* random start seed (hf_init == 0) */
  int fp32_corrections;  /* mixed mode, FP64 phase: 1 (default) = the sigmas of the correction
                            vectors in FP32 on the shifted operator, each run anchored by an
                            FP64 sigma of its start vector and closed by an FP64 sigma of the
                            result (its Rayleigh quotient and true residual are reported);
                            0 = every FP64-phase sigma in FP64 */
} doci_solve_opts;

typedef struct doci_solve_result {
  double energy;         /* lowest eigenvalue */
  double residual;       /* final ||H x - E x||_2 (Davidson) or ||g||^2 (CG) */
  int iterations;        /* total solver iterations (one sigma each) */
  int iterations_fp32;   /* of which in the FP32 phase (mixed mode) */
  int converged;         /* residual criterion met within max_its */
  int status_code;       /* reference-style return code of the solver */
  double energy_fp32;    /* energy at the end of the FP32 phase (mixed) */
  double seconds;        /* wall time of the solve */
  double sigma_seconds;  /* device time spent in sigma */
} doci_solve_result;

void doci_solve_opts_default(doci_solve_opts *opts);

/* Device-resident solve.  vec (host, D doubles) may be NULL; when given it is
 * the start vector if opts->hf_init < 0, and receives the eigenvector. */
int doci_solve(doci_ham *ham, const doci_solve_opts *opts, double *vec,
               doci_solve_result *result);

/* doci_solve that also records one entry per Davidson iteration into trace
 * (4 doubles each: phase 0 = FP32, 1 = FP64; residual norm; energy; seconds
 * since the call started), at most trace_len entries; *trace_count receives
 * the number written.  Used to time convergence. */
int doci_solve_trace(doci_ham *ham, const doci_solve_opts *opts, double *vec, doci_solve_result *result,
                     double *trace, int trace_len, int *trace_count);

/* Bytes of device memory a solve of ham with opts needs (admission). */
int64_t doci_solve_footprint(int L, int n_pairs, const doci_solve_opts *opts, int nroots);

/* ------------------------------------------------------------------------ */
/* Several roots, batched solves, request server.  No counterpart in the     */
/* reference (single Hamiltonian, lowest root: davidson.c:90, :117).          */
/* ------------------------------------------------------------------------ */

typedef struct doci_batch_opts {
  int nroots;          /* lowest eigenpairs per Hamiltonian, 1..8 (default 1) */
  int max_vec;         /* block-Davidson basis size, >= 2 nroots, <= 32 (16) */
  int max_its;         /* iteration limit (200) */
  double tol;          /* residual-norm tolerance of every root (1e-6) */
  int mode;            /* DOCI_MODE_MIXED (default) or DOCI_MODE_FP64 */
  double mixed_tol;    /* residual at which the FP32 phase hands over (1e-4) */
  int workers;         /* server: solves in flight at once, one CUDA stream each (8) */
  int64_t hbm_budget;  /* device bytes the solves in flight may hold; 0 = 85% of free */
  int keep;            /* basis vectors kept at a thick restart, nroots..max_vec - nroots;
                          0 = automatic (max(2 nroots, max_vec / 4)) */
} doci_batch_opts;

typedef struct doci_root_result {
  double energy[8];       /* lowest eigenvalues, ascending */
  double residual[8];     /* final FP64 residual norms */
  double energy_fp32[8];  /* energies at the end of the FP32 phase (mixed mode) */
  int nroots, iterations, iterations_fp32, sigmas, converged;
  int status;             /* doci_status of this solve */
  double queued_s, start_s, end_s;  /* server clock: submitted, admitted, finished */
} doci_root_result;

void doci_batch_opts_default(doci_batch_opts *opts);

/* Device bytes one solve of an (L, n_pairs) Hamiltonian holds (admission). */
int64_t doci_roots_footprint(int L, int n_pairs, const doci_batch_opts *opts);

/* Block-Davidson solve for the opts->nroots lowest eigenpairs (start vectors:
 * unit vectors on the lowest diagonal elements) on the batch engine with a
 * batch of one, so that the result is bit-identical to the same problem's in
 * doci_batch_solve or the server; vecs (host, D x nroots, column-major) may
 * be NULL. */
int doci_solve_roots(doci_ham *ham, const doci_batch_opts *opts, doci_root_result *result, double *vecs);

/* Autotuning of the batch engine's sigma for this handle's shape: time its
 * batched gather with tiles of 1, 2 or 4 determinants per thread of a
 * 256-thread tile, and the single-problem kernels (doci_sigma's path, one
 * call per vector), on nvec (1..8) vectors; keep the fastest for every
 * problem of the same (device, L, n_pairs) in the process.
 * *dets_per_thread (may be NULL) receives the tile, or 0 for the
 * single-problem kernels.  Untuned shapes use one determinant per thread
 * below 2^22 determinants and the single-problem kernels from there.  A tile
 * shape changes no result; the single-problem kernels reduce in another
 * order.  Synchronous.  No counterpart in the reference. */
int doci_engine_autotune(doci_ham *ham, int nvec, int *dets_per_thread);

/* Solve many Hamiltonians at once on the batch engine: every problem of a
 * group advances in lockstep, one device-resident, graph-captured block
 * Davidson iteration for the whole group (batched sigma over a shared space
 * of determinant tiles -- large problems take doci_sigma's kernels instead,
 * see doci_engine_autotune -- batched vector passes, one subspace
 * eigensolver per problem on the device); groups are formed in order so
 * that their solves fit opts->hbm_budget (0: 85% of the free memory).  A
 * result does not depend on the rest of the batch (bit for bit on the
 * batched path).  results[i] for hams[i] (start_s / end_s:
 * the group's run, seconds from the call). */
int doci_batch_solve(int n, doci_ham *const *hams, const doci_batch_opts *opts, doci_root_result *results);

/* Request server: submitted requests (integrals or an FCIDUMP path) are
 * admitted as workers and memory free up, built on the device and solved
 * concurrently, each on its own stream (continuous batching): one-root
 * requests by the single-root device Davidson (doci_solve's solver, mode and
 * mixed_tol from opts), several roots by the batch engine.  Tickets identify
 * requests. */
typedef struct doci_server doci_server;
int doci_server_create(const doci_batch_opts *opts, doci_server **out);
int doci_server_submit(doci_server *srv, int L, int n_pairs, double core, const double *one, const double *two,
                       int64_t *ticket);
int doci_server_submit_fcidump(doci_server *srv, const char *path, int64_t *ticket);
/* DOCI_ERR_PENDING while the request is queued or running */
int doci_server_poll(doci_server *srv, int64_t ticket, doci_root_result *out);
int doci_server_wait(doci_server *srv, int64_t ticket, doci_root_result *out);
int doci_server_stats(doci_server *srv, int64_t *submitted, int64_t *finished, int64_t *running,
                      int64_t *bytes_in_use);
/* Finishes the queued requests, then stops the workers. */
void doci_server_destroy(doci_server *srv);

#ifdef __cplusplus
}
#endif
#endif
