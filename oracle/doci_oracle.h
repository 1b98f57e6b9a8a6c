/*
 * doci_oracle.h -- CPU oracle for the DOCI sigma / Davidson / RQ-CG path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is a plain-C restatement of the
 * reference algorithm (klgunst/doci, src/doci.c, src/davidson.c, src/CG.c,
 * src/read_fcidump.c).  It is used by tests/, by __graft_entry__.smoke() and by
 * the cpu_baseline / --impl reference legs of bench.py, to check results and
 * to time the CPU path.  The product (doci_gb300/) never links, loads or calls
 * it.
 *
 * Parity pins: the oracle is checked (tests/test_oracle_pins.py) against
 *   - the published energies and Davidson traces in tests/coHF.out, lifHF.out;
 *   - the reference itself compiled from its sources into oracle/_ref/
 *     (addressing, diagonal, sigma, energies, iteration counts) when the
 *     reference sources are present;
 *   - an independent dense-H construction for small L.
 */
#ifndef DOCI_ORACLE_H
#define DOCI_ORACLE_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes returned instead of exit() (the reference exits) */
enum {
  ORC_OK = 0,
  ORC_ERR_OPEN = 1,       /* read_fcidump.c:27-30 */
  ORC_ERR_HEADER = 2,     /* read_fcidump.c:33-42 */
  ORC_ERR_LINE = 3,       /* read_fcidump.c:63-67 */
  ORC_ERR_NALPHA_NBETA = 4, /* doci.c:76-82 */
  ORC_ERR_TOO_MANY_ORBITALS = 5, /* doci.c:84-89 */
  ORC_ERR_ALLOC = 6,
  ORC_ERR_ARG = 7
};

typedef struct orc_ham {
  unsigned L, N;          /* orbitals, electron pairs */
  uint64_t D;             /* C(L, N) */
  double core;            /* core energy */
  double *one;            /* L*L, after transform_integrals (h') */
  double *two;            /* L^4, after transform_integrals */
  double *K;              /* L*L Viikk, K[i*L+a] = (ia|ia), K[i*L+i] = 0 */
  double *diag;           /* D diagonal (NULL when D was too large to keep) */
} orc_ham;

/* FCIDUMP reader, restating read_fcidump.c:18-82 (status instead of exit). */
int orc_read_fcidump(const char *path, unsigned *L, unsigned *Na, unsigned *Nb,
                     double *core, double **one, double **two, int *bad_line);

/* doci.c:630-665 */
void orc_transform_integrals(double *one, double *two, unsigned L);

/* doci.c:687-701: C(m, n) through a 64-bit product, then cast to 32 bits */
uint32_t orc_combination(unsigned n, unsigned m);
uint64_t orc_binom(unsigned n, unsigned k);

/* doci.c:472-548: all D bitstrings in lexical order */
void orc_bitstrings(unsigned N, unsigned L, uint32_t *out);
/* lexical rank of a bitstring (bit o = orbital o) */
uint64_t orc_rank(uint32_t bits, unsigned L, unsigned N);
uint32_t orc_unrank(uint64_t r, unsigned L, unsigned N);

/* doci.c:69-134 without the OpenMP partition: read, checks, transform, diag, K.
 * keep_diag = 0 skips the D-sized diagonal (large D samples). */
int orc_ham_create(const char *fcidump, int keep_diag, orc_ham **out);
void orc_ham_destroy(orc_ham *h);

/* doci.c:550-628 (same summation order) for determinants [first, first+count) */
void orc_diagonal_range(const orc_ham *h, uint64_t first, uint64_t count, double *out);

/* doci.c:164-238: diag part, lower-triangle enumeration with symmetric
 * scatter, per-thread partial vectors reduced at the end. nthreads <= 0 = all. */
void orc_matvec(const orc_ham *h, const double *x, double *y, int nthreads);

/* race-free gather form (doci.c:314-376, the commented doci_full_matvec) over
 * determinant chunks; used as the CPU baseline sample.  chunk_first/chunk_len
 * give nchunks ranges; y receives sigma for those rows only (packed). */
void orc_matvec_gather_rows(const orc_ham *h, const double *x, const double *diag_rows,
                            const uint64_t *chunk_first, const uint64_t *chunk_len,
                            int nchunks, double *y_rows, int nthreads);

/* Symmetric eigen-decomposition by cyclic Jacobi, ascending eigenvalues.
 * A is n x n column-major with leading dimension lda (upper triangle used),
 * eigenvectors returned column-major in V (ld = lda).  Replaces dsyev_. */
void orc_jacobi_eig(int n, const double *A, int lda, double *w, double *V);

/* davidson.c:33-128 (single root); trace (optional) receives per-iteration
 * residual and energy (2 doubles per iteration, up to max_its entries). */
int orc_davidson(const orc_ham *h, double *vec, double *energy, int max_vectors,
                 int keep_deflate, double tol, int max_its, int *its_out,
                 double *trace);

/* CG.c:13-164; precond != 0 uses the diagonal (CGP). */
int orc_ray_q(const orc_ham *h, double *vec, double *energy, double tol,
              int max_its, int precond, int *its_out, double *trace);

/* executable.c:270-299 HF_INIT=1: index of the lowest diagonal element */
uint64_t orc_hf_index(const orc_ham *h);

#ifdef __cplusplus
}
#endif
#endif
