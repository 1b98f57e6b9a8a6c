/*
 * doci_oracle.c -- CPU oracle (TEST INFRASTRUCTURE ONLY; see doci_oracle.h).
 *
 * A plain-C restatement of the reference's algorithm for the DOCI sigma
 * (matvec) path and the two solvers that call it.  Each function names the
 * reference lines it follows (paths relative to the klgunst/doci project).
 * Written independently: LAPACK's dsyev_/dsygv_ are replaced by a cyclic
 * Jacobi solver and a closed-form 2x2 generalised solver, BLAS by loops.
 */
#include "doci_oracle.h"

#include <ctype.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------------ */
/* FCIDUMP reader: read_fcidump.c:18-82                                     */
/* ------------------------------------------------------------------------ */

/* read_fcidump.c:88-110: equal iff the non-blank characters of line equal
 * the (blank-free) literal */
static int line_equals_ignoring_blanks(const char *line, const char *lit) {
  const unsigned char *p = (const unsigned char *)line;
  const unsigned char *q = (const unsigned char *)lit;
  for (;;) {
    while (*p && isspace(*p)) p++;
    if (!*p) return *q == 0;
    if (*q != *p) return 0;
    p++;
    q++;
  }
}

int orc_read_fcidump(const char *path, unsigned *L, unsigned *Na, unsigned *Nb,
                     double *core, double **one, double **two, int *bad_line) {
  char buf[255];
  int nelec = 0, ms2 = 0, line = 1;
  FILE *fp = fopen(path, "r");
  *one = *two = NULL;
  if (bad_line) *bad_line = 0;
  if (!fp) return ORC_ERR_OPEN;
  if (!fgets(buf, sizeof buf, fp) ||
      sscanf(buf, " &FCI NORB= %u , NELEC= %d , MS2= %d , ", L, &nelec, &ms2) != 3) {
    fclose(fp);
    if (bad_line) *bad_line = 1;
    return ORC_ERR_HEADER;
  }
  *Na = (unsigned)((nelec + ms2) / 2);
  *Nb = (unsigned)((nelec - ms2) / 2);
  *core = 0.0;
  if (*L == 0 || *L > 64) { fclose(fp); return ORC_ERR_HEADER; }
  const size_t n = *L, n2 = n * n, n4 = n2 * n2;
  *one = (double *)calloc(n2, sizeof(double));
  *two = (double *)calloc(n4, sizeof(double));
  if (!*one || !*two) { fclose(fp); free(*one); free(*two); *one = *two = NULL; return ORC_ERR_ALLOC; }

  /* skip the namelist (ORBSYM, ISYM, ...) up to &END, /END or / (:53-58) */
  while (fgets(buf, sizeof buf, fp)) {
    line++;
    if (line_equals_ignoring_blanks(buf, "&END") || line_equals_ignoring_blanks(buf, "/END") ||
        line_equals_ignoring_blanks(buf, "/"))
      break;
  }
  /* integral lines "value i j k l", chemical notation (:60-80) */
  while (fgets(buf, sizeof buf, fp)) {
    double v;
    int i, j, k, l;
    line++;
    if (sscanf(buf, " %lf %d %d %d %d ", &v, &i, &j, &k, &l) != 5) {
      fclose(fp);
      if (bad_line) *bad_line = line;
      free(*one); free(*two); *one = *two = NULL;
      return ORC_ERR_LINE;
    }
    double *slot;
    if (k != 0) {
      /* the reference indexes without checks; out-of-range is an error here */
      if (i < 1 || j < 1 || k < 1 || l < 1 || i > (int)n || j > (int)n || k > (int)n || l > (int)n) {
        fclose(fp);
        if (bad_line) *bad_line = line;
        free(*one); free(*two); *one = *two = NULL;
        return ORC_ERR_LINE;
      }
      slot = *two + (size_t)(l - 1) * n2 * n + (size_t)(k - 1) * n2 + (size_t)(j - 1) * n + (i - 1);
    } else if (i != 0) {
      if (i < 1 || j < 1 || i > (int)n || j > (int)n) {
        fclose(fp);
        if (bad_line) *bad_line = line;
        free(*one); free(*two); *one = *two = NULL;
        return ORC_ERR_LINE;
      }
      slot = *one + (size_t)(j - 1) * n + (i - 1);
    } else {
      slot = core;
    }
    if (fabs(*slot) >= 1e-14)
      fprintf(stderr, "Doubly inputted value at line %d, hope you don't mind\n", line);
    *slot = v;
  }
  fclose(fp);
  return ORC_OK;
}

/* ------------------------------------------------------------------------ */
/* doci.c:630-665: mirror h and the 8-fold two-body symmetry (propagating   */
/* only from the canonical loop domain i>=j, i>=k, k>=l), then              */
/* h'_kl = h_kl - 1/2 sum_j (kj|jl).                                        */
/* ------------------------------------------------------------------------ */
void orc_transform_integrals(double *one, double *two, unsigned L) {
  const size_t n = L, n2 = n * n, n3 = n2 * n;
  for (size_t i = 0; i < n; ++i)
    for (size_t j = 0; j <= i; ++j) one[i * n + j] = one[j * n + i];
  for (size_t i = 0; i < n; ++i)
    for (size_t j = 0; j <= i; ++j)
      for (size_t k = 0; k <= i; ++k)
        for (size_t l = 0; l <= k; ++l) {
          const double v = two[i + n * j + n2 * k + n3 * l];
          if (v == 0) continue;
          two[k + n * l + n2 * i + n3 * j] = v;
          two[j + n * i + n2 * l + n3 * k] = v;
          two[l + n * k + n2 * j + n3 * i] = v;
          two[j + n * i + n2 * k + n3 * l] = v;
          two[l + n * k + n2 * i + n3 * j] = v;
          two[i + n * j + n2 * l + n3 * k] = v;
          two[k + n * l + n2 * j + n3 * i] = v;
        }
  for (size_t k = 0; k < n; ++k)
    for (size_t l = 0; l < n; ++l) {
      double s = 0;
      for (size_t j = 0; j < n; ++j) s += two[k + j * n + j * n2 + l * n3];
      one[k + l * n] -= 0.5 * s;
    }
}

/* ------------------------------------------------------------------------ */
/* Addressing                                                               */
/* ------------------------------------------------------------------------ */
uint64_t orc_binom(unsigned n, unsigned k) {
  if (k > n) return 0;
  uint64_t r = 1;
  for (unsigned d = 1; d <= k; ++d) r = r * (n - k + d) / d;
  return r;
}

/* doci.c:687-701 */
uint32_t orc_combination(unsigned n, unsigned m) {
  if (n > m) return 0;
  unsigned long long r = 1;
  for (unsigned d = 1; d <= n; ++d) { r *= m--; r /= d; }
  return (uint32_t)r;
}

/* doci.c:472-548: lexical order of the sorted occupation list, the last pair
 * advanced first; bit o of the string = orbital o. */
void orc_bitstrings(unsigned N, unsigned L, uint32_t *out) {
  int occ[65];
  const uint64_t D = orc_binom(L, N);
  for (unsigned e = 0; e < N; ++e) occ[e] = (int)e;
  occ[N] = (int)L;
  for (uint64_t r = 0; r < D; ++r) {
    uint32_t b = 0;
    for (unsigned e = 0; e < N; ++e) b |= 1u << occ[e];
    out[r] = b;
    int e = (int)N - 1;
    while (e >= 0 && occ[e] + 1 == occ[e + 1]) --e;
    if (e < 0) break;
    occ[e]++;
    for (unsigned f = (unsigned)e + 1; f < N; ++f) occ[f] = occ[f - 1] + 1;
  }
}

/* rank = number of N-subsets that precede the sorted occupation list
 * lexicographically = D - 1 - sum_e C(L-1-c_e, N-e). */
uint64_t orc_rank(uint32_t bits, unsigned L, unsigned N) {
  uint64_t s = 0;
  unsigned e = 0;
  for (unsigned o = 0; o < L; ++o)
    if (bits >> o & 1u) { s += orc_binom(L - 1 - o, N - e); e++; }
  return orc_binom(L, N) - 1 - s;
}

uint32_t orc_unrank(uint64_t r, unsigned L, unsigned N) {
  uint64_t R = orc_binom(L, N) - 1 - r;
  uint32_t bits = 0;
  unsigned o = 0;
  for (unsigned e = 0; e < N; ++e) {
    /* smallest orbital o with C(L-1-o, N-e) <= R */
    while (orc_binom(L - 1 - o, N - e) > R) o++;
    R -= orc_binom(L - 1 - o, N - e);
    bits |= 1u << o;
    o++;
  }
  return bits;
}

static void occ_of(uint32_t bits, unsigned L, int *occ) {
  int e = 0;
  for (unsigned o = 0; o < L; ++o)
    if (bits >> o & 1u) occ[e++] = (int)o;
  occ[e] = (int)L;
}

/* ------------------------------------------------------------------------ */
/* doci.c:550-628: diagonal, same summation order (occupied pairs from the  */
/* last one down, orbitals ascending inside).                               */
/* ------------------------------------------------------------------------ */
static double diag_one(const orc_ham *h, const int *occ) {
  const size_t L = h->L, L2 = L * L, L3 = L2 * L;
  double t = h->core;
  for (int i = (int)h->N - 1; i >= 0; --i) {
    const size_t o1 = (size_t)occ[i];
    size_t idx_j = o1 * (L + 1), idx_k = o1 * (1 + L3);
    unsigned c = 0;
    t += 2 * h->one[o1 * (L + 1)];
    for (size_t o2 = 0; o2 < L; ++o2) {
      const int is_occ = occ[c] == (int)o2;
      c += (unsigned)is_occ;
      t += 2 * is_occ * h->two[idx_j];        /* 2 (ii|jj), j occupied */
      t += (1 - is_occ) * h->two[idx_k];      /* (ij|ji),  j virtual  */
      idx_j += L2 + L3;
      idx_k += L + L2;
    }
  }
  return t;
}

void orc_diagonal_range(const orc_ham *h, uint64_t first, uint64_t count, double *out) {
  /* large ranges are split over the host threads (a call from inside a
   * parallel region runs on its own thread) */
#pragma omp parallel for schedule(static) if (count > 65536)
  for (long long r = 0; r < (long long)count; ++r) {
    int occ[65];
    occ_of(orc_unrank(first + (uint64_t)r, h->L, h->N), h->L, occ);
    out[r] = diag_one(h, occ);
  }
}

/* doci.c:69-134 (setup) + doci.c:667-683 (Viikk) */
int orc_ham_create(const char *fcidump, int keep_diag, orc_ham **out) {
  unsigned L, Na, Nb;
  double core, *one, *two;
  int bad;
  *out = NULL;
  int st = orc_read_fcidump(fcidump, &L, &Na, &Nb, &core, &one, &two, &bad);
  if (st) return st;
  if (Na != Nb) { free(one); free(two); return ORC_ERR_NALPHA_NBETA; }
  if (L > 32) { free(one); free(two); return ORC_ERR_TOO_MANY_ORBITALS; }
  orc_transform_integrals(one, two, L);
  orc_ham *h = (orc_ham *)calloc(1, sizeof *h);
  h->L = L; h->N = Na; h->core = core; h->one = one; h->two = two;
  h->D = orc_binom(L, Na);
  h->K = (double *)malloc(sizeof(double) * L * L);
  for (size_t i = 0; i < L; ++i)
    for (size_t k = 0; k < L; ++k)
      h->K[i * L + k] = (i == k) ? 0.0 : two[i + k * L + i * L * L + k * L * L * L];
  if (keep_diag) {
    h->diag = (double *)malloc(sizeof(double) * h->D);
    if (!h->diag) { orc_ham_destroy(h); return ORC_ERR_ALLOC; }
#pragma omp parallel for schedule(static)
    for (long long c = 0; c < (long long)((h->D + 4095) / 4096); ++c) {
      uint64_t f = (uint64_t)c * 4096, n = h->D - f < 4096 ? h->D - f : 4096;
      orc_diagonal_range(h, f, n, h->diag + f);
    }
  }
  *out = h;
  return ORC_OK;
}

void orc_ham_destroy(orc_ham *h) {
  if (!h) return;
  free(h->one); free(h->two); free(h->K); free(h->diag); free(h);
}

/* ------------------------------------------------------------------------ */
/* doci.c:164-238: y = diag*x (:191-193); for every determinant T, every    */
/* lower neighbour T' = T\i u a with a < i (rank(T') < rank(T)) adds         */
/* K_ia x[T'] to y[T] and K_ia x[T] to y[T'] (:216-222), into per-thread     */
/* partial vectors (:173, :181) reduced at the end (:229-235).  Thread t    */
/* owns determinants [t*D/T, (t+1)*D/T) (doci.c:108-120).                   */
/* ------------------------------------------------------------------------ */
void orc_matvec(const orc_ham *h, const double *x, double *y, int nthreads) {
  const unsigned L = h->L, N = h->N;
  const uint64_t D = h->D;
  int T = 1;
#ifdef _OPENMP
  T = nthreads > 0 ? nthreads : omp_get_max_threads();
#else
  (void)nthreads;
#endif
  double *part = T > 1 ? (double *)calloc((size_t)D * (size_t)(T - 1), sizeof(double)) : NULL;
#pragma omp parallel num_threads(T)
  {
    int t = 0;
#ifdef _OPENMP
    t = omp_get_thread_num();
#endif
#pragma omp for schedule(static)
    for (long long c = 0; c < (long long)D; ++c) y[c] = x[c] * h->diag[c];
    double *acc = t ? part + (size_t)D * (size_t)(t - 1) : y;
    const uint64_t lo = (uint64_t)t * D / (uint64_t)T, hi = (uint64_t)(t + 1) * D / (uint64_t)T;
    int occ[65];
    for (uint64_t c = lo; c < hi; ++c) {
      const uint32_t b = orc_unrank(c, L, N);
      occ_of(b, L, occ);
      for (unsigned e = 0; e < N; ++e) {
        const unsigned i = (unsigned)occ[e];
        for (unsigned a = 0; a < i; ++a) {
          if (b >> a & 1u) continue;
          const uint64_t c2 = orc_rank((b & ~(1u << i)) | (1u << a), L, N);
          const double v = h->K[i * L + a];
          acc[c] += v * x[c2];
          acc[c2] += v * x[c];
        }
      }
    }
#pragma omp barrier
#pragma omp for schedule(static)
    for (long long c = 0; c < (long long)D; ++c)
      for (int q = 0; q < T - 1; ++q) y[c] += part[(size_t)c + (size_t)q * D];
  }
  free(part);
}

/* ------------------------------------------------------------------------ */
/* Race-free gather form (doci.c:314-376, the commented doci_full_matvec):   */
/* sigma[T] = diag[T] x[T] + sum_{i in T, a not in T} K_ia x[T\i u a].       */
/* Neighbour ranks come from prefix sums over the occupied orbitals, O(1)   */
/* per neighbour, as the reference's incremental Y-walk (doci.c:851-978)    */
/* gives O(1) per neighbour.  Used only to time a bounded CPU sample.       */
/* ------------------------------------------------------------------------ */
static uint64_t B_[34][34];
static void binom_table(void) {
  if (B_[1][1]) return;
  for (int n = 0; n < 34; ++n)
    for (int k = 0; k < 34; ++k) B_[n][k] = orc_binom((unsigned)n, (unsigned)k);
}

static double gather_row(const orc_ham *h, uint64_t r, const double *x, double diag_r) {
  const unsigned L = h->L, N = h->N;
  const uint64_t D = h->D;
  /* mirrored picture: bit d <-> orbital L-1-d; colex rank R = D-1-r */
  const uint32_t b = orc_unrank(r, L, N);
  unsigned m[33], q[33], nm = 0, nq = 0;
  for (unsigned d = 0; d < L; ++d) {
    if (b >> (L - 1 - d) & 1u) m[nm++] = d; else q[nq++] = d;
  }
  uint64_t PW[34], PU[34], PV[34];
  PW[0] = PU[0] = PV[0] = 0;
  for (unsigned j = 0; j < N; ++j) {
    PW[j + 1] = PW[j] + B_[m[j]][j + 1];
    PU[j + 1] = PU[j] + B_[m[j]][j];
    PV[j + 1] = PV[j] + B_[m[j]][j + 2];
  }
  const uint64_t R = D - 1 - r;
  double acc = diag_r * x[r];
  for (unsigned k = 0; k < N; ++k) {
    const uint64_t c1 = PV[k] + R - PW[k + 1], c2 = PW[k] - PU[k + 1];
    const double *Krow = h->K + (size_t)(L - 1 - m[k]) * L;
    for (unsigned t = 0; t < nq; ++t) {
      const unsigned qq = q[t], bb = qq - t;
      uint64_t colex;
      if (qq < m[k]) colex = PW[bb] - PV[bb] + B_[qq][bb + 1] + c1;
      else colex = PU[bb] + R - PW[bb] + B_[qq][bb] + c2;
      acc += Krow[L - 1 - qq] * x[D - 1 - colex];
    }
  }
  return acc;
}

void orc_matvec_gather_rows(const orc_ham *h, const double *x, const double *diag_rows,
                            const uint64_t *chunk_first, const uint64_t *chunk_len,
                            int nchunks, double *y_rows, int nthreads) {
  binom_table();
  uint64_t *off = (uint64_t *)malloc(sizeof(uint64_t) * ((size_t)nchunks + 1));
  off[0] = 0;
  for (int c = 0; c < nchunks; ++c) off[c + 1] = off[c] + chunk_len[c];
  const long long total = (long long)off[nchunks];
  int T = 1;
#ifdef _OPENMP
  T = nthreads > 0 ? nthreads : omp_get_max_threads();
#else
  (void)nthreads;
#endif
#pragma omp parallel for num_threads(T) schedule(dynamic, 256)
  for (long long p = 0; p < total; ++p) {
    int c = 0;
    while (off[c + 1] <= (uint64_t)p) c++;
    const uint64_t r = chunk_first[c] + ((uint64_t)p - off[c]);
    y_rows[p] = gather_row(h, r, x, diag_rows[p]);
  }
  free(off);
}

/* ------------------------------------------------------------------------ */
/* Dense symmetric eigensolver (replaces dsyev_ in davidson.c:81, :88).      */
/* ------------------------------------------------------------------------ */
void orc_jacobi_eig(int n, const double *A, int lda, double *w, double *V) {
  double *a = (double *)malloc(sizeof(double) * n * n);
  double *v = (double *)malloc(sizeof(double) * n * n);
  for (int c = 0; c < n; ++c)
    for (int r = 0; r < n; ++r) {
      a[r + c * n] = r <= c ? A[r + c * lda] : A[c + r * lda];
      v[r + c * n] = r == c;
    }
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0, tot = 0;
    for (int c = 0; c < n; ++c)
      for (int r = 0; r < n; ++r) {
        tot += a[r + c * n] * a[r + c * n];
        if (r != c) off += a[r + c * n] * a[r + c * n];
      }
    if (off <= 1e-30 * tot || off == 0) break;
    for (int p = 0; p < n - 1; ++p)
      for (int q = p + 1; q < n; ++q) {
        const double apq = a[p + q * n];
        if (apq == 0) continue;
        const double app = a[p + p * n], aqq = a[q + q * n];
        const double theta = (aqq - app) / (2 * apq);
        const double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1));
        const double c = 1 / sqrt(t * t + 1), s = t * c;
        for (int k = 0; k < n; ++k) {
          const double akp = a[k + p * n], akq = a[k + q * n];
          a[k + p * n] = c * akp - s * akq;
          a[k + q * n] = s * akp + c * akq;
        }
        for (int k = 0; k < n; ++k) {
          const double apk = a[p + k * n], aqk = a[q + k * n];
          a[p + k * n] = c * apk - s * aqk;
          a[q + k * n] = s * apk + c * aqk;
        }
        for (int k = 0; k < n; ++k) {
          const double vkp = v[k + p * n], vkq = v[k + q * n];
          v[k + p * n] = c * vkp - s * vkq;
          v[k + q * n] = s * vkp + c * vkq;
        }
      }
  }
  /* ascending order (selection sort keeps it simple for n <= 64) */
  int *idx = (int *)malloc(sizeof(int) * n);
  for (int i = 0; i < n; ++i) idx[i] = i;
  for (int i = 0; i < n; ++i)
    for (int j = i + 1; j < n; ++j)
      if (a[idx[j] + idx[j] * n] < a[idx[i] + idx[i] * n]) { int t = idx[i]; idx[i] = idx[j]; idx[j] = t; }
  for (int i = 0; i < n; ++i) {
    w[i] = a[idx[i] + idx[i] * n];
    for (int r = 0; r < n; ++r) V[r + i * lda] = v[r + idx[i] * n];
  }
  free(idx); free(a); free(v);
}

/* ------------------------------------------------------------------------ */
/* Davidson: davidson.c:33-128 with new_search_vector (:133-176),           */
/* expand_submatrix (:178-193), calculate_residue (:195-212),               */
/* create_new_vec_t (:214-227) and deflate (:229-255).                      */
/* ------------------------------------------------------------------------ */
static double dot(const double *a, const double *b, uint64_t n) {
  double s = 0;
  for (uint64_t i = 0; i < n; ++i) s += a[i] * b[i];
  return s;
}

int orc_davidson(const orc_ham *h, double *result, double *energy, int maxv, int keep,
                 double tol, int max_its, int *its_out, double *trace) {
  const uint64_t D = h->D;
  int its = 0, m = 0;
  double res = tol * 10;
  double *S = (double *)calloc((size_t)maxv * maxv, sizeof(double));
  double *Y = (double *)calloc((size_t)maxv * maxv, sizeof(double));
  double *w = (double *)calloc((size_t)maxv, sizeof(double));
  double *V = (double *)malloc(sizeof(double) * D * (size_t)maxv);
  double *VA = (double *)malloc(sizeof(double) * D * (size_t)maxv);
  double *t = (double *)malloc(sizeof(double) * D);
  double *tmp = (double *)malloc(sizeof(double) * D * (size_t)keep);
  memcpy(t, result, sizeof(double) * D);
  *energy = 0;
  while (res > tol && its++ < max_its) {
    /* modified Gram-Schmidt of t against V_0..V_{m-1}, normalise (:133-176) */
    for (int i = 0; i < m; ++i) {
      const double a = -dot(V + (size_t)i * D, t, D);
      for (uint64_t j = 0; j < D; ++j) t[j] += a * V[(size_t)i * D + j];
    }
    const double inv = 1.0 / sqrt(dot(t, t, D));
    for (uint64_t j = 0; j < D; ++j) t[j] *= inv;
    memcpy(V + (size_t)m * D, t, sizeof(double) * D);
    orc_matvec(h, V + (size_t)m * D, VA + (size_t)m * D, 0);
    for (int i = 0; i <= m; ++i) S[(size_t)m * maxv + i] = dot(V + (size_t)i * D, VA + (size_t)m * D, D);
    m++;
    orc_jacobi_eig(m, S, maxv, w, Y);
    if (m == maxv) {
      /* deflate: V[:, :keep] = V Y[:, :keep], same for VA; rebuild S (:229-255) */
      double *blocks[2] = {V, VA};
      for (int b = 0; b < 2; ++b) {
        for (int c = 0; c < keep; ++c)
          for (uint64_t j = 0; j < D; ++j) {
            double s = 0;
            for (int k = 0; k < maxv; ++k) s += blocks[b][(size_t)k * D + j] * Y[k + (size_t)c * maxv];
            tmp[(size_t)c * D + j] = s;
          }
        memcpy(blocks[b], tmp, sizeof(double) * D * (size_t)keep);
      }
      for (int c = 0; c < keep; ++c)
        for (int i = 0; i <= c; ++i) S[(size_t)c * maxv + i] = dot(V + (size_t)i * D, VA + (size_t)c * D, D);
      m = keep;
      orc_jacobi_eig(m, S, maxv, w, Y);
    }
    /* residual with the lowest Ritz pair (:195-212) */
    const double theta = w[0];
    double n2 = 0;
    for (uint64_t j = 0; j < D; ++j) {
      double xv = 0, rv = 0;
      for (int k = 0; k < m; ++k) {
        xv += V[j + (size_t)k * D] * Y[k];
        rv += VA[j + (size_t)k * D] * Y[k];
      }
      rv -= theta * xv;
      result[j] = xv;
      t[j] = rv;
      n2 += rv * rv;
    }
    res = sqrt(n2);
    *energy = theta;
    if (trace && its <= max_its) { trace[2 * (its - 1)] = res; trace[2 * (its - 1) + 1] = theta; }
    /* diagonal preconditioner with |D - theta| and a 1e-12 cutoff (:214-227) */
    for (uint64_t j = 0; j < D; ++j) {
      const double d = fabs(h->diag[j] - theta);
      t[j] = d > 1e-12 ? t[j] / d : t[j] / 1e-12;
    }
  }
  *energy = w[0];
  if (its_out) *its_out = its;
  free(S); free(Y); free(w); free(V); free(VA); free(t); free(tmp);
  return its >= max_its;
}

/* ------------------------------------------------------------------------ */
/* Rayleigh-quotient CG: CG.c:13-164.  The 2x2 problem A v = l B v           */
/* (dsygv_, ITYPE=1, upper triangles) is solved through the Cholesky factor */
/* of B, as dsygv does, giving B-normalised eigenvectors.                   */
/* ------------------------------------------------------------------------ */
static int gen_eig_2x2(const double A[4], const double B[4], double *lam, double vec[2]) {
  /* dsygv_ (ITYPE=1, UPLO='U'): B = U^T U, C = U^-T A U^-1, dsyev_(C), v = U^-1 z.
   * For n = 2 dsyev_ reduces to LAPACK's dlaev2 (published netlib algorithm)
   * applied to (c11, c12, c22) inside dsteqr, which stores the eigenvector
   * (cs1, sn1) of the larger-magnitude eigenvalue rt1 in column 1 and
   * (-sn1, cs1) in column 2, then sorts ascending.  The sign of that
   * eigenvector matters: CG.c:106-113 updates x but keeps p, so a flipped
   * x changes the next search direction (CG.c:92-94). */
  const double b11 = B[0], b12 = B[2], b22 = B[3];
  if (!(b11 > 0)) return 1;
  const double u11 = sqrt(b11), u12 = b12 / u11, s = b22 - u12 * u12;
  if (!(s > 0)) return 2;
  const double u22 = sqrt(s);
  const double i11 = 1 / u11, i12 = -u12 / (u11 * u22), i22 = 1 / u22;
  const double a11 = A[0], a12 = A[2], a22 = A[3];
  const double c11 = i11 * i11 * a11;
  const double c12 = i11 * (a11 * i12 + a12 * i22);
  const double c22 = i12 * i12 * a11 + 2 * i12 * i22 * a12 + i22 * i22 * a22;
  /* dlaev2(c11, c12, c22) */
  const double sm = c11 + c22, df = c11 - c22, adf = fabs(df), tb = c12 + c12, ab = fabs(tb);
  const double acmx = fabs(c11) > fabs(c22) ? c11 : c22, acmn = fabs(c11) > fabs(c22) ? c22 : c11;
  double rt, rt1, rt2, cs, cs1, sn1;
  int sgn1, sgn2;
  if (adf > ab) rt = adf * sqrt(1 + (ab / adf) * (ab / adf));
  else if (adf < ab) rt = ab * sqrt(1 + (adf / ab) * (adf / ab));
  else rt = ab * sqrt(2.0);
  if (sm < 0) { rt1 = 0.5 * (sm - rt); sgn1 = -1; rt2 = (acmx / rt1) * acmn - (c12 / rt1) * c12; }
  else if (sm > 0) { rt1 = 0.5 * (sm + rt); sgn1 = 1; rt2 = (acmx / rt1) * acmn - (c12 / rt1) * c12; }
  else { rt1 = 0.5 * rt; rt2 = -0.5 * rt; sgn1 = 1; }
  if (df >= 0) { cs = df + rt; sgn2 = 1; } else { cs = df - rt; sgn2 = -1; }
  if (fabs(cs) > ab) { const double ct = -tb / cs; sn1 = 1 / sqrt(1 + ct * ct); cs1 = ct * sn1; }
  else if (ab == 0) { cs1 = 1; sn1 = 0; }
  else { const double tn = -cs / tb; cs1 = 1 / sqrt(1 + tn * tn); sn1 = tn * cs1; }
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

int orc_ray_q(const orc_ham *h, double *vec, double *energy, double tol, int max_its,
              int precond, int *its_out, double *trace) {
  const uint64_t D = h->D;
  double *x = (double *)malloc(sizeof(double) * D * 2), *p = x + D;
  double *Ax = (double *)malloc(sizeof(double) * D * 2), *Ap = Ax + D;
  double *g = (double *)malloc(sizeof(double) * D);
  double *pinv = (double *)malloc(sizeof(double) * D);
  if (precond)
    for (uint64_t j = 0; j < D; ++j) pinv[j] = fabs(h->diag[j]) > 1e-12 ? 1 / h->diag[j] : 1 / 1e-12;
  int its = 0;
  memcpy(x, vec, sizeof(double) * D);
  orc_matvec(h, x, Ax, 0);
  double rho = dot(Ax, x, D);
  for (uint64_t j = 0; j < D; ++j) g[j] = 2 * (Ax[j] - rho * x[j]);
  double normq = dot(g, g, D);
  if (precond) for (uint64_t j = 0; j < D; ++j) g[j] *= pinv[j];
  double ng = dot(g, g, D), ng_prev = ng;
  while (normq > tol && its < max_its) {
    if (its != 0) {
      const double beta = ng / ng_prev;
      for (uint64_t j = 0; j < D; ++j) p[j] = beta * p[j] - g[j];
    } else {
      for (uint64_t j = 0; j < D; ++j) p[j] = -g[j];
    }
    orc_matvec(h, p, Ap, 0);
    double A[4], B[4], lam, v[2];
    A[0] = dot(x, Ax, D); A[1] = dot(p, Ax, D); A[2] = dot(x, Ap, D); A[3] = dot(p, Ap, D);
    B[0] = dot(x, x, D); B[1] = dot(p, x, D); B[2] = dot(x, p, D); B[3] = dot(p, p, D);
    if (gen_eig_2x2(A, B, &lam, v)) break;
    for (uint64_t j = 0; j < D; ++j) {
      x[j] = v[0] * x[j] + v[1] * p[j];
      Ax[j] = v[0] * Ax[j] + v[1] * Ap[j];
    }
    rho = lam;
    for (uint64_t j = 0; j < D; ++j) g[j] = 2 * (Ax[j] - rho * x[j]);
    normq = dot(g, g, D);
    if (precond) for (uint64_t j = 0; j < D; ++j) g[j] *= pinv[j];
    ng_prev = ng;
    ng = dot(g, g, D);
    if (trace && its < max_its) { trace[2 * its] = ng; trace[2 * its + 1] = rho; }
    its++;
  }
  memcpy(vec, x, sizeof(double) * D);
  *energy = rho;
  if (its_out) *its_out = its;
  free(x); free(Ax); free(g); free(pinv);
  return its <= max_its;
}

/* executable.c:276-288 */
uint64_t orc_hf_index(const orc_ham *h) {
  uint64_t ind = 0;
  double low = h->diag[0] + 1;
  for (uint64_t j = 0; j < h->D; ++j)
    if (low > h->diag[j]) { low = h->diag[j]; ind = j; }
  return ind;
}
