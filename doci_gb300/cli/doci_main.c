/*
 * doci_main.c -- the `doci` command-line program on libdoci_gb300.
 *
 * Same command line, input-file keys, defaults and printed lines as the
 * reference executable (src/executable.c): `doci [-m MODE] INPUTFILE`, keys
 * FCIDUMP, SOLVER (D/CG/CGP), MAX_ITS, TOL, DAVIDSON_KEEP, DAVIDSON_MAX_VEC,
 * HF_INIT (executable.c:201-230, defaults options.h:4-7), the input echo
 * (:232-268), the initial guess (:270-299) and the result block (:76-81),
 * so existing scripts and logs diff cleanly.  The solve runs through the
 * reference-compatible entry points (fill_doci_data, sparse_eigensolve with
 * doci_matvec), which keep it on the GPU.
 *
 * Extra environment knobs (absent in the reference): DOCI_SEED fixes the
 * random start of HF_INIT=0 (the reference seeds with time(NULL));
 * DOCI_MIXED=1 runs the mixed FP32/FP64 Davidson through doci_solve.
 */
#include <argp.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/time.h>
#include <time.h>

#include "doci_gb300.h"

#define DAVIDSON_MAX_VECS 30
#define DAVIDSON_KEEP_DEFLATE 2
#define SOLVER_TOL 1e-8
#define SOLVER_MAX_ITS 200

static int do_doci = 1;

const char *argp_program_version = "doci (GB300) 0.1";
static char doc[] =
    "doci -- An implementation of DOCI (Doubly Occupied Configuration Interaction)"
    "\n\n"
    "input-file\n"
    "----------\n"
    "\n"
    "FCIDUMP          = path to the FCIDUMP file.\n"
    "\n"
    "SOLVER           = The sparse solver to be used. (D for Davidson, CG for\n"
    "                   conjugate gradient and CGP for conjugate gradient with\n"
    "                   diagonal preconditioner). (default: D)\n"
    "\n"
    "MAX_ITS          = Maximum number of iterations. (default: 200)\n"
    "\n"
    "TOL              = The tolerance for convergence. (default: 1e-8)\n"
    "\n"
    "DAVIDSON_KEEP    = The vectors to be kept after deflation in the Davidson\n"
    "                   algorithm. (default: 2)\n"
    "\n"
    "DAVIDSON_MAX_VEC = The maximum dimension of the subspace optimization before\n"
    "                   Davidson deflates. (default: 30)\n"
    "\n"
    "HF_INIT          = Set to 1 if initial guess should be the Hartree-Fock\n"
    "                   solution. Set to 0 if the initial guess should be random.\n"
    "                   (default: 1)\n";
static char args_doc[] = "INPUTFILE";
static struct argp_option options[] = {
    {"mode", 'm', "WHICH_MODE", 0,
     "For Full Configuration Interaction calculations set mode to 1. "
     "For Double Occupied Configuration Ineraction set mode to 0. (default: 0)\n", 0},
    {0}};

struct arguments {
  char *inputfile;
};

static error_t parse_opt(int key, char *arg, struct argp_state *state) {
  struct arguments *a = state->input;
  switch (key) {
    case 'm':
      do_doci = atoi(arg) ? 0 : 1;
      break;
    case ARGP_KEY_ARG:
      if (state->arg_num > 1) argp_usage(state);
      a->inputfile = arg;
      break;
    case ARGP_KEY_END:
      if (state->arg_num < 1) argp_usage(state);
      break;
    default:
      return ARGP_ERR_UNKNOWN;
  }
  return 0;
}

static struct argp argp_parser = {options, parse_opt, args_doc, doc, 0, 0, 0};

typedef struct {
  char dumpfil[255];
  char solver[20];
  int max_its, keep, max_vec, hf_init;
  double tol;
} input_t;

/* executable.c:201-230: every line is tried against every key; a key with no
 * value (e.g. "DAVIDSON_KEEP=") leaves the default */
static void read_inputfile(const char *path, input_t *in) {
  char buf[255];
  FILE *fp = fopen(path, "r");
  if (!fp) {
    fprintf(stderr, "Error reading input file\n");
    exit(EXIT_FAILURE);
  }
  in->dumpfil[0] = 0;
  strcpy(in->solver, "D");
  in->max_its = SOLVER_MAX_ITS;
  in->tol = SOLVER_TOL;
  in->keep = DAVIDSON_KEEP_DEFLATE;
  in->max_vec = DAVIDSON_MAX_VECS;
  in->hf_init = 1;
  while (fgets(buf, sizeof buf, fp)) {
    sscanf(buf, " FCIDUMP = %254s ", in->dumpfil);
    sscanf(buf, " SOLVER = %19s ", in->solver);
    sscanf(buf, " MAX_ITS = %d ", &in->max_its);
    sscanf(buf, " TOL = %lf ", &in->tol);
    sscanf(buf, " DAVIDSON_KEEP = %d ", &in->keep);
    sscanf(buf, " DAVIDSON_MAX_VEC = %d ", &in->max_vec);
    sscanf(buf, " HF_INIT = %d ", &in->hf_init);
  }
  fclose(fp);
}

static void print_inputfile(const input_t *in) {  /* executable.c:232-268 */
  const char *name;
  if (strcmp(in->solver, "D") == 0) name = "DAVIDSON";
  else if (strcmp(in->solver, "CG") == 0) name = "CONJUGATE GRADIENT";
  else if (strcmp(in->solver, "CGP") == 0) name = "CONJUGATE GRADIENT WITH DIAGONAL PRECONDITIONER";
  else {
    printf("no correct solver inputted!\n");
    exit(EXIT_FAILURE);
  }
  printf(
      "doci -- An implementation of DOCI (Doubly Occupied Configuration Interaction)"
      "\n\n"
      "input-file\n"
      "----------\n"
      "\n"
      "FCIDUMP          = %s\n"
      "\n"
      "SOLVER           = %s\n"
      "\n"
      "MAX_ITS          = %d\n"
      "\n"
      "TOL              = %e\n"
      "\n"
      "DAVIDSON_KEEP    = %d\n"
      "\n"
      "DAVIDSON_MAX_VEC = %d\n"
      "\n"
      "INITIAL          = %s\n\n",
      in->dumpfil, name, in->max_its, in->tol, in->keep, in->max_vec, in->hf_init ? "Hartree-Fock" : "random");
}

/* executable.c:270-299 */
static double *make_init_guess(int hf_init, const double *diagonal, int n) {
  double *r = calloc((size_t)n, sizeof(double));
  if (!r) {
    fprintf(stderr, "out of memory\n");
    exit(EXIT_FAILURE);
  }
  if (hf_init) {
    int ind = 0;
    double low = diagonal[0] + 1;
    for (int i = 0; i < n; ++i)
      if (low > diagonal[i]) {
        low = diagonal[i];
        ind = i;
      }
    r[ind] = 1;
  } else {
    const char *s = getenv("DOCI_SEED");
    srand(s ? (unsigned)strtoul(s, NULL, 10) : (unsigned)time(NULL));
    double nrm = 0;
    for (int i = 0; i < n; ++i) {
      r[i] = rand();
      nrm += r[i] * r[i];
    }
    nrm = 1 / sqrt(nrm);
    for (int i = 0; i < n; ++i) r[i] *= nrm;
  }
  return r;
}

int main(int argc, char *argv[]) {
  struct timeval t0, t1;
  gettimeofday(&t0, NULL);
  setvbuf(stdout, NULL, _IOLBF, BUFSIZ);
  struct arguments args = {NULL};
  argp_parse(&argp_parser, argc, argv, 0, 0, &args);
  if (!do_doci) {
    fprintf(stderr, "Only DOCI works at this moment!\n");
    exit(EXIT_FAILURE);
  }
  input_t in;
  read_inputfile(args.inputfile, &in);
  print_inputfile(&in);
  void *dat = NULL;
  fill_doci_data(in.dumpfil, &dat);
  const int n = doci_get_basis_size(dat);
  double *diagonal = doci_get_diagonal(dat);
  double *result = make_init_guess(in.hf_init, diagonal, n);
  double energy = 0;
  int info;
  printf("--------------------------------------------------\n");
  const char *mixed = getenv("DOCI_MIXED");
  if (mixed && *mixed && strcmp(mixed, "0") != 0 && strcmp(in.solver, "D") == 0) {
    doci_solve_opts o;
    doci_solve_result res;
    doci_solve_opts_default(&o);
    o.max_its = in.max_its;
    o.tol = in.tol;
    o.davidson_keep = in.keep;
    o.davidson_max_vec = in.max_vec;
    o.hf_init = -1;
    o.mode = DOCI_MODE_MIXED;
    o.print_level = 1;
    int st = doci_solve((doci_ham *)dat, &o, result, &res);
    if (st) {
      fprintf(stderr, "doci_solve: %s\n", doci_status_string(st));
      exit(EXIT_FAILURE);
    }
    printf("\t\t ** FP32 ITERATIONS : %d (energy %.10lf)\n", res.iterations_fp32, res.energy_fp32);
    energy = res.energy;
    info = res.status_code;
  } else {
    info = sparse_eigensolve(result, n, &energy, doci_matvec, diagonal, NULL, in.tol, in.max_its, in.solver,
                             in.keep, in.max_vec, dat);
  }
  gettimeofday(&t1, NULL);
  const double el = (t1.tv_sec - t0.tv_sec) + 1e-6 * (t1.tv_usec - t0.tv_usec);
  printf(
      "\t\t ** EXIT CODE SOLVER : %d\n"
      "\t\t ** %s ENERGY : %.10lf\n"
      "\t\t ** ELAPSED TIME : %f\n"
      "--------------------------------------------------\n"
      "exiting...\n",
      info, do_doci ? "DOCI" : "FCI", energy, el);
  doci_cleanup_data(&dat);
  free(result);
  return EXIT_SUCCESS;
}
