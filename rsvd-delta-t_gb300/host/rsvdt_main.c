/*
 * rsvdt_main -- drop-in for the reference executable's main.c
 * (AliFarghadan/RSVD-Delta-t, SourceCode/main.c:85-152) on one GB300.
 *
 *   rsvdt_main -inputs variables.yaml
 *
 * Reads the same YAML keys with the same defaults and errors
 * (SourceCode/ReadUserInput.c:20-171), loads the same PETSc-binary operator,
 * weight and forcing files (paths are RootDir + <key>Dir, concatenated
 * without a separator as in SourceCode/LNSStructure.c:22), runs the
 * RSVD-Delta-t sequence through the C ABI (include/rsvdt.h) and writes the
 * same outputs into RootDir + ResultsDir + ResolventModes_<n>/
 * (SourceCode/CreateResultsDir.c:20-30, SourceCode/SaveResults.c:32-92).
 * With TransRun: true it runs the transient simulation instead
 * (SourceCode/main.c:119-124, SourceCode/TransientRunRK4.c:11-228) and
 * writes its snapshots and norms into RootDir + ResultsDir +
 * TransientSnapshots_<n>/.
 */
#include <ctype.h>
#include <errno.h>
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/stat.h>
#include <time.h>
#include <unistd.h>

#include "petsc_bin.h"
#include "rsvdt.h"

#define MAXOPT 256
#define PATHLEN 4096

typedef struct {
  char key[128];
  char val[PATHLEN];
} opt_t;

static opt_t g_opts[MAXOPT];
static int g_nopt = 0;

static void die(const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  fprintf(stderr, "[rsvdt] ERROR: ");
  vfprintf(stderr, fmt, ap);
  fprintf(stderr, "\n");
  va_end(ap);
  exit(1);
}

static char *trim(char *s) {
  while (isspace((unsigned char)*s)) ++s;
  char *e = s + strlen(s);
  while (e > s && isspace((unsigned char)e[-1])) *--e = '\0';
  return s;
}

/* Top-level "Key: value  # comment" lines of a YAML mapping (the subset
 * PetscOptionsInsertFileYAML turns into -Key value options). Quotes around
 * a value are removed. */
static void read_yaml(const char *path) {
  FILE *f = fopen(path, "r");
  if (!f) die("cannot open the inputs file %s", path);
  char line[PATHLEN + 256];
  while (fgets(line, sizeof line, f)) {
    char *s = line;
    if (*s == '#' || isspace((unsigned char)*s)) {
      s = trim(s);
      if (*s == '\0' || *s == '#') continue;
    }
    char *c = strchr(s, ':');
    if (!c) continue;
    *c = '\0';
    char *key = trim(s);
    char *val = c + 1;
    /* strip a comment that starts with whitespace + '#' */
    for (char *p = val; *p; ++p)
      if (*p == '#' && (p == val || isspace((unsigned char)p[-1]))) {
        *p = '\0';
        break;
      }
    val = trim(val);
    size_t n = strlen(val);
    if (n >= 2 && ((val[0] == '"' && val[n - 1] == '"') || (val[0] == '\'' && val[n - 1] == '\''))) {
      val[n - 1] = '\0';
      ++val;
    }
    if (!*key) continue;
    if (g_nopt >= MAXOPT) die("too many keys in %s", path);
    snprintf(g_opts[g_nopt].key, sizeof g_opts[g_nopt].key, "%s", key);
    snprintf(g_opts[g_nopt].val, sizeof g_opts[g_nopt].val, "%s", val);
    ++g_nopt;
  }
  fclose(f);
}

static const char *get(const char *key) {
  for (int i = g_nopt - 1; i >= 0; --i)
    if (strcmp(g_opts[i].key, key) == 0) return g_opts[i].val;
  return NULL;
}

static int get_real(const char *key, double *v) {
  const char *s = get(key);
  if (!s) return 0;
  char *end;
  errno = 0;
  double d = strtod(s, &end);
  if (end == s || *trim(end) != '\0' || errno) die("Input string %s for '%s' has no real value", s, key);
  *v = d;
  return 1;
}

static int get_int(const char *key, int64_t *v) {
  const char *s = get(key);
  if (!s) return 0;
  char *end;
  errno = 0;
  long long x = strtoll(s, &end, 10);
  if (end == s || *end != '\0' || errno)
    die("Input string %s for '%s' has no integer value (do not include . in it)", s, key);
  *v = x;
  return 1;
}

static int get_bool(const char *key, int *v) {
  const char *s = get(key);
  if (!s) return 0;
  char b[16];
  size_t n = strlen(s);
  if (n >= sizeof b) die("Unknown logical value: %s", s);
  for (size_t i = 0; i <= n; ++i) b[i] = (char)tolower((unsigned char)s[i]);
  if (!strcmp(b, "true") || !strcmp(b, "yes") || !strcmp(b, "on") || !strcmp(b, "1"))
    *v = 1;
  else if (!strcmp(b, "false") || !strcmp(b, "no") || !strcmp(b, "off") || !strcmp(b, "0"))
    *v = 0;
  else
    die("Unknown logical value: %s", s);
  return 1;
}

static int get_str(const char *key, char *out) {
  const char *s = get(key);
  if (!s) return 0;
  snprintf(out, PATHLEN, "%s", s);
  return 1;
}

static void warn_default_i(const char *key, long long v) {
  printf("Warning: '%s' variable not found. Setting '%s' to default value: %lld\n", key, key, v);
}

static void warn_default_g(const char *key, double v) {
  printf("Warning: '%s' variable not found. Setting '%s' to default value: %g\n", key, key, v);
}

typedef struct {
  char root[PATHLEN], results[PATHLEN], op[PATHLEN], forcing[PATHLEN];
  char wdir[5][PATHLEN];
  char folder[PATHLEN];
  int wflag[5];
  int input_forcing, trans_run, save_opt;
  /* SaveResumeQ (no counterpart in the reference): write the forcing of
   * every power sweep's direct action as a resume point. */
  int save_resume;
  int64_t rand_seed;
  /* Transient simulation (SourceCode/Variables.h TransRun_vars). */
  int trans_ic_flg;
  char icdir[PATHLEN];
  rsvdt_trans_params tp;
} drv_t;

static void join(char *out, const char *a, const char *b) {
  if (snprintf(out, PATHLEN, "%s%s", a, b) >= PATHLEN) die("path too long: %s%s", a, b);
}

/* SourceCode/ReadUserInput.c:20-171. */
static void read_user_input(rsvdt_params *p, drv_t *d) {
  int set, b;
  int64_t i;
  double r;
  if (!get_real("TransientLength", &p->TransientLength)) die("Must specify 'TransientLength'");
  if (!get_real("dt", &p->dt)) die("Must specify 'dt'");
  if (!get_real("w", &p->w)) die("Must specify 'dt'"); /* the reference's message for a missing w */
  static const char *wflag_keys[5] = {"InvInputWeightFlg", "InputMatrixFlg", "OutputMatrixFlg", "OutputWeightFlg",
                                      "InvOutputWeightFlg"};
  static const char *wdir_keys[5] = {"InvInputWeightDir", "InputMatrixDir", "OutputMatrixDir", "OutputWeightDir",
                                     "InvOutputWeightDir"};
  set = get_bool("InputForcingFlg", &d->input_forcing);
  if (!set) {
    d->input_forcing = 0;
    warn_default_i("InputForcingFlg", 0);
  } else if (d->input_forcing && !get_str("InputForcingDir", d->forcing))
    die("Must specify 'InputForcingDir'");
  for (int w = 0; w < 5; ++w) {
    set = get_bool(wflag_keys[w], &d->wflag[w]);
    if (!set) {
      d->wflag[w] = 0;
      warn_default_i(wflag_keys[w], 0);
    } else if (d->wflag[w] && !get_str(wdir_keys[w], d->wdir[w])) {
      die("Must specify '%s'", wdir_keys[w]);
    }
  }
  if (!get_bool("TwoPI", &b)) {
    b = 0;
    warn_default_i("TwoPI", 0);
  }
  p->TwoPI = b;
  if (!get_bool("TransRun", &d->trans_run)) {
    d->trans_run = 0;
    warn_default_i("TransRun", 0);
  }
  if (!get_bool("SaveResumeQ", &d->save_resume)) d->save_resume = 0;
  if (!get_bool("TransientRemoval", &b)) {
    b = 0;
    warn_default_i("TransientRemoval", 0);
  }
  p->TransientRemoval = b;
  if (!get_bool("DiscFlg", &b)) {
    b = 0;
    warn_default_i("DiscFlg", 0);
  }
  p->DiscFlg = b;
  if (!get_int("SaveResultsOpt", &i)) {
    i = 1;
    warn_default_i("SaveResultsOpt", 1);
  }
  d->save_opt = (int)i;
  if (!get_str("RootDir", d->root)) die("Must specify 'RootDir'");
  if (!get_str("ResultsDir", d->results)) die("Must specify 'ResultsDir'");
  if (!get_str("OperatorDir", d->op)) die("Must specify 'OperatorDir'");
  if (!get_int("k", &p->k)) {
    p->k = 3;
    warn_default_i("k", 3);
  }
  if (!get_int("q", &p->q)) {
    p->q = 0;
    warn_default_i("q", 0);
  }
  if (!get_int("Nw", &p->Nw)) die("Must specify 'Nw'");
  if (!get_int("RandSeed", &d->rand_seed)) {
    d->rand_seed = 1373;
    warn_default_i("RandSeed", 1373);
  }
  if (!get_int("Display", &i)) {
    i = 2;
    warn_default_i("Display", 2);
  }
  p->Display = (int32_t)i;
  set = get_real("beta", &r);
  if (!set && p->DiscFlg) die("Discounting flag is on! Either set Discounting to zero or specify 'beta'");
  p->beta = set ? r : 0.0;
  if (p->beta < 0 && p->DiscFlg) die("'beta' must be positive, current value: %g", p->beta);
  /* SourceCode/ReadUserInput.c:134-171: the transient-run keys get their
   * defaults (and warnings) only when TransRun is on; TransICDir is required
   * unless TransICFlg is absent in a transient run. */
  set = get_bool("TransICFlg", &d->trans_ic_flg);
  if (!set && d->trans_run) {
    d->trans_ic_flg = 0;
    warn_default_i("TransICFlg", 0);
  } else if (!get_str("TransICDir", d->icdir)) {
    die("Must specify 'TransICDir'");
  }
  rsvdt_trans_params *tp = &d->tp;
  b = 0;
  if (!get_real("TransDivVal", &tp->div_val) && d->trans_run) {
    tp->div_val = 1e3;
    warn_default_g("TransDivVal", tp->div_val);
  }
  if (!get_real("TransConVal", &tp->con_val) && d->trans_run) {
    tp->con_val = 1e-8;
    warn_default_g("TransConVal", tp->con_val);
  }
  if (!get_bool("TransSave", &b) && d->trans_run) {
    b = 0;
    warn_default_i("TransSave", 0);
  }
  tp->save = b;
  b = 0;
  if (!get_bool("TransRemovalEst", &b) && d->trans_run) {
    b = 0;
    warn_default_i("TransRemovalEst", 0);
  }
  tp->removal_est = b;
  if (!get_int("TransSaveMod", &tp->save_mod) && d->trans_run) {
    tp->save_mod = 100;
    warn_default_i("TransSaveMod", 100);
  }
  if (!get_int("TransPeriods", &tp->periods) && d->trans_run) {
    tp->periods = 1;
    warn_default_i("TransPeriods", 1);
  }
  printf("\n");
}

/* Resume point of power sweep j: the block that the sweep's direct action
 * takes as its forcing, written as Q_resume_sweep<j> in the results folder
 * (dense, MatView layout), readable through InputForcingDir; a run from it
 * with q - j power iterations continues this run exactly. */
typedef struct {
  const drv_t *d;
  int64_t rows, cols, q;
} resume_t;

static int write_resume_point(void *user, int32_t sweep, rsvdt_ctx *ctx) {
  const resume_t *rs = (const resume_t *)user;
  double *Q = (double *)malloc(sizeof(double) * 2 * (size_t)rs->rows * (size_t)rs->cols);
  if (!Q) {
    fprintf(stderr, "out of memory for the resume point\n");
    return 1;
  }
  char path[PATHLEN], name[64], err[512];
  int rc = rsvdt_get_block(ctx, Q, rs->rows, NULL) != RSVDT_OK;
  snprintf(name, sizeof name, "Q_resume_sweep%d", (int)sweep);
  join(path, rs->d->folder, name);
  if (!rc && pb_write_dense(path, Q, rs->rows, rs->cols, rs->rows, err, sizeof err)) {
    fprintf(stderr, "%s\n", err);
    rc = 1;
  }
  free(Q);
  if (!rc) printf("Resume point (InputForcingDir with q = %d): %s\n", (int)(rs->q - sweep), path);
  return rc;
}

/* SourceCode/CreateResultsDir.c:20-30. */
static void create_results_dir(drv_t *d, const char *prefix) {
  for (int ind = 0;; ++ind) {
    char name[256];
    snprintf(name, sizeof name, "%s%d/", prefix, ind);
    if (snprintf(d->folder, PATHLEN, "%s%s%s", d->root, d->results, name) >= PATHLEN) die("path too long");
    if (access(d->folder, F_OK) != 0) break;
  }
  if (mkdir(d->folder, 0775) != 0) die("cannot create the results folder %s (%s)", d->folder, strerror(errno));
}

static void check(rsvdt_ctx *ctx, rsvdt_status st, const char *what) {
  if (st != RSVDT_OK) die("%s: %s", what, rsvdt_last_error(ctx));
}

static void load_csr(const char *path, pb_csr *m) {
  char err[512];
  if (pb_read_mat(path, m, err, sizeof err)) die("%s", err);
}

/* SaveInputVarsCopy (SourceCode/SaveInputVarsCopy.c:26-38). */
static void save_inputs_copy(const char *inputs, const char *folder) {
  char path[PATHLEN];
  const char *base = strrchr(inputs, '/');
  base = base ? base + 1 : inputs;
  join(path, folder, base);
  FILE *src = fopen(inputs, "rb"), *dst = fopen(path, "wb");
  if (!src || !dst) die("cannot copy %s to %s", inputs, path);
  char buf[1024];
  size_t n;
  while ((n = fread(buf, 1, sizeof buf, src)) > 0) fwrite(buf, 1, n, dst);
  fclose(src);
  fclose(dst);
}

/* Uniform [0,1) real and imaginary parts, then normalised: the
 * distribution of VecSetRandom + VecNormalize in
 * SourceCode/TransientRunRK4.c:88-93, from a splitmix64 stream seeded by
 * RandSeed (PETSc's own generator is not reproduced). */
static void random_ic(double *q, int64_t n, uint64_t seed) {
  uint64_t x = seed;
  double s = 0;
  for (int64_t i = 0; i < 2 * n; ++i) {
    uint64_t z = (x += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    q[i] = (double)(z >> 11) * (1.0 / 9007199254740992.0);
    s += q[i] * q[i];
  }
  s = sqrt(s);
  for (int64_t i = 0; i < 2 * n; ++i) q[i] /= s;
}

typedef struct {
  const char *folder;
  char err[512];
} trans_io;

static int write_snapshot(void *user, int64_t pos, const double *q, int64_t n) {
  trans_io *io = (trans_io *)user;
  char path[PATHLEN], name[64];
  snprintf(name, sizeof name, "q_transient_%d", (int)pos);
  join(path, io->folder, name);
  return pb_write_vec(path, q, n, 1, io->err, sizeof io->err);
}

static int write_estimate(void *user, int64_t period, const double *initial, const double *updated,
                          int64_t count) {
  trans_io *io = (trans_io *)user;
  char path[PATHLEN], name[96];
  snprintf(name, sizeof name, "Initial_transient_norm_period_%d", (int)period);
  join(path, io->folder, name);
  if (pb_write_vec(path, initial, count, 0, io->err, sizeof io->err)) return 1;
  snprintf(name, sizeof name, "Updated_transient_norm_period_%d", (int)period);
  join(path, io->folder, name);
  return pb_write_vec(path, updated, count, 0, io->err, sizeof io->err);
}

/* PreProcessing for a transient run (SourceCode/PreProcessing.c:34-67:
 * no weights, no sketch) and TransientRunRK4
 * (SourceCode/TransientRunRK4.c:32-224). */
static int transient_run(rsvdt_params *p, drv_t *d, const char *inputs) {
  rsvdt_ctx *ctx = NULL;
  rsvdt_status st = rsvdt_create(p, &ctx);
  if (st != RSVDT_OK) die("%s", ctx ? rsvdt_last_error(ctx) : "context creation failed");
  char path[PATHLEN], err[512];
  pb_csr A;
  join(path, d->root, d->op);
  printf("Loading the operator: %s \n", path);
  load_csr(path, &A);
  if (A.rows != A.cols) die("the operator must be square, current size = %lld x %lld", (long long)A.rows,
                            (long long)A.cols);
  check(ctx, rsvdt_set_operator(ctx, A.rows, A.rowptr, A.col, A.val), "operator");
  printf("The operator is loaded (N = %lld)\n", (long long)A.rows);
  const int64_t N = A.rows;
  pb_free(&A);
  create_results_dir(d, "TransientSnapshots_");

  printf("\n********************************************\n************** Transient run ***************\n"
         "********************************************\n\n");
  rsvdt_trans_info info;
  check(ctx, rsvdt_trans_grid(ctx, &d->tp, &info), "transient grid");
  if (d->tp.save)
    printf("Total snapshots to be saved = %d\n", (int)info.n_saved);
  else
    printf("Saving snapshots is not requested\n");
  double *q = (double *)malloc(sizeof(double) * 2 * (size_t)N);
  double *norms = (double *)calloc((size_t)info.n_saved, sizeof(double));
  if (!q || !norms) die("out of memory");
  if (d->trans_ic_flg) {
    printf("Reading the initial vector\n");
    if (snprintf(path, PATHLEN, "%s%s%s", d->root, d->results, d->icdir) >= PATHLEN) die("path too long");
    double *v = NULL;
    int64_t n = 0;
    if (pb_read_vec(path, &v, &n, err, sizeof err)) die("%s", err);
    if (n != N) die("the initial vector has %lld entries, the operator %lld rows", (long long)n, (long long)N);
    memcpy(q, v, sizeof(double) * 2 * (size_t)N);
    free(v);
  } else {
    printf("Random vector is generated\n\n");
    random_ic(q, N, (uint64_t)d->rand_seed);
  }
  trans_io io;
  io.folder = d->folder;
  io.err[0] = '\0';
  const time_t t0 = time(NULL);
  st = rsvdt_trans_run(ctx, &d->tp, q, norms, write_snapshot, write_estimate, &io, &info);
  if (st != RSVDT_OK) die("transient run: %s%s%s", rsvdt_last_error(ctx), io.err[0] ? ": " : "", io.err);
  const int el = (int)difftime(time(NULL), t0);
  printf("*** Transient simulation elapsed time = %02d:%02d:%02d ***\n", el / 3600, (el / 60) % 60, el % 60);
  printf("\nThe results directory is: %s\n\n", d->folder);
  join(path, d->folder, "q_transient_norms");
  if (pb_write_vec(path, norms, info.n_saved, 0, err, sizeof err)) die("%s", err);
  join(path, d->folder, "q_transient_last_snapshot");
  if (pb_write_vec(path, q, N, 1, err, sizeof err)) die("%s", err);
  save_inputs_copy(inputs, d->folder);
  printf("DONE :))\n\n");
  free(q);
  free(norms);
  rsvdt_destroy(ctx);
  return 0;
}

int main(int argc, char **argv) {
  const char *inputs = NULL;
  for (int a = 1; a + 1 < argc; ++a)
    if (!strcmp(argv[a], "-inputs")) inputs = argv[a + 1];
  if (!inputs) die("Must specify inputs variables via -inputs");
  printf("\n*** Reading user inputs ***\n");
  read_yaml(inputs);
  rsvdt_params p;
  rsvdt_default_params(&p);
  drv_t d;
  memset(&d, 0, sizeof d);
  read_user_input(&p, &d);
  if (d.trans_run) return transient_run(&p, &d, inputs);

  rsvdt_ctx *ctx = NULL;
  rsvdt_status st = rsvdt_create(&p, &ctx);
  if (st != RSVDT_OK) die("%s", ctx ? rsvdt_last_error(ctx) : "context creation failed");

  /* Operator (SourceCode/LNSStructure.c:22-27). */
  char path[PATHLEN];
  pb_csr A;
  join(path, d.root, d.op);
  printf("Loading the operator: %s \n", path);
  load_csr(path, &A);
  if (A.rows != A.cols) die("the operator must be square, current size = %lld x %lld", (long long)A.rows,
                            (long long)A.cols);
  /* Problems whose resident buffers (five spectral blocks, the ring, the
   * operator and its conjugate transpose) would not fit in device memory
   * run in the capacity mode. */
  {
    int64_t dev_free = 0, dev_total = 0;
    if (rsvdt_device_memory(&dev_free, &dev_total) == RSVDT_OK) {
      const double blk = 16.0 * (double)A.rows * (double)p.Nw * (double)p.k;
      const double resident = 5 * blk + 16.0 * (double)(p.Nw + 1) * (double)A.rows * (double)p.k +
                              2 * 28.0 * (double)A.nnz;
      if (resident > 0.9 * (double)dev_free) {
        check(ctx, rsvdt_set_capacity_mode(ctx, 0, 0), "capacity mode");
        printf("Capacity mode: the resident buffers (%.1f GB) exceed the free device memory (%.1f GB)\n",
               resident / 1e9, dev_free / 1e9);
      }
    }
  }
  check(ctx, rsvdt_set_operator(ctx, A.rows, A.rowptr, A.col, A.val), "operator");
  printf("The operator is loaded (N = %lld)\n", (long long)A.rows);
  pb_free(&A);

  /* Weights (SourceCode/ReadWeightMats.c:26-99). */
  static const rsvdt_weight which[5] = {RSVDT_W_F_SQRT_INV, RSVDT_B, RSVDT_C, RSVDT_W_Q_SQRT, RSVDT_W_Q_SQRT_INV};
  for (int w = 0; w < 5; ++w) {
    if (!d.wflag[w]) continue;
    pb_csr M;
    join(path, d.root, d.wdir[w]);
    load_csr(path, &M);
    check(ctx, rsvdt_set_weight(ctx, which[w], M.rows, M.cols, M.rowptr, M.col, M.val), path);
    pb_free(&M);
  }
  rsvdt_grid g;
  check(ctx, rsvdt_get_grid(ctx, &g), "grid");
  printf("RSVD parameters:\n@ k        = %d\n@ q        = %d\n@ w        = %g\n\n", (int)p.k, (int)p.q, g.w);
  printf("Time-stepping parameters:\n@ TransientLength = %g\n@ dt              = %g\n@ Ns              = %d\n"
         "@ Nt              = %d\n",
         p.TransientLength, g.dt, (int)g.Ns, (int)g.Nt);
  printf("The effective number of frequencies, Nw = %d\n", (int)g.Nw_eff);

  /* Sketch (SourceCode/CreateRandomMat.c:23-39). */
  int64_t k = p.k;
  if (d.input_forcing) {
    pb_csr F;
    join(path, d.root, d.forcing);
    printf("Reading the input forcing matrix         : %s\n", path);
    load_csr(path, &F);
    if (F.rows != g.Nb)
      die("Input forcing must be have %d rows, current size = %d x %d", (int)g.Nb, (int)F.rows, (int)F.cols);
    /* Dense column-major copy. */
    double *Fd = (double *)calloc((size_t)(2 * F.rows * F.cols), sizeof(double));
    if (!Fd) die("out of memory");
    for (int64_t r = 0; r < F.rows; ++r)
      for (int64_t j = F.rowptr[r]; j < F.rowptr[r + 1]; ++j) {
        Fd[2 * (F.col[j] * F.rows + r)] = F.val[2 * j];
        Fd[2 * (F.col[j] * F.rows + r) + 1] = F.val[2 * j + 1];
      }
    check(ctx, rsvdt_set_sketch(ctx, Fd, F.rows, F.cols), "forcing");
    k = F.cols / g.Nw_eff;
    printf("Based on the input forcing: k = %d\n", (int)k);
    free(Fd);
    pb_free(&F);
  } else {
    printf("Generating a random forcing matrix\n");
    check(ctx, rsvdt_random_sketch(ctx, (uint64_t)d.rand_seed), "random sketch");
  }
  create_results_dir(&d, "ResolventModes_");
  resume_t rs = {&d, g.Nb, k * g.Nw_eff, p.q};
  if (d.save_resume) check(ctx, rsvdt_set_checkpoint(ctx, write_resume_point, &rs), "checkpoint");

  printf("\n********************************************\n*************** RSVD-\\Delta t **************\n"
         "********************************************\n");
  check(ctx, rsvdt_run(ctx), "RSVD-Delta-t");
  if (p.Display >= 1) {
    char js[1024];
    if (rsvdt_get_timings(ctx, js, sizeof js) == RSVDT_OK) printf("Timings: %s\n", js);
  }

  /* SaveResults (SourceCode/SaveResults.c:32-92), one file's columns at a
   * time (a file is N x Nw_eff or N x k; the whole U and V may not fit in
   * host memory). */
  const int64_t nwe = g.Nw_eff;
  double *S = (double *)malloc(sizeof(double) * k * nwe);
  if (!S) die("out of memory");
  check(ctx, rsvdt_get_results(ctx, NULL, 1, NULL, 1, S), "results");
  printf("\nThe results directory: %s\n\n", d.folder);
  char err[512];
  join(path, d.folder, "S_hat");
  if (pb_write_dense_real(path, S, k, nwe, k, err, sizeof err)) die("%s", err);
  const int64_t per = d.save_opt == 1 ? nwe : k;
  int64_t *cols = (int64_t *)malloc(sizeof(int64_t) * per);
  double *Ub = (double *)malloc(sizeof(double) * 2 * g.Nc * per);
  double *Vb = (double *)malloc(sizeof(double) * 2 * g.Nb * per);
  if (!cols || !Ub || !Vb) die("out of memory");
  const int64_t nfiles = d.save_opt == 1 ? k : nwe;
  for (int64_t f = 0; f < nfiles; ++f) {
    for (int64_t j = 0; j < per; ++j) cols[j] = d.save_opt == 1 ? j * k + f : f * k + j;
    check(ctx, rsvdt_get_result_cols(ctx, cols, per, Ub, g.Nc, Vb, g.Nb), "results");
    char name[128];
    if (d.save_opt == 1)
      snprintf(name, sizeof name, "U_hat_k%d_allFreqs", (int)f + 1);
    else
      snprintf(name, sizeof name, "U_hat_Freq%d_allK", (int)f);
    join(path, d.folder, name);
    if (pb_write_dense(path, Ub, g.Nc, per, g.Nc, err, sizeof err)) die("%s", err);
    name[0] = 'V';
    join(path, d.folder, name);
    if (pb_write_dense(path, Vb, g.Nb, per, g.Nb, err, sizeof err)) die("%s", err);
  }
  free(cols);
  free(Ub);
  free(Vb);
  save_inputs_copy(inputs, d.folder);
  printf("DONE :))\n\n");
  free(S);
  rsvdt_destroy(ctx);
  return 0;
}
