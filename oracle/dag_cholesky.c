/*
 * CPU restatement of Dagger.jl's datadeps tiled Cholesky and Cholesky solve,
 * and of the pivoted tiled LU (lu!(A, RowMaximum())).
 *
 * TEST INFRASTRUCTURE ONLY: this is the oracle's threaded form, used as the
 * checker at sizes the Python restatement is too slow for and as the CPU
 * baseline `bench.py` times ("CPU restatement of Dagger datadeps Cholesky",
 * not Dagger itself).  Nothing in the product library links it.
 *
 * What it restates (paths within JuliaParallel/Dagger.jl v0.22.0):
 *   src/array/cholesky.jl:38-53, :83-98   the POTRF/TRSM/SYRK/GEMM tile tasks
 *                                        and their In/InOut arguments
 *   src/array/trsm.jl:89-140               the left-side block solves ldiv! uses
 *   src/array/linalg.jl:386-403            ldiv! solve order per uplo
 *   src/array/lu.jl:263-304, :351-407      lu!(A, RowMaximum()) with the LAPACK
 *                                        panel (factor_panel_lapack!, InOut on
 *                                        every tile of the block column),
 *                                        swaprows_trail! per tile pair, TRSM,
 *                                        GEMM
 *   src/datadeps/queue.jl:43-53,
 *   src/datadeps/aliasing.jl:740-776       the dependency rules: a writer waits
 *                                        for the last writer and the readers
 *                                        since; a reader waits for the last
 *                                        writer
 * Tasks are run by a dependency-counting pool of worker threads (the
 * reference's ThreadProc workers), each calling single-threaded FP64 BLAS /
 * LAPACK tile routines.  The BLAS routine pointers are handed in at run time
 * (scipy's cython_blas / cython_lapack exports, LP64 Fortran ABI), so this
 * file needs no BLAS headers or link-time library.
 *
 * Matrices are column-major with leading dimension lda; tile (i, j) starts at
 * A + i*nb + j*nb*lda and is min(nb, n - i*nb) x min(nb, n - j*nb).
 */
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef void (*dgemm_fn)(char *, char *, int *, int *, int *, double *, double *, int *,
                         double *, int *, double *, double *, int *);
typedef void (*dtrsm_fn)(char *, char *, char *, char *, int *, int *, double *, double *,
                         int *, double *, int *);
typedef void (*dsyrk_fn)(char *, char *, int *, int *, double *, double *, int *, double *,
                         double *, int *);
typedef void (*dpotrf_fn)(char *, int *, double *, int *, int *);
typedef void (*dgetrf_fn)(int *, int *, double *, int *, int *, int *);

static dgemm_fn g_dgemm;
static dtrsm_fn g_dtrsm;
static dsyrk_fn g_dsyrk;
static dpotrf_fn g_dpotrf;
static dgetrf_fn g_dgetrf;

int oracle_set_getrf(void *dgetrf) {
  g_dgetrf = (dgetrf_fn)dgetrf;
  return dgetrf ? 0 : -1;
}

int oracle_set_blas(void *dgemm, void *dtrsm, void *dsyrk, void *dpotrf) {
  g_dgemm = (dgemm_fn)dgemm;
  g_dtrsm = (dtrsm_fn)dtrsm;
  g_dsyrk = (dsyrk_fn)dsyrk;
  g_dpotrf = (dpotrf_fn)dpotrf;
  return (dgemm && dtrsm && dsyrk && dpotrf) ? 0 : -1;
}

enum { T_POTRF, T_TRSM, T_SYRK, T_GEMM, T_GETRF, T_SWAP };

typedef struct {
  int kind;
  char side, uplo, ta, tb;
  double alpha, beta;
  int a, b, c;   /* tile ids: a, b read; c read-write (-1 = unused)    */
  int offset;    /* global row offset of a POTRF tile, for info       */
  char diag;     /* TRSM diag ('U' unit; 0 = 'N')                    */
  int span;      /* c .. c+span-1 are written (a panel); 0 or 1 = c  */
  int w2p1;      /* one more written tile + 1 (0 = none)             */
  int step;      /* LU: the block row k of a panel / interchange      */
} task_t;

typedef struct {
  /* tile geometry: tile id t -> pointer, rows, cols, ld */
  double **ptr;
  int *rows, *cols, *ld;
  task_t *tasks;
  int ntasks;
  int *npred;     /* remaining predecessor count */
  int **succ;     /* successor lists */
  int *nsucc;
  /* ready heap ordered by task index (submission order first) */
  int *heap;
  int heap_n;
  int done;
  int failed_info;
  int stop_on_info;  /* Cholesky: a failed POTRF stops the region; LU continues */
  /* LU: global 1-based pivots, the panels' local pivots, the block size */
  int *lu_ipiv, *lu_tmp, lu_n, lu_nb;
  pthread_mutex_t mu;
  pthread_cond_t cv;
} dag_t;

static void heap_push(dag_t *d, int t) {
  int i = d->heap_n++;
  d->heap[i] = t;
  while (i > 0) {
    int p = (i - 1) / 2;
    if (d->heap[p] <= d->heap[i]) break;
    int x = d->heap[p]; d->heap[p] = d->heap[i]; d->heap[i] = x;
    i = p;
  }
}

static int heap_pop(dag_t *d) {
  int top = d->heap[0];
  d->heap[0] = d->heap[--d->heap_n];
  int i = 0;
  for (;;) {
    int l = 2 * i + 1, r = l + 1, m = i;
    if (l < d->heap_n && d->heap[l] < d->heap[m]) m = l;
    if (r < d->heap_n && d->heap[r] < d->heap[m]) m = r;
    if (m == i) break;
    int x = d->heap[m]; d->heap[m] = d->heap[i]; d->heap[i] = x;
    i = m;
  }
  return top;
}

/* datadeps rules over whole tiles (tiles alias only themselves). */
static int build_edges(dag_t *d, int ntiles) {
  int *last_writer = malloc(sizeof(int) * ntiles);
  int **readers = calloc(ntiles, sizeof(int *));
  int *nreaders = calloc(ntiles, sizeof(int));
  int *capreaders = calloc(ntiles, sizeof(int));
  int *capsucc = calloc(d->ntasks, sizeof(int));
  if (!last_writer || !readers || !nreaders || !capreaders || !capsucc) return -1;
  for (int i = 0; i < ntiles; i++) last_writer[i] = -1;
  d->npred = calloc(d->ntasks, sizeof(int));
  d->succ = calloc(d->ntasks, sizeof(int *));
  d->nsucc = calloc(d->ntasks, sizeof(int));
  enum { kMaxPreds = 1024 };
  int preds[kMaxPreds];
#define ADD_PRED(p)                                              \
  do {                                                           \
    int _p = (p), _dup = 0;                                      \
    for (int _i = 0; _i < np; _i++) if (preds[_i] == _p) _dup = 1; \
    if (!_dup && np < kMaxPreds) preds[np++] = _p;               \
  } while (0)
  for (int t = 0; t < d->ntasks; t++) {
    task_t *k = &d->tasks[t];
    int np = 0;
    int rd[2] = {k->a, k->b};
    for (int r = 0; r < 2; r++)
      if (rd[r] >= 0 && last_writer[rd[r]] >= 0) ADD_PRED(last_writer[rd[r]]);
    /* written tiles: c (and c+1 .. c+span-1 for a panel), w2p1 - 1 */
    int wr[2 + 256], nw = 0;
    if (k->c >= 0)
      for (int q = 0; q < (k->span > 1 ? k->span : 1) && nw < 256; q++) wr[nw++] = k->c + q;
    if (k->w2p1 > 0) wr[nw++] = k->w2p1 - 1;
    for (int q = 0; q < nw; q++) {
      int w = wr[q];
      if (last_writer[w] >= 0) ADD_PRED(last_writer[w]);
      /* readers since the last write; kept bounded by the tile DAG's shape */
      for (int i = 0; i < nreaders[w]; i++) {
        int p = readers[w][i];
        int dup = 0;
        for (int j = 0; j < np; j++) if (preds[j] == p) dup = 1;
        if (!dup) {
          if (np >= kMaxPreds) return -2;
          preds[np++] = p;
        }
      }
    }
    for (int r = 0; r < 2; r++) {
      int tl = rd[r];
      if (tl < 0) continue;
      if (nreaders[tl] == capreaders[tl]) {
        capreaders[tl] = capreaders[tl] ? 2 * capreaders[tl] : 8;
        readers[tl] = realloc(readers[tl], sizeof(int) * capreaders[tl]);
      }
      readers[tl][nreaders[tl]++] = t;
    }
    for (int q = 0; q < nw; q++) {
      last_writer[wr[q]] = t;
      nreaders[wr[q]] = 0;
    }
    for (int i = 0; i < np; i++) {
      int p = preds[i];
      if (p == t) continue;
      if (d->nsucc[p] == capsucc[p]) {
        capsucc[p] = capsucc[p] ? 2 * capsucc[p] : 4;
        d->succ[p] = realloc(d->succ[p], sizeof(int) * capsucc[p]);
      }
      d->succ[p][d->nsucc[p]++] = t;
      d->npred[t]++;
    }
  }
#undef ADD_PRED
  for (int i = 0; i < ntiles; i++) free(readers[i]);
  free(readers); free(nreaders); free(capreaders); free(last_writer); free(capsucc);
  return 0;
}

static void run_task(dag_t *d, int t) {
  task_t *k = &d->tasks[t];
  if (k->kind == T_POTRF) {
    char uplo = k->uplo;
    int n = d->rows[k->c], lda = d->ld[k->c], info = 0;
    g_dpotrf(&uplo, &n, d->ptr[k->c], &lda, &info);
    if (info != 0) {
      pthread_mutex_lock(&d->mu);
      int g = k->offset + info;
      if (d->failed_info == 0 || g < d->failed_info) d->failed_info = g;
      pthread_mutex_unlock(&d->mu);
    }
  } else if (k->kind == T_GETRF) {
    /* factor_panel_lapack!: getrf on the block column from the diagonal down
     * (one column-major view of the whole matrix) */
    int r0 = k->step * d->lu_nb;
    int m = d->lu_n - r0, n = d->cols[k->c], lda = d->ld[k->c], info = 0;
    int *lp = d->lu_tmp + r0;
    g_dgetrf(&m, &n, d->ptr[k->c], &lda, lp, &info);
    int np = m < n ? m : n;
    for (int p = 0; p < np; p++) d->lu_ipiv[r0 + p] = r0 + lp[p];
    if (info > 0) {
      pthread_mutex_lock(&d->mu);
      int g = r0 + info;
      if (d->failed_info == 0 || g < d->failed_info) d->failed_info = g;
      pthread_mutex_unlock(&d->mu);
    }
  } else if (k->kind == T_SWAP) {
    /* swaprows_trail!(Ac[k, j], Ac[i, j], ipiv_k, i, nb): the pivots of step
     * k whose row lies in block i, in order */
    int nb = d->lu_nb, r0 = k->step * nb, i = k->offset;
    double *A = d->ptr[k->c], *M = d->ptr[k->w2p1 - 1];
    int ncols = d->cols[k->c], lda = d->ld[k->c], np = d->rows[k->c];
    for (int p = 0; p < np; p++) {
      int g = d->lu_ipiv[r0 + p] - 1;
      if (g / nb != i) continue;
      int r = g - i * nb;
      if (A + p == M + r) continue;
      for (int cc = 0; cc < ncols; cc++) {
        double x = A[p + (size_t)cc * lda];
        A[p + (size_t)cc * lda] = M[r + (size_t)cc * lda];
        M[r + (size_t)cc * lda] = x;
      }
    }
  } else if (k->kind == T_TRSM) {
    char side = k->side, uplo = k->uplo, ta = k->ta, diag = k->diag ? k->diag : 'N';
    int m = d->rows[k->c], n = d->cols[k->c];
    int lda = d->ld[k->a], ldb = d->ld[k->c];
    double alpha = k->alpha;
    if (m > 0 && n > 0) g_dtrsm(&side, &uplo, &ta, &diag, &m, &n, &alpha, d->ptr[k->a], &lda, d->ptr[k->c], &ldb);
  } else if (k->kind == T_SYRK) {
    char uplo = k->uplo, tr = k->ta;
    int n = d->rows[k->c];
    int kk = (tr == 'N') ? d->cols[k->a] : d->rows[k->a];
    int lda = d->ld[k->a], ldc = d->ld[k->c];
    double alpha = k->alpha, beta = k->beta;
    g_dsyrk(&uplo, &tr, &n, &kk, &alpha, d->ptr[k->a], &lda, &beta, d->ptr[k->c], &ldc);
  } else {
    char ta = k->ta, tb = k->tb;
    int m = d->rows[k->c], n = d->cols[k->c];
    int kk = (ta == 'N') ? d->cols[k->a] : d->rows[k->a];
    int lda = d->ld[k->a], ldb = d->ld[k->b], ldc = d->ld[k->c];
    double alpha = k->alpha, beta = k->beta;
    if (m > 0 && n > 0) g_dgemm(&ta, &tb, &m, &n, &kk, &alpha, d->ptr[k->a], &lda, d->ptr[k->b], &ldb, &beta, d->ptr[k->c], &ldc);
  }
}

static void *worker(void *arg) {
  dag_t *d = (dag_t *)arg;
  pthread_mutex_lock(&d->mu);
  for (;;) {
    while (d->heap_n == 0 && d->done < d->ntasks) pthread_cond_wait(&d->cv, &d->mu);
    if (d->done >= d->ntasks) break;
    int t = heap_pop(d);
    int skip = d->stop_on_info && d->failed_info != 0;  /* potrf_checked! stops the region */
    pthread_mutex_unlock(&d->mu);
    if (!skip) run_task(d, t);
    pthread_mutex_lock(&d->mu);
    d->done++;
    for (int i = 0; i < d->nsucc[t]; i++) {
      int s = d->succ[t][i];
      if (--d->npred[s] == 0) heap_push(d, s);
    }
    pthread_cond_broadcast(&d->cv);
  }
  pthread_mutex_unlock(&d->mu);
  return NULL;
}

static int run_dag(dag_t *d, int ntiles, int nthreads) {
  if (!g_dgemm) return -10;
  int rc = build_edges(d, ntiles);
  if (rc) return rc;
  d->heap = malloc(sizeof(int) * (d->ntasks + 1));
  d->heap_n = 0;
  d->done = 0;
  d->failed_info = 0;
  for (int t = 0; t < d->ntasks; t++)
    if (d->npred[t] == 0) heap_push(d, t);
  pthread_mutex_init(&d->mu, NULL);
  pthread_cond_init(&d->cv, NULL);
  if (nthreads < 1) nthreads = 1;
  pthread_t *th = malloc(sizeof(pthread_t) * nthreads);
  for (int i = 0; i < nthreads; i++) pthread_create(&th[i], NULL, worker, d);
  for (int i = 0; i < nthreads; i++) pthread_join(th[i], NULL);
  free(th);
  pthread_mutex_destroy(&d->mu);
  pthread_cond_destroy(&d->cv);
  for (int t = 0; t < d->ntasks; t++) free(d->succ[t]);
  free(d->succ); free(d->nsucc); free(d->npred); free(d->heap);
  return 0;
}

static void tile_geometry(dag_t *d, double *A, int lda, int nrows, int ncols, int nbr, int nbc,
                          int base) {
  int mt = (nrows + nbr - 1) / nbr, nt = (ncols + nbc - 1) / nbc;
  for (int j = 0; j < nt; j++)
    for (int i = 0; i < mt; i++) {
      int id = base + i + j * mt;
      d->ptr[id] = A + (size_t)i * nbr + (size_t)j * nbc * lda;
      d->rows[id] = (i + 1) * nbr <= nrows ? nbr : nrows - i * nbr;
      d->cols[id] = (j + 1) * nbc <= ncols ? nbc : ncols - j * nbc;
      d->ld[id] = lda;
    }
}

/* _chol! on an n x n column-major matrix with Blocks(nb, nb); returns info
 * (LAPACK order of the first non-positive leading minor, 0 on success). */
int oracle_chol_tiled(char uplo, int n, int nb, double *A, int lda, int nthreads) {
  if (n <= 0) return 0;
  int mt = (n + nb - 1) / nb;
  int ntiles = mt * mt;
  dag_t d;
  memset(&d, 0, sizeof d);
  d.stop_on_info = 1;
  d.ptr = malloc(sizeof(double *) * ntiles);
  d.rows = malloc(sizeof(int) * ntiles);
  d.cols = malloc(sizeof(int) * ntiles);
  d.ld = malloc(sizeof(int) * ntiles);
  tile_geometry(&d, A, lda, n, n, nb, nb, 0);
  long cap = (long)mt * (mt + 1) * (mt + 2) / 6 + 2L * mt * mt + 8;
  d.tasks = malloc(sizeof(task_t) * cap);
  int nt = 0;
#define TILE(i, j) ((i) + (j) * mt)
  for (int k = 0; k < mt; k++) {
    d.tasks[nt++] = (task_t){T_POTRF, 0, uplo, 0, 0, 0, 0, -1, -1, TILE(k, k), k * nb};
    if (uplo == 'U') {
      for (int j = k + 1; j < mt; j++)
        d.tasks[nt++] = (task_t){T_TRSM, 'L', 'U', 'T', 'N', 1.0, 0, TILE(k, k), -1, TILE(k, j), 0};
      for (int m = k + 1; m < mt; m++) {
        d.tasks[nt++] = (task_t){T_SYRK, 0, 'U', 'T', 0, -1.0, 1.0, TILE(k, m), -1, TILE(m, m), 0};
        for (int j = m + 1; j < mt; j++)
          d.tasks[nt++] = (task_t){T_GEMM, 0, 0, 'T', 'N', -1.0, 1.0, TILE(k, m), TILE(k, j), TILE(m, j), 0};
      }
    } else {
      for (int m = k + 1; m < mt; m++)
        d.tasks[nt++] = (task_t){T_TRSM, 'R', 'L', 'T', 'N', 1.0, 0, TILE(k, k), -1, TILE(m, k), 0};
      for (int j = k + 1; j < mt; j++) {
        d.tasks[nt++] = (task_t){T_SYRK, 0, 'L', 'N', 0, -1.0, 1.0, TILE(j, k), -1, TILE(j, j), 0};
        for (int m = j + 1; m < mt; m++)
          d.tasks[nt++] = (task_t){T_GEMM, 0, 0, 'N', 'T', -1.0, 1.0, TILE(m, k), TILE(j, k), TILE(m, j), 0};
      }
    }
  }
#undef TILE
  d.ntasks = nt;
  int rc = run_dag(&d, ntiles, nthreads);
  int info = d.failed_info;
  free(d.ptr); free(d.rows); free(d.cols); free(d.ld); free(d.tasks);
  return rc ? rc : info;
}

/* One left-side tiled triangular solve of trsm.jl:89-140 with alpha = 1
 * (its use in ldiv!), over an n x nrhs right-hand side B blocked
 * Blocks(nb, nb).  Tiles of the factor are ids [0, mt*mt), tiles of B follow. */
static int solve_pass(char uplo, char trans, int n, int nb, double *F, int ldf, int nrhs,
                      double *B, int ldb, int nthreads) {
  int mt = (n + nb - 1) / nb, bnt = (nrhs + nb - 1) / nb;
  int ntiles = mt * mt + mt * bnt;
  dag_t d;
  memset(&d, 0, sizeof d);
  d.ptr = malloc(sizeof(double *) * ntiles);
  d.rows = malloc(sizeof(int) * ntiles);
  d.cols = malloc(sizeof(int) * ntiles);
  d.ld = malloc(sizeof(int) * ntiles);
  tile_geometry(&d, F, ldf, n, n, nb, nb, 0);
  tile_geometry(&d, B, ldb, n, nrhs, nb, nb, mt * mt);
  d.tasks = malloc(sizeof(task_t) * ((long)mt * mt * bnt + (long)mt * bnt + 8));
  int nt = 0;
#define AT(i, j) ((i) + (j) * mt)
#define BT(i, j) (mt * mt + (i) + (j) * mt)
  /* forward when op(A) is lower, backward when upper; the GEMM's transA and
   * which A tile it reads follow trsm.jl:91-140 */
  int forward = (uplo == 'U') ? (trans != 'N') : (trans == 'N');
  for (int s = 0; s < mt; s++) {
    int k = forward ? s : mt - 1 - s;
    for (int c = 0; c < bnt; c++)
      d.tasks[nt++] = (task_t){T_TRSM, 'L', uplo, trans, 'N', 1.0, 0, AT(k, k), -1, BT(k, c), 0};
    for (int s2 = s + 1; s2 < mt; s2++) {
      int m = forward ? s2 : mt - 1 - s2;
      /* A tile: U'(k->m) reads A[k,m] with 'T'; U(k->m) reads A[m,k] 'N';
       * L(k->m) reads A[m,k] 'N'; L'(k->m) reads A[k,m] 'T' */
      int atile = (trans == 'N') ? AT(m, k) : AT(k, m);
      for (int c = 0; c < bnt; c++)
        d.tasks[nt++] = (task_t){T_GEMM, 0, 0, trans, 'N', -1.0, 1.0, atile, BT(k, c), BT(m, c), 0};
    }
  }
#undef AT
#undef BT
  d.ntasks = nt;
  int rc = run_dag(&d, ntiles, nthreads);
  free(d.ptr); free(d.rows); free(d.cols); free(d.ld); free(d.tasks);
  return rc;
}

/* ldiv!(cholesky, B) for a matrix right-hand side (linalg.jl:386-403). */
int oracle_solve_tiled(char uplo, int n, int nb, double *F, int ldf, int nrhs, double *B,
                       int ldb, int nthreads) {
  int rc;
  if (uplo == 'U') {
    rc = solve_pass('U', 'T', n, nb, F, ldf, nrhs, B, ldb, nthreads);
    if (!rc) rc = solve_pass('U', 'N', n, nb, F, ldf, nrhs, B, ldb, nthreads);
  } else {
    rc = solve_pass('L', 'N', n, nb, F, ldf, nrhs, B, ldb, nthreads);
    if (!rc) rc = solve_pass('L', 'T', n, nb, F, ldf, nrhs, B, ldb, nthreads);
  }
  return rc;
}

/* lu!(A, RowMaximum()) (lu.jl:351-407 with factor_panel_lapack!) on an n x n
 * column-major matrix with Blocks(nb, nb): per step k the panel task (getrf
 * of the block column from the diagonal down, InOut on all its tiles and on
 * the step's pivots), swaprows_trail! for every other block column j and
 * every block i >= k (InOut on tiles (k, j) and (i, j), In on the pivots),
 * TRSM('L','L','N','U') of tile (k, j) and GEMM('N','N',-1) of the trailing
 * tiles.  ipiv: n global 1-based pivots.  Returns LAPACK's info (the first
 * exactly zero pivot, 1-based; the factorization continues) or < 0. */
int oracle_lu_tiled(int n, int nb, double *A, int lda, int *ipiv, int nthreads) {
  if (n <= 0) return 0;
  if (!g_dgetrf) return -11;
  int mt = (n + nb - 1) / nb;
  if (mt > 256) return -12;
  int ntiles = mt * mt + mt;  /* the tiles, then one pivot chunk per step */
  dag_t d;
  memset(&d, 0, sizeof d);
  d.stop_on_info = 0;
  d.ptr = malloc(sizeof(double *) * ntiles);
  d.rows = malloc(sizeof(int) * ntiles);
  d.cols = malloc(sizeof(int) * ntiles);
  d.ld = malloc(sizeof(int) * ntiles);
  tile_geometry(&d, A, lda, n, n, nb, nb, 0);
  for (int k = 0; k < mt; k++) {
    d.ptr[mt * mt + k] = NULL;
    d.rows[mt * mt + k] = d.cols[mt * mt + k] = d.ld[mt * mt + k] = 0;
  }
  d.lu_ipiv = ipiv;
  d.lu_tmp = malloc(sizeof(int) * n);
  d.lu_n = n;
  d.lu_nb = nb;
  long cap = (long)mt * mt * mt + 4L * mt * mt + 8;
  d.tasks = malloc(sizeof(task_t) * cap);
  int nt = 0;
#define TILE(i, j) ((i) + (j) * mt)
#define PIV(k) (mt * mt + (k))
  for (int k = 0; k < mt; k++) {
    task_t t;
    memset(&t, 0, sizeof t);
    t.kind = T_GETRF; t.a = -1; t.b = -1; t.c = TILE(k, k); t.span = mt - k;
    t.w2p1 = PIV(k) + 1; t.step = k;
    d.tasks[nt++] = t;
    for (int j = 0; j < mt; j++) {
      if (j == k) continue;
      for (int i = k; i < mt; i++) {
        memset(&t, 0, sizeof t);
        t.kind = T_SWAP; t.a = PIV(k); t.b = -1; t.c = TILE(k, j);
        t.w2p1 = (i == k) ? 0 : TILE(i, j) + 1; t.offset = i; t.step = k;
        if (i == k) t.w2p1 = TILE(k, j) + 1;  /* swaps inside tile (k, j) */
        d.tasks[nt++] = t;
      }
    }
    for (int j = k + 1; j < mt; j++) {
      memset(&t, 0, sizeof t);
      t.kind = T_TRSM; t.side = 'L'; t.uplo = 'L'; t.ta = 'N'; t.diag = 'U'; t.alpha = 1.0;
      t.a = TILE(k, k); t.b = -1; t.c = TILE(k, j);
      d.tasks[nt++] = t;
      for (int i = k + 1; i < mt; i++) {
        memset(&t, 0, sizeof t);
        t.kind = T_GEMM; t.ta = 'N'; t.tb = 'N'; t.alpha = -1.0; t.beta = 1.0;
        t.a = TILE(i, k); t.b = TILE(k, j); t.c = TILE(i, j);
        d.tasks[nt++] = t;
      }
    }
  }
#undef TILE
#undef PIV
  d.ntasks = nt;
  int rc = run_dag(&d, ntiles, nthreads);
  int info = d.failed_info;
  free(d.ptr); free(d.rows); free(d.cols); free(d.ld); free(d.tasks); free(d.lu_tmp);
  return rc ? rc : info;
}
