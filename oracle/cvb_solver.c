/*
 * TEST INFRASTRUCTURE ONLY: the CPU baseline of the solve -- the reference's
 * algorithm (PoissonSolver_MG, poisson.c:1775-2017) restated without PETSc:
 *
 *   - the operator of every level is the assembled PoissonLHSNew matrix
 *     (orc_lhs_csr, rebuilt with the restricted nvert as the reference does);
 *   - KSP FGMRES(restart) right-preconditioned (control.dat: -ps_ksp_type fgmres),
 *     classical Gram-Schmidt without refinement (PETSc's default);
 *   - PCMG V-cycle, multiplicative, with MyRestriction / MyInterpolation
 *     transfers (poisson.c:1845-1877);
 *   - level smoothers: Richardson (control.dat -ps_mg_levels_N_ksp_type richardson)
 *     preconditioned by block Jacobi with ILU(0) in each block
 *     (PCBJACOBI, poisson.c:1896); one block per thread, as one block per MPI
 *     rank in the reference, over contiguous k-slabs of rows;
 *   - coarse solve: preonly + block Jacobi / ILU(0) (poisson.c:1912-1942);
 *   - convergence on the unpreconditioned residual ||b - A x|| <= rtol ||b||.
 *
 * Used only as bench.py's CPU-baseline leg and by tests; OpenMP over rows.
 */
#include <math.h>
#include <omp.h>
#include <stdlib.h>
#include <string.h>

#include "cvb_oracle.h"

typedef struct {
  int n;
  int *rp, *ci;
  double *v;
  /* block-Jacobi ILU(0): per block, factors stored in a copy of the block's rows */
  int nb;
  int *bstart;       /* [nb+1] row ranges */
  int *lrp, *lci;    /* block-local CSR (columns inside the block only) */
  double *lu;        /* ILU(0) factors in the block-local pattern */
  int *diag;         /* position of the diagonal in each local row */
} orc_mat;

typedef struct {
  int nlevels;
  orc_mat A[16];
  const orc_level *L[16];
  double *r[16], *e[16], *t[16];
  int nu;            /* Richardson iterations per smoothing */
} orc_mg;

static void mat_from_level(orc_mat *M, const orc_level *L) {
  int n = L->mx * L->my * L->mz;
  int cap = 19 * n + 16;
  M->n = n;
  M->rp = (int *)malloc(sizeof(int) * (n + 1));
  M->ci = (int *)malloc(sizeof(int) * cap);
  M->v = (double *)malloc(sizeof(double) * cap);
  orc_lhs_csr(L, M->rp, M->ci, M->v, cap);
}

static int cmp_int(const void *a, const void *b) { return *(const int *)a - *(const int *)b; }

/* ILU(0) of each diagonal block (rows/cols in [s,e)), couplings outside dropped. */
static void bjacobi_ilu(orc_mat *M, int nb, double shift) {
  int n = M->n;
  M->nb = nb;
  M->bstart = (int *)malloc(sizeof(int) * (nb + 1));
  for (int b = 0; b <= nb; b++) M->bstart[b] = (int)((long long)n * b / nb);
  M->lrp = (int *)malloc(sizeof(int) * (n + 1));
  M->lci = (int *)malloc(sizeof(int) * M->rp[n]);
  M->lu = (double *)malloc(sizeof(double) * M->rp[n]);
  M->diag = (int *)malloc(sizeof(int) * n);
  /* local pattern, sorted columns */
  int w = 0;
  M->lrp[0] = 0;
  for (int b = 0; b < nb; b++) {
    int s = M->bstart[b], e = M->bstart[b + 1];
    for (int r = s; r < e; r++) {
      int st = w;
      for (int q = M->rp[r]; q < M->rp[r + 1]; q++)
        if (M->ci[q] >= s && M->ci[q] < e) { M->lci[w] = M->ci[q]; M->lu[w] = M->v[q]; w++; }
      /* sort by column (insertion sort on <= 19 entries) */
      for (int a = st + 1; a < w; a++) {
        int c = M->lci[a]; double v = M->lu[a]; int z = a - 1;
        while (z >= st && M->lci[z] > c) { M->lci[z + 1] = M->lci[z]; M->lu[z + 1] = M->lu[z]; z--; }
        M->lci[z + 1] = c; M->lu[z + 1] = v;
      }
      M->lrp[r + 1] = w;
      M->diag[r] = -1;
      for (int q = st; q < w; q++) if (M->lci[q] == r) M->diag[r] = q;
    }
  }
  (void)cmp_int;
#pragma omp parallel for schedule(static, 1)
  for (int b = 0; b < nb; b++) {
    int s = M->bstart[b], e = M->bstart[b + 1];
    for (int i = s; i < e; i++) {
      for (int qk = M->lrp[i]; qk < M->lrp[i + 1] && M->lci[qk] < i; qk++) {
        int k = M->lci[qk];
        double piv = M->lu[M->diag[k]];
        if (fabs(piv) < shift) piv = piv < 0 ? -shift : shift;
        double f = M->lu[qk] / piv;
        M->lu[qk] = f;
        /* row_i -= f * row_k on the pattern of row i, columns > k */
        int qi = qk + 1;
        for (int qq = M->diag[k] + 1; qq < M->lrp[k + 1]; qq++) {
          int c = M->lci[qq];
          while (qi < M->lrp[i + 1] && M->lci[qi] < c) qi++;
          if (qi < M->lrp[i + 1] && M->lci[qi] == c) M->lu[qi] -= f * M->lu[qq];
        }
      }
    }
  }
}

/* z = (LU)^-1 r block by block */
static void ilu_solve(const orc_mat *M, const double *r, double *z) {
#pragma omp parallel for schedule(static, 1)
  for (int b = 0; b < M->nb; b++) {
    int s = M->bstart[b], e = M->bstart[b + 1];
    for (int i = s; i < e; i++) {
      double v = r[i];
      for (int q = M->lrp[i]; q < M->diag[i]; q++) v -= M->lu[q] * z[M->lci[q]];
      z[i] = v;
    }
    for (int i = e - 1; i >= s; i--) {
      double v = z[i];
      for (int q = M->diag[i] + 1; q < M->lrp[i + 1]; q++) v -= M->lu[q] * z[M->lci[q]];
      double d = M->lu[M->diag[i]];
      z[i] = v / (fabs(d) > 1e-300 ? d : 1e-10);
    }
  }
}

static void spmv(const orc_mat *M, const double *x, double *y) {
#pragma omp parallel for schedule(static)
  for (int r = 0; r < M->n; r++) {
    double s = 0.0;
    for (int q = M->rp[r]; q < M->rp[r + 1]; q++) s += M->v[q] * x[M->ci[q]];
    y[r] = s;
  }
}

static double dot(int n, const double *a, const double *b) {
  double s = 0.0;
#pragma omp parallel for reduction(+ : s) schedule(static)
  for (int i = 0; i < n; i++) s += a[i] * b[i];
  return s;
}

/* Richardson(nu) with the block-ILU preconditioner, from x (zero when zero_guess). */
static void smooth(orc_mg *G, int l, const double *b, double *x, int zero_guess) {
  orc_mat *M = &G->A[l];
  int n = M->n;
  double *r = G->t[l];
  double *z = (double *)malloc(sizeof(double) * n);
  for (int it = 0; it < G->nu; it++) {
    if (zero_guess && it == 0) {
      ilu_solve(M, b, z);
#pragma omp parallel for
      for (int i = 0; i < n; i++) x[i] = z[i];
      continue;
    }
    spmv(M, x, r);
#pragma omp parallel for
    for (int i = 0; i < n; i++) r[i] = b[i] - r[i];
    ilu_solve(M, r, z);
#pragma omp parallel for
    for (int i = 0; i < n; i++) x[i] += z[i];
  }
  free(z);
}

static void vcycle(orc_mg *G, int l, const double *b, double *x) {
  orc_mat *M = &G->A[l];
  int n = M->n;
  if (l == 0) { ilu_solve(M, b, x); return; }
  smooth(G, l, b, x, 1);
  double *r = G->t[l];
  spmv(M, x, r);
#pragma omp parallel for
  for (int i = 0; i < n; i++) r[i] = b[i] - r[i];
  orc_restrict(G->L[l], G->L[l - 1], r, G->r[l - 1]);
  vcycle(G, l - 1, G->r[l - 1], G->e[l - 1]);
  double *p = (double *)malloc(sizeof(double) * n);
  orc_interpolate(G->L[l - 1], G->L[l], G->e[l - 1], p);
#pragma omp parallel for
  for (int i = 0; i < n; i++) x[i] += p[i];
  free(p);
  smooth(G, l, b, x, 0);
}

/* Builds the hierarchy (operators + ILU), solves, reports times.  levels[0] is
 * the coarsest.  Returns iterations; *relres the final true relative residual. */
int orc_solve_mg(int nlevels, const orc_level *const *levels, const double *b, double *x, double rtol,
                 int max_it, int restart, int nu, int threads, double *relres, double *setup_s,
                 double *solve_s) {
  if (threads > 0) omp_set_num_threads(threads);
  int nth = omp_get_max_threads();
  double t0 = omp_get_wtime();
  orc_mg G;
  memset(&G, 0, sizeof(G));
  G.nlevels = nlevels;
  G.nu = nu;
  for (int l = 0; l < nlevels; l++) {
    G.L[l] = levels[l];
    mat_from_level(&G.A[l], levels[l]);
    bjacobi_ilu(&G.A[l], nth < G.A[l].n ? nth : 1, 1e-10);
    int n = G.A[l].n;
    G.r[l] = (double *)calloc(n, sizeof(double));
    G.e[l] = (double *)calloc(n, sizeof(double));
    G.t[l] = (double *)calloc(n, sizeof(double));
  }
  double t1 = omp_get_wtime();
  orc_mat *A = &G.A[nlevels - 1];
  int n = A->n, m = restart;
  double **V = (double **)malloc(sizeof(double *) * (m + 1));
  double **Z = (double **)malloc(sizeof(double *) * m);
  for (int q = 0; q <= m; q++) V[q] = (double *)malloc(sizeof(double) * n);
  for (int q = 0; q < m; q++) Z[q] = (double *)malloc(sizeof(double) * n);
  double *H = (double *)calloc((size_t)(m + 1) * m, sizeof(double));
  double *cs = (double *)malloc(sizeof(double) * m), *sn = (double *)malloc(sizeof(double) * m);
  double *g = (double *)malloc(sizeof(double) * (m + 1)), *y = (double *)malloc(sizeof(double) * m);
  double *r = (double *)malloc(sizeof(double) * n), *w = (double *)malloc(sizeof(double) * n);
  memset(x, 0, sizeof(double) * n);
  double bn = sqrt(dot(n, b, b));
  memcpy(r, b, sizeof(double) * n);
  double beta = bn;
  int total = 0;
  while (beta > rtol * bn && total < max_it) {
#pragma omp parallel for
    for (int i = 0; i < n; i++) V[0][i] = r[i] / beta;
    for (int q = 0; q <= m; q++) g[q] = 0.0;
    g[0] = beta;
    int j = 0;
    for (; j < m && total < max_it; j++) {
      memset(Z[j], 0, sizeof(double) * n);
      vcycle(&G, nlevels - 1, V[j], Z[j]);
      spmv(A, Z[j], w);
      for (int q = 0; q <= j; q++) H[q * m + j] = dot(n, V[q], w);
      for (int q = 0; q <= j; q++) {
        double h = H[q * m + j];
#pragma omp parallel for
        for (int i = 0; i < n; i++) w[i] -= h * V[q][i];
      }
      double hn = sqrt(dot(n, w, w));
      H[(j + 1) * m + j] = hn;
      total++;
      if (hn > 0) {
#pragma omp parallel for
        for (int i = 0; i < n; i++) V[j + 1][i] = w[i] / hn;
      }
      for (int q = 0; q < j; q++) {
        double t = cs[q] * H[q * m + j] + sn[q] * H[(q + 1) * m + j];
        H[(q + 1) * m + j] = -sn[q] * H[q * m + j] + cs[q] * H[(q + 1) * m + j];
        H[q * m + j] = t;
      }
      double a = H[j * m + j], bb = H[(j + 1) * m + j], rr = hypot(a, bb);
      cs[j] = rr > 0 ? a / rr : 1.0;
      sn[j] = rr > 0 ? bb / rr : 0.0;
      H[j * m + j] = rr;
      H[(j + 1) * m + j] = 0.0;
      g[j + 1] = -sn[j] * g[j];
      g[j] = cs[j] * g[j];
      if (fabs(g[j + 1]) <= rtol * bn || hn == 0.0) { j++; break; }
    }
    for (int q = j - 1; q >= 0; q--) {
      double t = g[q];
      for (int c = q + 1; c < j; c++) t -= H[q * m + c] * y[c];
      y[q] = t / H[q * m + q];
    }
    for (int q = 0; q < j; q++) {
      double yq = y[q];
#pragma omp parallel for
      for (int i = 0; i < n; i++) x[i] += yq * Z[q][i];
    }
    spmv(A, x, w);
#pragma omp parallel for
    for (int i = 0; i < n; i++) r[i] = b[i] - w[i];
    beta = sqrt(dot(n, r, r));
  }
  double t2 = omp_get_wtime();
  *relres = bn > 0 ? beta / bn : 0.0;
  *setup_s = t1 - t0;
  *solve_s = t2 - t1;
  for (int q = 0; q <= m; q++) free(V[q]);
  for (int q = 0; q < m; q++) free(Z[q]);
  free(V); free(Z); free(H); free(cs); free(sn); free(g); free(y); free(r); free(w);
  for (int l = 0; l < nlevels; l++) {
    free(G.A[l].rp); free(G.A[l].ci); free(G.A[l].v);
    free(G.A[l].bstart); free(G.A[l].lrp); free(G.A[l].lci); free(G.A[l].lu); free(G.A[l].diag);
    free(G.r[l]); free(G.e[l]); free(G.t[l]);
  }
  return total;
}
