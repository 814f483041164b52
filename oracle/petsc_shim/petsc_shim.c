/*
 * TEST INFRASTRUCTURE ONLY -- the single-process PETSc/MPI API stand-in used to
 * compile CURVIB's poisson.c / metrics.c / implicitsolver.c unmodified into
 * oracle/_ref/.  See petsc_shim.h for the semantics.  Nothing here is linked
 * into, or called by, the product library.
 */
#include <stdarg.h>
#include <stdint.h>
#include <stddef.h>
#include "petsc_shim.h"

struct tbl {
  void *user_ptr;      /* what DMDAVecGetArray handed out */
  void **rows;         /* j-row pointers */
  void ***planes;      /* k-plane pointers */
  struct tbl *next;
};

struct _p_DM {
  PetscInt M, N, P, dof, s;
  int per[3];
  DMDALocalInfo info;
  Vec coord_g, coord_l;
  DM cda;
};

struct _p_Vec {
  double *a;
  PetscInt n;
  DM dm;
  int local; /* 1: ghosted local vector, 0: global / natural */
  struct tbl *tables;
};

#define MAXROW 64
struct mrow { int n; int col[MAXROW]; double val[MAXROW]; };
struct _p_Mat {
  int shell;
  int nrows;
  struct mrow *rows;
  void *ctx;
  PetscErrorCode (*mult)(Mat, Vec, Vec);
};

struct _p_AO { int dummy; };
static struct _p_AO g_ao;

static int verbose(void) {
  const char *e = getenv("CVB_SHIM_VERBOSE");
  return e && *e && *e != '0';
}

PetscErrorCode PetscPrintf(MPI_Comm comm, const char *fmt, ...) {
  (void)comm;
  if (verbose()) { va_list ap; va_start(ap, fmt); vfprintf(stderr, fmt, ap); va_end(ap); }
  return 0;
}
PetscErrorCode PetscFPrintf(MPI_Comm comm, FILE *f, const char *fmt, ...) {
  (void)comm; (void)f;
  if (verbose()) { va_list ap; va_start(ap, fmt); vfprintf(stderr, fmt, ap); va_end(ap); }
  return 0;
}
PetscErrorCode PetscSynchronizedPrintf(MPI_Comm comm, const char *fmt, ...) {
  (void)comm;
  if (verbose()) { va_list ap; va_start(ap, fmt); vfprintf(stderr, fmt, ap); va_end(ap); }
  return 0;
}
PetscErrorCode PetscSynchronizedFlush(MPI_Comm comm, ...) { (void)comm; return 0; }
PetscErrorCode PetscBarrier(void *obj) { (void)obj; return 0; }
PetscErrorCode PetscTime(PetscLogDouble *t) { *t = 0.0; return 0; }

int MPI_Comm_rank(MPI_Comm c, int *r) { (void)c; *r = 0; return 0; }
int MPI_Comm_size(MPI_Comm c, int *s) { (void)c; *s = 1; return 0; }
int MPI_Allreduce(const void *s, void *r, int n, MPI_Datatype t, MPI_Op o, MPI_Comm c) {
  (void)o; (void)c;
  size_t sz = (t == MPI_DOUBLE) ? sizeof(double) : sizeof(int);
  if (s != r) memmove(r, s, sz * (size_t)n);
  return 0;
}
int MPI_Bcast(void *b, int n, MPI_Datatype t, int root, MPI_Comm c) {
  (void)b; (void)n; (void)t; (void)root; (void)c;
  return 0;
}

/* ---------------------------------------------------------------- DM --- */
static void set_info(DM da) {
  DMDALocalInfo *f = &da->info;
  memset(f, 0, sizeof(*f));
  f->dim = 3; f->dof = da->dof; f->sw = da->s;
  f->mx = da->M; f->my = da->N; f->mz = da->P;
  f->xs = 0; f->ys = 0; f->zs = 0;
  f->xm = da->M; f->ym = da->N; f->zm = da->P;
  f->gxs = da->per[0] ? -da->s : 0; f->gxm = da->M + (da->per[0] ? 2 * da->s : 0);
  f->gys = da->per[1] ? -da->s : 0; f->gym = da->N + (da->per[1] ? 2 * da->s : 0);
  f->gzs = da->per[2] ? -da->s : 0; f->gzm = da->P + (da->per[2] ? 2 * da->s : 0);
  f->bx = da->per[0] ? DM_BOUNDARY_PERIODIC : DM_BOUNDARY_NONE;
  f->by = da->per[1] ? DM_BOUNDARY_PERIODIC : DM_BOUNDARY_NONE;
  f->bz = da->per[2] ? DM_BOUNDARY_PERIODIC : DM_BOUNDARY_NONE;
  f->st = DMDA_STENCIL_BOX;
  f->da = da;
}

PetscErrorCode DMDACreate3d(MPI_Comm comm, DMBoundaryType bx, DMBoundaryType by, DMBoundaryType bz,
                            DMDAStencilType st, PetscInt M, PetscInt N, PetscInt P, PetscInt m,
                            PetscInt n, PetscInt p, PetscInt dof, PetscInt s, const PetscInt *lx,
                            const PetscInt *ly, const PetscInt *lz, DM *da) {
  (void)comm; (void)st; (void)m; (void)n; (void)p; (void)lx; (void)ly; (void)lz;
  DM d = (DM)calloc(1, sizeof(struct _p_DM));
  d->M = M; d->N = N; d->P = P; d->dof = dof; d->s = s;
  d->per[0] = bx == DM_BOUNDARY_PERIODIC;
  d->per[1] = by == DM_BOUNDARY_PERIODIC;
  d->per[2] = bz == DM_BOUNDARY_PERIODIC;
  set_info(d);
  *da = d;
  return 0;
}

PetscErrorCode DMDestroy(DM *da) {
  if (!da || !*da) return 0;
  if ((*da)->coord_g) VecDestroy(&(*da)->coord_g);
  if ((*da)->coord_l) VecDestroy(&(*da)->coord_l);
  if ((*da)->cda) { DM c = (*da)->cda; free(c); }
  free(*da);
  *da = NULL;
  return 0;
}

PetscErrorCode DMDAGetLocalInfo(DM da, DMDALocalInfo *info) { *info = da->info; return 0; }

PetscErrorCode DMDAGetInfo(DM da, PetscInt *dim, PetscInt *M, PetscInt *N, PetscInt *P, PetscInt *m,
                           PetscInt *n, PetscInt *p, PetscInt *dof, PetscInt *s,
                           DMBoundaryType *bx, DMBoundaryType *by, DMBoundaryType *bz,
                           DMDAStencilType *st) {
  if (dim) *dim = 3;
  if (M) *M = da->M;
  if (N) *N = da->N;
  if (P) *P = da->P;
  if (m) *m = 1;
  if (n) *n = 1;
  if (p) *p = 1;
  if (dof) *dof = da->dof;
  if (s) *s = da->s;
  if (bx) *bx = da->info.bx;
  if (by) *by = da->info.by;
  if (bz) *bz = da->info.bz;
  if (st) *st = DMDA_STENCIL_BOX;
  return 0;
}

static PetscInt nglobal(DM da) { return da->M * da->N * da->P * da->dof; }
static PetscInt nlocal(DM da) { return da->info.gxm * da->info.gym * da->info.gzm * da->dof; }

static Vec new_vec(DM da, int local) {
  Vec v = (Vec)calloc(1, sizeof(struct _p_Vec));
  v->dm = da;
  v->local = local;
  v->n = local ? nlocal(da) : nglobal(da);
  v->a = (double *)calloc((size_t)v->n, sizeof(double));
  return v;
}

PetscErrorCode DMCreateGlobalVector(DM da, Vec *v) { *v = new_vec(da, 0); return 0; }
PetscErrorCode DMCreateLocalVector(DM da, Vec *v) { *v = new_vec(da, 1); return 0; }
PetscErrorCode DMDACreateNaturalVector(DM da, Vec *v) { *v = new_vec(da, 0); return 0; }

PetscErrorCode DMGetCoordinateDM(DM da, DM *cda) {
  if (!da->cda) {
    DM c = (DM)calloc(1, sizeof(struct _p_DM));
    *c = *da;
    c->dof = 3;
    c->coord_g = NULL; c->coord_l = NULL; c->cda = NULL;
    set_info(c);
    da->cda = c;
  }
  *cda = da->cda;
  return 0;
}

PetscErrorCode DMDASetUniformCoordinates(DM da, PetscReal x0, PetscReal x1, PetscReal y0,
                                         PetscReal y1, PetscReal z0, PetscReal z1) {
  DM cda;
  DMGetCoordinateDM(da, &cda);
  if (!da->coord_g) da->coord_g = new_vec(cda, 0);
  if (!da->coord_l) da->coord_l = new_vec(cda, 1);
  double hx = da->M > 1 ? (x1 - x0) / (da->M - 1) : 0;
  double hy = da->N > 1 ? (y1 - y0) / (da->N - 1) : 0;
  double hz = da->P > 1 ? (z1 - z0) / (da->P - 1) : 0;
  for (int k = 0; k < da->P; k++)
    for (int j = 0; j < da->N; j++)
      for (int i = 0; i < da->M; i++) {
        double *c = da->coord_g->a + 3 * ((size_t)(k * da->N + j) * da->M + i);
        c[0] = x0 + i * hx; c[1] = y0 + j * hy; c[2] = z0 + k * hz;
      }
  DMGlobalToLocalBegin(cda, da->coord_g, INSERT_VALUES, da->coord_l);
  return 0;
}

PetscErrorCode DMGetCoordinates(DM da, Vec *c) {
  if (!da->coord_g) DMDASetUniformCoordinates(da, 0, 1, 0, 1, 0, 1);
  *c = da->coord_g;
  return 0;
}
PetscErrorCode DMGetCoordinatesLocal(DM da, Vec *c) {
  if (!da->coord_l) DMDASetUniformCoordinates(da, 0, 1, 0, 1, 0, 1);
  *c = da->coord_l;
  return 0;
}

/* [k][j][i] pointer tables indexed in global coordinates. */
PetscErrorCode DMDAVecGetArray(DM da, Vec v, void *array) {
  DMDALocalInfo *f = &da->info;
  int xs, ys, zs, xm, ym, zm;
  if (v->local) { xs = f->gxs; ys = f->gys; zs = f->gzs; xm = f->gxm; ym = f->gym; zm = f->gzm; }
  else { xs = 0; ys = 0; zs = 0; xm = f->mx; ym = f->my; zm = f->mz; }
  size_t es = sizeof(double) * (size_t)da->dof;
  if ((PetscInt)((size_t)xm * ym * zm * da->dof) != v->n) {
    fprintf(stderr, "petsc_shim: DMDAVecGetArray size mismatch (%d vs %d)\n",
            (int)((size_t)xm * ym * zm * da->dof), (int)v->n);
    abort();
  }
  struct tbl *t = (struct tbl *)calloc(1, sizeof(struct tbl));
  t->rows = (void **)malloc(sizeof(void *) * (size_t)ym * zm);
  t->planes = (void ***)malloc(sizeof(void **) * (size_t)zm);
  char *base = (char *)v->a;
  for (int kk = 0; kk < zm; kk++) {
    for (int jj = 0; jj < ym; jj++)
      t->rows[kk * ym + jj] = (void *)(base + ((size_t)(kk * ym + jj) * xm) * es - (ptrdiff_t)xs * (ptrdiff_t)es);
    t->planes[kk] = (void **)(t->rows + (size_t)kk * ym) - ys;
  }
  t->user_ptr = (void *)(t->planes - zs);
  t->next = v->tables;
  v->tables = t;
  *(void **)array = t->user_ptr;
  return 0;
}

PetscErrorCode DMDAVecRestoreArray(DM da, Vec v, void *array) {
  (void)da;
  void *p = *(void **)array;
  struct tbl **pp = &v->tables;
  while (*pp) {
    if ((*pp)->user_ptr == p) {
      struct tbl *t = *pp;
      *pp = t->next;
      free(t->rows); free(t->planes); free(t);
      break;
    }
    pp = &(*pp)->next;
  }
  return 0;
}

static inline int wrapi(int i, int n) { i %= n; return i < 0 ? i + n : i; }

/* Fill every point of a ghosted local array from the owned box of `src`
 * (global layout when src_local==0, or the owned part of a local array). */
static void fill_local(DM da, const double *src, int src_local, double *dst) {
  DMDALocalInfo *f = &da->info;
  int dof = da->dof;
  for (int kk = 0; kk < f->gzm; kk++) {
    int k = wrapi(kk + f->gzs, f->mz);
    for (int jj = 0; jj < f->gym; jj++) {
      int j = wrapi(jj + f->gys, f->my);
      for (int ii = 0; ii < f->gxm; ii++) {
        int i = wrapi(ii + f->gxs, f->mx);
        size_t s;
        if (src_local)
          s = ((size_t)((k - f->gzs) * f->gym + (j - f->gys)) * f->gxm + (i - f->gxs)) * dof;
        else
          s = ((size_t)(k * f->my + j) * f->mx + i) * dof;
        size_t d = ((size_t)(kk * f->gym + jj) * f->gxm + ii) * dof;
        for (int c = 0; c < dof; c++) dst[d + c] = src[s + c];
      }
    }
  }
}

PetscErrorCode DMGlobalToLocalBegin(DM da, Vec g, InsertMode m, Vec l) {
  (void)m;
  if (!l->local) { if (g != l) memcpy(l->a, g->a, sizeof(double) * (size_t)g->n); return 0; }
  fill_local(da, g->a, g->local, l->a);
  return 0;
}
PetscErrorCode DMGlobalToLocalEnd(DM da, Vec g, InsertMode m, Vec l) {
  (void)da; (void)g; (void)m; (void)l;
  return 0;
}

PetscErrorCode DMLocalToGlobalBegin(DM da, Vec l, InsertMode m, Vec g) {
  DMDALocalInfo *f = &da->info;
  int dof = da->dof;
  if (!l->local) { if (g != l) memcpy(g->a, l->a, sizeof(double) * (size_t)g->n); return 0; }
  for (int k = 0; k < f->mz; k++)
    for (int j = 0; j < f->my; j++)
      for (int i = 0; i < f->mx; i++) {
        size_t s = ((size_t)((k - f->gzs) * f->gym + (j - f->gys)) * f->gxm + (i - f->gxs)) * dof;
        size_t d = ((size_t)(k * f->my + j) * f->mx + i) * dof;
        for (int c = 0; c < dof; c++) {
          if (m == ADD_VALUES) g->a[d + c] += l->a[s + c];
          else g->a[d + c] = l->a[s + c];
        }
      }
  return 0;
}
PetscErrorCode DMLocalToGlobalEnd(DM da, Vec l, InsertMode m, Vec g) {
  (void)da; (void)l; (void)m; (void)g;
  return 0;
}

PetscErrorCode DMLocalToLocalBegin(DM da, Vec a, InsertMode m, Vec b) {
  (void)m;
  if (!a->local || !b->local) return DMGlobalToLocalBegin(da, a, m, b);
  if (a == b) {
    double *tmp = (double *)malloc(sizeof(double) * (size_t)a->n);
    memcpy(tmp, a->a, sizeof(double) * (size_t)a->n);
    fill_local(da, tmp, 1, b->a);
    free(tmp);
  } else {
    fill_local(da, a->a, 1, b->a);
  }
  return 0;
}
PetscErrorCode DMLocalToLocalEnd(DM da, Vec a, InsertMode m, Vec b) {
  (void)da; (void)a; (void)m; (void)b;
  return 0;
}

PetscErrorCode DMDAGetAO(DM da, AO *ao) { (void)da; *ao = &g_ao; return 0; }
PetscErrorCode AOApplicationToPetsc(AO ao, PetscInt n, PetscInt *idx) {
  (void)ao; (void)n; (void)idx; /* natural ordering on one rank */
  return 0;
}
PetscErrorCode DMDAGlobalToNaturalBegin(DM da, Vec g, InsertMode m, Vec n) {
  (void)da; (void)m;
  memcpy(n->a, g->a, sizeof(double) * (size_t)g->n);
  return 0;
}
PetscErrorCode DMDAGlobalToNaturalEnd(DM da, Vec g, InsertMode m, Vec n) {
  (void)da; (void)g; (void)m; (void)n;
  return 0;
}
PetscErrorCode DMDAGetGlobalIndices(DM da, PetscInt *n, const PetscInt **idx) {
  (void)da; (void)n; (void)idx;
  return 1;
}

/* ---------------------------------------------------------------- Vec --- */
PetscErrorCode VecDuplicate(Vec v, Vec *w) { *w = new_vec(v->dm, v->local); return 0; }
PetscErrorCode VecDestroy(Vec *v) {
  if (!v || !*v) return 0;
  while ((*v)->tables) {
    struct tbl *t = (*v)->tables;
    (*v)->tables = t->next;
    free(t->rows); free(t->planes); free(t);
  }
  free((*v)->a);
  free(*v);
  *v = NULL;
  return 0;
}
PetscErrorCode VecSet(Vec v, PetscScalar a) { for (PetscInt i = 0; i < v->n; i++) v->a[i] = a; return 0; }
PetscErrorCode VecCopy(Vec x, Vec y) { memcpy(y->a, x->a, sizeof(double) * (size_t)x->n); return 0; }
PetscErrorCode VecAYPX(Vec y, PetscScalar a, Vec x) {
  for (PetscInt i = 0; i < y->n; i++) y->a[i] = x->a[i] + a * y->a[i];
  return 0;
}
PetscErrorCode VecAXPY(Vec y, PetscScalar a, Vec x) {
  for (PetscInt i = 0; i < y->n; i++) y->a[i] += a * x->a[i];
  return 0;
}
PetscErrorCode VecWAXPY(Vec w, PetscScalar a, Vec x, Vec y) {
  for (PetscInt i = 0; i < w->n; i++) w->a[i] = a * x->a[i] + y->a[i];
  return 0;
}
PetscErrorCode VecScale(Vec x, PetscScalar a) { for (PetscInt i = 0; i < x->n; i++) x->a[i] *= a; return 0; }
PetscErrorCode VecNorm(Vec x, NormType t, PetscReal *r) {
  double s = 0;
  for (PetscInt i = 0; i < x->n; i++) {
    double v = fabs(x->a[i]);
    if (t == NORM_INFINITY) s = v > s ? v : s;
    else if (t == NORM_1) s += v;
    else s += v * v;
  }
  *r = (t == NORM_2) ? sqrt(s) : s;
  return 0;
}
/* The last VecMax result, for drivers of routines that only print it. */
static double g_last_max = 0.0;
static int g_last_at = -1;
void shim_last_vecmax(double *v, int *at) { *v = g_last_max; *at = g_last_at; }
PetscErrorCode VecMax(Vec x, PetscInt *p, PetscReal *r) {
  double m = -HUGE_VAL; int at = -1;
  for (PetscInt i = 0; i < x->n; i++) if (x->a[i] > m) { m = x->a[i]; at = i; }
  if (p) *p = at;
  *r = m;
  g_last_max = m;
  g_last_at = at;
  return 0;
}
PetscErrorCode VecMin(Vec x, PetscInt *p, PetscReal *r) {
  double m = HUGE_VAL; int at = -1;
  for (PetscInt i = 0; i < x->n; i++) if (x->a[i] < m) { m = x->a[i]; at = i; }
  if (p) *p = at;
  *r = m;
  return 0;
}
PetscErrorCode VecStrideMax(Vec x, PetscInt start, PetscInt *p, PetscReal *r) {
  int dof = x->dm->dof;
  double m = -HUGE_VAL;
  for (PetscInt i = start; i < x->n; i += dof) if (x->a[i] > m) m = x->a[i];
  if (p) *p = -1;
  *r = m;
  return 0;
}
PetscErrorCode VecStrideMin(Vec x, PetscInt start, PetscInt *p, PetscReal *r) {
  int dof = x->dm->dof;
  double m = HUGE_VAL;
  for (PetscInt i = start; i < x->n; i += dof) if (x->a[i] < m) m = x->a[i];
  if (p) *p = -1;
  *r = m;
  return 0;
}
PetscErrorCode VecGetLocalSize(Vec x, PetscInt *n) { *n = x->n; return 0; }
PetscErrorCode VecGetSize(Vec x, PetscInt *n) { *n = x->n; return 0; }
PetscErrorCode VecAssemblyBegin(Vec x) { (void)x; return 0; }
PetscErrorCode VecAssemblyEnd(Vec x) { (void)x; return 0; }

static int g_arrays_out = 0;
PetscErrorCode VecGetArray(Vec x, PetscScalar **a) {
  *a = x->a;
  g_arrays_out++;
  return 0;
}
PetscErrorCode VecRestoreArray(Vec x, PetscScalar **a) {
  if (*a != x->a) return 1;
  *a = NULL;
  g_arrays_out--;
  return 0;
}
int shim_arrays_out(void) { return g_arrays_out; }
PetscErrorCode DMDAGetGhostCorners(DM da, PetscInt *x, PetscInt *y, PetscInt *z, PetscInt *m,
                                   PetscInt *n, PetscInt *p) {
  if (x) *x = da->info.gxs;
  if (y) *y = da->info.gys;
  if (z) *z = da->info.gzs;
  if (m) *m = da->info.gxm;
  if (n) *n = da->info.gym;
  if (p) *p = da->info.gzm;
  return 0;
}

#define MAXOPT 64
static struct { char name[64], value[64]; } g_opt[MAXOPT];
static int g_nopt = 0;
PetscErrorCode PetscOptionsSetValue(const char name[], const char value[]) {
  int q = 0;
  while (q < g_nopt && strcmp(g_opt[q].name, name)) q++;
  if (q == MAXOPT || strlen(name) >= 64 || (value && strlen(value) >= 64)) return 1;
  if (q == g_nopt) g_nopt++;
  strcpy(g_opt[q].name, name);
  strcpy(g_opt[q].value, value ? value : "");
  return 0;
}
PetscErrorCode PetscOptionsClear(void) { g_nopt = 0; return 0; }
static const char *opt_find(const char pre[], const char name[]) {
  char full[160];
  /* PETSc inserts the prefix after the leading dash */
  snprintf(full, sizeof full, "-%s%s", pre ? pre : "", name[0] == '-' ? name + 1 : name);
  for (int q = 0; q < g_nopt; q++)
    if (!strcmp(g_opt[q].name, full)) return g_opt[q].value;
  return NULL;
}
PetscErrorCode PetscOptionsGetString(const char pre[], const char name[], char s[], size_t len,
                                     PetscBool *set) {
  const char *v = opt_find(pre, name);
  if (set) *set = v ? PETSC_TRUE : PETSC_FALSE;
  if (v && len) { strncpy(s, v, len - 1); s[len - 1] = 0; }
  return 0;
}
PetscErrorCode PetscOptionsGetReal(const char pre[], const char name[], PetscReal *r, PetscBool *set) {
  const char *v = opt_find(pre, name);
  if (set) *set = v ? PETSC_TRUE : PETSC_FALSE;
  if (v) *r = strtod(v, NULL);
  return 0;
}
PetscErrorCode PetscOptionsGetInt(const char pre[], const char name[], PetscInt *r, PetscBool *set) {
  const char *v = opt_find(pre, name);
  if (set) *set = v ? PETSC_TRUE : PETSC_FALSE;
  if (v) *r = (PetscInt)strtol(v, NULL, 10);
  return 0;
}

PetscErrorCode VecGetArray3d(Vec x, PetscInt m, PetscInt n, PetscInt p, PetscInt ms, PetscInt ns,
                             PetscInt ps, PetscScalar ****a) {
  (void)ms; (void)ns; (void)ps;
  double ***pl = (double ***)malloc(sizeof(double **) * (size_t)m);
  double **rw = (double **)malloc(sizeof(double *) * (size_t)m * n);
  for (int k = 0; k < m; k++) {
    pl[k] = rw + (size_t)k * n;
    for (int j = 0; j < n; j++) rw[(size_t)k * n + j] = x->a + ((size_t)k * n + j) * p;
  }
  *a = pl;
  return 0;
}
PetscErrorCode VecRestoreArray3d(Vec x, PetscInt m, PetscInt n, PetscInt p, PetscInt ms,
                                 PetscInt ns, PetscInt ps, PetscScalar ****a) {
  (void)x; (void)m; (void)n; (void)p; (void)ms; (void)ns; (void)ps;
  if (*a) { free((*a)[0]); free(*a); }
  *a = NULL;
  return 0;
}

struct _p_VecScatter { int dummy; };
PetscErrorCode VecScatterCreateToZero(Vec x, VecScatter *ctx, Vec *out) {
  *ctx = (VecScatter)calloc(1, sizeof(struct _p_VecScatter));
  *out = new_vec(x->dm, x->local);
  return 0;
}
PetscErrorCode VecScatterBegin(VecScatter ctx, Vec x, Vec y, InsertMode m, ScatterMode s) {
  (void)ctx; (void)m; (void)s;
  memcpy(y->a, x->a, sizeof(double) * (size_t)x->n);
  return 0;
}
PetscErrorCode VecScatterEnd(VecScatter ctx, Vec x, Vec y, InsertMode m, ScatterMode s) {
  (void)ctx; (void)x; (void)y; (void)m; (void)s;
  return 0;
}
PetscErrorCode VecScatterDestroy(VecScatter *ctx) { free(*ctx); *ctx = NULL; return 0; }

/* ---------------------------------------------------------------- Mat --- */
PetscErrorCode MatCreateAIJ(MPI_Comm comm, PetscInt m, PetscInt n, PetscInt M, PetscInt N,
                            PetscInt dnz, const PetscInt *dnnz, PetscInt onz,
                            const PetscInt *onnz, Mat *A) {
  (void)comm; (void)n; (void)N; (void)dnz; (void)dnnz; (void)onz; (void)onnz; (void)m;
  Mat a = (Mat)calloc(1, sizeof(struct _p_Mat));
  a->nrows = M;
  a->rows = (struct mrow *)calloc((size_t)M, sizeof(struct mrow));
  *A = a;
  return 0;
}
PetscErrorCode MatZeroEntries(Mat A) {
  for (int r = 0; r < A->nrows; r++)
    for (int c = 0; c < A->rows[r].n; c++) A->rows[r].val[c] = 0.0;
  return 0;
}
PetscErrorCode MatSetValues(Mat A, PetscInt m, const PetscInt *rows, PetscInt n,
                            const PetscInt *cols, const PetscScalar *v, InsertMode mode) {
  for (int a = 0; a < m; a++) {
    struct mrow *r = &A->rows[rows[a]];
    for (int b = 0; b < n; b++) {
      int c = cols[b], at = -1;
      for (int q = 0; q < r->n; q++) if (r->col[q] == c) { at = q; break; }
      if (at < 0) {
        if (r->n >= MAXROW) { fprintf(stderr, "petsc_shim: row overflow\n"); abort(); }
        at = r->n++;
        r->col[at] = c;
        r->val[at] = 0.0;
      }
      double x = v[(size_t)a * n + b];
      if (mode == ADD_VALUES) r->val[at] += x;
      else r->val[at] = x;
    }
  }
  return 0;
}
PetscErrorCode MatAssemblyBegin(Mat A, MatAssemblyType t) { (void)A; (void)t; return 0; }
PetscErrorCode MatAssemblyEnd(Mat A, MatAssemblyType t) { (void)A; (void)t; return 0; }
PetscErrorCode MatDestroy(Mat *A) {
  if (!A || !*A) return 0;
  free((*A)->rows);
  free(*A);
  *A = NULL;
  return 0;
}
PetscErrorCode MatMult(Mat A, Vec x, Vec y) {
  if (A->shell) return A->mult(A, x, y);
  for (int r = 0; r < A->nrows; r++) {
    double s = 0;
    for (int q = 0; q < A->rows[r].n; q++) s += A->rows[r].val[q] * x->a[A->rows[r].col[q]];
    y->a[r] = s;
  }
  return 0;
}
PetscErrorCode MatCreateShell(MPI_Comm comm, PetscInt m, PetscInt n, PetscInt M, PetscInt N,
                              void *ctx, Mat *A) {
  (void)comm; (void)m; (void)n; (void)N;
  Mat a = (Mat)calloc(1, sizeof(struct _p_Mat));
  a->shell = 1;
  a->nrows = M;
  a->ctx = ctx;
  *A = a;
  return 0;
}
PetscErrorCode MatShellSetOperation(Mat A, MatOperation op, void (*f)(void)) {
  if (op == MATOP_MULT) A->mult = (PetscErrorCode(*)(Mat, Vec, Vec))f;
  return 0;
}
PetscErrorCode MatShellGetContext(Mat A, void *ctx) { *(void **)ctx = A->ctx; return 0; }

/* Shim-only accessors used by the harness. */
int shim_mat_rows(Mat A) { return A->nrows; }
int shim_mat_row(Mat A, int r, const int **cols, const double **vals) {
  *cols = A->rows[r].col;
  *vals = A->rows[r].val;
  return A->rows[r].n;
}
double *shim_vec_data(Vec v) { return v->a; }
int shim_vec_size(Vec v) { return v->n; }

/* --------------------------------------------------- inert Krylov objects --- */
struct _p_MatNullSpace { int dummy; };
PetscErrorCode MatNullSpaceCreate(MPI_Comm c, PetscBool has_cnst, PetscInt n, const Vec *vecs,
                                  MatNullSpace *sp) {
  (void)c; (void)has_cnst; (void)n; (void)vecs;
  *sp = (MatNullSpace)calloc(1, sizeof(struct _p_MatNullSpace));
  return 0;
}
PetscErrorCode MatNullSpaceSetFunction(MatNullSpace sp, PetscErrorCode (*f)(MatNullSpace, Vec, void *),
                                       void *ctx) {
  (void)sp; (void)f; (void)ctx;
  return 0;
}
PetscErrorCode MatNullSpaceDestroy(MatNullSpace *sp) { free(*sp); *sp = NULL; return 0; }
PetscErrorCode MatSetNullSpace(Mat A, MatNullSpace sp) { (void)A; (void)sp; return 0; }

/* ---- binary viewer: VecView / VecLoad in PETSc's published binary layout
 * (big-endian int32 class id 1211214, int32 length, then the values as
 * big-endian doubles; with a block size above 1 a "<file>.info" holding
 * "-vecload_block_size <bs>").  A one-rank DMDA vector is written in its
 * [k][j][i] order with the DMDA's dof as block size.  Files are opened in the
 * directory shim_set_viewer_dir names (the harness points it at a test's
 * scratch directory; the reference names files relative to its cwd). */
struct _p_PetscViewer {
  FILE *f;
  int mode;
  char path[512];
};
static char g_viewer_dir[400] = ".";
void shim_set_viewer_dir(const char *dir) {
  snprintf(g_viewer_dir, sizeof g_viewer_dir, "%s", dir && *dir ? dir : ".");
}
PetscErrorCode PetscViewerBinaryOpen(MPI_Comm comm, const char name[], PetscFileMode mode, PetscViewer *v) {
  (void)comm;
  PetscViewer p = (PetscViewer)calloc(1, sizeof(*p));
  if (!p) return 1;
  snprintf(p->path, sizeof p->path, "%s/%s", g_viewer_dir, name);
  p->mode = mode;
  p->f = fopen(p->path, mode == FILE_MODE_WRITE ? "wb" : "rb");
  if (!p->f) { free(p); *v = NULL; return 1; }
  *v = p;
  return 0;
}
PetscErrorCode PetscViewerDestroy(PetscViewer *v) {
  if (v && *v) {
    if ((*v)->f) fclose((*v)->f);
    free(*v);
    *v = NULL;
  }
  return 0;
}
static void put_be32(FILE *f, uint32_t x) {
  unsigned char b[4] = {(unsigned char)(x >> 24), (unsigned char)(x >> 16), (unsigned char)(x >> 8), (unsigned char)x};
  fwrite(b, 1, 4, f);
}
static int get_be32(FILE *f, uint32_t *x) {
  unsigned char b[4];
  if (fread(b, 1, 4, f) != 4) return 1;
  *x = ((uint32_t)b[0] << 24) | ((uint32_t)b[1] << 16) | ((uint32_t)b[2] << 8) | b[3];
  return 0;
}
PetscErrorCode VecView(Vec x, PetscViewer v) {
  if (!v || !v->f || v->mode != FILE_MODE_WRITE) return 1;
  put_be32(v->f, 1211214u);
  put_be32(v->f, (uint32_t)x->n);
  for (PetscInt q = 0; q < x->n; q++) {
    uint64_t u;
    memcpy(&u, &x->a[q], 8);
    unsigned char b[8];
    for (int t = 0; t < 8; t++) b[t] = (unsigned char)(u >> (56 - 8 * t));
    fwrite(b, 1, 8, v->f);
  }
  const int bs = x->dm ? (int)x->dm->dof : 1;
  if (bs > 1) {
    char info[520];
    snprintf(info, sizeof info, "%s.info", v->path);
    FILE *g = fopen(info, "w");
    if (!g) return 1;
    fprintf(g, "-vecload_block_size %d\n", bs);
    fclose(g);
  }
  return 0;
}
PetscErrorCode VecLoad(Vec x, PetscViewer v) {
  if (!v || !v->f || v->mode != FILE_MODE_READ) return 1;
  uint32_t id, n;
  if (get_be32(v->f, &id) || id != 1211214u || get_be32(v->f, &n) || (PetscInt)n != x->n) return 1;
  for (PetscInt q = 0; q < x->n; q++) {
    unsigned char b[8];
    if (fread(b, 1, 8, v->f) != 8) return 1;
    uint64_t u = 0;
    for (int t = 0; t < 8; t++) u = (u << 8) | b[t];
    memcpy(&x->a[q], &u, 8);
  }
  return 0;
}
PetscErrorCode PetscOptionsClearValue(const char name[]) {
  for (int q = 0; q < g_nopt; q++)
    if (!strcmp(g_opt[q].name, name)) {
      g_opt[q] = g_opt[--g_nopt];
      break;
    }
  return 0;
}
