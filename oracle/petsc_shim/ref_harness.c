/*
 * TEST INFRASTRUCTURE ONLY.  Drives CURVIB's own poisson.c / metrics.c /
 * implicitsolver.c (compiled unmodified against the API shim) on the CPU so the
 * parity tests can compare against the reference's exact arithmetic.
 *
 * The level set-up mirrors MG_Initial (init.c:296-1060) for one block on one
 * rank: level sizes as MGDACreate (init.c:78-107), ghost width 3 when any
 * direction is periodic else 2 (init.c:116,155), coordinates injected fine ->
 * coarse (init.c:786-828), then FormMetrics (metrics.c:4) and, with periodic
 * directions, Update_Metrics_PBC (implicitsolver.c:2174).  The exported entry
 * points then call the reference functions named in each comment.
 *
 * Arrays cross this interface as the owned box [mz][my][mx] (x fastest), with
 * 3-vectors interleaved (x,y,z), i.e. exactly a PETSc global vector.
 */
#include "variables.h"
#include <string.h>
#include <unistd.h>

/* Globals the reference sources expect main.c to define. */
PetscInt block_number = 1, immersed = 0, MHV = 0, LV = 0, tistart = 0;
/* ti (the time step) is main.c's own: its object keeps that symbol global for
 * the restart routines, which name their files by it. */
extern PetscInt ti;
PetscInt NumberOfBodies = 1, blank = 0;
PetscInt imp_MAX_IT = 1, implicit_type = 0;
PetscReal imp_atol = 1e-8, imp_rtol = 1e-2, imp_stol = 1e-8;
PetscInt mg_idx = 0, mg_preItr = 1, mg_poItr = 1, mg_MAX_IT = 1;
int i_periodic = 0, j_periodic = 0, k_periodic = 0;
int ii_periodic = 0, jj_periodic = 0, kk_periodic = 0;
int les = 0, wallfunction = 0, rans = 0;
int i_homo_filter = 0, j_homo_filter = 0, k_homo_filter = 0;
int testfilter_ik = 0, testfilter_1d = 0;
int clark = 0;

/* Projection ends by calling these two (poisson.c:2902-2904); they belong to
 * the caller's side of the boundary, so the harness compares Ucont before them. */
PetscErrorCode Contra2Cart(UserCtx *user) { (void)user; return 0; }
PetscErrorCode GhostNodeVelocity(UserCtx *user) { (void)user; return 0; }
/* The reference's own two (rhs.c:25, bcs.c:3645), renamed in their objects by
 * oracle/build_ref.sh so that they do not collide with the inert pair above. */
PetscErrorCode cvbref_Contra2Cart(UserCtx *user);
PetscErrorCode cvbref_GhostNodeVelocity(UserCtx *user);
PetscErrorCode ibm_search_advanced(UserCtx *user, IBMNodes *ibm, PetscInt ibi);

PetscErrorCode FormMetrics(UserCtx *user);
PetscErrorCode Update_Metrics_PBC(UserCtx *user);
PetscErrorCode PoissonLHSNew(UserCtx *user);
PetscErrorCode PoissonRHS(UserCtx *user, Vec B);
PetscErrorCode VolumeFlux_rev(UserCtx *user, PetscReal *ibm_Flux, PetscReal *ibm_Area, PetscInt flg);
PetscErrorCode MyNvertRestriction(UserCtx *user_h, UserCtx *user_c);
PetscErrorCode FullyBlocked(UserCtx *user);
PetscErrorCode MyRestriction(Mat A, Vec X, Vec F);
PetscErrorCode MyInterpolation(Mat A, Vec X, Vec F);
PetscErrorCode PoissonNullSpaceFunction(MatNullSpace nullsp, Vec X, void *ctx);
PetscErrorCode UpdatePressure(UserCtx *user);
PetscErrorCode Projection(UserCtx *user);
PetscErrorCode GridRestriction(PetscInt i, PetscInt j, PetscInt k, PetscInt *ih, PetscInt *jh,
                               PetscInt *kh, UserCtx *user);

int shim_mat_rows(Mat A);
int shim_mat_row(Mat A, int r, const int **cols, const double **vals);
double *shim_vec_data(Vec v);
int shim_vec_size(Vec v);

static UserMG g_mg;
static int g_ready = 0;

static UserCtx *U(int l) { return &g_mg.mgctx[l].user[0]; }

static void make_vectors(UserCtx *u, int finest) {
  DMCreateGlobalVector(u->fda, &u->Csi);
  VecDuplicate(u->Csi, &u->Eta); VecDuplicate(u->Csi, &u->Zet);
  VecDuplicate(u->Csi, &u->ICsi); VecDuplicate(u->Csi, &u->IEta); VecDuplicate(u->Csi, &u->IZet);
  VecDuplicate(u->Csi, &u->JCsi); VecDuplicate(u->Csi, &u->JEta); VecDuplicate(u->Csi, &u->JZet);
  VecDuplicate(u->Csi, &u->KCsi); VecDuplicate(u->Csi, &u->KEta); VecDuplicate(u->Csi, &u->KZet);
  VecDuplicate(u->Csi, &u->Cent); VecDuplicate(u->Csi, &u->GridSpace);
  VecDuplicate(u->Csi, &u->Ucont);
  VecDuplicate(u->Csi, &u->Ucat);
  VecDuplicate(u->Csi, &u->Bcs.Ubcs);
  (void)finest;
  DMCreateGlobalVector(u->da, &u->Aj);
  VecDuplicate(u->Aj, &u->IAj); VecDuplicate(u->Aj, &u->JAj); VecDuplicate(u->Aj, &u->KAj);
  VecDuplicate(u->Aj, &u->Nvert); VecDuplicate(u->Aj, &u->Phi); VecDuplicate(u->Aj, &u->P);
  VecDuplicate(u->Aj, &u->Nvert_o);
  DMCreateLocalVector(u->fda, &u->lCsi);
  VecDuplicate(u->lCsi, &u->lEta); VecDuplicate(u->lCsi, &u->lZet);
  VecDuplicate(u->lCsi, &u->lICsi); VecDuplicate(u->lCsi, &u->lIEta); VecDuplicate(u->lCsi, &u->lIZet);
  VecDuplicate(u->lCsi, &u->lJCsi); VecDuplicate(u->lCsi, &u->lJEta); VecDuplicate(u->lCsi, &u->lJZet);
  VecDuplicate(u->lCsi, &u->lKCsi); VecDuplicate(u->lCsi, &u->lKEta); VecDuplicate(u->lCsi, &u->lKZet);
  VecDuplicate(u->lCsi, &u->lGridSpace); VecDuplicate(u->lCsi, &u->lCent);
  VecDuplicate(u->lCsi, &u->Centx); VecDuplicate(u->lCsi, &u->Centy); VecDuplicate(u->lCsi, &u->Centz);
  VecDuplicate(u->lCsi, &u->lUcont);
  VecDuplicate(u->lCsi, &u->lUcat);
  DMCreateLocalVector(u->da, &u->lAj);
  VecDuplicate(u->lAj, &u->lIAj); VecDuplicate(u->lAj, &u->lJAj); VecDuplicate(u->lAj, &u->lKAj);
  VecDuplicate(u->lAj, &u->lNvert); VecDuplicate(u->lAj, &u->lPhi); VecDuplicate(u->lAj, &u->lP);
  VecDuplicate(u->lAj, &u->lNvert_o);
}

void ref_free(void) {
  /* test-only: the process exits after use, leaks are harmless */
  g_ready = 0;
}

/* coords: KM*JM*IM nodes, x fastest, (x,y,z) interleaved. */
int ref_init(int nlevels, int IM, int JM, int KM, const int *bctype, int isc, int jsc, int ksc,
             const double *coords) {
  memset(&g_mg, 0, sizeof(g_mg));
  g_mg.mglevels = nlevels;
  g_mg.mgctx = (MGCtx *)calloc((size_t)nlevels, sizeof(MGCtx));
  for (int l = 0; l < nlevels; l++) {
    g_mg.mgctx[l].user = (UserCtx *)calloc(1, sizeof(UserCtx));
    g_mg.mgctx[l].thislevel = l;
    UserCtx *u = U(l);
    for (int q = 0; q < 6; q++) u->bctype[q] = bctype[q];
    u->isc = isc; u->jsc = jsc; u->ksc = ksc;
    u->cgrid = 0;
    u->st = 1.0; u->dt = 1.0;
    u->thislevel = l; u->mglevels = nlevels; u->_this = 0;
    u->assignedA = PETSC_FALSE; u->multinullspace = PETSC_FALSE;
  }
  U(nlevels - 1)->IM = IM; U(nlevels - 1)->JM = JM; U(nlevels - 1)->KM = KM;
  for (int l = nlevels - 2; l >= 0; l--) {
    UserCtx *u = U(l), *h = U(l + 1);
    u->IM = u->isc ? h->IM : (h->IM + 1) / 2;
    u->JM = u->jsc ? h->JM : (h->JM + 1) / 2;
    u->KM = u->ksc ? h->KM : (h->KM + 1) / 2;
  }
  int per = bctype[0] == 7 || bctype[2] == 7 || bctype[4] == 7;
  int s = per ? 3 : 2;
  for (int l = 0; l < nlevels; l++) {
    UserCtx *u = U(l);
    DMDACreate3d(PETSC_COMM_WORLD, bctype[0] == 7 ? DM_BOUNDARY_PERIODIC : DM_BOUNDARY_NONE,
                 bctype[2] == 7 ? DM_BOUNDARY_PERIODIC : DM_BOUNDARY_NONE,
                 bctype[4] == 7 ? DM_BOUNDARY_PERIODIC : DM_BOUNDARY_NONE, DMDA_STENCIL_BOX,
                 u->IM + 1, u->JM + 1, u->KM + 1, 1, 1, 1, 1, s, NULL, NULL, NULL, &u->da);
    DMDASetUniformCoordinates(u->da, 0.0, 1.0, 0.0, 1.0, 0.0, 1.0);
    DMGetCoordinateDM(u->da, &u->fda);
    DMDAGetLocalInfo(u->da, &u->info);
  }
  /* finest coordinates (init.c:655-744) */
  {
    UserCtx *u = U(nlevels - 1);
    Vec Coor, gCoor;
    Cmpnts ***coor;
    DMGetCoordinatesLocal(u->da, &Coor);
    VecSet(Coor, 0.0);
    DMDAVecGetArray(u->fda, Coor, &coor);
    for (int k = 0; k < u->info.mz; k++)
      for (int j = 0; j < u->info.my; j++)
        for (int i = 0; i < u->info.mx; i++)
          if (k < KM && j < JM && i < IM) {
            const double *c = coords + 3 * ((size_t)(k * JM + j) * IM + i);
            coor[k][j][i].x = c[0]; coor[k][j][i].y = c[1]; coor[k][j][i].z = c[2];
          }
    DMDAVecRestoreArray(u->fda, Coor, &coor);
    DMGetCoordinates(u->da, &gCoor);
    VecSet(gCoor, 0.0);
    DMLocalToGlobalBegin(u->fda, Coor, INSERT_VALUES, gCoor);
    DMLocalToGlobalEnd(u->fda, Coor, INSERT_VALUES, gCoor);
    DMGlobalToLocalBegin(u->fda, gCoor, INSERT_VALUES, Coor);
    DMGlobalToLocalEnd(u->fda, gCoor, INSERT_VALUES, Coor);
  }
  /* inject fine -> coarse (init.c:786-828) */
  for (int l = nlevels - 2; l >= 0; l--) {
    UserCtx *u = U(l), *h = U(l + 1);
    Vec Coor_high, Coor, gCoor;
    Cmpnts ***coor, ***coor_high;
    DMGetCoordinatesLocal(h->da, &Coor_high);
    DMGetCoordinates(u->da, &Coor);
    DMDAVecGetArray(h->fda, Coor_high, &coor_high);
    DMDAVecGetArray(u->fda, Coor, &coor);
    int xe = u->info.mx - 1, ye = u->info.my - 1, ze = u->info.mz - 1;
    for (int k = 0; k < ze; k++)
      for (int j = 0; j < ye; j++)
        for (int i = 0; i < xe; i++) {
          PetscInt ih, jh, kh;
          GridRestriction(i, j, k, &ih, &jh, &kh, u);
          coor[k][j][i] = coor_high[kh][jh][ih];
        }
    DMDAVecRestoreArray(u->fda, Coor, &coor);
    DMDAVecRestoreArray(h->fda, Coor_high, &coor_high);
    DMGetCoordinatesLocal(u->da, &gCoor);
    DMGlobalToLocalBegin(u->fda, Coor, INSERT_VALUES, gCoor);
    DMGlobalToLocalEnd(u->fda, Coor, INSERT_VALUES, gCoor);
  }
  /* level links and vectors (init.c:834-1060) */
  for (int l = nlevels - 1; l >= 0; l--) {
    UserCtx *u = U(l);
    if (l > 0) {
      u->da_c = &U(l - 1)->da;
      u->lNvert_c = &U(l - 1)->lNvert;
      u->user_c = U(l - 1);
    }
    if (l < nlevels - 1) {
      u->da_f = &U(l + 1)->da;
      u->user_f = U(l + 1);
    }
    make_vectors(u, l == nlevels - 1);
    FormMetrics(u);
    if (bctype[0] == 7 || bctype[2] == 7 || bctype[4] == 7) Update_Metrics_PBC(u);
  }
  g_ready = 1;
  return 0;
}

/* The hierarchy ref_init built, for drivers that call CURVIB-side code taking a
 * UserMG (the source-level binding's tests). */
UserMG *ref_usermg(void) { return g_ready ? &g_mg : NULL; }

int ref_dims(int level, int *mx, int *my, int *mz) {
  if (!g_ready || level < 0 || level >= g_mg.mglevels) return 1;
  *mx = U(level)->info.mx; *my = U(level)->info.my; *mz = U(level)->info.mz;
  return 0;
}

static Vec field(UserCtx *u, const char *name, int *dof) {
  struct { const char *n; Vec v; int dof; } t[] = {
    {"Csi", u->lCsi, 3}, {"Eta", u->lEta, 3}, {"Zet", u->lZet, 3},
    {"ICsi", u->lICsi, 3}, {"IEta", u->lIEta, 3}, {"IZet", u->lIZet, 3},
    {"JCsi", u->lJCsi, 3}, {"JEta", u->lJEta, 3}, {"JZet", u->lJZet, 3},
    {"KCsi", u->lKCsi, 3}, {"KEta", u->lKEta, 3}, {"KZet", u->lKZet, 3},
    {"Aj", u->lAj, 1}, {"IAj", u->lIAj, 1}, {"JAj", u->lJAj, 1}, {"KAj", u->lKAj, 1},
    {"Cent", u->lCent, 3}, {"Nvert", u->lNvert, 1}, {"Ucont", u->lUcont, 3},
    {"Phi", u->lPhi, 1}, {"P", u->lP, 1},
    {"gNvert", u->Nvert, 1}, {"gUcont", u->Ucont, 3}, {"gPhi", u->Phi, 1}, {"gP", u->P, 1},
  };
  for (size_t q = 0; q < sizeof(t) / sizeof(t[0]); q++)
    if (!strcmp(t[q].n, name)) { *dof = t[q].dof; return t[q].v; }
  return NULL;
}

/* Copy the owned box of a (local or global) vector out as [mz][my][mx](dof). */
static void copy_owned(UserCtx *u, Vec v, int dof, double *out, int to_vec) {
  DMDALocalInfo f = u->info;
  double *a = shim_vec_data(v);
  int n = shim_vec_size(v);
  int local = n != f.mx * f.my * f.mz * dof;
  int gxs = local ? f.gxs : 0, gys = local ? f.gys : 0, gzs = local ? f.gzs : 0;
  int gxm = local ? f.gxm : f.mx, gym = local ? f.gym : f.my;
  for (int k = 0; k < f.mz; k++)
    for (int j = 0; j < f.my; j++)
      for (int i = 0; i < f.mx; i++) {
        size_t s = ((size_t)((k - gzs) * gym + (j - gys)) * gxm + (i - gxs)) * dof;
        size_t d = ((size_t)(k * f.my + j) * f.mx + i) * dof;
        for (int c = 0; c < dof; c++) {
          if (to_vec) a[s + c] = out[d + c];
          else out[d + c] = a[s + c];
        }
      }
}

int ref_get_field(int level, const char *name, double *out) {
  if (!g_ready || level < 0 || level >= g_mg.mglevels) return 1;
  int dof;
  Vec v = field(U(level), name, &dof);
  if (!v) return 2;
  copy_owned(U(level), v, dof, out, 0);
  return 0;
}

/* Set a global field and refresh its local copy (G2L), as the reference keeps them. */
static int set_pair(UserCtx *u, Vec g, Vec l, int dof, const double *in, DM dm) {
  copy_owned(u, g, dof, (double *)in, 1);
  DMGlobalToLocalBegin(dm, g, INSERT_VALUES, l);
  DMGlobalToLocalEnd(dm, g, INSERT_VALUES, l);
  return 0;
}

int ref_set_nvert(int level, const double *nv) {
  if (!g_ready) return 1;
  UserCtx *u = U(level);
  return set_pair(u, u->Nvert, u->lNvert, 1, nv, u->da);
}
int ref_set_ucont(const double *uc) {
  UserCtx *u = U(g_mg.mglevels - 1);
  return set_pair(u, u->Ucont, u->lUcont, 3, uc, u->fda);
}

/* PoissonSolver_MG's immersed block (poisson.c:1794-1806): nvert restriction on
 * every level pair, then FullyBlocked on the coarsest level.  Returns
 * multinullspace in *mns and, when set, KSKE (2*mx*my ints) in kske. */
int ref_nvert_restrict(int *mns, int *kske) {
  if (!g_ready) return 1;
  int L = g_mg.mglevels;
  for (int l = L - 1; l > 0; l--) {
    U(l)->multinullspace = PETSC_FALSE;
    MyNvertRestriction(U(l), U(l - 1));
  }
  UserCtx *c = U(0);
  PetscMalloc(c->info.mx * c->info.my * 2 * sizeof(PetscInt), &c->KSKE);
  FullyBlocked(c);
  *mns = c->multinullspace;
  if (kske) memcpy(kske, c->KSKE, sizeof(int) * 2 * c->info.mx * c->info.my);
  return 0;
}

/* PoissonLHSNew (poisson.c:600) -> rows of (col,val); returns entries written. */
int ref_lhs(int level, int *rowptr, int *cols, double *vals, int cap) {
  if (!g_ready) return -1;
  UserCtx *u = U(level);
  u->assignedA = PETSC_FALSE;
  PoissonLHSNew(u);
  int nr = shim_mat_rows(u->A), w = 0;
  rowptr[0] = 0;
  for (int r = 0; r < nr; r++) {
    const int *c; const double *v;
    int n = shim_mat_row(u->A, r, &c, &v);
    for (int q = 0; q < n; q++) {
      if (w >= cap) return -2;
      cols[w] = c[q]; vals[w] = v[q]; w++;
    }
    rowptr[r + 1] = w;
  }
  MatDestroy(&u->A);
  u->assignedA = PETSC_FALSE;
  return w;
}

/* VolumeFlux_rev (poisson.c:3712) on the finest level; Ucont updated in place. */
int ref_volume_flux(double flux_intp_sum, int flg, double *ucont_inout, double *flux, double *area) {
  UserCtx *u = U(g_mg.mglevels - 1);
  set_pair(u, u->Ucont, u->lUcont, 3, ucont_inout, u->fda);
  u->FluxIntpSum = flux_intp_sum;
  VolumeFlux_rev(u, flux, area, flg);
  copy_owned(u, u->Ucont, 3, ucont_inout, 0);
  return 0;
}

/* PoissonRHS (poisson.c:1509) on the finest level from its current lUcont. */
int ref_rhs(double dt, double st, double *b, double *compat_sum) {
  UserCtx *u = U(g_mg.mglevels - 1);
  u->dt = dt; u->st = st;
  Vec B;
  VecDuplicate(u->P, &B);
  PoissonRHS(u, B);
  copy_owned(u, B, 1, b, 0);
  /* the reference prints this sum (poisson.c:1554-1568); recompute it identically */
  DMDALocalInfo f = u->info;
  double *bb = shim_vec_data(B), s = 0;
  double ***aj;
  DMDAVecGetArray(u->da, u->lAj, &aj);
  for (int k = 0; k < f.mz; k++)
    for (int j = 0; j < f.my; j++)
      for (int i = 0; i < f.mx; i++)
        s += bb[(size_t)(k * f.my + j) * f.mx + i] / aj[k][j][i] * dt / COEF_TIME_ACCURACY;
  DMDAVecRestoreArray(u->da, u->lAj, &aj);
  *compat_sum = s;
  VecDestroy(&B);
  return 0;
}

/* MyRestriction (poisson.c:129): fine level (coarse+1) vector -> coarse level vector. */
int ref_restrict(int coarse, const double *xf, double *fc) {
  UserCtx *c = U(coarse), *f = U(coarse + 1);
  Mat MR;
  Vec X, F;
  VecDuplicate(f->P, &X); VecDuplicate(c->P, &F);
  copy_owned(f, X, 1, (double *)xf, 1);
  MatCreateShell(PETSC_COMM_WORLD, 0, 0, c->info.mx * c->info.my * c->info.mz, 0, (void *)c, &MR);
  MatShellSetOperation(MR, MATOP_MULT, (void (*)(void))MyRestriction);
  MatMult(MR, X, F);
  copy_owned(c, F, 1, fc, 0);
  MatDestroy(&MR); VecDestroy(&X); VecDestroy(&F);
  return 0;
}

/* MyInterpolation (poisson.c:265): coarse level (fine-1) vector -> fine level vector. */
int ref_interpolate(int fine, const double *xc, double *ff) {
  UserCtx *f = U(fine), *c = U(fine - 1);
  Mat MP;
  Vec X, F;
  VecDuplicate(c->P, &X); VecDuplicate(f->P, &F);
  copy_owned(c, X, 1, (double *)xc, 1);
  copy_owned(f, F, 1, ff, 1); /* MyInterpolation leaves nothing unset, but be explicit */
  MatCreateShell(PETSC_COMM_WORLD, 0, 0, f->info.mx * f->info.my * f->info.mz, 0, (void *)f, &MP);
  MatShellSetOperation(MP, MATOP_MULT, (void (*)(void))MyInterpolation);
  MatMult(MP, X, F);
  copy_owned(f, F, 1, ff, 0);
  MatDestroy(&MP); VecDestroy(&X); VecDestroy(&F);
  return 0;
}

/* PoissonNullSpaceFunction (poisson.c:372) applied in place on one level. */
int ref_nullspace(int level, double *x) {
  UserCtx *u = U(level);
  Vec X;
  VecDuplicate(u->P, &X);
  copy_owned(u, X, 1, x, 1);
  PoissonNullSpaceFunction(NULL, X, (void *)u);
  copy_owned(u, X, 1, x, 0);
  VecDestroy(&X);
  return 0;
}

/* The tail of a time step on the finest level, in the reference's order:
 * G2L(Phi) (poisson.c:1985), UpdatePressure (poisson.c:2908), Projection
 * (poisson.c:2281).  p, phi and ucont are updated in place. */
int ref_update_and_project(double dt, double st, double *p, double *phi, double *ucont) {
  UserCtx *u = U(g_mg.mglevels - 1);
  u->dt = dt; u->st = st;
  set_pair(u, u->P, u->lP, 1, p, u->da);
  set_pair(u, u->Phi, u->lPhi, 1, phi, u->da);
  set_pair(u, u->Ucont, u->lUcont, 3, ucont, u->fda);
  UpdatePressure(u);
  Projection(u);
  copy_owned(u, u->P, 1, p, 0);
  copy_owned(u, u->Phi, 1, phi, 0);
  copy_owned(u, u->Ucont, 3, ucont, 0);
  return 0;
}

/* Contra2Cart (rhs.c:25-143) on the finest level: the Cartesian velocity at
 * the centres of the interior cells that are fluid (nvert < 0.1) or inside a
 * body (nvert > 7), from Ucont and the centre metrics.  ucont is the global
 * Ucont box; ucat (global Ucat box) is read for the cells the routine leaves
 * alone and written. */
int ref_contra2cart(const double *ucont, double *ucat) {
  if (!g_ready) return 1;
  UserCtx *u = U(g_mg.mglevels - 1);
  set_pair(u, u->Ucont, u->lUcont, 3, ucont, u->fda);
  set_pair(u, u->Ucat, u->lUcat, 3, ucat, u->fda);
  cvbref_Contra2Cart(u);
  copy_owned(u, u->Ucat, 3, ucat, 0);
  return 0;
}

/* The rheology plates' velocity (bcs.c's global U_bc) for GhostNodeVelocity. */
extern PetscReal U_bc;
void ref_set_u_bc(double v) { U_bc = v; }

/* GhostNodeVelocity (bcs.c:3645-4435) on the finest level: ubcs (Bcs.Ubcs) and
 * ucat (Ucat), global boxes, both read and written. */
int ref_ghost_node_velocity(double *ubcs, double *ucat) {
  if (!g_ready) return 1;
  UserCtx *u = U(g_mg.mglevels - 1);
  copy_owned(u, u->Bcs.Ubcs, 3, ubcs, 1);
  set_pair(u, u->Ucat, u->lUcat, 3, ucat, u->fda);
  cvbref_GhostNodeVelocity(u);
  copy_owned(u, u->Ucat, 3, ucat, 0);
  copy_owned(u, u->Bcs.Ubcs, 3, ubcs, 0);
  return 0;
}

/* ibm_search_advanced (ibm.c:4197-4740) on the finest level for body ibi of
 * nbodies.  The body is a closed triangle mesh: n_v nodes (xyz, x y z per
 * node), n_elmt triangles (nv, three node indices each) and their unit normals
 * (nf, x y z per triangle).  nvert_o is the previous step's Nvert_o; nvert is
 * Nvert, read and written (global boxes).  The routine also builds the body's
 * interpolation list, which is left in the harness. */
int ref_ibm_search(int n_v, const double *xyz, int n_elmt, const int *nv, const double *nf, int ibi, int nbodies,
                   const double *nvert_o, double *nvert) {
  if (!g_ready) return 1;
  UserCtx *u = U(g_mg.mglevels - 1);
  IBMNodes *ibm = (IBMNodes *)calloc(1, sizeof(IBMNodes));
  if (!ibm) return 2;
  ibm->n_v = n_v;
  ibm->n_elmt = n_elmt;
  ibm->x_bp = (double *)malloc(sizeof(double) * n_v);
  ibm->y_bp = (double *)malloc(sizeof(double) * n_v);
  ibm->z_bp = (double *)malloc(sizeof(double) * n_v);
  for (int q = 0; q < n_v; q++) {
    ibm->x_bp[q] = xyz[3 * q]; ibm->y_bp[q] = xyz[3 * q + 1]; ibm->z_bp[q] = xyz[3 * q + 2];
  }
  ibm->nv1 = (int *)malloc(sizeof(int) * n_elmt);
  ibm->nv2 = (int *)malloc(sizeof(int) * n_elmt);
  ibm->nv3 = (int *)malloc(sizeof(int) * n_elmt);
  ibm->nf_x = (double *)malloc(sizeof(double) * n_elmt);
  ibm->nf_y = (double *)malloc(sizeof(double) * n_elmt);
  ibm->nf_z = (double *)malloc(sizeof(double) * n_elmt);
  for (int e = 0; e < n_elmt; e++) {
    ibm->nv1[e] = nv[3 * e]; ibm->nv2[e] = nv[3 * e + 1]; ibm->nv3[e] = nv[3 * e + 2];
    ibm->nf_x[e] = nf[3 * e]; ibm->nf_y[e] = nf[3 * e + 1]; ibm->nf_z[e] = nf[3 * e + 2];
  }
  NumberOfBodies = nbodies;
  if (!u->ibmlist) u->ibmlist = (IBMList *)calloc((size_t)(nbodies > 16 ? nbodies : 16), sizeof(IBMList));
  set_pair(u, u->Nvert, u->lNvert, 1, nvert, u->da);
  set_pair(u, u->Nvert_o, u->lNvert_o, 1, nvert_o, u->da);
  int rc = ibm_search_advanced(u, ibm, ibi);
  copy_owned(u, u->Nvert, 1, nvert, 0);
  /* the interpolation list stays with the harness (test-only: leaks are harmless) */
  return rc;
}

/* MG_Initial (init.c:296-1060) run in dir, which holds its grid.dat and
 * bcs.dat (one block): the node coordinates it leaves on the finest level,
 * [KM][JM][IM][3], for the grid.dat reader's pinning.  -mg_level, -grid1d and
 * -chact_leng are set as given; L_dim is main.c's global. */
PetscErrorCode MG_Initial(UserMG *usermg, IBMNodes *ibm);
PetscReal L_dim = 1.0; /* main.c's length scale of grid.dat's coordinates */
static UserMG g_mg_initial;

/* The boundary types MG_Initial read from bcs.dat (init.c:478-490) in the
 * last ref_mg_initial_nodes call, and the i / j / k periodic flags it set. */
int ref_mg_initial_bctype(int *bctype, int *periodic) {
  if (!g_mg_initial.mgctx) return 1;
  UserCtx *u = &g_mg_initial.mgctx[g_mg_initial.mglevels - 1].user[0];
  for (int f = 0; f < 6; f++) bctype[f] = u->bctype[f];
  periodic[0] = i_periodic;
  periodic[1] = j_periodic;
  periodic[2] = k_periodic;
  return 0;
}

int ref_mg_initial_nodes(const char *dir, int nlevels, int grid1d, double cl, double l_dim, int *IM, int *JM,
                         int *KM, double *coords, long long cap) {
  char cwd[4096], val[64];
  if (!getcwd(cwd, sizeof cwd) || chdir(dir)) return 1;
  PetscOptionsClear();
  snprintf(val, sizeof val, "%d", nlevels); PetscOptionsSetValue("-mg_level", val);
  snprintf(val, sizeof val, "%d", grid1d); PetscOptionsSetValue("-grid1d", val);
  snprintf(val, sizeof val, "%.17g", cl); PetscOptionsSetValue("-chact_leng", val);
  L_dim = l_dim;
  block_number = 1;
  i_periodic = j_periodic = k_periodic = 0;
  UserMG *mgp = &g_mg_initial;
  memset(mgp, 0, sizeof *mgp);
  IBMNodes *ibm = (IBMNodes *)calloc(1, sizeof(IBMNodes));
  int rc = MG_Initial(mgp, ibm);
  if (chdir(cwd)) rc = rc ? rc : 2;
  PetscOptionsClear();
  if (rc) return rc;
  UserCtx *u = &mgp->mgctx[mgp->mglevels - 1].user[0];
  *IM = u->IM; *JM = u->JM; *KM = u->KM;
  if ((long long)3 * u->IM * u->JM * u->KM > cap) return 3;
  Vec Coor;
  Cmpnts ***coor;
  DMGetCoordinatesLocal(u->da, &Coor);
  DMDAVecGetArray(u->fda, Coor, &coor);
  for (int k = 0; k < u->KM; k++)
    for (int j = 0; j < u->JM; j++)
      for (int i = 0; i < u->IM; i++) {
        double *c = coords + 3 * (((size_t)k * u->JM + j) * u->IM + i);
        c[0] = coor[k][j][i].x; c[1] = coor[k][j][i].y; c[2] = coor[k][j][i].z;
      }
  DMDAVecRestoreArray(u->fda, Coor, &coor);
  return 0;
}

/* Divergence (main.c:469-593), run after Projection in Flow_Solver
 * (solvers.c:1084): max over the interior of |div Ucont| aj, zero next to a
 * body and on the ring, and its index in the [mz][my][mx] box, as VecMax
 * returns them (the routine itself only prints them). */
PetscErrorCode Divergence(UserCtx *user);
void shim_last_vecmax(double *v, int *at);
int ref_divergence(const double *ucont, double *maxdiv, int *at) {
  if (!g_ready) return 1;
  UserCtx *u = U(g_mg.mglevels - 1);
  set_pair(u, u->Ucont, u->lUcont, 3, ucont, u->fda);
  int rc = Divergence(u);
  shim_last_vecmax(maxdiv, at);
  return rc;
}

/* Convection (rhs.c:1463-1946) as FormFunction1 calls it (rhs.c:2651), on
 * lUcont and lUcat of the finest level, with -central set as given; conv is
 * the [mz][my][mx] box of the result. */
PetscErrorCode Convection(UserCtx *user, Vec Ucont, Vec Ucat, Vec Conv);
int ref_convection(const double *ucont, const double *ucat, int central, double *conv) {
  if (!g_ready) return 1;
  UserCtx *u = U(g_mg.mglevels - 1);
  set_pair(u, u->Ucont, u->lUcont, 3, ucont, u->fda);
  set_pair(u, u->Ucat, u->lUcat, 3, ucat, u->fda);
  PetscOptionsSetValue("-central", central ? "1" : "0");
  Vec Conv;
  VecDuplicate(u->Ucont, &Conv);
  int rc = Convection(u, u->lUcont, u->lUcat, Conv);
  copy_owned(u, Conv, 3, conv, 0);
  VecDestroy(&Conv);
  PetscOptionsSetValue("-central", "0");
  return rc;
}

/* MetricsDivergence (metrics.c:1551-1625), which MG_Initial runs on the
 * finest level once its metrics are formed (init.c:1054), over the metrics
 * this harness formed with the reference's FormMetrics. */
PetscErrorCode MetricsDivergence(UserCtx *user);
int ref_metrics_divergence(double *maxdiv, int *at) {
  if (!g_ready) return 1;
  int rc = MetricsDivergence(U(g_mg.mglevels - 1));
  shim_last_vecmax(maxdiv, at);
  return rc;
}


/* Ucont_P_Binary_Output (main.c:285): the reference's restart files for step
 * ti_ and block (user->_this) into dir -- nvert, ucont, ucat, p are the finest
 * level's global boxes Nvert, Ucont, Ucat, P. */
PetscErrorCode Ucont_P_Binary_Output(UserCtx *user);
PetscErrorCode Ucont_P_Binary_Input(UserCtx *user);
int ref_restart_write(const char *dir, int ti_, int block, const double *nvert, const double *ucont,
                      const double *ucat, const double *p) {
  if (!g_ready) return 1;
  UserCtx *u = U(g_mg.mglevels - 1);
  copy_owned(u, u->Nvert, 1, (double *)nvert, 1);
  copy_owned(u, u->Ucont, 3, (double *)ucont, 1);
  copy_owned(u, u->Ucat, 3, (double *)ucat, 1);
  copy_owned(u, u->P, 1, (double *)p, 1);
  ti = ti_;
  u->_this = block;
  shim_set_viewer_dir(dir);
  int rc = Ucont_P_Binary_Output(u);
  shim_set_viewer_dir(".");
  return rc;
}
/* Ucont_P_Binary_Input (main.c:75): reads Ucont, P and Nvert_o back. */
int ref_restart_read(const char *dir, int ti_, int block, double *ucont, double *p, double *nvert_o) {
  if (!g_ready) return 1;
  UserCtx *u = U(g_mg.mglevels - 1);
  ti = ti_;
  u->_this = block;
  shim_set_viewer_dir(dir);
  int rc = Ucont_P_Binary_Input(u);
  shim_set_viewer_dir(".");
  if (rc) return rc;
  copy_owned(u, u->Ucont, 3, ucont, 0);
  copy_owned(u, u->P, 1, p, 0);
  copy_owned(u, u->Nvert_o, 1, nvert_o, 0);
  return 0;
}

/* Viscous (rhs.c:1947), FormFunction1 (rhs.c:2567) and CalcRHS
 * (implicitsolver.c:6449) on the finest level.  FormFunction1 starts with
 * Contra2Cart, which in this library is the inert stand-in (see the top of
 * this file), so the harness runs the reference's own Contra2Cart first: its
 * result is what FormFunction1's call leaves. */
PetscErrorCode Viscous(UserCtx *user, Vec Ucont, Vec Ucat, Vec Visc);
PetscErrorCode FormFunction1(UserCtx *user, Vec Rhs);
PetscErrorCode CalcRHS(UserCtx *user, FSInfo *fsi);

int ref_viscous(const double *ucat, double ren, double *visc) {
  if (!g_ready) return 1;
  UserCtx *u = U(g_mg.mglevels - 1);
  set_pair(u, u->Ucat, u->lUcat, 3, ucat, u->fda);
  u->ren = ren;
  Vec V;
  VecDuplicate(u->lUcat, &V);
  int rc = Viscous(u, u->lUcont, u->lUcat, V);
  copy_owned(u, V, 3, visc, 0);
  VecDestroy(&V);
  return rc;
}

static void momentum_inputs(UserCtx *u, const double *ucont, const double *ucat, const double *p, double ren,
                            int central) {
  set_pair(u, u->Ucont, u->lUcont, 3, ucont, u->fda);
  set_pair(u, u->Ucat, u->lUcat, 3, ucat, u->fda);
  set_pair(u, u->P, u->lP, 1, p, u->da);
  u->ren = ren;
  PetscOptionsSetValue("-central", central ? "1" : "0");
  cvbref_Contra2Cart(u);
}

int ref_form_function1(const double *ucont, double *ucat, const double *p, double ren, int central, double *rhs) {
  if (!g_ready) return 1;
  UserCtx *u = U(g_mg.mglevels - 1);
  momentum_inputs(u, ucont, ucat, p, ren, central);
  Vec R;
  VecDuplicate(u->Ucont, &R);
  copy_owned(u, R, 3, rhs, 1);
  int rc = FormFunction1(u, R);
  copy_owned(u, R, 3, rhs, 0);
  copy_owned(u, u->Ucat, 3, ucat, 0);
  VecDestroy(&R);
  PetscOptionsSetValue("-central", "0");
  return rc;
}

int ref_calc_rhs(const double *ucont, const double *ucont_o, const double *ucont_rm1, double *ucat, const double *p,
                 double ren, double dt, int ti_, int tistart_, int central, double *rhs) {
  if (!g_ready) return 1;
  UserCtx *u = U(g_mg.mglevels - 1);
  momentum_inputs(u, ucont, ucat, p, ren, central);
  if (!u->Ucont_o) VecDuplicate(u->Ucont, &u->Ucont_o);
  if (!u->Ucont_rm1) VecDuplicate(u->Ucont, &u->Ucont_rm1);
  copy_owned(u, u->Ucont_o, 3, (double *)ucont_o, 1);
  copy_owned(u, u->Ucont_rm1, 3, (double *)ucont_rm1, 1);
  VecDuplicate(u->Ucont, &u->Rhs);
  copy_owned(u, u->Rhs, 3, rhs, 1);
  u->dt = dt;
  ti = ti_;
  tistart = tistart_;
  int rc = CalcRHS(u, NULL);
  copy_owned(u, u->Rhs, 3, rhs, 0);
  copy_owned(u, u->Ucat, 3, ucat, 0);
  VecDestroy(&u->Rhs);
  PetscOptionsSetValue("-central", "0");
  return rc;
}

/* InflowFlux (bcs.c:99-400) and FormBCS (bcs.c:4436-5889) on the finest
 * level.  Both read and write ucont (Ucont) and ubcs (Bcs.Ubcs); FormBCS also
 * ucat (Ucat) and p (P).  InflowFlux's result is the global FluxInSum, which
 * FormBCS's outlet reads (flux_in_sum here), beside the user's FluxIntpSum. */
extern PetscReal FluxInSum;
extern PetscInt inletprofile;
PetscErrorCode InflowFlux(UserCtx *user);
PetscErrorCode FormBCS(UserCtx *user);

/* CMx_c, CMy_c, CMz_c (main.c's globals), which the shaped inlet profiles
 * subtract from the face centres. */
extern PetscReal CMx_c, CMy_c, CMz_c;
void ref_set_cm(double x, double y, double z) { CMx_c = x; CMy_c = y; CMz_c = z; }
/* Flux_in (main.c:6) and ti, which the uniform inlet profiles read. */
extern PetscReal Flux_in;
void ref_set_inlet_globals(double flux_in, int ti_) { Flux_in = flux_in; ti = ti_; }
/* InletRead's table on the finest level: r as InletRead sets it (bcs.c:46),
 * uinr [101][1001] as given. */
void ref_set_inlet_table(const double *uinr) {
  UserCtx *u = &g_mg.mgctx[g_mg.mglevels - 1].user[0];
  for (int i = 0; i < 101; i++) u->r[i] = i * 0.005;
  memcpy(u->uinr, uinr, sizeof(u->uinr));
}

int ref_inflow_flux(double *ucont, double *ubcs, int profile, double *flux_in_sum) {
  if (!g_ready) return 1;
  UserCtx *u = U(g_mg.mglevels - 1);
  set_pair(u, u->Ucont, u->lUcont, 3, ucont, u->fda);
  copy_owned(u, u->Bcs.Ubcs, 3, ubcs, 1);
  inletprofile = profile;
  FluxInSum = *flux_in_sum;
  int rc = InflowFlux(u);
  *flux_in_sum = FluxInSum;
  copy_owned(u, u->Ucont, 3, ucont, 0);
  copy_owned(u, u->Bcs.Ubcs, 3, ubcs, 0);
  return rc;
}

int ref_form_bcs(double *ucont, double *ubcs, double *ucat, double *p, double flux_in_sum, double flux_intp_sum) {
  if (!g_ready) return 1;
  UserCtx *u = U(g_mg.mglevels - 1);
  set_pair(u, u->Ucont, u->lUcont, 3, ucont, u->fda);
  set_pair(u, u->Ucat, u->lUcat, 3, ucat, u->fda);
  set_pair(u, u->P, u->lP, 1, p, u->da);
  copy_owned(u, u->Bcs.Ubcs, 3, ubcs, 1);
  FluxInSum = flux_in_sum;
  u->FluxIntpSum = flux_intp_sum;
  int rc = FormBCS(u);
  copy_owned(u, u->Ucont, 3, ucont, 0);
  copy_owned(u, u->Bcs.Ubcs, 3, ubcs, 0);
  copy_owned(u, u->Ucat, 3, ucat, 0);
  copy_owned(u, u->P, 1, p, 0);
  return rc;
}

/* ImpRK (implicitsolver.c:7094-7257) on the finest level, one block, no
 * immersed body: ucont, ubcs, ucat and p (Ucont, Bcs.Ubcs, Ucat, P) read and
 * written, ucont_o / ucont_rm1 the two previous steps' fluxes; cfl, dt, st and
 * FluxIntpSum the block's, imp_atol / imp_rtol / imp_MAX_IT and inletprofile
 * from the arguments for this call.  The routine appends to the file
 * Converge_dU0 in the working directory, as the reference's rank 0 does. */
int ref_imp_rk(double *ucont, const double *ucont_o, const double *ucont_rm1, double *ucat, double *p,
               double *ubcs, double ren, double dt, double st, double cfl, int ti_, int tistart_, int central,
               double atol, double rtol, int max_it, int profile, double flux_intp_sum) {
  if (!g_ready) return 1;
  UserCtx *u = U(g_mg.mglevels - 1);
  set_pair(u, u->Ucont, u->lUcont, 3, ucont, u->fda);
  set_pair(u, u->Ucat, u->lUcat, 3, ucat, u->fda);
  set_pair(u, u->P, u->lP, 1, p, u->da);
  copy_owned(u, u->Bcs.Ubcs, 3, ubcs, 1);
  if (!u->Ucont_o) VecDuplicate(u->Ucont, &u->Ucont_o);
  if (!u->Ucont_rm1) VecDuplicate(u->Ucont, &u->Ucont_rm1);
  copy_owned(u, u->Ucont_o, 3, (double *)ucont_o, 1);
  copy_owned(u, u->Ucont_rm1, 3, (double *)ucont_rm1, 1);
  if (!u->psuedot) VecDuplicate(u->Ucont, &u->psuedot);
  VecSet(u->psuedot, 0.);
  u->ren = ren;
  u->dt = dt;
  u->st = st;
  u->cfl = cfl;
  u->FluxIntpSum = flux_intp_sum;
  inletprofile = profile;
  FluxInSum = 0.;
  PetscOptionsSetValue("-central", central ? "1" : "0");
  ti = ti_;
  tistart = tistart_;
  const PetscInt it0 = imp_MAX_IT;
  const PetscReal a0 = imp_atol, r0 = imp_rtol;
  imp_MAX_IT = max_it;
  imp_atol = atol;
  imp_rtol = rtol;
  int rc = ImpRK(u, NULL, NULL);
  imp_MAX_IT = it0;
  imp_atol = a0;
  imp_rtol = r0;
  PetscOptionsSetValue("-central", "0");
  copy_owned(u, u->Ucont, 3, ucont, 0);
  copy_owned(u, u->Bcs.Ubcs, 3, ubcs, 0);
  copy_owned(u, u->Ucat, 3, ucat, 0);
  copy_owned(u, u->P, 1, p, 0);
  return rc;
}
