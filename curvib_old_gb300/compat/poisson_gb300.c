/*
 * Source-level drop-in of CURVIB's pressure-projection path onto libcvb (see
 * poisson_gb300.h for what it replaces).  Compiled in the CURVIB tree:
 *
 *   cc -c poisson_gb300.c -I<curvib> -I<this repo>/include $(PETSC_CC_INCLUDES)
 *   link with -L<this repo>/curvib_old_gb300/_build -lcvb
 *
 * The arrays handed to libcvb are the PETSc vectors' own storage: VecGetArray
 * on a DMDA vector of one rank gives its box [k][j][i], i fastest, with
 * Cmpnts interleaved -- the layout cvb.h takes.  Local (ghosted) vectors give
 * the ghosted box that cvb_level_desc's gxs..gzm describe.  Nothing is
 * converted or copied on the host.
 */
#include <stdlib.h>
#include <string.h>
#include "variables.h"
#include "cvb.h"
#include "poisson_gb300.h"

extern PetscInt block_number, immersed; /* main.c, as poisson.c:6-7 declares them */
extern PetscInt wallfunction;           /* main.c, as bcs.c:3689 declares it */
extern PetscInt les;                    /* main.c, as rhs.c declares it */
extern PetscInt rans;                   /* main.c, as rhs.c declares it */
extern PetscInt ti, tistart;            /* main.c: the time step, as implicitsolver.c declares them */
extern PetscInt imp_MAX_IT;             /* main.c: the pseudo-time iteration's controls */
extern PetscReal imp_atol, imp_rtol;
extern PetscInt inletprofile;           /* main.c: InflowFlux's profile */
extern PetscReal FluxInSum;             /* main.c: InflowFlux's result, as bcs.c:5 declares it */
extern PetscReal U_bc;                  /* bcs.c:10: the rheology plates' velocity */
extern PetscReal CMx_c, CMy_c, CMz_c;   /* main.c: the centre the shaped inlet profiles take from the nodes */
extern PetscReal Flux_in;               /* main.c: the uniform inlet profiles' speed */
PetscErrorCode Contra2Cart(UserCtx *user);
PetscErrorCode GhostNodeVelocity(UserCtx *user);
PetscErrorCode ImpRK(UserCtx *user, IBMNodes *ibm, FSInfo *fsi); /* implicitsolver.c:7094 */

static cvb_ctx *g_cvb = NULL;
static cvb_solve_opts g_opts;
static int g_cent_given = 0; /* the cell centres went to the context (an annulus face) */

static PetscErrorCode report(int rc, const char *where) {
  if (rc)
    PetscPrintf(PETSC_COMM_WORLD, "%s: %s\n", where,
                g_cvb ? cvb_last_error(g_cvb) : "libcvb context not created");
  return rc;
}

static UserCtx *finest(UserMG *usermg) { return &usermg->mgctx[usermg->mglevels - 1].user[0]; }

/* The ghosted arrays of one level: the nine face-metric fields, the four
 * Jacobian fields, and on the finest level the three cell-centre metric fields
 * Projection reads.  Level 0 is the coarsest, as mgctx[0] (init.c:839-850). */
#define DESC_ARRAYS 16
static void desc_get(UserCtx *u, cvb_level_desc *d, int fine, PetscScalar *hold[DESC_ARRAYS]) {
  PetscInt gxs, gys, gzs, gxm, gym, gzm;
  DMDAGetGhostCorners(u->da, &gxs, &gys, &gzs, &gxm, &gym, &gzm);
  memset(d, 0, sizeof *d);
  d->mx = u->info.mx; d->my = u->info.my; d->mz = u->info.mz;
  d->gxs = gxs; d->gys = gys; d->gzs = gzs;
  d->gxm = gxm; d->gym = gym; d->gzm = gzm;
  for (int f = 0; f < 6; f++) d->bctype[f] = u->bctype[f];
  d->isc = u->isc; d->jsc = u->jsc; d->ksc = u->ksc;
  Vec v[DESC_ARRAYS] = {u->lICsi, u->lIEta, u->lIZet, u->lJCsi, u->lJEta, u->lJZet,
                        u->lKCsi, u->lKEta, u->lKZet, u->lIAj,  u->lJAj,  u->lKAj,
                        u->lAj,   u->lCsi,  u->lEta,  u->lZet};
  for (int q = 0; q < DESC_ARRAYS; q++) {
    hold[q] = NULL;
    if (q < 13 || fine) VecGetArray(v[q], &hold[q]);
  }
  d->icsi = hold[0]; d->ieta = hold[1]; d->izet = hold[2];
  d->jcsi = hold[3]; d->jeta = hold[4]; d->jzet = hold[5];
  d->kcsi = hold[6]; d->keta = hold[7]; d->kzet = hold[8];
  d->iaj = hold[9]; d->jaj = hold[10]; d->kaj = hold[11]; d->aj = hold[12];
  d->csi = hold[13]; d->eta = hold[14]; d->zet = hold[15];
}

static void desc_restore(UserCtx *u, PetscScalar *hold[DESC_ARRAYS]) {
  Vec v[DESC_ARRAYS] = {u->lICsi, u->lIEta, u->lIZet, u->lJCsi, u->lJEta, u->lJZet,
                        u->lKCsi, u->lKEta, u->lKZet, u->lIAj,  u->lJAj,  u->lKAj,
                        u->lAj,   u->lCsi,  u->lEta,  u->lZet};
  for (int q = 0; q < DESC_ARRAYS; q++)
    if (hold[q]) VecRestoreArray(v[q], &hold[q]);
}

/* PETSc's options database -> cvb_solve_opts.  The names are the ones the
 * reference's KSP reads under its "ps_" prefix (poisson.c:1829) and the
 * library's own; libcvb parses and checks the values. */
static PetscErrorCode read_options(void) {
  static const char *const names[] = {"-ps_ksp_rtol",    "-ps_ksp_atol",     "-ps_ksp_max_it",
                                      "-ps_ksp_gmres_restart", "-cvb_precision", "-cvb_smoother",
                                      "-cvb_pre_sweeps", "-cvb_post_sweeps", "-cvb_omega",
                                      "-cvb_coarse_dense_max"};
  enum { NOPT = sizeof names / sizeof names[0] };
  char values[NOPT][64];
  const char *tok[2 * NOPT];
  int n = 0;
  cvb_solve_opts_default(&g_opts);
  for (int q = 0; q < NOPT; q++) {
    PetscBool set = PETSC_FALSE;
    values[q][0] = 0;
    PetscOptionsGetString(PETSC_NULL, names[q], values[q], sizeof values[q], &set);
    if (set) { tok[n++] = names[q]; tok[n++] = values[q]; }
  }
  char bad[96] = "";
  int rc = cvb_solve_opts_from_args(n, tok, &g_opts, bad, (int)sizeof bad);
  if (rc) PetscPrintf(PETSC_COMM_WORLD, "PoissonSetup_GB300: bad option %s\n", bad);
  return rc;
}

PetscErrorCode PoissonSetup_GB300(UserMG *usermg) {
  const int nl = usermg->mglevels;
  if (block_number != 1 || nl < 1 || nl > 16) {
    PetscPrintf(PETSC_COMM_WORLD, "PoissonSetup_GB300: one block and 1-16 levels only\n");
    return CVB_BAD_INPUT;
  }
  int rc = read_options();
  if (rc) return rc;
  g_cent_given = 0;
  if (!g_cvb) {
    cvb_options o;
    memset(&o, 0, sizeof o); /* device 0, the context's own stream */
    rc = cvb_init(&g_cvb, &o);
    if (rc) return report(rc, "PoissonSetup_GB300");
  }
  cvb_level_desc d[16];
  PetscScalar *hold[16][DESC_ARRAYS];
  for (int l = 0; l < nl; l++) desc_get(&usermg->mgctx[l].user[0], &d[l], l == nl - 1, hold[l]);
  PetscScalar *nv;
  VecGetArray(finest(usermg)->lNvert, &nv);
  rc = cvb_setup_hierarchy(g_cvb, nl, d, nv);
  VecRestoreArray(finest(usermg)->lNvert, &nv);
  for (int l = 0; l < nl; l++) desc_restore(&usermg->mgctx[l].user[0], hold[l]);
  return report(rc, "PoissonSetup_GB300");
}

PetscErrorCode PoissonSetNvert_GB300(UserMG *usermg) {
  PetscScalar *nv;
  VecGetArray(finest(usermg)->lNvert, &nv);
  int rc = cvb_set_nvert(g_cvb, nv);
  VecRestoreArray(finest(usermg)->lNvert, &nv);
  return report(rc, "PoissonSetNvert_GB300");
}

/* VolumeFlux_rev(flg = immersed) corrects Ucont in place, PoissonRHS forms B
 * from it, and the solve writes Phi (poisson.c:1775-2017).  The ghosted copies
 * of what changed are refreshed as the reference leaves them: lPhi after the
 * solve (poisson.c:1985-1986) and lUcont, which VolumeFlux_rev's corrections
 * reach through the global vector. */
PetscErrorCode PoissonSolver_MG_GB300(UserMG *usermg) {
  UserCtx *u = finest(usermg);
  cvb_solve_stats st;
  PetscScalar *uc, *phi;
  memset(&st, 0, sizeof st);
  VecGetArray(u->Ucont, &uc);
  VecGetArray(u->Phi, &phi);
  int rc = cvb_poisson_solver_mg(g_cvb, uc, u->FluxIntpSum, (int)immersed, u->dt, u->st, phi, &g_opts, &st);
  VecRestoreArray(u->Phi, &phi);
  VecRestoreArray(u->Ucont, &uc);
  PetscPrintf(PETSC_COMM_WORLD, "PoissonSolver_MG_GB300: %d iterations, relative residual %e\n",
              st.iterations, st.rel_residual);
  DMGlobalToLocalBegin(u->fda, u->Ucont, INSERT_VALUES, u->lUcont);
  DMGlobalToLocalEnd(u->fda, u->Ucont, INSERT_VALUES, u->lUcont);
  DMGlobalToLocalBegin(u->da, u->Phi, INSERT_VALUES, u->lPhi);
  DMGlobalToLocalEnd(u->da, u->Phi, INSERT_VALUES, u->lPhi);
  return report(rc, "PoissonSolver_MG_GB300");
}

/* P += Phi with the periodic ring copies of both, then the ghosted copies
 * (poisson.c:2908-3248 ends with lP and lPhi refreshed). */
PetscErrorCode UpdatePressure_GB300(UserCtx *u) {
  PetscScalar *p, *phi;
  VecGetArray(u->P, &p);
  VecGetArray(u->Phi, &phi);
  int rc = cvb_update_pressure(g_cvb, p, phi);
  VecRestoreArray(u->Phi, &phi);
  VecRestoreArray(u->P, &p);
  DMGlobalToLocalBegin(u->da, u->P, INSERT_VALUES, u->lP);
  DMGlobalToLocalEnd(u->da, u->P, INSERT_VALUES, u->lP);
  DMGlobalToLocalBegin(u->da, u->Phi, INSERT_VALUES, u->lPhi);
  DMGlobalToLocalEnd(u->da, u->Phi, INSERT_VALUES, u->lPhi);
  return report(rc, "UpdatePressure_GB300");
}

/* GhostNodeVelocity's boundary types libcvb covers: all but the wall
 * function.  An annulus face (bctype[2] 11) reads the cell centres and a
 * rheology plate (13) the velocity U_bc; ghost_inputs hands them over (the
 * centres once per set-up). */
static int ghost_on_device(const UserCtx *u) {
  (void)u;
  return !wallfunction;
}

static int ghost_inputs(UserCtx *u) {
  int rc = 0;
  if (u->bctype[2] == 11 && !g_cent_given) {
    PetscScalar *cent;
    VecGetArray(u->Cent, &cent);
    rc = cvb_set_cell_centres(g_cvb, cent);
    VecRestoreArray(u->Cent, &cent);
    if (rc) return rc;
    g_cent_given = 1;
  }
  for (int f = 2; f < 6; f++)
    if (u->bctype[f] == 13) return cvb_set_plate_velocity(g_cvb, U_bc);
  return 0;
}

/* Projection (poisson.c:2281-2904): the flux correction, lUcont refreshed,
 * Contra2Cart and GhostNodeVelocity.  With covered boundary types all of it
 * runs on the device in one call (Ucat, Bcs.Ubcs and Ucont copied once);
 * otherwise the flux correction does, and the reference's own Contra2Cart and
 * GhostNodeVelocity follow on the host.  lUcont and lUcat end refreshed, as
 * the reference leaves them. */
PetscErrorCode Projection_GB300(UserCtx *u) {
  PetscScalar *phi, *uc;
  int rc;
  VecGetArray(u->Phi, &phi);
  VecGetArray(u->Ucont, &uc);
  if (ghost_on_device(u)) {
    PetscScalar *ub, *ucat;
    rc = ghost_inputs(u);
    if (rc) {
      VecRestoreArray(u->Ucont, &uc);
      VecRestoreArray(u->Phi, &phi);
      return report(rc, "Projection_GB300");
    }
    VecGetArray(u->Bcs.Ubcs, &ub);
    VecGetArray(u->Ucat, &ucat);
    rc = cvb_projection_cart(g_cvb, phi, u->dt, u->st, uc, ub, ucat);
    VecRestoreArray(u->Ucat, &ucat);
    VecRestoreArray(u->Bcs.Ubcs, &ub);
    VecRestoreArray(u->Ucont, &uc);
    VecRestoreArray(u->Phi, &phi);
    if (rc) return report(rc, "Projection_GB300");
    DMGlobalToLocalBegin(u->fda, u->Ucont, INSERT_VALUES, u->lUcont);
    DMGlobalToLocalEnd(u->fda, u->Ucont, INSERT_VALUES, u->lUcont);
    DMGlobalToLocalBegin(u->fda, u->Ucat, INSERT_VALUES, u->lUcat);
    DMGlobalToLocalEnd(u->fda, u->Ucat, INSERT_VALUES, u->lUcat);
    return 0;
  }
  rc = cvb_projection(g_cvb, phi, u->dt, u->st, uc);
  VecRestoreArray(u->Ucont, &uc);
  VecRestoreArray(u->Phi, &phi);
  if (rc) return report(rc, "Projection_GB300");
  DMGlobalToLocalBegin(u->fda, u->Ucont, INSERT_VALUES, u->lUcont);
  DMGlobalToLocalEnd(u->fda, u->Ucont, INSERT_VALUES, u->lUcont);
  Contra2Cart(u);
  GhostNodeVelocity(u);
  return 0;
}

/* Convection (rhs.c:1463-1946) with the reference's arguments (FormFunction1
 * passes lUcont and lUcat, rhs.c:2651), on the device for every boundary type.
 * -central or les selects the central form, as in the reference.  On one rank
 * without periodic faces the local vectors are the box itself and go to the
 * library as they are; a periodic DMDA's local vectors carry ghost planes, so
 * the owned box is taken out of them and Conv is written back into its owned
 * part (its ghost cells are 0, as the reference's VecSet leaves them).  nvert
 * is the one the context was last given (PoissonSetNvert_GB300 after a body
 * moves). */
PetscErrorCode Convection_GB300(UserCtx *u, Vec Ucont, Vec Ucat, Vec Conv) {
  const int mx = u->info.mx, my = u->info.my, mz = u->info.mz;
  const PetscInt box = 3 * (PetscInt)mx * my * mz;
  PetscInt gxs, gys, gzs, gxm, gym, gzm;
  DMDAGetGhostCorners(u->fda, &gxs, &gys, &gzs, &gxm, &gym, &gzm);
  const PetscInt ghosted = 3 * (PetscInt)gxm * gym * gzm;
  PetscInt n_uc = -1, n_ucat = -1, n_conv = -1;
  VecGetLocalSize(Ucont, &n_uc);
  VecGetLocalSize(Ucat, &n_ucat);
  VecGetLocalSize(Conv, &n_conv);
  const int as_box = n_uc == box && n_ucat == box && n_conv == box;
  const int as_ghosted = n_uc == ghosted && n_ucat == ghosted && n_conv == ghosted && gxs <= 0 && gys <= 0 &&
                         gzs <= 0 && gxs + gxm >= mx && gys + gym >= my && gzs + gzm >= mz;
  if (!as_box && !as_ghosted) {
    PetscPrintf(PETSC_COMM_WORLD, "Convection_GB300: vectors of %d/%d/%d values, box needs %d (one rank only)\n",
                (int)n_uc, (int)n_ucat, (int)n_conv, (int)box);
    return CVB_BAD_INPUT;
  }
  PetscInt central = 0;
  PetscOptionsGetInt(PETSC_NULL, "-central", &central, PETSC_NULL);
  PetscScalar *uc, *ucat, *conv;
  VecGetArray(Ucont, &uc);
  VecGetArray(Ucat, &ucat);
  VecGetArray(Conv, &conv);
  int rc;
  if (as_box) {
    rc = cvb_convection(g_cvb, uc, ucat, (les || central) ? 1 : 0, conv);
  } else {
    double *bu = (double *)malloc(sizeof(double) * box), *bc = (double *)malloc(sizeof(double) * box),
           *bo = (double *)malloc(sizeof(double) * box);
    rc = (bu && bc && bo) ? CVB_OK : CVB_OOM;
    for (int k = 0; k < mz && rc == CVB_OK; k++)
      for (int j = 0; j < my; j++)
        for (int i = 0; i < mx; i++) {
          const size_t b = 3 * (((size_t)k * my + j) * mx + i);
          const size_t l = 3 * (((size_t)(k - gzs) * gym + (j - gys)) * gxm + (i - gxs));
          for (int c = 0; c < 3; c++) { bu[b + c] = uc[l + c]; bc[b + c] = ucat[l + c]; }
        }
    if (rc == CVB_OK) rc = cvb_convection(g_cvb, bu, bc, (les || central) ? 1 : 0, bo);
    if (rc == CVB_OK) {
      memset(conv, 0, sizeof(double) * ghosted);
      for (int k = 0; k < mz; k++)
        for (int j = 0; j < my; j++)
          for (int i = 0; i < mx; i++) {
            const size_t b = 3 * (((size_t)k * my + j) * mx + i);
            const size_t l = 3 * (((size_t)(k - gzs) * gym + (j - gys)) * gxm + (i - gxs));
            for (int c = 0; c < 3; c++) conv[l + c] = bo[b + c];
          }
    }
    free(bu);
    free(bc);
    free(bo);
  }
  VecRestoreArray(Conv, &conv);
  VecRestoreArray(Ucat, &ucat);
  VecRestoreArray(Ucont, &uc);
  return report(rc, "Convection_GB300");
}

/* ImpRK (implicitsolver.c:7094-7257) with the reference's arguments.  On one
 * block with no immersed body, no LES / RANS / wall model, solid walls on the
 * x and y faces and on the k faces walls or an inlet (5, any profile; the
 * table ones, 0 and 5, for ti below 2000) with an outlet (4), the whole pseudo-time iteration runs on the device
 * (cvb_imp_rk: InflowFlux, FormBCS, CalcRHS, the Runge-Kutta stage updates,
 * the norms and the step halving), with the reference's -cfl, -imp_atol,
 * -imp_rtol, -imp_MAX_IT, -inlet (inletprofile) and -central and the block's
 * FluxIntpSum; Ucont, Bcs.Ubcs, Ucat and P come back and the local copies
 * are refreshed, as the reference leaves them.  Any other configuration runs
 * the reference's own ImpRK. */
/* The shaped inlet profiles read the k = 0 node plane of the local
 * coordinates (bcs.c:130-160) and CMx_c, CMy_c, CMz_c: copied out of the
 * ghosted local array and handed over before every ImpRK (the centre may
 * move). */
static int inlet_nodes(UserCtx *u) {
  const DMDALocalInfo *f = &u->info;
  const int mx = f->mx, my = f->my;
  double *plane = malloc(sizeof(double) * 3 * (size_t)mx * my);
  if (!plane) return CVB_OOM;
  Vec Coor;
  PetscScalar *c;
  DMGetCoordinatesLocal(u->da, &Coor);
  VecGetArray(Coor, &c);
  for (int j = 0; j < my; j++)
    for (int i = 0; i < mx; i++) {
      const size_t l = 3 * (((size_t)(0 - f->gzs) * f->gym + (j - f->gys)) * f->gxm + (i - f->gxs));
      for (int d = 0; d < 3; d++) plane[3 * ((size_t)j * mx + i) + d] = c[l + d];
    }
  VecRestoreArray(Coor, &c);
  const int rc = cvb_set_inlet_nodes(g_cvb, plane, CMx_c, CMy_c, CMz_c);
  free(plane);
  return rc;
}

PetscErrorCode ImpRK_GB300(UserCtx *u, IBMNodes *ibm, FSInfo *fsi) {
  const PetscInt *bt = u->bctype;
  int covered = bt[0] == 1 && bt[1] == 1 && bt[2] == 1 && bt[3] == 1 && (bt[4] == 1 || bt[4] == 5) &&
                (bt[5] == 1 || bt[5] == 4) && ((bt[4] == 5) == (bt[5] == 4));
  const int shaped = inletprofile == 2 || inletprofile == 4 || inletprofile == 7 || inletprofile == 10;
  const int uniform = inletprofile == 3 || inletprofile == 6 || inletprofile == 8;
  /* the table profiles, within the table (bcs.c:73) */
  const int table = (inletprofile == 0 || inletprofile == 5) && ti >= 0 && ti < 2000;
  if (bt[4] == 5)
    covered = covered && (inletprofile == 1 || inletprofile == -1 || inletprofile == 11 || shaped || uniform || table);
  if (!g_cvb || block_number != 1 || immersed || les || rans || wallfunction || !covered || !u->Ucont_o ||
      !u->Ucont_rm1)
    return ImpRK(u, ibm, fsi);
  if (bt[4] == 5 && (shaped || table)) {
    int rc = inlet_nodes(u);
    if (!rc && table) rc = cvb_set_inlet_table(g_cvb, &u->uinr[0][0]);
    if (rc) return report(rc, "ImpRK_GB300");
  }
  if (bt[4] == 5 && uniform) cvb_set_inlet_flux(g_cvb, Flux_in, (int)ti);
  PetscInt central = 0;
  PetscOptionsGetInt(PETSC_NULL, "-central", &central, PETSC_NULL);
  PetscScalar *uc, *uo, *urm, *ucat, *p, *ub;
  VecGetArray(u->Ucont, &uc);
  VecGetArray(u->Ucont_o, &uo);
  VecGetArray(u->Ucont_rm1, &urm);
  VecGetArray(u->Ucat, &ucat);
  VecGetArray(u->P, &p);
  VecGetArray(u->Bcs.Ubcs, &ub);
  cvb_imp_rk_opts o;
  cvb_imp_rk_opts_default(&o);
  o.ren = u->ren;
  o.dt = u->dt;
  o.st = u->st;
  o.cfl = u->cfl;
  o.ti = (int)ti;
  o.tistart = (int)tistart;
  o.central = central ? 1 : 0;
  o.imp_atol = imp_atol;
  o.imp_rtol = imp_rtol;
  o.imp_max_it = (int)imp_MAX_IT;
  o.inletprofile = (int)inletprofile;
  o.flux_intp_sum = u->FluxIntpSum;
  cvb_imp_rk_stats st;
  int rc = cvb_imp_rk(g_cvb, uc, uo, urm, ucat, p, ub, &o, &st);
  VecRestoreArray(u->Bcs.Ubcs, &ub);
  VecRestoreArray(u->P, &p);
  VecRestoreArray(u->Ucat, &ucat);
  VecRestoreArray(u->Ucont_rm1, &urm);
  VecRestoreArray(u->Ucont_o, &uo);
  VecRestoreArray(u->Ucont, &uc);
  if (rc) return report(rc, "ImpRK_GB300");
  if (bt[4] == 5) FluxInSum = u->FluxInSum = st.flux_in_sum; /* as InflowFlux leaves them (bcs.c:242, 383) */
  if (bt[4] == 5 && uniform) Flux_in = cvb_inlet_flux_in(g_cvb); /* profile 8 sets it (bcs.c:76) */
  PetscPrintf(PETSC_COMM_WORLD, "ImpRK_GB300: %d pseudo-time iterations (%d undone), |dU| %le, rel %le, |F| %le\n",
              st.pseudo_iterations, st.rejected, st.norm_du, st.rel_du, st.norm_f);
  DMGlobalToLocalBegin(u->fda, u->Ucont, INSERT_VALUES, u->lUcont);
  DMGlobalToLocalEnd(u->fda, u->Ucont, INSERT_VALUES, u->lUcont);
  DMGlobalToLocalBegin(u->fda, u->Ucat, INSERT_VALUES, u->lUcat);
  DMGlobalToLocalEnd(u->fda, u->Ucat, INSERT_VALUES, u->lUcat);
  DMGlobalToLocalBegin(u->da, u->P, INSERT_VALUES, u->lP);
  DMGlobalToLocalEnd(u->da, u->P, INSERT_VALUES, u->lP);
  return 0;
}

PetscErrorCode PoissonFinalize_GB300(void) {
  if (g_cvb) cvb_destroy(g_cvb);
  g_cvb = NULL;
  return 0;
}
