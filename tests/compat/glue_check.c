/*
 * TEST INFRASTRUCTURE ONLY.  Runs the source-level binding
 * (curvib_old_gb300/compat/poisson_gb300.c) on a CPU against a real UserMG:
 * the hierarchy is built by the reference's own MG_Initial steps and
 * FormMetrics through the oracle's harness, and libcvb is the recording
 * stand-in of cvb_record.c.  Checks that every array handed to the library is
 * the right vector's own storage, that sizes, ghost boxes, boundary types,
 * options and scalars arrive unchanged, that the ghosted copies are refreshed
 * after each call as the reference leaves them, that every VecGetArray is
 * restored, and that failures come back as the call's status.
 *
 * usage: glue_check  -> prints one line per failed check, exits with their count
 */
#include <stdio.h>
#include <string.h>
#include "variables.h"
#include "cvb_record.h"
#include "poisson_gb300.h"

extern PetscInt block_number, immersed, wallfunction, les;
extern PetscInt ti, tistart, imp_MAX_IT;
extern PetscReal imp_atol, imp_rtol, FluxInSum, U_bc, CMx_c, CMy_c, CMz_c, Flux_in;
extern PetscInt inletprofile;
int ref_init(int nlevels, int IM, int JM, int KM, const int *bctype, int isc, int jsc, int ksc,
             const double *coords);
UserMG *ref_usermg(void);
double *shim_vec_data(Vec v);

static int g_checks = 0, g_fail = 0;
#define CHECK(cond, ...)                                   \
  do {                                                     \
    g_checks++;                                            \
    if (!(cond)) {                                         \
      g_fail++;                                            \
      printf("FAIL %s:%d: ", __FILE__, __LINE__);          \
      printf(__VA_ARGS__);                                 \
      printf("\n");                                        \
    }                                                      \
  } while (0)

/* Index of owned-box cell (i, j, k) in a level's ghosted local array. */
static long local_index(UserCtx *u, int i, int j, int k) {
  const DMDALocalInfo *f = &u->info;
  return ((long)(k - f->gzs) * f->gym + (j - f->gys)) * f->gxm + (i - f->gxs);
}

int main(void) {
  /* 16 x 8 x 8 cells (17 x 9 x 9 nodes), periodic in x, three levels */
  enum { IM = 17, JM = 9, KM = 9, NL = 3 };
  static double coords[3 * IM * JM * KM];
  for (int k = 0; k < KM; k++)
    for (int j = 0; j < JM; j++)
      for (int i = 0; i < IM; i++) {
        double *c = coords + 3 * ((k * JM + j) * IM + i);
        c[0] = 2.0 * i / (IM - 1);
        c[1] = (double)j / (JM - 1) + 0.05 * (double)(j * (JM - 1 - j)) / (JM * JM);
        c[2] = (double)k / (KM - 1);
      }
  const int bctype[6] = {7, 7, 1, 1, 1, 1};
  if (ref_init(NL, IM, JM, KM, bctype, 0, 0, 0, coords)) { printf("FAIL ref_init\n"); return 1; }
  UserMG *mg = ref_usermg();
  UserCtx *fine = &mg->mgctx[NL - 1].user[0];

  /* options as control.dat would give them; -d_taw is not the solver's */
  PetscOptionsClear();
  PetscOptionsSetValue("-ps_ksp_rtol", "1e-9");
  PetscOptionsSetValue("-cvb_precision", "fp64");
  PetscOptionsSetValue("-d_taw", "1");
  immersed = 1;

  /* --- set-up --- */
  memset(&REC, 0, sizeof REC);
  CHECK(PoissonSetup_GB300(mg) == 0, "PoissonSetup_GB300 failed");
  CHECK(REC.n_init == 1 && REC.n_setup == 1, "init %d setup %d", REC.n_init, REC.n_setup);
  CHECK(REC.ntok == 4 && !strcmp(REC.tok[0], "-ps_ksp_rtol") && !strcmp(REC.tok[1], "1e-9") &&
            !strcmp(REC.tok[2], "-cvb_precision") && !strcmp(REC.tok[3], "fp64"),
        "options forwarded: %d tokens", REC.ntok);
  CHECK(REC.nlevels == NL, "levels %d", REC.nlevels);
  for (int l = 0; l < NL; l++) {
    UserCtx *u = &mg->mgctx[l].user[0];
    const cvb_level_desc *d = &REC.levels[l];
    const DMDALocalInfo *f = &u->info;
    CHECK(d->mx == f->mx && d->my == f->my && d->mz == f->mz, "level %d box %d %d %d", l, d->mx, d->my, d->mz);
    CHECK(d->gxs == f->gxs && d->gys == f->gys && d->gzs == f->gzs && d->gxm == f->gxm && d->gym == f->gym &&
              d->gzm == f->gzm,
          "level %d ghost box", l);
    CHECK(d->mx == (l == NL - 1 ? IM + 1 : l == NL - 2 ? 10 : 6), "level %d mx %d", l, d->mx);
    for (int q = 0; q < 6; q++) CHECK(d->bctype[q] == bctype[q], "level %d bctype[%d]", l, q);
    CHECK(d->isc == u->isc && d->jsc == u->jsc && d->ksc == u->ksc, "level %d semi-coarsening", l);
    const double *got[13] = {d->icsi, d->ieta, d->izet, d->jcsi, d->jeta, d->jzet, d->kcsi,
                             d->keta, d->kzet, d->iaj,  d->jaj,  d->kaj,  d->aj};
    Vec want[13] = {u->lICsi, u->lIEta, u->lIZet, u->lJCsi, u->lJEta, u->lJZet, u->lKCsi,
                    u->lKEta, u->lKZet, u->lIAj,  u->lJAj,  u->lKAj,  u->lAj};
    for (int q = 0; q < 13; q++) CHECK(got[q] == shim_vec_data(want[q]), "level %d array %d", l, q);
    if (l == NL - 1)
      CHECK(d->csi == shim_vec_data(u->lCsi) && d->eta == shim_vec_data(u->lEta) &&
                d->zet == shim_vec_data(u->lZet),
            "finest centre metrics");
    else
      CHECK(!d->csi && !d->eta && !d->zet, "level %d centre metrics must be NULL", l);
  }
  CHECK(REC.nvert == shim_vec_data(fine->lNvert), "finest nvert");
  CHECK(shim_arrays_out() == 0, "set-up left %d arrays out", shim_arrays_out());

  /* --- PoissonSolver_MG --- */
  const int mi = 5, mj = 4, mk = 6; /* an interior cell */
  const DMDALocalInfo *ff = &fine->info;
  REC.mark = ((long)mk * ff->my + mj) * ff->mx + mi;
  const long loc = local_index(fine, mi, mj, mk);
  fine->FluxIntpSum = 0.125;
  fine->dt = 0.01;
  fine->st = 2.0;
  CHECK(PoissonSolver_MG_GB300(mg) == 0, "PoissonSolver_MG_GB300 failed");
  CHECK(REC.n_solver_mg == 1, "solver_mg calls %d", REC.n_solver_mg);
  CHECK(REC.ucont == shim_vec_data(fine->Ucont) && REC.phi == shim_vec_data(fine->Phi), "Ucont / Phi storage");
  CHECK(REC.flux_intp_sum == 0.125 && REC.immersed == 1 && REC.dt == 0.01 && REC.st == 2.0,
        "scalars %g %d %g %g", REC.flux_intp_sum, REC.immersed, REC.dt, REC.st);
  CHECK(REC.opts.rtol == 1e-9 && REC.opts.precision == CVB_PRECISION_FP64, "options rtol %g precision %d",
        REC.opts.rtol, REC.opts.precision);
  CHECK(shim_vec_data(fine->lUcont)[3 * loc + 1] == 42.0, "lUcont not refreshed after the solve");
  CHECK(shim_vec_data(fine->lPhi)[loc] == 3.0, "lPhi not refreshed after the solve");
  CHECK(shim_arrays_out() == 0, "solve left %d arrays out", shim_arrays_out());

  /* --- UpdatePressure --- */
  CHECK(UpdatePressure_GB300(fine) == 0, "UpdatePressure_GB300 failed");
  CHECK(REC.p == shim_vec_data(fine->P) && REC.phi_up == shim_vec_data(fine->Phi), "P / Phi storage");
  CHECK(shim_vec_data(fine->lP)[loc] == 7.0, "lP not refreshed");
  CHECK(shim_arrays_out() == 0, "update left %d arrays out", shim_arrays_out());

  /* --- Projection: covered boundary types, all on the device in one call --- */
  CHECK(Projection_GB300(fine) == 0, "Projection_GB300 failed");
  CHECK(REC.n_projection_cart == 1 && REC.n_projection == 0, "one-call projection not used");
  CHECK(REC.phi_proj == shim_vec_data(fine->Phi) && REC.ucont_proj == shim_vec_data(fine->Ucont) &&
            REC.ubcs_proj == shim_vec_data(fine->Bcs.Ubcs) && REC.ucat_proj == shim_vec_data(fine->Ucat),
        "Phi / Ucont / Bcs.Ubcs / Ucat storage");
  CHECK(REC.dt_proj == 0.01 && REC.st_proj == 2.0, "projection dt %g st %g", REC.dt_proj, REC.st_proj);
  CHECK(shim_vec_data(fine->lUcont)[3 * loc] == 5.0, "lUcont not refreshed after the projection");
  CHECK(shim_vec_data(fine->lUcat)[3 * loc + 2] == 9.0, "lUcat not refreshed after the projection");
  CHECK(shim_arrays_out() == 0, "projection left %d arrays out", shim_arrays_out());
  /* an annulus face: its cell centres (Cent's storage) go to the context once,
   * then the one-call projection; a rheology plate: U_bc goes with it */
  fine->bctype[2] = 11;
  CHECK(Projection_GB300(fine) == 0 && REC.n_projection_cart == 2 && REC.n_set_cent == 1 &&
            REC.cent == shim_vec_data(fine->Cent),
        "annulus face: centres not given or projection not on the device");
  CHECK(Projection_GB300(fine) == 0 && REC.n_projection_cart == 3 && REC.n_set_cent == 1,
        "annulus face: centres given again");
  fine->bctype[2] = 1;
  fine->bctype[4] = 13;
  U_bc = 0.625;
  CHECK(Projection_GB300(fine) == 0 && REC.n_projection_cart == 4 && REC.u_bc == 0.625,
        "rheology plate: U_bc not passed");
  fine->bctype[4] = 1;
  /* the wall function: flux correction on the device, the reference's own
   * Contra2Cart / GhostNodeVelocity on the host */
  wallfunction = 1;
  CHECK(Projection_GB300(fine) == 0 && REC.n_projection == 1 && REC.n_projection_cart == 4,
        "wall function: host post-projection not used");
  wallfunction = 0;
  CHECK(shim_arrays_out() == 0, "host-path projections left %d arrays out", shim_arrays_out());

  /* --- Convection: walled faces on the device, -central and les passed on.
   * This box is periodic in x, so the faces are made walled for these calls
   * and the box-shaped global vectors stand in for lUcont and lUcat (on one
   * rank without periodic faces the two have the same layout). --- */
  Vec Conv;
  VecDuplicate(fine->Ucont, &Conv);
  fine->bctype[0] = fine->bctype[1] = 1;
  CHECK(Convection_GB300(fine, fine->Ucont, fine->Ucat, Conv) == 0 && REC.n_convection == 1 &&
            REC.central_conv == 0, "convection not on the device");
  CHECK(REC.ucont_conv == shim_vec_data(fine->Ucont) && REC.ucat_conv == shim_vec_data(fine->Ucat) &&
            REC.conv_conv == shim_vec_data(Conv), "Ucont / Ucat / Conv storage");
  CHECK(shim_vec_data(Conv)[3 * REC.mark] == 7.0, "Conv not written");
  PetscOptionsSetValue("-central", "1");
  CHECK(Convection_GB300(fine, fine->Ucont, fine->Ucat, Conv) == 0 && REC.central_conv == 1, "-central not passed");
  PetscOptionsSetValue("-central", "0");
  les = 1;
  CHECK(Convection_GB300(fine, fine->Ucont, fine->Ucat, Conv) == 0 && REC.central_conv == 1, "les not passed");
  les = 0;
  fine->bctype[0] = fine->bctype[1] = 7;
  VecDestroy(&Conv);
  /* the periodic box as FormFunction1 passes it: ghosted local vectors; the
   * owned box goes to the library and Conv's owned part comes back */
  Vec ConvL;
  VecDuplicate(fine->lUcont, &ConvL);
  const int nconv = REC.n_convection;
  CHECK(Convection_GB300(fine, fine->lUcont, fine->lUcat, ConvL) == 0 && REC.n_convection == nconv + 1,
        "periodic convection not on the device");
  CHECK(REC.ucont_conv != shim_vec_data(fine->lUcont) && REC.conv_conv != shim_vec_data(ConvL),
        "ghosted vectors passed as boxes");
  CHECK(shim_vec_data(ConvL)[3 * loc] == 7.0, "Conv's owned part not written back");
  CHECK(shim_vec_data(ConvL)[0] == 0.0, "Conv's ghost cells not 0");
  VecDestroy(&ConvL);
  CHECK(shim_arrays_out() == 0, "convection left %d arrays out", shim_arrays_out());

  /* --- ImpRK: one block, immersed 0, walls on every face: on the device with
   * the block's and the run's controls; a failure comes back as the status --- */
  int bsave[6];
  for (int f = 0; f < 6; f++) { bsave[f] = fine->bctype[f]; fine->bctype[f] = 1; }
  VecDuplicate(fine->Ucont, &fine->Ucont_o);
  VecDuplicate(fine->Ucont, &fine->Ucont_rm1);
  const PetscInt imm_keep = immersed;
  immersed = 0;
  fine->cfl = 0.3;
  fine->ren = 250.0;
  ti = 4;
  tistart = 1;
  imp_MAX_IT = 7;
  imp_atol = 2e-7;
  imp_rtol = 3e-4;
  CHECK(ImpRK_GB300(fine, NULL, NULL) == 0 && REC.n_imp_rk == 1, "ImpRK not on the device");
  CHECK(REC.ucont_imp == shim_vec_data(fine->Ucont) && REC.uo_imp == shim_vec_data(fine->Ucont_o) &&
            REC.urm_imp == shim_vec_data(fine->Ucont_rm1) && REC.ucat_imp == shim_vec_data(fine->Ucat) &&
            REC.p_imp == shim_vec_data(fine->P) && REC.ubcs_imp == shim_vec_data(fine->Bcs.Ubcs),
        "Ucont / Ucont_o / Ucont_rm1 / Ucat / P / Bcs.Ubcs storage");
  CHECK(REC.ren_imp == 250.0 && REC.dt_imp == fine->dt && REC.st_imp == fine->st && REC.cfl_imp == 0.3 &&
            REC.ti_imp == 4 && REC.tistart_imp == 1 && REC.central_imp == 0 && REC.atol_imp == 2e-7 &&
            REC.rtol_imp == 3e-4 && REC.max_it_imp == 7,
        "ImpRK controls");
  CHECK(shim_vec_data(fine->lUcont)[3 * loc] == 11.0 && shim_vec_data(fine->lUcat)[3 * loc + 1] == 12.0 &&
            shim_vec_data(fine->lP)[loc] == 13.0,
        "lUcont / lUcat / lP not refreshed after ImpRK");
  /* an inlet on k = 0 and an outlet on the last face: the profile, the
   * block's immersed-boundary flux, and FluxInSum back as InflowFlux leaves it */
  fine->bctype[4] = 5;
  fine->bctype[5] = 4;
  inletprofile = 11;
  fine->FluxIntpSum = 0.25;
  FluxInSum = 0.0;
  CHECK(ImpRK_GB300(fine, NULL, NULL) == 0 && REC.n_imp_rk == 2 && REC.profile_imp == 11 && REC.intp_imp == 0.25,
        "inlet / outlet ImpRK not on the device with its profile and FluxIntpSum");
  CHECK(FluxInSum == 0.5 && fine->FluxInSum == 0.5, "FluxInSum not set after ImpRK");
  CHECK(REC.n_inlet_nodes == 0, "inlet nodes handed over for a constant profile");
  /* a shaped profile: the k = 0 node plane and the centre go first */
  inletprofile = 4;
  CMx_c = 0.5, CMy_c = 0.25, CMz_c = 0.125;
  CHECK(ImpRK_GB300(fine, NULL, NULL) == 0 && REC.n_imp_rk == 3 && REC.profile_imp == 4 && REC.n_inlet_nodes == 1,
        "shaped-profile ImpRK not on the device with the inlet's nodes");
  CHECK(REC.inlet_cm[0] == 0.5 && REC.inlet_cm[1] == 0.25 && REC.inlet_cm[2] == 0.125, "CMx_c / CMy_c / CMz_c");
  {
    int bad = 0;
    const int mx = fine->info.mx;
    for (int j = 0; j < JM; j++)
      for (int i = 0; i < IM; i++)
        for (int d = 0; d < 3; d++) bad += REC.inlet_plane[3 * (j * mx + i) + d] != coords[3 * (j * IM + i) + d];
    CHECK(bad == 0, "k = 0 node plane: %d coordinates differ", bad);
  }
  CMx_c = CMy_c = CMz_c = 0.0;
  /* a uniform profile: Flux_in and ti go first, Flux_in comes back */
  inletprofile = 8;
  Flux_in = 0.125;
  CHECK(ImpRK_GB300(fine, NULL, NULL) == 0 && REC.n_imp_rk == 4 && REC.profile_imp == 8 && REC.n_inlet_flux == 1 &&
            REC.inlet_flux_in == 0.125 && REC.inlet_ti == 4,
        "uniform-profile ImpRK not on the device with Flux_in and ti");
  CHECK(Flux_in == 0.875, "Flux_in not set after ImpRK with profile 8");
  /* a table profile: the nodes and the finest level's uinr go first */
  inletprofile = 5;
  CHECK(ImpRK_GB300(fine, NULL, NULL) == 0 && REC.n_imp_rk == 5 && REC.profile_imp == 5 && REC.n_inlet_nodes == 2 &&
            REC.inlet_table == &fine->uinr[0][0],
        "table-profile ImpRK not on the device with the nodes and uinr");
  inletprofile = 11;
  CHECK(shim_vec_data(fine->Bcs.Ubcs)[3 * REC.mark + 2] == 14.0, "Bcs.Ubcs not written back");
  fine->bctype[4] = fine->bctype[5] = 1;
  PetscOptionsSetValue("-central", "1");
  CHECK(ImpRK_GB300(fine, NULL, NULL) == 0 && REC.central_imp == 1, "-central not passed to ImpRK");
  PetscOptionsSetValue("-central", "0");
  REC.fail_next = CVB_NAN_DETECTED;
  CHECK(ImpRK_GB300(fine, NULL, NULL) == CVB_NAN_DETECTED, "ImpRK failure not returned");
  CHECK(shim_arrays_out() == 0, "ImpRK left %d arrays out", shim_arrays_out());
  immersed = imm_keep;
  for (int f = 0; f < 6; f++) fine->bctype[f] = bsave[f];

  /* --- failures come back as the call's status, arrays restored --- */
  REC.fail_next = CVB_NOT_CONVERGED;
  int before = REC.n_last_error;
  CHECK(PoissonSolver_MG_GB300(mg) == CVB_NOT_CONVERGED, "non-convergence not returned");
  CHECK(REC.n_last_error == before + 1, "message not fetched");
  CHECK(shim_arrays_out() == 0, "failed solve left %d arrays out", shim_arrays_out());
  REC.fail_next = CVB_CUDA_ERROR;
  CHECK(Projection_GB300(fine) == CVB_CUDA_ERROR, "projection failure not returned");
  fine->bctype[4] = 13;
  REC.fail_next = CVB_CUDA_ERROR;
  CHECK(Projection_GB300(fine) == CVB_CUDA_ERROR, "host-path projection failure not returned");
  fine->bctype[4] = 1;
  CHECK(shim_arrays_out() == 0, "failed projection left %d arrays out", shim_arrays_out());

  /* --- moving body: new nvert --- */
  CHECK(PoissonSetNvert_GB300(mg) == 0 && REC.n_set_nvert == 1 && REC.nvert == shim_vec_data(fine->lNvert),
        "PoissonSetNvert_GB300");

  /* --- refused inputs: a bad option value, more than one block --- */
  PetscOptionsSetValue("-cvb_precision", "bad");
  CHECK(PoissonSetup_GB300(mg) == CVB_BAD_INPUT, "bad option accepted");
  PetscOptionsSetValue("-cvb_precision", "fp64");
  block_number = 2;
  int setups = REC.n_setup;
  CHECK(PoissonSetup_GB300(mg) == CVB_BAD_INPUT && REC.n_setup == setups, "two blocks accepted");
  block_number = 1;
  CHECK(shim_arrays_out() == 0, "refused set-ups left %d arrays out", shim_arrays_out());

  CHECK(PoissonFinalize_GB300() == 0 && REC.n_destroy == 1 && REC.n_init == 1, "finalize: destroy %d init %d",
        REC.n_destroy, REC.n_init);

  printf("glue_check: %d checks, %d failures\n", g_checks, g_fail);
  return g_fail;
}
