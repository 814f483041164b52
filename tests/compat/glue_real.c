/*
 * TEST INFRASTRUCTURE ONLY.  Runs the source-level binding
 * (curvib_old_gb300/compat/poisson_gb300.c) against the real libcvb on a GPU,
 * on a UserMG that the reference's own MG_Initial steps and FormMetrics built
 * (oracle harness), and compares what the binding leaves in CURVIB's vectors
 * with what the reference's own routines compute from the same inputs:
 *   PoissonSolver_MG_GB300  -> Ucont as VolumeFlux_rev leaves it (1e-13, the
 *                              flux sums are added in another order), and a
 *                              Phi that solves the reference's PoissonLHSNew
 *                              system for its PoissonRHS (mean removed);
 *   UpdatePressure_GB300    -> P and Phi bit for bit (UpdatePressure);
 *   Projection_GB300        -> Ucont bit for bit (Projection's flux correction)
 *                              and Ucat bit for bit (Contra2Cart, then
 *                              GhostNodeVelocity);
 *   Convection_GB300        -> Conv bit for bit (Convection);
 *   ImpRK_GB300             -> Ucont, Ucat and P bit for bit (ImpRK with
 *                              immersed 0, on the fields the projection left).
 *
 * usage: glue_real fp64|mixed  -> prints one line per failed check, exits with their count
 */
#include <execinfo.h>
#include <math.h>
#include <signal.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "variables.h"
#include "cvb.h"
#include "poisson_gb300.h"

extern PetscInt block_number, immersed;
int ref_init(int nlevels, int IM, int JM, int KM, const int *bctype, int isc, int jsc, int ksc,
             const double *coords);
UserMG *ref_usermg(void);
double *shim_vec_data(Vec v);
int ref_set_nvert(int level, const double *nv);
int ref_set_ucont(const double *uc);
int ref_volume_flux(double flux_intp_sum, int flg, double *ucont_inout, double *flux, double *area);
int ref_rhs(double dt, double st, double *b, double *compat_sum);
int ref_lhs(int level, int *rowptr, int *cols, double *vals, int cap);
int ref_update_and_project(double dt, double st, double *p, double *phi, double *ucont);
int ref_contra2cart(const double *ucont, double *ucat);
int ref_ghost_node_velocity(double *ubcs, double *ucat);
int ref_convection(const double *ucont, const double *ucat, int central, double *conv);
int ref_imp_rk(double *ucont, const double *ucont_o, const double *ucont_rm1, double *ucat, double *p,
               double *ubcs, double ren, double dt, double st, double cfl, int ti_, int tistart_, int central,
               double atol, double rtol, int max_it, int profile, double flux_intp_sum);
extern PetscInt ti, tistart, imp_MAX_IT;
extern PetscReal imp_atol, imp_rtol;

static int g_checks = 0, g_fail = 0;
#define CHECK(cond, ...)                          \
  do {                                            \
    g_checks++;                                   \
    if (!(cond)) {                                \
      g_fail++;                                   \
      printf("FAIL %s:%d: ", __FILE__, __LINE__); \
      printf(__VA_ARGS__);                        \
      printf("\n");                               \
    }                                             \
  } while (0)

static double *copy_of(const double *a, size_t n) {
  double *b = (double *)malloc(sizeof(double) * n);
  memcpy(b, a, sizeof(double) * n);
  return b;
}
static int same(const double *a, const double *b, size_t n) { return memcmp(a, b, sizeof(double) * n) == 0; }
static double maxabs(const double *a, size_t n) {
  double m = 0;
  for (size_t q = 0; q < n; q++) m = fabs(a[q]) > m ? fabs(a[q]) : m;
  return m;
}

static const char *volatile g_step = "start";
#define STEP(name) (g_step = name, printf("step: %s\n", name), fflush(stdout))

/* a fault names the step it came in and the call stack (link with -rdynamic) */
static void on_fault(int sig) {
  fprintf(stderr, "signal %d in step %s\n", sig, g_step);
  void *pc[48];
  backtrace_symbols_fd(pc, backtrace(pc, 48), 2);
  signal(sig, SIG_DFL);
  raise(sig);
}

int main(int argc, char **argv) {
  setvbuf(stdout, NULL, _IONBF, 0);
  signal(SIGSEGV, on_fault);
  signal(SIGBUS, on_fault);
  const int mixed = argc > 1 && !strcmp(argv[1], "mixed");
  /* 16 x 12 x 10 cells, walls everywhere, stretched and sheared, three levels */
  enum { IM = 17, JM = 13, KM = 11, NL = 3 };
  static double coords[3 * IM * JM * KM];
  for (int k = 0; k < KM; k++)
    for (int j = 0; j < JM; j++)
      for (int i = 0; i < IM; i++) {
        double *c = coords + 3 * ((k * JM + j) * IM + i);
        const double eta = (double)j / (JM - 1);
        c[0] = 1.5 * i / (IM - 1) + 0.03 * sin(6.283185307179586 * eta);
        c[1] = 0.5 * (1.0 + tanh(1.5 * (2.0 * eta - 1.0)) / tanh(1.5));
        c[2] = (double)k / (KM - 1);
      }
  const int bctype[6] = {1, 1, 1, 1, 1, 1};
  STEP("ref_init");
  if (ref_init(NL, IM, JM, KM, bctype, 0, 0, 0, coords)) { printf("FAIL ref_init\n"); return 1; }
  UserMG *mg = ref_usermg();
  UserCtx *fine = &mg->mgctx[NL - 1].user[0];
  const int mx = fine->info.mx, my = fine->info.my, mz = fine->info.mz;
  const size_t n = (size_t)mx * my * mz;

  /* a body: solid cells 3 in a box, an immersed-boundary layer 1 around them */
  double *nv = (double *)calloc(n, sizeof(double));
  for (int k = 1; k < mz - 1; k++)
    for (int j = 1; j < my - 1; j++)
      for (int i = 1; i < mx - 1; i++) {
        const int in = i >= 6 && i <= 9 && j >= 5 && j <= 7 && k >= 4 && k <= 6;
        const int near = i >= 5 && i <= 10 && j >= 4 && j <= 8 && k >= 3 && k <= 7;
        nv[((size_t)k * my + j) * mx + i] = in ? 3.0 : near ? 1.0 : 0.0;
      }
  STEP("nvert");
  ref_set_nvert(NL - 1, nv);
  /* fluxes on the interior faces, zero on the walls */
  double *uc0 = (double *)calloc(3 * n, sizeof(double));
  unsigned s = 12345u;
  for (int k = 1; k < mz - 1; k++)
    for (int j = 1; j < my - 1; j++)
      for (int i = 1; i < mx - 1; i++)
        for (int c = 0; c < 3; c++) {
          const int q[3] = {i, j, k}, m[3] = {mx, my, mz};
          s = s * 1664525u + 1013904223u;
          if (q[c] < m[c] - 2) uc0[3 * (((size_t)k * my + j) * mx + i) + c] = (double)(s >> 8) / 16777216.0 - 0.5;
        }
  STEP("ucont");
  ref_set_ucont(uc0);

  PetscOptionsClear();
  PetscOptionsSetValue("-ps_ksp_rtol", "1e-11");
  PetscOptionsSetValue("-cvb_precision", mixed ? "mixed" : "fp64");
  immersed = 1;
  block_number = 1;
  fine->FluxIntpSum = 0.0;
  fine->dt = 0.01;
  fine->st = 1.0;

  /* --- the binding on the real library (refonly: skipped, the reference half
   * runs on the initial fields, to check this driver without a GPU) --- */
  const int refonly = argc > 2 && !strcmp(argv[2], "refonly");
  if (refonly) {
    double *z = (double *)calloc(3 * n, sizeof(double));
    double *uc_b = copy_of(uc0, 3 * n), *phi_b = z, *p_b = z, *phi_b2 = z, *uc_b2 = uc_b, *ucat_b = z, *conv_b = z;
    (void)p_b; (void)phi_b2; (void)ucat_b; (void)conv_b;
    STEP("reference routines");
    double *uc_r = copy_of(uc0, 3 * n), flux, area;
    ref_volume_flux(0.0, 1, uc_r, &flux, &area);
    STEP("rhs");
    double *b = (double *)malloc(sizeof(double) * n), sum;
    ref_rhs(fine->dt, fine->st, b, &sum);
    STEP("lhs");
    const int cap = (int)n * 19;
    int *rowptr = (int *)malloc(sizeof(int) * (n + 1)), *cols = (int *)malloc(sizeof(int) * cap);
    double *vals = (double *)malloc(sizeof(double) * cap);
    printf("lhs entries %d\n", ref_lhs(NL - 1, rowptr, cols, vals, cap));
    STEP("update_and_project");
    double *p_r = (double *)calloc(n, sizeof(double)), *phi_r = copy_of(phi_b, n), *uc_r2 = copy_of(uc_b, 3 * n);
    ref_update_and_project(fine->dt, fine->st, p_r, phi_r, uc_r2);
    STEP("contra2cart");
    double *ucat_r = (double *)calloc(3 * n, sizeof(double)), *ubcs_r = (double *)calloc(3 * n, sizeof(double));
    ref_contra2cart(uc_r2, ucat_r);
    STEP("ghost");
    ref_ghost_node_velocity(ubcs_r, ucat_r);
    STEP("convection");
    double *conv_r = (double *)calloc(3 * n, sizeof(double));
    ref_convection(uc_b2, ucat_r, 0, conv_r);
    STEP("imp_rk");
    double *im_uo = copy_of(uc_r2, 3 * n), *im_urm = copy_of(uc_r2, 3 * n), *im_ub = calloc(3 * n, sizeof(double));
    for (size_t q = 0; q < 3 * n; q++) { im_uo[q] *= 0.99; im_urm[q] *= 0.97; }
    immersed = 0;
    ref_imp_rk(uc_r2, im_uo, im_urm, ucat_r, p_r, im_ub, 300.0, 2e-3, 1.0, 0.5, 5, 0, 0, 1e-7, 1e-4, 6, 1, 0.0);
    int finite = 1;
    for (size_t q = 0; q < 3 * n; q++) finite = finite && isfinite(uc_r2[q]);
    printf("imp_rk finite %d, max |Ucont| %.3e\n", finite, maxabs(uc_r2, 3 * n));
    STEP("done");
    return 0;
  }
  STEP("PoissonSetup_GB300");
  CHECK(PoissonSetup_GB300(mg) == 0, "PoissonSetup_GB300 failed");
  STEP("PoissonSolver_MG_GB300");
  CHECK(PoissonSolver_MG_GB300(mg) == 0, "PoissonSolver_MG_GB300 failed");
  double *uc_b = copy_of(shim_vec_data(fine->Ucont), 3 * n), *phi_b = copy_of(shim_vec_data(fine->Phi), n);
  STEP("UpdatePressure_GB300");
  CHECK(UpdatePressure_GB300(fine) == 0, "UpdatePressure_GB300 failed");
  double *p_b = copy_of(shim_vec_data(fine->P), n), *phi_b2 = copy_of(shim_vec_data(fine->Phi), n);
  STEP("Projection_GB300");
  CHECK(Projection_GB300(fine) == 0, "Projection_GB300 failed");
  double *uc_b2 = copy_of(shim_vec_data(fine->Ucont), 3 * n), *ucat_b = copy_of(shim_vec_data(fine->Ucat), 3 * n);
  Vec Conv;
  VecDuplicate(fine->Ucont, &Conv);
  STEP("Convection_GB300");
  CHECK(Convection_GB300(fine, fine->Ucont, fine->Ucat, Conv) == 0, "Convection_GB300 failed");
  double *conv_b = copy_of(shim_vec_data(Conv), 3 * n);
  /* the momentum equation's pseudo-time iteration on the projected fields:
   * previous steps' fluxes close to Ucont, no-slip walls, immersed 0 */
  STEP("ImpRK_GB300");
  const double imp_dt = 2e-3, imp_cfl = 0.5, imp_ren = 300.0;
  double *im_uc = copy_of(uc_b2, 3 * n), *im_uo = copy_of(uc_b2, 3 * n), *im_urm = copy_of(uc_b2, 3 * n);
  for (size_t q = 0; q < 3 * n; q++) { im_uo[q] *= 0.99; im_urm[q] *= 0.97; }
  double *im_ucat = copy_of(ucat_b, 3 * n), *im_p = copy_of(p_b, n), *im_ub = (double *)calloc(3 * n, sizeof(double));
  if (!fine->Ucont_o) VecDuplicate(fine->Ucont, &fine->Ucont_o);
  if (!fine->Ucont_rm1) VecDuplicate(fine->Ucont, &fine->Ucont_rm1);
  memcpy(shim_vec_data(fine->Ucont), im_uc, sizeof(double) * 3 * n);
  memcpy(shim_vec_data(fine->Ucont_o), im_uo, sizeof(double) * 3 * n);
  memcpy(shim_vec_data(fine->Ucont_rm1), im_urm, sizeof(double) * 3 * n);
  memcpy(shim_vec_data(fine->Ucat), im_ucat, sizeof(double) * 3 * n);
  memcpy(shim_vec_data(fine->P), im_p, sizeof(double) * n);
  memcpy(shim_vec_data(fine->Bcs.Ubcs), im_ub, sizeof(double) * 3 * n);
  const double dt_keep = fine->dt;
  fine->dt = imp_dt;
  fine->cfl = imp_cfl;
  fine->ren = imp_ren;
  immersed = 0;
  ti = 5;
  tistart = 0;
  imp_MAX_IT = 6;
  imp_atol = 1e-7;
  imp_rtol = 1e-4;
  CHECK(ImpRK_GB300(fine, NULL, NULL) == 0, "ImpRK_GB300 failed");
  double *im_uc_b = copy_of(shim_vec_data(fine->Ucont), 3 * n), *im_ucat_b = copy_of(shim_vec_data(fine->Ucat), 3 * n),
         *im_p_b = copy_of(shim_vec_data(fine->P), n);
  immersed = 1;
  fine->dt = dt_keep;
  CHECK(PoissonFinalize_GB300() == 0, "PoissonFinalize_GB300 failed");

  /* --- the reference's own routines on the same inputs --- */
  STEP("reference routines");
  double *uc_r = copy_of(uc0, 3 * n), flux, area;
  ref_volume_flux(0.0, 1, uc_r, &flux, &area);
  double dmax = 0;
  for (size_t q = 0; q < 3 * n; q++) dmax = fabs(uc_r[q] - uc_b[q]) > dmax ? fabs(uc_r[q] - uc_b[q]) : dmax;
  CHECK(dmax <= 1e-13 * maxabs(uc_r, 3 * n), "VolumeFlux_rev: Ucont differs by %.3e", dmax);
  double *b = (double *)malloc(sizeof(double) * n), sum;
  ref_rhs(fine->dt, fine->st, b, &sum);
  const int cap = (int)n * 19;
  int *rowptr = (int *)malloc(sizeof(int) * (n + 1)), *cols = (int *)malloc(sizeof(int) * cap);
  double *vals = (double *)malloc(sizeof(double) * cap);
  CHECK(ref_lhs(NL - 1, rowptr, cols, vals, cap) > 0, "ref_lhs failed");
  /* residual of the binding's Phi on the fluid cells, after removing the part
   * of b outside the operator's range (aj times the fluid mean of b / aj) */
  /* FormMetrics destroys the global Aj (metrics.c:1221); on this walled box
   * the ghosted lAj is the box itself */
  double *aj = shim_vec_data(fine->lAj);
  double cs = 0, cn = 0;
  for (size_t q = 0; q < n; q++) {
    const int i = (int)(q % mx), j = (int)((q / mx) % my), k = (int)(q / ((size_t)mx * my));
    if (i >= 1 && i <= mx - 2 && j >= 1 && j <= my - 2 && k >= 1 && k <= mz - 2 && nv[q] < 0.1) {
      cs += b[q] / aj[q];
      cn += 1;
    }
  }
  double rn = 0, bn = 0;
  for (size_t q = 0; q < n; q++) {
    const int i = (int)(q % mx), j = (int)((q / mx) % my), k = (int)(q / ((size_t)mx * my));
    if (!(i >= 1 && i <= mx - 2 && j >= 1 && j <= my - 2 && k >= 1 && k <= mz - 2 && nv[q] < 0.1)) continue;
    double ax = 0;
    for (int e = rowptr[q]; e < rowptr[q + 1]; e++) ax += vals[e] * phi_b[cols[e]];
    const double bq = b[q] - aj[q] * cs / cn;
    rn += (bq - ax) * (bq - ax);
    bn += bq * bq;
  }
  CHECK(sqrt(rn) <= 1e-9 * sqrt(bn), "PoissonSolver_MG: relative residual %.3e on the reference's operator",
        sqrt(rn / bn));
  double *p_r = (double *)calloc(n, sizeof(double)), *phi_r = copy_of(phi_b, n), *uc_r2 = copy_of(uc_b, 3 * n);
  ref_update_and_project(fine->dt, fine->st, p_r, phi_r, uc_r2);
  CHECK(same(p_r, p_b, n) && same(phi_r, phi_b2, n), "UpdatePressure: P / Phi differ");
  CHECK(same(uc_r2, uc_b2, 3 * n), "Projection: Ucont differs");
  double *ucat_r = (double *)calloc(3 * n, sizeof(double)), *ubcs_r = (double *)calloc(3 * n, sizeof(double));
  ref_contra2cart(uc_r2, ucat_r);
  ref_ghost_node_velocity(ubcs_r, ucat_r);
  CHECK(same(ucat_r, ucat_b, 3 * n), "Contra2Cart + GhostNodeVelocity: Ucat differs");
  double *conv_r = (double *)calloc(3 * n, sizeof(double));
  ref_convection(uc_b2, ucat_b, 0, conv_r);
  CHECK(same(conv_r, conv_b, 3 * n), "Convection: Conv differs");

  /* ImpRK's own run on the same inputs (it leaves Converge_dU0 in the
   * working directory) */
  STEP("ImpRK");
  immersed = 0;
  fine->FluxIntpSum = 0.0;
  ref_imp_rk(im_uc, im_uo, im_urm, im_ucat, im_p, im_ub, imp_ren, imp_dt, 1.0, imp_cfl, 5, 0, 0, 1e-7, 1e-4, 6, 1, 0.0);
  int finite = 1;
  for (size_t q = 0; q < 3 * n; q++) finite = finite && isfinite(im_uc[q]);
  CHECK(finite, "ImpRK: Ucont not finite");
  CHECK(same(im_uc, im_uc_b, 3 * n) && same(im_ucat, im_ucat_b, 3 * n) && same(im_p, im_p_b, n),
        "ImpRK: Ucont / Ucat / P differ");
  printf("glue_real (%s): %d checks, %d failures\n", mixed ? "mixed" : "fp64", g_checks, g_fail);
  return g_fail;
}
