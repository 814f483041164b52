/* TEST INFRASTRUCTURE ONLY: see cvb_record.h. */
#include <stdlib.h>
#include <string.h>
#include "cvb_record.h"

cvb_record REC;
static int g_ctx_token;

int cvb_solve_opts_default(cvb_solve_opts *o) {
  memset(o, 0, sizeof *o);
  o->precision = CVB_PRECISION_MIXED;
  o->rtol = 1e-8;
  o->max_it = 200;
  o->restart = 30;
  return CVB_OK;
}

/* Keeps the tokens; understands -ps_ksp_rtol and -cvb_precision, and refuses
 * the value "bad", which is all the binding's test needs (the real parser has
 * its own tests). */
int cvb_solve_opts_from_args(int argc, const char *const *argv, cvb_solve_opts *o, char *bad, int bad_len) {
  REC.ntok = 0;
  for (int q = 0; q < argc && q < REC_MAXTOK; q++) {
    strncpy(REC.tok[q], argv[q], 63);
    REC.tok[q][63] = 0;
    REC.ntok++;
  }
  for (int q = 0; q + 1 < argc; q += 2) {
    if (!strcmp(argv[q + 1], "bad")) {
      if (bad && bad_len > 0) { strncpy(bad, argv[q], (size_t)bad_len - 1); bad[bad_len - 1] = 0; }
      return CVB_BAD_INPUT;
    }
    if (!strcmp(argv[q], "-ps_ksp_rtol")) o->rtol = strtod(argv[q + 1], NULL);
    if (!strcmp(argv[q], "-cvb_precision")) o->precision = strcmp(argv[q + 1], "fp64") ? CVB_PRECISION_MIXED : CVB_PRECISION_FP64;
  }
  return CVB_OK;
}

int cvb_init(cvb_ctx **ctx, const cvb_options *opts) {
  (void)opts;
  REC.n_init++;
  *ctx = (cvb_ctx *)&g_ctx_token;
  return CVB_OK;
}
void cvb_destroy(cvb_ctx *ctx) {
  (void)ctx;
  REC.n_destroy++;
}
const char *cvb_last_error(const cvb_ctx *ctx) {
  (void)ctx;
  REC.n_last_error++;
  return "recorded failure";
}

static int take_status(void) {
  int rc = REC.fail_next;
  REC.fail_next = 0;
  return rc;
}

int cvb_setup_hierarchy(cvb_ctx *ctx, int nlevels, const cvb_level_desc *levels, const double *nvert_finest) {
  (void)ctx;
  REC.n_setup++;
  REC.nlevels = nlevels;
  for (int l = 0; l < nlevels && l < 16; l++) REC.levels[l] = levels[l];
  REC.nvert = nvert_finest;
  return take_status();
}
int cvb_set_nvert(cvb_ctx *ctx, const double *nvert_finest) {
  (void)ctx;
  REC.n_set_nvert++;
  REC.nvert = nvert_finest;
  return take_status();
}
int cvb_poisson_solver_mg(cvb_ctx *ctx, double *ucont, double flux_intp_sum, int immersed, double dt, double st,
                          double *phi, const cvb_solve_opts *opts, cvb_solve_stats *stats) {
  (void)ctx;
  REC.n_solver_mg++;
  REC.ucont = ucont; REC.phi = phi;
  REC.flux_intp_sum = flux_intp_sum; REC.immersed = immersed; REC.dt = dt; REC.st = st;
  REC.opts = *opts;
  ucont[3 * REC.mark + 1] = 42.0;
  phi[REC.mark] = 3.0;
  memset(stats, 0, sizeof *stats);
  stats->iterations = 6;
  stats->status = REC.fail_next;
  return take_status();
}
int cvb_update_pressure(cvb_ctx *ctx, double *p, double *phi) {
  (void)ctx;
  REC.n_update++;
  REC.p = p; REC.phi_up = phi;
  p[REC.mark] = 7.0;
  return take_status();
}
int cvb_projection(cvb_ctx *ctx, const double *phi, double dt, double st, double *ucont) {
  (void)ctx;
  REC.n_projection++;
  REC.phi_proj = phi; REC.dt_proj = dt; REC.st_proj = st; REC.ucont_proj = ucont;
  ucont[3 * REC.mark] = 5.0;
  return take_status();
}
int cvb_convection(cvb_ctx *ctx, const double *ucont, const double *ucat, int central, double *conv) {
  (void)ctx;
  REC.n_convection++;
  REC.ucont_conv = ucont; REC.ucat_conv = ucat; REC.central_conv = central; REC.conv_conv = conv;
  conv[3 * REC.mark] = 7.0;
  return take_status();
}
int cvb_set_cell_centres(cvb_ctx *ctx, const double *cent) {
  (void)ctx;
  REC.n_set_cent++;
  REC.cent = cent;
  return CVB_OK;
}
int cvb_set_inlet_nodes(cvb_ctx *ctx, const double *coor0, double cmx, double cmy, double cmz) {
  (void)ctx;
  REC.n_inlet_nodes++;
  memcpy(REC.inlet_plane, coor0, sizeof REC.inlet_plane);
  REC.inlet_cm[0] = cmx;
  REC.inlet_cm[1] = cmy;
  REC.inlet_cm[2] = cmz;
  return CVB_OK;
}
int cvb_set_inlet_flux(cvb_ctx *ctx, double flux_in, int ti) {
  (void)ctx;
  REC.n_inlet_flux++;
  REC.inlet_flux_in = flux_in;
  REC.inlet_ti = ti;
  return CVB_OK;
}
double cvb_inlet_flux_in(const cvb_ctx *ctx) {
  (void)ctx;
  return 0.875;
}
int cvb_set_inlet_table(cvb_ctx *ctx, const double *uinr) {
  (void)ctx;
  REC.inlet_table = uinr;
  return CVB_OK;
}
int cvb_set_plate_velocity(cvb_ctx *ctx, double u_bc) {
  (void)ctx;
  REC.u_bc = u_bc;
  return CVB_OK;
}
void cvb_imp_rk_opts_default(cvb_imp_rk_opts *o) {
  memset(o, 0, sizeof *o);
  o->ren = o->dt = o->st = 1.;
  o->cfl = 0.2;
  o->ti = 1;
  o->imp_atol = 1e-7;
  o->imp_rtol = 1e-4;
  o->imp_max_it = 50;
  o->inletprofile = 1;
}
int cvb_imp_rk(cvb_ctx *ctx, double *ucont, const double *ucont_o, const double *ucont_rm1, double *ucat, double *p,
               double *ubcs, const cvb_imp_rk_opts *o, cvb_imp_rk_stats *stats) {
  (void)ctx;
  REC.n_imp_rk++;
  REC.ucont_imp = ucont; REC.uo_imp = ucont_o; REC.urm_imp = ucont_rm1; REC.ucat_imp = ucat; REC.p_imp = p;
  REC.ubcs_imp = ubcs; REC.ren_imp = o->ren; REC.dt_imp = o->dt; REC.st_imp = o->st; REC.cfl_imp = o->cfl;
  REC.ti_imp = o->ti; REC.tistart_imp = o->tistart; REC.central_imp = o->central; REC.atol_imp = o->imp_atol;
  REC.rtol_imp = o->imp_rtol; REC.max_it_imp = o->imp_max_it; REC.profile_imp = o->inletprofile;
  REC.intp_imp = o->flux_intp_sum;
  ucont[3 * REC.mark] = 11.0;
  ucat[3 * REC.mark + 1] = 12.0;
  p[REC.mark] = 13.0;
  ubcs[3 * REC.mark + 2] = 14.0;
  if (stats) {
    memset(stats, 0, sizeof *stats);
    stats->flux_in_sum = 0.5;
  }
  return take_status();
}
int cvb_projection_cart(cvb_ctx *ctx, const double *phi, double dt, double st, double *ucont, double *ubcs,
                        double *ucat) {
  (void)ctx;
  REC.n_projection_cart++;
  REC.phi_proj = phi; REC.dt_proj = dt; REC.st_proj = st; REC.ucont_proj = ucont;
  REC.ubcs_proj = ubcs; REC.ucat_proj = ucat;
  ucont[3 * REC.mark] = 5.0;
  ucat[3 * REC.mark + 2] = 9.0;
  return take_status();
}
