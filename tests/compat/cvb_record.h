/*
 * TEST INFRASTRUCTURE ONLY.  A recording stand-in for the libcvb entry points
 * the source-level binding (curvib_old_gb300/compat/poisson_gb300.c) calls, so
 * that the binding can run on a CPU against a real UserMG and the test can see
 * exactly which arrays and values reach the library.  Each path call also
 * writes one marked cell of the arrays it may change, so the test can check
 * that the binding refreshes the ghosted copies afterwards.
 */
#ifndef CVB_RECORD_H
#define CVB_RECORD_H
#include "cvb.h"

#define REC_MAXTOK 32

typedef struct {
  int n_init, n_destroy, n_last_error, n_setup, n_set_nvert, n_solver_mg, n_update, n_projection,
      n_projection_cart, n_convection, central_conv, n_imp_rk, n_set_cent;
  const double *cent;
  double u_bc;
  int ntok;
  char tok[REC_MAXTOK][64];
  int nlevels;
  cvb_level_desc levels[16];
  const double *nvert;
  /* cvb_poisson_solver_mg */
  double *ucont, *phi, flux_intp_sum, dt, st;
  int immersed;
  cvb_solve_opts opts;
  /* cvb_update_pressure */
  double *p, *phi_up;
  /* cvb_projection, cvb_projection_cart */
  const double *phi_proj;
  double *ucont_proj, dt_proj, st_proj;
  double *ubcs_proj, *ucat_proj;
  const double *ucont_conv, *ucat_conv;
  double *conv_conv;
  /* cvb_imp_rk */
  double *ucont_imp, *ucat_imp, *p_imp, *ubcs_imp;
  const double *uo_imp, *urm_imp;
  double ren_imp, dt_imp, st_imp, cfl_imp, atol_imp, rtol_imp, intp_imp;
  int ti_imp, tistart_imp, central_imp, max_it_imp, profile_imp;
  /* cvb_set_inlet_nodes: calls, a copy of the plane and the centre */
  int n_inlet_nodes;
  double inlet_plane[3 * 64 * 64], inlet_cm[3];
  /* cvb_set_inlet_flux (cvb_inlet_flux_in returns 0.875) */
  int n_inlet_flux, inlet_ti;
  const double *inlet_table; /* cvb_set_inlet_table */
  double inlet_flux_in;
  /* the status the next path call returns, then 0 again */
  int fail_next;
  /* cell (box index) the path calls write: solver_mg sets ucont[3m+1] = 42 and
   * phi[m] = 3; update_pressure sets p[m] = 7; projection sets ucont[3m] = 5;
   * projection_cart sets ucont[3m] = 5 and ucat[3m+2] = 9; imp_rk sets
 * ucont[3m] = 11, ucat[3m+1] = 12, p[m] = 13 and ubcs[3m+2] = 14, and
 * returns FluxInSum 0.5 */
  long mark;
} cvb_record;

extern cvb_record REC;

#endif
