/*
 * cvb -- GB300 implementation of CURVIB's pressure-projection path behind a C ABI.
 *
 * Replaces, for one block on one GPU, the reference routines of poisson.c:
 *   PoissonRHS        (poisson.c:1509)  -> cvb_poisson_rhs
 *   PoissonLHSNew     (poisson.c:600)   -> built once by cvb_setup_hierarchy,
 *                                          applied matrix-free (cvb_apply_operator)
 *   PoissonSolver_MG  (poisson.c:1775)  -> cvb_poisson_solver_mg / cvb_poisson_solve
 *   VolumeFlux_rev    (poisson.c:3712)  -> cvb_volume_flux_rev
 *   MyNvertRestriction(poisson.c:1662), FullyBlocked (poisson.c:1578)
 *                                       -> cvb_setup_hierarchy / cvb_set_nvert
 *   UpdatePressure    (poisson.c:2908)  -> cvb_update_pressure
 *   Projection        (poisson.c:2281)  -> cvb_projection (flux correction), or
 *                                          cvb_projection_cart (with the trailing
 *                                          Contra2Cart and GhostNodeVelocity)
 *   Contra2Cart       (rhs.c:25)        -> cvb_contra2cart
 *   GhostNodeVelocity (bcs.c:3645)      -> cvb_ghost_node_velocity
 *   Divergence        (main.c:469)      -> cvb_divergence
 *   MetricsDivergence (metrics.c:1551)  -> cvb_metrics_divergence
 *   Convection        (rhs.c:1463)      -> cvb_convection
 *   Viscous           (rhs.c:1947)      -> cvb_viscous
 *   FormFunction1     (rhs.c:2567)      -> cvb_form_function1
 *   CalcRHS   (implicitsolver.c:6449)   -> cvb_calc_rhs
 *   InflowFlux (bcs.c:99)               -> cvb_inflow_flux
 *   FormBCS   (bcs.c:4436)              -> cvb_form_bcs
 *   ImpRK     (implicitsolver.c:7094)   -> cvb_imp_rk
 *   ibm_search_advanced (ibm.c:4197), its nvert classification
 *                                       -> cvb_ibm_search
 *
 * Conventions
 *  - Every entry point returns a cvb_status (0 = success, as PetscErrorCode).
 *    cvb_last_error() describes the last failure of a context.
 *  - Arrays are the reference's DMDA layouts, index [k][j][i] with i fastest and
 *    the boundary ring included (mx = IM+1 for IM grid nodes):
 *      * level metrics and nvert: the ghosted local arrays (lICsi, lAj, lNvert,
 *        ...) covering the box gxs..gxs+gxm-1 etc. given in cvb_level_desc;
 *      * vector fields (Ucont, B, P, Phi): the owned box [mz][my][mx], Ucont as
 *        Cmpnts (x,y,z interleaved).
 *  - Host pointers are caller-owned and only read/written during the call.
 *    Device buffers belong to the context and stay resident across calls.
 *  - A context is not reentrant; distinct contexts may be used from distinct
 *    threads (each runs on its own CUDA stream).
 */
#ifndef CVB_H
#define CVB_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct cvb_ctx cvb_ctx;

typedef enum {
  CVB_OK = 0,
  CVB_NOT_CONVERGED = 1, /* iteration budget exhausted above the tolerance */
  CVB_NAN_DETECTED = 2,  /* a NaN/Inf appeared in the residual */
  CVB_OOM = 3,           /* device allocation failed */
  CVB_BAD_INPUT = 4,     /* inconsistent sizes, missing arrays, bad options */
  CVB_TIMEOUT = 5,       /* a bounded device-side wait gave up */
  CVB_CUDA_ERROR = 6,    /* any other CUDA runtime error */
  CVB_NOT_SETUP = 7      /* cvb_setup_hierarchy has not run */
} cvb_status;

typedef enum { CVB_PRECISION_FP64 = 0, CVB_PRECISION_MIXED = 1 } cvb_precision;

typedef struct {
  int device;   /* CUDA device ordinal */
  void *stream; /* cudaStream_t to issue work on; NULL: the context creates one */
} cvb_options;

/* One multigrid level: a PETSc-free mirror of the UserCtx fields the path reads
 * (variables.h:155-304).  Level 0 is the coarsest, as mgctx[0] (init.c:839). */
typedef struct {
  int mx, my, mz;                   /* DMDALocalInfo mx, my, mz */
  int gxs, gys, gzs, gxm, gym, gzm; /* ghosted box covered by the arrays below */
  int bctype[6];                    /* UserCtx.bctype; 7 = periodic */
  int isc, jsc, ksc;                /* semi-coarsening flags of this level */
  const double *icsi, *ieta, *izet; /* lICsi, lIEta, lIZet (Cmpnts) */
  const double *jcsi, *jeta, *jzet; /* lJCsi, lJEta, lJZet */
  const double *kcsi, *keta, *kzet; /* lKCsi, lKEta, lKZet */
  const double *iaj, *jaj, *kaj;    /* lIAj, lJAj, lKAj */
  const double *aj;                 /* lAj */
  const double *csi, *eta, *zet;    /* lCsi, lEta, lZet: finest level only, else NULL */
} cvb_level_desc;

/* Solver controls.  The reference reads the equivalent -ps_ksp_* options from
 * control.dat (poisson.c:1829, 1975; control.dat rtol/atol/max_it). */
typedef struct {
  int precision;       /* cvb_precision: FP64 throughout, or FP32 V-cycles in FP64 FGMRES */
  double rtol;         /* stop when ||b - A phi|| <= rtol ||b|| ... */
  double atol;         /* ... or <= atol */
  int max_it;          /* total FGMRES iterations */
  int restart;         /* FGMRES restart length (<= 64) */
  int pre_sweeps;      /* smoothing sweeps before / after the coarse correction (zebra: one
                          sweep = both colors) */
  int post_sweeps;
  double omega;        /* relaxation factor (Jacobi: damping; zebra: over-relaxation) */
  int project_rhs;     /* remove b's component outside range(A) (fluid-weighted mean of b/aj) */
  int warm_start;      /* use phi's input values as the initial guess */
  int coarse_dense_max;/* largest coarsest-level box (ring included) solved exactly by a dense
                          inverse (default 6000); larger ones get 30 smoothing sweeps */
  int cgs_refine;      /* 1: second Gram-Schmidt pass when the first cancels most of w
                          (PETSc's KSPGMRESSetCGSRefinementType IFNEEDED); 0: never (its default) */
  int smoother;        /* cvb_smoother: the multigrid smoother */
} cvb_solve_opts;

typedef enum {
  CVB_SMOOTHER_JACOBI = 0, /* damped y-line Jacobi: every line from the same iterate */
  CVB_SMOOTHER_ZEBRA = 1   /* y-line Gauss-Seidel in two colors, (i + k) even then odd, in place */
} cvb_smoother;

typedef struct {
  int status;            /* cvb_status of the solve */
  int iterations;        /* FGMRES iterations (preconditioner applications) */
  int restarts;
  double rel_residual;   /* true ||b - A phi|| / ||b|| at exit (FP64) */
  double abs_residual;
  double rhs_norm;
  double rhs_projected;  /* size of the removed incompatible part of b, relative to ||b|| */
  double device_ms;      /* time on the device between the solve's first and last kernel */
} cvb_solve_stats;

int cvb_solve_opts_default(cvb_solve_opts *opts);
/* Update opts from options in the reference's control.dat syntax ("-name value"
 * per line, '#' starts a comment, later occurrences win), as PETSc's options
 * database reads them for PoissonSolver_MG (poisson.c:1829-1983;
 * control.dat~:65-74): -ps_ksp_rtol, -ps_ksp_atol, -ps_ksp_max_it,
 * -ps_ksp_gmres_restart, and this library's -cvb_precision {fp64|mixed},
 * -cvb_smoother {zebra|jacobi}, -cvb_pre_sweeps, -cvb_post_sweeps, -cvb_omega,
 * -cvb_coarse_dense_max.  Other options are ignored.  The _args form takes
 * argv-style tokens (command-line options override control.dat when applied
 * after it).  Returns CVB_BAD_INPUT, with the offending option in *bad (may be
 * NULL), for an unreadable file or a malformed value. */
int cvb_solve_opts_from_file(const char *path, cvb_solve_opts *opts, char *bad, int bad_len);
int cvb_solve_opts_from_args(int argc, const char *const *argv, cvb_solve_opts *opts, char *bad, int bad_len);

/* --- context ------------------------------------------------------------- */
int cvb_init(cvb_ctx **ctx, const cvb_options *opts);
void cvb_destroy(cvb_ctx *ctx);
const char *cvb_last_error(const cvb_ctx *ctx);

/* Upload the metrics of every level, restrict nvert down the hierarchy
 * (MyNvertRestriction + FullyBlocked), build each level's operator
 * (PoissonLHSNew), the smoother factors and the coarsest-level solver.
 * nvert_finest covers the finest level's ghosted box.  The reference rebuilds
 * all of this inside every PoissonSolver_MG call; here it stays resident. */
int cvb_setup_hierarchy(cvb_ctx *ctx, int nlevels, const cvb_level_desc *levels,
                        const double *nvert_finest);
/* Set up a hierarchy on the grid of a set-up donor context, with this
 * context's own nvert: the metrics stay resident once and are shared (they are
 * freed with the last context that uses them).  No counterpart in the
 * reference, which keeps one grid per run. */
int cvb_setup_like(cvb_ctx *ctx, const cvb_ctx *donor, const double *nvert_finest);
/* Upload a grid's metrics only: the context can then donate them to
 * cvb_setup_like but cannot solve itself. */
int cvb_setup_geometry(cvb_ctx *ctx, int nlevels, const cvb_level_desc *levels);
/* The immersed body moved: redo the nvert restriction and rebuild the operators. */
int cvb_set_nvert(cvb_ctx *ctx, const double *nvert_finest);
/* Restricted nvert of one level ([mz][my][mx]) and the FullyBlocked result. */
int cvb_get_nvert(cvb_ctx *ctx, int level, double *nvert, int *multinullspace);
int cvb_level_dims(const cvb_ctx *ctx, int level, int *mx, int *my, int *mz);

/* --- the path ------------------------------------------------------------ */
/* VolumeFlux_rev (poisson.c:3712): ucont corrected in place; flux/area are the
 * sums after the correction, as the reference leaves them in ibm_Flux/ibm_Area. */
int cvb_volume_flux_rev(cvb_ctx *ctx, double *ucont, double flux_intp_sum, int flg, double *flux,
                        double *area);
/* PoissonRHS (poisson.c:1509); compat_sum is the sum it prints ("Summation RHS"). */
int cvb_poisson_rhs(cvb_ctx *ctx, const double *ucont, double dt, double st, double *b,
                    double *compat_sum);
/* The multigrid-preconditioned FGMRES solve of A phi = b (KSPSolve, poisson.c:1983),
 * phi returned with the fluid mean removed and zero outside the fluid
 * (PoissonNullSpaceFunction, poisson.c:372). */
int cvb_poisson_solve(cvb_ctx *ctx, const double *b, double *phi, const cvb_solve_opts *opts,
                      cvb_solve_stats *stats);
/* Drop-in for PoissonSolver_MG (poisson.c:1775): VolumeFlux_rev(flg = immersed),
 * PoissonRHS(dt, st), then the solve.  ucont is corrected in place. */
int cvb_poisson_solver_mg(cvb_ctx *ctx, double *ucont, double flux_intp_sum, int immersed, double dt,
                          double st, double *phi, const cvb_solve_opts *opts, cvb_solve_stats *stats);
/* UpdatePressure (poisson.c:2908): p += phi, periodic ring copies of p and phi. */
int cvb_update_pressure(cvb_ctx *ctx, double *p, double *phi);
/* Projection's flux correction (poisson.c:2281-2900) with phi as UpdatePressure left it. */
int cvb_projection(cvb_ctx *ctx, const double *phi, double dt, double st, double *ucont);
/* Contra2Cart (rhs.c:25-143), which Projection calls next (poisson.c:2902): the
 * Cartesian velocity at the centre of every interior cell with nvert < 0.1 or
 * nvert > 7, from ucont and the finest level's centre metrics.  ucont and ucat
 * are [mz][my][mx][3]; ucat is read for the cells the routine leaves alone. */
int cvb_contra2cart(cvb_ctx *ctx, const double *ucont, double *ucat);
/* GhostNodeVelocity (bcs.c:3645-4435), Projection's last call (poisson.c:2904),
 * without the wall function: boundary velocities of slip (3), moving-lid
 * (bctype[5] 2), O-grid (bctype[3] 12), annulus (bctype[2] 11: from the cell
 * centres of cvb_set_cell_centres) and rheology-plate (13 on faces 2-5: the
 * velocity of cvb_set_plate_velocity) faces into ubcs (Bcs.Ubcs), the ring of
 * ucat from ubcs and the periodic images, the box's edges.  ubcs and ucat
 * ([mz][my][mx][3]) are read and written.  CVB_BAD_INPUT, with nothing
 * written, for an annulus face before the centres were given, or a periodic
 * face whose opposite is not. */
int cvb_ghost_node_velocity(cvb_ctx *ctx, double *ubcs, double *ucat);
/* The finest level's cell centres (FormMetrics' Cent, [mz][my][mx][3]) for an
 * annulus face's boundary velocity (bcs.c:3811-3826); they stay on the device
 * and are also the centres cvb_ibm_search reuses when given none. */
int cvb_set_cell_centres(cvb_ctx *ctx, const double *cent);
/* The rheology plates' velocity, bcs.c's global U_bc (-U_bc option), for
 * faces of bctype 13 (bcs.c:3963-4010); 0 until set, as the global starts. */
int cvb_set_plate_velocity(cvb_ctx *ctx, double u_bc);
/* Projection as Flow_Solver calls it (solvers.c:1068, poisson.c:2281-2904):
 * the flux correction, Contra2Cart and GhostNodeVelocity on the device in one
 * call, each array copied in and out once. */
int cvb_projection_cart(cvb_ctx *ctx, const double *phi, double dt, double st, double *ucont, double *ubcs,
                        double *ucat);
/* Divergence (main.c:469-593), the check Flow_Solver runs after Projection
 * (solvers.c:1084): the largest |(the cell's three flux differences) * aj|
 * over the interior cells, 0 where nvert of the cell and its face neighbours
 * sums above 0.1, and its index in the [mz][my][mx] box (the first one, as
 * VecMax).  ucont NULL uses the context's device copy of Ucont as the last
 * projection or VolumeFlux_rev left it. */
int cvb_divergence(cvb_ctx *ctx, const double *ucont, double *maxdiv, long long *at);
/* MetricsDivergence (metrics.c:1551-1625), the check of the finest level's
 * metrics MG_Initial runs once they are formed (init.c:1054): the largest
 * |(the nine differences of the centre metrics csi, eta, zet across the cell)
 * * aj| over the interior cells, 0 on the ring, and its first index in the
 * [mz][my][mx] box, as VecMax returns them.  Reads the metrics the context
 * holds on the device. */
int cvb_metrics_divergence(cvb_ctx *ctx, double *maxdiv, long long *at);
/* Convection (rhs.c:1463-1946), the convective term FormFunction1 starts the
 * momentum right-hand side with (rhs.c:2651): at every interior cell the sum
 * over its six faces of the face flux of ucat carried by Ucont/2, QUICK
 * upwinded (central != 0: central, the -central option), with the one-sided
 * forms of the reference next to the ring and next to cells of nvert above
 * 0.1; 0 on the ring.  ucont, ucat and conv are [mz][my][mx][3].  ucont NULL
 * uses the device copy of Ucont the last projection left, ucat NULL the device
 * Ucat of the last cvb_projection_cart.  The nvert it tests is the context's
 * finest-level nvert, as the last cvb_setup_hierarchy or cvb_set_nvert gave it
 * (the reference reads lNvert on every call: after a body moves, call
 * cvb_set_nvert first).  Along a periodic direction (bctype 7) the faces at
 * the seam read the periodic images the reference's ghost cells hold (cell
 * m - 3 for index -1, cell 2 for index m) and take the full QUICK form where
 * both sides are fluid, as the reference does (rhs.c:1546-1620). */
int cvb_convection(cvb_ctx *ctx, const double *ucont, const double *ucat, int central, double *conv);
/* The momentum right-hand side on the finest level: Viscous for any box,
 * FormFunction1 and CalcRHS for boxes with no periodic face (bctype 7 is
 * refused there with CVB_BAD_INPUT).  Vector fields are
 * [mz][my][mx][3], p is [mz][my][mx]; nvert is the context's (the last
 * cvb_setup_hierarchy or cvb_set_nvert); ucont / ucat NULL use the device copies
 * the last projection left.  Results equal the reference's bit for bit.
 *
 * Viscous (rhs.c:1947-2566), laminar (no LES / RANS model): at every interior
 * cell the sum over its faces of the viscous flux nu (G grad ucat), nu =
 * 1 / ren, with the reference's one-sided derivatives next to cells of nvert
 * in (0.5, 7); 0 on the ring.  It reads the box alone, so on a periodic box
 * ucat's ring must hold the periodic images (as GhostNodeVelocity leaves it). */
int cvb_viscous(cvb_ctx *ctx, const double *ucat, double ren, double *visc);
/* FormFunction1 (rhs.c:2567-3351): Contra2Cart (ucat's interior cells from
 * ucont; ucat is written back), Convection (QUICK, or central with central !=
 * 0), Viscous, their contravariant difference at the cell centres, and on
 * every face its average minus the pressure gradient (G grad p) with the
 * reference's one-sided differences, zero on faces next to blocked cells.
 * rhs's interior cells are written, its ring is left as passed.  Where the
 * reference assigns no tangential pressure derivative (a fluid cell between
 * two blocked cells, or under a wall with a blocked cell on the other side),
 * the value of the previous assignment in its loop order stands, as there. */
int cvb_form_function1(cvb_ctx *ctx, const double *ucont, double *ucat, const double *p, double ren, int central,
                       double *rhs);
/* CalcRHS (implicitsolver.c:6449-6713): FormFunction1, then rhs -= dU / dt with
 * dU = 1.5 ucont - 2 ucont_o + 0.5 ucont_rm1 (second-order backward,
 * COEF_TIME_ACCURACY 1.5) unless ti == tistart or ti == 1 (then ucont -
 * ucont_o), the faces next to blocked cells and walls zeroed, and the boundary
 * ring zeroed as the reference's six boundary loops leave it (bctype[5] 8 adds
 * the convective-outflow term on the last k face before those loops). */
int cvb_calc_rhs(cvb_ctx *ctx, const double *ucont, const double *ucont_o, const double *ucont_rm1, double *ucat,
                 const double *p, double ren, double dt, int ti, int tistart, int central, double *rhs);
/* The momentum equation's boundary conditions and pseudo-time iteration, one
 * block, for boxes with solid walls (bctype 1) on the x and y faces and, on
 * the k faces, walls or an inlet on k = 0 (bctype[4] 5) with an outlet on the
 * last (bctype[5] 4); other boxes are refused with CVB_BAD_INPUT.  Vector
 * fields are [mz][my][mx][3], p [mz][my][mx]; results equal the reference's
 * bit for bit.
 *
 * InflowFlux (bcs.c:99-400) on an inlet face with a constant profile
 * (inletprofile 1: speed 2; -1: speed -1; 11: 0.185; 3, 6, 8: see
 * cvb_set_inlet_flux) or a shaped one (2, 4, 7, 10, after
 * cvb_set_inlet_nodes; with cvb_set_inlet_table also the table's 0 and 5;
 * other profiles are refused): on the face's
 * interior cells above fluid cells ubcs = uin zet / |zet| and Ucont.z = uin
 * |zet|; *flux_in_sum (FluxInSum) = their sum in the reference's loop order.
 * On a walled k = 0 face nothing is written. */
int cvb_inflow_flux(cvb_ctx *ctx, double *ucont, double *ubcs, int inletprofile, double *flux_in_sum);
/* The inlet's nodes for the shaped profiles (bcs.c:152-195), which take the
 * speed from each face cell's centre (the mean of its four nodes) less
 * (cmx, cmy, cmz), the reference's CMx_c, CMy_c, CMz_c: profile 2 = 4 (1.5)
 * y (4.1 - y) / 4.1^2, 4 = 2 (1 - 4 r^2) within r = sqrt(y^2 + z^2) <= 0.5
 * and 0 outside, 7 = 1.5 (1 - 4 y^2), 10 = a square duct's fully developed
 * flow (x in [0, 1], y in [1, 2]; 20 terms of its series, formed on the host
 * with libm, once per call of this function).  coor0 holds the k = 0 node plane in
 * the box layout, [my][mx][3] (node (i, j) at [j][i], as the reference's
 * local coor array). */
int cvb_set_inlet_nodes(cvb_ctx *ctx, const double *coor0, double cmx, double cmy, double cmz);
/* The reference's Flux_in and ti globals for the uniform profiles that
 * InletInterpolation gives (bcs.c:67-82): 3 and 6 take uin = Flux_in, 8
 * uin = sin(2 (3.14159) ti / 200) and leaves it in Flux_in.  Flux_in starts
 * at the reference's 4.104388e-04 and ti at 0; cvb_imp_rk takes ti from its
 * options.  cvb_inlet_flux_in returns Flux_in as the last InflowFlux left it. */
int cvb_set_inlet_flux(cvb_ctx *ctx, double flux_in, int ti);
double cvb_inlet_flux_in(const cvb_ctx *ctx);
/* The table of the profiles 0 and 5 (bcs.c:40-96), InletRead's uinr
 * [101][1001]: uinr[i][t] the speed at radius 0.005 i in column t.  The speed
 * of a face cell is (for 5 minus) the table interpolated linearly at its
 * radius sqrt(y^2 + z^2) about (CMy_c, CMz_c) (cvb_set_inlet_nodes), in
 * column ti/2 - (ti/2000) 2000 (cvb_set_inlet_flux's or cvb_imp_rk's ti);
 * beyond radius 1 row 99's, between 0.5 and 1 zero.  Steps whose column
 * falls outside the table (ti >= 2000) are refused with CVB_BAD_INPUT. */
int cvb_set_inlet_table(cvb_ctx *ctx, const double *uinr);
/* FormBCS (bcs.c:4436-5889): three passes of the outlet's flux correction
 * (ratio = (flux_in_sum + flux_intp_sum - the outlet's flux) / its area; ubcs
 * on the last face = the ucat next to it; Ucont.z of the last interior face =
 * ubcs . zet + ratio |zet|), Contra2Cart of ucont into ucat's interior cells,
 * the ghost faces u = 2 ubcs - inner on the faces' interior cells, and the
 * means of ucat and p on the box's 12 edges.  ucont, ubcs, ucat and p are read
 * and written; flux_in_sum and flux_intp_sum (the block's FluxIntpSum) matter
 * only with an outlet. */
int cvb_form_bcs(cvb_ctx *ctx, double *ucont, double *ubcs, double *ucat, double *p, double flux_in_sum,
                 double flux_intp_sum);
/* ImpRK's controls: the block's ren, dt, st and cfl, the time step ti and
 * tistart (CalcRHS's BDF2 switch), -central, imp_atol / imp_rtol / imp_MAX_IT,
 * InflowFlux's inletprofile and the block's FluxIntpSum (the immersed-boundary
 * flux the outlet adds to the inlet's). */
typedef struct {
  double ren, dt, st, cfl;
  int ti, tistart, central;
  double imp_atol, imp_rtol;
  int imp_max_it;
  int inletprofile;
  double flux_intp_sum;
} cvb_imp_rk_opts;
/* The reference's defaults: cfl 0.2 (init.c:54), imp_atol 1e-7, imp_rtol
 * 1e-4, imp_MAX_IT 50 (main.c:21-26), inletprofile 1; ren, dt, st 1; ti 1,
 * tistart 0; FluxIntpSum 0. */
void cvb_imp_rk_opts_default(cvb_imp_rk_opts *opts);
/* What cvb_imp_rk did: the pseudo-time iterations kept (pseudot at the end),
 * those undone with the step halved, and the last iteration's norms. */
typedef struct {
  int pseudo_iterations;
  int rejected;
  double norm_du;   /* max |Ucont change| of the last iteration */
  double rel_du;    /* norm_du / its first value */
  double norm_f;    /* max |Rhs| after the last iteration */
  double rel_f;     /* norm_f / its first value */
  double lambda;    /* the pseudo-time step factor at the end (cfl, halved per undone iteration) */
  double flux_in_sum; /* FluxInSum of the last InflowFlux (0 with a walled k = 0 face) */
} cvb_imp_rk_stats;
/* ImpRK (implicitsolver.c:7094-7257), the momentum equation's pseudo-time
 * iteration, as the reference runs it with immersed 0 (no immersed-boundary
 * interpolation between iterations; nvert's blocked cells still mask the
 * fluxes): InflowFlux, OutflowFlux (it only sums a flux nothing here reads),
 * FormBCS and CalcRHS as above; per pseudo-time iteration four Runge-Kutta
 * stages Ucont = (lambda alfa_s dt st) Rhs + Ucont_prev with alfa 1/4, 1/3,
 * 1/2, 1 and lambda starting at cfl; an iteration whose |Rhs| and |dU| both
 * grew is undone with lambda halved (while lambda > 0.001); the loop ends when
 * |dU| <= imp_atol or |dU| / |dU|_first <= imp_rtol, or after imp_max_it
 * iterations.  ucont (Ucont), ucat (Ucat), p (P) and ubcs (Bcs.Ubcs) are read
 * and written, ucont_o / ucont_rm1 are the two previous steps' fluxes.  stats
 * may be NULL.  The iteration runs on the device; the host reads two norms per
 * iteration. */
int cvb_imp_rk(cvb_ctx *ctx, double *ucont, const double *ucont_o, const double *ucont_rm1, double *ucat, double *p,
               double *ubcs, const cvb_imp_rk_opts *opts, cvb_imp_rk_stats *stats);
/* The nvert classification of ibm_search_advanced (ibm.c:4197-4740), which the
 * reference reruns for moving bodies every step (solvers.c:201-571), for body
 * ibi of nbodies: a closed triangle mesh of n_v nodes (xyz, x y z per node) and
 * n_elmt triangles (tri, three node indices each; nf, their unit normals).
 * Every interior cell centre (cent, the finest level's lCent, [mz][my][mx][3])
 * gets the reference's ray-cast inside test; then the layer of cells next to
 * inside ones, the fix for cells that were solid in the previous step's
 * nvert_o ([mz][my][mx]), the codes 3 + ibi/1000 (inside) and 1 + ibi/1000
 * (layer), and the reference's two clean-up passes along k.  nvert
 * ([mz][my][mx]) is read and written, bit for bit as the reference leaves
 * it.  Bodies go one after another, ibi = 0 first (ibi 0 clears nvert below 5).
 * The reference retries singular rays (through an edge or a vertex) without
 * end; this tries 64 directions and then returns CVB_NOT_CONVERGED with nvert
 * untouched.  Feed the result to cvb_set_nvert.  cent may be NULL to reuse
 * the centres an earlier call uploaded (they stay on the device). */
int cvb_ibm_search(cvb_ctx *ctx, const double *cent, int n_v, const double *xyz, int n_elmt, const int *tri,
                   const double *nf, int ibi, int nbodies, const double *nvert_o, double *nvert);
/* --- files on either side of the path (host only, no context) ------------ */
/* PETSc binary vectors as VecView writes and VecLoad reads them: the int32
 * class id 1211214, the int32 length n, then n IEEE doubles, all big-endian;
 * with block_size > 1 also "<path>.info" holding "-vecload_block_size <bs>".
 * A one-rank DMDA vector is written in its [k][j][i] order. */
int cvb_petsc_vec_write(const char *path, const double *v, long long n, int block_size);
int cvb_petsc_vec_size(const char *path, long long *n);
/* CVB_BAD_INPUT unless the file holds a vector of exactly n values. */
int cvb_petsc_vec_read(const char *path, double *v, long long n);
/* The restart set of Ucont_P_Binary_Output / _Input (main.c:75-467) for step ti
 * and block: nvfield (Nvert), vfield (Ucont), ufield (Ucat), pfield (P), each
 * "<dir>/<name>%05d_%1d.dat" over a box of ncells cells.  NULL arrays are
 * skipped.  The read side fills Ucont, P and Nvert_o, as _Input does. */
int cvb_restart_write(const char *dir, int ti, int block, long long ncells, const double *nvert, const double *ucont,
                      const double *ucat, const double *p);
int cvb_restart_read(const char *dir, int ti, int block, long long ncells, double *ucont, double *p,
                     double *nvert_o);
/* bcs.dat as MG_Initial reads it (init.c:474-490): for each of nblocks
 * blocks one line of six boundary types ("%i": decimal, 0x hexadecimal or 0
 * octal), into bctype[6 b .. 6 b + 5]; periodic (may be NULL) gets the i, j, k
 * periodic flags the reference sets (1 where a block has type 7 on either
 * face of that direction).  A file with fewer than 6 nblocks numbers is
 * CVB_BAD_INPUT (the reference leaves those types unread). */
int cvb_bcs_dat_read(const char *path, int nblocks, int *bctype, int *periodic);
/* grid.dat as MG_Initial reads it (init.c:339-349, 606-735): the block count,
 * then per block "IM JM KM" and its nodes: all x, then all y, then all z in
 * [k][j][i] order, or with grid1d IM + JM + KM lines of "x y z" (one component
 * used per line).  Fills IM, JM, KM of the given block and, when coords is not
 * NULL, its node coordinates [KM][JM][IM][3] scaled as the reference does,
 * c / cl * l_dim; capacity is coords' length in doubles. */
int cvb_grid_dat_read(const char *path, int block, int grid1d, double cl, double l_dim, int *IM, int *JM, int *KM,
                      double *coords, long long capacity);

/* randomdirection's ray offsets for seeds 1 .. n (srand(seed); rand() scaled to
 * [-0.5, 0.5), ibm.c:101-104), from a private generator state: the caller's
 * rand() sequence is not disturbed.  Needs no context or GPU. */
int cvb_ibm_ray_offsets(int n, double *s);

/* --- device-resident form (inputs already in HBM) ---------------------- */
/* Device pointers of the context's finest-level rhs and solution ([mz][my][mx] FP64). */
double *cvb_device_rhs(cvb_ctx *ctx);
double *cvb_device_phi(cvb_ctx *ctx);
/* Copy a host rhs into the resident rhs, a host phi into the resident phi (a
 * warm start), the resident phi out to the host ([mz][my][mx] FP64, synchronous). */
int cvb_set_rhs(cvb_ctx *ctx, const double *b);
int cvb_set_phi(cvb_ctx *ctx, const double *phi);
int cvb_get_phi(cvb_ctx *ctx, double *phi);
/* Solve the context's resident rhs into its resident phi. */
int cvb_solve_resident(cvb_ctx *ctx, const cvb_solve_opts *opts, cvb_solve_stats *stats);
/* The context's CUDA stream (cudaStream_t). */
void *cvb_stream(cvb_ctx *ctx);

/* --- parity hooks ------------------------------------------------------- */
/* y = A_level x in FP64 (the assembled PoissonLHSNew rows), host arrays [mz][my][mx]. */
int cvb_apply_operator(cvb_ctx *ctx, int level, const double *x, double *y);
/* The same operator in FP32 flux form (the mixed V-cycle's operator). */
int cvb_apply_operator_f32(cvb_ctx *ctx, int level, const float *x, float *y);
/* The 19 stored weights of every row, [19][mz][my][mx], slots in the reference's
 * CP,EP,WP,NP,SP,TP,BP,NE,SE,NW,SW,TN,BN,TS,BS,TE,BE,TW,BW order. */
int cvb_get_weights(cvb_ctx *ctx, int level, double *w);
/* Whether the level's operator has cross-derivative terms: *cross32 for the FP32
 * flux form, *cross64 for the FP64 rows (any of the 12 edge weights non-zero).
 * On an orthogonal grid both are 0 and the operator kernels read the seven face
 * points only.  No counterpart in the reference (which always assembles 19). */
int cvb_level_cross(const cvb_ctx *ctx, int level, int *cross32, int *cross64);
/* One FP32 zebra half-sweep (the mixed V-cycle's smoother, y-line
 * Gauss-Seidel on the lines (i + k) % 2 == color, over-relaxed by omega) of
 * x in place for right-hand side b, host arrays [mz][my][mx], in a given
 * form: two kernels (residual, then line solves), one kernel, or one kernel
 * with its tiles staged by TMA bulk tensor copies in chunks of 4, 8 or 16 row
 * pairs.  The forms compute the same update; the set-up autotuner picks the
 * fastest per level (cvb_tuning_report).  CVB_BAD_INPUT when the form cannot
 * run on the level.  A parity and measurement hook with no counterpart in the
 * reference (its smoother is Richardson + ILU, poisson.c:1906-1935). */
enum {
  CVB_ZEBRA_SPLIT = 0,
  CVB_ZEBRA_FUSED = 1,
  CVB_ZEBRA_SPLIT4 = 2, /* the two forms above with 4 lines per line-solve tile instead of 8 */
  CVB_ZEBRA_FUSED4 = 3,
  CVB_ZEBRA_TMA4 = 4,
  CVB_ZEBRA_TMA8 = 8,
  CVB_ZEBRA_TMA16 = 16
};
int cvb_zebra_half_f32(cvb_ctx *ctx, int level, int form, int color, float omega, const float *b, float *x);
/* MyRestriction (poisson.c:129) from level+1 to level; MyInterpolation
 * (poisson.c:265) from level-1 to level (returned, not added). */
int cvb_restrict(cvb_ctx *ctx, int coarse_level, const double *xf, double *xc);
int cvb_interpolate(cvb_ctx *ctx, int fine_level, const double *xc, double *xf);
/* PoissonNullSpaceFunction (poisson.c:372) on one level, in place. */
int cvb_nullspace(cvb_ctx *ctx, int level, double *x);

/* --- allocation-free form ------------------------------------------------ */
/* PoissonRHS on device arrays without allocating any device memory.  This entry
 * point has no counterpart in the reference.  It is for callers that cannot call
 * cudaMalloc: hosts whose device memory is handed out by their own allocator or
 * pool (a PETSc or framework pool that must not be bypassed or fragmented), and
 * time-stepping loops that forbid allocation after start-up so that a long run
 * cannot fail half-way on memory.
 *
 * d_ucont ([mz][my][mx] Cmpnts), d_aj, d_nvert ([mz][my][mx]) and the outputs
 * d_b ([mz][my][mx]) and d_compat_sum (one double, the sum PoissonRHS prints)
 * are device pointers owned by the caller; stream is a cudaStream_t of the
 * current device (NULL: the legacy default stream).  Results equal
 * cvb_poisson_rhs's bit for bit.
 *
 * The only scratch is a fixed file-scope device array of 2*CVB_NOALLOC_MAX_BLOCKS
 * doubles (32 KB) that every GPU loading this library holds until the process
 * exits.  Boxes larger than CVB_NOALLOC_MAX_CELLS cells are rejected with
 * CVB_BAD_INPUT.  The first call on each device (and the first after that
 * device's context was replaced, e.g. by cudaDeviceReset) looks up the array's
 * device address (cudaGetSymbolAddress) with that device current; make that
 * first call before any stream capture.  Every call shares the array and leaves
 * its last contents there; each call overwrites every slot it reads, so nothing
 * needs clearing, but calls that overlap on the GPU (concurrent streams or host
 * threads) race on it and must be serialised by the caller. */
#define CVB_NOALLOC_MAX_BLOCKS 2048
#define CVB_NOALLOC_MAX_CELLS (64 * 1024 * 1024)
int cvb_poisson_rhs_noalloc(const double *d_ucont, const double *d_aj, const double *d_nvert, int mx, int my,
                            int mz, double dt, double st, double *d_b, double *d_compat_sum, void *stream);

/* --- batched and served solves ------------------------------------------ */
/* A batch runs many independent solves at once, each on its own set-up
 * context (its hierarchy stays resident there).  The reference has no
 * counterpart: it solves one block per PoissonSolver_MG call.
 *
 * Work proceeds in rounds on the batch's stream.  One round is one FGMRES
 * iteration of every active solve, and every phase of it (each V-cycle kernel,
 * each Krylov step) is one grouped kernel launch over a work-list of all the
 * solves' tiles.  The Krylov scalars (Gram-Schmidt column, Givens rotations,
 * convergence test) stay on the device; the host reads each solve's state one
 * round late, so it never stalls the GPU.  Solves may be submitted at any time
 * and join at the next round (continuous batching); finished ones are handed
 * back by cvb_batch_poll.  A solve's result does not depend on what else is
 * in the batch: every reduction has a fixed tree per problem size.
 *
 * Batch-wide settings (precision, restart, sweeps, omega) come from the
 * options given at creation; tolerances are per solve.  Limits: the context's
 * coarsest level must be solved densely (coarse_dense_max), y-lines of at most
 * 400 rows, at most 1024 solves in flight. */
typedef struct cvb_batch cvb_batch;
int cvb_batch_create(cvb_batch **batch, const cvb_options *opts, const cvb_solve_opts *solve_opts);
void cvb_batch_destroy(cvb_batch *batch);
const char *cvb_batch_last_error(const cvb_batch *batch);
/* Queue a solve of ctx's resident rhs (cvb_device_rhs) into its resident phi.
 * host_b (optional, [mz][my][mx]) is copied into the resident rhs first; if it
 * is pinned memory it must stay valid until the solve is polled.  The context
 * must not be used otherwise until its ticket is polled. */
int cvb_batch_submit(cvb_batch *batch, cvb_ctx *ctx, const double *host_b, double rtol, double atol, int max_it,
                     int warm_start, int project_rhs, int *ticket);
/* Admit queued solves and issue one round; *in_flight = solves not yet polled. */
int cvb_batch_step(cvb_batch *batch, int *in_flight);
/* A finished solve: *ticket (-1 if none is ready) and its statistics. */
int cvb_batch_poll(cvb_batch *batch, int *ticket, cvb_solve_stats *stats);
/* Copy a finished solve's phi to the host (on the batch's copy stream). */
int cvb_batch_read_phi(cvb_batch *batch, cvb_ctx *ctx, double *host_phi);
/* Submit n solves with the batch's options and run them to completion. */
int cvb_batch_solve(cvb_batch *batch, int n, cvb_ctx *const *ctxs, cvb_solve_stats *stats);
int cvb_batch_in_flight(const cvb_batch *batch);
/* Bound cvb_batch_solve's loop to `rounds` rounds (0: the default, 10^6).  When
 * the bound is reached with solves unfinished it returns CVB_TIMEOUT and the
 * batch stays usable: the unfinished solves are still in flight, and
 * cvb_batch_step / cvb_batch_poll carry them on to their results.  No
 * counterpart in the reference, whose KSPSolve has only max_it. */
int cvb_batch_set_round_limit(cvb_batch *batch, long long rounds);
/* Mixed-precision rounds replay their V-cycles from a CUDA graph while the set
 * of iterating problems stays the same (on by default; 0 turns it off, the
 * launches then run one by one with the same result).  No counterpart in the
 * reference, whose solves run one at a time (poisson.c:1775). */
int cvb_batch_set_graphs(cvb_batch *batch, int on);
/* Graphs instantiated, graphs updated in place, and graph launches so far. */
int cvb_batch_graph_stats(const cvb_batch *batch, long long *captures, long long *updates, long long *replays);
/* Device memory held by a context alone (operators, vectors, Krylov basis) and
 * by its grid's shared metrics, with an id that is equal for contexts sharing them. */
int cvb_device_bytes(const cvb_ctx *ctx, unsigned long long *bytes);
/* Cap the device memory this context may allocate (its own arrays, and the
 * grid's when it uploads one); 0 removes the cap.  An allocation beyond it
 * fails with CVB_OOM as a failed cudaMalloc would, and the context stays
 * usable: raise the cap and set up again.  For callers sharing a GPU, and for
 * exercising the out-of-memory paths.  No counterpart in the reference. */
int cvb_set_device_limit(cvb_ctx *ctx, unsigned long long bytes);
int cvb_geometry_bytes(const cvb_ctx *ctx, unsigned long long *bytes, unsigned long long *id);

/* --- measurement ------------------------------------------------------- */
/* Kernel launches this library has issued in the process (all contexts). */
long long cvb_kernel_launches(void);
enum {
  CVB_KERNEL_LINE_SWEEP_F32 = 0, /* fused residual + y-line Thomas sweep, FP32 (mixed V-cycle) */
  CVB_KERNEL_LINE_SWEEP_F64 = 1, /* the same in FP64 (plain FP64 V-cycle) */
  CVB_KERNEL_RESIDUAL_F32 = 2,   /* b - A x, FP32 flux form */
  CVB_KERNEL_RESIDUAL_F64 = 3,   /* b - A x, FP64 stored rows */
  CVB_KERNEL_ZEBRA_F32 = 4,      /* one zebra half-sweep (residual on one color + its line solves), FP32 */
  CVB_KERNEL_ZEBRA_F64 = 5,      /* the same in FP64 */
  CVB_KERNEL_VCYCLE_F32 = 6,     /* one FP32 V-cycle (default options) from the level down, replayed from a CUDA graph */
  CVB_KERNEL_VCYCLE_F64 = 7,     /* the same in FP64 */
  CVB_KERNEL_CONTRA2CART = 8,    /* Contra2Cart on the finest level (the level argument must name it) */
  CVB_KERNEL_GHOST_NODES = 9,    /* GhostNodeVelocity on the finest level */
  CVB_KERNEL_CONVECTION = 10,    /* Convection (QUICK) on the finest level: face fluxes, then their differences */
  CVB_KERNEL_VISCOUS = 11,       /* Viscous (laminar) on the finest level: face fluxes, then their differences */
  CVB_KERNEL_MOMENTUM_RHS = 12   /* CalcRHS on the finest level on device arrays: Contra2Cart, Convection,
                                    Viscous, FormFunction1's face values, the time term and masks */
};
/* JSON record of the set-up autotuner: per level, the measured time of the
 * fused and the split y-line sweep in each precision and the variant kept. */
int cvb_tuning_report(cvb_ctx *ctx, char *buf, int len);
/* Wall-clock milliseconds of the last set-up (cvb_setup_hierarchy,
 * cvb_setup_like or cvb_set_nvert) by phase: [0] the grid's metrics uploaded
 * (0 when shared or kept), [1] the level arrays allocated and nvert copied (0 for
 * cvb_set_nvert), [2] nvert restriction and the operators of every level
 * (MyNvertRestriction, FullyBlocked, PoissonLHSNew's weights, the FP32 copies,
 * the line factors), [3] the autotuner (0 when every level shape was timed
 * before in the process), [4] the coarsest solver (dense inverse).  The
 * reference rebuilds its operators and factors in every PoissonSolver_MG call
 * (poisson.c:1775). */
int cvb_setup_times(const cvb_ctx *ctx, double *ms5);
/* Average duration of `reps` back-to-back launches of one kernel on `level`
 * (CUDA events on the context's stream) and its algorithmic bytes per launch
 * (every array it needs, touched once). */
int cvb_time_kernel(cvb_ctx *ctx, int kernel, int level, int reps, double *avg_ms, double *bytes);

#ifdef __cplusplus
}
#endif
#endif /* CVB_H */
