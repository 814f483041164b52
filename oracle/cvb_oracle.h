/*
 * TEST INFRASTRUCTURE ONLY: the CPU oracle for the pressure-projection path.
 *
 * A plain-C restatement of the reference's arithmetic (CURVIB poisson.c), used
 * by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg as the
 * checker.  The product library never links or calls it.
 *
 * Arrays are the reference's DMDA global layout for one level: [mz][my][mx],
 * i fastest, boundary ring included; 3-vectors (Cmpnts) are interleaved x,y,z.
 * Periodic ring values are the ones Update_Metrics_PBC / UpdatePressure leave.
 */
#ifndef CVB_ORACLE_H
#define CVB_ORACLE_H
#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
  int mx, my, mz;
  int bctype[6];
  int isc, jsc, ksc;
  const double *icsi, *ieta, *izet;   /* I-face metrics (ICsi, IEta, IZet) */
  const double *jcsi, *jeta, *jzet;   /* J-face metrics */
  const double *kcsi, *keta, *kzet;   /* K-face metrics */
  const double *iaj, *jaj, *kaj, *aj; /* face and cell Jacobians */
  const double *csi, *eta, *zet;      /* cell metrics (VolumeFlux_rev) */
  const double *nvert;
} orc_level;

/* PoissonLHSNew (poisson.c:600-1507) assembled as CSR, columns in the
 * reference's CP,EP,WP,NP,SP,TP,BP,NE,SE,NW,SW,TN,BN,TS,BS,TE,BE,TW,BW order.
 * Returns nnz, or -1 if cap is too small. */
int orc_lhs_csr(const orc_level *L, int *rowptr, int *cols, double *vals, int cap);
/* y = A x with the CSR from orc_lhs_csr. */
void orc_csr_mult(int n, const int *rowptr, const int *cols, const double *vals,
                  const double *x, double *y);
/* PoissonRHS (poisson.c:1509-1576); returns the printed compatibility sum. */
double orc_poisson_rhs(const orc_level *L, const double *ucont, double dt, double st, double *b);
/* VolumeFlux_rev (poisson.c:3712-3944); ucont updated in place. */
void orc_volume_flux_rev(const orc_level *L, double *ucont, double flux_intp_sum, int flg,
                         double *flux_out, double *area_out);
/* MyNvertRestriction (poisson.c:1662-1773): coarse nvert from fine nvert. */
void orc_nvert_restrict(const orc_level *fine, int coarse_mx, int coarse_my, int coarse_mz,
                        int coarse_is_level0, int isc, int jsc, int ksc, double *nvert_c);
/* FullyBlocked (poisson.c:1578-1660): returns multinullspace; fills KSKE[2*mx*my]. */
int orc_fully_blocked(const orc_level *L, int *kske);
/* MyRestriction (poisson.c:129-226). */
void orc_restrict(const orc_level *fine, const orc_level *coarse, const double *xf, double *fc);
/* MyInterpolation (poisson.c:265-370). */
void orc_interpolate(const orc_level *coarse, const orc_level *fine, const double *xc, double *ff);
/* PoissonNullSpaceFunction (poisson.c:372-563) in place. */
void orc_nullspace(const orc_level *L, int multinullspace, const int *kske, double *x);
/* UpdatePressure (poisson.c:2908-3248): p += phi and the periodic ring copies
 * of p and phi. */
void orc_update_pressure(const orc_level *L, double *p, double *phi);
/* Projection (poisson.c:2281-2900), flux correction part; reads phi with its
 * periodic ring already filled (as after UpdatePressure). */
void orc_projection(const orc_level *L, const double *phi, double dt, double st, double *ucont);
/* Contra2Cart (rhs.c:25-143): Cartesian velocity at the centre of every
 * interior cell with nvert < 0.1 or nvert > 7, from the averaged contravariant
 * fluxes and centre metrics by Cramer's rule; other cells keep their ucat. */
void orc_contra2cart(const orc_level *L, const double *ucont, double *ucat);
/* GhostNodeVelocity (bcs.c:3645-4435) without the wall function: the boundary
 * velocity of moving-lid (bctype[5] 2), O-grid (bctype[3] 12) and slip (3)
 * faces into ubcs; every non-periodic ghost face from 2 ubcs - inner; the
 * periodic ring copies; the averages on the box's 12 edges; the second round
 * of ring copies.  Returns 0, or -1 (nothing written) for what it does not
 * restate: bctype 11 without the cell centres, or a periodic face whose
 * opposite is not; rheology faces (13) take a plate velocity of 0. */
int orc_ghost_node_velocity(const orc_level *L, double *ubcs, double *ucat);
/* The same with the annulus face (bctype[2] 11: ubcs from the cell centres
 * cent, [mz][my][mx][3], of the first interior row) and the rheology plates
 * (bctype 13 on faces 2-5: the plate velocity u_bc, bcs.c's U_bc). */
int orc_ghost_node_velocity_ext(const orc_level *L, double *ubcs, double *ucat, const double *cent, double u_bc);
/* The nvert classification of ibm_search_advanced (ibm.c:4197-4740) for body
 * ibi of nbodies, a closed triangle mesh (xyz: n_v nodes; tri: n_elmt node
 * triples; nf: their unit normals): each interior cell centre (cent,
 * [mz][my][mx][3]) inside the body's bounding box gets the ray-cast inside test
 * of point_cell_advanced (ibm.c:1285), rays aimed by randomdirection (ibm.c:87)
 * through a 40^3 bucket grid; then the 27-cell layer around inside cells, the
 * phase-change fix against nvert_o, the codes 1 / 3 + ibi/1000, and the two
 * clean-up passes along k.  nvert ([mz][my][mx]) is read and written.  The
 * reference retries a ray until it meets no singular pair of intersections;
 * this gives up after max_tries directions and returns -1 (0 on success). */
/* Divergence (main.c:469-593): |(the flux differences of the cell) * aj| on
 * interior cells, 0 where the cell or a face neighbour has nvert summing above
 * 0.1, 0 on the ring; returns the maximum and its first index in the box (as
 * VecMax). */
void orc_divergence(const orc_level *L, const double *ucont, double *maxdiv, long long *at);
/* MetricsDivergence (metrics.c:1551-1625): |(csi.x - csi_w.x + eta.x - eta_s.x
 * + zet.x - zet_b.x + the same for y and z) * aj| on interior cells, summed
 * left to right, 0 on the ring; the maximum and its first index (VecMax). */
void orc_metrics_divergence(const orc_level *L, double *maxdiv, long long *at);
/* Convection (rhs.c:1463-1946) for boxes with no periodic face: the face
 * fluxes of ucat carried by Ucont/2, QUICK (central != 0: central), with the
 * one-sided forms next to the ring and next to cells of nvert above 0.1, then
 * conv = the flux differences over each interior cell, 0 on the ring.  Where
 * the reference reads two cells past the i or j end of a row it reads, on one
 * rank, the first cells of the next row; flat indexing reads the same.
 * Returns -1 (conv untouched) when a face is periodic, else 0. */
int orc_convection(const orc_level *L, const double *ucont, const double *ucat, int central, double *conv);
/* randomdirection's offsets for seeds 1 .. n: srand(seed); rand() scaled to
 * [-0.5, 0.5), exactly as ibm.c:101-104 draws them (the global generator). */
void orc_ibm_ray_offsets(int n, double *s);
int orc_ibm_search(int mx, int my, int mz, const double *cent, int n_v, const double *xyz, int n_elmt,
                   const int *tri, const double *nf, int ibi, int nbodies, const double *nvert_o,
                   double *nvert, int max_tries);

#ifdef __cplusplus
}
#endif
/* Viscous (rhs.c:1947-2566), laminar: visc ([mz][my][mx][3]) from ucat with
 * nu = 1 / ren; 0 on the ring. */
void orc_viscous(const orc_level *L, const double *ucat, double ren, double *visc);
/* FormFunction1 (rhs.c:2567-3351) for a box with no periodic face: ucat's
 * interior is refreshed from ucont (Contra2Cart), rhs's interior cells are
 * written; -1 for a periodic box. */
int orc_form_function1(const orc_level *L, const double *ucont, double *ucat, const double *p, double ren,
                       int central, double *rhs);
/* CalcRHS (implicitsolver.c:6449-6713) for a box with no periodic face. */
int orc_calc_rhs(const orc_level *L, const double *ucont, const double *ucont_o, const double *ucont_rm1,
                 double *ucat, const double *p, double ren, double dt, int ti, int tistart, int central,
                 double *rhs);
/* The boxes the momentum equation's pseudo-time iteration is restated for:
 * solid walls (bctype 1) on the x and y faces, and on the k faces either
 * walls or an inlet (bctype[4] 5) with an outlet (bctype[5] 4).  1 if covered. */
int orc_bcs_covered(const int *bc);
/* InflowFlux's inlet speed for the constant profiles 1, -1 and 11
 * (bcs.c:161-200); 0 for the others. */
int orc_inlet_speed(int inletprofile, double *uin);
/* InflowFlux (bcs.c:99-400) with an inlet on the k = 0 face (bctype[4] 5) and
 * a constant profile: on the face's interior cells above fluid cells, ubcs =
 * uin zet / |zet| and Ucont.z = uin |zet|; *flux_in_sum = their sum, in the
 * reference's loop order.  Nothing for a wall (FluxInSum keeps its value);
 * -1 for a profile that is not restated. */
int orc_inflow_flux(const orc_level *L, double *ucont, double *ubcs, int inletprofile, double *flux_in_sum);
/* The same with the shaped profiles 2 (a parabola in y), 4 (a pipe) and 7
 * (a parabola in y about 0), whose speed depends on the face cell's centre:
 * coor, the k = 0 node plane in the box layout [my][mx][3] (the first plane
 * of a [mz][my][mx][3] box), and cm, (CMx_c, CMy_c, CMz_c).  -1 for a shaped
 * profile without them.  orc_inflow_flux and orc_imp_rk take them from
 * orc_set_inlet_nodes (NULL: none). */
void orc_set_inlet_nodes(const double *coor0, const double *cm);
int orc_inflow_flux_ext(const orc_level *L, double *ucont, double *ubcs, int inletprofile, const double *coor,
                        const double *cm, double *flux_in_sum);
double orc_duct_speed(double xc, double yc);
/* Flux_in and ti for the uniform profiles 3 and 6 (uin = Flux_in) and 8
 * (uin = Flux_in = sin(2 3.14159 ti / 200)); orc_imp_rk sets ti itself. */
void orc_set_inlet_globals(double flux_in, int ti);
/* The table profiles 0 and 5 (+- InletInterpolation of uinr [101][1001]
 * at the face cell's radius and ti; NULL: none); -1 where the reference's
 * step index ti / 2 - (ti / 2000) 2000 falls outside the table. */
void orc_set_inlet_table(const double *uinr);
double orc_inlet_shaped(int inletprofile, const double *coor, int mx, int my, int i, int j, const double *cm);
/* FormBCS (bcs.c:4436-5889) on a covered box (orc_bcs_covered): three passes
 * of the outlet's flux correction (bctype[5] 4, bcs.c:4914-4998: ubcs on the
 * last face = the ucat next to it, Ucont.z of the last interior face = ubcs .
 * zet + ratio |zet| with ratio = (FluxInSum + FluxIntpSum - the outlet flux)
 * / the outlet area), Contra2Cart, the ghost faces u = 2 ubcs - inner on the
 * faces' interior cells (bcs.c:5250-5318) and the averages of ucat and p on
 * the box's 12 edges (bcs.c:5439-5570).  ucont, ubcs, ucat and p are read and
 * written.  -1 (nothing written) for a box that is not covered. */
int orc_form_bcs(const orc_level *L, double *ucont, double *ubcs, double *ucat, double *p, double flux_in_sum,
                 double flux_intp_sum);
typedef struct {
  int pseudo_iterations; /* pseudot at the end */
  int rejected;          /* iterations undone with the pseudo-time step halved */
  double norm_du, rel_du, norm_f, rel_f, lambda;
} orc_imp_rk_stats;
/* ImpRK (implicitsolver.c:7094-7257) on a covered box (orc_bcs_covered), one
 * block, no immersed body: InflowFlux as orc_inflow_flux, OutflowFlux (which
 * only sums a flux nothing here reads), FormBCS as orc_form_bcs with the
 * user's FluxIntpSum, CalcRHS as orc_calc_rhs; four Runge-Kutta stages per
 * pseudo-time iteration, the step halved and the iteration undone when both
 * norms grew, until |dU| <= atol or |dU| / |dU|_1 <= rtol or max_it
 * iterations.  ucont, ubcs, ucat and p are read and written; -1 for a box or
 * inlet profile that is not covered. */
int orc_imp_rk(const orc_level *L, double *ucont, const double *ucont_o, const double *ucont_rm1, double *ucat,
               double *p, double *ubcs, double ren, double dt, double st, double cfl, int ti, int tistart,
               int central, double atol, double rtol, int max_it, int inletprofile, double flux_intp_sum,
               orc_imp_rk_stats *out);
#endif
