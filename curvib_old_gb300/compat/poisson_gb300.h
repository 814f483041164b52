/*
 * Source-level drop-in of CURVIB's pressure-projection path onto libcvb.
 *
 * poisson_gb300.c is compiled inside a CURVIB source tree, beside poisson.c,
 * against CURVIB's own variables.h and PETSc.  It replaces, one for one:
 *   PoissonSolver_MG(usermg)  (poisson.c:1775; called at solvers.c:1052)
 *   UpdatePressure(&user[bi]) (poisson.c:2908; called at solvers.c:1066)
 *   Projection(&user[bi])     (poisson.c:2281; called at solvers.c:1068),
 *                             with its Contra2Cart (rhs.c:25) and
 *                             GhostNodeVelocity (bcs.c:3645)
 * and adds the set-up the reference does inside every PoissonSolver_MG call
 * (PoissonLHSNew on every level, MyNvertRestriction, FullyBlocked), which here
 * runs once and stays resident on the GPU.
 *
 * Scope: one block (block_number == 1) on one rank, as libcvb's contexts.
 * Every function returns 0 or a cvb_status, as a PetscErrorCode.
 */
#ifndef POISSON_GB300_H
#define POISSON_GB300_H

/* After MG_Initial (init.c:853-1019): uploads every level's metrics and the
 * finest nvert, restricts nvert and builds the operators.  Solver controls are
 * read here from PETSc's options database (control.dat and the command line):
 * -ps_ksp_rtol, -ps_ksp_atol, -ps_ksp_max_it, -ps_ksp_gmres_restart and the
 * library's -cvb_* options (cvb_solve_opts_from_args). */
PetscErrorCode PoissonSetup_GB300(UserMG *usermg);
/* The immersed body moved: new finest nvert, operators rebuilt. */
PetscErrorCode PoissonSetNvert_GB300(UserMG *usermg);
PetscErrorCode PoissonSolver_MG_GB300(UserMG *usermg);
PetscErrorCode UpdatePressure_GB300(UserCtx *user);
PetscErrorCode Projection_GB300(UserCtx *user);
/* In place of Convection (rhs.c:1463), same arguments. */
PetscErrorCode Convection_GB300(UserCtx *user, Vec Ucont, Vec Ucat, Vec Conv);
/* In place of ImpRK (implicitsolver.c:7094; Flow_Solver's momentum solver
 * for implicit 3 or 7, solvers.c:1028 and 1036), same arguments: on the device
 * for one block with no immersed body and walls on every face, else the
 * reference's own ImpRK. */
PetscErrorCode ImpRK_GB300(UserCtx *user, IBMNodes *ibm, FSInfo *fsi);
/* At the end of the run. */
PetscErrorCode PoissonFinalize_GB300(void);

#endif
