/*
 * TEST INFRASTRUCTURE ONLY -- never linked into the product library.
 *
 * A single-process stand-in for the small part of the PETSc 3.6 / MPI API that
 * CURVIB's poisson.c, metrics.c and implicitsolver.c call.  It exists so that
 * those reference sources can be compiled unmodified into oracle/_ref/ and run
 * on the CPU to produce the reference's own numbers (assembled operator, RHS,
 * metrics, restriction/prolongation, projection) for the parity tests.
 *
 * Semantics follow the public PETSc DMDA documentation for ONE rank:
 *   - a global vector holds the owned box [0,mx)x[0,my)x[0,mz), i fastest;
 *   - a local vector holds the ghosted box; on one rank a periodic direction has
 *     s ghost layers on each side that wrap around, a non-periodic one has none;
 *   - DMDAVecGetArray returns [k][j][i] pointer tables indexed in global
 *     coordinates (ghost indices may be negative).
 * Krylov / preconditioner objects are inert: the harness never calls
 * PoissonSolver_MG, only the functions around it.
 */
#ifndef CVB_PETSC_SHIM_H
#define CVB_PETSC_SHIM_H

#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>

typedef int PetscInt;
typedef int PetscMPIInt;
typedef double PetscReal;
typedef double PetscScalar;
typedef int PetscErrorCode;
typedef int PetscLogDouble_i;
typedef double PetscLogDouble;
typedef enum { PETSC_FALSE = 0, PETSC_TRUE = 1 } PetscBool;
typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int InsertMode;
typedef int ScatterMode;
typedef int NormType;
typedef int MatAssemblyType;
typedef int MatOperation;
typedef int DMBoundaryType;
typedef int DMDAStencilType;
typedef int MatShiftType;
typedef int PCMGType;
typedef int PCMGCycleType;
typedef int ISColoringType;
typedef int MatStructure;
typedef int PetscFileMode;
typedef const char *KSPType;
typedef const char *PCType;
typedef const char *SNESType;
typedef const char *MatType;

#define PETSC_COMM_WORLD 0
#define PETSC_COMM_SELF 1
#define MPI_COMM_WORLD 0
#define MPI_DOUBLE 1
#define MPI_INT 2
#define MPIU_INT 2
#define MPIU_REAL 1
#define MPIU_SCALAR 1
#define MPI_SUM 1
#define MPI_MAX 2
#define MPI_MIN 3
#define PETSC_NULL 0
#define PETSC_DEFAULT (-2)
#define PETSC_DECIDE (-1)
#define PETSC_DETERMINE (-1)
#define PETSC_STDOUT stdout
#define INSERT_VALUES 1
#define ADD_VALUES 2
#define SCATTER_FORWARD 0
#define SCATTER_REVERSE 1
#define NORM_1 0
#define NORM_2 1
#define NORM_INFINITY 3
#define MAT_FINAL_ASSEMBLY 0
#define MAT_FLUSH_ASSEMBLY 1
#define MATOP_MULT 1
#define MATOP_MULT_ADD 2
#define MATOP_MULT_TRANSPOSE 3
#define DM_BOUNDARY_NONE 0
#define DM_BOUNDARY_PERIODIC 3
#define DMDA_STENCIL_STAR 0
#define DMDA_STENCIL_BOX 1
#define MAT_SHIFT_NONZERO 1
#define MAT_SHIFT_POSITIVE_DEFINITE 2
#define PC_MG_MULTIPLICATIVE 0
#define PC_MG_ADDITIVE 1
#define PC_MG_FULL 2
#define PC_MG_KASKADE 3
#define PC_MG_CYCLE_V 1
#define PC_MG_CYCLE_W 2
#define IS_COLORING_GLOBAL 0
#define IS_COLORING_GHOSTED 1
#define SAME_NONZERO_PATTERN 0
#define DIFFERENT_NONZERO_PATTERN 1
#define FILE_MODE_READ 0
#define FILE_MODE_WRITE 1
#define KSPGMRES "gmres"
#define KSPFGMRES "fgmres"
#define KSPBCGS "bcgs"
#define KSPBCGSL "bcgsl"
#define KSPPREONLY "preonly"
#define KSPRICHARDSON "richardson"
#define PCMG "mg"
#define PCLU "lu"
#define PCNONE "none"
#define PCBJACOBI "bjacobi"
#define PCJACOBI "jacobi"
#define PCILU "ilu"
#define SNESLS "ls"
#define SNESTR "tr"
#define SNESNEWTONTR "newtontr"
#define SNESNEWTONLS "newtonls"
#define MATAIJ "aij"
#define PETSC_VIEWER_STDOUT_WORLD 0
#define PETSC_VIEWER_STDOUT_SELF 0
#define PETSC_VIEWER_DRAW_WORLD 0
#define PETSC_ERR_ARG_OUTOFRANGE 63

#define PetscMax(a, b) (((a) < (b)) ? (b) : (a))
#define PetscMin(a, b) (((a) < (b)) ? (a) : (b))
#define PetscAbsScalar(a) fabs(a)
#define PetscAbsReal(a) fabs(a)
#define PetscSqrtScalar(a) sqrt(a)
#define PetscMalloc(sz, pp) ((*(void **)(pp) = calloc(1, (size_t)(sz) > 0 ? (size_t)(sz) : 1)) == NULL)
#define PetscFree(p) (free(p), (p) = NULL, 0)
#define PetscNew(pp) PetscMalloc(sizeof(**(pp)), (pp))
#define CHKERRQ(e) do { if (e) return (e); } while (0)
#define CHKMEMQ
#define SETERRQ(c, n, s) return (n)
#define SETERRQ1(c, n, s, a) return (n)
#define SETERRQ2(c, n, s, a, b) return (n)

/* Objects.  All are pointers to shim-owned structs. */
typedef struct _p_DM *DM;
typedef struct _p_Vec *Vec;
typedef struct _p_Mat *Mat;
typedef struct _p_AO *AO;
typedef struct _p_KSP *KSP;
typedef struct _p_PC *PC;
typedef struct _p_SNES *SNES;
typedef struct _p_MatNullSpace *MatNullSpace;
typedef struct _p_VecScatter *VecScatter;
typedef struct _p_ISColoring *ISColoring;
typedef struct _p_MatFDColoring *MatFDColoring;
typedef struct _p_KSPFischerGuess *KSPFischerGuess;
typedef struct _p_PetscViewer *PetscViewer;
typedef struct _p_DMMG *DMMG;
typedef struct _p_IS *IS;

typedef struct {
  PetscInt dim, dof, sw;
  PetscInt mx, my, mz;
  PetscInt xs, ys, zs;
  PetscInt xm, ym, zm;
  PetscInt gxs, gys, gzs;
  PetscInt gxm, gym, gzm;
  DMBoundaryType bx, by, bz;
  DMDAStencilType st;
  DM da;
} DMDALocalInfo;

/* --- the API subset (implemented in petsc_shim.c) --- */
PetscErrorCode PetscPrintf(MPI_Comm comm, const char *fmt, ...);
PetscErrorCode PetscFPrintf(MPI_Comm comm, FILE *f, const char *fmt, ...);
PetscErrorCode PetscSynchronizedPrintf(MPI_Comm comm, const char *fmt, ...);
PetscErrorCode PetscSynchronizedFlush(MPI_Comm comm, ...);
PetscErrorCode PetscBarrier(void *obj);
PetscErrorCode PetscTime(PetscLogDouble *t);

int MPI_Comm_rank(MPI_Comm c, int *r);
int MPI_Comm_size(MPI_Comm c, int *s);
int MPI_Allreduce(const void *s, void *r, int n, MPI_Datatype t, MPI_Op o, MPI_Comm c);
int MPI_Bcast(void *b, int n, MPI_Datatype t, int root, MPI_Comm c);

PetscErrorCode DMDACreate3d(MPI_Comm comm, DMBoundaryType bx, DMBoundaryType by, DMBoundaryType bz,
                            DMDAStencilType st, PetscInt M, PetscInt N, PetscInt P, PetscInt m,
                            PetscInt n, PetscInt p, PetscInt dof, PetscInt s, const PetscInt *lx,
                            const PetscInt *ly, const PetscInt *lz, DM *da);
PetscErrorCode DMDestroy(DM *da);
PetscErrorCode DMDAGetLocalInfo(DM da, DMDALocalInfo *info);
PetscErrorCode DMDAGetInfo(DM da, PetscInt *dim, PetscInt *M, PetscInt *N, PetscInt *P, PetscInt *m,
                           PetscInt *n, PetscInt *p, PetscInt *dof, PetscInt *s,
                           DMBoundaryType *bx, DMBoundaryType *by, DMBoundaryType *bz,
                           DMDAStencilType *st);
PetscErrorCode DMGetCoordinateDM(DM da, DM *cda);
PetscErrorCode DMGetCoordinates(DM da, Vec *c);
PetscErrorCode DMGetCoordinatesLocal(DM da, Vec *c);
PetscErrorCode DMDASetUniformCoordinates(DM da, PetscReal x0, PetscReal x1, PetscReal y0,
                                         PetscReal y1, PetscReal z0, PetscReal z1);
PetscErrorCode DMCreateGlobalVector(DM da, Vec *v);
PetscErrorCode DMCreateLocalVector(DM da, Vec *v);
PetscErrorCode DMDAVecGetArray(DM da, Vec v, void *array);
PetscErrorCode DMDAVecRestoreArray(DM da, Vec v, void *array);
PetscErrorCode DMGlobalToLocalBegin(DM da, Vec g, InsertMode m, Vec l);
PetscErrorCode DMGlobalToLocalEnd(DM da, Vec g, InsertMode m, Vec l);
PetscErrorCode DMLocalToGlobalBegin(DM da, Vec l, InsertMode m, Vec g);
PetscErrorCode DMLocalToGlobalEnd(DM da, Vec l, InsertMode m, Vec g);
PetscErrorCode DMLocalToLocalBegin(DM da, Vec a, InsertMode m, Vec b);
PetscErrorCode DMLocalToLocalEnd(DM da, Vec a, InsertMode m, Vec b);
PetscErrorCode DMDAGetAO(DM da, AO *ao);
PetscErrorCode AOApplicationToPetsc(AO ao, PetscInt n, PetscInt *idx);
PetscErrorCode DMDACreateNaturalVector(DM da, Vec *v);
PetscErrorCode DMDAGlobalToNaturalBegin(DM da, Vec g, InsertMode m, Vec n);
PetscErrorCode DMDAGlobalToNaturalEnd(DM da, Vec g, InsertMode m, Vec n);
PetscErrorCode DMDAGetGlobalIndices(DM da, PetscInt *n, const PetscInt **idx);

PetscErrorCode VecDuplicate(Vec v, Vec *w);
PetscErrorCode VecDestroy(Vec *v);
PetscErrorCode VecSet(Vec v, PetscScalar a);
PetscErrorCode VecCopy(Vec x, Vec y);
PetscErrorCode VecAYPX(Vec y, PetscScalar a, Vec x);
PetscErrorCode VecAXPY(Vec y, PetscScalar a, Vec x);
PetscErrorCode VecWAXPY(Vec w, PetscScalar a, Vec x, Vec y);
PetscErrorCode VecScale(Vec x, PetscScalar a);
PetscErrorCode VecNorm(Vec x, NormType t, PetscReal *r);
PetscErrorCode VecMax(Vec x, PetscInt *p, PetscReal *r);
PetscErrorCode VecMin(Vec x, PetscInt *p, PetscReal *r);
PetscErrorCode VecStrideMax(Vec x, PetscInt start, PetscInt *p, PetscReal *r);
PetscErrorCode VecStrideMin(Vec x, PetscInt start, PetscInt *p, PetscReal *r);
PetscErrorCode VecGetLocalSize(Vec x, PetscInt *n);
PetscErrorCode PetscViewerBinaryOpen(MPI_Comm comm, const char name[], PetscFileMode mode, PetscViewer *v);
PetscErrorCode PetscViewerDestroy(PetscViewer *v);
PetscErrorCode VecView(Vec x, PetscViewer v);
PetscErrorCode VecLoad(Vec x, PetscViewer v);
PetscErrorCode PetscOptionsClearValue(const char name[]);
void shim_set_viewer_dir(const char *dir);
PetscErrorCode VecGetSize(Vec x, PetscInt *n);
PetscErrorCode VecAssemblyBegin(Vec x);
PetscErrorCode VecAssemblyEnd(Vec x);
PetscErrorCode VecGetArray3d(Vec x, PetscInt m, PetscInt n, PetscInt p, PetscInt ms, PetscInt ns,
                             PetscInt ps, PetscScalar ****a);
PetscErrorCode VecRestoreArray3d(Vec x, PetscInt m, PetscInt n, PetscInt p, PetscInt ms,
                                 PetscInt ns, PetscInt ps, PetscScalar ****a);
/* The vector's own storage (a DMDA vector's box, dof interleaved).  Every Get
 * must be matched by a Restore; shim_arrays_out() counts the unmatched ones. */
PetscErrorCode VecGetArray(Vec x, PetscScalar **a);
PetscErrorCode VecRestoreArray(Vec x, PetscScalar **a);
int shim_arrays_out(void);
PetscErrorCode DMDAGetGhostCorners(DM da, PetscInt *x, PetscInt *y, PetscInt *z, PetscInt *m,
                                   PetscInt *n, PetscInt *p);
/* A flat options table ("-name" -> value string), as PETSc's options database
 * holds control.dat and the command line.  Get* leave the value untouched and
 * set *set = PETSC_FALSE when the option is absent. */
PetscErrorCode PetscOptionsSetValue(const char name[], const char value[]);
PetscErrorCode PetscOptionsClear(void);
PetscErrorCode PetscOptionsGetString(const char pre[], const char name[], char s[], size_t len,
                                     PetscBool *set);
PetscErrorCode PetscOptionsGetReal(const char pre[], const char name[], PetscReal *v, PetscBool *set);
PetscErrorCode PetscOptionsGetInt(const char pre[], const char name[], PetscInt *v, PetscBool *set);
PetscErrorCode VecScatterCreateToZero(Vec x, VecScatter *ctx, Vec *out);
PetscErrorCode VecScatterBegin(VecScatter ctx, Vec x, Vec y, InsertMode m, ScatterMode s);
PetscErrorCode VecScatterEnd(VecScatter ctx, Vec x, Vec y, InsertMode m, ScatterMode s);
PetscErrorCode VecScatterDestroy(VecScatter *ctx);

PetscErrorCode MatCreateAIJ(MPI_Comm comm, PetscInt m, PetscInt n, PetscInt M, PetscInt N,
                            PetscInt dnz, const PetscInt *dnnz, PetscInt onz,
                            const PetscInt *onnz, Mat *A);
PetscErrorCode MatZeroEntries(Mat A);
PetscErrorCode MatSetValues(Mat A, PetscInt m, const PetscInt *rows, PetscInt n,
                            const PetscInt *cols, const PetscScalar *v, InsertMode mode);
PetscErrorCode MatAssemblyBegin(Mat A, MatAssemblyType t);
PetscErrorCode MatAssemblyEnd(Mat A, MatAssemblyType t);
PetscErrorCode MatDestroy(Mat *A);
PetscErrorCode MatMult(Mat A, Vec x, Vec y);
PetscErrorCode MatCreateShell(MPI_Comm comm, PetscInt m, PetscInt n, PetscInt M, PetscInt N,
                              void *ctx, Mat *A);
PetscErrorCode MatShellSetOperation(Mat A, MatOperation op, void (*f)(void));
PetscErrorCode MatShellGetContext(Mat A, void *ctx);

/* Inert Krylov / PC / null-space objects: present so the sources link. */
PetscErrorCode MatNullSpaceCreate(MPI_Comm c, PetscBool has_cnst, PetscInt n, const Vec *vecs,
                                  MatNullSpace *sp);
PetscErrorCode MatNullSpaceSetFunction(MatNullSpace sp, PetscErrorCode (*f)(MatNullSpace, Vec, void *),
                                       void *ctx);
PetscErrorCode MatNullSpaceDestroy(MatNullSpace *sp);
PetscErrorCode MatSetNullSpace(Mat A, MatNullSpace sp);
/* Routines the sources pass as function pointers. */
PetscErrorCode PCMGResidualDefault(Mat A, Vec b, Vec x, Vec r);
PetscErrorCode PCMGDefaultResidual(Mat A, Vec b, Vec x, Vec r);
PetscErrorCode KSPMonitorTrueResidualNorm(KSP k, PetscInt n, PetscReal r, void *ctx);
PetscErrorCode MatMFFDComputeJacobian(SNES s, Vec x, Mat A, Mat B, void *ctx);

#endif
