// Grouped (batched) kernels: one launch runs one phase of the solve for every
// problem of a work-list.  Each task owns a contiguous range of the launch's
// blocks; a block finds its task by binary search over the tasks' first blocks
// and runs the same per-block body as the single-problem kernel.  The task list
// travels as a __grid_constant__ kernel parameter, so no table is copied to the
// device per launch and a captured graph keeps it.
#pragma once
#include "cvb_internal.h"

namespace cvb {

constexpr int kMaxTasks = 96;        // tasks per grouped launch (64-byte tasks, 6 KB of parameters)
constexpr int kBatchRestart = 64;    // Krylov basis slots per problem (same bound as a single solve)
constexpr int kSumSlots = kBatchRestart + 4;

struct GTask {
  const LevelDev *L;   // level of the task (restrict/prolong: the fine level; the coarse one is L - 1)
  const void *a;       // first input
  const void *b;       // second input (rhs / x / matrix)
  void *c;             // output
  const int *gate;     // skip the task while *gate != 0
  int block0;          // first block of the launch that belongs to this task
  int gx, gy;          // the task's grid in x and y (z: the rest)
  int p0, p1;          // kernel-specific integers
  int pad;
};
static_assert(sizeof(GTask) == 64, "GTask layout");

struct TaskList {
  int n;               // tasks in use
  int nblocks;         // total blocks (the launch's grid)
  GTask t[kMaxTasks];
};

// Per-problem Krylov state, resident on the device.  The FGMRES bookkeeping of a
// problem (Gram-Schmidt column, Givens rotations, convergence test, triangular
// solve) runs in one-block kernels on this state, so the host never waits for
// an iteration's scalars.
struct KState {
  double H[(kBatchRestart + 1) * kBatchRestart];  // column j at H[j*(m+1) ...]
  double cs[kBatchRestart], sn[kBatchRestart], g[kBatchRestart + 1], y[kBatchRestart];
  double beta;        // ||r|| at the start of the cycle
  double bnorm;       // ||b|| (after the range projection)
  double target;      // max(rtol*bnorm, atol)
  double est;         // |g_{j+1}|: the residual estimate of the current iterate
  double hn;          // ||w|| after orthogonalisation: the scale of the next basis vector
  double removed;     // range projection: fluid mean of b/aj that was removed
  int m;              // restart length
  int max_it;
  int j;              // basis vectors in the current cycle
  int iters;          // FGMRES iterations so far
  int cycles;         // completed restart cycles
  int pad;
};

// Host-visible flags of one problem, copied to pinned memory after every round.
struct BFlags {
  int gate;      // 1: the current cycle takes no more iterations (converged, broke down or full)
  int fin;       // 1: the solve is finished (result final, statistics below valid)
  int status;    // cvb_status once finished
  int iters;
  int cycles;
  int notfin;    // 1 - fin: gates the end-of-solve null-space removal
  double rel;    // true relative residual at the last cycle end
  double abs;
  double bnorm;
  double removed;
};

// One problem as the grouped Krylov kernels see it.
struct BProblem {
  size_t n;                  // finest-level cells
  int nb;                    // reduction blocks (a function of n only)
  int pad;
  double *b, *x, *w, *r;     // finest FP64 vectors
  double *const *V;          // device table of the FGMRES basis V[0..m]
  double *const *Z;          // device table of the preconditioned basis Z[0..m-1]
  double *partial;           // [rows][nb] first-stage sums
  double *sums;              // [kSumSlots] second-stage sums
  KState *ks;
  BFlags *fl;
  const LevelDev *F;         // finest level (device copy)
  const double *aj;          // finest aj (FP64)
};

// Reduction blocks of a problem of n cells: fixed by n alone, so a problem's
// sums have the same summation tree alone and in any batch.
inline int batch_reduce_blocks(size_t n) {
  size_t nb = (n + 8191) / 8192;
  return (int)(nb < 1 ? 1 : (nb > 608 ? 608 : nb));
}

// --- grouped launchers (kernels_batch.cu) ---------------------------------
// Stencil / V-cycle phases: L = device LevelDev, a/b/c per kernel.
void glaunch_residual32(const TaskList &tl, cudaStream_t s);   // a = x, b = rhs, c = r
void glaunch_residual64(const TaskList &tl, cudaStream_t s);   // a = x, b = rhs or null (apply), c = y
void glaunch_restrict(const TaskList &tl, bool f32, cudaStream_t s);     // a = fine, c = coarse
void glaunch_prolong(const TaskList &tl, bool f32, cudaStream_t s);      // a = coarse, c = fine (added)
// line sweeps: a = rhs (or residual), b = x (null: zero guess), c = xnew, p0 = mode (fused sweep);
// line solve: p1 = zebra color + 1 (0: every line)
void glaunch_line_sweep(const TaskList &tl, bool f32, float omega32, double omega64, size_t smem, cudaStream_t s);
// rr: the rows per lane shared by every task's level (1, 2, 4, 8), or 0
void glaunch_line_solve(const TaskList &tl, bool f32, float omega32, double omega64, size_t smem, int rr,
                        cudaStream_t s);
// zebra: residual on the cells of color p0 (a = x, b = rhs, c = r); zero fill of c[0..p0)
void glaunch_resid_color(const TaskList &tl, bool f32, cudaStream_t s);
void glaunch_zebra_fused(const TaskList &tl, bool f32, float omega32, double omega64, size_t smem, cudaStream_t s);
void glaunch_zero(const TaskList &tl, bool f32, cudaStream_t s);
// dense coarsest solve: a = r, b = Minv, c = e, p0 = n
void glaunch_dense(const TaskList &tl, bool f32, cudaStream_t s);
// element-wise: a = src, c = dst, p0 = n; kind 0 copy f32, 1 copy f64, 2 f64->f32, 3 f32->f64
void glaunch_elementwise(const TaskList &tl, int kind, cudaStream_t s);

// Krylov phases over problems: p0 = problem index into P (device array).
// multidot of w (a) with V[base .. base+cnt): p1 = base | (cnt << 8), pad = row of w.w
// (-1: none); cnt 0 with pad >= 0 is a plain norm.  Rows go to partial[row][nb].
void glaunch_multidot(const TaskList &tl, const BProblem *P, cudaStream_t s);
// finish: gx rows starting at partial row p1 into sums[p1 ...]; one block per row
void glaunch_finish(const TaskList &tl, const BProblem *P, cudaStream_t s);
// w -= sum_q sums[q] V_q for q < p1, then partial[kNormRow] = per-block |w|^2
void glaunch_multiaxpy_norm(const TaskList &tl, const BProblem *P, cudaStream_t s);
// dst = src / scalar: a = src, c = dst, b = scalar pointer, p0 = n
void glaunch_scale(const TaskList &tl, cudaStream_t s);
// x += Z y over the problem's current basis (count from its KState)
void glaunch_update(const TaskList &tl, const BProblem *P, cudaStream_t s);
// fluid sums (null space) / range projection sums and their corrections
void glaunch_fluid_sum(const TaskList &tl, const BProblem *P, cudaStream_t s);
void glaunch_add_fluid_const(const TaskList &tl, const BProblem *P, cudaStream_t s);
void glaunch_fluid_ratio(const TaskList &tl, const BProblem *P, cudaStream_t s);
void glaunch_remove_aj_mean(const TaskList &tl, const BProblem *P, cudaStream_t s);

// One-block-per-problem control kernels over a list of problems.
struct ProbList {
  int n;
  int idx[kMaxTasks];
};
// Opens a solve: ||b|| from sums[kNormRow] and the tolerances.
struct InitList {
  int n;
  int idx[kMaxTasks];
  int m[kMaxTasks], max_it[kMaxTasks];
  double rtol[kMaxTasks], atol[kMaxTasks];
};
constexpr int kNormRow = kBatchRestart + 1;  // partial row / sums slot of single norms
void launch_k_init(const InitList &il, const BProblem *P, cudaStream_t s);
// After the residual norm: finish the solve or open a (new) cycle.
void launch_k_cycle_start(const ProbList &pl, const BProblem *P, cudaStream_t s);
// One FGMRES iteration's scalar work (Gram-Schmidt column, Givens, convergence).
void launch_k_arnoldi(const ProbList &pl, const BProblem *P, cudaStream_t s);
// y = R^-1 g over the cycle's basis.
void launch_k_solve_y(const ProbList &pl, const BProblem *P, cudaStream_t s);
// The range projection's removed constant from sums[0..1] (after glaunch_fluid_ratio + finish).
void launch_k_removed(const ProbList &pl, const BProblem *P, cudaStream_t s);

}  // namespace cvb
