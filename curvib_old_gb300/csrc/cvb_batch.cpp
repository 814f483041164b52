// Batch engine: many independent pressure solves, each a set-up cvb_ctx, run in
// lockstep rounds on one stream.  One round is one FGMRES iteration for every
// active problem; each phase of it (every V-cycle kernel, each Krylov step) is
// ONE grouped launch over a work-list of all problems' tiles.  The FGMRES
// scalars live on the device (KState); the host only reads each problem's
// flags one round late, so the GPU always has the next round queued.  Problems
// join (submit) and leave (poll) between rounds: continuous batching.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <deque>
#include <map>
#include <string>
#include <vector>

#include "../../include/cvb.h"
#include "batch.h"
#include "cvb_ctx.h"
#include "stencil_body.cuh"

using namespace cvb;

namespace {

constexpr int kMaxSlots = 1024;
constexpr int kMaxLevels = 16;
constexpr int kMaxFusedRows = 400;
constexpr size_t kMaxSmem = 200 * 1024;

enum PState { P_NEW, P_ITER };

struct Prob {
  cvb_ctx *ctx = nullptr;
  int slot = -1;
  int ticket = -1;
  PState state = P_NEW;
  int host_j = 0;       // iterations issued in the current cycle
  int host_cycle = 0;   // cycles the host has closed
  int issued = 0;       // iterations issued in total
  bool warm = false, project = true;
  double rtol = 1e-8, atol = 0.0;
  int max_it = 200;
  int issue_cap = 0;        // iterations the host issues at most (a safety net over the device's budget)
  long long first_round = 0;
  bool close_next = false;  // the device closed the current cycle: close it in the next round
  const double *host_b = nullptr;  // optional host rhs copied in at admission
};

struct Done {
  int ticket;
  cvb_ctx *ctx;
  cvb_solve_stats st;
};

// Sink of the ops of one round, grouped by schedule key and kernel kind.
enum OpKind {
  OK_RES32, OK_RES64, OK_RESTRICT, OK_PROLONG, OK_SWEEP, OK_SOLVE, OK_DENSE, OK_COPY, OK_CONV, OK_WIDEN,
  OK_ZERO, OK_RESC, OK_ZFUSED,
  // line solves of levels whose lines have 1, 2, 4 or 8 rows per lane: one
  // launch each, so each runs the kernel specialised for its layout
  OK_SOLVE_R1, OK_SOLVE_R2, OK_SOLVE_R4, OK_SOLVE_R8, OK_COUNT
};

// The line-solve op kind of a level: by its lines' rows per lane.
static OpKind solve_kind(const LevelDev &L) {
  switch (LineLayout::of(L.g.my).R) {
    case 1: return OK_SOLVE_R1;
    case 2: return OK_SOLVE_R2;
    case 4: return OK_SOLVE_R4;
    case 8: return OK_SOLVE_R8;
    default: return OK_SOLVE;
  }
}


struct OpBatch {
  TaskList tl;
  size_t smem = 0;
};

}  // namespace

// cvb_batch_solve's bound on its host loop when the caller sets none
constexpr long long kDefaultRoundLimit = 1000000;

struct cvb_batch {
  int device = 0;
  cudaStream_t stream = nullptr, copy_stream = nullptr;
  bool own_stream = false;
  std::string err;
  cvb_solve_opts opts;
  bool mixed = true;
  int m = 30;
  // device state, one entry per slot
  BProblem *dP = nullptr;
  KState *dK = nullptr;
  BFlags *dF = nullptr;
  LevelDev *dL = nullptr;  // [slot][kMaxLevels]
  BFlags *hF[2] = {nullptr, nullptr};
  int hF_slots[2] = {0, 0};
  cudaEvent_t ev[2] = {nullptr, nullptr};
  long long round = 0;
  std::vector<int> free_slots;
  std::vector<Prob> active;
  std::deque<Prob> pending;
  std::deque<Done> done;
  int next_ticket = 0;
  long long launches_per_round = 0;
  long long round_limit = kDefaultRoundLimit;  // rounds cvb_batch_solve issues before CVB_TIMEOUT
  // the mixed-precision rounds' V-cycles as a CUDA graph (run_vcycles)
  bool graphs = true;
  std::vector<unsigned long long> vkey;  // (slot, ctx set-up id) of the iterating problems it was made for
  int vkey_rounds = 0;                   // rounds run with that key so far
  cudaGraphExec_t vexec = nullptr;
  bool vexec_ok = false;                 // vexec holds the program of vkey
  long long graph_captures = 0, graph_updates = 0, graph_replays = 0;
};

// ------------------------------------------------------------------ helpers
static int bfail(cvb_batch *b, int code, const char *fmt, ...) __attribute__((format(printf, 3, 4)));
static int bfail(cvb_batch *b, int code, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  if (b) b->err = buf;
  return code;
}
#define BCK(call)                                                                                   \
  do {                                                                                              \
    cudaError_t e_ = (call);                                                                        \
    if (e_ != cudaSuccess)                                                                          \
      return bfail(bt, e_ == cudaErrorMemoryAllocation ? CVB_OOM : CVB_CUDA_ERROR, "%s: %s (%s:%d)", \
                   #call, cudaGetErrorString(e_), __FILE__, __LINE__);                              \
  } while (0)
#define BTRY(expr)                 \
  do {                             \
    int s_ = (expr);               \
    if (s_ != CVB_OK) return s_;   \
  } while (0)

static inline int nblk(size_t n, int t) { return (int)((n + t - 1) / t); }
static int elem_blocks(size_t n) { return std::max(1, std::min(nblk(n, 256), 2048)); }

// Appends tasks to a list of TaskLists (a new list every kMaxTasks tasks).
struct Lists {
  std::vector<OpBatch> v;
  void add(const GTask &t0, int blocks, size_t smem = 0) {
    if (blocks <= 0) return;
    if (v.empty() || v.back().tl.n == kMaxTasks) {
      v.emplace_back();
      std::memset(&v.back().tl, 0, sizeof(TaskList));
    }
    OpBatch &ob = v.back();
    GTask t = t0;
    t.block0 = ob.tl.nblocks;
    ob.tl.t[ob.tl.n++] = t;
    ob.tl.nblocks += blocks;
    ob.smem = std::max(ob.smem, smem);
  }
};

static GTask task(const LevelDev *L, const void *a, const void *b, void *c, const int *gate, int gx = 0, int gy = 0,
                  int p0 = 0, int p1 = 0, int pad = 0) {
  GTask t;
  std::memset(&t, 0, sizeof t);
  t.L = L; t.a = a; t.b = b; t.c = c; t.gate = gate;
  t.gx = gx; t.gy = gy; t.p0 = p0; t.p1 = p1; t.pad = pad;
  return t;
}

// ------------------------------------------------------------ V-cycle program
// The ops of one problem's V-cycle, in the order of the single-solve vcycle(),
// each tagged with a schedule key: ops with equal keys (from all problems) run
// in one grouped launch, keys in increasing order.
struct VSink {
  std::map<long long, std::array<Lists, OK_COUNT>> *keyed;
  void add(long long key, OpKind k, const GTask &t, int blocks, size_t smem = 0) {
    (*keyed)[key][k].add(t, blocks, smem);
  }
};
static long long key_desc(int depth, int sub) { return (long long)depth * 1000 + sub; }
static long long key_coarse() { return 500000; }
static long long key_asc(int depth, int sub) { return 1000000 + (long long)(63 - depth) * 1000 + sub; }

template <typename T>
static T *lvec(LevelDev &L, int which);
template <>
float *lvec<float>(LevelDev &L, int which) {
  size_t n = L.g.n();
  return which == 0 ? L.r32 : which == 1 ? L.e32 : which == 2 ? L.t32 : L.t32 + n;
}
template <>
double *lvec<double>(LevelDev &L, int which) {
  size_t n = L.g.n();
  return which == 0 ? L.r64 : which == 1 ? L.e64 : which == 2 ? L.t64 : L.t64 + n;
}

// r = b - A x on one level: the FP32 kernel marches tiles of 31 x 7 cells in k,
// the FP64 one takes 32 x 4 cells per plane.
template <typename T>
static void add_residual(VSink &vs, long long key, LevelDev &L, const LevelDev *dLv, const T *x, const T *b, T *r,
                         const int *gate) {
  if (sizeof(T) == 4) {
    const MarchGrid m = MarchGrid::of(L.g);
    vs.add(key, OK_RES32, task(dLv, x, b, r, gate, m.gx, m.gy), m.blocks());
  } else {
    const int gx = plane_blocks(L.g);
    vs.add(key, OK_RES64, task(dLv, x, b, r, gate, gx, 1), gx * L.g.mz);
  }
}

template <typename T>
static void gen_sweep(VSink &vs, long long key0, long long key1, LevelDev &L, const LevelDev *dLv, const T *b,
                      const T *x, T *xnew, bool zero, const int *gate) {
  const bool f32 = sizeof(T) == 4;
  const int TW = f32 ? 32 : 16;                         // fused sweep tiles
  const int SW = f32 ? kSolveTW32 : kSolveTW64;         // line-solve tiles
  const size_t ssw = f32 ? line_sweep_smem<float, 32>(L.g) : line_sweep_smem<double, 16>(L.g);
  const size_t sso = f32 ? line_solve_smem<float, kSolveTW32>(L.g) : line_solve_smem<double, kSolveTW64>(L.g);
  const bool async = sso <= kMaxSmem;
  const int lblocks = nblk(L.g.mx, TW) * L.g.mz, sblocks = nblk(L.g.mx, SW) * L.g.mz;
  const int split = f32 ? L.sweep32 : L.sweep64;
  T *res = lvec<T>(L, 3);
  if (zero) {
    if (async) vs.add(key1, solve_kind(L), task(dLv, b, nullptr, xnew, gate, nblk(L.g.mx, SW)), sblocks, sso);
    else vs.add(key1, OK_SWEEP, task(dLv, b, nullptr, xnew, gate, nblk(L.g.mx, TW), 0, 0), lblocks, ssw);
  } else if (split == 1) {
    add_residual<T>(vs, key0, L, dLv, x, b, res, gate);
    if (async) vs.add(key1, solve_kind(L), task(dLv, res, x, xnew, gate, nblk(L.g.mx, SW)), sblocks, sso);
    else vs.add(key1, OK_SWEEP, task(dLv, res, x, xnew, gate, nblk(L.g.mx, TW), 0, 2), lblocks, ssw);
  } else {
    vs.add(key1, OK_SWEEP, task(dLv, b, x, xnew, gate, nblk(L.g.mx, TW), 0, 1), lblocks, ssw);
  }
}

// One zebra half-sweep of color `color`, in place on x (keys k0: residual, k1: solve).
template <typename T>
static void gen_zebra_half(VSink &vs, long long k0, long long k1, LevelDev &L, const LevelDev *dLv, const T *b, T *x,
                           int color, bool zero, const int *gate) {
  const bool f32 = sizeof(T) == 4;
  const int SW = f32 ? kSolveTW32 : kSolveTW64;
  const size_t sso = f32 ? line_solve_smem<float, kSolveTW32>(L.g) : line_solve_smem<double, kSolveTW64>(L.g);
  T *res = lvec<T>(L, 3);
  const bool fuse = f32 ? L.zfuse32 != 0 : L.zfuse64 != 0;
  if (!zero && fuse && zebra_fusable<T>(L) && L.g.my <= 400 && sso <= 200 * 1024) {
    const int gx = f32 ? solve_tiles_x<kSolveTW32>(L.g, color) : solve_tiles_x<kSolveTW64>(L.g, color);
    vs.add(k1, OK_ZFUSED, task(dLv, b, x, x, gate, gx, 0, 0, color + 1), gx * L.g.mz, sso);
    return;
  }
  const T *r = b;
  if (!zero) {
    const int gx = color_plane_blocks(L.g);
    vs.add(k0, OK_RESC, task(dLv, x, b, res, gate, gx, 1, color), gx * (L.g.mz - 2));
    r = res;
  }
  const int gx = f32 ? solve_tiles_x<kSolveTW32>(L.g, color) : solve_tiles_x<kSolveTW64>(L.g, color);
  (void)SW;
  vs.add(k1, solve_kind(L), task(dLv, r, zero ? nullptr : x, x, gate, gx, 0, 0, color + 1 + (zero ? 0 : 16)),
         gx * L.g.mz, sso);
}

template <typename T>
static void gen_vcycle(VSink &vs, cvb_ctx *ctx, const LevelDev *dLs, int l, int depth, const T *b, T *out,
                       const cvb_solve_opts &o, const int *gate);

// One zebra sweep (both colours) on x: the out-of-place one-kernel form through
// tmp (x -> tmp -> x) where the set-up chose it for a level with cross terms,
// else two half-sweeps.  ka/kb: the keys of the two colours' residual and solve.
template <typename T>
static void gen_zebra_sweep(VSink &vs, long long ka0, long long ka1, long long kb0, long long kb1, LevelDev &L,
                            const LevelDev *dLv, const T *b, T *x, T *tmp, bool zero_first, const int *gate) {
  const bool f32 = sizeof(T) == 4;
  const size_t sso = f32 ? line_solve_smem<float, kSolveTW32>(L.g) : line_solve_smem<double, kSolveTW64>(L.g);
  const bool fuse = f32 ? L.zfuse32 != 0 : L.zfuse64 != 0;
  if (!zero_first && fuse && !zebra_fusable<T>(L) && L.g.my <= 400 && sso <= 200 * 1024) {
    const int g0 = f32 ? solve_tiles_x<kSolveTW32>(L.g, 0) : solve_tiles_x<kSolveTW64>(L.g, 0);
    const int g1 = f32 ? solve_tiles_x<kSolveTW32>(L.g, 1) : solve_tiles_x<kSolveTW64>(L.g, 1);
    vs.add(ka1, OK_ZFUSED, task(dLv, b, x, tmp, gate, g0, 0, 0, 1), g0 * L.g.mz, sso);
    vs.add(kb1, OK_ZFUSED, task(dLv, b, tmp, x, gate, g1, 0, 0, 2), g1 * L.g.mz, sso);
    return;
  }
  gen_zebra_half<T>(vs, ka0, ka1, L, dLv, b, x, 0, zero_first, gate);
  gen_zebra_half<T>(vs, kb0, kb1, L, dLv, b, x, 1, false, gate);
}

template <typename T>
static void gen_vcycle_zebra(VSink &vs, cvb_ctx *ctx, const LevelDev *dLs, int l, int depth, const T *b, T *x,
                             const cvb_solve_opts &o, const int *gate) {
  LevelDev &L = ctx->L[l], &C = ctx->L[l - 1];
  const LevelDev *dLv = dLs + l;
  const size_t n = L.g.n();
  vs.add(key_desc(depth, 0), OK_ZERO, task(dLv, nullptr, nullptr, x, gate, elem_blocks(n), 0, (int)n),
         elem_blocks(n));
  T *tmp = lvec<T>(L, 2);
  const int pre = std::max(o.pre_sweeps, 1);
  for (int q = 0; q < pre; q++)
    gen_zebra_sweep<T>(vs, key_desc(depth, 1 + 10 * q), key_desc(depth, 2 + 10 * q), key_desc(depth, 4 + 10 * q),
                       key_desc(depth, 5 + 10 * q), L, dLv, b, x, tmp, q == 0, gate);
  T *res = lvec<T>(L, 3);
  add_residual<T>(vs, key_desc(depth, 100), L, dLv, x, b, res, gate);
  T *bc = lvec<T>(C, 0), *ec = lvec<T>(C, 1);
  const int cgx = plane_blocks(C.g);
  vs.add(key_desc(depth, 101), OK_RESTRICT, task(dLv, res, nullptr, bc, gate, cgx, 1), cgx * C.g.mz);
  gen_vcycle<T>(vs, ctx, dLs, l - 1, depth + 1, bc, ec, o, gate);
  vs.add(key_asc(depth, 0), OK_PROLONG, task(dLv, ec, nullptr, x, gate, plane_blocks(L.g), 1),
         plane_blocks(L.g) * L.g.mz);
  for (int q = 0; q < o.post_sweeps; q++)
    gen_zebra_sweep<T>(vs, key_asc(depth, 1 + 10 * q), key_asc(depth, 2 + 10 * q), key_asc(depth, 4 + 10 * q),
                       key_asc(depth, 5 + 10 * q), L, dLv, b, x, tmp, false, gate);
}

template <typename T>
static void gen_vcycle(VSink &vs, cvb_ctx *ctx, const LevelDev *dLs, int l, int depth, const T *b, T *out,
                       const cvb_solve_opts &o, const int *gate) {
  if (l == 0) {
    vs.add(key_coarse(), OK_DENSE, task(dLs, b, ctx->Minv, out, gate, 0, 0, ctx->ncoarse), nblk(ctx->ncoarse, 8));
    return;
  }
  if (o.smoother == CVB_SMOOTHER_ZEBRA) {
    gen_vcycle_zebra<T>(vs, ctx, dLs, l, depth, b, out, o, gate);
    return;
  }
  LevelDev &L = ctx->L[l], &C = ctx->L[l - 1];
  const LevelDev *dLv = dLs + l;
  T *x = out, *x2 = lvec<T>(L, 2);
  if (x2 == b) x2 = lvec<T>(L, 1);
  const int pre = std::max(o.pre_sweeps, 1);
  for (int q = 0; q < pre; q++) {
    gen_sweep<T>(vs, key_desc(depth, 2 * q), key_desc(depth, 2 * q + 1), L, dLv, b, q == 0 ? nullptr : x, x2,
                 q == 0, gate);
    std::swap(x, x2);
  }
  T *res = lvec<T>(L, 3);
  add_residual<T>(vs, key_desc(depth, 100), L, dLv, x, b, res, gate);
  T *bc = lvec<T>(C, 0), *ec = lvec<T>(C, 1);
  const int cgx = plane_blocks(C.g);
  vs.add(key_desc(depth, 101), OK_RESTRICT, task(dLv, res, nullptr, bc, gate, cgx, 1), cgx * C.g.mz);
  gen_vcycle<T>(vs, ctx, dLs, l - 1, depth + 1, bc, ec, o, gate);
  vs.add(key_asc(depth, 0), OK_PROLONG, task(dLv, ec, nullptr, x, gate, plane_blocks(L.g), 1),
         plane_blocks(L.g) * L.g.mz);
  for (int q = 0; q < o.post_sweeps; q++) {
    gen_sweep<T>(vs, key_asc(depth, 1 + 2 * q), key_asc(depth, 2 + 2 * q), L, dLv, b, x, x2, false, gate);
    std::swap(x, x2);
  }
  if (x != out) {
    size_t n = L.g.n();
    vs.add(key_asc(depth, 200), OK_COPY, task(dLv, x, nullptr, out, gate, elem_blocks(n), 0, (int)n),
           elem_blocks(n));
  }
}

// Launches every op of a keyed program in key order.
static void run_program(cvb_batch *bt, std::map<long long, std::array<Lists, OK_COUNT>> &prog, bool f32) {
  cudaStream_t s = bt->stream;
  const float w32 = (float)bt->opts.omega;
  const double w64 = bt->opts.omega;
  for (auto &kv : prog) {
    for (int k = 0; k < OK_COUNT; k++) {
      for (OpBatch &ob : kv.second[k].v) {
        switch (k) {
          case OK_RES32: glaunch_residual32(ob.tl, s); break;
          case OK_RES64: glaunch_residual64(ob.tl, s); break;
          case OK_RESTRICT: glaunch_restrict(ob.tl, f32, s); break;
          case OK_PROLONG: glaunch_prolong(ob.tl, f32, s); break;
          case OK_SWEEP: glaunch_line_sweep(ob.tl, f32, w32, w64, ob.smem, s); break;
          case OK_SOLVE: glaunch_line_solve(ob.tl, f32, w32, w64, ob.smem, 0, s); break;
          case OK_SOLVE_R1: glaunch_line_solve(ob.tl, f32, w32, w64, ob.smem, 1, s); break;
          case OK_SOLVE_R2: glaunch_line_solve(ob.tl, f32, w32, w64, ob.smem, 2, s); break;
          case OK_SOLVE_R4: glaunch_line_solve(ob.tl, f32, w32, w64, ob.smem, 4, s); break;
          case OK_SOLVE_R8: glaunch_line_solve(ob.tl, f32, w32, w64, ob.smem, 8, s); break;
          case OK_DENSE: glaunch_dense(ob.tl, f32, s); break;
          case OK_COPY: glaunch_elementwise(ob.tl, f32 ? 0 : 1, s); break;
          case OK_CONV: glaunch_elementwise(ob.tl, 2, s); break;
          case OK_WIDEN: glaunch_elementwise(ob.tl, 3, s); break;
          case OK_ZERO: glaunch_zero(ob.tl, f32, s); break;
          case OK_RESC: glaunch_resid_color(ob.tl, f32, s); break;
          case OK_ZFUSED: glaunch_zebra_fused(ob.tl, f32, w32, w64, ob.smem, s); break;
          default: break;
        }
      }
    }
  }
}

// The V-cycles of one round.  In mixed precision they read each problem's FP32
// input and write its FP32 output, whatever its Krylov index, so the round's
// V-cycle program depends only on which problems iterate: it is captured in a
// CUDA graph and replayed while that set stays the same.  A set's first round
// runs the launches eagerly (kernel attributes are set outside any capture), its
// second captures them -- updating the previous graph in place when the launch
// structure is the same, instantiating a new one otherwise -- and every round
// from the second on launches the graph alone.  FP64 rounds (whose V-cycles
// read V_j and write Z_j) run eagerly.  A capture the runtime refuses turns the
// graphs off for the batch; the launches then run eagerly, with the same result.
static void run_vcycles(cvb_batch *bt, std::map<long long, std::array<Lists, OK_COUNT>> &prog, bool f32,
                        const std::vector<Prob *> &iterating) {
  cudaStream_t s = bt->stream;
  if (!f32 || !bt->graphs || s == nullptr) {
    run_program(bt, prog, f32);
    return;
  }
  std::vector<unsigned long long> key;
  key.reserve(2 * iterating.size());
  for (Prob *p : iterating) {
    key.push_back((unsigned long long)p->slot);
    key.push_back(p->ctx->setup_id);
  }
  if (key != bt->vkey) {
    bt->vkey.swap(key);
    bt->vkey_rounds = 0;
    bt->vexec_ok = false;
  }
  if (++bt->vkey_rounds == 1) {
    run_program(bt, prog, f32);
    return;
  }
  if (!bt->vexec_ok) {
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
      run_program(bt, prog, f32);
      e = cudaStreamEndCapture(s, &graph);
    }
    if (e == cudaSuccess && graph && bt->vexec) {
      cudaGraphExecUpdateResultInfo info;
      if (cudaGraphExecUpdate(bt->vexec, graph, &info) == cudaSuccess) {
        bt->graph_updates++;
      } else {
        cudaGetLastError();
        cudaGraphExecDestroy(bt->vexec);
        bt->vexec = nullptr;
      }
    }
    if (e == cudaSuccess && graph && !bt->vexec) {
      e = cudaGraphInstantiate(&bt->vexec, graph, 0);
      if (e == cudaSuccess) bt->graph_captures++;
      else bt->vexec = nullptr;
    }
    if (graph) cudaGraphDestroy(graph);
    if (e != cudaSuccess || !bt->vexec) {
      cudaGetLastError();
      bt->graphs = false;
      run_program(bt, prog, f32);
      return;
    }
    bt->vexec_ok = true;
  }
  cudaGraphLaunch(bt->vexec, s);
  count_launch();
  bt->graph_replays++;
}

// ------------------------------------------------------------ Krylov rounds
static BProblem *dprob(cvb_batch *bt, int slot) { return bt->dP + slot; }
static KState *dks(cvb_batch *bt, int slot) { return bt->dK + slot; }
static BFlags *dfl(cvb_batch *bt, int slot) { return bt->dF + slot; }
static const LevelDev *dlev(cvb_batch *bt, int slot) { return bt->dL + (size_t)slot * kMaxLevels; }
static size_t fine_cells(cvb_ctx *c) { return c->L[c->nlevels - 1].g.n(); }

// Multidot tasks of w with V[0..nv) (+ w.w into self_row when self_row >= 0).
static void add_multidot(Lists &ls, const Prob &p, const double *w, int nv, int self_row, const int *gate) {
  const int nb = batch_reduce_blocks(fine_cells(p.ctx));
  if (nv == 0) {
    ls.add(task(nullptr, w, nullptr, nullptr, gate, 0, 0, p.slot, 0, self_row), nb);
    return;
  }
  for (int base = 0; base < nv; base += 8) {
    int cnt = std::min(8, nv - base);
    ls.add(task(nullptr, w, nullptr, nullptr, gate, 0, 0, p.slot, base | (cnt << 8), base == 0 ? self_row : -1), nb);
  }
}
static void add_finish(Lists &ls, const Prob &p, int row0, int rows, const int *gate) {
  ls.add(task(nullptr, nullptr, nullptr, nullptr, gate, rows, 0, p.slot, row0), rows);
}
static void launch_lists(Lists &ls, void (*fn)(const TaskList &, const BProblem *, cudaStream_t), cvb_batch *bt) {
  for (OpBatch &ob : ls.v) fn(ob.tl, bt->dP, bt->stream);
}
static void launch_lists2(Lists &ls, void (*fn)(const TaskList &, cudaStream_t), cvb_batch *bt) {
  for (OpBatch &ob : ls.v) fn(ob.tl, bt->stream);
}
template <typename L>
static void chunked(const std::vector<int> &slots, L &&fn) {
  for (size_t i = 0; i < slots.size(); i += kMaxTasks) {
    size_t e = std::min(slots.size(), i + (size_t)kMaxTasks);
    fn(i, e);
  }
}
static void launch_probs(cvb_batch *bt, const std::vector<int> &slots,
                         void (*fn)(const ProbList &, const BProblem *, cudaStream_t)) {
  chunked(slots, [&](size_t i, size_t e) {
    ProbList pl;
    pl.n = (int)(e - i);
    for (size_t q = i; q < e; q++) pl.idx[q - i] = slots[q];
    fn(pl, bt->dP, bt->stream);
  });
}

// Admission: device mirrors of the problem's levels and pointers.
static int admit(cvb_batch *bt, Prob &p) {
  cvb_ctx *c = p.ctx;
  BTRY(cvb_ensure_basis(c, bt->m, bt->mixed));
  if (c->stream) BCK(cudaStreamSynchronize(c->stream));
  LevelDev lv[kMaxLevels];
  for (int l = 0; l < c->nlevels; l++) {
    lv[l] = c->L[l];
    lv[l].gate = &dfl(bt, p.slot)->gate;
  }
  BCK(cudaMemcpyAsync((void *)dlev(bt, p.slot), lv, sizeof(LevelDev) * c->nlevels, cudaMemcpyHostToDevice,
                      bt->stream));
  BProblem P;
  std::memset(&P, 0, sizeof P);
  P.n = fine_cells(c);
  P.nb = batch_reduce_blocks(P.n);
  P.b = c->b; P.x = c->x; P.w = c->w; P.r = c->r;
  P.V = c->dV; P.Z = c->dZ64;
  P.partial = c->partial; P.sums = c->sums;
  P.ks = dks(bt, p.slot); P.fl = dfl(bt, p.slot);
  P.F = dlev(bt, p.slot) + (c->nlevels - 1);
  P.aj = c->aj64[c->nlevels - 1];
  BCK(cudaMemcpyAsync(dprob(bt, p.slot), &P, sizeof P, cudaMemcpyHostToDevice, bt->stream));
  BFlags f;
  std::memset(&f, 0, sizeof f);
  f.gate = 1;
  f.notfin = 1;
  BCK(cudaMemcpyAsync(dfl(bt, p.slot), &f, sizeof f, cudaMemcpyHostToDevice, bt->stream));
  if (p.host_b) BCK(cudaMemcpyAsync(c->b, p.host_b, sizeof(double) * P.n, cudaMemcpyHostToDevice, bt->stream));
  if (!p.warm) BCK(cudaMemsetAsync(c->x, 0, sizeof(double) * P.n, bt->stream));
  // (copies from pageable memory are staged before cudaMemcpyAsync returns)
  return CVB_OK;
}

// One round: start new problems, close finished cycles, one iteration for all.
static int issue_round(cvb_batch *bt, std::vector<Prob *> &starting, std::vector<Prob *> &closing,
                       std::vector<Prob *> &iterating) {
  cudaStream_t s = bt->stream;
  const bool f32 = bt->mixed;
  // --- starting: range projection, ||b||, tolerances
  if (!starting.empty()) {
    Lists ratio, fin01, rem, norm, finn;
    std::vector<int> proj_slots;
    InitList il;
    std::memset(&il, 0, sizeof il);
    for (Prob *p : starting) {
      const size_t n = fine_cells(p->ctx);
      const int nb = batch_reduce_blocks(n);
      const int *nog = nullptr;
      if (p->project) {
        ratio.add(task(nullptr, nullptr, nullptr, nullptr, nog, 0, 0, p->slot), nb);
        add_finish(fin01, *p, 0, 2, nog);
        rem.add(task(nullptr, nullptr, nullptr, nullptr, nog, elem_blocks(n), 0, p->slot), elem_blocks(n));
        proj_slots.push_back(p->slot);
      }
      add_multidot(norm, *p, p->ctx->b, 0, kNormRow, nog);
      add_finish(finn, *p, kNormRow, 1, nog);
    }
    launch_lists(ratio, glaunch_fluid_ratio, bt);
    launch_lists(fin01, glaunch_finish, bt);
    launch_lists(rem, glaunch_remove_aj_mean, bt);
    launch_probs(bt, proj_slots, launch_k_removed);
    launch_lists(norm, glaunch_multidot, bt);
    launch_lists(finn, glaunch_finish, bt);
    for (size_t i = 0; i < starting.size(); i += kMaxTasks) {
      size_t e = std::min(starting.size(), i + (size_t)kMaxTasks);
      il.n = (int)(e - i);
      for (size_t q = i; q < e; q++) {
        Prob *p = starting[q];
        il.idx[q - i] = p->slot;
        il.m[q - i] = bt->m;
        il.max_it[q - i] = p->max_it;
        il.rtol[q - i] = p->rtol;
        il.atol[q - i] = p->atol;
      }
      launch_k_init(il, bt->dP, s);
    }
  }
  // --- closing: y = R^-1 g, x += Z y
  if (!closing.empty()) {
    std::vector<int> slots;
    Lists upd;
    for (Prob *p : closing) {
      slots.push_back(p->slot);
      size_t n = fine_cells(p->ctx);
      upd.add(task(nullptr, nullptr, nullptr, nullptr, &dfl(bt, p->slot)->fin, elem_blocks(n), 0, p->slot),
              elem_blocks(n));
    }
    launch_probs(bt, slots, launch_k_solve_y);
    launch_lists(upd, glaunch_update, bt);
  }
  // --- (re)start of a cycle: r = b - A x, beta, V0; null space on finished ones
  std::vector<Prob *> restart(starting);
  restart.insert(restart.end(), closing.begin(), closing.end());
  if (!restart.empty()) {
    Lists res, norm, finn, scale, fsum, fin01, addc;
    std::vector<int> slots;
    for (Prob *p : restart) {
      cvb_ctx *c = p->ctx;
      LevelDev &F = c->L[c->nlevels - 1];
      const size_t n = F.g.n();
      const int *gfin = &dfl(bt, p->slot)->fin, *ggate = &dfl(bt, p->slot)->gate,
                *gnot = &dfl(bt, p->slot)->notfin;
      const int gx = plane_blocks(F.g);
      res.add(task(dlev(bt, p->slot) + (c->nlevels - 1), c->x, c->b, c->r, gfin, gx, 1), gx * F.g.mz);
      add_multidot(norm, *p, c->r, 0, kNormRow, gfin);
      add_finish(finn, *p, kNormRow, 1, gfin);
      scale.add(task(nullptr, c->r, &dks(bt, p->slot)->beta, c->V[0], ggate, elem_blocks(n), 0, (int)n),
                elem_blocks(n));
      fsum.add(task(nullptr, nullptr, nullptr, nullptr, gnot, 0, 0, p->slot), batch_reduce_blocks(n));
      add_finish(fin01, *p, 0, 2, gnot);
      addc.add(task(nullptr, nullptr, nullptr, nullptr, gnot, elem_blocks(n), 0, p->slot), elem_blocks(n));
      slots.push_back(p->slot);
    }
    launch_lists2(res, glaunch_residual64, bt);
    launch_lists(norm, glaunch_multidot, bt);
    launch_lists(finn, glaunch_finish, bt);
    launch_probs(bt, slots, launch_k_cycle_start);
    launch_lists2(scale, glaunch_scale, bt);
    launch_lists(fsum, glaunch_fluid_sum, bt);
    launch_lists(fin01, glaunch_finish, bt);
    launch_lists(addc, glaunch_add_fluid_const, bt);
  }
  // --- one FGMRES iteration for every iterating problem
  if (!iterating.empty()) {
    std::map<long long, std::array<Lists, OK_COUNT>> prog;
    VSink vs{&prog};
    Lists conv, widen, apply, mdot, fin, maxpy, finn, scale;
    std::vector<int> slots;
    for (Prob *p : iterating) {
      cvb_ctx *c = p->ctx;
      const int j = p->host_j;
      const int nl = c->nlevels;
      LevelDev &F = c->L[nl - 1];
      const size_t n = F.g.n();
      const int *gate = &dfl(bt, p->slot)->gate;
      const LevelDev *dLs = dlev(bt, p->slot);
      if (f32) {
        conv.add(task(nullptr, c->V[j], nullptr, c->b32, gate, elem_blocks(n), 0, (int)n), elem_blocks(n));
        gen_vcycle<float>(vs, c, dLs, nl - 1, 0, c->b32, c->Z32[0], bt->opts, gate);
        widen.add(task(nullptr, c->Z32[0], nullptr, c->Z64[j], gate, elem_blocks(n), 0, (int)n), elem_blocks(n));
      } else {
        gen_vcycle<double>(vs, c, dLs, nl - 1, 0, c->V[j], c->Z64[j], bt->opts, gate);
      }
      const int gx = plane_blocks(F.g);
      apply.add(task(dLs + (nl - 1), c->Z64[j], nullptr, c->w, gate, gx, 1), gx * F.g.mz);
      add_multidot(mdot, *p, c->w, j + 1, j + 1, gate);
      add_finish(fin, *p, 0, j + 2, gate);
      maxpy.add(task(nullptr, nullptr, nullptr, nullptr, gate, 0, 0, p->slot, j + 1), batch_reduce_blocks(n));
      add_finish(finn, *p, kNormRow, 1, gate);
      scale.add(task(nullptr, c->w, &dks(bt, p->slot)->hn, c->V[j + 1], gate, elem_blocks(n), 0, (int)n),
                elem_blocks(n));
      slots.push_back(p->slot);
    }
    for (OpBatch &ob : conv.v) glaunch_elementwise(ob.tl, 2, s);
    run_vcycles(bt, prog, f32, iterating);
    for (OpBatch &ob : widen.v) glaunch_elementwise(ob.tl, 3, s);
    launch_lists2(apply, glaunch_residual64, bt);
    launch_lists(mdot, glaunch_multidot, bt);
    launch_lists(fin, glaunch_finish, bt);
    launch_lists(maxpy, glaunch_multiaxpy_norm, bt);
    launch_lists(finn, glaunch_finish, bt);
    launch_probs(bt, slots, launch_k_arnoldi);
    launch_lists2(scale, glaunch_scale, bt);
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return bfail(bt, CVB_CUDA_ERROR, "round launch: %s", cudaGetErrorString(e));
  return CVB_OK;
}

static void record_done(cvb_batch *bt, Prob &p, const BFlags &f) {
  Done d;
  d.ticket = p.ticket;
  d.ctx = p.ctx;
  std::memset(&d.st, 0, sizeof d.st);
  d.st.status = f.status;
  d.st.iterations = f.iters;
  d.st.restarts = f.cycles > 0 ? f.cycles - 1 : 0;
  d.st.rel_residual = f.rel;
  d.st.abs_residual = f.abs;
  d.st.rhs_norm = f.bnorm;
  d.st.rhs_projected = f.removed;
  bt->done.push_back(d);
  bt->free_slots.push_back(p.slot);
}

// One step: admit, issue a round, read the previous round's flags.
static int step(cvb_batch *bt) {
  std::vector<Prob *> starting, closing, iterating;
  while (!bt->pending.empty() && !bt->free_slots.empty()) {
    Prob p = bt->pending.front();
    p.slot = bt->free_slots.back();
    int rc = admit(bt, p);
    if (rc != CVB_OK) return rc;
    bt->pending.pop_front();
    bt->free_slots.pop_back();
    p.state = P_NEW;
    bt->active.push_back(p);
  }
  const long long R = bt->round;
  for (Prob &p : bt->active) {
    if (p.state == P_NEW) {
      starting.push_back(&p);
      p.first_round = R;
    } else if (p.close_next || p.host_j >= bt->m || (p.issued >= p.issue_cap && p.host_j > 0)) {
      closing.push_back(&p);
    }
  }
  for (Prob *p : starting) { p->state = P_ITER; p->host_j = 0; }
  for (Prob *p : closing) { p->host_cycle++; p->host_j = 0; p->close_next = false; }
  for (Prob &p : bt->active)
    if (p.state == P_ITER && p.issued < p.issue_cap) iterating.push_back(&p);
  BTRY(issue_round(bt, starting, closing, iterating));
  for (Prob *p : iterating) { p->host_j++; p->issued++; }
  // this round's flags into the pinned buffer of its parity
  const int cur = (int)(R & 1);
  int nslot = 0;
  for (Prob &p : bt->active) nslot = std::max(nslot, p.slot + 1);
  bt->hF_slots[cur] = nslot;
  if (nslot) BCK(cudaMemcpyAsync(bt->hF[cur], bt->dF, sizeof(BFlags) * nslot, cudaMemcpyDeviceToHost, bt->stream));
  BCK(cudaEventRecord(bt->ev[cur], bt->stream));
  bt->round = R + 1;
  // the previous round's flags (that round has completed once its event has)
  if (R >= 1) {
    const int prev = cur ^ 1;
    BCK(cudaEventSynchronize(bt->ev[prev]));
    std::vector<Prob> keep;
    keep.reserve(bt->active.size());
    for (Prob &p : bt->active) {
      if (p.first_round > R - 1 || p.slot >= bt->hF_slots[prev]) { keep.push_back(p); continue; }
      const BFlags &f = bt->hF[prev][p.slot];
      if (f.fin) {
        record_done(bt, p, f);
        continue;
      }
      if (f.gate && f.cycles == p.host_cycle) p.close_next = true;
      if (p.issued >= p.issue_cap && !f.fin && p.host_j == 0 && f.cycles == p.host_cycle && !f.gate) {
        // the device keeps restarting without spending iterations: give up
        BFlags g = f;
        g.status = CVB_NOT_CONVERGED;
        record_done(bt, p, g);
        continue;
      }
      keep.push_back(p);
    }
    bt->active.swap(keep);
  }
  return CVB_OK;
}

static void destroy(cvb_batch *bt) {
  if (!bt) return;
  if (bt->stream) cudaStreamSynchronize(bt->stream);
  cudaFree(bt->dP);
  cudaFree(bt->dK);
  cudaFree(bt->dF);
  cudaFree(bt->dL);
  for (int q = 0; q < 2; q++) {
    if (bt->hF[q]) cudaFreeHost(bt->hF[q]);
    if (bt->ev[q]) cudaEventDestroy(bt->ev[q]);
  }
  if (bt->vexec) cudaGraphExecDestroy(bt->vexec);
  if (bt->copy_stream) cudaStreamDestroy(bt->copy_stream);
  if (bt->own_stream && bt->stream) cudaStreamDestroy(bt->stream);
  delete bt;
}

// ------------------------------------------------------------------ C ABI
extern "C" {

int cvb_batch_create(cvb_batch **out, const cvb_options *opts, const cvb_solve_opts *so) {
  if (!out) return CVB_BAD_INPUT;
  *out = nullptr;
  cvb_batch *bt = new cvb_batch();
  bt->device = opts ? opts->device : 0;
  cvb_solve_opts_default(&bt->opts);
  if (so) bt->opts = *so;
  const cvb_solve_opts &o = bt->opts;
  if (o.restart < 1 || o.restart > kBatchRestart || o.max_it < 0 || o.pre_sweeps < 0 || o.post_sweeps < 0 ||
      (o.precision != CVB_PRECISION_FP64 && o.precision != CVB_PRECISION_MIXED) ||
      (o.smoother != CVB_SMOOTHER_JACOBI && o.smoother != CVB_SMOOTHER_ZEBRA)) {
    delete bt;
    return CVB_BAD_INPUT;
  }
  bt->mixed = o.precision == CVB_PRECISION_MIXED;
  bt->m = o.restart;
  auto bad = [&](cudaError_t e) {
    if (e == cudaSuccess) return false;
    destroy(bt);
    return true;
  };
  if (bad(cudaSetDevice(bt->device))) return CVB_CUDA_ERROR;
  if (opts && opts->stream) {
    bt->stream = (cudaStream_t)opts->stream;
  } else {
    if (bad(cudaStreamCreateWithFlags(&bt->stream, cudaStreamNonBlocking))) return CVB_CUDA_ERROR;
    bt->own_stream = true;
  }
  if (bad(cudaStreamCreateWithFlags(&bt->copy_stream, cudaStreamNonBlocking))) return CVB_CUDA_ERROR;
  if (bad(cudaMalloc(&bt->dP, sizeof(BProblem) * kMaxSlots))) return CVB_OOM;
  if (bad(cudaMalloc(&bt->dK, sizeof(KState) * kMaxSlots))) return CVB_OOM;
  if (bad(cudaMalloc(&bt->dF, sizeof(BFlags) * kMaxSlots))) return CVB_OOM;
  if (bad(cudaMalloc(&bt->dL, sizeof(LevelDev) * kMaxSlots * kMaxLevels))) return CVB_OOM;
  if (bad(cudaMemset(bt->dF, 0, sizeof(BFlags) * kMaxSlots))) return CVB_CUDA_ERROR;
  for (int q = 0; q < 2; q++) {
    if (bad(cudaMallocHost(&bt->hF[q], sizeof(BFlags) * kMaxSlots))) return CVB_OOM;
    if (bad(cudaEventCreateWithFlags(&bt->ev[q], cudaEventDisableTiming))) return CVB_CUDA_ERROR;
  }
  for (int q = kMaxSlots - 1; q >= 0; q--) bt->free_slots.push_back(q);
  *out = bt;
  return CVB_OK;
}

void cvb_batch_destroy(cvb_batch *bt) { destroy(bt); }

const char *cvb_batch_last_error(const cvb_batch *bt) { return bt ? bt->err.c_str() : "no batch"; }

int cvb_batch_submit(cvb_batch *bt, cvb_ctx *ctx, const double *host_b, double rtol, double atol, int max_it,
                     int warm_start, int project_rhs, int *ticket) {
  if (!bt) return CVB_BAD_INPUT;
  if (!ctx || !ctx->ready) return bfail(bt, CVB_NOT_SETUP, "context is not set up");
  if (ctx->device != bt->device) return bfail(bt, CVB_BAD_INPUT, "context is on device %d, batch on %d", ctx->device,
                                              bt->device);
  if (!ctx->coarse_dense)
    return bfail(bt, CVB_BAD_INPUT, "batched solves need a dense coarsest level (%d cells > coarse_dense_max)",
                 ctx->ncoarse);
  if (ctx->nlevels > kMaxLevels) return bfail(bt, CVB_BAD_INPUT, "more than %d levels", kMaxLevels);
  for (int l = 0; l < ctx->nlevels; l++)
    if (ctx->L[l].g.my > kMaxFusedRows)
      return bfail(bt, CVB_BAD_INPUT, "level %d has %d rows per y-line (batched limit %d)", l, ctx->L[l].g.my,
                   kMaxFusedRows);
  if (!(rtol >= 0) || !(atol >= 0) || max_it < 0) return bfail(bt, CVB_BAD_INPUT, "bad tolerances");
  for (const Prob &p : bt->active)
    if (p.ctx == ctx) return bfail(bt, CVB_BAD_INPUT, "context already has a solve in this batch");
  for (const Prob &p : bt->pending)
    if (p.ctx == ctx) return bfail(bt, CVB_BAD_INPUT, "context already has a solve in this batch");
  Prob p;
  p.ctx = ctx;
  p.ticket = bt->next_ticket++;
  p.warm = warm_start != 0;
  p.project = project_rhs != 0;
  p.rtol = rtol;
  p.atol = atol;
  p.max_it = max_it;
  p.issue_cap = max_it + 4 * (max_it / std::max(bt->m, 1) + 2) + 8;
  p.host_b = host_b;
  bt->pending.push_back(p);
  if (ticket) *ticket = p.ticket;
  return CVB_OK;
}

int cvb_batch_step(cvb_batch *bt, int *in_flight) {
  if (!bt) return CVB_BAD_INPUT;
  if (cudaSetDevice(bt->device) != cudaSuccess) return bfail(bt, CVB_CUDA_ERROR, "cudaSetDevice failed");
  int rc = CVB_OK;
  if (!bt->active.empty() || !bt->pending.empty()) rc = step(bt);
  if (in_flight) *in_flight = (int)(bt->active.size() + bt->pending.size());
  return rc;
}

int cvb_batch_poll(cvb_batch *bt, int *ticket, cvb_solve_stats *st) {
  if (!bt || !ticket) return CVB_BAD_INPUT;
  *ticket = -1;
  if (bt->done.empty()) return CVB_OK;
  Done d = bt->done.front();
  bt->done.pop_front();
  *ticket = d.ticket;
  if (st) *st = d.st;
  return CVB_OK;
}

int cvb_batch_read_phi(cvb_batch *bt, cvb_ctx *ctx, double *host_phi) {
  if (!bt || !ctx || !host_phi || !ctx->ready) return CVB_BAD_INPUT;
  size_t n = fine_cells(ctx);
  BCK(cudaMemcpyAsync(host_phi, ctx->x, sizeof(double) * n, cudaMemcpyDeviceToHost, bt->copy_stream));
  BCK(cudaStreamSynchronize(bt->copy_stream));
  return CVB_OK;
}

int cvb_batch_solve(cvb_batch *bt, int n, cvb_ctx *const *ctxs, cvb_solve_stats *stats) {
  if (!bt || n < 0 || (n > 0 && !ctxs)) return CVB_BAD_INPUT;
  if (!bt->active.empty() || !bt->pending.empty())
    return bfail(bt, CVB_BAD_INPUT, "cvb_batch_solve needs an idle batch");
  std::map<int, int> where;
  const cvb_solve_opts &o = bt->opts;
  for (int q = 0; q < n; q++) {
    int t = -1;
    BTRY(cvb_batch_submit(bt, ctxs[q], nullptr, o.rtol, o.atol, o.max_it, o.warm_start, o.project_rhs, &t));
    where[t] = q;
  }
  cudaEvent_t e0, e1;
  BCK(cudaEventCreate(&e0));
  BCK(cudaEventCreate(&e1));
  BCK(cudaEventRecord(e0, bt->stream));
  int left = n, worst = CVB_OK;
  long long guard = 0;
  while (left > 0) {
    int inflight = 0;
    BTRY(cvb_batch_step(bt, &inflight));
    int t;
    cvb_solve_stats st;
    while (cvb_batch_poll(bt, &t, &st) == CVB_OK && t >= 0) {
      auto it = where.find(t);
      if (it != where.end()) {
        if (stats) stats[it->second] = st;
        if (st.status != CVB_OK && worst == CVB_OK) worst = st.status;
        left--;
      }
    }
    if (++guard >= bt->round_limit && left > 0) {
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      return bfail(bt, CVB_TIMEOUT, "batch did not finish within %lld rounds; %d solves still in flight",
                   bt->round_limit, left);
    }
  }
  BCK(cudaEventRecord(e1, bt->stream));
  BCK(cudaEventSynchronize(e1));
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (stats)
    for (int q = 0; q < n; q++) stats[q].device_ms = ms;
  if (worst != CVB_OK) return bfail(bt, worst, "%s", "at least one solve of the batch did not converge");
  return CVB_OK;
}

int cvb_batch_set_round_limit(cvb_batch *bt, long long rounds) {
  if (!bt || rounds < 0) return CVB_BAD_INPUT;
  bt->round_limit = rounds == 0 ? kDefaultRoundLimit : rounds;
  return CVB_OK;
}

int cvb_batch_set_graphs(cvb_batch *bt, int on) {
  if (!bt) return CVB_BAD_INPUT;
  bt->graphs = on != 0;
  bt->vkey.clear();
  bt->vkey_rounds = 0;
  bt->vexec_ok = false;
  return CVB_OK;
}

int cvb_batch_graph_stats(const cvb_batch *bt, long long *captures, long long *updates, long long *replays) {
  if (!bt) return CVB_BAD_INPUT;
  if (captures) *captures = bt->graph_captures;
  if (updates) *updates = bt->graph_updates;
  if (replays) *replays = bt->graph_replays;
  return CVB_OK;
}

int cvb_batch_in_flight(const cvb_batch *bt) {
  return bt ? (int)(bt->active.size() + bt->pending.size()) : 0;
}

}  // extern "C"
