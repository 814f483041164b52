// Host side of the cvb C ABI (include/cvb.h): device residency of one CURVIB
// block's multigrid hierarchy, the V-cycle, FP64 FGMRES and the path's entry points.
#include "../../include/cvb.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <array>
#include <cctype>
#include <chrono>
#include <cstdarg>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "cvb_ctx.h"

using namespace cvb;

// ------------------------------------------------------------------ helpers
static int fail(cvb_ctx *c, int code, const char *fmt, ...) __attribute__((format(printf, 3, 4)));
static int fail(cvb_ctx *c, int code, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  if (c) c->err = buf;
  return code;
}

#define CK(call)                                                                               \
  do {                                                                                         \
    cudaError_t e_ = (call);                                                                   \
    if (e_ != cudaSuccess)                                                                     \
      return fail(ctx, e_ == cudaErrorMemoryAllocation ? CVB_OOM : CVB_CUDA_ERROR, "%s: %s (%s:%d)", \
                  #call, cudaGetErrorString(e_), __FILE__, __LINE__);                          \
  } while (0)

#define CKL()                                                                                  \
  do {                                                                                         \
    cudaError_t e_ = cudaGetLastError();                                                       \
    if (e_ != cudaSuccess)                                                                     \
      return fail(ctx, CVB_CUDA_ERROR, "kernel launch: %s (%s:%d)", cudaGetErrorString(e_), __FILE__, \
                  __LINE__);                                                                   \
  } while (0)

#define TRY(expr)                  \
  do {                             \
    int s_ = (expr);               \
    if (s_ != CVB_OK) return s_;   \
  } while (0)

// Per-problem device memory comes from the device's stream-ordered pool, kept
// cached (release threshold at its maximum, a setting of this process's pool
// only): evicting one problem and setting up the next reuse memory without a
// device-wide synchronisation.
static void ensure_pool(int dev) {
  static std::mutex mu;
  static bool done[64] = {};
  std::lock_guard<std::mutex> lock(mu);
  if (dev < 0 || dev >= 64 || done[dev]) return;
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
    uint64_t thr = UINT64_MAX;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
  }
  done[dev] = true;
}

template <typename T>
static int dalloc(cvb_ctx *ctx, T **p, size_t count) {
  *p = nullptr;
  if (count == 0) count = 1;
  if (ctx->device_limit && ctx->device_bytes + sizeof(T) * count > ctx->device_limit)
    return fail(ctx, CVB_OOM, "device allocation of %zu bytes exceeds the context's limit (%zu of %zu bytes in use)",
                sizeof(T) * count, ctx->device_bytes, ctx->device_limit);
  cudaError_t e = cudaMallocAsync((void **)p, sizeof(T) * count, ctx->stream);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(ctx, CVB_OOM, "device allocation of %zu bytes failed: %s", sizeof(T) * count,
                cudaGetErrorString(e));
  }
  ctx->allocs.push_back((void *)*p);
  ctx->alloc_bytes.push_back(sizeof(T) * count);
  ctx->device_bytes += sizeof(T) * count;
  return CVB_OK;
}

// Returns one per-problem allocation to the pool (in stream order).
static void dfree(cvb_ctx *ctx, void *p) {
  for (size_t q = 0; q < ctx->allocs.size(); q++)
    if (ctx->allocs[q] == p) {
      ctx->device_bytes -= ctx->alloc_bytes[q];
      ctx->allocs.erase(ctx->allocs.begin() + q);
      ctx->alloc_bytes.erase(ctx->alloc_bytes.begin() + q);
      break;
    }
  cudaFreeAsync(p, ctx->stream);
}

// Geometry arrays: plain allocations owned by the shared Geometry.
template <typename T>
static int galloc(cvb_ctx *ctx, Geometry &G, T **p, size_t count) {
  *p = nullptr;
  if (count == 0) count = 1;
  if (ctx->device_limit && G.bytes + sizeof(T) * count > ctx->device_limit)
    return fail(ctx, CVB_OOM, "grid allocation of %zu bytes exceeds the context's limit (%zu of %zu bytes in use)",
                sizeof(T) * count, (size_t)G.bytes, ctx->device_limit);
  cudaError_t e = cudaMalloc((void **)p, sizeof(T) * count);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(ctx, CVB_OOM, "cudaMalloc of %zu bytes failed: %s", sizeof(T) * count, cudaGetErrorString(e));
  }
  G.allocs.push_back((void *)*p);
  G.bytes += sizeof(T) * count;
  return CVB_OK;
}

void drop_vcycle_graphs(cvb_ctx *ctx);

static void free_all(cvb_ctx *ctx) {
  drop_vcycle_graphs(ctx);
  for (void *p : ctx->allocs) cudaFreeAsync(p, ctx->stream);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  ctx->allocs.clear();
  ctx->alloc_bytes.clear();
  ctx->device_bytes = 0;
  ctx->L.clear();
  ctx->H.clear();
  ctx->geo.reset();
  ctx->fm.clear();
  ctx->iaj.clear(); ctx->jaj.clear(); ctx->kaj.clear(); ctx->aj64.clear();
  ctx->area3 = nullptr;
  ctx->inv_aj = nullptr;
  ctx->cm[0] = ctx->cm[1] = ctx->cm[2] = nullptr;
  ctx->nvert_tmp = nullptr;
  ctx->Minv = nullptr;
  ctx->cidx = nullptr;
  ctx->b = ctx->x = ctx->w = ctx->r = nullptr;
  for (int q = 0; q <= kMaxRestart; q++) ctx->V[q] = nullptr;
  for (int q = 0; q < kMaxRestart; q++) { ctx->Z64[q] = nullptr; ctx->Z32[q] = nullptr; }
  ctx->b32 = nullptr;
  ctx->dV = nullptr; ctx->dZ64 = nullptr; ctx->dZ32 = nullptr;
  ctx->partial = ctx->sums = ctx->hdev = nullptr;
  ctx->uc_dev = ctx->p_dev = nullptr;
  ctx->ucat_dev = ctx->ubcs_dev = nullptr;
  ctx->conv_dev = ctx->conv_fp = nullptr;
  ctx->visc_dev = ctx->rct_dev = ctx->rhs_dev = ctx->uo_dev = ctx->urm_dev = ctx->pu_dev = nullptr;
  ctx->imp_norms = nullptr;
  ctx->bc_scratch = nullptr;
  if (ctx->bc_host) cudaFreeHost(ctx->bc_host);
  ctx->bc_host = nullptr;
  ctx->ibm_cent = nullptr;
  ctx->ready = false;
}

// Copy the owned box [0,mx)x[0,my)x[0,mz) out of a ghosted local array.
static void extract_box(const cvb_level_desc &d, const double *src, int dof, std::vector<double> &out) {
  size_t n = (size_t)d.mx * d.my * d.mz;
  out.resize(n * dof);
  for (int k = 0; k < d.mz; k++)
    for (int j = 0; j < d.my; j++) {
      const double *row = src + (((size_t)(k - d.gzs) * d.gym + (j - d.gys)) * d.gxm + (0 - d.gxs)) * dof;
      std::memcpy(&out[((size_t)k * d.my + j) * d.mx * dof], row, sizeof(double) * d.mx * dof);
    }
}

// The owned box of an array: the array itself when its ghosted box is the owned
// box (no copy), else extracted into `scratch`.
static const double *box_view(const cvb_level_desc &d, const double *src, int dof, std::vector<double> &scratch) {
  if (d.gxs == 0 && d.gys == 0 && d.gzs == 0 && d.gxm == d.mx && d.gym == d.my && d.gzm == d.mz) return src;
  extract_box(d, src, dof, scratch);
  return scratch.data();
}

static int upload_box(cvb_ctx *ctx, Geometry &G, const cvb_level_desc &d, const double *src, int dof,
                      double **dst) {
  std::vector<double> h;
  const double *v = box_view(d, src, dof, h);
  const size_t count = (size_t)d.mx * d.my * d.mz * dof;
  TRY(galloc(ctx, G, dst, count));
  CK(cudaMemcpyAsync(*dst, v, sizeof(double) * count, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return CVB_OK;
}

static int check_desc(cvb_ctx *ctx, const cvb_level_desc &d, int level, bool finest) {
  if (d.mx < 3 || d.my < 3 || d.mz < 3) return fail(ctx, CVB_BAD_INPUT, "level %d: box %dx%dx%d too small", level, d.mx, d.my, d.mz);
  if ((long long)d.mx * d.my * d.mz >= (1LL << 31))
    return fail(ctx, CVB_BAD_INPUT, "level %d: box %dx%dx%d holds 2^31 cells or more", level, d.mx, d.my, d.mz);
  if (d.gxs > 0 || d.gys > 0 || d.gzs > 0 || d.gxs + d.gxm < d.mx || d.gys + d.gym < d.my || d.gzs + d.gzm < d.mz)
    return fail(ctx, CVB_BAD_INPUT, "level %d: ghosted box does not cover the owned box", level);
  const double *req[] = {d.icsi, d.ieta, d.izet, d.jcsi, d.jeta, d.jzet, d.kcsi, d.keta, d.kzet, d.iaj, d.jaj, d.kaj, d.aj};
  for (const double *p : req)
    if (!p) return fail(ctx, CVB_BAD_INPUT, "level %d: a metric array is NULL", level);
  if (finest && (!d.csi || !d.eta || !d.zet)) return fail(ctx, CVB_BAD_INPUT, "finest level needs lCsi/lEta/lZet");
  for (int a = 0; a < 3; a++) {
    bool p0 = d.bctype[2 * a] == 7, p1 = d.bctype[2 * a + 1] == 7;
    if (p0 != p1) return fail(ctx, CVB_BAD_INPUT, "level %d: direction %d is periodic on one side only", level, a);
    int m = a == 0 ? d.mx : (a == 1 ? d.my : d.mz);
    if (p0 && m - 2 < 3) return fail(ctx, CVB_BAD_INPUT, "level %d: periodic direction %d needs >= 3 cells", level, a);
  }
  return CVB_OK;
}

// Largest coarsest box (ring included) solved by a dense inverse unless the
// options say otherwise: 18^3 = 5832 holds a 16^3-cell coarsest level.
constexpr int kCoarseDenseMaxDefault = 6000;
// Largest coarsest block inverted on the host; larger ones go to the device.
constexpr int kHostInverseMax = 384;

// Gauss-Jordan inverse with partial pivoting (coarsest level, n <= kHostInverseMax).
static bool dense_inverse(std::vector<double> &A, int n, std::vector<double> &Inv) {
  Inv.assign((size_t)n * n, 0.0);
  for (int i = 0; i < n; i++) Inv[(size_t)i * n + i] = 1.0;
  for (int c = 0; c < n; c++) {
    int piv = c;
    double best = std::fabs(A[(size_t)c * n + c]);
    for (int r = c + 1; r < n; r++) {
      double v = std::fabs(A[(size_t)r * n + c]);
      if (v > best) { best = v; piv = r; }
    }
    if (!(best > 0.0)) return false;
    if (piv != c) {
      for (int q = 0; q < n; q++) {
        std::swap(A[(size_t)c * n + q], A[(size_t)piv * n + q]);
        std::swap(Inv[(size_t)c * n + q], Inv[(size_t)piv * n + q]);
      }
    }
    double inv = 1.0 / A[(size_t)c * n + c];
    for (int q = 0; q < n; q++) { A[(size_t)c * n + q] *= inv; Inv[(size_t)c * n + q] *= inv; }
    for (int r = 0; r < n; r++) {
      if (r == c) continue;
      double f = A[(size_t)r * n + c];
      if (f == 0.0) continue;
      double *ar = &A[(size_t)r * n], *ac = &A[(size_t)c * n];
      double *ir = &Inv[(size_t)r * n], *ic = &Inv[(size_t)c * n];
      for (int q = 0; q < n; q++) { ar[q] -= f * ac[q]; ir[q] -= f * ic[q]; }
    }
  }
  return true;
}

// Rows of the coarsest operator, made nonsingular: M = A + sum_r u_r v_r^T with
// v_r the indicator of fluid region r and u_r = s v_r.  A's left null vector on
// region r is 1/aj there, which is not orthogonal to u_r, so M is invertible; for a
// compatible right-hand side M^-1 b solves A e = b with zero region sums of e.
// The ring and the blocked cells are identity rows, so only the fluid block is
// inverted (e = r elsewhere) -- unless a fluid row couples to a non-fluid cell,
// in which case the whole box is.  cidx lists the inverted cells first.
static int build_coarse(cvb_ctx *ctx, const cvb_solve_opts *opt) {
  LevelDev &C = ctx->L[0];
  size_t n = C.g.n();
  ctx->ncoarse = (int)n;
  int dense_max = opt ? opt->coarse_dense_max : kCoarseDenseMaxDefault;
  ctx->coarse_dense = (int)n <= dense_max;
  if (!ctx->coarse_dense) return CVB_OK;
  std::vector<double> w(n * NSLOT), nv(n);
  CK(cudaMemcpyAsync(w.data(), C.w64, sizeof(double) * n * NSLOT, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaMemcpyAsync(nv.data(), C.nvert, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  const Geom &g = C.g;
  std::vector<int> region(n, -1), cols(n * NSLOT);
  std::vector<char> fluid(n, 0);
  for (int k = 0; k < g.mz; k++)
    for (int j = 0; j < g.my; j++)
      for (int i = 0; i < g.mx; i++) {
        size_t p = g.id(i, j, k);
        bool interior = i >= 1 && i <= g.mx - 2 && j >= 1 && j <= g.my - 2 && k >= 1 && k <= g.mz - 2;
        if (!interior || nv[p] > 0.1) continue;
        fluid[p] = 1;
        int iu = g.iu(i), id = g.id_(i), ju = g.ju(j), jd = g.jd(j), ku = g.ku(k), kd = g.kd(k);
        size_t c[NSLOT] = {g.id(i, j, k), g.id(iu, j, k), g.id(id, j, k), g.id(i, ju, k), g.id(i, jd, k),
                           g.id(i, j, ku), g.id(i, j, kd), g.id(iu, ju, k), g.id(iu, jd, k), g.id(id, ju, k),
                           g.id(id, jd, k), g.id(i, ju, ku), g.id(i, ju, kd), g.id(i, jd, ku), g.id(i, jd, kd),
                           g.id(iu, j, ku), g.id(iu, j, kd), g.id(id, j, ku), g.id(id, j, kd)};
        for (int m = 0; m < NSLOT; m++) cols[p * NSLOT + m] = (int)c[m];
        int reg = 0;
        if (ctx->multinullspace && k >= ctx->kske[2 * (j * g.mx + i)]) reg = 1;
        region[p] = reg;
      }
  bool compact = true;
  for (size_t p = 0; p < n && compact; p++)
    if (fluid[p])
      for (int m = 0; m < NSLOT; m++)
        if (w[(size_t)m * n + p] != 0.0 && !fluid[cols[p * NSLOT + m]]) { compact = false; break; }
  // the inverted cells first (fluid, or every cell), then the identity ones
  std::vector<int> idx, pos(n, -1);
  for (size_t p = 0; p < n; p++)
    if (!compact || fluid[p]) { pos[p] = (int)idx.size(); idx.push_back((int)p); }
  const int m = (int)idx.size();
  for (size_t p = 0; p < n; p++)
    if (pos[p] < 0) idx.push_back((int)p);
  std::vector<double> A((size_t)m * m, 0.0);
  double diag_sum = 0.0;
  int nfl = 0;
  for (int r = 0; r < m; r++) {
    size_t p = (size_t)idx[r];
    if (!fluid[p]) { A[(size_t)r * m + r] = 1.0; continue; }
    for (int q = 0; q < NSLOT; q++) A[(size_t)r * m + pos[cols[p * NSLOT + q]]] += w[(size_t)q * n + p];
    diag_sum += std::fabs(A[(size_t)r * m + r]);
    nfl++;
  }
  if (nfl > 0) {
    double s = diag_sum / nfl;
    for (int reg = 0; reg < 2; reg++) {
      int cnt = 0;
      for (int r = 0; r < m; r++) cnt += region[idx[r]] == reg;
      if (!cnt) continue;
      double sv = s / cnt;
      for (int r = 0; r < m; r++) {
        if (region[idx[r]] != reg) continue;
        for (int q = 0; q < m; q++)
          if (region[idx[q]] == reg) A[(size_t)r * m + q] += sv;
      }
    }
  }
  if (ctx->Minv) dfree(ctx, ctx->Minv);
  if (ctx->cidx) dfree(ctx, ctx->cidx);
  ctx->Minv = nullptr;
  ctx->cidx = nullptr;
  TRY(dalloc(ctx, &ctx->Minv, std::max((size_t)m * m, (size_t)1)));
  TRY(dalloc(ctx, &ctx->cidx, n));
  if (m > kHostInverseMax) {
    // thousands of unknowns (a 16^3 coarsest level): Gauss-Jordan on the device
    double *dA = nullptr, *dwork = nullptr;
    int *iwork = nullptr;
    TRY(dalloc(ctx, &dA, (size_t)m * m));
    int rc = dalloc(ctx, &dwork, 2 * (size_t)m);
    if (rc == CVB_OK) rc = dalloc(ctx, &iwork, 2 * (size_t)m + 1);
    bool ok = false;
    if (rc == CVB_OK && cudaMemcpyAsync(dA, A.data(), sizeof(double) * m * m, cudaMemcpyHostToDevice,
                                        ctx->stream) == cudaSuccess)
      ok = device_dense_inverse(dA, m, ctx->Minv, iwork, iwork + m, dwork, dwork + m, iwork + 2 * m, ctx->stream);
    if (iwork) dfree(ctx, iwork);
    if (dwork) dfree(ctx, dwork);
    dfree(ctx, dA);
    if (rc != CVB_OK) return rc;
    CK(cudaGetLastError());
    if (!ok) return fail(ctx, CVB_BAD_INPUT, "coarsest operator is singular after regularisation");
  } else if (m > 0) {
    std::vector<double> Inv;
    if (!dense_inverse(A, m, Inv)) return fail(ctx, CVB_BAD_INPUT, "coarsest operator is singular after regularisation");
    CK(cudaMemcpyAsync(ctx->Minv, Inv.data(), sizeof(double) * m * m, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
  }
  CK(cudaMemcpyAsync(ctx->cidx, idx.data(), sizeof(int) * n, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  C.cidx = ctx->cidx;
  C.cm = m;
  return CVB_OK;
}

// nvert restriction down the hierarchy and the operator build of every level.
static int build_operators(cvb_ctx *ctx) {
  int nl = ctx->nlevels;
  for (int l = nl - 2; l >= 0; l--) {
    LevelDev &F = ctx->L[l + 1], &C = ctx->L[l];
    launch_nvert_restrict(F.g, F.nvert, C.g, C.isc, C.jsc, C.ksc, C.nvert, ctx->nvert_tmp, ctx->stream);
    CKL();
  }
  // FullyBlocked on the coarsest level (poisson.c:1578-1660)
  {
    LevelDev &C = ctx->L[0];
    size_t n = C.g.n();
    std::vector<double> nv(n);
    CK(cudaMemcpyAsync(nv.data(), C.nvert, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    const Geom &g = C.g;
    ctx->kske.assign(2 * (size_t)g.mx * g.my, 0);
    int all = 1;
    for (int j = 1; j < g.my - 1; j++)
      for (int i = 1; i < g.mx - 1; i++) {
        int blocked = 0;
        for (int k = 0; k < g.mz; k++)
          if (nv[g.id(i, j, k)] > 0.1) {
            int &ks = ctx->kske[2 * (j * g.mx + i)];
            if (!blocked) { ks = k; blocked = 1; }
            else ks = std::min(ks, k);
          }
        if (!blocked) all = 0;
      }
    ctx->multinullspace = all;
  }
  double *g9 = nullptr;
  size_t nmax = 0;
  for (auto &lv : ctx->L) nmax = std::max(nmax, lv.g.n());
  TRY(dalloc(ctx, &g9, 9 * nmax));
  for (int l = 0; l < nl; l++) {
    LevelDev &lv = ctx->L[l];
    const Geom &g = lv.g;
    size_t n = g.n();
    const double *m[9];
    for (int q = 0; q < 9; q++) m[q] = ctx->fm[l][q];
    launch_gcoef(g, m, ctx->iaj[l], ctx->jaj[l], ctx->kaj[l], g9, ctx->stream);
    launch_codes(g, lv.nvert, lv.code, ctx->stream);
    launch_weight32(g, lv.nvert, lv.wgt32, ctx->stream);
    launch_weights(g, g9, ctx->aj64[l], lv.nvert, lv.code, lv.w64, ctx->stream);
    launch_line_factors(g, lv.w64, lv.line64, lv.line32, ctx->stream);
    launch_to_f32(g9, lv.gf32, 9 * n, ctx->stream);
    launch_scale_cross(g, lv.code, lv.gf32, ctx->stream);
    launch_to_f32(ctx->aj64[l], lv.ajf32, n, ctx->stream);
    CKL();
  }
  // g9 is a set-up temporary; return it to the pool
  dfree(ctx, g9);
  // which levels have cross-derivative terms (the kernels read 7 points on the
  // others, with the same results)
  int *flags = nullptr;
  TRY(dalloc(ctx, &flags, 2 * (size_t)nl));
  CK(cudaMemsetAsync(flags, 0, sizeof(int) * 2 * nl, ctx->stream));
  for (int l = 0; l < nl; l++) launch_cross_flags(ctx->L[l].g, ctx->L[l].gf32, ctx->L[l].w64, flags + 2 * l, ctx->stream);
  CKL();
  std::vector<int> hf(2 * nl);
  CK(cudaMemcpyAsync(hf.data(), flags, sizeof(int) * 2 * nl, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  dfree(ctx, flags);
  for (int l = 0; l < nl; l++) {
    ctx->L[l].cross32 = hf[2 * l];
    ctx->L[l].cross64 = hf[2 * l + 1];
  }
  // the colour-split coefficient copies of the levels without FP32 cross terms
  // (dropped where a rebuild gave the level cross terms)
  for (int l = 0; l < nl; l++) {
    LevelDev &lv = ctx->L[l];
    if (lv.cross32) {
      if (lv.cs32) dfree(ctx, lv.cs32);
      lv.cs32 = nullptr;
      continue;
    }
    if (!lv.cs32) TRY(dalloc(ctx, &lv.cs32, 5 * SplitRow::count(lv.g)));
    launch_split_coef(lv.g, lv.gf32, lv.ajf32, lv.code, lv.cs32, ctx->stream);
    CKL();
  }
  CK(cudaStreamSynchronize(ctx->stream));
  return CVB_OK;
}

// Set-up autotuner: times the fused and the split y-line sweep on every level
// and precision (CUDA events on the context stream, after one warm-up launch)
// and keeps the faster; the choice depends on the level's size and on how its
// lines fill the machine.
// The sweep variant depends on a level's shape only, so a choice is measured
// once per shape in the process and reused: contexts set up later (or while
// other work loads the GPU) take the same variant, and so the same rounding.
namespace {
struct ShapeKey {
  int mx, my, mz, px, py, pz, c32, c64;  // box, periodicity, cross-derivative flags
  bool operator<(const ShapeKey &o) const {
    return std::tie(mx, my, mz, px, py, pz, c32, c64) < std::tie(o.mx, o.my, o.mz, o.px, o.py, o.pz, o.c32, o.c64);
  }
};
std::mutex g_tune_mu;
std::map<ShapeKey, cvb_ctx::Tune> g_tune_cache;
bool g_tune_loaded = false;

// With CVB_TUNE_FILE set, measured choices persist in that text file (one
// shape per line: mx my mz px py pz, the two cross-term flags and the
// thirteen timings in microseconds), so a
// later process -- a profiler run, say, whose own timings would be distorted --
// makes the same choices.  Called with g_tune_mu held.
void tune_file_load() {
  if (g_tune_loaded) return;
  g_tune_loaded = true;
  const char *path = std::getenv("CVB_TUNE_FILE");
  if (!path || !*path) return;
  FILE *f = std::fopen(path, "r");
  if (!f) return;
  ShapeKey k;
  cvb_ctx::Tune t;
  while (std::fscanf(f, "%d %d %d %d %d %d %d %d %lf %lf %lf %lf %lf %lf %lf %lf %lf %lf %lf %lf %lf", &k.mx, &k.my,
                     &k.mz, &k.px, &k.py, &k.pz, &k.c32, &k.c64, &t.us32[0], &t.us32[1], &t.us64[0], &t.us64[1],
                     &t.zb32[0], &t.zb32[1], &t.zb64[0], &t.zb64[1], &t.zt32[0], &t.zt32[1], &t.zt32[2], &t.zw32[0],
                     &t.zw32[1]) == 21) {
    t.level = 0;
    t.cells = (size_t)k.mx * k.my * k.mz;
    g_tune_cache.emplace(k, t);
  }
  std::fclose(f);
}
void tune_file_append(const ShapeKey &k, const cvb_ctx::Tune &t) {
  const char *path = std::getenv("CVB_TUNE_FILE");
  if (!path || !*path) return;
  FILE *f = std::fopen(path, "a");
  if (!f) return;
  std::fprintf(f, "%d %d %d %d %d %d %d %d %.3f %.3f %.3f %.3f %.3f %.3f %.3f %.3f %.3f %.3f %.3f %.3f %.3f\n", k.mx,
               k.my, k.mz, k.px, k.py, k.pz, k.c32, k.c64, t.us32[0], t.us32[1], t.us64[0], t.us64[1], t.zb32[0],
               t.zb32[1], t.zb64[0], t.zb64[1], t.zt32[0], t.zt32[1], t.zt32[2], t.zw32[0], t.zw32[1]);
  std::fclose(f);
}
}  // namespace

static int autotune_sweeps(cvb_ctx *ctx) {
  ctx->tune.clear();
  for (int l = 0; l < ctx->nlevels; l++) {
    LevelDev &L = ctx->L[l];
    size_t n = L.g.n();
    const ShapeKey key{L.g.mx, L.g.my, L.g.mz, L.g.px, L.g.py, L.g.pz, L.cross32, L.cross64};
    // the faster form of each sweep: a zero fused timing means not fusable
    auto pick = [&L](const cvb_ctx::Tune &t) {
      L.sweep32 = t.us32[1] < t.us32[0] ? 1 : 0;
      L.sweep64 = t.us64[1] < t.us64[0] ? 1 : 0;
      // the fused zebra form only when clearly faster (3 %): near-ties keep the
      // two-kernel form, so the choice does not flip with timing noise
      L.zfuse32 = t.zb32[1] > 0.0 && t.zb32[1] < 0.97 * t.zb32[0] ? 1 : 0;
      L.zfuse64 = t.zb64[1] > 0.0 && t.zb64[1] < 0.97 * t.zb64[0] ? 1 : 0;
      // the FP32 forms with 4 lines per tile instead of 8, same rule
      L.ztw32 = 0;
      {
        double cur = L.zfuse32 ? t.zb32[1] : t.zb32[0];
        for (int v = 0; v < 2; v++)
          if (t.zw32[v] > 0.0 && t.zw32[v] < 0.97 * cur) {
            cur = t.zw32[v];
            L.ztw32 = 4;
            L.zfuse32 = v;
          }
      }
      // the TMA-staged FP32 half-sweep and its chunk of row pairs, on the same
      // 3 % rule against the better of the other two forms
      const double other = L.ztw32 ? t.zw32[L.zfuse32] : L.zfuse32 ? t.zb32[1] : t.zb32[0];
      L.ztma32 = 0;
      double best = 0.97 * other;
      const int rps[3] = {4, 8, 16};
      for (int v = 0; v < 3; v++)
        if (t.zt32[v] > 0.0 && t.zt32[v] < best) { best = t.zt32[v]; L.ztma32 = rps[v]; }
    };
    {
      std::lock_guard<std::mutex> lock(g_tune_mu);
      tune_file_load();
      auto it = g_tune_cache.find(key);
      if (it != g_tune_cache.end()) {
        cvb_ctx::Tune t = it->second;
        t.level = l;
        pick(t);
        ctx->tune.push_back(t);
        continue;
      }
    }
    cvb_ctx::Tune t;
    t.level = l;
    t.cells = n;
    CK(cudaMemsetAsync(L.r32, 0, sizeof(float) * n, ctx->stream));
    CK(cudaMemsetAsync(L.e32, 0, sizeof(float) * n, ctx->stream));
    CK(cudaMemsetAsync(L.r64, 0, sizeof(double) * n, ctx->stream));
    CK(cudaMemsetAsync(L.e64, 0, sizeof(double) * n, ctx->stream));
    for (int prec = 0; prec < 2; prec++)
      for (int v = 0; v < 2; v++) {
        if (prec == 0) L.sweep32 = v; else L.sweep64 = v;
        const int reps = 3;
        for (int q = 0; q <= reps; q++) {
          if (q == 1) CK(cudaEventRecord(ctx->ev0, ctx->stream));
          if (prec == 0) launch_line_smooth<float>(L, L.r32, L.e32, L.t32 + n, 0.85f, 0, ctx->stream);
          else launch_line_smooth<double>(L, L.r64, L.e64, L.t64 + n, 0.85, 0, ctx->stream);
        }
        CK(cudaEventRecord(ctx->ev1, ctx->stream));
        CK(cudaEventSynchronize(ctx->ev1));
        CKL();
        float ms = 0;
        CK(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
        (prec == 0 ? t.us32 : t.us64)[v] = 1e3 * ms / reps;
      }
    L.ztma32 = 0;
    // zebra sweep (both colours): two kernels per half-sweep, then one (in place
    // without cross terms, else out of place through t)
    for (int prec = 0; prec < 2; prec++)
      for (int v = 0; v < 2; v++) {
        double *zb = prec == 0 ? t.zb32 : t.zb64;
        if (prec == 0) L.zfuse32 = v; else L.zfuse64 = v;
        const int reps = 5;
        for (int q = 0; q <= reps; q++) {
          if (q == 1) CK(cudaEventRecord(ctx->ev0, ctx->stream));
          if (prec == 0) launch_zebra_sweep<float>(L, L.r32, L.e32, L.t32, L.t32 + n, 1.3f, false, ctx->stream);
          else launch_zebra_sweep<double>(L, L.r64, L.e64, L.t64, L.t64 + n, 1.3, false, ctx->stream);
        }
        CK(cudaEventRecord(ctx->ev1, ctx->stream));
        CK(cudaEventSynchronize(ctx->ev1));
        CKL();
        float ms = 0;
        CK(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
        zb[v] = 1e3 * ms / reps;
      }
    // the FP32 zebra sweep's two forms with 4 lines per tile
    L.ztw32 = 4;
    for (int v = 0; v < 2; v++) {
      t.zw32[v] = 0.0;
      L.zfuse32 = v;
      const int reps = 5;
      for (int q = 0; q <= reps; q++) {
        if (q == 1) CK(cudaEventRecord(ctx->ev0, ctx->stream));
        launch_zebra_sweep<float>(L, L.r32, L.e32, L.t32, L.t32 + n, 1.3f, false, ctx->stream);
      }
      CK(cudaEventRecord(ctx->ev1, ctx->stream));
      CK(cudaEventSynchronize(ctx->ev1));
      CKL();
      float ms = 0;
      CK(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
      t.zw32[v] = 1e3 * ms / reps;
    }
    L.ztw32 = 0;
    // the FP32 zebra sweep with TMA-staged tiles, each chunk size
    for (int v = 0; v < 3; v++) {
      t.zt32[v] = 0.0;
      const int rps[3] = {4, 8, 16};
      if (!zebra_tma_ok(L)) continue;
      const int reps = 5;
      bool ran = true;
      for (int q = 0; q <= reps && ran; q++) {
        if (q == 1) CK(cudaEventRecord(ctx->ev0, ctx->stream));
        for (int color = 0; color < 2 && ran; color++)
          ran = launch_zebra_tma(L, L.r32, L.e32, 1.3f, color, rps[v], ctx->stream);
      }
      if (!ran) {  // the tensor maps were refused: the form is not available here
        CK(cudaStreamSynchronize(ctx->stream));
        continue;
      }
      CK(cudaEventRecord(ctx->ev1, ctx->stream));
      CK(cudaEventSynchronize(ctx->ev1));
      CKL();
      float ms = 0;
      CK(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
      t.zt32[v] = 1e3 * ms / reps;
    }
    if (tma_timeout_take(ctx->stream) != 0) return fail(ctx, CVB_TIMEOUT, "a TMA-staged half-sweep gave up waiting");
    pick(t);
    ctx->tune.push_back(t);
    std::lock_guard<std::mutex> lock(g_tune_mu);
    if (g_tune_cache.emplace(key, t).second) tune_file_append(key, t);
  }
  return CVB_OK;
}

// Fills the [3][N] face-area block |csi|, |eta|, |zet| used by VolumeFlux_rev.
static void face_areas(const std::vector<double> &csi, const std::vector<double> &eta,
                       const std::vector<double> &zet, std::vector<double> &a3) {
  size_t n = csi.size() / 3;
  a3.resize(3 * n);
  const std::vector<double> *src[3] = {&csi, &eta, &zet};
  for (int d = 0; d < 3; d++)
    for (size_t p = 0; p < n; p++) {
      const double *v = &(*src[d])[3 * p];
      a3[d * n + p] = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    }
}

// ------------------------------------------------------------------ V-cycle
template <typename T>
static T *vptr(LevelDev &L, int which);
// which: 0 rhs, 1 e, 2 e2, 3 res.  Layout of the per-level allocation: r=rhs, e=e, t=[e2|res]
template <>
float *vptr<float>(LevelDev &L, int which) {
  size_t n = L.g.n();
  switch (which) {
    case 0: return L.r32;
    case 1: return L.e32;
    case 2: return L.t32;
    default: return L.t32 + n;
  }
}
template <>
double *vptr<double>(LevelDev &L, int which) {
  size_t n = L.g.n();
  switch (which) {
    case 0: return L.r64;
    case 1: return L.e64;
    case 2: return L.t64;
    default: return L.t64 + n;
  }
}

template <typename T>
static void smooth(LevelDev &L, const T *b, T *&x, T *&x2, T omega, int sweeps, bool zero_first, cudaStream_t s);
template <>
void smooth<float>(LevelDev &L, const float *b, float *&x, float *&x2, float omega, int sweeps, bool zero_first,
                   cudaStream_t s) {
  for (int q = 0; q < sweeps; q++) {
    bool z = zero_first && q == 0;
    // residual goes to the res buffer, Thomas writes x2, then swap
    LevelDev tmp = L;
    tmp.t32 = vptr<float>(L, 3);
    launch_line_smooth<float>(tmp, b, z ? nullptr : x, x2, omega, z, s);
    std::swap(x, x2);
  }
}
template <>
void smooth<double>(LevelDev &L, const double *b, double *&x, double *&x2, double omega, int sweeps,
                    bool zero_first, cudaStream_t s) {
  for (int q = 0; q < sweeps; q++) {
    bool z = zero_first && q == 0;
    LevelDev tmp = L;
    tmp.t64 = vptr<double>(L, 3);
    launch_line_smooth<double>(tmp, b, z ? nullptr : x, x2, omega, z, s);
    std::swap(x, x2);
  }
}

template <typename T>
static void coarse_solve(cvb_ctx *ctx, const T *b, T *x, const cvb_solve_opts *o);
template <>
void coarse_solve<float>(cvb_ctx *ctx, const float *b, float *x, const cvb_solve_opts *o) {
  LevelDev &C = ctx->L[0];
  if (ctx->coarse_dense) { launch_dense_apply_f32(C, ctx->Minv, b, x, ctx->stream); return; }
  float *a = x, *a2 = vptr<float>(C, 2);
  smooth<float>(C, b, a, a2, (float)o->omega, 30, true, ctx->stream);
  if (a != x) cudaMemcpyAsync(x, a, sizeof(float) * C.g.n(), cudaMemcpyDeviceToDevice, ctx->stream);
}
template <>
void coarse_solve<double>(cvb_ctx *ctx, const double *b, double *x, const cvb_solve_opts *o) {
  LevelDev &C = ctx->L[0];
  if (ctx->coarse_dense) { launch_dense_apply(C, ctx->Minv, b, x, ctx->stream); return; }
  double *a = x, *a2 = vptr<double>(C, 2);
  smooth<double>(C, b, a, a2, o->omega, 30, true, ctx->stream);
  if (a != x) cudaMemcpyAsync(x, a, sizeof(double) * C.g.n(), cudaMemcpyDeviceToDevice, ctx->stream);
}

template <typename T>
static void vcycle(cvb_ctx *ctx, int l, const T *b, T *out, const cvb_solve_opts *o, bool zeroed = false);

// The V-cycle with zebra smoothing: x (= out) is updated in place, each sweep
// one half-sweep per color.  zeroed: x is already zero (the restriction into
// this level cleared it).
template <typename T>
static void vcycle_zebra(cvb_ctx *ctx, int l, const T *b, T *x, const cvb_solve_opts *o, bool zeroed) {
  cudaStream_t s = ctx->stream;
  LevelDev &L = ctx->L[l], &C = ctx->L[l - 1];
  T *res = vptr<T>(L, 3);
  const T omega = (T)o->omega;
  if (!zeroed) cudaMemsetAsync(x, 0, sizeof(T) * L.g.n(), s);
  T *tmp = vptr<T>(L, 2);
  const int pre = std::max(o->pre_sweeps, 1);
  for (int q = 0; q < pre; q++) launch_zebra_sweep<T>(L, b, x, tmp, res, omega, q == 0, s);
  launch_residual<T>(L, b, x, res, s);
  T *bc = vptr<T>(C, 0), *ec = vptr<T>(C, 1);
  const bool clear = l - 1 > 0;  // the coarsest solve writes all of ec itself
  launch_restrict<T>(L, C, res, bc, s, clear ? ec : nullptr);
  vcycle<T>(ctx, l - 1, bc, ec, o, clear);
  launch_prolong_add<T>(C, L, ec, x, s);
  for (int q = 0; q < o->post_sweeps; q++) launch_zebra_sweep<T>(L, b, x, tmp, res, omega, false, s);
}

// One V-cycle on level l for A e = b, zero initial guess; result in `out`.
template <typename T>
static void vcycle(cvb_ctx *ctx, int l, const T *b, T *out, const cvb_solve_opts *o, bool zeroed) {
  cudaStream_t s = ctx->stream;
  if (l == 0) { coarse_solve<T>(ctx, b, out, o); return; }
  if (o->smoother == CVB_SMOOTHER_ZEBRA) { vcycle_zebra<T>(ctx, l, b, out, o, zeroed); return; }
  LevelDev &L = ctx->L[l], &C = ctx->L[l - 1];
  size_t n = L.g.n();
  T *x = out, *x2 = vptr<T>(L, 2);
  if (x2 == b) x2 = vptr<T>(L, 1);
  T omega = (T)o->omega;
  smooth<T>(L, b, x, x2, omega, std::max(o->pre_sweeps, 1), true, s);
  T *res = vptr<T>(L, 3);
  launch_residual<T>(L, b, x, res, s);
  T *bc = vptr<T>(C, 0), *ec = vptr<T>(C, 1);
  launch_restrict<T>(L, C, res, bc, s);
  vcycle<T>(ctx, l - 1, bc, ec, o);
  launch_prolong_add<T>(C, L, ec, x, s);
  smooth<T>(L, b, x, x2, omega, o->post_sweeps, false, s);
  if (x != out) cudaMemcpyAsync(out, x, sizeof(T) * n, cudaMemcpyDeviceToDevice, s);
}

// One V-cycle replayed from a CUDA graph: the first use of a (precision, input,
// output) triple runs it eagerly (kernel attributes get set outside any
// capture), the second captures it on the context's stream, later ones replay
// the graph -- one launch for the cycle's tens of kernels, most of them on
// coarse levels where a kernel is shorter than its launch.  Graphs are keyed
// by the cycle's options and dropped whenever the operators are rebuilt.
void drop_vcycle_graphs(cvb_ctx *ctx) {
  for (auto &kv : ctx->vgraphs)
    if (kv.second.exec) cudaGraphExecDestroy(kv.second.exec);
  ctx->vgraphs.clear();
}

template <typename T>
static int vcycle_graph(cvb_ctx *ctx, const cvb_solve_opts *o, int slot, const T *b, T *out) {
  const int key = (sizeof(T) == 4 ? 1000 : 0) + slot;
  VGraph &g = ctx->vgraphs[key];
  const bool same = g.omega == o->omega && g.pre == o->pre_sweeps && g.post == o->post_sweeps && g.b == (const void *)b &&
                    g.out == (void *)out && g.smoother == o->smoother;
  if (!same) {
    if (g.exec) cudaGraphExecDestroy(g.exec);
    g = VGraph();
    g.omega = o->omega; g.pre = o->pre_sweeps; g.post = o->post_sweeps; g.b = b; g.out = out;
    g.smoother = o->smoother;
  }
  if (g.exec) {
    CK(cudaGraphLaunch(g.exec, ctx->stream));
    count_launch(g.nodes);
    return CVB_OK;
  }
  if (g.uses++ == 0 || g.failed) {
    vcycle<T>(ctx, ctx->nlevels - 1, b, out, o);
    CKL();
    return CVB_OK;
  }
  cudaGraph_t graph = nullptr;
  const long long c0 = launch_count();
  CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
  vcycle<T>(ctx, ctx->nlevels - 1, b, out, o);
  cudaError_t e = cudaStreamEndCapture(ctx->stream, &graph);
  const long long nodes = launch_count() - c0;
  count_launch((int)-nodes);  // captured, not launched
  if (e == cudaSuccess && graph) e = cudaGraphInstantiate(&g.exec, graph, 0);
  if (graph) cudaGraphDestroy(graph);
  if (e != cudaSuccess || !g.exec) {
    cudaGetLastError();
    g.exec = nullptr;
    g.failed = true;  // keep to eager launches for this cycle
    vcycle<T>(ctx, ctx->nlevels - 1, b, out, o);
    CKL();
    return CVB_OK;
  }
  g.nodes = (int)nodes;
  CK(cudaGraphLaunch(g.exec, ctx->stream));
  count_launch(g.nodes);
  return CVB_OK;
}

// ------------------------------------------------------------------ solver
static int reduce_to_host(cvb_ctx *ctx, int nv, double *out) {
  launch_finish_sums(ctx->partial, nv, reduce_blocks(), ctx->sums, ctx->stream);
  CKL();
  CK(cudaMemcpyAsync(out, ctx->sums, sizeof(double) * nv, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return CVB_OK;
}

static int norm2(cvb_ctx *ctx, const double *v, size_t n, double *out) {
  // dot(v, v) with the multi-dot kernel; its one-entry pointer table is dV[kMaxRestart + 1]
  CK(cudaMemcpyAsync(ctx->dV + kMaxRestart + 1, &v, sizeof(double *), cudaMemcpyHostToDevice, ctx->stream));
  launch_multidot(ctx->dV + kMaxRestart + 1, 1, v, n, ctx->partial, ctx->stream);
  CKL();
  double s;
  TRY(reduce_to_host(ctx, 1, &s));
  *out = std::sqrt(s);
  return CVB_OK;
}

static int fluid_mean_zero(cvb_ctx *ctx, int level, double *x) {
  LevelDev &L = ctx->L[level];
  launch_fluid_mean_partial(L.g, L.code, x, ctx->partial, ctx->stream);
  launch_finish_sums(ctx->partial, 2, reduce_blocks(), ctx->sums, ctx->stream);
  launch_add_fluid_const(L.g, L.code, x, ctx->sums, 1, ctx->stream);
  CKL();
  return CVB_OK;
}

// Projects b onto range(A): b -= aj * (sum_fluid b/aj) / n_fluid on fluid cells.
static int project_rhs(cvb_ctx *ctx, double *b, double *removed);

static int fgmres(cvb_ctx *ctx, const cvb_solve_opts *o, cvb_solve_stats *st) {
  LevelDev &F = ctx->L[ctx->nlevels - 1];
  const size_t n = F.g.n();
  cudaStream_t s = ctx->stream;
  const bool mixed = o->precision == CVB_PRECISION_MIXED;
  const int m = std::min(std::max(o->restart, 1), kMaxRestart);
  double bnorm;
  TRY(norm2(ctx, ctx->b, n, &bnorm));
  st->rhs_norm = bnorm;
  if (!std::isfinite(bnorm)) return fail(ctx, CVB_NAN_DETECTED, "right-hand side is not finite");
  if (bnorm == 0.0) {
    CK(cudaMemsetAsync(ctx->x, 0, sizeof(double) * n, s));
    st->rel_residual = 0.0;
    st->abs_residual = 0.0;
    return CVB_OK;
  }
  // r0 = b - A x0: b itself for the zero initial guess (same bits, no apply)
  const double *rcur = ctx->r;
  double beta;
  if (!o->warm_start) {
    CK(cudaMemsetAsync(ctx->x, 0, sizeof(double) * n, s));
    rcur = ctx->b;
    beta = bnorm;
  } else {
    launch_residual<double>(F, ctx->b, ctx->x, ctx->r, s);
    CKL();
    TRY(norm2(ctx, ctx->r, n, &beta));
  }
  int total = 0, restarts = 0;
  double H[kMaxRestart + 1][kMaxRestart];
  double cs[kMaxRestart], sn[kMaxRestart], gv[kMaxRestart + 1], yv[kMaxRestart];
  int status = CVB_NOT_CONVERGED;
  const double target = std::max(o->rtol * bnorm, o->atol);
  while (true) {
    if (!std::isfinite(beta)) return fail(ctx, CVB_NAN_DETECTED, "residual became %g", beta);
    if (beta <= target) { status = CVB_OK; break; }
    if (total >= o->max_it) break;
    // V[0] = r / beta (k_scale divides by the device scalar)
    CK(cudaMemcpyAsync(ctx->hdev, &beta, sizeof(double), cudaMemcpyHostToDevice, s));
    // in mixed precision the scaling also writes the V-cycle's FP32 input
    float *in32 = mixed ? ctx->b32 : nullptr;
    launch_scale(ctx->V[0], rcur, ctx->hdev, n, s, nullptr, in32);
    CKL();
    for (int q = 0; q <= m; q++) gv[q] = 0.0;
    gv[0] = beta;
    int j = 0;
    double est = beta;
    for (; j < m && total < o->max_it; j++) {
      // z_j = M^-1 v_j
      if (mixed) {
        // ctx->b32 holds V[j] in FP32 (written by the scaling that formed V[j])
        // FP32 V-cycle; its result is widened once into the FP64 basis so the
        // FP64 operator and the final update read it without per-use conversions
        // (a conversion costs an FP64-pipe instruction on this part)
        TRY(vcycle_graph<float>(ctx, o, 0, ctx->b32, ctx->Z32[0]));
        launch_f32_to_f64(ctx->Z32[0], ctx->Z64[j], n, s);
        launch_apply<double>(F, ctx->Z64[j], ctx->w, s);
      } else {
        TRY(vcycle_graph<double>(ctx, o, j, ctx->V[j], ctx->Z64[j]));
        launch_apply<double>(F, ctx->Z64[j], ctx->w, s);
      }
      CKL();
      // classical Gram-Schmidt (PETSc's default for GMRES/FGMRES), with a second
      // pass only when the first one cancelled most of w (||w|| dropped below
      // half of its length before orthogonalisation).  The projections and the
      // norm stay on the device between the kernels (V_{j+1} = w / ||w|| is
      // formed there too); the host reads them back once per iteration.  The
      // norm of the updated w is summed from w itself: ||w||^2 - ||h||^2 would
      // save a pass, but on a basis whose orthogonality classical Gram-Schmidt
      // has eroded it is off by far more than rounding, and FGMRES then needed
      // 32 iterations instead of 6 on the channel.
      double h[kMaxRestart + 2], h2[kMaxRestart + 1], nw2;
      double *dsum = ctx->sums, *dnorm = ctx->sums + kMaxRestart + 2;
      launch_multidot(ctx->dV, j + 1, ctx->w, n, ctx->partial, s, 1);
      launch_finish_sums(ctx->partial, j + 2, reduce_blocks(), dsum, s);
      launch_multiaxpy_norm(ctx->w, ctx->dV, dsum, j + 1, n, ctx->partial, s);
      launch_finish_sums(ctx->partial, 1, reduce_blocks(), dnorm, s);
      launch_scale_sqrt(ctx->V[j + 1], ctx->w, dnorm, n, s, in32);
      CKL();
      CK(cudaMemcpyAsync(h, dsum, sizeof(double) * (j + 2), cudaMemcpyDeviceToHost, s));
      CK(cudaMemcpyAsync(&nw2, dnorm, sizeof(double), cudaMemcpyDeviceToHost, s));
      CK(cudaStreamSynchronize(s));
      const double w_before = h[j + 1];
      for (int q = 0; q <= j; q++) h2[q] = 0.0;
      if (o->cgs_refine && nw2 < 0.25 * w_before) {
        launch_multidot(ctx->dV, j + 1, ctx->w, n, ctx->partial, s);
        launch_finish_sums(ctx->partial, j + 1, reduce_blocks(), dsum, s);
        launch_multiaxpy_norm(ctx->w, ctx->dV, dsum, j + 1, n, ctx->partial, s);
        launch_finish_sums(ctx->partial, 1, reduce_blocks(), dnorm, s);
        launch_scale_sqrt(ctx->V[j + 1], ctx->w, dnorm, n, s, in32);
        CKL();
        CK(cudaMemcpyAsync(h2, dsum, sizeof(double) * (j + 1), cudaMemcpyDeviceToHost, s));
        CK(cudaMemcpyAsync(&nw2, dnorm, sizeof(double), cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
      }
      for (int q = 0; q <= j; q++) H[q][j] = h[q] + h2[q];
      double hn = std::sqrt(nw2);
      H[j + 1][j] = hn;
      total++;
      if (!std::isfinite(hn)) return fail(ctx, CVB_NAN_DETECTED, "Krylov vector became non-finite");
      // Givens rotations
      for (int q = 0; q < j; q++) {
        double t = cs[q] * H[q][j] + sn[q] * H[q + 1][j];
        H[q + 1][j] = -sn[q] * H[q][j] + cs[q] * H[q + 1][j];
        H[q][j] = t;
      }
      double a = H[j][j], bb = H[j + 1][j];
      double rr = std::hypot(a, bb);
      cs[j] = rr > 0 ? a / rr : 1.0;
      sn[j] = rr > 0 ? bb / rr : 0.0;
      H[j][j] = rr;
      H[j + 1][j] = 0.0;
      gv[j + 1] = -sn[j] * gv[j];
      gv[j] = cs[j] * gv[j];
      est = std::fabs(gv[j + 1]);
      if (est <= target || hn == 0.0) { j++; break; }
    }
    // y = H^-1 g ; x += Z y
    for (int q = j - 1; q >= 0; q--) {
      double t = gv[q];
      for (int c2 = q + 1; c2 < j; c2++) t -= H[q][c2] * yv[c2];
      yv[q] = t / H[q][q];
    }
    CK(cudaMemcpyAsync(ctx->hdev, yv, sizeof(double) * j, cudaMemcpyHostToDevice, s));
    launch_axpy_z(ctx->x, nullptr, ctx->dZ64, ctx->hdev, j, n, s);
    launch_residual<double>(F, ctx->b, ctx->x, ctx->r, s);
    CKL();
    TRY(norm2(ctx, ctx->r, n, &beta));
    rcur = ctx->r;
    restarts++;
  }
  TRY(fluid_mean_zero(ctx, ctx->nlevels - 1, ctx->x));
  st->iterations = total;
  st->restarts = restarts > 0 ? restarts - 1 : 0;
  st->abs_residual = beta;
  st->rel_residual = beta / bnorm;
  st->status = status;
  if (status != CVB_OK)
    return fail(ctx, status, "not converged: relative residual %.3e after %d iterations", beta / bnorm, total);
  return CVB_OK;
}

static int project_rhs(cvb_ctx *ctx, double *b, double *removed) {
  int l = ctx->nlevels - 1;
  LevelDev &F = ctx->L[l];
  launch_fluid_ratio_partial(F.g, F.code, b, ctx->inv_aj, ctx->partial, ctx->stream);
  launch_finish_sums(ctx->partial, 2, reduce_blocks(), ctx->sums, ctx->stream);
  launch_remove_aj_mean(F.g, F.code, ctx->aj64[l], b, ctx->sums, ctx->stream);
  CKL();
  double h[2];
  CK(cudaMemcpyAsync(h, ctx->sums, sizeof(double) * 2, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  // h = {sum b/aj, fluid count}; the removed part is aj * mean(b/aj) on fluid cells
  double c = h[1] > 0 ? h[0] / h[1] : 0.0;
  *removed = c;
  return CVB_OK;
}

static int solve_resident(cvb_ctx *ctx, const cvb_solve_opts *o, cvb_solve_stats *st) {
  if (!ctx->ready) return fail(ctx, CVB_NOT_SETUP, "cvb_setup_hierarchy has not run");
  cvb_solve_opts def;
  if (!o) { cvb_solve_opts_default(&def); o = &def; }
  if (o->restart < 1 || o->restart > kMaxRestart || o->max_it < 0 || !(o->rtol >= 0) || o->pre_sweeps < 0 ||
      o->post_sweeps < 0 || (o->precision != CVB_PRECISION_FP64 && o->precision != CVB_PRECISION_MIXED) ||
      (o->smoother != CVB_SMOOTHER_JACOBI && o->smoother != CVB_SMOOTHER_ZEBRA))
    return fail(ctx, CVB_BAD_INPUT, "bad solve options");
  cvb_solve_stats local;
  if (!st) st = &local;
  std::memset(st, 0, sizeof(*st));
  CK(cudaEventRecord(ctx->ev0, ctx->stream));
  if (o->project_rhs) TRY(project_rhs(ctx, ctx->b, &st->rhs_projected));
  int rc = fgmres(ctx, o, st);
  cudaEventRecord(ctx->ev1, ctx->stream);
  cudaEventSynchronize(ctx->ev1);
  float ms = 0;
  cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
  st->device_ms = ms;
  st->status = rc;
  bool tma = false;
  for (int l = 0; l < ctx->nlevels; l++) tma = tma || ctx->L[l].ztma32 != 0;
  if (tma && tma_timeout_take(ctx->stream) != 0) {
    st->status = CVB_TIMEOUT;
    return fail(ctx, CVB_TIMEOUT, "a TMA-staged half-sweep gave up waiting for its tiles; the result is not valid");
  }
  return rc;
}

// Per-problem part of a set-up on the context's geometry: level arrays, the
// finest level's nvert (owned box), operators, smoother factors, coarsest solver.
// nvert holds the reference's cell codes (0 fluid, 1..2 immersed boundary, 3+
// solid, ibm.c:4332-4438): finite and non-negative.
static int check_nvert(cvb_ctx *ctx, const double *v, size_t n) {
  for (size_t p = 0; p < n; p++)
    if (!std::isfinite(v[p]) || v[p] < 0.0)
      return fail(ctx, CVB_BAD_INPUT, "nvert[%zu] = %g is not a cell code (finite, >= 0)", p, v[p]);
  return CVB_OK;
}

static int setup_problem(cvb_ctx *ctx, const double *nvert_box) {
  using clk = std::chrono::steady_clock;
  auto ms_since = [](clk::time_point t) { return std::chrono::duration<double, std::milli>(clk::now() - t).count(); };
  clk::time_point t = clk::now();
  const int nlevels = ctx->nlevels;
  {
    const cvb_level_desc &d = ctx->H[nlevels - 1].d;
    TRY(check_nvert(ctx, nvert_box, (size_t)d.mx * d.my * d.mz));
  }
  Geometry &G = *ctx->geo;
  ctx->fm = G.fm;
  ctx->iaj = G.iaj; ctx->jaj = G.jaj; ctx->kaj = G.kaj; ctx->aj64 = G.aj64;
  ctx->area3 = G.area3;
  ctx->inv_aj = G.inv_aj;
  for (int c = 0; c < 3; c++) ctx->cm[c] = G.cm[c];
  ctx->L.assign(nlevels, LevelDev());
  size_t nmax = 0;
  for (int l = 0; l < nlevels; l++) {
    const cvb_level_desc &d = ctx->H[l].d;
    LevelDev &L = ctx->L[l];
    L.g.mx = d.mx; L.g.my = d.my; L.g.mz = d.mz;
    L.g.px = d.bctype[0] == 7; L.g.py = d.bctype[2] == 7; L.g.pz = d.bctype[4] == 7;
    L.isc = d.isc; L.jsc = d.jsc; L.ksc = d.ksc;
    size_t n = L.g.n();
    nmax = std::max(nmax, n);
    TRY(dalloc(ctx, &L.nvert, n));
    TRY(dalloc(ctx, &L.code, n));
    TRY(dalloc(ctx, &L.w64, (size_t)NSLOT * n));
    TRY(dalloc(ctx, &L.gf32, 9 * n));
    TRY(dalloc(ctx, &L.ajf32, n));
    TRY(dalloc(ctx, &L.wgt32, n));
    TRY(dalloc(ctx, &L.line32, LineFac::of(L.g).count(L.g)));
    TRY(dalloc(ctx, &L.line64, LineFac::of(L.g).count(L.g)));
    // t: [e2 | res]; res also holds a zebra residual in colour-split rows
    const size_t nt = n + std::max(n, SplitRow::count(L.g));
    TRY(dalloc(ctx, &L.r64, n)); TRY(dalloc(ctx, &L.e64, n)); TRY(dalloc(ctx, &L.t64, nt));
    TRY(dalloc(ctx, &L.r32, n)); TRY(dalloc(ctx, &L.e32, n)); TRY(dalloc(ctx, &L.t32, nt));
  }
  TRY(dalloc(ctx, &ctx->nvert_tmp, nmax));
  LevelDev &F = ctx->L[nlevels - 1];
  size_t n = F.g.n();
  CK(cudaMemcpyAsync(F.nvert, nvert_box, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  TRY(dalloc(ctx, &ctx->b, n)); TRY(dalloc(ctx, &ctx->x, n));
  TRY(dalloc(ctx, &ctx->w, n)); TRY(dalloc(ctx, &ctx->r, n));
  TRY(dalloc(ctx, &ctx->b32, n));
  TRY(dalloc(ctx, &ctx->uc_dev, 3 * n)); TRY(dalloc(ctx, &ctx->p_dev, n));
  TRY(dalloc(ctx, &ctx->dV, kMaxRestart + 2));
  TRY(dalloc(ctx, &ctx->dZ64, kMaxRestart));
  TRY(dalloc(ctx, &ctx->dZ32, kMaxRestart));
  int nb = reduce_blocks();
  TRY(dalloc(ctx, &ctx->partial, (size_t)nb * (kMaxRestart + 2)));
  TRY(dalloc(ctx, &ctx->sums, 2 * (kMaxRestart + 2)));
  TRY(dalloc(ctx, &ctx->hdev, kMaxRestart + 2));
  CK(cudaStreamSynchronize(ctx->stream));
  ctx->setup_ms[1] = ms_since(t);
  t = clk::now();
  TRY(build_operators(ctx));
  ctx->setup_ms[2] = ms_since(t);
  t = clk::now();
  TRY(autotune_sweeps(ctx));
  ctx->setup_ms[3] = ms_since(t);
  t = clk::now();
  cvb_solve_opts def;
  cvb_solve_opts_default(&def);
  TRY(build_coarse(ctx, &def));
  CK(cudaStreamSynchronize(ctx->stream));
  ctx->setup_ms[4] = ms_since(t);
  static std::atomic<unsigned long long> setups{0};
  ctx->setup_id = ++setups;
  ctx->ready = true;
  return CVB_OK;
}

// ------------------------------------------------------------------ C ABI
extern "C" {

int cvb_solve_opts_default(cvb_solve_opts *o) {
  if (!o) return CVB_BAD_INPUT;
  o->precision = CVB_PRECISION_MIXED;
  o->rtol = 1e-8;
  o->atol = 0.0;
  o->max_it = 200;
  o->restart = 30;
  o->pre_sweeps = 2;
  o->post_sweeps = 2;
  o->omega = 1.3;
  o->project_rhs = 1;
  o->warm_start = 0;
  o->coarse_dense_max = kCoarseDenseMaxDefault;
  o->cgs_refine = 0;
  o->smoother = CVB_SMOOTHER_ZEBRA;
  return CVB_OK;
}

}  // extern "C"

namespace {
// One "-name value" pair into opts; false when the value does not parse.
bool apply_option(const std::string &name, const std::string &val, cvb_solve_opts *o) {
  char *end = nullptr;
  auto real = [&](double *dst) {
    double v = std::strtod(val.c_str(), &end);
    if (val.empty() || *end || !std::isfinite(v)) return false;
    *dst = v;
    return true;
  };
  auto integer = [&](int *dst) {
    long v = std::strtol(val.c_str(), &end, 10);
    if (val.empty() || *end) return false;
    *dst = (int)v;
    return true;
  };
  if (name == "-ps_ksp_rtol") return real(&o->rtol);
  if (name == "-ps_ksp_atol") return real(&o->atol);
  if (name == "-ps_ksp_max_it") return integer(&o->max_it);
  if (name == "-ps_ksp_gmres_restart") return integer(&o->restart);
  if (name == "-cvb_pre_sweeps") return integer(&o->pre_sweeps);
  if (name == "-cvb_post_sweeps") return integer(&o->post_sweeps);
  if (name == "-cvb_omega") return real(&o->omega);
  if (name == "-cvb_coarse_dense_max") return integer(&o->coarse_dense_max);
  if (name == "-cvb_precision") {
    if (val == "fp64") o->precision = CVB_PRECISION_FP64;
    else if (val == "mixed") o->precision = CVB_PRECISION_MIXED;
    else return false;
    return true;
  }
  if (name == "-cvb_smoother") {
    if (val == "zebra") o->smoother = CVB_SMOOTHER_ZEBRA;
    else if (val == "jacobi") o->smoother = CVB_SMOOTHER_JACOBI;
    else return false;
    return true;
  }
  return true;  // not a solver option: ignored, as PETSc ignores unused options
}

// Tokens "-name [value]": a name followed by a token that is not itself an
// option name takes it as its value (a negative number is a value).
int apply_tokens(const std::vector<std::string> &tok, cvb_solve_opts *o, char *bad, int bad_len) {
  auto is_name = [](const std::string &t) {
    return t.size() > 1 && t[0] == '-' && !(std::isdigit((unsigned char)t[1]) || t[1] == '.');
  };
  for (size_t q = 0; q < tok.size(); q++) {
    if (!is_name(tok[q])) continue;
    std::string val;
    if (q + 1 < tok.size() && !is_name(tok[q + 1])) val = tok[++q];
    if (!apply_option(tok[q - (val.empty() ? 0 : 1)], val, o)) {
      if (bad && bad_len > 0) std::snprintf(bad, bad_len, "%s %s", tok[q - (val.empty() ? 0 : 1)].c_str(), val.c_str());
      return CVB_BAD_INPUT;
    }
  }
  return CVB_OK;
}
}  // namespace

extern "C" {

int cvb_solve_opts_from_args(int argc, const char *const *argv, cvb_solve_opts *opts, char *bad, int bad_len) {
  if (!opts || argc < 0 || (argc > 0 && !argv)) return CVB_BAD_INPUT;
  std::vector<std::string> tok;
  for (int q = 0; q < argc; q++)
    if (argv[q]) tok.emplace_back(argv[q]);
  return apply_tokens(tok, opts, bad, bad_len);
}

int cvb_solve_opts_from_file(const char *path, cvb_solve_opts *opts, char *bad, int bad_len) {
  if (!opts || !path) return CVB_BAD_INPUT;
  FILE *f = std::fopen(path, "r");
  if (!f) {
    if (bad && bad_len > 0) std::snprintf(bad, bad_len, "cannot read %s", path);
    return CVB_BAD_INPUT;
  }
  std::vector<std::string> tok;
  char line[4096];
  while (std::fgets(line, sizeof line, f)) {
    char *hash = std::strchr(line, '#');
    if (hash) *hash = 0;
    for (char *t = std::strtok(line, " \t\r\n"); t; t = std::strtok(nullptr, " \t\r\n")) tok.emplace_back(t);
  }
  std::fclose(f);
  return apply_tokens(tok, opts, bad, bad_len);
}

int cvb_init(cvb_ctx **out, const cvb_options *opts) {
  if (!out) return CVB_BAD_INPUT;
  cvb_ctx *ctx = new cvb_ctx();
  *out = ctx;
  ctx->device = opts ? opts->device : 0;
  CK(cudaSetDevice(ctx->device));
  if (opts && opts->stream) {
    ctx->stream = (cudaStream_t)opts->stream;
  } else {
    CK(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
    ctx->own_stream = true;
  }
  CK(cudaEventCreate(&ctx->ev0));
  CK(cudaEventCreate(&ctx->ev1));
  return CVB_OK;
}

void cvb_destroy(cvb_ctx *ctx) {
  if (!ctx) return;
  cudaSetDevice(ctx->device);
  free_all(ctx);
  if (ctx->ev0) cudaEventDestroy(ctx->ev0);
  if (ctx->ev1) cudaEventDestroy(ctx->ev1);
  if (ctx->own_stream && ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
}

const char *cvb_last_error(const cvb_ctx *ctx) { return ctx ? ctx->err.c_str() : "no context"; }

void *cvb_stream(cvb_ctx *ctx) { return ctx ? (void *)ctx->stream : nullptr; }

// Checks the level descriptors and uploads the grid's metrics into a new Geometry.
static int upload_geometry(cvb_ctx *ctx, int nlevels, const cvb_level_desc *lv) {
  CK(cudaSetDevice(ctx->device));
  ensure_pool(ctx->device);
  free_all(ctx);
  for (int l = 0; l < nlevels; l++) TRY(check_desc(ctx, lv[l], l, l == nlevels - 1));
  for (int l = 0; l + 1 < nlevels; l++) {
    const cvb_level_desc &c = lv[l], &f = lv[l + 1];
    int ex = c.isc ? f.mx : (f.mx - 2) / 2 + 2, ey = c.jsc ? f.my : (f.my - 2) / 2 + 2, ez = c.ksc ? f.mz : (f.mz - 2) / 2 + 2;
    if (c.mx != ex || c.my != ey || c.mz != ez)
      return fail(ctx, CVB_BAD_INPUT, "level %d box %dx%dx%d is not the coarsening of level %d (%dx%dx%d expected)", l,
                  c.mx, c.my, c.mz, l + 1, ex, ey, ez);
  }
  ctx->nlevels = nlevels;
  ctx->H.resize(nlevels);
  for (int l = 0; l < nlevels; l++) ctx->H[l].d = lv[l];
  // the grid's metrics: uploaded once, owned by a Geometry other contexts may share
  auto G = std::make_shared<Geometry>();
  G->device = ctx->device;
  G->fm.assign(nlevels, std::vector<double *>(9, nullptr));
  G->iaj.assign(nlevels, nullptr); G->jaj.assign(nlevels, nullptr);
  G->kaj.assign(nlevels, nullptr); G->aj64.assign(nlevels, nullptr);
  for (int l = 0; l < nlevels; l++) {
    const cvb_level_desc &d = lv[l];
    const double *srcs[9] = {d.icsi, d.ieta, d.izet, d.jcsi, d.jeta, d.jzet, d.kcsi, d.keta, d.kzet};
    for (int q = 0; q < 9; q++) TRY(upload_box(ctx, *G, d, srcs[q], 3, &G->fm[l][q]));
    TRY(upload_box(ctx, *G, d, d.iaj, 1, &G->iaj[l]));
    TRY(upload_box(ctx, *G, d, d.jaj, 1, &G->jaj[l]));
    TRY(upload_box(ctx, *G, d, d.kaj, 1, &G->kaj[l]));
    TRY(upload_box(ctx, *G, d, d.aj, 1, &G->aj64[l]));
  }
  {
    const cvb_level_desc &df = lv[nlevels - 1];
    size_t n = (size_t)df.mx * df.my * df.mz;
    std::vector<double> c1, c2, c3, a3;
    extract_box(df, df.csi, 3, c1);
    extract_box(df, df.eta, 3, c2);
    extract_box(df, df.zet, 3, c3);
    face_areas(c1, c2, c3, a3);
    TRY(galloc(ctx, *G, &G->area3, 3 * n));
    CK(cudaMemcpyAsync(G->area3, a3.data(), sizeof(double) * 3 * n, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    // centre metrics for Contra2Cart and the slip faces of GhostNodeVelocity
    const std::vector<double> *cv[3] = {&c1, &c2, &c3};
    for (int c = 0; c < 3; c++) {
      TRY(galloc(ctx, *G, &G->cm[c], 3 * n));
      CK(cudaMemcpyAsync(G->cm[c], cv[c]->data(), sizeof(double) * 3 * n, cudaMemcpyHostToDevice, ctx->stream));
    }
    CK(cudaStreamSynchronize(ctx->stream));
    TRY(galloc(ctx, *G, &G->inv_aj, n));
    launch_reciprocal(G->aj64[nlevels - 1], G->inv_aj, n, ctx->stream);
    CKL();
  }
  ctx->geo = G;
  return CVB_OK;
}

int cvb_setup_hierarchy(cvb_ctx *ctx, int nlevels, const cvb_level_desc *lv, const double *nvert_finest) {
  if (!ctx) return CVB_BAD_INPUT;
  if (nlevels < 1 || nlevels > 16 || !lv || !nvert_finest) return fail(ctx, CVB_BAD_INPUT, "bad hierarchy arguments");
  const auto t0 = std::chrono::steady_clock::now();
  TRY(upload_geometry(ctx, nlevels, lv));
  ctx->setup_ms[0] = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  std::vector<double> h;
  return setup_problem(ctx, box_view(lv[nlevels - 1], nvert_finest, 1, h));
}

int cvb_setup_geometry(cvb_ctx *ctx, int nlevels, const cvb_level_desc *lv) {
  if (!ctx) return CVB_BAD_INPUT;
  if (nlevels < 1 || nlevels > 16 || !lv) return fail(ctx, CVB_BAD_INPUT, "bad hierarchy arguments");
  return upload_geometry(ctx, nlevels, lv);
}

int cvb_setup_like(cvb_ctx *ctx, const cvb_ctx *donor, const double *nvert_finest) {
  if (!ctx || !donor || ctx == donor) return CVB_BAD_INPUT;
  if (!donor->geo) return fail(ctx, CVB_NOT_SETUP, "the donor context holds no grid");
  if (!nvert_finest) return fail(ctx, CVB_BAD_INPUT, "nvert is NULL");
  if (donor->device != ctx->device)
    return fail(ctx, CVB_BAD_INPUT, "donor is on device %d, context on %d", donor->device, ctx->device);
  CK(cudaSetDevice(ctx->device));
  ensure_pool(ctx->device);
  std::shared_ptr<Geometry> G = donor->geo;  // held before free_all in case the donor is reset meanwhile
  std::vector<LevelHost> H = donor->H;
  free_all(ctx);
  ctx->nlevels = (int)H.size();
  ctx->H = H;
  ctx->geo = G;
  ctx->setup_ms[0] = 0.0;  // the grid is the donor's
  std::vector<double> h;
  return setup_problem(ctx, box_view(ctx->H[ctx->nlevels - 1].d, nvert_finest, 1, h));
}

}  // extern "C"

// Krylov basis is allocated lazily, sized by the largest restart requested.
int cvb_ensure_basis(cvb_ctx *ctx, int m, bool mixed) {
  size_t n = ctx->L[ctx->nlevels - 1].g.n();
  bool changed = false;
  for (int q = 0; q <= m; q++)
    if (!ctx->V[q]) { TRY(dalloc(ctx, &ctx->V[q], n)); changed = true; }
  for (int q = 0; q < m; q++)
    if (!ctx->Z64[q]) { TRY(dalloc(ctx, &ctx->Z64[q], n)); changed = true; }
  if (mixed && !ctx->Z32[0]) { TRY(dalloc(ctx, &ctx->Z32[0], n)); changed = true; }
  if (changed) {
    CK(cudaMemcpyAsync(ctx->dV, ctx->V, sizeof(double *) * (kMaxRestart + 1), cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(ctx->dZ64, ctx->Z64, sizeof(double *) * kMaxRestart, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(ctx->dZ32, ctx->Z32, sizeof(float *) * kMaxRestart, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
  }
  return CVB_OK;
}

static size_t fine_n(cvb_ctx *ctx) { return ctx->L[ctx->nlevels - 1].g.n(); }

extern "C" {

int cvb_set_nvert(cvb_ctx *ctx, const double *nvert_finest) {
  if (!ctx) return CVB_BAD_INPUT;
  CK(cudaSetDevice(ctx->device));
  if (!ctx->ready) return fail(ctx, CVB_NOT_SETUP, "cvb_setup_hierarchy has not run");
  if (!nvert_finest) return fail(ctx, CVB_BAD_INPUT, "nvert is NULL");
  const cvb_level_desc &df = ctx->H[ctx->nlevels - 1].d;
  std::vector<double> h;
  const double *v = box_view(df, nvert_finest, 1, h);
  TRY(check_nvert(ctx, v, (size_t)df.mx * df.my * df.mz));
  drop_vcycle_graphs(ctx);
  CK(cudaMemcpyAsync(ctx->L[ctx->nlevels - 1].nvert, v, sizeof(double) * ctx->L[ctx->nlevels - 1].g.n(),
                     cudaMemcpyHostToDevice, ctx->stream));
  using clk = std::chrono::steady_clock;
  auto ms_since = [](clk::time_point t) { return std::chrono::duration<double, std::milli>(clk::now() - t).count(); };
  CK(cudaStreamSynchronize(ctx->stream));
  ctx->setup_ms[0] = ctx->setup_ms[1] = 0.0;  // the grid and the level arrays stay
  clk::time_point t = clk::now();
  TRY(build_operators(ctx));
  ctx->setup_ms[2] = ms_since(t);
  t = clk::now();
  TRY(autotune_sweeps(ctx));
  ctx->setup_ms[3] = ms_since(t);
  t = clk::now();
  cvb_solve_opts def;
  cvb_solve_opts_default(&def);
  TRY(build_coarse(ctx, &def));
  CK(cudaStreamSynchronize(ctx->stream));
  ctx->setup_ms[4] = ms_since(t);
  return CVB_OK;
}

int cvb_level_dims(const cvb_ctx *ctx, int level, int *mx, int *my, int *mz) {
  if (!ctx || !ctx->ready || level < 0 || level >= ctx->nlevels) return CVB_BAD_INPUT;
  *mx = ctx->L[level].g.mx; *my = ctx->L[level].g.my; *mz = ctx->L[level].g.mz;
  return CVB_OK;
}

int cvb_get_nvert(cvb_ctx *ctx, int level, double *nvert, int *mns) {
  if (!ctx) return CVB_BAD_INPUT;
  if (!ctx->ready) return fail(ctx, CVB_NOT_SETUP, "cvb_setup_hierarchy has not run");
  if (level < 0 || level >= ctx->nlevels) return fail(ctx, CVB_BAD_INPUT, "bad level %d", level);
  if (nvert)
    CK(cudaMemcpy(nvert, ctx->L[level].nvert, sizeof(double) * ctx->L[level].g.n(), cudaMemcpyDeviceToHost));
  if (mns) *mns = ctx->multinullspace;
  return CVB_OK;
}

int cvb_volume_flux_rev(cvb_ctx *ctx, double *ucont, double fis, int flg, double *flux, double *area) {
  if (!ctx) return CVB_BAD_INPUT;
  if (!ctx->ready) return fail(ctx, CVB_NOT_SETUP, "cvb_setup_hierarchy has not run");
  if (!ucont) return fail(ctx, CVB_BAD_INPUT, "ucont is NULL");
  LevelDev &F = ctx->L[ctx->nlevels - 1];
  size_t n = F.g.n();
  CK(cudaMemcpyAsync(ctx->uc_dev, ucont, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, ctx->stream));
  launch_ib_sums(F.g, ctx->uc_dev, ctx->area3, nullptr, nullptr, F.nvert, ctx->partial, ctx->stream);
  launch_finish_sums(ctx->partial, 2, reduce_blocks(), ctx->sums, ctx->stream);
  launch_ib_correct(F.g, ctx->uc_dev, ctx->area3, nullptr, nullptr, F.nvert, ctx->sums, fis, flg, ctx->stream);
  launch_ib_sums(F.g, ctx->uc_dev, ctx->area3, nullptr, nullptr, F.nvert, ctx->partial, ctx->stream);
  CKL();
  double fa[2];
  TRY(reduce_to_host(ctx, 2, fa));
  CK(cudaMemcpyAsync(ucont, ctx->uc_dev, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  if (flux) *flux = fa[0];
  if (area) *area = fa[1];
  return CVB_OK;
}

int cvb_poisson_rhs(cvb_ctx *ctx, const double *ucont, double dt, double st, double *b, double *compat) {
  if (!ctx) return CVB_BAD_INPUT;
  if (!ctx->ready) return fail(ctx, CVB_NOT_SETUP, "cvb_setup_hierarchy has not run");
  if (!ucont || !b || !(dt != 0.0) || !(st != 0.0)) return fail(ctx, CVB_BAD_INPUT, "bad PoissonRHS arguments");
  LevelDev &F = ctx->L[ctx->nlevels - 1];
  size_t n = F.g.n();
  CK(cudaMemcpyAsync(ctx->uc_dev, ucont, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, ctx->stream));
  launch_poisson_rhs(F.g, ctx->uc_dev, ctx->aj64[ctx->nlevels - 1], F.nvert, dt, st, ctx->b, ctx->partial, ctx->stream);
  CKL();
  double s;
  TRY(reduce_to_host(ctx, 1, &s));
  CK(cudaMemcpy(b, ctx->b, sizeof(double) * n, cudaMemcpyDeviceToHost));
  if (compat) *compat = s;
  return CVB_OK;
}

int cvb_solve_resident(cvb_ctx *ctx, const cvb_solve_opts *o, cvb_solve_stats *st) {
  if (!ctx) return CVB_BAD_INPUT;
  if (!ctx->ready) return fail(ctx, CVB_NOT_SETUP, "cvb_setup_hierarchy has not run");
  cvb_solve_opts def;
  if (!o) { cvb_solve_opts_default(&def); o = &def; }
  TRY(cvb_ensure_basis(ctx, std::min(std::max(o->restart, 1), kMaxRestart), o->precision == CVB_PRECISION_MIXED));
  return solve_resident(ctx, o, st);
}

double *cvb_device_rhs(cvb_ctx *ctx) { return ctx && ctx->ready ? ctx->b : nullptr; }
double *cvb_device_phi(cvb_ctx *ctx) { return ctx && ctx->ready ? ctx->x : nullptr; }

int cvb_poisson_solve(cvb_ctx *ctx, const double *b, double *phi, const cvb_solve_opts *o, cvb_solve_stats *st) {
  if (!ctx) return CVB_BAD_INPUT;
  if (!ctx->ready) return fail(ctx, CVB_NOT_SETUP, "cvb_setup_hierarchy has not run");
  if (!b || !phi) return fail(ctx, CVB_BAD_INPUT, "b/phi is NULL");
  cvb_solve_opts def;
  if (!o) { cvb_solve_opts_default(&def); o = &def; }
  size_t n = fine_n(ctx);
  CK(cudaMemcpyAsync(ctx->b, b, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
  if (o->warm_start) CK(cudaMemcpyAsync(ctx->x, phi, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
  int rc = cvb_solve_resident(ctx, o, st);
  if (rc == CVB_OK || rc == CVB_NOT_CONVERGED)
    CK(cudaMemcpyAsync(phi, ctx->x, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return rc;
}

// VolumeFlux_rev, PoissonRHS and the solve.  The corrected fluxes stay on the
// device for PoissonRHS and its right-hand side for the solve; the host gets
// the corrected ucont and phi back.
int cvb_poisson_solver_mg(cvb_ctx *ctx, double *ucont, double fis, int immersed, double dt, double st, double *phi,
                          const cvb_solve_opts *o, cvb_solve_stats *stats) {
  if (!ctx) return CVB_BAD_INPUT;
  if (!phi || !(dt != 0.0) || !(st != 0.0)) return fail(ctx, CVB_BAD_INPUT, "bad PoissonSolver_MG arguments");
  double flux, area;
  TRY(cvb_volume_flux_rev(ctx, ucont, fis, immersed, &flux, &area));
  LevelDev &F = ctx->L[ctx->nlevels - 1];
  const size_t n = F.g.n();
  launch_poisson_rhs(F.g, ctx->uc_dev, ctx->aj64[ctx->nlevels - 1], F.nvert, dt, st, ctx->b, ctx->partial, ctx->stream);
  CKL();
  cvb_solve_opts def;
  if (!o) { cvb_solve_opts_default(&def); o = &def; }
  if (o->warm_start) CK(cudaMemcpyAsync(ctx->x, phi, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
  int rc = cvb_solve_resident(ctx, o, stats);
  if (rc == CVB_OK || rc == CVB_NOT_CONVERGED)
    CK(cudaMemcpyAsync(phi, ctx->x, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return rc;
}

int cvb_update_pressure(cvb_ctx *ctx, double *p, double *phi) {
  if (!ctx) return CVB_BAD_INPUT;
  if (!ctx->ready) return fail(ctx, CVB_NOT_SETUP, "cvb_setup_hierarchy has not run");
  if (!p || !phi) return fail(ctx, CVB_BAD_INPUT, "p/phi is NULL");
  LevelDev &F = ctx->L[ctx->nlevels - 1];
  size_t n = F.g.n();
  CK(cudaMemcpyAsync(ctx->p_dev, p, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(ctx->w, phi, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
  launch_update_pressure(F.g, ctx->p_dev, ctx->w, ctx->stream);
  CKL();
  CK(cudaMemcpyAsync(p, ctx->p_dev, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaMemcpyAsync(phi, ctx->w, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return CVB_OK;
}

int cvb_projection(cvb_ctx *ctx, const double *phi, double dt, double st, double *ucont) {
  if (!ctx) return CVB_BAD_INPUT;
  if (!ctx->ready) return fail(ctx, CVB_NOT_SETUP, "cvb_setup_hierarchy has not run");
  if (!phi || !ucont) return fail(ctx, CVB_BAD_INPUT, "phi/ucont is NULL");
  int l = ctx->nlevels - 1;
  LevelDev &F = ctx->L[l];
  size_t n = F.g.n();
  CK(cudaMemcpyAsync(ctx->w, phi, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(ctx->uc_dev, ucont, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, ctx->stream));
  const double *fm[9];
  for (int q = 0; q < 9; q++) fm[q] = ctx->fm[l][q];
  launch_projection(F.g, fm, ctx->iaj[l], ctx->jaj[l], ctx->kaj[l], F.nvert, ctx->w, dt, st, ctx->uc_dev, ctx->stream);
  CKL();
  CK(cudaMemcpyAsync(ucont, ctx->uc_dev, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return CVB_OK;
}

// The boundary types GhostNodeVelocity is restated for: all but an annulus
// face (bctype[2] 11) before the cell centres it reads were given
// (cvb_set_cell_centres), and periodic faces without a periodic opposite.  The
// rheology plates (13 on faces 2-5) take the velocity of
// cvb_set_plate_velocity (0 until set, as the reference's global starts).
static int ghost_types_ok(cvb_ctx *ctx, const int *bc) {
  if (bc[2] == 11 && !ctx->ibm_cent)
    return fail(ctx, CVB_BAD_INPUT,
                "GhostNodeVelocity: an annulus face (bctype 11) needs the cell centres (cvb_set_cell_centres)");
  for (int d = 0; d < 3; d++)
    if ((bc[2 * d] == 7) != (bc[2 * d + 1] == 7))
      return fail(ctx, CVB_BAD_INPUT, "GhostNodeVelocity: periodic face %d without a periodic opposite", 2 * d);
  return CVB_OK;
}

static int ensure_c2c(cvb_ctx *ctx);
static int post_buffers(cvb_ctx *ctx, size_t n) {
  if (!ctx->ucat_dev) TRY(dalloc(ctx, &ctx->ucat_dev, 3 * n));
  if (!ctx->ubcs_dev) TRY(dalloc(ctx, &ctx->ubcs_dev, 3 * n));
  return ensure_c2c(ctx);
}

int cvb_contra2cart(cvb_ctx *ctx, const double *ucont, double *ucat) {
  if (!ctx) return CVB_BAD_INPUT;
  if (!ctx->ready) return fail(ctx, CVB_NOT_SETUP, "cvb_setup_hierarchy has not run");
  if (!ucont || !ucat) return fail(ctx, CVB_BAD_INPUT, "ucont/ucat is NULL");
  LevelDev &F = ctx->L[ctx->nlevels - 1];
  const size_t n = F.g.n();
  TRY(post_buffers(ctx, n));
  CK(cudaMemcpyAsync(ctx->uc_dev, ucont, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(ctx->ucat_dev, ucat, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, ctx->stream));
  launch_contra2cart(F.g, ctx->cm[0], ctx->cm[1], ctx->cm[2], F.nvert, ctx->uc_dev, ctx->ucat_dev, ctx->stream, 1,
                     -1, ctx->geo->c2c);
  CKL();
  CK(cudaMemcpyAsync(ucat, ctx->ucat_dev, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return CVB_OK;
}

int cvb_set_cell_centres(cvb_ctx *ctx, const double *cent) {
  if (!ctx) return CVB_BAD_INPUT;
  if (!ctx->ready) return fail(ctx, CVB_NOT_SETUP, "cvb_setup_hierarchy has not run");
  if (!cent) return fail(ctx, CVB_BAD_INPUT, "cent is NULL");
  const size_t n = ctx->L[ctx->nlevels - 1].g.n();
  if (!ctx->ibm_cent) TRY(dalloc(ctx, &ctx->ibm_cent, 3 * n));
  CK(cudaMemcpyAsync(ctx->ibm_cent, cent, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return CVB_OK;
}

int cvb_set_plate_velocity(cvb_ctx *ctx, double u_bc) {
  if (!ctx) return CVB_BAD_INPUT;
  ctx->u_bc = u_bc;
  return CVB_OK;
}

int cvb_ghost_node_velocity(cvb_ctx *ctx, double *ubcs, double *ucat) {
  if (!ctx) return CVB_BAD_INPUT;
  if (!ctx->ready) return fail(ctx, CVB_NOT_SETUP, "cvb_setup_hierarchy has not run");
  if (!ubcs || !ucat) return fail(ctx, CVB_BAD_INPUT, "ubcs/ucat is NULL");
  const int *bc = ctx->H[ctx->nlevels - 1].d.bctype;
  TRY(ghost_types_ok(ctx, bc));
  LevelDev &F = ctx->L[ctx->nlevels - 1];
  const size_t n = F.g.n();
  TRY(post_buffers(ctx, n));
  CK(cudaMemcpyAsync(ctx->ubcs_dev, ubcs, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(ctx->ucat_dev, ucat, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, ctx->stream));
  launch_ghost_node_velocity(F.g, bc, ctx->cm[0], ctx->cm[1], ctx->cm[2], ctx->ubcs_dev, ctx->ucat_dev, ctx->stream,
                             ctx->ibm_cent, ctx->u_bc);
  CKL();
  CK(cudaMemcpyAsync(ubcs, ctx->ubcs_dev, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaMemcpyAsync(ucat, ctx->ucat_dev, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return CVB_OK;
}

int cvb_projection_cart(cvb_ctx *ctx, const double *phi, double dt, double st, double *ucont, double *ubcs,
                        double *ucat) {
  if (!ctx) return CVB_BAD_INPUT;
  if (!ctx->ready) return fail(ctx, CVB_NOT_SETUP, "cvb_setup_hierarchy has not run");
  if (!phi || !ucont || !ubcs || !ucat) return fail(ctx, CVB_BAD_INPUT, "phi/ucont/ubcs/ucat is NULL");
  const int l = ctx->nlevels - 1;
  const int *bc = ctx->H[l].d.bctype;
  TRY(ghost_types_ok(ctx, bc));
  LevelDev &F = ctx->L[l];
  const size_t n = F.g.n();
  TRY(post_buffers(ctx, n));
  CK(cudaMemcpyAsync(ctx->w, phi, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(ctx->uc_dev, ucont, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(ctx->ubcs_dev, ubcs, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(ctx->ucat_dev, ucat, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, ctx->stream));
  const double *fm[9];
  for (int q = 0; q < 9; q++) fm[q] = ctx->fm[l][q];
  launch_projection(F.g, fm, ctx->iaj[l], ctx->jaj[l], ctx->kaj[l], F.nvert, ctx->w, dt, st, ctx->uc_dev, ctx->stream);
  launch_contra2cart(F.g, ctx->cm[0], ctx->cm[1], ctx->cm[2], F.nvert, ctx->uc_dev, ctx->ucat_dev, ctx->stream, 1,
                     -1, ctx->geo->c2c);
  launch_ghost_node_velocity(F.g, bc, ctx->cm[0], ctx->cm[1], ctx->cm[2], ctx->ubcs_dev, ctx->ucat_dev, ctx->stream,
                             ctx->ibm_cent, ctx->u_bc);
  CKL();
  CK(cudaMemcpyAsync(ucont, ctx->uc_dev, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaMemcpyAsync(ubcs, ctx->ubcs_dev, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaMemcpyAsync(ucat, ctx->ucat_dev, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return CVB_OK;
}

int cvb_convection(cvb_ctx *ctx, const double *ucont, const double *ucat, int central, double *conv) {
  if (!ctx) return CVB_BAD_INPUT;
  if (!ctx->ready) return fail(ctx, CVB_NOT_SETUP, "cvb_setup_hierarchy has not run");
  if (!conv) return fail(ctx, CVB_BAD_INPUT, "conv is NULL");
  if (!ucat && !ctx->ucat_dev) return fail(ctx, CVB_BAD_INPUT, "ucat is NULL and no projection has left Ucat on the device");
  LevelDev &F = ctx->L[ctx->nlevels - 1];
  const size_t n = F.g.n();
  TRY(post_buffers(ctx, n));
  if (!ctx->conv_dev) TRY(dalloc(ctx, &ctx->conv_dev, 3 * n));
  if (!ctx->conv_fp) TRY(dalloc(ctx, &ctx->conv_fp, 9 * n));
  if (ucont) CK(cudaMemcpyAsync(ctx->uc_dev, ucont, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, ctx->stream));
  if (ucat) CK(cudaMemcpyAsync(ctx->ucat_dev, ucat, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, ctx->stream));
  launch_convection(F.g, ctx->uc_dev, ctx->ucat_dev, F.nvert, central != 0, ctx->conv_fp, ctx->conv_dev, ctx->stream);
  CKL();
  CK(cudaMemcpyAsync(conv, ctx->conv_dev, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return CVB_OK;
}

// The grid's Contra2Cart factors (k_c2c_factors: the metric rows' minors and
// determinant of every interior cell), formed on first use and kept with the
// grid's metrics.
static int ensure_c2c(cvb_ctx *ctx) {
  Geometry &G = *ctx->geo;
  if (G.c2c) return CVB_OK;
  const int l = ctx->nlevels - 1;
  double *fac = nullptr;
  TRY(galloc(ctx, G, &fac, 10 * ctx->L[l].g.n()));
  launch_c2c_factors(ctx->L[l].g, ctx->cm[0], ctx->cm[1], ctx->cm[2], fac, ctx->stream);
  CKL();
  CK(cudaStreamSynchronize(ctx->stream));
  G.c2c = fac;
  return CVB_OK;
}

// --- the momentum right-hand side ------------------------------------------
// The grid's face metric products (k_face_gram), formed on first use and kept
// with the grid's metrics; the stream is synchronised once so that contexts
// sharing the grid on other streams see them.
static int ensure_face_gram(cvb_ctx *ctx) {
  Geometry &G = *ctx->geo;
  if (G.gram) return CVB_OK;
  const int l = ctx->nlevels - 1;
  double *gram = nullptr;
  TRY(galloc(ctx, G, &gram, 9 * ctx->L[l].g.n()));
  const double *fm[9];
  for (int q = 0; q < 9; q++) fm[q] = ctx->fm[l][q];
  launch_face_gram(ctx->L[l].g, fm, gram, ctx->stream);
  CKL();
  CK(cudaStreamSynchronize(ctx->stream));
  G.gram = gram;
  return CVB_OK;
}

// Device inputs of FormFunction1 / CalcRHS on the finest level: ucont, ucat,
// p and the incoming rhs copied in (NULL ucont / ucat: the device copies the
// last projection left), the scratch allocated on first use.
static int momentum_prepare(cvb_ctx *ctx, const char *who, const double *ucont, const double *ucat, const double *p,
                            const double *rhs) {
  if (!ctx) return CVB_BAD_INPUT;
  if (!ctx->ready) return fail(ctx, CVB_NOT_SETUP, "cvb_setup_hierarchy has not run");
  const int *bc = ctx->H[ctx->nlevels - 1].d.bctype;
  for (int f = 0; f < 6; f++)
    if (bc[f] == 7) return fail(ctx, CVB_BAD_INPUT, "%s: periodic faces (bctype 7) are not covered", who);
  if (!p || !rhs) return fail(ctx, CVB_BAD_INPUT, "%s: p / rhs is NULL", who);
  if (!ucat && !ctx->ucat_dev) return fail(ctx, CVB_BAD_INPUT, "%s: ucat is NULL and no projection has left Ucat on the device", who);
  LevelDev &F = ctx->L[ctx->nlevels - 1];
  const size_t n = F.g.n();
  TRY(post_buffers(ctx, n));
  if (!ctx->conv_dev) TRY(dalloc(ctx, &ctx->conv_dev, 3 * n));
  if (!ctx->conv_fp) TRY(dalloc(ctx, &ctx->conv_fp, 9 * n));
  if (!ctx->visc_dev) TRY(dalloc(ctx, &ctx->visc_dev, 3 * n));
  if (!ctx->rct_dev) TRY(dalloc(ctx, &ctx->rct_dev, 3 * n));
  if (!ctx->rhs_dev) TRY(dalloc(ctx, &ctx->rhs_dev, 3 * n));
  TRY(ensure_face_gram(ctx));
  if (ucont) CK(cudaMemcpyAsync(ctx->uc_dev, ucont, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, ctx->stream));
  if (ucat) CK(cudaMemcpyAsync(ctx->ucat_dev, ucat, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(ctx->p_dev, p, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(ctx->rhs_dev, rhs, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, ctx->stream));
  return CVB_OK;
}

// FormFunction1's kernels on the device copies: Contra2Cart, Convection,
// Viscous, then the face values into rhs_dev.
// cart = false: ucat's interior already holds Contra2Cart of the current
// ucont (FormBCS ran it), so FormFunction1's own call would rewrite the same
// values.
static void momentum_ff1(cvb_ctx *ctx, double ren, int central, bool cart = true) {
  const int l = ctx->nlevels - 1;
  LevelDev &F = ctx->L[l];
  const double *fm[9];
  for (int q = 0; q < 9; q++) fm[q] = ctx->fm[l][q];
  if (cart)
    launch_contra2cart(F.g, ctx->cm[0], ctx->cm[1], ctx->cm[2], F.nvert, ctx->uc_dev, ctx->ucat_dev, ctx->stream, 1,
                     -1, ctx->geo->c2c);
  launch_convection(F.g, ctx->uc_dev, ctx->ucat_dev, F.nvert, central != 0, ctx->conv_fp, ctx->conv_dev, ctx->stream);
  launch_viscous(F.g, F.nvert, ctx->ucat_dev, fm, ctx->iaj[l], ctx->jaj[l], ctx->kaj[l], ctx->geo->gram, 1. / ren,
                 ctx->conv_fp, ctx->visc_dev, ctx->stream);
  launch_form_function1(F.g, F.nvert, ctx->p_dev, ctx->conv_dev, ctx->visc_dev, ctx->cm[0], ctx->cm[1], ctx->cm[2],
                        ctx->aj64[l], fm, ctx->iaj[l], ctx->jaj[l], ctx->kaj[l], ctx->geo->gram, ctx->rct_dev,
                        ctx->rhs_dev, ctx->stream);
}

static int momentum_finish(cvb_ctx *ctx, double *ucat, double *rhs) {
  const size_t n = ctx->L[ctx->nlevels - 1].g.n();
  CKL();
  CK(cudaMemcpyAsync(rhs, ctx->rhs_dev, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, ctx->stream));
  if (ucat) CK(cudaMemcpyAsync(ucat, ctx->ucat_dev, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return CVB_OK;
}

int cvb_viscous(cvb_ctx *ctx, const double *ucat, double ren, double *visc) {
  if (!ctx) return CVB_BAD_INPUT;
  if (!ctx->ready) return fail(ctx, CVB_NOT_SETUP, "cvb_setup_hierarchy has not run");
  if (!visc || !(ren != 0.0)) return fail(ctx, CVB_BAD_INPUT, "Viscous: visc is NULL or ren is 0");
  // periodic boxes too: Viscous reads only the box, whose ring holds the
  // periodic images (rhs.c:2062-2490)
  const int l = ctx->nlevels - 1;
  if (!ucat && !ctx->ucat_dev) return fail(ctx, CVB_BAD_INPUT, "Viscous: ucat is NULL and no projection has left Ucat on the device");
  LevelDev &F = ctx->L[l];
  const size_t n = F.g.n();
  TRY(post_buffers(ctx, n));
  if (!ctx->conv_fp) TRY(dalloc(ctx, &ctx->conv_fp, 9 * n));
  if (!ctx->visc_dev) TRY(dalloc(ctx, &ctx->visc_dev, 3 * n));
  if (ucat) CK(cudaMemcpyAsync(ctx->ucat_dev, ucat, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, ctx->stream));
  TRY(ensure_face_gram(ctx));
  const double *fm[9];
  for (int q = 0; q < 9; q++) fm[q] = ctx->fm[l][q];
  launch_viscous(F.g, F.nvert, ctx->ucat_dev, fm, ctx->iaj[l], ctx->jaj[l], ctx->kaj[l], ctx->geo->gram, 1. / ren,
                 ctx->conv_fp, ctx->visc_dev, ctx->stream);
  CKL();
  CK(cudaMemcpyAsync(visc, ctx->visc_dev, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return CVB_OK;
}

int cvb_form_function1(cvb_ctx *ctx, const double *ucont, double *ucat, const double *p, double ren, int central,
                       double *rhs) {
  TRY(momentum_prepare(ctx, "FormFunction1", ucont, ucat, p, rhs));
  if (!(ren != 0.0)) return fail(ctx, CVB_BAD_INPUT, "FormFunction1: ren is 0");
  momentum_ff1(ctx, ren, central);
  return momentum_finish(ctx, ucat, rhs);
}

int cvb_calc_rhs(cvb_ctx *ctx, const double *ucont, const double *ucont_o, const double *ucont_rm1, double *ucat,
                 const double *p, double ren, double dt, int ti, int tistart, int central, double *rhs) {
  TRY(momentum_prepare(ctx, "CalcRHS", ucont, ucat, p, rhs));
  if (!(ren != 0.0) || !(dt != 0.0) || !ucont_o || !ucont_rm1)
    return fail(ctx, CVB_BAD_INPUT, "CalcRHS: ren / dt is 0 or ucont_o / ucont_rm1 is NULL");
  const int l = ctx->nlevels - 1;
  LevelDev &F = ctx->L[l];
  const size_t n = F.g.n();
  if (!ctx->uo_dev) TRY(dalloc(ctx, &ctx->uo_dev, 3 * n));
  if (!ctx->urm_dev) TRY(dalloc(ctx, &ctx->urm_dev, 3 * n));
  CK(cudaMemcpyAsync(ctx->uo_dev, ucont_o, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(ctx->urm_dev, ucont_rm1, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, ctx->stream));
  momentum_ff1(ctx, ren, central);
  // COEF_TIME_ACCURACY is 1.5 in the reference (variables.h:421): second-order
  // backward except on the first step
  const int bdf2 = (ti != tistart && ti != 1) ? 1 : 0;
  const int mz_end = ctx->H[l].d.bctype[5] == 8 ? F.g.mz - 2 : F.g.mz - 3;
  launch_calc_rhs(F.g, F.nvert, ctx->uc_dev, ctx->uo_dev, ctx->urm_dev, bdf2, -1. / dt, mz_end, ctx->rhs_dev,
                  ctx->stream);
  return momentum_finish(ctx, ucat, rhs);
}

// --- InflowFlux, FormBCS and ImpRK --------------------------------------------
// The boxes covered: walls (1) on the x and y faces; on the k faces walls, or
// an inlet on k = 0 (5) with an outlet on the last (4).
static int bc_covered(cvb_ctx *ctx, const char *who) {
  const int *bc = ctx->H[ctx->nlevels - 1].d.bctype;
  bool ok = true;
  for (int f = 0; f < 4; f++) ok = ok && bc[f] == 1;
  ok = ok && (bc[4] == 1 || bc[4] == 5) && (bc[5] == 1 || bc[5] == 4) && ((bc[4] == 5) == (bc[5] == 4));
  if (!ok)
    return fail(ctx, CVB_BAD_INPUT,
                "%s: bctype %d %d %d %d %d %d; covered are walls (1) on the x and y faces and on the k faces walls, "
                "or an inlet (5) on k = 0 with an outlet (4) on the last",
                who, bc[0], bc[1], bc[2], bc[3], bc[4], bc[5]);
  return CVB_OK;
}

// InflowFlux's profiles (bcs.c:152-200): the constant ones (1, -1, 11) and
// the shaped ones (2, 4, 7, 10), which need the k = 0 node plane
// (cvb_set_inlet_nodes).
struct InletProfile {
  double uin = 0.;
  int profile = 0;
  bool shaped = false;
  const double *uin_cell = nullptr;
};

// Profile 10 (bcs.c:180-195): fully developed laminar flow in a square duct,
// 1 - y'^2 less the first 20 terms of its Fourier series in y' = 2 (y - 1.5),
// x' = x - 0.5, each term's factors taken left to right.  Its pow, cosh and
// cos are libm's, as the reference's, so its speeds are formed here on the
// host, once per set of nodes.
static double duct_speed(double xc, double yc) {
  const double pi = 3.14159265358979323846264338327950288;
  const double y = (yc - 1.5) * 2., x = xc - 0.5, A = 1.;
  double u = 1 - y * y;
  for (int n = 0; n < 20; n++)
    u -= 4. * pow(2. / pi, 3) * pow(-1., n) / pow(2 * n + 1., 3.) * cosh((2 * n + 1) * pi * x / 2.) *
         cos((2. * n + 1) * pi * y / 2.) / cosh((2 * n + 1) * pi * A / 2.);
  return u;
}

// InletInterpolation's table (bcs.c:67-96) at radius r and table column
// tstep: uinr [101][1001], radius 0.005 i; beyond r = 1 the speed of row 99,
// between row 100's radius and 1 zero.
static double table_speed(const double *uinr, int tstep, double r) {
  const double *U = uinr + tstep;
  if (r > 1.) return U[99 * 1001];
  for (int i = 0; i < 100; i++) {
    const double ri = i * 0.005, ri1 = (i + 1) * 0.005;
    if (r >= ri && r < ri1) return U[i * 1001] + (U[(i + 1) * 1001] - U[i * 1001]) * (r - ri) / (ri1 - ri);
  }
  return 0;
}

// The reference's table column for time step ti (bcs.c:73), -1 outside the
// table.
static int table_step(int ti) {
  const int tstep = ti / 2 - ((ti / 2000) * 2000);
  return tstep >= 0 && tstep < 1001 ? tstep : -1;
}

// Speeds per inlet face cell formed on the host: profile 10 (libm's series)
// once per set of nodes, the table profiles 0 and 5 once per set of nodes,
// table and step.
static int host_speeds(cvb_ctx *ctx, int profile) {
  const int tstep = profile == 10 ? 0 : table_step(ctx->inlet_ti);
  const int key = profile * 10000 + tstep;
  if (ctx->inlet_uin_ready && ctx->inlet_uin_key == key) return CVB_OK;
  const Geom &g = ctx->L[ctx->nlevels - 1].g;
  const int ni = g.mx - 2, nj = g.my - 2;
  const double *P = ctx->inlet_plane_host.data(), *cm = ctx->inlet_cm;
  std::vector<double> u((size_t)ni * nj);
  for (int j = 1; j <= nj; j++)
    for (int i = 1; i <= ni; i++) {
      const double *a = P + 3 * ((size_t)j * g.mx + i), *b = P + 3 * ((size_t)(j - 1) * g.mx + i);
      const double *c = P + 3 * ((size_t)j * g.mx + i - 1), *d = P + 3 * ((size_t)(j - 1) * g.mx + i - 1);
      const double xc = (a[0] + b[0] + c[0] + d[0]) * 0.25 - cm[0];
      const double yc = (a[1] + b[1] + c[1] + d[1]) * 0.25 - cm[1];
      const double zc = (a[2] + b[2] + c[2] + d[2]) * 0.25 - cm[2];
      double s;
      if (profile == 10) {
        s = duct_speed(xc, yc);
      } else {
        s = table_speed(ctx->inlet_table.data(), tstep, sqrt(zc * zc + yc * yc));
        if (profile == 5) s = -s;
      }
      u[(size_t)(j - 1) * ni + i - 1] = s;
    }
  if (!ctx->inlet_uin) TRY(dalloc(ctx, &ctx->inlet_uin, u.size()));
  CK(cudaMemcpyAsync(ctx->inlet_uin, u.data(), sizeof(double) * u.size(), cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  ctx->inlet_uin_ready = true;
  ctx->inlet_uin_key = key;
  return CVB_OK;
}

static int inlet_speed(cvb_ctx *ctx, int profile, InletProfile *ip) {
  ip->profile = profile;
  ip->shaped = profile == 2 || profile == 4 || profile == 7 || profile == 10 || profile == 0 || profile == 5;
  if (profile == 1) ip->uin = 2.;
  else if (profile == -1) ip->uin = -1.;
  else if (profile == 11) ip->uin = 0.185;
  else if (profile == 3 || profile == 6) ip->uin = ctx->inlet_flux_in;
  else if (profile == 8)  // InletInterpolation (bcs.c:75-77) also leaves it in Flux_in
    ip->uin = ctx->inlet_flux_in = sin(2 * 3.14159 * ctx->inlet_ti / 200.);
  else if (!ip->shaped)
    return fail(ctx, CVB_BAD_INPUT,
                "InflowFlux: inletprofile %d is not covered (uniform profiles 1, -1, 11, 3, 6, 8, shaped 2, 4, 7, "
                "10 and the table's 0, 5 are)",
                profile);
  else if (!ctx->inlet_coor)
    return fail(ctx, CVB_BAD_INPUT, "InflowFlux: inletprofile %d needs the inlet's nodes (cvb_set_inlet_nodes)",
                profile);
  if (profile == 0 || profile == 5) {
    if (ctx->inlet_table.empty())
      return fail(ctx, CVB_BAD_INPUT, "InflowFlux: inletprofile %d needs the inlet table (cvb_set_inlet_table)",
                  profile);
    if (table_step(ctx->inlet_ti) < 0)
      return fail(ctx, CVB_BAD_INPUT,
                  "InflowFlux: inletprofile %d at ti %d: the table column ti/2 - (ti/2000) 2000 is outside the table",
                  profile, ctx->inlet_ti);
  }
  if (profile == 10 || profile == 0 || profile == 5) {
    TRY(host_speeds(ctx, profile));
    ip->uin_cell = ctx->inlet_uin;
  }
  return CVB_OK;
}

int cvb_set_inlet_flux(cvb_ctx *ctx, double flux_in, int ti) {
  if (!ctx) return CVB_BAD_INPUT;
  ctx->inlet_flux_in = flux_in;
  ctx->inlet_ti = ti;
  return CVB_OK;
}

double cvb_inlet_flux_in(const cvb_ctx *ctx) { return ctx ? ctx->inlet_flux_in : 0.; }

int cvb_set_inlet_table(cvb_ctx *ctx, const double *uinr) {
  if (!ctx) return CVB_BAD_INPUT;
  if (!uinr) return fail(ctx, CVB_BAD_INPUT, "uinr is NULL");
  ctx->inlet_table.assign(uinr, uinr + 101 * 1001);
  ctx->inlet_uin_ready = false;
  return CVB_OK;
}

int cvb_set_inlet_nodes(cvb_ctx *ctx, const double *coor0, double cmx, double cmy, double cmz) {
  if (!ctx) return CVB_BAD_INPUT;
  if (!ctx->ready) return fail(ctx, CVB_NOT_SETUP, "cvb_setup_hierarchy has not run");
  if (!coor0) return fail(ctx, CVB_BAD_INPUT, "coor0 is NULL");
  const Geom &g = ctx->L[ctx->nlevels - 1].g;
  const size_t n = (size_t)3 * g.mx * g.my;
  if (!ctx->inlet_coor) TRY(dalloc(ctx, &ctx->inlet_coor, n));
  CK(cudaMemcpyAsync(ctx->inlet_coor, coor0, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  ctx->inlet_plane_host.assign(coor0, coor0 + n);
  ctx->inlet_uin_ready = false;
  ctx->inlet_cm[0] = cmx;
  ctx->inlet_cm[1] = cmy;
  ctx->inlet_cm[2] = cmz;
  return CVB_OK;
}

static int bc_buffers(cvb_ctx *ctx) {
  const Geom &g = ctx->L[ctx->nlevels - 1].g;
  const size_t n2 = (size_t)(g.mx - 2) * (g.my - 2);
  if (!ctx->bc_scratch) TRY(dalloc(ctx, &ctx->bc_scratch, 2 * n2));
  if (!ctx->bc_host) {
    if (cudaMallocHost((void **)&ctx->bc_host, sizeof(double) * 2 * n2) != cudaSuccess) {
      cudaGetLastError();
      ctx->bc_host = nullptr;
      return fail(ctx, CVB_OOM, "pinned host buffer of %zu bytes failed", sizeof(double) * 2 * n2);
    }
  }
  return CVB_OK;
}

// The reference adds a plane's terms one after another in its (j, i) loop;
// the host does the same with the terms the kernels wrote in that order (a
// chain of dependent FP64 adds is far slower on the GPU).
static double ordered_sum(const double *t, size_t n) {
  double s = 0.;
  for (size_t q = 0; q < n; q++) s += t[q];
  return s;
}

// What InflowFlux leaves for FormBCS's outlet: FluxInSum, and the outlet's
// area (a sum over its fluid cells' |zet|, the same in every pass).
struct BcSums {
  double flux_in = 0.;
  bool have_flux_in = false;
  double area = 0.;
  bool have_area = false;
  int rc = CVB_OK;
};

// InflowFlux: the inlet face's ubcs and Ucont.z, and FluxInSum (summed once:
// its terms depend on the grid and nvert alone).
static int inflow_dev(cvb_ctx *ctx, const InletProfile &ip, BcSums &bs) {
  LevelDev &F = ctx->L[ctx->nlevels - 1];
  const size_t n2 = (size_t)(F.g.mx - 2) * (F.g.my - 2);
  launch_inflow(F.g, F.nvert, ctx->cm[2], ip.uin, ip.shaped ? ctx->inlet_coor : nullptr, ip.profile,
                ctx->inlet_cm[1], ctx->inlet_cm[2], ip.uin_cell, ctx->uc_dev, ctx->ubcs_dev, ctx->bc_scratch,
                ctx->stream);
  if (bs.have_flux_in) return CVB_OK;
  CKL();
  CK(cudaMemcpyAsync(ctx->bc_host, ctx->bc_scratch, sizeof(double) * n2, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  bs.flux_in = ordered_sum(ctx->bc_host, n2);
  bs.have_flux_in = true;
  return CVB_OK;
}

// FormBCS's three passes; with an outlet each pass sums its flux on the host
// and hands the kernel the ratio (bcs.c:4952-4956: FluxIn = FluxInSum +
// FarFluxInSum (0: no far-field face) + FluxIntpSum).
static int form_bcs_dev(cvb_ctx *ctx, double flux_intp_sum, BcSums &bs) {
  LevelDev &F = ctx->L[ctx->nlevels - 1];
  const Geom &g = F.g;
  const size_t n2 = (size_t)(g.mx - 2) * (g.my - 2);
  std::function<void()> outlet;
  if (ctx->H[ctx->nlevels - 1].d.bctype[5] == 4)
    outlet = [ctx, &F, &g, n2, flux_intp_sum, &bs]() {
      if (bs.rc) return;
      launch_outlet_terms(g, F.nvert, ctx->cm[2], ctx->ucat_dev, ctx->bc_scratch, ctx->stream);
      const size_t nt = bs.have_area ? n2 : 2 * n2;
      if (cudaMemcpyAsync(ctx->bc_host, ctx->bc_scratch, sizeof(double) * nt, cudaMemcpyDeviceToHost, ctx->stream) !=
              cudaSuccess ||
          cudaStreamSynchronize(ctx->stream) != cudaSuccess) {
        bs.rc = fail(ctx, CVB_CUDA_ERROR, "FormBCS outlet: %s", cudaGetErrorString(cudaGetLastError()));
        return;
      }
      const double flux_out = ordered_sum(ctx->bc_host, n2);
      if (!bs.have_area) {
        bs.area = ordered_sum(ctx->bc_host + n2, n2);
        bs.have_area = true;
      }
      const double flux_in = bs.flux_in + 0. + flux_intp_sum;
      const double ratio = (flux_in - flux_out) / bs.area;
      launch_outlet_apply(g, F.nvert, ctx->cm[2], ctx->ucat_dev, ratio, ctx->uc_dev, ctx->ubcs_dev, ctx->stream);
    };
  launch_form_bcs(g, ctx->cm[0], ctx->cm[1], ctx->cm[2], ctx->geo->c2c, F.nvert, ctx->uc_dev, ctx->ubcs_dev,
                  ctx->ucat_dev, ctx->p_dev, outlet, ctx->stream);
  return bs.rc;
}

int cvb_inflow_flux(cvb_ctx *ctx, double *ucont, double *ubcs, int inletprofile, double *flux_in_sum) {
  if (!ctx) return CVB_BAD_INPUT;
  if (!ctx->ready) return fail(ctx, CVB_NOT_SETUP, "cvb_setup_hierarchy has not run");
  if (!ucont || !ubcs || !flux_in_sum) return fail(ctx, CVB_BAD_INPUT, "InflowFlux: ucont/ubcs/flux_in_sum is NULL");
  TRY(bc_covered(ctx, "InflowFlux"));
  if (ctx->H[ctx->nlevels - 1].d.bctype[4] != 5) return CVB_OK;  // FluxIn 0; FluxInSum keeps its value
  InletProfile uin;
  TRY(inlet_speed(ctx, inletprofile, &uin));
  const size_t n = ctx->L[ctx->nlevels - 1].g.n();
  TRY(post_buffers(ctx, n));
  TRY(bc_buffers(ctx));
  CK(cudaMemcpyAsync(ctx->uc_dev, ucont, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(ctx->ubcs_dev, ubcs, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, ctx->stream));
  BcSums bs;
  TRY(inflow_dev(ctx, uin, bs));
  CKL();
  CK(cudaMemcpyAsync(ucont, ctx->uc_dev, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaMemcpyAsync(ubcs, ctx->ubcs_dev, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  *flux_in_sum = bs.flux_in;
  return CVB_OK;
}

int cvb_form_bcs(cvb_ctx *ctx, double *ucont, double *ubcs, double *ucat, double *p, double flux_in_sum,
                 double flux_intp_sum) {
  if (!ctx) return CVB_BAD_INPUT;
  if (!ctx->ready) return fail(ctx, CVB_NOT_SETUP, "cvb_setup_hierarchy has not run");
  if (!ucont || !ubcs || !ucat || !p) return fail(ctx, CVB_BAD_INPUT, "FormBCS: ucont/ubcs/ucat/p is NULL");
  TRY(bc_covered(ctx, "FormBCS"));
  const size_t n = ctx->L[ctx->nlevels - 1].g.n();
  TRY(post_buffers(ctx, n));
  TRY(bc_buffers(ctx));
  CK(cudaMemcpyAsync(ctx->uc_dev, ucont, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(ctx->ubcs_dev, ubcs, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(ctx->ucat_dev, ucat, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(ctx->p_dev, p, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
  BcSums bs;
  bs.flux_in = flux_in_sum;
  bs.have_flux_in = true;
  TRY(form_bcs_dev(ctx, flux_intp_sum, bs));
  CKL();
  CK(cudaMemcpyAsync(ucont, ctx->uc_dev, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaMemcpyAsync(ubcs, ctx->ubcs_dev, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaMemcpyAsync(ucat, ctx->ucat_dev, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaMemcpyAsync(p, ctx->p_dev, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return CVB_OK;
}

// The two norms of k_imp_norms, back on the host.
static int imp_norms(cvb_ctx *ctx, size_t n3, bool du, double *f, double *d) {
  launch_imp_norms(n3, ctx->rhs_dev, du ? ctx->pu_dev : nullptr, ctx->uc_dev, ctx->imp_norms, ctx->stream);
  CKL();
  unsigned long long h[2];
  CK(cudaMemcpyAsync(h, ctx->imp_norms, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  std::memcpy(f, &h[0], sizeof(double));
  if (d) std::memcpy(d, &h[1], sizeof(double));
  return CVB_OK;
}

void cvb_imp_rk_opts_default(cvb_imp_rk_opts *o) {
  if (!o) return;
  o->ren = 1.;
  o->dt = 1.;
  o->st = 1.;
  o->cfl = 0.2;        // init.c:54
  o->ti = 1;
  o->tistart = 0;
  o->central = 0;
  o->imp_atol = 1e-7;  // main.c:26
  o->imp_rtol = 1e-4;
  o->imp_max_it = 50;  // main.c:21
  o->inletprofile = 1;
  o->flux_intp_sum = 0.;
}

int cvb_imp_rk(cvb_ctx *ctx, double *ucont, const double *ucont_o, const double *ucont_rm1, double *ucat, double *p,
               double *ubcs, const cvb_imp_rk_opts *o, cvb_imp_rk_stats *stats) {
  if (!ctx) return CVB_BAD_INPUT;
  if (!ctx->ready) return fail(ctx, CVB_NOT_SETUP, "cvb_setup_hierarchy has not run");
  if (!ucont || !ucont_o || !ucont_rm1 || !ucat || !p || !ubcs || !o)
    return fail(ctx, CVB_BAD_INPUT, "ImpRK: ucont/ucont_o/ucont_rm1/ucat/p/ubcs/opts is NULL");
  const double ren = o->ren, dt = o->dt, st = o->st, cfl = o->cfl, imp_atol = o->imp_atol, imp_rtol = o->imp_rtol;
  const int ti = o->ti, tistart = o->tistart, central = o->central, imp_max_it = o->imp_max_it;
  if (!(ren != 0.0) || !(dt != 0.0)) return fail(ctx, CVB_BAD_INPUT, "ImpRK: ren / dt is 0");
  TRY(bc_covered(ctx, "ImpRK"));
  const bool inlet = ctx->H[ctx->nlevels - 1].d.bctype[4] == 5;
  InletProfile uin;
  ctx->inlet_ti = ti;  // InletInterpolation reads the global ti
  if (inlet) TRY(inlet_speed(ctx, o->inletprofile, &uin));
  const int l = ctx->nlevels - 1;
  LevelDev &F = ctx->L[l];
  const size_t n = F.g.n(), n3 = 3 * n;
  TRY(post_buffers(ctx, n));
  if (!ctx->conv_dev) TRY(dalloc(ctx, &ctx->conv_dev, n3));
  if (!ctx->conv_fp) TRY(dalloc(ctx, &ctx->conv_fp, 9 * n));
  if (!ctx->visc_dev) TRY(dalloc(ctx, &ctx->visc_dev, n3));
  if (!ctx->rct_dev) TRY(dalloc(ctx, &ctx->rct_dev, n3));
  if (!ctx->rhs_dev) TRY(dalloc(ctx, &ctx->rhs_dev, n3));
  if (!ctx->uo_dev) TRY(dalloc(ctx, &ctx->uo_dev, n3));
  if (!ctx->urm_dev) TRY(dalloc(ctx, &ctx->urm_dev, n3));
  if (!ctx->pu_dev) TRY(dalloc(ctx, &ctx->pu_dev, n3));
  if (!ctx->imp_norms) TRY(dalloc(ctx, &ctx->imp_norms, 2));
  TRY(bc_buffers(ctx));
  TRY(ensure_face_gram(ctx));
  CK(cudaMemcpyAsync(ctx->uc_dev, ucont, sizeof(double) * n3, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(ctx->uo_dev, ucont_o, sizeof(double) * n3, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(ctx->urm_dev, ucont_rm1, sizeof(double) * n3, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(ctx->ucat_dev, ucat, sizeof(double) * n3, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(ctx->p_dev, p, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(ctx->ubcs_dev, ubcs, sizeof(double) * n3, cudaMemcpyHostToDevice, ctx->stream));
  // InflowFlux (a wall k = 0 face: nothing), OutflowFlux (it only sums a flux
  // nothing here reads), FormBCS
  BcSums bs;
  auto boundary = [&]() -> int {
    if (inlet) TRY(inflow_dev(ctx, uin, bs));
    return form_bcs_dev(ctx, o->flux_intp_sum, bs);
  };
  // Rhs starts at 0 (VecSet, implicitsolver.c:7140); CalcRHS leaves part of
  // its ring as it was
  CK(cudaMemsetAsync(ctx->rhs_dev, 0, sizeof(double) * n3, ctx->stream));
  const int bdf2 = (ti != tistart && ti != 1) ? 1 : 0;  // COEF_TIME_ACCURACY 1.5 (variables.h:421)
  const int mz_end = F.g.mz - 3;                        // no convective outflow on an all-wall box
  auto calc_rhs = [&]() {
    momentum_ff1(ctx, ren, central, false);
    launch_calc_rhs(F.g, F.nvert, ctx->uc_dev, ctx->uo_dev, ctx->urm_dev, bdf2, -1. / dt, mz_end, ctx->rhs_dev,
                    ctx->stream);
  };
  // before the loop (implicitsolver.c:7124-7148): the boundary conditions,
  // pUcont = Ucont, CalcRHS
  TRY(boundary());
  CK(cudaMemcpyAsync(ctx->pu_dev, ctx->uc_dev, sizeof(double) * n3, cudaMemcpyDeviceToDevice, ctx->stream));
  calc_rhs();
  double normF0, normF1 = 1000., normdU1 = 1000., lambda = cfl;
  TRY(imp_norms(ctx, n3, false, &normF0, nullptr));
  const double alfa[4] = {0.25, 1 / 3., 0.5, 1.};  // implicitsolver.c:7111
  double normdU = 10., reldU = 1., normdU_bk = 0., reldU_bk = 1., normdU0 = 0., normF_bk = 0., relF_bk = 0.;
  int pseudot = 0, rejected = 0;
  // implicitsolver.c:7149-7239; the loop ends: pseudot grows by one per kept
  // iteration, and an undone one halves lambda, which stops at 0.001
  while (((normdU > imp_atol && reldU > imp_rtol) || pseudot < 1) && pseudot < imp_max_it) {
    pseudot++;
    for (int s = 0; s < 4; s++) {
      const double a = lambda * alfa[s] * dt * st;
      launch_imp_waxpy(n3, a, ctx->rhs_dev, ctx->pu_dev, ctx->uc_dev, ctx->stream);
      TRY(boundary());
      calc_rhs();
    }
    normdU1 = normdU_bk;
    const double normF_prev = normF_bk;
    TRY(imp_norms(ctx, n3, true, &normF_bk, &normdU_bk));
    if (pseudot == 1) {
      normdU0 = normdU_bk;
      reldU_bk = 1.;
    } else if (normdU0 > 1.e-10) {
      reldU_bk = normdU_bk / normdU0;
    }
    // normF1 takes the previous iteration's |Rhs|, as the reference orders
    // its statements (implicitsolver.c:7196-7197)
    if (pseudot > 1) normF1 = normF_prev;
    if (pseudot == 1) normF0 = normF_bk;
    relF_bk = normF_bk / normF0;
    normdU = normdU_bk;
    reldU = reldU_bk;
    if (pseudot > 1 && normF_bk > normF1 && normdU_bk > normdU1 && lambda > 0.001) {
      lambda = 0.5 * lambda;
      pseudot--;
      rejected++;
      CK(cudaMemcpyAsync(ctx->uc_dev, ctx->pu_dev, sizeof(double) * n3, cudaMemcpyDeviceToDevice, ctx->stream));
    } else {
      CK(cudaMemcpyAsync(ctx->pu_dev, ctx->uc_dev, sizeof(double) * n3, cudaMemcpyDeviceToDevice, ctx->stream));
      normF1 = normF_bk;
      normdU1 = normdU_bk;
    }
  }
  CKL();
  CK(cudaMemcpyAsync(ucont, ctx->uc_dev, sizeof(double) * n3, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaMemcpyAsync(ucat, ctx->ucat_dev, sizeof(double) * n3, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaMemcpyAsync(p, ctx->p_dev, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaMemcpyAsync(ubcs, ctx->ubcs_dev, sizeof(double) * n3, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  if (stats) {
    stats->flux_in_sum = bs.flux_in;
    stats->pseudo_iterations = pseudot;
    stats->rejected = rejected;
    stats->norm_du = normdU;
    stats->rel_du = reldU;
    stats->norm_f = normF_bk;
    stats->rel_f = relF_bk;
    stats->lambda = lambda;
  }
  return CVB_OK;
}

// Divergence (flow) or MetricsDivergence (metrics) of the finest level.
static int max_divergence(cvb_ctx *ctx, bool metrics, const double *ucont, double *maxdiv, long long *at) {
  if (!ctx) return CVB_BAD_INPUT;
  if (!ctx->ready) return fail(ctx, CVB_NOT_SETUP, "cvb_setup_hierarchy has not run");
  if (!maxdiv || !at) return fail(ctx, CVB_BAD_INPUT, "maxdiv/at is NULL");
  const int l = ctx->nlevels - 1;
  LevelDev &F = ctx->L[l];
  const size_t n = F.g.n();
  if (ucont) CK(cudaMemcpyAsync(ctx->uc_dev, ucont, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, ctx->stream));
  // 1024 partial (value, index) pairs and the result, from the pool for this call
  double *pv = nullptr;
  TRY(dalloc(ctx, &pv, 2 * 1024 + 2));
  long long *pi = reinterpret_cast<long long *>(pv + 1024);
  double *out = pv + 2048;
  if (metrics)
    launch_metrics_divergence(F.g, ctx->cm[0], ctx->cm[1], ctx->cm[2], ctx->aj64[l], pv, pi, out,
                              reinterpret_cast<long long *>(out + 1), ctx->stream);
  else
    launch_divergence(F.g, ctx->uc_dev, ctx->aj64[l], F.nvert, pv, pi, out, reinterpret_cast<long long *>(out + 1),
                      ctx->stream);
  double h[2];
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(h, out, sizeof h, cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  dfree(ctx, pv);
  if (e != cudaSuccess) return fail(ctx, CVB_CUDA_ERROR, "divergence: %s", cudaGetErrorString(e));
  *maxdiv = h[0];
  std::memcpy(at, h + 1, sizeof(long long));
  return CVB_OK;
}

int cvb_divergence(cvb_ctx *ctx, const double *ucont, double *maxdiv, long long *at) {
  return max_divergence(ctx, false, ucont, maxdiv, at);
}

int cvb_metrics_divergence(cvb_ctx *ctx, double *maxdiv, long long *at) {
  return max_divergence(ctx, true, nullptr, maxdiv, at);
}

// randomdirection's ray offsets (ibm.c:101-104): the first rand() after
// srand(seed), scaled to [-0.5, 0.5), for seeds 1 .. n.  They are drawn from a
// private generator state (initstate / random / setstate; in glibc rand() is
// random() and srand() seeds the same kind of state), so the caller's own
// rand() sequence is left where it was.
int cvb_ibm_ray_offsets(int n, double *s) {
  if (n < 0 || (n > 0 && !s)) return CVB_BAD_INPUT;
  static std::mutex mu;
  std::lock_guard<std::mutex> lock(mu);
  alignas(16) static char state[128];
  char *prev = nullptr;
  for (int q = 0; q < n; q++) {
    char *old = initstate((unsigned)(q + 1), state, sizeof state);
    if (q == 0) prev = old;
    s[q] = random() / ((double)RAND_MAX + 1) - 0.5;
  }
  if (prev) setstate(prev);
  return CVB_OK;
}

int cvb_ibm_search(cvb_ctx *ctx, const double *cent, int n_v, const double *xyz, int n_elmt, const int *tri,
                   const double *nf, int ibi, int nbodies, const double *nvert_o, double *nvert) {
  if (!ctx) return CVB_BAD_INPUT;
  if (!ctx->ready) return fail(ctx, CVB_NOT_SETUP, "cvb_setup_hierarchy has not run");
  if (!xyz || !tri || !nf || !nvert_o || !nvert) return fail(ctx, CVB_BAD_INPUT, "NULL array");
  if (!cent && !ctx->ibm_cent) return fail(ctx, CVB_BAD_INPUT, "cent is NULL and no earlier call gave the centres");
  if (n_v < 3 || n_elmt < 1) return fail(ctx, CVB_BAD_INPUT, "a body needs 3 nodes and 1 triangle");
  if (nbodies < 1 || ibi < 0 || ibi >= nbodies) return fail(ctx, CVB_BAD_INPUT, "body %d of %d", ibi, nbodies);
  for (long e = 0; e < 3L * n_elmt; e++)
    if (tri[e] < 0 || tri[e] >= n_v) return fail(ctx, CVB_BAD_INPUT, "triangle %ld names node %d", e / 3, tri[e]);
  LevelDev &F = ctx->L[ctx->nlevels - 1];
  const size_t n = F.g.n();
  IbmArgs A;
  std::memset(&A, 0, sizeof A);
  A.g = F.g;
  // bounding box and buckets (ibm.c:4250-4318)
  for (int c = 0; c < 3; c++) { A.min[c] = 1.e23; A.max[c] = -1.e23; }
  for (int q = 0; q < n_v; q++)
    for (int c = 0; c < 3; c++) {
      const double x = xyz[3 * q + c];
      A.min[c] = A.min[c] < x ? A.min[c] : x;
      A.max[c] = A.max[c] < x ? x : A.max[c];
    }
  for (int c = 0; c < 3; c++) {
    A.dc[c] = (A.max[c] - A.min[c]) / (kIbmBuckets - 1.);
    if (!(A.dc[c] > 0)) return fail(ctx, CVB_BAD_INPUT, "the body is flat in direction %d", c);
  }
  // each triangle's bucket ranges; the column lists keep, per (i, k) column,
  // its triangles and the end of their range in j
  const int ncol = kIbmBuckets * kIbmBuckets;
  std::vector<int> start(ncol + 1, 0);
  std::vector<std::array<int, 6>> rng(n_elmt);
  for (int e = 0; e < n_elmt; e++) {
    for (int c = 0; c < 3; c++) {
      const double a = xyz[3 * tri[3 * e] + c], b = xyz[3 * tri[3 * e + 1] + c], d = xyz[3 * tri[3 * e + 2] + c];
      double lo = a < b ? a : b, hi = a < b ? b : a;
      lo = lo < d ? lo : d;
      hi = hi < d ? d : hi;
      const int imin = (int)std::floor((lo - A.min[c]) / A.dc[c]);
      const int imax = (int)std::floor((hi - A.min[c]) / A.dc[c]) + 1;
      rng[e][2 * c] = imin < 0 ? 0 : imin;
      rng[e][2 * c + 1] = imax > kIbmBuckets ? kIbmBuckets : imax;
    }
    if (rng[e][2] >= rng[e][3]) continue;
    for (int k = rng[e][4]; k < rng[e][5]; k++)
      for (int i = rng[e][0]; i < rng[e][1]; i++) start[k * kIbmBuckets + i + 1]++;
  }
  for (int q = 0; q < ncol; q++) start[q + 1] += start[q];
  std::vector<int2> ent(std::max(start[ncol], 1));
  {
    std::vector<int> fill(ncol, 0);
    for (int e = 0; e < n_elmt; e++) {
      if (rng[e][2] >= rng[e][3]) continue;
      for (int k = rng[e][4]; k < rng[e][5]; k++)
        for (int i = rng[e][0]; i < rng[e][1]; i++) {
          const int col = k * kIbmBuckets + i;
          ent[start[col] + fill[col]++] = make_int2(e, rng[e][3]);
        }
    }
  }
  // per triangle: v0, the edges v1 - v0 and v2 - v0 (the subtractions the ray
  // test would repeat for every ray), the unit normal
  std::vector<double> tdata(12 * (size_t)n_elmt);
  for (int e = 0; e < n_elmt; e++) {
    const double *v0 = xyz + 3 * tri[3 * e], *v1 = xyz + 3 * tri[3 * e + 1], *v2 = xyz + 3 * tri[3 * e + 2];
    double *T = tdata.data() + 12 * (size_t)e;
    for (int c = 0; c < 3; c++) {
      T[c] = v0[c];
      T[3 + c] = v1[c] - v0[c];
      T[6 + c] = v2[c] - v0[c];
      T[9 + c] = nf[3 * e + c];
    }
  }
  double off[kIbmMaxTries];
  cvb_ibm_ray_offsets(kIbmMaxTries, off);
  // device copies, from the context's pool for this call
  // the cell centres stay on the device for later calls with cent == NULL
  if (!ctx->ibm_cent) TRY(dalloc(ctx, &ctx->ibm_cent, 3 * n));
  double *d_cent = ctx->ibm_cent;
  double *d_nv = nullptr, *d_nvo = nullptr, *d_tmp = nullptr, *d_tri = nullptr, *d_off = nullptr;
  int *d_start = nullptr, *d_flag = nullptr, *d_work = nullptr;
  int2 *d_ent = nullptr;
  void *bufs[10] = {};
  int rc = CVB_OK;
  auto release = [&]() {
    for (void *b : bufs)
      if (b) dfree(ctx, b);
  };
  rc = dalloc(ctx, &d_nv, n);
  if (!rc) { bufs[1] = d_nv; rc = dalloc(ctx, &d_nvo, n); }
  if (!rc) { bufs[2] = d_nvo; rc = dalloc(ctx, &d_tmp, n); }
  if (!rc) { bufs[3] = d_tmp; rc = dalloc(ctx, &d_tri, tdata.size()); }
  if (!rc) { bufs[4] = d_tri; rc = dalloc(ctx, &d_off, (size_t)kIbmMaxTries); }
  if (!rc) { bufs[5] = d_off; rc = dalloc(ctx, &d_start, start.size()); }
  if (!rc) { bufs[6] = d_start; rc = dalloc(ctx, &d_ent, ent.size()); }
  if (!rc) { bufs[7] = d_ent; rc = dalloc(ctx, &d_flag, 1); }
  // key and list per interior cell, count / start / fill per column, a total
  const size_t inner = (size_t)(F.g.mx - 2) * (F.g.my - 2) * (F.g.mz - 2);
  if (!rc) { bufs[8] = d_flag; rc = dalloc(ctx, &d_work, 2 * inner + 3 * (size_t)ncol + 1 + (n + 3) / 4); }
  if (rc) {
    release();
    return rc;
  }
  bufs[9] = d_work;
  IbmWork W;
  W.key = d_work;
  W.list = d_work + inner;
  W.count = d_work + 2 * inner;
  W.start = W.count + ncol;
  W.fill = W.start + ncol;
  W.total = W.fill + ncol;
  W.in4 = reinterpret_cast<unsigned char *>(W.total + 1);
  cudaStream_t s = ctx->stream;
  if (cent) CK(cudaMemcpyAsync(d_cent, cent, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(d_nv, nvert, sizeof(double) * n, cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(d_nvo, nvert_o, sizeof(double) * n, cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(d_tri, tdata.data(), sizeof(double) * tdata.size(), cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(d_off, off, sizeof off, cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(d_start, start.data(), sizeof(int) * start.size(), cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(d_ent, ent.data(), sizeof(int2) * ent.size(), cudaMemcpyHostToDevice, s));
  CK(cudaMemsetAsync(d_flag, 0, sizeof(int), s));
  A.col_start = d_start; A.col_ent = d_ent; A.tri = d_tri; A.offsets = d_off; A.tries = kIbmMaxTries;
  A.cent = d_cent; A.nvert = d_nv; A.nvert_o = d_nvo; A.ibi = ibi; A.nbodies = nbodies; A.failed = d_flag;
  launch_ibm_search(A, W, d_tmp, s);
  CKL();
  int flag = 0;
  CK(cudaMemcpyAsync(&flag, d_flag, sizeof(int), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  if (flag) {
    release();
    return fail(ctx, CVB_NOT_CONVERGED,
                "IB search: a cell centre found no ray clear of edges and vertices in %d directions", kIbmMaxTries);
  }
  CK(cudaMemcpyAsync(nvert, d_tmp, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  release();
  return CVB_OK;
}

static int level_ok(cvb_ctx *ctx, int level) {
  if (!ctx) return CVB_BAD_INPUT;
  if (!ctx->ready) return fail(ctx, CVB_NOT_SETUP, "cvb_setup_hierarchy has not run");
  if (level < 0 || level >= ctx->nlevels) return fail(ctx, CVB_BAD_INPUT, "bad level %d", level);
  return CVB_OK;
}

int cvb_apply_operator(cvb_ctx *ctx, int level, const double *x, double *y) {
  TRY(level_ok(ctx, level));
  LevelDev &L = ctx->L[level];
  size_t n = L.g.n();
  CK(cudaMemcpyAsync(L.r64, x, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
  launch_apply<double>(L, L.r64, L.e64, ctx->stream);
  CKL();
  CK(cudaMemcpyAsync(y, L.e64, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return CVB_OK;
}

int cvb_apply_operator_f32(cvb_ctx *ctx, int level, const float *x, float *y) {
  TRY(level_ok(ctx, level));
  LevelDev &L = ctx->L[level];
  size_t n = L.g.n();
  CK(cudaMemcpyAsync(L.r32, x, sizeof(float) * n, cudaMemcpyHostToDevice, ctx->stream));
  launch_apply<float>(L, L.r32, L.e32, ctx->stream);
  CKL();
  CK(cudaMemcpyAsync(y, L.e32, sizeof(float) * n, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return CVB_OK;
}

int cvb_zebra_half_f32(cvb_ctx *ctx, int level, int form, int color, float omega, const float *b, float *x) {
  TRY(level_ok(ctx, level));
  LevelDev &L = ctx->L[level];
  if (color != 0 && color != 1) return fail(ctx, CVB_BAD_INPUT, "colour %d is not 0 or 1", color);
  const int keep_tma = L.ztma32, keep_fuse = L.zfuse32, keep_tw = L.ztw32;
  L.ztw32 = 0;
  switch (form) {
    case CVB_ZEBRA_SPLIT: L.ztma32 = 0; L.zfuse32 = 0; break;
    case CVB_ZEBRA_FUSED: L.ztma32 = 0; L.zfuse32 = 1; break;
    case CVB_ZEBRA_SPLIT4: L.ztma32 = 0; L.zfuse32 = 0; L.ztw32 = 4; break;
    case CVB_ZEBRA_FUSED4: L.ztma32 = 0; L.zfuse32 = 1; L.ztw32 = 4; break;
    case CVB_ZEBRA_TMA4: case CVB_ZEBRA_TMA8: case CVB_ZEBRA_TMA16: L.ztma32 = form; L.zfuse32 = 0; break;
    default: return fail(ctx, CVB_BAD_INPUT, "unknown zebra form %d", form);
  }
  const bool ok = form == CVB_ZEBRA_SPLIT || form == CVB_ZEBRA_SPLIT4 ? true
                  : form == CVB_ZEBRA_FUSED || form == CVB_ZEBRA_FUSED4 ? zebra_fusable<float>(L)
                                                                        : zebra_tma_ok(L);
  if (!ok) {
    L.ztma32 = keep_tma;
    L.zfuse32 = keep_fuse;
    L.ztw32 = keep_tw;
    return fail(ctx, CVB_BAD_INPUT, "zebra form %d cannot run on level %d", form, level);
  }
  const size_t n = L.g.n();
  int rc = CVB_OK;
  if (cudaMemcpyAsync(L.r32, b, sizeof(float) * n, cudaMemcpyHostToDevice, ctx->stream) != cudaSuccess ||
      cudaMemcpyAsync(L.e32, x, sizeof(float) * n, cudaMemcpyHostToDevice, ctx->stream) != cudaSuccess)
    rc = CVB_CUDA_ERROR;
  if (rc == CVB_OK) {
    launch_zebra_half<float>(L, L.r32, L.e32, L.t32 + n, omega, color, false, ctx->stream);
    if (cudaGetLastError() != cudaSuccess ||
        cudaMemcpyAsync(x, L.e32, sizeof(float) * n, cudaMemcpyDeviceToHost, ctx->stream) != cudaSuccess ||
        cudaStreamSynchronize(ctx->stream) != cudaSuccess)
      rc = CVB_CUDA_ERROR;
  }
  L.ztma32 = keep_tma;
  L.zfuse32 = keep_fuse;
  L.ztw32 = keep_tw;
  if (rc != CVB_OK) return fail(ctx, rc, "zebra half-sweep failed");
  if (form >= CVB_ZEBRA_TMA4 && tma_timeout_take(ctx->stream) != 0)
    return fail(ctx, CVB_TIMEOUT, "a TMA-staged half-sweep gave up waiting for its tiles");
  return CVB_OK;
}

int cvb_set_device_limit(cvb_ctx *ctx, unsigned long long bytes) {
  if (!ctx) return CVB_BAD_INPUT;
  ctx->device_limit = (size_t)bytes;
  return CVB_OK;
}

int cvb_level_cross(const cvb_ctx *ctx, int level, int *cross32, int *cross64) {
  if (!ctx || !ctx->ready || level < 0 || level >= ctx->nlevels) return CVB_BAD_INPUT;
  if (cross32) *cross32 = ctx->L[level].cross32;
  if (cross64) *cross64 = ctx->L[level].cross64;
  return CVB_OK;
}

int cvb_get_weights(cvb_ctx *ctx, int level, double *w) {
  TRY(level_ok(ctx, level));
  LevelDev &L = ctx->L[level];
  CK(cudaMemcpy(w, L.w64, sizeof(double) * NSLOT * L.g.n(), cudaMemcpyDeviceToHost));
  return CVB_OK;
}

int cvb_restrict(cvb_ctx *ctx, int coarse, const double *xf, double *xc) {
  TRY(level_ok(ctx, coarse));
  TRY(level_ok(ctx, coarse + 1));
  LevelDev &C = ctx->L[coarse], &F = ctx->L[coarse + 1];
  CK(cudaMemcpyAsync(F.r64, xf, sizeof(double) * F.g.n(), cudaMemcpyHostToDevice, ctx->stream));
  launch_restrict<double>(F, C, F.r64, C.e64, ctx->stream);
  CKL();
  CK(cudaMemcpyAsync(xc, C.e64, sizeof(double) * C.g.n(), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return CVB_OK;
}

int cvb_interpolate(cvb_ctx *ctx, int fine, const double *xc, double *xf) {
  TRY(level_ok(ctx, fine));
  TRY(level_ok(ctx, fine - 1));
  LevelDev &C = ctx->L[fine - 1], &F = ctx->L[fine];
  CK(cudaMemcpyAsync(C.r64, xc, sizeof(double) * C.g.n(), cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemsetAsync(F.e64, 0, sizeof(double) * F.g.n(), ctx->stream));
  launch_prolong_add<double>(C, F, C.r64, F.e64, ctx->stream);
  CKL();
  CK(cudaMemcpyAsync(xf, F.e64, sizeof(double) * F.g.n(), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return CVB_OK;
}

long long cvb_kernel_launches(void) { return launch_count(); }

int cvb_set_rhs(cvb_ctx *ctx, const double *b) {
  if (!ctx || !b) return CVB_BAD_INPUT;
  if (!ctx->ready) return fail(ctx, CVB_NOT_SETUP, "cvb_setup_hierarchy has not run");
  CK(cudaMemcpyAsync(ctx->b, b, sizeof(double) * fine_n(ctx), cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return CVB_OK;
}

int cvb_set_phi(cvb_ctx *ctx, const double *phi) {
  if (!ctx || !phi) return CVB_BAD_INPUT;
  if (!ctx->ready) return fail(ctx, CVB_NOT_SETUP, "cvb_setup_hierarchy has not run");
  CK(cudaMemcpyAsync(ctx->x, phi, sizeof(double) * fine_n(ctx), cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return CVB_OK;
}

int cvb_get_phi(cvb_ctx *ctx, double *phi) {
  if (!ctx || !phi) return CVB_BAD_INPUT;
  if (!ctx->ready) return fail(ctx, CVB_NOT_SETUP, "cvb_setup_hierarchy has not run");
  CK(cudaMemcpyAsync(phi, ctx->x, sizeof(double) * fine_n(ctx), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return CVB_OK;
}

int cvb_device_bytes(const cvb_ctx *ctx, unsigned long long *bytes) {
  if (!ctx || !bytes) return CVB_BAD_INPUT;
  *bytes = (unsigned long long)ctx->device_bytes;
  return CVB_OK;
}

int cvb_geometry_bytes(const cvb_ctx *ctx, unsigned long long *bytes, unsigned long long *id) {
  if (!ctx || !bytes) return CVB_BAD_INPUT;
  *bytes = ctx->geo ? (unsigned long long)ctx->geo->bytes : 0ull;
  if (id) *id = (unsigned long long)(uintptr_t)ctx->geo.get();
  return CVB_OK;
}

int cvb_setup_times(const cvb_ctx *ctx, double *ms5) {
  if (!ctx || !ms5) return CVB_BAD_INPUT;
  for (int q = 0; q < 5; q++) ms5[q] = ctx->setup_ms[q];
  return CVB_OK;
}

int cvb_tuning_report(cvb_ctx *ctx, char *buf, int len) {
  if (!ctx) return CVB_BAD_INPUT;
  if (!ctx->ready) return fail(ctx, CVB_NOT_SETUP, "cvb_setup_hierarchy has not run");
  std::string o = "{\"line_sweep\": [";
  for (size_t q = 0; q < ctx->tune.size(); q++) {
    const auto &t = ctx->tune[q];
    char row[768];
    const LevelDev &L = ctx->L[t.level];
    char z32[16];
    if (L.ztma32) snprintf(z32, sizeof z32, "tma%d", L.ztma32);
    else snprintf(z32, sizeof z32, "%s%s", L.zfuse32 ? "fused" : "split", L.ztw32 == 4 ? "4" : "");
    snprintf(row, sizeof row,
             "%s{\"level\": %d, \"cells\": %zu, \"f32\": {\"fused_us\": %.2f, \"split_us\": %.2f, \"choice\": \"%s\"}, "
             "\"f64\": {\"fused_us\": %.2f, \"split_us\": %.2f, \"choice\": \"%s\"}, "
             "\"zebra_f32\": {\"split_us\": %.2f, \"fused_us\": %.2f, \"split4_us\": %.2f, \"fused4_us\": %.2f, "
             "\"tma4_us\": %.2f, \"tma8_us\": %.2f, \"tma16_us\": %.2f, \"choice\": \"%s\"}, "
             "\"zebra_f64\": {\"split_us\": %.2f, \"fused_us\": %.2f, \"choice\": \"%s\"}}",
             q ? ", " : "", t.level, t.cells, t.us32[0], t.us32[1], L.sweep32 ? "split" : "fused", t.us64[0],
             t.us64[1], L.sweep64 ? "split" : "fused", t.zb32[0], t.zb32[1], t.zw32[0], t.zw32[1], t.zt32[0],
             t.zt32[1], t.zt32[2], z32,
             t.zb64[0], t.zb64[1], L.zfuse64 ? "fused" : "split");
    o += row;
  }
  o += "]}";
  if (!buf || len <= (int)o.size()) return fail(ctx, CVB_BAD_INPUT, "report needs %zu bytes", o.size() + 1);
  std::memcpy(buf, o.c_str(), o.size() + 1);
  return CVB_OK;
}

// One V-cycle from `level` down with the default options: run once eagerly,
// captured into a graph, then the graph replayed `reps` times between events.
static int time_vcycle(cvb_ctx *ctx, int kernel, int level, int reps, double *avg_ms, double *bytes) {
  if (level < 1) return fail(ctx, CVB_BAD_INPUT, "a V-cycle needs a level above the coarsest");
  cvb_solve_opts o;
  cvb_solve_opts_default(&o);
  LevelDev &L = ctx->L[level];
  const size_t n = L.g.n();
  const bool f32 = kernel == CVB_KERNEL_VCYCLE_F32;
  auto run = [&]() {
    if (f32) vcycle<float>(ctx, level, L.r32, L.e32, &o);
    else vcycle<double>(ctx, level, L.r64, L.e64, &o);
  };
  CK(cudaMemsetAsync(L.r32, 0, sizeof(float) * n, ctx->stream));
  CK(cudaMemsetAsync(L.r64, 0, sizeof(double) * n, ctx->stream));
  run();
  CKL();
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
  const long long c0 = launch_count();
  run();
  count_launch((int)(c0 - launch_count()));  // captured, not launched
  CK(cudaStreamEndCapture(ctx->stream, &graph));
  cudaError_t e = cudaGraphInstantiate(&exec, graph, 0);
  cudaGraphDestroy(graph);
  CK(e);
  for (int q = 0; q < 3; q++) cudaGraphLaunch(exec, ctx->stream);
  cudaEventRecord(ctx->ev0, ctx->stream);
  for (int q = 0; q < reps; q++) cudaGraphLaunch(exec, ctx->stream);
  cudaEventRecord(ctx->ev1, ctx->stream);
  e = cudaEventSynchronize(ctx->ev1);
  cudaGraphExecDestroy(exec);
  CK(e);
  CKL();
  float ms = 0;
  CK(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
  if (avg_ms) *avg_ms = ms / reps;
  if (bytes) *bytes = 0.0;
  return CVB_OK;
}

int cvb_time_kernel(cvb_ctx *ctx, int kernel, int level, int reps, double *avg_ms, double *bytes) {
  TRY(level_ok(ctx, level));
  if (reps < 1) return fail(ctx, CVB_BAD_INPUT, "reps < 1");
  LevelDev &L = ctx->L[level];
  size_t n = L.g.n();
  double per_cell;
  auto launch = [&]() {
    switch (kernel) {
      case CVB_KERNEL_LINE_SWEEP_F32: launch_line_smooth<float>(L, L.r32, L.e32, L.t32 + n, 0.85f, 0, ctx->stream); break;
      case CVB_KERNEL_LINE_SWEEP_F64: launch_line_smooth<double>(L, L.r64, L.e64, L.t64 + n, 0.85, 0, ctx->stream); break;
      case CVB_KERNEL_RESIDUAL_F32: launch_residual<float>(L, L.r32, L.e32, L.t32, ctx->stream); break;
      case CVB_KERNEL_RESIDUAL_F64: launch_residual<double>(L, L.r64, L.e64, L.t64, ctx->stream); break;
      case CVB_KERNEL_ZEBRA_F32: launch_zebra_half<float>(L, L.r32, L.e32, L.t32 + n, 1.3f, 1, false, ctx->stream); break;
      case CVB_KERNEL_CONTRA2CART:
        launch_contra2cart(L.g, ctx->cm[0], ctx->cm[1], ctx->cm[2], L.nvert, ctx->uc_dev, ctx->ucat_dev, ctx->stream,
                           1, -1, ctx->geo->c2c);
        break;
      case CVB_KERNEL_GHOST_NODES:
        launch_ghost_node_velocity(L.g, ctx->H[level].d.bctype, ctx->cm[0], ctx->cm[1], ctx->cm[2], ctx->ubcs_dev,
                                   ctx->ucat_dev, ctx->stream);
        break;
      case CVB_KERNEL_CONVECTION:
        launch_convection(L.g, ctx->uc_dev, ctx->ucat_dev, L.nvert, 0, ctx->conv_fp, ctx->conv_dev, ctx->stream);
        break;
      case CVB_KERNEL_VISCOUS: {
        const double *fm[9];
        for (int q = 0; q < 9; q++) fm[q] = ctx->fm[level][q];
        launch_viscous(L.g, L.nvert, ctx->ucat_dev, fm, ctx->iaj[level], ctx->jaj[level], ctx->kaj[level],
                       ctx->geo->gram, 1. / 300., ctx->conv_fp, ctx->visc_dev, ctx->stream);
        break;
      }
      case CVB_KERNEL_MOMENTUM_RHS:
        momentum_ff1(ctx, 300., 0);
        launch_calc_rhs(L.g, L.nvert, ctx->uc_dev, ctx->uo_dev, ctx->urm_dev, 1, -1. / 2e-3, L.g.mz - 3, ctx->rhs_dev,
                        ctx->stream);
        break;
      default: launch_zebra_half<double>(L, L.r64, L.e64, L.t64 + n, 1.3, 1, false, ctx->stream); break;
    }
  };
  if (kernel == CVB_KERNEL_VCYCLE_F32 || kernel == CVB_KERNEL_VCYCLE_F64) return time_vcycle(ctx, kernel, level, reps, avg_ms, bytes);
  const bool momentum = kernel == CVB_KERNEL_VISCOUS || kernel == CVB_KERNEL_MOMENTUM_RHS;
  if (kernel == CVB_KERNEL_CONTRA2CART || kernel == CVB_KERNEL_GHOST_NODES || kernel == CVB_KERNEL_CONVECTION ||
      momentum) {
    if (level != ctx->nlevels - 1) return fail(ctx, CVB_BAD_INPUT, "kernel %d runs on the finest level only", kernel);
    if (kernel == CVB_KERNEL_GHOST_NODES) TRY(ghost_types_ok(ctx, ctx->H[level].d.bctype));
    if (momentum)
      for (int f = 0; f < 6; f++)
        if (ctx->H[level].d.bctype[f] == 7) return fail(ctx, CVB_BAD_INPUT, "periodic faces are not covered");
    TRY(post_buffers(ctx, n));
    CK(cudaMemsetAsync(ctx->uc_dev, 0, sizeof(double) * 3 * n, ctx->stream));
    CK(cudaMemsetAsync(ctx->ucat_dev, 0, sizeof(double) * 3 * n, ctx->stream));
    CK(cudaMemsetAsync(ctx->ubcs_dev, 0, sizeof(double) * 3 * n, ctx->stream));
  }
  if (kernel == CVB_KERNEL_CONVECTION || momentum) {
    if (!ctx->conv_dev) TRY(dalloc(ctx, &ctx->conv_dev, 3 * n));
    if (!ctx->conv_fp) TRY(dalloc(ctx, &ctx->conv_fp, 9 * n));
    if (momentum) {
      for (double **b : {&ctx->visc_dev, &ctx->rct_dev, &ctx->rhs_dev, &ctx->uo_dev, &ctx->urm_dev})
        if (!*b) TRY(dalloc(ctx, b, 3 * n));
      CK(cudaMemsetAsync(ctx->p_dev, 0, sizeof(double) * n, ctx->stream));
      CK(cudaMemsetAsync(ctx->rhs_dev, 0, sizeof(double) * 3 * n, ctx->stream));
      CK(cudaMemsetAsync(ctx->uo_dev, 0, sizeof(double) * 3 * n, ctx->stream));
      CK(cudaMemsetAsync(ctx->urm_dev, 0, sizeof(double) * 3 * n, ctx->stream));
      TRY(ensure_face_gram(ctx));
    }
    // a velocity field of mixed signs in [-1, 1] (zero fluxes would send every
    // face through the full QUICK expression)
    std::vector<double> v(3 * n);
    for (size_t q = 0; q < v.size(); q++) v[q] = (double)((q * 2654435761ull) % 2001) / 1000.0 - 1.0;
    CK(cudaMemcpyAsync(ctx->uc_dev, v.data(), sizeof(double) * 3 * n, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(ctx->ucat_dev, v.data() + 1, sizeof(double) * (3 * n - 1), cudaMemcpyHostToDevice,
                       ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
  }
  // algorithmic bytes per cell: every array the kernel needs, touched once.
  // The coefficients are the 9 face coefficients (FP32) or 19 weights (FP64),
  // 3 or 7 on a level without cross-derivative terms (an orthogonal grid).
  const double g32 = L.cross32 ? 36 : 12, w64 = L.cross64 ? 152 : 56;
  switch (kernel) {
    case CVB_KERNEL_LINE_SWEEP_F32: per_cell = 4 + 4 + g32 + 4 + 4 + 12 + 4; break;   // x b g aj code fac xnew
    case CVB_KERNEL_LINE_SWEEP_F64: per_cell = 8 + 8 + w64 + 4 + 24 + 8; break;       // x b w code fac xnew
    case CVB_KERNEL_RESIDUAL_F32: per_cell = 4 + 4 + g32 + 4 + 4 + 4; break;          // x b g aj code r
    case CVB_KERNEL_RESIDUAL_F64: per_cell = 8 + 8 + w64 + 4 + 8; break;              // x b w code r
    // one zebra half-sweep: x read everywhere; coefficients, b, r and the line
    // solve's r, factors, x in/out on the half of the cells of the color
    case CVB_KERNEL_ZEBRA_F32: per_cell = 4 + 0.5 * (4 + g32 + 4 + 4 + 4) + 0.5 * (4 + 12 + 4 + 4); break;
    case CVB_KERNEL_ZEBRA_F64: per_cell = 8 + 0.5 * (8 + w64 + 4 + 8) + 0.5 * (8 + 24 + 8 + 8); break;
    case CVB_KERNEL_CONTRA2CART: per_cell = 72 + 24 + 8 + 24; break;  // centre metrics, ucont, nvert, ucat
    case CVB_KERNEL_CONVECTION: per_cell = 24 + 24 + 8 + 24; break;   // ucont, ucat, nvert, conv
    // ucat, nvert, the nine face metrics and three face Jacobians, visc
    case CVB_KERNEL_VISCOUS: per_cell = 24 + 8 + 216 + 24 + 24; break;
    // Contra2Cart (centre metrics, ucont, nvert, ucat), Convection and Viscous
    // as above, FormFunction1's faces (conv, visc, aj, rct, p, face metrics and
    // Jacobians, rhs) and the time term (ucont, ucont_o, ucont_rm1, rhs in/out)
    case CVB_KERNEL_MOMENTUM_RHS:
      per_cell = (72 + 24 + 8 + 24) + (24 + 24 + 8 + 24) + (24 + 8 + 216 + 24 + 24) +
                 (24 + 24 + 8 + 24 + 8 + 216 + 24 + 24) + (24 * 3 + 48);
      break;
    case CVB_KERNEL_GHOST_NODES: {
      // the ring cells only: ucat read and written, ubcs read
      const double inner = (double)(L.g.mx - 2) * (L.g.my - 2) * (L.g.mz - 2);
      per_cell = 72 * ((double)n - inner) / (double)n;
      break;
    }
    default: return fail(ctx, CVB_BAD_INPUT, "unknown kernel id %d", kernel);
  }
  CK(cudaMemsetAsync(L.r32, 0, sizeof(float) * n, ctx->stream));
  CK(cudaMemsetAsync(L.e32, 0, sizeof(float) * n, ctx->stream));
  CK(cudaMemsetAsync(L.r64, 0, sizeof(double) * n, ctx->stream));
  CK(cudaMemsetAsync(L.e64, 0, sizeof(double) * n, ctx->stream));
  for (int q = 0; q < 3; q++) launch();
  CK(cudaEventRecord(ctx->ev0, ctx->stream));
  for (int q = 0; q < reps; q++) launch();
  CK(cudaEventRecord(ctx->ev1, ctx->stream));
  CK(cudaEventSynchronize(ctx->ev1));
  CKL();
  float ms = 0;
  CK(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
  if (avg_ms) *avg_ms = ms / reps;
  if (bytes) *bytes = per_cell * (double)n;
  return CVB_OK;
}

int cvb_nullspace(cvb_ctx *ctx, int level, double *x) {
  TRY(level_ok(ctx, level));
  LevelDev &L = ctx->L[level];
  CK(cudaMemcpyAsync(L.r64, x, sizeof(double) * L.g.n(), cudaMemcpyHostToDevice, ctx->stream));
  TRY(fluid_mean_zero(ctx, level, L.r64));
  CK(cudaMemcpyAsync(x, L.r64, sizeof(double) * L.g.n(), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return CVB_OK;
}

}  // extern "C"
