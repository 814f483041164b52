// Grouped kernels of the batch engine: each launch runs one phase of the solve
// for every problem of a work-list (TaskList), with the per-block bodies of the
// single-problem kernels; plus the one-block-per-problem FGMRES control kernels
// that keep the Krylov scalars on the device.
#include <cmath>

#include "../../include/cvb.h"
#include "batch.h"
#include "stencil_body.cuh"

namespace cvb {

static const int kRed = 256;

__device__ __forceinline__ int find_task(const TaskList &tl, int b) {
  int lo = 0, hi = tl.n - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (tl.t[mid].block0 <= b) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// Decode a 3-D block coordinate of a task from the launch's linear block.
struct Blk3 {
  int x, y, z;
};
__device__ __forceinline__ Blk3 blk3(const GTask &T, int b) {
  int lb = b - T.block0;
  Blk3 r;
  r.x = lb % T.gx;
  int q = lb / T.gx;
  r.y = q % T.gy;
  r.z = q / T.gy;
  return r;
}

// ------------------------------------------------------------ stencil phases
__global__ void __launch_bounds__(256) kg_apply32(const __grid_constant__ TaskList tl) {
  dep_sync();
  const GTask &T = tl.t[find_task(tl, blockIdx.x)];
  if (gated(T.gate)) return;
  const LevelDev L = *T.L;
  Blk3 q = blk3(T, blockIdx.x);
  if (L.cross32)
    apply32_march_body<true>(L.g, L.gf32, L.ajf32, L.code, (const float *)T.a, (const float *)T.b, (float *)T.c, q.x,
                             q.y, q.z);
  else
    apply32_march_body<false>(L.g, L.gf32, L.ajf32, L.code, (const float *)T.a, (const float *)T.b, (float *)T.c,
                              q.x, q.y, q.z);
}
__global__ void __launch_bounds__(128) kg_apply64(const __grid_constant__ TaskList tl) {
  dep_sync();
  const GTask &T = tl.t[find_task(tl, blockIdx.x)];
  if (gated(T.gate)) return;
  const LevelDev L = *T.L;
  Blk3 q = blk3(T, blockIdx.x);
  if (L.cross64)
    apply64_body<double, true>(L.g, L.w64, L.code, (const double *)T.a, (const double *)T.b, (double *)T.c, q.x, q.y,
                               q.z);
  else
    apply64_body<double, false>(L.g, L.w64, L.code, (const double *)T.a, (const double *)T.b, (double *)T.c, q.x, q.y,
                                q.z);
}
template <typename T>
__global__ void __launch_bounds__(128) kg_restrict(const __grid_constant__ TaskList tl) {
  dep_sync();
  const GTask &K = tl.t[find_task(tl, blockIdx.x)];
  if (gated(K.gate)) return;
  const LevelDev F = K.L[0], C = K.L[-1];
  Blk3 q = blk3(K, blockIdx.x);
  restrict_body<T>(F, C, (const T *)K.a, (T *)K.c, q.x, q.y, q.z);
}
template <typename T>
__global__ void __launch_bounds__(128) kg_prolong(const __grid_constant__ TaskList tl) {
  dep_sync();
  const GTask &K = tl.t[find_task(tl, blockIdx.x)];
  if (gated(K.gate)) return;
  const LevelDev F = K.L[0], C = K.L[-1];
  Blk3 q = blk3(K, blockIdx.x);
  prolong_body<T>(C, F, (const T *)K.a, (T *)K.c, q.x, q.y, q.z);
}
template <typename T, int TW>
__global__ void __launch_bounds__(256, 2) kg_line_sweep(const __grid_constant__ TaskList tl, T omega) {
  dep_sync();
  const GTask &K = tl.t[find_task(tl, blockIdx.x)];
  if (gated(K.gate)) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const LevelDev L = *K.L;
  int lb = blockIdx.x - K.block0;
  if (has_cross<T>(L))
    line_sweep_body<T, TW, true>(L, (const T *)K.a, (const T *)K.b, (T *)K.c, omega, K.p0, lb % K.gx, lb / K.gx,
                                 smem_raw);
  else
    line_sweep_body<T, TW, false>(L, (const T *)K.a, (const T *)K.b, (T *)K.c, omega, K.p0, lb % K.gx, lb / K.gx,
                                  smem_raw);
}
// RR: rows per lane of every task's level (0: each task's own, at run time)
template <typename T, int TW, int RR>
__global__ void __launch_bounds__(kSolveThreads, 4) kg_line_solve(const __grid_constant__ TaskList tl, T omega) {
  dep_sync();
  const GTask &K = tl.t[find_task(tl, blockIdx.x)];
  if (gated(K.gate)) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const LevelDev L = *K.L;
  int lb = blockIdx.x - K.block0;
  // p1: colour + 1 (0: all lines), plus 16 when the residual is colour-split
  line_solve_body<T, TW, RR>(L, (const T *)K.a, (const T *)K.b, (T *)K.c, omega, lb % K.gx, lb / K.gx, smem_raw,
                             (K.p1 & 15) - 1, (K.p1 >> 4) != 0);
}
// zebra half-sweep in one kernel: b = a, x from b into c (in place when b == c),
// colour p1 - 1
template <typename T, int TW>
__global__ void __launch_bounds__(kSolveThreads, 4) kg_zebra_fused(const __grid_constant__ TaskList tl, T omega) {
  dep_sync();
  const GTask &K = tl.t[find_task(tl, blockIdx.x)];
  if (gated(K.gate)) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const LevelDev L = *K.L;
  int lb = blockIdx.x - K.block0;
  if (has_cross<T>(L))
    zebra_fused_body<T, TW, 0, true>(L, (const T *)K.a, (const T *)K.b, (T *)K.c, omega, lb % K.gx, lb / K.gx,
                                     smem_raw, K.p1 - 1);
  else
    zebra_fused_body<T, TW, 0, false>(L, (const T *)K.a, (const T *)K.b, (T *)K.c, omega, lb % K.gx, lb / K.gx,
                                      smem_raw, K.p1 - 1);
}
// zebra: residual on the cells of color p0
template <typename T>
__global__ void __launch_bounds__(128) kg_resid_color(const __grid_constant__ TaskList tl) {
  dep_sync();
  const GTask &K = tl.t[find_task(tl, blockIdx.x)];
  if (gated(K.gate)) return;
  const LevelDev L = *K.L;
  Blk3 q = blk3(K, blockIdx.x);
  if (has_cross<T>(L)) resid_color_body<T, true>(L, (const T *)K.a, (const T *)K.b, (T *)K.c, K.p0, q.x, q.y, q.z);
  else resid_color_body<T, false>(L, (const T *)K.a, (const T *)K.b, (T *)K.c, K.p0, q.x, q.y, q.z);
}
// c[0 .. p0) = 0
template <typename T>
__global__ void kg_zero(const __grid_constant__ TaskList tl) {
  dep_sync();
  const GTask &K = tl.t[find_task(tl, blockIdx.x)];
  if (gated(K.gate)) return;
  T *c = (T *)K.c;
  const size_t n = (size_t)K.p0;
  for (size_t p = (size_t)(blockIdx.x - K.block0) * 256 + threadIdx.x; p < n; p += (size_t)K.gx * 256) c[p] = T(0);
}
void glaunch_resid_color(const TaskList &tl, bool f32, cudaStream_t s) {
  if (!tl.n) return;
  if (f32) launch_dep(kg_resid_color<float>, tl.nblocks, kFlat, 0, s, tl);
  else launch_dep(kg_resid_color<double>, tl.nblocks, kFlat, 0, s, tl);
}
void glaunch_zero(const TaskList &tl, bool f32, cudaStream_t s) {
  if (!tl.n) return;
  if (f32) launch_dep(kg_zero<float>, tl.nblocks, 256, 0, s, tl);
  else launch_dep(kg_zero<double>, tl.nblocks, 256, 0, s, tl);
}
// e = Minv r on the coarsest level's inverted cells, e = r on the others; one
// warp per row (8 rows per block)
template <typename T>
__device__ __forceinline__ void dense_rows_g(const double *__restrict__ M, const int *__restrict__ idx, int m, int n,
                                             const T *__restrict__ r, T *__restrict__ e, int row) {
  const int lane = threadIdx.x & 31;
  if (row >= n) return;
  if (row >= m) {
    if (lane == 0) e[idx[row]] = r[idx[row]];
    return;
  }
  double s = 0.0;
  for (int c = lane; c < m; c += 32) s = fma(M[(size_t)row * m + c], (double)r[idx[c]], s);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if (lane == 0) e[idx[row]] = (T)s;
}
template <typename T>
__global__ void kg_dense(const __grid_constant__ TaskList tl) {
  dep_sync();
  const GTask &K = tl.t[find_task(tl, blockIdx.x)];
  if (gated(K.gate)) return;
  const LevelDev &C = *K.L;
  const int row = (blockIdx.x - K.block0) * 8 + (threadIdx.x >> 5);
  dense_rows_g<T>((const double *)K.b, C.cidx, C.cm, K.p0, (const T *)K.a, (T *)K.c, row);
}
template <typename TS, typename TD>
__global__ void kg_elem(const __grid_constant__ TaskList tl) {
  dep_sync();
  const GTask &K = tl.t[find_task(tl, blockIdx.x)];
  if (gated(K.gate)) return;
  const TS *a = (const TS *)K.a;
  TD *c = (TD *)K.c;
  const size_t n = (size_t)K.p0;
  for (size_t p = (size_t)(blockIdx.x - K.block0) * 256 + threadIdx.x; p < n; p += (size_t)K.gx * 256)
    c[p] = (TD)a[p];
}

void glaunch_residual32(const TaskList &tl, cudaStream_t s) {
  if (!tl.n) return;
  launch_dep(kg_apply32, tl.nblocks, dim3(32, 8), 0, s, tl);
}
void glaunch_residual64(const TaskList &tl, cudaStream_t s) {
  if (!tl.n) return;
  launch_dep(kg_apply64, tl.nblocks, kFlat, 0, s, tl);
}
void glaunch_restrict(const TaskList &tl, bool f32, cudaStream_t s) {
  if (!tl.n) return;
  if (f32) launch_dep(kg_restrict<float>, tl.nblocks, kFlat, 0, s, tl);
  else launch_dep(kg_restrict<double>, tl.nblocks, kFlat, 0, s, tl);
}
void glaunch_prolong(const TaskList &tl, bool f32, cudaStream_t s) {
  if (!tl.n) return;
  if (f32) launch_dep(kg_prolong<float>, tl.nblocks, kFlat, 0, s, tl);
  else launch_dep(kg_prolong<double>, tl.nblocks, kFlat, 0, s, tl);
}
template <typename K>
static void allow_smem(K kernel) {
  cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
}
void glaunch_line_sweep(const TaskList &tl, bool f32, float omega32, double omega64, size_t smem, cudaStream_t s) {
  if (!tl.n) return;
  static bool attr = false;
  if (!attr) {
    allow_smem(kg_line_sweep<float, 32>);
    allow_smem(kg_line_sweep<double, 16>);
    attr = true;
  }
  if (f32) launch_dep(kg_line_sweep<float, 32>, tl.nblocks, 256, smem, s, tl, omega32);
  else launch_dep(kg_line_sweep<double, 16>, tl.nblocks, 256, smem, s, tl, omega64);
}
template <typename T, int TW, int RR>
static void line_solve_rr(const TaskList &tl, T omega, size_t smem, cudaStream_t s) {
  static bool attr = false;
  if (!attr) {
    allow_smem(kg_line_solve<T, TW, RR>);
    attr = true;
  }
  launch_dep(kg_line_solve<T, TW, RR>, tl.nblocks, kSolveThreads, smem, s, tl, omega);
}
template <typename T, int TW>
static void line_solve_r(const TaskList &tl, T omega, size_t smem, int rr, cudaStream_t s) {
  switch (rr) {
    case 1: line_solve_rr<T, TW, 1>(tl, omega, smem, s); break;
    case 2: line_solve_rr<T, TW, 2>(tl, omega, smem, s); break;
    case 4: line_solve_rr<T, TW, 4>(tl, omega, smem, s); break;
    case 8: line_solve_rr<T, TW, 8>(tl, omega, smem, s); break;
    default: line_solve_rr<T, TW, 0>(tl, omega, smem, s); break;
  }
}
void glaunch_line_solve(const TaskList &tl, bool f32, float omega32, double omega64, size_t smem, int rr,
                        cudaStream_t s) {
  if (!tl.n) return;
  if (f32) line_solve_r<float, kSolveTW32>(tl, omega32, smem, rr, s);
  else line_solve_r<double, kSolveTW64>(tl, omega64, smem, rr, s);
}
void glaunch_zebra_fused(const TaskList &tl, bool f32, float omega32, double omega64, size_t smem, cudaStream_t s) {
  if (!tl.n) return;
  static bool attr = false;
  if (!attr) {
    allow_smem(kg_zebra_fused<float, kSolveTW32>);
    allow_smem(kg_zebra_fused<double, kSolveTW64>);
    attr = true;
  }
  if (f32) launch_dep(kg_zebra_fused<float, kSolveTW32>, tl.nblocks, kSolveThreads, smem, s, tl, omega32);
  else launch_dep(kg_zebra_fused<double, kSolveTW64>, tl.nblocks, kSolveThreads, smem, s, tl, omega64);
}
void glaunch_dense(const TaskList &tl, bool f32, cudaStream_t s) {
  if (!tl.n) return;
  if (f32) launch_dep(kg_dense<float>, tl.nblocks, 256, 0, s, tl);
  else launch_dep(kg_dense<double>, tl.nblocks, 256, 0, s, tl);
}
void glaunch_elementwise(const TaskList &tl, int kind, cudaStream_t s) {
  if (!tl.n) return;
  switch (kind) {
    case 0: launch_dep(kg_elem<float, float>, tl.nblocks, 256, 0, s, tl); break;
    case 1: launch_dep(kg_elem<double, double>, tl.nblocks, 256, 0, s, tl); break;
    case 2: launch_dep(kg_elem<double, float>, tl.nblocks, 256, 0, s, tl); break;
    default: launch_dep(kg_elem<float, double>, tl.nblocks, 256, 0, s, tl); break;
  }
}

// ------------------------------------------------------------ Krylov phases
// Sums of NR per-thread accumulators over the block into partial[row_q][nb].
template <int NR>
__device__ __forceinline__ void block_store(double (&acc)[NR], double *partial, int nb, int lb, const int *rows) {
  __shared__ double sh[NR][kRed / 32];
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < NR; q++) {
    double v = acc[q];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) sh[q][wid] = v;
  }
  __syncthreads();
  if (threadIdx.x < NR) {
    double v = 0.0;
#pragma unroll
    for (int w = 0; w < kRed / 32; w++) v += sh[threadIdx.x][w];
    partial[(size_t)rows[threadIdx.x] * nb + lb] = v;
  }
}

template <int NV, bool SELF>
__device__ __forceinline__ void multidot_body(const BProblem &P, const double *w, int base, int self_row, int lb) {
  constexpr int NR = NV + (SELF ? 1 : 0);
  double acc[NR > 0 ? NR : 1];
#pragma unroll
  for (int q = 0; q < NR; q++) acc[q] = 0.0;
  const double *v[NV > 0 ? NV : 1];
#pragma unroll
  for (int q = 0; q < NV; q++) v[q] = P.V[base + q];
  const size_t n = P.n;
  for (size_t p = (size_t)lb * kRed + threadIdx.x; p < n; p += (size_t)P.nb * kRed) {
    double wp = w[p];
#pragma unroll
    for (int q = 0; q < NV; q++) acc[q] = fma(v[q][p], wp, acc[q]);
    if (SELF) acc[NV] = fma(wp, wp, acc[NV]);
  }
  int rows[NR > 0 ? NR : 1];
#pragma unroll
  for (int q = 0; q < NV; q++) rows[q] = base + q;
  if (SELF) rows[NV] = self_row;
  block_store<NR>(acc, P.partial, P.nb, lb, rows);
}

__global__ void __launch_bounds__(kRed) kg_multidot(const __grid_constant__ TaskList tl, const BProblem *__restrict__ PP) {
  dep_sync();
  const GTask &K = tl.t[find_task(tl, blockIdx.x)];
  if (gated(K.gate)) return;
  const BProblem P = PP[K.p0];
  const double *w = (const double *)K.a;
  const int base = K.p1 & 0xff, cnt = (K.p1 >> 8) & 0xff, self_row = K.pad;
  const int lb = blockIdx.x - K.block0;
  if (self_row >= 0) {
    switch (cnt) {
      case 0: multidot_body<0, true>(P, w, base, self_row, lb); break;
      case 1: multidot_body<1, true>(P, w, base, self_row, lb); break;
      case 2: multidot_body<2, true>(P, w, base, self_row, lb); break;
      case 3: multidot_body<3, true>(P, w, base, self_row, lb); break;
      case 4: multidot_body<4, true>(P, w, base, self_row, lb); break;
      case 5: multidot_body<5, true>(P, w, base, self_row, lb); break;
      case 6: multidot_body<6, true>(P, w, base, self_row, lb); break;
      case 7: multidot_body<7, true>(P, w, base, self_row, lb); break;
      default: multidot_body<8, true>(P, w, base, self_row, lb); break;
    }
  } else {
    switch (cnt) {
      case 1: multidot_body<1, false>(P, w, base, 0, lb); break;
      case 2: multidot_body<2, false>(P, w, base, 0, lb); break;
      case 3: multidot_body<3, false>(P, w, base, 0, lb); break;
      case 4: multidot_body<4, false>(P, w, base, 0, lb); break;
      case 5: multidot_body<5, false>(P, w, base, 0, lb); break;
      case 6: multidot_body<6, false>(P, w, base, 0, lb); break;
      case 7: multidot_body<7, false>(P, w, base, 0, lb); break;
      default: multidot_body<8, false>(P, w, base, 0, lb); break;
    }
  }
}
void glaunch_multidot(const TaskList &tl, const BProblem *P, cudaStream_t s) {
  if (!tl.n) return;
  launch_dep(kg_multidot, tl.nblocks, kRed, 0, s, tl, P);
}

// sums[p1 + r] = sum_b partial[p1 + r][b], one block per row r < gx
__global__ void __launch_bounds__(kRed) kg_finish(const __grid_constant__ TaskList tl, const BProblem *__restrict__ PP) {
  dep_sync();
  const GTask &K = tl.t[find_task(tl, blockIdx.x)];
  if (gated(K.gate)) return;
  const BProblem P = PP[K.p0];
  const int row = K.p1 + (blockIdx.x - K.block0);
  __shared__ double sh[kRed];
  double v = 0.0;
  for (int b = threadIdx.x; b < P.nb; b += kRed) v += P.partial[(size_t)row * P.nb + b];
  sh[threadIdx.x] = v;
  __syncthreads();
  for (int o = kRed / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) P.sums[row] = sh[0];
}
void glaunch_finish(const TaskList &tl, const BProblem *P, cudaStream_t s) {
  if (!tl.n) return;
  launch_dep(kg_finish, tl.nblocks, kRed, 0, s, tl, P);
}

// w -= sum_{q < nv} sums[q] V_q ; partial[kNormRow][lb] = sum of w^2 over the block
__global__ void __launch_bounds__(kRed) kg_multiaxpy_norm(const __grid_constant__ TaskList tl,
                                                          const BProblem *__restrict__ PP) {
  dep_sync();
  const GTask &K = tl.t[find_task(tl, blockIdx.x)];
  if (gated(K.gate)) return;
  const BProblem P = PP[K.p0];
  const int nv = K.p1, lb = blockIdx.x - K.block0;
  __shared__ double hs[kBatchRestart + 1];
  if (threadIdx.x < nv) hs[threadIdx.x] = P.sums[threadIdx.x];
  __syncthreads();
  double acc = 0.0;
  double *w = P.w;
  for (size_t p = (size_t)lb * kRed + threadIdx.x; p < P.n; p += (size_t)P.nb * kRed) {
    double v = w[p];
    for (int q = 0; q < nv; q++) v = fma(-hs[q], P.V[q][p], v);
    w[p] = v;
    acc = fma(v, v, acc);
  }
  double a1[1] = {acc};
  int rows[1] = {kNormRow};
  block_store<1>(a1, P.partial, P.nb, lb, rows);
}
void glaunch_multiaxpy_norm(const TaskList &tl, const BProblem *P, cudaStream_t s) {
  if (!tl.n) return;
  launch_dep(kg_multiaxpy_norm, tl.nblocks, kRed, 0, s, tl, P);
}

// dst = src / *scal
__global__ void kg_scale(const __grid_constant__ TaskList tl) {
  dep_sync();
  const GTask &K = tl.t[find_task(tl, blockIdx.x)];
  if (gated(K.gate)) return;
  const double inv = 1.0 / *(const double *)K.b;
  const double *a = (const double *)K.a;
  double *c = (double *)K.c;
  const size_t n = (size_t)K.p0;
  for (size_t p = (size_t)(blockIdx.x - K.block0) * 256 + threadIdx.x; p < n; p += (size_t)K.gx * 256)
    c[p] = a[p] * inv;
}
void glaunch_scale(const TaskList &tl, cudaStream_t s) {
  if (!tl.n) return;
  launch_dep(kg_scale, tl.nblocks, 256, 0, s, tl);
}

// x += sum_{q < j} y[q] Z_q with j and y from the problem's Krylov state
__global__ void kg_update(const __grid_constant__ TaskList tl, const BProblem *__restrict__ PP) {
  dep_sync();
  const GTask &K = tl.t[find_task(tl, blockIdx.x)];
  if (gated(K.gate)) return;
  const BProblem P = PP[K.p0];
  __shared__ double ys[kBatchRestart];
  const int nz = P.ks->j;
  if (threadIdx.x < nz) ys[threadIdx.x] = P.ks->y[threadIdx.x];
  __syncthreads();
  for (size_t p = (size_t)(blockIdx.x - K.block0) * 256 + threadIdx.x; p < P.n; p += (size_t)K.gx * 256) {
    double v = P.x[p];
    for (int q = 0; q < nz; q++) v = fma(ys[q], P.Z[q][p], v);
    P.x[p] = v;
  }
}
void glaunch_update(const TaskList &tl, const BProblem *P, cudaStream_t s) {
  if (!tl.n) return;
  launch_dep(kg_update, tl.nblocks, 256, 0, s, tl, P);
}

// Null space (PoissonNullSpaceFunction, poisson.c:411-558) on the finest level:
// sums and counts of x over interior fluid cells into partial rows 0, 1.
__device__ __forceinline__ bool fluid_cell(const uint32_t *code, size_t p) { return (code[p] & CODE_FLUID) != 0; }
__global__ void __launch_bounds__(kRed) kg_fluid_sum(const __grid_constant__ TaskList tl, const BProblem *__restrict__ PP) {
  dep_sync();
  const GTask &K = tl.t[find_task(tl, blockIdx.x)];
  if (gated(K.gate)) return;
  const BProblem P = PP[K.p0];
  const Geom g = P.F->g;
  const uint32_t *cd = P.F->code;
  const int lb = blockIdx.x - K.block0;
  double acc[2] = {0.0, 0.0};
  for (size_t p = (size_t)lb * kRed + threadIdx.x; p < P.n; p += (size_t)P.nb * kRed)
    if (fluid_cell(cd, p)) {
      acc[0] += P.x[p];
      acc[1] += 1.0;
    }
  int rows[2] = {0, 1};
  block_store<2>(acc, P.partial, P.nb, lb, rows);
}
__global__ void kg_add_fluid_const(const __grid_constant__ TaskList tl, const BProblem *__restrict__ PP) {
  dep_sync();
  const GTask &K = tl.t[find_task(tl, blockIdx.x)];
  if (gated(K.gate)) return;
  const BProblem P = PP[K.p0];
  const Geom g = P.F->g;
  const uint32_t *cd = P.F->code;
  const double shift = P.sums[1] > 0.0 ? P.sums[0] / (-1.0 * P.sums[1]) : 0.0;
  for (size_t p = (size_t)(blockIdx.x - K.block0) * 256 + threadIdx.x; p < P.n; p += (size_t)K.gx * 256) {
    if (fluid_cell(cd, p)) P.x[p] += shift;
    else P.x[p] = 0.0;
  }
}
// range projection of b: sums of b/aj and counts over fluid cells (rows 0, 1)
__global__ void __launch_bounds__(kRed) kg_fluid_ratio(const __grid_constant__ TaskList tl,
                                                       const BProblem *__restrict__ PP) {
  dep_sync();
  const GTask &K = tl.t[find_task(tl, blockIdx.x)];
  if (gated(K.gate)) return;
  const BProblem P = PP[K.p0];
  const Geom g = P.F->g;
  const uint32_t *cd = P.F->code;
  const int lb = blockIdx.x - K.block0;
  double acc[2] = {0.0, 0.0};
  for (size_t p = (size_t)lb * kRed + threadIdx.x; p < P.n; p += (size_t)P.nb * kRed)
    if (fluid_cell(cd, p)) {
      acc[0] += quot_newton(P.b[p], P.aj[p]);
      acc[1] += 1.0;
    }
  int rows[2] = {0, 1};
  block_store<2>(acc, P.partial, P.nb, lb, rows);
}
__global__ void kg_remove_aj_mean(const __grid_constant__ TaskList tl, const BProblem *__restrict__ PP) {
  dep_sync();
  const GTask &K = tl.t[find_task(tl, blockIdx.x)];
  if (gated(K.gate)) return;
  const BProblem P = PP[K.p0];
  const Geom g = P.F->g;
  const uint32_t *cd = P.F->code;
  const double c = P.sums[1] > 0.0 ? P.sums[0] / P.sums[1] : 0.0;
  for (size_t p = (size_t)(blockIdx.x - K.block0) * 256 + threadIdx.x; p < P.n; p += (size_t)K.gx * 256)
    if (fluid_cell(cd, p)) P.b[p] -= P.aj[p] * c;
}
void glaunch_fluid_sum(const TaskList &tl, const BProblem *P, cudaStream_t s) {
  if (!tl.n) return;
  launch_dep(kg_fluid_sum, tl.nblocks, kRed, 0, s, tl, P);
}
void glaunch_add_fluid_const(const TaskList &tl, const BProblem *P, cudaStream_t s) {
  if (!tl.n) return;
  launch_dep(kg_add_fluid_const, tl.nblocks, 256, 0, s, tl, P);
}
void glaunch_fluid_ratio(const TaskList &tl, const BProblem *P, cudaStream_t s) {
  if (!tl.n) return;
  launch_dep(kg_fluid_ratio, tl.nblocks, kRed, 0, s, tl, P);
}
void glaunch_remove_aj_mean(const TaskList &tl, const BProblem *P, cudaStream_t s) {
  if (!tl.n) return;
  launch_dep(kg_remove_aj_mean, tl.nblocks, 256, 0, s, tl, P);
}

// ------------------------------------------------------------ control kernels
// One thread per problem does the scalar work (a few hundred flops at most).
__global__ void k_init(const __grid_constant__ InitList il, const BProblem *__restrict__ PP) {
  dep_sync();
  if (threadIdx.x != 0) return;
  const int q = blockIdx.x;
  const BProblem &P = PP[il.idx[q]];
  KState *ks = P.ks;
  BFlags *fl = P.fl;
  const double bnorm = sqrt(P.sums[kNormRow]);
  ks->bnorm = bnorm;
  ks->target = fmax(il.rtol[q] * bnorm, il.atol[q]);
  ks->m = il.m[q];
  ks->max_it = il.max_it[q];
  ks->j = 0;
  ks->iters = 0;
  ks->cycles = 0;
  ks->est = 0.0;
  fl->bnorm = bnorm;
  fl->iters = 0;
  fl->cycles = 0;
  fl->status = CVB_OK;
  fl->rel = 0.0;
  fl->abs = 0.0;
  fl->fin = 0;
  fl->notfin = 1;
  fl->gate = 0;
  if (!isfinite(bnorm)) {
    fl->status = CVB_NAN_DETECTED;
    fl->fin = 1;
  } else if (bnorm == 0.0) {
    fl->fin = 1;  // zero right-hand side: phi stays as it is (zero unless warm-started)
  }
  if (fl->fin) { fl->gate = 1; fl->notfin = 0; }
}
void launch_k_init(const InitList &il, const BProblem *P, cudaStream_t s) {
  if (!il.n) return;
  launch_dep(k_init, il.n, 32, 0, s, il, P);
}

__global__ void k_removed(const __grid_constant__ ProbList pl, const BProblem *__restrict__ PP) {
  dep_sync();
  if (threadIdx.x != 0) return;
  const BProblem &P = PP[pl.idx[blockIdx.x]];
  double c = P.sums[1] > 0.0 ? P.sums[0] / P.sums[1] : 0.0;
  P.ks->removed = c;
  P.fl->removed = c;
}
void launch_k_removed(const ProbList &pl, const BProblem *P, cudaStream_t s) {
  if (!pl.n) return;
  launch_dep(k_removed, pl.n, 32, 0, s, pl, P);
}

// After r = b - A x and sums[kNormRow] = |r|^2: stop (converged, budget spent,
// NaN) or open a new cycle with beta = |r| (V_0 = r / beta follows, gated).
__global__ void k_cycle_start(const __grid_constant__ ProbList pl, const BProblem *__restrict__ PP) {
  dep_sync();
  if (threadIdx.x != 0) return;
  const BProblem &P = PP[pl.idx[blockIdx.x]];
  KState *ks = P.ks;
  BFlags *fl = P.fl;
  if (fl->fin) return;
  const double beta = sqrt(P.sums[kNormRow]);
  fl->abs = beta;
  fl->rel = ks->bnorm > 0.0 ? beta / ks->bnorm : 0.0;
  fl->iters = ks->iters;
  fl->cycles = ks->cycles;
  int fin = 0, status = CVB_OK;
  if (!isfinite(beta)) { fin = 1; status = CVB_NAN_DETECTED; }
  else if (beta <= ks->target) { fin = 1; status = CVB_OK; }
  else if (ks->iters >= ks->max_it) { fin = 1; status = CVB_NOT_CONVERGED; }
  if (fin) {
    fl->status = status;
    fl->gate = 1;
    fl->notfin = 0;
    __threadfence();
    fl->fin = 1;
    return;
  }
  ks->beta = beta;
  ks->j = 0;
  for (int q = 0; q <= ks->m; q++) ks->g[q] = 0.0;
  ks->g[0] = beta;
  ks->est = beta;
  fl->gate = 0;
}
void launch_k_cycle_start(const ProbList &pl, const BProblem *P, cudaStream_t s) {
  if (!pl.n) return;
  launch_dep(k_cycle_start, pl.n, 32, 0, s, pl, P);
}

// After the Gram-Schmidt sums of iteration j: H(:, j), the Givens rotations and
// the residual estimate; closes the cycle (gate) when it converged, broke down,
// is full or spent the iteration budget.
__global__ void k_arnoldi(const __grid_constant__ ProbList pl, const BProblem *__restrict__ PP) {
  dep_sync();
  if (threadIdx.x != 0) return;
  const BProblem &P = PP[pl.idx[blockIdx.x]];
  KState *ks = P.ks;
  BFlags *fl = P.fl;
  if (fl->gate) return;
  const int j = ks->j, m1 = ks->m + 1;
  double *Hc = ks->H + (size_t)j * m1;
  for (int q = 0; q <= j; q++) Hc[q] = P.sums[q];
  const double hn = sqrt(P.sums[kNormRow]);
  Hc[j + 1] = hn;
  ks->hn = hn;
  for (int q = 0; q < j; q++) {
    double t = ks->cs[q] * Hc[q] + ks->sn[q] * Hc[q + 1];
    Hc[q + 1] = -ks->sn[q] * Hc[q] + ks->cs[q] * Hc[q + 1];
    Hc[q] = t;
  }
  const double a = Hc[j], bb = Hc[j + 1];
  const double rr = hypot(a, bb);
  ks->cs[j] = rr > 0 ? a / rr : 1.0;
  ks->sn[j] = rr > 0 ? bb / rr : 0.0;
  Hc[j] = rr;
  Hc[j + 1] = 0.0;
  ks->g[j + 1] = -ks->sn[j] * ks->g[j];
  ks->g[j] = ks->cs[j] * ks->g[j];
  const double est = fabs(ks->g[j + 1]);
  ks->est = est;
  ks->j = j + 1;
  ks->iters += 1;
  fl->iters = ks->iters;
  if (!isfinite(hn) || !isfinite(est) || est <= ks->target || hn == 0.0 || j + 1 == ks->m ||
      ks->iters >= ks->max_it)
    fl->gate = 1;
}
void launch_k_arnoldi(const ProbList &pl, const BProblem *P, cudaStream_t s) {
  if (!pl.n) return;
  launch_dep(k_arnoldi, pl.n, 32, 0, s, pl, P);
}

// y = R^-1 g over the cycle's j basis vectors (back substitution).
__global__ void k_solve_y(const __grid_constant__ ProbList pl, const BProblem *__restrict__ PP) {
  dep_sync();
  if (threadIdx.x != 0) return;
  const BProblem &P = PP[pl.idx[blockIdx.x]];
  KState *ks = P.ks;
  if (P.fl->fin) return;
  const int j = ks->j, m1 = ks->m + 1;
  for (int q = j - 1; q >= 0; q--) {
    double t = ks->g[q];
    for (int c = q + 1; c < j; c++) t -= ks->H[(size_t)c * m1 + q] * ks->y[c];
    ks->y[q] = t / ks->H[(size_t)q * m1 + q];
  }
  ks->cycles += 1;
}
void launch_k_solve_y(const ProbList &pl, const BProblem *P, cudaStream_t s) {
  if (!pl.n) return;
  launch_dep(k_solve_y, pl.n, 32, 0, s, pl, P);
}

}  // namespace cvb
