// Krylov support: fused multi-dot products, multi-axpy with norm, null-space
// removal and the coarsest-level dense solve.  Every reduction is two-stage with
// a fixed block count and a fixed summation tree, so a solve's result does not
// depend on timing or on what else shares the GPU.
#include <algorithm>

#include "launch.cuh"

namespace cvb {

static long long g_launches = 0;
void count_launch(int n) { __atomic_add_fetch(&g_launches, (long long)n, __ATOMIC_RELAXED); }
long long launch_count() { return __atomic_load_n(&g_launches, __ATOMIC_RELAXED); }

static const int kRedThreads = 256;
static int g_red_blocks = 0;

int sm_count() {
  static int sms = 0;
  if (!sms) {
    int dev = 0, v = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
    sms = v > 0 ? v : 148;
  }
  return sms;
}

int reduce_blocks() {
  if (!g_red_blocks) g_red_blocks = sm_count() * 4;
  return g_red_blocks;
}

template <int NV>
__device__ __forceinline__ void block_reduce_store(double (&acc)[NV], double *partial, int nblocks, int base) {
  __shared__ double sh[NV][kRedThreads / 32];
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < NV; q++) {
    double v = acc[q];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) sh[q][wid] = v;
  }
  __syncthreads();
  if (threadIdx.x < NV) {
    double v = 0.0;
#pragma unroll
    for (int w = 0; w < kRedThreads / 32; w++) v += sh[threadIdx.x][w];
    partial[(size_t)(base + threadIdx.x) * nblocks + blockIdx.x] = v;
  }
}

// partial[q][block] = sum over this block's elements of V_q[i] * w[i] for NV
// vectors starting at `base`; with `self` the w.w sum goes to row `self_row`.
// The vector count is a template parameter: predicated-off products would still
// occupy the FP64 pipe, which bounds this kernel on this part.
template <typename TV, int NV, bool SELF>
__global__ void __launch_bounds__(kRedThreads) k_multidot(const TV *const *V, int base, const double *__restrict__ w,
                                                           size_t n, double *partial, int self_row,
                                                           const int *gate) {
  dep_sync();
  if (gated(gate)) return;
  double acc[NV + 1];
#pragma unroll
  for (int q = 0; q <= NV; q++) acc[q] = 0.0;
  const TV *v[NV];
#pragma unroll
  for (int q = 0; q < NV; q++) v[q] = V[base + q];
  for (size_t p = blockIdx.x * (size_t)kRedThreads + threadIdx.x; p < n; p += (size_t)gridDim.x * kRedThreads) {
    double wp = w[p];
#pragma unroll
    for (int q = 0; q < NV; q++) acc[q] = fma((double)v[q][p], wp, acc[q]);
    if (SELF) acc[NV] = fma(wp, wp, acc[NV]);
  }
  __shared__ double sh[NV + 1][kRedThreads / 32];
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  constexpr int NR = SELF ? NV + 1 : NV;
#pragma unroll
  for (int q = 0; q < NR; q++) {
    double x = acc[q];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0) sh[q][wid] = x;
  }
  __syncthreads();
  if (threadIdx.x < NR) {
    double x = 0.0;
#pragma unroll
    for (int ww = 0; ww < kRedThreads / 32; ww++) x += sh[threadIdx.x][ww];
    int row = (SELF && threadIdx.x == NV) ? self_row : base + threadIdx.x;
    partial[(size_t)row * gridDim.x + blockIdx.x] = x;
  }
}

template <typename TV, bool SELF>
static void multidot_chunk(const TV *const *V, int base, int cnt, const double *w, size_t n, double *partial,
                           int self_row, cudaStream_t s, const int *gate = nullptr) {
  int nb = reduce_blocks();
  switch (cnt) {
    case 1: launch_dep(k_multidot<TV, 1, SELF>, nb, kRedThreads, 0, s, V, base, w, n, partial, self_row, gate); break;
    case 2: launch_dep(k_multidot<TV, 2, SELF>, nb, kRedThreads, 0, s, V, base, w, n, partial, self_row, gate); break;
    case 3: launch_dep(k_multidot<TV, 3, SELF>, nb, kRedThreads, 0, s, V, base, w, n, partial, self_row, gate); break;
    case 4: launch_dep(k_multidot<TV, 4, SELF>, nb, kRedThreads, 0, s, V, base, w, n, partial, self_row, gate); break;
    case 5: launch_dep(k_multidot<TV, 5, SELF>, nb, kRedThreads, 0, s, V, base, w, n, partial, self_row, gate); break;
    case 6: launch_dep(k_multidot<TV, 6, SELF>, nb, kRedThreads, 0, s, V, base, w, n, partial, self_row, gate); break;
    case 7: launch_dep(k_multidot<TV, 7, SELF>, nb, kRedThreads, 0, s, V, base, w, n, partial, self_row, gate); break;
    default: launch_dep(k_multidot<TV, 8, SELF>, nb, kRedThreads, 0, s, V, base, w, n, partial, self_row, gate); break;
  }
}

// Dots of w with V_0..V_{nv-1} in chunks of up to 8 vectors (each chunk reads w
// once more); with `self`, w.w lands in row nv of the partials.
void launch_multidot(const double *const *V, int nv, const double *w, size_t n, double *partial, cudaStream_t s,
                     int self, const int *gate) {
  for (int base = 0; base < nv; base += 8) {
    int cnt = nv - base < 8 ? nv - base : 8;
    if (self && base == 0) multidot_chunk<double, true>(V, base, cnt, w, n, partial, nv, s, gate);
    else multidot_chunk<double, false>(V, base, cnt, w, n, partial, nv, s, gate);
  }
}
void launch_multidot_f32(const float *const *V, int nv, const double *w, size_t n, double *partial, cudaStream_t s) {
  for (int base = 0; base < nv; base += 8)
    multidot_chunk<float, false>(V, base, nv - base < 8 ? nv - base : 8, w, n, partial, nv, s);
}

// out[q] = sum_b partial[q][b], one block per q, fixed tree.
__global__ void k_finish(const double *__restrict__ partial, int nblocks, double *__restrict__ out,
                         const int *gate) {
  dep_sync();
  if (gated(gate)) return;
  __shared__ double sh[kRedThreads];
  int q = blockIdx.x;
  double v = 0.0;
  for (int b = threadIdx.x; b < nblocks; b += kRedThreads) v += partial[(size_t)q * nblocks + b];
  sh[threadIdx.x] = v;
  __syncthreads();
  for (int o = kRedThreads / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[q] = sh[0];
}
void launch_finish_sums(const double *partial, int nv, int nblocks, double *out, cudaStream_t s, const int *gate) {
  launch_dep(k_finish, nv, kRedThreads, 0, s, partial, nblocks, out, gate);
}

// w -= sum_q h[q] V_q ; partial[block] = sum of w^2 over the block.
__global__ void __launch_bounds__(kRedThreads) k_multiaxpy_norm(double *__restrict__ w, const double *const *V,
                                                                 const double *__restrict__ h, int nv, size_t n,
                                                                 double *partial, const int *gate) {
  dep_sync();
  if (gated(gate)) return;
  __shared__ double hs[64];
  if (threadIdx.x < nv) hs[threadIdx.x] = h[threadIdx.x];
  __syncthreads();
  double acc = 0.0;
  for (size_t p = blockIdx.x * (size_t)kRedThreads + threadIdx.x; p < n; p += (size_t)gridDim.x * kRedThreads) {
    double v = w[p];
    for (int q = 0; q < nv; q++) v = fma(-hs[q], V[q][p], v);
    w[p] = v;
    acc = fma(v, v, acc);
  }
  double a1[1] = {acc};
  block_reduce_store<1>(a1, partial, gridDim.x, 0);
}
void launch_multiaxpy_norm(double *w, const double *const *V, const double *h_dev, int nv, size_t n,
                           double *partial, cudaStream_t s, const int *gate) {
  launch_dep(k_multiaxpy_norm, reduce_blocks(), kRedThreads, 0, s, w, V, h_dev, nv, n, partial, gate);
}

// dst = src / *scal, or src / sqrt(*scal); with dst32 also its FP32 copy (the
// next V-cycle's input in mixed precision)
template <bool SQRT>
__global__ void k_scale(double *__restrict__ dst, const double *__restrict__ src, const double *__restrict__ scal,
                        size_t n, const int *gate, float *__restrict__ dst32) {
  dep_sync();
  if (gated(gate)) return;
  double inv = 1.0 / (SQRT ? sqrt(*scal) : *scal);
  for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < n; p += (size_t)gridDim.x * blockDim.x) {
    const double v = src[p] * inv;
    dst[p] = v;
    if (dst32) dst32[p] = (float)v;
  }
}
void launch_scale(double *dst, const double *src, const double *scal_dev, size_t n, cudaStream_t s,
                  const int *gate, float *dst32) {
  launch_dep(k_scale<false>, reduce_blocks(), 256, 0, s, dst, src, scal_dev, n, gate, dst32);
}
void launch_scale_sqrt(double *dst, const double *src, const double *sq_dev, size_t n, cudaStream_t s,
                       float *dst32, const int *gate) {
  launch_dep(k_scale<true>, reduce_blocks(), 256, 0, s, dst, src, sq_dev, n, gate, dst32);
}

__global__ void k_reciprocal(const double *__restrict__ a, double *__restrict__ out, size_t n) {
  dep_sync();
  for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < n; p += (size_t)gridDim.x * blockDim.x)
    out[p] = 1.0 / a[p];
}
void launch_reciprocal(const double *a, double *out, size_t n, cudaStream_t s) {
  launch_dep(k_reciprocal, reduce_blocks(), 256, 0, s, a, out, n);
}

// x += sum_q y[q] Z_q (Z stored FP32 in mixed mode, FP64 in plain mode)
__global__ void k_axpy_z(double *__restrict__ x, const float *const *Z32, const double *const *Z64,
                         const double *__restrict__ y, int nz, size_t n) {
  dep_sync();
  __shared__ double ys[64];
  if (threadIdx.x < nz) ys[threadIdx.x] = y[threadIdx.x];
  __syncthreads();
  for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < n; p += (size_t)gridDim.x * blockDim.x) {
    double v = x[p];
    if (Z32)
      for (int q = 0; q < nz; q++) v = fma(ys[q], (double)Z32[q][p], v);
    else
      for (int q = 0; q < nz; q++) v = fma(ys[q], Z64[q][p], v);
    x[p] = v;
  }
}
void launch_axpy_z(double *x, const float *const *Z32, const double *const *Z64, const double *y_dev, int nz,
                   size_t n, cudaStream_t s) {
  launch_dep(k_axpy_z, reduce_blocks(), 256, 0, s, x, Z32, Z64, y_dev, nz, n);
}

// Null space (PoissonNullSpaceFunction, poisson.c:411-558): sums and counts of x
// over interior fluid cells (nvert < 0.1).
__global__ void __launch_bounds__(kRedThreads) k_fluid_sum(Geom g, const uint32_t *__restrict__ code,
                                                           const double *__restrict__ x, double *partial) {
  dep_sync();
  double acc[2] = {0.0, 0.0};
  size_t n = g.n();
  for (size_t p = blockIdx.x * (size_t)kRedThreads + threadIdx.x; p < n; p += (size_t)gridDim.x * kRedThreads) {
    if (code[p] & CODE_FLUID) {
      acc[0] += x[p];
      acc[1] += 1.0;
    }
  }
  block_reduce_store<2>(acc, partial, gridDim.x, 0);
}
void launch_fluid_mean_partial(const Geom &g, const uint32_t *code, const double *x, double *partial,
                               cudaStream_t s) {
  launch_dep(k_fluid_sum, reduce_blocks(), kRedThreads, 0, s, g, code, x, partial);
}
// x += -sum/count on interior fluid cells; with zero_outside the ring and the
// non-fluid cells are set to zero.
__global__ void k_add_fluid_const(Geom g, const uint32_t *__restrict__ code, double *__restrict__ x,
                                  const double *__restrict__ sc, int zero_outside) {
  dep_sync();
  double shift = sc[1] > 0.0 ? sc[0] / (-1.0 * sc[1]) : 0.0;
  size_t n = g.n();
  for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < n; p += (size_t)gridDim.x * blockDim.x) {
    const uint32_t c = code[p];
    if (c & CODE_FLUID) x[p] += shift;
    if (zero_outside && (c & CODE_IDENTITY)) x[p] = 0.0;  // the ring and nvert > 0.1
  }
}
void launch_add_fluid_const(const Geom &g, const uint32_t *code, double *x, const double *sumcnt, int zero_outside,
                            cudaStream_t s) {
  launch_dep(k_add_fluid_const, reduce_blocks(), 256, 0, s, g, code, x, sumcnt, zero_outside);
}

// The range projection's sums over the fluid cells: of b / aj, as b times the
// stored 1 / aj (the FP64 pipe is this part's bound, and a division costs
// several of its instructions), and the cell count, counted in an integer.
__global__ void __launch_bounds__(kRedThreads) k_fluid_ratio(Geom g, const uint32_t *__restrict__ code,
                                                             const double *__restrict__ b,
                                                             const double *__restrict__ inv_aj, double *partial) {
  dep_sync();
  double acc[2] = {0.0, 0.0};
  unsigned cnt = 0;
  size_t n = g.n();
  for (size_t p = blockIdx.x * (size_t)kRedThreads + threadIdx.x; p < n; p += (size_t)gridDim.x * kRedThreads) {
    if (code[p] & CODE_FLUID) {
      acc[0] = fma(b[p], inv_aj[p], acc[0]);
      cnt++;
    }
  }
  acc[1] = (double)cnt;
  block_reduce_store<2>(acc, partial, gridDim.x, 0);
}
void launch_fluid_ratio_partial(const Geom &g, const uint32_t *code, const double *b, const double *inv_aj,
                                double *partial, cudaStream_t s) {
  launch_dep(k_fluid_ratio, reduce_blocks(), kRedThreads, 0, s, g, code, b, inv_aj, partial);
}
__global__ void k_remove_aj_mean(Geom g, const uint32_t *__restrict__ code, const double *__restrict__ aj,
                                 double *__restrict__ b, const double *__restrict__ sums) {
  dep_sync();
  double c = sums[1] > 0.0 ? sums[0] / sums[1] : 0.0;
  size_t n = g.n();
  for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < n; p += (size_t)gridDim.x * blockDim.x) {
    if (code[p] & CODE_FLUID)
      b[p] -= aj[p] * c;
  }
}
void launch_remove_aj_mean(const Geom &g, const uint32_t *code, const double *aj, double *b, const double *sums,
                           cudaStream_t s) {
  launch_dep(k_remove_aj_mean, reduce_blocks(), 256, 0, s, g, code, aj, b, sums);
}

// Coarsest level: e = Minv r with a dense FP64 inverse over the cells idx[0..m),
// e = r on the identity cells idx[m..n).  A block first gathers r over the
// inverted cells into shared memory, in the inverse's column order and in FP64;
// its warps then take rows, each lane two adjacent columns per step with one
// 16-byte load of the row (rows are 16-byte aligned for even m) into two
// accumulators, four steps in flight, then a shuffle sum.  The inverse is the
// bulk of the bytes (8 m^2), read once per apply.  STAGED false (m beyond what
// shared memory holds): r is read through idx at every step instead.
template <typename T, bool STAGED>
__global__ void __launch_bounds__(256) k_dense(const double *__restrict__ M, const int *__restrict__ idx, int m, int n,
                                               const T *__restrict__ r, T *__restrict__ e, const int *gate) {
  extern __shared__ __align__(16) double rc[];
  dep_sync();
  if (gated(gate)) return;
  if (STAGED) {
    for (int c = threadIdx.x; c < m; c += blockDim.x) rc[c] = (double)r[idx[c]];
    __syncthreads();
  }
  const int lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  const int tw = gridDim.x * nw;
  for (int row = blockIdx.x * nw + (threadIdx.x >> 5); row < n; row += tw) {
    if (row >= m) {
      if (lane == 0) e[idx[row]] = r[idx[row]];
      continue;
    }
    const double *Mr = M + (size_t)row * m;
    double s0 = 0.0, s1 = 0.0;
    if (STAGED && (m & 1) == 0) {
      const double2 *M2 = reinterpret_cast<const double2 *>(Mr);
      const double2 *R2 = reinterpret_cast<const double2 *>(rc);
#pragma unroll 4
      for (int c2 = lane; c2 < (m >> 1); c2 += 32) {
        const double2 v = __ldg(M2 + c2), x = R2[c2];
        s0 = fma(v.x, x.x, s0);
        s1 = fma(v.y, x.y, s1);
      }
    } else {
      for (int c = lane; c < m; c += 32) s0 = fma(__ldg(Mr + c), STAGED ? rc[c] : (double)r[idx[c]], s0);
    }
    double sum = s0 + s1;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) sum += __shfl_down_sync(0xffffffffu, sum, o);
    if (lane == 0) e[idx[row]] = (T)sum;
  }
}
template <typename T>
static void dense_apply(const LevelDev &C, const double *Minv, const T *r, T *e, cudaStream_t s, const int *gate) {
  constexpr int kMaxStaged = 8192;  // 64 KB of staged FP64 input
  const int n = (int)C.g.n();
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_dense<T, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, 8 * kMaxStaged);
    attr = true;
  }
  const int rows_per_block = 8, blocks = std::max(1, std::min((n + rows_per_block - 1) / rows_per_block, 4 * sm_count()));
  if (C.cm <= kMaxStaged)
    launch_dep(k_dense<T, true>, blocks, 256, sizeof(double) * (size_t)C.cm, s, Minv, C.cidx, C.cm, n, r, e, gate);
  else
    launch_dep(k_dense<T, false>, blocks, 256, 0, s, Minv, C.cidx, C.cm, n, r, e, gate);
}
void launch_dense_apply(const LevelDev &C, const double *Minv, const double *r, double *e, cudaStream_t s,
                        const int *gate) {
  dense_apply<double>(C, Minv, r, e, s, gate);
}
void launch_dense_apply_f32(const LevelDev &C, const double *Minv, const float *r, float *e, cudaStream_t s,
                            const int *gate) {
  dense_apply<float>(C, Minv, r, e, s, gate);
}

}  // namespace cvb
