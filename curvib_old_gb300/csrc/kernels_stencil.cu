// Single-problem kernels of the operator, smoother and transfers, and their
// launchers.  The per-cell arithmetic lives in stencil_body.cuh.
#include "stencil_body.cuh"

namespace cvb {

static inline unsigned nblk(size_t n, int t) { return (unsigned)((n + t - 1) / t); }

// X (every operator kernel): the level has cross-derivative terms; kernels for
// an orthogonal level (X false) read the seven face points only.
template <typename TX, bool X>
__global__ void __launch_bounds__(128) k_apply64(Geom g, const double *__restrict__ w, const uint32_t *__restrict__ code,
                                                 const TX *__restrict__ x, const double *__restrict__ b,
                                                 double *__restrict__ y, const int *gate) {
  dep_sync();
  if (gated(gate)) return;
  apply64_body<TX, X>(g, w, code, x, b, y, blockIdx.x, blockIdx.y, blockIdx.z);
}

template <bool X>
__global__ void __launch_bounds__(256) k_apply32(Geom g, const float *__restrict__ gf, const float *__restrict__ aj,
                                                 const uint32_t *__restrict__ code, const float *__restrict__ x,
                                                 const float *__restrict__ b, float *__restrict__ y, const int *gate) {
  dep_sync();
  if (gated(gate)) return;
  apply32_march_body<X>(g, gf, aj, code, x, b, y, blockIdx.x, blockIdx.y, blockIdx.z);
}
static dim3 march_grid(const Geom &g) {
  MarchGrid m = MarchGrid::of(g);
  return dim3(m.gx, m.gy, m.gz);
}
static const dim3 kMarchBlk(32, 8, 1);

static dim3 grid3(const Geom &g) { return dim3(nblk(g.mx, 32), nblk(g.my, 4), g.mz); }
static const dim3 kBlk(32, 4, 1);

template <typename TX>
static void apply64(const LevelDev &L, const TX *x, const double *b, double *y, cudaStream_t s) {
  const dim3 grd(plane_blocks(L.g), 1, L.g.mz);
  if (L.cross64) launch_dep(k_apply64<TX, true>, grd, kFlat, 0, s, L.g, L.w64, L.code, x, b, y, L.gate);
  else launch_dep(k_apply64<TX, false>, grd, kFlat, 0, s, L.g, L.w64, L.code, x, b, y, L.gate);
}
static void apply32(const LevelDev &L, const float *x, const float *b, float *y, cudaStream_t s) {
  if (L.cross32)
    launch_dep(k_apply32<true>, march_grid(L.g), kMarchBlk, 0, s, L.g, L.gf32, L.ajf32, L.code, x, b, y, L.gate);
  else
    launch_dep(k_apply32<false>, march_grid(L.g), kMarchBlk, 0, s, L.g, L.gf32, L.ajf32, L.code, x, b, y, L.gate);
}
template <>
void launch_apply<double>(const LevelDev &L, const double *x, double *y, cudaStream_t s) {
  apply64<double>(L, x, nullptr, y, s);
}
template <>
void launch_residual<double>(const LevelDev &L, const double *b, const double *x, double *r, cudaStream_t s) {
  apply64<double>(L, x, b, r, s);
}
void launch_apply64_from32(const LevelDev &L, const float *x, double *y, cudaStream_t s) {
  apply64<float>(L, x, nullptr, y, s);
}
template <>
void launch_apply<float>(const LevelDev &L, const float *x, float *y, cudaStream_t s) {
  apply32(L, x, nullptr, y, s);
}
template <>
void launch_residual<float>(const LevelDev &L, const float *b, const float *x, float *r, cudaStream_t s) {
  apply32(L, x, b, r, s);
}

template <typename T, int TW, bool X>
__global__ void __launch_bounds__(256, 3) k_line_sweep(LevelDev L, const T *__restrict__ b, const T *__restrict__ x,
                                                       T *__restrict__ xnew, T omega, int mode) {
  dep_sync();
  if (gated(L.gate)) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  line_sweep_body<T, TW, X>(L, b, x, xnew, omega, mode, blockIdx.x, blockIdx.y, smem_raw);
}

// RR: the line layout's rows per lane fixed at compile time (0: read from my)
template <typename T, int TW, int RR>
__global__ void __launch_bounds__(kSolveThreads, kTileMinBlocks<T, TW, RR>) k_line_solve(LevelDev L, const T *__restrict__ r, const T *x,
                                                                 T *xnew, T omega, int color, int rsplit) {
  dep_sync();
  if (gated(L.gate)) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  line_solve_body<T, TW, RR>(L, r, x, xnew, omega, blockIdx.x, blockIdx.y, smem_raw, color, rsplit != 0);
}

template <typename T, int TW, int RR, bool X>
__global__ void __launch_bounds__(kSolveThreads, X ? 4 : kTileMinBlocks<T, TW, RR>) k_zebra_fused(LevelDev L, const T *__restrict__ b, const T *xin,
                                                                  T *xout, T omega, int color) {
  dep_sync();
  if (gated(L.gate)) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  zebra_fused_body<T, TW, RR, X>(L, b, xin, xout, omega, blockIdx.x, blockIdx.y, smem_raw, color);
}

template <typename T, bool X>
__global__ void __launch_bounds__(128) k_resid_color(LevelDev L, const T *__restrict__ x, const T *__restrict__ b,
                                                     T *__restrict__ r, int color) {
  dep_sync();
  if (gated(L.gate)) return;
  resid_color_body<T, X>(L, x, b, r, color, blockIdx.x, blockIdx.y, blockIdx.z);
}
// mode 0: zero initial guess (residual = b); 1: residual b - A x computed in
// the sweep (fused); 2: `b` already holds the residual of x (split variant).
template <typename T, int TW>
static void line_sweep(const LevelDev &L, const T *b, const T *x, T *xnew, T omega, int mode, cudaStream_t s) {
  size_t smem = sizeof(T) * 4 * (size_t)L.g.my * TW;
  dim3 grd(nblk(L.g.mx, TW), L.g.mz);
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_line_sweep<T, TW, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    cudaFuncSetAttribute(k_line_sweep<T, TW, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    attr = true;
  }
  if (has_cross<T>(L)) launch_dep(k_line_sweep<T, TW, true>, grd, 256, smem, s, L, b, x, xnew, omega, mode);
  else launch_dep(k_line_sweep<T, TW, false>, grd, 256, smem, s, L, b, x, xnew, omega, mode);
}


template <typename T, int TW, int RR>
static void line_solve_r(const LevelDev &L, const T *r, const T *x, T *xnew, T omega, cudaStream_t s, int color,
                         int rsplit) {
  dim3 grd(solve_tiles_x<TW>(L.g, color), L.g.mz);
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_line_solve<T, TW, RR>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    attr = true;
  }
  launch_dep(k_line_solve<T, TW, RR>, grd, kSolveThreads, line_solve_smem_rr<T, TW>(L.g, RR), s, L, r, x, xnew, omega,
             color, rsplit);
}
template <typename T, int TW>
static void line_solve(const LevelDev &L, const T *r, const T *x, T *xnew, T omega, cudaStream_t s, int color = -1,
                       int rsplit = 0) {
  switch (LineLayout::of(L.g.my).R) {
    case 1: line_solve_r<T, TW, 1>(L, r, x, xnew, omega, s, color, rsplit); break;
    case 2: line_solve_r<T, TW, 2>(L, r, x, xnew, omega, s, color, rsplit); break;
    case 4: line_solve_r<T, TW, 4>(L, r, x, xnew, omega, s, color, rsplit); break;
    case 8: line_solve_r<T, TW, 8>(L, r, x, xnew, omega, s, color, rsplit); break;
    default: line_solve_r<T, TW, 0>(L, r, x, xnew, omega, s, color, rsplit); break;
  }
}

// Lines longer than the shared-memory tile allows fall back to a residual
// kernel plus a one-thread-per-line Thomas kernel.
template <typename T>
__global__ void k_line_thomas(Geom g, const T *__restrict__ fac, const T *__restrict__ r,
                              const T *__restrict__ x, T *__restrict__ xnew, T omega, int zero_guess,
                              const int *gate) {
  dep_sync();
  if (gated(gate)) return;
  size_t n = g.n();
  int i = blockIdx.x * blockDim.x + threadIdx.x, k = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= g.mx || k >= g.mz) return;
  bool ring = (i == 0 || i == g.mx - 1 || k == 0 || k == g.mz - 1);
  if (ring) {
    for (int j = 0; j < g.my; j++) {
      size_t p = g.id(i, j, k);
      xnew[p] = zero_guess ? T(0) : x[p];
    }
    return;
  }
  const LineFac F = LineFac::of(g);
  const T *a = fac + F.line(i, k) - 1, *minv = a + F.Q, *cp = minv + F.Q;  // indexed by j
  T dprev = T(0);
  size_t p0 = g.id(i, 0, k);
  xnew[p0] = zero_guess ? T(0) : x[p0];
  for (int j = 1; j <= g.my - 2; j++) {
    size_t p = g.id(i, j, k);
    T d = (r[p] - a[j] * dprev) * minv[j];
    xnew[p] = d;
    dprev = d;
  }
  size_t pe = g.id(i, g.my - 1, k);
  xnew[pe] = zero_guess ? T(0) : x[pe];
  T dn = T(0);
  for (int j = g.my - 2; j >= 1; j--) {
    size_t p = g.id(i, j, k);
    T d = xnew[p] - cp[j] * dn;
    dn = d;
    xnew[p] = zero_guess ? omega * d : x[p] + omega * d;
  }
}

static const int kMaxFusedRows = 400;
static const size_t kMaxSmem = 200 * 1024;

// Sweep variants: fused (residual inside the tile kernel) or split (a full-
// occupancy residual kernel into L.t32 / L.t64, then the asynchronous-copy
// line solve on it).  A zero-guess sweep is the line solve on b.
// The set-up autotuner stores the faster one per level in L.sweep32 / L.sweep64.
template <>
void launch_line_smooth<float>(const LevelDev &L, const float *b, const float *x, float *xnew, float omega,
                               int zero_guess, cudaStream_t s) {
  if (L.g.my <= kMaxFusedRows) {
    const bool async = line_solve_smem<float, kSolveTW32>(L.g) <= kMaxSmem;
    if (zero_guess) {
      if (async) line_solve<float, kSolveTW32>(L, b, nullptr, xnew, omega, s);
      else line_sweep<float, 32>(L, b, x, xnew, omega, 0, s);
    } else if (L.sweep32 == 1) {
      launch_residual<float>(L, b, x, L.t32, s);
      if (async) line_solve<float, kSolveTW32>(L, L.t32, x, xnew, omega, s);
      else line_sweep<float, 32>(L, L.t32, x, xnew, omega, 2, s);
    } else {
      line_sweep<float, 32>(L, b, x, xnew, omega, 1, s);
    }
    return;
  }
  const float *r = b;
  if (!zero_guess) { launch_residual<float>(L, b, x, L.t32, s); r = L.t32; }
  dim3 blk(32, 4), grd(nblk(L.g.mx, 32), nblk(L.g.mz, 4));
  launch_dep(k_line_thomas<float>, grd, blk, 0, s, L.g, L.line32, r, x, xnew, omega, zero_guess, L.gate);
}
template <>
void launch_line_smooth<double>(const LevelDev &L, const double *b, const double *x, double *xnew, double omega,
                                int zero_guess, cudaStream_t s) {
  if (L.g.my <= kMaxFusedRows) {
    const bool async = line_solve_smem<double, kSolveTW64>(L.g) <= kMaxSmem;
    if (zero_guess) {
      if (async) line_solve<double, kSolveTW64>(L, b, nullptr, xnew, omega, s);
      else line_sweep<double, 16>(L, b, x, xnew, omega, 0, s);
    } else if (L.sweep64 == 1) {
      launch_residual<double>(L, b, x, L.t64, s);
      if (async) line_solve<double, kSolveTW64>(L, L.t64, x, xnew, omega, s);
      else line_sweep<double, 16>(L, L.t64, x, xnew, omega, 2, s);
    } else {
      line_sweep<double, 16>(L, b, x, xnew, omega, 1, s);
    }
    return;
  }
  const double *r = b;
  if (!zero_guess) { launch_residual<double>(L, b, x, L.t64, s); r = L.t64; }
  dim3 blk(32, 4), grd(nblk(L.g.mx, 32), nblk(L.g.mz, 4));
  launch_dep(k_line_thomas<double>, grd, blk, 0, s, L.g, L.line64, r, x, xnew, omega, zero_guess, L.gate);
}

// Zebra (two-color) y-line relaxation: one half-sweep updates the lines of one
// color, (i + k) % 2 == color, in place: residual on those lines, then their
// line solves.  zero: x is zero on entry (the caller zeroed it); only the
// solves run, on r = b.
template <typename T, int TW, int RR, bool X>
static void zebra_fused_rx(const LevelDev &L, const T *b, const T *xin, T *xout, T omega, int color, cudaStream_t s) {
  dim3 grd(solve_tiles_x<TW>(L.g, color), L.g.mz);
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_zebra_fused<T, TW, RR, X>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    attr = true;
  }
  launch_dep(k_zebra_fused<T, TW, RR, X>, grd, kSolveThreads, line_solve_smem_rr<T, TW>(L.g, RR), s, L, b, xin, xout, omega,
             color);
}
template <typename T, int TW, int RR>
static void zebra_fused_r(const LevelDev &L, const T *b, const T *xin, T *xout, T omega, int color, cudaStream_t s) {
  if (has_cross<T>(L)) zebra_fused_rx<T, TW, RR, true>(L, b, xin, xout, omega, color, s);
  else zebra_fused_rx<T, TW, RR, false>(L, b, xin, xout, omega, color, s);
}
// One-kernel half-sweep, xin -> xout (in place when they are equal), TW lines
// per block.
template <typename T, int TW>
static void zebra_fused_tw(const LevelDev &L, const T *b, const T *xin, T *xout, T omega, int color,
                           cudaStream_t s) {
  switch (LineLayout::of(L.g.my).R) {
    case 1: zebra_fused_r<T, TW, 1>(L, b, xin, xout, omega, color, s); break;
    case 2: zebra_fused_r<T, TW, 2>(L, b, xin, xout, omega, color, s); break;
    case 4: zebra_fused_r<T, TW, 4>(L, b, xin, xout, omega, color, s); break;
    case 8: zebra_fused_r<T, TW, 8>(L, b, xin, xout, omega, color, s); break;
    default: zebra_fused_r<T, TW, 0>(L, b, xin, xout, omega, color, s); break;
  }
}
// The tile width the level's set-up chose: FP32 4 or 8 lines per block, FP64 4.
template <typename T>
static void zebra_fused(const LevelDev &L, const T *b, const T *xin, T *xout, T omega, int color, cudaStream_t s) {
  if (sizeof(T) == 4 && L.ztw32 == 4) zebra_fused_tw<T, 4>(L, b, xin, xout, omega, color, s);
  else zebra_fused_tw<T, sizeof(T) == 4 ? kSolveTW32 : kSolveTW64>(L, b, xin, xout, omega, color, s);
}
template <typename T>
static bool fused_ok(const LevelDev &L) {
  constexpr int TW = sizeof(T) == 4 ? kSolveTW32 : kSolveTW64;
  const bool chosen = sizeof(T) == 4 ? L.zfuse32 != 0 : L.zfuse64 != 0;
  return chosen && L.g.my <= kMaxFusedRows && line_solve_smem<T, TW>(L.g) <= kMaxSmem;
}

template <typename T>
void launch_zebra_half(const LevelDev &L, const T *b, T *x, T *res, T omega, int color, bool zero, cudaStream_t s) {
  constexpr int TW = sizeof(T) == 4 ? kSolveTW32 : kSolveTW64;
  if constexpr (sizeof(T) == 4) {
    if (!zero && L.ztma32 &&
        launch_zebra_tma(L, reinterpret_cast<const float *>(b), reinterpret_cast<float *>(x), (float)omega, color,
                         L.ztma32, s))
      return;
  }
  if (!zero && fused_ok<T>(L) && zebra_fusable<T>(L)) {
    zebra_fused<T>(L, b, x, x, omega, color, s);
    return;
  }
  const T *r = b;
  if (!zero) {
    dim3 grd(color_plane_blocks(L.g), 1, L.g.mz - 2);
    if (has_cross<T>(L)) launch_dep(k_resid_color<T, true>, grd, kFlat, 0, s, L, x, b, res, color);
    else launch_dep(k_resid_color<T, false>, grd, kFlat, 0, s, L, x, b, res, color);
    r = res;
  }
  if (sizeof(T) == 4 && L.ztw32 == 4) line_solve<T, 4>(L, r, zero ? nullptr : x, x, omega, s, color, zero ? 0 : 1);
  else line_solve<T, TW>(L, r, zero ? nullptr : x, x, omega, s, color, zero ? 0 : 1);
}

template <typename T>
void launch_zebra_sweep(const LevelDev &L, const T *b, T *x, T *tmp, T *res, T omega, bool zero_first,
                        cudaStream_t s) {
  if (!zero_first && fused_ok<T>(L) && !zebra_fusable<T>(L)) {
    // one-kernel half-sweeps out of place: x -> tmp -> x
    zebra_fused<T>(L, b, x, tmp, omega, 0, s);
    zebra_fused<T>(L, b, tmp, x, omega, 1, s);
    return;
  }
  launch_zebra_half<T>(L, b, x, res, omega, 0, zero_first, s);
  launch_zebra_half<T>(L, b, x, res, omega, 1, false, s);
}
template void launch_zebra_sweep<float>(const LevelDev &, const float *, float *, float *, float *, float, bool,
                                        cudaStream_t);
template void launch_zebra_sweep<double>(const LevelDev &, const double *, double *, double *, double *, double, bool,
                                         cudaStream_t);
template void launch_zebra_half<float>(const LevelDev &, const float *, float *, float *, float, int, bool,
                                       cudaStream_t);
template void launch_zebra_half<double>(const LevelDev &, const double *, double *, double *, double, int, bool,
                                        cudaStream_t);

// ------------------------------------------------------------------ transfers
// zero_c, when set, is zeroed over the coarse grid in the same pass (the next
// level's correction, which its V-cycle updates in place).
template <typename T>
__global__ void k_restrict(const __grid_constant__ LevelDev F, const __grid_constant__ LevelDev C,
                           const T *__restrict__ xf, T *__restrict__ xc, T *__restrict__ zero_c) {
  dep_sync();
  if (gated(F.gate)) return;
  if (zero_c) {
    const int idx = blockIdx.x * kFlat + threadIdx.x, pl = C.g.mx * C.g.my;
    if (idx < pl) zero_c[(size_t)blockIdx.z * pl + idx] = T(0);
  }
  restrict_body<T>(F, C, xf, xc, blockIdx.x, blockIdx.y, blockIdx.z);
}

template <typename T>
__global__ void k_prolong_add(const __grid_constant__ LevelDev C, const __grid_constant__ LevelDev F,
                              const T *__restrict__ xc, T *__restrict__ xf) {
  dep_sync();
  if (gated(F.gate)) return;
  prolong_body<T>(C, F, xc, xf, blockIdx.x, blockIdx.y, blockIdx.z);
}

template <typename T>
void launch_restrict(const LevelDev &F, const LevelDev &C, const T *xf, T *xc, cudaStream_t s, T *zero_c) {
  launch_dep(k_restrict<T>, dim3(plane_blocks(C.g), 1, C.g.mz), kFlat, 0, s, F, C, xf, xc, zero_c);
}
template <typename T>
void launch_prolong_add(const LevelDev &C, const LevelDev &F, const T *xc, T *xf, cudaStream_t s) {
  launch_dep(k_prolong_add<T>, dim3(plane_blocks(F.g), 1, F.g.mz), kFlat, 0, s, C, F, xc, xf);
}
template void launch_restrict<float>(const LevelDev &, const LevelDev &, const float *, float *, cudaStream_t,
                                     float *);
template void launch_restrict<double>(const LevelDev &, const LevelDev &, const double *, double *, cudaStream_t,
                                      double *);
template void launch_prolong_add<float>(const LevelDev &, const LevelDev &, const float *, float *, cudaStream_t);
template void launch_prolong_add<double>(const LevelDev &, const LevelDev &, const double *, double *, cudaStream_t);

}  // namespace cvb
