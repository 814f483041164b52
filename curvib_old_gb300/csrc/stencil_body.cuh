// Device code of the curvilinear pressure operator, its y-line smoother and the
// grid transfers, shared by the single-problem kernels (kernels_stencil.cu) and
// the grouped kernels of the batch engine (kernels_batch.cu).
//
// FP64: y = A x with the 19 stored weights per row (the reference's assembled
//       PoissonLHSNew rows), 19 FMAs per cell -- the cheapest FP64 form on a
//       part whose FP64 rate is a small fraction of its FP32 rate.
// FP32: the same operator matrix-free in flux form: for each face the flux
//       F = g_nn (x_Q - x_P) + two cross terms whose form (central / one-sided /
//       none) comes from the cell's switching code; row P is
//       -aj_P * (F_E - F_W + F_N - F_S + F_T - F_B), each term taken only where
//       the face is active from P's side.  Reads 9 face coefficients, aj and a
//       code per cell: ~52 B/cell.
#pragma once
#include "cvb_internal.h"
#include "launch.cuh"

namespace cvb {


// ------------------------------------------------------ per-plane blocks
// The per-cell kernels (FP64 rows, zebra residual, transfers) take 1-D blocks
// of kFlat threads over the cells of one plane, flattened i-fastest: a warp
// covers 32 consecutive cells whatever the row length, so narrow boxes (the
// 32^3..128^3 problems of a batch) leave no lanes idle at the row ends.
constexpr int kFlat = 128;
__host__ __device__ inline int plane_blocks(const Geom &g) { return (g.mx * g.my + kFlat - 1) / kFlat; }
// interior cells of one zebra colour in a plane: at most (mx-1)/2 per row
__host__ __device__ inline int color_plane_blocks(const Geom &g) {
  return (((g.mx - 1) / 2) * (g.my - 2) + kFlat - 1) / kFlat;
}

// ------------------------------------------------------------ neighbourhood
// 32-bit offsets of the six face neighbours, with the reference's periodic wrap
// of column indices (poisson.c:1329-1450) folded into the offset at seam cells.
struct Off {
  int e, w, n, s, t, b;
};
__device__ __forceinline__ Off offsets(const Geom &g, int i, int j, int k) {
  const int sy = g.mx, sz = g.mx * g.my;
  Off o;
  o.e = (g.px && i == g.mx - 2) ? -(g.mx - 3) : 1;
  o.w = (g.px && i == 1) ? (g.mx - 3) : -1;
  o.n = (g.py && j == g.my - 2) ? -(g.my - 3) * sy : sy;
  o.s = (g.py && j == 1) ? (g.my - 3) * sy : -sy;
  o.t = (g.pz && k == g.mz - 2) ? -(g.mz - 3) * sz : sz;
  o.b = (g.pz && k == 1) ? (g.mz - 3) * sz : -sz;
  return o;
}

// The 19 values of x around an interior cell, in registers.
template <typename T>
struct Star {
  T P, E, W, N, S, Tt, B, NE, SE, NW, SW, TN, BN, TS, BS, TE, BE, TW, BW;
};
template <typename T, typename TX>
__device__ __forceinline__ Star<T> load_star(const TX *__restrict__ x, int p, const Off &o) {
  Star<T> s;
  s.P = (T)x[p];
  s.E = (T)x[p + o.e]; s.W = (T)x[p + o.w]; s.N = (T)x[p + o.n]; s.S = (T)x[p + o.s];
  s.Tt = (T)x[p + o.t]; s.B = (T)x[p + o.b];
  s.NE = (T)x[p + o.e + o.n]; s.SE = (T)x[p + o.e + o.s]; s.NW = (T)x[p + o.w + o.n]; s.SW = (T)x[p + o.w + o.s];
  s.TN = (T)x[p + o.t + o.n]; s.BN = (T)x[p + o.b + o.n]; s.TS = (T)x[p + o.t + o.s]; s.BS = (T)x[p + o.b + o.s];
  s.TE = (T)x[p + o.t + o.e]; s.BE = (T)x[p + o.b + o.e]; s.TW = (T)x[p + o.t + o.w]; s.BW = (T)x[p + o.b + o.w];
  return s;
}

// ----------------------------------------------------------------- FP64 rows
// (A x)_p with the 19 stored weights; identity rows return x_p.  Every load of
// the row is issued before anything depends on one of them (the row's code
// included), so a row costs one memory latency, not a chain of them.
// X: the level has cross-derivative weights; without them (an orthogonal grid,
// the 12 edge slots all zero) only the seven face slots are read, which gives
// the same sum: every skipped term is an fma with a zero weight.
template <typename TX, bool X = true>
__device__ __forceinline__ double row64(const Geom &g, const double *__restrict__ w, const uint32_t *__restrict__ code,
                                        const TX *__restrict__ x, int i, int j, int k, int p, int n) {
  if (i < 1 || i > g.mx - 2 || j < 1 || j > g.my - 2 || k < 1 || k > g.mz - 2) return (double)x[p];
  Off o = offsets(g, i, j, k);
  uint32_t c = __ldg(code + p);
  Star<double> s = load_star<double>(x, p, o);
  const double *wp = w + p;
  double r = __ldg(wp + (size_t)CP * n) * s.P;
  r = fma(__ldg(wp + (size_t)EP * n), s.E, r); r = fma(__ldg(wp + (size_t)WP * n), s.W, r);
  r = fma(__ldg(wp + (size_t)NP * n), s.N, r); r = fma(__ldg(wp + (size_t)SP * n), s.S, r);
  r = fma(__ldg(wp + (size_t)TP * n), s.Tt, r); r = fma(__ldg(wp + (size_t)BP * n), s.B, r);
  if constexpr (X) {
    r = fma(__ldg(wp + (size_t)NE * n), s.NE, r); r = fma(__ldg(wp + (size_t)SE * n), s.SE, r);
    r = fma(__ldg(wp + (size_t)NW * n), s.NW, r); r = fma(__ldg(wp + (size_t)SW * n), s.SW, r);
    r = fma(__ldg(wp + (size_t)TN * n), s.TN, r); r = fma(__ldg(wp + (size_t)BN * n), s.BN, r);
    r = fma(__ldg(wp + (size_t)TS * n), s.TS, r); r = fma(__ldg(wp + (size_t)BS * n), s.BS, r);
    r = fma(__ldg(wp + (size_t)TE * n), s.TE, r); r = fma(__ldg(wp + (size_t)BE * n), s.BE, r);
    r = fma(__ldg(wp + (size_t)TW * n), s.TW, r); r = fma(__ldg(wp + (size_t)BW * n), s.BW, r);
  }
  return (c & CODE_IDENTITY) ? s.P : r;
}

// ----------------------------------------------------------------- FP32 rows
// Cross term of a face flux: g * (cu*s_up + c0*s_level + cd*s_down) for the
// central / lower / upper forms (branch 1/2/3), zero for branch 0.
// Cross term of a face flux.  The coefficient gs was scaled at set-up by the
// form's weight (central 1/4, one-sided 1/2, none 0), so the term is
// gs * (sA - sB) with (sA, sB) = (s_up, s_down) central, (s_level, s_down) lower,
// (s_up, s_level) upper.
__device__ __forceinline__ float cross32(int br, float gs, float su, float s0, float sd) {
  return gs * ((br == 2 ? s0 : su) - (br == 3 ? s0 : sd));
}
__device__ __forceinline__ float act(uint32_t c, uint32_t bit) { return (c & bit) ? 1.0f : 0.0f; }

// (A x)_p in flux form: each active face flux from its cell's coefficients and
// branch codes; the lower faces are the upper faces of the W/S/B neighbours.
// Loads first (all unconditional, in bounds for interior cells), then the
// arithmetic with the activity bits as 0/1 factors.
// X: the level has cross-derivative coefficients; without them (an orthogonal
// grid) each face flux is its normal term alone and only the seven face
// values of x are read.
template <typename TX, bool X = true>
__device__ __forceinline__ float row32(const Geom &g, const float *__restrict__ gf, const float *__restrict__ aj,
                                       const uint32_t *__restrict__ code, const TX *__restrict__ x, int i, int j,
                                       int k, int p, int n) {
  if (i < 1 || i > g.mx - 2 || j < 1 || j > g.my - 2 || k < 1 || k > g.mz - 2) return (float)x[p];
  Off o = offsets(g, i, j, k);
  const int pw = p - 1, ps = p - g.mx, pb = p - g.mx * g.my;  // lower neighbours (never wrapped)
  const uint32_t c = __ldg(code + p), cw = __ldg(code + pw), cs = __ldg(code + ps), cb = __ldg(code + pb);
  Star<float> s = load_star<float>(x, p, o);
  const float g11 = __ldg(gf + p), g12 = __ldg(gf + n + p), g13 = __ldg(gf + 2 * n + p);
  const float g21 = __ldg(gf + 3 * n + p), g22 = __ldg(gf + 4 * n + p), g23 = __ldg(gf + 5 * n + p);
  const float g31 = __ldg(gf + 6 * n + p), g32 = __ldg(gf + 7 * n + p), g33 = __ldg(gf + 8 * n + p);
  const float w11 = __ldg(gf + pw), w12 = __ldg(gf + n + pw), w13 = __ldg(gf + 2 * n + pw);
  const float s21 = __ldg(gf + 3 * n + ps), s22 = __ldg(gf + 4 * n + ps), s23 = __ldg(gf + 5 * n + ps);
  const float b31 = __ldg(gf + 6 * n + pb), b32 = __ldg(gf + 7 * n + pb), b33 = __ldg(gf + 8 * n + pb);
  const float ajp = __ldg(aj + p);
  float fe = g11 * (s.E - s.P), fw = w11 * (s.P - s.W), fn = g22 * (s.N - s.P);
  float fs = s22 * (s.P - s.S), ft = g33 * (s.Tt - s.P), fb = b33 * (s.P - s.B);
  if constexpr (X) {
    fe = fe + cross32(code_branch(c, 0, 0), g12, s.N + s.NE, s.P + s.E, s.S + s.SE) +
         cross32(code_branch(c, 0, 1), g13, s.Tt + s.TE, s.P + s.E, s.B + s.BE);
    fw = fw + cross32(code_branch(cw, 0, 0), w12, s.NW + s.N, s.W + s.P, s.SW + s.S) +
         cross32(code_branch(cw, 0, 1), w13, s.TW + s.Tt, s.W + s.P, s.BW + s.B);
    fn = fn + cross32(code_branch(c, 1, 0), g21, s.E + s.NE, s.P + s.N, s.W + s.NW) +
         cross32(code_branch(c, 1, 1), g23, s.Tt + s.TN, s.P + s.N, s.B + s.BN);
    fs = fs + cross32(code_branch(cs, 1, 0), s21, s.SE + s.E, s.S + s.P, s.SW + s.W) +
         cross32(code_branch(cs, 1, 1), s23, s.TS + s.Tt, s.S + s.P, s.BS + s.B);
    ft = ft + cross32(code_branch(c, 2, 0), g31, s.E + s.TE, s.P + s.Tt, s.W + s.TW) +
         cross32(code_branch(c, 2, 1), g32, s.N + s.TN, s.P + s.Tt, s.S + s.TS);
    fb = fb + cross32(code_branch(cb, 2, 0), b31, s.BE + s.E, s.B + s.P, s.BW + s.W) +
         cross32(code_branch(cb, 2, 1), b32, s.BN + s.N, s.B + s.P, s.BS + s.S);
  }
  float acc = act(c, CODE_ACT_E) * fe - act(c, CODE_ACT_W) * fw + act(c, CODE_ACT_N) * fn -
              act(c, CODE_ACT_S) * fs + act(c, CODE_ACT_T) * ft - act(c, CODE_ACT_B) * fb;
  return (c & CODE_IDENTITY) ? s.P : -ajp * acc;
}

// (A x)_p without cross terms from the colour-split copies of the coefficients
// (L.cs32: g11, g22, g33, aj and the code's bits, SplitRow::count values each):
// the cells of one zebra colour sit side by side there, so a half-sweep, which
// needs the coefficients of one colour's cells, reads whole sectors of them
// instead of every other value.  The same operands, flux form and order as
// row32<TX, false>; the W, S and B faces are the E, N and T faces of the
// neighbours i - 1, j - 1, k - 1 (never wrapped).  Interior cells only (the
// zebra kernels' cells): their split positions follow from the cell's own, q,
// with the row of the other colour h away -- i - 1 and k - 1 are of the other
// colour, j - 1 of the same.  (The same copies of the nine 19-point
// coefficients made that residual slower on the GB300, 119 against 115 us per
// half-sweep at 192^3: there the W, S and B neighbours' reads share cache lines
// with the other cells' own in the caller's layout, and the kernel is bound by
// its instructions more than by DRAM.)
__device__ __forceinline__ float row32_split(const Geom &g, const float *__restrict__ cs,
                                             const float *__restrict__ x, int i, int j, int k, int p) {
  const int h = SplitRow::half(g), c2 = (i + k) & 1;
  const size_t S = (size_t)g.my * g.mz * 2 * h;
  const int q = ((k * g.my + j) * 2 + c2) * h + (i >> 1);
  const int other = c2 ? -h : h;  // own colour's row -> the other colour's
  const int qw = q + other + ((i - 1) >> 1) - (i >> 1), qs = q - 2 * h, qb = q - g.my * 2 * h + other;
  const Off o = offsets(g, i, j, k);
  const uint32_t c = __float_as_uint(__ldg(cs + 4 * S + q));
  const float P = x[p], E = x[p + o.e], W = x[p + o.w], N = x[p + o.n], Sv = x[p + o.s], T = x[p + o.t],
              B = x[p + o.b];
  const float g11 = __ldg(cs + q), w11 = __ldg(cs + qw), g22 = __ldg(cs + S + q), s22 = __ldg(cs + S + qs);
  const float g33 = __ldg(cs + 2 * S + q), b33 = __ldg(cs + 2 * S + qb), ajp = __ldg(cs + 3 * S + q);
  const float fe = g11 * (E - P), fw = w11 * (P - W), fn = g22 * (N - P);
  const float fs = s22 * (P - Sv), ft = g33 * (T - P), fb = b33 * (P - B);
  const float acc = act(c, CODE_ACT_E) * fe - act(c, CODE_ACT_W) * fw + act(c, CODE_ACT_N) * fn -
                    act(c, CODE_ACT_S) * fs + act(c, CODE_ACT_T) * ft - act(c, CODE_ACT_B) * fb;
  return (c & CODE_IDENTITY) ? P : -ajp * acc;
}

// ------------------------------------------------------- apply / residual
// y = A x (b == nullptr) or y = b - A x.  One thread per cell.
// Bodies take the block's coordinates explicitly so that the grouped (batched)
// kernels can run them for any problem of a work-list: (bx, bz) = (block of the
// plane, plane), kFlat threads.
template <typename TX, bool X = true>
__device__ __forceinline__ void apply64_body(const Geom &g, const double *__restrict__ w,
                                             const uint32_t *__restrict__ code, const TX *__restrict__ x,
                                             const double *__restrict__ b, double *__restrict__ y, int bx, int by,
                                             int bz) {
  (void)by;
  const int pl = g.mx * g.my, idx = bx * kFlat + threadIdx.x;
  if (idx >= pl) return;
  const int j = idx / g.mx, i = idx - j * g.mx, k = bz;
  const int n = (int)g.n(), p = k * pl + idx;
  double ax = row64<TX, X>(g, w, code, x, i, j, k, p, n);
  y[p] = b ? b[p] - ax : ax;
}


// ---------------------------------------------- FP32 apply, face fluxes shared
// Each face flux is computed once: a thread owns its cell's three upper faces
// (E, N, T); its W face is the E face of the lane to its left (a shuffle), its S
// face the N face of the warp below (shared memory), its B face its own T face
// of the previous plane (the block marches in k).  Tiles overlap by one cell in
// x and y (lane 0 and warp 0 only supply fluxes).  x is read at wrapped
// coordinates (a ring cell of a periodic direction reads its image), the
// coefficients and codes at the cell's own position -- as row32 does, with the
// same operations in the same order.  About 20 loads and 3 face fluxes per
// cell instead of 42 and 6.
// A tile marches kd planes: 16 where the level has blocks to spare, fewer
// (down to 2) until the grid has kMarchMinBlocks blocks, so that small levels
// still spread over the SMs instead of running a few long marches.
#ifndef CVB_MARCH_MIN_BLOCKS
#define CVB_MARCH_MIN_BLOCKS 2432
#endif
constexpr int kMarchX = 31, kMarchY = 7, kMarchK = 16, kMarchMinBlocks = CVB_MARCH_MIN_BLOCKS;

struct MarchGrid {
  int gx, gy, gz, kd;
  __host__ __device__ static MarchGrid of(const Geom &g) {
    MarchGrid m;
    m.gx = (g.mx + kMarchX - 1) / kMarchX;
    m.gy = (g.my + kMarchY - 1) / kMarchY;
    m.kd = kMarchK;
    while (m.kd > 2 && m.gx * m.gy * ((g.mz + m.kd - 1) / m.kd) < kMarchMinBlocks) m.kd >>= 1;
    m.gz = (g.mz + m.kd - 1) / m.kd;
    return m;
  }
  __host__ __device__ int blocks() const { return gx * gy * gz; }
};

// coordinate of x read for column i of a box of m cells (periodic: the ring
// and beyond fold onto the image; otherwise clamped -- such values are unused)
__device__ __forceinline__ int wrap_read(int i, int m, int per) {
  if (per) {
    if (i <= 0) i += m - 2;
    else if (i >= m - 1) i -= m - 2;
  }
  return i < 0 ? 0 : (i > m - 1 ? m - 1 : i);  // always inside the box
}

// y = A x (b == nullptr) or y = b - A x on the tile (bx, by, bz); 32 x 8 threads.
// X: the level has cross-derivative coefficients (see row32).
template <bool X = true>
__device__ __forceinline__ void apply32_march_body(const Geom &g, const float *__restrict__ gf,
                                                   const float *__restrict__ aj, const uint32_t *__restrict__ code,
                                                   const float *__restrict__ x, const float *__restrict__ b,
                                                   float *__restrict__ y, int bx, int by, int bz) {
  __shared__ float shn[2][8][32];
  const int lane = threadIdx.x, w = threadIdx.y;
  const int mx = g.mx, my = g.my, mz = g.mz, n = (int)g.n(), pl = mx * my;
  const int i = bx * kMarchX - 1 + lane, j = by * kMarchY - 1 + w;
  const int kd = MarchGrid::of(g).kd;
  const int k0 = bz * kd, k1 = min(k0 + kd, mz);
  const bool col = i >= 0 && i < mx && j >= 0 && j < my;
  const bool out = col && lane >= 1 && w >= 1;
  // columns (wrapped) of the values this thread reads in every plane
  const int iw = wrap_read(i, mx, g.px), ie = wrap_read(i + 1, mx, g.px), iv = wrap_read(i - 1, mx, g.px);
  const int jw = wrap_read(j, my, g.py), jn = wrap_read(j + 1, my, g.py), js = wrap_read(j - 1, my, g.py);
  const int cP = jw * mx + iw, cE = jw * mx + ie, cW = jw * mx + iv, cN = jn * mx + iw, cS = js * mx + iw;
  const int cNE = jn * mx + ie, cSE = js * mx + ie, cNW = jn * mx + iv;
  const int cown = (j < 0 ? 0 : (j >= my ? my - 1 : j)) * mx + (i < 0 ? 0 : (i >= mx ? mx - 1 : i));
  // the previous plane (k0 - 1): its cell values and its T face flux
  float P, E, N, W, S, B, BE, BN, ftp = 0.0f;
  {
    const int kb = k0 - 1;
    const int ob = wrap_read(kb, mz, g.pz) * pl, ot = wrap_read(k0, mz, g.pz) * pl;
    P = x[ob + cP]; E = x[ob + cE]; N = x[ob + cN];
    W = X ? x[ob + cW] : 0.f;
    S = X ? x[ob + cS] : 0.f;
    const float T = x[ot + cP], TE = x[ot + cE], TN = x[ot + cN];
    const float TW = X ? x[ot + cW] : 0.f, TS = X ? x[ot + cS] : 0.f;
    if (kb >= 0 && col) {
      const int q = kb * pl + cown;
      const float g33 = __ldg(gf + 8 * n + q);
      ftp = g33 * (T - P);
      if constexpr (X) {
        const uint32_t c = __ldg(code + q);
        const float g31 = __ldg(gf + 6 * n + q), g32 = __ldg(gf + 7 * n + q);
        ftp = ftp + cross32(code_branch(c, 2, 0), g31, E + TE, P + T, W + TW) +
              cross32(code_branch(c, 2, 1), g32, N + TN, P + T, S + TS);
      }
    }
    B = P; BE = E; BN = N;
    P = T; E = TE; N = TN; W = TW; S = TS;
  }
  // per-plane inputs; those of plane k + 1 are loaded while plane k computes
  struct Plane {
    float T, TE, TN, TW, TS, NE, SE, NW;
    float g11, g12, g13, g21, g22, g23, g31, g32, g33, ajp, bp, xo;
    uint32_t c;
  };
  auto load = [&](int k, Plane &v) {
    const int op = wrap_read(k, mz, g.pz) * pl, ot = wrap_read(k + 1, mz, g.pz) * pl;
    v.T = x[ot + cP]; v.TE = x[ot + cE]; v.TN = x[ot + cN];
    v.TW = v.TS = v.NE = v.SE = v.NW = 0.f;
    if constexpr (X) {
      v.TW = x[ot + cW]; v.TS = x[ot + cS];
      v.NE = x[op + cNE]; v.SE = x[op + cSE]; v.NW = x[op + cNW];
    }
    v.c = CODE_IDENTITY;
    v.g11 = v.g12 = v.g13 = v.g21 = v.g22 = v.g23 = v.g31 = v.g32 = v.g33 = 0.f;
    v.ajp = v.bp = v.xo = 0.f;
    if (col) {
      const int q = k * pl + cown;
      v.c = __ldg(code + q);
      v.g11 = __ldg(gf + q); v.g22 = __ldg(gf + 4 * n + q); v.g33 = __ldg(gf + 8 * n + q);
      if constexpr (X) {
        v.g12 = __ldg(gf + n + q); v.g13 = __ldg(gf + 2 * n + q);
        v.g21 = __ldg(gf + 3 * n + q); v.g23 = __ldg(gf + 5 * n + q);
        v.g31 = __ldg(gf + 6 * n + q); v.g32 = __ldg(gf + 7 * n + q);
      }
      v.ajp = __ldg(aj + q);
      if (b && out) v.bp = b[q];
      if (out && (i == 0 || i == mx - 1 || j == 0 || j == my - 1 || k == 0 || k == mz - 1)) v.xo = x[q];
    }
  };
  Plane nx;
  load(k0, nx);
  for (int k = k0; k < k1; k++) {
    const Plane v = nx;
    if (k + 1 < k1) load(k + 1, nx);
    const uint32_t c = v.c;
    const float T = v.T, TE = v.TE, TN = v.TN, TW = v.TW, TS = v.TS, NE = v.NE, SE = v.SE, NW = v.NW;
    const int q = k * pl + cown;
    const bool ring = i == 0 || i == mx - 1 || j == 0 || j == my - 1 || k == 0 || k == mz - 1;
    const float xo = ring ? v.xo : P;
    float fe = v.g11 * (E - P), fn = v.g22 * (N - P), ft = v.g33 * (T - P);
    if constexpr (X) {
      fe = fe + cross32(code_branch(c, 0, 0), v.g12, N + NE, P + E, S + SE) +
           cross32(code_branch(c, 0, 1), v.g13, T + TE, P + E, B + BE);
      fn = fn + cross32(code_branch(c, 1, 0), v.g21, E + NE, P + N, W + NW) +
           cross32(code_branch(c, 1, 1), v.g23, T + TN, P + N, B + BN);
      ft = ft + cross32(code_branch(c, 2, 0), v.g31, E + TE, P + T, W + TW) +
           cross32(code_branch(c, 2, 1), v.g32, N + TN, P + T, S + TS);
    }
    const float fw = __shfl_up_sync(0xffffffffu, fe, 1);
    shn[k & 1][w][lane] = fn;
    __syncthreads();
    const float fs = w >= 1 ? shn[k & 1][w - 1][lane] : 0.0f;
    const float fb = ftp;
    if (out) {
      float acc = act(c, CODE_ACT_E) * fe - act(c, CODE_ACT_W) * fw + act(c, CODE_ACT_N) * fn -
                  act(c, CODE_ACT_S) * fs + act(c, CODE_ACT_T) * ft - act(c, CODE_ACT_B) * fb;
      const float ax = (c & CODE_IDENTITY) ? xo : -v.ajp * acc;
      y[q] = b ? v.bp - ax : ax;
    }
    ftp = ft;
    B = P; BE = E; BN = N;
    P = T; E = TE; N = TN; W = TW; S = TS;
  }
}

// ------------------------------------------------------------ y-line smoother
// One damped line-Jacobi sweep, fused: xnew = x + omega * T^-1 (b - A x), T the
// tridiagonal in-line (j) part of A with Thomas factors from set-up.
// A block owns a tile of TW consecutive i over all j at one k.  Phase 1: all
// threads compute the tile's residual into shared memory and stage the three
// factor arrays there (coalesced, many loads in flight; read from global inside
// the recurrence they would cost a memory latency per step).  Phase 2: TW threads
// run the forward/backward recurrences out of shared memory, one line each.
// Phase 3: all threads write x + omega*delta.  Zero guess: the residual is b.
template <typename T>
struct RowOf;
template <>
struct RowOf<float> {
  template <bool X = true>
  __device__ static float r(const Geom &g, const LevelDev &L, const float *x, int i, int j, int k, int p, int n) {
    return row32<float, X>(g, L.gf32, L.ajf32, L.code, x, i, j, k, p, n);
  }
  __device__ static const float *fac(const LevelDev &L) { return L.line32; }
};
template <>
struct RowOf<double> {
  template <bool X = true>
  __device__ static double r(const Geom &g, const LevelDev &L, const double *x, int i, int j, int k, int p, int n) {
    return row64<double, X>(g, L.w64, L.code, x, i, j, k, p, n);
  }
  __device__ static const double *fac(const LevelDev &L) { return L.line64; }
};

// Solves one line's tridiagonal system in place with one warp.  The Thomas
// passes are first-order affine recurrences, d_j = gamma_j + beta_j d_{j-1}
// (forward: gamma = m r, beta = -m a; backward: gamma = d, beta = -c), and
// affine maps compose associatively: each lane composes the maps of its
// contiguous rows, a shuffle scan combines the lanes, each lane replays its rows.
// r/a/m/c: this line's arrays in shared memory, indexed by row j = 1..nr.
template <typename T>
__device__ __forceinline__ void warp_line_solve(T *r, const T *a, const T *m, const T *c, int nr, int lane) {
  const int R = (nr + 31) >> 5;
  const int q0 = lane * R, q1 = min(q0 + R, nr);
  // forward: d_q = m_q (r_q - a_q d_{q-1})
  T B = T(1), G = T(0);
  for (int q = q0; q < q1; q++) {
    T mq = m[q + 1];
    T beta = -mq * a[q + 1], gamma = mq * r[q + 1];
    B = beta * B;
    G = beta * G + gamma;
  }
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    T Bp = __shfl_up_sync(0xffffffffu, B, o), Gp = __shfl_up_sync(0xffffffffu, G, o);
    if (lane >= o) { G = B * Gp + G; B = B * Bp; }
  }
  T d = __shfl_up_sync(0xffffffffu, G, 1);
  if (lane == 0) d = T(0);
  for (int q = q0; q < q1; q++) {
    T mq = m[q + 1];
    d = mq * r[q + 1] - mq * a[q + 1] * d;
    r[q + 1] = d;
  }
  __syncwarp();
  // backward: x_q = d_q - c_q x_{q+1}
  B = T(1); G = T(0);
  for (int q = q1 - 1; q >= q0; q--) {
    T beta = -c[q + 1], gamma = r[q + 1];
    B = beta * B;
    G = beta * G + gamma;
  }
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    T Bn = __shfl_down_sync(0xffffffffu, B, o), Gn = __shfl_down_sync(0xffffffffu, G, o);
    if (lane + o < 32) { G = B * Gn + G; B = B * Bn; }
  }
  T xs = __shfl_down_sync(0xffffffffu, G, 1);
  if (lane == 31) xs = T(0);
  for (int q = q1 - 1; q >= q0; q--) {
    xs = r[q + 1] - c[q + 1] * xs;
    r[q + 1] = xs;
  }
  __syncwarp();
}

// One damped line-Jacobi sweep, fused: xnew = x + omega * T^-1 (b - A x).
// A block owns TW lines (consecutive i at one k) over all j.  Phase 1: all
// threads compute the tile's residuals and stage the Thomas factors in shared
// memory (laid out line by line).  Phase 2: each warp solves TW/8 lines with
// warp_line_solve.  Phase 3: all threads write x + omega*delta.
template <typename T, int TW, bool X = true>
__device__ __forceinline__ void line_sweep_body(const LevelDev &L, const T *__restrict__ b, const T *__restrict__ x,
                                                T *__restrict__ xnew, T omega, int mode, int bx, int bk,
                                                unsigned char *smem_raw) {
  const Geom g = L.g;
  const int my = g.my, n = (int)g.n();
  T *sr = reinterpret_cast<T *>(smem_raw);  // [TW][my] residual -> line solution
  T *sa = sr + my * TW, *sm = sa + my * TW, *sc = sm + my * TW;
  const int tx = threadIdx.x % TW, ty = threadIdx.x / TW, ny = blockDim.x / TW;
  const int i0 = bx * TW, k = bk;
  const int i = i0 + tx;
  const bool kin = k >= 1 && k <= g.mz - 2;
  const T *fa = RowOf<T>::fac(L);
  const LineFac F = LineFac::of(g);
#pragma unroll 4
  for (int j = ty; j < my; j += ny) {
    const bool line = i >= 1 && i <= g.mx - 2 && kin;
    int p = (k * my + j) * g.mx + i;
    T r = T(0), a = T(0), m = T(1), c = T(0);
    if (line && j >= 1 && j <= my - 2) {
      const T *f = fa + F.line(i, k) + (j - 1);
      a = __ldg(f); m = __ldg(f + F.Q); c = __ldg(f + 2 * F.Q);
      r = (mode == 1) ? b[p] - RowOf<T>::template r<X>(g, L, x, i, j, k, p, n) : b[p];
    }
    sr[tx * my + j] = r; sa[tx * my + j] = a; sm[tx * my + j] = m; sc[tx * my + j] = c;
  }
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = blockDim.x >> 5;
  for (int t = warp; t < TW; t += nwarps) {
    int it = i0 + t;
    if (it >= 1 && it <= g.mx - 2 && kin)
      warp_line_solve<T>(sr + t * my, sa + t * my, sm + t * my, sc + t * my, my - 2, lane);
  }
  __syncthreads();
  if (i >= g.mx) return;
  const bool line = i >= 1 && i <= g.mx - 2 && kin;
#pragma unroll 4
  for (int j = ty; j < my; j += ny) {
    int p = (k * my + j) * g.mx + i;
    T d = sr[tx * my + j];
    T xo = (mode == 0) ? T(0) : x[p];
    xnew[p] = (line && j >= 1 && j <= my - 2) ? xo + omega * d : xo;
  }
}


// ---- line solve on a given residual, inputs staged by asynchronous copies ----
// The row pitch of a level (mx * sizeof(T), mx = IM+1) is not a multiple of 16
// bytes, so neither TMA tensor maps nor 16-byte bulk copies can address the
// tile; element-wise cp.async moves it instead.  Every thread issues all of its
// copies at once (no register staging, so no load latency per row), and the
// block waits once.
__device__ __forceinline__ void cp_async_el(float *dst, const float *src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"((unsigned)__cvta_generic_to_shared(dst)),
               "l"(src)
               : "memory");
}
__device__ __forceinline__ void cp_async_el(double *dst, const double *src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"((unsigned)__cvta_generic_to_shared(dst)),
               "l"(src)
               : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// Shared-memory layout of one line for the warp solve: lane l owns rows
// [l*R, l*R + R) (R a power of two) and keeps row l*R + t at t*33 + l, so at
// each step of its serial passes a warp reads 32 consecutive words of a row of
// 33 (no bank conflicts), and the four rows of a 16-byte load of the factors
// land in four different banks.  Lines are ls = 33*R words apart.
struct LineLayout {
  int nr, R, ls, sh;
  __host__ __device__ static LineLayout of(int my) {
    LineLayout o;
    o.nr = my - 2;
    int need = (o.nr + 31) >> 5;
    o.R = 1;
    o.sh = 0;
    while (o.R < need) { o.R <<= 1; o.sh++; }
    o.ls = 33 * o.R;
    return o;
  }
  // the layout with R fixed at compile time (RR > 0; the caller checked that it
  // is the layout of `my`), else the layout of `my`
  template <int RR>
  __host__ __device__ static LineLayout fixed(int my) {
    if (RR == 0) return of(my);
    LineLayout o;
    o.nr = my - 2;
    o.R = RR;
    o.sh = RR >= 16 ? 4 : RR >= 8 ? 3 : RR >= 4 ? 2 : RR >= 2 ? 1 : 0;
    o.ls = 33 * RR;
    return o;
  }
  __device__ int pos(int q) const { return (q & (R - 1)) * 33 + (q >> sh); }  // q = row - 1
};

// Runs f(t) for t = 0..cnt-1 (cnt <= R): unrolled when R is a compile-time RR.
template <int RR, typename F>
__device__ __forceinline__ void rows_up(int cnt, F f) {
  if constexpr (RR > 0) {
#pragma unroll
    for (int t = 0; t < RR; t++)
      if (t < cnt) f(t);
  } else {
    for (int t = 0; t < cnt; t++) f(t);
  }
}
template <int RR, typename F>
__device__ __forceinline__ void rows_down(int cnt, F f) {
  if constexpr (RR > 0) {
#pragma unroll
    for (int t = RR - 1; t >= 0; t--)
      if (t < cnt) f(t);
  } else {
    for (int t = cnt - 1; t >= 0; t--) f(t);
  }
}

// Lines per block of the line-solve kernel (128 threads, two lines per warp in
// FP32): small tiles, so that six share an SM (the register limit) and one
// tile's copies overlap another's solve.  Measured on the channel's finest
// level: 16 lines per block 92.9 us per zebra half-sweep, 8 lines 82.1 us.
constexpr int kSolveTW32 = 8, kSolveTW64 = 4, kSolveThreads = 128;

// Dynamic shared memory of the two line kernels for a level.
template <typename T, int TW>
inline size_t line_sweep_smem(const Geom &g) { return sizeof(T) * 4 * (size_t)g.my * TW; }
template <typename T, int TW>
inline size_t line_solve_smem(const Geom &g) { return sizeof(T) * 5 * (size_t)LineLayout::of(g.my).ls * TW; }

// Solves NL lines at once with one warp (line l at offset l * stride, laid out
// as LineLayout), interleaved: the recurrences and shuffle scans of different
// lines are independent, so their latencies overlap.  The Thomas passes are
// first-order affine recurrences, d_j = gamma_j + beta_j d_{j-1} (forward:
// gamma = m r, beta = -m a; backward: gamma = d, beta = -c), and affine maps
// compose associatively: each lane composes the maps of its R rows, a shuffle
// scan combines the lanes, each lane replays its rows.
// Where the warp solve finds the Thomas factors of row t of its line l: in
// shared memory beside the residual (offset o of the line layout), or in the
// lane's registers (LaneFactors).
template <typename T>
struct SmemFactors {
  const T *sa, *sm, *sc;
  __device__ T a(int, int, int o) const { return sa[o]; }
  __device__ T m(int, int, int o) const { return sm[o]; }
  __device__ T c(int, int, int o) const { return sc[o]; }
};
template <typename T, int NL, int R>
struct LaneFactors {
  T a_[NL][R], m_[NL][R], c_[NL][R];
  __device__ T a(int l, int t, int) const { return a_[l][t]; }
  __device__ T m(int l, int t, int) const { return m_[l][t]; }
  __device__ T c(int l, int t, int) const { return c_[l][t]; }
};

template <typename T, int NL, int RR = 0, typename FAC>
__device__ __forceinline__ void warp_lines_solve(T *sr, const FAC &fac, int stride, const LineLayout &Lo,
                                                 int lane) {
  const int q0 = lane * Lo.R, cnt = max(0, min(Lo.R, Lo.nr - q0));
  T B[NL], G[NL], d[NL];
#pragma unroll
  for (int l = 0; l < NL; l++) { B[l] = T(1); G[l] = T(0); }
  rows_up<RR>(cnt, [&](int t) {
#pragma unroll
    for (int l = 0; l < NL; l++) {
      const int o = l * stride + t * 33 + lane;
      T mq = fac.m(l, t, o);
      T beta = -mq * fac.a(l, t, o), gamma = mq * sr[o];
      B[l] = beta * B[l];
      G[l] = beta * G[l] + gamma;
    }
  });
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
#pragma unroll
    for (int l = 0; l < NL; l++) {
      T Bp = __shfl_up_sync(0xffffffffu, B[l], o), Gp = __shfl_up_sync(0xffffffffu, G[l], o);
      if (lane >= o) { G[l] = B[l] * Gp + G[l]; B[l] = B[l] * Bp; }
    }
  }
#pragma unroll
  for (int l = 0; l < NL; l++) {
    d[l] = __shfl_up_sync(0xffffffffu, G[l], 1);
    if (lane == 0) d[l] = T(0);
  }
  rows_up<RR>(cnt, [&](int t) {
#pragma unroll
    for (int l = 0; l < NL; l++) {
      const int o = l * stride + t * 33 + lane;
      T mq = fac.m(l, t, o);
      d[l] = mq * sr[o] - mq * fac.a(l, t, o) * d[l];
      sr[o] = d[l];
    }
  });
  __syncwarp();
#pragma unroll
  for (int l = 0; l < NL; l++) { B[l] = T(1); G[l] = T(0); }
  rows_down<RR>(cnt, [&](int t) {
#pragma unroll
    for (int l = 0; l < NL; l++) {
      const int o = l * stride + t * 33 + lane;
      T beta = -fac.c(l, t, o), gamma = sr[o];
      B[l] = beta * B[l];
      G[l] = beta * G[l] + gamma;
    }
  });
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
#pragma unroll
    for (int l = 0; l < NL; l++) {
      T Bn = __shfl_down_sync(0xffffffffu, B[l], o), Gn = __shfl_down_sync(0xffffffffu, G[l], o);
      if (lane + o < 32) { G[l] = B[l] * Gn + G[l]; B[l] = B[l] * Bn; }
    }
  }
#pragma unroll
  for (int l = 0; l < NL; l++) {
    d[l] = __shfl_down_sync(0xffffffffu, G[l], 1);
    if (lane == 31) d[l] = T(0);
  }
  rows_down<RR>(cnt, [&](int t) {
#pragma unroll
    for (int l = 0; l < NL; l++) {
      const int o = l * stride + t * 33 + lane;
      d[l] = sr[o] - fac.c(l, t, o) * d[l];
      sr[o] = d[l];
    }
  });
  __syncwarp();
}

// xnew = x + omega * T^-1 r on interior lines, x elsewhere; r is the residual of
// x (split sweep) or, with x == nullptr, the right-hand side (zero guess).
// A tile is TW consecutive lines (i) at one k.  (A persistent, double-buffered
// form of this kernel -- prefetching a block's next tile while it solves the
// current one -- ran slower here: with two tiles per block only two blocks fit
// on an SM, and four independent blocks hide the copies better.)

// Line of lane tx in tile bx at plane k: all lines (color < 0), or the lines of
// one zebra color, (i + k) % 2 == color, two cells apart.
__device__ __forceinline__ int tile_line(int bx, int tx, int k, int TW, int color) {
  return color < 0 ? bx * TW + tx : 2 * (bx * TW + tx) + ((color + k) & 1);
}

template <typename T>
struct Vec16;
template <>
struct Vec16<float> {
  using V = float4;
  static constexpr int W = 4;
  __device__ static float at(const V &v, int u) { return u == 0 ? v.x : u == 1 ? v.y : u == 2 ? v.z : v.w; }
};
template <>
struct Vec16<double> {
  using V = double2;
  static constexpr int W = 2;
  __device__ static double at(const V &v, int u) { return u == 0 ? v.x : v.y; }
};

// Thomas factors straight into the lanes' registers, for R <= 4 rows per
// lane: a lane's rows q0 .. q0 + R - 1 of a line are one piece of each of the
// line's runs (a, 1/m, c'), aligned to R values since runs hold a multiple of 4
// values and start 16-byte aligned.  Saves the factors' trip through shared
// memory (a store and two to four loads per value).
// Also for R = 8 in FP32 where a warp solves one line (tiles of 4 lines): the
// same 3 R values per lane as two lines of R = 4.
__host__ __device__ constexpr bool reg_factors(int bytes, int tw, int rr) {
  return rr >= 1 && (rr <= 4 || (rr == 8 && bytes == 4 && tw == kSolveThreads / 32));
}
template <typename T, int TW, int RR>
constexpr bool kRegFactors = reg_factors(sizeof(T), TW, RR);
// Rows of a line-solve tile in shared memory: the residual, then the three
// Thomas factor runs (only where they are not in registers), then x.
template <typename T, int TW, int RR>
constexpr int kTileRows = kRegFactors<T, TW, RR> ? 2 : 5;
// Shared memory of a line-solve / one-kernel zebra tile for a kernel compiled
// with RR (R at compile time; 0 = at run time).
template <typename T, int TW>
inline size_t line_solve_smem_rr(const Geom &g, int rr) {
  return sizeof(T) * (reg_factors(sizeof(T), TW, rr) ? 2 : 5) * (size_t)LineLayout::of(g.my).ls * TW;
}
// Resident blocks per SM the tile kernels are compiled for: with the factors in
// registers they fit in 48 registers, ten blocks of 128 threads (R = 8: eight).
template <typename T, int TW, int RR>
constexpr int kTileMinBlocks = kRegFactors<T, TW, RR> ? (RR == 8 ? 8 : 10) : 4;

template <int N>
__device__ __forceinline__ void ld_run(const float *p, float (&o)[N]) {
  if constexpr (N == 8) {
    const float4 v = __ldg(reinterpret_cast<const float4 *>(p));
    const float4 w = __ldg(reinterpret_cast<const float4 *>(p) + 1);
    o[0] = v.x; o[1] = v.y; o[2] = v.z; o[3] = v.w;
    o[4] = w.x; o[5] = w.y; o[6] = w.z; o[7] = w.w;
  } else if constexpr (N == 4) {
    const float4 v = __ldg(reinterpret_cast<const float4 *>(p));
    o[0] = v.x; o[1] = v.y; o[2] = v.z; o[3] = v.w;
  } else if constexpr (N == 2) {
    const float2 v = __ldg(reinterpret_cast<const float2 *>(p));
    o[0] = v.x; o[1] = v.y;
  } else {
    o[0] = __ldg(p);
  }
}
template <int N>
__device__ __forceinline__ void ld_run(const double *p, double (&o)[N]) {
  if constexpr (N == 4) {
    const double2 v = __ldg(reinterpret_cast<const double2 *>(p));
    const double2 w = __ldg(reinterpret_cast<const double2 *>(p) + 1);
    o[0] = v.x; o[1] = v.y; o[2] = w.x; o[3] = w.y;
  } else if constexpr (N == 2) {
    const double2 v = __ldg(reinterpret_cast<const double2 *>(p));
    o[0] = v.x; o[1] = v.y;
  } else {
    o[0] = __ldg(p);
  }
}

// The factors of the lines one warp solves in a tile: lines warp, warp + NW, ...
template <typename T, int TW, int RR>
using TileLaneFactors = LaneFactors<T, TW / (kSolveThreads / 32), (RR > 0 ? RR : 1)>;

template <typename T, int TW, int RR>
__device__ __forceinline__ void lane_factors_load(const LevelDev &L, int bx, int k, int color,
                                                  TileLaneFactors<T, TW, RR> &f) {
  constexpr int NW = kSolveThreads / 32, NL = TW / NW, R = RR > 0 ? RR : 1;
  const Geom &g = L.g;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, q0 = lane * R;
  const bool kin = k >= 1 && k <= g.mz - 2;
  const LineFac F = LineFac::of(g);
  const T *fa = RowOf<T>::fac(L);
#pragma unroll
  for (int l = 0; l < NL; l++) {
    const int il = tile_line(bx, warp + l * NW, k, TW, color);
    if (kin && il >= 1 && il <= g.mx - 2 && q0 < g.my - 2) {
      const T *p = fa + F.line(il, k) + q0;
      ld_run<R>(p, f.a_[l]);
      ld_run<R>(p + F.Q, f.m_[l]);
      ld_run<R>(p + 2 * (size_t)F.Q, f.c_[l]);
    } else {
#pragma unroll
      for (int t = 0; t < R; t++) f.a_[l][t] = f.m_[l][t] = f.c_[l][t] = T(0);
    }
  }
}

// Stage a tile: the residual (and x) rows by element copies (the lines are one
// or two cells apart in rows of the caller's layout), the Thomas factors by
// 16-byte loads of the lines' contiguous runs -- each warp takes whole runs,
// all of its loads in flight before it stores any.
// rx: stage r and x (else only the factors, the caller fills r and x).
// fac: stage the factors (else the caller holds them in registers).
template <typename T, int TW, int RR = 0>
__device__ __forceinline__ void solve_tile_load(const LevelDev &L, const T *__restrict__ r, const T *__restrict__ x,
                                                int bx, int k, T *st, int color = -1, bool rsplit = false,
                                                bool rx = true, bool fac = true) {
  const Geom &g = L.g;
  const int my = g.my, mx = g.mx;
  if (!(k >= 1 && k <= g.mz - 2)) return;
  const LineLayout Lo = LineLayout::fixed<RR>(my);
  T *sr = st, *sa = sr + Lo.ls * TW, *sx = st + (kTileRows<T, TW, RR> - 1) * Lo.ls * TW;
  const int tx = threadIdx.x % TW, ty = threadIdx.x / TW;
  constexpr int ny = kSolveThreads / TW;
  const int i = tile_line(bx, tx, k, TW, color);
  if (rx && i >= 1 && i <= mx - 2) {
    const int col = (k * my) * mx + i;
    for (int j = 1 + ty; j <= my - 2; j += ny) {
      const int p = col + j * mx;
      const int s = tx * Lo.ls + Lo.pos(j - 1);
      cp_async_el(sr + s, r + (rsplit ? SplitRow::at(g, i, j, k) : p));
      if (x) cp_async_el(sx + s, x + p);
    }
  }
  if (!fac) return;
  using VT = Vec16<T>;
  using V = typename VT::V;
  constexpr int W = VT::W, NW = kSolveThreads / 32, RUNS = (3 * TW + NW - 1) / NW;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const LineFac F = LineFac::of(g);
  const int per_arr = F.Q / W;
  const T *fa = RowOf<T>::fac(L);
  for (int v0 = 0; v0 < per_arr; v0 += 32) {
    const int v = v0 + lane;
    V val[RUNS];
    bool ok[RUNS];
#pragma unroll
    for (int u = 0; u < RUNS; u++) {
      const int run = warp + u * NW, lt = run / 3, arr = run - 3 * lt;
      const int il = tile_line(bx, lt, k, TW, color);
      ok[u] = run < 3 * TW && v < per_arr && il >= 1 && il <= mx - 2;
      if (ok[u]) val[u] = __ldg(reinterpret_cast<const V *>(fa + F.line(il, k) + (size_t)arr * F.Q) + v);
    }
#pragma unroll
    for (int u = 0; u < RUNS; u++) {
      if (!ok[u]) continue;
      const int run = warp + u * NW, lt = run / 3, arr = run - 3 * lt;
      T *dst = sa + (arr * TW + lt) * Lo.ls;
#pragma unroll
      for (int w = 0; w < W; w++)
        if (v * W + w < Lo.nr) dst[Lo.pos(v * W + w)] = VT::at(val[u], w);
    }
  }
}

// Solve the tile's lines in shared memory and write it out (the tile's copies
// have landed and the block is synchronised when this is entered).
template <typename T, int TW, int RR = 0>
__device__ __forceinline__ void solve_tile_finish(const LevelDev &L, const T *__restrict__ x, T *__restrict__ xnew,
                                                  T omega, int bx, int k, T *st, int color,
                                                  const TileLaneFactors<T, TW, RR> &lf) {
  const Geom &g = L.g;
  const int my = g.my, mx = g.mx;
  const LineLayout Lo = LineLayout::fixed<RR>(my);
  T *sr = st, *sa = sr + Lo.ls * TW, *sm = sa + Lo.ls * TW, *sc = sm + Lo.ls * TW;
  T *sx = st + (kTileRows<T, TW, RR> - 1) * Lo.ls * TW;
  const int tx = threadIdx.x % TW, ty = threadIdx.x / TW;
  constexpr int ny = kSolveThreads / TW;
  const int i = tile_line(bx, tx, k, TW, color);
  const bool kin = k >= 1 && k <= g.mz - 2;
  const bool line = i >= 1 && i <= mx - 2 && kin;
  // every warp solves TW / 4 lines (warp, warp + 4, ...) together; lines off
  // the interior hold stale shared memory whose results are never read
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  constexpr int NW = kSolveThreads / 32, NL = TW / NW;
  if (kin) {
    const int o = warp * Lo.ls;
    if constexpr (kRegFactors<T, TW, RR>) {
      warp_lines_solve<T, NL, RR>(sr + o, lf, NW * Lo.ls, Lo, lane);
    } else {
      const SmemFactors<T> fac{sa + o, sm + o, sc + o};
      warp_lines_solve<T, NL, RR>(sr + o, fac, NW * Lo.ls, Lo, lane);
    }
  }
  __syncthreads();
  if (i >= mx) return;
  const int col = (k * my) * mx + i;
  if (color >= 0) {
    // zebra: only the colour's interior rows change (x in place, or zeroed by
    // the caller for a zero guess)
    if (!line) return;
    for (int j = 1 + ty; j <= my - 2; j += ny) {
      const int s = tx * Lo.ls + Lo.pos(j - 1);
      const T xo = x ? sx[s] : T(0);
      xnew[col + j * mx] = xo + omega * sr[s];
    }
    return;
  }
  for (int j = ty; j < my; j += ny) {
    const int p = col + j * mx;
    if (line && j >= 1 && j <= my - 2) {
      const int s = tx * Lo.ls + Lo.pos(j - 1);
      T xo = x ? sx[s] : T(0);
      xnew[p] = xo + omega * sr[s];
    } else {
      xnew[p] = x ? x[p] : T(0);
    }
  }
}

// One tile per block: issue every copy, wait once, solve, write.
// color >= 0: zebra half-sweep on the lines of that color only, x updated in
// place (xnew == x; a tile reads its lines' x before it writes them) -- or,
// with x == nullptr, written on those lines only (the caller zeroed the rest).
// rsplit: r is in the colour-split row layout (a zebra residual), else in the
// level's own layout.
template <typename T, int TW, int RR = 0>
__device__ __forceinline__ void line_solve_body(const LevelDev &L, const T *__restrict__ r, const T *x, T *xnew,
                                                T omega, int bx, int k, unsigned char *smem_raw, int color = -1,
                                                bool rsplit = false) {
  T *st = reinterpret_cast<T *>(smem_raw);
  TileLaneFactors<T, TW, RR> lf;
  solve_tile_load<T, TW, RR>(L, r, x, bx, k, st, color, rsplit, true, !kRegFactors<T, TW, RR>);
  if constexpr (kRegFactors<T, TW, RR>) lane_factors_load<T, TW, RR>(L, bx, k, color, lf);
  cp_async_wait_all();
  __syncthreads();
  solve_tile_finish<T, TW, RR>(L, x, xnew, omega, bx, k, st, color, lf);
}

// Tiles of a line solve: all lines or one color's.
template <int TW>
__host__ __device__ inline int solve_tiles_x(const Geom &g, int color) {
  return color < 0 ? (g.mx + TW - 1) / TW : ((g.mx + 1) / 2 + TW - 1) / TW;
}

// Residual b - A x on the interior cells of one zebra color ((i + k) % 2 ==
// color), one thread per cell, kFlat threads per block over the colour's cells
// of one interior plane, written in the colour-split row layout (SplitRow).
template <typename T>
struct ColorRow;
template <>
struct ColorRow<float> {
  template <bool X>
  __device__ static float r(const Geom &g, const LevelDev &L, const float *x, int i, int j, int k, int p, int n) {
    if constexpr (!X) {
      if (L.cs32) return row32_split(g, L.cs32, x, i, j, k, p);
    }
    return row32<float, X>(g, L.gf32, L.ajf32, L.code, x, i, j, k, p, n);
  }
};
template <>
struct ColorRow<double> {
  template <bool X>
  __device__ static double r(const Geom &g, const LevelDev &L, const double *x, int i, int j, int k, int p, int n) {
    return row64<double, X>(g, L.w64, L.code, x, i, j, k, p, n);
  }
};
template <typename T, bool X = true>
__device__ __forceinline__ void resid_color_body(const LevelDev &L, const T *__restrict__ x, const T *__restrict__ b,
                                                 T *__restrict__ r, int color, int bx, int by, int plane) {
  const Geom g = L.g;
  // interior plane k = plane + 1; the colour's interior cells of the plane, row
  // by row, i = first, first + 2, ...
  (void)by;
  const int k = plane + 1;
  const int first = ((color + k) & 1) ? 1 : 2;
  const int nci = first <= g.mx - 2 ? (g.mx - 2 - first) / 2 + 1 : 0;
  const int idx = bx * kFlat + threadIdx.x;
  if (idx >= nci * (g.my - 2)) return;
  // idx / nci from a float reciprocal, corrected to the exact quotient
  int jj = (int)(((float)idx + 0.5f) * __frcp_rn((float)nci));
  jj -= jj * nci > idx;
  jj += (jj + 1) * nci <= idx;
  const int i = first + 2 * (idx - jj * nci), j = 1 + jj;
  const int n = (int)g.n(), p = (k * g.my + j) * g.mx + i;
  r[SplitRow::at(g, i, j, k)] = b[p] - ColorRow<T>::template r<X>(g, L, x, i, j, k, p, n);
}

// A zebra half-sweep in one kernel: a tile of one colour's lines computes its
// residual straight into shared memory, solves, and writes its lines.
//  - In place (xout == xin), for levels without cross-derivative terms: the
//    7-point rows couple a line (i, k) only to the lines (i +- 1, k) and
//    (i, k +- 1), all of the other colour, so a tile never reads a line that
//    another tile writes.  A periodic wrap in x (z) keeps the colours apart only
//    when mx (mz) is even (zebra_fusable).
//  - Out of place (xout != xin), for any level: the residual reads xin only,
//    which no tile writes, so the diagonal couplings of the 19-point rows are
//    no race either.  Each block also copies the rest of its 2 TW columns of the
//    plane (the other colour's lines and the ring) from xin to xout, so xout is
//    complete after the launch.
// Either way the results equal the two-kernel form, whose residual also sees x
// as it was before the half-sweep.
template <typename T, int TW, int RR = 0, bool X = false>
__device__ __forceinline__ void zebra_fused_body(const LevelDev &L, const T *__restrict__ b, const T *xin, T *xout,
                                                 T omega, int bx, int k, unsigned char *smem_raw, int color) {
  const Geom &g = L.g;
  const int my = g.my, mx = g.mx, n = (int)g.n();
  T *st = reinterpret_cast<T *>(smem_raw);
  const bool kin = k >= 1 && k <= g.mz - 2;
  if (kin) {
    const LineLayout Lo = LineLayout::fixed<RR>(my);
    T *sr = st, *sx = st + (kTileRows<T, TW, RR> - 1) * Lo.ls * TW;
    const int tx = threadIdx.x % TW, ty = threadIdx.x / TW;
    constexpr int ny = kSolveThreads / TW;
    const int i = tile_line(bx, tx, k, TW, color);
    if (i >= 1 && i <= mx - 2) {
      const int col = (k * my) * mx + i;
#pragma unroll 4
      for (int j = 1 + ty; j <= my - 2; j += ny) {
        const int p = col + j * mx;
        const int s = tx * Lo.ls + Lo.pos(j - 1);
        sr[s] = b[p] - ColorRow<T>::template r<X>(g, L, xin, i, j, k, p, n);
        sx[s] = xin[p];
      }
    }
    // the factors, as the line solve stages them (nothing to copy asynchronously)
    if constexpr (!kRegFactors<T, TW, RR>) solve_tile_load<T, TW, RR>(L, nullptr, nullptr, bx, k, st, color, false, false);
  }
  if (xout != xin) {
    // the block's columns [2 TW bx, 2 TW (bx + 1)) of plane k, except the cells
    // its line solves write
    const int c0 = 2 * TW * bx, par = (color + k) & 1;
    for (int e = threadIdx.x; e < 2 * TW * my; e += kSolveThreads) {
      const int j = e / (2 * TW), i = c0 + (e - j * 2 * TW);
      if (i >= mx) continue;
      const bool solved = kin && i >= 1 && i <= mx - 2 && j >= 1 && j <= my - 2 && (i & 1) == par;
      if (!solved) {
        const int p = (k * my + j) * mx + i;
        xout[p] = xin[p];
      }
    }
  }
  // register factors after the residual loop, so that they do not add to its
  // registers
  TileLaneFactors<T, TW, RR> lf;
  if constexpr (kRegFactors<T, TW, RR>) lane_factors_load<T, TW, RR>(L, bx, k, color, lf);
  __syncthreads();
  solve_tile_finish<T, TW, RR>(L, xin, xout, omega, bx, k, st, color, lf);
}


// ------------------------------------------------------------------ transfers
// Products in the transfers are rounded on their own (no fused multiply-add), as
// the reference's C evaluates them, so FP64 transfers match it bit for bit.
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double div_rn(double a, double b) { return __ddiv_rn(a, b); }
__device__ __forceinline__ float div_rn(float a, float b) { return __fdiv_rn(a, b); }
// Restriction weight of a fine cell, max(0, 1 - nvert): FP64 from nvert (as the
// reference), FP32 from the set-up copy of the same value rounded to float.
template <typename T>
struct FineWeight;
template <>
struct FineWeight<double> {
  __device__ static double w(const LevelDev &F, int q) {
    double wt = 1.0 - F.nvert[q];
    return wt > 0.0 ? wt : 0.0;
  }
};
template <>
struct FineWeight<float> {
  __device__ static float w(const LevelDev &F, int q) { return F.wgt32[q]; }
};

// MyRestriction (poisson.c:129-226): coarse = 0.125 * sum over the 8 children of
// x * max(0, 1 - nvert_fine) (children coincide along a semi-coarsened
// direction); zero on the ring and on blocked coarse cells.  The children are
// summed in the reference's order.  Index arithmetic in int: a level holds
// fewer than 2^31 cells (checked at set-up).
template <typename T>
__device__ __forceinline__ void restrict_body(const LevelDev &F, const LevelDev &C, const T *__restrict__ xf,
                                              T *__restrict__ xc, int bx, int by, int bz) {
  const int cmx = C.g.mx, cmy = C.g.my, cmz = C.g.mz;
  (void)by;
  const int idx = bx * kFlat + threadIdx.x;
  if (idx >= cmx * cmy) return;
  const int j = idx / cmx, i = idx - j * cmx, k = bz;
  const int p = k * cmx * cmy + idx;
  if (i == 0 || i == cmx - 1 || j == 0 || j == cmy - 1 || k == 0 || k == cmz - 1 || (C.code[p] & CODE_BLOCKED)) {
    xc[p] = T(0);
    return;
  }
  const int isc = C.isc, jsc = C.jsc, ksc = C.ksc;
  const int ih = isc ? i : 2 * i, jh = jsc ? j : 2 * j, kh = ksc ? k : 2 * k;
  const int fmx = F.g.mx, fpl = fmx * F.g.my;
  const int q = (kh * F.g.my + jh) * fmx + ih;
  const int oi = isc ? 0 : 1, oj = jsc ? 0 : fmx, ok = ksc ? 0 : fpl;
  auto W = [&](int o) { return mul_rn(xf[q - o], FineWeight<T>::w(F, q - o)); };
  T s = W(0);
  s = add_rn(s, W(oi));
  s = add_rn(s, W(oj));
  s = add_rn(s, W(ok));
  s = add_rn(s, W(oi + oj));
  s = add_rn(s, W(oj + ok));
  s = add_rn(s, W(oi + ok));
  s = add_rn(s, W(oi + oj + ok));
  xc[p] = mul_rn(T(0.125), s);
}

// MyInterpolation (poisson.c:228-370), added into xf: cell-centred trilinear
// weights 27/9/9/3/9/3/3/1 over 64 toward the neighbour on the child's side,
// falling back to injection next to walls and blocked coarse cells.  The
// blocked tests read the codes' blocked bit (nvert > 0.1); the divisions by 64
// are multiplications by 1/64, which round identically (an exact power of two).
template <typename T>
__device__ __forceinline__ void prolong_body(const LevelDev &C, const LevelDev &F, const T *__restrict__ xc,
                                             T *__restrict__ xf, int bx, int by, int bz) {
  const int fmx = F.g.mx, fmy = F.g.my, fmz = F.g.mz;
  (void)by;
  const int idx = bx * kFlat + threadIdx.x;
  if (idx >= fmx * fmy) return;
  const int j = idx / fmx, i = idx - j * fmx, k = bz;
  if (i == 0 || i == fmx - 1 || j == 0 || j == fmy - 1 || k == 0 || k == fmz - 1) return;
  const int p = k * fmx * fmy + idx;
  if (F.code[p] & CODE_BLOCKED) return;
  const int isc = F.isc, jsc = F.jsc, ksc = F.ksc;
  int ic, jc, kc, ia, ja, ka;
  if (isc) { ic = i; ia = 0; } else { ic = (i + 1) / 2; ia = (i - 2 * ic) == 0 ? 1 : -1; if (i == 1 || i == fmx - 2) ia = 0; }
  if (jsc) { jc = j; ja = 0; } else { jc = (j + 1) / 2; ja = (j - 2 * jc) == 0 ? 1 : -1; if (j == 1 || j == fmy - 2) ja = 0; }
  if (ksc) { kc = k; ka = 0; } else { kc = (k + 1) / 2; ka = (k - 2 * kc) == 0 ? 1 : -1; if (k == 1 || k == fmz - 2) ka = 0; }
  const int cmx = C.g.mx, cpl = cmx * C.g.my;
  const int q = (kc * C.g.my + jc) * cmx + ic;
  const uint32_t *cc = C.code;
  if (ka != 0 && (cc[q + ka * cpl] & CODE_BLOCKED)) ka = 0;
  if (ja != 0 && (cc[q + ja * cmx] & CODE_BLOCKED)) ja = 0;
  if (ia != 0 && (cc[q + ia] & CODE_BLOCKED)) ia = 0;
  const int oj = ja * cmx, ok = ka * cpl;
  T s1 = add_rn(add_rn(add_rn(mul_rn(xc[q], T(9)), mul_rn(xc[q + oj], T(3))), mul_rn(xc[q + ia], T(3))),
                xc[q + ia + oj]);
  T s2 = add_rn(add_rn(add_rn(mul_rn(xc[q + ok], T(9)), mul_rn(xc[q + oj + ok], T(3))), mul_rn(xc[q + ia + ok], T(3))),
                xc[q + ia + oj + ok]);
  T v = add_rn(mul_rn(mul_rn(s1, T(3)), T(0.015625)), mul_rn(s2, T(0.015625)));
  xf[p] = add_rn(xf[p], v);
}


}  // namespace cvb
